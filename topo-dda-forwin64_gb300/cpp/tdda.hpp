// tdda.hpp -- C++ drop-in for the reference's AProductCore / DDAModel solve path.
//
// Header-only, over the C ABI of libtdda (include/tdda.h).  The classes keep
// the reference's constructor arguments, method names and call sequence
// (AProductCore.h:51-80, DDAModel.h:34-74), so the reference's callers
// (main.cpp:245-251, EvoDDAModel.cpp:433-457, 596-610) compile against them:
//
//     tdda::AProductCore Core(&CStr, lam, material, nback, "LDR");
//     tdda::DDAModel TestModel(&Core, n_K, E0, n_E0);
//     TestModel.bicgstab(MAX_ITERATION_DDA, MAX_ERROR);
//     TestModel.update_E_in_structure();
//
// Type parameters keep it independent of Eigen:
//   * the structure (CStr) may be any class with the reference CoreStructure's
//     getters get_N/get_Nx/get_Ny/get_Nz/get_d, get_R() -> pointer to an
//     integer vector and get_diel_old() -> pointer to a double vector (the
//     reference's own CoreStructure qualifies, CoreStructure.h:44-52);
//   * complex vectors are any contiguous container of std::complex<double>
//     with data()/size() and a size constructor (Eigen::VectorXcd,
//     std::vector<std::complex<double>>), chosen by DDAModelT's parameter.
//
// With Eigen (included before this header, as the reference's own headers do
// through Tools.h, or TDDA_WITH_EIGEN defined with Eigen on the include path)
// the getters and tensors take the reference's Eigen types, so its callers
// compile unchanged: A_dic_generator / LDR_inter return Matrix3cd, get_R()
// VectorXi*, get_diel_old() VectorXd*, get_material() VectorXcd*, and
// DDAModel::get_nK / get_nE0 Vector3d (AProductCore.h:51-80, DDAModel.h:34-74;
// ObjDDAModel.cpp:20-60 uses them so).  Without Eigen they are std::array /
// std::vector.
//
// Behaviour matches the reference where it is observable: the material is
// normalised and a vacuum permittivity bumped to 1.01 (AProductCore.cpp:19-24);
// bicgstab prints its progress when verbose and leaves get_ITERATION()
// unchanged when it does not converge (DDAModel.cpp:256-259); an unknown
// method string throws std::invalid_argument (AProductCore.cpp:567-569).  CUDA
// or argument errors, which the reference never checks, throw
// std::runtime_error.  The method string selects the interaction tensor:
// "LDR" or "FCD" (AProductCore.cpp:560-571), both built on the device.
#pragma once

#include <array>
#include <cmath>
#include <complex>
#include <cstdio>
#include <fstream>
#include <functional>
#include <iostream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "tdda.h"

#if defined(TDDA_WITH_EIGEN) && !defined(EIGEN_WORLD_VERSION)
#include <Eigen/Core>
#endif
#if defined(EIGEN_WORLD_VERSION)
#define TDDA_EIGEN_TYPES 1
#else
#define TDDA_EIGEN_TYPES 0
#endif

namespace tdda {

using cplx = std::complex<double>;

// the reference's value types (Eigen), or their plain stand-ins
#if TDDA_EIGEN_TYPES
using Tensor3 = Eigen::Matrix3cd;
using IndexVec = Eigen::VectorXi;
using RealVec = Eigen::VectorXd;
using MaterialVec = Eigen::VectorXcd;
using Vec3 = Eigen::Vector3d;
inline Tensor3 make_tensor(const cplx (&a)[6]) {
    Tensor3 m;
    m << a[0], a[1], a[2], a[1], a[3], a[4], a[2], a[4], a[5];
    return m;
}
inline Vec3 make_vec3(const double (&v)[3]) { return Vec3(v[0], v[1], v[2]); }
inline void scale(Tensor3& m, double f) { m *= f; }
#else
using Tensor3 = std::array<std::array<cplx, 3>, 3>;
using IndexVec = std::vector<int>;
using RealVec = std::vector<double>;
using MaterialVec = std::vector<cplx>;
using Vec3 = std::array<double, 3>;
inline Tensor3 make_tensor(const cplx (&a)[6]) { return {{{a[0], a[1], a[2]}, {a[1], a[3], a[4]}, {a[2], a[4], a[5]}}}; }
inline Vec3 make_vec3(const double (&v)[3]) { return {v[0], v[1], v[2]}; }
inline void scale(Tensor3& m, double f) {
    for (auto& row : m)
        for (auto& v : row) v *= f;
}
#endif

inline void check(tdda_status st, const char* where) {
    if (st != TDDA_OK) throw std::runtime_error(std::string(where) + ": " + tdda_last_error());
}

template <class V> inline const double* dptr(const V& v) { return reinterpret_cast<const double*>(v.data()); }
template <class V> inline double* dptr(V& v) { return reinterpret_cast<double*>(v.data()); }

class AProductCore {
   public:
    // AProductCore(CoreStructure*, double lam, VectorXcd material, double nback, string method)
    template <class CStrT, class MatVec>
    AProductCore(CStrT* CStr, double lam, const MatVec& material, double nback, const std::string& method,
                 int max_rhs = 1, int device = 0)
        : lam_(lam), nback_(nback) {
        init(CStr, material, method, max_rhs, device, false);
    }
    // AProductCore(CoreStructure*, double lam, VectorXcd material, double nback, int MAXm, int MAXn,
    //              double Lm, double Ln, string method)     AProductCore.cpp:251-536
    template <class CStrT, class MatVec>
    AProductCore(CStrT* CStr, double lam, const MatVec& material, double nback, int MAXm, int MAXn, double Lm,
                 double Ln, const std::string& method, int max_rhs = 1, int device = 0)
        : lam_(lam), nback_(nback), MAXm_(MAXm), MAXn_(MAXn), Lm_(Lm), Ln_(Ln) {
        init(CStr, material, method, max_rhs, device, true);
    }
    AProductCore(const AProductCore&) = delete;
    AProductCore& operator=(const AProductCore&) = delete;
    ~AProductCore() { tdda_core_destroy(h_); }

   private:
    template <class CStrT, class MatVec>
    void init(CStrT* CStr, const MatVec& material, const std::string& method, int max_rhs, int device,
              bool periodic) {
        const double lam = lam_, nback = nback_;
        if (method != "LDR" && method != "FCD")
            throw std::invalid_argument("\"" + method + "\" is not a valid polarizabiliy calculation method.");
        N_ = CStr->get_N();
        Nx_ = CStr->get_Nx();
        Ny_ = CStr->get_Ny();
        Nz_ = CStr->get_Nz();
        d_ = CStr->get_d();
        const auto* R = CStr->get_R();
        R_.resize(3 * (size_t)N_);
        for (size_t i = 0; i < (size_t)R_.size(); i++) R_[i] = (int)(*R)(i);
        diel_old_ = [CStr](std::vector<double>& out) {
            const auto* dv = CStr->get_diel_old();
            out.resize((size_t)dv->size());
            for (size_t i = 0; i < out.size(); i++) out[i] = (*dv)(i);
        };
        // get_diel_old() hands out the structure's own vector, as the reference does
        // (AProductCore::get_diel_old returns CStr->get_diel_old())
        if constexpr (std::is_convertible<decltype(CStr->get_diel_old()), RealVec*>::value)
            diel_ptr_ = [CStr]() -> RealVec* { return CStr->get_diel_old(); };
        std::vector<double> mat(2 * (size_t)material.size());
        for (size_t i = 0; i < (size_t)material.size(); i++) {
            mat[2 * i] = std::real(material[i]);
            mat[2 * i + 1] = std::imag(material[i]);
        }
        tdda_core_desc desc;
        desc.Nx = Nx_;
        desc.Ny = Ny_;
        desc.Nz = Nz_;
        desc.N = N_;
        desc.R = R_.data();
        desc.d = d_;
        desc.lam = lam;
        desc.nback = nback;
        desc.material = mat.data();
        desc.nmat = (int)material.size();
        desc.method = method == "LDR" ? TDDA_METHOD_LDR : TDDA_METHOD_FCD;
        desc.max_rhs = max_rhs;
        desc.device = device;
        if (periodic)
            check(tdda_core_create_periodic(&desc, MAXm_, MAXn_, Lm_, Ln_, &h_), "AProductCore");
        else
            check(tdda_core_create(&desc, &h_), "AProductCore");
        material_.resize(material.size());
        check(tdda_core_info(h_, &K_, grid_.data(), reinterpret_cast<double*>(material_.data())), "AProductCore");
    }

   public:

    // VectorXcd Aproduct(VectorXcd& b)     AProductCore.cpp:697-758
    template <class V> V Aproduct(const V& b) {
        V y(b.size());
        check(tdda_aproduct(h_, TDDA_FP64, dptr(b), dptr(y), TDDA_MEM_HOST), "Aproduct");
        return y;
    }
    // Matrix3cd LDR_inter(double x, double y, double z)     AProductCore.cpp:588-623
    Tensor3 LDR_inter(double x, double y, double z) const {
        double t[12];
        check(tdda_core_ldr_inter(h_, x, y, z, t), "LDR_inter");
        cplx a[6];
        for (int l = 0; l < 6; l++) a[l] = cplx(t[2 * l], t[2 * l + 1]);
        return make_tensor(a);
    }
    // Matrix3cd A_dic_generator(double x, double y, double z)     AProductCore.cpp:560-571 (LDR or FCD)
    Tensor3 A_dic_generator(double x, double y, double z) const {
        double t[12];
        check(tdda_core_interaction(h_, x, y, z, t), "A_dic_generator");
        cplx a[6];
        for (int l = 0; l < 6; l++) a[l] = cplx(t[2 * l], t[2 * l + 1]);
        return make_tensor(a);
    }
    // Matrix3cd A_dic_generator(double x, double y, double z, int m, int n)     AProductCore.cpp:573-586
    Tensor3 A_dic_generator(double x, double y, double z, int m, int n) const {
        x = x + m * Lm_;
        y = y + n * Ln_;
        Tensor3 r = A_dic_generator(x, y, z);
        scale(r, std::exp(-std::pow(0.01 * K_ * std::sqrt(x * x + y * y + z * z), 4)));
        return r;
    }

    int get_N() const { return N_; }
    int get_Nx() const { return Nx_; }
    int get_Ny() const { return Ny_; }
    int get_Nz() const { return Nz_; }
    double get_d() const { return d_; }
    double get_lam() const { return lam_; }
    double get_K() const { return K_; }
    double get_nback() const { return nback_; }
    double get_Lm() const { return Lm_; }
    double get_Ln() const { return Ln_; }
    // VectorXcd* get_material(), VectorXi* get_R(), VectorXd* get_diel_old()   AProductCore.h:66-75
    MaterialVec* get_material() { return &material_; }
    const MaterialVec* get_material() const { return &material_; }
    IndexVec* get_R() { return &R_; }
    const IndexVec* get_R() const { return &R_; }
    RealVec* get_diel_old() {
        if (diel_ptr_) return diel_ptr_();
        std::vector<double> tmp;
        diel_old_(tmp);
        diel_copy_.resize(tmp.size());
        for (size_t i = 0; i < tmp.size(); i++) diel_copy_[i] = tmp[i];
        return &diel_copy_;
    }
    std::array<int, 3> grid() const { return grid_; }
    tdda_core* handle() const { return h_; }
    // Not in the reference: times the FP32 x pass's forms and tiles on this core's
    // A-product of nrhs right-hand sides and keeps the fastest (tdda_core_autotune).
    tdda_xpass_tune autotune(int nrhs = 1, int reps = 10) {
        tdda_xpass_tune t{};
        check(tdda_core_autotune(h_, nrhs, reps, &t), "autotune");
        return t;
    }
    // the structure's current densities (CoreStructure::get_diel_old)
    void read_diel_old(std::vector<double>& out) const { diel_old_(out); }

   private:
    tdda_core* h_ = nullptr;
    int N_ = 0, Nx_ = 0, Ny_ = 0, Nz_ = 0;
    double d_ = 0, lam_ = 0, nback_ = 1, K_ = 0;
    IndexVec R_;
    MaterialVec material_;
    std::array<int, 3> grid_{{0, 0, 0}};
    std::function<void(std::vector<double>&)> diel_old_;
    std::function<RealVec*()> diel_ptr_;
    RealVec diel_copy_;  // get_diel_old() of a structure whose vector is of another type
    int MAXm_ = 0, MAXn_ = 0;  // periodic images (AProductCore.h members of the periodic ctor)
    double Lm_ = 0, Ln_ = 0;
};

// DDAModel over a complex vector type VectorXcd (Eigen::VectorXcd or
// std::vector<std::complex<double>>).
template <class VectorXcd = std::vector<cplx>> class DDAModelT {
   public:
    // DDAModel(AProductCore*, Vector3d n_K, double E0, Vector3d n_E0, bool verbose = true)
    template <class V3>
    DDAModelT(AProductCore* Core, const V3& n_K, double E0, const V3& n_E0, bool verbose = true)
        : core_(Core), E0_(E0), verbose_(verbose) {
        for (int j = 0; j < 3; j++) {
            nK_[j] = n_K[j];
            nE0_[j] = n_E0[j];
        }
        std::vector<double> diel;
        Core->read_diel_old(diel);
        check(tdda_model_create(Core->handle(), nK_, E0, nE0_, diel.data(), &h_), "DDAModel");
        n3_ = 3 * (size_t)Core->get_N();
        P_ = VectorXcd(n3_);
        Einternal_ = VectorXcd(n3_);
        al_ = VectorXcd(n3_);
        EResult_ = VectorXcd(n3_);  // VectorXcd::Zero(N*3) until solve_E (DDAModel.cpp:46)
        for (size_t i = 0; i < n3_; i++) EResult_[i] = cplx(0.0, 0.0);
        fetch(TDDA_FIELD_AL, al_);
    }
    // DDAModel(AProductCore*, Vector3d n_K, double E0, Vector3d n_E0, VectorXi* RResult,
    // bool verbose = true) (DDAModel.cpp:71-108): solve_E evaluates the field at the lattice
    // points RResult (3 integers per point, in units of d)
    template <class V3, class VI>
    DDAModelT(AProductCore* Core, const V3& n_K, double E0, const V3& n_E0, const VI* RResult, bool verbose = true)
        : DDAModelT(Core, n_K, E0, n_E0, verbose) {
        if (RResult->size() % 3 != 0) throw std::invalid_argument("RResult does not have a size with 3*integer");
        rresult_.resize(RResult->size());
        for (size_t i = 0; i < rresult_.size(); i++) rresult_[i] = Core->get_d() * (double)(*RResult)[i];
        EResult_ = VectorXcd(rresult_.size());
    }
    DDAModelT(const DDAModelT&) = delete;
    DDAModelT& operator=(const DDAModelT&) = delete;
    ~DDAModelT() { tdda_model_destroy(h_); }

    // void bicgstab(int MAX_ITERATION, double MAX_ERROR)     DDAModel.cpp:131-260
    void bicgstab(int MAX_ITERATION, double MAX_ERROR) { solve(MAX_ITERATION, MAX_ERROR, TDDA_FP64); }
    // bicgstab(int, double, int EVOITERATION) (DDAModel.h:41, a debug overload that prints
    // at one optimisation step): the same solve
    void bicgstab(int MAX_ITERATION, double MAX_ERROR, int /*EVOITERATION*/) { bicgstab(MAX_ITERATION, MAX_ERROR); }
    // the same solve with the FP32 convolution and FP64 refinement
    void bicgstab_mixed(int MAX_ITERATION, double MAX_ERROR) { solve(MAX_ITERATION, MAX_ERROR, TDDA_FP32_REFINE); }
    // the same with the inner solve right-preconditioned by diag(al) (TDDA_FP32_JACOBI)
    void bicgstab_jacobi(int MAX_ITERATION, double MAX_ERROR) { solve(MAX_ITERATION, MAX_ERROR, TDDA_FP32_JACOBI); }

    void change_E(const VectorXcd& E) { check(tdda_model_change_E(h_, dptr(E), TDDA_MEM_HOST), "change_E"); }
    void reset_E() { check(tdda_model_reset_E(h_), "reset_E"); }
    // UpdateAlpha: reads the structure's current densities, as the reference does
    void UpdateAlpha() {
        std::vector<double> diel;
        core_->read_diel_old(diel);
        check(tdda_model_update_alpha(h_, diel.data()), "UpdateAlpha");
        fetch(TDDA_FIELD_AL, al_);
    }
    void UpdateAlphaSingle(int idx) {
        std::vector<double> diel;
        core_->read_diel_old(diel);
        check(tdda_model_update_alpha_single(h_, idx, diel.at(3 * (size_t)idx)), "UpdateAlphaSingle");
        fetch(TDDA_FIELD_AL, al_);
    }
    void InitializeP(const VectorXcd& P) {
        check(tdda_model_initialize_P(h_, dptr(P), TDDA_MEM_HOST), "InitializeP");
        P_ = P;
    }
    VectorXcd Aproductwithalb(const VectorXcd& b) {
        VectorXcd y(b.size());
        check(tdda_model_aproduct_with_alb(h_, dptr(b), dptr(y), TDDA_MEM_HOST), "Aproductwithalb");
        return y;
    }
    void update_E_in_structure() {
        check(tdda_model_update_E_in_structure(h_), "update_E_in_structure");
        fetch(TDDA_FIELD_EINTERNAL, Einternal_);
    }
    // DDAModel.cpp:530-565: with RResult, E = E_ext - sum_i A(r - d R_i) P_i at d * RResult
    // (the incident field as ObjDDAModel.cpp:42-44 writes it; the reference's solve_E mixes
    // up the coordinates in two of its three phase terms, :544-545); without, Einternal.
    void solve_E() {
        if (rresult_.empty()) {
            EResult_ = Einternal_;
            return;
        }
        check(tdda_model_field_at(h_, (int)(rresult_.size() / 3), rresult_.data(), dptr(EResult_), TDDA_MEM_HOST),
              "solve_E");
    }
    VectorXcd* get_EResult() { return &EResult_; }

    // DDAModel::output_to_file(string save_position, int iteration, int ModelLabel)   DDAModel.cpp:618-656:
    // EResult then P, one "re+imj" / "re-imj" per line
    void output_to_file(const std::string& save_position, int iteration, int ModelLabel) {
        std::ofstream fout(save_position + "Model_results" + std::to_string(ModelLabel) + "it" +
                           std::to_string(iteration) + ".txt");
        write_complex(fout, EResult_);
        write_complex(fout, P_);
    }
    // DDAModel::output_to_file(string save_position, int iteration)   DDAModel.cpp:658-697: EResult only
    void output_to_file(const std::string& save_position, int iteration) {
        std::ofstream fout(save_position + "Model_results" + "it" + std::to_string(iteration) + ".txt");
        write_complex(fout, EResult_);
    }

    VectorXcd* get_P() { return &P_; }
    VectorXcd* get_Einternal() { return &Einternal_; }
    VectorXcd* get_al() { return &al_; }
    int get_ITERATION() const { return tdda_model_iterations(h_); }
    double get_E0() const { return E0_; }
    // Vector3d get_nE0() / get_nK()   DDAModel.h:52-53
    Vec3 get_nE0() const { return make_vec3(nE0_); }
    Vec3 get_nK() const { return make_vec3(nK_); }
    AProductCore* get_Core() { return core_; }
    // the core's getters, forwarded as DDAModel.h:63-73 declares them
    int get_N() const { return core_->get_N(); }
    int get_Nx() const { return core_->get_Nx(); }
    int get_Ny() const { return core_->get_Ny(); }
    int get_Nz() const { return core_->get_Nz(); }
    IndexVec* get_R() { return core_->get_R(); }
    double get_d() const { return core_->get_d(); }
    double get_lam() const { return core_->get_lam(); }
    double get_K() const { return core_->get_K(); }
    RealVec* get_diel_old() { return core_->get_diel_old(); }
    MaterialVec* get_material() { return core_->get_material(); }
    const tdda_solve_info& last_info() const { return info_; }
    tdda_model* handle() const { return h_; }

   private:
    std::vector<double> rresult_;  // d * RResult, nm
    VectorXcd EResult_;
    static void write_complex(std::ostream& f, const VectorXcd& v) {
        for (size_t i = 0; i < (size_t)v.size(); i++) {
            if (v[i].imag() < 0)
                f << v[i].real() << v[i].imag() << "j" << std::endl;
            else
                f << v[i].real() << "+" << v[i].imag() << "j" << std::endl;
        }
    }
    void fetch(int field, VectorXcd& out) {
        check(tdda_model_get(h_, field, dptr(out), TDDA_MEM_HOST), "DDAModel get");
    }
    void solve(int max_it, double max_err, int precision) {
        if (verbose_) std::cout << "--------------Calculation start. Iterative method used: BICGSTAB---------------\n\n";
        tdda_model* one[1] = {h_};
        const tdda_status st = precision == TDDA_FP64          ? tdda_model_bicgstab(h_, max_it, max_err, &info_)
                               : precision == TDDA_FP32_JACOBI ? tdda_solve_batch(one, 1, TDDA_FP32_JACOBI, max_it,
                                                                                  max_err, &info_)
                                                               : tdda_model_solve_mixed(h_, max_it, max_err, &info_);
        if (st != TDDA_OK && st != TDDA_NOT_CONVERGED && st != TDDA_BREAKDOWN) check(st, "bicgstab");
        fetch(TDDA_FIELD_P, P_);
        if (st == TDDA_NOT_CONVERGED) {
            std::cout << "                ERROR:does not converge in " << max_it << " iterations" << std::endl;
        } else if (verbose_) {
            if (st == TDDA_BREAKDOWN)
                std::cout << "----------------------------r0dotrl==(0,0), nan is going to occur so stop now"
                             "------------------------\n";
            std::cout << "              Error: " << info_.error << "\n              Iteration: " << get_ITERATION()
                      << "\n"
                      << std::endl;
        }
    }

    AProductCore* core_;
    tdda_model* h_ = nullptr;
    double nK_[3], nE0_[3], E0_;
    bool verbose_;
    size_t n3_ = 0;
    VectorXcd P_, Einternal_, al_;
    tdda_solve_info info_{};
};

using DDAModel = DDAModelT<>;

}  // namespace tdda
