/*
 * ref_driver.cpp -- drives the reference's own classes (compiled unchanged
 * from its sources, see oracle/Makefile target `ref`) to produce golden
 * outputs for the checker.  It builds the structure the way the reference's
 * "DDA input" task does (main.cpp:165-226: build_a_bulk -> Space ->
 * Structure -> SpacePara -> CoreStructure), then constructs
 * AProductCore(..., "LDR") and DDAModel and calls Aproduct /
 * Aproductwithalb / bicgstab / update_E_in_structure.
 *
 * I/O is raw little-endian binary (see tests/golden/make_golden.py):
 *   in : int32 mode (0 aprod, 1 solve, 2 ldr, 3 solve then the point-field
 *        objective ObjPointEDDAModel::GetVal at points, 4 aprod on the
 *        periodic core); int32 Nx Ny Nz N;
 *        f64 d lam nback; int32 nmat; f64 material[2 nmat]; f64 nK[3] E0 nE0[3];
 *        int32 max_it; f64 max_err; int32 R[3N]; f64 diel_old[3N];
 *        int32 nvec; f64 vec[nvec][6N]   (mode 2: vec = nvec points of 3 f64)
 *        mode 3 appends int32 npts; f64 pts[npts][3]
 *        mode 4 (A-products on the periodic core, AProductCore.cpp:251-536)
 *        appends int32 MAXm MAXn; f64 Lm Ln
 *        mode 5: A-products with the FCD tensor (AProductCore.cpp:625-695); its
 *        SiCi tables are read from the working directory (SiCi.cpp:8-25)
 *        mode 6: a solve, then the reference's text writers into the working
 *        directory: CoreStructure::output_to_file (CoreStructure.cpp:155-185,
 *        both modes), DDAModel::output_to_file (DDAModel.cpp:589-697) and the
 *        commondata.txt lines of main.cpp:282-289
 *        mode 7: timing.  Appends int32 reps, int32 solve (0/1).  Times the
 *        constructor AProductCore(...) + DDAModel(...), then `reps`
 *        Aproduct(vec[0]) calls, then (solve = 1) one bicgstab(max_it,
 *        max_err) from P = 0.  Writes f64 ctor_s, f64 aprod_s[reps],
 *        int32 iterations, f64 solve_s (the final error is on stdout).  Built against the CPU
 *        stand-ins (oracle/_ref/ref_timer) or against the CUDA runtime and
 *        cuFFT with kernel.cu for the GPU (oracle/_ref/ref_cufft): the
 *        reference's host<->device copies per product are part of its design
 *        and are inside the timed calls.  The process ends without running
 *        the destructors (AProductCore.cpp:540-541 frees ADev twice).
 *   out: see the per-mode writers below.
 */
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <cstdint>
#include <iostream>
#include <stdexcept>
#include <vector>

#include "AProductCore.h"
#include "CoreStructure.h"
#include "DDAModel.h"
#include "ObjDDAModel.h"
#include "Space.h"
#include "SpacePara.h"
#include "Structure.h"
#include "Tools.h"

namespace {

struct Reader {
    FILE* f;
    template <class T> T get() {
        T v;
        if (std::fread(&v, sizeof(T), 1, f) != 1) throw std::runtime_error("short read");
        return v;
    }
    template <class T> void get(T* p, size_t n) {
        if (n && std::fread(p, sizeof(T), n, f) != n) throw std::runtime_error("short read");
    }
};

void put_cvec(FILE* f, const VectorXcd& v) {
    for (int i = 0; i < v.size(); i++) {
        double re = v(i).real(), im = v(i).imag();
        std::fwrite(&re, 8, 1, f);
        std::fwrite(&im, 8, 1, f);
    }
}

VectorXcd to_cvec(const std::vector<double>& raw, size_t off, int n) {
    VectorXcd v(n);
    for (int i = 0; i < n; i++) v(i) = std::complex<double>(raw[off + 2 * i], raw[off + 2 * i + 1]);
    return v;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: ref_driver in.bin out.bin\n");
        return 2;
    }
#ifdef REF_GPU_BUILD
    // the reference checks no CUDA call: without a device it would run on garbage
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
        std::fprintf(stderr, "ref_driver: no CUDA device\n");
        return 3;
    }
#endif
    FILE* fi = std::fopen(argv[1], "rb");
    if (!fi) return 2;
    Reader rd{fi};
    int mode = rd.get<int32_t>();
    int Nx = rd.get<int32_t>(), Ny = rd.get<int32_t>(), Nz = rd.get<int32_t>(), N = rd.get<int32_t>();
    double d = rd.get<double>(), lam = rd.get<double>(), nback = rd.get<double>();
    int nmat = rd.get<int32_t>();
    std::vector<double> mat(2 * nmat);
    rd.get(mat.data(), mat.size());
    Vector3d nK, nE0;
    for (int j = 0; j < 3; j++) nK(j) = rd.get<double>();
    double E0 = rd.get<double>();
    for (int j = 0; j < 3; j++) nE0(j) = rd.get<double>();
    int max_it = rd.get<int32_t>();
    double max_err = rd.get<double>();
    std::vector<int32_t> Rraw(3 * N);
    rd.get(Rraw.data(), Rraw.size());
    std::vector<double> dielraw(3 * N);
    rd.get(dielraw.data(), dielraw.size());
    int nvec = rd.get<int32_t>();
    size_t veclen = mode == 2 ? 3 : 6 * (size_t)N;  // modes 0, 1, 3, 4: 3N complex
    std::vector<double> vecs(nvec * veclen);
    rd.get(vecs.data(), vecs.size());
    int MAXm = 0, MAXn = 0;
    double Lm = 0, Ln = 0;
    if (mode == 4) {
        MAXm = rd.get<int32_t>();
        MAXn = rd.get<int32_t>();
        Lm = rd.get<double>();
        Ln = rd.get<double>();
    }
    int reps = 0, do_solve = 0;
    if (mode == 7) {
        reps = rd.get<int32_t>();
        do_solve = rd.get<int32_t>();
    }
    std::vector<double> pts;
    if (mode == 3) {
        int npts = rd.get<int32_t>();
        pts.resize(3 * (size_t)npts);
        rd.get(pts.data(), pts.size());
    }
    std::fclose(fi);

    // main.cpp:176-220 ("DDA input"): bulk space, one structure, SpacePara, CoreStructure
    VectorXi inputGeo(3 * N);
    VectorXd inputDiel(3 * N);
    for (int i = 0; i < 3 * N; i++) {
        inputGeo(i) = Rraw[i];
        inputDiel(i) = dielraw[i];
    }
    VectorXi total_space = build_a_bulk(Nx, Ny, Nz);
    vector<Structure> ln;
    Space S(&total_space, Nx, Ny, Nz, 0, &ln);
    Structure s1(S.get_total_space(), &inputGeo);
    S = S + s1;
    Vector3i bind(1, 1, 1);
    SpacePara spacepara(&S, bind, &inputGeo, &inputDiel);
    CoreStructure CStr(&spacepara, d);

    VectorXcd material(nmat);
    for (int i = 0; i < nmat; i++) material(i) = std::complex<double>(mat[2 * i], mat[2 * i + 1]);
    using clk = std::chrono::steady_clock;
    const auto t_ctor = clk::now();
    AProductCore Core = mode == 4 ? AProductCore(&CStr, lam, material, nback, MAXm, MAXn, Lm, Ln, "LDR")
                                  : AProductCore(&CStr, lam, material, nback, mode == 5 ? "FCD" : "LDR");

    FILE* fo = std::fopen(argv[2], "wb");
    if (!fo) return 2;
    if (mode == 2) {
        double K = Core.get_K();
        std::fwrite(&K, 8, 1, fo);
        for (int v = 0; v < nvec; v++) {
            Matrix3cd A = Core.LDR_inter(vecs[3 * v], vecs[3 * v + 1], vecs[3 * v + 2]);
            const int fi6[6] = {0, 0, 0, 1, 1, 2}, se6[6] = {0, 1, 2, 1, 2, 2};
            for (int l = 0; l < 6; l++) {
                double re = A(fi6[l], se6[l]).real(), im = A(fi6[l], se6[l]).imag();
                std::fwrite(&re, 8, 1, fo);
                std::fwrite(&im, 8, 1, fo);
            }
        }
        std::fclose(fo);
        return 0;
    }

    DDAModel Model(&Core, nK, E0, nE0, true);
    if (mode == 7) {
        const double ctor_s = std::chrono::duration<double>(clk::now() - t_ctor).count();
        std::fwrite(&ctor_s, 8, 1, fo);
        VectorXcd b = to_cvec(vecs, 0, 3 * N);
        for (int k = 0; k < reps; k++) {
            const auto t0 = clk::now();
            VectorXcd y = Core.Aproduct(b);
            const double s = std::chrono::duration<double>(clk::now() - t0).count();
            std::fwrite(&s, 8, 1, fo);
        }
        int32_t it = 0;
        double solve_s = 0;
        if (do_solve) {  // the reference prints the final Error on stdout (DDAModel.cpp:236-255)
            const auto t0 = clk::now();
            Model.bicgstab(max_it, max_err);
            solve_s = std::chrono::duration<double>(clk::now() - t0).count();
            it = Model.get_ITERATION();
        }
        std::fwrite(&it, 4, 1, fo);
        std::fwrite(&solve_s, 8, 1, fo);
        std::fclose(fo);
#ifdef REF_GPU_BUILD
        const cudaError_t e = cudaDeviceSynchronize();
        const cudaError_t e2 = cudaGetLastError();
        if (e != cudaSuccess || e2 != cudaSuccess) {
            std::fprintf(stderr, "ref_driver: CUDA error %d / %d in the reference's calls\n", (int)e, (int)e2);
            std::fflush(stdout);
            std::_Exit(4);
        }
#endif
        std::fflush(stdout);
        std::_Exit(0);
    }
    VectorXi* Rs = CStr.get_R();
    for (int i = 0; i < 3 * N; i++) {
        int32_t r = (*Rs)(i);
        std::fwrite(&r, 4, 1, fo);
    }
    put_cvec(fo, *Model.get_al());
    if (mode == 0 || mode == 4 || mode == 5) {
        for (int v = 0; v < nvec; v++) {
            VectorXcd b = to_cvec(vecs, v * veclen, 3 * N);
            VectorXcd y = Core.Aproduct(b);
            put_cvec(fo, y);
            VectorXcd yw = Model.Aproductwithalb(b);
            put_cvec(fo, yw);
        }
    } else {  // modes 1, 3, 6
        if (nvec >= 1) {
            VectorXcd P0 = to_cvec(vecs, 0, 3 * N);
            Model.InitializeP(P0);
        }
        if (nvec >= 2) Model.change_E(to_cvec(vecs, veclen, 3 * N));
        Model.bicgstab(max_it, max_err);
        Model.update_E_in_structure();
        int32_t it = Model.get_ITERATION();
        std::fwrite(&it, 4, 1, fo);
        put_cvec(fo, *Model.get_P());
        put_cvec(fo, *Model.get_Einternal());
        if (mode == 6) {
            CStr.output_to_file("", 7, "normal");   // CoreStructure7.txt
            CStr.output_to_file("s", 8, "simple");  // sCoreStructure8.txt
            Model.solve_E();                        // EResult = Einternal (DDAModel.cpp:560-562)
            Model.output_to_file("", 3, 1);         // Model_results1it3.txt
            std::ofstream Common("commondata.txt");  // main.cpp:282-289
            Common << CStr.get_Nx() << std::endl << CStr.get_Ny() << std::endl << CStr.get_Nz() << std::endl
                   << CStr.get_N() << std::endl;
            Common << (spacepara.get_geometry()) << std::endl;
            Common << d << std::endl;
            Common << nE0 << std::endl;
            Common << nK << std::endl;
        }
        if (mode == 3) {
            // ObjDDAModel.cpp:20-96: |E| at each point from the solved P
            for (size_t p = 0; p + 2 < pts.size(); p += 3) {
                ObjPointEDDAModel obj(std::vector<double>{pts[p], pts[p + 1], pts[p + 2]}, &Model);
                double v = obj.GetVal();
                std::fwrite(&v, 8, 1, fo);
            }
        }
    }
    std::fclose(fo);
    return 0;
}
