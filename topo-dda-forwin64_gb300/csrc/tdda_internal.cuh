// tdda_internal.cuh -- device data layout and kernel launchers shared by the
// C-ABI implementation (tdda_api.cu) and the kernels (tdda_kernels.cu).
//
// HBM layout of one core (one lattice at one wavelength):
//   cellmap   int32 [Nx][Ny][Nz]          dipole index of each cell, -1 if empty
//   green64   double2 [Hy][Hx][Hz][6]     folded Green spectrum / (Mx My Mz)
//   green32   float2  [Hy][Hx][3][Hz][2]  the same rounded to FP32 (mixed path), as
//                                         planes of component pairs (xx|xy, xz|yy, yz|zz)
//   tw{x,y,z} double2/float2 [M]          exp(-2 pi i m / M)
//   grid      cx<T> [nrhs][3][Nx][My][Mz]  FFT work grid (x kept to the lattice)
// with H = M/2 + 1 per axis (the tensor components are even or odd in each
// axis, so the spectrum at M-k equals +/- the spectrum at k).
#pragma once

#include <cuda_runtime.h>

#include "tdda_fft.cuh"
#include "tdda_tensor.cuh"

namespace tdda {

struct Geom {
    int Nx, Ny, Nz;    // lattice box
    int N;             // dipoles
    AxisPlan px, py, pz;
    int Hx, Hy, Hz;    // folded Green extents
    long long sy, sx, sc, sb;  // grid strides (y, x, component, rhs) in elements
    int dense;         // 1: the full box in build_a_bulk order, dipole (x Ny + y) Nz + z
                       // in every cell (tools.cpp:497-510), so no cellmap lookup
    // FP32 x pass (set by tdda_core_set_xpass / tdda_core_autotune):
    int x_form;        // 0: the register form on a two-stage plan where one is compiled,
                       // 1: the shared-memory form on the length's compiled plan
    int x_tile;        // z-columns per block of the register form: 8, 16, or 0 for
                       // the built-in choice (16 for M = 128, else 8)
    int multi;         // 1: a cross-lattice batch -- every right-hand side brings its own
                       // lattice (RhsVecs::Nx ... green); Nx, Ny, Nz, N above are the
                       // largest the grid shape holds (the strides follow them)
    int early;         // the fused FP32 pass kernels launched early (launch_early): 0 no;
                       // 1 the next kernel released after the wait; 2 before the last
                       // stage; 3 per launch: 1 for at most `sms` blocks, else 2
    int sms;           // streaming multiprocessors of the core's device
};

// The release point of an early launch of `blocks` blocks.  Released right after
// its wait, a kernel of more blocks than SMs had the next kernel's blocks stack
// up on the SMs its own blocks left free first (64x64x16 solve: -6%); released
// before its last stage, it keeps the ordinary placement.
inline Geom early_geom(Geom g, long long blocks) {
    if (g.early == 3) g.early = blocks <= g.sms ? 1 : 2;
    return g;
}

// A launch that lets the kernel's blocks start while the previous kernel of the
// stream is still running (programmatic dependent launch), when `early` is set:
// the blocks stage their constants (twiddles, the lattice), then wait in
// grid_dep_wait() for the previous kernel's completion and memory before they
// touch anything another kernel writes.  Only kernels that call grid_dep_wait
// on every path that reads or writes such memory may be launched this way.
// Inside a stream capture the dependency becomes a programmatic graph edge.
template <typename... P, typename... A>
cudaError_t launch_early(bool early, void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                         A... args) {
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cfg.attrs = at;
    cfg.numAttrs = early ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, args...);
}

// solver status values (mirrored in include/tdda.h)
enum : int { ST_RUNNING = 0, ST_CONVERGED = 1, ST_BREAKDOWN = 2, ST_MAXITER = 3, ST_NAN = 4 };

// FP64 scalars of one BiCGSTAB right-hand side (DDAModel.cpp:153-156, 186-255)
struct SolveState {
    double2 alpha, beta, zeta;
    double2 rho;       // r0 . r      (current residual)
    double2 rho_prev;  // r0 . rl     (previous residual)
    double rnorm2;     // |r|^2
    double Enorm;      // |E|
    double tol;
    double error;      // |r| / |E| at the end
    int status;
    int it;            // completed loop iterations
    int max_it;
    int iterations;    // ITERATION as the reference reports it
    int init;          // the next step finalisation is the initial one (no convergence check)
    int pending;       // deferred update of P and r not yet applied (FP64 deferred form)
    // The FP32 inner solve keeps its step scalars in FP32 (its kernels use
    // them so), in two slots: step k (parity p = k & 1) reads the slots q = p ^ 1
    // of step k - 1 and writes slot p, so no kernel reads a field one of its own
    // blocks writes (the scalars are formed by the consuming kernels).
    float2 alpha32[2], beta32[2], zeta32[2], rho32[2];
    int it32[2];       // completed steps after step k
    int init32[2];     // slot q of the first step: the initial products (no convergence check)
    int last_slot;     // slot of the step whose update is pending when the solve stopped, or -1
    float Enorm32, tol32;
    // the device-side loop of the FP32 inner solve (kept in the state of the
    // first right-hand side of a batch): chunks of steps run, and the limit
    int chunks, chunk_limit;
};

// per right-hand side: the vectors of one solve.  FP64 vectors (and the
// double-float residual product, which reads them) are AoS [x,y,z] per dipole,
// the layout of the C ABI; the FP32 vectors of the inner solve, internal to
// the library, are SoA [c][dipole], so the gather and scatter of a pass block
// (one component of one x-plane) read and write whole sectors.
template <typename T> struct RhsVecs {
    cx<T>* P;
    cx<T>* E;
    cx<T>* r;
    cx<T>* r0;
    cx<T>* p;
    cx<T>* u;
    cx<T>* t;
    cx<T>* Ap;
    cx<T>* At;
    const cx<T>* al;
    // FP32 inner solve with Jacobi right preconditioning (TDDA_FP32_JACOBI): the
    // gathers scatter pre v = v / al onto the grid and the sinks add 1 v (al
    // then points to ones), so every product is A D^-1 v with D = diag(al);
    // the correction is D^-1 of the inner solution.  nullptr otherwise.
    const cx<T>* pre;
    SolveState* st;
    double* part;        // reduction partials, kPartSlots x maxblk doubles
    unsigned int* cnt;   // last-block counters, kCounters
    // Cross-lattice batches (the FP32 fused passes on one FFT grid shape): the
    // lattice of this right-hand side when it is not the launch's own -- its
    // box, dipole count, build_a_bulk flag, cellmap and folded Green spectrum.
    // Read only when Geom::multi is set.
    const int* cellmap;
    const cx<T>* green;
    int Nx, Ny, Nz, N, dense;
};
// the lattice a pass kernel works on for one right-hand side: its own (cross-lattice
// batches) or the launch's
struct Lat {
    int Nx, Ny, Nz, N, dense;
    const int* cellmap;
};
template <typename T>
__host__ __device__ __forceinline__ Lat lattice_of(const Geom& g, const RhsVecs<T>& R, const int* cellmap) {
    if (g.multi) return Lat{R.Nx, R.Ny, R.Nz, R.N, R.dense, R.cellmap};
    return Lat{g.Nx, g.Ny, g.Nz, g.N, g.dense, cellmap};
}
// entry of component c of dipole i in a vector of N dipoles
template <typename T> __host__ __device__ __forceinline__ long long vec_index(long long i, int c, int N) {
    if constexpr (sizeof(T) == 4) return (long long)c * N + i;
    return 3 * i + c;
}
constexpr int kPartSlots = 8;
constexpr int kCounters = 8;

// what the first z-pass transforms (the fused vector update of the solver)
enum SrcMode : int {
    SRC_IN = 0,      // v = in
    SRC_PUPD = 1,    // p = r + beta (p - u)         (DDAModel.cpp:219)
    SRC_TUPD = 2,    // t = r - alpha Ap             (DDAModel.cpp:222)
    SRC_P = 3,       // v = P                        (DDAModel.cpp:164)
    SRC_PUPD_DEF = 4,  // apply the deferred update of the previous step
                       // (u = zeta Ap, P += alpha p + zeta r - alpha u,
                       // r = t - zeta At), then p = r + beta (p - u)
};
// what the last z-pass does with A v
enum SnkMode : int {
    SNK_OUT = 0,     // out = A v
    SNK_ALB = 1,     // out = A v + al v             (DDAModel.cpp:577-586)
    SNK_AP = 2,      // Ap = A p + al p, alpha = (r0.r) / (r0.Ap)
    SNK_AT = 3,      // At = A t + al t, zeta = (At.t) / (At.At)
    SNK_RES = 4,     // r = r0 = p = E - (A P + al P), rho = r0.r   (DDAModel.cpp:164-168)
    SNK_AT_DEF = 5,  // At = A t + al t; zeta, and r0.r and |r|^2 of r = t - zeta At from
                     // r0.t, r0.At, t.t, At.t, At.At; the step logic of launch_update;
                     // the update of P and r is left pending (SRC_PUPD_DEF, launch_finish)
};

// -------------------------------------------------------------- pass dispatch
// The five passes of one A-product.  Each length-specialised translation unit
// (tdda_pass_z.cu, tdda_pass_xy.cu) holds kernels for a set of FFT lengths;
// tdda_pass_generic.cu holds the runtime-plan kernels for every length.
enum PassId : int { PASS_ZFWD = 0, PASS_YFWD = 1, PASS_XPASS = 2, PASS_YINV = 3, PASS_ZINV = 4 };
template <typename T> struct PassArgs {
    Geom g;
    int nrhs;
    const RhsVecs<T>* rhs;
    const cx<T>* green;
    const cx<T>* twx;
    const cx<T>* twy;
    const cx<T>* twz;
    const int* cellmap;
    cx<T>* grid;
    cudaStream_t stream;
    int slot;       // FP32 deferred step: parity of the step (state slots)
    int prod_nblk;  // FP32 deferred step: blocks of the sink pass whose partials this gather reads
};
// mode: SrcMode for PASS_ZFWD, SnkMode for PASS_ZINV, unused otherwise
template <typename T> cudaError_t pass_generic(int pass, int mode, const PassArgs<T>& a);
// return false (nothing launched) when the length has no specialised kernel
template <typename T> bool pass_ct_z(int pass, int mode, const PassArgs<T>& a, cudaError_t* err);
template <typename T> bool pass_ct_xy(int pass, int mode, const PassArgs<T>& a, cudaError_t* err);
// fused z+y passes: pass PASS_ZFWD launches k_zyfwd (z and y forward), pass
// PASS_ZINV launches k_yzinv (y and z inverse); only for the planes zy_fused()
// accepts (FP32, compiled (My, Mz) pairs); false means nothing was launched
template <typename T> bool pass_zy(int pass, int mode, const PassArgs<T>& a, cudaError_t* err);
bool zy_fused(const Geom& g, bool fp32);
cudaError_t configure_pass_zy();
// the double-float A-product (tdda_pass_dd.cu): residual r = E - (A P + al P)
// of the FP64 vectors of rhs (laid out as RhsVecs<double>), for the grids
// dd_lengths() accepts
bool dd_lengths(const Geom& g);
cudaError_t launch_residual_dd(const Geom& g, int nrhs, const RhsVecs<dd>* rhs, const dd2* green, const dd2* twx,
                               const dd2* twy, const dd2* twz, const int* cellmap, dd2* grid, cudaStream_t stream);
cudaError_t configure_pass_dd();
// dst = src split into double-float pairs
cudaError_t launch_to_dd(long long n, const double2* src, dd2* dst, cudaStream_t stream);
cudaError_t configure_pass_generic();
cudaError_t configure_pass_ct_z();
cudaError_t configure_pass_ct_xy();
// the FFT lengths with specialised kernels
bool ct_has_z(int Mz);
bool ct_has_xy(int M);
// FFT x lengths whose FP32 x pass is the register form (k_xpass2)
bool xpass2_length(int M);
// the further x / y lengths of tdda_pass_xy2.cu
template <typename T> bool pass_ct_xy2(int pass, int mode, const PassArgs<T>& a, cudaError_t* err);
bool ct_has_xy2(int M);
bool xpass2_length2(int M);
cudaError_t configure_pass_ct_xy2();
constexpr size_t kMaxPassSmem = 200 * 1024;

// -------------------------------------------------------------- launchers
// All launchers enqueue on `stream` and return cudaGetLastError().

// images of a lattice periodic in x and y (AProductCore.cpp:251-536)
struct PeriodicImages {
    int MAXm, MAXn;  // images m in [-MAXm, MAXm] (x), n in [-MAXn, MAXn] (y)
    double Lm, Ln;   // periods, nm
};

// Green spectrum: LDR tensor on the full grid (the sum over the images when pi
// is given, through the octant table oct of 6 Nx Ny Nz entries), 3-D forward
// FFT, fold, scale.
cudaError_t launch_green(const Geom& g, double K, double d, const double2* tw64x, const double2* tw64y,
                         const double2* tw64z, double2* full6 /* 6*Mx*My*Mz scratch */, double2* green64,
                         float2* green32, cudaStream_t stream, const Interaction& it,
                         const PeriodicImages* pi = nullptr, double2* oct = nullptr);
// the FCD Si/Ci tables (kSiCiN entries each)
cudaError_t launch_sici_table(double* si, double* ci, cudaStream_t stream);

// One A-product over nrhs right-hand sides.  rhs[] lives in device memory.
// ev, when given, holds 6 events recorded before K1..K5 and after K5; with
// the fused z+y passes ev[1] = ev[2] and ev[4] = ev[5] (K2 and K4 take no time).
// For SRC_IN with SNK_OUT / SNK_ALB the vectors used are rhs[b].p (input)
// and rhs[b].Ap (output); SNK_RES reads P and E and writes r, r0, p.
template <typename T>
cudaError_t launch_aproduct(const Geom& g, int src, int snk, int nrhs, const RhsVecs<T>* rhs,
                            const cx<T>* green, const cx<T>* twx, const cx<T>* twy, const cx<T>* twz,
                            const int* cellmap, cx<T>* grid, cudaStream_t stream, cudaEvent_t* ev = nullptr,
                            int slot = 0);
// blocks of the last pass of an A-product at precision T (the producer of the
// dot-product partials)
template <typename T> int sink_blocks(const Geom& g);
// chunks of FP32 steps one launch of the device-side loop runs at most.  A
// bounded launch keeps the host in the loop now and then: while a device-side
// loop runs, driver operations of other streams on the GPU (graph
// instantiation and destruction, module loads) can wait for it.
constexpr int kLoopChunks = 8;
// FP32 deferred step, end of a chunk of steps inside the device-side loop: one
// block forms the step end of every right-hand side for the step of parity
// `slot` (the computation the next gather repeats), counts the chunk and sets
// the loop's condition: another chunk while a right-hand side is running, fewer
// than chunk_limit chunks have run, and this launch has not run kLoopChunks.
// in_loop: launched inside the conditional node of the device-side loop (else
// the host launches each chunk and the condition is not set)
cudaError_t launch_chunk_end(const Geom& g, int nrhs, const RhsVecs<float>* rhs, int slot,
                             cudaGraphConditionalHandle loop, bool in_loop, cudaStream_t stream);

// u = zeta Ap; z = zeta r - alpha u; P += alpha p + z; r = t - zeta At;
// rho_prev = rho; rho = r0.r; convergence / breakdown / iteration limit;
// beta for the next iteration.  is_init marks the step after the three
// initial products (DDAModel.cpp:177-182), which checks no convergence.
template <typename T>
cudaError_t launch_update(const Geom& g, int nrhs, const RhsVecs<T>* rhs, int is_init, cudaStream_t stream);

// Applies the pending deferred update of P and r (SNK_AT_DEF) of every
// right-hand side that has one; the end of the FP32 inner solve.
template <typename T>
cudaError_t launch_finish(const Geom& g, int nrhs, const RhsVecs<T>* rhs, cudaStream_t stream);

// |E| of every right-hand side into st->Enorm, and reset of the state.
template <typename T>
cudaError_t launch_solve_begin(const Geom& g, int nrhs, const RhsVecs<T>* rhs, cudaStream_t stream);

// When P = 0 the initial residual is E: r = r0 = p = E, rho = r0.r.
template <typename T>
cudaError_t launch_residual_is_rhs(const Geom& g, int nrhs, const RhsVecs<T>* rhs, cudaStream_t stream);

// eps by linear interpolation in the material table and al = 1 / alpha_LDR(eps)
// for 3N densities (DDAModel.cpp:54-63, tools.cpp:617-630), FP64.
constexpr int kMaxMaterials = 16;
struct AlphaParams {
    double a1c;   // 3 d^3 / (4 pi)
    double d3;    // d^3
    double Kd2;   // (K d)^2
    double rad;   // (2/3) (K d)^3
    double S;     // sum_i (nE0_i nK_i)^2
    int nmat;
    double2 mat[kMaxMaterials];
};
cudaError_t launch_model_alpha(int n3, const double* diel_old, const AlphaParams& ap, double2* diel, double2* al,
                               float2* fal, cudaStream_t stream);

// E_inc = E0 n_E0 exp(i K d n_K . R)         (DDAModel.cpp:47-51)
cudaError_t launch_model_incident(int N, const int* R, double3 nK, double3 nE0, double E0, double K, double d,
                                  double2* E, cudaStream_t stream);

// E at npts points (nm): E_ext - sum_i A(r - d R_i) P_i, FP64 (ObjDDAModel.cpp:42-96).
// part holds 3 * field_blocks(N, npts) * npts double2.
int field_blocks(int N, int npts);
cudaError_t launch_field_at(int N, const int* R, double d, double K, const Interaction& it, const double2* P, int npts,
                            const double* pts, double3 nK, double3 nE0, double E0, double2* part, double2* E,
                            cudaStream_t stream);

// Adjoint sensitivity per design parameter (EvoDDAModel.cpp:610-638):
//   s_i = sum_{q in [off_i, off_i+1)} Re( sum_c lam_{3j+c} dal_j/drho_j P_{3j+c} ), j = dip_q,
//   lam = sum_k coef_k lam_k.  FP64, one thread per parameter in list order.
struct GradArgs {
    int nadj;
    const double2* lam[8];
    double2 coef[8];
};
cudaError_t launch_density_gradient(int nparam, const int* off, const int* dip, const double2* P, const double2* eps,
                                    const double* diel_old, const AlphaParams& ap, const GradArgs& ga, double* s,
                                    cudaStream_t stream);

// Einternal = al P / ((2 + eps) / 3)       (DDAModel.cpp:567-575)
cudaError_t launch_einternal(int n3, const double2* al, const double2* P, const double2* diel, double2* Ein,
                             cudaStream_t stream);

// mixed precision helpers: dst32 = (float) src64 ; P64 += (double) d32 ; zero
cudaError_t launch_to_f32(int n3, const double2* src, float2* dst, cudaStream_t stream);
// *flag = 1 when one of the n values is not +-0 (mode 0), or lies outside
// [0, hi) or is NaN (mode 1); else 0
cudaError_t launch_scan(long long n, const double* v, int mode, double hi, unsigned int* flag, cudaStream_t stream);
cudaError_t launch_accumulate(int n3, const float2* d, double2* P, cudaStream_t stream);
// Jacobi preconditioning: pre = 1 / al (FP32 SoA from the FP32 al), P += d pre, v = 1
cudaError_t launch_recip_f32(int n3, const float2* al, float2* pre, cudaStream_t stream);
cudaError_t launch_accumulate_scaled(int n3, const float2* d, const float2* pre, double2* P, cudaStream_t stream);
cudaError_t launch_fill_ones(long long n, float2* v, cudaStream_t stream);
// max and min |al|^2 of a model's FP32 al (as float bits) into out[0], out[1]
cudaError_t launch_al_range(int n3, const float2* al, unsigned int* out, cudaStream_t stream);
template <typename T> cudaError_t launch_zero(long long n, cx<T>* v, cudaStream_t stream);

// generic in-place 3-D FFT of a contiguous (n0, n1, n2) double2 array
cudaError_t launch_fft3d_f64(double2* data, const AxisPlan& p0, const AxisPlan& p1, const AxisPlan& p2,
                             const double2* tw0, const double2* tw1, const double2* tw2, int sign,
                             cudaStream_t stream);

int max_blocks_per_rhs(const Geom& g);
// largest dynamic shared memory any pass kernel needs for this geometry
size_t max_pass_smem(const Geom& g);

// raise the dynamic shared-memory limit of every pass kernel (once per device,
// outside any stream capture)
cudaError_t configure_kernels();

}  // namespace tdda
