// tdda_api.cu -- implementation of the C ABI in include/tdda.h.
//
// Host responsibilities: argument checks, the FFT plan per axis, the
// incident field and polarisabilities (O(N), host FP64 std::complex exactly
// as DDAModel.cpp:47-63 / tools.cpp:617-630), device memory, and the solve
// drivers.  Every O(grid) operation runs on the device (tdda_kernels.cu).
// One BiCGSTAB iteration (11 kernels) is captured once per core, precision
// and batch width as a CUDA graph and replayed; the host reads the solver
// status every few iterations.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/tdda.h"
#include "tdda_internal.cuh"
#include "tdda_session.h"

using tdda::AxisPlan;
using tdda::Geom;
using tdda::RhsVecs;
using tdda::SolveState;
using tdda::dd;
using tdda::dd2;
using cd = std::complex<double>;

namespace {

thread_local std::string g_err;

void set_err(const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
}

tdda_status cuda_fail(cudaError_t e, const char* what) {
    set_err("%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? TDDA_ERR_OUT_OF_MEMORY : TDDA_ERR_CUDA;
}

#define TDDA_CK(call)                                                   \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) return cuda_fail(e_, #call);             \
    } while (0)

// kernels launched by this library (graph replays included); a stream
// capture records launches without running them, so it does not count
std::atomic<unsigned long long> g_launches{0};
thread_local bool t_capturing = false;
inline void count_launches(int n) {
    if (!t_capturing) g_launches += (unsigned long long)n;
}
#define TDDA_CK1(call)          \
    do {                        \
        count_launches(1);      \
        TDDA_CK(call);          \
    } while (0)

constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr int kChunk = 4;        // iterations between status reads
constexpr int kMaxOuter = 10;    // refinement steps of the mixed solve

bool smooth7(int m) {
    for (int p : {2, 3, 5, 7})
        while (m % p == 0) m /= p;
    return m == 1;
}
int smooth_size(int n) {
    int m = std::max(1, n);
    while (!smooth7(m)) m++;
    return m;
}
// FFT length of an axis of N cells: the smallest 7-smooth length >= 2N - 1,
// or the next length with compiled passes when that holds at most 25% more
// points.  Any length >= 2N - 1 gives the same linear convolution
// (AProductCore.cpp:41-43 uses 2N - 1).
int fft_length(int N, bool z_axis) {
    static const int kZ[] = {20, 32, 40, 48, 56, 64};
    static const int kXY[] = {32, 40, 48, 56, 64, 80, 96, 112, 128, 160, 192, 224, 256};
    const int m = smooth_size(2 * N - 1);
    const int* f = z_axis ? kZ : kXY;
    const int nf = z_axis ? 6 : 13;
    for (int k = 0; k < nf; k++)
        if (f[k] >= m) return 4 * f[k] <= 5 * m ? f[k] : m;
    return m;
}

// radix plan: 8s and 4s (no lone 2 unless the power of two is 2), then 3, 5, 7
bool make_plan(int M, AxisPlan* ap) {
    std::memset(ap, 0, sizeof(*ap));
    ap->M = M;
    int m = M, a = 0;
    while (m % 2 == 0) { m /= 2; a++; }
    std::vector<int> r;
    while (a >= 3 && a != 4) { r.push_back(8); a -= 3; }
    while (a >= 2) { r.push_back(4); a -= 2; }
    if (a == 1) r.push_back(2);
    for (int p : {3, 5, 7})
        while (m % p == 0) { r.push_back(p); m /= p; }
    if (m != 1 || (int)r.size() > tdda::kMaxStages) return false;
    ap->nstages = (int)r.size();
    ap->rmin = 8;
    int span = 1;
    for (size_t i = 0; i < r.size(); i++) {
        ap->radix[i] = r[i];
        ap->rmin = std::min(ap->rmin, r[i]);
        ap->ns[i] = tdda::fastdiv_make((unsigned)span);
        span *= r[i];
    }
    if (r.empty()) ap->rmin = 1;
    return true;
}

void twiddles(int M, std::vector<double2>& w64, std::vector<float2>& w32) {
    w64.resize(M);
    w32.resize(M);
    for (int m = 0; m < M; m++) {
        long double a = 2.0L * 3.141592653589793238462643383279502884L * (long double)m / (long double)M;
        double c = (double)std::cos(a), s = -(double)std::sin(a);
        w64[m] = make_double2(c, s);
        w32[m] = make_float2((float)c, (float)s);
    }
}

// AProductCore::LDR_inter (AProductCore.cpp:588-623), host FP64
void ldr_host(double K, double x, double y, double z, cd out[6]) {
    using namespace std::complex_literals;
    double xs = x * x, ys = y * y, zs = z * z;
    double rn = std::sqrt(xs + ys + zs);
    if (rn == 0.0) {
        for (int l = 0; l < 6; l++) out[l] = 0.0;
        return;
    }
    double xy = x * y, yz = y * z, zx = z * x;
    double rsq = rn * rn, rcu = rn * rn * rn;
    cd c1 = 1i * K * rn;
    c1 = std::exp(c1) / rcu;
    cd c2 = (1.0 - K * rn * 1i);
    c2 = c2 / rsq;
    cd c3 = K * K - 3.0 * c2;
    out[0] = c1 * (c2 * (rsq - 3 * xs) - K * K * (ys + zs));
    out[1] = c1 * (xy * c3);
    out[2] = c1 * (zx * c3);
    out[3] = c1 * (c2 * (rsq - 3 * ys) - K * K * (zs + xs));
    out[4] = c1 * (yz * c3);
    out[5] = c1 * (c2 * (rsq - 3 * zs) - K * K * (xs + ys));
}

template <typename T> struct Graphs {
    cudaGraphExec_t iter[65] = {};  // the steps of a solve, by batch width
};

}  // namespace

struct tdda_core_s {
    int device = 0;
    cudaStream_t stream = nullptr;
    Geom g{};
    int N = 0, nmat = 0, max_rhs = 1, method = 0, maxblk = 1;
    double d = 0, lam = 0, nback = 1, K = 0;
    std::vector<cd> material;  // normalised
    std::vector<int> R;
    int* cellmap = nullptr;
    int* Rdev = nullptr;  // 3N lattice indices
    double2* green64 = nullptr;
    // FP32 inner solve as a device-side loop (conditional graph node); TDDA_DEVICE_LOOP=0 in the
    // environment makes the host launch each chunk instead (profilers see the kernels of a
    // host-launched graph, not those of a device-side loop's body)
    bool device_loop = true;
    float2* ones32 = nullptr;  // 3N entries of 1 (the sinks' diagonal of a Jacobi-preconditioned solve)
    // batch schedule of the FP32 products: right-hand sides per launch (0: all of a
    // batch in one launch per pass).  Groups run one after another, each through all
    // of its passes, so a group's FFT work grid can stay in L2 between the passes.
    int group = 0;
    dd2* green_dd = nullptr;            // double-float copies for the residual product (on first use)
    dd2* tw_dd[3] = {nullptr, nullptr, nullptr};
    float2* green32 = nullptr;
    double2* tw64[3] = {nullptr, nullptr, nullptr};
    float2* tw32[3] = {nullptr, nullptr, nullptr};
    double2* grid64 = nullptr;
    float2* grid32 = nullptr;
    double2 *vin64 = nullptr, *vout64 = nullptr;
    float2 *vin32 = nullptr, *vout32 = nullptr;
    RhsVecs<double>* rhs64 = nullptr;  // device, max_rhs + 1 entries (last: plain products)
    RhsVecs<float>* rhs32 = nullptr;
    SolveState* st64 = nullptr;        // device, max_rhs
    SolveState* st32 = nullptr;
    SolveState* hst = nullptr;         // pinned host, max_rhs
    SolveState* hst_first = nullptr;   // pinned host, max_rhs: the first residual's states (solve_mixed)
    unsigned int* flag = nullptr;      // device: result of launch_scan
    unsigned int* hflag = nullptr;     // pinned host copy of it
    double* part = nullptr;
    unsigned int* cnt = nullptr;
    Graphs<double> g64;
    Graphs<float> g32;
    std::vector<void*> allocs;
    bool is_periodic = false;
    tdda::PeriodicImages periodic{};
    tdda::Interaction inter{};  // LDR, or FCD with this device's Si/Ci tables
};

struct tdda_model_s {
    tdda_core* core = nullptr;
    double nK[3] = {0, 0, 0}, nE0[3] = {0, 0, 0}, E0 = 1;
    std::vector<double> diel_old;
    // FP64 state: P, E, al, diel, Einternal and the Krylov vectors
    double2 *P = nullptr, *E = nullptr, *al = nullptr, *diel = nullptr, *Ein = nullptr;
    double* dold = nullptr;  // the 3N densities on the device
    double2 *r = nullptr, *r0 = nullptr, *p = nullptr, *u = nullptr, *t = nullptr, *Ap = nullptr, *At = nullptr;
    // FP32 Krylov vectors of the mixed solve (allocated on first use)
    float2 *fP = nullptr, *fE = nullptr, *fal = nullptr, *fr = nullptr, *fr0 = nullptr, *fp = nullptr, *fu = nullptr,
           *ft = nullptr, *fAp = nullptr, *fAt = nullptr;
    // Jacobi right preconditioning of the FP32 inner solve (TDDA_FP32_JACOBI):
    // whether the model's current solve uses it, and 1 / al as FP32 SoA
    bool jacobi = false;
    float2* fpre = nullptr;
    // UpdateAlpha keeps the previous densities on the device (restored when the new
    // ones are refused) and leaves the host copy diel_old stale until it is needed
    double* dold_bak = nullptr;
    bool dold_host_stale = false;
    std::vector<void*> allocs;
    bool P_zero = true;
    int ITERATION = 0;
    double Error = 0.0;
};

namespace {

// Device buffers are stream-ordered allocations from the device's memory pool
// (cudaMallocAsync / cudaFreeAsync on the owner's stream): creating and
// destroying cores and models never synchronises the device, so several can
// be set up and torn down while other solves run (the serving loop).
template <typename T> tdda_status dalloc(std::vector<void*>& list, T** p, size_t count, cudaStream_t stream) {
    void* q = nullptr;
    cudaError_t e = cudaMallocAsync(&q, sizeof(T) * std::max<size_t>(count, 1), stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync");
    list.push_back(q);
    *p = (T*)q;
    return TDDA_OK;
}

#define TDDA_TRY(call)                         \
    do {                                       \
        tdda_status s_ = (call);               \
        if (s_ != TDDA_OK) return s_;          \
    } while (0)

void free_all(std::vector<void*>& list, cudaStream_t stream) {
    for (void* q : list) cudaFreeAsync(q, stream);
    list.clear();
}

// raise the kernels' shared-memory limits once per device
std::mutex g_cfg_mu;
bool g_cfg_ready[64];
tdda_status configure_once(int device) {
    std::lock_guard<std::mutex> lk(g_cfg_mu);
    if (device >= 0 && device < 64 && g_cfg_ready[device]) return TDDA_OK;
    cudaError_t e = tdda::configure_kernels();
    if (e != cudaSuccess) return cuda_fail(e, "configure_kernels");
    if (device >= 0 && device < 64) g_cfg_ready[device] = true;
    return TDDA_OK;
}

// Small pinned host buffers (solve states, flags) come from a process-wide
// free list by size class and go back to it: freeing pinned memory
// synchronises the whole device, so a core destroyed while other streams run
// solves would wait for all of their queued work.
std::mutex g_pin_mu;
std::vector<std::pair<size_t, void*>> g_pin_free;
size_t pin_class(size_t bytes) {
    size_t c = 256;
    while (c < bytes) c *= 2;
    return c;
}
cudaError_t pinned_get(void** p, size_t bytes) {
    const size_t cls = pin_class(bytes);
    {
        std::lock_guard<std::mutex> lk(g_pin_mu);
        for (size_t i = 0; i < g_pin_free.size(); i++) {
            if (g_pin_free[i].first == cls) {
                *p = g_pin_free[i].second;
                g_pin_free.erase(g_pin_free.begin() + (long)i);
                return cudaSuccess;
            }
        }
    }
    return cudaMallocHost(p, cls);
}
void pinned_put(void* p, size_t bytes) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(g_pin_mu);
    g_pin_free.emplace_back(pin_class(bytes), p);
}

// keep freed pool memory cached for reuse instead of returning it to the
// driver at every synchronisation (once per device)
std::mutex g_pool_mu;
bool g_pool_ready[64];
tdda_status ensure_pool(int device) {
    if (device < 0 || device >= 64) return TDDA_OK;
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (g_pool_ready[device]) return TDDA_OK;
    cudaMemPool_t pool;
    cudaError_t e = cudaDeviceGetDefaultMemPool(&pool, device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetDefaultMemPool");
    unsigned long long thr = ~0ull;
    e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMemPoolSetAttribute");
    g_pool_ready[device] = true;
    return TDDA_OK;
}

template <typename T> tdda_status dalloc_c(tdda_core* c, T** p, size_t count) {
    return dalloc(c->allocs, p, count, c->stream);
}

cudaMemcpyKind kind_in(int mem) { return mem == TDDA_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice; }
cudaMemcpyKind kind_out(int mem) { return mem == TDDA_MEM_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost; }

RhsVecs<double> vecs64(tdda_core* c, tdda_model* m, int slot) {
    RhsVecs<double> v{};
    v.P = m->P; v.E = m->E; v.r = m->r; v.r0 = m->r0; v.p = m->p; v.u = m->u; v.t = m->t;
    v.Ap = m->Ap; v.At = m->At; v.al = m->al;
    v.st = c->st64 + slot;
    v.part = c->part + (size_t)slot * tdda::kPartSlots * c->maxblk;
    v.cnt = c->cnt + (size_t)slot * tdda::kCounters;
    return v;
}
RhsVecs<float> vecs32(tdda_core* c, tdda_model* m, int slot) {
    RhsVecs<float> v{};
    v.P = m->fP; v.E = m->fE; v.r = m->fr; v.r0 = m->fr0; v.p = m->fp; v.u = m->fu; v.t = m->ft;
    v.Ap = m->fAp; v.At = m->fAt; v.al = m->fal;
    if (m->jacobi) {  // products A D^-1 v: the gathers scale by 1 / al, the sinks add 1 v
        v.pre = m->fpre;
        v.al = m->core->ones32;
    }
    v.st = c->st32 + slot;
    v.part = c->part + (size_t)slot * tdda::kPartSlots * c->maxblk;
    v.cnt = c->cnt + (size_t)slot * tdda::kCounters;
    return v;
}

// incident field and polarisability of a model (DDAModel.cpp:47-63)

// LDR polarisability constants of one model (tools.cpp:617-630) and the
// normalised material table (AProductCore.cpp:19-24)
tdda::AlphaParams alpha_params(const tdda_model* m) {
    const tdda_core* c = m->core;
    tdda::AlphaParams ap;
    std::memset(&ap, 0, sizeof(ap));
    ap.a1c = 3 * std::pow(c->d, 3) / (4 * kPi);
    ap.d3 = std::pow(c->d, 3);
    ap.Kd2 = std::pow(c->K * c->d, 2);
    ap.rad = (2.0 / 3.0) * std::pow(c->K * c->d, 3);
    ap.S = std::pow(m->nE0[0] * m->nK[0], 2) + std::pow(m->nE0[1] * m->nK[1], 2) + std::pow(m->nE0[2] * m->nK[2], 2);
    ap.nmat = c->nmat;
    for (int k = 0; k < c->nmat; k++) ap.mat[k] = make_double2(c->material[k].real(), c->material[k].imag());
    return ap;
}

tdda_status model_upload_fields(tdda_model* m, bool field_E, bool field_al, const double* diel_old = nullptr) {
    tdda_core* c = m->core;
    const int N = c->N;
    if (field_E) {
        // E_inc = E0 n_E0 exp(i K d n_K . R) on the device (DDAModel.cpp:47-51)
        TDDA_CK1(tdda::launch_model_incident(N, c->Rdev, make_double3(m->nK[0], m->nK[1], m->nK[2]),
                                             make_double3(m->nE0[0], m->nE0[1], m->nE0[2]), m->E0, c->K, c->d, m->E,
                                             c->stream));
        TDDA_CK(cudaStreamSynchronize(c->stream));
    }
    if (field_al) {
        // eps and al on the device (DDAModel.cpp:54-63, tools.cpp:617-630) from
        // the densities the caller checked with densities_in_table
        const tdda::AlphaParams ap = alpha_params(m);
        TDDA_CK(cudaMemcpyAsync(m->dold, diel_old ? diel_old : m->diel_old.data(), sizeof(double) * 3 * (size_t)N,
                                cudaMemcpyHostToDevice, c->stream));
        TDDA_CK1(tdda::launch_model_alpha(3 * N, m->dold, ap, m->diel, m->al, m->fal, c->stream));
        TDDA_CK(cudaStreamSynchronize(c->stream));
    }
    return TDDA_OK;
}

// Every density indexes the material table of the interpolation of
// DDAModel.cpp:54-63: with lf = floor(v) and ln = (lf >= 1 ? lf : lf + 1), both
// lf and ln lie in [0, nmat), which holds exactly when nmat >= 2 and
// 0 <= v < nmat (NaN fails).  Checked in branch-free chunks the compiler
// vectorises; on failure *bad is the first offending entry.
bool densities_in_table(const double* v, size_t n, int nmat, size_t* bad) {
    const double hi = (double)nmat;
    constexpr size_t kChunk = 4096;
    for (size_t i0 = 0; i0 < n; i0 += kChunk) {
        const size_t i1 = std::min(n, i0 + kChunk);
        int ok = nmat >= 2;
        for (size_t i = i0; i < i1; i++) ok &= (v[i] >= 0.0) & (v[i] < hi);
        if (!ok) {
            size_t i = i0;
            while (i < i1 && nmat >= 2 && v[i] >= 0.0 && v[i] < hi) i++;
            *bad = std::min(i, i1 - 1);
            return false;
        }
    }
    return true;
}


tdda_status model_alloc_f32(tdda_model* m) {
    if (m->fP) return TDDA_OK;
    const size_t n3 = 3 * (size_t)m->core->N;
    float2** v[] = {&m->fP, &m->fE, &m->fal, &m->fr, &m->fr0, &m->fp, &m->fu, &m->ft, &m->fAp, &m->fAt};
    for (float2** q : v) TDDA_TRY(dalloc(m->allocs, q, n3, m->core->stream));
    TDDA_CK1(tdda::launch_to_f32((int)n3, m->al, m->fal, m->core->stream));
    return TDDA_OK;
}

// The state of a Jacobi-preconditioned FP32 solve of model m: 1 / al of its
// current polarisabilities (from the FP32 al, which model_alloc_f32 and every
// UpdateAlpha keep current) and its core's vector of ones (on the model's core
// stream, before the solve's first product).
tdda_status prepare_jacobi(tdda_model* m) {
    tdda_core* c = m->core;
    const size_t n3 = 3 * (size_t)c->N;
    if (!m->fpre) TDDA_TRY(dalloc(m->allocs, &m->fpre, n3, c->stream));
    if (!c->ones32) {
        TDDA_TRY(dalloc_c(c, &c->ones32, n3));
        TDDA_CK1(tdda::launch_fill_ones(n3, c->ones32, c->stream));
    }
    TDDA_CK1(tdda::launch_recip_f32((int)n3, m->fal, m->fpre, c->stream));
    return TDDA_OK;
}

// TDDA_FP32_AUTO: precondition when |al| varies by more than kJacobiSpread
// over the model's dipoles (the preconditioner pays its extra load where al is
// nearly constant, and cuts the steps 5-10x where low- and high-density dipoles
// mix).  Reads the FP32 al, so after model_alloc_f32.
constexpr float kJacobiSpread = 4.f;
tdda_status wants_jacobi(tdda_model* m, bool* out) {
    tdda_core* c = m->core;
    TDDA_CK1(tdda::launch_al_range(3 * c->N, m->fal, c->flag + 1, c->stream));
    TDDA_CK(cudaMemcpyAsync(c->hflag + 1, c->flag + 1, 2 * sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream));
    TDDA_CK(cudaStreamSynchronize(c->stream));
    float hi, lo;
    std::memcpy(&hi, &c->hflag[1], sizeof(float));
    std::memcpy(&lo, &c->hflag[2], sizeof(float));
    *out = hi > kJacobiSpread * kJacobiSpread * lo;
    return TDDA_OK;
}

// the preconditioning of a model's FP32 inner solves: mode 0 none, 1 Jacobi,
// 2 chosen by wants_jacobi (TDDA_FP32_REFINE, _JACOBI, _AUTO)
tdda_status set_preconditioner(tdda_model* m, int mode) {
    bool j = mode == 1;
    if (mode == 2) TDDA_TRY(wants_jacobi(m, &j));
    m->jacobi = j;
    if (j) TDDA_TRY(prepare_jacobi(m));
    return TDDA_OK;
}
int precond_mode(int precision) {
    return precision == TDDA_FP32_JACOBI ? 1 : precision == TDDA_FP32_AUTO ? 2 : 0;
}

// P (FP64) += the inner solve's correction: d, or D^-1 d for a Jacobi-preconditioned solve
tdda_status accumulate_correction(tdda_model* m, cudaStream_t stream) {
    const int n3 = 3 * m->core->N;
    if (m->jacobi) TDDA_CK1(tdda::launch_accumulate_scaled(n3, m->fP, m->fpre, m->P, stream));
    else TDDA_CK1(tdda::launch_accumulate(n3, m->fP, m->P, stream));
    return TDDA_OK;
}

template <typename T> struct Prec;
template <> struct Prec<double> {
    static RhsVecs<double>* rhs(tdda_core* c) { return c->rhs64; }
    static SolveState* st(tdda_core* c) { return c->st64; }
    static const double2* green(tdda_core* c) { return c->green64; }
    static double2* grid(tdda_core* c) { return c->grid64; }
    static const double2* tw(tdda_core* c, int a) { return c->tw64[a]; }
    static cudaGraphExec_t& graph(tdda_core* c, int n) { return c->g64.iter[n]; }
};
template <> struct Prec<float> {
    static RhsVecs<float>* rhs(tdda_core* c) { return c->rhs32; }
    static SolveState* st(tdda_core* c) { return c->st32; }
    static const float2* green(tdda_core* c) { return c->green32; }
    static float2* grid(tdda_core* c) { return c->grid32; }
    static const float2* tw(tdda_core* c, int a) { return c->tw32[a]; }
    static cudaGraphExec_t& graph(tdda_core* c, int n) { return c->g32.iter[n]; }
};

// kernels of one A-product at precision T: 3 with the fused z+y passes, else 5
template <typename T> int product_kernels(const tdda_core* c) { return tdda::zy_fused(c->g, sizeof(T) == 4) ? 3 : 5; }

// right-hand sides per launch of a batch of n: the core's FP32 batch schedule
template <typename T> int group_size(const tdda_core* c, int n) {
    return (sizeof(T) == 4 && c->group > 0 && c->group < n) ? c->group : n;
}
template <typename T> int group_count(const tdda_core* c, int n) {
    const int gs = group_size<T>(c, n);
    return (n + gs - 1) / gs;
}

// One A-product of n right-hand sides: one launch per pass, or, with an FP32
// batch schedule of groups, each group through all of its passes in turn (the
// group's right-hand sides use the first slices of the work grid).  ev (the
// six pass events) is recorded for an ungrouped product only.
template <typename T>
cudaError_t aprod(tdda_core* c, int src, int snk, int n, const RhsVecs<T>* rhs, cudaEvent_t* ev = nullptr,
                  int slot = 0) {
    const int gs = group_size<T>(c, n);
    for (int g0 = 0; g0 < n; g0 += gs) {
        count_launches(product_kernels<T>(c));
        const cudaError_t e = tdda::launch_aproduct<T>(
            c->g, src, snk, std::min(gs, n - g0), rhs + g0, Prec<T>::green(c), Prec<T>::tw(c, 0), Prec<T>::tw(c, 1),
            Prec<T>::tw(c, 2), c->cellmap, Prec<T>::grid(c), c->stream, gs == n ? ev : nullptr, slot);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

// One BiCGSTAB step.  FP64 (the drop-in): the reference's recurrence with its
// three reductions, the update of P and r in k_update.  FP32 (the inner solve
// of the mixed form): the update is deferred into the next step's gather and
// r0.r, |r|^2 follow from sums taken with At (SNK_AT_DEF), so a step is two
// products and no separate update kernel.  The FP32 sink passes only publish
// block partials; the next gather forms alpha, or the end of the previous step
// (zeta, r0.r, convergence, beta), in every block, and its block 0 records
// them in the state slots of the step's parity `slot`.
template <typename T> constexpr bool kDeferred = sizeof(T) == 4;

template <typename T> int step_kernels(const tdda_core* c, int n) {
    return 2 * product_kernels<T>(c) * group_count<T>(c, n) + (kDeferred<T> ? 0 : 1);
}

template <typename T> cudaError_t enqueue_iteration(tdda_core* c, int n, int slot) {
    const RhsVecs<T>* rhs = Prec<T>::rhs(c);
    cudaError_t e;
    if constexpr (kDeferred<T>) {
        // update, p, Ap
        if ((e = aprod<T>(c, tdda::SRC_PUPD_DEF, tdda::SNK_AP, n, rhs, nullptr, slot))) return e;
        return aprod<T>(c, tdda::SRC_TUPD, tdda::SNK_AT_DEF, n, rhs, nullptr, slot);  // alpha, t, At
    } else {
        if ((e = aprod<T>(c, tdda::SRC_PUPD, tdda::SNK_AP, n, rhs))) return e;  // p, Ap, alpha
        if ((e = aprod<T>(c, tdda::SRC_TUPD, tdda::SNK_AT, n, rhs))) return e;  // t, At, zeta
        count_launches(1);
        return tdda::launch_update<T>(c->g, n, rhs, 0, c->stream);  // u, P, r, rho, beta
    }
}

// kChunk steps (parities 0, 1, 0, 1 ...); FP32 ends the chunk with the step
// end for the next step (parity 0) and the condition of the device-side loop
template <typename T>
cudaError_t enqueue_chunk(tdda_core* c, int n, cudaGraphConditionalHandle loop, bool in_loop) {
    for (int k = 0; k < kChunk; k++) {
        cudaError_t e = enqueue_iteration<T>(c, n, k & 1);
        if (e != cudaSuccess) return e;
    }
    if constexpr (kDeferred<T>) return tdda::launch_chunk_end(c->g, n, Prec<T>::rhs(c), 0, loop, in_loop, c->stream);
    return cudaSuccess;
}
template <typename T> int chunk_kernels(const tdda_core* c, int n) {
    return kChunk * step_kernels<T>(c, n) + (kDeferred<T> ? 1 : 0);
}

// The graph of the steps.  FP64: one chunk, launched by the host until the
// states it reads stop.  FP32: a conditional WHILE node whose body is one
// chunk; k_chunk_end sets its condition, so the inner solve runs to its end
// without a host round trip (at most chunk_limit chunks).
template <typename T> tdda_status get_iteration_graph(tdda_core* c, int n, cudaGraphExec_t* out) {
    cudaGraphExec_t& ex = Prec<T>::graph(c, n);
    if (!ex) {
        cudaGraph_t gr = nullptr;
        cudaError_t e = cudaSuccess, e2 = cudaSuccess;
        if (kDeferred<T> && c->device_loop) {
            TDDA_CK(cudaGraphCreate(&gr, 0));
            cudaGraphConditionalHandle loop = 0;
            e = cudaGraphConditionalHandleCreate(&loop, gr, 1, cudaGraphCondAssignDefault);
            cudaGraphNodeParams cp{};
            cp.type = cudaGraphNodeTypeConditional;
            cp.conditional.handle = loop;
            cp.conditional.type = cudaGraphCondTypeWhile;
            cp.conditional.size = 1;
            cudaGraphNode_t node = nullptr;
            if (e == cudaSuccess) e = cudaGraphAddNode(&node, gr, nullptr, nullptr, 0, &cp);
            if (e != cudaSuccess) {
                cudaGraphDestroy(gr);
                return cuda_fail(e, "conditional node of the inner solve");
            }
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            TDDA_CK(cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
            t_capturing = true;
            e = enqueue_chunk<T>(c, n, loop, true);
            t_capturing = false;
            cudaGraph_t captured = nullptr;
            e2 = cudaStreamEndCapture(c->stream, &captured);
        } else {
            TDDA_CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            t_capturing = true;
            e = enqueue_chunk<T>(c, n, 0, false);
            t_capturing = false;
            e2 = cudaStreamEndCapture(c->stream, &gr);
        }
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (gr) cudaGraphDestroy(gr);
            return cuda_fail(e != cudaSuccess ? e : e2, "capture of the BiCGSTAB steps");
        }
        e = cudaGraphInstantiate(&ex, gr, 0);
        cudaGraphDestroy(gr);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
    }
    *out = ex;
    return TDDA_OK;
}

// The FP64 residual r = E - (A P + al P) of the refinement: the double-float
// product (about 44 bits, on the FP32 pipes) where its passes are compiled,
// else the FP64 passes.  The double-float spectrum and twiddles are split from
// the FP64 ones on first use.
tdda_status residual_product(tdda_core* c, int n) {
    if (tdda::dd_lengths(c->g)) {
        if (!c->green_dd) {
            const long long H6 = 6LL * c->g.Hx * c->g.Hy * c->g.Hz;
            const int M[3] = {c->g.px.M, c->g.py.M, c->g.pz.M};
            TDDA_TRY(dalloc_c(c, &c->green_dd, (size_t)H6));
            for (int a = 0; a < 3; a++) TDDA_TRY(dalloc_c(c, &c->tw_dd[a], (size_t)M[a]));
            TDDA_CK1(tdda::launch_to_dd(H6, c->green64, c->green_dd, c->stream));
            for (int a = 0; a < 3; a++) TDDA_CK1(tdda::launch_to_dd(M[a], c->tw64[a], c->tw_dd[a], c->stream));
        }
        count_launches(5);
        TDDA_CK1(tdda::launch_residual_dd(c->g, n, reinterpret_cast<const RhsVecs<dd>*>(c->rhs64), c->green_dd,
                                          c->tw_dd[0], c->tw_dd[1], c->tw_dd[2], c->cellmap,
                                          reinterpret_cast<dd2*>(c->grid64), c->stream));
        return TDDA_OK;
    }
    TDDA_CK(aprod<double>(c, tdda::SRC_P, tdda::SNK_RES, n, c->rhs64));
    return TDDA_OK;
}

// BiCGSTAB on n right-hand sides whose RhsVecs<T> and states are uploaded.
// DDAModel.cpp:164-255.  p_zero: every P is zero, so r = E without a product.
template <typename T> tdda_status krylov(tdda_core* c, int n, bool p_zero, int max_it) {
    const RhsVecs<T>* rhs = Prec<T>::rhs(c);
    if (p_zero) {
        TDDA_CK1(tdda::launch_residual_is_rhs<T>(c->g, n, rhs, c->stream));
    } else {
        TDDA_CK1(tdda::launch_solve_begin<T>(c->g, n, rhs, c->stream));
        TDDA_CK(aprod<T>(c, tdda::SRC_P, tdda::SNK_RES, n, rhs));  // r = r0 = p = E - A P
    }
    if (kDeferred<T>) {  // the initial products are step -1 (parity 1)
        TDDA_CK(aprod<T>(c, tdda::SRC_IN, tdda::SNK_AP, n, rhs, nullptr, 1));     // Ap0
        TDDA_CK(aprod<T>(c, tdda::SRC_TUPD, tdda::SNK_AT_DEF, n, rhs, nullptr, 1));  // alpha, t, At0
    } else {
        TDDA_CK(aprod<T>(c, tdda::SRC_IN, tdda::SNK_AP, n, rhs));  // Ap0, alpha
        TDDA_CK(aprod<T>(c, tdda::SRC_TUPD, tdda::SNK_AT, n, rhs));  // t, At0, zeta
        TDDA_CK1(tdda::launch_update<T>(c->g, n, rhs, 1, c->stream));
    }
    cudaGraphExec_t ex;
    TDDA_TRY(get_iteration_graph<T>(c, n, &ex));
    if constexpr (kDeferred<T>) {  // device-side loop, up to kLoopChunks chunks per launch (else one)
        for (;;) {
            TDDA_CK(cudaGraphLaunch(ex, c->stream));
            TDDA_CK(cudaMemcpyAsync(c->hst, Prec<T>::st(c), sizeof(SolveState) * n, cudaMemcpyDeviceToHost,
                                    c->stream));
            TDDA_CK(cudaStreamSynchronize(c->stream));
            bool running = false;
            for (int i = 0; i < n; i++) running |= c->hst[i].status == tdda::ST_RUNNING;
            if (!running || c->hst[0].chunks >= c->hst[0].chunk_limit) break;
        }
        count_launches(c->hst[0].chunks * chunk_kernels<T>(c, n));
        TDDA_CK1(tdda::launch_finish<T>(c->g, n, rhs, c->stream));  // the last step's update
        return TDDA_OK;
    }
    int done_it = 0;
    for (;;) {
        TDDA_CK(cudaMemcpyAsync(c->hst, Prec<T>::st(c), sizeof(SolveState) * n, cudaMemcpyDeviceToHost, c->stream));
        TDDA_CK(cudaStreamSynchronize(c->stream));
        bool running = false;
        for (int i = 0; i < n; i++) running |= c->hst[i].status == tdda::ST_RUNNING;
        if (!running || done_it > max_it) break;
        count_launches(chunk_kernels<T>(c, n));
        TDDA_CK(cudaGraphLaunch(ex, c->stream));
        done_it += kChunk;
    }
    return TDDA_OK;
}

tdda_status status_of(const SolveState& s) {
    switch (s.status) {
        case tdda::ST_CONVERGED: return TDDA_OK;
        case tdda::ST_BREAKDOWN: return TDDA_BREAKDOWN;
        case tdda::ST_MAXITER: return TDDA_NOT_CONVERGED;
        case tdda::ST_NAN: return TDDA_ERR_NAN;
        default: return TDDA_ERR_CUDA;
    }
}

SolveState fresh_state(double tol, int max_it, int iterations) {
    SolveState s;
    std::memset(&s, 0, sizeof(s));
    s.tol = tol;
    s.max_it = max_it;
    s.iterations = iterations;
    s.status = tdda::ST_RUNNING;
    s.init = 1;
    s.tol32 = (float)tol;
    s.init32[1] = 1;  // the FP32 initial products are step -1 (slot 1)
    s.last_slot = -1;
    s.chunks = 0;
    s.chunk_limit = max_it / kChunk + 2;  // max_it steps and the chunk that detects the stop
    return s;
}

tdda_status check_batch(tdda_model* const* ms, int n) {
    if (!ms || n < 1) {
        set_err("empty batch");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    tdda_core* c = ms[0] ? ms[0]->core : nullptr;
    if (!c) {
        set_err("null model");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    if (n > c->max_rhs) {
        set_err("batch of %d exceeds the core's max_rhs %d", n, c->max_rhs);
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    for (int i = 0; i < n; i++) {
        if (!ms[i] || ms[i]->core != c) {
            set_err("models of a batch must share one core");
            return TDDA_ERR_INVALID_ARGUMENT;
        }
        for (int j = 0; j < i; j++)
            if (ms[j] == ms[i]) {
                set_err("a model appears twice in a batch");
                return TDDA_ERR_INVALID_ARGUMENT;
            }
    }
    return TDDA_OK;
}

tdda_status solve_fp64(tdda_model* const* ms, int n, int max_it, double tol, tdda_solve_info* infos) {
    tdda_core* c = ms[0]->core;
    std::vector<RhsVecs<double>> hv(n);
    bool p_zero = true;
    for (int i = 0; i < n; i++) {
        hv[i] = vecs64(c, ms[i], i);
        c->hst[i] = fresh_state(tol, max_it, ms[i]->ITERATION);
        p_zero &= ms[i]->P_zero;
    }
    TDDA_CK(cudaMemcpyAsync(c->rhs64, hv.data(), sizeof(RhsVecs<double>) * n, cudaMemcpyHostToDevice, c->stream));
    TDDA_CK(cudaMemcpyAsync(c->st64, c->hst, sizeof(SolveState) * n, cudaMemcpyHostToDevice, c->stream));
    if (max_it <= 0) {
        // the reference still runs its three initial products and the update
        TDDA_TRY(krylov<double>(c, n, p_zero, 0));
    } else {
        TDDA_TRY(krylov<double>(c, n, p_zero, max_it));
    }
    tdda_status worst = TDDA_OK;
    for (int i = 0; i < n; i++) {
        const SolveState& s = c->hst[i];
        tdda_model* m = ms[i];
        m->P_zero = false;
        tdda_status st = status_of(s);
        if (s.status == tdda::ST_CONVERGED || s.status == tdda::ST_BREAKDOWN) {
            m->ITERATION = s.iterations;
            m->Error = s.error;
        }
        if (infos) {
            infos[i].status = st;
            infos[i].iterations = m->ITERATION;
            infos[i].error = s.error;
            infos[i].true_residual = -1.0;
            infos[i].outer_iterations = 0;
            infos[i].inner_iterations = s.it;
        }
        if (st != TDDA_OK && worst == TDDA_OK) worst = st;
    }
    return worst;
}

// Mixed precision: FP32 BiCGSTAB on the FP64 residual, FP64 accumulation of
// the correction, FP64 residual check, until |E - A P| / |E| <= tol.
tdda_status solve_mixed(tdda_model* const* ms, int n, int max_it, double tol, tdda_solve_info* infos,
                        int precond = 0) {
    tdda_core* c = ms[0]->core;
    for (int i = 0; i < n; i++) {
        TDDA_TRY(model_alloc_f32(ms[i]));
        TDDA_TRY(set_preconditioner(ms[i], precond));
    }
    std::vector<RhsVecs<double>> h64(n);
    std::vector<RhsVecs<float>> h32(n);
    std::vector<int> done(n, 0), inner(n, 0), outer(n, 0);
    std::vector<double> Enorm(n, 0.0), res(n, 1.0), prev_res(n, 1e300);
    std::vector<tdda_status> stat(n, TDDA_NOT_CONVERGED);
    bool all_p_zero = true;
    for (int i = 0; i < n; i++) {
        h64[i] = vecs64(c, ms[i], i);
        h32[i] = vecs32(c, ms[i], i);
        all_p_zero &= ms[i]->P_zero;
    }
    TDDA_CK(cudaMemcpyAsync(c->rhs64, h64.data(), sizeof(RhsVecs<double>) * n, cudaMemcpyHostToDevice, c->stream));
    TDDA_CK(cudaMemcpyAsync(c->rhs32, h32.data(), sizeof(RhsVecs<float>) * n, cudaMemcpyHostToDevice, c->stream));
    // With every P zero the first residual is E itself, |r| / |E| = 1 exactly for a finite,
    // nonzero E, so the first inner solve starts without the host reading that residual back
    // (one host round trip less).  The first residual's states land in hst_first and are
    // checked with the inner solve's: a right-hand side whose E is zero or not finite ends
    // as the check would have ended it, and its inner result is dropped.
    const bool ahead = all_p_zero && max_it > 0 && tol < 1.0;
    if (ahead && !c->hst_first) TDDA_CK(pinned_get((void**)&c->hst_first, sizeof(SolveState) * c->max_rhs));
    for (int outer_it = 0; outer_it <= kMaxOuter; outer_it++) {
        const bool first_ahead = ahead && outer_it == 0;
        SolveState* hs = first_ahead ? c->hst_first : c->hst;
        // FP64 residual r = E - (A P + al P) of the right-hand sides still open
        for (int i = 0; i < n; i++) {
            hs[i] = fresh_state(tol, 0, 0);
            if (done[i]) hs[i].status = tdda::ST_CONVERGED;
        }
        TDDA_CK(cudaMemcpyAsync(c->st64, hs, sizeof(SolveState) * n, cudaMemcpyHostToDevice, c->stream));
        if (outer_it == 0 && all_p_zero) {
            // P = 0: the residual is E exactly (A 0 = 0), no product needed
            TDDA_CK1(tdda::launch_residual_is_rhs<double>(c->g, n, c->rhs64, c->stream));
        } else {
            TDDA_CK1(tdda::launch_solve_begin<double>(c->g, n, c->rhs64, c->stream));
            TDDA_TRY(residual_product(c, n));
        }
        TDDA_CK(cudaMemcpyAsync(hs, c->st64, sizeof(SolveState) * n, cudaMemcpyDeviceToHost, c->stream));
        bool open = false;
        if (first_ahead) {
            for (int i = 0; i < n; i++) res[i] = prev_res[i] = 1.0;
            open = true;
        } else {
            TDDA_CK(cudaStreamSynchronize(c->stream));
        }
        for (int i = 0; i < n && !first_ahead; i++) {
            if (done[i]) continue;
            const SolveState& s = c->hst[i];
            if (s.status == tdda::ST_NAN) {
                done[i] = 1;
                stat[i] = TDDA_ERR_NAN;
                continue;
            }
            Enorm[i] = s.Enorm;
            // a NaN in E makes |E| NaN, which the zero-E test below would take for 0
            res[i] = !std::isfinite(Enorm[i]) ? Enorm[i] : (Enorm[i] > 0 ? std::sqrt(s.rnorm2) / Enorm[i] : 0.0);
            if (!std::isfinite(res[i])) {
                done[i] = 1;
                stat[i] = TDDA_ERR_NAN;
            } else if (res[i] <= tol) {
                done[i] = 1;
                stat[i] = TDDA_OK;
            } else if (outer_it == kMaxOuter || inner[i] >= max_it || res[i] >= prev_res[i]) {
                done[i] = 1;
                stat[i] = TDDA_NOT_CONVERGED;
            } else {
                open = true;
            }
            prev_res[i] = res[i];
        }
        if (!open) break;
        // FP32 correction: A d = r, d0 = 0, to a relative tolerance that brings
        // the true residual under tol with margin (0.9 tol: the FP32 recurrence
        // residual tracks the true one to ~1e-8 of |E| at these tolerances; the
        // outer check catches the rest)
        for (int i = 0; i < n; i++) {
            tdda_model* m = ms[i];
            double tin = std::min(0.5, std::max(2e-6, 0.9 * tol / std::max(res[i], 1e-300)));
            c->hst[i] = fresh_state(tin, max_it - inner[i], 0);
            if (done[i]) {
                c->hst[i].status = tdda::ST_CONVERGED;
                continue;
            }
            TDDA_CK1(tdda::launch_to_f32(3 * c->N, m->r, m->fE, c->stream));
            TDDA_CK1(tdda::launch_zero<float>(3LL * c->N, m->fP, c->stream));
        }
        // the device-side loop reads its limit from the first state: the largest of the batch
        for (int i = 1; i < n; i++) c->hst[0].chunk_limit = std::max(c->hst[0].chunk_limit, c->hst[i].chunk_limit);
        TDDA_CK(cudaMemcpyAsync(c->st32, c->hst, sizeof(SolveState) * n, cudaMemcpyHostToDevice, c->stream));
        TDDA_TRY(krylov<float>(c, n, true, max_it));  // ends with the stream synchronised
        for (int i = 0; i < n && first_ahead; i++) {
            // the first residual's check, as above for r = E
            const SolveState& s = c->hst_first[i];
            Enorm[i] = s.Enorm;
            if (s.status == tdda::ST_NAN) {
                done[i] = 1;
                stat[i] = TDDA_ERR_NAN;
            } else if (!std::isfinite(s.Enorm)) {
                done[i] = 1;
                stat[i] = TDDA_ERR_NAN;
                res[i] = s.Enorm;
            } else if (!(s.Enorm > 0)) {
                done[i] = 1;
                stat[i] = TDDA_OK;
                res[i] = 0.0;
            }
        }
        for (int i = 0; i < n; i++) {
            if (done[i]) continue;
            const SolveState& s = c->hst[i];
            inner[i] += s.it;
            outer[i] += 1;
            if (s.status == tdda::ST_NAN) {
                done[i] = 1;
                stat[i] = TDDA_ERR_NAN;
                continue;
            }
            TDDA_TRY(accumulate_correction(ms[i], c->stream));
        }
    }
    TDDA_CK(cudaStreamSynchronize(c->stream));
    tdda_status worst = TDDA_OK;
    for (int i = 0; i < n; i++) {
        tdda_model* m = ms[i];
        m->P_zero = false;
        if (stat[i] == TDDA_OK) {
            m->ITERATION = inner[i];
            m->Error = res[i];
        }
        if (infos) {
            infos[i].status = stat[i];
            infos[i].iterations = inner[i];
            infos[i].error = res[i];
            infos[i].true_residual = res[i];
            infos[i].outer_iterations = outer[i];
            infos[i].inner_iterations = inner[i];
        }
        if (stat[i] != TDDA_OK && worst == TDDA_OK) worst = stat[i];
    }
    return worst;
}

tdda_status set_device(int dev) {
    cudaError_t e = cudaSetDevice(dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    return TDDA_OK;
}

// ------------------------------------------------- allocation-free A-product
// Some callers cannot call cudaMalloc while they run the product: code that
// runs under an external memory budget with every byte pre-reserved, or a host
// framework that forbids device allocation once its own setup is done.  For
// them tdda_aproduct_noalloc keeps the FFT work grid of the product in this
// fixed, file-scope device array instead of the core's buffers.  Every GPU that
// loads the library holds it (64 MiB) until the process exits.
constexpr size_t kNoAllocGridElems = 4u << 20;  // complex128 entries: 64 MiB
static __device__ __align__(256) double2 g_noalloc_grid[kNoAllocGridElems];
static __device__ __align__(256) RhsVecs<double> g_noalloc_rhs;

struct NoAllocSlot {
    bool ready = false;
    double2* grid = nullptr;
    RhsVecs<double>* rhs = nullptr;
};
constexpr int kNoAllocDevices = 64;
NoAllocSlot g_noalloc_slots[kNoAllocDevices];
std::mutex g_noalloc_mu;

// Device addresses of the two arrays, looked up once per device with that
// device current.  In host code the arrays' names are host-side stand-ins, not
// device addresses, so only these looked-up pointers reach a kernel.
tdda_status noalloc_setup(int device, NoAllocSlot* out) {
    if (device < 0 || device >= kNoAllocDevices) {
        set_err("device %d out of range for the allocation-free product", device);
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    NoAllocSlot& slot = g_noalloc_slots[device];
    if (!slot.ready) {
        void* g = nullptr;
        void* r = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&g, g_noalloc_grid);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_grid)");
        e = cudaGetSymbolAddress(&r, g_noalloc_rhs);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_rhs)");
        slot.grid = (double2*)g;
        slot.rhs = (RhsVecs<double>*)r;
        slot.ready = true;
    }
    *out = slot;
    return TDDA_OK;
}

}  // namespace


// ============================================================ cross-lattice sessions
// The FP32+refine solve of solve_mixed, one right-hand side per slot, on a
// "shape" core: a core of one FFT grid shape with no lattice of its own
// (Geom::multi), whose pass kernels read each slot's lattice, cellmap and Green
// spectrum from its RhsVecs.  Each slot follows solve_mixed's sequence for its
// model alone: the refinement residual on the model's own core, the inner
// solve's start with that core's vector-length reductions, the steps of the
// shape's batched launches, the end (k_finish) and the accumulation of the
// correction; so its result is bit-identical to tdda_model_solve_mixed.
namespace tdda_session {
namespace {

enum Phase : int { kFree = 0, kResidual = 1, kInner = 2 };

struct Slot {
    tdda_model* m = nullptr;
    int phase = kFree;
    int inner = 0, outer = 0, nres = 0, max_it = 0;
    double tol = 0, res = 1.0, prev_res = 1e300;
};

}  // namespace

struct Shape {
    tdda_core* c = nullptr;   // the shape core (g.multi = 1, no lattice)
    int cap = 0;
    std::vector<Slot> slots;
    std::vector<RhsVecs<float>> h32;  // the full-width slot array, host copy
    RhsVecs<float>* rhs32c = nullptr;  // device: a subset of slots for one launch
    bool dirty = true;                 // h32 differs from the device copy
};

void core_grid(const tdda_core* c, int grid[3]) {
    grid[0] = c->g.px.M;
    grid[1] = c->g.py.M;
    grid[2] = c->g.pz.M;
}
int core_device(const tdda_core* c) { return c->device; }
void grid_of_box(int Nx, int Ny, int Nz, int grid[3]) {
    grid[0] = fft_length(Nx, false);
    grid[1] = fft_length(Ny, false);
    grid[2] = fft_length(Nz, true);
}

namespace {
// The largest lattice a grid shape holds on each axis: M >= 2N - 1
int cap_of(int M) { return (M + 1) / 2; }

// Geometry of a shape core: the plans of its lengths, strides for the largest
// lattice, and the cross-lattice flag
bool shape_geom(const int grid[3], Geom* g) {
    std::memset(g, 0, sizeof(*g));
    AxisPlan* plans[3] = {&g->px, &g->py, &g->pz};
    for (int a = 0; a < 3; a++)
        if (grid[a] < 1 || !make_plan(grid[a], plans[a])) return false;
    g->Nx = cap_of(grid[0]);
    g->Ny = cap_of(grid[1]);
    g->Nz = cap_of(grid[2]);
    g->N = g->Nx * g->Ny * g->Nz;
    g->Hx = g->px.M / 2 + 1;
    g->Hy = g->py.M / 2 + 1;
    g->Hz = g->pz.M / 2 + 1;
    g->sy = g->pz.M;
    g->sx = (long long)g->py.M * g->pz.M;
    g->sc = (long long)g->Nx * g->sx;
    g->sb = 3 * g->sc;
    g->dense = 0;
    g->multi = 1;
    return true;
}

// the slot's entry of the shape's RhsVecs array: the model's FP32 vectors with
// its own lattice, or an empty lattice (every pass block of a free slot returns)
RhsVecs<float> slot_vecs(Shape* s, int k) {
    RhsVecs<float> v{};
    tdda_core* c = s->c;
    v.st = c->st32 + k;
    v.part = c->part + (size_t)k * tdda::kPartSlots * c->maxblk;
    v.cnt = c->cnt + (size_t)k * tdda::kCounters;
    const tdda_model* m = s->slots[k].m;
    if (!m) return v;
    const tdda_core* oc = m->core;
    v = vecs32(c, const_cast<tdda_model*>(m), k);
    v.cellmap = oc->cellmap;
    v.green = oc->green32;
    v.Nx = oc->g.Nx;
    v.Ny = oc->g.Ny;
    v.Nz = oc->g.Nz;
    v.N = oc->g.N;
    v.dense = oc->g.dense;
    return v;
}

// the refinement residual r = E - (A P + al P) of the model on its own core
// (solve_mixed's outer step for one right-hand side); the state read back
tdda_status own_residual(tdda_model* m, SolveState* out) {
    tdda_core* oc = m->core;
    RhsVecs<double> v = vecs64(oc, m, 0);
    oc->hst[0] = fresh_state(0.0, 0, 0);
    TDDA_CK(cudaMemcpyAsync(oc->rhs64, &v, sizeof(v), cudaMemcpyHostToDevice, oc->stream));
    TDDA_CK(cudaMemcpyAsync(oc->st64, oc->hst, sizeof(SolveState), cudaMemcpyHostToDevice, oc->stream));
    if (m->P_zero) {
        // P = 0: the residual is E exactly (A 0 = 0), no product needed
        TDDA_CK1(tdda::launch_residual_is_rhs<double>(oc->g, 1, oc->rhs64, oc->stream));
    } else {
        TDDA_CK1(tdda::launch_solve_begin<double>(oc->g, 1, oc->rhs64, oc->stream));
        TDDA_TRY(residual_product(oc, 1));
    }
    TDDA_CK(cudaMemcpyAsync(oc->hst, oc->st64, sizeof(SolveState), cudaMemcpyDeviceToHost, oc->stream));
    TDDA_CK(cudaStreamSynchronize(oc->stream));
    *out = oc->hst[0];
    return TDDA_OK;
}

void finish_slot(Shape* s, int k, tdda_status st, std::vector<Done>* done) {
    Slot& sl = s->slots[k];
    tdda_model* m = sl.m;
    m->P_zero = false;
    if (st == TDDA_OK) {
        m->ITERATION = sl.inner;
        m->Error = sl.res;
    }
    Done d;
    d.slot = k;
    d.model = m;
    d.info.status = st;
    d.info.iterations = sl.inner;
    d.info.error = sl.res;
    d.info.true_residual = sl.res;
    d.info.outer_iterations = sl.outer;
    d.info.inner_iterations = sl.inner;
    done->push_back(d);
    sl = Slot{};
    s->h32[k] = slot_vecs(s, k);
    s->dirty = true;
}

tdda_status upload_subset(Shape* s, const std::vector<int>& ks) {
    std::vector<RhsVecs<float>> v(ks.size());
    for (size_t i = 0; i < ks.size(); i++) v[i] = s->h32[ks[i]];
    TDDA_CK(cudaMemcpyAsync(s->rhs32c, v.data(), sizeof(RhsVecs<float>) * v.size(), cudaMemcpyHostToDevice,
                            s->c->stream));
    return TDDA_OK;
}
}  // namespace

double core_bytes(int Nx, int Ny, int Nz, int N, int max_rhs) {
    const double Mx = fft_length(Nx, false), My = fft_length(Ny, false), Mz = fft_length(Nz, true);
    const double H = (Mx / 2 + 1) * (My / 2 + 1) * (Mz / 2 + 1);
    const double n3 = 3.0 * N;
    const double grid = 3.0 * Nx * My * Mz * max_rhs;  // FFT work grid entries
    return (double)Nx * Ny * Nz * 4 + n3 * 4           // cellmap, R
           + 6 * H * (16 + 8 + 16)                     // Green spectra (FP64, FP32, double-float)
           + grid * (16 + 8)                           // FP64 and FP32 grids
           + n3 * 2 * (16 + 8)                         // product staging
           + 6 * Mx * My * Mz * 16                     // full Green grid while the core is built
           + 1e6;                                      // reduction partials, states, twiddles
}

double model_bytes(int N, int precision) {
    const double n3 = 3.0 * N;
    double model = n3 * (12 * 16 + 8);  // FP64 vectors and densities
    if (precision == TDDA_FP32_REFINE) model += n3 * 10 * 8;
    if (precision == TDDA_FP32_JACOBI || precision == TDDA_FP32_AUTO) model += n3 * 11 * 8;  // and 1 / al
    return model;
}

double shape_bytes(const int grid[3], int cap) {
    Geom g;
    if (!shape_geom(grid, &g)) return 0.0;
    const double blk = tdda::max_blocks_per_rhs(g);
    return (double)g.sb * cap * 8 + cap * (tdda::kPartSlots * blk * 8 + 2 * sizeof(SolveState) +
                                           2 * sizeof(RhsVecs<float>) + tdda::kCounters * 4) +
           8.0 * (grid[0] + grid[1] + grid[2]) + 1e5;
}

tdda_status shape_create(int device, const int grid[3], int cap, Shape** out) {
    if (!out || !grid || cap < 1 || cap > 64) {
        set_err("invalid shape");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    Geom g;
    if (!shape_geom(grid, &g)) {
        set_err("no radix plan for the FFT grid %dx%dx%d", grid[0], grid[1], grid[2]);
        return TDDA_ERR_UNSUPPORTED;
    }
    if (tdda::max_pass_smem(g) > tdda::kMaxPassSmem) {
        set_err("FFT grid %dx%dx%d needs more shared memory per tile than a block has", grid[0], grid[1], grid[2]);
        return TDDA_ERR_UNSUPPORTED;
    }
    TDDA_TRY(set_device(device));
    TDDA_TRY(ensure_pool(device));
    TDDA_TRY(configure_once(device));
    Shape* s = new Shape();
    tdda_core* c = new tdda_core_s();
    s->c = c;
    s->cap = cap;
    c->device = device;
    c->max_rhs = cap;
    c->g = g;
    c->N = g.N;
    c->maxblk = tdda::max_blocks_per_rhs(g);
    auto fail = [&](tdda_status st) {
        shape_destroy(s);
        return st;
    };
#define TDDA_SHAPE_CK(call)                                \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return fail(cuda_fail(e_, #call)); \
    } while (0)
#define TDDA_SHAPE_TRY(call)                    \
    do {                                        \
        tdda_status s_ = (call);                \
        if (s_ != TDDA_OK) return fail(s_);     \
    } while (0)
    TDDA_SHAPE_CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    {
        const char* v = std::getenv("TDDA_DEVICE_LOOP");
        c->device_loop = !(v && v[0] == '0');
        // early launch of the fused FP32 pass kernels (Geom::early; 0: every kernel the ordinary way)
        const char* el = std::getenv("TDDA_EARLY_LAUNCH");
        c->g.early = el ? std::atoi(el) : 3;
        if (cudaDeviceGetAttribute(&c->g.sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess) c->g.sms = 0;
    }
    for (int a = 0; a < 3; a++) TDDA_SHAPE_TRY(dalloc_c(c, &c->tw32[a], (size_t)grid[a]));
    TDDA_SHAPE_TRY(dalloc_c(c, &c->grid32, (size_t)(g.sb * cap)));
    TDDA_SHAPE_TRY(dalloc_c(c, &c->rhs32, (size_t)cap + 1));
    TDDA_SHAPE_TRY(dalloc_c(c, &s->rhs32c, (size_t)cap));
    TDDA_SHAPE_TRY(dalloc_c(c, &c->st32, (size_t)cap));
    TDDA_SHAPE_TRY(dalloc_c(c, &c->part, (size_t)cap * tdda::kPartSlots * c->maxblk));
    TDDA_SHAPE_TRY(dalloc_c(c, &c->cnt, (size_t)cap * tdda::kCounters));
    TDDA_SHAPE_CK(pinned_get((void**)&c->hst, sizeof(SolveState) * cap));
    TDDA_SHAPE_CK(cudaMemsetAsync(c->cnt, 0, sizeof(unsigned int) * cap * tdda::kCounters, c->stream));
    for (int a = 0; a < 3; a++) {
        std::vector<double2> w64;
        std::vector<float2> w32;
        twiddles(grid[a], w64, w32);
        TDDA_SHAPE_CK(cudaMemcpyAsync(c->tw32[a], w32.data(), sizeof(float2) * w32.size(), cudaMemcpyHostToDevice,
                                      c->stream));
        TDDA_SHAPE_CK(cudaStreamSynchronize(c->stream));
    }
    // every slot starts free: a stopped state, an empty lattice
    s->slots.assign(cap, Slot{});
    s->h32.resize(cap);
    for (int k = 0; k < cap; k++) {
        c->hst[k] = fresh_state(0.0, 0, 0);
        c->hst[k].status = tdda::ST_CONVERGED;
        s->h32[k] = slot_vecs(s, k);
    }
    TDDA_SHAPE_CK(cudaMemcpyAsync(c->st32, c->hst, sizeof(SolveState) * cap, cudaMemcpyHostToDevice, c->stream));
    TDDA_SHAPE_CK(cudaMemcpyAsync(c->rhs32, s->h32.data(), sizeof(RhsVecs<float>) * cap, cudaMemcpyHostToDevice,
                                  c->stream));
    TDDA_SHAPE_CK(cudaStreamSynchronize(c->stream));
    s->dirty = false;
#undef TDDA_SHAPE_CK
#undef TDDA_SHAPE_TRY
    *out = s;
    return TDDA_OK;
}

void shape_destroy(Shape* s) {
    if (!s) return;
    if (s->c) tdda_core_destroy(s->c);
    delete s;
}

bool shape_accepts(const Shape* s, const tdda_model* m) {
    if (!s || !m) return false;
    const tdda_core* oc = m->core;
    return oc->device == s->c->device && oc->g.px.M == s->c->g.px.M && oc->g.py.M == s->c->g.py.M &&
           oc->g.pz.M == s->c->g.pz.M && oc->g.Nx <= s->c->g.Nx && oc->g.Ny <= s->c->g.Ny && oc->g.Nz <= s->c->g.Nz;
}
int shape_cap(const Shape* s) { return s ? s->cap : 0; }
int shape_active(const Shape* s) {
    int n = 0;
    if (s)
        for (const Slot& sl : s->slots) n += sl.phase != kFree;
    return n;
}

tdda_status shape_admit(Shape* s, tdda_model* m, int max_it, double tol, int* slot, int precond) {
    if (!shape_accepts(s, m)) {
        set_err("the model's core does not share the shape's FFT grid");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    int k = 0;
    while (k < s->cap && s->slots[k].phase != kFree) k++;
    if (k == s->cap) {
        set_err("no free slot");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    TDDA_TRY(set_device(s->c->device));
    TDDA_TRY(model_alloc_f32(m));
    TDDA_TRY(set_preconditioner(m, precond));
    TDDA_CK(cudaStreamSynchronize(m->core->stream));
    Slot& sl = s->slots[k];
    sl = Slot{};
    sl.m = m;
    sl.phase = kResidual;
    sl.max_it = max_it;
    sl.tol = tol;
    s->h32[k] = slot_vecs(s, k);
    s->dirty = true;
    if (slot) *slot = k;
    return TDDA_OK;
}

tdda_status shape_step(Shape* s, std::vector<Done>* done) {
    tdda_core* c = s->c;
    TDDA_TRY(set_device(c->device));
    // the shape's previous round (accumulations of the corrections) before the
    // residuals read P on the models' own streams
    TDDA_CK(cudaStreamSynchronize(c->stream));
    // 1. refinement residuals, on each model's own core (solve_mixed's outer step)
    std::vector<int> start;
    for (int k = 0; k < s->cap; k++) {
        Slot& sl = s->slots[k];
        if (sl.phase != kResidual) continue;
        SolveState st;
        TDDA_TRY(own_residual(sl.m, &st));
        const int nres = sl.nres++;
        if (st.status == tdda::ST_NAN) {
            finish_slot(s, k, TDDA_ERR_NAN, done);
            continue;
        }
        const double En = st.Enorm;
        sl.res = !std::isfinite(En) ? En : (En > 0 ? std::sqrt(st.rnorm2) / En : 0.0);
        tdda_status fin = TDDA_OK;
        bool open = false;
        if (!std::isfinite(sl.res)) fin = TDDA_ERR_NAN;
        else if (sl.res <= sl.tol) fin = TDDA_OK;
        else if (nres == kMaxOuter || sl.inner >= sl.max_it || sl.res >= sl.prev_res) fin = TDDA_NOT_CONVERGED;
        else open = true;
        sl.prev_res = sl.res;
        if (!open) {
            finish_slot(s, k, fin, done);
            continue;
        }
        // 2. the inner solve's start: FP32 right-hand side r, correction 0, a fresh state
        tdda_model* m = sl.m;
        const double tin = std::min(0.5, std::max(2e-6, 0.9 * sl.tol / std::max(sl.res, 1e-300)));
        c->hst[k] = fresh_state(tin, sl.max_it - sl.inner, 0);
        TDDA_CK(cudaMemcpyAsync(c->st32 + k, &c->hst[k], sizeof(SolveState), cudaMemcpyHostToDevice, c->stream));
        TDDA_CK1(tdda::launch_to_f32(3 * m->core->N, m->r, m->fE, c->stream));
        TDDA_CK1(tdda::launch_zero<float>(3LL * m->core->N, m->fP, c->stream));
        sl.phase = kInner;
        start.push_back(k);
    }
    if (s->dirty) {
        TDDA_CK(cudaMemcpyAsync(c->rhs32, s->h32.data(), sizeof(RhsVecs<float>) * s->cap, cudaMemcpyHostToDevice,
                                c->stream));
        s->dirty = false;
    }
    if (!start.empty()) {
        // r = r0 = p = E (the FP32 right-hand side), |E| and r0.r, each with its own
        // lattice's vector-length reduction, as its solve alone forms them
        for (int k : start) {
            TDDA_TRY(upload_subset(s, {k}));
            TDDA_CK1(tdda::launch_residual_is_rhs<float>(s->slots[k].m->core->g, 1, s->rhs32c, c->stream));
        }
        // the initial products of the new inner solves (step -1, parity 1), in one launch per pass
        TDDA_TRY(upload_subset(s, start));
        const int n = (int)start.size();
        TDDA_CK(aprod<float>(c, tdda::SRC_IN, tdda::SNK_AP, n, s->rhs32c, nullptr, 1));
        TDDA_CK(aprod<float>(c, tdda::SRC_TUPD, tdda::SNK_AT_DEF, n, s->rhs32c, nullptr, 1));
    }
    // the launch covers the slots up to the last one in an inner solve (slots are
    // taken lowest first, so a lightly loaded shape launches few right-hand sides)
    int width = 0;
    for (int k = 0; k < s->cap; k++)
        if (s->slots[k].phase == kInner) width = k + 1;
    if (width == 0) return TDDA_OK;
    // 3. one launch of the steps of those slots (the device-side loop: at most
    // kLoopChunks chunks of kChunk steps, or one host-launched chunk); the chunk
    // count of the launch restarts in the first slot's state
    const int zero_limit[2] = {0, 1 << 30};
    TDDA_CK(cudaMemcpyAsync(&c->st32[0].chunks, zero_limit, sizeof(zero_limit), cudaMemcpyHostToDevice, c->stream));
    cudaGraphExec_t ex;
    TDDA_TRY(get_iteration_graph<float>(c, width, &ex));
    TDDA_CK(cudaGraphLaunch(ex, c->stream));
    TDDA_CK(cudaMemcpyAsync(c->hst, c->st32, sizeof(SolveState) * width, cudaMemcpyDeviceToHost, c->stream));
    TDDA_CK(cudaStreamSynchronize(c->stream));
    count_launches(std::max(1, c->hst[0].chunks) * chunk_kernels<float>(c, width));
    // 4. inner solves that stopped: the pending update, then P += the correction
    std::vector<int> stopped;
    for (int k = 0; k < width; k++)
        if (s->slots[k].phase == kInner && c->hst[k].status != tdda::ST_RUNNING) stopped.push_back(k);
    if (stopped.empty()) return TDDA_OK;
    TDDA_TRY(upload_subset(s, stopped));
    TDDA_CK1(tdda::launch_finish<float>(c->g, (int)stopped.size(), s->rhs32c, c->stream));
    for (int k : stopped) {
        Slot& sl = s->slots[k];
        const SolveState& st = c->hst[k];
        sl.inner += st.it;
        sl.outer += 1;
        if (st.status == tdda::ST_NAN) {
            finish_slot(s, k, TDDA_ERR_NAN, done);
            continue;
        }
        TDDA_TRY(accumulate_correction(sl.m, c->stream));
        sl.m->P_zero = false;
        sl.phase = kResidual;
    }
    TDDA_CK(cudaStreamSynchronize(c->stream));
    return TDDA_OK;
}

tdda_status model_reinit(tdda_model* m, const double* nK, double E0, const double* nE0, const double* diel_old) {
    if (!m || !nK || !nE0 || !diel_old) {
        set_err("null argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    tdda_core* c = m->core;
    size_t bad = 0;
    if (!densities_in_table(diel_old, 3 * (size_t)c->N, c->nmat, &bad)) {
        set_err("density %g of entry %zu is outside the material table", diel_old[bad], bad);
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    TDDA_TRY(set_device(c->device));
    for (int j = 0; j < 3; j++) {
        m->nK[j] = nK[j];
        m->nE0[j] = nE0[j];
    }
    m->E0 = E0;
    m->dold_host_stale = true;  // uploaded straight from the caller; the host copy follows on demand
    const size_t n3 = 3 * (size_t)c->N;
    TDDA_CK(cudaMemsetAsync(m->P, 0, sizeof(double2) * n3, c->stream));
    TDDA_CK(cudaMemsetAsync(m->Ein, 0, sizeof(double2) * n3, c->stream));
    TDDA_TRY(model_upload_fields(m, true, true, diel_old));
    m->P_zero = true;
    m->ITERATION = 0;
    m->Error = 0.0;
    return TDDA_OK;
}

}  // namespace tdda_session

// ======================================================================= ABI
extern "C" {

int tdda_abi_version(void) { return TDDA_ABI_VERSION; }
const char* tdda_last_error(void) { return g_err.c_str(); }
int tdda_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

namespace {
tdda_status core_create(const tdda_core_desc* desc, const tdda::PeriodicImages* pi, tdda_core** out);

// The FCD tensor's Si/Ci tables, built once per device by k_sici_table and
// kept for the life of the process (2 x 8 MB).
std::mutex g_sici_mu;
double* g_sici[64][2];
tdda_status sici_tables(int device, cudaStream_t stream, const double** si, const double** ci) {
    std::lock_guard<std::mutex> lk(g_sici_mu);
    if (device < 0 || device >= 64) {
        set_err("device %d out of range", device);
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    if (!g_sici[device][0]) {
        double *a = nullptr, *b = nullptr;
        cudaError_t e = cudaMalloc((void**)&a, sizeof(double) * tdda::kSiCiN);
        if (e == cudaSuccess) e = cudaMalloc((void**)&b, sizeof(double) * tdda::kSiCiN);
        if (e == cudaSuccess) e = tdda::launch_sici_table(a, b, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) {
            if (a) cudaFree(a);
            if (b) cudaFree(b);
            return cuda_fail(e, "Si/Ci tables");
        }
        count_launches(1);
        g_sici[device][0] = a;
        g_sici[device][1] = b;
    }
    *si = g_sici[device][0];
    *ci = g_sici[device][1];
    return TDDA_OK;
}
}  // namespace

tdda_status tdda_core_create(const tdda_core_desc* desc, tdda_core** out) { return core_create(desc, nullptr, out); }

tdda_status tdda_core_create_periodic(const tdda_core_desc* desc, int MAXm, int MAXn, double Lm, double Ln,
                                      tdda_core** out) {
    g_err.clear();
    if (MAXm < 0 || MAXn < 0 || MAXm > 4096 || MAXn > 4096 || !std::isfinite(Lm) || !std::isfinite(Ln)) {
        set_err("invalid periodic images (MAXm %d, MAXn %d, Lm %g, Ln %g)", MAXm, MAXn, Lm, Ln);
        if (out) *out = nullptr;
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    const tdda::PeriodicImages pi{MAXm, MAXn, Lm, Ln};
    return core_create(desc, &pi, out);
}

namespace {
tdda_status core_create(const tdda_core_desc* desc, const tdda::PeriodicImages* pi, tdda_core** out) {
    g_err.clear();
    if (!desc || !out) {
        set_err("null argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    if (desc->Nx < 1 || desc->Ny < 1 || desc->Nz < 1 || desc->N < 1 || !desc->R || desc->nmat < 1 ||
        !desc->material || !(desc->d > 0) || !(desc->lam > 0) || !(desc->nback > 0) || desc->max_rhs < 1 ||
        desc->max_rhs > 64) {
        set_err("invalid core description");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    if (desc->nmat > tdda::kMaxMaterials) {
        set_err("at most %d materials", tdda::kMaxMaterials);
        return TDDA_ERR_UNSUPPORTED;
    }
    if (desc->method != TDDA_METHOD_LDR && desc->method != TDDA_METHOD_FCD) {
        set_err("unknown interaction method %d", desc->method);
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    if (desc->method == TDDA_METHOD_FCD) {
        // the smallest Si/Ci argument is (pi/d - K) d = pi - K d (nearest neighbours), and
        // the reference's tables start at 0.1 (SiCi.cpp:27-47)
        const double Kd = 2 * kPi / (desc->lam / desc->nback) * desc->d;
        if (!(kPi - Kd >= tdda::kSiCiDis)) {
            set_err("FCD needs K d <= pi - 0.1 (K d = %g): the spacing is too coarse for the wavelength", Kd);
            return TDDA_ERR_UNSUPPORTED;
        }
    }
    if ((long long)desc->Nx * desc->Ny * desc->Nz > (1LL << 28)) {
        set_err("lattice box too large");
        return TDDA_ERR_UNSUPPORTED;
    }
    if (tdda_device_count() < 1) {
        set_err("no CUDA device");
        return TDDA_ERR_NO_DEVICE;
    }
    tdda_status s = set_device(desc->device);
    if (s != TDDA_OK) return s;
    tdda_core* c = new tdda_core_s();
    c->device = desc->device;
    c->N = desc->N;
    c->nmat = desc->nmat;
    c->max_rhs = desc->max_rhs;
    c->method = desc->method;
    c->d = desc->d;
    c->lam = desc->lam;
    c->nback = desc->nback;
    c->K = 2 * kPi / (c->lam / c->nback);  // AProductCore.cpp:17
    c->material.resize(c->nmat);
    for (int i = 0; i < c->nmat; i++) {  // AProductCore.cpp:19-24 (the periodic ctor, :263-268, bumps below 1.01)
        cd m(desc->material[2 * i], desc->material[2 * i + 1]);
        m = m / (c->nback * c->nback);
        const double a = std::sqrt(std::norm(m));
        if (pi ? a < 1.01 : a <= 1.01) m = m + 0.01;
        c->material[i] = m;
    }
    c->R.assign(desc->R, desc->R + 3 * (size_t)desc->N);
    Geom& g = c->g;
    g.Nx = desc->Nx;
    g.Ny = desc->Ny;
    g.Nz = desc->Nz;
    g.N = desc->N;
    std::vector<int> cellmap((size_t)g.Nx * g.Ny * g.Nz, -1);
    for (int i = 0; i < g.N; i++) {
        int x = c->R[3 * i], y = c->R[3 * i + 1], z = c->R[3 * i + 2];
        if (x < 0 || x >= g.Nx || y < 0 || y >= g.Ny || z < 0 || z >= g.Nz) {
            set_err("dipole %d at (%d,%d,%d) lies outside the %dx%dx%d box", i, x, y, z, g.Nx, g.Ny, g.Nz);
            delete c;
            return TDDA_ERR_INVALID_ARGUMENT;
        }
        int& cell = cellmap[((size_t)x * g.Ny + y) * g.Nz + z];
        if (cell >= 0) {
            set_err("dipoles %d and %d occupy the same lattice site", cell, i);
            delete c;
            return TDDA_ERR_INVALID_ARGUMENT;
        }
        cell = i;
    }
    g.dense = 1;
    for (size_t k = 0; k < cellmap.size() && g.dense; k++) g.dense = cellmap[k] == (int)k;
    // FFT length per axis (fft_length)
    int Ms[3] = {fft_length(g.Nx, false), fft_length(g.Ny, false), fft_length(g.Nz, true)};
    AxisPlan* plans[3] = {&g.px, &g.py, &g.pz};
    for (int a = 0; a < 3; a++) {
        if (!make_plan(Ms[a], plans[a])) {
            set_err("no radix plan for FFT length %d", Ms[a]);
            delete c;
            return TDDA_ERR_UNSUPPORTED;
        }
    }
    g.Hx = g.px.M / 2 + 1;
    g.Hy = g.py.M / 2 + 1;
    g.Hz = g.pz.M / 2 + 1;
    g.sy = g.pz.M;
    g.sx = (long long)g.py.M * g.pz.M;
    g.sc = (long long)g.Nx * g.sx;
    g.sb = 3 * g.sc;
    if (tdda::max_pass_smem(g) > tdda::kMaxPassSmem) {
        set_err("FFT grid %dx%dx%d needs more shared memory per tile than a block has", g.px.M, g.py.M, g.pz.M);
        delete c;
        return TDDA_ERR_UNSUPPORTED;
    }
    c->maxblk = tdda::max_blocks_per_rhs(g);

#define TDDA_CORE_TRY(call)          \
    do {                             \
        tdda_status s_ = (call);     \
        if (s_ != TDDA_OK) {         \
            tdda_core_destroy(c);    \
            return s_;               \
        }                            \
    } while (0)
#define TDDA_CORE_CK(call)                                     \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) {                               \
            tdda_status s_ = cuda_fail(e_, #call);             \
            tdda_core_destroy(c);                              \
            return s_;                                         \
        }                                                      \
    } while (0)

    TDDA_CORE_CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
    {
        const char* v = std::getenv("TDDA_DEVICE_LOOP");
        c->device_loop = !(v && v[0] == '0');
        // early launch of the fused FP32 pass kernels (Geom::early; 0: every kernel the ordinary way)
        const char* el = std::getenv("TDDA_EARLY_LAUNCH");
        c->g.early = el ? std::atoi(el) : 3;
        if (cudaDeviceGetAttribute(&c->g.sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess) c->g.sms = 0;
    }
    const size_t n3 = 3 * (size_t)g.N;
    const long long H6 = 6LL * g.Hx * g.Hy * g.Hz;
    const long long Mfull = (long long)g.px.M * g.py.M * g.pz.M;
    TDDA_CORE_TRY(ensure_pool(c->device));
    TDDA_CORE_TRY(dalloc_c(c, &c->cellmap, cellmap.size()));
    TDDA_CORE_TRY(dalloc_c(c, &c->Rdev, 3 * (size_t)g.N));
    TDDA_CORE_TRY(dalloc_c(c, &c->green64, (size_t)H6));
    TDDA_CORE_TRY(dalloc_c(c, &c->green32, (size_t)H6));
    for (int a = 0; a < 3; a++) {
        TDDA_CORE_TRY(dalloc_c(c, &c->tw64[a], (size_t)plans[a]->M));
        TDDA_CORE_TRY(dalloc_c(c, &c->tw32[a], (size_t)plans[a]->M));
    }
    TDDA_CORE_TRY(dalloc_c(c, &c->grid64, (size_t)(g.sb * c->max_rhs)));
    TDDA_CORE_TRY(dalloc_c(c, &c->grid32, (size_t)(g.sb * c->max_rhs)));
    TDDA_CORE_TRY(dalloc_c(c, &c->vin64, n3));
    TDDA_CORE_TRY(dalloc_c(c, &c->vout64, n3));
    TDDA_CORE_TRY(dalloc_c(c, &c->vin32, n3));
    TDDA_CORE_TRY(dalloc_c(c, &c->vout32, n3));
    TDDA_CORE_TRY(dalloc_c(c, &c->rhs64, (size_t)c->max_rhs + 1));
    TDDA_CORE_TRY(dalloc_c(c, &c->rhs32, (size_t)c->max_rhs + 1));
    TDDA_CORE_TRY(dalloc_c(c, &c->st64, (size_t)c->max_rhs));
    TDDA_CORE_TRY(dalloc_c(c, &c->st32, (size_t)c->max_rhs));
    TDDA_CORE_TRY(dalloc_c(c, &c->part, (size_t)c->max_rhs * tdda::kPartSlots * c->maxblk));
    TDDA_CORE_TRY(dalloc_c(c, &c->cnt, (size_t)c->max_rhs * tdda::kCounters));
    TDDA_CORE_CK(pinned_get((void**)&c->hst, sizeof(SolveState) * c->max_rhs));
    // flag[0]: launch_scan's result; flag[1..2]: the |al|^2 range of TDDA_FP32_AUTO
    TDDA_CORE_TRY(dalloc_c(c, &c->flag, 3));
    TDDA_CORE_CK(pinned_get((void**)&c->hflag, 3 * sizeof(unsigned int)));
    TDDA_CORE_CK(cudaMemsetAsync(c->cnt, 0, sizeof(unsigned int) * c->max_rhs * tdda::kCounters, c->stream));
    TDDA_CORE_CK(cudaMemcpyAsync(c->cellmap, cellmap.data(), sizeof(int) * cellmap.size(), cudaMemcpyHostToDevice,
                                 c->stream));
    TDDA_CORE_CK(cudaMemcpyAsync(c->Rdev, c->R.data(), sizeof(int) * c->R.size(), cudaMemcpyHostToDevice, c->stream));
    for (int a = 0; a < 3; a++) {
        std::vector<double2> w64;
        std::vector<float2> w32;
        twiddles(plans[a]->M, w64, w32);
        TDDA_CORE_CK(cudaMemcpyAsync(c->tw64[a], w64.data(), sizeof(double2) * w64.size(), cudaMemcpyHostToDevice,
                                     c->stream));
        TDDA_CORE_CK(cudaMemcpyAsync(c->tw32[a], w32.data(), sizeof(float2) * w32.size(), cudaMemcpyHostToDevice,
                                     c->stream));
        TDDA_CORE_CK(cudaStreamSynchronize(c->stream));
    }
    // plain-product slots (the entry after the batch slots)
    RhsVecs<double> p64{};
    p64.p = c->vin64;
    p64.Ap = c->vout64;
    RhsVecs<float> p32{};
    p32.p = c->vin32;
    p32.Ap = c->vout32;
    TDDA_CORE_CK(cudaMemcpyAsync(c->rhs64 + c->max_rhs, &p64, sizeof(p64), cudaMemcpyHostToDevice, c->stream));
    TDDA_CORE_CK(cudaMemcpyAsync(c->rhs32 + c->max_rhs, &p32, sizeof(p32), cudaMemcpyHostToDevice, c->stream));
    TDDA_CORE_TRY(configure_once(c->device));
    c->inter.fcd = c->method == TDDA_METHOD_FCD;
    if (c->inter.fcd) TDDA_CORE_TRY(sici_tables(c->device, c->stream, &c->inter.si, &c->inter.ci));
    // Green spectrum (AProductCore.cpp:53-229; periodic: :300-520), on a temporary full grid
    double2* full6 = nullptr;
    double2* oct = nullptr;
    TDDA_CORE_CK(cudaMallocAsync((void**)&full6, sizeof(double2) * 6 * (size_t)Mfull, c->stream));
    // the octant of lattice offsets (both forms: the tensor is even or odd in each axis)
    TDDA_CORE_CK(cudaMallocAsync((void**)&oct, sizeof(double2) * 6 * (size_t)g.Nx * g.Ny * g.Nz, c->stream));
    count_launches(6);
    cudaError_t ge = tdda::launch_green(g, c->K, c->d, c->tw64[0], c->tw64[1], c->tw64[2], full6, c->green64,
                                        c->green32, c->stream, c->inter, pi, oct);
    cudaError_t fe = cudaFreeAsync(full6, c->stream);
    if (oct && fe == cudaSuccess) fe = cudaFreeAsync(oct, c->stream);
    TDDA_CORE_CK(ge);
    TDDA_CORE_CK(fe);
    TDDA_CORE_CK(cudaStreamSynchronize(c->stream));
    if (pi) c->periodic = *pi, c->is_periodic = true;
#undef TDDA_CORE_TRY
#undef TDDA_CORE_CK
    *out = c;
    return TDDA_OK;
}
}  // namespace

tdda_status tdda_core_destroy(tdda_core* c) {
    if (!c) return TDDA_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& e : c->g64.iter)
        if (e) cudaGraphExecDestroy(e);
    for (auto& e : c->g32.iter)
        if (e) cudaGraphExecDestroy(e);
    free_all(c->allocs, c->stream);
    if (c->stream) cudaStreamSynchronize(c->stream);
    pinned_put(c->hst, sizeof(SolveState) * c->max_rhs);
    if (c->hst_first) pinned_put(c->hst_first, sizeof(SolveState) * c->max_rhs);
    pinned_put(c->hflag, 3 * sizeof(unsigned int));
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return TDDA_OK;
}

tdda_status tdda_core_info(const tdda_core* c, double* K, int* grid3, double* material_norm) {
    if (!c) {
        set_err("null core");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    if (K) *K = c->K;
    if (grid3) {
        grid3[0] = c->g.px.M;
        grid3[1] = c->g.py.M;
        grid3[2] = c->g.pz.M;
    }
    if (material_norm)
        for (int i = 0; i < c->nmat; i++) {
            material_norm[2 * i] = c->material[i].real();
            material_norm[2 * i + 1] = c->material[i].imag();
        }
    return TDDA_OK;
}

tdda_status tdda_core_ldr_inter(const tdda_core* c, double x, double y, double z, double* out12) {
    if (!c || !out12) {
        set_err("null argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    cd t[6];
    ldr_host(c->K, x, y, z, t);
    for (int l = 0; l < 6; l++) {
        out12[2 * l] = t[l].real();
        out12[2 * l + 1] = t[l].imag();
    }
    return TDDA_OK;
}

tdda_status tdda_core_interaction(const tdda_core* c, double x, double y, double z, double* out12) {
    if (!c || !out12) {
        set_err("null argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    double2 t[6];
    tdda::Interaction it{c->inter.fcd, nullptr, nullptr};  // host: Si/Ci node values evaluated directly
    tdda::interaction_tensor(it, c->K, c->d, x, y, z, t);
    for (int l = 0; l < 6; l++) {
        out12[2 * l] = t[l].x;
        out12[2 * l + 1] = t[l].y;
    }
    return TDDA_OK;
}

tdda_status tdda_aproduct(tdda_core* c, int precision, const double* b, double* y, int mem) {
    if (!c || !b || !y || (precision != TDDA_FP64 && precision != TDDA_FP32_REFINE)) {
        set_err("invalid argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    TDDA_TRY(set_device(c->device));
    const size_t n3 = 3 * (size_t)c->N;
    TDDA_CK(cudaMemcpyAsync(c->vin64, b, sizeof(double2) * n3, kind_in(mem), c->stream));
    if (precision == TDDA_FP64) {
        TDDA_CK(aprod<double>(c, tdda::SRC_IN, tdda::SNK_OUT, 1, c->rhs64 + c->max_rhs));
    } else {
        TDDA_CK1(tdda::launch_to_f32((int)n3, c->vin64, c->vin32, c->stream));
        TDDA_CK(aprod<float>(c, tdda::SRC_IN, tdda::SNK_OUT, 1, c->rhs32 + c->max_rhs));
        TDDA_CK1(tdda::launch_zero<double>((long long)n3, c->vout64, c->stream));
        TDDA_CK1(tdda::launch_accumulate((int)n3, c->vout32, c->vout64, c->stream));
    }
    TDDA_CK(cudaMemcpyAsync(y, c->vout64, sizeof(double2) * n3, kind_out(mem), c->stream));
    TDDA_CK(cudaStreamSynchronize(c->stream));
    return TDDA_OK;
}

tdda_status tdda_model_create(tdda_core* c, const double* nK, double E0, const double* nE0, const double* diel_old,
                              tdda_model** out) {
    if (!c || !nK || !nE0 || !diel_old || !out) {
        set_err("null argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    *out = nullptr;
    {
        size_t bad = 0;
        if (!densities_in_table(diel_old, 3 * (size_t)c->N, c->nmat, &bad)) {
            set_err("density %g of entry %zu is outside the material table", diel_old[bad], bad);
            return TDDA_ERR_INVALID_ARGUMENT;
        }
    }
    TDDA_TRY(set_device(c->device));
    tdda_model* m = new tdda_model_s();
    m->core = c;
    for (int j = 0; j < 3; j++) {
        m->nK[j] = nK[j];
        m->nE0[j] = nE0[j];
    }
    m->E0 = E0;
    const size_t n3 = 3 * (size_t)c->N;
    m->dold_host_stale = true;  // uploaded straight from the caller; the host copy follows on demand
    double2** v[] = {&m->P, &m->E, &m->al, &m->diel, &m->Ein, &m->r, &m->r0, &m->p, &m->u, &m->t, &m->Ap, &m->At};
    for (double2** q : v) {
        tdda_status s = dalloc(m->allocs, q, n3, c->stream);
        if (s != TDDA_OK) {
            tdda_model_destroy(m);
            return s;
        }
    }
    {
        tdda_status s = dalloc(m->allocs, &m->dold, n3, c->stream);
        if (s != TDDA_OK) {
            tdda_model_destroy(m);
            return s;
        }
    }
    cudaError_t e = cudaMemsetAsync(m->P, 0, sizeof(double2) * n3, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->Ein, 0, sizeof(double2) * n3, c->stream);
    if (e != cudaSuccess) {
        tdda_model_destroy(m);
        return cuda_fail(e, "cudaMemsetAsync");
    }
    tdda_status s = model_upload_fields(m, true, true, diel_old);
    if (s != TDDA_OK) {
        tdda_model_destroy(m);
        return s;
    }
    *out = m;
    return TDDA_OK;
}

tdda_status tdda_model_destroy(tdda_model* m) {
    if (!m) return TDDA_OK;
    cudaSetDevice(m->core->device);
    cudaStreamSynchronize(m->core->stream);
    free_all(m->allocs, m->core->stream);
    delete m;
    return TDDA_OK;
}

tdda_status tdda_model_update_alpha(tdda_model* m, const double* diel_old) {
    if (!m || !diel_old) {
        set_err("null argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    TDDA_TRY(set_device(m->core->device));
    tdda_core* c = m->core;
    const size_t n3 = 3 * (size_t)c->N;
    if (!m->dold_bak) TDDA_TRY(dalloc(m->allocs, &m->dold_bak, n3, c->stream));
    // keep the current densities, upload, then check the range on the device
    // before anything that depends on the densities changes (the host scan below
    // only names the entry)
    TDDA_CK(cudaMemcpyAsync(m->dold_bak, m->dold, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->stream));
    TDDA_CK(cudaMemcpyAsync(m->dold, diel_old, sizeof(double) * n3, cudaMemcpyHostToDevice, c->stream));
    TDDA_CK1(tdda::launch_scan((long long)n3, m->dold, 1, (double)c->nmat, c->flag, c->stream));
    TDDA_CK(cudaMemcpyAsync(c->hflag, c->flag, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream));
    TDDA_CK(cudaStreamSynchronize(c->stream));
    if (*c->hflag || c->nmat < 2) {
        size_t bad = 0;
        densities_in_table(diel_old, n3, c->nmat, &bad);
        TDDA_CK(cudaMemcpyAsync(m->dold, m->dold_bak, sizeof(double) * n3, cudaMemcpyDeviceToDevice, c->stream));
        TDDA_CK(cudaStreamSynchronize(c->stream));  // the model keeps its densities
        set_err("density %g of entry %zu is outside the material table", diel_old[bad], bad);
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    // no wait for the alpha kernel: the caller's densities were read before the scan's
    // synchronisation, and everything that reads al runs on the core's stream or waits
    // for it (the cross-lattice sessions synchronise a model's stream at admission)
    TDDA_CK1(tdda::launch_model_alpha((int)n3, m->dold, alpha_params(m), m->diel, m->al, m->fal, c->stream));
    m->dold_host_stale = true;  // the device holds the densities; the host copy follows on demand
    return TDDA_OK;
}

// the host copy of the densities, refreshed from the device after UpdateAlpha
static tdda_status host_densities(tdda_model* m) {
    if (!m->dold_host_stale) return TDDA_OK;
    tdda_core* c = m->core;
    m->diel_old.resize(3 * (size_t)c->N);
    TDDA_CK(cudaMemcpyAsync(m->diel_old.data(), m->dold, sizeof(double) * 3 * (size_t)c->N, cudaMemcpyDeviceToHost,
                            c->stream));
    TDDA_CK(cudaStreamSynchronize(c->stream));
    m->dold_host_stale = false;
    return TDDA_OK;
}

tdda_status tdda_model_update_alpha_single(tdda_model* m, int idx, double value) {
    if (!m || idx < 0 || idx >= m->core->N) {
        set_err("invalid argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    TDDA_TRY(set_device(m->core->device));
    TDDA_TRY(host_densities(m));
    std::vector<double> d = m->diel_old;
    d[3 * (size_t)idx] = d[3 * (size_t)idx + 1] = d[3 * (size_t)idx + 2] = value;
    return tdda_model_update_alpha(m, d.data());
}

tdda_status tdda_model_change_E(tdda_model* m, const double* E, int mem) {
    if (!m || !E) {
        set_err("null argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    TDDA_TRY(set_device(m->core->device));
    TDDA_CK(cudaMemcpyAsync(m->E, E, sizeof(double2) * 3 * (size_t)m->core->N, kind_in(mem), m->core->stream));
    TDDA_CK(cudaStreamSynchronize(m->core->stream));
    return TDDA_OK;
}

tdda_status tdda_model_reset_E(tdda_model* m) {
    if (!m) {
        set_err("null model");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    TDDA_TRY(set_device(m->core->device));
    return model_upload_fields(m, true, false);
}

tdda_status tdda_model_initialize_P(tdda_model* m, const double* P, int mem) {
    if (!m) {
        set_err("null model");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    TDDA_TRY(set_device(m->core->device));
    const size_t n = 6 * (size_t)m->core->N;
    if (!P) {  // P = 0 without a transfer
        TDDA_CK(cudaMemsetAsync(m->P, 0, sizeof(double) * n, m->core->stream));
        TDDA_CK(cudaStreamSynchronize(m->core->stream));
        m->P_zero = true;
        return TDDA_OK;
    }
    tdda_core* c = m->core;
    TDDA_CK(cudaMemcpyAsync(m->P, P, sizeof(double) * n, kind_in(mem), c->stream));
    TDDA_CK1(tdda::launch_scan((long long)n, reinterpret_cast<const double*>(m->P), 0, 0.0, c->flag, c->stream));
    TDDA_CK(cudaMemcpyAsync(c->hflag, c->flag, sizeof(unsigned int), cudaMemcpyDeviceToHost, c->stream));
    TDDA_CK(cudaStreamSynchronize(c->stream));
    const bool zero = *c->hflag == 0;
    m->P_zero = zero;  // A 0 = 0 exactly, so the solve may skip its first product
    return TDDA_OK;
}

tdda_status tdda_model_aproduct_with_alb(tdda_model* m, const double* b, double* y, int mem) {
    if (!m || !b || !y) {
        set_err("null argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    tdda_core* c = m->core;
    TDDA_TRY(set_device(c->device));
    const size_t n3 = 3 * (size_t)c->N;
    RhsVecs<double> v{};
    v.p = c->vin64;
    v.Ap = c->vout64;
    v.al = m->al;
    TDDA_CK(cudaMemcpyAsync(c->rhs64 + c->max_rhs, &v, sizeof(v), cudaMemcpyHostToDevice, c->stream));
    TDDA_CK(cudaMemcpyAsync(c->vin64, b, sizeof(double2) * n3, kind_in(mem), c->stream));
    TDDA_CK(aprod<double>(c, tdda::SRC_IN, tdda::SNK_ALB, 1, c->rhs64 + c->max_rhs));
    TDDA_CK(cudaMemcpyAsync(y, c->vout64, sizeof(double2) * n3, kind_out(mem), c->stream));
    v.al = nullptr;
    TDDA_CK(cudaMemcpyAsync(c->rhs64 + c->max_rhs, &v, sizeof(v), cudaMemcpyHostToDevice, c->stream));
    TDDA_CK(cudaStreamSynchronize(c->stream));
    return TDDA_OK;
}

tdda_status tdda_solve_batch(tdda_model* const* ms, int n, int precision, int max_it, double max_err,
                             tdda_solve_info* infos) {
    g_err.clear();
    TDDA_TRY(check_batch(ms, n));
    if (!(max_err >= 0) || (precision != TDDA_FP64 && precision != TDDA_FP32_REFINE &&
                            precision != TDDA_FP32_JACOBI && precision != TDDA_FP32_AUTO)) {
        set_err("invalid tolerance or precision");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    TDDA_TRY(set_device(ms[0]->core->device));
    if (precision == TDDA_FP64) return solve_fp64(ms, n, max_it, max_err, infos);
    return solve_mixed(ms, n, max_it, max_err, infos, precond_mode(precision));
}

namespace {
// shapes of tdda_solve_multi, kept per (device, grid, width) for the next call
struct ShapeKey {
    int device, Mx, My, Mz, cap;
    bool operator==(const ShapeKey& o) const {
        return device == o.device && Mx == o.Mx && My == o.My && Mz == o.Mz && cap == o.cap;
    }
};
std::mutex g_shape_mu;
std::vector<std::pair<ShapeKey, tdda_session::Shape*>> g_shapes;  // idle shapes
}  // namespace

tdda_status tdda_solve_multi(tdda_model* const* ms, int n, int max_it, double max_err, tdda_solve_info* infos) {
    return tdda_solve_multi_precision(ms, n, TDDA_FP32_REFINE, max_it, max_err, infos);
}

tdda_status tdda_solve_multi_precision(tdda_model* const* ms, int n, int precision, int max_it, double max_err,
                                       tdda_solve_info* infos) {
    g_err.clear();
    if (!ms || n < 1 || n > 64 || !(max_err >= 0) ||
        (precision != TDDA_FP32_REFINE && precision != TDDA_FP32_JACOBI && precision != TDDA_FP32_AUTO)) {
        set_err("invalid batch, precision, tolerance or size (1..64 right-hand sides)");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    for (int i = 0; i < n; i++) {
        if (!ms[i]) {
            set_err("null model");
            return TDDA_ERR_INVALID_ARGUMENT;
        }
        for (int j = 0; j < i; j++)
            if (ms[j] == ms[i]) {
                set_err("a model appears twice in a batch");
                return TDDA_ERR_INVALID_ARGUMENT;
            }
    }
    int grid[3];
    tdda_session::core_grid(ms[0]->core, grid);
    const int device = ms[0]->core->device;
    for (int i = 1; i < n; i++) {
        int gi[3];
        tdda_session::core_grid(ms[i]->core, gi);
        if (ms[i]->core->device != device || gi[0] != grid[0] || gi[1] != grid[1] || gi[2] != grid[2]) {
            set_err("models of a cross-lattice batch share one device and FFT grid shape (%dx%dx%d and %dx%dx%d)",
                    grid[0], grid[1], grid[2], gi[0], gi[1], gi[2]);
            return TDDA_ERR_INVALID_ARGUMENT;
        }
    }
    const ShapeKey key{device, grid[0], grid[1], grid[2], n};
    tdda_session::Shape* sh = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_shape_mu);
        for (size_t k = 0; k < g_shapes.size(); k++)
            if (g_shapes[k].first == key) {
                sh = g_shapes[k].second;
                g_shapes.erase(g_shapes.begin() + (long)k);
                break;
            }
    }
    if (!sh) TDDA_TRY(tdda_session::shape_create(device, grid, n, &sh));
    tdda_status worst = TDDA_OK;
    tdda_status st = TDDA_OK;
    for (int i = 0; i < n && st == TDDA_OK; i++)
        st = tdda_session::shape_admit(sh, ms[i], max_it, max_err, nullptr, precond_mode(precision));
    std::vector<tdda_session::Done> done;
    while (st == TDDA_OK && tdda_session::shape_active(sh) > 0) st = tdda_session::shape_step(sh, &done);
    if (st != TDDA_OK) {
        tdda_session::shape_destroy(sh);  // slots may hold models mid-solve
        return st;
    }
    for (const auto& d : done) {
        for (int i = 0; i < n; i++)
            if (ms[i] == d.model && infos) infos[i] = d.info;
        if (d.info.status != TDDA_OK && worst == TDDA_OK) worst = (tdda_status)d.info.status;
    }
    {
        std::lock_guard<std::mutex> lk(g_shape_mu);
        g_shapes.emplace_back(key, sh);
        if (g_shapes.size() > 16) {  // keep a few shapes; the oldest goes
            tdda_session::shape_destroy(g_shapes.front().second);
            g_shapes.erase(g_shapes.begin());
        }
    }
    return worst;
}

tdda_status tdda_model_bicgstab(tdda_model* m, int max_it, double max_err, tdda_solve_info* info) {
    return tdda_solve_batch(&m, 1, TDDA_FP64, max_it, max_err, info);
}

tdda_status tdda_model_solve_mixed(tdda_model* m, int max_it, double max_err, tdda_solve_info* info) {
    return tdda_solve_batch(&m, 1, TDDA_FP32_REFINE, max_it, max_err, info);
}

tdda_status tdda_model_update_E_in_structure(tdda_model* m) {
    if (!m) {
        set_err("null model");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    TDDA_TRY(set_device(m->core->device));
    TDDA_CK1(tdda::launch_einternal(3 * m->core->N, m->al, m->P, m->diel, m->Ein, m->core->stream));
    TDDA_CK(cudaStreamSynchronize(m->core->stream));
    return TDDA_OK;
}

tdda_status tdda_model_get(const tdda_model* m, int field, double* out, int mem) {
    if (!m || !out) {
        set_err("null argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    const double2* src = field == TDDA_FIELD_P ? m->P
                         : field == TDDA_FIELD_E ? m->E
                         : field == TDDA_FIELD_AL ? m->al
                         : field == TDDA_FIELD_DIEL ? m->diel
                         : field == TDDA_FIELD_EINTERNAL ? m->Ein
                                                         : nullptr;
    if (!src) {
        set_err("unknown field %d", field);
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    TDDA_TRY(set_device(m->core->device));
    TDDA_CK(cudaMemcpyAsync(out, src, sizeof(double2) * 3 * (size_t)m->core->N, kind_out(mem), m->core->stream));
    TDDA_CK(cudaStreamSynchronize(m->core->stream));
    return TDDA_OK;
}

int tdda_model_iterations(const tdda_model* m) { return m ? m->ITERATION : -1; }

tdda_status tdda_model_density_gradient(const tdda_model* fwd, int nadj, tdda_model* const* adj, const double* coef,
                                        int nparam, const int* offsets, const int* dipoles, double* s_out) {
    if (!fwd || nadj < 1 || nadj > 8 || !adj || !coef || nparam < 0 || !offsets || !dipoles || !s_out) {
        set_err("invalid argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    tdda_core* c = fwd->core;
    for (int k = 0; k < nadj; k++)
        if (!adj[k] || adj[k]->core != c) {
            set_err("adjoint model %d is missing or on another core", k);
            return TDDA_ERR_INVALID_ARGUMENT;
        }
    const int nd = nparam > 0 ? offsets[nparam] : 0;
    if (offsets[0] != 0) {
        set_err("offsets[0] must be 0");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    for (int i = 0; i < nparam; i++)
        if (offsets[i + 1] < offsets[i]) {
            set_err("offsets must not decrease (parameter %d)", i);
            return TDDA_ERR_INVALID_ARGUMENT;
        }
    for (int q = 0; q < nd; q++)
        if (dipoles[q] < 0 || dipoles[q] >= c->N) {
            set_err("dipole %d of the parameter map is outside 0..%d", dipoles[q], c->N - 1);
            return TDDA_ERR_INVALID_ARGUMENT;
        }
    if (nparam == 0) return TDDA_OK;
    TDDA_TRY(set_device(c->device));
    tdda::GradArgs ga{};
    ga.nadj = nadj;
    for (int k = 0; k < nadj; k++) {
        ga.lam[k] = adj[k]->P;
        ga.coef[k] = make_double2(coef[2 * k], coef[2 * k + 1]);
    }
    std::vector<void*> tmp;
    int *doff = nullptr, *ddip = nullptr;
    double* dout = nullptr;
    tdda_status st = dalloc(tmp, &doff, (size_t)nparam + 1, c->stream);
    if (st == TDDA_OK) st = dalloc(tmp, &ddip, (size_t)std::max(nd, 1), c->stream);
    if (st == TDDA_OK) st = dalloc(tmp, &dout, (size_t)nparam, c->stream);
    cudaError_t e = cudaSuccess;
    if (st == TDDA_OK) {
        e = cudaMemcpyAsync(doff, offsets, sizeof(int) * ((size_t)nparam + 1), cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess && nd > 0)
            e = cudaMemcpyAsync(ddip, dipoles, sizeof(int) * (size_t)nd, cudaMemcpyHostToDevice, c->stream);
        count_launches(1);
        if (e == cudaSuccess)
            e = tdda::launch_density_gradient(nparam, doff, ddip, fwd->P, fwd->diel, fwd->dold, alpha_params(fwd), ga,
                                              dout, c->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s_out, dout, sizeof(double) * (size_t)nparam, cudaMemcpyDeviceToHost, c->stream);
    }
    free_all(tmp, c->stream);
    if (st != TDDA_OK) return st;
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "density gradient");
    return TDDA_OK;
}

tdda_status tdda_model_field_at(tdda_model* m, int npts, const double* points, double* E, int mem) {
    if (!m || npts < 0 || (npts > 0 && (!points || !E))) {
        set_err("invalid argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    if (npts == 0) return TDDA_OK;
    tdda_core* c = m->core;
    TDDA_TRY(set_device(c->device));
    const int nb = tdda::field_blocks(c->N, npts);
    std::vector<void*> tmp;
    double* dpts = nullptr;
    double2 *part = nullptr, *dE = nullptr;
    tdda_status st = dalloc(tmp, &part, 3 * (size_t)nb * npts, c->stream);
    if (st == TDDA_OK && mem != TDDA_MEM_DEVICE) st = dalloc(tmp, &dpts, 3 * (size_t)npts, c->stream);
    if (st == TDDA_OK && mem != TDDA_MEM_DEVICE) st = dalloc(tmp, &dE, 3 * (size_t)npts, c->stream);
    cudaError_t e = cudaSuccess;
    if (st == TDDA_OK) {
        if (mem != TDDA_MEM_DEVICE) {
            e = cudaMemcpyAsync(dpts, points, sizeof(double) * 3 * (size_t)npts, cudaMemcpyHostToDevice, c->stream);
        } else {
            dpts = const_cast<double*>(points);
            dE = reinterpret_cast<double2*>(E);
        }
        count_launches(2 * ((npts + 32767) / 32768));
        if (e == cudaSuccess)
            e = tdda::launch_field_at(c->N, c->Rdev, c->d, c->K, c->inter, m->P, npts, dpts, make_double3(m->nK[0], m->nK[1], m->nK[2]),
                                      make_double3(m->nE0[0], m->nE0[1], m->nE0[2]), m->E0, part, dE, c->stream);
        if (e == cudaSuccess && mem != TDDA_MEM_DEVICE)
            e = cudaMemcpyAsync(E, dE, sizeof(double2) * 3 * (size_t)npts, cudaMemcpyDeviceToHost, c->stream);
    }
    free_all(tmp, c->stream);
    if (st != TDDA_OK) return st;
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "field at points");
    return TDDA_OK;
}

tdda_status tdda_fft3d(double* data, int n0, int n1, int n2, int sign) {
    AxisPlan p[3];
    int n[3] = {n0, n1, n2};
    if (!data || (sign != -1 && sign != 1)) {
        set_err("invalid argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    for (int a = 0; a < 3; a++)
        if (n[a] < 1 || !make_plan(n[a], &p[a]) || n[a] > 2048) {
            set_err("FFT length %d is not supported", n[a]);
            return TDDA_ERR_UNSUPPORTED;
        }
    std::vector<void*> tmp;
    double2* tw[3];
    for (int a = 0; a < 3; a++) {
        std::vector<double2> w64;
        std::vector<float2> w32;
        twiddles(n[a], w64, w32);
        tdda_status s = dalloc(tmp, &tw[a], (size_t)n[a], (cudaStream_t)0);
        if (s != TDDA_OK) {
            free_all(tmp, 0);
            return s;
        }
        cudaMemcpy(tw[a], w64.data(), sizeof(double2) * n[a], cudaMemcpyHostToDevice);
    }
    cudaError_t e = tdda::configure_kernels();
    count_launches(3);
    if (e == cudaSuccess) e = tdda::launch_fft3d_f64((double2*)data, p[0], p[1], p[2], tw[0], tw[1], tw[2], sign, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    free_all(tmp, 0);
    cudaStreamSynchronize(0);
    if (e != cudaSuccess) return cuda_fail(e, "tdda_fft3d");
    return TDDA_OK;
}

tdda_status tdda_core_stream(const tdda_core* c, void** stream) {
    if (!c || !stream) {
        set_err("null argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    *stream = (void*)c->stream;
    return TDDA_OK;
}

unsigned long long tdda_kernel_launches(void) { return g_launches.load(); }

const char* tdda_core_pass_name(const tdda_core* c, int precision, int pass) {
    if (!c || pass < 0 || pass > 4 || (precision != TDDA_FP64 && precision != TDDA_FP32_REFINE)) return nullptr;
    const bool fp32 = precision == TDDA_FP32_REFINE;
    const bool fused = tdda::zy_fused(c->g, fp32);
    switch (pass) {
        case 0: return fused ? "k_zyfwd" : "k_zfwd";
        case 1: return fused ? "" : "k_ypass";
        case 2: return fp32 && c->g.x_form == 0 && tdda::xpass2_length(c->g.px.M) ? "k_xpass2" : "k_xpass";
        case 3: return fused ? "k_yzinv" : "k_ypass";
        default: return fused ? "" : "k_zinv";
    }
}

int tdda_core_pass_count(const tdda_core* c, int precision) {
    if (!c || (precision != TDDA_FP64 && precision != TDDA_FP32_REFINE)) return -1;
    return tdda::zy_fused(c->g, precision == TDDA_FP32_REFINE) ? 3 : 5;
}

namespace {
// the five pass times of `reps` plain products (arguments checked by the caller)
tdda_status profile_products(tdda_core* c, int precision, int nrhs, int reps, double* ms5) {
    // nrhs plain products on the core's input / output vectors (the same
    // vectors for every right-hand side: the passes read and write the
    // grid slot of each right-hand side separately)
    std::vector<RhsVecs<double>> h64(nrhs, RhsVecs<double>{});
    std::vector<RhsVecs<float>> h32(nrhs, RhsVecs<float>{});
    for (int i = 0; i < nrhs; i++) {
        h64[i].p = c->vin64;
        h64[i].Ap = c->vout64;
        h32[i].p = c->vin32;
        h32[i].Ap = c->vout32;
    }
    TDDA_CK(cudaMemcpyAsync(c->rhs64, h64.data(), sizeof(RhsVecs<double>) * nrhs, cudaMemcpyHostToDevice, c->stream));
    TDDA_CK(cudaMemcpyAsync(c->rhs32, h32.data(), sizeof(RhsVecs<float>) * nrhs, cudaMemcpyHostToDevice, c->stream));
    cudaEvent_t ev[6];
    for (auto& e : ev) TDDA_CK(cudaEventCreate(&e));
    double acc[5] = {0, 0, 0, 0, 0};
    tdda_status st = TDDA_OK;
    // an FP32 batch schedule of groups: each group's passes are timed and the
    // groups' times of a pass added
    const int gs = precision == TDDA_FP64 ? nrhs : group_size<float>(c, nrhs);
    for (int r = 0; r < reps + 1 && st == TDDA_OK; r++) {  // the first run is a warm-up
        for (int g0 = 0; g0 < nrhs && st == TDDA_OK; g0 += gs) {
            const int n = std::min(gs, nrhs - g0);
            count_launches(precision == TDDA_FP64 ? product_kernels<double>(c) : product_kernels<float>(c));
            cudaError_t e =
                precision == TDDA_FP64
                    ? tdda::launch_aproduct<double>(c->g, tdda::SRC_IN, tdda::SNK_OUT, n, c->rhs64 + g0, c->green64,
                                                    c->tw64[0], c->tw64[1], c->tw64[2], c->cellmap, c->grid64,
                                                    c->stream, ev, 0)
                    : tdda::launch_aproduct<float>(c->g, tdda::SRC_IN, tdda::SNK_OUT, n, c->rhs32 + g0, c->green32,
                                                   c->tw32[0], c->tw32[1], c->tw32[2], c->cellmap, c->grid32,
                                                   c->stream, ev, 0);
            if (e == cudaSuccess) e = cudaEventSynchronize(ev[5]);
            if (e != cudaSuccess) {
                st = cuda_fail(e, "profiled A-product");
                break;
            }
            for (int k = 0; k < 5 && r > 0; k++) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, ev[k], ev[k + 1]);
                acc[k] += ms;
            }
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    for (int k = 0; k < 5; k++) ms5[k] = acc[k] / reps;
    return st;
}

// A captured solve step holds its pass kernels and their Geom: a new FP32 x-pass
// configuration drops the FP32 step graphs (captured again on next use).
tdda_status set_xpass(tdda_core* c, int form, int tile) {
    if (c->g.x_form == form && c->g.x_tile == tile) return TDDA_OK;
    TDDA_CK(cudaStreamSynchronize(c->stream));
    for (auto& e : c->g32.iter)
        if (e) cudaGraphExecDestroy(e), e = nullptr;
    c->g.x_form = form;
    c->g.x_tile = tile;
    return TDDA_OK;
}

// The batch schedule is part of the captured FP32 steps: a new one drops them.
tdda_status set_batch_group(tdda_core* c, int group) {
    if (c->group == group) return TDDA_OK;
    TDDA_CK(cudaStreamSynchronize(c->stream));
    for (auto& e : c->g32.iter)
        if (e) cudaGraphExecDestroy(e), e = nullptr;
    c->group = group;
    return TDDA_OK;
}
}  // namespace

tdda_status tdda_profile_aproduct(tdda_core* c, int precision, int nrhs, int reps, double* ms5) {
    if (!c || !ms5 || reps < 1 || nrhs < 1 || nrhs > c->max_rhs ||
        (precision != TDDA_FP64 && precision != TDDA_FP32_REFINE)) {
        set_err("invalid argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    TDDA_TRY(set_device(c->device));
    return profile_products(c, precision, nrhs, reps, ms5);
}

tdda_status tdda_core_set_xpass(tdda_core* c, int form, int tile) {
    if (!c || (form != 0 && form != 1) || (tile != 0 && tile != 8 && tile != 16) || (form == 1 && tile != 0)) {
        set_err("invalid argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    TDDA_TRY(set_device(c->device));
    return set_xpass(c, form, tile);
}

tdda_status tdda_core_autotune(tdda_core* c, int nrhs, int reps, tdda_xpass_tune* out) {
    if (!c || !out || reps < 1 || nrhs < 1 || nrhs > c->max_rhs) {
        set_err("invalid argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    TDDA_TRY(set_device(c->device));
    *out = tdda_xpass_tune{};
    // candidates: the register form with 8 and 16 z-columns a block, where the
    // x length has a two-stage plan, and the shared-memory form
    int nc = 0;
    if (tdda::xpass2_length(c->g.px.M)) {
        out->form[nc] = 0, out->tile[nc++] = 8;
        out->form[nc] = 0, out->tile[nc++] = 16;
    }
    out->form[nc] = 1, out->tile[nc++] = 0;
    out->ncand = nc;
    const int form0 = c->g.x_form, tile0 = c->g.x_tile;
    int best = -1;
    for (int k = 0; k < nc; k++) {
        double ms5[5];
        tdda_status st = set_xpass(c, out->form[k], out->tile[k]);
        if (st == TDDA_OK) st = profile_products(c, TDDA_FP32_REFINE, nrhs, reps, ms5);
        if (st != TDDA_OK) {
            set_xpass(c, form0, tile0);
            return st;
        }
        out->ms[k] = ms5[0] + ms5[1] + ms5[2] + ms5[3] + ms5[4];
        if (best < 0 || out->ms[k] < out->ms[best]) best = k;
    }
    out->x_form = out->form[best];
    out->x_tile = out->tile[best];
    return set_xpass(c, out->x_form, out->x_tile);
}

tdda_status tdda_core_set_batch_group(tdda_core* c, int group) {
    if (!c || group < 0 || group > c->max_rhs) {
        set_err("invalid argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    TDDA_TRY(set_device(c->device));
    return set_batch_group(c, group);
}

tdda_status tdda_core_autotune_batch(tdda_core* c, int nrhs, int reps, tdda_batch_tune* out) {
    if (!c || !out || reps < 1 || nrhs < 1 || nrhs > c->max_rhs) {
        set_err("invalid argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    TDDA_TRY(set_device(c->device));
    *out = tdda_batch_tune{};
    // candidates: the whole batch in one launch per pass (0), then halves of it
    int nc = 0;
    out->groups[nc++] = 0;
    for (int g = nrhs / 2; g >= 1 && nc < 4; g /= 2)
        if (g < nrhs) out->groups[nc++] = g;
    out->ncand = nc;
    const int group0 = c->group;
    int best = -1;
    for (int k = 0; k < nc; k++) {
        double ms5[5];
        tdda_status st = set_batch_group(c, out->groups[k]);
        if (st == TDDA_OK) st = profile_products(c, TDDA_FP32_REFINE, nrhs, reps, ms5);
        if (st != TDDA_OK) {
            set_batch_group(c, group0);
            return st;
        }
        out->ms[k] = ms5[0] + ms5[1] + ms5[2] + ms5[3] + ms5[4];
        if (best < 0 || out->ms[k] < out->ms[best]) best = k;
    }
    out->group = out->groups[best];
    return set_batch_group(c, out->group);
}

tdda_status tdda_aproduct_noalloc(tdda_core* c, const double* b, double* y) {
    if (!c || !b || !y) {
        set_err("null argument");
        return TDDA_ERR_INVALID_ARGUMENT;
    }
    const size_t need = (size_t)c->g.sb;  // 3 x Nx x My x Mz complex128 entries
    if (need > kNoAllocGridElems) {
        set_err("allocation-free A-product: FFT work grid of %zu complex128 entries exceeds the static "
                "maximum of %zu (64 MiB); use tdda_aproduct",
                need, kNoAllocGridElems);
        return TDDA_ERR_UNSUPPORTED;
    }
    TDDA_TRY(set_device(c->device));
    NoAllocSlot slot;
    TDDA_TRY(noalloc_setup(c->device, &slot));
    RhsVecs<double> v{};
    v.p = (double2*)b;
    v.Ap = (double2*)y;
    TDDA_CK(cudaMemcpyAsync(slot.rhs, &v, sizeof(v), cudaMemcpyHostToDevice, c->stream));
    count_launches(5);
    TDDA_CK(tdda::launch_aproduct<double>(c->g, tdda::SRC_IN, tdda::SNK_OUT, 1, slot.rhs, c->green64, c->tw64[0],
                                          c->tw64[1], c->tw64[2], c->cellmap, slot.grid, c->stream));
    TDDA_CK(cudaStreamSynchronize(c->stream));
    return TDDA_OK;
}

double tdda_request_bytes(int Nx, int Ny, int Nz, int N, int nrhs, int precision) {
    if (Nx < 1 || Ny < 1 || Nz < 1 || N < 1 || nrhs < 1) return 0.0;
    return tdda_session::core_bytes(Nx, Ny, Nz, N, nrhs) + nrhs * tdda_session::model_bytes(N, precision);
}

}  // extern "C"
