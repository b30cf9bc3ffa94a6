// tdda_device.cuh -- device helpers shared by the kernel translation units:
// tile sizes of the pass kernels, FP64 complex scalar arithmetic, the
// deterministic block / grid reductions and the per-RHS early exit.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <type_traits>

#include "tdda_internal.cuh"

namespace tdda {
namespace dev {

constexpr int kNT = 256;  // threads of every pass and vector kernel

__host__ __device__ constexpr int iclamp(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
__host__ __device__ constexpr int floor_pow2(int v) {
    int p = 1;
    while (p * 2 <= v) p *= 2;
    return p;
}

__host__ __device__ constexpr int pad_odd(int m) { return (m % 2 == 0) ? m + 1 : m; }

// Tiles are sized so that the two ping-pong buffers of a block stay within
// kSmemBudget (two resident blocks per SM at the largest grids).
constexpr int kSmemBudget = 64 * 1024;

// lines of a z-pass tile: 3 components x LZ (x, y) columns, for Mz
template <typename T> __host__ __device__ constexpr int z_lines(int Mz) {
    return iclamp((kSmemBudget - Mz * (int)sizeof(cx<T>)) / (2 * 3 * pad_odd(Mz) * (int)sizeof(cx<T>)), 1, 16);
}
// z-tile of a y-pass, for My
template <typename T> __host__ __device__ constexpr int y_tile(int My) {
    return iclamp(floor_pow2((kSmemBudget - My * (int)sizeof(cx<T>)) / (2 * My * (int)sizeof(cx<T>))), 1, 16);
}
// z-tile of the x-pass (3 components per z), for Mx
template <typename T> __host__ __device__ constexpr int x_tile(int Mx) {
    return iclamp(floor_pow2((kSmemBudget - Mx * (int)sizeof(cx<T>)) / (2 * 3 * Mx * (int)sizeof(cx<T>))), 1, 16);
}
template <typename T> __host__ __device__ constexpr size_t zsmem(int Mz) {
    return sizeof(cx<T>) * (size_t)(Mz + 2 * 3 * z_lines<T>(Mz) * pad_odd(Mz));
}
template <typename T> __host__ __device__ constexpr size_t ysmem(int My) {
    return sizeof(cx<T>) * (size_t)(My + 2 * My * (y_tile<T>(My) + 1));
}
template <typename T> __host__ __device__ constexpr size_t xsmem(int Mx) {
    return sizeof(cx<T>) * (size_t)(Mx + 2 * Mx * (3 * x_tile<T>(Mx) + 1));
}
// lines of a generic row FFT and z-tile of a generic column FFT (FP64)
__host__ __device__ constexpr int row_lines(const AxisPlan& p) {
    return iclamp((kSmemBudget - p.M * 16) / (2 * pad_odd(p.M) * 16), 1, 32);
}
__host__ __device__ constexpr int col_tile(const AxisPlan& p) {
    return iclamp(floor_pow2((kSmemBudget - p.M * 16) / (2 * p.M * 16)), 1, 16);
}

template <typename T> __device__ __forceinline__ cx<T> ld(const cx<T>* p) { return *p; }

__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
    // Smith's algorithm (R. L. Smith, CACM 5(8), 1962)
    if (fabs(b.x) >= fabs(b.y)) {
        double r = b.y / b.x, den = b.x + b.y * r;
        return make_double2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
    }
    double r = b.x / b.y, den = b.x * r + b.y;
    return make_double2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
}
__device__ __forceinline__ double2 dmul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ bool finite2(double2 a) { return isfinite(a.x) && isfinite(a.y); }

template <typename T> __device__ __forceinline__ cx<T> from_d(double2 a) { return mk<T>(T(a.x), T(a.y)); }

// ------------------------------------------------------------ reductions
// Block-wide sum of NV doubles in a fixed order; the result is valid in
// thread 0.  sred must hold NV * blockDim.x doubles.  The partials go through
// shared memory and one warp adds them: on GB300 every FP64 warp instruction
// occupies the narrow FP64 pipe for many cycles, so one warp summing the block
// costs far less than a shuffle tree run by every warp.
template <int NV> __device__ __forceinline__ void block_sum(double (&v)[NV], double* sred) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nt = blockDim.x;
#pragma unroll
    for (int k = 0; k < NV; k++) sred[k * nt + threadIdx.x] = v[k];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
            double a = 0.0;
            for (int i = lane; i < nt; i += 32) a += sred[k * nt + i];
            for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
            v[k] = a;
        }
    }
    __syncthreads();
}

// Accumulator of the per-thread partial sums.  The FP64 kernels add in FP64.
// The FP32 kernels (the inner solve of the mixed form) keep GB300's narrow
// FP64 pipe out of their reductions: each thread adds its few products (at
// most 8 in the vector kernels, at most 24 in the passes) in FP32, and the
// warp, block and grid sums are double-float (hi, lo) pairs of FP32 values
// added with Knuth's TwoSum, about 44 bits.  Every order is fixed, so the
// sums are deterministic.
template <typename T> using acc_t = typename std::conditional<sizeof(T) == 4, float, double>::type;

// (a.x + a.y) + (b.x + b.y) as a double-float pair (TwoSum of the high parts,
// D. E. Knuth, TAOCP vol. 2, 4.2.2; the low parts added; renormalised)
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
    // explicit round-to-nearest operations: no contraction or reassociation
    const float s = __fadd_rn(a.x, b.x);
    const float bp = __fsub_rn(s, a.x);
    const float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bp)), __fsub_rn(b.x, bp));
    const float lo = __fadd_rn(__fadd_rn(e, a.y), b.y);
    const float hi = __fadd_rn(s, lo);
    return make_float2(hi, __fsub_rn(lo, __fsub_rn(hi, s)));
}

// Block sum of double-float values, result in v[] of every thread.  Each
// warp sums its lanes with a shuffle tree, then warp k adds the per-warp sums
// of value k with a second tree (NV <= warps per block), so no thread runs a
// serial loop.  sred must hold 32 * NV float2; the caller puts a barrier
// between two calls on the same sred.
template <int NV> __device__ __forceinline__ void block_sum(float2 (&v)[NV], float2* sred) {
    static_assert(NV <= kNT / 32, "one warp per summed value");
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
        float2 a = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            a = df_add(a, make_float2(__shfl_down_sync(0xffffffffu, a.x, o), __shfl_down_sync(0xffffffffu, a.y, o)));
        if (lane == 0) sred[k * 32 + warp] = a;
    }
    __syncthreads();
    if (warp < NV) {
        float2 a = lane < nw ? sred[warp * 32 + lane] : make_float2(0.f, 0.f);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            a = df_add(a, make_float2(__shfl_down_sync(0xffffffffu, a.x, o), __shfl_down_sync(0xffffffffu, a.y, o)));
        if (lane == 0) sred[warp * 32] = a;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; k++) v[k] = sred[k * 32];
}

// Publish this block's sums (valid in thread 0); the last block of the grid
// (for this right-hand side) sums all partials in block order and returns
// true in every thread of that block, with the totals in tot (valid in
// thread 0).
template <int NV>
__device__ bool publish_total(const double (&v)[NV], double* part, int nblk, int bid, unsigned int* cnt, double* sred,
                              double (&tot)[NV]) {
    __shared__ int s_last;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) part[k * nblk + bid] = v[k];
        __threadfence();
        unsigned int prev = atomicAdd(cnt, 1u);
        s_last = (prev == (unsigned int)(nblk - 1));
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
#pragma unroll
    for (int k = 0; k < NV; k++) {
        double a = 0.0;
        for (int i = threadIdx.x; i < nblk; i += blockDim.x) a += __ldcg(part + k * nblk + i);
        tot[k] = a;
    }
    block_sum<NV>(tot, sred);
    if (threadIdx.x == 0) *cnt = 0u;
    return true;
}

template <int NV>
__device__ bool last_block_total(double (&v)[NV], double* part, int nblk, int bid, unsigned int* cnt, double* sred,
                                 double (&tot)[NV]) {
    block_sum<NV>(v, sred);
    return publish_total<NV>(v, part, nblk, bid, cnt, sred, tot);
}
// FP32 partials: double-float block and grid sums; the partial slots hold one
// float2 (hi, lo) each.  tot: the double-float totals (valid in thread 0).
// sred must hold 32 * NV float2, i.e. 32 * NV doubles (a float2 is 8 bytes).
template <int NV>
__device__ bool last_block_total(float (&v)[NV], double* part, int nblk, int bid, unsigned int* cnt, double* sred,
                                 float2 (&tot)[NV]) {
    __shared__ int s_last;
    float2* sr2 = reinterpret_cast<float2*>(sred);
    float2* part2 = reinterpret_cast<float2*>(part);
#pragma unroll
    for (int k = 0; k < NV; k++) tot[k] = make_float2(v[k], 0.f);
    block_sum<NV>(tot, sr2);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) part2[k * nblk + bid] = tot[k];
        __threadfence();
        unsigned int prev = atomicAdd(cnt, 1u);
        s_last = (prev == (unsigned int)(nblk - 1));
    }
    __syncthreads();
    if (!s_last) return false;
    __threadfence();
#pragma unroll
    for (int k = 0; k < NV; k++) {
        float2 q = make_float2(0.f, 0.f);
        for (int i = threadIdx.x; i < nblk; i += blockDim.x) q = df_add(q, __ldcg(part2 + k * nblk + i));
        tot[k] = q;
    }
    block_sum<NV>(tot, sr2);
    if (threadIdx.x == 0) *cnt = 0u;
    return true;
}

// grid totals of a reduction kernel: FP64, or double-float pairs for FP32
template <typename T> using tot_t = typename std::conditional<sizeof(T) == 4, float2, double>::type;

// Shared scratch of a reduction kernel, in doubles: NV * nt for the FP64
// block sum, 32 * NV float2 (8 bytes each, one per warp slot) for the
// double-float one.
template <typename T, int NV> __host__ __device__ constexpr int sred_size() {
    static_assert(sizeof(float2) == sizeof(double), "a float2 slot is one double");
    return sizeof(T) == 4 ? 32 * NV : NV * kNT;
}

// The end of one BiCGSTAB step, given r0.r and |r|^2 of the new residual
// (DDAModel.cpp:218-255): convergence (not after the initial products,
// DDAModel.cpp:177-182), the iteration limit, breakdown on r0.rl = 0
// (DDAModel.cpp:193-215) and beta for the next step.  Run by one thread.
__device__ __forceinline__ void finish_step(SolveState* st, double2 rho, double rn2, bool is_init) {
    st->rho_prev = st->rho;
    st->rho = rho;
    st->rnorm2 = rn2;
    const double err = sqrt(rn2) / st->Enorm;
    if (!is_init) {
        st->it += 1;
        if (err <= st->tol) {  // DDAModel.cpp:232-235
            st->status = ST_CONVERGED;
            st->iterations = st->it;
            st->error = err;
            return;
        }
    }
    if (st->it >= st->max_it) {  // the loop of DDAModel.cpp:186 ends
        st->status = ST_MAXITER;
        st->error = err;
        return;
    }
    if (st->rho_prev.x == 0.0 && st->rho_prev.y == 0.0) {  // DDAModel.cpp:193-215
        st->status = ST_BREAKDOWN;
        st->iterations = st->it + 1;
        st->error = err;
        return;
    }
    // beta = (alpha / zeta) * (r0 . r) / (r0 . rl)      DDAModel.cpp:218
    st->beta = cdiv(dmul(cdiv(st->alpha, st->zeta), st->rho), st->rho_prev);
    // the reference would iterate on NaN up to the limit; stop and report it
    if (!finite2(st->rho) || !isfinite(err) || !finite2(st->beta)) {
        st->status = ST_NAN;
        st->error = err;
    }
}

// The step end of the deferred-update form (SNK_AT_DEF) from the five sums
// At.t, At.At, r0.t, r0.At, t.t: zeta = At.t / At.At, and for
// r = t - zeta At: r0.r = r0.t - zeta r0.At and
// |r|^2 = t.t - 2 Re(conj(zeta) At.t) + |zeta|^2 At.At.
__device__ __forceinline__ void finish_step_deferred(SolveState* st, const double (&tot)[8]) {
    const double2 Att = make_double2(tot[0], tot[1]);
    const double AtAt = tot[2];
    const double2 r0t = make_double2(tot[3], tot[4]), r0At = make_double2(tot[5], tot[6]);
    const double tt = tot[7];
    const double2 zeta = cdiv(Att, make_double2(AtAt, 0.0));  // DDAModel.cpp:225
    st->zeta = zeta;
    const double2 zr = dmul(zeta, r0At);
    const double2 rho = make_double2(r0t.x - zr.x, r0t.y - zr.y);
    double rn2 = tt - 2.0 * (zeta.x * Att.x + zeta.y * Att.y) + (zeta.x * zeta.x + zeta.y * zeta.y) * AtAt;
    if (!(rn2 > 0.0)) rn2 = isnan(rn2) ? rn2 : 0.0;
    const bool init = st->init != 0;
    st->init = 0;
    st->pending = 1;
    finish_step(st, rho, rn2, init);
}

// The FP32 inner solve forms its step scalars in FP32 from the hi parts of
// the double-float totals (its kernels use them in FP32), and keeps them in
// the FP32 fields of the state; nothing on its critical path touches the
// FP64 pipe.
__device__ __forceinline__ float2 fmul2(float2 a, float2 b) { return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ float2 fdiv2(float2 a, float2 b) {
    // Smith's algorithm (R. L. Smith, CACM 5(8), 1962)
    if (fabsf(b.x) >= fabsf(b.y)) {
        const float r = b.y / b.x, den = b.x + b.y * r;
        return make_float2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
    }
    const float r = b.x / b.y, den = b.x * r + b.y;
    return make_float2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
}

// ---- the FP32 deferred step, formed by the consuming kernels ---------------
// The sink passes of an FP32 step only publish block partials (publish_partials).
// Every block of the next gather sums them (sum_partials) and forms the step
// scalars itself; block 0 records them in the state slot of the step.

// Block partials as double-float pairs into part slots k * nblk + bid (thread 0).
template <int NV>
__device__ __forceinline__ void publish_partials(float (&v)[NV], double* part, int nblk, int bid, double* sred) {
    float2 a[NV];
#pragma unroll
    for (int k = 0; k < NV; k++) a[k] = make_float2(v[k], 0.f);
    block_sum<NV>(a, reinterpret_cast<float2*>(sred));
    if (threadIdx.x == 0) {
        float2* part2 = reinterpret_cast<float2*>(part);
#pragma unroll
        for (int k = 0; k < NV; k++) part2[k * nblk + bid] = a[k];
    }
}

// The totals of nblk published partials (every thread).  Warp k adds value k:
// lane l takes the partials l, l + 32, ... (loads issued eight at a time), then
// a shuffle tree; one barrier.  The order is fixed.  sred: NV float2 of shared
// scratch.
template <int NV>
__device__ __forceinline__ void sum_partials(const double* part, int nblk, float2* sred, float2 (&tot)[NV]) {
    static_assert(NV <= kNT / 32, "one warp per summed value");
    const float2* part2 = reinterpret_cast<const float2*>(part);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (warp < NV) {
        const float2* src = part2 + (long long)warp * nblk;
        float2 a = make_float2(0.f, 0.f);
        for (int i0 = lane; i0 < nblk; i0 += 32 * 8) {
            float2 v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) v[u] = i0 + 32 * u < nblk ? __ldcg(src + i0 + 32 * u) : make_float2(0.f, 0.f);
#pragma unroll
            for (int u = 0; u < 8; u++) a = df_add(a, v[u]);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            a = df_add(a, make_float2(__shfl_down_sync(0xffffffffu, a.x, o), __shfl_down_sync(0xffffffffu, a.y, o)));
        if (lane == 0) sred[warp] = a;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; k++) tot[k] = sred[k];
}

// The state fields the end of step k - 1 reads, loaded together ahead of the
// partial sums (one round trip instead of a chain of dependent ones).
struct StepIn {
    float2 alpha, rho;  // alpha and r0.r of step k - 1
    int it, init, status, max_it;
    float Enorm, tol;
};
__device__ __forceinline__ StepIn load_step_in(const SolveState* st, int p) {
    const int q = p ^ 1;
    StepIn s;
    s.alpha = st->alpha32[q];
    s.rho = st->rho32[q];
    s.it = st->it32[q];
    s.init = st->init32[q];
    s.status = st->status;
    s.max_it = st->max_it;
    s.Enorm = st->Enorm32;
    s.tol = st->tol32;
    return s;
}

// The end of step k - 1 as seen by step k (parity p): zeta = At.t / At.At in
// FP32; r0.r and |r|^2 of r = t - zeta At as FP64 multiply-adds on the
// double-float totals (they cancel as r gets small next to t); then the
// logic of DDAModel.cpp:218-255: convergence (not after the initial
// products), the iteration limit, breakdown on r0.rl = 0, beta.
struct StepEnd {
    float2 zeta, rho, beta;
    float err;
    int it, stop, set_iterations, iterations;
};
__device__ __forceinline__ double df_d(float2 a) { return (double)a.x + (double)a.y; }
__device__ __forceinline__ StepEnd step_end_f32(const StepIn& st, const float2 (&tot)[8]) {
    StepEnd e;
    e.zeta = fdiv2(make_float2(tot[0].x, tot[1].x), make_float2(tot[2].x, 0.f));  // DDAModel.cpp:225
    const double zx = e.zeta.x, zy = e.zeta.y;
    const double ax = df_d(tot[0]), ay = df_d(tot[1]), bb = df_d(tot[2]);
    const double tx = df_d(tot[3]), ty = df_d(tot[4]), ux = df_d(tot[5]), uy = df_d(tot[6]), cc = df_d(tot[7]);
    e.rho = make_float2((float)(tx - (zx * ux - zy * uy)), (float)(ty - (zx * uy + zy * ux)));
    double rn2 = cc - 2.0 * (zx * ax + zy * ay) + (zx * zx + zy * zy) * bb;
    if (!(rn2 > 0.0)) rn2 = isnan(rn2) ? rn2 : 0.0;
    e.err = sqrtf((float)rn2) / st.Enorm;
    const bool init = st.init != 0;
    e.it = st.it + (init ? 0 : 1);
    e.stop = ST_RUNNING;
    e.set_iterations = 0;
    e.iterations = 0;
    e.beta = make_float2(0.f, 0.f);
    const float2 rho_prev = st.rho;
    if (!init && e.err <= st.tol) {  // DDAModel.cpp:232-235
        e.stop = ST_CONVERGED;
        e.set_iterations = 1;
        e.iterations = e.it;
    } else if (e.it >= st.max_it) {  // the loop of DDAModel.cpp:186 ends
        e.stop = ST_MAXITER;
    } else if (rho_prev.x == 0.f && rho_prev.y == 0.f) {  // DDAModel.cpp:193-215
        e.stop = ST_BREAKDOWN;
        e.set_iterations = 1;
        e.iterations = e.it + 1;
    } else {
        // beta = (alpha / zeta) * (r0 . r) / (r0 . rl)      DDAModel.cpp:218
        e.beta = fdiv2(fmul2(fdiv2(st.alpha, e.zeta), e.rho), rho_prev);
        if (!isfinite(e.rho.x) || !isfinite(e.rho.y) || !isfinite(e.err) || !isfinite(e.beta.x) ||
            !isfinite(e.beta.y))
            e.stop = ST_NAN;
    }
    return e;
}
// records step_end_f32's result (one thread of one block)
__device__ __forceinline__ void write_step_end(SolveState* st, const StepEnd& e, int p) {
    const int q = p ^ 1;
    st->zeta32[q] = e.zeta;
    st->rho32[p] = e.rho;
    st->beta32[p] = e.beta;
    st->it32[p] = e.it;
    st->init32[p] = 0;
    st->it = e.it;
    if (e.stop != ST_RUNNING) {
        st->status = e.stop;
        st->error = e.err;
        st->last_slot = q;
        if (e.set_iterations) st->iterations = e.iterations;
    }
}

// The scalars a sink pass forms from its grid totals (thread 0 of the last block).
template <typename T, int SNK, int NV> __device__ __forceinline__ void finalize_sink(SolveState* st, const tot_t<T> (&tot)[NV]) {
    if constexpr (sizeof(T) == 4) {
        // the FP32 step forms its scalars in the consuming kernels; the initial
        // residual r0.r seeds slot 1 (the initial products are step -1)
        if constexpr (SNK == SNK_RES) st->rho32[1] = make_float2(tot[0].x, 0.f);
    } else {
        if constexpr (SNK == SNK_RES) {
            st->rho = make_double2(tot[0], 0.0);  // r0 . r with r0 = r
            st->rnorm2 = tot[0];
        } else if constexpr (SNK == SNK_AT_DEF) {
            finish_step_deferred(st, tot);
        } else if constexpr (SNK == SNK_AP) {
            st->alpha = cdiv(st->rho, make_double2(tot[0], tot[1]));  // DDAModel.cpp:221
        } else if constexpr (SNK == SNK_AT) {
            st->zeta = cdiv(make_double2(tot[0], tot[1]), make_double2(tot[2], 0.0));  // DDAModel.cpp:225
        }
    }
}

// step scalars as the kernels of precision T use them
template <typename T> __device__ __forceinline__ cx<T> st_alpha(const SolveState* s, int slot = 0) {
    if constexpr (sizeof(T) == 4) return s->alpha32[slot]; else return s->alpha;
}
template <typename T> __device__ __forceinline__ cx<T> st_beta(const SolveState* s, int slot = 0) {
    if constexpr (sizeof(T) == 4) return s->beta32[slot]; else return s->beta;
}
template <typename T> __device__ __forceinline__ cx<T> st_zeta(const SolveState* s, int slot = 0) {
    if constexpr (sizeof(T) == 4) return s->zeta32[slot]; else return s->zeta;
}

__device__ __forceinline__ bool rhs_done(const SolveState* st) {
    return st != nullptr && *((volatile const int*)&st->status) != ST_RUNNING;
}

// Programmatic dependent launch (launch_early): grid_dep_wait() returns once the
// previous kernel of the stream has completed and its writes are visible;
// grid_dep_release() lets the stream's next kernel start launching its blocks
// (they wait in their own grid_dep_wait).  Both do nothing in a kernel launched
// the ordinary way.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename T> __device__ __forceinline__ void stage_tw(cx<T>* stw, const cx<T>* tw, int M) {
    for (int i = threadIdx.x; i < M; i += blockDim.x) stw[i] = tw[i];
}

}  // namespace dev
}  // namespace tdda
