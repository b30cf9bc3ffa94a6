// tdda_device.cuh -- device helpers shared by the kernel translation units:
// tile sizes of the pass kernels, FP64 complex scalar arithmetic, the
// deterministic block / grid reductions and the per-RHS early exit.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

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

// Publish this block's partials; the last block of the grid (for this
// right-hand side) sums all partials in block order and returns true in
// every thread of that block, with the totals in tot (valid in thread 0).
template <int NV>
__device__ bool last_block_total(double (&v)[NV], double* part, int nblk, int bid, unsigned int* cnt, double* sred,
                                 double (&tot)[NV]) {
    __shared__ int s_last;
    block_sum<NV>(v, sred);
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

__device__ __forceinline__ bool rhs_done(const SolveState* st) {
    return st != nullptr && *((volatile const int*)&st->status) != ST_RUNNING;
}

template <typename T> __device__ __forceinline__ void stage_tw(cx<T>* stw, const cx<T>* tw, int M) {
    for (int i = threadIdx.x; i < M; i += blockDim.x) stw[i] = tw[i];
}

}  // namespace dev
}  // namespace tdda
