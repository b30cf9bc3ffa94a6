// tdda_fft_ct.cuh -- the shared-memory Stockham FFT with a compile-time plan.
//
// Same algorithm as smem_fft() in tdda_fft.cuh (radix stages, ping-pong
// buffers, one barrier per stage), but the length M, the radix sequence, the
// number of lines L, their strides and the thread count NT are template
// constants: every index, twiddle step and loop trip count folds at compile
// time and the per-thread butterfly loops unroll.  The pass kernels use it for
// the axis lengths of the common lattices and fall back to the runtime plan
// otherwise.
#pragma once

#include "tdda_fft.cuh"

namespace tdda {

// radix plan: the host's make_plan() (8s and 4s, no lone 2 unless the power
// of two is 2, then 3, 5, 7).  With big set (the FP32 passes, latency-bound)
// some lengths take a two-stage plan of larger in-register radices, which
// needs fewer shared-memory passes; the FP64 passes, bound by the FP64 pipe,
// keep the plan with the fewest multiplications.
__host__ __device__ constexpr int ct_nrad(int M, int which, bool big = false) {
    if (big && M == 128) return which < 0 ? 2 : (which == 0 ? 16 : 8);
    if (big && M == 192) return which < 0 ? 2 : (which == 0 ? 16 : 12);
    if (big && M == 160) return which < 0 ? 2 : (which == 0 ? 16 : 10);
    if (big && M == 48) return which < 0 ? 2 : (which == 0 ? 16 : 3);
    if (big && M == 56) return which < 0 ? 2 : (which == 0 ? 8 : 7);
    if (big && M == 80) return which < 0 ? 2 : (which == 0 ? 16 : 5);
    if (big && M == 112) return which < 0 ? 2 : (which == 0 ? 16 : 7);
    if (big && M == 96) return which < 0 ? 2 : (which == 0 ? 12 : 8);
    int m = M, a = 0;
    while (m % 2 == 0) { m /= 2; a++; }
    int r[16] = {};
    int n = 0;
    while (a >= 3 && a != 4) { r[n++] = 8; a -= 3; }
    while (a >= 2) { r[n++] = 4; a -= 2; }
    if (a == 1) r[n++] = 2;
    while (m % 3 == 0) { r[n++] = 3; m /= 3; }
    while (m % 5 == 0) { r[n++] = 5; m /= 5; }
    while (m % 7 == 0) { r[n++] = 7; m /= 7; }
    return which < 0 ? n : r[which];
}
__host__ __device__ constexpr int ct_nstages(int M, bool big) { return ct_nrad(M, -1, big); }
// The two-stage plan of the register-form x pass, M = R1 R2: the FP32 plan,
// except 192 = 24 x 8.  Its first and last stages have 3 ZT R2 tasks for ZT R1
// threads, one each when R1 = 3 R2, and the spectra of its second stage take
// 3 R2 complex registers.
__host__ __device__ constexpr int x2_radix(int M, int which) {
    if (M == 192) return which == 0 ? 24 : 8;
    return ct_nrad(M, which, true);
}
__host__ __device__ constexpr int ct_radix(int M, int st, bool big) { return ct_nrad(M, st, big); }

// PIN (first stage only): the inputs idx >= M / 2 are zero padding (nvalid
// <= M / 2), so the butterfly inputs r >= (R + 1) / 2 are neither read nor
// added.  POUT (last stage only): outputs idx >= M / 2 are never stored (nout
// <= M / 2), so the butterfly outputs q >= (R + 1) / 2 are not formed.
template <int R, int SIGN, typename T, int M, int NS, int L, int LS, int MS, int NT, bool PIN, bool POUT>
__device__ __forceinline__ void ct_stage(const cx<T>* __restrict__ x, cx<T>* __restrict__ y, const cx<T>* tw,
                                         int nvalid, int nout) {
    constexpr int m = M / R;
    constexpr int nb = L * m;
    constexpr int twstep = M / (NS * R);
    static_assert(!PIN || NS == 1, "input pruning on the first stage");
    static_assert(!POUT || NS * R == M, "output pruning on the last stage");
    constexpr int RIN = PIN ? (R + 1) / 2 : R;
    constexpr int ROUT = POUT ? (R + 1) / 2 : R;
#pragma unroll 4
    for (int w = threadIdx.x; w < nb; w += NT) {
        const int j = w / L;
        const int l = w - j * L;
        const cx<T>* xb = x + l * LS;
        cx<T> v[R];
#pragma unroll
        for (int r = 0; r < RIN; r++) {
            const int idx = j + r * m;
            v[r] = idx < nvalid ? xb[idx * MS] : czero<T>();
        }
        const int k = j % NS;
        if (NS > 1) {
#pragma unroll
            for (int r = 1; r < R; r++) {
                cx<T> t = tw[r * k * twstep];
                if (SIGN > 0) t.y = -t.y;
                v[r] = cmul<T>(v[r], t);
            }
        }
        BflyIn<R, SIGN, T, RIN>::run(v);
        cx<T>* yb = y + l * LS;
        const int ob = (j - k) * R + k;
#pragma unroll
        for (int q = 0; q < ROUT; q++) {
            const int idx = ob + q * NS;
            if (idx < nout) yb[idx * MS] = v[q];
        }
    }
    __syncthreads();
}

// HIN: nvalid <= M / 2 (a zero-padded forward input); HOUT: nout <= M / 2 (an
// inverse whose upper half is discarded).  M even for either.
template <int SIGN, typename T, int M, int L, int LS, int MS, int NT, bool HIN = false, bool HOUT = false, int ST = 0,
          int NS = 1>
__device__ __forceinline__ cx<T>* ct_fft(cx<T>* a, cx<T>* b, const cx<T>* tw, int nvalid, int nout) {
    constexpr bool big = sizeof(T) == 4;
    static_assert(!(HIN || HOUT) || M % 2 == 0, "halving needs an even length");
    if constexpr (ST == ct_nstages(M, big)) {
        return a;
    } else {
        constexpr int R = ct_radix(M, ST, big);
        constexpr bool last = ST == ct_nstages(M, big) - 1;
        ct_stage<R, SIGN, T, M, NS, L, LS, MS, NT, HIN && ST == 0, HOUT && last>(a, b, tw, ST == 0 ? nvalid : M,
                                                                                 last ? nout : M);
        return ct_fft<SIGN, T, M, L, LS, MS, NT, HIN, HOUT, ST + 1, NS * R>(b, a, tw, nvalid, nout);
    }
}

}  // namespace tdda
