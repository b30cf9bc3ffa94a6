// tdda_kernels.cu -- sm_103a kernels of the DDA solve path.
//
//   K0  green      LDR tensor on the padded grid (AProductCore.cpp:53-194,
//                  588-623), forward 3-D FFT, fold to the octant, scale 1/M
//   K1  zfwd       gather the dipole vector onto the grid (+ the fused
//                  BiCGSTAB vector update), z-axis forward FFT, pruned input
//   K2  ypass      y-axis forward FFT over the x < Nx planes, pruned input
//   K3  xpass      x-axis forward FFT, symmetric 3x3 spectral product with
//                  the six Green components (kernel.cu:74-85), inverse x FFT,
//                  pruned output
//   K4  ypass      y-axis inverse FFT, pruned output
//   K5  zinv       z-axis inverse FFT, pruned output, scatter to dipoles,
//                  + al*v and the fused dot products of the solver
//   K6  update     BiCGSTAB vector update and dots (DDAModel.cpp:225-232)
// The pass structure replaces the reference's host scatter, H2D copy, six
// cuFFT calls, three element-wise kernels and D2H copy per product
// (AProductCore.cpp:697-758).  All reductions are deterministic: fixed
// per-block trees and a fixed-order sum of block partials by the last block.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include <algorithm>

#include "tdda_device.cuh"
#include "tdda_tensor.cuh"

namespace tdda {

namespace {

using namespace dev;
// ================================================================ K6 update
template <typename T>
__global__ void __launch_bounds__(kNT) k_update(int n3, const RhsVecs<T>* __restrict__ rhs, int is_init) {
    static_assert(sizeof(T) == 8, "the FP32 step is the deferred form");
    __shared__ double sred[sred_size<T, 4>()];
    const int b = blockIdx.y;
    const RhsVecs<T> R = rhs[b];
    if (rhs_done(R.st)) return;
    const cx<T> alpha = st_alpha<T>(R.st), zeta = st_zeta<T>(R.st);
    acc_t<T> acc[4] = {0, 0, 0, 0};
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n3; e += gridDim.x * blockDim.x) {
        const cx<T> Ap = R.Ap[e], r = R.r[e], p = R.p[e], t = R.t[e], At = R.At[e], r0 = R.r0[e];
        cx<T> P = R.P[e];
        const cx<T> u = cmul<T>(zeta, Ap);                              // u = zeta Ap
        const cx<T> z = csub<T>(cmul<T>(zeta, r), cmul<T>(alpha, u));  // z = zeta r - alpha u
        P = cadd<T>(cadd<T>(P, cmul<T>(alpha, p)), z);                 // P = P + alpha p + z
        const cx<T> rn = csub<T>(t, cmul<T>(zeta, At));                // r = t - zeta At
        R.u[e] = u;
        R.P[e] = P;
        R.r[e] = rn;
        acc[0] += r0.x * rn.x + r0.y * rn.y;
        acc[1] += r0.x * rn.y - r0.y * rn.x;
        acc[2] += rn.x * rn.x + rn.y * rn.y;
    }
    tot_t<T> tot[4];
    if (!last_block_total<4>(acc, R.part, gridDim.x, blockIdx.x, R.cnt + 3, sred, tot)) return;
    if (threadIdx.x != 0) return;
    finish_step(R.st, make_double2(tot[0], tot[1]), tot[2], is_init != 0);
}

// The deferred update of the last step (SNK_AT_DEF) for every right-hand side
// that has one pending: u = zeta Ap; P += alpha p + zeta r - alpha u;
// r = t - zeta At.
template <typename T>
__global__ void __launch_bounds__(kNT) k_finish(int n3, int multi, const RhsVecs<T>* __restrict__ rhs) {
    const RhsVecs<T> R = rhs[blockIdx.y];
    if (R.st == nullptr) return;
    if (multi) n3 = 3 * R.N;  // a cross-lattice batch: this right-hand side's dipoles
    cx<T> alpha, zeta;
    if constexpr (sizeof(T) == 4) {
        const int q = R.st->last_slot;  // the step whose update is pending
        if (q < 0) return;
        alpha = R.st->alpha32[q];
        zeta = R.st->zeta32[q];
    } else {
        if (!R.st->pending) return;
        alpha = R.st->alpha;
        zeta = R.st->zeta;
    }
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n3; e += gridDim.x * blockDim.x) {
        const cx<T> u = cmul<T>(zeta, R.Ap[e]);
        const cx<T> r = R.r[e];
        const cx<T> z = csub<T>(cmul<T>(zeta, r), cmul<T>(alpha, u));
        R.P[e] = cadd<T>(cadd<T>(R.P[e], cmul<T>(alpha, R.p[e])), z);
        R.r[e] = csub<T>(R.t[e], cmul<T>(zeta, R.At[e]));
    }
}

// |E| of each right-hand side
template <typename T>
__global__ void __launch_bounds__(kNT) k_solve_begin(int n3, int multi, const RhsVecs<T>* __restrict__ rhs,
                                                     int resid_is_rhs) {
    __shared__ double sred[sred_size<T, 4>()];
    const int b = blockIdx.y;
    const RhsVecs<T> R = rhs[b];
    if (rhs_done(R.st)) return;
    if (multi) n3 = 3 * R.N;  // a cross-lattice batch: this right-hand side's dipoles
    acc_t<T> acc[4] = {0, 0, 0, 0};
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n3; e += gridDim.x * blockDim.x) {
        const cx<T> v = R.E[e];
        acc[0] += v.x * v.x + v.y * v.y;
        if (resid_is_rhs) {
            R.r[e] = v;
            R.r0[e] = v;
            R.p[e] = v;
        }
    }
    tot_t<T> tot[4];
    if (!last_block_total<4>(acc, R.part, gridDim.x, blockIdx.x, R.cnt + 4, sred, tot)) return;
    if (threadIdx.x != 0) return;
    if constexpr (sizeof(T) == 4) {
        R.st->Enorm32 = sqrtf(tot[0].x);
        if (resid_is_rhs) R.st->rho32[1] = make_float2(tot[0].x, 0.f);  // r0.r of the initial products (step -1)
    } else {
        R.st->Enorm = sqrt(tot[0]);
        if (resid_is_rhs) {
            R.st->rho = make_double2(tot[0], 0.0);
            R.st->rnorm2 = tot[0];
        }
    }
}

// The end of a chunk of FP32 steps: for each right-hand side the step end
// before the step of parity `slot`, from the At-pass partials (the computation
// every block of the next gather repeats, so the state the host reads after
// the loop is current), then the condition of the device-side loop.  One block.
__global__ void __launch_bounds__(kNT) k_chunk_end(const RhsVecs<float>* __restrict__ rhs, int nrhs, int slot,
                                                   int prod_nblk, cudaGraphConditionalHandle loop, int in_loop) {
    __shared__ float2 sred[8];
    __shared__ int s_running;
    grid_dep_wait();  // the partials and states are the previous kernel's
    if (threadIdx.x == 0) s_running = 0;
    for (int b = 0; b < nrhs; b++) {
        const RhsVecs<float> R = rhs[b];
        StepIn in;
        if (threadIdx.x == 0) in = load_step_in(R.st, slot);
        float2 tot[8];
        sum_partials<8>(R.part, prod_nblk, sred, tot);
        if (threadIdx.x == 0 && in.status == ST_RUNNING) {
            const StepEnd e = step_end_f32(in, tot);
            write_step_end(R.st, e, slot);
            if (e.stop == ST_RUNNING) s_running = 1;
        }
        __syncthreads();  // sred is reused for the next right-hand side
    }
    if (threadIdx.x == 0) {
        SolveState* st0 = rhs[0].st;
        const int chunks = st0->chunks + 1;
        st0->chunks = chunks;
        // another chunk inside this launch, unless the launch has run its
        // kLoopChunks (the host then reads the states and launches again)
        const bool more = s_running && chunks < st0->chunk_limit && chunks % kLoopChunks != 0;
        if (in_loop) cudaGraphSetConditional(loop, more ? 1u : 0u);
    }
}

// ================================================================ K0 green

// ================================================================ field at points
// E(r_p) = E_ext(r_p) - sum_i A(r_p - d R_i) P_i (ObjDDAModel.cpp:42-96,
// DDAModel.cpp:530-565), FP64.  Pass 1: block (b, p) sums the dipoles
// i = b*nt + t, b*nt + t + gridDim.x*nt, ... for point p in a fixed order and
// writes its three complex partials; pass 2 adds the nb partials of each point
// in block order and subtracts them from the incident field.
__global__ void __launch_bounds__(kNT) k_field_partial(int N, const int* __restrict__ R, double d, double K,
                                                       Interaction it, const double2* __restrict__ P,
                                                       const double* __restrict__ pts, double2* __restrict__ part) {
    __shared__ double sred[6 * kNT];
    const int p = blockIdx.y;
    const double x = pts[3 * p], y = pts[3 * p + 1], z = pts[3 * p + 2];
    double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        double2 t[6];
        interaction_tensor(it, K, d, x - d * R[3 * i], y - d * R[3 * i + 1], z - d * R[3 * i + 2], t);
        const double2 px = P[3 * i], py = P[3 * i + 1], pz = P[3 * i + 2];
        const double2 s0 = dmul(t[0], px), s1 = dmul(t[1], py), s2 = dmul(t[2], pz);
        const double2 u0 = dmul(t[1], px), u1 = dmul(t[3], py), u2 = dmul(t[4], pz);
        const double2 w0 = dmul(t[2], px), w1 = dmul(t[4], py), w2 = dmul(t[5], pz);
        acc[0] += s0.x + s1.x + s2.x;
        acc[1] += s0.y + s1.y + s2.y;
        acc[2] += u0.x + u1.x + u2.x;
        acc[3] += u0.y + u1.y + u2.y;
        acc[4] += w0.x + w1.x + w2.x;
        acc[5] += w0.y + w1.y + w2.y;
    }
    block_sum<6>(acc, sred);
    if (threadIdx.x == 0) {
        double2* o = part + ((long long)p * gridDim.x + blockIdx.x) * 3;
        o[0] = make_double2(acc[0], acc[1]);
        o[1] = make_double2(acc[2], acc[3]);
        o[2] = make_double2(acc[4], acc[5]);
    }
}

__global__ void k_field_sum(int npts, int nb, const double2* __restrict__ part, const double* __restrict__ pts,
                            double3 nK, double3 nE0, double E0, double K, double2* __restrict__ E) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    double sn, cs;
    sincos(K * (nK.x * pts[3 * p] + nK.y * pts[3 * p + 1] + nK.z * pts[3 * p + 2]), &sn, &cs);
    const double amp[3] = {E0 * nE0.x, E0 * nE0.y, E0 * nE0.z};
    for (int j = 0; j < 3; j++) {
        double2 s = make_double2(0.0, 0.0);
        for (int b = 0; b < nb; b++) {
            const double2 v = part[((long long)p * nb + b) * 3 + j];
            s.x += v.x;
            s.y += v.y;
        }
        E[3 * p + j] = make_double2(amp[j] * cs - s.x, amp[j] * sn - s.y);
    }
}

// Periodic lattice (AProductCore.cpp:251-536): the tensor at offset o is the
// sum over the images (m, n) of LDR(o d + (m Lm, n Ln, 0)), each damped by
// exp(-(gamma K r)^4), gamma = 0.01 (AProductCore.cpp:573-586).  The image sum
// is symmetric in m and n, so every component keeps the parity of the
// free-space tensor and the octant o >= 0 determines the rest.  One block
// per octant offset sums the (2 MAXm + 1)(2 MAXn + 1) images in a fixed order.
__global__ void __launch_bounds__(kNT) k_green_periodic_octant(Geom g, double K, double d, PeriodicImages pi,
                                                               Interaction it, double2* __restrict__ oct) {
    __shared__ double sred[12 * kNT];
    const int o = blockIdx.x;  // (ox Ny + oy) Nz + oz
    const int oz = o % g.Nz, oy = (o / g.Nz) % g.Ny, ox = o / (g.Nz * g.Ny);
    const int nm = 2 * pi.MAXm + 1, nimg = nm * (2 * pi.MAXn + 1);
    double acc[12];
#pragma unroll
    for (int l = 0; l < 12; l++) acc[l] = 0.0;
    for (int q = threadIdx.x; q < nimg; q += blockDim.x) {
        const int m = q % nm - pi.MAXm, n = q / nm - pi.MAXn;
        const double x = d * ox + m * pi.Lm, y = d * oy + n * pi.Ln, z = d * oz;
        double2 t[6];
        interaction_tensor(it, K, d, x, y, z, t);
        const double gk = 0.01 * K * sqrt(x * x + y * y + z * z);
        const double g2 = gk * gk;
        const double ph = exp(-(g2 * g2));
#pragma unroll
        for (int l = 0; l < 6; l++) {
            acc[2 * l] += t[l].x * ph;
            acc[2 * l + 1] += t[l].y * ph;
        }
    }
    block_sum<12>(acc, sred);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int l = 0; l < 6; l++) oct[(long long)o * 6 + l] = make_double2(acc[2 * l], acc[2 * l + 1]);
    }
}

// the full padded grid from the octant: xx, yy, zz even in every axis; xy odd
// in x and y, xz in x and z, yz in y and z
// The tensor at the octant of lattice offsets (0 <= o < N on each axis), one
// thread per offset: every other offset differs only by the sign of the odd
// components (xy odd in x and y, xz in x and z, yz in y and z), which
// k_green_expand applies, so the FP64 tensor is evaluated Nx Ny Nz times
// instead of once per grid point.
__global__ void k_green_octant(Geom g, double K, double d, Interaction it, double2* __restrict__ oct) {
    const long long n = (long long)g.Nx * g.Ny * g.Nz;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const int oz = (int)(e % g.Nz);
        const int oy = (int)((e / g.Nz) % g.Ny);
        const int ox = (int)(e / ((long long)g.Nz * g.Ny));
        double2 t[6];
        interaction_tensor(it, K, d, d * ox, d * oy, d * oz, t);
#pragma unroll
        for (int l = 0; l < 6; l++) oct[e * 6 + l] = t[l];
    }
}
__global__ void k_green_expand(Geom g, const double2* __restrict__ oct, double2* __restrict__ full6) {
    const int Mx = g.px.M, My = g.py.M, Mz = g.pz.M;
    const long long M = (long long)Mx * My * Mz;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < M; e += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(e % Mz);
        const int j = (int)((e / Mz) % My);
        const int i = (int)(e / ((long long)Mz * My));
        int ox = i < g.Nx ? i : (i > Mx - g.Nx ? i - Mx : INT32_MIN);
        int oy = j < g.Ny ? j : (j > My - g.Ny ? j - My : INT32_MIN);
        int oz = k < g.Nz ? k : (k > Mz - g.Nz ? k - Mz : INT32_MIN);
        double2 t[6];
        if (ox != INT32_MIN && oy != INT32_MIN && oz != INT32_MIN) {
            const double sx = ox < 0 ? -1.0 : 1.0, sy = oy < 0 ? -1.0 : 1.0, sz = oz < 0 ? -1.0 : 1.0;
            const double2* src = oct + (((long long)abs(ox) * g.Ny + abs(oy)) * g.Nz + abs(oz)) * 6;
            const double sg[6] = {1.0, sx * sy, sx * sz, 1.0, sy * sz, 1.0};
#pragma unroll
            for (int l = 0; l < 6; l++) t[l] = make_double2(sg[l] * src[l].x, sg[l] * src[l].y);
        } else {
#pragma unroll
            for (int l = 0; l < 6; l++) t[l] = make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int l = 0; l < 6; l++) full6[l * M + e] = t[l];
    }
}

// the Si/Ci tables of the FCD tensor: Si(0.1 k), Ci(0.1 k), k = 1 .. kSiCiN
__global__ void k_sici_table(double* __restrict__ si, double* __restrict__ ci) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < kSiCiN; k += gridDim.x * blockDim.x)
        sici(kSiCiDis * (k + 1), &si[k], &ci[k]);
}

// fold the spectrum to the octant, scale by 1/M, write FP64 and FP32 copies
__global__ void k_green_fold(Geom g, const double2* __restrict__ full6, double2* __restrict__ green64,
                             float2* __restrict__ green32) {
    const int Mx = g.px.M, My = g.py.M, Mz = g.pz.M;
    const long long M = (long long)Mx * My * Mz;
    const long long H = (long long)g.Hx * g.Hy * g.Hz;
    const double inv = 1.0 / (double)M;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < H * 6; e += (long long)gridDim.x * blockDim.x) {
        const int l = (int)(e % 6);
        const long long q = e / 6;
        const int fz = (int)(q % g.Hz);
        const int fx = (int)((q / g.Hz) % g.Hx);
        const int fy = (int)(q / ((long long)g.Hx * g.Hz));
        const double2 v = full6[l * M + ((long long)fx * My + fy) * Mz + fz];
        const double2 w = make_double2(v.x * inv, v.y * inv);
        green64[e] = w;
        // FP32: planes of component pairs, [fy][fx][l / 2][fz][l % 2]
        green32[((((long long)fy * g.Hx + fx) * 3 + l / 2) * g.Hz + fz) * 2 + (l & 1)] =
            make_float2((float)w.x, (float)w.y);
    }
}

// ------------------------------------------------------- generic FFT passes
// rows: nrows contiguous lines of length M
// nout: outputs m >= nout are neither formed in the last stage nor stored (the
// Green spectrum keeps only the octant k <= M / 2 of each axis)
__global__ void __launch_bounds__(kNT) k_fft_rows(double2* __restrict__ data, long long nrows, AxisPlan p,
                                                  const double2* __restrict__ tw, int sign, int nout) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int M = p.M;
    const int L = row_lines(p);
    const int MP = pad_odd(M);
    double2* stw = reinterpret_cast<double2*>(smem_raw);
    double2* s = stw + M;
    double2* s2 = s + L * MP;
    stage_tw<double>(stw, tw, M);
    const long long r0 = (long long)blockIdx.x * L;
    const int nl = (int)min((long long)L, nrows - r0);
    for (int e = threadIdx.x; e < nl * M; e += blockDim.x) {
        const int line = e / M, m = e - (e / M) * M;
        s[line * MP + m] = data[(r0 + line) * M + m];
    }
    __syncthreads();
    const double2* res = sign < 0 ? smem_fft<-1, double>(s, s2, L, MP, 1, p, stw, M, nout)
                                  : smem_fft<+1, double>(s, s2, L, MP, 1, p, stw, M, nout);
    for (int e = threadIdx.x; e < nl * M; e += blockDim.x) {
        const int line = e / M, m = e - (e / M) * M;
        if (m < nout) data[(r0 + line) * M + m] = res[line * MP + m];
    }
}

// columns: element m of line (o, t) at off(o) + t + m*ms, t in [0, ninner)
// contiguous; off(o) = (o / o1) * s1 + (o % o1) * s2
__global__ void __launch_bounds__(kNT) k_fft_cols(double2* __restrict__ data, int nouter, int o1, long long s1,
                                                  long long s2, long long ms, int ninner, AxisPlan p,
                                                  const double2* __restrict__ tw, int sign, int nout) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int M = p.M;
    const int ZT = col_tile(p);
    const int nt = (ninner + ZT - 1) / ZT;
    const int o = blockIdx.x / nt, t0 = (blockIdx.x - o * nt) * ZT;
    const int zn = min(ZT, ninner - t0);
    double2* stw = reinterpret_cast<double2*>(smem_raw);
    double2* s = stw + M;
    double2* sb2 = s + M * ZT;
    stage_tw<double>(stw, tw, M);
    double2* base = data + (long long)(o / o1) * s1 + (long long)(o % o1) * s2 + t0;
    for (int e = threadIdx.x; e < M * ZT; e += blockDim.x) {
        const int m = e / ZT, zl = e - (e / ZT) * ZT;
        s[e] = zl < zn ? base[m * ms + zl] : make_double2(0.0, 0.0);
    }
    __syncthreads();
    const double2* res = sign < 0 ? smem_fft<-1, double>(s, sb2, ZT, 1, ZT, p, stw, M, nout)
                                  : smem_fft<+1, double>(s, sb2, ZT, 1, ZT, p, stw, M, nout);
    for (int e = threadIdx.x; e < nout * ZT; e += blockDim.x) {
        const int m = e / ZT, zl = e - (e / ZT) * ZT;
        if (zl < zn) base[m * ms + zl] = res[e];
    }
}

// ------------------------------------------------------------ polarisability
__device__ __forceinline__ double2 dadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 dscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }

// eps and al = 1 / alpha_LDR(eps) of one density (DDAModel.cpp:54-63, tools.cpp:617-630)
__device__ __forceinline__ void model_alpha_one(double v, const AlphaParams& ap, double2& eps, double2& inv) {
    const double b1 = -1.891531, b2 = 0.1648469, b3 = -1.7700004;  // LDR coefficients (tools.cpp:618-620)
    int lf = (int)floor(v);
    int ln = lf + 1;
    if (lf >= 1) ln = lf;
    lf = lf < 0 ? 0 : (lf >= ap.nmat ? ap.nmat - 1 : lf);  // the host checked the range
    ln = ln >= ap.nmat ? ap.nmat - 1 : ln;
    const double2 mf = ap.mat[lf], mn = ap.mat[ln];
    const double w = v - (double)lf;
    eps = make_double2(mf.x + w * (mn.x - mf.x), mf.y + w * (mn.y - mf.y));
    // a1 = (3 d^3 / (4 pi)) (eps - 1) / (eps + 2)
    const double2 a1 = cdiv(dscale(make_double2(eps.x - 1.0, eps.y), ap.a1c), make_double2(eps.x + 2.0, eps.y));
    // result = 1 + (a1 / d^3) ((b1 + eps b2 + eps b3 S) (K d)^2 - i (2/3)(K d)^3)
    const double2 q = dadd(dadd(make_double2(b1, 0.0), dscale(eps, b2)), dscale(dscale(eps, b3), ap.S));
    const double2 t = make_double2(q.x * ap.Kd2, q.y * ap.Kd2 - ap.rad);
    const double2 res = dadd(make_double2(1.0, 0.0), dmul(make_double2(a1.x / ap.d3, a1.y / ap.d3), t));
    const double2 alpha = cdiv(a1, res);
    inv = cdiv(make_double2(1.0, 0.0), alpha);
}

__global__ void k_to_dd(long long n, const double2* __restrict__ src, dd2* __restrict__ dst) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        dst[e] = dd2(src[e]);
}

// *flag |= 1 when an entry is neither +0 nor -0 (mode 0: A 0 = 0 exactly), or
// when a density lies outside [0, hi) or is NaN (mode 1: the material table,
// DDAModel.cpp:54-63).  An OR, so the result does not depend on the order.
__global__ void k_scan(long long n, const double* __restrict__ v, int mode, double hi, unsigned int* __restrict__ flag) {
    unsigned int any = 0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
        const double x = v[e];
        if (mode == 0) any |= (__double_as_longlong(x) & 0x7fffffffffffffffll) != 0;
        else any |= !(x >= 0.0 && x < hi);
    }
    any = __any_sync(0xffffffffu, any);
    if (any && (threadIdx.x & 31) == 0) atomicOr(flag, 1u);
}

// One thread per dipole: the three entries of a dipole normally hold the same
// density (CoreStructure.cpp:22-27), whose values are formed once.
__global__ void k_model_alpha(int n3, const double* __restrict__ diel_old, AlphaParams ap, double2* __restrict__ diel,
                              double2* __restrict__ al, float2* __restrict__ fal) {
    const int n = n3 / 3;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double2 eps, inv;
        double vprev = 0.0;
        for (int c = 0; c < 3; c++) {
            const int e = 3 * i + c;
            const double v = diel_old[e];
            if (c == 0 || !(v == vprev)) model_alpha_one(v, ap, eps, inv);
            vprev = v;
            diel[e] = eps;
            al[e] = inv;
            if (fal) fal[(long long)c * n + i] = make_float2((float)inv.x, (float)inv.y);  // FP32: SoA
        }
    }
}

// d(al)/d(rho) for entry e: al = 1 / alpha_LDR(eps) = 1/a_CM + (b1 + b2 eps + b3 S eps)(Kd)^2/d^3
// - i(2/3)(Kd)^3/d^3 (tools.cpp:617-630), so dal/deps = -3 / (c (eps - 1)^2) + (b2 + b3 S)(Kd)^2/d^3
// with c = 3 d^3 / (4 pi); eps interpolates the material table linearly in rho below 1
// (DDAModel.cpp:54-63), so deps/drho = mat[1] - mat[0] there (the left derivative at rho = 1);
// above 1 the table is piecewise constant and the derivative is 0.
__device__ __forceinline__ double2 dal_drho(double2 eps, double v, const AlphaParams& ap) {
    const double b2 = 0.1648469, b3 = -1.7700004;  // LDR coefficients (tools.cpp:618-620)
    if (v > 1.0 || ap.nmat < 2) return make_double2(0.0, 0.0);
    const double2 em1 = make_double2(eps.x - 1.0, eps.y);
    const double2 sq = dmul(em1, em1);
    const double2 t = cdiv(make_double2(-3.0 / ap.a1c, 0.0), sq);
    const double2 dal = make_double2(t.x + (b2 + b3 * ap.S) * ap.Kd2 / ap.d3, t.y);
    return dmul(dal, make_double2(ap.mat[1].x - ap.mat[0].x, ap.mat[1].y - ap.mat[0].y));
}

__global__ void k_density_gradient(int nparam, const int* __restrict__ off, const int* __restrict__ dip,
                                   const double2* __restrict__ P, const double2* __restrict__ eps,
                                   const double* __restrict__ diel_old, AlphaParams ap, GradArgs ga,
                                   double* __restrict__ s) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nparam) return;
    double acc = 0.0;
    for (int q = off[i]; q < off[i + 1]; q++) {
        const int j = dip[q];
        for (int c = 0; c < 3; c++) {
            const int e = 3 * j + c;
            double2 lam = make_double2(0.0, 0.0);
            for (int k = 0; k < ga.nadj; k++) lam = dadd(lam, dmul(ga.coef[k], ga.lam[k][e]));
            const double2 t = dmul(dmul(lam, dal_drho(eps[e], diel_old[e], ap)), P[e]);
            acc += t.x;
        }
    }
    s[i] = acc;
}

__global__ void k_model_incident(int N, const int* __restrict__ R, double3 nK, double3 nE0, double E0, double K,
                                 double d, double2* __restrict__ E) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
        const double ph = K * d * (nK.x * R[3 * i] + nK.y * R[3 * i + 1] + nK.z * R[3 * i + 2]);
        double sn, cs;
        sincos(ph, &sn, &cs);
        const double a[3] = {E0 * nE0.x, E0 * nE0.y, E0 * nE0.z};
#pragma unroll
        for (int j = 0; j < 3; j++) E[3 * i + j] = make_double2(a[j] * cs, a[j] * sn);
    }
}

// ------------------------------------------------------------ small kernels
__global__ void k_einternal(int n3, const double2* al, const double2* P, const double2* diel, double2* Ein) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n3; e += gridDim.x * blockDim.x) {
        const double2 lf = make_double2((2.0 + diel[e].x) / 3.0, diel[e].y / 3.0);
        Ein[e] = cdiv(dmul(al[e], P[e]), lf);
    }
}
// FP64 AoS vector -> FP32 SoA vector (the layouts of RhsVecs<double> and <float>)
__global__ void k_to_f32(int n3, const double2* src, float2* dst) {
    const int n = n3 / 3;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n3; e += gridDim.x * blockDim.x) {
        const int c = e / n, i = e - c * n;  // consecutive threads write consecutive entries
        const double2 v = src[3LL * i + c];
        dst[e] = make_float2((float)v.x, (float)v.y);
    }
}
// P (FP64 AoS) += d (FP32 SoA)
__global__ void k_accumulate(int n3, const float2* d, double2* P) {
    const int n = n3 / 3;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n3; e += gridDim.x * blockDim.x) {
        const int i = e / 3, c = e - 3 * i;
        const float2 v = d[(long long)c * n + i];
        P[e] = make_double2(P[e].x + (double)v.x, P[e].y + (double)v.y);
    }
}
// Jacobi preconditioning of the FP32 inner solve: pre = 1 / al from the FP32
// al (SoA; al is well away from 0, so FP32 is enough for a preconditioner), and
// P += d pre (the correction's product in FP32, like the correction itself,
// accumulated in FP64), and a vector of ones
__global__ void k_recip_f32(int n3, const float2* al, float2* pre) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n3; e += gridDim.x * blockDim.x) {
        const float2 a = al[e];
        const float m = a.x * a.x + a.y * a.y;
        pre[e] = make_float2(a.x / m, -a.y / m);
    }
}
__global__ void k_accumulate_scaled(int n3, const float2* d, const float2* pre, double2* P) {
    const int n = n3 / 3;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n3; e += gridDim.x * blockDim.x) {
        const int i = e / 3, c = e - 3 * i;
        const long long s = (long long)c * n + i;
        const float2 v = d[s], q = pre[s];
        const float vx = v.x * q.x - v.y * q.y, vy = v.x * q.y + v.y * q.x;
        P[e] = make_double2(P[e].x + (double)vx, P[e].y + (double)vy);
    }
}
// the largest and smallest |al|^2 of a model (positive floats compare as their
// bit patterns): out[0] max, out[1] min, set to 0 and ~0 before the launch
__global__ void k_al_range(int n3, const float2* __restrict__ al, unsigned int* __restrict__ out) {
    float hi = 0.f, lo = 3.0e38f;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n3; e += gridDim.x * blockDim.x) {
        const float2 a = al[e];
        const float m = a.x * a.x + a.y * a.y;
        hi = fmaxf(hi, m);
        lo = fminf(lo, m);
    }
    for (int o = 16; o > 0; o >>= 1) {
        hi = fmaxf(hi, __shfl_down_sync(0xffffffffu, hi, o));
        lo = fminf(lo, __shfl_down_sync(0xffffffffu, lo, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, __float_as_uint(hi));
        atomicMin(out + 1, __float_as_uint(lo));
    }
}
__global__ void k_fill_ones(long long n, float2* v) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        v[e] = make_float2(1.f, 0.f);
}
template <typename T> __global__ void k_zero(long long n, cx<T>* v) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        v[e] = czero<T>();
}

int grid1d(long long n, int nt) {
    long long b = (n + nt - 1) / nt;
    if (b > 152 * 16) b = 152 * 16;  // 16 resident blocks per SM on 152 SMs at most
    return (int)(b < 1 ? 1 : b);
}
// reductions over a vector: four entries per thread keeps the FP64 block
// sums few while leaving enough threads to cover memory latency
// blocks of a grid-stride reduction over n entries.  FP64 kernels: 4 entries
// per thread, at most 8 blocks per SM (each block's FP64 block sum occupies
// the narrow FP64 pipe).  FP32 kernels: 2 entries per thread for latency
// hiding, and at most 8 per thread (their per-thread partials are FP32).
int grid_reduce(long long n, bool fp32) {
    long long b;
    if (fp32) {
        b = std::min((n + 2LL * kNT - 1) / (2LL * kNT), std::max(152LL * 16, (n + 8LL * kNT - 1) / (8LL * kNT)));
    } else {
        b = (n + 4LL * kNT - 1) / (4LL * kNT);
        if (b > 152 * 8) b = 152 * 8;
    }
    return (int)(b < 1 ? 1 : b);
}

size_t rowsmem(const AxisPlan& p) { return sizeof(double2) * (size_t)(p.M + 2 * row_lines(p) * pad_odd(p.M)); }
size_t colsmem(const AxisPlan& p) { return sizeof(double2) * (size_t)(p.M + 2 * p.M * col_tile(p)); }


}  // namespace

cudaError_t configure_kernels() {
    cudaError_t e = configure_pass_generic();
    if (e == cudaSuccess) e = configure_pass_ct_z();
    if (e == cudaSuccess) e = configure_pass_ct_xy();
    if (e == cudaSuccess) e = configure_pass_ct_xy2();
    if (e == cudaSuccess) e = configure_pass_zy();
    if (e == cudaSuccess) e = configure_pass_dd();
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute((const void*)k_fft_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxPassSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute((const void*)k_fft_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxPassSmem);
    return e;
}

size_t max_pass_smem(const Geom& g) {
    size_t m = 0;
    m = std::max(m, zsmem<double>(g.pz.M));
    m = std::max(m, ysmem<double>(g.py.M));
    m = std::max(m, xsmem<double>(g.px.M));
    m = std::max(m, rowsmem(g.pz));
    m = std::max(m, colsmem(g.py));
    m = std::max(m, colsmem(g.px));
    return m;  // the FP32 tiles are never larger than the FP64 ones
}

int max_blocks_per_rhs(const Geom& g) {
    const int lz = std::min(z_lines<float>(g.pz.M), z_lines<double>(g.pz.M));
    int nz = (g.Nx * g.Ny + lz - 1) / lz;
    int nv = std::max(grid_reduce(3LL * g.N, false), grid_reduce(3LL * g.N, true));
    int nzy = 3 * g.Nx;  // fused z+y passes: one block per (x plane, component)
    return std::max(nz, std::max(nv, nzy));
}

// ------------------------------------------------------------------ launchers
namespace {
cudaError_t fft_rows(double2* data, long long nrows, const AxisPlan& p, const double2* tw, int sign,
                     cudaStream_t stream, int nout = 0) {
    const int L = row_lines(p);
    k_fft_rows<<<(unsigned)((nrows + L - 1) / L), kNT, rowsmem(p), stream>>>(data, nrows, p, tw, sign,
                                                                              nout > 0 ? nout : p.M);
    return cudaGetLastError();
}
cudaError_t fft_cols(double2* data, int nouter, int o1, long long s1, long long s2, long long ms, int ninner,
                     const AxisPlan& p, const double2* tw, int sign, cudaStream_t stream, int nout = 0) {
    const int ZT = col_tile(p);
    const int nt = (ninner + ZT - 1) / ZT;
    k_fft_cols<<<(unsigned)(nouter * nt), kNT, colsmem(p), stream>>>(data, nouter, o1, s1, s2, ms, ninner, p, tw,
                                                                      sign, nout > 0 ? nout : p.M);
    return cudaGetLastError();
}
}  // namespace

cudaError_t launch_green(const Geom& g, double K, double d, const double2* twx, const double2* twy, const double2* twz,
                         double2* full6, double2* green64, float2* green32, cudaStream_t stream,
                         const Interaction& it, const PeriodicImages* pi, double2* oct) {
    const int Mx = g.px.M, My = g.py.M, Mz = g.pz.M;
    const long long M = (long long)Mx * My * Mz;
    cudaError_t err;
    if (pi) {
        k_green_periodic_octant<<<g.Nx * g.Ny * g.Nz, kNT, 0, stream>>>(g, K, d, *pi, it, oct);
        err = cudaGetLastError();
        if (!err) {
            k_green_expand<<<grid1d(M, kNT), kNT, 0, stream>>>(g, oct, full6);
            err = cudaGetLastError();
        }
    } else {
        const long long n = (long long)g.Nx * g.Ny * g.Nz;
        k_green_octant<<<grid1d(n, kNT), kNT, 0, stream>>>(g, K, d, it, oct);
        err = cudaGetLastError();
        if (!err) {
            k_green_expand<<<grid1d(M, kNT), kNT, 0, stream>>>(g, oct, full6);
            err = cudaGetLastError();
        }
    }
    // the six components form a (6 Mx, My, Mz) array for the z and y axes;
    // the x axis runs over the outer pairs (component, y).  Only the octant
    // k <= M / 2 of each axis is folded, so each axis forms only those outputs,
    // and the later axes transform only the lines of the kept indices: the y
    // pass the columns kz < Hz, the x pass the columns ky < Hy, kz < Hz.
    if (!err) err = fft_rows(full6, 6LL * Mx * My, g.pz, twz, -1, stream, g.Hz);
    if (!err) err = fft_cols(full6, 6 * Mx, 6 * Mx, 0, (long long)My * Mz, Mz, g.Hz, g.py, twy, -1, stream, g.Hy);
    if (!err) err = fft_cols(full6, 6 * g.Hy, g.Hy, M, Mz, (long long)My * Mz, g.Hz, g.px, twx, -1, stream, g.Hx);
    if (err) return err;
    const long long H6 = 6LL * g.Hx * g.Hy * g.Hz;
    k_green_fold<<<grid1d(H6, kNT), kNT, 0, stream>>>(g, full6, green64, green32);
    return cudaGetLastError();
}

cudaError_t launch_fft3d_f64(double2* data, const AxisPlan& p0, const AxisPlan& p1, const AxisPlan& p2,
                             const double2* tw0, const double2* tw1, const double2* tw2, int sign,
                             cudaStream_t stream) {
    const int n0 = p0.M, n1 = p1.M, n2 = p2.M;
    cudaError_t err = fft_rows(data, (long long)n0 * n1, p2, tw2, sign, stream);
    if (!err) err = fft_cols(data, n0, n0, 0, (long long)n1 * n2, n2, n2, p1, tw1, sign, stream);
    if (!err) err = fft_cols(data, n1, n1, 0, n2, (long long)n1 * n2, n2, p0, tw0, sign, stream);
    return err;
}

template <typename T>
cudaError_t launch_aproduct(const Geom& g, int src, int snk, int nrhs, const RhsVecs<T>* rhs, const cx<T>* green,
                            const cx<T>* twx, const cx<T>* twy, const cx<T>* twz, const int* cellmap, cx<T>* grid,
                            cudaStream_t stream, cudaEvent_t* ev, int slot) {
    const PassArgs<T> a{g, nrhs, rhs, green, twx, twy, twz, cellmap, grid, stream, slot, sink_blocks<T>(g)};
    if (zy_fused(g, sizeof(T) == 4)) {
        cudaError_t err = cudaSuccess;
        if (ev) cudaEventRecord(ev[0], stream);
        if (!pass_zy<T>(PASS_ZFWD, src, a, &err)) return cudaErrorInvalidValue;
        if (err != cudaSuccess) return err;
        if (ev) cudaEventRecord(ev[1], stream), cudaEventRecord(ev[2], stream);
        if (!pass_ct_xy<T>(PASS_XPASS, 0, a, &err) && !pass_ct_xy2<T>(PASS_XPASS, 0, a, &err))
            err = pass_generic<T>(PASS_XPASS, 0, a);
        if (err != cudaSuccess) return err;
        if (ev) cudaEventRecord(ev[3], stream);
        if (!pass_zy<T>(PASS_ZINV, snk, a, &err)) return cudaErrorInvalidValue;
        if (err != cudaSuccess) return err;
        if (ev) cudaEventRecord(ev[4], stream), cudaEventRecord(ev[5], stream);
        return cudaSuccess;
    }
    const int passes[5] = {PASS_ZFWD, PASS_YFWD, PASS_XPASS, PASS_YINV, PASS_ZINV};
    const int modes[5] = {src, 0, 0, 0, snk};
    for (int k = 0; k < 5; k++) {
        if (ev) cudaEventRecord(ev[k], stream);
        cudaError_t err = cudaSuccess;
        const bool done = pass_ct_z<T>(passes[k], modes[k], a, &err) || pass_ct_xy<T>(passes[k], modes[k], a, &err) ||
                          pass_ct_xy2<T>(passes[k], modes[k], a, &err);
        if (!done) err = pass_generic<T>(passes[k], modes[k], a);
        if (err != cudaSuccess) return err;
    }
    if (ev) cudaEventRecord(ev[5], stream);
    return cudaSuccess;
}

template <typename T> int sink_blocks(const Geom& g) {
    if (zy_fused(g, sizeof(T) == 4)) return 3 * g.Nx;  // one block per (x plane, component)
    const int lz = z_lines<T>(g.pz.M);
    return (g.Nx * g.Ny + lz - 1) / lz;
}

cudaError_t launch_chunk_end(const Geom& g, int nrhs, const RhsVecs<float>* rhs, int slot,
                             cudaGraphConditionalHandle loop, bool in_loop, cudaStream_t stream) {
    const cudaError_t e = launch_early(g.early != 0, k_chunk_end, dim3(1), dim3(kNT), 0, stream, rhs, nrhs, slot,
                                       sink_blocks<float>(g), loop, in_loop ? 1 : 0);
    return e != cudaSuccess ? e : cudaGetLastError();
}

template <typename T>
cudaError_t launch_update(const Geom& g, int nrhs, const RhsVecs<T>* rhs, int is_init, cudaStream_t stream) {
    const dim3 gr(grid_reduce(3LL * g.N, sizeof(T) == 4), nrhs);
    k_update<T><<<gr, kNT, 0, stream>>>(3 * g.N, rhs, is_init);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_finish(const Geom& g, int nrhs, const RhsVecs<T>* rhs, cudaStream_t stream) {
    const dim3 gr(grid1d(3LL * g.N, kNT), nrhs);
    k_finish<T><<<gr, kNT, 0, stream>>>(3 * g.N, g.multi, rhs);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_solve_begin(const Geom& g, int nrhs, const RhsVecs<T>* rhs, cudaStream_t stream) {
    const dim3 gr(grid_reduce(3LL * g.N, sizeof(T) == 4), nrhs);
    k_solve_begin<T><<<gr, kNT, 0, stream>>>(3 * g.N, g.multi, rhs, 0);
    return cudaGetLastError();
}

template <typename T>
cudaError_t launch_residual_is_rhs(const Geom& g, int nrhs, const RhsVecs<T>* rhs, cudaStream_t stream) {
    const dim3 gr(grid_reduce(3LL * g.N, sizeof(T) == 4), nrhs);
    k_solve_begin<T><<<gr, kNT, 0, stream>>>(3 * g.N, g.multi, rhs, 1);
    return cudaGetLastError();
}

cudaError_t launch_sici_table(double* si, double* ci, cudaStream_t stream) {
    k_sici_table<<<grid1d(kSiCiN, 128), 128, 0, stream>>>(si, ci);
    return cudaGetLastError();
}

int field_blocks(int N, int npts) {
    const int per_point = std::max(1, (N + kNT - 1) / kNT);
    const int fill = std::max(1, (152 * 8) / std::max(1, npts));
    return std::min(per_point, fill);
}

cudaError_t launch_field_at(int N, const int* R, double d, double K, const Interaction& it, const double2* P, int npts,
                            const double* pts, double3 nK, double3 nE0, double E0, double2* part, double2* E,
                            cudaStream_t stream) {
    const int nb = field_blocks(N, npts);
    constexpr int kChunk = 32768;  // points per launch (gridDim.y <= 65535)
    for (int p0 = 0; p0 < npts; p0 += kChunk) {
        const int np = std::min(kChunk, npts - p0);
        double2* pp = part + 3LL * nb * p0;
        k_field_partial<<<dim3(nb, np), kNT, 0, stream>>>(N, R, d, K, it, P, pts + 3LL * p0, pp);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        k_field_sum<<<grid1d(np, 128), 128, 0, stream>>>(np, nb, pp, pts + 3LL * p0, nK, nE0, E0, K, E + 3LL * p0);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_einternal(int n3, const double2* al, const double2* P, const double2* diel, double2* Ein,
                             cudaStream_t stream) {
    k_einternal<<<grid1d(n3, kNT), kNT, 0, stream>>>(n3, al, P, diel, Ein);
    return cudaGetLastError();
}
cudaError_t launch_scan(long long n, const double* v, int mode, double hi, unsigned int* flag, cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(unsigned int), stream);
    if (e != cudaSuccess) return e;
    k_scan<<<std::min(grid1d(n, kNT), 152 * 8), kNT, 0, stream>>>(n, v, mode, hi, flag);
    return cudaGetLastError();
}
cudaError_t launch_model_alpha(int n3, const double* diel_old, const AlphaParams& ap, double2* diel, double2* al,
                               float2* fal, cudaStream_t stream) {
    k_model_alpha<<<grid1d(n3 / 3, kNT), kNT, 0, stream>>>(n3, diel_old, ap, diel, al, fal);
    return cudaGetLastError();
}
cudaError_t launch_density_gradient(int nparam, const int* off, const int* dip, const double2* P, const double2* eps,
                                    const double* diel_old, const AlphaParams& ap, const GradArgs& ga, double* s,
                                    cudaStream_t stream) {
    k_density_gradient<<<grid1d(nparam, 128), 128, 0, stream>>>(nparam, off, dip, P, eps, diel_old, ap, ga, s);
    return cudaGetLastError();
}
cudaError_t launch_model_incident(int N, const int* R, double3 nK, double3 nE0, double E0, double K, double d,
                                  double2* E, cudaStream_t stream) {
    k_model_incident<<<grid1d(N, kNT), kNT, 0, stream>>>(N, R, nK, nE0, E0, K, d, E);
    return cudaGetLastError();
}
cudaError_t launch_to_dd(long long n, const double2* src, dd2* dst, cudaStream_t stream) {
    k_to_dd<<<std::min(grid1d(n, kNT), 152 * 8), kNT, 0, stream>>>(n, src, dst);
    return cudaGetLastError();
}
cudaError_t launch_to_f32(int n3, const double2* src, float2* dst, cudaStream_t stream) {
    k_to_f32<<<grid1d(n3, kNT), kNT, 0, stream>>>(n3, src, dst);
    return cudaGetLastError();
}
cudaError_t launch_recip_f32(int n3, const float2* al, float2* pre, cudaStream_t stream) {
    k_recip_f32<<<grid1d(n3, kNT), kNT, 0, stream>>>(n3, al, pre);
    return cudaGetLastError();
}
cudaError_t launch_accumulate_scaled(int n3, const float2* d, const float2* pre, double2* P, cudaStream_t stream) {
    k_accumulate_scaled<<<grid1d(n3, kNT), kNT, 0, stream>>>(n3, d, pre, P);
    return cudaGetLastError();
}
cudaError_t launch_al_range(int n3, const float2* al, unsigned int* out, cudaStream_t stream) {
    // out[0] = 0 (max), out[1] = ~0 (min), without a host buffer
    cudaError_t e = cudaMemsetAsync(out, 0, sizeof(unsigned int), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(out + 1, 0xff, sizeof(unsigned int), stream);
    if (e != cudaSuccess) return e;
    k_al_range<<<std::min(grid1d(n3, kNT), 152 * 8), kNT, 0, stream>>>(n3, al, out);
    return cudaGetLastError();
}
cudaError_t launch_fill_ones(long long n, float2* v, cudaStream_t stream) {
    k_fill_ones<<<grid1d(n, kNT), kNT, 0, stream>>>(n, v);
    return cudaGetLastError();
}
cudaError_t launch_accumulate(int n3, const float2* d, double2* P, cudaStream_t stream) {
    k_accumulate<<<grid1d(n3, kNT), kNT, 0, stream>>>(n3, d, P);
    return cudaGetLastError();
}
template <typename T> cudaError_t launch_zero(long long n, cx<T>* v, cudaStream_t stream) {
    k_zero<T><<<grid1d(n, kNT), kNT, 0, stream>>>(n, v);
    return cudaGetLastError();
}

#define TDDA_INST(T)                                                                                               \
    template cudaError_t launch_aproduct<T>(const Geom&, int, int, int, const RhsVecs<T>*, const cx<T>*,          \
                                            const cx<T>*, const cx<T>*, const cx<T>*, const int*, cx<T>*,         \
                                            cudaStream_t, cudaEvent_t*, int);                                      \
    template int sink_blocks<T>(const Geom&);                                                                      \
    template cudaError_t launch_finish<T>(const Geom&, int, const RhsVecs<T>*, cudaStream_t);                      \
    template cudaError_t launch_solve_begin<T>(const Geom&, int, const RhsVecs<T>*, cudaStream_t);                 \
    template cudaError_t launch_residual_is_rhs<T>(const Geom&, int, const RhsVecs<T>*, cudaStream_t);             \
    template cudaError_t launch_zero<T>(long long, cx<T>*, cudaStream_t);
TDDA_INST(float)
TDDA_INST(double)
#undef TDDA_INST
template cudaError_t launch_update<double>(const Geom&, int, const RhsVecs<double>*, int, cudaStream_t);

}  // namespace tdda
