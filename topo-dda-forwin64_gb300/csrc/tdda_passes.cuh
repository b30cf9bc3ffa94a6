// tdda_passes.cuh -- the five A-product passes K1..K5 (see tdda_kernels.cu for
// the pass structure) and their launch helpers.
//
// Every pass kernel takes CM, the FFT length of its axis, as a template
// parameter.  CM > 0 compiles the plan, the tile and every stride into the
// kernel (tdda_fft_ct.cuh); CM = 0 reads the plan from the geometry at run
// time (tdda_fft.cuh) and serves every other length.  Each translation unit
// that includes this header instantiates its own set of lengths:
// tdda_pass_generic.cu (CM = 0), tdda_pass_z.cu (z lengths) and
// tdda_pass_xy.cu (x / y lengths).
#pragma once

#include "tdda_device.cuh"
#include "tdda_fft_ct.cuh"

namespace tdda {
namespace dev {

// One entry of the deferred-update step (SRC_PUPD_DEF): the update of the
// previous step (DDAModel.cpp:226-230: u = zeta Ap, z = zeta r - alpha u,
// P += alpha p + z, r = t - zeta At), then the new direction
// p = r + beta (p - u) (DDAModel.cpp:219), which is returned.
// Vector access of the pass kernels.  The double-float product reads and
// writes the FP64 vectors (double2 in memory) and converts at the gather and
// the scatter; the other precisions load and store their own type.
template <typename T> __device__ __forceinline__ cx<T> ldv(const cx<T>* p, long long i) {
    if constexpr (is_dd<T>) return dd2(reinterpret_cast<const double2*>(p)[i]);
    else return p[i];
}
template <typename T> __device__ __forceinline__ void stv(cx<T>* p, long long i, cx<T> v) {
    if constexpr (is_dd<T>) reinterpret_cast<double2*>(p)[i] = v.to_double2();
    else p[i] = v;
}
template <typename T> __device__ __forceinline__ acc_t<T> cnorm2(cx<T> v) {
    if constexpr (is_dd<T>) {
        const double2 d = v.to_double2();
        return d.x * d.x + d.y * d.y;
    } else {
        return v.x * v.x + v.y * v.y;
    }
}

template <typename T>
__device__ __forceinline__ cx<T> deferred_step(const RhsVecs<T>& R, long long o, cx<T> alpha, cx<T> zeta, cx<T> beta) {
    const cx<T> Ap = R.Ap[o], r = R.r[o], p = R.p[o], t = R.t[o], At = R.At[o];
    const cx<T> u = cmul<T>(zeta, Ap);
    const cx<T> z = csub<T>(cmul<T>(zeta, r), cmul<T>(alpha, u));
    R.P[o] = cadd<T>(cadd<T>(R.P[o], cmul<T>(alpha, p)), z);
    const cx<T> rn = csub<T>(t, cmul<T>(zeta, At));
    R.r[o] = rn;
    const cx<T> pn = cadd<T>(rn, cmul<T>(beta, csub<T>(p, u)));
    R.p[o] = pn;
    return pn;
}

// The FP32 step's scalars in a gather pass (SRC_PUPD_DEF: the end of the
// previous step from the At partials; SRC_TUPD: alpha from the Ap partials),
// formed by every block from the partials the previous sink pass published;
// block 0 records them.  The state is read here, with the partials: a
// right-hand side whose solve has stopped returns false without writing.
// scratch: 8 float2 of shared memory that is free until the gather.  Returns
// false when the solve does not continue.
template <int SRC>
__device__ __forceinline__ bool fp32_step_scalars(const RhsVecs<float>& R, int slot, int prod_nblk, float2* scratch,
                                                  float2& alpha, float2& beta, float2& zeta) {
    __shared__ float2 s_sc[3];
    __shared__ int s_stop;
    if constexpr (SRC == SRC_PUPD_DEF) {
        StepIn in;
        if (threadIdx.x == 0) in = load_step_in(R.st, slot);
        float2 tot[8];
        sum_partials<8>(R.part, prod_nblk, scratch, tot);
        if (threadIdx.x == 0) {
            if (in.status != ST_RUNNING) {
                s_stop = in.status;
            } else {
                const StepEnd e = step_end_f32(in, tot);
                if (blockIdx.x == 0) write_step_end(R.st, e, slot);
                s_sc[0] = e.zeta;
                s_sc[1] = e.beta;
                s_sc[2] = in.alpha;
                s_stop = e.stop;
            }
        }
        __syncthreads();
        if (s_stop != ST_RUNNING) return false;
        zeta = s_sc[0];
        beta = s_sc[1];
        alpha = s_sc[2];
    } else {
        float2 rho;
        int status;
        if (threadIdx.x == 0) rho = R.st->rho32[slot], status = R.st->status;
        float2 tot[2];
        sum_partials<2>(R.part, prod_nblk, scratch, tot);
        if (threadIdx.x == 0) {
            const float2 a = fdiv2(rho, make_float2(tot[0].x, tot[1].x));  // DDAModel.cpp:221
            if (status == ST_RUNNING && blockIdx.x == 0) R.st->alpha32[slot] = a;
            s_sc[0] = a;
            s_stop = status;
        }
        __syncthreads();
        if (s_stop != ST_RUNNING) return false;
        alpha = s_sc[0];
    }
    return true;
}

// ------------------------------------------------------------ K1 zfwd
template <typename T, int SRC, int CM>
__global__ void __launch_bounds__(kNT) k_zfwd(Geom g, const RhsVecs<T>* __restrict__ rhs,
                                              const cx<T>* __restrict__ twz, const int* __restrict__ cellmap,
                                              cx<T>* __restrict__ grid, int slot, int prod_nblk) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr bool kStep32 = sizeof(T) == 4 && (SRC == SRC_PUPD_DEF || SRC == SRC_TUPD);
    __shared__ double s_scratch[kStep32 ? 8 : 1];
    const int b = blockIdx.y;
    const RhsVecs<T> R = rhs[b];
    if constexpr (!kStep32) {  // the FP32 step reads the status with its scalars
        if (rhs_done(R.st)) return;
    }
    constexpr int cLZ = CM > 0 ? z_lines<T>(CM) : 1;
    constexpr int cMzP = CM > 0 ? pad_odd(CM) : 1;
    const int Mz = CM > 0 ? CM : g.pz.M, Nz = g.multi ? R.Nz : g.Nz;
    const int LZ = CM > 0 ? cLZ : z_lines<T>(Mz), MzP = CM > 0 ? cMzP : pad_odd(Mz);
    cx<T>* stw = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* s = stw + Mz;
    cx<T>* s2 = s + 3 * LZ * MzP;
    // the lattice of this right-hand side (its own in a cross-lattice batch, whose
    // blocks past its lines return: the grid shape's launch covers the largest)
    const Lat L = lattice_of<T>(g, R, cellmap);
    const int nlines = L.Nx * L.Ny;
    const int l0 = blockIdx.x * LZ;
    const int nl = min(LZ, nlines - l0);
    if (nl <= 0) return;
    stage_tw<T>(stw, twz, Mz);

    cx<T> beta, alpha, zeta;
    if constexpr (kStep32) {
        if (!fp32_step_scalars<SRC>(R, slot, prod_nblk, reinterpret_cast<float2*>(s_scratch), alpha, beta, zeta))
            return;
    } else {
        if (SRC == SRC_PUPD || SRC == SRC_PUPD_DEF) beta = st_beta<T>(R.st);
        if (SRC == SRC_TUPD || SRC == SRC_PUPD_DEF) alpha = st_alpha<T>(R.st);
        if (SRC == SRC_PUPD_DEF) zeta = st_zeta<T>(R.st);
    }
    const cx<T>* src = SRC == SRC_IN ? R.p : R.P;
    for (int e = threadIdx.x; e < nl * Nz; e += blockDim.x) {
        const int line = e / Nz, z = e - (e / Nz) * Nz;
        const int i = L.cellmap[(long long)(l0 + line) * Nz + z];
        cx<T> v[3];
        if (i >= 0) {
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const long long o = vec_index<T>(i, c, L.N);
                if (SRC == SRC_PUPD) {
                    cx<T> pc = R.p[o], uc = R.u[o], rc = R.r[o];
                    v[c] = cadd<T>(rc, cmul<T>(beta, csub<T>(pc, uc)));
                    R.p[o] = v[c];
                } else if (SRC == SRC_PUPD_DEF) {
                    v[c] = deferred_step<T>(R, o, alpha, zeta, beta);
                } else if (SRC == SRC_TUPD) {
                    cx<T> rc = R.r[o], ac = R.Ap[o];
                    v[c] = csub<T>(rc, cmul<T>(alpha, ac));
                    R.t[o] = v[c];
                } else {
                    v[c] = ldv<T>(src, o);
                }
                if constexpr (sizeof(T) == 4) {  // Jacobi preconditioning: the grid gets D^-1 v
                    if (SRC != SRC_P && R.pre) v[c] = cmul<T>(v[c], R.pre[o]);
                }
            }
        } else {
            v[0] = v[1] = v[2] = czero<T>();
        }
#pragma unroll
        for (int c = 0; c < 3; c++) s[(c * LZ + line) * MzP + z] = v[c];
    }
    __syncthreads();
    const cx<T>* res;
    if constexpr (CM > 0) res = ct_fft<-1, T, CM, 3 * cLZ, cMzP, 1, kNT, true, false>(s, s2, stw, Nz, CM);
    else res = smem_fft<-1, T>(s, s2, 3 * LZ, MzP, 1, g.pz, stw, Nz, Mz);
    cx<T>* gb = grid + (long long)b * g.sb;
    for (int e = threadIdx.x; e < 3 * nl * Mz; e += blockDim.x) {
        const int cl = e / Mz, z = e - (e / Mz) * Mz;
        const int c = cl / nl, line = cl - (cl / nl) * nl;
        const int l = l0 + line, x = l / L.Ny, y = l - (l / L.Ny) * L.Ny;
        gb[c * g.sc + x * g.sx + y * g.sy + z] = res[(c * LZ + line) * MzP + z];
    }
}

// ------------------------------------------------------------ K2/K4 ypass
template <typename T, int SIGN, int CM>
__global__ void __launch_bounds__(kNT) k_ypass(Geom g, const RhsVecs<T>* __restrict__ rhs,
                                               const cx<T>* __restrict__ twy, cx<T>* __restrict__ grid) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = blockIdx.z;
    if (rhs_done(rhs[b].st)) return;
    constexpr int cZT = CM > 0 ? y_tile<T>(CM) : 1;
    const int My = CM > 0 ? CM : g.py.M, Mz = g.pz.M;
    const int ZT = CM > 0 ? cZT : y_tile<T>(My);
    const int nzt = (Mz + ZT - 1) / ZT;
    const int x = blockIdx.x / nzt, z0 = (blockIdx.x - x * nzt) * ZT;
    // a cross-lattice batch: this right-hand side's own x extent and rows
    const int Ny = g.multi ? rhs[b].Ny : g.Ny;
    if (g.multi && x >= rhs[b].Nx) return;
    const int c = blockIdx.y;
    const int zn = min(ZT, Mz - z0);
    cx<T>* stw = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* s = stw + My;
    const int ZP = ZT + 1;  // padded row stride: consecutive rows start in different banks
    cx<T>* s2 = s + My * ZP;
    stage_tw<T>(stw, twy, My);
    cx<T>* gp = grid + (long long)b * g.sb + c * g.sc + (long long)x * g.sx + z0;
    const int nin = SIGN < 0 ? Ny : My;
    const int nout = SIGN < 0 ? My : Ny;
    for (int e = threadIdx.x; e < nin * ZT; e += blockDim.x) {
        const int y = e / ZT, zl = e - (e / ZT) * ZT;
        if (zl < zn) s[y * ZP + zl] = gp[(long long)y * g.sy + zl];
    }
    __syncthreads();
    const cx<T>* res;
    if constexpr (CM > 0) res = ct_fft<SIGN, T, CM, cZT, 1, cZT + 1, kNT, (SIGN < 0), (SIGN > 0)>(s, s2, stw, nin, nout);
    else res = smem_fft<SIGN, T>(s, s2, ZT, 1, ZP, g.py, stw, nin, nout);
    for (int e = threadIdx.x; e < nout * ZT; e += blockDim.x) {
        const int y = e / ZT, zl = e - (e / ZT) * ZT;
        if (zl < zn) gp[(long long)y * g.sy + zl] = res[y * ZP + zl];
    }
}

// ------------------------------------------------------------ K3 xpass
// folding of a spectral index and the parity of each tensor component:
// xx, yy, zz even in all axes; xy odd in x,y; xz odd in x,z; yz odd in y,z
__device__ __forceinline__ int fold(int k, int M) { return 2 * k > M ? M - k : k; }

// the six components of one spectral point: 48 (FP32) or 96 (FP64) contiguous,
// 16-byte aligned bytes, read as 16-byte vectors
template <typename T>
__device__ __forceinline__ void load_green6(const cx<T>* gg, cx<T>& a0, cx<T>& a1, cx<T>& a2, cx<T>& a3, cx<T>& a4,
                                            cx<T>& a5) {
    if constexpr (is_dd<T>) {
        const float4* q = reinterpret_cast<const float4*>(gg);
        a0 = dd2(__ldg(q)); a1 = dd2(__ldg(q + 1)); a2 = dd2(__ldg(q + 2));
        a3 = dd2(__ldg(q + 3)); a4 = dd2(__ldg(q + 4)); a5 = dd2(__ldg(q + 5));
    } else if constexpr (sizeof(cx<T>) == 8) {
        const float4* q = reinterpret_cast<const float4*>(gg);
        const float4 u = __ldg(q), v = __ldg(q + 1), w = __ldg(q + 2);
        a0 = mk<T>(u.x, u.y); a1 = mk<T>(u.z, u.w);
        a2 = mk<T>(v.x, v.y); a3 = mk<T>(v.z, v.w);
        a4 = mk<T>(w.x, w.y); a5 = mk<T>(w.z, w.w);
    } else {
        a0 = __ldg(gg); a1 = __ldg(gg + 1); a2 = __ldg(gg + 2);
        a3 = __ldg(gg + 3); a4 = __ldg(gg + 4); a5 = __ldg(gg + 5);
    }
}

// The six components at folded point (fy, fx, fz).  FP64 and double-float
// tables hold the six contiguously ([Hy][Hx][Hz][6]).  The FP32 table holds
// them as three planes of component pairs ([Hy][Hx][3][Hz] float4: xx|xy,
// xz|yy, yz|zz), so the threads of a warp that walk z read whole 128-byte
// lines with each 16-byte load instead of a third of three lines each.
template <typename T>
__device__ __forceinline__ void load_green(const cx<T>* green, const Geom& g, int fy, int fx, int fz, cx<T>& a0,
                                           cx<T>& a1, cx<T>& a2, cx<T>& a3, cx<T>& a4, cx<T>& a5) {
    if constexpr (sizeof(cx<T>) == 8) {
        const float4* q = reinterpret_cast<const float4*>(green) + ((long long)fy * g.Hx + fx) * 3 * g.Hz + fz;
        const float4 u = __ldg(q), v = __ldg(q + g.Hz), w = __ldg(q + 2 * g.Hz);
        a0 = mk<T>(u.x, u.y); a1 = mk<T>(u.z, u.w);
        a2 = mk<T>(v.x, v.y); a3 = mk<T>(v.z, v.w);
        a4 = mk<T>(w.x, w.y); a5 = mk<T>(w.z, w.w);
    } else {
        load_green6<T>(green + (((long long)fy * g.Hx + fx) * g.Hz + fz) * 6, a0, a1, a2, a3, a4, a5);
    }
}

template <typename T, int CM>
__global__ void __launch_bounds__(kNT) k_xpass(Geom g, const RhsVecs<T>* __restrict__ rhs,
                                               const cx<T>* __restrict__ green, const cx<T>* __restrict__ twx,
                                               cx<T>* __restrict__ grid) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = blockIdx.y;
    if (rhs_done(rhs[b].st)) return;
    constexpr int cZT = CM > 0 ? x_tile<T>(CM) : 1;
    // a right-hand side of a cross-lattice batch brings its own box and spectrum
    const int Mx = CM > 0 ? CM : g.px.M, My = g.py.M, Mz = g.pz.M, Nx = g.multi ? rhs[b].Nx : g.Nx;
    if (g.multi) green = rhs[b].green;
    const int ZT = CM > 0 ? cZT : x_tile<T>(Mx);
    const int nzt = (Mz + ZT - 1) / ZT;
    const int y = blockIdx.x / nzt, z0 = (blockIdx.x - y * nzt) * ZT;
    const int zn = min(ZT, Mz - z0);
    const int W = 3 * ZT;  // lines: 3 components x ZT
    const int WP = W + 1;   // padded row stride: consecutive rows start in different banks
    cx<T>* stw = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* s = stw + Mx;
    cx<T>* s2 = s + Mx * WP;
    stage_tw<T>(stw, twx, Mx);
    cx<T>* gp = grid + (long long)b * g.sb + (long long)y * g.sy + z0;
    for (int e = threadIdx.x; e < Nx * W; e += blockDim.x) {
        const int x = e / W, r = e - (e / W) * W;
        const int c = r / ZT, zl = r - (r / ZT) * ZT;
        if (zl < zn) s[x * WP + r] = gp[c * g.sc + (long long)x * g.sx + zl];
        else s[x * WP + r] = czero<T>();
    }
    __syncthreads();
    cx<T>* res;
    if constexpr (CM > 0) res = ct_fft<-1, T, CM, 3 * cZT, 1, 3 * cZT + 1, kNT, true, false>(s, s2, stw, Nx, CM);
    else res = smem_fft<-1, T>(s, s2, W, 1, WP, g.px, stw, Nx, Mx);

    // spectral product: C = A b with the symmetric 3x3 Green tensor
    const int fy = fold(y, My);
    const bool uy = 2 * y > My;
    for (int e = threadIdx.x; e < Mx * ZT; e += blockDim.x) {
        const int kx = e / ZT, zl = e - (e / ZT) * ZT;
        const int z = z0 + zl;
        if (zl >= zn) continue;
        const int fx = fold(kx, Mx), fz = fold(z, Mz);
        const bool ux = 2 * kx > Mx, uz = 2 * z > Mz;
        cx<T> a0, a1, a2, a3, a4, a5;
        load_green<T>(green, g, fy, fx, fz, a0, a1, a2, a3, a4, a5);
        if (ux != uy) a1 = mk<T>(-a1.x, -a1.y);  // xy: odd in x and y
        if (ux != uz) a2 = mk<T>(-a2.x, -a2.y);  // xz: odd in x and z
        if (uy != uz) a4 = mk<T>(-a4.x, -a4.y);  // yz: odd in y and z
        cx<T>* p = res + kx * WP + zl;
        const cx<T> bx = p[0], by = p[ZT], bz = p[2 * ZT];
        p[0] = cadd<T>(cadd<T>(cmul<T>(a0, bx), cmul<T>(a1, by)), cmul<T>(a2, bz));
        p[ZT] = cadd<T>(cadd<T>(cmul<T>(a1, bx), cmul<T>(a3, by)), cmul<T>(a4, bz));
        p[2 * ZT] = cadd<T>(cadd<T>(cmul<T>(a2, bx), cmul<T>(a4, by)), cmul<T>(a5, bz));
    }
    __syncthreads();
    cx<T>* other = res == s ? s2 : s;
    const cx<T>* out;
    if constexpr (CM > 0) out = ct_fft<+1, T, CM, 3 * cZT, 1, 3 * cZT + 1, kNT, false, true>(res, other, stw, CM, Nx);
    else out = smem_fft<+1, T>(res, other, W, 1, WP, g.px, stw, Mx, Nx);
    for (int e = threadIdx.x; e < Nx * W; e += blockDim.x) {
        const int x = e / W, r = e - (e / W) * W;
        const int c = r / ZT, zl = r - (r / ZT) * ZT;
        if (zl < zn) gp[c * g.sc + (long long)x * g.sx + zl] = out[x * WP + r];
    }
}

// ------------------------------------------------------------ K3, register form
// x pass for an FFT length with a two-stage plan M = R1 R2 (the FP32 plans of
// tdda_fft_ct.cuh).  Stockham order: the forward's first stage (radix R1,
// butterfly j < R2) reads x = j + R2 r and writes j R1 + q; its second stage
// (radix R2, butterfly j < R1, twiddles w^(r j)) leaves the spectrum at
// kx = j + R1 q in the registers of one thread; the inverse's first stage
// (radix R2, no twiddles) needs exactly those values, so the second forward
// stage, the spectral product and the first inverse stage run in registers,
// for the three components of one (y, z) column.  The first and last stages
// read and write the grid directly.  Two shared-memory round trips instead of
// six, three barriers.  One block: ZT z-columns of one y row, NT = ZT R1
// threads (one register-stage task each).
template <typename T, int M, int ZT, int MINB>
__global__ void __launch_bounds__(ZT * x2_radix(M, 0), MINB) k_xpass2(Geom g, const RhsVecs<T>* __restrict__ rhs,
                                                                   const cx<T>* __restrict__ green,
                                                                   const cx<T>* __restrict__ twx,
                                                                   cx<T>* __restrict__ grid) {
    constexpr int R1 = x2_radix(M, 0), R2 = x2_radix(M, 1);
    static_assert(R1 * R2 == M, "two-stage plan");
    constexpr int NT = ZT * R1, W = 3 * ZT;
    // Shared rows of W lines.  With 8 z-columns (W = 24) a half warp's 8-byte
    // accesses span two rows, whose banks must differ by 8: the rows of the
    // first exchange (stage 1 -> stage 2) shift by 8 entries every R1 rows,
    // those of the second every R2 rows (R2 even), so that each of the four
    // access patterns takes the minimum two wavefronts per warp.  With 16
    // z-columns a half warp stays in one row and no shift is needed.
    constexpr int SA = ZT == 8 ? 8 : 0, SB = (ZT == 8 && R2 % 2 == 0) ? 8 : 0;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    cx<T>* stw = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* s = stw + M;  // M rows of W, plus the row shifts
    const int b = blockIdx.y;
    const SolveState* st = rhs[b].st;
    // a right-hand side of a cross-lattice batch brings its own box and spectrum
    const int My = g.py.M, Mz = g.pz.M, Nx = g.multi ? rhs[b].Nx : g.Nx;
    if (g.multi) green = rhs[b].green;
    const int nzt = (Mz + ZT - 1) / ZT;
    const int y = blockIdx.x / nzt, z0 = (blockIdx.x - y * nzt) * ZT;
    const int zn = min(ZT, Mz - z0);
    stage_tw<T>(stw, twx, M);
    cx<T>* gp = grid + (long long)b * g.sb + (long long)y * g.sy + z0;
    grid_dep_wait();  // the grid and the solve's state are the previous kernel's
    if (g.early == 1) grid_dep_release();

    // forward stage 1: radix R1 over x = j + R2 r < Nx, grid -> s[j R1 + q][line].
    // Nx <= M / 2, so the inputs r >= R1 / 2 are zero padding: not read, not added.
    static_assert(R1 % 2 == 0, "even first radix");
    constexpr int RH = R1 / 2;
    // a compile-time count of tasks per thread, so the loads of all of a
    // thread's tasks can be issued before the first butterfly
    constexpr int T1 = (W * R2 + NT - 1) / NT;
#pragma unroll
    for (int k = 0; k < T1; k++) {
        const int w = threadIdx.x + k * NT;
        if (T1 * NT > W * R2 && w >= W * R2) break;
        const int l = w % W, j = w / W;
        const int c = l / ZT, zl = l - c * ZT;
        const cx<T>* src = gp + c * g.sc + zl;
        cx<T> v[R1];
#pragma unroll
        for (int r = 0; r < RH; r++) {
            const int xx = j + R2 * r;
            v[r] = (zl < zn && xx < Nx) ? src[(long long)xx * g.sx] : czero<T>();
        }
        BflyIn<R1, -1, T, RH>::run(v);
        cx<T>* d = s + j * (R1 * W + SA) + l;  // row j R1 + q, shifted SA j
#pragma unroll
        for (int q = 0; q < R1; q++) d[q * W] = v[q];
    }
    // a stopped solve is checked here, after the first loads are issued: nothing
    // has been written to global memory yet
    if (rhs_done(st)) return;
    __syncthreads();

    // forward stage 2, spectral product, inverse stage 1: task (zl, j), j < R1
    const int zl = threadIdx.x % ZT, j = threadIdx.x / ZT;
    cx<T> X[3][R2];
#pragma unroll
    for (int c = 0; c < 3; c++) {
#pragma unroll
        for (int r = 0; r < R2; r++) {
            cx<T> t = s[(j + R1 * r) * W + SA * r + c * ZT + zl];  // row j + R1 r
            if (r > 0) t = cmul<T>(t, stw[r * j]);
            X[c][r] = t;
        }
        Bfly<R2, -1, T>::run(X[c]);  // X[c][q]: spectrum at kx = j + R1 q
    }
    if (zl < zn) {  // columns past Mz (a partial tile) hold zeros and are never stored
        const int z = z0 + zl;
        const int fy = fold(y, My), fz = fold(z, Mz);
        const bool uy = 2 * y > My, uz = 2 * z > Mz;
#pragma unroll
        for (int q = 0; q < R2; q++) {
            const int kx = j + R1 * q;
            const int fx = fold(kx, M);
            const bool ux = 2 * kx > M;
            cx<T> a0, a1, a2, a3, a4, a5;
            load_green<T>(green, g, fy, fx, fz, a0, a1, a2, a3, a4, a5);
            if (ux != uy) a1 = mk<T>(-a1.x, -a1.y);  // xy: odd in x and y
            if (ux != uz) a2 = mk<T>(-a2.x, -a2.y);  // xz: odd in x and z
            if (uy != uz) a4 = mk<T>(-a4.x, -a4.y);  // yz: odd in y and z
            const cx<T> bx = X[0][q], by = X[1][q], bz = X[2][q];
            X[0][q] = cadd<T>(cadd<T>(cmul<T>(a0, bx), cmul<T>(a1, by)), cmul<T>(a2, bz));
            X[1][q] = cadd<T>(cadd<T>(cmul<T>(a1, bx), cmul<T>(a3, by)), cmul<T>(a4, bz));
            X[2][q] = cadd<T>(cadd<T>(cmul<T>(a2, bx), cmul<T>(a4, by)), cmul<T>(a5, bz));
        }
    }
#pragma unroll
    for (int c = 0; c < 3; c++) Bfly<R2, +1, T>::run(X[c]);  // inverse stage 1: outputs j R2 + q
    __syncthreads();  // every stage-2 read of s is done
#pragma unroll
    for (int c = 0; c < 3; c++)
#pragma unroll
        for (int q = 0; q < R2; q++) s[(j * R2 + q) * W + SB * j + c * ZT + zl] = X[c][q];  // row j R2 + q
    __syncthreads();

    if (g.early == 2) grid_dep_release();  // the next kernel's blocks start during the last stage
    // inverse stage 2: radix R1, butterfly j < R2, twiddles conj(w^(r j)), outputs x = j + R2 q < Nx
    for (int w = threadIdx.x; w < W * R2; w += NT) {
        const int l = w % W, jj = w / W;
        const int c = l / ZT, zz = l - c * ZT;
        cx<T> v[R1];
#pragma unroll
        for (int r = 0; r < R1; r++) {
            cx<T> t = s[(jj + R2 * r) * W + SB * r + l];  // row jj + R2 r
            if (r > 0) {
                cx<T> tw = stw[r * jj];
                tw.y = -tw.y;
                t = cmul<T>(t, tw);
            }
            v[r] = t;
        }
        Bfly<R1, +1, T>::run(v);
        cx<T>* dst = gp + c * g.sc + zz;
#pragma unroll
        for (int q = 0; q < RH; q++) {  // outputs x >= M / 2 >= Nx are never stored
            const int xx = jj + R2 * q;
            if (zz < zn && xx < Nx) dst[(long long)xx * g.sx] = v[q];
        }
    }
}

template <typename T, int M, int ZT, int MINB = 1> struct XLaunch2 {
    static constexpr int NT = ZT * x2_radix(M, 0);
    // twiddles, M rows of 3 ZT lines, the row shifts (at most 8 max(R1, R2))
    static constexpr size_t smem =
        sizeof(cx<T>) * (size_t)(M + M * 3 * ZT + 8 * (x2_radix(M, 0) > x2_radix(M, 1) ? x2_radix(M, 0)
                                                                                         : x2_radix(M, 1)));
    static cudaError_t run(const PassArgs<T>& a) {
        const dim3 grid(a.g.py.M * ((a.g.pz.M + ZT - 1) / ZT), a.nrhs);
        const Geom g = early_geom(a.g, (long long)grid.x * grid.y);
        const cudaError_t e =
            launch_early(g.early, k_xpass2<T, M, ZT, MINB>, grid, dim3(NT), smem, a.stream, g, a.rhs, a.green, a.twx, a.grid);
        return e != cudaSuccess ? e : cudaGetLastError();
    }
    static cudaError_t configure() {
        return cudaFuncSetAttribute((const void*)k_xpass2<T, M, ZT, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kMaxPassSmem);
    }
};

// blocks per SM the register form is compiled for: 16 warps per SM (a register
// cap of 128 a thread), 24 for M = 128 and 192, whose spectra fit in 85
template <int M, int ZT> constexpr int x2_minb() {
    constexpr int n = ((M == 128 || M == 192) ? 24 : 16) * 32 / (ZT * x2_radix(M, 0));
    return n > 0 ? n : 1;
}
// The register form with 8 or 16 z-columns a block (Geom::x_tile; 0 takes 16
// for M = 128, else 8).  The tile changes only which block transforms a column:
// results are bit-identical.
template <typename T, int M> struct X2Launch {
    using Narrow = XLaunch2<T, M, 8, x2_minb<M, 8>()>;
    using Wide = XLaunch2<T, M, 16, x2_minb<M, 16>()>;
    static cudaError_t run(const PassArgs<T>& a) {
        const bool wide = a.g.x_tile ? a.g.x_tile == 16 : M == 128;
        return wide ? Wide::run(a) : Narrow::run(a);
    }
    static cudaError_t configure() {
        const cudaError_t e = Narrow::configure();
        return e != cudaSuccess ? e : Wide::configure();
    }
};

// ------------------------------------------------------------ K5 zinv
template <typename T, int SRC, int SNK, int CM>
__global__ void __launch_bounds__(kNT) k_zinv(Geom g, const RhsVecs<T>* __restrict__ rhs,
                                              const cx<T>* __restrict__ twz, const int* __restrict__ cellmap,
                                              cx<T>* __restrict__ grid) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int NV = SNK == SNK_AT_DEF ? 8 : 4;
    __shared__ double sred[sred_size<T, NV>()];
    const int b = blockIdx.y;
    const RhsVecs<T> R = rhs[b];
    if (rhs_done(R.st)) return;
    constexpr int cLZ = CM > 0 ? z_lines<T>(CM) : 1;
    constexpr int cMzP = CM > 0 ? pad_odd(CM) : 1;
    // the lattice of this right-hand side (its own in a cross-lattice batch)
    const Lat L = lattice_of<T>(g, R, cellmap);
    const int Mz = CM > 0 ? CM : g.pz.M, Nz = L.Nz;
    const int LZ = CM > 0 ? cLZ : z_lines<T>(Mz), MzP = CM > 0 ? cMzP : pad_odd(Mz);
    cx<T>* stw = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* s = stw + Mz;
    cx<T>* s2 = s + 3 * LZ * MzP;
    const int nlines = L.Nx * L.Ny;
    const int l0 = blockIdx.x * LZ;
    // a cross-lattice batch launches the grid shape's largest line count: a block past
    // this right-hand side's lines adds zeros to its sums
    const int nl = max(0, min(LZ, nlines - l0));
    acc_t<T> acc[NV] = {};
    if (nl > 0) {
    stage_tw<T>(stw, twz, Mz);
    const cx<T>* gb = grid + (long long)b * g.sb;
    for (int e = threadIdx.x; e < 3 * nl * Mz; e += blockDim.x) {
        const int cl = e / Mz, z = e - (e / Mz) * Mz;
        const int c = cl / nl, line = cl - (cl / nl) * nl;
        const int l = l0 + line, x = l / L.Ny, y = l - (l / L.Ny) * L.Ny;
        s[(c * LZ + line) * MzP + z] = gb[c * g.sc + x * g.sx + y * g.sy + z];
    }
    __syncthreads();
    const cx<T>* res;
    if constexpr (CM > 0) res = ct_fft<+1, T, CM, 3 * cLZ, cMzP, 1, kNT, false, true>(s, s2, stw, CM, Nz);
    else res = smem_fft<+1, T>(s, s2, 3 * LZ, MzP, 1, g.pz, stw, Mz, Nz);

    // scatter to the dipoles, fused diagonal term and dot products
    const cx<T>* vsrc = (SRC == SRC_TUPD) ? R.t : (SRC == SRC_P ? R.P : R.p);
    for (int e = threadIdx.x; e < nl * Nz; e += blockDim.x) {
        const int line = e / Nz, z = e - (e / Nz) * Nz;
        const int i = L.cellmap[(long long)(l0 + line) * Nz + z];
        if (i < 0) continue;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            const long long o = vec_index<T>(i, c, L.N);
            cx<T> val = res[(c * LZ + line) * MzP + z];
            if (SNK == SNK_OUT) {
                R.Ap[o] = val;
                continue;
            }
            const cx<T> vv = ldv<T>(vsrc, o);
            const cx<T> w = cadd<T>(val, cmul<T>(vv, ldv<T>(R.al, o)));
            if (SNK == SNK_ALB) {
                R.Ap[o] = w;
            } else if (SNK == SNK_AP) {
                R.Ap[o] = w;
                const cx<T> q = R.r0[o];  // r0 . Ap
                acc[0] += q.x * w.x + q.y * w.y;
                acc[1] += q.x * w.y - q.y * w.x;
            } else if (SNK == SNK_AT || SNK == SNK_AT_DEF) {
                R.At[o] = w;
                const cx<T> tt = vv;  // At . t and At . At
                acc[0] += w.x * tt.x + w.y * tt.y;
                acc[1] += w.x * tt.y - w.y * tt.x;
                acc[2] += w.x * w.x + w.y * w.y;
                if constexpr (SNK == SNK_AT_DEF) {  // r0 . t, r0 . At, t . t
                    const cx<T> q = R.r0[o];
                    acc[3] += q.x * tt.x + q.y * tt.y;
                    acc[4] += q.x * tt.y - q.y * tt.x;
                    acc[5] += q.x * w.x + q.y * w.y;
                    acc[6] += q.x * w.y - q.y * w.x;
                    acc[7] += tt.x * tt.x + tt.y * tt.y;
                }
            } else if (SNK == SNK_RES) {
                const cx<T> res = csub<T>(ldv<T>(R.E, o), w);
                stv<T>(R.r, o, res);
                stv<T>(R.r0, o, res);
                stv<T>(R.p, o, res);
                acc[0] += cnorm2<T>(res);
            }
        }
    }
    }  // nl > 0
    if (SNK == SNK_OUT || SNK == SNK_ALB) return;
    if constexpr (sizeof(T) == 4 && (SNK == SNK_AP || SNK == SNK_AT_DEF)) {
        publish_partials<NV>(acc, R.part, gridDim.x, blockIdx.x, sred);  // the next gather forms the scalars
        return;
    }
    tot_t<T> tot[NV];
    const int nblk = gridDim.x;
    const int slot = SNK == SNK_AP ? 0 : (SNK == SNK_AT || SNK == SNK_AT_DEF ? 1 : 2);
    if (!last_block_total<NV>(acc, R.part, nblk, blockIdx.x, R.cnt + slot, sred, tot)) return;
    if (threadIdx.x != 0) return;
    finalize_sink<T, SNK, NV>(R.st, tot);
}

// ------------------------------------------------------------ fused z+y passes
// For the FP32 passes of the compiled (My, Mz) pairs one block holds the whole
// My x Mz plane of one component of one x-plane in shared memory, so K1+K2
// become one kernel (k_zyfwd) and K4+K5 another (k_yzinv): the plane makes no
// round trip through L2 between the z and y transforms and an A-product is
// three launches instead of five.  Grid: (3 Nx, nrhs), block (x, c) =
// (blockIdx.x / 3, blockIdx.x % 3).  Plane layout in shared memory: [y][z],
// row stride ZP.  Lattice data occupies rows y < Ny <= LY and columns
// z < Nz <= LZ (M >= 2N - 1 on every axis).
// Gather of CH entries of one component: o[q] = 3 i + c of the dipole in
// cell q, or -1 for an empty or padding cell (v[q] = 0).  GatherIn holds the
// vectors a gather reads: load() issues every load, combine() forms the grid
// values with the step scalars and stores the updated vectors, so a kernel can
// form the scalars while the loads are in flight.  All loads come before the
// first store.
template <typename T, int SRC, int CH> struct GatherIn {
    static constexpr int NL = SRC == SRC_PUPD_DEF ? 6 : (SRC == SRC_PUPD ? 3 : (SRC == SRC_TUPD ? 2 : 1));
    // FP32 gathers of a Jacobi-preconditioned solve scale the grid values by pre
    static constexpr bool kPre = sizeof(T) == 4 && (SRC == SRC_IN || SRC == SRC_PUPD || SRC == SRC_TUPD ||
                                                    SRC == SRC_PUPD_DEF);
    cx<T> a[NL][CH];
    __device__ __forceinline__ void load(const RhsVecs<T>& R, const long long (&o)[CH], const cx<T>* src) {
#pragma unroll
        for (int q = 0; q < CH; q++) {
            if (o[q] < 0) continue;
            const long long i = o[q];
            if constexpr (SRC == SRC_PUPD_DEF) {
                a[0][q] = R.Ap[i]; a[1][q] = R.r[i]; a[2][q] = R.p[i];
                a[3][q] = R.t[i]; a[4][q] = R.At[i]; a[5][q] = R.P[i];
            } else if constexpr (SRC == SRC_PUPD) {
                a[0][q] = R.p[i]; a[1][q] = R.u[i]; a[2][q] = R.r[i];
            } else if constexpr (SRC == SRC_TUPD) {
                a[0][q] = R.r[i]; a[1][q] = R.Ap[i];
            } else {
                a[0][q] = src[i];
            }
        }
    }
    __device__ __forceinline__ void combine(const RhsVecs<T>& R, const long long (&o)[CH], cx<T> (&v)[CH], cx<T> alpha,
                                            cx<T> beta, cx<T> zeta) const {
#pragma unroll
        for (int q = 0; q < CH; q++) {
            v[q] = czero<T>();
            if (o[q] < 0) continue;
            const long long i = o[q];
            if constexpr (SRC == SRC_PUPD_DEF) {
                // the previous step's update (DDAModel.cpp:226-230), then p (DDAModel.cpp:219)
                const cx<T> Ap = a[0][q], r = a[1][q], p = a[2][q], t = a[3][q], At = a[4][q], P = a[5][q];
                const cx<T> u = cmul<T>(zeta, Ap);
                const cx<T> z = csub<T>(cmul<T>(zeta, r), cmul<T>(alpha, u));
                R.P[i] = cadd<T>(cadd<T>(P, cmul<T>(alpha, p)), z);
                const cx<T> rn = csub<T>(t, cmul<T>(zeta, At));
                R.r[i] = rn;
                v[q] = cadd<T>(rn, cmul<T>(beta, csub<T>(p, u)));
                R.p[i] = v[q];
            } else if constexpr (SRC == SRC_PUPD) {
                v[q] = cadd<T>(a[2][q], cmul<T>(beta, csub<T>(a[0][q], a[1][q])));  // p = r + beta (p - u)
                R.p[i] = v[q];
            } else if constexpr (SRC == SRC_TUPD) {
                v[q] = csub<T>(a[0][q], cmul<T>(alpha, a[1][q]));  // t = r - alpha Ap
                R.t[i] = v[q];
            } else {
                v[q] = a[0][q];
            }
            if constexpr (kPre) {  // the stored vectors stay unscaled; the grid gets D^-1 v
                if (R.pre) v[q] = cmul<T>(v[q], R.pre[i]);
            }
        }
    }
};
template <typename T, int SRC, int CH>
__device__ __forceinline__ void gather_chunk(const RhsVecs<T>& R, const long long (&o)[CH], cx<T> (&v)[CH],
                                             const cx<T>* src, cx<T> alpha, cx<T> beta, cx<T> zeta) {
    GatherIn<T, SRC, CH> in;
    in.load(R, o, src);
    in.combine(R, o, v, alpha, beta, zeta);
}

// Scatter of CH entries of one component (A v in val[q], dipole entry o[q] or
// -1) with the sink's diagonal term, stores and dot-product terms.  All loads come before
// the first store.
template <typename T, int SRC, int SNK, int CH, int NV>
__device__ __forceinline__ void scatter_chunk(const RhsVecs<T>& R, const long long (&o)[CH], const cx<T> (&val)[CH],
                                              acc_t<T> (&acc)[NV]) {
    const cx<T>* vsrc = (SRC == SRC_TUPD) ? R.t : (SRC == SRC_P ? R.P : R.p);
    cx<T> vv[CH], al[CH], q2[CH];
#pragma unroll
    for (int q = 0; q < CH; q++) {
        if (o[q] < 0) continue;
        if constexpr (SNK != SNK_OUT) { vv[q] = vsrc[o[q]]; al[q] = R.al[o[q]]; }
        if constexpr (SNK == SNK_AP || SNK == SNK_AT_DEF) q2[q] = R.r0[o[q]];
        if constexpr (SNK == SNK_RES) q2[q] = R.E[o[q]];
    }
#pragma unroll
    for (int q = 0; q < CH; q++) {
        if (o[q] < 0) continue;
        if constexpr (SNK == SNK_OUT) {
            R.Ap[o[q]] = val[q];
            continue;
        } else {
            const cx<T> w = cadd<T>(val[q], cmul<T>(vv[q], al[q]));
            if constexpr (SNK == SNK_ALB) {
                R.Ap[o[q]] = w;
            } else if constexpr (SNK == SNK_AP) {
                R.Ap[o[q]] = w;
                const cx<T> r0 = q2[q];  // r0 . Ap
                acc[0] += r0.x * w.x + r0.y * w.y;
                acc[1] += r0.x * w.y - r0.y * w.x;
            } else if constexpr (SNK == SNK_AT || SNK == SNK_AT_DEF) {
                R.At[o[q]] = w;
                const cx<T> t = vv[q];
                acc[0] += w.x * t.x + w.y * t.y;  // At . t
                acc[1] += w.x * t.y - w.y * t.x;
                acc[2] += w.x * w.x + w.y * w.y;  // At . At
                if constexpr (SNK == SNK_AT_DEF) {  // r0 . t, r0 . At, t . t
                    const cx<T> r0 = q2[q];
                    acc[3] += r0.x * t.x + r0.y * t.y;
                    acc[4] += r0.x * t.y - r0.y * t.x;
                    acc[5] += r0.x * w.x + r0.y * w.y;
                    acc[6] += r0.x * w.y - r0.y * w.x;
                    acc[7] += t.x * t.x + t.y * t.y;
                }
            } else {  // SNK_RES
                const cx<T> rr = csub<T>(q2[q], w);
                R.r[o[q]] = rr;
                R.r0[o[q]] = rr;
                R.p[o[q]] = rr;
                acc[0] += rr.x * rr.x + rr.y * rr.y;
            }
        }
    }
}

template <typename T, int MY, int MZ> struct ZyPlane {
    static constexpr int ZP = pad_odd(MZ);
    static constexpr int LY = (MY + 1) / 2;
    static constexpr int LZ = (MZ + 1) / 2;
    // twiddles, buffer A of My rows and buffer B of LY rows (the z stages and
    // the lattice side never need more than LY rows)
    static constexpr size_t smem = sizeof(cx<T>) * (size_t)(MY + MZ + (MY + LY) * ZP);
};

// Both axes use their two-stage plans (z: Mz = A1 A2, y: My = B1 B2): the
// first z stage gathers its inputs straight from the dipole vectors and the
// last y stage writes the grid (k_zyfwd); the first y stage reads the grid
// and the last z stage scatters straight to the dipoles (k_yzinv).  Three
// barriers per kernel.  Row-wise stages map consecutive threads to
// consecutive rows y (odd row stride ZP: no bank conflicts), column-wise
// stages to consecutive z.
template <typename T, int SRC, int MY, int MZ>
__global__ void __launch_bounds__(kNT) k_zyfwd(Geom g, const RhsVecs<T>* __restrict__ rhs,
                                               const cx<T>* __restrict__ twy, const cx<T>* __restrict__ twz,
                                               const int* __restrict__ cellmap, cx<T>* __restrict__ grid, int slot,
                                               int prod_nblk) {
    constexpr bool kStep32 = sizeof(T) == 4 && (SRC == SRC_PUPD_DEF || SRC == SRC_TUPD);
    using PL = ZyPlane<T, MY, MZ>;
    constexpr int A1 = ct_radix(MZ, 0, true), A2 = ct_radix(MZ, 1, true);
    constexpr int B1 = ct_radix(MY, 0, true), B2 = ct_radix(MY, 1, true);
    static_assert(ct_nstages(MZ, true) == 2 && ct_nstages(MY, true) == 2, "two-stage plans");
    constexpr int ZP = PL::ZP, LY = PL::LY;
    static_assert(!kStep32 || LY * ZP >= 8, "buffer B holds the scratch of the step scalars");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = blockIdx.y;
    const RhsVecs<T> R = rhs[b];
    const Lat L = lattice_of<T>(g, R, cellmap);
    const int x = blockIdx.x / 3, c = blockIdx.x - 3 * (blockIdx.x / 3);
    if (x >= L.Nx) return;  // past this right-hand side's lattice (cross-lattice batches)
    const int Ny = L.Ny, Nz = L.Nz;
    cx<T>* stwy = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* stwz = stwy + MY;
    cx<T>* sA = stwz + MZ;     // My rows
    cx<T>* sB = sA + MY * ZP;  // LY rows
    stage_tw<T>(stwy, twy, MY);
    stage_tw<T>(stwz, twz, MZ);
    grid_dep_wait();  // the vectors, partials and states are the previous kernels'
    if (g.early == 1) grid_dep_release();
    if constexpr (!kStep32) {  // the FP32 step reads the status with its scalars
        if (rhs_done(R.st)) return;
    }

    cx<T> beta, alpha, zeta;
    if constexpr (!kStep32) {
        if (SRC == SRC_PUPD || SRC == SRC_PUPD_DEF) beta = st_beta<T>(R.st);
        if (SRC == SRC_TUPD || SRC == SRC_PUPD_DEF) alpha = st_alpha<T>(R.st);
        if (SRC == SRC_PUPD_DEF) zeta = st_zeta<T>(R.st);
    }
    const cx<T>* src = SRC == SRC_IN ? R.p : R.P;
    const int* cm = L.cellmap + (long long)x * Ny * Nz;
    const int ibase = x * Ny * Nz;

    // gather: consecutive threads take consecutive cells (y, z), z fastest, in
    // chunks of CH cells whose loads are issued before their stores
    constexpr int LZ = PL::LZ, NCELL = LY * LZ, NE = (NCELL + kNT - 1) / kNT, CH = NE < 4 ? NE : 4;
#pragma unroll
    for (int c0 = 0; c0 < NE; c0 += CH) {
        int sidx[CH];
        long long o[CH];
#pragma unroll
        for (int q = 0; q < CH; q++) {
            const int e = threadIdx.x + (c0 + q) * kNT;
            const int y = e / LZ, z = e - (e / LZ) * LZ;
            const bool cell = c0 + q < NE && e < NCELL;
            sidx[q] = cell ? y * ZP + z : -1;
            int i = -1;
            if (cell && y < Ny && z < Nz) i = L.dense ? ibase + y * Nz + z : cm[y * Nz + z];
            o[q] = i >= 0 ? vec_index<T>(i, c, L.N) : -1LL;
        }
        GatherIn<T, SRC, CH> in;
        in.load(R, o, src);
        if constexpr (kStep32) {
            // the FP32 step scalars, formed while the first chunk's loads are in
            // flight (buffer B is free until the chunk's stores)
            if (c0 == 0 &&
                !fp32_step_scalars<SRC>(R, slot, prod_nblk, reinterpret_cast<float2*>(sB), alpha, beta, zeta))
                return;
        }
        cx<T> v[CH];
        in.combine(R, o, v, alpha, beta, zeta);
#pragma unroll
        for (int q = 0; q < CH; q++)
            if (sidx[q] >= 0) sB[sidx[q]] = v[q];
    }
    __syncthreads();  // also publishes the twiddles
    // z stage 1: task (y < LY, j < A2) reads z = j + A2 r < LZ (columns past LZ
    // are not gathered: zero), writes j A1 + q
    constexpr int RV = (LZ + A2 - 1) / A2;
    for (int w = threadIdx.x; w < LY * A2; w += kNT) {
        const int y = w % LY, j = w / LY;
        cx<T> v[A1];
#pragma unroll
        for (int r = 0; r < RV; r++) v[r] = j + A2 * r < LZ ? sB[y * ZP + j + A2 * r] : czero<T>();
        BflyIn<A1, -1, T, RV>::run(v);
#pragma unroll
        for (int q = 0; q < A1; q++) sA[y * ZP + j * A1 + q] = v[q];
    }
    __syncthreads();
    // z stage 2: task (y, j < A1) reads j + A1 r with twiddles w^(r j), writes j + A1 q
    for (int w = threadIdx.x; w < LY * A1; w += kNT) {
        const int y = w % LY, j = w / LY;
        cx<T> v[A2];
#pragma unroll
        for (int r = 0; r < A2; r++) {
            cx<T> t = sA[y * ZP + j + A1 * r];
            if (r > 0) t = cmul<T>(t, stwz[r * j]);
            v[r] = t;
        }
        Bfly<A2, -1, T>::run(v);
#pragma unroll
        for (int q = 0; q < A2; q++) sB[y * ZP + j + A1 * q] = v[q];
    }
    __syncthreads();
    // y stage 1: task (kz < Mz, j < B2) reads rows y = j + B2 r < Ny (r < RY:
    // Ny <= LY)
    constexpr int RY = (LY + B2 - 1) / B2;
    for (int w = threadIdx.x; w < MZ * B2; w += kNT) {
        const int kz = w % MZ, j = w / MZ;
        cx<T> v[B1];
#pragma unroll
        for (int r = 0; r < RY; r++) {
            const int y = j + B2 * r;
            v[r] = y < Ny ? sB[y * ZP + kz] : czero<T>();
        }
        BflyIn<B1, -1, T, RY>::run(v);
#pragma unroll
        for (int q = 0; q < B1; q++) sA[(j * B1 + q) * ZP + kz] = v[q];
    }
    __syncthreads();
    if (g.early == 2) grid_dep_release();  // the next kernel's blocks start during the last stage
    // y stage 2 to the grid plane [y][z]: task (kz, j < B1), rows j + B1 q
    cx<T>* gp = grid + (long long)b * g.sb + c * g.sc + (long long)x * g.sx;
    for (int w = threadIdx.x; w < MZ * B1; w += kNT) {
        const int kz = w % MZ, j = w / MZ;
        cx<T> v[B2];
#pragma unroll
        for (int r = 0; r < B2; r++) {
            cx<T> t = sA[(j + B1 * r) * ZP + kz];
            if (r > 0) t = cmul<T>(t, stwy[r * j]);
            v[r] = t;
        }
        Bfly<B2, -1, T>::run(v);
#pragma unroll
        for (int q = 0; q < B2; q++) gp[(long long)(j + B1 * q) * g.sy + kz] = v[q];
    }
}

template <typename T, int SRC, int SNK, int MY, int MZ>
__global__ void __launch_bounds__(kNT) k_yzinv(Geom g, const RhsVecs<T>* __restrict__ rhs,
                                               const cx<T>* __restrict__ twy, const cx<T>* __restrict__ twz,
                                               const int* __restrict__ cellmap, cx<T>* __restrict__ grid) {
    using PL = ZyPlane<T, MY, MZ>;
    constexpr int A1 = ct_radix(MZ, 0, true), A2 = ct_radix(MZ, 1, true);
    constexpr int B1 = ct_radix(MY, 0, true), B2 = ct_radix(MY, 1, true);
    static_assert(ct_nstages(MZ, true) == 2 && ct_nstages(MY, true) == 2, "two-stage plans");
    constexpr int ZP = PL::ZP, LY = PL::LY;
    constexpr int NV = SNK == SNK_AT_DEF ? 8 : 4;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double sred[sred_size<T, NV>()];
    const int b = blockIdx.y;
    const RhsVecs<T> R = rhs[b];
    const Lat L = lattice_of<T>(g, R, cellmap);
    const int x = blockIdx.x / 3, c = blockIdx.x - 3 * (blockIdx.x / 3);
    if (x >= L.Nx) {
        // past this right-hand side's lattice (cross-lattice batches): its sums over the
        // grid shape's blocks take zeros here, which leave them exactly as its own
        // blocks form them
        if (SNK == SNK_OUT || SNK == SNK_ALB) return;
        grid_dep_wait();
        acc_t<T> zero[NV] = {};
        if constexpr (sizeof(T) == 4 && (SNK == SNK_AP || SNK == SNK_AT_DEF)) {
            publish_partials<NV>(zero, R.part, gridDim.x, blockIdx.x, sred);
        } else {
            tot_t<T> tot[NV];
            const int slot = SNK == SNK_AP ? 0 : (SNK == SNK_AT || SNK == SNK_AT_DEF ? 1 : 2);
            if (last_block_total<NV>(zero, R.part, gridDim.x, blockIdx.x, R.cnt + slot, sred, tot) &&
                threadIdx.x == 0)
                finalize_sink<T, SNK, NV>(R.st, tot);
        }
        return;
    }
    const int nblk = gridDim.x;
    const int Ny = L.Ny, Nz = L.Nz;
    cx<T>* stwy = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* stwz = stwy + MY;
    cx<T>* sA = stwz + MZ;     // My rows
    cx<T>* sB = sA + MY * ZP;  // LY rows
    stage_tw<T>(stwy, twy, MY);
    stage_tw<T>(stwz, twz, MZ);
    const cx<T>* gp = grid + (long long)b * g.sb + c * g.sc + (long long)x * g.sx;
    grid_dep_wait();  // the grid and the solve's state are the previous kernel's
    if (g.early == 1) grid_dep_release();

    // y stage 1 on the grid plane: task (kz < Mz, j < B2) reads rows j + B2 r
    for (int w = threadIdx.x; w < MZ * B2; w += kNT) {
        const int kz = w % MZ, j = w / MZ;
        cx<T> v[B1];
#pragma unroll
        for (int r = 0; r < B1; r++) v[r] = gp[(long long)(j + B2 * r) * g.sy + kz];
        Bfly<B1, +1, T>::run(v);
#pragma unroll
        for (int q = 0; q < B1; q++) sA[(j * B1 + q) * ZP + kz] = v[q];
    }
    // a stopped solve is checked here, after the plane's loads are issued:
    // nothing has been written to global memory yet
    if (rhs_done(R.st)) return;
    __syncthreads();  // also publishes the twiddles
    // y stage 2: task (kz, j < B1), twiddles conj(w^(r j)), rows j + B1 q < Ny kept
    for (int w = threadIdx.x; w < MZ * B1; w += kNT) {
        const int kz = w % MZ, j = w / MZ;
        cx<T> v[B2];
#pragma unroll
        for (int r = 0; r < B2; r++) {
            cx<T> t = sA[(j + B1 * r) * ZP + kz];
            if (r > 0) {
                cx<T> tw = stwy[r * j];
                tw.y = -tw.y;
                t = cmul<T>(t, tw);
            }
            v[r] = t;
        }
        Bfly<B2, +1, T>::run(v);
        constexpr int QY = (LY + B1 - 1) / B1;  // rows past LY >= Ny are never kept
#pragma unroll
        for (int q = 0; q < QY; q++) {
            const int y = j + B1 * q;
            if (y < Ny) sB[y * ZP + kz] = v[q];
        }
    }
    __syncthreads();
    // z stage 1 on the rows y < Ny: task (y, j < A2) reads z = j + A2 r
    for (int w = threadIdx.x; w < LY * A2; w += kNT) {
        const int y = w % LY, j = w / LY;
        if (y >= Ny) continue;
        cx<T> v[A1];
#pragma unroll
        for (int r = 0; r < A1; r++) v[r] = sB[y * ZP + j + A2 * r];
        Bfly<A1, +1, T>::run(v);
#pragma unroll
        for (int q = 0; q < A1; q++) sA[y * ZP + j * A1 + q] = v[q];
    }
    __syncthreads();
    if (g.early == 2) grid_dep_release();  // the next kernel's blocks start during the last stage
    // z stage 2: task (y, j < A1), twiddles conj(w^(r j)), outputs z = j + A1 q < LZ
    constexpr int LZ = PL::LZ, QV = (LZ + A1 - 1) / A1;
    for (int w = threadIdx.x; w < LY * A1; w += kNT) {
        const int y = w % LY, j = w / LY;
        if (y >= Ny) continue;
        cx<T> v[A2];
#pragma unroll
        for (int r = 0; r < A2; r++) {
            cx<T> t = sA[y * ZP + j + A1 * r];
            if (r > 0) {
                cx<T> tw = stwz[r * j];
                tw.y = -tw.y;
                t = cmul<T>(t, tw);
            }
            v[r] = t;
        }
        Bfly<A2, +1, T>::run(v);
#pragma unroll
        for (int q = 0; q < QV; q++)
            if (j + A1 * q < LZ) sB[y * ZP + j + A1 * q] = v[q];
    }
    __syncthreads();
    // scatter component c: consecutive threads take consecutive cells (y, z),
    // in chunks of CH whose loads are issued before their stores
    const int* cm = L.cellmap + (long long)x * Ny * Nz;
    const int ibase = x * Ny * Nz;
    acc_t<T> acc[NV] = {};
    // the sink's operand loads of all the thread's cells at once, up to 9 cells
    constexpr int NCELL = LY * LZ, NE = (NCELL + kNT - 1) / kNT;
    constexpr int CH = (SNK != SNK_OUT && NE <= 9) || NE < 4 ? NE : 4;
#pragma unroll
    for (int c0 = 0; c0 < NE; c0 += CH) {
        long long o[CH];
        cx<T> vo[CH];
#pragma unroll
        for (int q = 0; q < CH; q++) {
            const int e = threadIdx.x + (c0 + q) * kNT;
            const int y = e / LZ, z = e - (e / LZ) * LZ;
            const bool cell = c0 + q < NE && e < NCELL && y < Ny && z < Nz;
            int i = -1;
            if (cell) i = L.dense ? ibase + y * Nz + z : cm[y * Nz + z];
            o[q] = i >= 0 ? vec_index<T>(i, c, L.N) : -1LL;
            vo[q] = i >= 0 ? sB[y * ZP + z] : czero<T>();
        }
        scatter_chunk<T, SRC, SNK, CH, NV>(R, o, vo, acc);
    }
    if (SNK == SNK_OUT || SNK == SNK_ALB) return;
    if constexpr (sizeof(T) == 4 && (SNK == SNK_AP || SNK == SNK_AT_DEF)) {
        publish_partials<NV>(acc, R.part, nblk, blockIdx.x, sred);  // the next gather forms the scalars
        return;
    }
    tot_t<T> tot[NV];
    const int slot = SNK == SNK_AP ? 0 : (SNK == SNK_AT || SNK == SNK_AT_DEF ? 1 : 2);
    if (!last_block_total<NV>(acc, R.part, nblk, blockIdx.x, R.cnt + slot, sred, tot)) return;
    if (threadIdx.x != 0) return;
    finalize_sink<T, SNK, NV>(R.st, tot);
}

template <typename T, int MY, int MZ> struct ZyLaunch {
    // pass: PASS_ZFWD (k_zyfwd, mode = SrcMode) or PASS_ZINV (k_yzinv, mode = SnkMode)
    static cudaError_t run(int pass, int mode, const PassArgs<T>& a) {
        const dim3 grid(3 * a.g.Nx, a.nrhs);
        const size_t sm = ZyPlane<T, MY, MZ>::smem;
        const Geom g = early_geom(a.g, (long long)grid.x * grid.y);
        cudaError_t e = cudaSuccess;
        if (pass == PASS_ZFWD) {
            switch (mode) {
                case SRC_IN: e = launch_early(g.early, k_zyfwd<T, SRC_IN, MY, MZ>, grid, dim3(kNT), sm, a.stream, g, a.rhs, a.twy, a.twz, a.cellmap, a.grid, a.slot, a.prod_nblk); break;
                case SRC_PUPD: e = launch_early(g.early, k_zyfwd<T, SRC_PUPD, MY, MZ>, grid, dim3(kNT), sm, a.stream, g, a.rhs, a.twy, a.twz, a.cellmap, a.grid, a.slot, a.prod_nblk); break;
                case SRC_TUPD: e = launch_early(g.early, k_zyfwd<T, SRC_TUPD, MY, MZ>, grid, dim3(kNT), sm, a.stream, g, a.rhs, a.twy, a.twz, a.cellmap, a.grid, a.slot, a.prod_nblk); break;
                case SRC_PUPD_DEF: e = launch_early(g.early, k_zyfwd<T, SRC_PUPD_DEF, MY, MZ>, grid, dim3(kNT), sm, a.stream, g, a.rhs, a.twy, a.twz, a.cellmap, a.grid, a.slot, a.prod_nblk); break;
                default: e = launch_early(g.early, k_zyfwd<T, SRC_P, MY, MZ>, grid, dim3(kNT), sm, a.stream, g, a.rhs, a.twy, a.twz, a.cellmap, a.grid, a.slot, a.prod_nblk); break;
            }
        } else {
            switch (mode) {
                case SNK_OUT: e = launch_early(g.early, k_yzinv<T, SRC_IN, SNK_OUT, MY, MZ>, grid, dim3(kNT), sm, a.stream, g, a.rhs, a.twy, a.twz, a.cellmap, a.grid); break;
                case SNK_ALB: e = launch_early(g.early, k_yzinv<T, SRC_IN, SNK_ALB, MY, MZ>, grid, dim3(kNT), sm, a.stream, g, a.rhs, a.twy, a.twz, a.cellmap, a.grid); break;
                case SNK_AP: e = launch_early(g.early, k_yzinv<T, SRC_PUPD, SNK_AP, MY, MZ>, grid, dim3(kNT), sm, a.stream, g, a.rhs, a.twy, a.twz, a.cellmap, a.grid); break;
                case SNK_AT: e = launch_early(g.early, k_yzinv<T, SRC_TUPD, SNK_AT, MY, MZ>, grid, dim3(kNT), sm, a.stream, g, a.rhs, a.twy, a.twz, a.cellmap, a.grid); break;
                case SNK_AT_DEF: e = launch_early(g.early, k_yzinv<T, SRC_TUPD, SNK_AT_DEF, MY, MZ>, grid, dim3(kNT), sm, a.stream, g, a.rhs, a.twy, a.twz, a.cellmap, a.grid); break;
                default: e = launch_early(g.early, k_yzinv<T, SRC_P, SNK_RES, MY, MZ>, grid, dim3(kNT), sm, a.stream, g, a.rhs, a.twy, a.twz, a.cellmap, a.grid); break;
            }
        }
        return e != cudaSuccess ? e : cudaGetLastError();
    }
    static cudaError_t configure() {
        const void* ks[] = {(const void*)k_zyfwd<T, SRC_IN, MY, MZ>, (const void*)k_zyfwd<T, SRC_PUPD, MY, MZ>,
                            (const void*)k_zyfwd<T, SRC_TUPD, MY, MZ>, (const void*)k_zyfwd<T, SRC_P, MY, MZ>,
                            (const void*)k_zyfwd<T, SRC_PUPD_DEF, MY, MZ>, (const void*)k_yzinv<T, SRC_TUPD, SNK_AT_DEF, MY, MZ>,
                            (const void*)k_yzinv<T, SRC_IN, SNK_OUT, MY, MZ>, (const void*)k_yzinv<T, SRC_IN, SNK_ALB, MY, MZ>,
                            (const void*)k_yzinv<T, SRC_PUPD, SNK_AP, MY, MZ>, (const void*)k_yzinv<T, SRC_TUPD, SNK_AT, MY, MZ>,
                            (const void*)k_yzinv<T, SRC_P, SNK_RES, MY, MZ>};
        for (const void* k : ks) {
            cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxPassSmem);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
};

// ------------------------------------------------------------ launchers
// Launches pass `pass` (PASS_*) of an A-product for the length CM (0: runtime).
template <typename T, int CM> struct PassLaunch {
    static cudaError_t run(int pass, int mode, const PassArgs<T>& a) {
        if (pass == PASS_ZFWD || pass == PASS_ZINV) return run_z(pass, mode, a);
        if (pass == PASS_YFWD || pass == PASS_YINV) return run_y(pass, a);
        return run_x(a);
    }
    static cudaError_t run_z(int pass, int mode, const PassArgs<T>& a) {
        const Geom& g = a.g;
        {
            const int Mz = CM > 0 ? CM : g.pz.M;
            const int LZ = z_lines<T>(Mz);
            const dim3 grid((g.Nx * g.Ny + LZ - 1) / LZ, a.nrhs);
            const size_t sm = zsmem<T>(Mz);
            if constexpr (is_dd<T>) {  // the double-float product forms residuals only
                if (pass == PASS_ZFWD) {
                    k_zfwd<T, SRC_P, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid, a.slot,
                                                                      a.prod_nblk);
                } else {
                    k_zinv<T, SRC_P, SNK_RES, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid);
                }
                return cudaGetLastError();
            }
            if (pass == PASS_ZFWD) {
                switch (mode) {
                    case SRC_IN: k_zfwd<T, SRC_IN, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid, a.slot, a.prod_nblk); break;
                    case SRC_PUPD: k_zfwd<T, SRC_PUPD, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid, a.slot, a.prod_nblk); break;
                    case SRC_TUPD: k_zfwd<T, SRC_TUPD, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid, a.slot, a.prod_nblk); break;
                    case SRC_PUPD_DEF: k_zfwd<T, SRC_PUPD_DEF, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid, a.slot, a.prod_nblk); break;
                    default: k_zfwd<T, SRC_P, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid, a.slot, a.prod_nblk); break;
                }
            } else {
                switch (mode) {
                    case SNK_OUT: k_zinv<T, SRC_IN, SNK_OUT, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid); break;
                    case SNK_ALB: k_zinv<T, SRC_IN, SNK_ALB, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid); break;
                    case SNK_AP: k_zinv<T, SRC_PUPD, SNK_AP, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid); break;
                    case SNK_AT: k_zinv<T, SRC_TUPD, SNK_AT, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid); break;
                    case SNK_AT_DEF: k_zinv<T, SRC_TUPD, SNK_AT_DEF, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid); break;
                    default: k_zinv<T, SRC_P, SNK_RES, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid); break;
                }
            }
        }
        return cudaGetLastError();
    }
    static cudaError_t run_y(int pass, const PassArgs<T>& a) {
        const Geom& g = a.g;
        {
            const int My = CM > 0 ? CM : g.py.M;
            const int YT = y_tile<T>(My);
            const dim3 grid(g.Nx * ((g.pz.M + YT - 1) / YT), 3, a.nrhs);
            const size_t sm = ysmem<T>(My);
            if (pass == PASS_YFWD) k_ypass<T, -1, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twy, a.grid);
            else k_ypass<T, +1, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twy, a.grid);
        }
        return cudaGetLastError();
    }
    static cudaError_t run_x(const PassArgs<T>& a) {
        const Geom& g = a.g;
        {
            const int Mx = CM > 0 ? CM : g.px.M;
            const int XT = x_tile<T>(Mx);
            const dim3 grid(g.py.M * ((g.pz.M + XT - 1) / XT), a.nrhs);
            k_xpass<T, CM><<<grid, kNT, xsmem<T>(Mx), a.stream>>>(g, a.rhs, a.green, a.twx, a.grid);
        }
        return cudaGetLastError();
    }

    // raise the dynamic shared-memory limit of the kernels of this length
    static cudaError_t set_attr(const void* k) {
        return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxPassSmem);
    }
    static cudaError_t configure_z() {
        if constexpr (is_dd<T>) {
            cudaError_t e = set_attr((const void*)k_zfwd<T, SRC_P, CM>);
            return e != cudaSuccess ? e : set_attr((const void*)k_zinv<T, SRC_P, SNK_RES, CM>);
        }
        const void* ks[] = {(const void*)k_zfwd<T, SRC_IN, CM>, (const void*)k_zfwd<T, SRC_PUPD, CM>,
                            (const void*)k_zfwd<T, SRC_TUPD, CM>, (const void*)k_zfwd<T, SRC_P, CM>,
                            (const void*)k_zfwd<T, SRC_PUPD_DEF, CM>, (const void*)k_zinv<T, SRC_TUPD, SNK_AT_DEF, CM>,
                            (const void*)k_zinv<T, SRC_IN, SNK_OUT, CM>, (const void*)k_zinv<T, SRC_IN, SNK_ALB, CM>,
                            (const void*)k_zinv<T, SRC_PUPD, SNK_AP, CM>, (const void*)k_zinv<T, SRC_TUPD, SNK_AT, CM>,
                            (const void*)k_zinv<T, SRC_P, SNK_RES, CM>};
        for (const void* k : ks) {
            cudaError_t e = set_attr(k);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
    static cudaError_t configure_xy() {
        const void* ks[] = {(const void*)k_ypass<T, -1, CM>, (const void*)k_ypass<T, +1, CM>,
                            (const void*)k_xpass<T, CM>};
        for (const void* k : ks) {
            cudaError_t e = set_attr(k);
            if (e != cudaSuccess) return e;
        }
        return cudaSuccess;
    }
};

}  // namespace dev
}  // namespace tdda
