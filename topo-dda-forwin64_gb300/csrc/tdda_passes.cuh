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

// ------------------------------------------------------------ K1 zfwd
template <typename T, int SRC, int CM>
__global__ void __launch_bounds__(kNT) k_zfwd(Geom g, const RhsVecs<T>* __restrict__ rhs,
                                              const cx<T>* __restrict__ twz, const int* __restrict__ cellmap,
                                              cx<T>* __restrict__ grid) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = blockIdx.y;
    const RhsVecs<T> R = rhs[b];
    if (rhs_done(R.st)) return;
    constexpr int cLZ = CM > 0 ? z_lines<T>(CM) : 1;
    constexpr int cMzP = CM > 0 ? pad_odd(CM) : 1;
    const int Mz = CM > 0 ? CM : g.pz.M, Nz = g.Nz;
    const int LZ = CM > 0 ? cLZ : z_lines<T>(Mz), MzP = CM > 0 ? cMzP : pad_odd(Mz);
    cx<T>* stw = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* s = stw + Mz;
    cx<T>* s2 = s + 3 * LZ * MzP;
    stage_tw<T>(stw, twz, Mz);
    const int nlines = g.Nx * g.Ny;
    const int l0 = blockIdx.x * LZ;
    const int nl = min(LZ, nlines - l0);

    cx<T> beta, alpha;
    if (SRC == SRC_PUPD) beta = from_d<T>(R.st->beta);
    if (SRC == SRC_TUPD) alpha = from_d<T>(R.st->alpha);
    const cx<T>* src = SRC == SRC_IN ? R.p : R.P;
    for (int e = threadIdx.x; e < nl * Nz; e += blockDim.x) {
        const int line = e / Nz, z = e - (e / Nz) * Nz;
        const int i = cellmap[(long long)(l0 + line) * Nz + z];
        cx<T> v[3];
        if (i >= 0) {
            const long long o = 3LL * i;
#pragma unroll
            for (int c = 0; c < 3; c++) {
                if (SRC == SRC_PUPD) {
                    cx<T> pc = R.p[o + c], uc = R.u[o + c], rc = R.r[o + c];
                    v[c] = cadd<T>(rc, cmul<T>(beta, csub<T>(pc, uc)));
                    R.p[o + c] = v[c];
                } else if (SRC == SRC_TUPD) {
                    cx<T> rc = R.r[o + c], ac = R.Ap[o + c];
                    v[c] = csub<T>(rc, cmul<T>(alpha, ac));
                    R.t[o + c] = v[c];
                } else {
                    v[c] = src[o + c];
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
    if constexpr (CM > 0) res = ct_fft<-1, T, CM, 3 * cLZ, cMzP, 1, kNT>(s, s2, stw, Nz, CM);
    else res = smem_fft<-1, T>(s, s2, 3 * LZ, MzP, 1, g.pz, stw, Nz, Mz);
    cx<T>* gb = grid + (long long)b * g.sb;
    for (int e = threadIdx.x; e < 3 * nl * Mz; e += blockDim.x) {
        const int cl = e / Mz, z = e - (e / Mz) * Mz;
        const int c = cl / nl, line = cl - (cl / nl) * nl;
        const int l = l0 + line, x = l / g.Ny, y = l - (l / g.Ny) * g.Ny;
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
    const int c = blockIdx.y;
    const int zn = min(ZT, Mz - z0);
    cx<T>* stw = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* s = stw + My;
    const int ZP = ZT + 1;  // padded row stride: consecutive rows start in different banks
    cx<T>* s2 = s + My * ZP;
    stage_tw<T>(stw, twy, My);
    cx<T>* gp = grid + (long long)b * g.sb + c * g.sc + (long long)x * g.sx + z0;
    const int nin = SIGN < 0 ? g.Ny : My;
    const int nout = SIGN < 0 ? My : g.Ny;
    for (int e = threadIdx.x; e < nin * ZT; e += blockDim.x) {
        const int y = e / ZT, zl = e - (e / ZT) * ZT;
        if (zl < zn) s[y * ZP + zl] = gp[(long long)y * g.sy + zl];
    }
    __syncthreads();
    const cx<T>* res;
    if constexpr (CM > 0) res = ct_fft<SIGN, T, CM, cZT, 1, cZT + 1, kNT>(s, s2, stw, nin, nout);
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
    if constexpr (sizeof(cx<T>) == 8) {
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

template <typename T, int CM>
__global__ void __launch_bounds__(kNT) k_xpass(Geom g, const RhsVecs<T>* __restrict__ rhs,
                                               const cx<T>* __restrict__ green, const cx<T>* __restrict__ twx,
                                               cx<T>* __restrict__ grid) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int b = blockIdx.y;
    if (rhs_done(rhs[b].st)) return;
    constexpr int cZT = CM > 0 ? x_tile<T>(CM) : 1;
    const int Mx = CM > 0 ? CM : g.px.M, My = g.py.M, Mz = g.pz.M, Nx = g.Nx;
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
    if constexpr (CM > 0) res = ct_fft<-1, T, CM, 3 * cZT, 1, 3 * cZT + 1, kNT>(s, s2, stw, Nx, CM);
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
        const cx<T>* gg = green + (((long long)fy * g.Hx + fx) * g.Hz + fz) * 6;
        cx<T> a0, a1, a2, a3, a4, a5;
        load_green6<T>(gg, a0, a1, a2, a3, a4, a5);
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
    if constexpr (CM > 0) out = ct_fft<+1, T, CM, 3 * cZT, 1, 3 * cZT + 1, kNT>(res, other, stw, CM, Nx);
    else out = smem_fft<+1, T>(res, other, W, 1, WP, g.px, stw, Mx, Nx);
    for (int e = threadIdx.x; e < Nx * W; e += blockDim.x) {
        const int x = e / W, r = e - (e / W) * W;
        const int c = r / ZT, zl = r - (r / ZT) * ZT;
        if (zl < zn) gp[c * g.sc + (long long)x * g.sx + zl] = out[x * WP + r];
    }
}

// ------------------------------------------------------------ K5 zinv
template <typename T, int SRC, int SNK, int CM>
__global__ void __launch_bounds__(kNT) k_zinv(Geom g, const RhsVecs<T>* __restrict__ rhs,
                                              const cx<T>* __restrict__ twz, const int* __restrict__ cellmap,
                                              cx<T>* __restrict__ grid) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double sred[4 * kNT];
    const int b = blockIdx.y;
    const RhsVecs<T> R = rhs[b];
    if (rhs_done(R.st)) return;
    constexpr int cLZ = CM > 0 ? z_lines<T>(CM) : 1;
    constexpr int cMzP = CM > 0 ? pad_odd(CM) : 1;
    const int Mz = CM > 0 ? CM : g.pz.M, Nz = g.Nz;
    const int LZ = CM > 0 ? cLZ : z_lines<T>(Mz), MzP = CM > 0 ? cMzP : pad_odd(Mz);
    cx<T>* stw = reinterpret_cast<cx<T>*>(smem_raw);
    cx<T>* s = stw + Mz;
    cx<T>* s2 = s + 3 * LZ * MzP;
    stage_tw<T>(stw, twz, Mz);
    const int nlines = g.Nx * g.Ny;
    const int l0 = blockIdx.x * LZ;
    const int nl = min(LZ, nlines - l0);
    const cx<T>* gb = grid + (long long)b * g.sb;
    for (int e = threadIdx.x; e < 3 * nl * Mz; e += blockDim.x) {
        const int cl = e / Mz, z = e - (e / Mz) * Mz;
        const int c = cl / nl, line = cl - (cl / nl) * nl;
        const int l = l0 + line, x = l / g.Ny, y = l - (l / g.Ny) * g.Ny;
        s[(c * LZ + line) * MzP + z] = gb[c * g.sc + x * g.sx + y * g.sy + z];
    }
    __syncthreads();
    const cx<T>* res;
    if constexpr (CM > 0) res = ct_fft<+1, T, CM, 3 * cLZ, cMzP, 1, kNT>(s, s2, stw, CM, Nz);
    else res = smem_fft<+1, T>(s, s2, 3 * LZ, MzP, 1, g.pz, stw, Mz, Nz);

    // scatter to the dipoles, fused diagonal term and dot products
    const cx<T>* vsrc = (SRC == SRC_TUPD) ? R.t : (SRC == SRC_P ? R.P : R.p);
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int e = threadIdx.x; e < nl * Nz; e += blockDim.x) {
        const int line = e / Nz, z = e - (e / Nz) * Nz;
        const int i = cellmap[(long long)(l0 + line) * Nz + z];
        if (i < 0) continue;
        const long long o = 3LL * i;
#pragma unroll
        for (int c = 0; c < 3; c++) {
            cx<T> val = res[(c * LZ + line) * MzP + z];
            if (SNK == SNK_OUT) {
                R.Ap[o + c] = val;
                continue;
            }
            const cx<T> vv = vsrc[o + c];
            const cx<T> w = cadd<T>(val, cmul<T>(vv, R.al[o + c]));
            if (SNK == SNK_ALB) {
                R.Ap[o + c] = w;
            } else if (SNK == SNK_AP) {
                R.Ap[o + c] = w;
                const cx<T> q = R.r0[o + c];  // r0 . Ap
                acc[0] += (double)q.x * (double)w.x + (double)q.y * (double)w.y;
                acc[1] += (double)q.x * (double)w.y - (double)q.y * (double)w.x;
            } else if (SNK == SNK_AT) {
                R.At[o + c] = w;
                const cx<T> tt = vv;  // At . t and At . At
                acc[0] += (double)w.x * (double)tt.x + (double)w.y * (double)tt.y;
                acc[1] += (double)w.x * (double)tt.y - (double)w.y * (double)tt.x;
                acc[2] += (double)w.x * (double)w.x + (double)w.y * (double)w.y;
            } else if (SNK == SNK_RES) {
                const cx<T> res = csub<T>(R.E[o + c], w);
                R.r[o + c] = res;
                R.r0[o + c] = res;
                R.p[o + c] = res;
                acc[0] += (double)res.x * (double)res.x + (double)res.y * (double)res.y;
            }
        }
    }
    if (SNK == SNK_OUT || SNK == SNK_ALB) return;
    double tot[4];
    const int nblk = gridDim.x;
    const int slot = SNK == SNK_AP ? 0 : (SNK == SNK_AT ? 1 : 2);
    if (!last_block_total<4>(acc, R.part, nblk, blockIdx.x, R.cnt + slot, sred, tot)) return;
    if (threadIdx.x != 0) return;
    SolveState* st = R.st;
    if (SNK == SNK_AP) {
        double2 r0Ap = make_double2(tot[0], tot[1]);
        st->alpha = cdiv(st->rho, r0Ap);  // DDAModel.cpp:221
    } else if (SNK == SNK_AT) {
        st->zeta = cdiv(make_double2(tot[0], tot[1]), make_double2(tot[2], 0.0));  // DDAModel.cpp:225
    } else {
        st->rho = make_double2(tot[0], 0.0);  // r0 . r with r0 = r
        st->rnorm2 = tot[0];
    }
}

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
            if (pass == PASS_ZFWD) {
                switch (mode) {
                    case SRC_IN: k_zfwd<T, SRC_IN, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid); break;
                    case SRC_PUPD: k_zfwd<T, SRC_PUPD, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid); break;
                    case SRC_TUPD: k_zfwd<T, SRC_TUPD, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid); break;
                    default: k_zfwd<T, SRC_P, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid); break;
                }
            } else {
                switch (mode) {
                    case SNK_OUT: k_zinv<T, SRC_IN, SNK_OUT, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid); break;
                    case SNK_ALB: k_zinv<T, SRC_IN, SNK_ALB, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid); break;
                    case SNK_AP: k_zinv<T, SRC_PUPD, SNK_AP, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid); break;
                    case SNK_AT: k_zinv<T, SRC_TUPD, SNK_AT, CM><<<grid, kNT, sm, a.stream>>>(g, a.rhs, a.twz, a.cellmap, a.grid); break;
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
        const void* ks[] = {(const void*)k_zfwd<T, SRC_IN, CM>, (const void*)k_zfwd<T, SRC_PUPD, CM>,
                            (const void*)k_zfwd<T, SRC_TUPD, CM>, (const void*)k_zfwd<T, SRC_P, CM>,
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
