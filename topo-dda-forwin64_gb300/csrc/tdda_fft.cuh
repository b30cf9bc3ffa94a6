// tdda_fft.cuh -- complex helpers and the shared-memory Stockham FFT used by
// every pass of the A-product (sm_103a; float and double instantiations).
//
// A pass kernel stages a tile of L independent lines of length M in shared
// memory (line l at s + l*ls, element m at + m*ms) and calls smem_fft().  Each
// radix-R stage maps butterfly j of every line (Stockham autosort, span Ns):
//     k = j mod Ns,  v[r] = x[j + r M/R] * W^(r k M/(Ns R)),  V = DFT_R(v),
//     y[(j-k) R + k + q Ns] = V[q]
// from one shared buffer to the other (ping-pong), one barrier per stage.
// The radix-2/3/4/5/7/8 butterflies are written from the DFT definition; the
// twiddle table W[m] = exp(-2 pi i m / M) is computed on the host in extended
// precision and staged into shared memory by the kernel.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace tdda {

template <typename T> struct cplx_t;
template <> struct cplx_t<float> { typedef float2 type; };
template <> struct cplx_t<double> { typedef double2 type; };

// Double-float scalar: an unevaluated sum hi + lo of two FP32 values (about 44
// significant bits), for products that need more than FP32 and run on the
// FP32 pipes.  Addition is the TwoSum of the high parts with the low parts
// added (D. E. Knuth, TAOCP vol. 2, 4.2.2; the "sloppy" double-double add of
// Hida, Li and Bailey's QD library): its error is bounded by about 2^-44 of
// |a| + |b|, the bound an FFT needs.  Multiplication takes the exact error of
// hi*hi from one FMA (Dekker's product with a fused multiply-add).  Every
// operation is rounded explicitly, so no contraction or reordering applies.
struct dd {
    float hi, lo;
    __host__ __device__ dd() {}
    __host__ __device__ constexpr dd(float h, float l) : hi(h), lo(l) {}
    __host__ __device__ dd(double v) : hi((float)v), lo((float)(v - (double)(float)v)) {}
    __host__ __device__ dd(int v) : dd((double)v) {}
    __host__ __device__ operator double() const { return (double)hi + (double)lo; }
};
__device__ __forceinline__ dd dd_fast2sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return dd(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ dd operator+(dd a, dd b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bp = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bp)), __fsub_rn(b.hi, bp));
    return dd_fast2sum(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ dd operator-(dd a) { return dd(-a.hi, -a.lo); }
__device__ __forceinline__ dd operator-(dd a, dd b) { return a + (-b); }
__device__ __forceinline__ dd operator*(dd a, dd b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return dd_fast2sum(p, e);
}
__device__ __forceinline__ dd& operator+=(dd& a, dd b) { return a = a + b; }
// complex double-float: 16 bytes, (re.hi, re.lo, im.hi, im.lo)
struct __align__(16) dd2 {
    dd x, y;
    __host__ __device__ dd2() {}
    __host__ __device__ dd2(dd re, dd im) : x(re), y(im) {}
    __host__ __device__ dd2(double2 v) : x(v.x), y(v.y) {}
    __host__ __device__ explicit dd2(float4 v) : x(v.x, v.y), y(v.z, v.w) {}
    __host__ __device__ double2 to_double2() const { return make_double2((double)x, (double)y); }
};
template <> struct cplx_t<dd> { typedef dd2 type; };
template <typename T> constexpr bool is_dd = false;
template <> constexpr bool is_dd<dd> = true;

template <typename T> using cx = typename cplx_t<T>::type;

template <typename T> __host__ __device__ __forceinline__ cx<T> mk(T re, T im) {
    cx<T> c;
    c.x = re;
    c.y = im;
    return c;
}
template <typename T> __device__ __forceinline__ cx<T> cadd(cx<T> a, cx<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ cx<T> csub(cx<T> a, cx<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T> __device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
    return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// conj(a) * b
template <typename T> __device__ __forceinline__ cx<T> cmulc(cx<T> a, cx<T> b) {
    return mk<T>(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
template <typename T> __device__ __forceinline__ cx<T> cscale(cx<T> a, T s) { return mk<T>(a.x * s, a.y * s); }
// multiply by (sign * i): sign = -1 gives -i (forward), +1 gives +i (inverse)
template <int SIGN, typename T> __device__ __forceinline__ cx<T> cmul_i(cx<T> a) {
    return SIGN < 0 ? mk<T>(a.y, -a.x) : mk<T>(-a.y, a.x);
}
template <typename T> __device__ __forceinline__ cx<T> czero() { return mk<T>(T(0), T(0)); }

// Butterfly arithmetic.  For FP32 the real and imaginary parts of a complex
// value are one 64-bit register pair, and sm_100-family GPUs add, subtract and
// fused-multiply-add such pairs in one instruction (PTX add / sub / fma.rn.f32x2):
// each is exactly two rn operations, so the results are those of the scalar
// forms, at half the instruction count.  Other types use the scalar forms.
__device__ __forceinline__ unsigned long long f2_pack(float2 a) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
    return r;
}
__device__ __forceinline__ float2 f2_unpack(unsigned long long r) {
    float2 a;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
    return a;
}
template <typename T> __device__ __forceinline__ cx<T> badd(cx<T> a, cx<T> b) { return cadd<T>(a, b); }
template <typename T> __device__ __forceinline__ cx<T> bsub(cx<T> a, cx<T> b) { return csub<T>(a, b); }
// acc + c a for a real constant c
template <typename T> __device__ __forceinline__ cx<T> bfma(cx<T> a, T c, cx<T> acc) {
    return mk<T>(acc.x + c * a.x, acc.y + c * a.y);
}
template <> __device__ __forceinline__ float2 badd<float>(float2 a, float2 b) {
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
    return f2_unpack(r);
}
template <> __device__ __forceinline__ float2 bsub<float>(float2 a, float2 b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(b)));
    return f2_unpack(r);
}
template <> __device__ __forceinline__ float2 bfma<float>(float2 a, float c, float2 acc) {
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(f2_pack(a)), "l"(f2_pack(make_float2(c, c))),
        "l"(f2_pack(acc)));
    return f2_unpack(r);
}

// Up to 8 radix stages per axis (M <= 8^8 is far beyond any lattice here).
constexpr int kMaxStages = 8;

// Exact unsigned division by a fixed divisor d via a 32x32 multiply-high:
// q = umulhi(n, ceil(2^32 / d)) equals floor(n / d) whenever n * d < 2^32,
// which every index here satisfies (n < 2^20, d <= 2^11).
struct FastDiv {
    unsigned d, m;  // m = 0 encodes d = 1
};
__host__ __device__ inline FastDiv fastdiv_make(unsigned d) {
    FastDiv f;
    f.d = d;
    f.m = d <= 1 ? 0u : (unsigned)(((1ull << 32) + d - 1) / d);
    return f;
}
__device__ __forceinline__ unsigned fastdiv(unsigned n, FastDiv f) { return f.m ? __umulhi(n, f.m) : n; }

struct AxisPlan {
    int M;                  // FFT length
    int nstages;
    int radix[kMaxStages];  // applied first to last
    int rmin;               // smallest radix
    FastDiv ns[kMaxStages]; // division by the span Ns of each stage
};

// ---------------------------------------------------------------- butterflies
// In-place DFT of v[0..R-1]: V[q] = sum_r v[r] exp(SIGN 2 pi i r q / R).
template <int R, int SIGN, typename T> struct Bfly;

template <int SIGN, typename T> struct Bfly<2, SIGN, T> {
    static __device__ __forceinline__ void run(cx<T>* v) {
        cx<T> a = v[0], b = v[1];
        v[0] = badd<T>(a, b);
        v[1] = bsub<T>(a, b);
    }
};

template <int SIGN, typename T> struct Bfly<4, SIGN, T> {
    static __device__ __forceinline__ void run(cx<T>* v) {
        cx<T> t0 = badd<T>(v[0], v[2]);
        cx<T> t1 = bsub<T>(v[0], v[2]);
        cx<T> t2 = badd<T>(v[1], v[3]);
        cx<T> t3 = cmul_i<SIGN, T>(bsub<T>(v[1], v[3]));
        v[0] = badd<T>(t0, t2);
        v[2] = bsub<T>(t0, t2);
        v[1] = badd<T>(t1, t3);
        v[3] = bsub<T>(t1, t3);
    }
};

// DFT of length R whose inputs v[NIN .. R) are zero: they are neither read
// nor added (the zero-padded half of a first stage).  Pruned forms for NIN =
// R / 2 with R = 4, 8, 16 (the first radices of the two-stage plans); any
// other NIN runs the full butterfly on zeros.
template <int R, int SIGN, typename T, int NIN> struct BflyIn {
    static __device__ __forceinline__ void run(cx<T>* v) {
#pragma unroll
        for (int r = NIN; r < R; r++) v[r] = czero<T>();
        Bfly<R, SIGN, T>::run(v);
    }
};
template <int SIGN, typename T> struct BflyIn<4, SIGN, T, 4> {
    static __device__ __forceinline__ void run(cx<T>* v) { Bfly<4, SIGN, T>::run(v); }
};
template <int SIGN, typename T> struct BflyIn<4, SIGN, T, 2> {
    // v[0] + W^q v[1], W = exp(SIGN i pi / 2)
    static __device__ __forceinline__ void run(cx<T>* v) {
        const cx<T> a = v[0], b = v[1], wb = cmul_i<SIGN, T>(b);
        v[0] = badd<T>(a, b);
        v[1] = badd<T>(a, wb);
        v[2] = bsub<T>(a, b);
        v[3] = bsub<T>(a, wb);
    }
};

// Radix 8: even / odd 4-point DFTs combined with W8^q.  NIN4 < 4: only the
// first NIN4 inputs of each 4-point DFT (v[0 .. 2 NIN4)) are non-zero.
template <int SIGN, typename T, int NIN4> struct Bfly8 {
    static __device__ __forceinline__ void run(cx<T>* v) {
        const T h = T(0.70710678118654752440084436210484904);  // sqrt(1/2)
        cx<T> e[4], o[4];
#pragma unroll
        for (int k = 0; k < NIN4; k++) e[k] = v[2 * k], o[k] = v[2 * k + 1];
        BflyIn<4, SIGN, T, NIN4>::run(e);
        BflyIn<4, SIGN, T, NIN4>::run(o);
        // W8^1 = (1 + SIGN i) sqrt(1/2), W8^2 = SIGN i, W8^3 = (-1 + SIGN i) sqrt(1/2)
        cx<T> o1 = mk<T>((o[1].x - T(SIGN) * o[1].y) * h, (o[1].y + T(SIGN) * o[1].x) * h);
        cx<T> o2 = cmul_i<SIGN, T>(o[2]);
        cx<T> o3 = mk<T>((-o[3].x - T(SIGN) * o[3].y) * h, (-o[3].y + T(SIGN) * o[3].x) * h);
        v[0] = badd<T>(e[0], o[0]);
        v[4] = bsub<T>(e[0], o[0]);
        v[1] = badd<T>(e[1], o1);
        v[5] = bsub<T>(e[1], o1);
        v[2] = badd<T>(e[2], o2);
        v[6] = bsub<T>(e[2], o2);
        v[3] = badd<T>(e[3], o3);
        v[7] = bsub<T>(e[3], o3);
    }
};
template <int SIGN, typename T> struct Bfly<8, SIGN, T> : Bfly8<SIGN, T, 4> {};

// odd prime radices: V[q] = v0 + sum_{r=1}^{(R-1)/2} [ c_{rq} (v_r + v_{R-r}) + SIGN i s_{rq} (v_r - v_{R-r}) ]
// with c_m = cos(2 pi m / R), s_m = sin(2 pi m / R)
template <int R> struct OddConst;
template <> struct OddConst<3> {
    static __device__ __forceinline__ double c(int m) { return m % 3 == 0 ? 1.0 : -0.5; }
    static __device__ __forceinline__ double s(int m) {
        int k = m % 3;
        return k == 0 ? 0.0 : (k == 1 ? 0.86602540378443864676372317075293618 : -0.86602540378443864676372317075293618);
    }
};
template <> struct OddConst<5> {
    static __device__ __forceinline__ double c(int m) {
        int k = m % 5;
        return k == 0 ? 1.0 : (k == 1 || k == 4) ? 0.30901699437494742410229341718281906 : -0.80901699437494742410229341718281906;
    }
    static __device__ __forceinline__ double s(int m) {
        int k = m % 5;
        const double s1 = 0.95105651629515357211643933337938214, s2 = 0.58778525229247312916870595463907277;
        return k == 0 ? 0.0 : k == 1 ? s1 : k == 2 ? s2 : k == 3 ? -s2 : -s1;
    }
};
template <> struct OddConst<7> {
    static __device__ __forceinline__ double c(int m) {
        int k = m % 7;
        const double c1 = 0.62348980185873353052500488400423981, c2 = -0.22252093395631440428890256449679476,
                     c3 = -0.90096886790241912623610231950744505;
        return k == 0 ? 1.0 : (k == 1 || k == 6) ? c1 : (k == 2 || k == 5) ? c2 : c3;
    }
    static __device__ __forceinline__ double s(int m) {
        int k = m % 7;
        const double s1 = 0.78183148246802980870844452667405775, s2 = 0.97492791218182360701813168299393122,
                     s3 = 0.43388373911755812047576833284835875;
        return k == 0 ? 0.0 : k == 1 ? s1 : k == 2 ? s2 : k == 3 ? s3 : k == 4 ? -s3 : k == 5 ? -s2 : -s1;
    }
};

template <int R, int SIGN, typename T> struct BflyOdd {
    static __device__ __forceinline__ void run(cx<T>* v) {
        constexpr int H = (R - 1) / 2;
        cx<T> sp[H], sm[H];
#pragma unroll
        for (int r = 1; r <= H; r++) {
            sp[r - 1] = badd<T>(v[r], v[R - r]);
            sm[r - 1] = bsub<T>(v[r], v[R - r]);
        }
        cx<T> out[R];
        cx<T> s0 = v[0];
#pragma unroll
        for (int r = 0; r < H; r++) s0 = badd<T>(s0, sp[r]);
        out[0] = s0;
#pragma unroll
        for (int q = 1; q <= H; q++) {
            cx<T> re = v[0];
            cx<T> im = czero<T>();
#pragma unroll
            for (int r = 1; r <= H; r++) {
                const T c = T(OddConst<R>::c(r * q));
                const T s = T(OddConst<R>::s(r * q));
                re = bfma<T>(sp[r - 1], c, re);
                im = bfma<T>(sm[r - 1], s, im);
            }
            cx<T> rot = cmul_i<SIGN, T>(im);  // SIGN i * im
            out[q] = badd<T>(re, rot);
            out[R - q] = bsub<T>(re, rot);
        }
#pragma unroll
        for (int q = 0; q < R; q++) v[q] = out[q];
    }
};
template <int SIGN, typename T> struct Bfly<3, SIGN, T> : BflyOdd<3, SIGN, T> {};
template <int SIGN, typename T> struct Bfly<5, SIGN, T> : BflyOdd<5, SIGN, T> {};
template <int SIGN, typename T> struct Bfly<7, SIGN, T> : BflyOdd<7, SIGN, T> {};

// ------------------------------------------------------ composite butterflies
// DFT of length R = R1 R2 in registers: with n = R2 n1 + n2 and k = k1 + R1 k2,
//   X[k] = sum_n2 W_R^(n2 k1) W_R2^(n2 k2) sum_n1 x[R2 n1 + n2] W_R1^(n1 k1):
// R2 DFTs of length R1, twiddles W_R^(n2 k1), R1 DFTs of length R2.  The
// constants cos / sin(2 pi m / R) are tabulated below.
template <int R> struct RootTab;
template <> struct RootTab<10> {
    static __device__ __forceinline__ double c(int m) {
        constexpr double t[10] = {1, 0.80901699437494745, 0.30901699437494745, -0.30901699437494734, -0.80901699437494734, -1, -0.80901699437494756, -0.30901699437494756, 0.30901699437494723, 0.80901699437494734};
        return t[m % 10];
    }
    static __device__ __forceinline__ double s(int m) {
        constexpr double t[10] = {0, 0.58778525229247314, 0.95105651629515353, 0.95105651629515364, 0.58778525229247325, 1.2246467991473532e-16, -0.58778525229247303, -0.95105651629515353, -0.95105651629515364, -0.58778525229247336};
        return t[m % 10];
    }
};
template <> struct RootTab<12> {
    static __device__ __forceinline__ double c(int m) {
        constexpr double t[12] = {1, 0.86602540378443871, 0.50000000000000011, 6.123233995736766e-17, -0.49999999999999978, -0.86602540378443871, -1, -0.86602540378443882, -0.50000000000000044, -1.8369701987210297e-16, 0.50000000000000011, 0.86602540378443837};
        return t[m % 12];
    }
    static __device__ __forceinline__ double s(int m) {
        constexpr double t[12] = {0, 0.49999999999999994, 0.8660254037844386, 1, 0.86602540378443871, 0.49999999999999994, 1.2246467991473532e-16, -0.49999999999999972, -0.86602540378443837, -1, -0.8660254037844386, -0.50000000000000044};
        return t[m % 12];
    }
};
template <> struct RootTab<16> {
    static __device__ __forceinline__ double c(int m) {
        constexpr double t[16] = {1, 0.92387953251128674, 0.70710678118654757, 0.38268343236508984, 6.123233995736766e-17, -0.38268343236508973, -0.70710678118654746, -0.92387953251128674, -1, -0.92387953251128685, -0.70710678118654768, -0.38268343236509034, -1.8369701987210297e-16, 0.38268343236509, 0.70710678118654735, 0.92387953251128652};
        return t[m % 16];
    }
    static __device__ __forceinline__ double s(int m) {
        constexpr double t[16] = {0, 0.38268343236508978, 0.70710678118654746, 0.92387953251128674, 1, 0.92387953251128674, 0.70710678118654757, 0.38268343236508989, 1.2246467991473532e-16, -0.38268343236508967, -0.70710678118654746, -0.92387953251128652, -1, -0.92387953251128663, -0.70710678118654768, -0.38268343236509039};
        return t[m % 16];
    }
};

template <> struct RootTab<24> {
    static __device__ __forceinline__ double c(int m) {
        constexpr double t[24] = {1.0, 0.9659258262890683, 0.8660254037844387, 0.7071067811865476, 0.5000000000000001, 0.25881904510252074, 6.123233995736766e-17, -0.25881904510252063, -0.4999999999999998, -0.7071067811865475, -0.8660254037844387, -0.9659258262890682, -1.0, -0.9659258262890683, -0.8660254037844388, -0.7071067811865479, -0.5000000000000004, -0.25881904510252063, -1.8369701987210297e-16, 0.2588190451025203, 0.5000000000000001, 0.7071067811865474, 0.8660254037844384, 0.9659258262890681};
        return t[m % 24];
    }
    static __device__ __forceinline__ double s(int m) {
        constexpr double t[24] = {0.0, 0.25881904510252074, 0.49999999999999994, 0.7071067811865475, 0.8660254037844386, 0.9659258262890683, 1.0, 0.9659258262890683, 0.8660254037844387, 0.7071067811865476, 0.49999999999999994, 0.258819045102521, 1.2246467991473532e-16, -0.2588190451025208, -0.4999999999999997, -0.7071067811865471, -0.8660254037844384, -0.9659258262890683, -1.0, -0.9659258262890684, -0.8660254037844386, -0.7071067811865477, -0.5000000000000004, -0.25881904510252157};
        return t[m % 24];
    }
};

// NIN1 < R1: only inputs n1 < NIN1 of each inner DFT (v[0 .. R2 NIN1)) are
// non-zero.
template <int R1, int R2, int SIGN, typename T, int NIN1 = R1> struct BflyComp {
    static __device__ __forceinline__ void run(cx<T>* v) {
        constexpr int R = R1 * R2;
        cx<T> y[R2][R1];
#pragma unroll
        for (int n2 = 0; n2 < R2; n2++) {
            cx<T> a[R1];
#pragma unroll
            for (int n1 = 0; n1 < NIN1; n1++) a[n1] = v[R2 * n1 + n2];
            BflyIn<R1, SIGN, T, NIN1>::run(a);
#pragma unroll
            for (int k1 = 0; k1 < R1; k1++) {
                if (n2 > 0 && k1 > 0) {
                    const T c = T(RootTab<R>::c(n2 * k1)), s = T(SIGN) * T(RootTab<R>::s(n2 * k1));
                    a[k1] = mk<T>(a[k1].x * c - a[k1].y * s, a[k1].x * s + a[k1].y * c);
                }
                y[n2][k1] = a[k1];
            }
        }
#pragma unroll
        for (int k1 = 0; k1 < R1; k1++) {
            cx<T> b[R2];
#pragma unroll
            for (int n2 = 0; n2 < R2; n2++) b[n2] = y[n2][k1];
            Bfly<R2, SIGN, T>::run(b);
#pragma unroll
            for (int k2 = 0; k2 < R2; k2++) v[k1 + R1 * k2] = b[k2];
        }
    }
};
template <int SIGN, typename T> struct Bfly<16, SIGN, T> : BflyComp<4, 4, SIGN, T> {};
template <int SIGN, typename T> struct BflyIn<8, SIGN, T, 4> : Bfly8<SIGN, T, 2> {};
template <int SIGN, typename T> struct BflyIn<16, SIGN, T, 8> : BflyComp<4, 4, SIGN, T, 2> {};
template <int SIGN, typename T> struct Bfly<24, SIGN, T> : BflyComp<8, 3, SIGN, T> {};
template <int SIGN, typename T> struct BflyIn<24, SIGN, T, 12> : BflyComp<8, 3, SIGN, T, 4> {};
template <int SIGN, typename T> struct BflyIn<12, SIGN, T, 6> : BflyComp<4, 3, SIGN, T, 2> {};
template <int SIGN, typename T> struct Bfly<12, SIGN, T> : BflyComp<4, 3, SIGN, T> {};
template <int SIGN, typename T> struct Bfly<10, SIGN, T> : BflyComp<2, 5, SIGN, T> {};

// ----------------------------------------------------------------- one stage
// Out-of-place (ping-pong) stage: reads x, writes y, then a barrier.  Each
// thread loops over butterflies, holding one radix-R butterfly in registers.
// nvalid: inputs with index >= nvalid are zero (first stage only); nout:
// outputs with index >= nout are not stored (last stage only).
template <int R, int SIGN, typename T>
__device__ __forceinline__ void fft_stage(const cx<T>* __restrict__ x, cx<T>* __restrict__ y, int L, FastDiv fl,
                                          int ls, int ms, int M, int Ns, FastDiv fns, const cx<T>* tw, int nvalid,
                                          int nout) {
    const int m = M / R;
    const int nb = L * m;
    const int twstep = M / (Ns * R);
    for (int w = threadIdx.x; w < nb; w += blockDim.x) {
        const int j = (int)fastdiv((unsigned)w, fl);
        const int l = w - j * L;
        const cx<T>* xb = x + l * ls;
        cx<T> v[R];
#pragma unroll
        for (int r = 0; r < R; r++) {
            const int idx = j + r * m;
            v[r] = idx < nvalid ? xb[idx * ms] : czero<T>();
        }
        const int k = j - (int)fastdiv((unsigned)j, fns) * Ns;
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; r++) {
                cx<T> t = tw[r * k * twstep];
                if (SIGN > 0) t.y = -t.y;
                v[r] = cmul<T>(v[r], t);
            }
        }
        Bfly<R, SIGN, T>::run(v);
        cx<T>* yb = y + l * ls;
        const int ob = (j - k) * R + k;
#pragma unroll
        for (int q = 0; q < R; q++) {
            const int idx = ob + q * Ns;
            if (idx < nout) yb[idx * ms] = v[q];
        }
    }
    __syncthreads();
}

// Full transform of the L lines held in buffer a (b is scratch of the same
// shape).  SIGN = -1 forward, +1 inverse; unnormalised.  Returns the buffer
// that holds the result.
template <int SIGN, typename T>
__device__ __forceinline__ cx<T>* smem_fft(cx<T>* a, cx<T>* b, int L, int ls, int ms, const AxisPlan& ap,
                                           const cx<T>* tw, int nvalid, int nout) {
    int Ns = 1;
    const int M = ap.M;
    const FastDiv fl = fastdiv_make((unsigned)L);
    for (int st = 0; st < ap.nstages; st++) {
        const int R = ap.radix[st];
        const int nv = st == 0 ? nvalid : M;
        const int no = st == ap.nstages - 1 ? nout : M;
        const FastDiv fns = ap.ns[st];
        switch (R) {
            case 2: fft_stage<2, SIGN, T>(a, b, L, fl, ls, ms, M, Ns, fns, tw, nv, no); break;
            case 3: fft_stage<3, SIGN, T>(a, b, L, fl, ls, ms, M, Ns, fns, tw, nv, no); break;
            case 4: fft_stage<4, SIGN, T>(a, b, L, fl, ls, ms, M, Ns, fns, tw, nv, no); break;
            case 5: fft_stage<5, SIGN, T>(a, b, L, fl, ls, ms, M, Ns, fns, tw, nv, no); break;
            case 7: fft_stage<7, SIGN, T>(a, b, L, fl, ls, ms, M, Ns, fns, tw, nv, no); break;
            default: fft_stage<8, SIGN, T>(a, b, L, fl, ls, ms, M, Ns, fns, tw, nv, no); break;
        }
        Ns *= R;
        cx<T>* t = a;
        a = b;
        b = t;
    }
    return a;
}

}  // namespace tdda
