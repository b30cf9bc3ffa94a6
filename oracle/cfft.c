/*
 * cfft.c -- CPU mixed-radix Stockham FFT for the oracle (test infrastructure).
 *
 * Algorithm: Stockham autosort.  For n = R_1 R_2 ... R_s, stage i with radix
 * R and "span" Ns = R_1...R_{i-1} maps, for every butterfly j in [0, n/R):
 *     k    = j mod Ns
 *     v[r] = x[j + r n/R] * exp(sign 2 pi i r k / (Ns R))      r = 0..R-1
 *     V    = DFT_R(v)        (V[q] = sum_r v[r] exp(sign 2 pi i r q / R))
 *     y[(j - k) R + k + q Ns] = V[q]
 * and the output of the last stage is in natural order.  The radix-R DFTs
 * are written from their definition; the twiddles come from a table
 * W[m] = exp(-2 pi i m / n) evaluated with the C library's cos/sin.
 *
 * Conventions follow cuFFT as the reference uses it: forward sign -1,
 * inverse sign +1, no normalisation (AProductCore.cpp:719-739, :752).
 */
#include "cfft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define OC_MAX_FACTORS 40

struct oc_plan1d {
    int n;
    int nfac;
    int fac[OC_MAX_FACTORS];
    oc_cplx* w; /* W[m] = exp(-2 pi i m / n) */
};

static void factorize(int n, int* fac, int* nfac) {
    int k = 0;
    while (n % 4 == 0 && k < OC_MAX_FACTORS) { fac[k++] = 4; n /= 4; }
    if (n % 2 == 0 && k < OC_MAX_FACTORS) { fac[k++] = 2; n /= 2; }
    for (int p = 3; n > 1 && k < OC_MAX_FACTORS; p += 2) {
        while (n % p == 0 && k < OC_MAX_FACTORS) { fac[k++] = p; n /= p; }
        if ((long long)p * p > n && n > 1) { fac[k++] = n; n = 1; }
    }
    *nfac = k;
}

oc_plan1d* oc_plan1d_create(int n) {
    if (n < 1) return NULL;
    oc_plan1d* p = (oc_plan1d*)calloc(1, sizeof(oc_plan1d));
    if (!p) return NULL;
    p->n = n;
    factorize(n, p->fac, &p->nfac);
    p->w = (oc_cplx*)malloc(sizeof(oc_cplx) * (size_t)n);
    if (!p->w) { free(p); return NULL; }
    const double two_pi = 6.283185307179586476925286766559;
    for (int m = 0; m < n; m++) {
        double a = two_pi * (double)m / (double)n;
        p->w[m].re = cos(a);
        p->w[m].im = -sin(a);
    }
    return p;
}

void oc_plan1d_destroy(oc_plan1d* p) {
    if (!p) return;
    free(p->w);
    free(p);
}

int oc_plan1d_len(const oc_plan1d* p) { return p->n; }

static inline oc_cplx cmul(oc_cplx a, oc_cplx b) {
    oc_cplx c;
    c.re = a.re * b.re - a.im * b.im;
    c.im = a.re * b.im + a.im * b.re;
    return c;
}

/* exp(sign * 2 pi i * a / L) for a < L, L dividing n */
static inline oc_cplx twiddle(const oc_plan1d* p, long a, long L, int sign) {
    oc_cplx t = p->w[a * (p->n / L)];
    if (sign > 0) t.im = -t.im;
    return t;
}

static void stage(const oc_plan1d* p, const oc_cplx* x, oc_cplx* y, int R, int Ns, int sign) {
    const int n = p->n;
    const int m = n / R;
    oc_cplx v[64];
    oc_cplx V[64];
    oc_cplx* vv = v;
    oc_cplx* VV = V;
    oc_cplx* heap = NULL;
    if (R > 64) {
        heap = (oc_cplx*)malloc(sizeof(oc_cplx) * 2 * (size_t)R);
        vv = heap;
        VV = heap + R;
    }
    for (int j = 0; j < m; j++) {
        const int k = j % Ns;
        for (int r = 0; r < R; r++) {
            oc_cplx a = x[j + r * m];
            if (Ns > 1 && r > 0) a = cmul(a, twiddle(p, (long)r * k, (long)Ns * R, sign));
            vv[r] = a;
        }
        if (R == 2) {
            VV[0].re = vv[0].re + vv[1].re; VV[0].im = vv[0].im + vv[1].im;
            VV[1].re = vv[0].re - vv[1].re; VV[1].im = vv[0].im - vv[1].im;
        } else if (R == 4) {
            oc_cplx t0 = {vv[0].re + vv[2].re, vv[0].im + vv[2].im};
            oc_cplx t1 = {vv[0].re - vv[2].re, vv[0].im - vv[2].im};
            oc_cplx t2 = {vv[1].re + vv[3].re, vv[1].im + vv[3].im};
            oc_cplx d = {vv[1].re - vv[3].re, vv[1].im - vv[3].im};
            /* t3 = (sign * i) * d : forward multiplies by -i */
            oc_cplx t3;
            if (sign < 0) { t3.re = d.im; t3.im = -d.re; }
            else { t3.re = -d.im; t3.im = d.re; }
            VV[0].re = t0.re + t2.re; VV[0].im = t0.im + t2.im;
            VV[2].re = t0.re - t2.re; VV[2].im = t0.im - t2.im;
            VV[1].re = t1.re + t3.re; VV[1].im = t1.im + t3.im;
            VV[3].re = t1.re - t3.re; VV[3].im = t1.im - t3.im;
        } else {
            for (int q = 0; q < R; q++) {
                oc_cplx s = vv[0];
                for (int r = 1; r < R; r++) {
                    long e = ((long)r * q) % R;
                    oc_cplx t = twiddle(p, e, R, sign);
                    oc_cplx prod = cmul(vv[r], t);
                    s.re += prod.re;
                    s.im += prod.im;
                }
                VV[q] = s;
            }
        }
        const int base = (j - k) * R + k;
        for (int q = 0; q < R; q++) y[base + q * Ns] = VV[q];
    }
    free(heap);
}

void oc_fft1d(const oc_plan1d* p, oc_cplx* data, ptrdiff_t stride, int sign, oc_cplx* work) {
    const int n = p->n;
    oc_cplx* a = work;
    oc_cplx* b = work + n;
    for (int i = 0; i < n; i++) a[i] = data[(ptrdiff_t)i * stride];
    int Ns = 1;
    for (int s = 0; s < p->nfac; s++) {
        stage(p, a, b, p->fac[s], Ns, sign);
        Ns *= p->fac[s];
        oc_cplx* t = a; a = b; b = t;
    }
    for (int i = 0; i < n; i++) data[(ptrdiff_t)i * stride] = a[i];
}

int oc_fft3d(int n0, int n1, int n2, oc_cplx* data, int sign) {
    oc_plan1d* p0 = oc_plan1d_create(n0);
    oc_plan1d* p1 = oc_plan1d_create(n1);
    oc_plan1d* p2 = oc_plan1d_create(n2);
    int nmax = n0 > n1 ? n0 : n1;
    if (n2 > nmax) nmax = n2;
    oc_cplx* work = (oc_cplx*)malloc(sizeof(oc_cplx) * 2 * (size_t)nmax);
    if (!p0 || !p1 || !p2 || !work) {
        oc_plan1d_destroy(p0); oc_plan1d_destroy(p1); oc_plan1d_destroy(p2); free(work);
        return 1;
    }
    const ptrdiff_t s1 = n2, s0 = (ptrdiff_t)n1 * n2;
    for (int i = 0; i < n0; i++)
        for (int j = 0; j < n1; j++) oc_fft1d(p2, data + i * s0 + j * s1, 1, sign, work);
    for (int i = 0; i < n0; i++)
        for (int k = 0; k < n2; k++) oc_fft1d(p1, data + i * s0 + k, s1, sign, work);
    for (int j = 0; j < n1; j++)
        for (int k = 0; k < n2; k++) oc_fft1d(p0, data + j * s1 + k, s0, sign, work);
    oc_plan1d_destroy(p0); oc_plan1d_destroy(p1); oc_plan1d_destroy(p2);
    free(work);
    return 0;
}

/* ------------------------------------------------------------------------
 * Lengths with a large prime factor, for timing the reference's CPU path.
 *
 * oc_fft3d_fast gives the same transform as oc_fft3d (to rounding) but runs a
 * line whose length has a prime factor above 7 through Bluestein's chirp-z
 * algorithm (L. I. Bluestein, "A linear filtering approach to the
 * computation of the discrete Fourier transform", 1970): with
 * k q = (k^2 + q^2 - (q - k)^2) / 2 and c_k = exp(sign pi i k^2 / n),
 *     X_q = c_q sum_k (x_k c_k) conj(c_{q - k}),
 * a circular convolution of length L >= 2n - 1 (a power of two) evaluated
 * with the radix-4/2 FFT above.  The reference's 2N - 1 grids (127, 31, 191,
 * ...) are such lengths; the direct O(p^2) prime DFT of oc_fft3d is kept for
 * the checker itself, whose outputs are pinned to fixtures.
 */
typedef struct {
    int n, L;
    oc_plan1d* sub;   /* length L */
    oc_cplx* chirp;   /* c_k for sign -1, k < n (sign +1 is the conjugate) */
    oc_cplx* bhat[2]; /* FFT_L of the conjugate chirp, for sign -1 and +1 */
} oc_blue;

static int largest_prime_factor(int n) {
    int p = 1;
    for (int f = 2; (long long)f * f <= n; f++)
        while (n % f == 0) { p = f; n /= f; }
    return n > 1 ? n : p;
}

static void blue_destroy(oc_blue* b) {
    if (!b) return;
    oc_plan1d_destroy(b->sub);
    free(b->chirp);
    free(b->bhat[0]);
    free(b->bhat[1]);
    free(b);
}

static oc_blue* blue_create(int n) {
    oc_blue* b = (oc_blue*)calloc(1, sizeof(oc_blue));
    if (!b) return NULL;
    b->n = n;
    b->L = 1;
    while (b->L < 2 * n - 1) b->L *= 2;
    const int L = b->L;
    b->sub = oc_plan1d_create(L);
    b->chirp = (oc_cplx*)malloc(sizeof(oc_cplx) * (size_t)n);
    b->bhat[0] = (oc_cplx*)calloc((size_t)L, sizeof(oc_cplx));
    b->bhat[1] = (oc_cplx*)calloc((size_t)L, sizeof(oc_cplx));
    oc_cplx* work = (oc_cplx*)malloc(sizeof(oc_cplx) * 2 * (size_t)L);
    if (!b->sub || !b->chirp || !b->bhat[0] || !b->bhat[1] || !work) {
        free(work);
        blue_destroy(b);
        return NULL;
    }
    const double pi = 3.14159265358979323846264338327950288;
    for (int k = 0; k < n; k++) {
        /* k^2 mod 2n keeps the angle's argument small and exact */
        const long long e = ((long long)k * k) % (2LL * n);
        const double a = pi * (double)e / (double)n;
        b->chirp[k].re = cos(a);
        b->chirp[k].im = -sin(a);
    }
    for (int s = 0; s < 2; s++) {
        const double sg = s == 0 ? -1.0 : 1.0; /* the transform's sign */
        oc_cplx* h = b->bhat[s];
        for (int k = 0; k < n; k++) {
            /* conj(c_k) of that sign: c_k(sign) = (re, sign * |im|) */
            oc_cplx c = b->chirp[k];
            if (sg > 0) c.im = -c.im;
            oc_cplx cc = {c.re, -c.im};
            h[k] = cc;
            if (k > 0) h[L - k] = cc;
        }
        oc_fft1d(b->sub, h, 1, -1, work);
    }
    free(work);
    return b;
}

/* one line through the chirp-z convolution; scratch holds 3 L elements */
static void blue_line(const oc_blue* b, oc_cplx* data, ptrdiff_t stride, int sign, oc_cplx* scratch) {
    const int n = b->n, L = b->L;
    oc_cplx* a = scratch;
    oc_cplx* work = scratch + L;
    for (int k = 0; k < n; k++) {
        oc_cplx c = b->chirp[k];
        if (sign > 0) c.im = -c.im;
        a[k] = cmul(data[(ptrdiff_t)k * stride], c);
    }
    for (int k = n; k < L; k++) a[k].re = a[k].im = 0.0;
    oc_fft1d(b->sub, a, 1, -1, work);
    const oc_cplx* h = b->bhat[sign > 0 ? 1 : 0];
    for (int k = 0; k < L; k++) a[k] = cmul(a[k], h[k]);
    oc_fft1d(b->sub, a, 1, 1, work);
    const double inv = 1.0 / (double)L;
    for (int q = 0; q < n; q++) {
        oc_cplx c = b->chirp[q];
        if (sign > 0) c.im = -c.im;
        oc_cplx v = cmul(a[q], c);
        v.re *= inv;
        v.im *= inv;
        data[(ptrdiff_t)q * stride] = v;
    }
}

typedef struct {
    oc_plan1d* p;
    oc_blue* b;
} oc_axis;

static int axis_create(oc_axis* ax, int n) {
    ax->p = NULL;
    ax->b = NULL;
    if (largest_prime_factor(n) > 7) ax->b = blue_create(n);
    else ax->p = oc_plan1d_create(n);
    return ax->p || ax->b ? 0 : 1;
}

static void axis_line(const oc_axis* ax, oc_cplx* data, ptrdiff_t stride, int sign, oc_cplx* scratch) {
    if (ax->b) blue_line(ax->b, data, stride, sign, scratch);
    else oc_fft1d(ax->p, data, stride, sign, scratch);
}

static int axis_scratch(const oc_axis* ax) { return ax->b ? 3 * ax->b->L : 2 * oc_plan1d_len(ax->p); }

int oc_fft3d_fast(int n0, int n1, int n2, oc_cplx* data, int sign) {
    oc_axis a0, a1, a2;
    int err = axis_create(&a0, n0);
    err |= axis_create(&a1, n1);
    err |= axis_create(&a2, n2);
    int ns = axis_scratch(&a0);
    if (axis_scratch(&a1) > ns) ns = axis_scratch(&a1);
    if (axis_scratch(&a2) > ns) ns = axis_scratch(&a2);
    oc_cplx* scratch = err ? NULL : (oc_cplx*)malloc(sizeof(oc_cplx) * (size_t)ns);
    if (!scratch) err = 1;
    if (!err) {
        const ptrdiff_t s1 = n2, s0 = (ptrdiff_t)n1 * n2;
        for (int i = 0; i < n0; i++)
            for (int j = 0; j < n1; j++) axis_line(&a2, data + i * s0 + j * s1, 1, sign, scratch);
        for (int i = 0; i < n0; i++)
            for (int k = 0; k < n2; k++) axis_line(&a1, data + i * s0 + k, s1, sign, scratch);
        for (int j = 0; j < n1; j++)
            for (int k = 0; k < n2; k++) axis_line(&a0, data + j * s1 + k, s0, sign, scratch);
    }
    free(scratch);
    oc_plan1d_destroy(a0.p); oc_plan1d_destroy(a1.p); oc_plan1d_destroy(a2.p);
    blue_destroy(a0.b); blue_destroy(a1.b); blue_destroy(a2.b);
    return err;
}
