/*
 * tdda_oracle.c -- CPU restatement of the reference's DDA solve path.
 * TEST INFRASTRUCTURE ONLY (see tdda_oracle.h): the checker, never the
 * thing measured or shipped.
 */
#include "tdda_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "cfft.h"

typedef double _Complex cd;

static const double OR_PI = 3.14159265358979323846264338327950288;

static inline cd ld(const double* p, long i) { return p[2 * i] + I * p[2 * i + 1]; }
static inline void st(double* p, long i, cd v) { p[2 * i] = creal(v); p[2 * i + 1] = cimag(v); }

/* AProductCore.cpp:19-24: material / nback^2, then +0.01 when |eps| <= 1.01 */
void or_normalize_material(int nmat, const double* mat_in, double nback, double* mat_out) {
    for (int i = 0; i < nmat; i++) {
        cd m = ld(mat_in, i) / (nback * nback);
        if (sqrt(creal(m) * creal(m) + cimag(m) * cimag(m)) <= 1.01) m = m + 0.01;
        st(mat_out, i, m);
    }
}

/* AProductCore.cpp:588-623.  out12 = xx, xy, xz, yy, yz, zz (re, im).
 * r = 0 gives the zero tensor (the reference leaves the off-diagonals of
 * that case unset; they are defined as 0 here). */
void or_ldr_inter(double K, double x, double y, double z, double* out12) {
    double xs = x * x, ys = y * y, zs = z * z;
    double rn = sqrt(xs + ys + zs);
    if (rn == 0.0) {
        memset(out12, 0, 12 * sizeof(double));
        return;
    }
    double xy = x * y, yz = y * z, zx = z * x;
    double rsq = rn * rn;
    double rcu = rn * rn * rn;
    cd c1 = cexp(I * (K * rn)) / rcu;
    cd c2 = (1.0 - I * (K * rn)) / rsq;
    cd c3 = K * K - 3.0 * c2;
    cd t[6];
    t[0] = c2 * (rsq - 3 * xs) - K * K * (ys + zs);
    t[1] = xy * c3;
    t[2] = zx * c3;
    t[3] = c2 * (rsq - 3 * ys) - K * K * (zs + xs);
    t[4] = yz * c3;
    t[5] = c2 * (rsq - 3 * zs) - K * K * (xs + ys);
    for (int l = 0; l < 6; l++) st(out12, l, c1 * t[l]);
}

/* Sine and cosine integrals Si(x) = int_0^x sin t / t dt and
 * Ci(x) = gamma + ln x + int_0^x (cos t - 1) / t dt for x > 0, to double
 * precision, from the formulas of Abramowitz & Stegun:
 *  - x <= 4: the power series 5.2.14 and 5.2.16, summed until the terms no
 *    longer change the sum;
 *  - x > 4: E1(ix) = -Ci(x) + i (Si(x) - pi/2) (5.2.23), with E1(z) from its
 *    even continued fraction 5.1.22, e^{-z} / (z + 1 - 1/(z + 3 - 4/(z + 5 - ...))),
 *    evaluated by the modified Lentz method (W. J. Lentz, Appl. Opt. 15, 1976;
 *    Thompson & Barnett, J. Comput. Phys. 64, 1986). */
void or_sici(double x, double* si, double* ci) {
    const double euler = 0.57721566490153286061;
    if (x <= 4.0) {
        double s = 0.0, c = 0.0, term = x; /* term = (-1)^k x^(2k+1) / (2k+1)! */
        for (int k = 0; k < 60; k++) {
            const double sk = term / (2 * k + 1);
            s += sk;
            const double tc = -term * x / (2 * k + 2); /* (-1)^(k+1) x^(2k+2) / (2k+2)! */
            const double ck = tc / (2 * k + 2);
            c += ck;
            term = tc * x / (2 * k + 3);
            if (fabs(sk) <= 1e-17 * fabs(s) && fabs(ck) <= 1e-17 * (fabs(c) + 1e-300)) break;
        }
        *si = s;
        *ci = euler + log(x) + c;
        return;
    }
    /* Lentz on f = b0 + a1/(b1 + a2/(b2 + ...)) with b_j = z + 2j + 1 and
     * a_j = -j^2, then E1 = e^{-z} / f, z = i x */
    const cd z = x * I;
    const double tiny = 1e-300;
    cd b = z + 1.0;
    cd f = b, C = b, D = 0.0;
    for (int j = 1; j < 1000; j++) {
        const double a = -(double)j * (double)j;
        b = b + 2.0;
        D = b + a * D;
        if (cabs(D) < tiny) D = tiny;
        C = b + a / C;
        if (cabs(C) < tiny) C = tiny;
        D = 1.0 / D;
        const cd delta = C * D;
        f = f * delta;
        if (cabs(delta - 1.0) < 1e-16) break;
    }
    const cd e1 = cexp(-z) / f;
    *ci = -creal(e1);
    *si = OR_PI / 2 + cimag(e1);
}

/* The Si/Ci tables of SiCi/SiCi.py (read by SiCi.cpp:8-25): the values at
 * x = 0.1 k, k = 1 .. 999999, here evaluated with or_sici. */
enum { SICI_N = 999999 };
static const double SICI_DIS = 0.1;
static double* g_si = NULL;
static double* g_ci = NULL;
static void sici_tables(void) {
    if (g_si) return;
    double* si = (double*)malloc(sizeof(double) * SICI_N);
    double* ci = (double*)malloc(sizeof(double) * SICI_N);
    for (int k = 0; k < SICI_N; k++) or_sici(SICI_DIS * (k + 1), &si[k], &ci[k]);
    g_ci = ci;
    g_si = si;
}
/* SiCi::get_Si / get_Ci (SiCi.cpp:27-47): linear interpolation between the
 * nodes (floor(x/dis)) dis and (ceil(x/dis)) dis.  Where the reference divides
 * 0 by 0 (x on a node) this returns the node value; below the first node and
 * past the last it extends the end intervals (the reference reads outside
 * its table there). */
static double sici_interp(const double* tab, double x) {
    double q = x / SICI_DIS;
    if (!(q >= 0.0)) q = 0.0;
    if (q > (double)SICI_N) q = (double)SICI_N;
    int p1 = (int)floor(q) - 1, p2 = (int)ceil(q) - 1;
    if (p1 < 0) p1 = 0, p2 = 1;
    if (p2 > SICI_N - 1) p2 = SICI_N - 1, p1 = SICI_N - 2;
    if (p1 == p2) return tab[p1];
    const double v1 = tab[p1], v2 = tab[p2];
    const double a1 = (p1 + 1) * SICI_DIS, a2 = (p2 + 1) * SICI_DIS;
    return v1 + ((v2 - v1) / (a2 - a1)) * (x - a1);
}

/* AProductCore::FCD_inter (AProductCore.cpp:625-695): the filtered coupled
 * dipole tensor with the cut-off Kf = pi / d. */
void or_fcd_inter(double K, double d, double x, double y, double z, double* out12) {
    sici_tables();
    const double xs = x * x, ys = y * y, zs = z * z;
    const double rn = sqrt(xs + ys + zs);
    if (rn == 0.0) {
        memset(out12, 0, 12 * sizeof(double));
        return;
    }
    const double xy = x * y, yz = y * z, zx = z * x;
    const double rsq = rn * rn, rcu = rn * rn * rn;
    const double Kf = OR_PI / d;
    const double Cz = sici_interp(g_ci, (Kf + K) * rn), Cf = sici_interp(g_ci, (Kf - K) * rn);
    const double Sz = sici_interp(g_si, (Kf + K) * rn), Sf = sici_interp(g_si, (Kf - K) * rn);
    const double Cz1 = cos((Kf + K) * rn) / rn, Cf1 = cos((Kf - K) * rn) / rn;
    const double Sz1 = sin((Kf + K) * rn) / rn, Sf1 = sin((Kf - K) * rn) / rn;
    const double Cz2 = (-((Kf + K) * rn) * sin((Kf + K) * rn) - cos((Kf + K) * rn)) / rsq;
    const double Cf2 = (-((Kf - K) * rn) * sin((Kf - K) * rn) - cos((Kf - K) * rn)) / rsq;
    const double Sz2 = (((Kf + K) * rn) * cos((Kf + K) * rn) - sin((Kf + K) * rn)) / rsq;
    const double Sf2 = (((Kf - K) * rn) * cos((Kf - K) * rn) - sin((Kf - K) * rn)) / rsq;
    const double kr = K * rn;
    const double sikr = sin(kr), cskr = cos(kr);
    const double sikfr = sin(Kf * rn), cskfr = cos(Kf * rn);
    const cd CC = OR_PI * I + Cf - Cz;
    const double C1C1 = Cf1 - Cz1, C2C2 = Cf2 - Cz2;
    const double SS = Sz + Sf, S1S1 = Sz1 + Sf1, S2S2 = Sz2 + Sf2;
    const cd gf = (sikr * CC + cskr * SS) / (OR_PI * rn);
    const cd const1 = (kr * cskr - sikr) * CC - (kr * sikr + cskr) * SS + rn * sikr * C1C1 + rn * cskr * S1S1;
    const cd const2 = (-K * kr * sikr) * CC - (K * kr * cskr) * SS + (2 * kr * cskr) * C1C1 - (2 * kr * sikr) * S1S1 +
                      rn * sikr * C2C2 + rn * cskr * S2S2;
    const cd gf1 = const1 / (OR_PI * rsq);
    const cd gf2 = (rn * const2 - 2.0 * const1) / (OR_PI * rcu);
    const double hr = (sikfr - Kf * rn * cskfr) / (2.0 * OR_PI * OR_PI * rcu);
    const cd term1 = K * K * gf + gf1 / rn + (4.0 * OR_PI / 3.0) * hr;
    const cd term2 = (gf2 - gf1 / rn) / rsq;
    const cd t[6] = {term1 + xs * term2, xy * term2, zx * term2, term1 + ys * term2, yz * term2, term1 + zs * term2};
    for (int l = 0; l < 6; l++) st(out12, l, -1.0 * t[l]);
}

/* tools.cpp:617-630: LDR polarisability.  The three lattice-dispersion
 * coefficients are the published LDR constants the reference uses. */
void or_get_alpha(double lam, double K, double d, double eps_re, double eps_im,
                  const double* nE0, const double* nK, double* out2) {
    (void)lam;
    const double b1 = -1.891531;
    const double b2 = 0.1648469;
    const double b3 = -1.7700004;
    cd eps = eps_re + I * eps_im;
    cd a1 = (3 * pow(d, 3) / (4 * OR_PI)) * (eps - 1.0) / (eps + 2.0);
    cd res = 0.0 + I * ((2.0 / 3.0) * pow(K * d, 3));
    double S = pow(nE0[0] * nK[0], 2) + pow(nE0[1] * nK[1], 2) + pow(nE0[2] * nK[2], 2);
    res = 1.0 + (a1 / pow(d, 3)) * ((b1 + eps * b2 + eps * b3 * S) * pow(K * d, 2) - res);
    res = a1 / res;
    out2[0] = creal(res);
    out2[1] = cimag(res);
}

struct or_core {
    int Nx, Ny, Nz, N;
    int* R;
    double d, lam, nback, K;
    int nmat;
    double* material; /* normalised */
    int Mx, My, Mz;
    long M;
    int pruned;
    int method;       /* 0 LDR, 1 FCD */
    oc_cplx* A[6];    /* spectra of xx, xy, xz, yy, yz, zz */
    oc_cplx* bg[3];   /* padded b grids */
    oc_plan1d *px, *py, *pz;
    oc_cplx* work;
};

static inline long gidx(const or_core* c, long i, long j, long k) {
    return k + (long)c->Mz * (j + (long)c->My * i);
}

/* offset on the periodic grid: index i of an axis of length M with Nn
 * lattice points -> signed lattice offset, or INT32 sentinel if unused */
static int grid_offset(int i, int Nn, int M, int* off) {
    if (i < Nn) { *off = i; return 1; }
    if (i > M - Nn) { *off = i - M; return 1; }
    return 0;
}

static void fft3(or_core* c, oc_cplx* g, int sign, int prune_in, int prune_out) {
    /* forward with prune_in: data nonzero only for x<Nx, y<Ny, z<Nz.
     * inverse with prune_out: only x<Nx, y<Ny, z<Nz outputs are read. */
    const long sy = c->Mz, sx = (long)c->My * c->Mz;
    if (sign < 0) {
        int ix = prune_in ? c->Nx : c->Mx, iy = prune_in ? c->Ny : c->My;
        for (int i = 0; i < ix; i++)
            for (int j = 0; j < iy; j++) oc_fft1d(c->pz, g + i * sx + j * sy, 1, sign, c->work);
        for (int i = 0; i < ix; i++)
            for (int k = 0; k < c->Mz; k++) oc_fft1d(c->py, g + i * sx + k, sy, sign, c->work);
        for (int j = 0; j < c->My; j++)
            for (int k = 0; k < c->Mz; k++) oc_fft1d(c->px, g + j * sy + k, sx, sign, c->work);
    } else {
        /* the inverse runs the axes in the same order as the forward one */
        int ox = prune_out ? c->Nx : c->Mx, oy = prune_out ? c->Ny : c->My;
        if (!prune_out) {
            for (int i = 0; i < c->Mx; i++)
                for (int j = 0; j < c->My; j++) oc_fft1d(c->pz, g + i * sx + j * sy, 1, sign, c->work);
            for (int i = 0; i < c->Mx; i++)
                for (int k = 0; k < c->Mz; k++) oc_fft1d(c->py, g + i * sx + k, sy, sign, c->work);
            for (int j = 0; j < c->My; j++)
                for (int k = 0; k < c->Mz; k++) oc_fft1d(c->px, g + j * sy + k, sx, sign, c->work);
        } else {
            /* same transform, axes taken in the reverse order so that
             * only lines feeding the kept outputs are computed */
            for (int j = 0; j < c->My; j++)
                for (int k = 0; k < c->Mz; k++) oc_fft1d(c->px, g + j * sy + k, sx, sign, c->work);
            for (int i = 0; i < ox; i++)
                for (int k = 0; k < c->Mz; k++) oc_fft1d(c->py, g + i * sx + k, sy, sign, c->work);
            for (int i = 0; i < ox; i++)
                for (int j = 0; j < oy; j++) oc_fft1d(c->pz, g + i * sx + j * sy, 1, sign, c->work);
        }
    }
}

/* AProductCore::A_dic_generator(x, y, z, m, n) (AProductCore.cpp:573-586):
 * the LDR tensor of the image (m, n) of a lattice periodic in x and y with
 * periods Lm, Ln, damped by exp(-(gamma K r)^4), gamma = 0.01 */
/* AProductCore::A_dic_generator(x, y, z) (AProductCore.cpp:560-571) */
static void a_dic(int method, double K, double d, double x, double y, double z, double* t) {
    if (method == 1) or_fcd_inter(K, d, x, y, z, t);
    else or_ldr_inter(K, x, y, z, t);
}

static void ldr_image(int method, double K, double d, double x, double y, double z, int m, int n, double Lm,
                      double Ln, double* t) {
    const double gamma = 0.01;
    x = x + m * Lm;
    y = y + n * Ln;
    a_dic(method, K, d, x, y, z, t);
    const double ph = exp(-pow(gamma * K * sqrt(x * x + y * y + z * z), 4));
    for (int l = 0; l < 12; l++) t[l] *= ph;
}

static or_core* core_create(int Nx, int Ny, int Nz, int N, const int* R, double d, double lam, double nback,
                            int nmat, const double* material, int Mx, int My, int Mz, int periodic, int MAXm,
                            int MAXn, double Lm, double Ln, int method);

or_core* or_core_create(int Nx, int Ny, int Nz, int N, const int* R, double d, double lam,
                        double nback, int nmat, const double* material, int Mx, int My, int Mz) {
    return core_create(Nx, Ny, Nz, N, R, d, lam, nback, nmat, material, Mx, My, Mz, 0, 0, 0, 0.0, 0.0, 0);
}

or_core* or_core_create_periodic(int Nx, int Ny, int Nz, int N, const int* R, double d, double lam, double nback,
                                 int nmat, const double* material, int MAXm, int MAXn, double Lm, double Ln,
                                 int Mx, int My, int Mz) {
    if (MAXm < 0 || MAXn < 0) return NULL;
    return core_create(Nx, Ny, Nz, N, R, d, lam, nback, nmat, material, Mx, My, Mz, 1, MAXm, MAXn, Lm, Ln, 0);
}

or_core* or_core_create_method(int Nx, int Ny, int Nz, int N, const int* R, double d, double lam, double nback,
                               int nmat, const double* material, int method, int periodic, int MAXm, int MAXn,
                               double Lm, double Ln, int Mx, int My, int Mz) {
    if (method != 0 && method != 1) return NULL;
    if (periodic && (MAXm < 0 || MAXn < 0)) return NULL;
    return core_create(Nx, Ny, Nz, N, R, d, lam, nback, nmat, material, Mx, My, Mz, periodic, MAXm, MAXn, Lm, Ln,
                       method);
}

static or_core* core_create(int Nx, int Ny, int Nz, int N, const int* R, double d, double lam, double nback,
                            int nmat, const double* material, int Mx, int My, int Mz, int periodic, int MAXm,
                            int MAXn, double Lm, double Ln, int method) {
    if (Nx < 1 || Ny < 1 || Nz < 1 || N < 0 || nmat < 1) return NULL;
    or_core* c = (or_core*)calloc(1, sizeof(or_core));
    if (!c) return NULL;
    c->Nx = Nx; c->Ny = Ny; c->Nz = Nz; c->N = N;
    c->d = d; c->lam = lam; c->nback = nback;
    c->method = method;
    c->K = 2 * OR_PI / (lam / nback); /* AProductCore.cpp:17 */
    c->nmat = nmat;
    c->material = (double*)malloc(sizeof(double) * 2 * nmat);
    or_normalize_material(nmat, material, nback, c->material);
    c->R = (int*)malloc(sizeof(int) * 3 * (size_t)(N > 0 ? N : 1));
    if (N > 0) memcpy(c->R, R, sizeof(int) * 3 * (size_t)N);
    for (int i = 0; i < N; i++) {
        if (R[3 * i] < 0 || R[3 * i] >= Nx || R[3 * i + 1] < 0 || R[3 * i + 1] >= Ny ||
            R[3 * i + 2] < 0 || R[3 * i + 2] >= Nz) {
            or_core_destroy(c);
            return NULL;
        }
    }
    c->Mx = Mx > 0 ? Mx : 2 * Nx - 1; /* AProductCore.cpp:41-44 */
    c->My = My > 0 ? My : 2 * Ny - 1;
    c->Mz = Mz > 0 ? Mz : 2 * Nz - 1;
    if (c->Mx < 2 * Nx - 1 || c->My < 2 * Ny - 1 || c->Mz < 2 * Nz - 1) {
        or_core_destroy(c);
        return NULL;
    }
    c->M = (long)c->Mx * c->My * c->Mz;
    c->px = oc_plan1d_create(c->Mx);
    c->py = oc_plan1d_create(c->My);
    c->pz = oc_plan1d_create(c->Mz);
    int nmax = c->Mx > c->My ? c->Mx : c->My;
    if (c->Mz > nmax) nmax = c->Mz;
    c->work = (oc_cplx*)malloc(sizeof(oc_cplx) * 2 * (size_t)nmax);
    for (int l = 0; l < 6; l++) c->A[l] = (oc_cplx*)calloc((size_t)c->M, sizeof(oc_cplx));
    for (int l = 0; l < 3; l++) c->bg[l] = (oc_cplx*)calloc((size_t)c->M, sizeof(oc_cplx));
    /* AProductCore.cpp:53-194: the tensor at every signed lattice offset */
    double t[12];
    for (int i = 0; i < c->Mx; i++) {
        int ox;
        if (!grid_offset(i, Nx, c->Mx, &ox)) continue;
        for (int j = 0; j < c->My; j++) {
            int oy;
            if (!grid_offset(j, Ny, c->My, &oy)) continue;
            for (int k = 0; k < c->Mz; k++) {
                int oz;
                if (!grid_offset(k, Nz, c->Mz, &oz)) continue;
                if (periodic) {
                    /* AProductCore.cpp:300-328: the sum over the images, m outer, n inner */
                    double ti[12];
                    memset(t, 0, sizeof(t));
                    for (int m = -MAXm; m <= MAXm; m++)
                        for (int n = -MAXn; n <= MAXn; n++) {
                            ldr_image(method, c->K, d, d * ox, d * oy, d * oz, m, n, Lm, Ln, ti);
                            for (int l = 0; l < 12; l++) t[l] = t[l] + ti[l];
                        }
                } else {
                    a_dic(method, c->K, d, d * ox, d * oy, d * oz, t);
                }
                long g = gidx(c, i, j, k);
                for (int l = 0; l < 6; l++) {
                    c->A[l][g].re = t[2 * l];
                    c->A[l][g].im = t[2 * l + 1];
                }
            }
        }
    }
    /* AProductCore.cpp:212-229: forward transforms of the six components */
    for (int l = 0; l < 6; l++) fft3(c, c->A[l], -1, 0, 0);
    return c;
}

void or_core_destroy(or_core* c) {
    if (!c) return;
    for (int l = 0; l < 6; l++) free(c->A[l]);
    for (int l = 0; l < 3; l++) free(c->bg[l]);
    oc_plan1d_destroy(c->px);
    oc_plan1d_destroy(c->py);
    oc_plan1d_destroy(c->pz);
    free(c->work);
    free(c->material);
    free(c->R);
    free(c);
}

void or_core_set_pruned(or_core* c, int pruned) { c->pruned = pruned; }
double or_core_K(const or_core* c) { return c->K; }
void or_core_material(const or_core* c, double* out) {
    memcpy(out, c->material, sizeof(double) * 2 * c->nmat);
}
void or_core_grid(const or_core* c, int* out3) {
    out3[0] = c->Mx; out3[1] = c->My; out3[2] = c->Mz;
}

/* AProductCore.cpp:697-758 (B2Bs / Conv / Conv2B of kernel.cu:44-125 are
 * the deinterleave, the symmetric 3x3 spectral product and the
 * re-interleave, done here directly on the three component grids) */
int or_aproduct(or_core* c, const double* b, double* y) {
    const long M = c->M;
    for (int l = 0; l < 3; l++) memset(c->bg[l], 0, sizeof(oc_cplx) * (size_t)M);
    for (int i = 0; i < c->N; i++) {
        long g = gidx(c, c->R[3 * i], c->R[3 * i + 1], c->R[3 * i + 2]);
        for (int j = 0; j < 3; j++) {
            c->bg[j][g].re = b[2 * (3 * i + j)];
            c->bg[j][g].im = b[2 * (3 * i + j) + 1];
        }
    }
    for (int l = 0; l < 3; l++) fft3(c, c->bg[l], -1, c->pruned, 0);
    for (long g = 0; g < M; g++) {
        cd bx = c->bg[0][g].re + I * c->bg[0][g].im;
        cd by = c->bg[1][g].re + I * c->bg[1][g].im;
        cd bz = c->bg[2][g].re + I * c->bg[2][g].im;
        cd a[6];
        for (int l = 0; l < 6; l++) a[l] = c->A[l][g].re + I * c->A[l][g].im;
        cd cx = (a[0] * bx + a[1] * by) + a[2] * bz;
        cd cy = (a[1] * bx + a[3] * by) + a[4] * bz;
        cd cz = (a[2] * bx + a[4] * by) + a[5] * bz;
        c->bg[0][g].re = creal(cx); c->bg[0][g].im = cimag(cx);
        c->bg[1][g].re = creal(cy); c->bg[1][g].im = cimag(cy);
        c->bg[2][g].re = creal(cz); c->bg[2][g].im = cimag(cz);
    }
    for (int l = 0; l < 3; l++) fft3(c, c->bg[l], +1, 0, c->pruned);
    for (int i = 0; i < c->N; i++) {
        long g = gidx(c, c->R[3 * i], c->R[3 * i + 1], c->R[3 * i + 2]);
        for (int j = 0; j < 3; j++) {
            y[2 * (3 * i + j)] = c->bg[j][g].re / (double)M;
            y[2 * (3 * i + j) + 1] = c->bg[j][g].im / (double)M;
        }
    }
    return 0;
}

int or_aproduct_direct(int N, const int* R, double d, double K, const double* b, double* y) {
    double t[12];
    for (int i = 0; i < N; i++) {
        cd s[3] = {0, 0, 0};
        for (int j = 0; j < N; j++) {
            or_ldr_inter(K, d * (R[3 * i] - R[3 * j]), d * (R[3 * i + 1] - R[3 * j + 1]),
                         d * (R[3 * i + 2] - R[3 * j + 2]), t);
            cd a[6];
            for (int l = 0; l < 6; l++) a[l] = t[2 * l] + I * t[2 * l + 1];
            cd bx = ld(b, 3 * j), by = ld(b, 3 * j + 1), bz = ld(b, 3 * j + 2);
            s[0] += a[0] * bx + a[1] * by + a[2] * bz;
            s[1] += a[1] * bx + a[3] * by + a[4] * bz;
            s[2] += a[2] * bx + a[4] * by + a[5] * bz;
        }
        for (int c = 0; c < 3; c++) st(y, 3 * i + c, s[c]);
    }
    return 0;
}

struct or_model {
    or_core* core;
    double nK[3], nE0[3], E0;
    long n3;
    cd *P, *E, *al, *diel, *Ein;
    double *tmp_in, *tmp_out;
};

/* DDAModel.cpp:47-51 and :463-467 */
static void model_incident(or_model* m) {
    const or_core* c = m->core;
    for (int i = 0; i < c->N; i++) {
        double ph = c->K * c->d *
                    (m->nK[0] * c->R[3 * i] + m->nK[1] * c->R[3 * i + 1] + m->nK[2] * c->R[3 * i + 2]);
        cd e = cos(ph) + I * sin(ph);
        for (int j = 0; j < 3; j++) m->E[3 * i + j] = m->E0 * m->nE0[j] * e;
    }
}

/* DDAModel.cpp:54-63 / :470-487: eps by linear interpolation in the
 * material table, al = 1 / alpha_LDR(eps) */
int or_model_update_alpha(or_model* m, const double* diel_old) {
    const or_core* c = m->core;
    for (long i = 0; i < m->n3; i++) {
        double v = diel_old[i];
        int lf = (int)floor(v);
        int ln = lf + 1;
        if (lf >= 1) ln = lf;
        if (lf < 0 || lf >= c->nmat || ln >= c->nmat) return 1;
        cd mf = ld(c->material, lf), mn = ld(c->material, ln);
        cd eps = mf + (v - (double)lf) * (mn - mf);
        m->diel[i] = eps;
        double a[2];
        or_get_alpha(c->lam, c->K, c->d, creal(eps), cimag(eps), m->nE0, m->nK, a);
        m->al[i] = 1.0 / (a[0] + I * a[1]);
    }
    return 0;
}

or_model* or_model_create(or_core* c, const double* nK, double E0, const double* nE0,
                          const double* diel_old) {
    or_model* m = (or_model*)calloc(1, sizeof(or_model));
    if (!m) return NULL;
    m->core = c;
    for (int j = 0; j < 3; j++) { m->nK[j] = nK[j]; m->nE0[j] = nE0[j]; }
    m->E0 = E0;
    m->n3 = 3L * c->N;
    size_t nb = sizeof(cd) * (size_t)(m->n3 > 0 ? m->n3 : 1);
    m->P = (cd*)calloc(1, nb);
    m->E = (cd*)calloc(1, nb);
    m->al = (cd*)calloc(1, nb);
    m->diel = (cd*)calloc(1, nb);
    m->Ein = (cd*)calloc(1, nb);
    m->tmp_in = (double*)calloc(1, nb);
    m->tmp_out = (double*)calloc(1, nb);
    model_incident(m);
    if (or_model_update_alpha(m, diel_old)) {
        or_model_destroy(m);
        return NULL;
    }
    return m;
}

void or_model_destroy(or_model* m) {
    if (!m) return;
    free(m->P); free(m->E); free(m->al); free(m->diel); free(m->Ein);
    free(m->tmp_in); free(m->tmp_out);
    free(m);
}

void or_model_change_E(or_model* m, const double* E) {
    for (long i = 0; i < m->n3; i++) m->E[i] = ld(E, i);
}
void or_model_reset_E(or_model* m) { model_incident(m); }
void or_model_initialize_P(or_model* m, const double* P) {
    for (long i = 0; i < m->n3; i++) m->P[i] = ld(P, i);
}

/* DDAModel.cpp:577-586 */
static void awa(or_model* m, const cd* b, cd* out) {
    for (long i = 0; i < m->n3; i++) st(m->tmp_in, i, b[i]);
    or_aproduct(m->core, m->tmp_in, m->tmp_out);
    for (long i = 0; i < m->n3; i++) out[i] = ld(m->tmp_out, i) + b[i] * m->al[i];
}

int or_model_aproduct_with_alb(or_model* m, const double* b, double* y) {
    cd* bb = (cd*)malloc(sizeof(cd) * (size_t)m->n3);
    cd* yy = (cd*)malloc(sizeof(cd) * (size_t)m->n3);
    for (long i = 0; i < m->n3; i++) bb[i] = ld(b, i);
    awa(m, bb, yy);
    for (long i = 0; i < m->n3; i++) st(y, i, yy[i]);
    free(bb);
    free(yy);
    return 0;
}

/* Eigen's a.dot(b) = sum conj(a_i) b_i (eigen Dot.h:62), summed in the
 * order Eigen 3.3's linear-vectorised reduction uses for complex<double>
 * with SSE2 packets of one element (eigen Redux.h:227-281): two running
 * sums over the even and the odd indices, added together, then the last
 * element when n is odd.  Reproducing the order makes the restatement
 * bit-identical to the reference's solve. */
static cd dotc(const cd* a, const cd* b, long n) {
    if (n <= 0) return 0;
    if (n == 1) return conj(a[0]) * b[0];
    cd s0 = conj(a[0]) * b[0];
    cd s1 = conj(a[1]) * b[1];
    long i = 2;
    for (; i + 1 < n; i += 2) {
        s0 += conj(a[i]) * b[i];
        s1 += conj(a[i + 1]) * b[i + 1];
    }
    s0 += s1;
    if (i < n) s0 += conj(a[i]) * b[i];
    return s0;
}
static double nrm(const cd* a, long n) {
    double s = 0;
    for (long i = 0; i < n; i++) s += creal(a[i]) * creal(a[i]) + cimag(a[i]) * cimag(a[i]);
    return sqrt(s);
}

/* DDAModel.cpp:131-260.  Returns OR_CONVERGED, OR_BREAKDOWN or OR_MAXITER.
 * *iterations / *error follow the reference: the loop index + 1 on
 * convergence or breakdown; left unchanged when the iteration limit is
 * reached (the reference keeps its previous ITERATION then). */
int or_model_bicgstab(or_model* m, int max_it, double max_err, int* iterations, double* error) {
    const long n = m->n3;
    cd* buf = (cd*)calloc((size_t)(10 * (n > 0 ? n : 1)), sizeof(cd));
    cd *p = buf, *t = buf + n, *r = buf + 2 * n, *r0 = buf + 3 * n, *rl = buf + 4 * n;
    cd *u = buf + 5 * n, *z = buf + 6 * n, *Ap = buf + 7 * n, *At = buf + 8 * n, *Ax = buf + 9 * n;
    cd alpha, beta, zeta;
    int status = OR_MAXITER;

    awa(m, m->P, Ax);
    for (long i = 0; i < n; i++) { r[i] = m->E[i] - Ax[i]; r0[i] = r[i]; p[i] = r[i]; }
    awa(m, p, Ap);
    alpha = dotc(r0, r, n) / dotc(r0, Ap, n);
    for (long i = 0; i < n; i++) t[i] = r[i] - alpha * Ap[i];
    awa(m, t, At);
    zeta = dotc(At, t, n) / dotc(At, At, n);
    for (long i = 0; i < n; i++) {
        u[i] = zeta * Ap[i];
        z[i] = zeta * r[i] - alpha * u[i];
        m->P[i] = m->P[i] + alpha * p[i] + z[i];
        rl[i] = r[i];
        r[i] = t[i] - zeta * At[i];
    }
    const double En = nrm(m->E, n);
    for (int it = 0; it < max_it; it++) {
        cd r0rl = dotc(r0, rl, n);
        if (creal(r0rl) == 0 && cimag(r0rl) == 0) {
            *error = nrm(r, n) / En;
            *iterations = it + 1;
            status = OR_BREAKDOWN;
            break;
        }
        beta = (alpha / zeta) * dotc(r0, r, n) / r0rl;
        for (long i = 0; i < n; i++) p[i] = r[i] + beta * (p[i] - u[i]);
        awa(m, p, Ap);
        alpha = dotc(r0, r, n) / dotc(r0, Ap, n);
        for (long i = 0; i < n; i++) t[i] = r[i] - alpha * Ap[i];
        awa(m, t, At);
        zeta = dotc(At, t, n) / dotc(At, At, n);
        for (long i = 0; i < n; i++) {
            u[i] = zeta * Ap[i];
            z[i] = zeta * r[i] - alpha * u[i];
            m->P[i] = m->P[i] + alpha * p[i] + z[i];
            rl[i] = r[i];
            r[i] = t[i] - zeta * At[i];
        }
        double e = nrm(r, n) / En;
        if (e <= max_err) {
            *error = e;
            *iterations = it + 1;
            status = OR_CONVERGED;
            break;
        }
    }
    free(buf);
    return status;
}

/* DDAModel.cpp:567-575 */
void or_model_update_E_in_structure(or_model* m) {
    for (long i = 0; i < m->n3; i++) {
        cd lf = (2.0 + m->diel[i]) / 3.0;
        m->Ein[i] = m->al[i] * m->P[i] / lf;
    }
}

/* The field at off-lattice points: E(r) = E_ext(r) - sum_i A(r - d R_i) P_i
 * with E_ext = E0 nE0 exp(i K nK.r), accumulated as ObjPointEDDAModel does
 * (ObjDDAModel.cpp:42-44 for E_ext, :57-66 for the terms, :83-96 for the
 * order: start at E_ext, subtract dipole by dipole).  DDAModel::solve_E
 * (DDAModel.cpp:530-565) sums the same terms.  pts: npts x 3 in nm;
 * E_out: npts x 3 complex, interleaved. */
void or_model_field_at(const or_model* m, int npts, const double* pts, double* E_out) {
    const or_core* c = m->core;
    double A[12];
    for (int p = 0; p < npts; p++) {
        const double x = pts[3 * p], y = pts[3 * p + 1], z = pts[3 * p + 2];
        const double ph = c->K * (m->nK[0] * x + m->nK[1] * y + m->nK[2] * z);
        const cd e = cos(ph) + sin(ph) * I;
        cd s[3];
        for (int j = 0; j < 3; j++) s[j] = (m->E0 * m->nE0[j]) * e;
        for (int i = 0; i < c->N; i++) {
            a_dic(c->method, c->K, c->d, x - c->d * c->R[3 * i], y - c->d * c->R[3 * i + 1], z - c->d * c->R[3 * i + 2],
                  A);
            const cd a00 = A[0] + A[1] * I, a01 = A[2] + A[3] * I, a02 = A[4] + A[5] * I;
            const cd a11 = A[6] + A[7] * I, a12 = A[8] + A[9] * I, a22 = A[10] + A[11] * I;
            const cd px = m->P[3 * i], py = m->P[3 * i + 1], pz = m->P[3 * i + 2];
            s[0] -= a00 * px + a01 * py + a02 * pz;
            s[1] -= a01 * px + a11 * py + a12 * pz;
            s[2] -= a02 * px + a12 * py + a22 * pz;
        }
        for (int j = 0; j < 3; j++) st(E_out, 3L * p + j, s[j]);
    }
}

void or_model_get(const or_model* m, int what, double* out) {
    const cd* src = what == 0 ? m->P : what == 1 ? m->E : what == 2 ? m->al : what == 3 ? m->diel : m->Ein;
    for (long i = 0; i < m->n3; i++) st(out, i, src[i]);
}
