// tdda_tensor.cuh -- the dipole interaction tensors, for device kernels and
// host code alike: LDR (AProductCore.cpp:588-623) and FCD (AProductCore.cpp:
// 625-695), the latter with the sine and cosine integrals interpolated in the
// tables the reference reads (SiCi.cpp:8-47, written by SiCi/SiCi.py at
// x = 0.1 k, k = 1 .. 999999).  Each returns the six components xx, xy, xz,
// yy, yz, zz; r = 0 gives the zero tensor.
#pragma once

#include <cuda_runtime.h>
#include <math.h>

namespace tdda {

constexpr int kSiCiN = 999999;
constexpr double kSiCiDis = 0.1;
constexpr double kPiT = 3.14159265358979323846;

// which tensor a kernel evaluates; si / ci: the device tables (FCD only)
struct Interaction {
    int fcd;
    const double* si;
    const double* ci;
};

__host__ __device__ inline double2 t_mul(double2 a, double2 b) {
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ inline double2 t_div(double2 a, double2 b) {
    // Smith's algorithm (R. L. Smith, CACM 5(8), 1962)
    if (fabs(b.x) >= fabs(b.y)) {
        const double r = b.y / b.x, den = b.x + b.y * r;
        return make_double2((a.x + a.y * r) / den, (a.y - a.x * r) / den);
    }
    const double r = b.x / b.y, den = b.x * r + b.y;
    return make_double2((a.x * r + a.y) / den, (a.y * r - a.x) / den);
}

// LDR_inter (AProductCore.cpp:588-623) at the offset (x, y, z) nm
__host__ __device__ inline void ldr_tensor(double K, double x, double y, double z, double2 (&t)[6]) {
    const double xs = x * x, ys = y * y, zs = z * z;
    const double rn = sqrt(xs + ys + zs);
    if (rn == 0.0) {
        for (int l = 0; l < 6; l++) t[l] = make_double2(0.0, 0.0);
        return;
    }
    const double rsq = rn * rn, rcu = rn * rn * rn;
    const double sn = sin(K * rn), cs = cos(K * rn);
    const double2 c1 = make_double2(cs / rcu, sn / rcu);        // e^{iKr} / r^3
    const double2 c2 = make_double2(1.0 / rsq, -(K * rn) / rsq);  // (1 - iKr) / r^2
    const double2 c3 = make_double2(K * K - 3.0 * c2.x, -3.0 * c2.y);
    double2 v[6];
    v[0] = make_double2(c2.x * (rsq - 3 * xs) - K * K * (ys + zs), c2.y * (rsq - 3 * xs));
    v[1] = make_double2(x * y * c3.x, x * y * c3.y);
    v[2] = make_double2(z * x * c3.x, z * x * c3.y);
    v[3] = make_double2(c2.x * (rsq - 3 * ys) - K * K * (zs + xs), c2.y * (rsq - 3 * ys));
    v[4] = make_double2(y * z * c3.x, y * z * c3.y);
    v[5] = make_double2(c2.x * (rsq - 3 * zs) - K * K * (xs + ys), c2.y * (rsq - 3 * zs));
    for (int l = 0; l < 6; l++) t[l] = t_mul(c1, v[l]);
}

// Si(x) and Ci(x), x > 0, from Abramowitz & Stegun: the power series 5.2.14 /
// 5.2.16 for x <= 4; above, E1(ix) = -Ci(x) + i (Si(x) - pi/2) (5.2.23) with
// E1(z) from its even continued fraction 5.1.22, e^{-z} / (z + 1 - 1/(z + 3 -
// 4/(z + 5 - ...))), by the modified Lentz method (Thompson & Barnett,
// J. Comput. Phys. 64, 1986).
__host__ __device__ inline void sici(double x, double* si, double* ci) {
    const double euler = 0.57721566490153286061;
    if (x <= 4.0) {
        double s = 0.0, c = 0.0, term = x;  // term = (-1)^k x^(2k+1) / (2k+1)!
        for (int k = 0; k < 60; k++) {
            const double sk = term / (2 * k + 1);
            s += sk;
            const double tc = -term * x / (2 * k + 2);
            const double ck = tc / (2 * k + 2);
            c += ck;
            term = tc * x / (2 * k + 3);
            if (fabs(sk) <= 1e-17 * fabs(s) && fabs(ck) <= 1e-17 * (fabs(c) + 1e-300)) break;
        }
        *si = s;
        *ci = euler + log(x) + c;
        return;
    }
    const double tiny = 1e-300;
    double2 b = make_double2(1.0, x);
    double2 f = b, C = b, D = make_double2(0.0, 0.0);
    for (int j = 1; j < 1000; j++) {
        const double a = -(double)j * (double)j;
        b.x += 2.0;
        D = make_double2(b.x + a * D.x, b.y + a * D.y);
        if (hypot(D.x, D.y) < tiny) D = make_double2(tiny, 0.0);
        C = t_div(make_double2(a, 0.0), C);
        C = make_double2(b.x + C.x, b.y + C.y);
        if (hypot(C.x, C.y) < tiny) C = make_double2(tiny, 0.0);
        D = t_div(make_double2(1.0, 0.0), D);
        const double2 delta = t_mul(C, D);
        f = t_mul(f, delta);
        if (hypot(delta.x - 1.0, delta.y) < 1e-16) break;
    }
    const double2 e1 = t_div(make_double2(cos(x), -sin(x)), f);  // e^{-ix} / f
    *ci = -e1.x;
    *si = kPiT / 2 + e1.y;
}

// SiCi::get_Si / get_Ci (SiCi.cpp:27-47): linear interpolation between the
// table nodes floor(x/dis) dis and ceil(x/dis) dis.  On a node it returns the
// node value (the reference divides 0 by 0 there); below the first node and
// past the last it extends the end interval (the reference reads outside its
// table).  tab == nullptr evaluates the node values with sici() (host).
__host__ __device__ inline double sici_table_value(const double* tab, int p, bool want_si) {
    if (tab) return tab[p];
    double s, c;
    sici(kSiCiDis * (p + 1), &s, &c);
    return want_si ? s : c;
}
__host__ __device__ inline double sici_interp(const double* tab, double x, bool want_si) {
    double q = x / kSiCiDis;
    if (!(q >= 0.0)) q = 0.0;                    // NaN or negative: the first interval
    if (q > (double)kSiCiN) q = (double)kSiCiN;  // past the table: the last interval
    int p1 = (int)floor(q) - 1, p2 = (int)ceil(q) - 1;
    if (p1 < 0) p1 = 0, p2 = 1;
    if (p2 > kSiCiN - 1) p2 = kSiCiN - 1, p1 = kSiCiN - 2;
    if (p1 == p2) return sici_table_value(tab, p1, want_si);
    const double v1 = sici_table_value(tab, p1, want_si), v2 = sici_table_value(tab, p2, want_si);
    const double a1 = (p1 + 1) * kSiCiDis, a2 = (p2 + 1) * kSiCiDis;
    return v1 + ((v2 - v1) / (a2 - a1)) * (x - a1);
}

// FCD_inter (AProductCore.cpp:625-695), cut-off Kf = pi / d
__host__ __device__ inline void fcd_tensor(double K, double d, double x, double y, double z, const double* si_tab,
                                           const double* ci_tab, double2 (&t)[6]) {
    const double xs = x * x, ys = y * y, zs = z * z;
    const double rn = sqrt(xs + ys + zs);
    if (rn == 0.0) {
        for (int l = 0; l < 6; l++) t[l] = make_double2(0.0, 0.0);
        return;
    }
    const double xy = x * y, yz = y * z, zx = z * x;
    const double rsq = rn * rn, rcu = rn * rn * rn;
    const double Kf = kPiT / d;
    const double ap = (Kf + K) * rn, am = (Kf - K) * rn;
    const double Cz = sici_interp(ci_tab, ap, false), Cf = sici_interp(ci_tab, am, false);
    const double Sz = sici_interp(si_tab, ap, true), Sf = sici_interp(si_tab, am, true);
    const double cp = cos(ap), sp = sin(ap), cm = cos(am), sm = sin(am);
    const double Cz1 = cp / rn, Cf1 = cm / rn, Sz1 = sp / rn, Sf1 = sm / rn;
    const double Cz2 = (-ap * sp - cp) / rsq, Cf2 = (-am * sm - cm) / rsq;
    const double Sz2 = (ap * cp - sp) / rsq, Sf2 = (am * cm - sm) / rsq;
    const double kr = K * rn;
    const double sikr = sin(kr), cskr = cos(kr);
    const double sikfr = sin(Kf * rn), cskfr = cos(Kf * rn);
    const double2 CC = make_double2(Cf - Cz, kPiT);  // pi i + Cf - Cz
    const double C1C1 = Cf1 - Cz1, C2C2 = Cf2 - Cz2;
    const double SS = Sz + Sf, S1S1 = Sz1 + Sf1, S2S2 = Sz2 + Sf2;
    // gf = (sin(kr) CC + cos(kr) SS) / (pi r)
    const double2 gf = make_double2((sikr * CC.x + cskr * SS) / (kPiT * rn), sikr * CC.y / (kPiT * rn));
    const double a1 = kr * cskr - sikr, b1 = -(kr * sikr + cskr);
    const double2 const1 = make_double2(a1 * CC.x + b1 * SS + rn * sikr * C1C1 + rn * cskr * S1S1, a1 * CC.y);
    const double a2 = -K * kr * sikr, b2 = -K * kr * cskr;
    const double2 const2 = make_double2(a2 * CC.x + b2 * SS + 2 * kr * cskr * C1C1 - 2 * kr * sikr * S1S1 +
                                            rn * sikr * C2C2 + rn * cskr * S2S2,
                                        a2 * CC.y);
    const double2 gf1 = make_double2(const1.x / (kPiT * rsq), const1.y / (kPiT * rsq));
    const double2 gf2 = make_double2((rn * const2.x - 2.0 * const1.x) / (kPiT * rcu),
                                     (rn * const2.y - 2.0 * const1.y) / (kPiT * rcu));
    const double hr = (sikfr - Kf * rn * cskfr) / (2.0 * kPiT * kPiT * rcu);
    const double2 term1 = make_double2(K * K * gf.x + gf1.x / rn + (4.0 * kPiT / 3.0) * hr, K * K * gf.y + gf1.y / rn);
    const double2 term2 = make_double2((gf2.x - gf1.x / rn) / rsq, (gf2.y - gf1.y / rn) / rsq);
    t[0] = make_double2(-(term1.x + xs * term2.x), -(term1.y + xs * term2.y));
    t[1] = make_double2(-xy * term2.x, -xy * term2.y);
    t[2] = make_double2(-zx * term2.x, -zx * term2.y);
    t[3] = make_double2(-(term1.x + ys * term2.x), -(term1.y + ys * term2.y));
    t[4] = make_double2(-yz * term2.x, -yz * term2.y);
    t[5] = make_double2(-(term1.x + zs * term2.x), -(term1.y + zs * term2.y));
}

// AProductCore::A_dic_generator (AProductCore.cpp:560-571)
__host__ __device__ inline void interaction_tensor(const Interaction& it, double K, double d, double x, double y, double z,
                                                   double2 (&t)[6]) {
    if (it.fcd) fcd_tensor(K, d, x, y, z, it.si, it.ci, t);
    else ldr_tensor(K, x, y, z, t);
}

}  // namespace tdda
