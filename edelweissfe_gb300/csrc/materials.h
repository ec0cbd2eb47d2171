// Small-strain constitutive updates of the element kernel: linear elasticity and J2 plasticity
// with isotropic hardening, in FP64.
//
// Plain C++ on doubles (exp, sqrt, fabs of <math.h>), so that the same source compiles for the
// device (elements.cu) and for the host, where a test runs it on random states against the
// oracle (tests/native/materials_check.cpp).
//
// props: the reference's material row [E, nu, fy0, HLin, dfy, delta] (J2) or [E, nu], plus
// lambda and G in slots 6 and 7.  Stress and strain are Voigt 6-vectors in the reference's order
// [11, 22, 33, 12, 13, 23] with engineering shear strains.
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define EF_MAT_HD __host__ __device__ __forceinline__
#define EF_MAT_UNROLL _Pragma("unroll")
#else
#define EF_MAT_HD inline
#define EF_MAT_UNROLL
#endif

namespace ef {

struct MatOut {
    double lt, mt, c1;  // tangent C = lt 1x1 + 2 mt I_s - c1 n x n (Voigt, engineering shear)
    double n[6];
};

// Linear elastic update: stress += Ei dStrain; tangent Ei  (linearelastic.py:185-210)
// props[6], props[7] hold lambda = E nu / ((1 + nu)(1 - 2 nu)) and G = E / (2 (1 + nu)), formed
// once on the host (two FP64 divisions per Gauss point fewer)
EF_MAT_HD void mat_linear_elastic(const double* props, double* sig, const double* de, MatOut& o) {
    const double lam = props[6], mu = props[7];
    const double tr = de[0] + de[1] + de[2];
    sig[0] += lam * tr + 2.0 * mu * de[0];
    sig[1] += lam * tr + 2.0 * mu * de[1];
    sig[2] += lam * tr + 2.0 * mu * de[2];
    sig[3] += mu * de[3];
    sig[4] += mu * de[4];
    sig[5] += mu * de[5];
    o.lt = lam;
    o.mt = mu;
    o.c1 = 0.0;
}

// J2 radial return with isotropic hardening fy = fy0 + H k + dfy (1 - exp(-delta k)) (vonmises.py:186-254)
// returns false where the reference raises CutbackRequest
EF_MAT_HD bool mat_von_mises(const double* props, double* sig, double* kappa, const double* de, MatOut& o) {
    const double fy0 = props[2], HL = props[3], dfy = props[4], dl = props[5];
    const double lam = props[6], G = props[7];  // formed on the host (see mat_linear_elastic)
    o.lt = lam;
    o.mt = G;
    o.c1 = 0.0;
    const double nde2 = de[0] * de[0] + de[1] * de[1] + de[2] * de[2] + de[3] * de[3] + de[4] * de[4] + de[5] * de[5];
    if (nde2 < 1e-28) return true;  // zero-increment shortcut |de| < 1e-14: stress and kappa unchanged, C = Ei
    double t[6];
    const double tr = de[0] + de[1] + de[2];
    t[0] = sig[0] + lam * tr + 2.0 * G * de[0];
    t[1] = sig[1] + lam * tr + 2.0 * G * de[1];
    t[2] = sig[2] + lam * tr + 2.0 * G * de[2];
    t[3] = sig[3] + G * de[3];
    t[4] = sig[4] + G * de[4];
    t[5] = sig[5] + G * de[5];
    const double p = (t[0] + t[1] + t[2]) * (1.0 / 3.0);
    double d[6] = {t[0] - p, t[1] - p, t[2] - p, t[3], t[4], t[5]};
    const double dn2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2] + 2.0 * (d[3] * d[3] + d[4] * d[4] + d[5] * d[5]);
    const double k0 = *kappa;
    const double s23 = 0.81649658092772603;  // sqrt(2/3)
    const double s6 = 2.4494897427831781;    // sqrt(6)
    // with dfy = 0 the exponential terms are exact zeros: skipped (FP64 exp is expensive here)
    const bool expo = dfy != 0.0;
    const double fyk = fy0 + HL * k0 + (expo ? dfy * (1.0 - exp(-dl * k0)) : 0.0);
    const double lim = s23 * fyk;
    // yield test |dev t| - sqrt(2/3) fy > 0, on squares (the square root only where plastic)
    if (lim <= 0.0 || dn2 > lim * lim) {
        const double dn = sqrt(dn2);
        double dk = 0.0;
        double R = dn - s23 * fyk;
        int it = 0;
        while (fabs(R) > 1e-12) {
            if (it == 15) return false;
            const double dR = -s6 * G - s23 * (HL + (expo ? dfy * dl * exp(-dl * (k0 + dk)) : 0.0));
            dk -= R / dR;
            ++it;
            const double kk = k0 + dk;
            R = dn - s6 * G * dk - s23 * (fy0 + HL * kk + (expo ? dfy * (1.0 - exp(-dl * kk)) : 0.0));
        }
        const double dLam = 1.2247448713915889 * dk;  // sqrt(3/2)
        const double k1 = k0 + dk;
        *kappa = k1;
        const double inv = 1.0 / dn;
EF_MAT_UNROLL
        for (int i = 0; i < 6; ++i) {
            o.n[i] = d[i] * inv;
            sig[i] = t[i] - 2.0 * G * dLam * o.n[i];
        }
        const double hp = HL + (expo ? dfy * dl * exp(-dl * k1) : 0.0);
        const double c1 = 2.0 * G * (1.0 / (1.0 + hp / (3.0 * G)) - 2.0 * G * dLam * inv);
        const double c2 = 4.0 * G * G * dLam * inv;
        o.c1 = c1;
        o.lt = lam + c2 * (1.0 / 3.0);
        o.mt = G - 0.5 * c2;
    } else {
EF_MAT_UNROLL
        for (int i = 0; i < 6; ++i) sig[i] = t[i];
    }
    return true;
}

}  // namespace ef

#undef EF_MAT_HD
#undef EF_MAT_UNROLL
