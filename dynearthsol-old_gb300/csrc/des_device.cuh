// Device arithmetic of the DynEarthSol3D step, FP64.
//
// Every function restates one reference routine with the same sequence of
// IEEE operations (the file is compiled with -fmad=false, so no multiply-add
// is fused, and CUDA's double division and square root are correctly
// rounded), which makes the results bit-identical to the reference's own
// functions wherever no transcendental is involved.  sin/cos/atan2/tan/pow/
// exp are CUDA's; where their argument is a material constant the host-side
// libm value is used instead (MatTable), which is exactly what the reference
// computes.
#pragma once

#include <cstdint>

#include "des_softf64.cuh"

namespace des {

constexpr double kDeg2Rad = 3.1415926535897932384626433832795 / 180;   // constants.hpp:76
constexpr double kEps = 2.220446049250313080847263336181640625e-16;     // DBL_EPSILON
constexpr unsigned kBoundX0 = 1, kBoundX1 = 2, kBoundY0 = 4, kBoundY1 = 8, kBoundZ0 = 16,
                   kBoundZ1 = 32, kBoundAny = 0x3ff;
constexpr int kMaxMat = 16;
constexpr int kMaxMix = 256;

// Static material data of one "mix": a distinct vector of per-element marker
// counts (the rows of elemmarkers).  Means that depend only on the counts are
// computed on the host with the reference's arithmetic (matprops.cxx:436-461).
struct Mix {
    double bulkm, shearm, cp, k;   // harmonic / arithmetic means
    double rho_qs;                 // bulkm / (pseudo_speed^2)  (geometry.cxx:356-357)
    double dt_maxwell;             // 0.5 visc_min / (1e-40 + shearm)  (geometry.cxx:303-304)
    int    count[kMaxMat];
    int    n;                      // total markers
    int    single;                 // >= 0: the only material present, with a power-of-two count
};

// Per-material constants (matprops.cxx:553-569 vectors, expanded to nmat).
struct MatTable {
    int    nmat, nmix;
    double rho0[kMaxMat], alpha[kMaxMat];
    double vexp_pw[kMaxMat], vexp_pw1[kMaxMat], vcoef_pow[kMaxMat], vQ[kMaxMat], vnR[kMaxMat];
    double pls0[kMaxMat], pls1[kMaxMat], c0[kMaxMat], c1[kMaxMat], f0[kMaxMat], f1[kMaxMat];
    double d0[kMaxMat], d1[kMaxMat];
    double hslope[kMaxMat];        // (c1 - c0) / (pls1 - pls0)
    // libm values for the friction/dilation angle of material 0 (used when the
    // element's averaged angle equals it exactly)
    double phi_c, sphi_c, tphi_c, anphi_c, sqanphi_c;
    double psi_c, spsi_c, anpsi_c;
    // the same for the fully weakened angles of material 0 (friction_angle1,
    // dilation_angle1), which every element past pls1 uses
    double phi_w, tphi_w, anphi_w, sqanphi_w;
    double psi_w, anpsi_w;
    double visc_min, visc_max, tension_max;
    // FP32 copies for the quick elastic bound (quick_elastic)
    float pls0f[kMaxMat], pls1f[kMaxMat], c0f[kMaxMat], c1f[kMaxMat], f0f[kMaxMat], f1f[kMaxMat];
    float phi_cf, anphi_cf, sqanphi_cf, tphi_cf, phi_wf, anphi_wf, sqanphi_wf, tphi_wf, tension_maxf;
    Mix    mix[kMaxMix];
};

__device__ __forceinline__ double smin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }
// The templated helpers below are instantiated with double for the FP64 form
// (identical operation order to the reference) and with float for the FP32
// form; literals are cast to R so that a float instantiation stays in FP32.
template <class R>
__device__ __forceinline__ R tr3(const R *s) { return s[0] + s[1] + s[2]; }

// utils.hpp:78-87
template <class R>
__device__ __forceinline__ R second_invariant2(const R *t)
{
    R a = (t[0] + t[1] + t[2]) / R(3);
    return (R(0.5) * ((t[0] - a) * (t[0] - a) + (t[1] - a) * (t[1] - a) + (t[2] - a) * (t[2] - a)) +
            t[3] * t[3] + t[4] * t[4] + t[5] * t[5]);
}

// ---- MatProps -------------------------------------------------------------

// Exact steps in the element's arithmetic type: for FP64 on the integer
// pipes (0 + x, 2 x, x / 4, x / 3 as the FP64 unit rounds them, sf::*), for
// FP32 the FP32 instructions themselves
__device__ __forceinline__ double padd0(double x) { return sf::add0(x); }
__device__ __forceinline__ float padd0(float x) { return 0.f + x; }
__device__ __forceinline__ double ptwice(double x) { return sf::twice(x); }
__device__ __forceinline__ float ptwice(float x) { return 2 * x; }
__device__ __forceinline__ double pquarter(double x) { return sf::quarter(x); }
__device__ __forceinline__ float pquarter(float x) { return x / 4; }
__device__ __forceinline__ double pdiv3(double x) { return sf::div3(x); }
__device__ __forceinline__ float pdiv3(float x) { return x / 3; }

// element mean temperature (matprops.cxx:613-618): ((((0 + a) + b) + c) + d) / 4
template <class R>
__device__ __forceinline__ R elem_mean4(R a, R b, R c, R d)
{
    R t = padd0(a);
    t += b;
    t += c;
    t += d;
    return pquarter(t);
}

// matprops.cxx:707-728
__device__ __forceinline__ double mat_rho(const MatTable &M, const Mix &x, double T)
{
    double TinCelsius = T - 273;
    if (x.single >= 0) {
        // (r * k) / k with k a power of two is r exactly
        int m = x.single;
        return M.rho0[m] * (1 - M.alpha[m] * TinCelsius);
    }
    double result = 0;
    int n = 0;
    for (int m = 0; m < M.nmat; m++) {
        result += M.rho0[m] * (1 - M.alpha[m] * TinCelsius) * x.count[m];
        n += x.count[m];
    }
    return result / n;
}

// matprops.cxx:607-643; edot_ii = second invariant of the (corrected) strain rate
__device__ __forceinline__ double mat_visc(const MatTable &M, const Mix &x, double T,
                                           const double *srate)
{
    double edot = sqrt(second_invariant2(srate));
    edot = smax(edot, 1e-30);
    double result = 0;
    int n = 0;
    for (int m = 0; m < M.nmat; m++) {
        if (x.single >= 0 && m != x.single) continue;   // zero-count terms add +0
        double visc0 = 0.25 * pow(edot, M.vexp_pw[m]) * M.vcoef_pow[m] *
                       exp(M.vQ[m] / (M.vnR[m] * T)) * 1e6;
        result += x.count[m] / visc0;
        n += x.count[m];
    }
    double v = n / result;
    return smin(smax(v, M.visc_min), M.visc_max);
}

// matprops.cxx:646-704
__device__ __forceinline__ void plastic_props(const MatTable &M, const Mix &x, double pls,
                                              double &amc, double &anphi, double &anpsi,
                                              double &hardn, double &ten_max)
{
    double cohesion, phi, psi;
    if (x.single >= 0) {
        // one material, power-of-two count: (v * k) / k == v
        int m = x.single;
        if (pls < M.pls0[m]) {
            cohesion = M.c0[m];
            phi = M.f0[m];
            psi = M.d0[m];
            hardn = 0;
        } else if (pls < M.pls1[m]) {
            double p = (pls - M.pls0[m]) / (M.pls1[m] - M.pls0[m]);
            cohesion = M.c0[m] + p * (M.c1[m] - M.c0[m]);
            phi = M.f0[m] + p * (M.f1[m] - M.f0[m]);
            psi = M.d0[m] + p * (M.d1[m] - M.d0[m]);
            hardn = M.hslope[m];
        } else {
            cohesion = M.c1[m];
            phi = M.f1[m];
            psi = M.d1[m];
            hardn = 0;
        }
    } else {
        double c = 0, f = 0, d = 0, h = 0;
        int n = 0;
        for (int m = 0; m < M.nmat; m++) {
            int k = x.count[m];
            if (k == 0) continue;
            n += k;
            if (pls < M.pls0[m]) {
                c += M.c0[m] * k;
                f += M.f0[m] * k;
                d += M.d0[m] * k;
                h += 0;
            } else if (pls < M.pls1[m]) {
                double p = (pls - M.pls0[m]) / (M.pls1[m] - M.pls0[m]);
                c += (M.c0[m] + p * (M.c1[m] - M.c0[m])) * k;
                f += (M.f0[m] + p * (M.f1[m] - M.f0[m])) * k;
                d += (M.d0[m] + p * (M.d1[m] - M.d0[m])) * k;
                h += M.hslope[m] * k;
            } else {
                c += M.c1[m] * k;
                f += M.f1[m] * k;
                d += M.d1[m] * k;
                h += 0;
            }
        }
        cohesion = c / n;
        phi = f / n;
        psi = d / n;
        hardn = h / n;
    }
    double sqanphi, tphi;
    if (phi == M.phi_c) {
        anphi = M.anphi_c;
        sqanphi = M.sqanphi_c;
        tphi = M.tphi_c;
    } else if (phi == M.phi_w) {
        anphi = M.anphi_w;
        sqanphi = M.sqanphi_w;
        tphi = M.tphi_w;
    } else {
        double sphi = sin(phi * kDeg2Rad);
        anphi = (1 + sphi) / (1 - sphi);
        sqanphi = sqrt(anphi);
        tphi = tan(phi * kDeg2Rad);
    }
    if (psi == M.psi_c) {
        anpsi = M.anpsi_c;
    } else if (psi == M.psi_w) {
        anpsi = M.anpsi_w;
    } else {
        double spsi = sin(psi * kDeg2Rad);
        anpsi = (1 + spsi) / (1 - spsi);
    }
    amc = 2 * cohesion * sqanphi;
    ten_max = (phi == 0) ? M.tension_max : smin(M.tension_max, cohesion / tphi);
}

// ---- 3x3 symmetric eigen-solver -------------------------------------------
// Restated from Kopp, arXiv physics/0610206 (the reference's 3x3-C library:
// dsyevc3.c:31-81, dsytrd3.c:28-105, dsyevq3.c:29-135, dsyevh3.c:31-135).
// A holds a00 a11 a22 a01 a02 a12.

__device__ __forceinline__ double sq(double x) { return x * x; }

// (the products on the integer pipes, sf::mul, rounded as the FP64 unit
// rounds them; the square roots, atan2 and sincos on the FP64 unit)
__device__ __forceinline__ void eig_cardano(const double *A, double w[3])
{
    using sf::mul;
    const double a00 = A[0], a11 = A[1], a22 = A[2], a01 = A[3], a02 = A[4], a12 = A[5];
    double de = mul(a01, a12);
    double dd = mul(a01, a01);
    double ee = mul(a12, a12);
    double ff = mul(a02, a02);
    double m = a00 + a11 + a22;
    double c1 = (mul(a00, a11) + mul(a00, a22) + mul(a11, a22)) - (dd + ee + ff);
    double c0 = mul(a22, dd) + mul(a00, ee) + mul(a11, ff) - mul(mul(a00, a11), a22) - mul(mul(2.0, a02), de);
    double p = mul(m, m) - mul(3.0, c1);
    double q = mul(m, p - mul(3.0 / 2.0, c1)) - mul(27.0 / 2.0, c0);
    double sqrt_p = sqrt(fabs(p));
    double phi = mul(27.0, mul(mul(0.25, mul(c1, c1)), p - c1) + mul(c0, q + mul(27.0 / 4.0, c0)));
    phi = mul(1.0 / 3.0, atan2(sqrt(fabs(phi)), q));
    double sp, cp;
    sincos(phi, &sp, &cp);
    double c = mul(sqrt_p, cp);
    double s = mul(mul(1.0 / 1.73205080756887729352744634151, sqrt_p), sp);
    w[1] = mul(1.0 / 3.0, m - c);
    w[2] = w[1] + s;
    w[0] = w[1] + c;
    w[1] -= s;
}

static __device__ __noinline__ int eig_ql(const double *A, double Q[3][3], double w[3])
{
    const double a00 = A[0], a11 = A[1], a22 = A[2], a01 = A[3], a02 = A[4], a12 = A[5];
    double e[3];
    // Householder reduction (dsytrd3.c:28-105)
    {
        double u1, u2, q1, q2, omega, f, K, h, g;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) Q[i][j] = (i == j) ? 1.0 : 0.0;
        h = sq(a01) + sq(a02);
        if (a01 > 0)
            g = -sqrt(h);
        else
            g = sqrt(h);
        e[0] = g;
        f = g * a01;
        u1 = a01 - g;
        u2 = a02;
        omega = h - f;
        if (omega > 0.0) {
            omega = 1.0 / omega;
            K = 0.0;
            f = a11 * u1 + a12 * u2;      // A[1][1] u1 + A[1][2] u2
            q1 = omega * f;
            K += u1 * f;
            f = a12 * u1 + a22 * u2;      // A[1][2] u1 + A[2][2] u2
            q2 = omega * f;
            K += u2 * f;
            K *= 0.5 * sq(omega);
            q1 = q1 - K * u1;
            q2 = q2 - K * u2;
            w[0] = a00;
            w[1] = a11 - 2.0 * q1 * u1;
            w[2] = a22 - 2.0 * q2 * u2;
            f = omega * u1;
            Q[1][1] = Q[1][1] - f * u1;
            Q[2][1] = Q[2][1] - f * u2;
            f = omega * u2;
            Q[1][2] = Q[1][2] - f * u1;
            Q[2][2] = Q[2][2] - f * u2;
            e[1] = a12 - q1 * u2 - u1 * q2;
        } else {
            w[0] = a00;
            w[1] = a11;
            w[2] = a22;
            e[1] = a12;
        }
    }
    // implicit-shift QL (dsyevq3.c:58-132)
    double g, r, p, f, b, s, c, t;
    for (int l = 0; l < 2; l++) {
        int nIter = 0;
        int m;
        while (1) {
            for (m = l; m <= 1; m++) {
                g = fabs(w[m]) + fabs(w[m + 1]);
                if (fabs(e[m]) + g == g) break;
            }
            if (m == l) break;
            if (nIter++ >= 30) return -1;
            g = (w[l + 1] - w[l]) / (e[l] + e[l]);
            r = sqrt(sq(g) + 1.0);
            if (g > 0)
                g = w[m] - w[l] + e[l] / (g + r);
            else
                g = w[m] - w[l] + e[l] / (g - r);
            s = c = 1.0;
            p = 0.0;
            for (int i = m - 1; i >= l; i--) {
                f = s * e[i];
                b = c * e[i];
                if (fabs(f) > fabs(g)) {
                    c = g / f;
                    r = sqrt(sq(c) + 1.0);
                    e[i + 1] = f * r;
                    c *= (s = 1.0 / r);
                } else {
                    s = f / g;
                    r = sqrt(sq(s) + 1.0);
                    e[i + 1] = g * r;
                    s *= (c = 1.0 / r);
                }
                g = w[i + 1] - p;
                r = (w[i] - g) * s + 2.0 * c * b;
                p = s * r;
                w[i + 1] = g + p;
                g = c * r - b;
                for (int k = 0; k < 3; k++) {
                    t = Q[k][i + 1];
                    Q[k][i + 1] = s * Q[k][i] + c * t;
                    Q[k][i] = c * Q[k][i] - s * t;
                }
            }
            w[l] -= p;
            e[l] = g;
            e[m] = 0.0;
        }
    }
    return 0;
}

// returns 0 (Cardano + cross products), 1 (QL fallback), -1 (QL did not converge)
__device__ __forceinline__ int eig_hybrid(const double *A, double Q[3][3], double w[3])
{
    const double a00 = A[0], a11 = A[1], a01 = A[3], a02 = A[4], a12 = A[5];
    double norm, error, t, u;
    using sf::mul;
    eig_cardano(A, w);
    t = fabs(w[0]);
    if ((u = fabs(w[1])) > t) t = u;
    if ((u = fabs(w[2])) > t) t = u;
    if (t < 1.0)
        u = t;
    else
        u = mul(t, t);
    error = mul(mul(256.0, kEps), mul(u, u));
    double q01 = mul(a01, a12) - mul(a02, a11);
    double q11 = mul(a02, a01) - mul(a12, a00);
    double q21 = mul(a01, a01);
    Q[0][0] = q01 + mul(a02, w[0]);
    Q[1][0] = q11 + mul(a12, w[0]);
    Q[2][0] = mul(a00 - w[0], a11 - w[0]) - q21;
    norm = mul(Q[0][0], Q[0][0]) + mul(Q[1][0], Q[1][0]) + mul(Q[2][0], Q[2][0]);
    if (norm <= error) return eig_ql(A, Q, w) == 0 ? 1 : -1;
    norm = sqrt(1.0 / norm);
    for (int j = 0; j < 3; j++) Q[j][0] = mul(Q[j][0], norm);
    Q[0][1] = q01 + mul(a02, w[1]);
    Q[1][1] = q11 + mul(a12, w[1]);
    Q[2][1] = mul(a00 - w[1], a11 - w[1]) - q21;
    norm = mul(Q[0][1], Q[0][1]) + mul(Q[1][1], Q[1][1]) + mul(Q[2][1], Q[2][1]);
    if (norm <= error) return eig_ql(A, Q, w) == 0 ? 1 : -1;
    norm = sqrt(1.0 / norm);
    for (int j = 0; j < 3; j++) Q[j][1] = mul(Q[j][1], norm);
    Q[0][2] = mul(Q[1][0], Q[2][1]) - mul(Q[2][0], Q[1][1]);
    Q[1][2] = mul(Q[2][0], Q[0][1]) - mul(Q[0][0], Q[2][1]);
    Q[2][2] = mul(Q[0][0], Q[1][1]) - mul(Q[1][0], Q[0][1]);
    return 0;
}

// rheology.cxx:16-71
__device__ __forceinline__ int principal3(const double *s, double p[3], double v[3][3])
{
    int rc = eig_hybrid(s, v, p);
#define DES_SWAP_COL(i, j)                                   \
    {                                                        \
        double tmp = p[i];                                   \
        p[i] = p[j];                                         \
        p[j] = tmp;                                          \
        for (int r = 0; r < 3; ++r) {                        \
            double bb = v[r][i];                             \
            v[r][i] = v[r][j];                               \
            v[r][j] = bb;                                    \
        }                                                    \
    }
    if (p[0] > p[1]) DES_SWAP_COL(0, 1)
    if (p[1] > p[2]) DES_SWAP_COL(1, 2)
    if (p[0] > p[1]) DES_SWAP_COL(0, 1)
#undef DES_SWAP_COL
    return rc;
}

// ---- rheology (rheology.cxx:108-302, 3D) ----------------------------------

// a product as the FP64 unit rounds it, on the integer pipes for FP64
// (sf::mul); FP32 products stay on the FP32 pipe
__device__ __forceinline__ double pmul(double a, double b) { return sf::mul(a, b); }
__device__ __forceinline__ float pmul(float a, float b) { return a * b; }

template <class R>
__device__ __forceinline__ void elastic(R bulkm, R shearm, const R *de, R *s)
{
    R lambda = bulkm - R(2.) / R(3) * shearm;
    R dev = tr3(de);
    const R g2 = ptwice(shearm);
    for (int i = 0; i < 3; ++i) s[i] += pmul(g2, de[i]) + pmul(lambda, dev);
    for (int i = 3; i < 6; ++i) s[i] += pmul(g2, de[i]);
}

template <class R>
__device__ __forceinline__ void maxwell(R bulkm, R shearm, R viscosity, R dt, R dv, const R *de, R *s)
{
    R tmp = R(0.5) * dt * shearm / viscosity;
    R f1 = 1 - tmp;
    R f2 = 1 / (1 + tmp);
    R dev = pdiv3(tr3(de));
    R s0 = pdiv3(tr3(s));
    const R g2 = ptwice(shearm);
    for (int i = 0; i < 3; ++i)
        s[i] = ((s[i] - s0) * f1 + g2 * (de[i] - dev)) * f2 + s0 + bulkm * dv;
    for (int i = 3; i < 6; ++i) s[i] = (s[i] * f1 + g2 * de[i]) * f2;
}

template <class R>
__device__ __forceinline__ void viscous(R bulkm, R viscosity, R total_dv, const R *edot, R *s)
{
    R dev = pdiv3(tr3(edot));
    const R v2 = ptwice(viscosity);
    for (int i = 0; i < 3; ++i) s[i] = v2 * (edot[i] - dev) + bulkm * total_dv;
    for (int i = 3; i < 6; ++i) s[i] = v2 * edot[i];
}

// Conservative test that the reference's composite yield check
// (rheology.cxx:190-196) reports "no failure" for the trial stress s.  The
// eigenvalues of s lie in [m - R, m + R] with m = tr/3 and
// R = sqrt(2/3 * |dev s|^2).  The margin covers the error of the reference's
// Cardano eigenvalues: near an isotropic stress p = tr^2 - 3 c1 cancels, so
// sqrt(p) carries an absolute error up to about sqrt(5 eps) |tr|, i.e. about
// 1e-7 |m| in each eigenvalue; the margin is 1e-6 (|m| + R) per unit of
// (1 + anphi).  When this returns true the reference returns the trial stress
// unchanged, which needs no eigen-decomposition.
__device__ __forceinline__ bool surely_elastic(const double *s, double anphi, double amc,
                                               double ten_max)
{
    double m = (s[0] + s[1] + s[2]) * (1.0 / 3.0);
    double a = s[0] - m, b = s[1] - m, c = s[2] - m;
    double dev2 = a * a + b * b + c * c + 2.0 * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]);
    double R = sqrt(dev2 * (2.0 / 3.0)) * (1.0 + 1e-12);
    double scale = fabs(m) + R;
    double margin = 1e-6 * scale * (1.0 + anphi) + 1e-300;
    double fs_lo = (m - R) - anphi * (m + R) + amc;
    double ft_hi = (m + R) - ten_max;
    return fs_lo > margin && ft_hi < -margin;
}

// The same bound in FP32 from FP32 plastic properties, before any FP64 work on
// the element: where it holds, the element's stress is the trial and its
// plastic properties are never needed.  The margin (1e-4 of the stress scale
// times 1 + anphi) covers the FP32 rounding of the stress, of the properties
// and of the bound many times over.
__device__ __forceinline__ bool quick_elastic(const MatTable &M, const Mix &x, double pls, const double *s)
{
    const float pl = (float)pls;
    float c = 0.f, f = 0.f;
    int n = 0;
    for (int m = 0; m < M.nmat; ++m) {
        const int k = x.count[m];
        if (k == 0) continue;
        n += k;
        float cm, fm;
        if (pl < M.pls0f[m]) {
            cm = M.c0f[m];
            fm = M.f0f[m];
        } else if (pl < M.pls1f[m]) {
            const float q = (pl - M.pls0f[m]) / (M.pls1f[m] - M.pls0f[m]);
            cm = M.c0f[m] + q * (M.c1f[m] - M.c0f[m]);
            fm = M.f0f[m] + q * (M.f1f[m] - M.f0f[m]);
        } else {
            cm = M.c1f[m];
            fm = M.f1f[m];
        }
        c += cm * (float)k;
        f += fm * (float)k;
    }
    const float cohesion = c / (float)n, phi = f / (float)n;
    float anphi, sq, tph;
    if (phi == M.phi_cf) {
        anphi = M.anphi_cf;
        sq = M.sqanphi_cf;
        tph = M.tphi_cf;
    } else if (phi == M.phi_wf) {
        anphi = M.anphi_wf;
        sq = M.sqanphi_wf;
        tph = M.tphi_wf;
    } else {
        const float sp = sinf(phi * (float)kDeg2Rad);
        anphi = (1.f + sp) / (1.f - sp);
        sq = sqrtf(anphi);
        tph = tanf(phi * (float)kDeg2Rad);
    }
    const float amc = 2.f * cohesion * sq;
    const float ten_max = (phi == 0.f) ? M.tension_maxf : fminf(M.tension_maxf, cohesion / tph);
    float sf[6];
    for (int i = 0; i < 6; ++i) sf[i] = (float)s[i];
    const float mp = (sf[0] + sf[1] + sf[2]) * (1.f / 3.f);
    const float a = sf[0] - mp, b = sf[1] - mp, cc = sf[2] - mp;
    const float dev2 = a * a + b * b + cc * cc + 2.f * (sf[3] * sf[3] + sf[4] * sf[4] + sf[5] * sf[5]);
    const float R = sqrtf(dev2 * (2.f / 3.f)) * (1.f + 1e-5f);
    const float margin = 1e-4f * (fabsf(mp) + R) * (1.f + anphi) + 1e-30f;
    return ((mp - R) - anphi * (mp + R) + amc) > margin && ((mp + R) - ten_max) < -margin;
}

// The return map of elasto_plastic (rheology.cxx:154-302) from the trial s;
// returns 1 when the principal stresses were computed (+2 when QL was used,
// +4 when QL failed to converge, +16 for a shear return, +32 for a tensile one)
__device__ __forceinline__ int plastic_return(double bulkm, double shearm, double amc, double anphi,
                                              double anpsi, double hardn, double ten_max, double &depls,
                                              double *s)
{
    depls = 0;
    if (surely_elastic(s, anphi, amc, ten_max)) return 0;
    double p[3];
    double v[3][3];
    int rc = principal3(s, p, v);
    int flags = 1 | (rc == 1 ? 2 : 0) | (rc < 0 ? 6 : 0);
    double fs = p[0] - p[2] * anphi + amc;
    double ft = p[2] - ten_max;
    if (fs > 0 && ft < 0) return flags;
    double pa = sqrt(1 + anphi * anphi) + anphi;
    double ps = ten_max * anphi - amc;
    double h = p[2] - ten_max + pa * (p[0] - ps);
    double a1 = bulkm + 4. / 3 * shearm;
    double a2 = bulkm - 2. / 3 * shearm;
    double alam;
    if (h < 0) {
        flags |= 16;
        alam = fs / (a1 - a2 * anpsi + a1 * anphi * anpsi - a2 * anphi + 2 * sqrt(anphi) * hardn);
        p[0] -= alam * (a1 - a2 * anpsi);
        p[1] -= alam * (a2 - a2 * anpsi);
        p[2] -= alam * (a2 - a1 * anpsi);
        depls = fabs(alam) * sqrt((7 + 4 * anpsi + 7 * anpsi * anpsi) / 18);
    } else {
        flags |= 32;
        alam = ft / a1;
        p[0] -= alam * a2;
        p[1] -= alam * a2;
        p[2] -= alam * a1;
        depls = fabs(alam) * sqrt(7. / 18);
    }
    // (the reconstruction's products on the integer pipes, sf::mul)
    using sf::mul;
    double ss00 = 0, ss11 = 0, ss22 = 0, ss01 = 0, ss02 = 0, ss12 = 0;
    for (int k = 0; k < 3; k++) {
        ss00 += mul(mul(v[0][k], v[0][k]), p[k]);
        ss01 += mul(mul(v[0][k], v[1][k]), p[k]);
        ss02 += mul(mul(v[0][k], v[2][k]), p[k]);
        ss11 += mul(mul(v[1][k], v[1][k]), p[k]);
        ss12 += mul(mul(v[1][k], v[2][k]), p[k]);
        ss22 += mul(mul(v[2][k], v[2][k]), p[k]);
    }
    s[0] = ss00;
    s[1] = ss11;
    s[2] = ss22;
    s[3] = ss01;
    s[4] = ss02;
    s[5] = ss12;
    return flags;
}

// elasto_plastic (rheology.cxx:154-302): elastic trial, then the return map
__device__ __forceinline__ int elasto_plastic(double bulkm, double shearm, double amc, double anphi,
                                              double anpsi, double hardn, double ten_max,
                                              const double *de, double &depls, double *s)
{
    elastic(bulkm, shearm, de, s);
    return plastic_return(bulkm, shearm, amc, anphi, anpsi, hardn, ten_max, depls, s);
}

// ---- geometry -------------------------------------------------------------

// geometry.cxx:29-49
__device__ __forceinline__ double tet_volume(const double *d0, const double *d1, const double *d2,
                                             const double *d3)
{
    double x01 = d0[0] - d1[0];
    double x12 = d1[0] - d2[0];
    double x23 = d2[0] - d3[0];
    double y01 = d0[1] - d1[1];
    double y12 = d1[1] - d2[1];
    double y23 = d2[1] - d3[1];
    double z01 = d0[2] - d1[2];
    double z12 = d1[2] - d2[2];
    double z23 = d2[2] - d3[2];
    // (the division by 6 on the integer pipes, sf::div6)
    return sf::div6(x01 * (y23 * z12 - y12 * z23) + x12 * (y01 * z23 - y23 * z01) +
                    x23 * (y12 * z01 - y01 * z12));
}

// geometry.cxx:53-83 (3D): the squared norm of the facet's cross product,
// whose sqrt / 2 is the facet's area
__device__ __forceinline__ double tri_area2(const double *a, const double *b, const double *c)
{
    double ab0 = b[0] - a[0], ab1 = b[1] - a[1];
    double ac0 = c[0] - a[0], ac1 = c[1] - a[1];
    double ab2 = b[2] - a[2], ac2 = c[2] - a[2];
    double d0 = ab1 * ac2 - ab2 * ac1;
    double d1 = ab2 * ac0 - ab0 * ac2;
    double d2 = ab0 * ac1 - ab1 * ac0;
    return d0 * d0 + d1 * d1 + d2 * d2;
}

// geometry.cxx:53-83 (3D)
__device__ __forceinline__ double tri_area(const double *a, const double *b, const double *c)
{
    return sqrt(tri_area2(a, b, c)) / 2;
}

// geometry.cxx:472-509 (3D): 216 sqrt(3) V^2 / (sum of the face areas)^3, 1
// for the regular tetrahedron; nf = 216 sqrt(3) from the host's libm
__device__ __forceinline__ double elem_quality(const double X[4][3], double vol, double nf)
{
    double area_sum = (tri_area(X[0], X[1], X[2]) + tri_area(X[0], X[1], X[3]) + tri_area(X[2], X[3], X[0]) +
                       tri_area(X[2], X[3], X[1]));
    return nf * vol * vol / (area_sum * area_sum * area_sum);
}

// geometry.cxx:410-452; X[v][d] are the four vertex coordinates.  r1 and
// r3 receive the bracketed cross products of nodes 1 and 3 (before the
// scaling by iv); they are, bit for bit, the cross products tri_area forms
// for the facets (2, 3, 0) and (0, 1, 2): each edge difference here is the
// other's or its exact negative, and the products commute.
__device__ __forceinline__ void shape_fn(const double X[4][3], double vol, double dx[4], double dy[4],
                                         double dz[4], double r1[3], double r3[3])
{
    const double *d0 = X[0], *d1 = X[1], *d2 = X[2], *d3 = X[3];
    double iv = 1 / (6 * vol);
    double x01 = d0[0] - d1[0], x02 = d0[0] - d2[0], x03 = d0[0] - d3[0];
    double x12 = d1[0] - d2[0], x13 = d1[0] - d3[0], x23 = d2[0] - d3[0];
    double y01 = d0[1] - d1[1], y02 = d0[1] - d2[1], y03 = d0[1] - d3[1];
    double y12 = d1[1] - d2[1], y13 = d1[1] - d3[1], y23 = d2[1] - d3[1];
    double z01 = d0[2] - d1[2], z02 = d0[2] - d2[2], z03 = d0[2] - d3[2];
    double z12 = d1[2] - d2[2], z13 = d1[2] - d3[2], z23 = d2[2] - d3[2];
    r1[0] = y02 * z23 - y23 * z02;
    r1[1] = z02 * x23 - z23 * x02;
    r1[2] = x02 * y23 - x23 * y02;
    r3[0] = y01 * z02 - y02 * z01;
    r3[1] = z01 * x02 - z02 * x01;
    r3[2] = x01 * y02 - x02 * y01;
    dx[0] = iv * (y13 * z12 - y12 * z13);
    dx[1] = iv * r1[0];
    dx[2] = iv * (y13 * z03 - y03 * z13);
    dx[3] = iv * r3[0];
    dy[0] = iv * (z13 * x12 - z12 * x13);
    dy[1] = iv * r1[1];
    dy[2] = iv * (z13 * x03 - z03 * x13);
    dy[3] = iv * r3[1];
    dz[0] = iv * (x13 * y12 - x12 * y13);
    dz[1] = iv * r1[2];
    dz[2] = iv * (x13 * y03 - x03 * y13);
    dz[3] = iv * r3[2];
}

__device__ __forceinline__ void shape_fn(const double X[4][3], double vol, double dx[4], double dy[4],
                                         double dz[4])
{
    double r1[3], r3[3];
    shape_fn(X, vol, dx, dy, dz, r1, r3);
}

// fields.cxx:193-241: D = sym(grad v) from the four nodal velocities V[i][d]
template <class R>
__device__ __forceinline__ void strain_rate(const R V[4][3], const R *dx, const R *dy, const R *dz, R *s)
{
    s[0] = 0;
    for (int i = 0; i < 4; ++i) s[0] += V[i][0] * dx[i];
    s[1] = 0;
    for (int i = 0; i < 4; ++i) s[1] += V[i][1] * dy[i];
    s[2] = 0;
    for (int i = 0; i < 4; ++i) s[2] += V[i][2] * dz[i];
    s[3] = 0;
    for (int i = 0; i < 4; ++i) s[3] += R(0.5) * (V[i][0] * dy[i] + V[i][1] * dx[i]);
    s[4] = 0;
    for (int i = 0; i < 4; ++i) s[4] += R(0.5) * (V[i][0] * dz[i] + V[i][2] * dx[i]);
    s[5] = 0;
    for (int i = 0; i < 4; ++i) s[5] += R(0.5) * (V[i][1] * dz[i] + V[i][2] * dy[i]);
}

// fields.cxx:483-504: spin components
template <class R>
__device__ __forceinline__ void spin(const R V[4][3], const R *dx, const R *dy, const R *dz, R &w3,
                                     R &w4, R &w5)
{
    w3 = 0;
    for (int i = 0; i < 4; ++i) w3 += R(0.5) * (V[i][0] * dy[i] - V[i][1] * dx[i]);
    w4 = 0;
    for (int i = 0; i < 4; ++i) w4 += R(0.5) * (V[i][0] * dz[i] - V[i][2] * dx[i]);
    w5 = 0;
    for (int i = 0; i < 4; ++i) w5 += R(0.5) * (V[i][1] * dz[i] - V[i][2] * dy[i]);
}

// FP64: the spin (fields.cxx:483-504) and the strain rate (fields.cxx:193-241)
// of the same velocities and gradients share their products V_i,a dN_i/db,
// formed once here.  Both sum 0.5 (bracket) over the four nodes; scaling by
// 0.5 is exact and commutes with rounding, so 0.5 times the sum of the
// brackets equals the reference's sum bit for bit (for terms above the
// subnormal range).
//
// Each sum starts from zero in the reference; its first addition, 0 + x, is
// x except for -0 and is formed on the integer pipes (sf::add0), as are the
// exact scalings by 0.5 (sf::half).
__device__ __forceinline__ void spin_and_rate(const double V[4][3], const double *dx, const double *dy,
                                              const double *dz, double &w3, double &w4, double &w5,
                                              double D[6])
{
    D[0] = sf::add0(V[0][0] * dx[0]);
    for (int i = 1; i < 4; ++i) D[0] += V[i][0] * dx[i];
    D[1] = sf::add0(V[0][1] * dy[0]);
    for (int i = 1; i < 4; ++i) D[1] += V[i][1] * dy[i];
    D[2] = sf::add0(V[0][2] * dz[0]);
    for (int i = 1; i < 4; ++i) D[2] += V[i][2] * dz[i];
    double t3, t4, t5, u3, u4, u5;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const double xy = V[i][0] * dy[i], yx = V[i][1] * dx[i];
        const double xz = V[i][0] * dz[i], zx = V[i][2] * dx[i];
        const double yz = V[i][1] * dz[i], zy = V[i][2] * dy[i];
        if (i == 0) {
            t3 = sf::add0(xy + yx);
            u3 = sf::add0(xy - yx);
            t4 = sf::add0(xz + zx);
            u4 = sf::add0(xz - zx);
            t5 = sf::add0(yz + zy);
            u5 = sf::add0(yz - zy);
        } else {
            t3 += xy + yx;
            u3 += xy - yx;
            t4 += xz + zx;
            u4 += xz - zx;
            t5 += yz + zy;
            u5 += yz - zy;
        }
    }
    D[3] = sf::half(t3);
    D[4] = sf::half(t4);
    D[5] = sf::half(t5);
    w3 = sf::half(u3);
    w4 = sf::half(u4);
    w5 = sf::half(u5);
}

// fields.cxx:419-433 in FP64: the reference's 2 s_ab w products appear twice
// each; 2 (s_ab w) is formed once per pair and the factor 2 applied to the
// sum (exact, as above; an exponent step on the integer pipes, sf::twice)
__device__ __forceinline__ void jaumann64(double *s, double dt, double w3, double w4, double w5)
{
    // (products on the integer pipes, sf::mul)
    const double p3 = sf::mul(s[3], w3), p4 = sf::mul(s[4], w4), p5 = sf::mul(s[5], w5);
    double inc[6];
    inc[0] = sf::twice(-p3 - p4);
    inc[1] = sf::twice(p3 - p5);
    inc[2] = sf::twice(p4 + p5);
    inc[3] = sf::mul(s[0], w3) - sf::mul(s[1], w3) - sf::mul(s[4], w5) - sf::mul(s[5], w4);
    inc[4] = sf::mul(s[0], w4) - sf::mul(s[2], w4) + sf::mul(s[3], w5) - sf::mul(s[5], w3);
    inc[5] = sf::mul(s[1], w5) - sf::mul(s[2], w5) + sf::mul(s[3], w4) + sf::mul(s[4], w3);
    for (int i = 0; i < 6; ++i) s[i] += sf::mul(dt, inc[i]);
}

// fields.cxx:419-433
template <class R>
__device__ __forceinline__ void jaumann(R *s, R dt, R w3, R w4, R w5)
{
    R inc[6];
    inc[0] = R(-2.0) * s[3] * w3 - R(2.0) * s[4] * w4;
    inc[1] = R(2.0) * s[3] * w3 - R(2.0) * s[5] * w5;
    inc[2] = R(2.0) * s[4] * w4 + R(2.0) * s[5] * w5;
    inc[3] = s[0] * w3 - s[1] * w3 - s[4] * w5 - s[5] * w4;
    inc[4] = s[0] * w4 - s[2] * w4 + s[3] * w5 - s[5] * w3;
    inc[5] = s[1] * w5 - s[2] * w5 + s[3] * w4 + s[4] * w3;
    for (int i = 0; i < 6; ++i) s[i] += dt * inc[i];
}

// fields.cxx:130-143: element conduction vector tr[i] = kv sum_j (gradNi.gradNj) T_j.
// gradNi.gradNj and gradNj.gradNi round identically (the products commute and
// are summed in the same order), so the 10 distinct dot products are formed once.
__device__ __forceinline__ void conduction(const double *dx, const double *dy, const double *dz,
                                           const double Tn[4], double kv, double tr[4])
{
    // (products on the integer pipes, sf::mul)
    double D[4][4];
    for (int i = 0; i < 4; ++i)
        for (int j = i; j < 4; ++j) {
            D[i][j] = sf::mul(dx[i], dx[j]) + sf::mul(dy[i], dy[j]) + sf::mul(dz[i], dz[j]);
            D[j][i] = D[i][j];
        }
    // (the loops stay rolled: in E-A the shorter code runs faster than the
    // matrix held in registers, which unrolling them would give)
    for (int i = 0; i < 4; ++i) {
        double diffusion = sf::add0(sf::mul(D[i][0], Tn[0]));    // 0 + x (sf::add0)
        for (int j = 1; j < 4; ++j) diffusion += sf::mul(D[i][j], Tn[j]);
        tr[i] = sf::mul(diffusion, kv);
    }
}

// geometry.cxx:280-293 for one element: 3 V / (largest facet area).  The
// largest area is taken among the squared norms and rooted once: a correctly
// rounded sqrt and the exact halving keep the order (equal roots of unequal
// squares are equal values) and NaN stays NaN, so smax selects the same
// value as among the four areas.
__device__ __forceinline__ double min_height(const double X[4][3], double vol)
{
    double m2 = smax(smax(tri_area2(X[0], X[1], X[2]), tri_area2(X[0], X[1], X[3])),
                     smax(tri_area2(X[2], X[3], X[0]), tri_area2(X[2], X[3], X[1])));
    double maxa = sqrt(m2) / 2;
    return 3 * vol / maxa;
}

// the same with the cross products of the facets (0, 1, 2) and (2, 3, 0)
// taken from shape_fn (r3 and r1).  Out of line: E-A calls it every tenth
// step, and kept apart its registers leave the pass's own allocation (E-A
// 5.08 -> 5.01 ms per step on config 2).
static __device__ __noinline__ double min_height(const double X[4][3], double vol, const double r1[3],
                                                 const double r3[3])
{
    double m2 = smax(smax(r3[0] * r3[0] + r3[1] * r3[1] + r3[2] * r3[2], tri_area2(X[0], X[1], X[3])),
                     smax(r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2], tri_area2(X[2], X[3], X[1])));
    double maxa = sqrt(m2) / 2;
    return 3 * vol / maxa;
}

// !(x > 0) from the bits (integer pipes): zero, negative or NaN
__device__ __forceinline__ bool not_positive(double x)
{
    const long long b = __double_as_longlong(x);
    return b <= 0 || b > 0x7ff0000000000000ll;
}

// true for NaN or +-Inf, from the exponent bits (integer pipes)
__device__ __forceinline__ bool not_finite(double x)
{
    return ((unsigned long long)__double_as_longlong(x) & 0x7ff0000000000000ull) == 0x7ff0000000000000ull;
}

// orderable 64-bit image of a double (total order for non-NaN values)
__device__ __forceinline__ unsigned long long order_bits(double x)
{
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ULL);
}
__device__ __forceinline__ double from_order_bits(unsigned long long b)
{
    unsigned long long r = (b >> 63) ? (b & 0x7fffffffffffffffULL) : ~b;
    return __longlong_as_double((long long)r);
}

}  // namespace des
