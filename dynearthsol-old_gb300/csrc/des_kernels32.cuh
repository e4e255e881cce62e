// Kernels of the FP32 mixed-precision step.
//
// FP64 is kept where stability needs it: coordinates and the update
// x += v dt, element volumes and the evaluation of the shape derivatives from
// the coordinates, the plastic-strain and temperature accumulators, and the
// stable-dt reduction.  Everything else -- stress, strain, strain rate,
// velocity, forces, nodal masses, the element force / conduction / dvoldt
// contributions -- is stored and computed in FP32.  Elements whose trial
// stress the FP32 yield bound cannot prove elastic take the exact FP64 return
// map (the same device code as the FP64 form), so plastic decisions never
// rest on FP32 eigenvalues.  The six passes and their order are those of the
// FP64 form (des_kernels.cuh).
//
// Stress split.  Each element's stress is held as an FP64 isotropic reference
// s0 (its mean stress when the state was set, the lithostatic pressure after
// init) plus an FP32 deviation sigma'.  Nodal forces are the residual of
// element contributions sigma.grad(N).V of about 1e15 N that cancel to 1e-4 of
// that; in FP32 the rounding of a 1e8 Pa stress alone exceeds the residual.
// With the split, the large s0 and rho0 g parts of every element force vector
// are formed in FP64 from the FP64 geometry (f0, one pass later gathered in
// FP64) and only sigma' and the thermal density change go through FP32.  Every
// constitutive update used here is equivariant under an isotropic shift
// (elastic, Maxwell, Jaumann, NMD, the second invariant), so it acts on
// sigma' directly; the yield test and the FP64 return map add s0 back.
#pragma once

#include "des_kernels.cuh"

namespace des {

struct MixF {
    float bulkm, shearm, cp, k, rho_qs;
    float rho_alpha;        // sum_m k_m rho0_m alpha_m / n: thermal part of the density
    double rho_ref;         // sum_m k_m rho0_m / n: density at 273 K
    double rho_g4;          // rho_ref g / 4: an element's buoyancy per node and unit volume
    int single;
    int count[kMaxMat];
    int n;
};

struct ConstsF {
    int nmat, nmix;
    MixF mix[kMaxMix];
    float rho0[kMaxMat], alpha[kMaxMat];
    float vexp_pw[kMaxMat], vlog_coef[kMaxMat], vQ[kMaxMat], vnR[kMaxMat];
    float pls0[kMaxMat], pls1[kMaxMat], c0[kMaxMat], c1[kMaxMat], f0[kMaxMat], f1[kMaxMat];
    float d0[kMaxMat], d1[kMaxMat], hslope[kMaxMat];
    float phi_c, anphi_c, sqanphi_c, tphi_c, psi_c, anpsi_c;
    float visc_min, visc_max, tension_max;
    float gravity, surface_temperature, therm_diff_max;
    int rheol, thermal, is_qs;
};

struct DevF {
    int nnode, nelem;
    const int4 *conn;
    const int *sup_off;
    const unsigned *sup_ent;
    const unsigned *bcflag;
    const unsigned char *mix;
    double *x, *y, *z, *x0, *y0, *z0;   // FP64
    double *T, *vol, *vol_old, *pls;    // FP64
    float *vx, *vy, *vz, *fx, *fy, *fz;
    float *mass, *tmass, *vol_n, *ntmp;
    float *dpls, *edvoldt, *dp, *tmp_sg;
    float *stress, *strain, *srate, *srate_next;   // [6][E]
    float *shp, *tmp;                               // [12][E]
    float *c_vol, *c_mass, *c_tmass, *c_trdv;
    double *s0;                                     // [E] isotropic reference stress
    double *f0;                                     // [12][E] FP64 part of the force vectors
    const Consts *K;
    const ConstsF *F;
    Clock *clk;
    BdryFacets bf;
    int *pend, *exact;                              // [E] element lists of the stress pass
};

__device__ __forceinline__ void f_load_vel4(const DevF &d, int4 c, float V[4][3])
{
    const int n[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        V[i][0] = __ldg(d.vx + n[i]);
        V[i][1] = __ldg(d.vy + n[i]);
        V[i][2] = __ldg(d.vz + n[i]);
    }
}
__device__ __forceinline__ void f_load_xyz4(const DevF &d, int4 c, double X[4][3])
{
    const int n[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        X[i][0] = __ldg(d.x + n[i]);
        X[i][1] = __ldg(d.y + n[i]);
        X[i][2] = __ldg(d.z + n[i]);
    }
}
__device__ __forceinline__ void f_load_shp(const DevF &d, int e, float dx[4], float dy[4], float dz[4])
{
    const size_t E = d.nelem;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        dx[i] = d.shp[(0 + i) * E + e];
        dy[i] = d.shp[(4 + i) * E + e];
        dz[i] = d.shp[(8 + i) * E + e];
    }
}
__device__ __forceinline__ void f_load6(const float *a, size_t E, int e, float s[6])
{
#pragma unroll
    for (int i = 0; i < 6; ++i) s[i] = a[i * E + e];
}
__device__ __forceinline__ void f_store6(float *a, size_t E, int e, const float s[6])
{
#pragma unroll
    for (int i = 0; i < 6; ++i) a[i * E + e] = s[i];
}
// element mean temperature in FP32 (from the FP64 accumulator)
__device__ __forceinline__ float f_elem_T(const DevF &d, int4 c)
{
    return elem_mean4(sf::to_float(__ldg(d.T + c.x)), sf::to_float(__ldg(d.T + c.y)),
                      sf::to_float(__ldg(d.T + c.z)), sf::to_float(__ldg(d.T + c.w)));
}

// matprops.cxx:707-728 in FP32
__device__ __forceinline__ float f_rho(const ConstsF &F, const MixF &x, float T)
{
    float Tc = T - 273.f;
    if (x.single >= 0) return F.rho0[x.single] * (1.f - F.alpha[x.single] * Tc);
    float r = 0.f;
    int n = 0;
    for (int m = 0; m < F.nmat; ++m) {
        r += F.rho0[m] * (1.f - F.alpha[m] * Tc) * (float)x.count[m];
        n += x.count[m];
    }
    return r / (float)n;
}

// matprops.cxx:607-643 in FP32, evaluated in the log domain so that the
// power law cannot overflow FP32 before the [visc_min, visc_max] clip
__device__ __forceinline__ float f_visc(const ConstsF &F, const MixF &x, float T, const float *srate)
{
    float edot = sqrtf(second_invariant2(srate));
    edot = fmaxf(edot, 1e-30f);
    float le = __logf(edot);
    float inv = 0.f;
    int n = 0;
    for (int m = 0; m < F.nmat; ++m) {
        if (x.count[m] == 0) continue;
        float lv = F.vlog_coef[m] + F.vexp_pw[m] * le + F.vQ[m] / (F.vnR[m] * T);
        inv += (float)x.count[m] * expf(-lv);
        n += x.count[m];
    }
    float v = (inv > 0.f) ? (float)n / inv : F.visc_max;
    return fminf(fmaxf(v, F.visc_min), F.visc_max);
}

// matprops.cxx:646-704 in FP32
__device__ __forceinline__ void f_plastic_props(const ConstsF &F, const MixF &x, float pls, float &amc,
                                                float &anphi, float &ten_max)
{
    float c = 0.f, f = 0.f;
    int n = 0;
    for (int m = 0; m < F.nmat; ++m) {
        int k = x.count[m];
        if (k == 0) continue;
        n += k;
        float cm, fm;
        if (pls < F.pls0[m]) {
            cm = F.c0[m];
            fm = F.f0[m];
        } else if (pls < F.pls1[m]) {
            float p = (pls - F.pls0[m]) / (F.pls1[m] - F.pls0[m]);
            cm = F.c0[m] + p * (F.c1[m] - F.c0[m]);
            fm = F.f0[m] + p * (F.f1[m] - F.f0[m]);
        } else {
            cm = F.c1[m];
            fm = F.f1[m];
        }
        c += cm * (float)k;
        f += fm * (float)k;
    }
    float cohesion = c / (float)n, phi = f / (float)n;
    float sq, tph;
    if (phi == F.phi_c) {
        anphi = F.anphi_c;
        sq = F.sqanphi_c;
        tph = F.tphi_c;
    } else {
        float sp = sinf(phi * (float)kDeg2Rad);
        anphi = (1.f + sp) / (1.f - sp);
        sq = sqrtf(anphi);
        tph = tanf(phi * (float)kDeg2Rad);
    }
    amc = 2.f * cohesion * sq;
    ten_max = (phi == 0.f) ? F.tension_max : fminf(F.tension_max, cohesion / tph);
}

// FP32 counterpart of surely_elastic: a margin of 1e-4 of the stress scale
// covers FP32 rounding of the bound many times over
__device__ __forceinline__ bool f_surely_elastic(const float *s, float s0, float anphi, float amc,
                                                 float ten_max)
{
    float mp = (s[0] + s[1] + s[2]) * (1.f / 3.f);
    float a = s[0] - mp, b = s[1] - mp, c = s[2] - mp;
    float m = s0 + mp;
    float dev2 = a * a + b * b + c * c + 2.f * (s[3] * s[3] + s[4] * s[4] + s[5] * s[5]);
    float R = sqrtf(dev2 * (2.f / 3.f)) * (1.f + 1e-5f);
    float margin = 1e-4f * (fabsf(m) + R) * (1.f + anphi) + 1e-30f;
    return ((m - R) - anphi * (m + R) + amc) > margin && ((m + R) - ten_max) < -margin;
}

// FP32 principal values: eigenvalues of a symmetric 3x3 (xx yy zz xy xz yz) from the invariants of its
// deviator (trigonometric form), ascending; the isotropic shift m is added
// after, so a large pressure does not cancel the deviatoric part
__device__ __forceinline__ void f_principal_values(const float *s, float shift, float p[3])
{
    float m = (s[0] + s[1] + s[2]) * (1.f / 3.f);
    float a = s[0] - m, b = s[1] - m, c = s[2] - m;
    float j2 = 0.5f * (a * a + b * b + c * c) + s[3] * s[3] + s[4] * s[4] + s[5] * s[5];
    float j3 = a * b * c + 2.f * s[3] * s[4] * s[5] - a * s[5] * s[5] - b * s[4] * s[4] - c * s[3] * s[3];
    float r = sqrtf(j2 * (1.f / 3.f));
    float cos3 = (r > 0.f) ? j3 / (2.f * r * r * r) : 0.f;
    cos3 = fminf(fmaxf(cos3, -1.f), 1.f);
    float th = acosf(cos3) * (1.f / 3.f);
    float hi = 2.f * r * cosf(th), lo = 2.f * r * cosf(th + 2.0943951023931953f);
    float mid = -(hi + lo);
    p[0] = lo + m + shift;
    p[1] = mid + m + shift;
    p[2] = hi + m + shift;
    if (p[1] < p[0]) { float tmp = p[0]; p[0] = p[1]; p[1] = tmp; }
    if (p[2] < p[1]) { float tmp = p[1]; p[1] = p[2]; p[2] = tmp; }
    if (p[1] < p[0]) { float tmp = p[0]; p[0] = p[1]; p[1] = tmp; }
}

// "No failure" (rheology.cxx:193, fs > 0 and ft < 0) from the FP32 principal
// values of the trial (deviation form, plus s0), with a margin of 1e-2 of the
// yield function's scale: the trigonometric eigenvalues are off by up to
// about 2e-3 of the deviator's size next to a double eigenvalue, and the
// FP32 sums by far less.
__device__ __forceinline__ bool f_clearly_elastic(const float p[3], float s0f, float anphi, float amc,
                                                  float ten_max)
{
    const float lo = p[0] + s0f, hi = p[2] + s0f;
    const float margin = 1e-2f * (fabsf(lo) + anphi * fabsf(hi) + amc);
    return lo - anphi * hi + amc > margin && hi - ten_max < -margin;
}

// the exact FP64 return map for one element (rheology.cxx:578-598), from the
// FP32 state; returns eigen flags
__device__ __noinline__ int ep_fp64(const Consts &K, const Mix &x, double pls, double s0,
                                    const float *s_in, const float *de_in, float *s_out, double &depls)
{
    double s[6], de[6];
    for (int i = 0; i < 6; ++i) {
        s[i] = (double)s_in[i] + (i < 3 ? s0 : 0.0);
        de[i] = de_in[i];
    }
    double amc, anphi, anpsi, hardn, ten_max;
    plastic_props(K.M, x, pls, amc, anphi, anpsi, hardn, ten_max);
    int flags = elasto_plastic(x.bulkm, x.shearm, amc, anphi, anpsi, hardn, ten_max, de, depls, s);
    for (int i = 0; i < 6; ++i) s_out[i] = (float)(s[i] - (i < 3 ? s0 : 0.0));
    return flags | 8;
}

// elastic trial + bound; FP64 return map only where the bound fails
__device__ __forceinline__ int f_elasto_plastic(const DevF &d, const MixF &xf, int e, double pls,
                                                double s0, const float *s_old, const float *de,
                                                float *s_new, double &depls)
{
    const ConstsF &F = *d.F;
    float amc, anphi, ten_max;
    f_plastic_props(F, xf, (float)pls, amc, anphi, ten_max);
    for (int i = 0; i < 6; ++i) s_new[i] = s_old[i];
    elastic(xf.bulkm, xf.shearm, de, s_new);
    depls = 0;
    if (f_surely_elastic(s_new, (float)s0, anphi, amc, ten_max)) return 0;
    float p[3];
    f_principal_values(s_new, 0.f, p);
    if (f_clearly_elastic(p, (float)s0, anphi, amc, ten_max)) return 0;
    const Consts &K = *d.K;
    return ep_fp64(K, K.M.mix[d.mix[e]], pls, s0, s_old, de, s_new, depls);
}

// rheology.cxx:628-638 decides between the Maxwell stress sv and the
// elasto-plastic stress sp by the smaller second invariant.  Where sp is the
// elastic trial (no plastic correction) the two invariants differ by a
// relative 1e-7 for cold, stiff elements, below FP32 resolution, so the
// difference is formed exactly instead: with a = dev(s), b = 2G dev(de) and
// t = dt G / (2 eta), sv - sp = -t/(1+t) (2a + b) on the deviator, and
// J2(sv) - J2(sp) = B(sv - sp, sv + sp) for the bilinear form B of J2.
__device__ __forceinline__ float j2_bilinear(const float *u, const float *v)
{
    float mu = (u[0] + u[1] + u[2]) * (1.f / 3.f), mv = (v[0] + v[1] + v[2]) * (1.f / 3.f);
    return 0.5f * ((u[0] - mu) * (v[0] - mv) + (u[1] - mu) * (v[1] - mv) + (u[2] - mu) * (v[2] - mv)) +
           u[3] * v[3] + u[4] * v[4] + u[5] * v[5];
}
__device__ __forceinline__ bool f_viscous_wins(const MixF &xf, const float *s, const float *de,
                                               const float *sv, const float *sp, double depls,
                                               float dt, float visc)
{
    if (depls != 0) return second_invariant2(sv) < second_invariant2(sp);
    const float t = 0.5f * dt * xf.shearm / visc;
    const float k = t / (1.f + t);
    const float ms = tr3(s) * (1.f / 3.f), mde = tr3(de) * (1.f / 3.f);
    float dvec[6], w[6];
    for (int i = 0; i < 6; ++i) {
        float a = (i < 3) ? s[i] - ms : s[i];
        float b = 2.f * xf.shearm * ((i < 3) ? de[i] - mde : de[i]);
        dvec[i] = -k * (2.f * a + b);
        w[i] = 2.f * sp[i] + dvec[i];
    }
    return j2_bilinear(dvec, w) < 0.f;
}

// ---- fused passes ----------------------------------------------------------

__device__ __forceinline__ void f_next_contrib(const DevF &d, int e, int4 c, const float V[4][3],
                                               const float dx[4], const float dy[4], const float dz[4],
                                               float volf)
{
    const size_t E = d.nelem;
    float D[6];
    strain_rate(V, dx, dy, dz, D);
    f_store6(d.srate_next, E, e, D);
    d.c_trdv[e] = tr3(D) * volf;
    if (d.F->thermal) {
        // conduction vector kv (grad N_i . grad T) with grad T from temperature
        // differences (sum_j grad N_j = 0), differences taken in FP64
        double T0 = __ldg(d.T + c.x);
        float t1 = sf::to_float(__ldg(d.T + c.y) - T0), t2 = sf::to_float(__ldg(d.T + c.z) - T0),
              t3 = sf::to_float(__ldg(d.T + c.w) - T0);
        float gx = dx[1] * t1 + dx[2] * t2 + dx[3] * t3;
        float gy = dy[1] * t1 + dy[2] * t2 + dy[3] * t3;
        float gz = dz[1] * t1 + dz[2] * t2 + dz[3] * t3;
        float kv = d.F->mix[d.mix[e]].k * volf;
        for (int i = 0; i < 4; ++i) d.tmp[i * E + e] = kv * (dx[i] * gx + dy[i] * gy + dz[i] * gz);
    }
}

// FP64 geometry of the FP32 form: edge vectors from node 0, their cross
// products c_i = 6 V grad(N_i) (the cofactors; c_0 = -(c_1 + c_2 + c_3)) and
// the volume det / 6, the same quantities compute_volume (geometry.cxx:29-49)
// and compute_shape_fn (geometry.cxx:388-470) form, grouped so that the
// volume and the four gradients share one set of products.
__device__ __forceinline__ double f_cofactors(const double X[4][3], double cf[4][3])
{
    double a[3], b[3], q[3];
    for (int k = 0; k < 3; ++k) {
        a[k] = X[1][k] - X[0][k];
        b[k] = X[2][k] - X[0][k];
        q[k] = X[3][k] - X[0][k];
    }
    // (fused multiply-adds: this form is held to a tolerance, not to the
    // reference's rounding)
    // (the plain products on the integer pipes, sf::mul, rounded as the FP64
    // unit rounds them)
    cf[1][0] = fma(b[1], q[2], -sf::mul(b[2], q[1]));
    cf[1][1] = fma(b[2], q[0], -sf::mul(b[0], q[2]));
    cf[1][2] = fma(b[0], q[1], -sf::mul(b[1], q[0]));
    cf[2][0] = fma(q[1], a[2], -sf::mul(q[2], a[1]));
    cf[2][1] = fma(q[2], a[0], -sf::mul(q[0], a[2]));
    cf[2][2] = fma(q[0], a[1], -sf::mul(q[1], a[0]));
    cf[3][0] = fma(a[1], b[2], -sf::mul(a[2], b[1]));
    cf[3][1] = fma(a[2], b[0], -sf::mul(a[0], b[2]));
    cf[3][2] = fma(a[0], b[1], -sf::mul(a[1], b[0]));
    for (int k = 0; k < 3; ++k) cf[0][k] = -(cf[1][k] + cf[2][k] + cf[3][k]);
    return fma(a[0], cf[1][0], fma(a[1], cf[1][1], sf::mul(a[2], cf[1][2])));     // 6 V
}

// FP64 part of the element force vectors for the next step: s0 grad(N_i) V
// = s0 c_i / 6, plus rho_ref g V / 4 on z (fields.cxx:336-340 with the split
// stress)
__device__ __forceinline__ void f_reference_force(const DevF &d, int e, const double cf[4][3], double vol)
{
    const size_t E = d.nelem;
    const double s6 = sf::mul(d.s0[e], 1.0 / 6.0);
    const double buoy = d.F->gravity != 0.f ? sf::mul(d.F->mix[d.mix[e]].rho_g4, vol) : 0.0;
    for (int i = 0; i < 4; ++i) {
        d.f0[(i)*E + e] = s6 * cf[i][0];
        d.f0[(i + 4) * E + e] = s6 * cf[i][1];
        d.f0[(i + 8) * E + e] = fma(s6, cf[i][2], buoy);
    }
}

__global__ void kf_prime(DevF d)
{
    int e = gtid();
    if (e >= d.nelem) return;
    int4 c = d.conn[e];
    float V[4][3], dx[4], dy[4], dz[4];
    f_load_vel4(d, c, V);
    f_load_shp(d, e, dx, dy, dz);
    {
        double X[4][3], cf[4][3];
        f_load_xyz4(d, c, X);
        f_cofactors(X, cf);
        f_reference_force(d, e, cf, d.vol[e]);
    }
    f_next_contrib(d, e, c, V, dx, dy, dz, (float)d.vol[e]);
}

// N-A
__global__ void kf_fn_a(DevF d)
{
    int n = gtid();
    const ConstsF &F = *d.F;
    const double dt = d.clk->dt;
    if (n == 0) {
        d.clk->steps += 1;
        d.clk->time += dt;
        d.clk->npend = 0;
        d.clk->nexact = 0;
    }
    if (n >= d.nnode) return;
    const size_t E = d.nelem;
    const int q0 = d.sup_off[n], q1 = d.sup_off[n + 1];
    float vn, tm;
    if (d.clk->mass_valid) {
        vn = d.vol_n[n];
        tm = d.tmass[n];
    } else {
        float m = 0.f;
        vn = 0.f;
        tm = 0.f;
        for (int q = q0; q < q1; ++q) {
            size_t e = __ldg(d.sup_ent + q) >> 2;
            vn += d.c_vol[e];
            m += d.c_mass[e];
            if (F.thermal) tm += d.c_tmass[e];
        }
        d.vol_n[n] = vn;
        d.mass[n] = m;
        d.tmass[n] = tm;
    }
    if (F.thermal) {
        float tdot = 0.f;
        for (int q = q0; q < q1; ++q) {
            unsigned p = __ldg(d.sup_ent + q);
            tdot += d.tmp[(p & 3u) * E + (p >> 2)];
        }
        if (d.bcflag[n] & kBoundZ1)
            d.T[n] = d.K->surface_temperature;
        else
            d.T[n] -= (double)tdot * dt / (double)tm;
    }
    float dv = 0.f;
    for (int q = q0; q < q1; ++q) dv += d.c_trdv[__ldg(d.sup_ent + q) >> 2];
    d.ntmp[n] = dv / vn;
}

// E-B: edvoldt + update_stress (FP32 with the FP64 return map where needed),
// over the elements from e0 (a multiple of the block size)
__global__ void kf_fe_b(DevF d, int e0)
{
    int e = e0 + gtid();
    if (e == 0) d.clk->mass_valid = 1;
    bool live = e < d.nelem;
    int flags = 0;
    if (live) {
        const size_t E = d.nelem;
        const ConstsF &F = *d.F;
        int4 c = d.conn[e];
        const MixF &xf = F.mix[d.mix[e]];
        float edv = (d.ntmp[c.x] + d.ntmp[c.y] + d.ntmp[c.z] + d.ntmp[c.w]) * 0.25f;
        d.edvoldt[e] = edv;
        float s[6], es[6], edot[6];
        f_load6(d.stress, E, e, s);
        f_load6(d.strain, E, e, es);
        f_load6(d.srate_next, E, e, edot);
        double pls = d.pls[e];
        const double s0 = d.s0[e];
        float dpls = d.dpls[e];
        const float dt = (float)d.clk->dt;
        float old_s = tr3(s);
        float div = tr3(edot);
        for (int i = 0; i < 3; ++i) edot[i] += (edv - div) * (1.f / 3.f);
        float de[6];
        for (int i = 0; i < 6; ++i) {
            es[i] += edot[i] * dt;
            de[i] = edot[i] * dt;
        }
        switch (F.rheol) {
        case 1:
            elastic(xf.bulkm, xf.shearm, de, s);
            break;
        case 2: {
            float visc = f_visc(F, xf, f_elem_T(d, c), edot);
            viscous(xf.bulkm, visc, tr3(es), edot, s);      // a full stress, not an increment
            for (int i = 0; i < 3; ++i) s[i] = (float)((double)s[i] - s0);
        } break;
        case 3: {
            float visc = f_visc(F, xf, f_elem_T(d, c), edot);
            float dv = (float)(d.vol[e] / d.vol_old[e] - 1);
            maxwell(xf.bulkm, xf.shearm, visc, dt, dv, de, s);
        } break;
        case 5: {
            double depls;
            float sn[6];
            flags = f_elasto_plastic(d, xf, e, pls, s0, s, de, sn, depls);
            for (int i = 0; i < 6; ++i) s[i] = sn[i];
            pls += depls;
            dpls = (float)depls;
        } break;
        case 7: {
            float visc = f_visc(F, xf, f_elem_T(d, c), edot);
            float dv = (float)(d.vol[e] / d.vol_old[e] - 1);
            float sv[6];
            for (int i = 0; i < 6; ++i) sv[i] = s[i];
            maxwell(xf.bulkm, xf.shearm, visc, dt, dv, de, sv);
            double depls;
            float sp[6];
            flags = f_elasto_plastic(d, xf, e, pls, s0, s, de, sp, depls);
            if (f_viscous_wins(xf, s, de, sv, sp, depls, dt, visc)) {
                for (int i = 0; i < 6; ++i) s[i] = sv[i];
            } else {
                for (int i = 0; i < 6; ++i) s[i] = sp[i];
                pls += depls;
                dpls = (float)depls;
            }
        } break;
        }
        float dp = tr3(s) - old_s;
        f_store6(d.stress, E, e, s);
        f_store6(d.strain, E, e, es);
        f_store6(d.srate, E, e, edot);
        d.pls[e] = pls;
        d.dpls[e] = dpls;
        d.dp[e] = dp;
        d.tmp_sg[e] = dp * d.c_vol[e];
    }
    unsigned solved = __ballot_sync(0xffffffffu, flags & 1);
    unsigned ql = __ballot_sync(0xffffffffu, flags & 2);
    if ((threadIdx.x & 31) == 0) {
        if (solved) atomicAdd(&d.clk->eig, (unsigned long long)__popc(solved));
        if (ql) atomicAdd(&d.clk->ql, (unsigned long long)__popc(ql));
    }
}

// N-B
__global__ void kf_sg_gather(DevF d)
{
    int n = gtid();
    if (n >= d.nnode) return;
    float s = 0.f;
    for (int q = d.sup_off[n]; q < d.sup_off[n + 1]; ++q) s += d.tmp_sg[__ldg(d.sup_ent + q) >> 2];
    d.ntmp[n] = s / d.vol_n[n];
}

// E-C (registers bounded for 12 blocks of 128 per SM: 0.231 -> 0.225 ms on
// config 2)
__global__ void __launch_bounds__(128, 12) kf_fe_c(DevF d)
{
    int e = gtid();
    if (e >= d.nelem) return;
    const size_t E = d.nelem;
    const ConstsF &F = *d.F;
    int4 c = d.conn[e];
    float dp_el = (d.ntmp[c.x] + d.ntmp[c.y] + d.ntmp[c.z] + d.ntmp[c.w]) * 0.25f;
    float ddp = (dp_el - d.dp[e]) * (1.f / 3.f);
    float s[6];
    f_load6(d.stress, E, e, s);
    for (int i = 0; i < 3; ++i) {
        s[i] += ddp;
        d.stress[i * E + e] = s[i];
    }
    float dx[4], dy[4], dz[4];
    f_load_shp(d, e, dx, dy, dz);
    float vol = d.c_vol[e];
    // FP32 part of the buoyancy: the thermal change of the density (the
    // rho0 g V / 4 part is in f0)
    float buoy = 0.f;
    if (F.gravity != 0.f)
        buoy = -F.mix[d.mix[e]].rho_alpha * (f_elem_T(d, c) - 273.f) * F.gravity * 0.25f;
    for (int i = 0; i < 4; ++i) {
        d.tmp[(i)*E + e] = (s[0] * dx[i] + s[3] * dy[i] + s[4] * dz[i]) * vol;
        d.tmp[(i + 4) * E + e] = (s[3] * dx[i] + s[1] * dy[i] + s[5] * dz[i]) * vol;
        d.tmp[(i + 8) * E + e] = (s[4] * dx[i] + s[5] * dy[i] + s[2] * dz[i] + buoy) * vol;
    }
}

// N-C
__global__ void kf_fn_c(DevF d)
{
    int n = gtid();
    if (n >= d.nnode) return;
    const size_t E = d.nelem;
    const Consts &K = *d.K;
    const double dt = d.clk->dt;
    const float dtf = (float)dt;
    float g[3] = {0.f, 0.f, 0.f};
    double h[3] = {0.0, 0.0, 0.0};
    // the FP64 reference part and the FP32 part in two walks over the
    // support list, each streaming its own arrays (one walk over both:
    // 282 against 194 B per element read from DRAM, 0.46 against 0.35 ms
    // on config 2)
    const int q0 = d.sup_off[n], q1 = d.sup_off[n + 1];
    for (int q = q0; q < q1; ++q) {
        unsigned p = __ldg(d.sup_ent + q);
        size_t e = p >> 2, i = p & 3u;
        h[0] -= d.f0[(i)*E + e];
        h[1] -= d.f0[(i + 4) * E + e];
        h[2] -= d.f0[(i + 8) * E + e];
    }
    for (int q = q0; q < q1; ++q) {
        unsigned p = __ldg(d.sup_ent + q);
        size_t e = p >> 2, i = p & 3u;
        g[0] -= d.tmp[(i)*E + e];
        g[1] -= d.tmp[(i + 4) * E + e];
        g[2] -= d.tmp[(i + 8) * E + e];
    }
    // the boundary tractions balance the FP64 reference part: FP64 as well
    stress_bc_node(K, d.bf, n, d.bcflag[n], d.z[n], d.z0[n], h);
    float f[3] = {(float)(h[0] + (double)g[0]), (float)(h[1] + (double)g[1]),
                  (float)(h[2] + (double)g[2])};
    float v[3] = {d.vx[n], d.vy[n], d.vz[n]};
    if (d.F->is_qs) {
        f[0] = damp(K, f[0], v[0]);
        f[1] = damp(K, f[1], v[1]);
        f[2] = damp(K, f[2], v[2]);
    }
    d.fx[n] = f[0];
    d.fy[n] = f[1];
    d.fz[n] = f[2];
    float m = d.mass[n];
    for (int j = 0; j < 3; ++j) v[j] += dtf * f[j] / m;
    vbc_node(K, d.bcflag[n], v);
    d.vx[n] = v[0];
    d.vy[n] = v[1];
    d.vz[n] = v[2];
    const double x = d.x[n] + (double)v[0] * dt, y = d.y[n] + (double)v[1] * dt,
                 z = d.z[n] + (double)v[2] * dt;
    d.x[n] = x;
    d.y[n] = y;
    d.z[n] = z;
    if (not_finite(x) || not_finite(y) || not_finite(z)) atomicOr(&d.clk->status, 0x2u);
}

// FP64 volume and shape derivatives of one element, rounded to FP32 for use;
// also forms f0 from the FP64 derivatives.  With c2max, the largest squared
// cofactor norm: |c_i| is twice the area of the face opposite node i.
__device__ __forceinline__ double f_geometry(const DevF &d, int e, int4 c, float dx[4], float dy[4],
                                             float dz[4], double *c2max)
{
    const size_t E = d.nelem;
    double X[4][3];
    f_load_xyz4(d, c, X);
    double cf[4][3];
    const double det = f_cofactors(X, cf);
    const double vol = sf::mul(det, 1.0 / 6.0);
    f_reference_force(d, e, cf, vol);
    if (c2max) {
        double m = 0;
        for (int i = 0; i < 4; ++i) m = fmax(m, fma(cf[i][0], cf[i][0], fma(cf[i][1], cf[i][1], cf[i][2] * cf[i][2])));
        *c2max = m;
    }
    // the gradients themselves are FP32: c_i / (6 V)
    const float iv = 1.f / sf::to_float(det);
    for (int i = 0; i < 4; ++i) {
        dx[i] = sf::to_float(cf[i][0]) * iv;
        dy[i] = sf::to_float(cf[i][1]) * iv;
        dz[i] = sf::to_float(cf[i][2]) * iv;
        d.shp[(0 + i) * E + e] = dx[i];
        d.shp[(4 + i) * E + e] = dy[i];
        d.shp[(8 + i) * E + e] = dz[i];
    }
    return vol;
}

// E-A, over the elements from e0 (a multiple of the block size); the pass
// has nblocks blocks in all.  Registers bounded for 9 blocks of 128 per SM
// (1.07 -> 1.01 ms on config 2).
__global__ void __launch_bounds__(128, 9) kf_fe_a(DevF d, int e0, unsigned nblocks)
{
    int e = e0 + gtid();
    const Consts &K = *d.K;
    const ConstsF &F = *d.F;
    const bool dt_step = (K.fixed_dt == 0) && (d.clk->steps % 10 == 0);
    if (e == 0) d.clk->mass_valid = 0;
    bool live = e < d.nelem;
    double minh = 0;
    if (live) {
        const size_t E = d.nelem;
        int4 c = d.conn[e];
        float dx[4], dy[4], dz[4];
        double c2max = 0;
        double vol = f_geometry(d, e, c, dx, dy, dz, dt_step ? &c2max : nullptr);
        d.vol_old[e] = d.vol[e];
        d.vol[e] = vol;
        if (not_positive(vol)) atomicOr(&d.clk->status, 0x4u);
        float volf = sf::to_float(vol);
        d.c_vol[e] = volf;
        const MixF &xf = F.mix[d.mix[e]];
        {
            float rT = f_rho(F, xf, f_elem_T(d, c));
            d.c_mass[e] = (F.is_qs ? xf.rho_qs : rT) * volf * 0.25f;
            if (F.thermal) d.c_tmass[e] = rT * xf.cp * volf * 0.25f;
        }
        float V[4][3];
        f_load_vel4(d, c, V);
        if (F.rheol & 1) {
            float w3, w4, w5, s[6];
            spin(V, dx, dy, dz, w3, w4, w5);
            const float dt = (float)d.clk->dt;
            f_load6(d.stress, E, e, s);
            jaumann(s, dt, w3, w4, w5);
            f_store6(d.stress, E, e, s);
            f_load6(d.strain, E, e, s);
            jaumann(s, dt, w3, w4, w5);
            f_store6(d.strain, E, e, s);
        }
        f_next_contrib(d, e, c, V, dx, dy, dz, volf);
        if (dt_step) {
            // the reference's 3 V / (largest face area) (geometry.cxx:280-293)
            // from the cofactors: 6 V / max |c_i|
            minh = 6 * vol / sqrt(c2max);
        }
    }
    if (dt_step) {
        Dev dd;
        dd.conn = d.conn;
        dd.T = d.T;
        dd.mix = d.mix;
        dd.K = d.K;
        dd.clk = d.clk;
        dt_reduce_and_finalize(dd, minh, live, nblocks);
    }
}

__global__ void kf_mass_flush(DevF d)
{
    int n = gtid();
    if (n == 0) d.clk->mass_valid = 1;
    if (n >= d.nnode) return;
    const bool thermal = d.F->thermal;
    float vn = 0.f, m = 0.f, tm = 0.f;
    for (int q = d.sup_off[n]; q < d.sup_off[n + 1]; ++q) {
        size_t e = __ldg(d.sup_ent + q) >> 2;
        vn += d.c_vol[e];
        m += d.c_mass[e];
        if (thermal) tm += d.c_tmass[e];
    }
    d.vol_n[n] = vn;
    d.mass[n] = m;
    d.tmass[n] = tm;
}

// ---- init() for the FP32 form ----------------------------------------------

// geometry.cxx:354-381 with T = 0 (the first compute_mass of init)
__global__ void kf_init_geometry(DevF d)
{
    int e = gtid();
    if (e >= d.nelem) return;
    int4 c = d.conn[e];
    float dx[4], dy[4], dz[4];
    double vol = f_geometry(d, e, c, dx, dy, dz, nullptr);
    d.vol[e] = vol;
    d.vol_old[e] = vol;
    float volf = (float)vol;
    d.c_vol[e] = volf;
    const ConstsF &F = *d.F;
    const MixF &xf = F.mix[d.mix[e]];
    float r0 = f_rho(F, xf, 0.f);
    d.c_mass[e] = (F.is_qs ? xf.rho_qs : r0) * volf * 0.25f;
    d.c_tmass[e] = F.thermal ? r0 * xf.cp * volf * 0.25f : 0.f;
}

// volume, shape derivatives and mass contributions from the current
// coordinates and temperature, as E-A leaves them at the end of a step (the
// host-buffer path derives them instead of uploading them)
__global__ void kf_derive_geometry(DevF d)
{
    int e = gtid();
    if (e >= d.nelem) return;
    int4 c = d.conn[e];
    float dx[4], dy[4], dz[4];
    double vol = f_geometry(d, e, c, dx, dy, dz, nullptr);
    d.vol[e] = vol;
    float volf = (float)vol;
    d.c_vol[e] = volf;
    const ConstsF &F = *d.F;
    const MixF &xf = F.mix[d.mix[e]];
    float rT = f_rho(F, xf, f_elem_T(d, c));
    d.c_mass[e] = (F.is_qs ? xf.rho_qs : rT) * volf * 0.25f;
    if (F.thermal) d.c_tmass[e] = rT * xf.cp * volf * 0.25f;
}

__global__ void kf_vbcs(DevF d)
{
    int n = gtid();
    if (n >= d.nnode) return;
    unsigned flag = d.bcflag[n];
    if (!(flag & kBoundAny)) return;
    float v[3] = {d.vx[n], d.vy[n], d.vz[n]};
    vbc_node(*d.K, flag, v);
    d.vx[n] = v[0];
    d.vy[n] = v[1];
    d.vz[n] = v[2];
}

// ic.cxx:100-131, evaluated in FP64
__global__ void kf_init_stress(DevF d)
{
    int e = gtid();
    if (e >= d.nelem) return;
    const size_t E = d.nelem;
    const Consts &K = *d.K;
    const double ks = K.M.mix[d.mix[K.ref_pressure_option != 0 ? e : 0]].bulkm;
    int4 c = d.conn[e];
    double zc = elem_mean4(__ldg(d.z + c.x), __ldg(d.z + c.y), __ldg(d.z + c.z), __ldg(d.z + c.w));
    double p = ref_pressure(K.ref_pressure_option, K.rho0_0, K.gravity, zc);
    d.s0[e] = -p;
    for (int i = 0; i < 3; ++i) {
        d.stress[i * E + e] = 0.f;
        d.strain[i * E + e] = (float)(-p / ks / 3);
    }
}

// host stress rows (AoS, FP64) <-> s0 (mean of the diagonal) + FP32 deviation
__global__ void k_stress_split(const double *src, double *s0, float *dst, long long rows, long long row0,
                               long long ld)
{
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const double *a = src + 6 * r;
    double m = (a[0] + a[1] + a[2]) / 3;
    s0[row0 + r] = m;
    for (int c = 0; c < 6; ++c) dst[c * ld + row0 + r] = (float)(a[c] - (c < 3 ? m : 0.0));
}
__global__ void k_stress_join(const double *s0, const float *src, double *dst, long long rows,
                              long long row0, long long ld)
{
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    double m = s0[row0 + r];
    for (int c = 0; c < 6; ++c) dst[6 * r + c] = (double)src[c * ld + row0 + r] + (c < 3 ? m : 0.0);
}

// the same split for page-locked host rows read in place: a block moves 256
// rows through shared memory so that the host side is read in whole
// contiguous runs
__global__ void k_stress_split_tiled(const double *src, double *s0, float *dst, long long rows)
{
    __shared__ double t[256 * 6];
    const long long r0 = (long long)blockIdx.x * 256;
    const int nr = (int)min(256LL, rows - r0);
    for (int i = threadIdx.x; i < nr * 6; i += blockDim.x) t[i] = src[r0 * 6 + i];
    __syncthreads();
    const int r = threadIdx.x;
    if (r >= nr) return;
    const double *a = t + 6 * r;
    double m = (a[0] + a[1] + a[2]) / 3;
    s0[r0 + r] = m;
    for (int c = 0; c < 6; ++c) dst[c * rows + r0 + r] = (float)(a[c] - (c < 3 ? m : 0.0));
}

// ---- Output::average_fields (output.cxx:227-267) after a step ---------------
// Both forms: the element sources are FP64 arrays or FP32 arrays (the FP32
// stress adding the reference stress s0 back).
struct AvgArgs {
    int nnode, nelem, interval;
    const Clock *clk;
    const double *coord;                        // SoA x | y | z
    const double *stress, *strain, *dpls;       // FP64 form
    const float *stress_f, *strain_f, *dpls_f;  // FP32 form
    const double *s0;
    double *c0, *strain0, *stress_sum, *dpls_sum, *time0;
};
__global__ void k_average_fields(AvgArgs a)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const bool first = (a.clk->steps % a.interval) == 1;
    if (i == 0 && first) *a.time0 = a.clk->time;
    if (first && i < 3LL * a.nnode) a.c0[i] = a.coord[i];
    if (i >= a.nelem) return;
    const size_t E = a.nelem;
    for (int c = 0; c < 6; ++c) {
        double sv, ev;
        if (a.stress) {
            sv = a.stress[c * E + i];
            ev = a.strain[c * E + i];
        } else {
            sv = (double)a.stress_f[c * E + i] + (c < 3 ? a.s0[i] : 0.0);
            ev = (double)a.strain_f[c * E + i];
        }
        if (first) {
            a.strain0[c * E + i] = ev;
            a.stress_sum[c * E + i] = sv;
        } else {
            a.stress_sum[c * E + i] += sv;
        }
    }
    const double dp = a.dpls ? a.dpls[i] : (double)a.dpls_f[i];
    if (first)
        a.dpls_sum[i] = dp;
    else
        a.dpls_sum[i] += dp;
}

__global__ void k_vol_to_f(const double *vol, float *volf, long long n)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) volf[i] = (float)vol[i];
}

// ---- layout conversion with FP64 <-> FP32 ----------------------------------
__global__ void k_aos_to_soa_f(const double *src, float *dst, int ncomp, long long rows, long long row0,
                               long long ld)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * ncomp) return;
    long long r = i / ncomp;
    int c = (int)(i - r * ncomp);
    dst[c * ld + row0 + r] = (float)src[i];
}
__global__ void k_soa_to_aos_f(const float *src, double *dst, int ncomp, long long rows, long long row0,
                               long long ld)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * ncomp) return;
    long long r = i / ncomp;
    int c = (int)(i - r * ncomp);
    dst[i] = (double)src[c * ld + row0 + r];
}

}  // namespace des
