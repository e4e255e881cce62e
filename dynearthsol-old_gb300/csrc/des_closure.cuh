// The learned return-map closure inside the FP32 stress pass (E-B).
//
// For the elasto-plastic rheologies the reference computes the principal
// stresses of the elastic trial with dsyevh3 and returns the trial to the
// Mohr-Coulomb surface (rheology.cxx:180-240); the FP32 form does that in
// FP64 for every element the cheap elastic bound cannot clear.  With a
// closure set, the pass sorts those elements per CTA:
//
//   network candidates  the FP32 principal values of the trial say "shear
//                       return, clearly": fs < -tol S and h < -tol S
//   exact               everything else (near the yield surface, the tensile
//                       or corner branches, inputs outside the training
//                       envelope)
//
// Candidates are compacted into 16-row tiles and evaluated by the MLP on the
// tensor cores.  Each prediction is then judged in FP32: the predicted
// stress must lie on the yield surface, |fs(sigma) - 2 sqrt(anphi) hardn
// alam| <= tol S (the hardening term is the residual the reference's own
// return leaves), inside the tensile cutoff, with a positive plastic-strain
// increment; for rh_evp the Maxwell/plastic choice must also be clear.
// Rejected candidates join the exact queue, and the exact queue is
// compacted onto the first threads of the CTA, which run the FP64 return
// map, so that the FP64 work is not spread over every warp.
//
// Network input (14; 8 used): four quantities, functions of the old stress,
// the strain increment and the plastic strain,
//   the principal values of the unit deviator n of the elastic trial   3
//   plastic strain capped at the largest pls1                           1
// normalised as x = (raw - in_mean) * in_scale, each entering as a pair of
// BF16 values (x = hi + lo / 256).  The temperature does not enter the
// shear return (it acts through the viscosity, outside the network).
// Network output (7, raw = y * out_scale; 4 used): a, b D, c D and
// depls / |alam|, where the return per unit plastic multiplier is
//   R = (trial - new stress) / (2 G alam) = a I + b n + c dev(n n)
// (an isotropic function of the trial, so three coefficients describe it,
// Cayley-Hamilton) and D = (3 l_min^2 - 1)(3 l_max^2 - 1) clears the poles
// b and c have where two principal values meet.  alam = fs / (a1 - a2 anpsi
// + a1 anphi anpsi - a2 anphi + 2 sqrt(anphi) hardn) comes from the FP32
// principal values of the trial.
#pragma once

#include "des_kernels32.cuh"
#include "des_mlp.cuh"

namespace des {

constexpr int kNnBlock = 128;

struct NnSmem {
    __nv_bfloat16 w1[kMlpHid * kMlpIn], w2[kMlpHid * kMlpHid], w3[kMlpOut * kMlpHid];
    float b1[kMlpHid], b2[kMlpHid], b3[kMlpOut];
    __nv_bfloat16 x[kNnBlock * kMlpIn];
    __nv_bfloat16 h1[kNnBlock / 32][16 * kHStride], h2[kNnBlock / 32][16 * kHStride];
    float y[kNnBlock * kMlpOut];
    float so[6][kNnBlock], de[6][kNnBlock];      // inputs of the exact return map
    float res[6][kNnBlock];                      // its outputs
    double resd[kNnBlock];
    int queue[kNnBlock];
    int wcount[kNnBlock / 32];
};

// FP32 plastic properties with the dilation factor and the hardening slope
// (matprops.cxx:646-704)
__device__ __forceinline__ void f_plastic_full(const ConstsF &F, const MixF &x, float pls, float &amc,
                                               float &anphi, float &anpsi, float &hardn, float &ten_max)
{
    float c = 0.f, f = 0.f, dd = 0.f, h = 0.f;
    int n = 0;
    for (int m = 0; m < F.nmat; ++m) {
        int k = x.count[m];
        if (k == 0) continue;
        n += k;
        float cm, fm, dm, hm = 0.f;
        if (pls < F.pls0[m]) {
            cm = F.c0[m];
            fm = F.f0[m];
            dm = F.d0[m];
        } else if (pls < F.pls1[m]) {
            float p = (pls - F.pls0[m]) / (F.pls1[m] - F.pls0[m]);
            cm = F.c0[m] + p * (F.c1[m] - F.c0[m]);
            fm = F.f0[m] + p * (F.f1[m] - F.f0[m]);
            dm = F.d0[m] + p * (F.d1[m] - F.d0[m]);
            hm = F.hslope[m];
        } else {
            cm = F.c1[m];
            fm = F.f1[m];
            dm = F.d1[m];
        }
        c += cm * (float)k;
        f += fm * (float)k;
        dd += dm * (float)k;
        h += hm * (float)k;
    }
    const float cohesion = c / (float)n, phi = f / (float)n, psi = dd / (float)n;
    hardn = h / (float)n;
    const float sphi = sinf(phi * (float)kDeg2Rad), spsi = sinf(psi * (float)kDeg2Rad);
    anphi = (1.f + sphi) / (1.f - sphi);
    anpsi = (1.f + spsi) / (1.f - spsi);
    amc = 2.f * cohesion * sqrtf(anphi);
    ten_max = (phi == 0.f) ? F.tension_max : fminf(F.tension_max, cohesion / tanf(phi * (float)kDeg2Rad));
}

// The unit deviator n of the trial (deviation form st), dev(n n), and the
// eigenvalues of n from the trial's principal values p (ascending).
__device__ __forceinline__ bool nn_basis(const float *st, const float p[3], float n[6], float q[6], float lam[3])
{
    const float m = (st[0] + st[1] + st[2]) * (1.f / 3.f);
    n[0] = st[0] - m;
    n[1] = st[1] - m;
    n[2] = st[2] - m;
    n[3] = st[3];
    n[4] = st[4];
    n[5] = st[5];
    const float j2 = 0.5f * (n[0] * n[0] + n[1] * n[1] + n[2] * n[2]) + n[3] * n[3] + n[4] * n[4] + n[5] * n[5];
    if (!(j2 > 0.f)) return false;
    const float inv = rsqrtf(j2);
    for (int i = 0; i < 6; ++i) n[i] *= inv;
    q[0] = n[0] * n[0] + n[3] * n[3] + n[4] * n[4];
    q[1] = n[3] * n[3] + n[1] * n[1] + n[5] * n[5];
    q[2] = n[4] * n[4] + n[5] * n[5] + n[2] * n[2];
    q[3] = n[0] * n[3] + n[3] * n[1] + n[4] * n[5];
    q[4] = n[0] * n[4] + n[3] * n[5] + n[4] * n[2];
    q[5] = n[3] * n[4] + n[1] * n[5] + n[5] * n[2];
    const float mq = (q[0] + q[1] + q[2]) * (1.f / 3.f);
    for (int i = 0; i < 3; ++i) {
        q[i] -= mq;
        lam[i] = (p[i] - m) * inv;
    }
    return true;
}

// (3 l_min^2 - 1)(3 l_max^2 - 1), zero where the least or the most compressive
// principal direction is not unique: the poles of the return's coefficients
__device__ __forceinline__ float nn_pole(const float lam[3])
{
    return (3.f * lam[0] * lam[0] - 1.f) * (3.f * lam[2] * lam[2] - 1.f);
}

// what a candidate needs to turn the network output into a stress and to
// judge it
struct NnCand {
    float alam, S, cf, anphi, hardn, ft_shift;
};

// kind: 0 = done (elastic), 1 = network candidate, 2 = exact FP64 return map
template <int RHEOL>
__global__ void __launch_bounds__(kNnBlock) kf_fe_b_nn(DevF d, const MlpDev *__restrict__ net)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    NnSmem &S = *reinterpret_cast<NnSmem *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int e = blockIdx.x * kNnBlock + tid;
    if (e == 0) d.clk->mass_valid = 1;
    const bool live = e < d.nelem;
    const size_t E = d.nelem;
    const ConstsF &F = *d.F;
    const float tol = net->tol;

    int kind = 0;
    float so[6], de[6];      // old stress and strain increment (deviation form)
    float s[6], sv[6];       // trial, Maxwell stress (rh_evp)
    float visc = 0.f, dpls = 0.f, dt = 0.f;
    double pls = 0.0, s0 = 0.0;
    NnCand cd = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    float raw[kMlpIn];
    int mixid = 0;
    if (live) {
        int4 c = d.conn[e];
        mixid = d.mix[e];
        const MixF &xf = F.mix[mixid];
        float edv = (d.ntmp[c.x] + d.ntmp[c.y] + d.ntmp[c.z] + d.ntmp[c.w]) * 0.25f;
        d.edvoldt[e] = edv;
        float es[6], edot[6];
        f_load6(d.stress, E, e, so);
        f_load6(d.strain, E, e, es);
        f_load6(d.srate_next, E, e, edot);
        pls = d.pls[e];
        s0 = d.s0[e];
        dpls = d.dpls[e];
        dt = (float)d.clk->dt;
        float div = tr3(edot);
        for (int i = 0; i < 3; ++i) edot[i] += (edv - div) * (1.f / 3.f);
        for (int i = 0; i < 6; ++i) {
            es[i] += edot[i] * dt;
            de[i] = edot[i] * dt;
            s[i] = so[i];
        }
        f_store6(d.strain, E, e, es);
        f_store6(d.srate, E, e, edot);
        const float Te = f_elem_T(d, c);
        if (RHEOL == 7) {
            visc = f_visc(F, xf, Te, edot);
            float dv = (float)(d.vol[e] / d.vol_old[e] - 1);
            for (int i = 0; i < 6; ++i) sv[i] = so[i];
            maxwell(xf.bulkm, xf.shearm, visc, dt, dv, de, sv);
        }
        float amc, anphi, anpsi, hardn, ten_max;
        // the elastic tests exactly as the pass without a closure applies them
        const float plsf = (float)pls, s0f = (float)s0;
        f_plastic_props(F, xf, plsf, amc, anphi, ten_max);
        elastic(xf.bulkm, xf.shearm, de, s);
        float p[3];
        if (!f_surely_elastic(s, s0f, anphi, amc, ten_max) &&
            (f_principal_values(s, 0.f, p), !f_clearly_elastic(p, s0f, anphi, amc, ten_max))) {
            kind = 2;
            // FP32 throughout: the tests below have margins of tol S, and the
            // FP32 sums are good to about 1e-7 S
            f_plastic_full(F, xf, plsf, amc, anphi, anpsi, hardn, ten_max);
            cd.anphi = anphi;
            cd.hardn = hardn;
            cd.cf = (1.f - anphi) * s0f + amc;
            cd.ft_shift = s0f - ten_max;
            cd.S = fabsf(p[0] + s0f) + anphi * fabsf(p[2] + s0f) + amc;
            const float fs = p[0] - anphi * p[2] + cd.cf;
            const float pa = sqrtf(1.f + anphi * anphi) + anphi;
            const float ps = ten_max * anphi - amc;
            const float h = p[2] + s0f - ten_max + pa * (p[0] + s0f - ps);
            const float a1 = xf.bulkm + (4.f / 3.f) * xf.shearm, a2 = xf.bulkm - (2.f / 3.f) * xf.shearm;
            const float den = a1 - a2 * anpsi + a1 * anphi * anpsi - a2 * anphi + 2.f * sqrtf(anphi) * hardn;
            cd.alam = fs / den;
            // past the largest pls1 the plastic properties no longer change,
            // so the network sees the plastic strain saturated there
            float pls_sat = 0.f;
            for (int m = 0; m < F.nmat; ++m) pls_sat = fmaxf(pls_sat, F.pls1[m]);
            float nb[6], qb[6], lam[3];
            if (fs < -tol * cd.S && h < -tol * cd.S && nn_basis(s, p, nb, qb, lam)) {
                raw[0] = lam[0];
                raw[1] = lam[1];
                raw[2] = lam[2];
                raw[3] = fminf(plsf, pls_sat);
                for (int i = 4; i < kMlpIn; ++i) raw[i] = 0.f;
                bool inside = true;
                for (int i = 0; i < kMlpInUsed; ++i) {
                    raw[i] = (raw[i] - net->in_mean[i]) * net->in_scale[i];
                    inside = inside && raw[i] >= net->env_lo[i] && raw[i] <= net->env_hi[i];
                }
                if (inside) {
                    kind = 1;
                    // each input enters as a BF16 pair, x = hi + lo / 256, so that
                    // the network sees it to about 16 significant bits
                    for (int i = 3; i >= 0; --i) {
                        const float x = raw[i];
                        const float hi = __bfloat162float(__float2bfloat16(x));
                        raw[2 * i] = hi;
                        raw[2 * i + 1] = (x - hi) * 256.f;
                    }
                }
            }
            for (int i = 0; i < 6; ++i) {
                S.so[i][tid] = so[i];
                S.de[i][tid] = de[i];
            }
        }
    }

    float sp[6];
    double depls = 0.0;
    // CTAs whose elements are all elastic skip the network and the queue
    if (__syncthreads_or(kind != 0)) {
        // ---- compaction of the network candidates ------------------------
        const unsigned cmask = __ballot_sync(0xffffffffu, kind == 1);
        if (lane == 0) S.wcount[w] = __popc(cmask);
        __syncthreads();
        int nc = 0, slot = 0;
        for (int i = 0; i < kNnBlock / 32; ++i) {
            if (i == w) slot = nc + __popc(cmask & ((1u << lane) - 1u));
            nc += S.wcount[i];
        }
        if (kind == 1) {
            __nv_bfloat16 *xr = S.x + slot * kMlpIn;
            for (int i = 0; i < kMlpIn; i += 2)
                *reinterpret_cast<uint32_t *>(xr + i) = pack_bf16(i < kMlpInUsed ? raw[i] : 0.f,
                                                                  i + 1 < kMlpInUsed ? raw[i + 1] : 0.f);
        }
        const int ntile = (nc + 15) >> 4;
        if (tid >= nc && tid < ntile * 16)      // zero rows that pad the last tile
            for (int i = 0; i < kMlpIn; i += 2) *reinterpret_cast<uint32_t *>(S.x + tid * kMlpIn + i) = 0u;
        if (nc > 0) {
            // the network's parameters, once per CTA that has candidates
            const uint4 *src = reinterpret_cast<const uint4 *>(net->w1);
            uint4 *dst = reinterpret_cast<uint4 *>(S.w1);
            constexpr int nvec = (int)(sizeof(S.w1) + sizeof(S.w2) + sizeof(S.w3)) / 16;
            for (int i = tid; i < nvec; i += kNnBlock) dst[i] = __ldg(src + i);
            for (int i = tid; i < kMlpHid; i += kNnBlock) {
                S.b1[i] = net->b1[i];
                S.b2[i] = net->b2[i];
            }
            if (tid < kMlpOut) S.b3[tid] = net->b3[tid];
        }
        __syncthreads();
        for (int t = w; t < ntile; t += kNnBlock / 32)
            mlp_forward16(S.x + t * 16 * kMlpIn, S.w1, S.w2, S.w3, S.b1, S.b2, S.b3, S.h1[w], S.h2[w],
                          S.y + t * 16 * kMlpOut);
        __syncthreads();

        // ---- judge the predictions ---------------------------------------
        if (kind == 1) {
            // R = a I + (b / D) n + (c / D) dev(n n), the return per unit
            // multiplier; sigma = trial - 2 G alam R
            const MixF &xf = F.mix[mixid];
            const float *yo = S.y + slot * kMlpOut;
            float nb[6], qb[6], lam[3], p[3];
            f_principal_values(s, 0.f, p);
            nn_basis(s, p, nb, qb, lam);
            const float D = nn_pole(lam);
            const float a = yo[0] * net->out_scale[0];
            const float b = yo[1] * net->out_scale[1] / D, c = yo[2] * net->out_scale[2] / D;
            const float g2 = 2.f * xf.shearm * cd.alam;
            for (int i = 0; i < 6; ++i) sp[i] = s[i] - g2 * ((i < 3 ? a : 0.f) + b * nb[i] + c * qb[i]);
            const float dp = fabsf(cd.alam) * yo[3] * net->out_scale[3];
            f_principal_values(sp, 0.f, p);
            const float r = p[0] - cd.anphi * p[2] + cd.cf - 2.f * sqrtf(cd.anphi) * cd.hardn * cd.alam;
            bool ok = fabsf(D) > 1e-4f && dp > 0.f && fabsf(r) <= tol * cd.S && p[2] + cd.ft_shift < 0.f;
            for (int i = 0; i < 6; ++i) ok = ok && isfinite(sp[i]);
            if (RHEOL == 7 && ok) {
                // the Maxwell/plastic choice of rheology.cxx:628-638 must be clear
                const float jv = second_invariant2(sv), jp = second_invariant2(sp);
                ok = fabsf(jv - jp) > tol * fmaxf(jv, jp);
            }
            if (ok)
                depls = dp;
            else
                kind = 2;
        }
        const unsigned amask = __ballot_sync(0xffffffffu, kind == 1);
        const unsigned xmask = __ballot_sync(0xffffffffu, kind == 2);
        if (lane == 0) {
            if (cmask) atomicAdd(&d.clk->nn_cand, (unsigned long long)__popc(cmask));
            if (amask) atomicAdd(&d.clk->nn_accept, (unsigned long long)__popc(amask));
            if (xmask) atomicAdd(&d.clk->fp64_returns, (unsigned long long)__popc(xmask));
        }

        // ---- exact FP64 return map for the compacted rest -----------------
        __syncthreads();     // every warp has read its wcount entry above
        if (lane == 0) S.wcount[w] = __popc(xmask);
        __syncthreads();
        int nx = 0, xslot = 0;
        for (int i = 0; i < kNnBlock / 32; ++i) {
            if (i == w) xslot = nx + __popc(xmask & ((1u << lane) - 1u));
            nx += S.wcount[i];
        }
        if (kind == 2) S.queue[xslot] = tid;
        __syncthreads();
        int flags = 0;
        if (tid < nx) {
            const int j = S.queue[tid];
            const int ej = blockIdx.x * kNnBlock + j;
            float sj[6], dej[6], out[6];
            for (int i = 0; i < 6; ++i) {
                sj[i] = S.so[i][j];
                dej[i] = S.de[i][j];
            }
            const Consts &K = *d.K;
            double dpj;
            flags = ep_fp64(K, K.M.mix[d.mix[ej]], d.pls[ej], d.s0[ej], sj, dej, out, dpj);
            for (int i = 0; i < 6; ++i) S.res[i][j] = out[i];
            S.resd[j] = dpj;
        }
        __syncthreads();
        unsigned solved = __ballot_sync(0xffffffffu, flags & 1), ql = __ballot_sync(0xffffffffu, flags & 2);
        if (lane == 0) {
            if (solved) atomicAdd(&d.clk->eig, (unsigned long long)__popc(solved));
            if (ql) atomicAdd(&d.clk->ql, (unsigned long long)__popc(ql));
        }
    }
    if (!live) return;

    // ---- results -------------------------------------------------------------
    if (kind == 2) {
        for (int i = 0; i < 6; ++i) sp[i] = S.res[i][tid];
        depls = S.resd[tid];
    } else if (kind == 0) {
        for (int i = 0; i < 6; ++i) sp[i] = s[i];
        depls = 0.0;
    }
    bool plastic = true;
    if (RHEOL == 7) {
        if (kind == 1)
            plastic = second_invariant2(sv) >= second_invariant2(sp);
        else
            plastic = !f_viscous_wins(F.mix[mixid], so, de, sv, sp, depls, dt, visc);
    }
    if (plastic) {
        for (int i = 0; i < 6; ++i) s[i] = sp[i];
        pls += depls;
        dpls = (float)depls;
    } else {
        for (int i = 0; i < 6; ++i) s[i] = sv[i];
    }
    float dpv = tr3(s) - tr3(so);
    f_store6(d.stress, E, e, s);
    d.pls[e] = pls;
    d.dpls[e] = dpls;
    d.dp[e] = dpv;
    d.tmp_sg[e] = dpv * d.c_vol[e];
}

}  // namespace des
