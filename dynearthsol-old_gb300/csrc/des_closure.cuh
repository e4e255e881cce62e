// The FP32 form's elasto-(visco-)plastic stress pass (E-B) and the learned
// return-map closure inside it.
//
// For the elasto-plastic rheologies the reference computes the principal
// stresses of the elastic trial with dsyevh3 and returns the trial to the
// Mohr-Coulomb surface (rheology.cxx:180-240); the FP32 form does that in
// FP64 for every element the cheap elastic bounds cannot clear.  Those
// elements are listed (E-B1) and returned by a dense pass (E-B3).  With a
// closure set, a pass in between (E-B2) sorts the listed elements:
//
//   network candidates  the FP32 principal values of the trial say "shear
//                       return, clearly": fs < -tol S and h < -tol S
//   exact               everything else (near the yield surface, the tensile
//                       or corner branches, inputs outside the training
//                       envelope)
//
// Candidates are packed into 16-row tiles and evaluated by the MLP on the
// tensor cores.  Each prediction is then judged in FP32: the predicted
// stress must lie on the yield surface, |fs(sigma) - 2 sqrt(anphi) hardn
// alam| <= tol S (the hardening term is the residual the reference's own
// return leaves), inside the tensile cutoff, with a positive plastic-strain
// increment; for rh_evp the Maxwell/plastic choice must also be clear.
// Rejected candidates join the exact list.
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

// ---- the elasto-(visco-)plastic stress pass as three dense kernels -------
//
// E-B1 (kf_fe_b_ep) corrects the strain rate, updates the strain and forms
// the elastic trial of every element, and finishes every element the FP32
// bounds prove elastic; each other element goes to the pending list.  With a
// closure, E-B2 (kf_nn_list) takes the pending list 32 entries per warp,
// evaluates the network on the candidates among them in full 16-row tiles
// (the weights staged once per CTA) and judges each prediction; the rest join
// the exact list.  E-B3 (kf_exact_list) runs the FP64 return map on the
// pending list (no closure) or the exact list, with every lane busy.  The
// later kernels recompute an element's trial from what E-B1 left (the old
// stress still in place, the corrected strain rate in srate) with the same
// FP32 arithmetic, so the result does not depend on which kernel finishes an
// element.

// one element's stress-update inputs
struct FTrial {
    float so[6], de[6], s[6], sv[6];   // old stress, increment, elastic trial, Maxwell stress (rh_evp)
    float visc, dt;
    double pls, s0;
    int4 c;
    int mix;
};

template <int RHEOL>
__device__ __forceinline__ void f_trial_from_state(const DevF &d, int e, FTrial &q)
{
    const size_t E = d.nelem;
    const ConstsF &F = *d.F;
    q.c = d.conn[e];
    q.mix = d.mix[e];
    const MixF &xf = F.mix[q.mix];
    float edot[6];
    f_load6(d.stress, E, e, q.so);
    f_load6(d.srate, E, e, edot);
    q.pls = d.pls[e];
    q.s0 = d.s0[e];
    q.dt = (float)d.clk->dt;
    for (int i = 0; i < 6; ++i) {
        q.de[i] = edot[i] * q.dt;
        q.s[i] = q.so[i];
    }
    elastic(xf.bulkm, xf.shearm, q.de, q.s);
    q.visc = 0.f;
    if (RHEOL == 7) {
        q.visc = f_visc(F, xf, f_elem_T(d, q.c), edot);
        const float dv = (float)(d.vol[e] / d.vol_old[e] - 1);
        for (int i = 0; i < 6; ++i) q.sv[i] = q.so[i];
        maxwell(xf.bulkm, xf.shearm, q.visc, q.dt, dv, q.de, q.sv);
    }
}

// the element's new stress from the plastic candidate sp (rheology.cxx:578-598,
// 628-638 for rh_evp), plastic strain, dpressure and its volume-weighted share
template <int RHEOL>
__device__ __forceinline__ void f_finish(const DevF &d, int e, const FTrial &q, const float sp[6], double depls,
                                         bool from_network)
{
    const size_t E = d.nelem;
    bool plastic = true;
    if (RHEOL == 7) {
        plastic = from_network ? second_invariant2(q.sv) >= second_invariant2(sp)
                               : !f_viscous_wins(d.F->mix[q.mix], q.so, q.de, q.sv, sp, depls, q.dt, q.visc);
    }
    float s[6];
    if (plastic) {
        for (int i = 0; i < 6; ++i) s[i] = sp[i];
        d.pls[e] = q.pls + depls;
        d.dpls[e] = (float)depls;
    } else {
        for (int i = 0; i < 6; ++i) s[i] = q.sv[i];
    }
    const float dpv = tr3(s) - tr3(q.so);
    f_store6(d.stress, E, e, s);
    d.dp[e] = dpv;
    d.tmp_sg[e] = dpv * d.c_vol[e];
}

// appends e (where take) to list with one atomic per warp; every lane of the
// warp calls it
__device__ __forceinline__ void list_append(unsigned *count, int *list, bool take, int e)
{
    const unsigned m = __ballot_sync(0xffffffffu, take);
    if (!m) return;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    unsigned base = 0;
    if (lane == leader) base = atomicAdd(count, (unsigned)__popc(m));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (take) list[base + __popc(m & ((1u << lane) - 1u))] = e;
}

// E-B1, over the elements from e0 (a multiple of the block size); registers
// bounded for 12 blocks of 128 per SM (E-B1 0.331 -> 0.317 ms on config 2)
template <int RHEOL>
__global__ void __launch_bounds__(128, 12) kf_fe_b_ep(DevF d, int e0)
{
    const int e = e0 + gtid();
    if (e == 0) d.clk->mass_valid = 1;
    const bool live = e < d.nelem;
    bool pending = false;
    if (live) {
        const size_t E = d.nelem;
        const ConstsF &F = *d.F;
        const int4 c = d.conn[e];
        const MixF &xf = F.mix[d.mix[e]];
        const float edv = (d.ntmp[c.x] + d.ntmp[c.y] + d.ntmp[c.z] + d.ntmp[c.w]) * 0.25f;
        d.edvoldt[e] = edv;
        float so[6], es[6], edot[6];
        f_load6(d.stress, E, e, so);
        f_load6(d.strain, E, e, es);
        f_load6(d.srate_next, E, e, edot);
        const float dt = (float)d.clk->dt;
        const float div = tr3(edot);
        for (int i = 0; i < 3; ++i) edot[i] += (edv - div) * (1.f / 3.f);
        float de[6], st[6];
        for (int i = 0; i < 6; ++i) {
            es[i] += edot[i] * dt;
            de[i] = edot[i] * dt;
            st[i] = so[i];
        }
        f_store6(d.strain, E, e, es);
        f_store6(d.srate, E, e, edot);
        elastic(xf.bulkm, xf.shearm, de, st);
        const float s0f = (float)d.s0[e];
        float amc, anphi, ten_max;
        f_plastic_props(F, xf, (float)d.pls[e], amc, anphi, ten_max);
        bool clear = f_surely_elastic(st, s0f, anphi, amc, ten_max);
        if (!clear) {
            float p[3];
            f_principal_values(st, 0.f, p);
            clear = f_clearly_elastic(p, s0f, anphi, amc, ten_max);
        }
        if (clear) {
            float s[6];
            bool plastic = true;
            if (RHEOL == 7) {
                const float visc = f_visc(F, xf, f_elem_T(d, c), edot);
                const float dv = (float)(d.vol[e] / d.vol_old[e] - 1);
                float sv[6];
                for (int i = 0; i < 6; ++i) sv[i] = so[i];
                maxwell(xf.bulkm, xf.shearm, visc, dt, dv, de, sv);
                if (f_viscous_wins(xf, so, de, sv, st, 0.0, dt, visc)) {
                    plastic = false;
                    for (int i = 0; i < 6; ++i) s[i] = sv[i];
                }
            }
            if (plastic) {
                for (int i = 0; i < 6; ++i) s[i] = st[i];
                d.dpls[e] = 0.f;
            }
            const float dpv = tr3(s) - tr3(so);
            f_store6(d.stress, E, e, s);
            d.dp[e] = dpv;
            d.tmp_sg[e] = dpv * d.c_vol[e];
        } else {
            pending = true;
        }
    }
    list_append(&d.clk->npend, d.pend, pending, e);
}

constexpr int kNnListBlock = 128;

struct NnListSmem {
    __nv_bfloat16 w1[kMlpHid * kMlpIn], w2[kMlpHid * kMlpHid], w3[kMlpOut * kMlpHid];
    float b1[kMlpHid], b2[kMlpHid], b3[kMlpOut];
    __nv_bfloat16 x[kNnListBlock / 32][32 * kMlpIn];       // two 16-row tiles per warp
    __nv_bfloat16 h1[kNnListBlock / 32][16 * kHStride], h2[kNnListBlock / 32][16 * kHStride];
    float y[kNnListBlock / 32][32 * kMlpOut];
};

// E-B2
template <int RHEOL>
__global__ void __launch_bounds__(kNnListBlock) kf_nn_list(DevF d, const MlpDev *__restrict__ net)
{
    const unsigned npend = d.clk->npend;
    if (npend == 0) return;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    NnListSmem &S = *reinterpret_cast<NnListSmem *>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    {
        const uint4 *src = reinterpret_cast<const uint4 *>(net->w1);
        uint4 *dst = reinterpret_cast<uint4 *>(S.w1);
        constexpr int nvec = (int)(sizeof(S.w1) + sizeof(S.w2) + sizeof(S.w3)) / 16;
        for (int i = tid; i < nvec; i += kNnListBlock) dst[i] = __ldg(src + i);
        for (int i = tid; i < kMlpHid; i += kNnListBlock) {
            S.b1[i] = net->b1[i];
            S.b2[i] = net->b2[i];
        }
        if (tid < kMlpOut) S.b3[tid] = net->b3[tid];
    }
    __syncthreads();
    const ConstsF &F = *d.F;
    const float tol = net->tol;
    float pls_sat = 0.f;       // past the largest pls1 the plastic properties no longer change
    for (int m = 0; m < F.nmat; ++m) pls_sat = fmaxf(pls_sat, F.pls1[m]);
    unsigned long long ncand = 0, naccept = 0;
    const unsigned nwarp = gridDim.x * (kNnListBlock / 32);
    for (unsigned base = (blockIdx.x * (kNnListBlock / 32) + w) * 32u; base < npend; base += nwarp * 32u) {
        const unsigned j = base + lane;
        const bool valid = j < npend;
        const int e = valid ? d.pend[j] : 0;
        FTrial q;
        NnCand cd = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        float raw[kMlpIn];
        bool cand = false;
        if (valid) {
            f_trial_from_state<RHEOL>(d, e, q);
            const MixF &xf = F.mix[q.mix];
            const float plsf = (float)q.pls, s0f = (float)q.s0;
            float amc, anphi, anpsi, hardn, ten_max, p[3];
            f_principal_values(q.s, 0.f, p);
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
            float nb[6], qb[6], lam[3];
            if (fs < -tol * cd.S && h < -tol * cd.S && nn_basis(q.s, p, nb, qb, lam)) {
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
                    cand = true;
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
        }
        // the candidates of this warp, packed into one or two 16-row tiles
        const unsigned cm = __ballot_sync(0xffffffffu, cand);
        const int nc = __popc(cm), slot = __popc(cm & ((1u << lane) - 1u));
        const int ntile = (nc + 15) >> 4;
        __nv_bfloat16 *X = S.x[w];
        if (cand)
            for (int i = 0; i < kMlpIn; i += 2)
                *reinterpret_cast<uint32_t *>(X + slot * kMlpIn + i) =
                    pack_bf16(i < kMlpInUsed ? raw[i] : 0.f, i + 1 < kMlpInUsed ? raw[i + 1] : 0.f);
        if (lane >= nc && lane < ntile * 16)      // rows that pad the last tile
            for (int i = 0; i < kMlpIn; i += 2) *reinterpret_cast<uint32_t *>(X + lane * kMlpIn + i) = 0u;
        __syncwarp();
        for (int t = 0; t < ntile; ++t)
            mlp_forward16(X + t * 16 * kMlpIn, S.w1, S.w2, S.w3, S.b1, S.b2, S.b3, S.h1[w], S.h2[w],
                          S.y[w] + t * 16 * kMlpOut);
        __syncwarp();
        bool accepted = false;
        if (cand) {
            // R = a I + (b / D) n + (c / D) dev(n n), the return per unit
            // multiplier; sigma = trial - 2 G alam R
            const MixF &xf = F.mix[q.mix];
            const float *yo = S.y[w] + slot * kMlpOut;
            float nb[6], qb[6], lam[3], p[3], sp[6];
            f_principal_values(q.s, 0.f, p);
            nn_basis(q.s, p, nb, qb, lam);
            const float D = nn_pole(lam);
            const float a = yo[0] * net->out_scale[0];
            const float b = yo[1] * net->out_scale[1] / D, c = yo[2] * net->out_scale[2] / D;
            const float g2 = 2.f * xf.shearm * cd.alam;
            for (int i = 0; i < 6; ++i) sp[i] = q.s[i] - g2 * ((i < 3 ? a : 0.f) + b * nb[i] + c * qb[i]);
            const float dpl = fabsf(cd.alam) * yo[3] * net->out_scale[3];
            f_principal_values(sp, 0.f, p);
            const float r = p[0] - cd.anphi * p[2] + cd.cf - 2.f * sqrtf(cd.anphi) * cd.hardn * cd.alam;
            bool ok = fabsf(D) > 1e-4f && dpl > 0.f && fabsf(r) <= tol * cd.S && p[2] + cd.ft_shift < 0.f;
            for (int i = 0; i < 6; ++i) ok = ok && isfinite(sp[i]);
            if (RHEOL == 7 && ok) {
                // the Maxwell/plastic choice of rheology.cxx:628-638 must be clear
                const float jv = second_invariant2(q.sv), jp = second_invariant2(sp);
                ok = fabsf(jv - jp) > tol * fmaxf(jv, jp);
            }
            if (ok) {
                accepted = true;
                f_finish<RHEOL>(d, e, q, sp, dpl, true);
            }
        }
        ncand += nc;
        naccept += __popc(__ballot_sync(0xffffffffu, accepted));
        list_append(&d.clk->nexact, d.exact, valid && !accepted, e);
        __syncwarp();      // the tile buffers are reused by the next round
    }
    if (lane == 0) {
        if (ncand) atomicAdd(&d.clk->nn_cand, ncand);
        if (naccept) atomicAdd(&d.clk->nn_accept, naccept);
    }
}

// E-B3: the exact FP64 return map over a list
template <int RHEOL>
__global__ void kf_exact_list(DevF d, int from_pending)
{
    const unsigned n = from_pending ? d.clk->npend : d.clk->nexact;
    const int *list = from_pending ? d.pend : d.exact;
    unsigned nsolved = 0, nql = 0, nret = 0;
    for (unsigned j = gtid(); j < n; j += gridDim.x * blockDim.x) {
        const int e = list[j];
        FTrial q;
        f_trial_from_state<RHEOL>(d, e, q);
        const Consts &K = *d.K;
        float sp[6];
        double depls;
        const int flags = ep_fp64(K, K.M.mix[q.mix], q.pls, q.s0, q.so, q.de, sp, depls);
        f_finish<RHEOL>(d, e, q, sp, depls, false);
        nsolved += (flags & 1) ? 1u : 0u;
        nql += (flags & 2) ? 1u : 0u;
        ++nret;
    }
    for (int o = 16; o > 0; o >>= 1) {
        nsolved += __shfl_down_sync(0xffffffffu, nsolved, o);
        nql += __shfl_down_sync(0xffffffffu, nql, o);
        nret += __shfl_down_sync(0xffffffffu, nret, o);
    }
    if ((threadIdx.x & 31) == 0) {
        if (nsolved) atomicAdd(&d.clk->eig, (unsigned long long)nsolved);
        if (nql) atomicAdd(&d.clk->ql, (unsigned long long)nql);
        if (nret) atomicAdd(&d.clk->fp64_returns, (unsigned long long)nret);
    }
}

}  // namespace des
