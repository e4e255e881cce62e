// C ABI of the GB300 time-step library: device state, upload/download, the
// per-function entry points and the captured whole-step graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <new>
#include <vector>

#include "des_gpu.h"
#include "des_closure.cuh"
#include "des_support.cuh"
#include "des_topology.h"

using namespace des;

namespace {

const int kElemBlock = 128;
const int kNodeBlock = 256;
const int kStepKernels = 6;
const int kEaChunks = 8;   // E-A launches of the host-buffer step (downloads overlap them)
const int kEbChunks = 8;   // E-B launches of the host-buffer step (its inputs come up chunk by chunk)

inline int blocks(long long n, int b) { return (int)((n + b - 1) / b); }

}  // namespace

struct des_gpu {
    int device = 0;
    int sms = 1;                          // multiprocessors of the device
    cudaStream_t stream = nullptr;
    int nnode = 0, nelem = 0, nmat = 0;
    des_params P;
    Consts hK;
    std::vector<std::vector<int>> mix_counts;
    Dev d;
    Consts *dK = nullptr;
    Clock *dclk = nullptr;
    std::vector<void *> allocs;
    long long bytes = 0;
    double *staging = nullptr;
    long long staging_elems = 0;
    cudaGraphExec_t graph = nullptr;
    bool primed = false;
    int prec = DES_PREC_FP64;
    DevF f;
    ConstsF hF;
    ConstsF *dF = nullptr;
    bool stress_bcs = false;
    int bfacets_count[DES_NBDRY] = {0};
    MlpDev *dnet = nullptr;      // the learned closure (FP32 form), when set
    bool closure = false;
    unsigned long long *qout = nullptr;   // mesh-quality reductions
    // output snapshot: the selected fields as FP64 AoS rows in device memory,
    // copied to the host on their own stream while the steps go on
    double *snap = nullptr;
    long long snap_bytes = 0;
    unsigned snap_mask = 0;
    Clock *snap_clk = nullptr;
    cudaStream_t copy_stream = nullptr;
    double *dl = nullptr;                 // host-layout rows of an overlapped download
    long long dl_elems = 0;
    cudaEvent_t head_done = nullptr;      // a step's passes before E-A are done
    cudaEvent_t up_done = nullptr;        // the copy stream's uploads are done
    // host-to-device copies of the host-buffer step, on their own stream so
    // that they run beside the device-to-host copies of the copy stream;
    // one event per element chunk
    cudaStream_t up_stream = nullptr;
    cudaEvent_t up_chunk[kEbChunks] = {};
    cudaEvent_t snap_ready = nullptr, snap_done = nullptr;
    int avg_interval = 0;                 // Output::average_fields every step when > 0
    double *avg_c0 = nullptr, *avg_strain0 = nullptr, *avg_stress = nullptr, *avg_dpls = nullptr,
           *avg_time0 = nullptr;
};

namespace {

int cuda_rc(cudaError_t e) { return e == cudaSuccess ? DES_OK : DES_ERR_CUDA; }
#define DES_CUDA(call)                          \
    do {                                        \
        cudaError_t _e = (call);                \
        if (_e != cudaSuccess) return DES_ERR_CUDA; \
    } while (0)
#define DES_LAUNCH()                                        \
    do {                                                    \
        if (cudaGetLastError() != cudaSuccess) return DES_ERR_CUDA; \
    } while (0)

template <class T>
int dev_alloc(des_gpu *g, T **p, size_t n)
{
    void *q = nullptr;
    size_t bytes = sizeof(T) * (n ? n : 1);
    if (cudaMalloc(&q, bytes) != cudaSuccess) return DES_ERR_NOMEM;
    g->allocs.push_back(q);
    g->bytes += (long long)bytes;
    if (cudaMemset(q, 0, bytes) != cudaSuccess) return DES_ERR_CUDA;
    *p = static_cast<T *>(q);
    return DES_OK;
}

double mv(const des_matvec &v, int m) { return v.len == 1 ? v.v[0] : v.v[m]; }

// matprops.cxx:436-461
double arith_mean(const des_matvec &s, const std::vector<int> &n)
{
    if (s.len == 1) return s.v[0];
    double result = 0;
    int m = 0;
    for (int i = 0; i < s.len; i++) {
        result += n[i] * s.v[i];
        m += n[i];
    }
    return result / m;
}
double harm_mean(const des_matvec &s, const std::vector<int> &n)
{
    if (s.len == 1) return s.v[0];
    double result = 0;
    int m = 0;
    for (int i = 0; i < s.len; i++) {
        result += n[i] / s.v[i];
        m += n[i];
    }
    return m / result;
}

int check_params(const des_params &p, int nmat)
{
    if (p.nmat != nmat || nmat < 1 || nmat > DES_MAX_MAT) return DES_ERR_ARG;
    if (p.is_plane_strain) return DES_ERR_UNSUPPORTED;
    // bc.cxx:765-777: 0 none, 1 diffusion, 101 the custom template
    if (p.surface_process_option != 0 && p.surface_process_option != 1 && p.surface_process_option != 101)
        return DES_ERR_OPTION;
    if (p.rheol_type != DES_RH_ELASTIC && p.rheol_type != DES_RH_VISCOUS &&
        p.rheol_type != DES_RH_MAXWELL && p.rheol_type != DES_RH_EP && p.rheol_type != DES_RH_EVP)
        return DES_ERR_OPTION;
    if (p.damping_option < 0 || p.damping_option > 4) return DES_ERR_OPTION;
    if (p.ref_pressure_option < 0 || p.ref_pressure_option > 2) return DES_ERR_OPTION;
    if (p.precision != DES_PREC_FP64 && p.precision != DES_PREC_FP32) return DES_ERR_UNSUPPORTED;
    const des_matvec *vs[] = {&p.rho0, &p.alpha, &p.bulk_modulus, &p.shear_modulus,
                              &p.visc_exponent, &p.visc_coefficient, &p.visc_activation_energy,
                              &p.heat_capacity, &p.therm_cond, &p.pls0, &p.pls1, &p.cohesion0,
                              &p.cohesion1, &p.friction_angle0, &p.friction_angle1,
                              &p.dilation_angle0, &p.dilation_angle1};
    for (const des_matvec *v : vs)
        if (!(v->len == nmat || (v->len == 1 && nmat != 1) || (v->len == 1 && nmat == 1)))
            return DES_ERR_TOPOLOGY;   // VectorBase::create rejects it (matprops.cxx:509-520)
    return DES_OK;
}

// The distinct marker-count vectors ("mixes") of elemmarkers [nelem][nmat]
// in order of first appearance, and the element -> mix map.  Every material
// property MatProps derives from an element's counts (matprops.cxx:193-331)
// is a function of its mix.
int build_mix(const int *elemmarkers, int nelem, int nmat, std::vector<std::vector<int>> &counts,
              std::vector<unsigned char> &mix)
{
    counts.clear();
    mix.assign((size_t)nelem, 0);
    std::map<std::vector<int>, int> ids;
    std::vector<int> prev, cur((size_t)nmat);
    int prev_id = -1;
    for (int e = 0; e < nelem; ++e) {
        const int *c = elemmarkers + (size_t)nmat * e;
        cur.assign(c, c + nmat);
        int n = 0;
        for (int k = 0; k < nmat; ++k) {
            if (cur[k] < 0) return DES_ERR_TOPOLOGY;
            n += cur[k];
        }
        if (n <= 0) return DES_ERR_TOPOLOGY;   // MarkerSet rejects an element without markers
        if (prev_id >= 0 && cur == prev) {
            mix[e] = (unsigned char)prev_id;
            continue;
        }
        auto it = ids.find(cur);
        int id;
        if (it == ids.end()) {
            id = (int)ids.size();
            if (id >= kMaxMix) return DES_ERR_SIZE;
            ids[cur] = id;
            counts.push_back(cur);
        } else {
            id = it->second;
        }
        mix[e] = (unsigned char)id;
        prev = cur;
        prev_id = id;
    }
    return DES_OK;
}

// Consts from params and the distinct marker-count vectors
int build_consts(des_gpu *g)
{
    const des_params &p = g->P;
    Consts &K = g->hK;
    std::memset(&K, 0, sizeof(K));
    MatTable &M = K.M;
    M.nmat = g->nmat;
    M.nmix = (int)g->mix_counts.size();
    const double gas_constant = 8.3144;
    for (int m = 0; m < g->nmat; ++m) {
        M.rho0[m] = mv(p.rho0, m);
        M.alpha[m] = mv(p.alpha, m);
        double ve = mv(p.visc_exponent, m);
        M.vexp_pw[m] = 1 / ve - 1;
        M.vexp_pw1[m] = -1 / ve;
        M.vcoef_pow[m] = std::pow(0.75 * mv(p.visc_coefficient, m), M.vexp_pw1[m]);
        M.vQ[m] = mv(p.visc_activation_energy, m);
        M.vnR[m] = ve * gas_constant;
        M.pls0[m] = mv(p.pls0, m);
        M.pls1[m] = mv(p.pls1, m);
        M.c0[m] = mv(p.cohesion0, m);
        M.c1[m] = mv(p.cohesion1, m);
        M.f0[m] = mv(p.friction_angle0, m);
        M.f1[m] = mv(p.friction_angle1, m);
        M.d0[m] = mv(p.dilation_angle0, m);
        M.d1[m] = mv(p.dilation_angle1, m);
        M.hslope[m] = (M.c1[m] - M.c0[m]) / (M.pls1[m] - M.pls0[m]);
    }
    const double deg2rad = 3.1415926535897932384626433832795 / 180;
    M.phi_c = M.f0[0];
    double sphi = std::sin(M.phi_c * deg2rad);
    M.sphi_c = sphi;
    M.anphi_c = (1 + sphi) / (1 - sphi);
    M.sqanphi_c = std::sqrt(M.anphi_c);
    M.tphi_c = std::tan(M.phi_c * deg2rad);
    M.psi_c = M.d0[0];
    double spsi = std::sin(M.psi_c * deg2rad);
    M.spsi_c = spsi;
    M.anpsi_c = (1 + spsi) / (1 - spsi);
    M.phi_w = M.f1[0];
    double sphi_w = std::sin(M.phi_w * deg2rad);
    M.anphi_w = (1 + sphi_w) / (1 - sphi_w);
    M.sqanphi_w = std::sqrt(M.anphi_w);
    M.tphi_w = std::tan(M.phi_w * deg2rad);
    M.psi_w = M.d1[0];
    double spsi_w = std::sin(M.psi_w * deg2rad);
    M.anpsi_w = (1 + spsi_w) / (1 - spsi_w);
    for (int m = 0; m < g->nmat; ++m) {
        M.pls0f[m] = (float)M.pls0[m];
        M.pls1f[m] = (float)M.pls1[m];
        M.c0f[m] = (float)M.c0[m];
        M.c1f[m] = (float)M.c1[m];
        M.f0f[m] = (float)M.f0[m];
        M.f1f[m] = (float)M.f1[m];
    }
    M.phi_cf = (float)M.phi_c;
    M.anphi_cf = (float)M.anphi_c;
    M.sqanphi_cf = (float)M.sqanphi_c;
    M.tphi_cf = (float)M.tphi_c;
    M.phi_wf = (float)M.phi_w;
    M.anphi_wf = (float)M.anphi_w;
    M.sqanphi_wf = (float)M.sqanphi_w;
    M.tphi_wf = (float)M.tphi_w;
    M.visc_min = p.visc_min;
    M.visc_max = p.visc_max;
    M.tension_max = p.tension_max;
    M.tension_maxf = (float)p.tension_max;
    double pseudo_speed = p.max_vbc_val * p.inertial_scaling;
    for (int i = 0; i < M.nmix; ++i) {
        const std::vector<int> &cnt = g->mix_counts[i];
        Mix &x = M.mix[i];
        x.bulkm = harm_mean(p.bulk_modulus, cnt);
        x.shearm = harm_mean(p.shear_modulus, cnt);
        x.cp = arith_mean(p.heat_capacity, cnt);
        x.k = arith_mean(p.therm_cond, cnt);
        x.rho_qs = x.bulkm / (pseudo_speed * pseudo_speed);
        x.dt_maxwell = 0.5 * p.visc_min / (1e-40 + x.shearm);
        int n = 0, nonzero = 0, which = -1;
        for (int m = 0; m < g->nmat; ++m) {
            x.count[m] = cnt[m];
            n += cnt[m];
            if (cnt[m] != 0) {
                ++nonzero;
                which = m;
            }
        }
        x.n = n;
        bool pow2 = which >= 0 && (cnt[which] & (cnt[which] - 1)) == 0;
        x.single = (nonzero == 1 && pow2) ? which : -1;
    }
    K.gravity = p.gravity;
    K.damping_factor = p.damping_factor;
    K.surface_temperature = p.surface_temperature;
    K.dt_fraction = p.dt_fraction;
    K.fixed_dt = p.fixed_dt;
    K.inertial_scaling = p.inertial_scaling;
    K.max_vbc_val = p.max_vbc_val;
    K.therm_diff_max = p.therm_diff_max;
    K.zlength = p.zlength;
    K.rho0_0 = p.rho0.v[0];
    K.compensation_pressure = p.compensation_pressure;
    K.damping_option = p.damping_option;
    K.is_qs = p.is_quasi_static ? 1 : 0;
    K.thermal = p.has_thermal_diffusion ? 1 : 0;
    K.rheol = p.rheol_type;
    for (int i = 0; i < DES_NBDRY; ++i) {
        K.vbc_types[i] = p.vbc_types[i];
        K.vbc_values[i] = p.vbc_values[i];
        for (int k = 0; k < 3; ++k) K.bnormals[i][k] = p.bnormals[i][k];
        for (int j = 0; j < DES_NBDRY; ++j)
            for (int k = 0; k < 3; ++k) K.edge[i][j][k] = p.edge_vectors[i][j][k];
    }
    // apply_stress_bcs (bc.cxx:503-595): the sides whose facets carry a
    // traction, and the elastic foundation (both only with gravity)
    K.stress_bc_sides = 0;
    if (p.gravity != 0) {
        for (int i = 0; i < DES_NBDRY; ++i) {
            int t = p.vbc_types[i];
            if (t != 0 && t != 2 && t != 4) continue;
            if (i == 4 && !p.has_winkler_foundation) continue;
            if (i == 5 && !p.has_water_loading) continue;
            if (g->bfacets_count[i] > 0) K.stress_bc_sides |= 1u << i;
        }
    }
    K.elastic_foundation = (p.gravity != 0 && p.has_elastic_foundation) ? 1 : 0;
    K.elastic_foundation_constant = p.elastic_foundation_constant;
    K.winkler_delta_rho = p.winkler_delta_rho;
    K.surface_process_option = p.surface_process_option;
    K.ref_pressure_option = p.ref_pressure_option;
    K.surface_diffusivity = p.surface_diffusivity;
    g->stress_bcs = K.stress_bc_sides != 0 || K.elastic_foundation;
    if (cudaMemcpyAsync(g->dK, &g->hK, sizeof(Consts), cudaMemcpyHostToDevice, g->stream) !=
        cudaSuccess)
        return DES_ERR_CUDA;
    if (g->dF) {
        ConstsF &F = g->hF;
        std::memset(&F, 0, sizeof(F));
        F.nmat = M.nmat;
        F.nmix = M.nmix;
        for (int i = 0; i < M.nmix; ++i) {
            const Mix &x = M.mix[i];
            MixF &y = F.mix[i];
            y.bulkm = (float)x.bulkm;
            y.shearm = (float)x.shearm;
            y.cp = (float)x.cp;
            y.k = (float)x.k;
            y.rho_qs = (float)x.rho_qs;
            double rr = 0, ra = 0;
            int nn = 0;
            for (int m = 0; m < M.nmat; ++m) {
                rr += M.rho0[m] * x.count[m];
                ra += M.rho0[m] * M.alpha[m] * x.count[m];
                nn += x.count[m];
            }
            y.rho_ref = rr / nn;
            y.rho_g4 = y.rho_ref * p.gravity / 4;
            y.rho_alpha = (float)(ra / nn);
            y.single = x.single;
            y.n = x.n;
            for (int m = 0; m < kMaxMat; ++m) y.count[m] = x.count[m];
        }
        for (int m = 0; m < M.nmat; ++m) {
            F.rho0[m] = (float)M.rho0[m];
            F.alpha[m] = (float)M.alpha[m];
            F.vexp_pw[m] = (float)M.vexp_pw[m];
            F.vlog_coef[m] = (float)std::log(0.25 * M.vcoef_pow[m] * 1e6);
            F.vQ[m] = (float)M.vQ[m];
            F.vnR[m] = (float)M.vnR[m];
            F.pls0[m] = (float)M.pls0[m];
            F.pls1[m] = (float)M.pls1[m];
            F.c0[m] = (float)M.c0[m];
            F.c1[m] = (float)M.c1[m];
            F.f0[m] = (float)M.f0[m];
            F.f1[m] = (float)M.f1[m];
            F.d0[m] = (float)M.d0[m];
            F.d1[m] = (float)M.d1[m];
            F.hslope[m] = (float)M.hslope[m];
        }
        F.phi_c = (float)M.phi_c;
        F.anphi_c = (float)M.anphi_c;
        F.sqanphi_c = (float)M.sqanphi_c;
        F.tphi_c = (float)M.tphi_c;
        F.psi_c = (float)M.psi_c;
        F.anpsi_c = (float)M.anpsi_c;
        F.visc_min = (float)M.visc_min;
        F.visc_max = (float)M.visc_max;
        F.tension_max = (float)M.tension_max;
        F.gravity = (float)p.gravity;
        F.surface_temperature = (float)p.surface_temperature;
        F.therm_diff_max = (float)p.therm_diff_max;
        F.rheol = p.rheol_type;
        F.thermal = K.thermal;
        F.is_qs = K.is_qs;
        if (cudaMemcpyAsync(g->dF, &g->hF, sizeof(ConstsF), cudaMemcpyHostToDevice, g->stream) !=
            cudaSuccess)
            return DES_ERR_CUDA;
    }
    return cudaStreamSynchronize(g->stream) == cudaSuccess ? DES_OK : DES_ERR_CUDA;
}

// ---- host <-> device field transfers --------------------------------------
// Page-locked host arrays (des_host_register, cudaHostAlloc) are reachable from
// the GPU (on GB300 over NVLink-C2C): uploads read the host rows in place, in
// one pass with the layout change (as fast as the copy engine, ~200 GB/s
// here).  Downloads go through the staging buffer and the copy engine, which
// writes host memory faster (~190 GB/s) than kernel stores (~150 GB/s); other
// host memory goes through the staging buffer both ways.
const void *mapped(const void *host)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, host) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (a.type == cudaMemoryTypeHost) ? a.devicePointer : nullptr;
}

int upload_field(des_gpu *g, const double *host, double *dst, int ncomp, long long rows)
{
    if (!host) return DES_ERR_ARG;
    if (const double *m = static_cast<const double *>(mapped(host))) {
        k_aos_to_soa<<<blocks(rows * ncomp, 256), 256, 0, g->stream>>>(m, dst, ncomp, rows, 0, rows);
        DES_LAUNCH();
        return DES_OK;
    }
    long long chunk_rows = std::max(1LL, g->staging_elems / ncomp);
    for (long long r0 = 0; r0 < rows; r0 += chunk_rows) {
        long long nr = std::min(chunk_rows, rows - r0);
        DES_CUDA(cudaMemcpyAsync(g->staging, host + r0 * ncomp, sizeof(double) * nr * ncomp,
                                 cudaMemcpyHostToDevice, g->stream));
        k_aos_to_soa<<<blocks(nr * ncomp, 256), 256, 0, g->stream>>>(g->staging, dst, ncomp, nr, r0,
                                                                       rows);
        DES_LAUNCH();
    }
    return DES_OK;
}
// device SoA -> host rows through the staging buffer stg, on stream st
int download_field(des_gpu *g, double *host, const double *src, int ncomp, long long rows,
                   cudaStream_t st, double *stg)
{
    if (!host) return DES_ERR_ARG;
    long long chunk_rows = std::max(1LL, g->staging_elems / ncomp);
    for (long long r0 = 0; r0 < rows; r0 += chunk_rows) {
        long long nr = std::min(chunk_rows, rows - r0);
        k_soa_to_aos<<<blocks(nr * ncomp, 256), 256, 0, st>>>(src, stg, ncomp, nr, r0, rows);
        DES_LAUNCH();
        DES_CUDA(cudaMemcpyAsync(host + r0 * ncomp, stg, sizeof(double) * nr * ncomp,
                                 cudaMemcpyDeviceToHost, st));
    }
    return DES_OK;
}

int upload_field(des_gpu *g, const double *host, float *dst, int ncomp, long long rows)
{
    if (!host) return DES_ERR_ARG;
    if (const double *m = static_cast<const double *>(mapped(host))) {
        k_aos_to_soa_f<<<blocks(rows * ncomp, 256), 256, 0, g->stream>>>(m, dst, ncomp, rows, 0, rows);
        DES_LAUNCH();
        return DES_OK;
    }
    long long chunk_rows = std::max(1LL, g->staging_elems / ncomp);
    for (long long r0 = 0; r0 < rows; r0 += chunk_rows) {
        long long nr = std::min(chunk_rows, rows - r0);
        DES_CUDA(cudaMemcpyAsync(g->staging, host + r0 * ncomp, sizeof(double) * nr * ncomp,
                                 cudaMemcpyHostToDevice, g->stream));
        k_aos_to_soa_f<<<blocks(nr * ncomp, 256), 256, 0, g->stream>>>(g->staging, dst, ncomp, nr,
                                                                         r0, rows);
        DES_LAUNCH();
    }
    return DES_OK;
}
int read_clock(des_gpu *g, Clock &c)
{
    DES_CUDA(cudaMemcpyAsync(&c, g->dclk, sizeof(Clock), cudaMemcpyDeviceToHost, g->stream));
    DES_CUDA(cudaStreamSynchronize(g->stream));
    return DES_OK;
}

// nodal masses current and fused-pass priming invalidated before a
// per-function call
int begin_fn(des_gpu *g)
{
    if (!g) return DES_ERR_ARG;
    Clock c;
    int rc = read_clock(g, c);
    if (rc) return rc;
    if (!c.mass_valid) {
        if (g->prec == DES_PREC_FP32)
            kf_mass_flush<<<blocks(g->nnode, kNodeBlock), kNodeBlock, 0, g->stream>>>(g->f);
        else
            k_mass_flush<<<blocks(g->nnode, kNodeBlock), kNodeBlock, 0, g->stream>>>(g->d);
        DES_LAUNCH();
    }
    g->primed = false;
    return DES_OK;
}

// the per-function entry points operate on the FP64 form's fields
int begin_fn64(des_gpu *g)
{
    if (!g) return DES_ERR_ARG;
    if (g->prec != DES_PREC_FP64) return DES_ERR_UNSUPPORTED;
    return begin_fn(g);
}

int prime(des_gpu *g)
{
    if (g->primed) return DES_OK;
    if (g->prec == DES_PREC_FP32)
        kf_prime<<<blocks(g->nelem, kElemBlock), kElemBlock, 0, g->stream>>>(g->f);
    else
        k_prime<<<blocks(g->nelem, kElemBlock), kElemBlock, 0, g->stream>>>(g->d);
    DES_LAUNCH();
    g->primed = true;
    return DES_OK;
}

// surface_processes (bc.cxx:760-782), after update_coordinate
void launch_surface(des_gpu *g)
{
    const int opt = g->P.surface_process_option;
    if (opt == 0) return;
    if (opt == 1 && g->d.bf.nbf > 0)
        k_surface_facets<<<blocks(g->d.bf.nbf, 128), 128, 0, g->stream>>>(g->d);
    k_surface_nodes<<<blocks(g->nnode, kNodeBlock), kNodeBlock, 0, g->stream>>>(g->d);
}

// the first kernel of pass E-B over the element blocks [b0, b1)
void launch_eb_first(des_gpu *g, int b0, int b1)
{
    cudaStream_t st = g->stream;
    const int n = b1 - b0, e0 = b0 * kElemBlock;
    if (g->prec == DES_PREC_FP32) {
        if (g->hF.rheol == 7)
            kf_fe_b_ep<7><<<n, kElemBlock, 0, st>>>(g->f, e0);
        else if (g->hF.rheol == 5)
            kf_fe_b_ep<5><<<n, kElemBlock, 0, st>>>(g->f, e0);
        else
            kf_fe_b<<<n, kElemBlock, 0, st>>>(g->f, e0);
    } else if (g->d.ret_log) {
        k_fe_b_t<true><<<n, kElemBlock, 0, st>>>(g->d, e0);
    } else {
        k_fe_b_t<false><<<n, kElemBlock, 0, st>>>(g->d, e0);
    }
}

// the rest of pass E-B once its first kernel has covered every element: in
// the FP32 form with rh_ep / rh_evp, the network (with a closure) and the
// exact return map, each over the dense list the first kernel left
void launch_eb_rest(des_gpu *g)
{
    if (g->prec != DES_PREC_FP32 || (g->hF.rheol != 5 && g->hF.rheol != 7)) return;
    cudaStream_t st = g->stream;
    const DevF &f = g->f;
    const int nn_grid = 4 * g->sms, exact_grid = 8 * g->sms;
    if (g->hF.rheol == 7) {
        if (g->closure) kf_nn_list<7><<<nn_grid, kNnListBlock, sizeof(NnListSmem), st>>>(f, g->dnet);
        kf_exact_list<7><<<exact_grid, 128, 0, st>>>(f, g->closure ? 0 : 1);
    } else {
        if (g->closure) kf_nn_list<5><<<nn_grid, kNnListBlock, sizeof(NnListSmem), st>>>(f, g->dnet);
        kf_exact_list<5><<<exact_grid, 128, 0, st>>>(f, g->closure ? 0 : 1);
    }
}

// pass k of N-A, E-B, N-B, E-C, N-C (0..4) of one step
void launch_pass(des_gpu *g, int k)
{
    const int nb = blocks(g->nnode, kNodeBlock), eb = blocks(g->nelem, kElemBlock);
    cudaStream_t st = g->stream;
    if (k == 1) {
        launch_eb_first(g, 0, eb);
        launch_eb_rest(g);
        return;
    }
    if (g->prec == DES_PREC_FP32) {
        const DevF &f = g->f;
        switch (k) {
        case 0: kf_fn_a<<<nb, kNodeBlock, 0, st>>>(f); break;
        case 2: kf_sg_gather<<<nb, kNodeBlock, 0, st>>>(f); break;
        case 3: kf_fe_c<<<eb, kElemBlock, 0, st>>>(f); break;
        default:
            if (g->hK.stress_bc_sides && g->d.bf.nbf > 0)
                k_stress_bc_facets<<<blocks(g->d.bf.nbf, 128), 128, 0, st>>>(g->d);
            kf_fn_c<<<nb, kNodeBlock, 0, st>>>(f);
            launch_surface(g);
            break;
        }
    } else {
        const Dev &d = g->d;
        switch (k) {
        case 0: k_fn_a<<<nb, kNodeBlock, 0, st>>>(d); break;
        case 2: k_sg_gather<<<nb, kNodeBlock, 0, st>>>(d); break;
        case 3: k_fe_c<<<eb, kElemBlock, 0, st>>>(d); break;
        default:
            if (g->hK.stress_bc_sides && d.bf.nbf > 0)
                k_stress_bc_facets<<<blocks(d.bf.nbf, 128), 128, 0, st>>>(d);
            k_fn_c<<<nb, kNodeBlock, 0, st>>>(d);
            launch_surface(g);
            break;
        }
    }
}

// passes N-A .. N-C of one step
void launch_head(des_gpu *g, cudaEvent_t *ev)
{
    for (int k = 0; k < 5; ++k) {
        if (ev) cudaEventRecord(ev[k], g->stream);
        launch_pass(g, k);
    }
}

// E-A over the element blocks [b0, b1) of its nblocks
void launch_ea(des_gpu *g, int b0, int b1)
{
    const int nb = blocks(g->nelem, kElemBlock);
    if (g->prec == DES_PREC_FP32)
        kf_fe_a<<<b1 - b0, kElemBlock, 0, g->stream>>>(g->f, b0 * kElemBlock, nb);
    else
        k_fe_a<<<b1 - b0, kElemBlock, 0, g->stream>>>(g->d, b0 * kElemBlock, nb);
}

// the averaging of the output fields after a step (Output::average_fields)
void launch_average(des_gpu *g)
{
    cudaStream_t st = g->stream;
    if (g->avg_interval > 0) {
        AvgArgs a;
        a.nnode = g->nnode;
        a.nelem = g->nelem;
        a.interval = g->avg_interval;
        a.clk = g->dclk;
        a.coord = g->d.x;
        const bool f32 = g->prec == DES_PREC_FP32;
        a.stress = f32 ? nullptr : g->d.stress;
        a.strain = f32 ? nullptr : g->d.strain;
        a.dpls = f32 ? nullptr : g->d.dpls;
        a.stress_f = f32 ? g->f.stress : nullptr;
        a.strain_f = f32 ? g->f.strain : nullptr;
        a.dpls_f = f32 ? g->f.dpls : nullptr;
        a.s0 = f32 ? g->f.s0 : nullptr;
        a.c0 = g->avg_c0;
        a.strain0 = g->avg_strain0;
        a.stress_sum = g->avg_stress;
        a.dpls_sum = g->avg_dpls;
        a.time0 = g->avg_time0;
        const long long n = std::max(3LL * g->nnode, (long long)g->nelem);
        k_average_fields<<<blocks(n, 256), 256, 0, st>>>(a);
    }
}

// pass E-A (and the averaging of the output fields) of one step
void launch_tail(des_gpu *g, cudaEvent_t *ev)
{
    if (ev) cudaEventRecord(ev[5], g->stream);
    launch_ea(g, 0, blocks(g->nelem, kElemBlock));
    if (ev) cudaEventRecord(ev[6], g->stream);
    launch_average(g);
}

// the six passes of one step, in order, on g's stream (captured or not)
void launch_step(des_gpu *g, cudaEvent_t *ev)
{
    launch_head(g, ev);
    launch_tail(g, ev);
}

int finish(des_gpu *g)
{
    DES_CUDA(cudaGetLastError());
    DES_CUDA(cudaStreamSynchronize(g->stream));
    return DES_OK;
}

// the second stream (output copies, downloads overlapping E-A) and its events
int ensure_copy_stream(des_gpu *g)
{
    if (!g->copy_stream) DES_CUDA(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking));
    if (!g->head_done) DES_CUDA(cudaEventCreateWithFlags(&g->head_done, cudaEventDisableTiming));
    if (!g->up_done) DES_CUDA(cudaEventCreateWithFlags(&g->up_done, cudaEventDisableTiming));
    if (!g->up_stream) DES_CUDA(cudaStreamCreateWithFlags(&g->up_stream, cudaStreamNonBlocking));
    for (cudaEvent_t &e : g->up_chunk)
        if (!e) DES_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    return DES_OK;
}

// the overlapped download's buffer, grown to n doubles when smaller
int ensure_download_buffer(des_gpu *g, long long n)
{
    if (n <= g->dl_elems) return DES_OK;
    if (g->dl) {
        g->allocs.erase(std::find(g->allocs.begin(), g->allocs.end(), static_cast<void *>(g->dl)));
        g->bytes -= (long long)sizeof(double) * (g->dl_elems ? g->dl_elems : 1);
        DES_CUDA(cudaFree(g->dl));
        g->dl = nullptr;
        g->dl_elems = 0;
    }
    int rc = dev_alloc(g, &g->dl, (size_t)n);
    if (rc) return rc;
    g->dl_elems = n;
    return DES_OK;
}

int capture_step_graph(des_gpu *g)
{
    cudaGraph_t graph;
    DES_CUDA(cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal));
    launch_step(g, nullptr);
    cudaError_t e = cudaStreamEndCapture(g->stream, &graph);
    if (e != cudaSuccess) return DES_ERR_CUDA;
    e = cudaGraphInstantiate(&g->graph, graph, 0);
    cudaGraphDestroy(graph);
    return cuda_rc(e);
}

__device__ __forceinline__ unsigned long long check_mix(unsigned long long z)
{
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// sf::mul, sf::to_float, sf::add0, sf::twice, sf::half, sf::div6, sf::div3
// and sf::quarter against the FP64 unit's multiply, conversion, addition and
// division
__global__ void k_softf64_check(unsigned long long *bad, long long n, unsigned long long seed)
{
    unsigned long long nb[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
        const unsigned long long r1 = check_mix(seed + 2 * i + 1), r2 = check_mix(seed + 2 * i + 2);
        const unsigned long long keep = 0x800fffffffffffffull;
        const double x = sf::from_bits(r1), y = sf::from_bits(r2);
        const double x1 = sf::from_bits((r1 & keep) | ((963ull + r2 % 121) << 52));
        const double y1 = sf::from_bits((r2 & keep) | ((963ull + (r1 >> 7) % 121) << 52));
        const double xf = sf::from_bits((r1 & keep) | ((870ull + (r2 >> 11) % 310) << 52));
        // every other operand with an exponent field of 0-8 (subnormals, results near them)
        const double xs = (i & 1) ? x : sf::from_bits((r1 & keep) | ((r2 % 9) << 52));
        double h = __dmul_rn(x, y), g = sf::mul(x, y);
        nb[0] += sf::bits(h) != sf::bits(g) && !(h != h && g != g);
        h = __dmul_rn(x1, y1);
        g = sf::mul(x1, y1);
        nb[1] += sf::bits(h) != sf::bits(g);
        float hf = __double2float_rn(x), gf = sf::to_float(x);
        nb[2] += __float_as_uint(hf) != __float_as_uint(gf) && !(hf != hf && gf != gf);
        hf = __double2float_rn(xf);
        gf = sf::to_float(xf);
        nb[3] += __float_as_uint(hf) != __float_as_uint(gf);
        h = __dadd_rn(0.0, xs);
        g = sf::add0(xs);
        nb[4] += sf::bits(h) != sf::bits(g) && !(h != h && g != g);
        h = __dmul_rn(xs, 2.0);
        g = sf::twice(xs);
        nb[5] += sf::bits(h) != sf::bits(g) && !(h != h && g != g);
        h = __dmul_rn(xs, 0.5);
        g = sf::half(xs);
        nb[6] += sf::bits(h) != sf::bits(g) && !(h != h && g != g);
        h = __ddiv_rn(xs, 6.0);
        g = sf::div6(xs);
        nb[7] += sf::bits(h) != sf::bits(g) && !(h != h && g != g);
        h = __ddiv_rn(xs, 3.0);
        g = sf::div3(xs);
        nb[8] += sf::bits(h) != sf::bits(g) && !(h != h && g != g);
        h = __dmul_rn(xs, 0.25);
        g = sf::quarter(xs);
        nb[9] += sf::bits(h) != sf::bits(g) && !(h != h && g != g);
    }
    for (int k = 0; k < 10; ++k)
        if (nb[k]) atomicAdd(bad + k, nb[k]);
}

}  // namespace

extern "C" {

int des_gpu_softf64_check(int device, long long n, unsigned long long seed, unsigned long long mismatches[10])
{
    if (n < 0 || !mismatches) return DES_ERR_ARG;
    DES_CUDA(cudaSetDevice(device));
    unsigned long long *bad = nullptr;
    DES_CUDA(cudaMalloc(&bad, 10 * sizeof(unsigned long long)));
    cudaError_t e = cudaMemset(bad, 0, 10 * sizeof(unsigned long long));
    int sms = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) {
        k_softf64_check<<<sms * 8, 256>>>(bad, n, seed);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(mismatches, bad, 10 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    cudaFree(bad);
    return cuda_rc(e);
}

const char *des_gpu_error_string(int code)
{
    switch (code) {
    case DES_OK: return "ok";
    case DES_ERR_OPTION: return "unknown rheology or option";
    case DES_ERR_ARG: return "bad argument";
    case DES_ERR_CUDA: return "CUDA runtime error";
    case DES_ERR_NOMEM: return "device allocation failed";
    case DES_ERR_UNSUPPORTED: return "option not supported by this library";
    case DES_ERR_SIZE: return "size above the entry point's limit";
    case DES_ERR_DT: return "dt <= 0 or non-finite coordinates";
    case DES_ERR_TOPOLOGY: return "inconsistent mesh topology";
    default: return "unknown error";
    }
}

// create_support (mesh.cxx:1703-1717) from the device connectivity into the
// CSR the node passes gather over (des_support.cuh)
static int build_support(des_gpu *g, const int *conn, int *sup_off, unsigned *sup_ent)
{
    const int N = g->nnode;
    const long long nent = 4LL * g->nelem, n1 = (long long)N + 1;
    const int nb = (int)((n1 + kScanBlock - 1) / kScanBlock);
    cudaStream_t s = g->stream;
    int *sums = nullptr, *cursor = nullptr;
    int rc = DES_OK;
    if (cudaMalloc(&sums, sizeof(int) * (size_t)nb) != cudaSuccess ||
        cudaMalloc(&cursor, sizeof(int) * (size_t)N) != cudaSuccess)
        rc = DES_ERR_NOMEM;
    if (!rc) rc = cuda_rc(cudaMemsetAsync(sup_off, 0, sizeof(int) * (size_t)n1, s));
    if (!rc) rc = cuda_rc(cudaMemsetAsync(cursor, 0, sizeof(int) * (size_t)N, s));
    if (!rc) {
        k_sup_count<<<blocks(nent, 256), 256, 0, s>>>(nent, conn, sup_off);
        k_scan_blocks<<<nb, kScanBlock, 0, s>>>(sup_off, n1, sums);
        k_scan_sums<<<1, kScanBlock, 0, s>>>(sums, nb);
        k_scan_add<<<nb, kScanBlock, 0, s>>>(sup_off, n1, sums);
        k_sup_fill<<<blocks(nent, 256), 256, 0, s>>>(nent, conn, sup_off, cursor, sup_ent);
        k_sup_sort<<<blocks(N, kNodeBlock), kNodeBlock, 0, s>>>(N, sup_off, sup_ent);
        rc = cuda_rc(cudaGetLastError());
    }
    if (!rc) rc = cuda_rc(cudaStreamSynchronize(s));
    cudaFree(sums);
    cudaFree(cursor);
    return rc;
}

int des_gpu_create(const des_mesh_view *m, const des_params *p, int device, des_gpu **out)
{
    if (!m || !p || !out || !m->elemmarkers) return DES_ERR_ARG;
    int rc = check_params(*p, m->nmat);
    if (rc) return rc;
    des_topology *topo = nullptr;
    rc = topology_build(m, &topo, false);   // support lists: built on the device below
    if (rc) return rc;
    des_gpu *g = new (std::nothrow) des_gpu();   // value-initialised: every device pointer starts null
    if (!g) {
        des_topology_free(topo);
        return DES_ERR_NOMEM;
    }
    if (device >= 0 && cudaSetDevice(device) != cudaSuccess) {
        des_topology_free(topo);
        delete g;
        return DES_ERR_CUDA;
    }
    cudaGetDevice(&g->device);
    cudaDeviceGetAttribute(&g->sms, cudaDevAttrMultiProcessorCount, g->device);
    if (g->sms < 1) g->sms = 1;
    g->P = *p;
    g->nnode = m->nnode;
    g->nelem = m->nelem;
    g->nmat = m->nmat;
    for (int i = 0; i < DES_NBDRY; ++i) g->bfacets_count[i] = topo->bfacets_count[i];

    std::vector<unsigned char> mix;
    if ((rc = build_mix(m->elemmarkers, m->nelem, m->nmat, g->mix_counts, mix))) {
        des_topology_free(topo);
        delete g;
        return rc;
    }

    auto fail = [&](int code) {
        des_topology_free(topo);
        des_gpu_destroy(g);
        return code;
    };
    if (cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(DES_ERR_CUDA);
    const size_t N = m->nnode, E = m->nelem;
    g->prec = p->precision;
    Dev &d = g->d;
    d.nnode = m->nnode;
    d.nelem = m->nelem;
    double *coord, *coord0;
    int4 *conn;
    int *sup_off;
    unsigned *sup_ent, *bcflag;
    unsigned char *dmix;
    // arrays both forms keep in FP64 (and the topology)
    if ((rc = dev_alloc(g, &coord, 3 * N)) || (rc = dev_alloc(g, &coord0, 3 * N)) ||
        (rc = dev_alloc(g, &d.T, N)) || (rc = dev_alloc(g, &bcflag, N)) ||
        (rc = dev_alloc(g, &sup_off, N + 1)) || (rc = dev_alloc(g, &sup_ent, 4 * E)) ||
        (rc = dev_alloc(g, &conn, E)) || (rc = dev_alloc(g, &dmix, E)) ||
        (rc = dev_alloc(g, &d.vol, E)) || (rc = dev_alloc(g, &d.vol_old, E)) ||
        (rc = dev_alloc(g, &d.pls, E)) || (rc = dev_alloc(g, &g->dK, 1)) ||
        (rc = dev_alloc(g, &g->dclk, 1)))
        return fail(rc);
    d.x = coord; d.y = coord + N; d.z = coord + 2 * N;
    d.x0 = coord0; d.y0 = coord0 + N; d.z0 = coord0 + 2 * N;
    d.conn = conn;
    d.sup_off = sup_off;
    d.sup_ent = sup_ent;
    d.bcflag = bcflag;
    d.mix = dmix;
    d.K = g->dK;
    d.clk = g->dclk;
    if (g->prec == DES_PREC_FP64) {
        double *vel, *force;
        if ((rc = dev_alloc(g, &vel, 3 * N)) || (rc = dev_alloc(g, &force, 3 * N)) ||
            (rc = dev_alloc(g, &d.mass, N)) || (rc = dev_alloc(g, &d.tmass, N)) ||
            (rc = dev_alloc(g, &d.vol_n, N)) || (rc = dev_alloc(g, &d.ntmp, N)) ||
            (rc = dev_alloc(g, &d.edvoldt, E)) || (rc = dev_alloc(g, &d.dpls, E)) ||
            (rc = dev_alloc(g, &d.dp, E)) || (rc = dev_alloc(g, &d.tmp_sg, E)) ||
            (rc = dev_alloc(g, &d.stress, 6 * E)) || (rc = dev_alloc(g, &d.strain, 6 * E)) ||
            (rc = dev_alloc(g, &d.srate, 6 * E)) || (rc = dev_alloc(g, &d.srate_next, 6 * E)) ||
            (rc = dev_alloc(g, &d.shp, 12 * E)) || (rc = dev_alloc(g, &d.tmp, 12 * E)) ||
            (rc = dev_alloc(g, &d.c_mass, E)) || (rc = dev_alloc(g, &d.c_tmass, E)) ||
            (rc = dev_alloc(g, &d.c_trdv, E)))
            return fail(rc);
        d.vx = vel; d.vy = vel + N; d.vz = vel + 2 * N;
        d.fx = force; d.fy = force + N; d.fz = force + 2 * N;
    } else {
        DevF &f = g->f;
        float *vel, *force;
        if ((rc = dev_alloc(g, &vel, 3 * N)) || (rc = dev_alloc(g, &force, 3 * N)) ||
            (rc = dev_alloc(g, &f.mass, N)) || (rc = dev_alloc(g, &f.tmass, N)) ||
            (rc = dev_alloc(g, &f.vol_n, N)) || (rc = dev_alloc(g, &f.ntmp, N)) ||
            (rc = dev_alloc(g, &f.edvoldt, E)) || (rc = dev_alloc(g, &f.dpls, E)) ||
            (rc = dev_alloc(g, &f.dp, E)) || (rc = dev_alloc(g, &f.tmp_sg, E)) ||
            (rc = dev_alloc(g, &f.stress, 6 * E)) || (rc = dev_alloc(g, &f.strain, 6 * E)) ||
            (rc = dev_alloc(g, &f.srate, 6 * E)) || (rc = dev_alloc(g, &f.srate_next, 6 * E)) ||
            (rc = dev_alloc(g, &f.shp, 12 * E)) || (rc = dev_alloc(g, &f.tmp, 12 * E)) ||
            (rc = dev_alloc(g, &f.c_vol, E)) || (rc = dev_alloc(g, &f.c_mass, E)) ||
            (rc = dev_alloc(g, &f.c_tmass, E)) || (rc = dev_alloc(g, &f.c_trdv, E)) ||
            (rc = dev_alloc(g, &f.s0, E)) || (rc = dev_alloc(g, &f.f0, 12 * E)) ||
            (rc = dev_alloc(g, &f.pend, E)) || (rc = dev_alloc(g, &f.exact, E)) ||
            (rc = dev_alloc(g, &g->dF, 1)))
            return fail(rc);
        f.nnode = d.nnode;
        f.nelem = d.nelem;
        f.conn = conn;
        f.sup_off = sup_off;
        f.sup_ent = sup_ent;
        f.bcflag = bcflag;
        f.mix = dmix;
        f.x = d.x; f.y = d.y; f.z = d.z;
        f.x0 = d.x0; f.y0 = d.y0; f.z0 = d.z0;
        f.T = d.T;
        f.vol = d.vol;
        f.vol_old = d.vol_old;
        f.pls = d.pls;
        f.vx = vel; f.vy = vel + N; f.vz = vel + 2 * N;
        f.fx = force; f.fy = force + N; f.fz = force + 2 * N;
        f.K = g->dK;
        f.F = g->dF;
        f.clk = g->dclk;
    }
    g->staging_elems = std::min<long long>(12LL * (long long)E, 1LL << 25);
    g->staging_elems = std::max<long long>(g->staging_elems, 3LL * (long long)N < (1LL << 25) ? 3LL * (long long)N : (1LL << 25));
    if ((rc = dev_alloc(g, &g->staging, (size_t)g->staging_elems))) return fail(rc);

    // apply_stress_bcs: every boundary facet, and each node's facets in the
    // order bc.cxx:568-590 subtracts them (side by side, facets in bfacets
    // order)
    {
        static const int kFacetHost[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};   // constants.hpp:61-67
        int nbf = 0;
        for (int i = 0; i < DES_NBDRY; ++i) nbf += topo->bfacets_count[i];
        std::vector<int> belem((size_t)nbf), off(N + 1, 0), nodes(3 * (size_t)nbf);
        std::vector<unsigned char> bsf((size_t)nbf);
        int k = 0;
        for (int i = 0; i < DES_NBDRY; ++i)
            for (int j = 0; j < topo->bfacets_count[i]; ++j, ++k) {
                const int e = topo->bfacets[i][2 * j], f = topo->bfacets[i][2 * j + 1];
                belem[k] = e;
                bsf[k] = (unsigned char)((i << 2) | f);
                for (int q = 0; q < 3; ++q) {
                    nodes[3 * (size_t)k + q] = m->connectivity[4 * (size_t)e + kFacetHost[f][q]];
                    ++off[nodes[3 * (size_t)k + q] + 1];
                }
            }
        for (size_t n = 0; n < N; ++n) off[n + 1] += off[n];
        std::vector<int> fill(off.begin(), off.end() - 1), nf((size_t)off[N]);
        for (int q = 0; q < 3 * nbf; ++q) nf[(size_t)fill[nodes[q]]++] = q / 3;
        int *d_elem, *d_off, *d_nf;
        unsigned char *d_sf;
        double *d_val, *d_surf;
        if ((rc = dev_alloc(g, &d_elem, (size_t)nbf)) || (rc = dev_alloc(g, &d_sf, (size_t)nbf)) ||
            (rc = dev_alloc(g, &d_val, 3 * (size_t)nbf)) || (rc = dev_alloc(g, &d_surf, 4 * (size_t)nbf)) ||
            (rc = dev_alloc(g, &d_off, N + 1)) ||
            (rc = dev_alloc(g, &d_nf, (size_t)off[N])))
            return fail(rc);
        if (cudaMemcpy(d_elem, belem.data(), sizeof(int) * nbf, cudaMemcpyHostToDevice) ||
            cudaMemcpy(d_sf, bsf.data(), (size_t)nbf, cudaMemcpyHostToDevice) ||
            cudaMemcpy(d_off, off.data(), sizeof(int) * (N + 1), cudaMemcpyHostToDevice) ||
            cudaMemcpy(d_nf, nf.data(), sizeof(int) * nf.size(), cudaMemcpyHostToDevice))
            return fail(DES_ERR_CUDA);
        BdryFacets sb;
        sb.nbf = nbf;
        sb.elem = d_elem;
        sb.side_f = d_sf;
        sb.val = d_val;
        sb.surf = d_surf;
        sb.node_off = d_off;
        sb.node_facet = d_nf;
        g->d.bf = sb;
        g->f.bf = sb;
    }

    if (cudaMemcpy(conn, m->connectivity, sizeof(int) * 4 * E, cudaMemcpyHostToDevice) ||
        cudaMemcpy(bcflag, topo->bcflag, sizeof(unsigned) * N, cudaMemcpyHostToDevice) ||
        cudaMemcpy(dmix, mix.data(), E, cudaMemcpyHostToDevice))
        return fail(DES_ERR_CUDA);
    if ((rc = build_support(g, reinterpret_cast<const int *>(conn), sup_off, sup_ent))) return fail(rc);
    des_topology_free(topo);
    topo = nullptr;
    Clock c0;
    std::memset(&c0, 0, sizeof(c0));
    c0.minl = ~0ULL;
    if (cudaMemcpy(g->dclk, &c0, sizeof(Clock), cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(DES_ERR_CUDA);
    if ((rc = build_consts(g))) return fail(rc);
    *out = g;
    return DES_OK;
}

int des_gpu_download_support(des_gpu *g, int *offsets, int *elems, int *slots)
{
    if (!g || !offsets || !elems || !slots) return DES_ERR_ARG;
    const size_t N = g->nnode, E = g->nelem;
    std::vector<unsigned> ent(4 * E);
    DES_CUDA(cudaStreamSynchronize(g->stream));
    DES_CUDA(cudaMemcpy(offsets, g->d.sup_off, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost));
    DES_CUDA(cudaMemcpy(ent.data(), g->d.sup_ent, sizeof(unsigned) * 4 * E, cudaMemcpyDeviceToHost));
    for (size_t q = 0; q < 4 * E; ++q) {
        elems[q] = (int)(ent[q] >> 2);
        slots[q] = (int)(ent[q] & 3u);
    }
    return DES_OK;
}

int des_gpu_destroy(des_gpu *g)
{
    if (!g) return DES_OK;
    if (g->copy_stream) {
        cudaStreamSynchronize(g->copy_stream);
        cudaStreamDestroy(g->copy_stream);
    }
    if (g->up_stream) {
        cudaStreamSynchronize(g->up_stream);
        cudaStreamDestroy(g->up_stream);
    }
    for (cudaEvent_t e : g->up_chunk)
        if (e) cudaEventDestroy(e);
    if (g->snap_ready) cudaEventDestroy(g->snap_ready);
    if (g->head_done) cudaEventDestroy(g->head_done);
    if (g->up_done) cudaEventDestroy(g->up_done);
    if (g->snap_done) cudaEventDestroy(g->snap_done);
    if (g->stream) cudaStreamSynchronize(g->stream);
    if (g->graph) cudaGraphExecDestroy(g->graph);
    for (void *p : g->allocs) cudaFree(p);
    if (g->stream) cudaStreamDestroy(g->stream);
    delete g;
    return DES_OK;
}

int des_gpu_set_params(des_gpu *g, const des_params *p)
{
    if (!g || !p) return DES_ERR_ARG;
    int rc = check_params(*p, g->nmat);
    if (rc) return rc;
    if (p->precision != g->prec) return DES_ERR_ARG;   // the device layout depends on it
    g->P = *p;
    g->primed = false;
    rc = build_consts(g);
    if (rc) return rc;
    // the captured step depends on the rheology (closure) and on whether
    // boundary tractions apply
    if (g->graph) cudaGraphExecDestroy(g->graph);
    g->graph = nullptr;
    if (g->closure && g->hF.rheol != 5 && g->hF.rheol != 7) g->closure = false;
    return DES_OK;
}

int des_gpu_set_elemmarkers(des_gpu *g, const int *elemmarkers)
{
    if (!g || !elemmarkers) return DES_ERR_ARG;
    std::vector<std::vector<int>> counts;
    std::vector<unsigned char> mix;
    int rc = build_mix(elemmarkers, g->nelem, g->nmat, counts, mix);
    if (rc) return rc;
    // the network was trained on one material mix
    if (g->closure && counts != g->mix_counts) return DES_ERR_UNSUPPORTED;
    DES_CUDA(cudaMemcpyAsync(const_cast<unsigned char *>(g->d.mix), mix.data(), (size_t)g->nelem,
                             cudaMemcpyHostToDevice, g->stream));
    DES_CUDA(cudaStreamSynchronize(g->stream));
    g->mix_counts.swap(counts);
    if ((rc = build_consts(g))) return rc;
    // the conduction and (FP32 form) reference-force terms prepared for the
    // next step depend on the mix
    g->primed = false;
    return DES_OK;
}

long long des_gpu_device_bytes(const des_gpu *g) { return g ? g->bytes : 0; }
int des_gpu_kernels_per_step(const des_gpu *g)
{
    if (!g) return 0;
    int n = kStepKernels + ((g->hK.stress_bc_sides && g->d.bf.nbf > 0) ? 1 : 0);
    if (g->P.surface_process_option == 1) n += g->d.bf.nbf > 0 ? 2 : 1;
    if (g->P.surface_process_option == 101) n += 1;
    // the FP32 form's elasto-plastic stress pass: the exact list, the network
    if (g->prec == DES_PREC_FP32 && (g->hF.rheol == 5 || g->hF.rheol == 7)) n += g->closure ? 2 : 1;
    return n + (g->avg_interval > 0 ? 1 : 0);
}

int des_gpu_upload(des_gpu *g, const des_state_view *h, unsigned mask)
{
    if (!g || !h || h->nnode != g->nnode || h->nelem != g->nelem) return DES_ERR_ARG;
    if (mask & ~(unsigned)DES_F_ALL) return DES_ERR_ARG;
    const long long N = g->nnode, E = g->nelem;
    Dev &d = g->d;
    int rc = DES_OK;
    const bool f32 = g->prec == DES_PREC_FP32;
    DevF &f = g->f;
#define UP(flag, ptr, dst, nc, rows) \
    if ((mask & (flag)) && (rc = upload_field(g, h->ptr, dst, nc, rows))) return rc;
    // fields of the form's precision (FP32 copies in the mixed form)
#define UPX(flag, ptr, fld, off, nc, rows)                                                    \
    if (mask & (flag)) {                                                                     \
        rc = f32 ? upload_field(g, h->ptr, f.fld + (off), nc, rows)                          \
                 : upload_field(g, h->ptr, d.fld + (off), nc, rows);                         \
        if (rc) return rc;                                                                   \
    }
    UP(DES_F_COORD, coord, d.x, 3, N)
    UP(DES_F_COORD0, coord0, d.x0, 3, N)
    UPX(DES_F_VEL, vel, vx, 0, 3, N)
    UPX(DES_F_FORCE, force, fx, 0, 3, N)
    UP(DES_F_TEMPERATURE, temperature, d.T, 1, N)
    UPX(DES_F_MASS, mass, mass, 0, 1, N)
    UPX(DES_F_MASS, tmass, tmass, 0, 1, N)
    UPX(DES_F_MASS, volume_n, vol_n, 0, 1, N)
    UPX(DES_F_NTMP, ntmp, ntmp, 0, 1, N)
    UP(DES_F_VOLUME, volume, d.vol, 1, E)
    UP(DES_F_VOLUME, volume_old, d.vol_old, 1, E)
    if (mask & DES_F_STRESS) {
        if (f32) {
            if (!h->stress) return DES_ERR_ARG;
            if (const double *m = static_cast<const double *>(mapped(h->stress))) {
                k_stress_split_tiled<<<blocks(E, 256), 256, 0, g->stream>>>(m, f.s0, f.stress, E);
                DES_LAUNCH();
            } else {
                long long chunk = std::max(1LL, g->staging_elems / 6);
                for (long long r0 = 0; r0 < E; r0 += chunk) {
                    long long nr = std::min(chunk, E - r0);
                    DES_CUDA(cudaMemcpyAsync(g->staging, h->stress + 6 * r0, sizeof(double) * 6 * nr,
                                             cudaMemcpyHostToDevice, g->stream));
                    k_stress_split<<<blocks(nr, 256), 256, 0, g->stream>>>(g->staging, f.s0, f.stress, nr,
                                                                            r0, E);
                    DES_LAUNCH();
                }
            }
        } else if ((rc = upload_field(g, h->stress, d.stress, 6, E))) {
            return rc;
        }
    }
    UPX(DES_F_STRAIN, strain, strain, 0, 6, E)
    UPX(DES_F_STRAIN_RATE, strain_rate, srate, 0, 6, E)
    UP(DES_F_PLSTRAIN, plstrain, d.pls, 1, E)
    UPX(DES_F_PLSTRAIN, delta_plstrain, dpls, 0, 1, E)
    UPX(DES_F_DPRESSURE, dpressure, dp, 0, 1, E)
    UPX(DES_F_EDVOLDT, edvoldt, edvoldt, 0, 1, E)
    UPX(DES_F_SHAPE, shpdx, shp, 0, 4, E)
    UPX(DES_F_SHAPE, shpdy, shp, 4 * E, 4, E)
    UPX(DES_F_SHAPE, shpdz, shp, 8 * E, 4, E)
    UPX(DES_F_TMP_RESULT, tmp_result, tmp, 0, 12, E)
    UPX(DES_F_TMP_RESULT, tmp_result_sg, tmp_sg, 0, 1, E)
#undef UP
#undef UPX
    if (f32 && (mask & DES_F_VOLUME)) {
        // FP32 copy of the volumes used as element weights
        k_vol_to_f<<<blocks(E, 256), 256, 0, g->stream>>>(d.vol, f.c_vol, E);
        DES_LAUNCH();
    }
    if (mask & (DES_F_SCALARS | DES_F_MASS)) {
        Clock c;
        if ((rc = read_clock(g, c))) return rc;
        if (mask & DES_F_SCALARS) {
            c.time = h->time;
            c.dt = h->dt;
            c.steps = h->steps;
        }
        if (mask & DES_F_MASS) c.mass_valid = 1;
        k_clock_set<<<1, 32, 0, g->stream>>>(g->dclk, c.time, c.dt, c.steps, c.mass_valid);
        DES_LAUNCH();
    }
    g->primed = false;
    return finish(g);
}

// One field of a download: its host rows and its device source (FP64 or
// FP32 structure of arrays, or the FP32 form's split stress s0 + s').
struct DownPart {
    double *host;
    const double *src64;
    const float *src32;
    bool stress_join;
    int ncomp;
    long long rows;
    bool elem;          // one row per element (else per node)
};

// the mask fields in download order; DES_ERR_ARG for a missing host array
static int down_parts(des_gpu *g, des_state_view *h, unsigned mask, std::vector<DownPart> &out)
{
    const long long N = g->nnode, E = g->nelem;
    const Dev &d = g->d;
    const DevF &f = g->f;
    const bool f32 = g->prec == DES_PREC_FP32;
    out.clear();
    bool ok = true;
    // x: a field kept in the form's precision (FP32 in the mixed form)
    auto add = [&](unsigned flag, double *host, const double *s64, const float *s32, bool x, int nc, bool elem) {
        if (!ok || !(mask & flag)) return;
        if (!host) {
            ok = false;
            return;
        }
        const bool use32 = x && f32;
        out.push_back({host, use32 ? nullptr : s64, use32 ? s32 : nullptr, false, nc, elem ? E : N, elem});
    };
    add(DES_F_COORD, h->coord, d.x, nullptr, false, 3, false);
    add(DES_F_COORD0, h->coord0, d.x0, nullptr, false, 3, false);
    add(DES_F_VEL, h->vel, d.vx, f.vx, true, 3, false);
    add(DES_F_FORCE, h->force, d.fx, f.fx, true, 3, false);
    add(DES_F_TEMPERATURE, h->temperature, d.T, nullptr, false, 1, false);
    add(DES_F_MASS, h->mass, d.mass, f.mass, true, 1, false);
    add(DES_F_MASS, h->tmass, d.tmass, f.tmass, true, 1, false);
    add(DES_F_MASS, h->volume_n, d.vol_n, f.vol_n, true, 1, false);
    add(DES_F_NTMP, h->ntmp, d.ntmp, f.ntmp, true, 1, false);
    add(DES_F_VOLUME, h->volume, d.vol, nullptr, false, 1, true);
    add(DES_F_VOLUME, h->volume_old, d.vol_old, nullptr, false, 1, true);
    if (ok && (mask & DES_F_STRESS)) {
        if (!h->stress) return DES_ERR_ARG;
        out.push_back({h->stress, f32 ? nullptr : d.stress, nullptr, f32, 6, E, true});
    }
    add(DES_F_STRAIN, h->strain, d.strain, f.strain, true, 6, true);
    add(DES_F_STRAIN_RATE, h->strain_rate, d.srate, f.srate, true, 6, true);
    add(DES_F_PLSTRAIN, h->plstrain, d.pls, nullptr, false, 1, true);
    add(DES_F_PLSTRAIN, h->delta_plstrain, d.dpls, f.dpls, true, 1, true);
    add(DES_F_DPRESSURE, h->dpressure, d.dp, f.dp, true, 1, true);
    add(DES_F_EDVOLDT, h->edvoldt, d.edvoldt, f.edvoldt, true, 1, true);
    add(DES_F_SHAPE, h->shpdx, d.shp, f.shp, true, 4, true);
    add(DES_F_SHAPE, h->shpdy, d.shp + 4 * E, f.shp + 4 * E, true, 4, true);
    add(DES_F_SHAPE, h->shpdz, d.shp + 8 * E, f.shp + 8 * E, true, 4, true);
    add(DES_F_TMP_RESULT, h->tmp_result, d.tmp, f.tmp, true, 12, true);
    add(DES_F_TMP_RESULT, h->tmp_result_sg, d.tmp_sg, f.tmp_sg, true, 1, true);
    return ok ? DES_OK : DES_ERR_ARG;
}

// rows [r0, r0 + nr) of one part as host-layout rows at dst, on stream st
static int convert_part(des_gpu *g, const DownPart &q, long long r0, long long nr, double *dst, cudaStream_t st)
{
    if (q.stress_join)
        k_stress_join<<<blocks(nr, 256), 256, 0, st>>>(g->f.s0, g->f.stress, dst, nr, r0, q.rows);
    else if (q.src64)
        k_soa_to_aos<<<blocks(nr * q.ncomp, 256), 256, 0, st>>>(q.src64, dst, q.ncomp, nr, r0, q.rows);
    else
        k_soa_to_aos_f<<<blocks(nr * q.ncomp, 256), 256, 0, st>>>(q.src32, dst, q.ncomp, nr, r0, q.rows);
    DES_LAUNCH();
    return DES_OK;
}

// The mask fields into the host rows through the staging buffer, on g's
// stream (current nodal masses and the clock are the caller's part).
static int download_fields(des_gpu *g, des_state_view *h, unsigned mask)
{
    std::vector<DownPart> parts;
    int rc = down_parts(g, h, mask, parts);
    if (rc) return rc;
    for (const DownPart &q : parts) {
        const long long chunk = std::max(1LL, g->staging_elems / q.ncomp);
        for (long long r0 = 0; r0 < q.rows; r0 += chunk) {
            const long long nr = std::min(chunk, q.rows - r0);
            if ((rc = convert_part(g, q, r0, nr, g->staging, g->stream))) return rc;
            DES_CUDA(cudaMemcpyAsync(q.host + r0 * q.ncomp, g->staging, sizeof(double) * nr * q.ncomp,
                                     cudaMemcpyDeviceToHost, g->stream));
        }
    }
    return DES_OK;
}

// Overlapped form: each part is converted whole on g's stream into the
// download buffer at *offset and copied to the host on the copy stream as
// soon as its conversion is done, so conversions, copies and later kernels
// of g's stream run side by side.  The caller synchronises the copy stream.
// rows [r0, r0 + nr) of part q: converted on g's stream into its place in
// the download buffer (the part starts at base), then copied on the copy stream
static int download_rows_async(des_gpu *g, const DownPart &q, long long base, long long r0, long long nr)
{
    double *dst = g->dl + base + r0 * q.ncomp;
    int rc = convert_part(g, q, r0, nr, dst, g->stream);
    if (rc) return rc;
    DES_CUDA(cudaEventRecord(g->head_done, g->stream));
    DES_CUDA(cudaStreamWaitEvent(g->copy_stream, g->head_done, 0));
    DES_CUDA(cudaMemcpyAsync(q.host + r0 * q.ncomp, dst, sizeof(double) * q.ncomp * nr, cudaMemcpyDeviceToHost,
                             g->copy_stream));
    return DES_OK;
}

static int download_async(des_gpu *g, const std::vector<DownPart> &parts, long long *offset)
{
    for (const DownPart &q : parts) {
        int rc = download_rows_async(g, q, *offset, 0, q.rows);
        if (rc) return rc;
        *offset += q.ncomp * q.rows;
    }
    return DES_OK;
}

// nodal masses from the last E-A's contributions, before they are read
static int flush_masses(des_gpu *g, const Clock &c)
{
    if (c.mass_valid) return DES_OK;
    if (g->prec == DES_PREC_FP32)
        kf_mass_flush<<<blocks(g->nnode, kNodeBlock), kNodeBlock, 0, g->stream>>>(g->f);
    else
        k_mass_flush<<<blocks(g->nnode, kNodeBlock), kNodeBlock, 0, g->stream>>>(g->d);
    DES_LAUNCH();
    return DES_OK;
}

int des_gpu_download(des_gpu *g, des_state_view *h, unsigned mask)
{
    if (!g || !h || h->nnode != g->nnode || h->nelem != g->nelem) return DES_ERR_ARG;
    if (mask & ~(unsigned)DES_F_ALL) return DES_ERR_ARG;
    Clock c;
    int rc = read_clock(g, c);
    if (rc) return rc;
    if ((mask & DES_F_MASS) && (rc = flush_masses(g, c))) return rc;
    if ((rc = download_fields(g, h, mask))) return rc;
    if (mask & DES_F_SCALARS) {
        h->time = c.time;
        h->dt = c.dt;
        h->steps = c.steps;
    }
    return finish(g);
}

int des_gpu_report(des_gpu *g, des_step_report *r)
{
    if (!g || !r) return DES_ERR_ARG;
    Clock c;
    int rc = read_clock(g, c);
    if (rc) return rc;
    r->steps = c.steps;
    r->time = c.time;
    r->dt = c.dt;
    r->status = c.status;
    r->ql_fallbacks = (long long)c.ql;
    r->eigen_solves = (long long)c.eig;
    r->closure_candidates = (long long)c.nn_cand;
    r->closure_accepted = (long long)c.nn_accept;
    r->exact_returns = (long long)c.fp64_returns;
    return DES_OK;
}

// host inverse of order_bits
static double from_bits(unsigned long long b)
{
    unsigned long long r = (b >> 63) ? (b & 0x7fffffffffffffffULL) : ~b;
    double x;
    std::memcpy(&x, &r, sizeof x);
    return x;
}

// elem_quality of every element into the scratch array (and the reductions of
// the remesh checks into g->qout); returns the scratch array
static int run_quality(des_gpu *g, const des_remesh_check *c, double **q)
{
    if (int rc = begin_fn(g)) return rc;     // the scratch array holds state of the fused passes
    if (!g->qout) {
        int rc = dev_alloc(g, &g->qout, 4);
        if (rc) return rc;
    }
    QualityArgs a;
    const Dev &d = g->d;
    a.nelem = g->nelem;
    a.nnode = g->nnode;
    a.conn = d.conn;
    a.x = d.x;
    a.y = d.y;
    a.z = d.z;
    a.vol = d.vol;
    a.bcflag = d.bcflag;
    a.nf = 216 * std::sqrt(3.0);                          // geometry.cxx:491
    a.smallest_vol = c ? c->smallest_size * 0.118 * std::pow(c->resolution, 3) : 0.0;   // remeshing.cxx:83,1905
    a.bottom = c ? -c->zlength : 0.0;
    a.dist = c ? c->max_boundary_distortion * c->resolution : 0.0;
    a.check_bottom = c && (c->remeshing_option == 1 || c->remeshing_option == 2 || c->remeshing_option == 11);
    a.q = g->prec == DES_PREC_FP32 ? reinterpret_cast<double *>(g->f.tmp) : d.tmp;
    a.out = g->qout;
    DES_CUDA(cudaMemsetAsync(g->qout, 0xff, 4 * sizeof(unsigned long long), g->stream));
    const int eb = blocks(g->nelem, kElemBlock), nb = blocks(g->nnode, kNodeBlock);
    k_quality<<<eb, kElemBlock, 0, g->stream>>>(a);
    k_quality_worst<<<eb, kElemBlock, 0, g->stream>>>(a);
    if (a.check_bottom) k_bottom_distortion<<<nb, kNodeBlock, 0, g->stream>>>(a);
    DES_LAUNCH();
    *q = a.q;
    return DES_OK;
}

int des_gpu_bad_mesh_quality(des_gpu *g, const des_remesh_check *c, int *code, int *index,
                             double *worst_quality)
{
    if (!g || !c || !code || !index) return DES_ERR_ARG;
    double *q;
    if (int rc = run_quality(g, c, &q)) return rc;
    unsigned long long out[4];
    DES_CUDA(cudaMemcpyAsync(out, g->qout, sizeof out, cudaMemcpyDeviceToHost, g->stream));
    DES_CUDA(cudaStreamSynchronize(g->stream));
    // worst_elem_quality (geometry.cxx:512-526) starts from q = 1, element 0
    double qw = 1;
    int worst = 0;
    if (out[0] != ~0ull && from_bits(out[0]) < 1) {
        qw = from_bits(out[0]);
        worst = (int)out[1];
    }
    qw = std::pow(qw, 1.0 / 3);                             // remeshing.cxx:1946
    if (worst_quality) *worst_quality = qw;
    // remeshing.cxx:1905-1954: tiny elements, then the bottom, then distortion
    if (out[2] != ~0ull) {
        *code = 3;
        *index = (int)out[2];
    } else if (out[3] != ~0ull) {
        *code = 2;
        *index = (int)out[3];
    } else if (qw < c->min_quality) {
        *code = 1;
        *index = worst;
    } else {
        *code = 0;
    }
    return DES_OK;
}

int des_gpu_elem_quality(des_gpu *g, double *quality)
{
    if (!g || !quality) return DES_ERR_ARG;
    double *q;
    if (int rc = run_quality(g, nullptr, &q)) return rc;
    DES_CUDA(cudaMemcpyAsync(quality, q, sizeof(double) * g->nelem, cudaMemcpyDeviceToHost, g->stream));
    DES_CUDA(cudaStreamSynchronize(g->stream));
    return DES_OK;
}

// ---- output snapshots ---------------------------------------------------
// fields a snapshot can hold, in this order, with their AoS row widths
namespace {
constexpr unsigned kSnapFields = DES_F_COORD | DES_F_VEL | DES_F_FORCE | DES_F_TEMPERATURE | DES_F_VOLUME |
                                 DES_F_STRESS | DES_F_STRAIN | DES_F_STRAIN_RATE | DES_F_PLSTRAIN | DES_F_COORD0;
struct SnapPart {
    unsigned flag;
    int ncomp;
    bool node;
    double *des_state_view::*host;
};
const SnapPart kSnap[] = {
    {DES_F_COORD, 3, true, &des_state_view::coord},
    {DES_F_VEL, 3, true, &des_state_view::vel},
    {DES_F_FORCE, 3, true, &des_state_view::force},
    {DES_F_TEMPERATURE, 1, true, &des_state_view::temperature},
    {DES_F_COORD0, 3, true, &des_state_view::coord0},
    {DES_F_VOLUME, 1, false, &des_state_view::volume},
    {DES_F_VOLUME, 1, false, &des_state_view::volume_old},
    {DES_F_STRESS, 6, false, &des_state_view::stress},
    {DES_F_STRAIN, 6, false, &des_state_view::strain},
    {DES_F_STRAIN_RATE, 6, false, &des_state_view::strain_rate},
    {DES_F_PLSTRAIN, 1, false, &des_state_view::plstrain},
    {DES_F_PLSTRAIN, 1, false, &des_state_view::delta_plstrain},
};
}  // namespace

int des_gpu_output_snapshot(des_gpu *g, unsigned mask)
{
    if (!g || (mask & ~kSnapFields)) return DES_ERR_ARG;
    const long long N = g->nnode, E = g->nelem;
    if (!g->snap) {
        long long n = 0;
        for (const SnapPart &s : kSnap) n += (long long)s.ncomp * (s.node ? N : E);
        int rc;
        if ((rc = dev_alloc(g, &g->snap, (size_t)n)) || (rc = dev_alloc(g, &g->snap_clk, 1))) return rc;
        g->snap_bytes = n * (long long)sizeof(double);
        if ((rc = ensure_copy_stream(g))) return rc;
        DES_CUDA(cudaEventCreateWithFlags(&g->snap_ready, cudaEventDisableTiming));
        DES_CUDA(cudaEventCreateWithFlags(&g->snap_done, cudaEventDisableTiming));
        DES_CUDA(cudaEventRecord(g->snap_done, g->copy_stream));
    }
    // the previous snapshot's copies must have left the buffer
    DES_CUDA(cudaStreamWaitEvent(g->stream, g->snap_done, 0));
    const bool f32 = g->prec == DES_PREC_FP32;
    const Dev &d = g->d;
    const DevF &f = g->f;
    double *dst = g->snap;
    cudaStream_t st = g->stream;
    for (const SnapPart &s : kSnap) {
        const long long rows = s.node ? N : E;
        if (mask & s.flag) {
            const int nb = blocks(rows * s.ncomp, 256);
            const bool shared64 = s.host == &des_state_view::coord || s.host == &des_state_view::coord0 ||
                                  s.host == &des_state_view::temperature || s.host == &des_state_view::volume ||
                                  s.host == &des_state_view::volume_old || s.host == &des_state_view::plstrain;
            if (s.host == &des_state_view::stress && f32) {
                k_stress_join<<<blocks(E, 256), 256, 0, st>>>(f.s0, f.stress, dst, E, 0, E);
            } else if (shared64 || !f32) {
                const double *src = s.host == &des_state_view::coord ? d.x
                                  : s.host == &des_state_view::coord0 ? d.x0
                                  : s.host == &des_state_view::temperature ? d.T
                                  : s.host == &des_state_view::volume ? d.vol
                                  : s.host == &des_state_view::volume_old ? d.vol_old
                                  : s.host == &des_state_view::plstrain ? d.pls
                                  : s.host == &des_state_view::vel ? d.vx
                                  : s.host == &des_state_view::force ? d.fx
                                  : s.host == &des_state_view::stress ? d.stress
                                  : s.host == &des_state_view::strain ? d.strain
                                  : s.host == &des_state_view::strain_rate ? d.srate
                                  : d.dpls;
                k_soa_to_aos<<<nb, 256, 0, st>>>(src, dst, s.ncomp, rows, 0, rows);
            } else {
                const float *src = s.host == &des_state_view::vel ? f.vx
                                 : s.host == &des_state_view::force ? f.fx
                                 : s.host == &des_state_view::strain ? f.strain
                                 : s.host == &des_state_view::strain_rate ? f.srate
                                 : f.dpls;
                k_soa_to_aos_f<<<nb, 256, 0, st>>>(src, dst, s.ncomp, rows, 0, rows);
            }
            DES_LAUNCH();
        }
        dst += rows * s.ncomp;
    }
    DES_CUDA(cudaMemcpyAsync(g->snap_clk, g->dclk, sizeof(Clock), cudaMemcpyDeviceToDevice, st));
    DES_CUDA(cudaEventRecord(g->snap_ready, st));
    g->snap_mask = mask;
    return DES_OK;
}

int des_gpu_output_fetch(des_gpu *g, des_state_view *h)
{
    if (!g || !h || !g->snap || h->nnode != g->nnode || h->nelem != g->nelem) return DES_ERR_ARG;
    const long long N = g->nnode, E = g->nelem;
    for (const SnapPart &s : kSnap)
        if ((g->snap_mask & s.flag) && !(h->*(s.host))) return DES_ERR_ARG;
    cudaStream_t cs = g->copy_stream;
    DES_CUDA(cudaStreamWaitEvent(cs, g->snap_ready, 0));
    const double *src = g->snap;
    for (const SnapPart &s : kSnap) {
        const long long n = (s.node ? N : E) * s.ncomp;
        if (g->snap_mask & s.flag)
            DES_CUDA(cudaMemcpyAsync(h->*(s.host), src, sizeof(double) * n, cudaMemcpyDeviceToHost, cs));
        src += n;
    }
    DES_CUDA(cudaEventRecord(g->snap_done, cs));
    return DES_OK;
}

int des_gpu_output_wait(des_gpu *g, des_state_view *h)
{
    if (!g || !g->copy_stream) return DES_ERR_ARG;
    DES_CUDA(cudaStreamSynchronize(g->copy_stream));
    if (h) {
        Clock c;
        DES_CUDA(cudaMemcpy(&c, g->snap_clk, sizeof(Clock), cudaMemcpyDeviceToHost));
        h->time = c.time;
        h->dt = c.dt;
        h->steps = c.steps;
    }
    return DES_OK;
}

int des_gpu_set_averaging(des_gpu *g, int interval)
{
    if (!g || interval < 0) return DES_ERR_ARG;
    if (interval > 0 && !g->avg_c0) {
        const size_t N = g->nnode, E = g->nelem;
        int rc;
        if ((rc = dev_alloc(g, &g->avg_c0, 3 * N)) || (rc = dev_alloc(g, &g->avg_strain0, 6 * E)) ||
            (rc = dev_alloc(g, &g->avg_stress, 6 * E)) || (rc = dev_alloc(g, &g->avg_dpls, E)) ||
            (rc = dev_alloc(g, &g->avg_time0, 1)))
            return rc;
    }
    if (g->graph) cudaGraphExecDestroy(g->graph);
    g->graph = nullptr;
    g->avg_interval = interval;
    return DES_OK;
}

int des_gpu_download_averages(des_gpu *g, double *coord0, double *strain0, double *stress_sum,
                              double *dpls_sum, double *time0)
{
    if (!g) return DES_ERR_ARG;
    if (!g->avg_c0) return DES_ERR_UNSUPPORTED;
    int rc;
    if (coord0 && (rc = download_field(g, coord0, g->avg_c0, 3, g->nnode, g->stream, g->staging))) return rc;
    if (strain0 && (rc = download_field(g, strain0, g->avg_strain0, 6, g->nelem, g->stream, g->staging))) return rc;
    if (stress_sum && (rc = download_field(g, stress_sum, g->avg_stress, 6, g->nelem, g->stream,
                                                 g->staging))) return rc;
    if (dpls_sum && (rc = download_field(g, dpls_sum, g->avg_dpls, 1, g->nelem, g->stream, g->staging))) return rc;
    if (time0) DES_CUDA(cudaMemcpyAsync(time0, g->avg_time0, sizeof(double), cudaMemcpyDeviceToHost, g->stream));
    return finish(g);
}

int des_gpu_set_closure(des_gpu *g, const des_mlp *net)
{
    if (!g) return DES_ERR_ARG;
    if (g->graph) cudaGraphExecDestroy(g->graph);
    g->graph = nullptr;
    if (!net) {
        g->closure = false;
        return DES_OK;
    }
    if (g->prec != DES_PREC_FP32 || (g->hF.rheol != 5 && g->hF.rheol != 7)) return DES_ERR_UNSUPPORTED;
    // the network knows one material mix: its inputs carry no composition
    if (g->hF.nmix != 1) return DES_ERR_UNSUPPORTED;
    if (!(net->tol > 0.f) || !std::isfinite(net->tol)) return DES_ERR_ARG;
    MlpDev h;
    std::memset(&h, 0, sizeof(h));
    for (int o = 0; o < kMlpHid; ++o)
        for (int i = 0; i < kMlpIn; ++i) h.w1[o * kMlpIn + i] = __float2bfloat16(net->w1[o][i]);
    for (int o = 0; o < kMlpHid; ++o)
        for (int i = 0; i < kMlpHid; ++i) h.w2[o * kMlpHid + i] = __float2bfloat16(net->w2[o][i]);
    for (int o = 0; o < kMlpOut; ++o)
        for (int i = 0; i < kMlpHid; ++i)
            h.w3[o * kMlpHid + i] = __float2bfloat16(o < kMlpOutUsed ? net->w3[o][i] : 0.f);
    for (int i = 0; i < kMlpHid; ++i) {
        h.b1[i] = net->b1[i];
        h.b2[i] = net->b2[i];
    }
    for (int i = 0; i < kMlpOut; ++i) {
        h.b3[i] = i < kMlpOutUsed ? net->b3[i] : 0.f;
        h.out_scale[i] = net->out_scale[i];
    }
    for (int i = 0; i < kMlpIn; ++i) {
        h.in_mean[i] = net->in_mean[i];
        h.in_scale[i] = net->in_scale[i];
        h.env_lo[i] = net->env_lo[i];
        h.env_hi[i] = net->env_hi[i];
    }
    h.tol = net->tol;
    if (!g->dnet) {
        int rc = dev_alloc(g, &g->dnet, 1);
        if (rc) return rc;
    }
    DES_CUDA(cudaMemcpyAsync(g->dnet, &h, sizeof(h), cudaMemcpyHostToDevice, g->stream));
    DES_CUDA(cudaStreamSynchronize(g->stream));
    g->closure = true;
    return DES_OK;
}

int des_gpu_log_returns(des_gpu *g, int nsteps, float *records, long long capacity, long long *count)
{
    if (!g || nsteps < 1 || capacity < 1 || !records || !count) return DES_ERR_ARG;
    if (g->prec != DES_PREC_FP64) return DES_ERR_UNSUPPORTED;
    if (int rc = prime(g)) return rc;
    float *buf = nullptr;
    if (cudaMalloc(&buf, sizeof(float) * kRetRecord * (size_t)capacity) != cudaSuccess) return DES_ERR_NOMEM;
    const unsigned long long zero = 0;
    int rc = cuda_rc(cudaMemcpyAsync(&g->dclk->nlog, &zero, sizeof(zero), cudaMemcpyHostToDevice, g->stream));
    if (!rc) {
        g->d.ret_log = buf;
        g->d.ret_cap = capacity;
        for (int s = 0; s < nsteps; ++s) launch_step(g, nullptr);
        g->d.ret_log = nullptr;
        g->d.ret_cap = 0;
        rc = finish(g);
    }
    Clock c;
    if (!rc) rc = read_clock(g, c);
    if (!rc) {
        *count = (long long)c.nlog;
        const long long n = std::min<long long>((long long)c.nlog, capacity);
        if (n > 0)
            rc = cuda_rc(cudaMemcpy(records, buf, sizeof(float) * kRetRecord * (size_t)n, cudaMemcpyDeviceToHost));
    }
    cudaFree(buf);
    return rc;
}

int des_gpu_step(des_gpu *g, int nsteps, des_step_report *report)
{
    if (!g || nsteps < 0) return DES_ERR_ARG;
    if (int rc = prime(g)) return rc;
    if (!g->graph) {
        int rc = capture_step_graph(g);
        if (rc) return rc;
    }
    for (int i = 0; i < nsteps; ++i) DES_CUDA(cudaGraphLaunch(g->graph, g->stream));
    if (!report) return DES_OK;
    int rc = des_gpu_report(g, report);
    if (rc) return rc;
    // the reference stops with exit code 11 on both (geometry.cxx:321-325,
    // output.cxx:195-208)
    if (report->status & (DES_STATUS_DT_NONPOSITIVE | DES_STATUS_NONFINITE)) return DES_ERR_DT;
    return DES_OK;
}

int des_gpu_time_steps(des_gpu *g, int nsteps, double *ms)
{
    if (!g || nsteps < 0 || !ms) return DES_ERR_ARG;
    if (int rc = prime(g)) return rc;
    if (!g->graph) {
        int rc = capture_step_graph(g);
        if (rc) return rc;
    }
    cudaEvent_t a, b;
    DES_CUDA(cudaEventCreate(&a));
    DES_CUDA(cudaEventCreate(&b));
    DES_CUDA(cudaStreamSynchronize(g->stream));
    DES_CUDA(cudaEventRecord(a, g->stream));
    for (int i = 0; i < nsteps; ++i) DES_CUDA(cudaGraphLaunch(g->graph, g->stream));
    DES_CUDA(cudaEventRecord(b, g->stream));
    DES_CUDA(cudaEventSynchronize(b));
    float f = 0;
    DES_CUDA(cudaEventElapsedTime(&f, a, b));
    *ms = f;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return DES_OK;
}

int des_gpu_profile_steps(des_gpu *g, int nsteps, double ms[6])
{
    if (!g || nsteps < 0 || !ms) return DES_ERR_ARG;
    if (int rc = prime(g)) return rc;
    cudaEvent_t ev[7];
    for (int i = 0; i < 7; ++i) DES_CUDA(cudaEventCreate(&ev[i]));
    for (int k = 0; k < 6; ++k) ms[k] = 0;
    DES_CUDA(cudaStreamSynchronize(g->stream));
    for (int s = 0; s < nsteps; ++s) {
        launch_step(g, ev);
        DES_LAUNCH();
        DES_CUDA(cudaEventSynchronize(ev[6]));
        for (int k = 0; k < 6; ++k) {
            float f = 0;
            cudaEventElapsedTime(&f, ev[k], ev[k + 1]);
            ms[k] += f;
        }
    }
    for (int i = 0; i < 7; ++i) cudaEventDestroy(ev[i]);
    return DES_OK;
}

int des_host_register(void *ptr, long long bytes)
{
    if (!ptr || bytes <= 0) return DES_ERR_ARG;
    return cuda_rc(cudaHostRegister(ptr, (size_t)bytes, cudaHostRegisterDefault));
}
int des_host_unregister(void *ptr)
{
    if (!ptr) return DES_ERR_ARG;
    return cuda_rc(cudaHostUnregister(ptr));
}
void des_abi_sizes(long long out[5])
{
    out[0] = sizeof(des_params);
    out[1] = sizeof(des_mesh_view);
    out[2] = sizeof(des_state_view);
    out[3] = sizeof(des_topology);
    out[4] = sizeof(des_step_report);
}

// fields the loop body overwrites before it reads them (update_force,
// update_strain_rate, compute_edvoldt, update_stress, the scratch arrays):
// des_gpu_step_host downloads but does not upload them
constexpr unsigned kStepOutputs =
    DES_F_FORCE | DES_F_NTMP | DES_F_STRAIN_RATE | DES_F_DPRESSURE | DES_F_EDVOLDT | DES_F_TMP_RESULT;
// fields that no pass after pass k (N-A, E-B, N-B, E-C, N-C) writes; E-A
// writes none of them (coordinates, velocity and temperature it only reads)
constexpr unsigned kFinishedAfterPass[5] = {
    DES_F_TEMPERATURE | DES_F_COORD0,
    DES_F_PLSTRAIN | DES_F_STRAIN_RATE | DES_F_DPRESSURE | DES_F_EDVOLDT,
    DES_F_NTMP,
    0,
    DES_F_COORD | DES_F_VEL | DES_F_FORCE};
constexpr unsigned kBeforeLastPass = kFinishedAfterPass[0] | kFinishedAfterPass[1] | kFinishedAfterPass[2] |
                                     kFinishedAfterPass[3] | kFinishedAfterPass[4];

// One element field of the overlapped upload: its host rows and where they go.
struct UpPart {
    const double *host;
    int ncomp;
    double *dst64;
    float *dst32;
    bool stress_split;
};

static std::vector<UpPart> up_parts(des_gpu *g, const des_state_view *h, unsigned later)
{
    const bool f32 = g->prec == DES_PREC_FP32;
    std::vector<UpPart> out;
    out.push_back({h->volume_old, 1, g->d.vol_old, nullptr, false});
    if (later & DES_F_STRESS) out.push_back({h->stress, 6, g->d.stress, nullptr, false});
    if (later & DES_F_STRAIN)
        out.push_back({h->strain, 6, f32 ? nullptr : g->d.strain, f32 ? g->f.strain : nullptr, false});
    if (later & DES_F_PLSTRAIN) {
        out.push_back({h->plstrain, 1, g->d.pls, nullptr, false});
        out.push_back({h->delta_plstrain, 1, f32 ? nullptr : g->d.dpls, f32 ? g->f.dpls : nullptr, false});
    }
    return out;
}

// the host rows of volume_old and the `later` fields into the download
// buffer (sized here for this call's downloads too, `down` doubles), by the
// copy engine on the copy stream
static int upload_elements_async(des_gpu *g, const des_state_view *h, unsigned later, long long down)
{
    const long long E = g->nelem;
    std::vector<UpPart> parts = up_parts(g, h, later);
    long long need = 0;
    for (const UpPart &q : parts) {
        if (!q.host) return DES_ERR_ARG;
        need += q.ncomp * E;
    }
    int rc;
    if ((rc = ensure_copy_stream(g)) || (rc = ensure_download_buffer(g, std::max(need, down)))) return rc;
    // the buffer's previous contents have left on the copy stream
    DES_CUDA(cudaStreamSynchronize(g->copy_stream));
    long long off = 0;
    for (const UpPart &q : parts) {
        DES_CUDA(cudaMemcpyAsync(g->dl + off, q.host, sizeof(double) * q.ncomp * E, cudaMemcpyHostToDevice,
                                 g->copy_stream));
        off += q.ncomp * E;
    }
    DES_CUDA(cudaEventRecord(g->up_done, g->copy_stream));
    return DES_OK;
}

// the uploaded rows into the device's arrays, once the copies are done
static int finish_elements_async(des_gpu *g, const des_state_view *h, unsigned later)
{
    const long long E = g->nelem;
    DES_CUDA(cudaStreamWaitEvent(g->stream, g->up_done, 0));
    long long off = 0;
    for (const UpPart &q : up_parts(g, h, later)) {
        const double *src = g->dl + off;
        if (q.dst64)
            k_aos_to_soa<<<blocks(E * q.ncomp, 256), 256, 0, g->stream>>>(src, q.dst64, q.ncomp, E, 0, E);
        else
            k_aos_to_soa_f<<<blocks(E * q.ncomp, 256), 256, 0, g->stream>>>(src, q.dst32, q.ncomp, E, 0, E);
        DES_LAUNCH();
        off += q.ncomp * E;
    }
    g->primed = false;
    return DES_OK;
}

// volume, shape derivatives and nodal masses from the device's coordinates
// and temperature, the values update_mesh (dynearthsol.cxx:237-261) leaves
static int derive_geometry(des_gpu *g)
{
    const int eb = blocks(g->nelem, kElemBlock), nb = blocks(g->nnode, kNodeBlock);
    cudaStream_t s = g->stream;
    if (g->prec == DES_PREC_FP32) {
        kf_derive_geometry<<<eb, kElemBlock, 0, s>>>(g->f);
        kf_mass_flush<<<nb, kNodeBlock, 0, s>>>(g->f);
    } else {
        k_volume<<<eb, kElemBlock, 0, s>>>(g->d, 0);
        k_shape<<<eb, kElemBlock, 0, s>>>(g->d);
        k_mass_elem<<<eb, kElemBlock, 0, s>>>(g->d, g->d.T);
        k_mass_node<<<nb, kNodeBlock, 0, s>>>(g->d);
    }
    DES_LAUNCH();
    Clock c;
    if (int rc = read_clock(g, c)) return rc;
    k_clock_set<<<1, 32, 0, g->stream>>>(g->dclk, c.time, c.dt, c.steps, 1);
    DES_LAUNCH();
    g->primed = false;
    return finish(g);
}

// the end of a host-buffer step once passes N-A .. N-C are queued and their
// fields are on their way down (the download buffer filled up to off): E-A in
// element chunks, each chunk's rows of the element fields going to the host
// while the next chunk computes, then the averaging, the clock, the nodal
// masses and the late nodal fields
static int step_host_tail(des_gpu *g, des_state_view *host, unsigned mask, const std::vector<DownPart> &late,
                          long long off, des_step_report *report)
{
    int rc = DES_OK;
    std::vector<DownPart> late_elem, late_node;
    for (const DownPart &q : late) (q.elem ? late_elem : late_node).push_back(q);
    const int nb = blocks(g->nelem, kElemBlock), nchunk = std::min(kEaChunks, nb);
    std::vector<long long> base(late_elem.size());
    for (size_t i = 0; i < late_elem.size(); ++i) {
        base[i] = off;
        off += late_elem[i].ncomp * late_elem[i].rows;
    }
    for (int k = 0; k < nchunk && !rc; ++k) {
        const int b0 = (int)((long long)nb * k / nchunk), b1 = (int)((long long)nb * (k + 1) / nchunk);
        launch_ea(g, b0, b1);
        rc = cuda_rc(cudaGetLastError());
        const long long r0 = (long long)b0 * kElemBlock;
        const long long r1 = std::min<long long>((long long)b1 * kElemBlock, g->nelem);
        for (size_t i = 0; i < late_elem.size() && !rc; ++i)
            rc = download_rows_async(g, late_elem[i], base[i], r0, r1 - r0);
    }
    if (!rc) {
        launch_average(g);
        rc = cuda_rc(cudaGetLastError());
    }
    Clock c = {};
    if (!rc) rc = read_clock(g, c);
    if (!rc && report && (rc = des_gpu_report(g, report)) == DES_OK &&
        (report->status & (DES_STATUS_DT_NONPOSITIVE | DES_STATUS_NONFINITE)))
        rc = DES_ERR_DT;
    if (!rc && (mask & DES_F_MASS)) rc = flush_masses(g, c);
    if (!rc) rc = download_async(g, late_node, &off);
    const cudaError_t ce = cudaStreamSynchronize(g->copy_stream);
    if (rc) return rc;
    if (ce != cudaSuccess) return DES_ERR_CUDA;
    if (mask & DES_F_SCALARS) {
        host->time = c.time;
        host->dt = c.dt;
        host->steps = c.steps;
    }
    return finish(g);
}

// One step from host buffers with the element fields E-B reads (`later`)
// coming up chunk by chunk on the upload stream while the geometry is
// derived and N-A runs: E-B runs on each chunk as it lands, and in the FP64
// form the fields E-B finishes go down chunk by chunk on the copy stream
// while later chunks still come up, so the two directions of the host link
// run at once.  (The FP32 form's list kernels follow the last chunk, so its
// E-B fields go down whole.)
static int step_host_pipelined(des_gpu *g, des_state_view *host, unsigned mask, unsigned later,
                               des_step_report *report)
{
    const long long E = g->nelem;
    int rc;
    const std::vector<UpPart> ups = up_parts(g, host, later);
    long long U = 0;
    for (const UpPart &q : ups) {
        if (!q.host) return DES_ERR_ARG;
        U += q.ncomp * E;
    }
    std::vector<DownPart> all, late, eb;
    if ((rc = down_parts(g, host, mask, all)) || (rc = down_parts(g, host, mask & ~kBeforeLastPass, late)) ||
        (rc = down_parts(g, host, mask & kFinishedAfterPass[1], eb)))
        return rc;
    long long D = 0;
    for (const DownPart &q : all) D += q.ncomp * q.rows;
    if ((rc = ensure_copy_stream(g)) || (rc = ensure_download_buffer(g, U + D))) return rc;
    // the buffer's previous contents have left
    DES_CUDA(cudaStreamSynchronize(g->copy_stream));
    DES_CUDA(cudaStreamSynchronize(g->up_stream));
    const int nb = blocks(E, kElemBlock), nchunk = std::min(kEbChunks, nb);
    auto chunk_block = [&](int k) { return (int)((long long)nb * k / nchunk); };
    auto block_row = [&](int b) { return std::min<long long>((long long)b * kElemBlock, E); };
    // uploads into the buffer's first U doubles: each part's host rows at the
    // part's place, chunk by chunk, one event per chunk
    for (int k = 0; k < nchunk; ++k) {
        const long long r0 = block_row(chunk_block(k)), r1 = block_row(chunk_block(k + 1));
        long long uoff = 0;
        for (const UpPart &q : ups) {
            DES_CUDA(cudaMemcpyAsync(g->dl + uoff + r0 * q.ncomp, q.host + r0 * q.ncomp,
                                     sizeof(double) * q.ncomp * (r1 - r0), cudaMemcpyHostToDevice,
                                     g->up_stream));
            uoff += q.ncomp * E;
        }
        DES_CUDA(cudaEventRecord(g->up_chunk[k], g->up_stream));
    }
    // volume, shape derivatives and masses from the coordinates, the
    // next-step contributions (neither reads the `later` fields), N-A
    if ((rc = derive_geometry(g)) || (rc = prime(g))) return rc;
    long long off = U;
    launch_pass(g, 0);
    if ((rc = cuda_rc(cudaGetLastError()))) return rc;
    {
        std::vector<DownPart> done;
        if ((rc = down_parts(g, host, mask & kFinishedAfterPass[0], done)) || (rc = download_async(g, done, &off)))
            return rc;
    }
    // E-B chunk by chunk as its inputs land
    std::vector<long long> ebase(eb.size());
    for (size_t i = 0; i < eb.size(); ++i) {
        ebase[i] = off;
        off += eb[i].ncomp * eb[i].rows;
    }
    const bool per_chunk = g->prec == DES_PREC_FP64;
    for (int k = 0; k < nchunk && !rc; ++k) {
        const int b0 = chunk_block(k), b1 = chunk_block(k + 1);
        const long long r0 = block_row(b0), nr = block_row(b1) - r0;
        DES_CUDA(cudaStreamWaitEvent(g->stream, g->up_chunk[k], 0));
        long long uoff = 0;
        for (const UpPart &q : ups) {
            const double *src = g->dl + uoff + r0 * q.ncomp;
            if (q.dst64)
                k_aos_to_soa<<<blocks(nr * q.ncomp, 256), 256, 0, g->stream>>>(src, q.dst64, q.ncomp, nr, r0, E);
            else
                k_aos_to_soa_f<<<blocks(nr * q.ncomp, 256), 256, 0, g->stream>>>(src, q.dst32, q.ncomp, nr, r0, E);
            uoff += q.ncomp * E;
        }
        launch_eb_first(g, b0, b1);
        rc = cuda_rc(cudaGetLastError());
        if (per_chunk)
            for (size_t i = 0; i < eb.size() && !rc; ++i) rc = download_rows_async(g, eb[i], ebase[i], r0, nr);
    }
    if (rc) return rc;
    launch_eb_rest(g);
    if ((rc = cuda_rc(cudaGetLastError()))) return rc;
    if (!per_chunk)
        for (size_t i = 0; i < eb.size() && !rc; ++i) rc = download_rows_async(g, eb[i], ebase[i], 0, eb[i].rows);
    // N-B, E-C, N-C, each field going down after the pass that finishes it
    for (int k = 2; k < 5 && !rc; ++k) {
        launch_pass(g, k);
        rc = cuda_rc(cudaGetLastError());
        std::vector<DownPart> done;
        if (!rc) rc = down_parts(g, host, mask & kFinishedAfterPass[k], done);
        if (!rc) rc = download_async(g, done, &off);
    }
    if (rc) return rc;
    return step_host_tail(g, host, mask, late, off, report);
}

int des_gpu_step_host(des_gpu *g, des_state_view *host, unsigned mask, int nsteps,
                      des_step_report *report)
{
    if (!g || !host || nsteps < 0) return DES_ERR_ARG;
    unsigned up = mask & ~kStepOutputs;
    // with coordinates and temperature in hand, volume, shape derivatives and
    // masses are recomputed on the device rather than copied (1.0 GB fewer
    // host-to-device bytes per step for 9.6M elements); volume_old is copied
    const unsigned derived = DES_F_VOLUME | DES_F_SHAPE | DES_F_MASS;
    const bool derive = (up & DES_F_COORD) && (up & DES_F_TEMPERATURE) && (up & derived) == derived;
    if (derive) up &= ~derived;
    // while the geometry is derived, the element fields it does not read come
    // over the copy engine on a second stream (the FP32 form's derivation
    // reads the reference stress, so its stress is uploaded first)
    unsigned later = 0;
    if (derive) later = up & (DES_F_STRAIN | DES_F_PLSTRAIN | (g->prec == DES_PREC_FP64 ? DES_F_STRESS : 0u));
    int rc = des_gpu_upload(g, host, up & ~later);
    if (rc) return rc;
    if (derive && host->nelem == g->nelem && host->volume_old && nsteps == 1)
        return step_host_pipelined(g, host, mask, later, report);
    if (derive) {
        if (host->nelem != g->nelem || !host->volume_old) return DES_ERR_ARG;
        std::vector<DownPart> all;
        if ((rc = down_parts(g, host, mask, all))) return rc;
        long long down = 0;
        for (const DownPart &q : all) down += q.ncomp * q.rows;
        if ((rc = upload_elements_async(g, host, later, down))) return rc;
        if ((rc = derive_geometry(g))) return rc;
        if ((rc = finish_elements_async(g, host, later))) return rc;
    }
    if (nsteps == 0) return des_gpu_download(g, host, mask);
    // every step but the last as the graph; the last as its passes, so that
    // the fields finished before E-A download on the copy stream while E-A
    // runs (the host link is the bound of this entry point)
    if (nsteps > 1 && (rc = des_gpu_step(g, nsteps - 1, nullptr))) return rc;
    if ((rc = prime(g))) return rc;
    std::vector<DownPart> all, late;
    if ((rc = down_parts(g, host, mask, all)) || (rc = down_parts(g, host, mask & ~kBeforeLastPass, late)))
        return rc;
    long long need = 0;
    for (const DownPart &q : all) need += q.ncomp * q.rows;
    if ((rc = ensure_copy_stream(g)) || (rc = ensure_download_buffer(g, need))) return rc;
    long long off = 0;
    // each field downloads after the pass that finishes it
    for (int k = 0; k < 5 && !rc; ++k) {
        launch_pass(g, k);
        rc = cuda_rc(cudaGetLastError());
        std::vector<DownPart> done;
        if (!rc) rc = down_parts(g, host, mask & kFinishedAfterPass[k], done);
        if (!rc) rc = download_async(g, done, &off);
    }
    if (rc) return rc;
    return step_host_tail(g, host, mask, late, off, report);
}

// remesh (remeshing.cxx:1963-2067) after the host's new mesh, interpolation
// and marker remap: a fresh device state for the new mesh takes the handle's
// place, with the interpolated fields and the handle's clock, closure and
// averaging settings
int des_gpu_remesh(des_gpu *g, const des_mesh_view *mesh, const des_state_view *host,
                   int reset_bottom_coord0)
{
    if (!g || !mesh || !host) return DES_ERR_ARG;
    if (host->nnode != mesh->nnode || host->nelem != mesh->nelem || mesh->nmat != g->nmat) return DES_ERR_ARG;
    if (!host->coord || !host->coord0 || !host->vel || !host->temperature || !host->plstrain ||
        !host->delta_plstrain || !host->strain || !host->stress)
        return DES_ERR_ARG;
    Clock c;
    int rc = read_clock(g, c);
    if (rc) return rc;
    if (g->copy_stream) DES_CUDA(cudaStreamSynchronize(g->copy_stream));
    des_gpu *ng = nullptr;
    if ((rc = des_gpu_create(mesh, &g->P, g->device, &ng))) return rc;
    auto fail = [&](int code) {
        des_gpu_destroy(ng);
        return code;
    };
    if (g->closure) {
        // the network was trained on one material mix
        if (ng->mix_counts != g->mix_counts) return fail(DES_ERR_UNSUPPORTED);
        if ((rc = dev_alloc(ng, &ng->dnet, 1))) return fail(rc);
        if (cudaMemcpy(ng->dnet, g->dnet, sizeof(MlpDev), cudaMemcpyDeviceToDevice) != cudaSuccess)
            return fail(DES_ERR_CUDA);
        ng->closure = true;
    }
    // averaging restarts with the next step (remeshing falls on an
    // interval's last step, output.cxx:229-233)
    if (g->avg_interval > 0 && (rc = des_gpu_set_averaging(ng, g->avg_interval))) return fail(rc);
    // the fields remesh interpolates (brc-interpolation.cxx:219-242,
    // nn-interpolation.cxx:290-325); the rest is reallocated (fields.cxx:57-105)
    const unsigned interpolated = DES_F_COORD | DES_F_COORD0 | DES_F_VEL | DES_F_TEMPERATURE |
                                  DES_F_PLSTRAIN | DES_F_STRAIN | DES_F_STRESS;
    if ((rc = des_gpu_upload(ng, host, interpolated))) return fail(rc);
    if (reset_bottom_coord0) {
        k_reset_bottom_coord0<<<blocks(ng->nnode, kNodeBlock), kNodeBlock, 0, ng->stream>>>(ng->d,
                                                                                       -ng->P.zlength);
        if (cudaGetLastError() != cudaSuccess) return fail(DES_ERR_CUDA);
    }
    k_clock_set<<<1, 32, 0, ng->stream>>>(ng->dclk, c.time, c.dt, c.steps, 1);
    if (cudaGetLastError() != cudaSuccess) return fail(DES_ERR_CUDA);
    // compute_volume, volume_old = volume, compute_mass, compute_shape_fn
    if ((rc = derive_geometry(ng))) return fail(rc);
    if (cudaMemcpyAsync(ng->d.vol_old, ng->d.vol, sizeof(double) * (size_t)ng->nelem,
                        cudaMemcpyDeviceToDevice, ng->stream) != cudaSuccess)
        return fail(DES_ERR_CUDA);
    if ((rc = finish(ng))) return fail(rc);
    std::swap(*g, *ng);
    des_gpu_destroy(ng);
    return DES_OK;
}

#define ELEM_GRID(g) blocks((g)->nelem, kElemBlock), kElemBlock, 0, (g)->stream
#define NODE_GRID(g) blocks((g)->nnode, kNodeBlock), kNodeBlock, 0, (g)->stream

int des_gpu_update_temperature(des_gpu *g)
{
    int rc = begin_fn64(g);
    if (rc) return rc;
    k_temp_elem<<<ELEM_GRID(g)>>>(g->d);
    k_temp_node<<<NODE_GRID(g)>>>(g->d);
    return finish(g);
}
int des_gpu_update_strain_rate(des_gpu *g)
{
    int rc = begin_fn64(g);
    if (rc) return rc;
    k_srate<<<ELEM_GRID(g)>>>(g->d, g->d.srate);
    return finish(g);
}
int des_gpu_compute_dvoldt(des_gpu *g)
{
    int rc = begin_fn64(g);
    if (rc) return rc;
    k_dvoldt_elem<<<ELEM_GRID(g)>>>(g->d);
    k_sg_gather<<<NODE_GRID(g)>>>(g->d);
    return finish(g);
}
int des_gpu_compute_edvoldt(des_gpu *g)
{
    int rc = begin_fn64(g);
    if (rc) return rc;
    k_edvoldt<<<ELEM_GRID(g)>>>(g->d);
    return finish(g);
}
int des_gpu_update_stress(des_gpu *g)
{
    int rc = begin_fn64(g);
    if (rc) return rc;
    k_stress<<<ELEM_GRID(g)>>>(g->d);
    return finish(g);
}
int des_gpu_NMD_stress(des_gpu *g)
{
    int rc = begin_fn64(g);
    if (rc) return rc;
    k_dp_elem<<<ELEM_GRID(g)>>>(g->d);
    k_sg_gather<<<NODE_GRID(g)>>>(g->d);
    k_nmd_apply<<<ELEM_GRID(g)>>>(g->d);
    return finish(g);
}
int des_gpu_update_force(des_gpu *g)
{
    int rc = begin_fn64(g);
    if (rc) return rc;
    k_force_elem<<<ELEM_GRID(g)>>>(g->d);
    if (g->hK.stress_bc_sides && g->d.bf.nbf > 0)
        k_stress_bc_facets<<<blocks(g->d.bf.nbf, 128), 128, 0, g->stream>>>(g->d);
    k_force_node<<<NODE_GRID(g)>>>(g->d, g->hK.is_qs);
    return finish(g);
}
int des_gpu_update_velocity(des_gpu *g)
{
    int rc = begin_fn64(g);
    if (rc) return rc;
    k_velocity<<<NODE_GRID(g)>>>(g->d);
    return finish(g);
}
int des_gpu_apply_vbcs(des_gpu *g)
{
    int rc = begin_fn64(g);
    if (rc) return rc;
    k_vbcs<<<NODE_GRID(g)>>>(g->d);
    return finish(g);
}
int des_gpu_update_coordinate(des_gpu *g)
{
    int rc = begin_fn64(g);
    if (rc) return rc;
    k_coord<<<NODE_GRID(g)>>>(g->d);
    return finish(g);
}
int des_gpu_compute_volume(des_gpu *g)
{
    int rc = begin_fn64(g);
    if (rc) return rc;
    k_volume<<<ELEM_GRID(g)>>>(g->d, 0);
    return finish(g);
}
int des_gpu_compute_mass(des_gpu *g)
{
    int rc = begin_fn64(g);
    if (rc) return rc;
    k_mass_elem<<<ELEM_GRID(g)>>>(g->d, g->d.T);
    k_mass_node<<<NODE_GRID(g)>>>(g->d);
    k_clock_mass_valid<<<1, 32, 0, g->stream>>>(g->dclk, 1);
    return finish(g);
}
int des_gpu_compute_shape_fn(des_gpu *g)
{
    int rc = begin_fn64(g);
    if (rc) return rc;
    k_shape<<<ELEM_GRID(g)>>>(g->d);
    return finish(g);
}
int des_gpu_update_mesh(des_gpu *g)
{
    int rc = begin_fn64(g);
    if (rc) return rc;
    k_coord<<<NODE_GRID(g)>>>(g->d);
    launch_surface(g);
    k_volume<<<ELEM_GRID(g)>>>(g->d, 1);
    k_mass_elem<<<ELEM_GRID(g)>>>(g->d, g->d.T);
    k_mass_node<<<NODE_GRID(g)>>>(g->d);
    k_clock_mass_valid<<<1, 32, 0, g->stream>>>(g->dclk, 1);
    k_shape<<<ELEM_GRID(g)>>>(g->d);
    return finish(g);
}
int des_gpu_rotate_stress(des_gpu *g)
{
    int rc = begin_fn64(g);
    if (rc) return rc;
    k_rotate<<<ELEM_GRID(g)>>>(g->d);
    return finish(g);
}
int des_gpu_compute_dt(des_gpu *g, double *dt_out)
{
    int rc = begin_fn(g);
    if (rc) return rc;
    if (g->P.fixed_dt != 0) {
        k_clock_dt<<<1, 32, 0, g->stream>>>(g->dclk, g->P.fixed_dt);
    } else {
        k_dt<<<ELEM_GRID(g)>>>(g->d);
    }
    if ((rc = finish(g))) return rc;
    Clock c;
    if ((rc = read_clock(g, c))) return rc;
    if (dt_out) *dt_out = c.dt;
    return (c.dt > 0) ? DES_OK : DES_ERR_DT;
}

// compute_volume on caller arrays in the reference layout (AoS coordinates)
__global__ void k_volume_rows(int nelem, const double *__restrict__ coord,
                              const int4 *__restrict__ conn, double *__restrict__ vol)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nelem) return;
    int4 q = conn[e];
    const int n[4] = {q.x, q.y, q.z, q.w};
    double X[4][3];
    for (int i = 0; i < 4; ++i)
        for (int k = 0; k < 3; ++k) X[i][k] = coord[3LL * n[i] + k];
    vol[e] = tet_volume(X[0], X[1], X[2], X[3]);
}

int des_compute_volume(int nnode, int nelem, const double *coord, const int *connectivity,
                       double *volume)
{
    if (nnode < 1 || nelem < 1 || !coord || !connectivity || !volume) return DES_ERR_ARG;
    double *dx = nullptr, *dv = nullptr;
    int *dc = nullptr;
    cudaStream_t s = nullptr;
    int rc = cuda_rc(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    if (!rc && (cudaMalloc(&dx, sizeof(double) * 3 * (size_t)nnode) != cudaSuccess ||
                cudaMalloc(&dc, sizeof(int) * 4 * (size_t)nelem) != cudaSuccess ||
                cudaMalloc(&dv, sizeof(double) * (size_t)nelem) != cudaSuccess))
        rc = DES_ERR_NOMEM;
    if (!rc) rc = cuda_rc(cudaMemcpyAsync(dx, coord, sizeof(double) * 3 * (size_t)nnode,
                                          cudaMemcpyHostToDevice, s));
    if (!rc) rc = cuda_rc(cudaMemcpyAsync(dc, connectivity, sizeof(int) * 4 * (size_t)nelem,
                                          cudaMemcpyHostToDevice, s));
    if (!rc) {
        k_volume_rows<<<blocks(nelem, kElemBlock), kElemBlock, 0, s>>>(
            nelem, dx, reinterpret_cast<const int4 *>(dc), dv);
        rc = cuda_rc(cudaGetLastError());
    }
    if (!rc) rc = cuda_rc(cudaMemcpyAsync(volume, dv, sizeof(double) * (size_t)nelem,
                                          cudaMemcpyDeviceToHost, s));
    if (!rc) rc = cuda_rc(cudaStreamSynchronize(s));
    cudaFree(dx);
    cudaFree(dc);
    cudaFree(dv);
    if (s) cudaStreamDestroy(s);
    return rc;
}

static int init_fields_fp32(des_gpu *g)
{
    const size_t N = g->nnode, E = g->nelem;
    DevF &f = g->f;
    cudaStream_t s = g->stream;
    g->primed = false;
    DES_CUDA(cudaMemsetAsync(f.vx, 0, sizeof(float) * 3 * N, s));
    DES_CUDA(cudaMemsetAsync(f.fx, 0, sizeof(float) * 3 * N, s));
    DES_CUDA(cudaMemsetAsync(f.stress, 0, sizeof(float) * 6 * E, s));
    DES_CUDA(cudaMemsetAsync(f.s0, 0, sizeof(double) * E, s));
    DES_CUDA(cudaMemsetAsync(f.strain, 0, sizeof(float) * 6 * E, s));
    DES_CUDA(cudaMemsetAsync(f.srate, 0, sizeof(float) * 6 * E, s));
    DES_CUDA(cudaMemcpyAsync(f.x0, f.x, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, s));
    kf_init_geometry<<<ELEM_GRID(g)>>>(f);
    kf_mass_flush<<<NODE_GRID(g)>>>(f);
    k_clock_set<<<1, 32, 0, s>>>(g->dclk, 0.0, 0.0, 0, 1);
    kf_vbcs<<<NODE_GRID(g)>>>(f);
    if (g->P.gravity != 0) kf_init_stress<<<ELEM_GRID(g)>>>(f);
    return DES_OK;
}

int des_gpu_init_fields(des_gpu *g)
{
    if (!g) return DES_ERR_ARG;
    if (g->prec == DES_PREC_FP32) {
        int rc = init_fields_fp32(g);
        if (rc) return rc;
        g->P.compensation_pressure =
            g->P.gravity != 0 ? ref_pressure(g->P.ref_pressure_option, g->P.rho0.v[0], g->P.gravity, -g->P.zlength)
                              : 0;
        g->hK.compensation_pressure = g->P.compensation_pressure;
        DES_CUDA(cudaMemcpyAsync(&g->dK->compensation_pressure, &g->hK.compensation_pressure,
                                 sizeof(double), cudaMemcpyHostToDevice, g->stream));
        if ((rc = finish(g))) return rc;
        double dt;
        return des_gpu_compute_dt(g, &dt);
    }
    const size_t N = g->nnode, E = g->nelem;
    Dev &d = g->d;
    g->primed = false;
    cudaStream_t s = g->stream;
    DES_CUDA(cudaMemsetAsync(d.vx, 0, sizeof(double) * 3 * N, s));
    DES_CUDA(cudaMemsetAsync(d.fx, 0, sizeof(double) * 3 * N, s));
    DES_CUDA(cudaMemsetAsync(d.stress, 0, sizeof(double) * 6 * E, s));
    DES_CUDA(cudaMemsetAsync(d.strain, 0, sizeof(double) * 6 * E, s));
    DES_CUDA(cudaMemsetAsync(d.srate, 0, sizeof(double) * 6 * E, s));
    DES_CUDA(cudaMemcpyAsync(d.x0, d.x, sizeof(double) * 3 * N, cudaMemcpyDeviceToDevice, s));
    k_volume<<<ELEM_GRID(g)>>>(d, 0);
    DES_CUDA(cudaMemcpyAsync(d.vol_old, d.vol, sizeof(double) * E, cudaMemcpyDeviceToDevice, s));
    k_mass_elem<<<ELEM_GRID(g)>>>(d, nullptr);
    k_mass_node<<<NODE_GRID(g)>>>(d);
    k_clock_set<<<1, 32, 0, s>>>(g->dclk, 0.0, 0.0, 0, 1);
    k_shape<<<ELEM_GRID(g)>>>(d);
    k_vbcs<<<NODE_GRID(g)>>>(d);
    if (g->P.gravity != 0) {
        k_init_stress<<<ELEM_GRID(g)>>>(d);
        g->P.compensation_pressure =
            ref_pressure(g->P.ref_pressure_option, g->P.rho0.v[0], g->P.gravity, -g->P.zlength);
    } else {
        g->P.compensation_pressure = 0;
    }
    g->hK.compensation_pressure = g->P.compensation_pressure;
    DES_CUDA(cudaMemcpyAsync(&g->dK->compensation_pressure, &g->hK.compensation_pressure,
                             sizeof(double), cudaMemcpyHostToDevice, s));
    int rc = finish(g);
    if (rc) return rc;
    double dt;
    return des_gpu_compute_dt(g, &dt);
}

}  // extern "C"
