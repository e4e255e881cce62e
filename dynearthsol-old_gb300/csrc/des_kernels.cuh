// Kernels of the FP64 step.  Two families share the device arithmetic of
// des_device.cuh:
//  * one kernel (or elem + node pair) per reference function, operating on
//    the reference's fields, used by the per-function entry points;
//  * six fused passes per time step (node / element alternating), captured
//    into one CUDA graph:
//      N-A  nodal masses (if stale), dvoldt gather, tdot gather + T update
//      E-B  edvoldt, update_stress, dp * volume
//      N-B  dp_nd gather
//      E-C  NMD correction, element force vectors
//      N-C  force gather, damping, velocity, velocity BCs, coordinates
//      E-A  volume, shape functions, mass contributions, rotate_stress,
//           next strain rate, dvoldt and conduction contributions, dt minimum
// Every nodal sum runs over the node's support list in ascending element
// order, as the reference's node loops do, so sums are bit-identical and
// no atomics are needed.
#pragma once

#include "des_device.cuh"

namespace des {

// ref_pressure (matprops.cxx:523-535): rho0[0] g depth, or the pressure of the
// PREM model interpolated in depth (option 1, matprops.cxx:20-62) or of PREM
// with an average continental crust (option 2, matprops.cxx:66-108); 0 above
// the surface.  Depths every 100 m and pressures every 1e7 Pa, as integers.
__host__ __device__ inline double ref_pressure(int option, double rho0, double gravity, double z)
{
    const double depth = -z;
    if (option == 0) return rho0 * gravity * depth;
    const int km_x10[46] = {0,     30,    150,   244,   400,   600,   800,   1150,  1500,  1850,
                            2200,  2650,  3100,  3550,  4000,  4500,  5000,  5500,  6000,  6350,
                            6700,  7210,  7710,  8710,  9710,  10710, 11710, 12710, 13710, 14710,
                            15710, 16710, 17710, 18710, 19710, 20710, 21710, 22710, 23710, 24710,
                            25710, 26710, 27410, 27710, 28710, 28910};
    const int kbar_x10[46] = {0,     3,     33,    60,    112,   178,   245,   361,   478,   594,
                              711,   864,   1020,  1177,  1335,  1522,  1713,  1907,  2104,  2243,
                              2383,  2607,  2829,  3276,  3728,  4186,  4648,  5116,  5589,  6068,
                              6552,  7041,  7535,  8036,  8543,  9056,  9576,  10103, 10638, 11182,
                              11734, 12297, 12697, 12870, 13456, 13575};
    // the crust of option 2: 0.82, 4.1 and 6.7 kbar at 3, 15 and 24.4 km
    const int crust_x100[3] = {82, 410, 670};
    if (depth <= 0) return 0;
    int n = 1;
    while (n < 45 && depth > km_x10[n] * 100.0) ++n;
    auto press = [&](int i) {
        if (option == 2 && i >= 1 && i <= 3) return crust_x100[i - 1] * 1e6;
        return kbar_x10[i] * 1e7;
    };
    const double d0 = km_x10[n - 1] * 100.0, d1 = km_x10[n] * 100.0;
    return press(n - 1) + (press(n) - press(n - 1)) * (depth - d0) / (d1 - d0);
}

struct Consts {
    MatTable M;
    double gravity, damping_factor, surface_temperature, dt_fraction, fixed_dt;
    double inertial_scaling, max_vbc_val, therm_diff_max, zlength, rho0_0;
    double compensation_pressure;
    double winkler_delta_rho, elastic_foundation_constant;
    unsigned stress_bc_sides;   // sides whose facets carry apply_stress_bcs' tractions
    int elastic_foundation;     // the bottom restoring force of apply_stress_bcs
    int surface_process_option;
    double surface_diffusivity;
    int ref_pressure_option;
    int damping_option, is_qs, thermal, rheol;
    int vbc_types[10];
    double vbc_values[10];
    double bnormals[10][3];
    double edge[10][10][3];
};

struct Clock {
    double dt, time;
    int steps, mass_valid;
    unsigned long long minl;           // order_bits of the running minimum height
    unsigned blocks_done, status;
    unsigned long long ql, eig;
    unsigned long long nlog;                    // return-map records seen (logging launches)
    unsigned long long nn_cand, nn_accept, fp64_returns;   // learned-closure counters
    unsigned npend, nexact;          // list lengths of the FP32 form's stress pass
};

// The boundary facets (mesh.cxx:1633-1682, bfacets side by side) and, for
// every node, the facets it belongs to in that order: the order in which
// apply_stress_bcs (bc.cxx:503-595) and the surface diffusion (bc.cxx:598-730)
// accumulate facet terms at a node.
struct BdryFacets {
    int nbf;
    const int *elem;                // [nbf] element of each facet
    const unsigned char *side_f;    // [nbf] side << 2 | facet of the element
    double *val;                    // [3][nbf] traction p n / 3 on each of its nodes
    double *surf;                   // [4][nbf] top facets: projected area, slope term of each node
    const int *node_off;            // [nnode + 1]
    const int *node_facet;          // facet indices
};

struct Dev {
    int nnode, nelem;
    const int4 *conn;
    const int *sup_off;
    const unsigned *sup_ent;     // (element << 2) | local slot
    const unsigned *bcflag;
    const unsigned char *mix;
    double *x, *y, *z, *vx, *vy, *vz, *fx, *fy, *fz, *x0, *y0, *z0;
    double *T, *mass, *tmass, *vol_n, *ntmp;
    double *vol, *vol_old, *edvoldt, *pls, *dpls, *dp, *tmp_sg;
    double *stress, *strain, *srate, *srate_next;   // [6][E]
    double *shp;                                     // [12][E] dx0..3 dy0..3 dz0..3
    double *tmp;                                     // [12][E]
    double *c_mass, *c_tmass, *c_trdv;               // fused-pass contributions
    const Consts *K;
    Clock *clk;
    float *ret_log;                  // return-map records (logging launches only)
    long long ret_cap;
    BdryFacets bf;
};

__device__ __forceinline__ int gtid() { return blockIdx.x * blockDim.x + threadIdx.x; }

__device__ __forceinline__ void load_xyz4(const Dev &d, int4 c, double X[4][3])
{
    const int n[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        X[i][0] = __ldg(d.x + n[i]);
        X[i][1] = __ldg(d.y + n[i]);
        X[i][2] = __ldg(d.z + n[i]);
    }
}
__device__ __forceinline__ void load_vel4(const Dev &d, int4 c, double V[4][3])
{
    const int n[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        V[i][0] = __ldg(d.vx + n[i]);
        V[i][1] = __ldg(d.vy + n[i]);
        V[i][2] = __ldg(d.vz + n[i]);
    }
}
__device__ __forceinline__ void load_nodal4(const double *a, int4 c, double out[4])
{
    out[0] = __ldg(a + c.x);
    out[1] = __ldg(a + c.y);
    out[2] = __ldg(a + c.z);
    out[3] = __ldg(a + c.w);
}
__device__ __forceinline__ void load_shp(const Dev &d, int e, double dx[4], double dy[4],
                                         double dz[4])
{
    const size_t E = d.nelem;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        dx[i] = d.shp[(0 + i) * E + e];
        dy[i] = d.shp[(4 + i) * E + e];
        dz[i] = d.shp[(8 + i) * E + e];
    }
}
__device__ __forceinline__ void store_shp(const Dev &d, int e, const double dx[4], const double dy[4],
                                          const double dz[4])
{
    const size_t E = d.nelem;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        d.shp[(0 + i) * E + e] = dx[i];
        d.shp[(4 + i) * E + e] = dy[i];
        d.shp[(8 + i) * E + e] = dz[i];
    }
}
__device__ __forceinline__ void load6(const double *a, size_t E, int e, double s[6])
{
#pragma unroll
    for (int i = 0; i < 6; ++i) s[i] = a[i * E + e];
}
__device__ __forceinline__ void store6(double *a, size_t E, int e, const double s[6])
{
#pragma unroll
    for (int i = 0; i < 6; ++i) a[i * E + e] = s[i];
}

// ---- shared per-element / per-node bodies ---------------------------------

// rheology.cxx:525-646 for one element; returns eigen flags (bit0 solved,
// bit1 QL, bit2 QL failed)
// the plastic branch of elasto_plastic (rheology.cxx:154-302), out of line:
// few elements take it
static __device__ __noinline__ int plastic_branch(const MatTable &M, const Mix &x, double pls, double &depls,
                                                  double s[6])
{
    double amc, anphi, anpsi, hardn, ten_max;
    plastic_props(M, x, pls, amc, anphi, anpsi, hardn, ten_max);
    return plastic_return(x.bulkm, x.shearm, amc, anphi, anpsi, hardn, ten_max, depls, s);
}

__device__ __forceinline__ int stress_body(const Dev &d, int e, int4 c, double edv, double dt,
                                           double s[6], double es[6], double edot[6], double &pls,
                                           double &dpls, double &dpress)
{
    const Consts &K = *d.K;
    const MatTable &M = K.M;
    const Mix &x = M.mix[d.mix[e]];
    double old_s = tr3(s);
    {
        double div = tr3(edot);
        const double corr = sf::div3(edv - div);
        for (int i = 0; i < 3; ++i) edot[i] += corr;
    }
    // (products on the integer pipes, sf::mul)
    double de[6];
    for (int i = 0; i < 6; ++i) de[i] = sf::mul(edot[i], dt);
    for (int i = 0; i < 6; ++i) es[i] += de[i];
    int flags = 0;
    switch (K.rheol) {
    case 1:   // elastic
        elastic(x.bulkm, x.shearm, de, s);
        break;
    case 2: { // viscous
        double Tn[4];
        load_nodal4(d.T, c, Tn);
        double viscosity = mat_visc(M, x, elem_mean4(Tn[0], Tn[1], Tn[2], Tn[3]), edot);
        viscous(x.bulkm, viscosity, tr3(es), edot, s);
    } break;
    case 3: { // maxwell
        double Tn[4];
        load_nodal4(d.T, c, Tn);
        double viscosity = mat_visc(M, x, elem_mean4(Tn[0], Tn[1], Tn[2], Tn[3]), edot);
        double dv = d.vol[e] / d.vol_old[e] - 1;
        maxwell(x.bulkm, x.shearm, viscosity, dt, dv, de, s);
    } break;
    case 5: { // elasto-plastic
        double depls = 0;
        elastic(x.bulkm, x.shearm, de, s);
        if (!quick_elastic(M, x, pls, s)) flags = plastic_branch(M, x, pls, depls, s);
        pls += depls;
        dpls = depls;
    } break;
    case 7: { // elasto-visco-plastic
        double depls = 0;
        double Tn[4];
        load_nodal4(d.T, c, Tn);
        double viscosity = mat_visc(M, x, elem_mean4(Tn[0], Tn[1], Tn[2], Tn[3]), edot);
        double dv = d.vol[e] / d.vol_old[e] - 1;
        double sv[6];
        for (int i = 0; i < 6; ++i) sv[i] = s[i];
        maxwell(x.bulkm, x.shearm, viscosity, dt, dv, de, sv);
        double svII = second_invariant2(sv);
        double sp[6];
        for (int i = 0; i < 6; ++i) sp[i] = s[i];
        elastic(x.bulkm, x.shearm, de, sp);
        if (!quick_elastic(M, x, pls, sp)) flags = plastic_branch(M, x, pls, depls, sp);
        double spII = second_invariant2(sp);
        if (svII < spII) {
            for (int i = 0; i < 6; ++i) s[i] = sv[i];
            flags &= ~48;    // the plastic return was not taken
        } else {
            for (int i = 0; i < 6; ++i) s[i] = sp[i];
            pls += depls;
            dpls = depls;
        }
    } break;
    }
    dpress = tr3(s) - old_s;
    return flags;
}

__device__ __forceinline__ void count_eigen(const Dev &d, int flags)
{
    // warp-aggregated counters of eigen-solves and QL fallbacks
    unsigned solved = __ballot_sync(0xffffffffu, flags & 1);
    unsigned ql = __ballot_sync(0xffffffffu, flags & 2);
    unsigned bad = __ballot_sync(0xffffffffu, flags & 4);
    if ((threadIdx.x & 31) == 0) {
        if (solved) atomicAdd(&d.clk->eig, (unsigned long long)__popc(solved));
        if (ql) atomicAdd(&d.clk->ql, (unsigned long long)__popc(ql));
        if (bad) atomicOr(&d.clk->status, 0x8u);
    }
}

// fields.cxx:264-297 for one component
template <class R>
__device__ __forceinline__ R damp(const Consts &K, R f, R v)
{
    const R fac = R(K.damping_factor);
    switch (K.damping_option) {
    case 1:
        if (fabs(v) > R(1e-13)) f -= fac * copysign(f, v);
        break;
    case 2:
        f -= fac * f;
        break;
    case 3:
        if ((f < 0) == (v < 0))
            f -= fac * f;
        else
            f += (1 - fac) * f;
        break;
    default:
        break;
    }
    return f;
}

// bc.cxx:201-496 for one node
template <class R>
__device__ __forceinline__ void vbc_node(const Consts &K, unsigned flag, R v[3])
{
    if (!(flag & kBoundAny)) return;
    const int vx0 = K.vbc_types[0], vx1 = K.vbc_types[1], vy0 = K.vbc_types[2],
              vy1 = K.vbc_types[3], vz0 = K.vbc_types[4], vz1 = K.vbc_types[5];
    const R ux0 = R(K.vbc_values[0]), ux1 = R(K.vbc_values[1]), uy0 = R(K.vbc_values[2]),
            uy1 = R(K.vbc_values[3]), uz0 = R(K.vbc_values[4]), uz1 = R(K.vbc_values[5]);
    if (flag & kBoundX0) {
        switch (vx0) {
        case 1: v[0] = ux0; break;
        case 2: v[1] = 0; v[2] = 0; break;
        case 3: v[0] = ux0; v[1] = 0; v[2] = 0; break;
        case 4: v[1] = ux0; v[2] = 0; break;
        case 5: v[0] = 0; v[1] = ux0; v[2] = 0; break;
        case 7: v[0] = ux0; v[1] = 0; break;
        }
    }
    if (flag & kBoundX1) {
        switch (vx1) {
        case 1: v[0] = ux1; break;
        case 2: v[1] = 0; v[2] = 0; break;
        case 3: v[0] = ux1; v[1] = 0; v[2] = 0; break;
        case 4: v[1] = ux1; v[2] = 0; break;
        case 5: v[0] = 0; v[1] = ux1; v[2] = 0; break;
        case 7: v[0] = ux1; v[1] = 0; break;
        }
    }
    if (flag & kBoundY0) {
        switch (vy0) {
        case 1: v[1] = uy0; break;
        case 2: v[0] = 0; v[2] = 0; break;
        case 3: v[0] = 0; v[1] = uy0; v[2] = 0; break;
        case 4: v[0] = uy0; v[2] = 0; break;
        case 5: v[0] = uy0; v[1] = 0; v[2] = 0; break;
        case 7: v[0] = 0; v[1] = uy0; break;
        }
    }
    if (flag & kBoundY1) {
        switch (vy1) {
        case 1: v[1] = uy1; break;
        case 2: v[0] = 0; v[2] = 0; break;
        case 3: v[0] = uy1; v[1] = 0; v[2] = 0; break;
        case 4: v[0] = uy1; v[2] = 0; break;
        case 5: v[0] = uy1; v[1] = 0; v[2] = 0; break;
        case 7: v[0] = 0; v[1] = uy1; break;
        }
    }
    if (flag & 0x3c0u) {
        for (int ib = 6; ib <= 9; ib++) {
            if (!(flag & (1u << ib))) continue;
            const R n[3] = {R(K.bnormals[ib][0]), R(K.bnormals[ib][1]), R(K.bnormals[ib][2])};
            const R val = R(K.vbc_values[ib]);
            R fac = 0;
            switch (K.vbc_types[ib]) {
            case 1:
                if (flag == (1u << ib)) {
                    R vn = 0;
                    for (int dd = 0; dd < 3; dd++) vn += v[dd] * n[dd];
                    for (int dd = 0; dd < 3; dd++) v[dd] += (val - vn) * n[dd];
                } else {
                    for (int ic = 0; ic < ib; ic++) {
                        if (!(flag & (1u << ic))) continue;
                        if (K.vbc_types[ic] == 0) {
                            R vn = 0;
                            for (int dd = 0; dd < 3; dd++) vn += v[dd] * n[dd];
                            for (int dd = 0; dd < 3; dd++) v[dd] += (val - vn) * n[dd];
                        } else if (K.vbc_types[ic] == 1) {
                            const R edge[3] = {R(K.edge[ic][ib][0]), R(K.edge[ic][ib][1]),
                                               R(K.edge[ic][ib][2])};
                            R ve = 0;
                            for (int dd = 0; dd < 3; dd++) ve += v[dd] * edge[dd];
                            for (int dd = 0; dd < 3; dd++) v[dd] = ve * edge[dd];
                        }
                    }
                }
                break;
            case 3:
                for (int dd = 0; dd < 3; dd++) v[dd] = val * n[dd];
                break;
            case 11:
                fac = 1 / sqrt(1 - n[2] * n[2]);
                if (flag == (1u << ib)) {
                    R vn = 0;
                    for (int dd = 0; dd < 2; dd++) vn += v[dd] * n[dd];
                    for (int dd = 0; dd < 2; dd++) v[dd] += (val * fac - vn) * n[dd];
                } else {
                    for (int ic = 0; ic < ib; ic++) {
                        if (!(flag & (1u << ic))) continue;
                        if (K.vbc_types[ic] == 0) {
                            R vn = 0;
                            for (int dd = 0; dd < 2; dd++) vn += v[dd] * n[dd];
                            for (int dd = 0; dd < 2; dd++) v[dd] += (val * fac - vn) * n[dd];
                        } else if (K.vbc_types[ic] == 1) {
                            const R edge[3] = {R(K.edge[ic][ib][0]), R(K.edge[ic][ib][1]),
                                               R(K.edge[ic][ib][2])};
                            R ve = 0;
                            for (int dd = 0; dd < 3; dd++) ve += v[dd] * edge[dd];
                            for (int dd = 0; dd < 3; dd++) v[dd] = ve * edge[dd];
                        }
                    }
                }
                break;
            case 13:
                fac = 1 / sqrt(1 - n[2] * n[2]);
                for (int dd = 0; dd < 2; dd++) v[dd] = val * fac * n[dd];
                v[2] = 0;
                break;
            }
        }
    }
    if (vz0 == 0 && vz1 == 0) return;
    if (flag & kBoundZ0) {
        switch (vz0) {
        case 1: v[2] = uz0; break;
        case 2: v[0] = 0; v[1] = 0; break;
        case 3: v[0] = 0; v[1] = 0; v[2] = uz0; break;
        }
    }
    if (flag & kBoundZ1) {
        switch (vz1) {
        case 1: v[2] = uz1; break;
        case 2: v[0] = 0; v[1] = 0; break;
        case 3: v[0] = 0; v[1] = 0; v[2] = uz1; break;
        }
    }
}

// block-level minimum of the elements' heights + the last block turns the
// global minimum into dt (geometry.cxx:311-325).  No thread waits on another
// block.  nblocks: the blocks of every launch that contributes (E-A may run
// as several launches over consecutive element ranges); the last to finish
// forms dt.  The reference's dt_diffusion, the minimum over the elements of
// 0.5 h h / therm_diff_max (geometry.cxx:305-307), is that expression of the
// minimum height: for h >= 0 it is non-decreasing in h under round to
// nearest (0.5 h exact, then a product and a quotient by a positive
// constant, each rounded monotonically), so the minimum commutes with it;
// where a height is negative, dt_advection <= 0 is the smaller term either
// way.
__device__ void dt_reduce_and_finalize(const Dev &d, double minh, bool active, unsigned nblocks)
{
    __shared__ unsigned long long s_min[32];
    __shared__ bool s_last;
    unsigned long long a = active ? order_bits(minh) : ~0ULL;
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long a2 = __shfl_down_sync(0xffffffffu, a, o);
        a = a2 < a ? a2 : a;
    }
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_min[warp] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long ma = ~0ULL;
        for (int w = 0; w < (int)(blockDim.x + 31) / 32; ++w) ma = s_min[w] < ma ? s_min[w] : ma;
        if (ma != ~0ULL) atomicMin(&d.clk->minl, ma);
        __threadfence();
        unsigned done = atomicAdd(&d.clk->blocks_done, 1u);
        s_last = (done == nblocks - 1);
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        __threadfence();
        const Consts &K = *d.K;
        unsigned long long bl = atomicAdd(&d.clk->minl, 0ULL);
        double minl = from_order_bits(bl);
        double dt_diffusion = K.thermal ? 0.5 * minl * minl / K.therm_diff_max : 1.7976931348623157e308;
        double dt_maxwell = 1.7976931348623157e308;
        for (int i = 0; i < K.M.nmix; ++i) dt_maxwell = smin(dt_maxwell, K.M.mix[i].dt_maxwell);
        double dt_advection = 0.5 * minl / K.max_vbc_val;
        double dt_elastic;
        if (K.is_qs) {
            dt_elastic = 0.5 * minl / (K.max_vbc_val * K.inertial_scaling);
        } else {
            int4 c0 = d.conn[0];
            double Tn[4];
            load_nodal4(d.T, c0, Tn);
            const Mix &x0 = K.M.mix[d.mix[0]];
            double rho0 = mat_rho(K.M, x0, elem_mean4(Tn[0], Tn[1], Tn[2], Tn[3]));
            dt_elastic = 0.5 * minl / sqrt(x0.bulkm / rho0);
        }
        double dt = smin(smin(dt_elastic, dt_maxwell), smin(dt_advection, dt_diffusion)) * K.dt_fraction;
        d.clk->dt = dt;
        if (!(dt > 0)) atomicOr(&d.clk->status, 0x1u);
        d.clk->minl = ~0ULL;
        d.clk->blocks_done = 0;
    }
}

// ===========================================================================
// per-function kernels
// ===========================================================================

// fields.cxx:119-144
__global__ void k_temp_elem(Dev d)
{
    int e = gtid();
    if (e >= d.nelem) return;
    const size_t E = d.nelem;
    int4 c = d.conn[e];
    double dx[4], dy[4], dz[4], Tn[4], tr[4];
    load_shp(d, e, dx, dy, dz);
    load_nodal4(d.T, c, Tn);
    double kv = d.K->M.mix[d.mix[e]].k * d.vol[e];
    conduction(dx, dy, dz, Tn, kv, tr);
    for (int i = 0; i < 4; ++i) d.tmp[i * E + e] = tr[i];
}

// fields.cxx:149-168
__global__ void k_temp_node(Dev d)
{
    int n = gtid();
    if (n >= d.nnode) return;
    const size_t E = d.nelem;
    double tdot = 0;
    for (int q = d.sup_off[n]; q < d.sup_off[n + 1]; ++q) {
        unsigned p = __ldg(d.sup_ent + q);
        tdot += d.tmp[(p & 3u) * E + (p >> 2)];
    }
    d.ntmp[n] = tdot;
    const Consts &K = *d.K;
    if (d.bcflag[n] & kBoundZ1)
        d.T[n] = K.surface_temperature;
    else
        d.T[n] -= tdot * d.clk->dt / d.tmass[n];
}

// fields.cxx:184-243; out = srate or srate_next
__global__ void k_srate(Dev d, double *out)
{
    int e = gtid();
    if (e >= d.nelem) return;
    double V[4][3], dx[4], dy[4], dz[4], s[6];
    load_vel4(d, d.conn[e], V);
    load_shp(d, e, dx, dy, dz);
    strain_rate(V, dx, dy, dz, s);
    store6(out, d.nelem, e, s);
}

// geometry.cxx:128-134 (src = srate) and 200-204 (dp)
__global__ void k_dvoldt_elem(Dev d)
{
    int e = gtid();
    if (e >= d.nelem) return;
    const size_t E = d.nelem;
    double dj = d.srate[e] + d.srate[E + e] + d.srate[2 * E + e];
    d.tmp_sg[e] = dj * d.vol[e];
}
__global__ void k_dp_elem(Dev d)
{
    int e = gtid();
    if (e >= d.nelem) return;
    d.tmp_sg[e] = d.dp[e] * d.vol[e];
}

// geometry.cxx:138-143 and 208-213: ntmp[n] = sum(tmp_sg) / volume_n
__global__ void k_sg_gather(Dev d)
{
    int n = gtid();
    if (n >= d.nnode) return;
    double s = 0.;
    for (int q = d.sup_off[n]; q < d.sup_off[n + 1]; ++q) s += d.tmp_sg[__ldg(d.sup_ent + q) >> 2];
    s /= d.vol_n[n];
    d.ntmp[n] = s;
}

// geometry.cxx:166-174
__global__ void k_edvoldt(Dev d)
{
    int e = gtid();
    if (e >= d.nelem) return;
    double a[4];
    load_nodal4(d.ntmp, d.conn[e], a);
    double dj = sf::add0(a[0]);
    for (int i = 1; i < 4; ++i) dj += a[i];
    d.edvoldt[e] = sf::quarter(dj);
}

// rheology.cxx:525-650
__global__ void k_stress(Dev d)
{
    int e = gtid();
    bool live = e < d.nelem;
    int flags = 0;
    if (live) {
        const size_t E = d.nelem;
        double s[6], es[6], edot[6];
        load6(d.stress, E, e, s);
        load6(d.strain, E, e, es);
        load6(d.srate, E, e, edot);
        double pls = d.pls[e], dpls = d.dpls[e], dpress;
        flags = stress_body(d, e, d.conn[e], d.edvoldt[e], d.clk->dt, s, es, edot, pls, dpls, dpress);
        store6(d.stress, E, e, s);
        store6(d.strain, E, e, es);
        store6(d.srate, E, e, edot);
        d.pls[e] = pls;
        d.dpls[e] = dpls;
        d.dp[e] = dpress;
    }
    count_eigen(d, flags);
}

// geometry.cxx:221-250
__global__ void k_nmd_apply(Dev d)
{
    int e = gtid();
    if (e >= d.nelem) return;
    const size_t E = d.nelem;
    double a[4];
    load_nodal4(d.ntmp, d.conn[e], a);
    double dpe = sf::add0(a[0]);
    for (int i = 1; i < 4; ++i) dpe += a[i];
    double dp_el = sf::quarter(dpe);
    double ddp = sf::div3(-d.dp[e] + dp_el);
    for (int i = 0; i < 3; ++i) d.stress[i * E + e] += ddp;
}

// fields.cxx:321-346: element force vectors into tmp[12][E]
__device__ __forceinline__ void force_elem_body(const Dev &d, int e, int4 c, const double s[6])
{
    const size_t E = d.nelem;
    const Consts &K = *d.K;
    double dx[4], dy[4], dz[4];
    load_shp(d, e, dx, dy, dz);
    double vol = d.vol[e];
    double buoy = 0;
    if (K.gravity != 0) {
        double Tn[4];
        load_nodal4(d.T, c, Tn);
        buoy = sf::quarter(mat_rho(K.M, K.M.mix[d.mix[e]], elem_mean4(Tn[0], Tn[1], Tn[2], Tn[3])) * K.gravity);
    }
    // (products on the integer pipes, sf::mul)
    for (int i = 0; i < 4; ++i) {
        d.tmp[(i)*E + e] = sf::mul(sf::mul(s[0], dx[i]) + sf::mul(s[3], dy[i]) + sf::mul(s[4], dz[i]), vol);
        d.tmp[(i + 4) * E + e] =
            sf::mul(sf::mul(s[3], dx[i]) + sf::mul(s[1], dy[i]) + sf::mul(s[5], dz[i]), vol);
        d.tmp[(i + 8) * E + e] =
            sf::mul(sf::mul(s[4], dx[i]) + sf::mul(s[5], dy[i]) + sf::mul(s[2], dz[i]) + buoy, vol);
    }
}
__global__ void k_force_elem(Dev d)
{
    int e = gtid();
    if (e >= d.nelem) return;
    double s[6];
    load6(d.stress, d.nelem, e, s);
    force_elem_body(d, e, d.conn[e], s);
}

// node j of facet f of a tetrahedron (constants.hpp:61-67: {1,2,3},
// {0,3,2}, {0,1,3}, {0,2,1}), two bits per entry
__device__ __forceinline__ int facet_node(int f, int j)
{
    constexpr unsigned kPacked = (1u << 0) | (2u << 2) | (3u << 4) | (0u << 6) | (3u << 8) | (2u << 10) |
                                 (0u << 12) | (1u << 14) | (3u << 16) | (0u << 18) | (2u << 20) | (1u << 22);
    return (kPacked >> (2 * (3 * f + j))) & 3u;
}

// bc.cxx:528-566 for one boundary facet: its outward normal n with the
// facet's area as length (bc.cxx:15-36), the pressure p of its side and the
// traction p n / 3 each of its three nodes receives
__global__ void k_stress_bc_facets(Dev d)
{
    const int k = gtid();
    const BdryFacets &b = d.bf;
    if (k >= b.nbf) return;
    const Consts &K = *d.K;
    const int side = b.side_f[k] >> 2, f = b.side_f[k] & 3;
    if (!(K.stress_bc_sides & (1u << side))) return;
    const int e = b.elem[k];
    const int4 c4 = d.conn[e];
    auto pick = [&](int i) { return i == 0 ? c4.x : i == 1 ? c4.y : i == 2 ? c4.z : c4.w; };
    const int n0 = pick(facet_node(f, 0)), n1 = pick(facet_node(f, 1)), n2 = pick(facet_node(f, 2));
    const double v01[3] = {d.x[n1] - d.x[n0], d.y[n1] - d.y[n0], d.z[n1] - d.z[n0]};
    const double v02[3] = {d.x[n2] - d.x[n0], d.y[n2] - d.y[n0], d.z[n2] - d.z[n0]};
    double normal[3];
    normal[0] = (v01[1] * v02[2] - v01[2] * v02[1]) / 2;
    normal[1] = (v01[2] * v02[0] - v01[0] * v02[2]) / 2;
    normal[2] = (v01[0] * v02[1] - v01[1] * v02[0]) / 2;
    const double zcenter = (d.z[n0] + d.z[n1] + d.z[n2]) / 3;
    double p;
    if (side == 4) {
        // Winkler foundation under the bottom
        double Tn[4];
        load_nodal4(d.T, c4, Tn);
        const double rho = mat_rho(K.M, K.M.mix[d.mix[e]], elem_mean4(Tn[0], Tn[1], Tn[2], Tn[3]));
        p = K.compensation_pressure - (rho + K.winkler_delta_rho) * K.gravity * (zcenter + K.zlength);
    } else if (side == 5) {
        // water loading on the surface below sea level (0)
        p = 0;
        if (zcenter < 0) p = 1030 * K.gravity * (0 - zcenter);
    } else {
        p = ref_pressure(K.ref_pressure_option, K.rho0_0, K.gravity, zcenter);
    }
    for (int j = 0; j < 3; ++j) b.val[j * b.nbf + k] = p * normal[j] / 3;
}

// bc.cxx:616-700 (simple_diffusion, 3D) for one facet of the top boundary:
// its projected area and, for each of its nodes, the FEM slope term that the
// node's total_slope receives
__global__ void k_surface_facets(Dev d)
{
    const int k = gtid();
    const BdryFacets &b = d.bf;
    if (k >= b.nbf || (b.side_f[k] >> 2) != 5) return;
    const int f = b.side_f[k] & 3;
    const int4 c4 = d.conn[b.elem[k]];
    auto pick = [&](int i) { return i == 0 ? c4.x : i == 1 ? c4.y : i == 2 ? c4.z : c4.w; };
    const int n[3] = {pick(facet_node(f, 0)), pick(facet_node(f, 1)), pick(facet_node(f, 2))};
    const double X[3] = {d.x[n[0]], d.x[n[1]], d.x[n[2]]};
    const double Y[3] = {d.y[n[0]], d.y[n[1]], d.y[n[2]]};
    const double Z[3] = {d.z[n[0]], d.z[n[1]], d.z[n[2]]};
    const double x01 = X[1] - X[0], y01 = Y[1] - Y[0], x02 = X[2] - X[0], y02 = Y[2] - Y[0];
    const double projected_area = 0.5 * (x01 * y02 - y01 * x02);
    const double iv = 1 / (2 * projected_area);
    const double sx[3] = {iv * (Y[1] - Y[2]), iv * (Y[2] - Y[0]), iv * (Y[0] - Y[1])};
    const double sy[3] = {iv * (X[2] - X[1]), iv * (X[0] - X[2]), iv * (X[1] - X[0])};
    b.surf[k] = projected_area;
    for (int j = 0; j < 3; ++j) {
        double slope = 0;
        for (int i = 0; i < 3; ++i) {
            const double D = sx[j] * sx[i] + sy[j] * sy[i];
            slope += D * Z[i];
        }
        b.surf[(1 + j) * b.nbf + k] = slope * projected_area;
    }
}

// bc.cxx:702-712 (option 1) for one node of the top boundary: its totals over
// its top facets in facet order, then the height change; option 101 (the
// reference's custom template, bc.cxx:735-757) adds dh = 0
__global__ void k_surface_nodes(Dev d)
{
    const int n = gtid();
    if (n >= d.nnode || !(d.bcflag[n] & kBoundZ1)) return;
    const Consts &K = *d.K;
    if (K.surface_process_option != 1) {
        d.z[n] += 0.0;
        return;
    }
    const BdryFacets &b = d.bf;
    double total_dx = 0, total_slope = 0;
    for (int q = b.node_off[n]; q < b.node_off[n + 1]; ++q) {
        const int k = b.node_facet[q];
        if ((b.side_f[k] >> 2) != 5) continue;
        const int f = b.side_f[k] & 3;
        const int4 c4 = d.conn[b.elem[k]];
        auto pick = [&](int i) { return i == 0 ? c4.x : i == 1 ? c4.y : i == 2 ? c4.z : c4.w; };
        const int j = pick(facet_node(f, 0)) == n ? 0 : pick(facet_node(f, 1)) == n ? 1 : 2;
        total_dx += b.surf[k];
        total_slope += b.surf[(1 + j) * b.nbf + k];
    }
    const double dh = K.surface_diffusivity * d.clk->dt * total_slope / total_dx;
    d.z[n] -= dh;
}

// bc.cxx:568-590 for node n after update_force's gather: the tractions of its
// boundary facets, then the elastic foundation's restoring force on the bottom
__device__ __forceinline__ void stress_bc_node(const Consts &K, const BdryFacets &b, int n, unsigned flag,
                                               double z, double z0, double f[3])
{
    if (K.stress_bc_sides && (flag & kBoundAny)) {
        for (int q = b.node_off[n]; q < b.node_off[n + 1]; ++q) {
            const int k = b.node_facet[q];
            if (!(K.stress_bc_sides & (1u << (b.side_f[k] >> 2)))) continue;
            for (int j = 0; j < 3; ++j) f[j] -= b.val[j * b.nbf + k];
        }
    }
    if (K.elastic_foundation && (flag & kBoundZ0)) f[2] -= K.elastic_foundation_constant * (z - z0);
}

// fields.cxx:351-365 + apply_damping (fields.cxx:250-309)
__device__ __forceinline__ void force_gather(const Dev &d, int n, double f[3])
{
    const size_t E = d.nelem;
    f[0] = f[1] = f[2] = 0;
    for (int q = d.sup_off[n]; q < d.sup_off[n + 1]; ++q) {
        unsigned p = __ldg(d.sup_ent + q);
        size_t e = p >> 2, i = p & 3u;
        f[0] -= d.tmp[(i)*E + e];
        f[1] -= d.tmp[(i + 4) * E + e];
        f[2] -= d.tmp[(i + 8) * E + e];
    }
}
__global__ void k_force_node(Dev d, int damping)
{
    int n = gtid();
    if (n >= d.nnode) return;
    double f[3];
    force_gather(d, n, f);
    stress_bc_node(*d.K, d.bf, n, d.bcflag[n], d.z[n], d.z0[n], f);
    if (damping) {
        const Consts &K = *d.K;
        f[0] = damp(K, f[0], d.vx[n]);
        f[1] = damp(K, f[1], d.vy[n]);
        f[2] = damp(K, f[2], d.vz[n]);
    }
    d.fx[n] = f[0];
    d.fy[n] = f[1];
    d.fz[n] = f[2];
}

// fields.cxx:386-389
__global__ void k_velocity(Dev d)
{
    int n = gtid();
    if (n >= d.nnode) return;
    double dt = d.clk->dt, m = d.mass[n];
    d.vx[n] += dt * d.fx[n] / m;
    d.vy[n] += dt * d.fy[n] / m;
    d.vz[n] += dt * d.fz[n] / m;
}

// remeshing.cxx:2046-2054: the bottom nodes' coord0 back on z = -zlength
// (bnodes[iboundz0] are the nodes flagged on that boundary, mesh.cxx:1553-1566)
__global__ void k_reset_bottom_coord0(Dev d, double zbottom)
{
    int n = gtid();
    if (n >= d.nnode) return;
    if (d.bcflag[n] & kBoundZ0) d.z0[n] = zbottom;
}

__global__ void k_vbcs(Dev d)
{
    int n = gtid();
    if (n >= d.nnode) return;
    unsigned flag = d.bcflag[n];
    if (!(flag & kBoundAny)) return;
    double v[3] = {d.vx[n], d.vy[n], d.vz[n]};
    vbc_node(*d.K, flag, v);
    d.vx[n] = v[0];
    d.vy[n] = v[1];
    d.vz[n] = v[2];
}

// fields.cxx:406-408
__global__ void k_coord(Dev d)
{
    int n = gtid();
    if (n >= d.nnode) return;
    double dt = d.clk->dt;
    d.x[n] += d.vx[n] * dt;
    d.y[n] += d.vy[n] * dt;
    d.z[n] += d.vz[n] * dt;
    // output.cxx:195-208 stops on NaN/Inf coordinates
    if (not_finite(d.x[n]) || not_finite(d.y[n]) || not_finite(d.z[n])) atomicOr(&d.clk->status, 0x2u);
}

// geometry.cxx:94-110; save_old copies volume into volume_old first
__global__ void k_volume(Dev d, int save_old)
{
    int e = gtid();
    if (e >= d.nelem) return;
    double X[4][3];
    load_xyz4(d, d.conn[e], X);
    double v = tet_volume(X[0], X[1], X[2], X[3]);
    if (save_old) d.vol_old[e] = d.vol[e];
    d.vol[e] = v;
    if (!(v > 0)) atomicOr(&d.clk->status, 0x4u);
}

// geometry.cxx:354-365; Tsrc = NULL means T = 0 (the first compute_mass of init)
__global__ void k_mass_elem(Dev d, const double *Tsrc)
{
    int e = gtid();
    if (e >= d.nelem) return;
    const size_t E = d.nelem;
    const Consts &K = *d.K;
    const Mix &x = K.M.mix[d.mix[e]];
    double Tn[4] = {0, 0, 0, 0};
    if (Tsrc) load_nodal4(Tsrc, d.conn[e], Tn);
    double rT = mat_rho(K.M, x, elem_mean4(Tn[0], Tn[1], Tn[2], Tn[3]));
    double vol = d.vol[e];
    double rho = K.is_qs ? x.rho_qs : rT;
    double m = rho * vol / 4;
    double tm = rT * x.cp * vol / 4;
    d.tmp[e] = vol;
    d.tmp[E + e] = m;
    if (K.thermal) d.tmp[2 * E + e] = tm;
}

// geometry.cxx:370-381 from tmp[0..2]
__global__ void k_mass_node(Dev d)
{
    int n = gtid();
    if (n >= d.nnode) return;
    const size_t E = d.nelem;
    const bool thermal = d.K->thermal;
    double vn = 0, m = 0, tm = 0;
    for (int q = d.sup_off[n]; q < d.sup_off[n + 1]; ++q) {
        size_t e = __ldg(d.sup_ent + q) >> 2;
        vn += d.tmp[e];
        m += d.tmp[E + e];
        if (thermal) tm += d.tmp[2 * E + e];
    }
    d.vol_n[n] = vn;
    d.mass[n] = m;
    d.tmass[n] = tm;
}

// geometry.cxx:400-466
__global__ void k_shape(Dev d)
{
    int e = gtid();
    if (e >= d.nelem) return;
    double X[4][3], dx[4], dy[4], dz[4];
    load_xyz4(d, d.conn[e], X);
    shape_fn(X, d.vol[e], dx, dy, dz);
    store_shp(d, e, dx, dy, dz);
}

// fields.cxx:478-529
__global__ void k_rotate(Dev d)
{
    int e = gtid();
    if (e >= d.nelem) return;
    const size_t E = d.nelem;
    double V[4][3], dx[4], dy[4], dz[4], w3, w4, w5, s[6];
    load_vel4(d, d.conn[e], V);
    load_shp(d, e, dx, dy, dz);
    spin(V, dx, dy, dz, w3, w4, w5);
    double dt = d.clk->dt;
    load6(d.stress, E, e, s);
    jaumann(s, dt, w3, w4, w5);
    store6(d.stress, E, e, s);
    load6(d.strain, E, e, s);
    jaumann(s, dt, w3, w4, w5);
    store6(d.strain, E, e, s);
}

// geometry.cxx:270-325
__global__ void k_dt(Dev d)
{
    int e = gtid();
    bool live = e < d.nelem;
    double minh = 0;
    if (live) {
        double X[4][3];
        load_xyz4(d, d.conn[e], X);
        minh = min_height(X, d.vol[e]);
    }
    dt_reduce_and_finalize(d, minh, live, gridDim.x);
}

// ic.cxx:100-131
__global__ void k_init_stress(Dev d)
{
    int e = gtid();
    if (e >= d.nelem) return;
    const size_t E = d.nelem;
    const Consts &K = *d.K;
    // bulkm(0), or the element's own with a PREM reference pressure
    const double ks = K.M.mix[d.mix[K.ref_pressure_option != 0 ? e : 0]].bulkm;
    double zn[4];
    load_nodal4(d.z, d.conn[e], zn);
    double zcenter = elem_mean4(zn[0], zn[1], zn[2], zn[3]);
    double p = ref_pressure(K.ref_pressure_option, K.rho0_0, K.gravity, zcenter);
    for (int i = 0; i < 3; ++i) {
        d.stress[i * E + e] = -p;
        d.strain[i * E + e] = -p / ks / 3;
    }
}

// ===========================================================================
// fused passes
// ===========================================================================

// contributions for the next N-A pass from the current state: next strain
// rate, tr(D) * volume, conduction vector
// with the next step's strain rate D already formed
__device__ __forceinline__ void next_step_contrib_d(const Dev &d, int e, int4 c, const double D[6],
                                                    const double dx[4], const double dy[4],
                                                    const double dz[4], double vol)
{
    const size_t E = d.nelem;
    store6(d.srate_next, E, e, D);
    d.c_trdv[e] = tr3(D) * vol;
    if (d.K->thermal) {
        double Tn[4], tr[4];
        load_nodal4(d.T, c, Tn);
        conduction(dx, dy, dz, Tn, d.K->M.mix[d.mix[e]].k * vol, tr);
        for (int i = 0; i < 4; ++i) d.tmp[i * E + e] = tr[i];
    }
}

__device__ __forceinline__ void next_step_contrib(const Dev &d, int e, int4 c, const double V[4][3],
                                                  const double dx[4], const double dy[4],
                                                  const double dz[4], double vol)
{
    double D[6];
    strain_rate(V, dx, dy, dz, D);
    next_step_contrib_d(d, e, c, D, dx, dy, dz, vol);
}

__global__ void k_prime(Dev d)
{
    int e = gtid();
    if (e >= d.nelem) return;
    int4 c = d.conn[e];
    double V[4][3], dx[4], dy[4], dz[4];
    load_vel4(d, c, V);
    load_shp(d, e, dx, dy, dz);
    next_step_contrib(d, e, c, V, dx, dy, dz, d.vol[e]);
}

// N-A: start of a step (dynearthsol.cxx:358-362, 365 node half)
__global__ void k_fn_a(Dev d)
{
    int n = gtid();
    const Consts &K = *d.K;
    const double dt = d.clk->dt;
    if (n == 0) {
        d.clk->steps += 1;
        d.clk->time += dt;
    }
    if (n >= d.nnode) return;
    const size_t E = d.nelem;
    const int q0 = d.sup_off[n], q1 = d.sup_off[n + 1];
    double vn, tm;
    if (d.clk->mass_valid) {
        vn = d.vol_n[n];
        tm = d.tmass[n];
    } else {
        double m = 0;
        vn = 0;
        tm = 0;
        for (int q = q0; q < q1; ++q) {
            size_t e = __ldg(d.sup_ent + q) >> 2;
            vn += d.vol[e];
            m += d.c_mass[e];
            if (K.thermal) tm += d.c_tmass[e];
        }
        d.vol_n[n] = vn;
        d.mass[n] = m;
        d.tmass[n] = tm;
    }
    if (K.thermal) {
        double tdot = 0;
        for (int q = q0; q < q1; ++q) {
            unsigned p = __ldg(d.sup_ent + q);
            tdot += d.tmp[(p & 3u) * E + (p >> 2)];
        }
        if (d.bcflag[n] & kBoundZ1)
            d.T[n] = K.surface_temperature;
        else
            d.T[n] -= tdot * dt / tm;
    }
    double dv = 0.;
    for (int q = q0; q < q1; ++q) dv += d.c_trdv[__ldg(d.sup_ent + q) >> 2];
    dv /= vn;
    d.ntmp[n] = dv;
}

// E-B: edvoldt + update_stress + dp * volume
// One return-map record: the inputs and outputs of elasto_plastic for an
// element that took the shear return (rheology.cxx:180-240 via :578-640).
constexpr int kRetRecord = 24;
// [0:6] stress before, [6:12] strain increment, [12] element temperature,
// [13] plastic strain before, [14:20] stress after, [20] plastic-strain
// increment, [21] element index (int bits), [22] step (int bits), [23] the
// dilation factor anpsi of the return

// (over the elements from e0, a multiple of the block size).  Registers
// bounded for 8 blocks of 128 per SM, with the return map out of line
// (plastic_branch): the spills fall there, where few elements go; config 2's
// E-B 1.08 -> 0.86 ms, the yielding workload's 1.61 -> 1.42 ms.
template <bool LOG>
__global__ void __launch_bounds__(128, 8) k_fe_b_t(Dev d, int e0)
{
    int e = e0 + gtid();
    if (e == 0) d.clk->mass_valid = 1;
    bool live = e < d.nelem;
    int flags = 0;
    float rec[kRetRecord];
    if (live) {
        const size_t E = d.nelem;
        int4 c = d.conn[e];
        double a[4];
        load_nodal4(d.ntmp, c, a);
        double dj = sf::add0(a[0]);            // 0 + a0, then the rest; / 4
        for (int i = 1; i < 4; ++i) dj += a[i];
        double edv = sf::quarter(dj);
        d.edvoldt[e] = edv;
        double s[6], es[6], edot[6];
        load6(d.stress, E, e, s);
        load6(d.strain, E, e, es);
        load6(d.srate_next, E, e, edot);
        double pls = d.pls[e], dpls = d.dpls[e], dpress;
        const double pls_in = pls;
        if (LOG)
            for (int i = 0; i < 6; ++i) rec[i] = (float)s[i];
        flags = stress_body(d, e, c, edv, d.clk->dt, s, es, edot, pls, dpls, dpress);
        if (LOG) {
            double Tn[4];
            load_nodal4(d.T, c, Tn);
            for (int i = 0; i < 6; ++i) {
                rec[6 + i] = (float)(edot[i] * d.clk->dt);
                rec[14 + i] = (float)s[i];
            }
            double amc, anphi, anpsi, hardn, ten_max;
            plastic_props(d.K->M, d.K->M.mix[d.mix[e]], pls_in, amc, anphi, anpsi, hardn, ten_max);
            rec[12] = (float)elem_mean4(Tn[0], Tn[1], Tn[2], Tn[3]);
            rec[13] = (float)pls_in;
            rec[20] = (float)dpls;
            rec[21] = __int_as_float(e);
            rec[22] = __int_as_float(d.clk->steps);
            rec[23] = (float)anpsi;
        }
        store6(d.stress, E, e, s);
        store6(d.strain, E, e, es);
        store6(d.srate, E, e, edot);
        d.pls[e] = pls;
        d.dpls[e] = dpls;
        d.dp[e] = dpress;
        d.tmp_sg[e] = dpress * d.vol[e];
    }
    count_eigen(d, flags);
    if (LOG) {
        const bool w = live && (flags & 16);
        const unsigned m = __ballot_sync(0xffffffffu, w);
        if (m) {
            const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
            unsigned long long base = 0;
            if (lane == leader) base = atomicAdd(&d.clk->nlog, (unsigned long long)__popc(m));
            base = __shfl_sync(0xffffffffu, base, leader);
            const long long idx = (long long)base + __popc(m & ((1u << lane) - 1u));
            if (w && idx < d.ret_cap)
                for (int i = 0; i < kRetRecord; ++i) d.ret_log[idx * kRetRecord + i] = rec[i];
        }
    }
}

// E-C: NMD correction + element force vectors (registers bounded for 9
// blocks of 128 per SM: 1.06 -> 0.99 ms on config 2)
__global__ void __launch_bounds__(128, 9) k_fe_c(Dev d)
{
    int e = gtid();
    if (e >= d.nelem) return;
    const size_t E = d.nelem;
    int4 c = d.conn[e];
    double a[4];
    load_nodal4(d.ntmp, c, a);
    double dpe = sf::add0(a[0]);                // 0 + a0, then the rest; / 4, / 3
    for (int i = 1; i < 4; ++i) dpe += a[i];
    double dp_el = sf::quarter(dpe);
    double ddp = sf::div3(-d.dp[e] + dp_el);
    double s[6];
    load6(d.stress, E, e, s);
    for (int i = 0; i < 3; ++i) s[i] += ddp;
    for (int i = 0; i < 3; ++i) d.stress[i * E + e] = s[i];
    force_elem_body(d, e, c, s);
}

// N-C: force gather, damping, velocity, velocity BCs, coordinates
__global__ void k_fn_c(Dev d)
{
    int n = gtid();
    if (n >= d.nnode) return;
    const Consts &K = *d.K;
    const double dt = d.clk->dt;
    double f[3];
    force_gather(d, n, f);
    stress_bc_node(K, d.bf, n, d.bcflag[n], d.z[n], d.z0[n], f);
    double v[3] = {d.vx[n], d.vy[n], d.vz[n]};
    if (K.is_qs) {
        f[0] = damp(K, f[0], v[0]);
        f[1] = damp(K, f[1], v[1]);
        f[2] = damp(K, f[2], v[2]);
    }
    d.fx[n] = f[0];
    d.fy[n] = f[1];
    d.fz[n] = f[2];
    double m = d.mass[n];
    for (int j = 0; j < 3; ++j) v[j] += dt * f[j] / m;
    vbc_node(K, d.bcflag[n], v);
    d.vx[n] = v[0];
    d.vy[n] = v[1];
    d.vz[n] = v[2];
    const double x = d.x[n] + v[0] * dt, y = d.y[n] + v[1] * dt, z = d.z[n] + v[2] * dt;
    d.x[n] = x;
    d.y[n] = y;
    d.z[n] = z;
    // output.cxx:195-208 stops on NaN/Inf coordinates
    if (not_finite(x) || not_finite(y) || not_finite(z)) atomicOr(&d.clk->status, 0x2u);
}

// E-A: update_mesh element half, rotate_stress, next-step contributions, dt;
// this launch covers the elements from e0 (a multiple of the block size), the
// pass nblocks blocks in all.  Six blocks of 128 per SM (80 registers, a few
// spilled): the pass waits on FP64 results and on instruction fetch more than
// on any pipe, and the extra warps hide more of that (measured 5.16 against
// 5.27 ms at five blocks on config 2)
__global__ void __launch_bounds__(128, 6) k_fe_a(Dev d, int e0, unsigned nblocks)
{
    int e = e0 + gtid();
    const Consts &K = *d.K;
    const bool dt_step = (K.fixed_dt == 0) && (d.clk->steps % 10 == 0);
    if (e == 0) d.clk->mass_valid = 0;
    bool live = e < d.nelem;
    double minh = 0;
    if (live) {
        const size_t E = d.nelem;
        int4 c = d.conn[e];
        double X[4][3];
        load_xyz4(d, c, X);
        double vol = tet_volume(X[0], X[1], X[2], X[3]);
        d.vol_old[e] = d.vol[e];
        d.vol[e] = vol;
        if (not_positive(vol)) atomicOr(&d.clk->status, 0x4u);
        double dx[4], dy[4], dz[4], r1[3], r3[3];
        shape_fn(X, vol, dx, dy, dz, r1, r3);
        store_shp(d, e, dx, dy, dz);
        // the element's dt candidates here, so that the coordinates are dead
        // before the rotation's registers are needed (geometry.cxx:280-300)
        if (dt_step) {
            minh = min_height(X, vol, r1, r3);
        }
        const Mix &x = K.M.mix[d.mix[e]];
        {
            double Tn[4];
            load_nodal4(d.T, c, Tn);
            double rT = mat_rho(K.M, x, elem_mean4(Tn[0], Tn[1], Tn[2], Tn[3]));
            double rho = K.is_qs ? x.rho_qs : rT;
            d.c_mass[e] = rho * vol / 4;
            if (K.thermal) d.c_tmass[e] = rT * x.cp * vol / 4;
        }
        double V[4][3];
        load_vel4(d, c, V);
        double w3, w4, w5, D[6];
        spin_and_rate(V, dx, dy, dz, w3, w4, w5, D);
        if (K.rheol & 1) {
            double s[6];
            const double dt = d.clk->dt;
            load6(d.stress, E, e, s);
            jaumann64(s, dt, w3, w4, w5);
            store6(d.stress, E, e, s);
            load6(d.strain, E, e, s);
            jaumann64(s, dt, w3, w4, w5);
            store6(d.strain, E, e, s);
        }
        next_step_contrib_d(d, e, c, D, dx, dy, dz, vol);
    }
    if (dt_step) dt_reduce_and_finalize(d, minh, live, nblocks);
}

// nodal masses from the fused-pass contributions (used before a download)
__global__ void k_mass_flush(Dev d)
{
    int n = gtid();
    if (n == 0) d.clk->mass_valid = 1;
    if (n >= d.nnode) return;
    const bool thermal = d.K->thermal;
    double vn = 0, m = 0, tm = 0;
    for (int q = d.sup_off[n]; q < d.sup_off[n + 1]; ++q) {
        size_t e = __ldg(d.sup_ent + q) >> 2;
        vn += d.vol[e];
        m += d.c_mass[e];
        if (thermal) tm += d.c_tmass[e];
    }
    d.vol_n[n] = vn;
    d.mass[n] = m;
    d.tmass[n] = tm;
}

// ---- layout conversion ----------------------------------------------------
// rows [row0, row0 + rows) of an AoS block with ncomp components <-> SoA
__global__ void k_aos_to_soa(const double *src, double *dst, int ncomp, long long rows,
                             long long row0, long long ld)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * ncomp) return;
    long long r = i / ncomp;
    int c = (int)(i - r * ncomp);
    dst[c * ld + row0 + r] = src[i];
}
__global__ void k_soa_to_aos(const double *src, double *dst, int ncomp, long long rows,
                             long long row0, long long ld)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * ncomp) return;
    long long r = i / ncomp;
    int c = (int)(i - r * ncomp);
    dst[i] = src[c * ld + row0 + r];
}

// ---- mesh-quality checks (the remesh trigger) --------------------------------
// Arrays both forms keep in FP64.  out[0] = minimum quality (order bits),
// out[1] = first element with that quality, out[2] = first element smaller
// than smallest_vol, out[3] = first bottom node farther than dist from the
// bottom (each ~0ull when there is none).
struct QualityArgs {
    int nelem, nnode;
    const int4 *conn;
    const double *x, *y, *z, *vol;
    const unsigned *bcflag;
    double nf, smallest_vol, bottom, dist;
    int check_bottom;
    double *q;                       // per-element quality (scratch, E doubles)
    unsigned long long *out;
};

__device__ __forceinline__ unsigned long long warp_min64(unsigned long long v)
{
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
    }
    return v;
}
// minimum over the block, one atomicMin by thread 0; every thread of the
// block calls it (blockDim.x a multiple of 32, at most 1024)
__device__ __forceinline__ void block_min_to(unsigned long long v, unsigned long long *dst)
{
    __shared__ unsigned long long part[32];
    v = warp_min64(v);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = part[0];
        for (int i = 1; i < (int)(blockDim.x >> 5); ++i) m = part[i] < m ? part[i] : m;
        if (m != ~0ull) atomicMin(dst, m);
    }
    __syncthreads();     // part is reused by the next call
}

// elem_quality of every element, its minimum, and the first element below
// smallest_vol (remeshing.cxx:1905-1914)
__global__ void k_quality(QualityArgs a)
{
    const int e = gtid();
    unsigned long long qb = ~0ull, tiny = ~0ull;
    if (e < a.nelem) {
        const int4 c = a.conn[e];
        const int n[4] = {c.x, c.y, c.z, c.w};
        double X[4][3];
        for (int i = 0; i < 4; ++i) {
            X[i][0] = __ldg(a.x + n[i]);
            X[i][1] = __ldg(a.y + n[i]);
            X[i][2] = __ldg(a.z + n[i]);
        }
        const double v = a.vol[e];
        const double q = elem_quality(X, v, a.nf);
        a.q[e] = q;
        qb = order_bits(q);
        if (v < a.smallest_vol) tiny = (unsigned long long)e;
    }
    block_min_to(qb, &a.out[0]);
    block_min_to(tiny, &a.out[2]);
}
// the first element with the minimum quality (worst_elem_quality's strict <)
__global__ void k_quality_worst(QualityArgs a)
{
    const int e = gtid();
    unsigned long long w = ~0ull;
    if (e < a.nelem && order_bits(a.q[e]) == a.out[0]) w = (unsigned long long)e;
    block_min_to(w, &a.out[1]);
}
// the first bottom node too far from the bottom (remeshing.cxx:1917-1934)
__global__ void k_bottom_distortion(QualityArgs a)
{
    const int n = gtid();
    unsigned long long f = ~0ull;
    if (n < a.nnode && (a.bcflag[n] & kBoundZ0) && fabs(a.z[n] - a.bottom) > a.dist) f = (unsigned long long)n;
    block_min_to(f, &a.out[3]);
}

__global__ void k_clock_set(Clock *clk, double time, double dt, int steps, int mass_valid)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        clk->time = time;
        clk->dt = dt;
        clk->steps = steps;
        clk->mass_valid = mass_valid;
    }
}
__global__ void k_clock_mass_valid(Clock *clk, int v)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) clk->mass_valid = v;
}
__global__ void k_clock_dt(Clock *clk, double dt)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) clk->dt = dt;
}

}  // namespace des
