// TEST INFRASTRUCTURE -- CPU restatement of the DynEarthSol3D explicit step
// (the parity oracle and the "port" CPU baseline).  Not part of the product.
//
// Layout and loop structure follow the reference: arrays of structures with N
// components per row (array2d.hpp:86-87), OpenMP loops per function, node sums
// gathered over the support lists in ascending element order, the linear
// search for a node's slot in update_temperature / update_force.  Every
// floating-point expression is written with the evaluation order of the
// reference line cited next to it.
#include "des_oracle.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <new>
#include <unordered_map>
#include <utility>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double kYear2Sec = 365.2422 * 86400;                  // constants.hpp:75
const double kPi = 3.1415926535897932384626433832795;
const double kDeg2Rad = kPi / 180;                          // constants.hpp:76
const int kFacet[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};   // constants.hpp:61-67
const unsigned kBoundX0 = 1, kBoundX1 = 2, kBoundY0 = 4, kBoundY1 = 8, kBoundZ0 = 16,
               kBoundZ1 = 32;
const unsigned kBoundAny = 0x3ff;

// std::min / std::max semantics (first argument wins ties and NaN comparisons)
inline double smin(double a, double b) { return (b < a) ? b : a; }
inline double smax(double a, double b) { return (a < b) ? b : a; }

inline double mv(const des_matvec &v, int m) { return v.len == 1 ? v.v[0] : v.v[m]; }

inline double trace3(const double *s) { return s[0] + s[1] + s[2]; }   // utils.hpp:68-75

// utils.hpp:78-87
inline double second_invariant2(const double *t)
{
    double a = (t[0] + t[1] + t[2]) / 3;
    return (0.5 * ((t[0] - a) * (t[0] - a) + (t[1] - a) * (t[1] - a) + (t[2] - a) * (t[2] - a)) +
            t[3] * t[3] + t[4] * t[4] + t[5] * t[5]);
}
inline double second_invariant(const double *t) { return std::sqrt(second_invariant2(t)); }

}  // namespace

struct dso {
    des_params P;
    int nnode = 0, nelem = 0, nmat = 0;
    std::vector<int> conn;            // [nelem][4]
    std::vector<int> markers;         // [nelem][nmat]
    std::vector<unsigned> bcflag;     // [nnode]
    std::vector<int> sup_off, sup_el; // CSR of support lists
    std::vector<int> bnodes[DES_NBDRY];
    std::vector<std::pair<int, int>> bfacets[DES_NBDRY];
    std::vector<double> zeros_n;      // temperature used by compute_mass at init (all zero)

    const int *em(int e) const { return &markers[(size_t)nmat * e]; }

    // ---- MatProps (matprops.cxx:436-461, 595-740) ------------------------
    double arithmetic_mean(const des_matvec &s, int e) const
    {
        if (s.len == 1) return s.v[0];
        const int *n = em(e);
        double result = 0;
        int m = 0;
        for (int i = 0; i < s.len; i++) {
            result += n[i] * s.v[i];
            m += n[i];
        }
        return result / m;
    }
    double harmonic_mean(const des_matvec &s, int e) const
    {
        if (s.len == 1) return s.v[0];
        const int *n = em(e);
        double result = 0;
        int m = 0;
        for (int i = 0; i < s.len; i++) {
            result += n[i] / s.v[i];
            m += n[i];
        }
        return m / result;
    }
    double bulkm(int e) const { return harmonic_mean(P.bulk_modulus, e); }
    double shearm(int e) const { return harmonic_mean(P.shear_modulus, e); }
    double cp(int e) const { return arithmetic_mean(P.heat_capacity, e); }
    double kcond(int e) const { return arithmetic_mean(P.therm_cond, e); }

    double elem_T(int e, const double *T) const
    {
        const int *c = &conn[4 * (size_t)e];
        double t = 0;
        for (int i = 0; i < 4; ++i) t += T[c[i]];
        t /= 4;
        return t;
    }
    double rho(int e, const double *T) const            // matprops.cxx:707-728
    {
        const double celsius0 = 273;
        double t = elem_T(e, T);
        double TinCelsius = t - celsius0;
        double result = 0;
        int n = 0;
        const int *k = em(e);
        for (int m = 0; m < nmat; m++) {
            result += mv(P.rho0, m) * (1 - mv(P.alpha, m) * TinCelsius) * k[m];
            n += k[m];
        }
        return result / n;
    }
    double visc(int e, const double *T, const double *srate) const    // matprops.cxx:607-643
    {
        const double gas_constant = 8.3144;
        const double min_strain_rate = 1e-30;
        double t = elem_T(e, T);
        double edot = second_invariant(srate + 6 * (size_t)e);
        edot = smax(edot, min_strain_rate);
        double result = 0;
        int n = 0;
        const int *k = em(e);
        for (int m = 0; m < nmat; m++) {
            double ve = mv(P.visc_exponent, m);
            double pw = 1 / ve - 1;
            double pw1 = -1 / ve;
            double visc0 = 0.25 * std::pow(edot, pw) * std::pow(0.75 * mv(P.visc_coefficient, m), pw1) *
                           std::exp(mv(P.visc_activation_energy, m) / (ve * gas_constant * t)) * 1e6;
            result += k[m] / visc0;
            n += k[m];
        }
        double v = n / result;
        v = smin(smax(v, P.visc_min), P.visc_max);
        return v;
    }
    void plastic_weakening(int e, double pls, double &cohesion, double &friction_angle,
                           double &dilation_angle, double &hardening) const   // matprops.cxx:646-684
    {
        double c, f, d, h;
        c = f = d = h = 0;
        int n = 0;
        const int *kk = em(e);
        for (int m = 0; m < nmat; m++) {
            int k = kk[m];
            if (k == 0) continue;
            n += k;
            double p0 = mv(P.pls0, m), p1 = mv(P.pls1, m);
            double c0 = mv(P.cohesion0, m), c1 = mv(P.cohesion1, m);
            double f0 = mv(P.friction_angle0, m), f1 = mv(P.friction_angle1, m);
            double d0 = mv(P.dilation_angle0, m), d1 = mv(P.dilation_angle1, m);
            if (pls < p0) {
                c += c0 * k;
                f += f0 * k;
                d += d0 * k;
                h += 0;
            } else if (pls < p1) {
                double p = (pls - p0) / (p1 - p0);
                c += (c0 + p * (c1 - c0)) * k;
                f += (f0 + p * (f1 - f0)) * k;
                d += (d0 + p * (d1 - d0)) * k;
                h += (c1 - c0) / (p1 - p0) * k;
            } else {
                c += c1 * k;
                f += f1 * k;
                d += d1 * k;
                h += 0;
            }
        }
        cohesion = c / n;
        friction_angle = f / n;
        dilation_angle = d / n;
        hardening = h / n;
    }
    void plastic_props(int e, double pls, double &amc, double &anphi, double &anpsi,
                       double &hardn, double &ten_max) const             // matprops.cxx:687-704
    {
        double cohesion, phi, psi;
        plastic_weakening(e, pls, cohesion, phi, psi, hardn);
        double sphi = std::sin(phi * kDeg2Rad);
        double spsi = std::sin(psi * kDeg2Rad);
        anphi = (1 + sphi) / (1 - sphi);
        anpsi = (1 + spsi) / (1 - spsi);
        amc = 2 * cohesion * std::sqrt(anphi);
        ten_max = (phi == 0) ? P.tension_max : smin(P.tension_max, cohesion / std::tan(phi * kDeg2Rad));
    }

    // index of node n among the element's vertices (fields.cxx:154-159)
    int slot_of(int e, int n) const
    {
        const int *c = &conn[4 * (size_t)e];
        for (int i = 0; i < 4; i++)
            if (n == c[i]) return i;
        return -1;
    }
};

// ---------------------------------------------------------------------------
// 3x3 symmetric eigen-solver: oracle/des_oracle_eig.cpp (a translation unit of
// its own, so it can be built with the reference's 3x3-C flags as well)
// ---------------------------------------------------------------------------
extern "C" int dso_eig_hybrid(const double A[3][3], double Q[3][3], double w[3]);

namespace {

inline int eig_hybrid(const double A[3][3], double Q[3][3], double w[3])
{
    return dso_eig_hybrid(A, Q, w);
}

// rheology.cxx:16-71: eigen-decomposition, then sort p ascending with the
// matching eigenvector columns
void principal3(const double *s, double p[3], double v[3][3])
{
    double a[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    a[0][0] = s[0];
    a[1][1] = s[1];
    a[2][2] = s[2];
    a[0][1] = s[3];
    a[0][2] = s[4];
    a[1][2] = s[5];
    eig_hybrid(a, v, p);
    auto swap_cols = [&](int i, int j) {
        double tmp = p[i];
        p[i] = p[j];
        p[j] = tmp;
        for (int r = 0; r < 3; ++r) {
            double b = v[r][i];
            v[r][i] = v[r][j];
            v[r][j] = b;
        }
    };
    if (p[0] > p[1]) swap_cols(0, 1);
    if (p[1] > p[2]) swap_cols(1, 2);
    if (p[0] > p[1]) swap_cols(0, 1);
}

// ---------------------------------------------------------------------------
// rheology.cxx:108-302 (3D forms)
// ---------------------------------------------------------------------------
void elastic(double bulkm, double shearm, const double *de, double *s)
{
    double lambda = bulkm - 2. / 3 * shearm;
    double dev = trace3(de);
    for (int i = 0; i < 3; ++i) s[i] += 2 * shearm * de[i] + lambda * dev;
    for (int i = 3; i < 6; ++i) s[i] += 2 * shearm * de[i];
}

void maxwell(double bulkm, double shearm, double viscosity, double dt, double dv,
             const double *de, double *s)
{
    double tmp = 0.5 * dt * shearm / viscosity;
    double f1 = 1 - tmp;
    double f2 = 1 / (1 + tmp);
    double dev = trace3(de) / 3;
    double s0 = trace3(s) / 3;
    for (int i = 0; i < 3; ++i)
        s[i] = ((s[i] - s0) * f1 + 2 * shearm * (de[i] - dev)) * f2 + s0 + bulkm * dv;
    for (int i = 3; i < 6; ++i) s[i] = (s[i] * f1 + 2 * shearm * de[i]) * f2;
}

void viscous(double bulkm, double viscosity, double total_dv, const double *edot, double *s)
{
    double dev = trace3(edot) / 3;
    for (int i = 0; i < 3; ++i) s[i] = 2 * viscosity * (edot[i] - dev) + bulkm * total_dv;
    for (int i = 3; i < 6; ++i) s[i] = 2 * viscosity * edot[i];
}

void elasto_plastic(double bulkm, double shearm, double amc, double anphi, double anpsi,
                    double hardn, double ten_max, const double *de, double &depls, double *s,
                    int &failure_mode)
{
    elastic(bulkm, shearm, de, s);
    depls = 0;
    failure_mode = 0;
    double p[3];
    double v[3][3];
    principal3(s, p, v);
    double fs = p[0] - p[2] * anphi + amc;
    double ft = p[2] - ten_max;
    if (fs > 0 && ft < 0) return;
    double pa = std::sqrt(1 + anphi * anphi) + anphi;
    double ps = ten_max * anphi - amc;
    double h = p[2] - ten_max + pa * (p[0] - ps);
    double a1 = bulkm + 4. / 3 * shearm;
    double a2 = bulkm - 2. / 3 * shearm;
    double alam;
    if (h < 0) {
        failure_mode = 10;
        alam = fs / (a1 - a2 * anpsi + a1 * anphi * anpsi - a2 * anphi + 2 * std::sqrt(anphi) * hardn);
        p[0] -= alam * (a1 - a2 * anpsi);
        p[1] -= alam * (a2 - a2 * anpsi);
        p[2] -= alam * (a2 - a1 * anpsi);
        depls = std::fabs(alam) * std::sqrt((7 + 4 * anpsi + 7 * anpsi * anpsi) / 18);
    } else {
        failure_mode = 1;
        alam = ft / a1;
        p[0] -= alam * a2;
        p[1] -= alam * a2;
        p[2] -= alam * a1;
        depls = std::fabs(alam) * std::sqrt(7. / 18);
    }
    double ss[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int m = 0; m < 3; m++)
        for (int n = m; n < 3; n++)
            for (int k = 0; k < 3; k++) ss[m][n] += v[m][k] * v[n][k] * p[k];
    s[0] = ss[0][0];
    s[1] = ss[1][1];
    s[2] = ss[2][2];
    s[3] = ss[0][1];
    s[4] = ss[0][2];
    s[5] = ss[1][2];
}

// bc.cxx:15-36
void facet_normal(int f, const int *c, const double *coord, double *normal, double &zcenter)
{
    int n0 = c[kFacet[f][0]], n1 = c[kFacet[f][1]], n2 = c[kFacet[f][2]];
    double v01[3], v02[3];
    for (int i = 0; i < 3; ++i) {
        v01[i] = coord[3 * (size_t)n1 + i] - coord[3 * (size_t)n0 + i];
        v02[i] = coord[3 * (size_t)n2 + i] - coord[3 * (size_t)n0 + i];
    }
    normal[0] = (v01[1] * v02[2] - v01[2] * v02[1]) / 2;
    normal[1] = (v01[2] * v02[0] - v01[0] * v02[2]) / 2;
    normal[2] = (v01[0] * v02[1] - v01[1] * v02[0]) / 2;
    zcenter = (coord[3 * (size_t)n0 + 2] + coord[3 * (size_t)n1 + 2] + coord[3 * (size_t)n2 + 2]) / 3;
}

// geometry.cxx:29-49
double tet_volume(const double *d0, const double *d1, const double *d2, const double *d3)
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
    return (x01 * (y23 * z12 - y12 * z23) + x12 * (y01 * z23 - y23 * z01) +
            x23 * (y12 * z01 - y01 * z12)) / 6;
}

// geometry.cxx:53-83 (3D)
double tri_area(const double *a, const double *b, const double *c)
{
    double ab0 = b[0] - a[0], ab1 = b[1] - a[1];
    double ac0 = c[0] - a[0], ac1 = c[1] - a[1];
    double ab2 = b[2] - a[2], ac2 = c[2] - a[2];
    double d0 = ab1 * ac2 - ab2 * ac1;
    double d1 = ab2 * ac0 - ab0 * ac2;
    double d2 = ab0 * ac1 - ab1 * ac0;
    return std::sqrt(d0 * d0 + d1 * d1 + d2 * d2) / 2;
}

// fields.cxx:419-433
void jaumann(double *s, double dt, double w3, double w4, double w5)
{
    double inc[6];
    inc[0] = -2.0 * s[3] * w3 - 2.0 * s[4] * w4;
    inc[1] = 2.0 * s[3] * w3 - 2.0 * s[5] * w5;
    inc[2] = 2.0 * s[4] * w4 + 2.0 * s[5] * w5;
    inc[3] = s[0] * w3 - s[1] * w3 - s[4] * w5 - s[5] * w4;
    inc[4] = s[0] * w4 - s[2] * w4 + s[3] * w5 - s[5] * w3;
    inc[5] = s[1] * w5 - s[2] * w5 + s[3] * w4 + s[4] * w3;
    for (int i = 0; i < 6; ++i) s[i] += dt * inc[i];
}

// matprops.cxx:523-535, option 0 (lithostatic); the PREM options are not restated
// matprops.cxx:20-108: the pressure of the PREM model (kbar -> 1e8 Pa) at
// tabulated depths, linearly interpolated; `modified` takes the average
// continental crust of option 2 for the top three depths
double prem_pressure(double depth, bool modified)
{
    static const double km[46] = {0,    3,    15,   24.4, 40,   60,   80,   115,  150,  185,  220,  265,
                                  310,  355,  400,  450,  500,  550,  600,  635,  670,  721,  771,  871,
                                  971,  1071, 1171, 1271, 1371, 1471, 1571, 1671, 1771, 1871, 1971, 2071,
                                  2171, 2271, 2371, 2471, 2571, 2671, 2741, 2771, 2871, 2891};
    static const double kbar[46] = {0,      0.3,    3.3,    6.0,    11.2,   17.8,   24.5,   36.1,   47.8,
                                    59.4,   71.1,   86.4,   102.0,  117.7,  133.5,  152.2,  171.3,  190.7,
                                    210.4,  224.3,  238.3,  260.7,  282.9,  327.6,  372.8,  418.6,  464.8,
                                    511.6,  558.9,  606.8,  655.2,  704.1,  753.5,  803.6,  854.3,  905.6,
                                    957.6,  1010.3, 1063.8, 1118.2, 1173.4, 1229.7, 1269.7, 1287.0, 1345.6,
                                    1357.5};
    static const double crust[3] = {0.82, 4.1, 6.7};
    // the reference writes each value as a literal (3e3, 0.3e8, ...); the
    // products below are exact for every entry, so they are the same doubles
    auto d = [](int i) { return std::round(km[i] * 10) * 100.0; };
    auto p = [&](int i) {
        return (modified && i >= 1 && i <= 3) ? std::round(crust[i - 1] * 100) * 1e6 : std::round(kbar[i] * 10) * 1e7;
    };
    if (depth <= 0) return 0;
    int n;
    for (n = 1; n < 46; n++)
        if (depth <= d(n)) break;
    if (n == 46) n = 45;
    return p(n - 1) + (p(n) - p(n - 1)) * (depth - d(n - 1)) / (d(n) - d(n - 1));
}

// matprops.cxx:523-535
double ref_pressure(const des_params &P, double z)
{
    double depth = -z;
    if (P.ref_pressure_option == 1) return prem_pressure(depth, false);
    if (P.ref_pressure_option == 2) return prem_pressure(depth, true);
    return P.rho0.v[0] * P.gravity * depth;
}

}  // namespace

// ===========================================================================
extern "C" {

int dso_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int dso_set_params(dso *o, const des_params *p)
{
    if (!o || !p) return DES_ERR_ARG;
    o->P = *p;
    return DES_OK;
}

// MatProps reads var.elemmarkers through a reference (matprops.cxx:165), so
// the counts phase_changes writes (phasechanges.cxx:248-254) take effect in
// the next property lookup
int dso_set_elemmarkers(dso *o, const int *elemmarkers)
{
    if (!o || !elemmarkers) return DES_ERR_ARG;
    o->markers.assign(elemmarkers, elemmarkers + (size_t)o->nmat * o->nelem);
    return DES_OK;
}

int dso_create(const des_mesh_view *m, const des_params *p, dso **out)
{
    if (!m || !p || !out || m->nnode < 1 || m->nelem < 1 || m->nmat < 1) return DES_ERR_ARG;
    dso *o = new (std::nothrow) dso;
    if (!o) return DES_ERR_NOMEM;
    o->P = *p;
    o->nnode = m->nnode;
    o->nelem = m->nelem;
    o->nmat = m->nmat;
    o->conn.assign(m->connectivity, m->connectivity + 4 * (size_t)m->nelem);
    if (m->elemmarkers)
        o->markers.assign(m->elemmarkers, m->elemmarkers + (size_t)m->nmat * m->nelem);
    else
        o->markers.assign((size_t)m->nmat * m->nelem, 0);
    o->zeros_n.assign(m->nnode, 0.0);

    // create_boundary_flags2 (mesh.cxx:1529-1539)
    o->bcflag.assign(m->nnode, 0u);
    for (int i = 0; i < m->nseg; ++i) {
        unsigned flag = static_cast<unsigned>(m->segflag[i]);
        const int *n = m->segment + 3 * (size_t)i;
        for (int j = 0; j < 3; ++j) o->bcflag[n[j]] |= flag;
    }
    // create_boundary_nodes (mesh.cxx:1553-1566)
    for (int i = 0; i < m->nnode; ++i)
        for (int j = 0; j < DES_NBDRY; ++j)
            if (o->bcflag[i] & (1u << j)) o->bnodes[j].push_back(i);
    // create_boundary_facets (mesh.cxx:1633-1682): the reference scan for small
    // meshes, an exact hash lookup otherwise (same result: the scan takes the
    // first facet with the segment's node set)
    auto ordered = [](int x, int y, int z) {
        int a[3] = {x, y, z};
        std::sort(a, a + 3);
        return std::make_pair(((uint64_t)(uint32_t)a[0] << 32) | (uint32_t)a[1], a[2]);
    };
    bool small = (long long)m->nseg * m->nelem <= 400000000LL;
    std::map<std::pair<uint64_t, int>, int> first_owner;
    if (!small) {
        for (int e = m->nelem - 1; e >= 0; --e) {
            const int *c = &o->conn[4 * (size_t)e];
            for (int f = 3; f >= 0; --f) {
                int a = c[kFacet[f][0]], b = c[kFacet[f][1]], d = c[kFacet[f][2]];
                if ((o->bcflag[a] & o->bcflag[b] & o->bcflag[d]) == 0u) continue;
                first_owner[ordered(a, b, d)] = 4 * e + f;
            }
        }
    }
    for (int i = 0; i < m->nseg; ++i) {
        unsigned flag = static_cast<unsigned>(m->segflag[i]);
        if ((flag & kBoundAny) == 0) continue;
        const int *sg = m->segment + 3 * (size_t)i;
        auto af = ordered(sg[0], sg[1], sg[2]);
        bool found = false;
        if (small) {
            for (int e = 0; e < m->nelem && !found; ++e) {
                const int *c = &o->conn[4 * (size_t)e];
                for (int f = 0; f < 4 && !found; ++f) {
                    if ((flag & o->bcflag[c[kFacet[f][0]]] & o->bcflag[c[kFacet[f][1]]] &
                         o->bcflag[c[kFacet[f][2]]]) == 0u)
                        continue;
                    if (ordered(c[kFacet[f][0]], c[kFacet[f][1]], c[kFacet[f][2]]) == af) {
                        for (int k = 0; k < DES_NBDRY; ++k) {
                            if (flag == (1u << k)) {
                                o->bfacets[k].push_back(std::make_pair(e, f));
                                found = true;
                                break;
                            }
                        }
                    }
                }
            }
        } else {
            auto it = first_owner.find(af);
            if (it != first_owner.end()) {
                for (int k = 0; k < DES_NBDRY; ++k) {
                    if (flag == (1u << k)) {
                        o->bfacets[k].push_back(std::make_pair(it->second >> 2, it->second & 3));
                        found = true;
                        break;
                    }
                }
            }
        }
        if (!found) {
            delete o;
            return DES_ERR_TOPOLOGY;
        }
    }
    // create_support (mesh.cxx:1703-1717) as CSR
    o->sup_off.assign(m->nnode + 1, 0);
    for (size_t q = 0; q < o->conn.size(); ++q) o->sup_off[o->conn[q] + 1]++;
    for (int n = 0; n < m->nnode; ++n) o->sup_off[n + 1] += o->sup_off[n];
    o->sup_el.assign(o->conn.size(), 0);
    std::vector<int> cur(o->sup_off.begin(), o->sup_off.end() - 1);
    for (int e = 0; e < m->nelem; ++e)
        for (int i = 0; i < 4; ++i) o->sup_el[cur[o->conn[4 * (size_t)e + i]]++] = e;
    *out = o;
    return DES_OK;
}

void dso_destroy(dso *o) { delete o; }

int dso_bcflag(const dso *o, unsigned *bcflag)
{
    std::memcpy(bcflag, o->bcflag.data(), sizeof(unsigned) * o->nnode);
    return DES_OK;
}
int dso_support(const dso *o, int *offsets, int *elems)
{
    std::memcpy(offsets, o->sup_off.data(), sizeof(int) * (o->nnode + 1));
    std::memcpy(elems, o->sup_el.data(), sizeof(int) * o->sup_el.size());
    return DES_OK;
}
int dso_bnodes(const dso *o, int b, int *count, int *nodes)
{
    if (b < 0 || b >= DES_NBDRY) return DES_ERR_ARG;
    *count = (int)o->bnodes[b].size();
    if (nodes) std::memcpy(nodes, o->bnodes[b].data(), sizeof(int) * o->bnodes[b].size());
    return DES_OK;
}
int dso_bfacets(const dso *o, int b, int *count, int *pairs)
{
    if (b < 0 || b >= DES_NBDRY) return DES_ERR_ARG;
    *count = (int)o->bfacets[b].size();
    if (pairs)
        for (size_t q = 0; q < o->bfacets[b].size(); ++q) {
            pairs[2 * q] = o->bfacets[b][q].first;
            pairs[2 * q + 1] = o->bfacets[b][q].second;
        }
    return DES_OK;
}

// bc.cxx:90-179
int dso_boundary_normals(dso *o, const double *coord, des_params *p)
{
    for (int i = 0; i < DES_NBDRY; i++) {
        double normal[3] = {0};
        if (o->bfacets[i].size() == 0) continue;
        for (auto j = o->bfacets[i].begin(); j < o->bfacets[i].end(); ++j) {
            double tmp;
            facet_normal(j->second, &o->conn[4 * (size_t)j->first], coord, normal, tmp);
            double len = 0;
            for (int d = 0; d < 3; d++) len += normal[d] * normal[d];
            len = std::sqrt(len);
            for (int d = 0; d < 3; d++) normal[d] = normal[d] / len;
            if (j == o->bfacets[i].begin()) {
                for (int d = 0; d < 3; d++) p->bnormals[i][d] = normal[d];
                if (i < 6) break;
            } else {
                double diff2 = 0;
                for (int d = 0; d < 3; d++)
                    diff2 += (p->bnormals[i][d] - normal[d]) * (p->bnormals[i][d] - normal[d]);
                if (diff2 > 1e-12) return DES_ERR_OPTION;
            }
        }
    }
    for (int i = 0; i < DES_NBDRY; i++) {
        if (o->bfacets[i].size() == 0) continue;
        for (int j = i + 1; j < DES_NBDRY; j++) {
            if (o->bfacets[j].size() == 0) continue;
            double *s = p->edge_vectors[i][j];
            if (std::abs(p->bnormals[i][2]) < 1e-15 && std::abs(p->bnormals[j][2]) < 1e-15) {
                s[0] = s[1] = 0;
                s[2] = 1;
            } else {
                s[0] = p->bnormals[i][1] * p->bnormals[j][2] - p->bnormals[i][2] * p->bnormals[j][1];
                s[1] = p->bnormals[i][2] * p->bnormals[j][0] - p->bnormals[i][0] * p->bnormals[j][2];
                s[2] = p->bnormals[i][0] * p->bnormals[j][1] - p->bnormals[i][1] * p->bnormals[j][0];
            }
        }
    }
    o->P = *p;
    return DES_OK;
}

// fields.cxx:108-172
int dso_update_temperature(dso *o, des_state_view *s)
{
    const double surface_temperature = o->P.surface_temperature;
    double *T = s->temperature;
    #pragma omp parallel for
    for (int e = 0; e < o->nelem; e++) {
        const int *conn = &o->conn[4 * (size_t)e];
        double *tr = s->tmp_result + 12 * (size_t)e;
        double kv = o->kcond(e) * s->volume[e];
        const double *dx = s->shpdx + 4 * (size_t)e;
        const double *dy = s->shpdy + 4 * (size_t)e;
        const double *dz = s->shpdz + 4 * (size_t)e;
        for (int i = 0; i < 4; ++i) {
            double diffusion = 0.;
            for (int j = 0; j < 4; ++j)
                diffusion += (dx[i] * dx[j] + dy[i] * dy[j] + dz[i] * dz[j]) * T[conn[j]];
            tr[i] = diffusion * kv;
        }
    }
    #pragma omp parallel for
    for (int n = 0; n < o->nnode; n++) {
        double *tdot = s->ntmp;
        tdot[n] = 0;
        for (int q = o->sup_off[n]; q < o->sup_off[n + 1]; ++q) {
            int e = o->sup_el[q];
            int i = o->slot_of(e, n);
            tdot[n] += s->tmp_result[12 * (size_t)e + i];
        }
        if (o->bcflag[n] & kBoundZ1)
            T[n] = surface_temperature;
        else
            T[n] -= tdot[n] * s->dt / s->tmass[n];
    }
    return DES_OK;
}

// fields.cxx:175-247
int dso_update_strain_rate(dso *o, des_state_view *st)
{
    #pragma omp parallel for
    for (int e = 0; e < o->nelem; ++e) {
        const int *conn = &o->conn[4 * (size_t)e];
        const double *dx = st->shpdx + 4 * (size_t)e;
        const double *dy = st->shpdy + 4 * (size_t)e;
        const double *dz = st->shpdz + 4 * (size_t)e;
        double *s = st->strain_rate + 6 * (size_t)e;
        const double *v[4];
        for (int i = 0; i < 4; ++i) v[i] = st->vel + 3 * (size_t)conn[i];
        s[0] = 0;
        for (int i = 0; i < 4; ++i) s[0] += v[i][0] * dx[i];
        s[1] = 0;
        for (int i = 0; i < 4; ++i) s[1] += v[i][1] * dy[i];
        s[2] = 0;
        for (int i = 0; i < 4; ++i) s[2] += v[i][2] * dz[i];
        s[3] = 0;
        for (int i = 0; i < 4; ++i) s[3] += 0.5 * (v[i][0] * dy[i] + v[i][1] * dx[i]);
        s[4] = 0;
        for (int i = 0; i < 4; ++i) s[4] += 0.5 * (v[i][0] * dz[i] + v[i][2] * dx[i]);
        s[5] = 0;
        for (int i = 0; i < 4; ++i) s[5] += 0.5 * (v[i][1] * dz[i] + v[i][2] * dy[i]);
    }
    return DES_OK;
}

// geometry.cxx:117-151
int dso_compute_dvoldt(dso *o, des_state_view *s)
{
    #pragma omp parallel for
    for (int e = 0; e < o->nelem; e++) {
        double dj = trace3(s->strain_rate + 6 * (size_t)e);
        s->tmp_result_sg[e] = dj * s->volume[e];
    }
    #pragma omp parallel for
    for (int n = 0; n < o->nnode; n++) {
        double *dvoldt = s->ntmp;
        dvoldt[n] = 0.;
        for (int q = o->sup_off[n]; q < o->sup_off[n + 1]; ++q) dvoldt[n] += s->tmp_result_sg[o->sup_el[q]];
        dvoldt[n] /= s->volume_n[n];
    }
    return DES_OK;
}

// geometry.cxx:154-182
int dso_compute_edvoldt(dso *o, des_state_view *s)
{
    #pragma omp parallel for
    for (int e = 0; e < o->nelem; ++e) {
        const int *conn = &o->conn[4 * (size_t)e];
        double dj = 0;
        for (int i = 0; i < 4; ++i) dj += s->ntmp[conn[i]];
        s->edvoldt[e] = dj / 4;
    }
    return DES_OK;
}

// rheology.cxx:513-654 (3D)
int dso_update_stress(dso *o, des_state_view *st)
{
    const int rheol = o->P.rheol_type;
    if (rheol != DES_RH_ELASTIC && rheol != DES_RH_VISCOUS && rheol != DES_RH_MAXWELL &&
        rheol != DES_RH_EP && rheol != DES_RH_EVP)
        return DES_ERR_OPTION;
    const double dt = st->dt;
    #pragma omp parallel for
    for (int e = 0; e < o->nelem; ++e) {
        double *s = st->stress + 6 * (size_t)e;
        double *es = st->strain + 6 * (size_t)e;
        double *edot = st->strain_rate + 6 * (size_t)e;
        double old_s = trace3(s);
        {
            double div = trace3(edot);
            for (int i = 0; i < 3; ++i) edot[i] += (st->edvoldt[e] - div) / 3;
        }
        for (int i = 0; i < 6; ++i) es[i] += edot[i] * dt;
        double de[6];
        for (int i = 0; i < 6; ++i) de[i] = edot[i] * dt;
        switch (rheol) {
        case DES_RH_ELASTIC:
            elastic(o->bulkm(e), o->shearm(e), de, s);
            break;
        case DES_RH_VISCOUS: {
            double bulkm = o->bulkm(e);
            double viscosity = o->visc(e, st->temperature, st->strain_rate);
            double total_dv = trace3(es);
            viscous(bulkm, viscosity, total_dv, edot, s);
        } break;
        case DES_RH_MAXWELL: {
            double bulkm = o->bulkm(e);
            double shearm = o->shearm(e);
            double viscosity = o->visc(e, st->temperature, st->strain_rate);
            double dv = st->volume[e] / st->volume_old[e] - 1;
            maxwell(bulkm, shearm, viscosity, dt, dv, de, s);
        } break;
        case DES_RH_EP: {
            double depls = 0;
            double bulkm = o->bulkm(e);
            double shearm = o->shearm(e);
            double amc, anphi, anpsi, hardn, ten_max;
            o->plastic_props(e, st->plstrain[e], amc, anphi, anpsi, hardn, ten_max);
            int failure_mode;
            elasto_plastic(bulkm, shearm, amc, anphi, anpsi, hardn, ten_max, de, depls, s, failure_mode);
            st->plstrain[e] += depls;
            st->delta_plstrain[e] = depls;
        } break;
        case DES_RH_EVP: {
            double depls = 0;
            double bulkm = o->bulkm(e);
            double shearm = o->shearm(e);
            double viscosity = o->visc(e, st->temperature, st->strain_rate);
            double dv = st->volume[e] / st->volume_old[e] - 1;
            double sv[6];
            for (int i = 0; i < 6; ++i) sv[i] = s[i];
            maxwell(bulkm, shearm, viscosity, dt, dv, de, sv);
            double svII = second_invariant2(sv);
            double amc, anphi, anpsi, hardn, ten_max;
            o->plastic_props(e, st->plstrain[e], amc, anphi, anpsi, hardn, ten_max);
            double sp[6];
            for (int i = 0; i < 6; ++i) sp[i] = s[i];
            int failure_mode;
            elasto_plastic(bulkm, shearm, amc, anphi, anpsi, hardn, ten_max, de, depls, sp, failure_mode);
            double spII = second_invariant2(sp);
            if (svII < spII) {
                for (int i = 0; i < 6; ++i) s[i] = sv[i];
            } else {
                for (int i = 0; i < 6; ++i) s[i] = sp[i];
                st->plstrain[e] += depls;
                st->delta_plstrain[e] = depls;
            }
        } break;
        }
        st->dpressure[e] = trace3(s) - old_s;
    }
    return DES_OK;
}

// geometry.cxx:185-254
int dso_NMD_stress(dso *o, des_state_view *st)
{
    #pragma omp parallel for
    for (int e = 0; e < o->nelem; e++) st->tmp_result_sg[e] = st->dpressure[e] * st->volume[e];
    #pragma omp parallel for
    for (int n = 0; n < o->nnode; n++) {
        double *dp_nd = st->ntmp;
        dp_nd[n] = 0;
        for (int q = o->sup_off[n]; q < o->sup_off[n + 1]; ++q) dp_nd[n] += st->tmp_result_sg[o->sup_el[q]];
        dp_nd[n] /= st->volume_n[n];
    }
    #pragma omp parallel for
    for (int e = 0; e < o->nelem; ++e) {
        const int *conn = &o->conn[4 * (size_t)e];
        double dp = 0;
        for (int i = 0; i < 4; ++i) dp += st->ntmp[conn[i]];
        double dp_el = dp / 4;
        double *s = st->stress + 6 * (size_t)e;
        double dp_orig = st->dpressure[e];
        double ddp = (-dp_orig + dp_el) / 3;
        for (int i = 0; i < 3; ++i) s[i] += ddp;
    }
    return DES_OK;
}

namespace {

// bc.cxx:503-595
void apply_stress_bcs(dso *o, des_state_view *st)
{
    const des_params &P = o->P;
    if (P.gravity == 0) return;
    for (int i = 0; i < DES_NBDRY; i++) {
        if (P.vbc_types[i] != 0 && P.vbc_types[i] != 2 && P.vbc_types[i] != 4) continue;
        if (i == 4 && !P.has_winkler_foundation) continue;
        if (i == 5 && !P.has_water_loading) continue;
        const auto &bdry = o->bfacets[i];
        const int nbound = (int)bdry.size();
        std::vector<double> tmp_val(3 * (size_t)nbound);
        std::vector<int> tmp_ind(3 * (size_t)nbound);
        for (int n = 0; n < nbound; ++n) {
            int e = bdry[n].first;
            int f = bdry[n].second;
            const int *conn = &o->conn[4 * (size_t)e];
            double normal[3];
            double zcenter;
            facet_normal(f, conn, st->coord, normal, zcenter);
            double p;
            if (i == 4 && P.has_winkler_foundation) {
                p = P.compensation_pressure -
                    (o->rho(e, st->temperature) + P.winkler_delta_rho) * P.gravity * (zcenter + P.zlength);
            } else if (i == 5 && P.has_water_loading) {
                const double sea_level = 0;
                p = 0;
                if (zcenter < sea_level) {
                    const double sea_water_density = 1030;
                    p = sea_water_density * P.gravity * (sea_level - zcenter);
                }
            } else {
                p = ref_pressure(P, zcenter);
            }
            for (int j = 0; j < 3; ++j) tmp_ind[3 * n + j] = conn[kFacet[f][j]];
            for (int d = 0; d < 3; ++d) tmp_val[3 * n + d] = p * normal[d] / 3;
        }
        for (size_t jj = 0; jj < o->bnodes[i].size(); jj++) {
            int node = o->bnodes[i][jj];
            for (int facet = 0; facet < nbound; ++facet)
                for (int j = 0; j < 3; ++j)
                    if (tmp_ind[3 * facet + j] == node) {
                        for (int d = 0; d < 3; ++d) st->force[3 * (size_t)node + d] -= tmp_val[3 * facet + d];
                        break;
                    }
        }
    }
    if (P.has_elastic_foundation && st->coord0) {
        for (int n : o->bnodes[4])
            st->force[3 * (size_t)n + 2] -=
                P.elastic_foundation_constant * (st->coord[3 * (size_t)n + 2] - st->coord0[3 * (size_t)n + 2]);
    }
}

// fields.cxx:250-309
int apply_damping(dso *o, des_state_view *st)
{
    double *ff = st->force;
    const double *v = st->vel;
    const double small_vel = 1e-13;
    const double fac = o->P.damping_factor;
    const int n3 = o->nnode * 3;
    switch (o->P.damping_option) {
    case 0:
        break;
    case 1:
        #pragma omp parallel for
        for (int i = 0; i < n3; ++i)
            if (std::fabs(v[i]) > small_vel) ff[i] -= fac * std::copysign(ff[i], v[i]);
        break;
    case 2:
        #pragma omp parallel for
        for (int i = 0; i < n3; ++i) ff[i] -= fac * ff[i];
        break;
    case 3:
        #pragma omp parallel for
        for (int i = 0; i < n3; ++i) {
            if ((ff[i] < 0) == (v[i] < 0))
                ff[i] -= fac * ff[i];
            else
                ff[i] += (1 - fac) * ff[i];
        }
        break;
    case 4:
        break;
    default:
        return DES_ERR_OPTION;
    }
    return DES_OK;
}

}  // namespace

// fields.cxx:312-375
int dso_update_force(dso *o, des_state_view *st)
{
    const double gravity = o->P.gravity;
    #pragma omp parallel for
    for (int e = 0; e < o->nelem; e++) {
        const double *dx = st->shpdx + 4 * (size_t)e;
        const double *dy = st->shpdy + 4 * (size_t)e;
        const double *dz = st->shpdz + 4 * (size_t)e;
        const double *s = st->stress + 6 * (size_t)e;
        const double vol = st->volume[e];
        double *tr = st->tmp_result + 12 * (size_t)e;
        double buoy = 0;
        if (gravity != 0) buoy = o->rho(e, st->temperature) * gravity / 4;
        for (int i = 0; i < 4; ++i) {
            tr[i] = (s[0] * dx[i] + s[3] * dy[i] + s[4] * dz[i]) * vol;
            tr[i + 4] = (s[3] * dx[i] + s[1] * dy[i] + s[5] * dz[i]) * vol;
            tr[i + 8] = (s[4] * dx[i] + s[5] * dy[i] + s[2] * dz[i] + buoy) * vol;
        }
    }
    #pragma omp parallel for
    for (int n = 0; n < o->nnode; n++) {
        double *f = st->force + 3 * (size_t)n;
        f[0] = f[1] = f[2] = 0;
        for (int q = o->sup_off[n]; q < o->sup_off[n + 1]; ++q) {
            int e = o->sup_el[q];
            int i = o->slot_of(e, n);
            const double *tr = st->tmp_result + 12 * (size_t)e;
            for (int j = 0; j < 3; j++) f[j] -= tr[i + 4 * j];
        }
    }
    apply_stress_bcs(o, st);
    if (o->P.is_quasi_static) return apply_damping(o, st);
    return DES_OK;
}

// fields.cxx:378-393
int dso_update_velocity(dso *o, des_state_view *st)
{
    const double dt = st->dt;
    #pragma omp parallel for
    for (int i = 0; i < o->nnode; ++i)
        for (int j = 0; j < 3; j++) st->vel[3 * (size_t)i + j] += dt * st->force[3 * (size_t)i + j] / st->mass[i];
    return DES_OK;
}

// bc.cxx:182-500 (3D)
int dso_apply_vbcs(dso *o, des_state_view *st)
{
    const des_params &P = o->P;
    const int vx0 = P.vbc_types[0], vx1 = P.vbc_types[1], vy0 = P.vbc_types[2],
              vy1 = P.vbc_types[3], vz0 = P.vbc_types[4], vz1 = P.vbc_types[5];
    const double ux0 = P.vbc_values[0], ux1 = P.vbc_values[1], uy0 = P.vbc_values[2],
                 uy1 = P.vbc_values[3], uz0 = P.vbc_values[4], uz1 = P.vbc_values[5];
    #pragma omp parallel for
    for (int i = 0; i < o->nnode; ++i) {
        uint32_t flag = o->bcflag[i];
        if (!(flag & kBoundAny)) continue;
        double *v = st->vel + 3 * (size_t)i;
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
        for (int ib = 6; ib <= 9; ib++) {
            const double *n = P.bnormals[ib];
            if (!(flag & (1u << ib))) continue;
            double fac = 0;
            switch (P.vbc_types[ib]) {
            case 1:
                if (flag == (1u << ib)) {
                    double vn = 0;
                    for (int d = 0; d < 3; d++) vn += v[d] * n[d];
                    for (int d = 0; d < 3; d++) v[d] += (P.vbc_values[ib] - vn) * n[d];
                } else {
                    for (int ic = 0; ic < ib; ic++) {
                        if (!(flag & (1u << ic))) continue;
                        if (P.vbc_types[ic] == 0) {
                            double vn = 0;
                            for (int d = 0; d < 3; d++) vn += v[d] * n[d];
                            for (int d = 0; d < 3; d++) v[d] += (P.vbc_values[ib] - vn) * n[d];
                        } else if (P.vbc_types[ic] == 1) {
                            const double *edge = P.edge_vectors[ic][ib];
                            double ve = 0;
                            for (int d = 0; d < 3; d++) ve += v[d] * edge[d];
                            for (int d = 0; d < 3; d++) v[d] = ve * edge[d];
                        }
                    }
                }
                break;
            case 3:
                for (int d = 0; d < 3; d++) v[d] = P.vbc_values[ib] * n[d];
                break;
            case 11:
                fac = 1 / std::sqrt(1 - n[2] * n[2]);
                if (flag == (1u << ib)) {
                    double vn = 0;
                    for (int d = 0; d < 2; d++) vn += v[d] * n[d];
                    for (int d = 0; d < 2; d++) v[d] += (P.vbc_values[ib] * fac - vn) * n[d];
                } else {
                    for (int ic = 0; ic < ib; ic++) {
                        if (!(flag & (1u << ic))) continue;
                        if (P.vbc_types[ic] == 0) {
                            double vn = 0;
                            for (int d = 0; d < 2; d++) vn += v[d] * n[d];
                            for (int d = 0; d < 2; d++) v[d] += (P.vbc_values[ib] * fac - vn) * n[d];
                        } else if (P.vbc_types[ic] == 1) {
                            const double *edge = P.edge_vectors[ic][ib];
                            double ve = 0;
                            for (int d = 0; d < 3; d++) ve += v[d] * edge[d];
                            for (int d = 0; d < 3; d++) v[d] = ve * edge[d];
                        }
                    }
                }
                break;
            case 13:
                fac = 1 / std::sqrt(1 - n[2] * n[2]);
                for (int d = 0; d < 2; d++) v[d] = P.vbc_values[ib] * fac * n[d];
                v[2] = 0;
                break;
            }
        }
        if (vz0 == 0 && vz1 == 0) continue;
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
    return DES_OK;
}

// fields.cxx:396-412
int dso_update_coordinate(dso *o, des_state_view *st)
{
    const double dt = st->dt;
    const int n3 = o->nnode * 3;
    #pragma omp parallel for
    for (int i = 0; i < n3; ++i) st->coord[i] += st->vel[i] * dt;
    return DES_OK;
}

// geometry.cxx:86-114
int dso_compute_volume(dso *o, des_state_view *st)
{
    #pragma omp parallel for
    for (int e = 0; e < o->nelem; ++e) {
        const int *c = &o->conn[4 * (size_t)e];
        st->volume[e] = tet_volume(st->coord + 3 * (size_t)c[0], st->coord + 3 * (size_t)c[1],
                                   st->coord + 3 * (size_t)c[2], st->coord + 3 * (size_t)c[3]);
    }
    return DES_OK;
}

namespace {
// geometry.cxx:333-385 with an explicit temperature array
void compute_mass_T(dso *o, des_state_view *st, const double *T)
{
    const des_params &P = o->P;
    double pseudo_speed = P.max_vbc_val * P.inertial_scaling;
    const bool qs = P.is_quasi_static, thermal = P.has_thermal_diffusion;
    #pragma omp parallel for
    for (int e = 0; e < o->nelem; e++) {
        double *tr = st->tmp_result + 12 * (size_t)e;
        double rho = qs ? o->bulkm(e) / (pseudo_speed * pseudo_speed) : o->rho(e, T);
        double m = rho * st->volume[e] / 4;
        double tm = o->rho(e, T) * o->cp(e) * st->volume[e] / 4;
        tr[0] = st->volume[e];
        tr[1] = m;
        if (thermal) tr[2] = tm;
    }
    #pragma omp parallel for
    for (int n = 0; n < o->nnode; n++) {
        st->volume_n[n] = 0;
        st->mass[n] = 0;
        st->tmass[n] = 0;
        for (int q = o->sup_off[n]; q < o->sup_off[n + 1]; ++q) {
            const double *tr = st->tmp_result + 12 * (size_t)o->sup_el[q];
            st->volume_n[n] += tr[0];
            st->mass[n] += tr[1];
            if (thermal) st->tmass[n] += tr[2];
        }
    }
}
}  // namespace

int dso_compute_mass(dso *o, des_state_view *st)
{
    compute_mass_T(o, st, st->temperature);
    return DES_OK;
}

// geometry.cxx:388-470 (3D)
int dso_compute_shape_fn(dso *o, des_state_view *st)
{
    #pragma omp parallel for
    for (int e = 0; e < o->nelem; e++) {
        const int *c = &o->conn[4 * (size_t)e];
        const double *d0 = st->coord + 3 * (size_t)c[0];
        const double *d1 = st->coord + 3 * (size_t)c[1];
        const double *d2 = st->coord + 3 * (size_t)c[2];
        const double *d3 = st->coord + 3 * (size_t)c[3];
        double iv = 1 / (6 * st->volume[e]);
        double x01 = d0[0] - d1[0], x02 = d0[0] - d2[0], x03 = d0[0] - d3[0];
        double x12 = d1[0] - d2[0], x13 = d1[0] - d3[0], x23 = d2[0] - d3[0];
        double y01 = d0[1] - d1[1], y02 = d0[1] - d2[1], y03 = d0[1] - d3[1];
        double y12 = d1[1] - d2[1], y13 = d1[1] - d3[1], y23 = d2[1] - d3[1];
        double z01 = d0[2] - d1[2], z02 = d0[2] - d2[2], z03 = d0[2] - d3[2];
        double z12 = d1[2] - d2[2], z13 = d1[2] - d3[2], z23 = d2[2] - d3[2];
        double *px = st->shpdx + 4 * (size_t)e, *py = st->shpdy + 4 * (size_t)e,
               *pz = st->shpdz + 4 * (size_t)e;
        px[0] = iv * (y13 * z12 - y12 * z13);
        px[1] = iv * (y02 * z23 - y23 * z02);
        px[2] = iv * (y13 * z03 - y03 * z13);
        px[3] = iv * (y01 * z02 - y02 * z01);
        py[0] = iv * (z13 * x12 - z12 * x13);
        py[1] = iv * (z02 * x23 - z23 * x02);
        py[2] = iv * (z13 * x03 - z03 * x13);
        py[3] = iv * (z01 * x02 - z02 * x01);
        pz[0] = iv * (x13 * y12 - x12 * y13);
        pz[1] = iv * (x02 * y23 - x23 * y02);
        pz[2] = iv * (x13 * y03 - x03 * y13);
        pz[3] = iv * (x01 * y02 - x02 * y01);
    }
    return DES_OK;
}

namespace {
// bc.cxx:598-730 (simple_diffusion, 3D): the heights of the top surface
// diffuse; every top facet adds its horizontal projected area to its nodes'
// total_dx and its FEM slope term to their total_slope, in bfacets order
void surface_diffusion(dso *o, des_state_view *st)
{
    double *x = st->coord;
    std::vector<double> total_dx(o->nnode, 0.0), total_slope(o->nnode, 0.0);
    for (const auto &fc : o->bfacets[5]) {
        const int *c = &o->conn[4 * (size_t)fc.first];
        const int n[3] = {c[kFacet[fc.second][0]], c[kFacet[fc.second][1]], c[kFacet[fc.second][2]]};
        auto X = [&](int i, int d) { return x[3 * (size_t)n[i] + d]; };
        const double x01 = X(1, 0) - X(0, 0), y01 = X(1, 1) - X(0, 1);
        const double x02 = X(2, 0) - X(0, 0), y02 = X(2, 1) - X(0, 1);
        const double projected_area = 0.5 * (x01 * y02 - y01 * x02);
        for (int i = 0; i < 3; ++i) total_dx[n[i]] += projected_area;
        const double iv = 1 / (2 * projected_area);
        const double sx[3] = {iv * (X(1, 1) - X(2, 1)), iv * (X(2, 1) - X(0, 1)), iv * (X(0, 1) - X(1, 1))};
        const double sy[3] = {iv * (X(2, 0) - X(1, 0)), iv * (X(0, 0) - X(2, 0)), iv * (X(1, 0) - X(0, 0))};
        for (int j = 0; j < 3; ++j) {
            double slope = 0;
            for (int k = 0; k < 3; ++k) {
                const double D = sx[j] * sx[k] + sy[j] * sy[k];
                slope += D * X(k, 2);
            }
            total_slope[n[j]] += slope * projected_area;
        }
    }
    for (int nd : o->bnodes[5]) {
        const double dh = o->P.surface_diffusivity * st->dt * total_slope[nd] / total_dx[nd];
        x[3 * (size_t)nd + 2] -= dh;
    }
}

// bc.cxx:760-782: option 1 diffuses the surface; option 101 is the
// reference's template for a custom rule, which adds dh = 0 to each top node
int surface_processes(dso *o, des_state_view *st)
{
    switch (o->P.surface_process_option) {
    case 0: return DES_OK;
    case 1: surface_diffusion(o, st); return DES_OK;
    case 101:
        for (int nd : o->bnodes[5]) st->coord[3 * (size_t)nd + 2] += 0.0;
        return DES_OK;
    default: return DES_ERR_OPTION;
    }
}
}  // namespace

// dynearthsol.cxx:237-261
int dso_update_mesh(dso *o, des_state_view *st)
{
    dso_update_coordinate(o, st);
    if (int rc = surface_processes(o, st)) return rc;
    // the reference swaps the two vectors (dynearthsol.cxx:248); the caller's
    // buffers stay in place here, so copy instead
    std::memcpy(st->volume_old, st->volume, sizeof(double) * o->nelem);
    dso_compute_volume(o, st);
    dso_compute_mass(o, st);
    dso_compute_shape_fn(o, st);
    return DES_OK;
}

// fields.cxx:455-533 (3D)
int dso_rotate_stress(dso *o, des_state_view *st)
{
    const double dt = st->dt;
    #pragma omp parallel for
    for (int e = 0; e < o->nelem; ++e) {
        const int *conn = &o->conn[4 * (size_t)e];
        double w3, w4, w5;
        {
            const double *dx = st->shpdx + 4 * (size_t)e;
            const double *dy = st->shpdy + 4 * (size_t)e;
            const double *dz = st->shpdz + 4 * (size_t)e;
            const double *v[4];
            for (int i = 0; i < 4; ++i) v[i] = st->vel + 3 * (size_t)conn[i];
            w3 = 0;
            for (int i = 0; i < 4; ++i) w3 += 0.5 * (v[i][0] * dy[i] - v[i][1] * dx[i]);
            w4 = 0;
            for (int i = 0; i < 4; ++i) w4 += 0.5 * (v[i][0] * dz[i] - v[i][2] * dx[i]);
            w5 = 0;
            for (int i = 0; i < 4; ++i) w5 += 0.5 * (v[i][1] * dz[i] - v[i][2] * dy[i]);
        }
        jaumann(st->stress + 6 * (size_t)e, dt, w3, w4, w5);
        jaumann(st->strain + 6 * (size_t)e, dt, w3, w4, w5);
    }
    return DES_OK;
}

// geometry.cxx:257-330 (3D)
int dso_compute_dt(dso *o, des_state_view *st, double *dt_out)
{
    const des_params &P = o->P;
    if (P.fixed_dt != 0) {
        *dt_out = P.fixed_dt;
        return DES_OK;
    }
    double dt_maxwell = std::numeric_limits<double>::max();
    double dt_diffusion = std::numeric_limits<double>::max();
    double minl = std::numeric_limits<double>::max();
    for (int e = 0; e < o->nelem; ++e) {
        const int *c = &o->conn[4 * (size_t)e];
        const double *a = st->coord + 3 * (size_t)c[0];
        const double *b = st->coord + 3 * (size_t)c[1];
        const double *cc = st->coord + 3 * (size_t)c[2];
        const double *d = st->coord + 3 * (size_t)c[3];
        double maxa = smax(smax(tri_area(a, b, cc), tri_area(a, b, d)),
                           smax(tri_area(cc, d, a), tri_area(cc, d, b)));
        double minh = 3 * st->volume[e] / maxa;
        dt_maxwell = smin(dt_maxwell, 0.5 * P.visc_min / (1e-40 + o->shearm(e)));
        if (P.has_thermal_diffusion) dt_diffusion = smin(dt_diffusion, 0.5 * minh * minh / P.therm_diff_max);
        minl = smin(minl, minh);
    }
    double dt_advection = 0.5 * minl / P.max_vbc_val;
    double dt_elastic = P.is_quasi_static ? 0.5 * minl / (P.max_vbc_val * P.inertial_scaling)
                                          : 0.5 * minl / std::sqrt(o->bulkm(0) / o->rho(0, st->temperature));
    double dt = smin(smin(dt_elastic, dt_maxwell), smin(dt_advection, dt_diffusion)) * P.dt_fraction;
    *dt_out = dt;
    if (dt <= 0) return DES_ERR_DT;
    return DES_OK;
}

// dynearthsol.cxx:86-105 after the mesh: coord0, volume, mass (T = 0), shape
// functions, vbcs, lithostatic stress (ic.cxx:96-132); T and plstrain come in s
int dso_init_fields(dso *o, des_state_view *st)
{
    const des_params &P = o->P;
    if (st->coord0) std::memcpy(st->coord0, st->coord, sizeof(double) * 3 * o->nnode);
    dso_compute_volume(o, st);
    std::memcpy(st->volume_old, st->volume, sizeof(double) * o->nelem);
    compute_mass_T(o, st, o->zeros_n.data());
    dso_compute_shape_fn(o, st);
    dso_apply_vbcs(o, st);
    if (P.gravity == 0) {
        o->P.compensation_pressure = 0;
    } else {
        if (P.ref_pressure_option < 0 || P.ref_pressure_option > 2) return DES_ERR_OPTION;
        double ks = o->bulkm(0);
        for (int e = 0; e < o->nelem; ++e) {
            const int *c = &o->conn[4 * (size_t)e];
            double zcenter = 0;
            for (int i = 0; i < 4; ++i) zcenter += st->coord[3 * (size_t)c[i] + 2];
            zcenter /= 4;
            double p = ref_pressure(P, zcenter);
            if (P.ref_pressure_option == 1 || P.ref_pressure_option == 2) ks = o->bulkm(e);
            for (int i = 0; i < 3; ++i) {
                st->stress[6 * (size_t)e + i] = -p;
                st->strain[6 * (size_t)e + i] = -p / ks / 3;
            }
        }
        o->P.compensation_pressure = ref_pressure(P, -P.zlength);
    }
    st->time = 0;
    st->steps = 0;
    double dt;
    int rc = dso_compute_dt(o, st, &dt);
    st->dt = dt;
    return rc;
}

// dynearthsol.cxx:358-394
int dso_step(dso *o, des_state_view *st, int nsteps)
{
    const des_params &P = o->P;
    for (int it = 0; it < nsteps; ++it) {
        st->steps++;
        st->time += st->dt;
        if (P.has_thermal_diffusion) dso_update_temperature(o, st);
        dso_update_strain_rate(o, st);
        dso_compute_dvoldt(o, st);
        dso_compute_edvoldt(o, st);
        int rc = dso_update_stress(o, st);
        if (rc) return rc;
        dso_NMD_stress(o, st);
        rc = dso_update_force(o, st);
        if (rc) return rc;
        dso_update_velocity(o, st);
        dso_apply_vbcs(o, st);
        if (int rc = dso_update_mesh(o, st)) return rc;
        if (P.rheol_type & DES_RH_ELASTIC) dso_rotate_stress(o, st);
        if (st->steps % 10 == 0) {
            double dt;
            rc = dso_compute_dt(o, st, &dt);
            st->dt = dt;
            if (rc) return rc;
        }
    }
    return DES_OK;
}

int dso_dsyevh3(const double a[9], double q[9], double w[3])
{
    double A[3][3], Q[3][3];
    for (int i = 0; i < 9; ++i) A[i / 3][i % 3] = a[i];
    int rc = eig_hybrid(A, Q, w);
    for (int i = 0; i < 9; ++i) q[i] = Q[i / 3][i % 3];
    return rc;
}

void dso_principal_stresses3(const double s[6], double p[3], double v[9])
{
    double V[3][3];
    principal3(s, p, V);
    for (int i = 0; i < 9; ++i) v[i] = V[i / 3][i % 3];
}

void dso_elasto_plastic(double bulkm, double shearm, double amc, double anphi, double anpsi,
                        double hardn, double ten_max, const double de[6], double *depls,
                        double s[6], int *failure_mode)
{
    elasto_plastic(bulkm, shearm, amc, anphi, anpsi, hardn, ten_max, de, *depls, s, *failure_mode);
}

// geometry.cxx:472-509 (3D)
static double elem_quality(const double *coord, const int *conn, const double *volume, int e)
{
    const int *c = conn + 4 * (size_t)e;
    const double *a = coord + 3 * (size_t)c[0], *b = coord + 3 * (size_t)c[1];
    const double *cc = coord + 3 * (size_t)c[2], *d = coord + 3 * (size_t)c[3];
    const double vol = volume[e];
    const double nf = 216 * std::sqrt(3.0);
    double area_sum = (tri_area(a, b, cc) + tri_area(a, b, d) + tri_area(cc, d, a) + tri_area(cc, d, b));
    return nf * vol * vol / (area_sum * area_sum * area_sum);
}

void dso_elem_quality(const dso *o, const des_state_view *s, double *quality)
{
    for (int e = 0; e < o->nelem; ++e) quality[e] = elem_quality(s->coord, o->conn.data(), s->volume, e);
}

// remeshing.cxx:1893-1960 (3D: sizefactor 0.118, remeshing.cxx:83)
void dso_bad_mesh_quality(const dso *o, const des_state_view *s, const des_remesh_check *c, int *code,
                          int *index, double *worst_quality)
{
    const double smallest_vol = c->smallest_size * 0.118 * std::pow(c->resolution, 3);
    // worst_elem_quality (geometry.cxx:512-526)
    double q = 1;
    int worst = 0;
    for (int e = 0; e < o->nelem; ++e) {
        double qe = elem_quality(s->coord, o->conn.data(), s->volume, e);
        if (qe < q) {
            q = qe;
            worst = e;
        }
    }
    q = std::pow(q, 1.0 / 3);
    if (worst_quality) *worst_quality = q;
    *code = 0;
    for (int e = 0; e < o->nelem; ++e)
        if (s->volume[e] < smallest_vol) {
            *code = 3;
            *index = e;
            return;
        }
    if (c->remeshing_option == 1 || c->remeshing_option == 2 || c->remeshing_option == 11) {
        const double bottom = -c->zlength, dist = c->max_boundary_distortion * c->resolution;
        for (int i = 0; i < o->nnode; ++i)
            if ((o->bcflag[i] & 16u) && std::fabs(s->coord[3 * (size_t)i + 2] - bottom) > dist) {
                *code = 2;
                *index = i;
                return;
            }
    }
    if (q < c->min_quality) {
        *code = 1;
        *index = worst;
    }
}

void dso_plastic_props(const dso *o, int e, double pls, double out[7])
{
    out[0] = o->bulkm(e);
    out[1] = o->shearm(e);
    o->plastic_props(e, pls, out[2], out[3], out[4], out[5], out[6]);
}

}  // extern "C"
