// Seeded synthetic inputs: structured box of Kuhn-split hexahedra, marker
// counts, temperature profile.  See include/des_workload.h for the contract.
//
// All arithmetic here is plain IEEE double without libm calls, so the same
// seed gives bit-identical inputs on x86-64 and aarch64 (build with
// -ffp-contract=off).
#include "des_workload.h"

#include <algorithm>
#include <cstdint>
#include <vector>

namespace {

inline uint64_t mix64(uint64_t z)
{
    // splitmix64 finaliser (Steele, Lea & Flood 2014)
    z += 0x9e3779b97f4a7c15ULL;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
    return z ^ (z >> 31);
}

// uniform double in [0,1) from counter (seed, stream, index)
inline double u01(uint64_t seed, uint64_t stream, uint64_t index)
{
    uint64_t r = mix64(mix64(seed ^ (stream * 0xd1b54a32d192ed03ULL)) + index);
    return static_cast<double>(r >> 11) * (1.0 / 9007199254740992.0);
}

// Signed tetrahedron volume with the arithmetic of geometry.cxx:29-49, used
// only to orient the six Kuhn tetrahedra of the unit cube once.
double signed_volume(const double *d0, const double *d1, const double *d2, const double *d3)
{
    double x01 = d0[0] - d1[0], x12 = d1[0] - d2[0], x23 = d2[0] - d3[0];
    double y01 = d0[1] - d1[1], y12 = d1[1] - d2[1], y23 = d2[1] - d3[1];
    double z01 = d0[2] - d1[2], z12 = d1[2] - d2[2], z23 = d2[2] - d3[2];
    return (x01 * (y23 * z12 - y12 * z23) + x12 * (y01 * z23 - y23 * z01) +
            x23 * (y12 * z01 - y01 * z12)) / 6;
}

// local facet numbering of a tetrahedron (constants.hpp:61-67)
const int kFacet[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};

struct KuhnTable {
    int corner[6][4];   // corner index a + 2b + 4c of the unit cube, per tet
    KuhnTable()
    {
        const int perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
        for (int t = 0; t < 6; ++t) {
            int step0 = 1 << perm[t][0];
            int step1 = step0 | (1 << perm[t][1]);
            int c[4] = {0, step0, step1, 7};
            double p[4][3];
            for (int v = 0; v < 4; ++v)
                for (int d = 0; d < 3; ++d) p[v][d] = (c[v] >> d) & 1;
            if (signed_volume(p[0], p[1], p[2], p[3]) < 0) std::swap(c[1], c[2]);
            for (int v = 0; v < 4; ++v) corner[t][v] = c[v];
        }
    }
};

}  // namespace

extern "C" int des_box_sizes(const des_box_spec *s, int *nnode, int *nelem, int *nseg)
{
    if (!s || s->nx < 1 || s->ny < 1 || s->nz < 1) return 2;
    long long nn = (long long)(s->nx + 1) * (s->ny + 1) * (s->nz + 1);
    long long ne = 6LL * s->nx * s->ny * s->nz;
    long long ns = 4LL * ((long long)s->ny * s->nz + (long long)s->nx * s->nz + (long long)s->nx * s->ny);
    if (ne > (1LL << 30) || nn > (1LL << 30)) return 6;
    if (nnode) *nnode = (int)nn;
    if (nelem) *nelem = (int)ne;
    if (nseg) *nseg = (int)ns;
    return 0;
}

extern "C" int des_box_fill(const des_box_spec *s, double *coord, int *conn, int *segment,
                            int *segflag)
{
    int nnode, nelem, nseg;
    int rc = des_box_sizes(s, &nnode, &nelem, &nseg);
    if (rc) return rc;
    if (!coord || !conn || !segment || !segflag) return 2;
    const int nx = s->nx, ny = s->ny, nz = s->nz;
    auto node_id = [=](int i, int j, int k) { return (i * (ny + 1) + j) * (nz + 1) + k; };

    const double hx = s->xlength / nx, hy = s->ylength / ny, hz = s->zlength / nz;
    #pragma omp parallel for schedule(static)
    for (int i = 0; i <= nx; ++i) {
        for (int j = 0; j <= ny; ++j) {
            for (int k = 0; k <= nz; ++k) {
                int n = node_id(i, j, k);
                double x = (s->xlength * i) / nx;
                double y = (s->ylength * j) / ny;
                double z = (k == nz) ? 0.0 : -((s->zlength * (nz - k)) / nz);
                if (s->jitter != 0) {
                    if (i > 0 && i < nx) x += s->jitter * hx * (2 * u01(s->seed, 1, 3ULL * n + 0) - 1);
                    if (j > 0 && j < ny) y += s->jitter * hy * (2 * u01(s->seed, 1, 3ULL * n + 1) - 1);
                    if (k > 0 && k < nz) z += s->jitter * hz * (2 * u01(s->seed, 1, 3ULL * n + 2) - 1);
                }
                coord[3LL * n + 0] = x;
                coord[3LL * n + 1] = y;
                coord[3LL * n + 2] = z;
            }
        }
    }

    static const KuhnTable kuhn;
    #pragma omp parallel for schedule(static)
    for (int i = 0; i < nx; ++i) {
        for (int j = 0; j < ny; ++j) {
            for (int k = 0; k < nz; ++k) {
                long long hex = ((long long)i * ny + j) * nz + k;
                for (int t = 0; t < 6; ++t) {
                    int *c = conn + 4 * (6 * hex + t);
                    for (int v = 0; v < 4; ++v) {
                        int cc = kuhn.corner[t][v];
                        c[v] = node_id(i + (cc & 1), j + ((cc >> 1) & 1), k + ((cc >> 2) & 1));
                    }
                }
            }
        }
    }

    // Boundary triangles, in ascending (element, facet) order.
    auto face_flag = [=](int n) {
        int k = n % (nz + 1);
        int j = (n / (nz + 1)) % (ny + 1);
        int i = n / ((nz + 1) * (ny + 1));
        unsigned f = 0;
        if (i == 0) f |= 1u;
        if (i == nx) f |= 2u;
        if (j == 0) f |= 4u;
        if (j == ny) f |= 8u;
        if (k == 0) f |= 16u;
        if (k == nz) f |= 32u;
        return f;
    };
    int ns = 0;
    for (int e = 0; e < nelem; ++e) {
        const int *c = conn + 4LL * e;
        for (int f = 0; f < 4; ++f) {
            int a = c[kFacet[f][0]], b = c[kFacet[f][1]], d = c[kFacet[f][2]];
            unsigned common = face_flag(a) & face_flag(b) & face_flag(d);
            if (!common) continue;
            if (ns >= nseg) return 12;
            segment[3 * ns + 0] = a;
            segment[3 * ns + 1] = b;
            segment[3 * ns + 2] = d;
            segflag[ns] = (int)common;   // three non-collinear nodes share one wall
            ++ns;
        }
    }
    return ns == nseg ? 0 : 12;
}

extern "C" int des_markers_layered(int nelem, int nmat, const double *coord, const int *conn,
                                   int mpe, double zlength, int nlayers,
                                   const int *layer_mattypes, const double *layer_depths,
                                   unsigned long long seed, int *elemmarkers)
{
    if (nelem < 0 || nmat < 1 || mpe < 1 || nlayers < 1 || !elemmarkers || !layer_mattypes)
        return 2;
    for (int l = 0; l < nlayers; ++l)
        if (layer_mattypes[l] < 0 || layer_mattypes[l] >= nmat) return 2;
    if (nlayers > 1 && (!coord || !conn || !layer_depths)) return 2;
    #pragma omp parallel for schedule(static)
    for (int e = 0; e < nelem; ++e) {
        int *cnt = elemmarkers + (long long)nmat * e;
        for (int m = 0; m < nmat; ++m) cnt[m] = 0;
        for (int q = 0; q < mpe; ++q) {
            int mt = layer_mattypes[0];
            if (nlayers > 1) {
                // uniform point in the tetrahedron: sorted uniforms -> barycentric weights
                double u[3];
                for (int r = 0; r < 3; ++r) u[r] = u01(seed, 2, (4ULL * mpe) * e + 4ULL * q + r);
                std::sort(u, u + 3);
                double eta[4] = {u[0], u[1] - u[0], u[2] - u[1], 1 - u[2]};
                double z = 0;
                for (int v = 0; v < 4; ++v) z += coord[3LL * conn[4LL * e + v] + 2] * eta[v];
                mt = layer_mattypes[nlayers - 1];
                for (int l = 0; l < nlayers - 1; ++l) {
                    if (z >= -zlength * layer_depths[l]) {
                        mt = layer_mattypes[l];
                        break;
                    }
                }
            }
            ++cnt[mt];
        }
    }
    return 0;
}

extern "C" int des_temperature_linear(int nnode, const double *coord, double zlength,
                                      double t_top, double t_bottom, double sigma,
                                      unsigned long long seed, double *temperature)
{
    if (nnode < 0 || !coord || !temperature || zlength <= 0) return 2;
    #pragma omp parallel for schedule(static)
    for (int n = 0; n < nnode; ++n) {
        double z = coord[3LL * n + 2];
        if (z >= 0) {
            temperature[n] = t_top;
            continue;
        }
        double t = t_top + (t_bottom - t_top) * (-z / zlength);
        if (sigma > 0) {
            // Irwin-Hall: sum of 12 uniforms minus 6 has mean 0 and variance 1
            double g = -6.0;
            for (int r = 0; r < 12; ++r) g += u01(seed, 3, 12ULL * n + r);
            t += sigma * g;
        }
        temperature[n] = t;
    }
    return 0;
}
