// Boundary topology and node->element support lists, built on the host once
// per mesh.  Orderings follow the reference exactly so that every list is
// bit-identical to what mesh.cxx produces:
//   bcflag          mesh.cxx:1529-1550  OR of segment flags per node
//   bnodes[i]       mesh.cxx:1553-1573  ascending node id
//   bfacets[i]      mesh.cxx:1633-1700  segment order; (e,f) is the first
//                                       facet in ascending (e,f) order whose
//                                       node set equals the segment's
//   support         mesh.cxx:1703-1717  ascending element id per node
// The facet search uses a sorted key table instead of the O(nseg*nelem) scan.
#include "des_gpu.h"
#include "des_topology.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

namespace {

const int kFacet[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};   // constants.hpp:61-67
const unsigned kBoundAny = 0x3ffu;                                       // constants.hpp:50-51

struct FacetKey {
    int a, b, c;     // sorted node ids
    int ef;          // 4 * element + facet
    bool operator<(const FacetKey &o) const
    {
        if (a != o.a) return a < o.a;
        if (b != o.b) return b < o.b;
        if (c != o.c) return c < o.c;
        return ef < o.ef;
    }
};

inline void sort3(int &x, int &y, int &z)
{
    if (x > y) std::swap(x, y);
    if (y > z) std::swap(y, z);
    if (x > y) std::swap(x, y);
}

template <class T>
T *alloc_array(size_t n)
{
    return static_cast<T *>(std::malloc(sizeof(T) * (n ? n : 1)));
}

}  // namespace

extern "C" void des_topology_free(des_topology *t)
{
    if (!t) return;
    std::free(t->bcflag);
    std::free(t->support_offsets);
    std::free(t->support_elems);
    std::free(t->support_slots);
    for (int i = 0; i < DES_NBDRY; ++i) {
        std::free(t->bnodes[i]);
        std::free(t->bfacets[i]);
    }
    std::free(t);
}

extern "C" int des_topology_build(const des_mesh_view *m, des_topology **out)
{
    return des::topology_build(m, out, true);
}

int des::topology_build(const des_mesh_view *m, des_topology **out, bool support)
{
    if (!m || !out || m->nnode < 1 || m->nelem < 1 || !m->connectivity) return DES_ERR_ARG;
    if (m->nseg > 0 && (!m->segment || !m->segflag)) return DES_ERR_ARG;
    const int nn = m->nnode, ne = m->nelem;
    for (long long q = 0; q < 4LL * ne; ++q)
        if (m->connectivity[q] < 0 || m->connectivity[q] >= nn) return DES_ERR_ARG;
    for (long long q = 0; q < 3LL * m->nseg; ++q)
        if (m->segment[q] < 0 || m->segment[q] >= nn) return DES_ERR_ARG;

    des_topology *t = static_cast<des_topology *>(std::calloc(1, sizeof(des_topology)));
    if (!t) return DES_ERR_NOMEM;
    t->nnode = nn;
    t->nelem = ne;
    t->bcflag = alloc_array<unsigned>(nn);
    if (support) {
        t->support_offsets = alloc_array<int>((size_t)nn + 1);
        t->support_elems = alloc_array<int>(4 * (size_t)ne);
        t->support_slots = alloc_array<int>(4 * (size_t)ne);
    }
    if (!t->bcflag || (support && (!t->support_offsets || !t->support_elems || !t->support_slots))) {
        des_topology_free(t);
        return DES_ERR_NOMEM;
    }

    // boundary flags
    std::memset(t->bcflag, 0, sizeof(unsigned) * nn);
    for (int s = 0; s < m->nseg; ++s) {
        unsigned flag = static_cast<unsigned>(m->segflag[s]);
        for (int j = 0; j < 3; ++j) t->bcflag[m->segment[3 * s + j]] |= flag;
    }

    // boundary nodes
    for (int b = 0; b < DES_NBDRY; ++b) {
        int count = 0;
        for (int n = 0; n < nn; ++n) count += (t->bcflag[n] >> b) & 1u;
        t->bnodes_count[b] = count;
        t->bnodes[b] = alloc_array<int>(count);
        if (!t->bnodes[b]) { des_topology_free(t); return DES_ERR_NOMEM; }
        int q = 0;
        for (int n = 0; n < nn; ++n)
            if ((t->bcflag[n] >> b) & 1u) t->bnodes[b][q++] = n;
    }

    // boundary facets: table of every element facet whose three nodes are all
    // on some boundary, sorted by node set then by (e,f)
    std::vector<FacetKey> keys;
    for (int e = 0; e < ne; ++e) {
        const int *c = m->connectivity + 4LL * e;
        for (int f = 0; f < 4; ++f) {
            int a = c[kFacet[f][0]], b = c[kFacet[f][1]], d = c[kFacet[f][2]];
            if ((t->bcflag[a] & t->bcflag[b] & t->bcflag[d]) == 0u) continue;
            sort3(a, b, d);
            keys.push_back(FacetKey{a, b, d, 4 * e + f});
        }
    }
    std::sort(keys.begin(), keys.end());
    std::vector<int> facet_of_seg(m->nseg > 0 ? m->nseg : 1, -1);
    std::vector<int> kind_of_seg(m->nseg > 0 ? m->nseg : 1, -1);
    for (int s = 0; s < m->nseg; ++s) {
        unsigned flag = static_cast<unsigned>(m->segflag[s]);
        if ((flag & kBoundAny) == 0u) continue;
        int kind = -1;
        for (int k = 0; k < DES_NBDRY; ++k)
            if (flag == (1u << k)) kind = k;
        int a = m->segment[3 * s], b = m->segment[3 * s + 1], d = m->segment[3 * s + 2];
        sort3(a, b, d);
        FacetKey probe{a, b, d, -1};
        auto it = std::lower_bound(keys.begin(), keys.end(), probe);
        bool found = false;
        for (; it != keys.end() && it->a == a && it->b == b && it->c == d; ++it) {
            int e = it->ef >> 2, f = it->ef & 3;
            const int *c = m->connectivity + 4LL * e;
            unsigned shared = flag & t->bcflag[c[kFacet[f][0]]] & t->bcflag[c[kFacet[f][1]]] &
                              t->bcflag[c[kFacet[f][2]]];
            if (shared == 0u) continue;
            if (kind >= 0) {       // a single-flag segment is taken by its first facet
                facet_of_seg[s] = it->ef;
                kind_of_seg[s] = kind;
                found = true;
                break;
            }
        }
        if (!found) { des_topology_free(t); return DES_ERR_TOPOLOGY; }
    }
    for (int b = 0; b < DES_NBDRY; ++b) {
        int count = 0;
        for (int s = 0; s < m->nseg; ++s) count += (kind_of_seg[s] == b);
        t->bfacets_count[b] = count;
        t->bfacets[b] = alloc_array<int>(2 * (size_t)count);
        if (!t->bfacets[b]) { des_topology_free(t); return DES_ERR_NOMEM; }
        int q = 0;
        for (int s = 0; s < m->nseg; ++s) {
            if (kind_of_seg[s] != b) continue;
            t->bfacets[b][2 * q] = facet_of_seg[s] >> 2;
            t->bfacets[b][2 * q + 1] = facet_of_seg[s] & 3;
            ++q;
        }
    }

    if (!support) {
        *out = t;
        return DES_OK;
    }
    // support lists as CSR, elements ascending within each node
    std::vector<int> count(nn, 0);
    for (long long q = 0; q < 4LL * ne; ++q) ++count[m->connectivity[q]];
    t->support_offsets[0] = 0;
    for (int n = 0; n < nn; ++n) t->support_offsets[n + 1] = t->support_offsets[n] + count[n];
    std::vector<int> cursor(t->support_offsets, t->support_offsets + nn);
    for (int e = 0; e < ne; ++e) {
        for (int i = 0; i < 4; ++i) {
            int n = m->connectivity[4LL * e + i];
            int p = cursor[n]++;
            t->support_elems[p] = e;
            t->support_slots[p] = i;
        }
    }
    *out = t;
    return DES_OK;
}

// bc.cxx:90-179, restated.  Normal of a facet as bc.cxx:15-36 computes it.
extern "C" int des_boundary_normals(const des_topology *t, const int *conn, const double *coord,
                                    des_params *p)
{
    if (!t || !conn || !coord || !p) return DES_ERR_ARG;
    for (int i = 0; i < DES_NBDRY; ++i) {
        if (t->bfacets_count[i] == 0) continue;
        for (int q = 0; q < t->bfacets_count[i]; ++q) {
            int e = t->bfacets[i][2 * q], f = t->bfacets[i][2 * q + 1];
            const int *c = conn + 4LL * e;
            const double *x0 = coord + 3LL * c[kFacet[f][0]];
            const double *x1 = coord + 3LL * c[kFacet[f][1]];
            const double *x2 = coord + 3LL * c[kFacet[f][2]];
            double v01[3], v02[3], nrm[3];
            for (int d = 0; d < 3; ++d) {
                v01[d] = x1[d] - x0[d];
                v02[d] = x2[d] - x0[d];
            }
            nrm[0] = (v01[1] * v02[2] - v01[2] * v02[1]) / 2;
            nrm[1] = (v01[2] * v02[0] - v01[0] * v02[2]) / 2;
            nrm[2] = (v01[0] * v02[1] - v01[1] * v02[0]) / 2;
            double len = 0;
            for (int d = 0; d < 3; ++d) len += nrm[d] * nrm[d];
            len = std::sqrt(len);
            for (int d = 0; d < 3; ++d) nrm[d] = nrm[d] / len;
            if (q == 0) {
                for (int d = 0; d < 3; ++d) p->bnormals[i][d] = nrm[d];
                if (i < 6) break;    // only the slanted boundaries must be planar
            } else {
                double diff2 = 0;
                for (int d = 0; d < 3; ++d)
                    diff2 += (p->bnormals[i][d] - nrm[d]) * (p->bnormals[i][d] - nrm[d]);
                if (diff2 > 1e-12) return DES_ERR_OPTION;
            }
        }
    }
    for (int i = 0; i < DES_NBDRY; ++i) {
        if (t->bfacets_count[i] == 0) continue;
        for (int j = i + 1; j < DES_NBDRY; ++j) {
            if (t->bfacets_count[j] == 0) continue;
            double *s = p->edge_vectors[i][j];
            const double *a = p->bnormals[i], *b = p->bnormals[j];
            if (std::fabs(a[2]) < 1e-15 && std::fabs(b[2]) < 1e-15) {
                s[0] = s[1] = 0;
                s[2] = 1;
            } else {
                s[0] = a[1] * b[2] - a[2] * b[1];
                s[1] = a[2] * b[0] - a[0] * b[2];
                s[2] = a[0] * b[1] - a[1] * b[0];
            }
        }
    }
    return DES_OK;
}
