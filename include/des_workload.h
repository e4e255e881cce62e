/*
 * des_workload.h -- seeded synthetic inputs for the time-step library.
 *
 * The reference meshes with TetGen (mesh.cxx:334-512); the benchmark boxes are
 * instead structured: nx*ny*nz hexahedra, each cut into 6 tetrahedra that share
 * the hex's main diagonal (Kuhn split, conforming when every hex uses the same
 * orientation).  Node positions are jittered by a counter-based PRNG
 * (splitmix64 of seed and node id): interior nodes in 3D, face nodes in their
 * plane, edge nodes along their edge, corners fixed, so the six walls stay
 * planar.  Every tetrahedron is oriented so that the reference's signed volume
 * (geometry.cxx:29-49) is positive.  The boundary triangles become segments
 * with the reference's flags (constants.hpp:39-44), as create_new_mesh leaves
 * them after discarding internal segments.
 *
 * Host-only; no GPU is needed.
 */
#ifndef DES_WORKLOAD_H
#define DES_WORKLOAD_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct des_box_spec {
    int    nx, ny, nz;               /* hexahedra along x, y, z */
    double xlength, ylength, zlength;/* box [0,xl] x [0,yl] x [-zl,0] in metres */
    double jitter;                   /* fraction of the spacing, e.g. 0.05 */
    unsigned long long seed;
} des_box_spec;

/* Sizes of the box mesh: nnode = (nx+1)(ny+1)(nz+1), nelem = 6 nx ny nz,
 * nseg = 4 (ny nz + nx nz + nx ny). */
int des_box_sizes(const des_box_spec *spec, int *nnode, int *nelem, int *nseg);

/* Fills coord[nnode][3], connectivity[nelem][4], segment[nseg][3], segflag[nseg]. */
int des_box_fill(const des_box_spec *spec, double *coord, int *connectivity,
                 int *segment, int *segflag);

/* Marker counts per element (the int_vec2D elemmarkers).  Each element gets
 * markers_per_elem markers at seeded random barycentric positions; a marker
 * takes material layer_mattypes[i] of the first layer i with
 * z >= -zlength * layer_depths[i], else the last entry, as
 * MarkerSet::layered_initial_mattype does (markerset.cxx:328-341).  With
 * nlayers == 1 every marker is material layer_mattypes[0]. */
int des_markers_layered(int nelem, int nmat, const double *coord, const int *connectivity,
                        int markers_per_elem, double zlength, int nlayers,
                        const int *layer_mattypes, const double *layer_depths,
                        unsigned long long seed, int *elemmarkers);

/* Temperature in Kelvin: T = t_top + (t_bottom - t_top) * (-z / zlength), plus
 * a seeded N(0, sigma) perturbation per node when sigma > 0 (Box-Muller on the
 * same counter PRNG).  Nodes with z >= 0 keep t_top exactly. */
int des_temperature_linear(int nnode, const double *coord, double zlength, double t_top,
                           double t_bottom, double sigma, unsigned long long seed,
                           double *temperature);

#ifdef __cplusplus
}
#endif
#endif /* DES_WORKLOAD_H */
