/*
 * des_oracle.h -- TEST INFRASTRUCTURE.  CPU restatement of the DynEarthSol3D
 * time-step loop used only as the parity checker (tests/, __graft_entry__.smoke)
 * and as the timed CPU baseline of bench.py.  Nothing in the product links it.
 *
 * Each function operates on host arrays in the reference layout (des_state_view)
 * and follows the reference function cited beside it statement by statement,
 * so that double arithmetic is evaluated in the same order.  Build with
 * -ffp-contract=off so no multiply-add is fused on any host.
 */
#ifndef DES_ORACLE_H
#define DES_ORACLE_H

#include "../include/des_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dso dso;

int  dso_create(const des_mesh_view *mesh, const des_params *params, dso **out);
void dso_destroy(dso *o);
int  dso_set_params(dso *o, const des_params *params);
/* the counts phase_changes leaves in var.elemmarkers (phasechanges.cxx:232-258) */
int  dso_set_elemmarkers(dso *o, const int *elemmarkers);
int  dso_num_threads(void);

/* topology as mesh.cxx builds it (the naive facet scan for small meshes) */
int  dso_bcflag(const dso *o, unsigned *bcflag);
int  dso_support(const dso *o, int *offsets, int *elems);
int  dso_bnodes(const dso *o, int b, int *count, int *nodes);
int  dso_bfacets(const dso *o, int b, int *count, int *pairs);
int  dso_boundary_normals(dso *o, const double *coord, des_params *params);

/* init() order (dynearthsol.cxx:86-105) given coord, T and plstrain in s */
int  dso_init_fields(dso *o, des_state_view *s);

int  dso_update_temperature(dso *o, des_state_view *s);
int  dso_update_strain_rate(dso *o, des_state_view *s);
int  dso_compute_dvoldt(dso *o, des_state_view *s);
int  dso_compute_edvoldt(dso *o, des_state_view *s);
int  dso_update_stress(dso *o, des_state_view *s);
int  dso_NMD_stress(dso *o, des_state_view *s);
int  dso_update_force(dso *o, des_state_view *s);
int  dso_update_velocity(dso *o, des_state_view *s);
int  dso_apply_vbcs(dso *o, des_state_view *s);
int  dso_update_coordinate(dso *o, des_state_view *s);
int  dso_compute_volume(dso *o, des_state_view *s);
int  dso_compute_mass(dso *o, des_state_view *s);
int  dso_compute_shape_fn(dso *o, des_state_view *s);
int  dso_update_mesh(dso *o, des_state_view *s);
int  dso_rotate_stress(dso *o, des_state_view *s);
int  dso_compute_dt(dso *o, des_state_view *s, double *dt);

/* one or more iterations of dynearthsol.cxx:358-394 */
int  dso_step(dso *o, des_state_view *s, int nsteps);

/* dsyevh3 and principal_stresses3 on one symmetric matrix (upper part of a) */
int  dso_dsyevh3(const double a[9], double q[9], double w[3]);
void dso_principal_stresses3(const double s[6], double p[3], double v[9]);
/* elasto_plastic (rheology.cxx:154-302) on one stress */
void dso_elasto_plastic(double bulkm, double shearm, double amc, double anphi, double anpsi,
                        double hardn, double ten_max, const double de[6], double *depls,
                        double s[6], int *failure_mode);
/* elem_quality (geometry.cxx:472-509) of every element of the state */
void dso_elem_quality(const dso *o, const des_state_view *s, double *quality);
/* bad_mesh_quality (remeshing.cxx:1893-1960); see des_gpu_bad_mesh_quality */
void dso_bad_mesh_quality(const dso *o, const des_state_view *s, const des_remesh_check *c, int *code,
                          int *index, double *worst_quality);
/* element e's moduli and plastic properties at plastic strain pls
 * (matprops.cxx:595-604, 687-704): out = bulkm, shearm, amc, anphi, anpsi,
 * hardn, ten_max */
void dso_plastic_props(const dso *o, int e, double pls, double out[7]);

#ifdef __cplusplus
}
#endif
#endif
