// TEST INFRASTRUCTURE -- driver around the reference's own, unmodified
// functions (compiled from the reference tree by oracle/ref.mk into
// oracle/_ref/libdesref.so).  It injects a mesh and state into the reference's
// Variables the way restart() does (dynearthsol.cxx:162-234), replaces
// input.cxx (boost is absent) by filling Param from des_params, and runs the
// loop body of dynearthsol.cxx:358-394 without output and remeshing.
// Used only to pin oracle/des_oracle.cpp and to write the golden fixtures.
#include <cstring>
#include <string>
#include <limits>
#include <new>
#include <utility>
#include <vector>

#include "constants.hpp"
#include "parameters.hpp"
#include "bc.hpp"
#include "fields.hpp"
#include "geometry.hpp"
#include "ic.hpp"
#include "markerset.hpp"
#include "matprops.hpp"
#include "mesh.hpp"
#include "output.hpp"
#include "rheology.hpp"
#include "3x3-C/dsyevh3.h"

#include "../include/des_gpu.h"

struct dsr {
    Param param;
    Variables var;
    Output *out = nullptr;       // the reference's own output writer, when set up
    bool marker_output = false;  // sim.has_marker_output of the next output_begin
};

namespace {

void fill_vec(double_vec &dst, const des_matvec &src)
{
    dst.assign(src.v, src.v + src.len);
}

void fill_param(Param &p, const des_params &q, int nmat)
{
    p.sim.max_steps = std::numeric_limits<int>::max();
    p.sim.max_time_in_yr = std::numeric_limits<double>::max();
    p.sim.is_restarting = false;
    p.mesh.zlength = q.zlength;
    p.mesh.quality_check_step_interval = std::numeric_limits<int>::max();
    p.control.gravity = q.gravity;
    p.control.characteristic_speed = 0;
    p.control.inertial_scaling = q.inertial_scaling;
    p.control.dt_fraction = q.dt_fraction;
    p.control.fixed_dt = q.fixed_dt;
    p.control.damping_factor = q.damping_factor;
    p.control.damping_option = q.damping_option;
    p.control.ref_pressure_option = q.ref_pressure_option;
    p.control.surface_process_option = q.surface_process_option;
    p.control.surface_diffusivity = q.surface_diffusivity;
    p.control.is_quasi_static = q.is_quasi_static != 0;
    p.control.has_thermal_diffusion = q.has_thermal_diffusion != 0;
    p.control.has_hydration_processes = false;
    p.bc.surface_temperature = q.surface_temperature;
    p.bc.mantle_temperature = q.surface_temperature;
    p.bc.winkler_delta_rho = q.winkler_delta_rho;
    p.bc.has_winkler_foundation = q.has_winkler_foundation != 0;
    p.bc.elastic_foundation_constant = q.elastic_foundation_constant;
    p.bc.has_elastic_foundation = q.has_elastic_foundation != 0;
    p.bc.has_water_loading = q.has_water_loading != 0;
    int *types[10] = {&p.bc.vbc_x0, &p.bc.vbc_x1, &p.bc.vbc_y0, &p.bc.vbc_y1, &p.bc.vbc_z0,
                      &p.bc.vbc_z1, &p.bc.vbc_n0, &p.bc.vbc_n1, &p.bc.vbc_n2, &p.bc.vbc_n3};
    double *vals[10] = {&p.bc.vbc_val_x0, &p.bc.vbc_val_x1, &p.bc.vbc_val_y0, &p.bc.vbc_val_y1,
                        &p.bc.vbc_val_z0, &p.bc.vbc_val_z1, &p.bc.vbc_val_n0, &p.bc.vbc_val_n1,
                        &p.bc.vbc_val_n2, &p.bc.vbc_val_n3};
    for (int i = 0; i < 10; ++i) {
        *types[i] = q.vbc_types[i];
        *vals[i] = q.vbc_values[i];
    }
    p.ic.weakzone_option = 0;
    p.mat.rheol_type = q.rheol_type;
    p.mat.phase_change_option = 0;
    p.mat.nmat = nmat;
    p.mat.is_plane_strain = false;
    p.mat.visc_min = q.visc_min;
    p.mat.visc_max = q.visc_max;
    p.mat.tension_max = q.tension_max;
    p.mat.therm_diff_max = q.therm_diff_max;
    fill_vec(p.mat.rho0, q.rho0);
    fill_vec(p.mat.alpha, q.alpha);
    fill_vec(p.mat.bulk_modulus, q.bulk_modulus);
    fill_vec(p.mat.shear_modulus, q.shear_modulus);
    fill_vec(p.mat.visc_exponent, q.visc_exponent);
    fill_vec(p.mat.visc_coefficient, q.visc_coefficient);
    fill_vec(p.mat.visc_activation_energy, q.visc_activation_energy);
    fill_vec(p.mat.heat_capacity, q.heat_capacity);
    fill_vec(p.mat.therm_cond, q.therm_cond);
    fill_vec(p.mat.pls0, q.pls0);
    fill_vec(p.mat.pls1, q.pls1);
    fill_vec(p.mat.cohesion0, q.cohesion0);
    fill_vec(p.mat.cohesion1, q.cohesion1);
    fill_vec(p.mat.friction_angle0, q.friction_angle0);
    fill_vec(p.mat.friction_angle1, q.friction_angle1);
    fill_vec(p.mat.dilation_angle0, q.dilation_angle0);
    fill_vec(p.mat.dilation_angle1, q.dilation_angle1);
    p.debug.dt = false;
}

template <class A>
void copy_in(A &dst, const double *src, size_t n)
{
    if (src) std::memcpy(dst.data(), src, sizeof(double) * n);
}
template <class A>
void copy_out(const A &src, double *dst, size_t n)
{
    if (dst) std::memcpy(dst, src.data(), sizeof(double) * n);
}

}  // namespace

extern "C" {

int dsr_create(const des_mesh_view *m, const des_params *q, dsr **out)
{
    dsr *h = new (std::nothrow) dsr();
    if (!h) return DES_ERR_NOMEM;
    Param &p = h->param;
    Variables &var = h->var;
    fill_param(p, *q, m->nmat);
    // init_var (dynearthsol.cxx:32-68)
    var.time = 0;
    var.steps = 0;
    var.max_vbc_val = find_max_vbc(p.bc);
    for (int i = 0; i < 10; ++i) {
        var.vbc_types[i] = q->vbc_types[i];
        var.vbc_values[i] = q->vbc_values[i];
    }
    var.nnode = m->nnode;
    var.nelem = m->nelem;
    var.nseg = m->nseg;
    var.coord = new array_t(m->nnode, 0.0);
    var.connectivity = new conn_t(m->nelem);
    std::memcpy(var.connectivity->data(), m->connectivity, sizeof(int) * 4 * (size_t)m->nelem);
    var.segment = new segment_t(m->nseg);
    std::memcpy(var.segment->data(), m->segment, sizeof(int) * 3 * (size_t)m->nseg);
    var.segflag = new segflag_t(m->nseg);
    std::memcpy(var.segflag->data(), m->segflag, sizeof(int) * (size_t)m->nseg);
    var.regattr = nullptr;
    var.bcflag = nullptr;
    var.phch = nullptr;
    create_boundary_flags(var);
    create_boundary_nodes(var);
    create_boundary_facets(var);
    create_support(var);
    var.elemmarkers = new int_vec2D(var.nelem, std::vector<int>(m->nmat, 0));
    for (int e = 0; e < var.nelem; ++e)
        for (int k = 0; k < m->nmat; ++k) (*var.elemmarkers)[e][k] = m->elemmarkers[(size_t)m->nmat * e + k];
    allocate_variables(p, var);
    *out = h;
    return DES_OK;
}

double dsr_max_vbc_val(const dsr *h) { return h->var.max_vbc_val; }

// writes the counts in place, as phase_changes does (phasechanges.cxx:248-254):
// MatProps holds a reference to var.elemmarkers
int dsr_set_elemmarkers(dsr *h, const int *em)
{
    int_vec2D &k = *h->var.elemmarkers;
    const int nmat = (int)k[0].size();
    for (int e = 0; e < h->var.nelem; ++e)
        for (int m = 0; m < nmat; ++m) k[e][m] = em[(size_t)nmat * e + m];
    return 0;
}

int dsr_bcflag(const dsr *h, unsigned *bcflag)
{
    for (int i = 0; i < h->var.nnode; ++i) bcflag[i] = (*h->var.bcflag)[i];
    return DES_OK;
}
int dsr_support(const dsr *h, int *offsets, int *elems)
{
    int q = 0;
    offsets[0] = 0;
    for (int n = 0; n < h->var.nnode; ++n) {
        for (int e : (*h->var.support)[n]) elems[q++] = e;
        offsets[n + 1] = q;
    }
    return DES_OK;
}
int dsr_bnodes(const dsr *h, int b, int *count, int *nodes)
{
    *count = (int)h->var.bnodes[b].size();
    if (nodes)
        for (size_t i = 0; i < h->var.bnodes[b].size(); ++i) nodes[i] = h->var.bnodes[b][i];
    return DES_OK;
}
int dsr_bfacets(const dsr *h, int b, int *count, int *pairs)
{
    *count = (int)h->var.bfacets[b].size();
    if (pairs)
        for (size_t i = 0; i < h->var.bfacets[b].size(); ++i) {
            pairs[2 * i] = h->var.bfacets[b][i].first;
            pairs[2 * i + 1] = h->var.bfacets[b][i].second;
        }
    return DES_OK;
}
int dsr_normals(const dsr *h, double *bnormals30, double *edge300)
{
    for (int i = 0; i < 10; ++i)
        for (int d = 0; d < 3; ++d) bnormals30[3 * i + d] = h->var.bnormals[i][d];
    for (auto &kv : h->var.edge_vectors)
        for (int d = 0; d < 3; ++d) edge300[(kv.first.first * 10 + kv.first.second) * 3 + d] = kv.second[d];
    return DES_OK;
}
double dsr_compensation_pressure(const dsr *h) { return h->var.compensation_pressure; }

// the Variables members remesh leaves as they were (boundary normals and edge
// vectors from init, the compensation pressure), for a harness built on the
// remeshed mesh
int dsr_inherit(dsr *h, const dsr *from)
{
    for (int i = 0; i < nbdrytypes; ++i)
        for (int d = 0; d < NDIMS; ++d) h->var.bnormals[i][d] = from->var.bnormals[i][d];
    h->var.edge_vectors = from->var.edge_vectors;
    h->var.compensation_pressure = from->var.compensation_pressure;
    return 0;
}

int dsr_set_state(dsr *h, const des_state_view *s, unsigned mask)
{
    Variables &v = h->var;
    const size_t n = v.nnode, e = v.nelem;
    if (mask & DES_F_COORD) copy_in(*v.coord, s->coord, 3 * n);
    if (mask & DES_F_COORD0) copy_in(*v.coord0, s->coord0, 3 * n);
    if (mask & DES_F_VEL) copy_in(*v.vel, s->vel, 3 * n);
    if (mask & DES_F_FORCE) copy_in(*v.force, s->force, 3 * n);
    if (mask & DES_F_TEMPERATURE) copy_in(*v.temperature, s->temperature, n);
    if (mask & DES_F_MASS) {
        copy_in(*v.mass, s->mass, n);
        copy_in(*v.tmass, s->tmass, n);
        copy_in(*v.volume_n, s->volume_n, n);
    }
    if (mask & DES_F_NTMP) copy_in(*v.ntmp, s->ntmp, n);
    if (mask & DES_F_VOLUME) {
        copy_in(*v.volume, s->volume, e);
        copy_in(*v.volume_old, s->volume_old, e);
    }
    if (mask & DES_F_STRESS) copy_in(*v.stress, s->stress, 6 * e);
    if (mask & DES_F_STRAIN) copy_in(*v.strain, s->strain, 6 * e);
    if (mask & DES_F_STRAIN_RATE) copy_in(*v.strain_rate, s->strain_rate, 6 * e);
    if (mask & DES_F_PLSTRAIN) {
        copy_in(*v.plstrain, s->plstrain, e);
        copy_in(*v.delta_plstrain, s->delta_plstrain, e);
    }
    if (mask & DES_F_DPRESSURE) copy_in(*v.dpressure, s->dpressure, e);
    if (mask & DES_F_EDVOLDT) copy_in(*v.edvoldt, s->edvoldt, e);
    if (mask & DES_F_SHAPE) {
        copy_in(*v.shpdx, s->shpdx, 4 * e);
        copy_in(*v.shpdy, s->shpdy, 4 * e);
        copy_in(*v.shpdz, s->shpdz, 4 * e);
    }
    if (mask & DES_F_TMP_RESULT) {
        copy_in(*v.tmp_result, s->tmp_result, 12 * e);
        copy_in(*v.tmp_result_sg, s->tmp_result_sg, e);
    }
    if (mask & DES_F_SCALARS) {
        v.time = s->time;
        v.dt = s->dt;
        v.steps = s->steps;
    }
    return DES_OK;
}

int dsr_get_state(const dsr *h, des_state_view *s, unsigned mask)
{
    const Variables &v = h->var;
    const size_t n = v.nnode, e = v.nelem;
    if (mask & DES_F_COORD) copy_out(*v.coord, s->coord, 3 * n);
    if (mask & DES_F_COORD0) copy_out(*v.coord0, s->coord0, 3 * n);
    if (mask & DES_F_VEL) copy_out(*v.vel, s->vel, 3 * n);
    if (mask & DES_F_FORCE) copy_out(*v.force, s->force, 3 * n);
    if (mask & DES_F_TEMPERATURE) copy_out(*v.temperature, s->temperature, n);
    if (mask & DES_F_MASS) {
        copy_out(*v.mass, s->mass, n);
        copy_out(*v.tmass, s->tmass, n);
        copy_out(*v.volume_n, s->volume_n, n);
    }
    if (mask & DES_F_NTMP) copy_out(*v.ntmp, s->ntmp, n);
    if (mask & DES_F_VOLUME) {
        copy_out(*v.volume, s->volume, e);
        copy_out(*v.volume_old, s->volume_old, e);
    }
    if (mask & DES_F_STRESS) copy_out(*v.stress, s->stress, 6 * e);
    if (mask & DES_F_STRAIN) copy_out(*v.strain, s->strain, 6 * e);
    if (mask & DES_F_STRAIN_RATE) copy_out(*v.strain_rate, s->strain_rate, 6 * e);
    if (mask & DES_F_PLSTRAIN) {
        copy_out(*v.plstrain, s->plstrain, e);
        copy_out(*v.delta_plstrain, s->delta_plstrain, e);
    }
    if (mask & DES_F_DPRESSURE) copy_out(*v.dpressure, s->dpressure, e);
    if (mask & DES_F_EDVOLDT) copy_out(*v.edvoldt, s->edvoldt, e);
    if (mask & DES_F_SHAPE) {
        copy_out(*v.shpdx, s->shpdx, 4 * e);
        copy_out(*v.shpdy, s->shpdy, 4 * e);
        copy_out(*v.shpdz, s->shpdz, 4 * e);
    }
    if (mask & DES_F_TMP_RESULT) {
        copy_out(*v.tmp_result, s->tmp_result, 12 * e);
        copy_out(*v.tmp_result_sg, s->tmp_result_sg, e);
    }
    if (mask & DES_F_SCALARS) {
        s->time = v.time;
        s->dt = v.dt;
        s->steps = v.steps;
    }
    return DES_OK;
}

// init() from allocate_variables on (dynearthsol.cxx:88-105); coord, T and
// plstrain are taken from s, the full state is written back to s.
int dsr_init_fields(dsr *h, des_state_view *s)
{
    Param &param = h->param;
    Variables &var = h->var;
    copy_in(*var.coord, s->coord, 3 * (size_t)var.nnode);
    for (int i = 0; i < var.nnode; i++)
        for (int d = 0; d < NDIMS; d++) (*var.coord0)[i][d] = (*var.coord)[i][d];
    compute_volume(*var.coord, *var.connectivity, *var.volume);
    *var.volume_old = *var.volume;
    compute_mass(param, var, *var.connectivity, *var.volume, *var.mat, var.max_vbc_val, *var.volume_n,
                 *var.mass, *var.tmass, *var.tmp_result, *var.support);
    compute_shape_fn(var, *var.coord, *var.connectivity, *var.volume, *var.shpdx, *var.shpdy, *var.shpdz);
    create_boundary_normals(var, var.bnormals, var.edge_vectors);
    apply_vbcs(param, var, *var.vel);
    copy_in(*var.temperature, s->temperature, (size_t)var.nnode);     // in place of initial_temperature
    initial_stress_state(param, var, *var.stress, *var.stressyy, *var.strain, var.compensation_pressure);
    copy_in(*var.plstrain, s->plstrain, (size_t)var.nelem);           // in place of initial_weak_zone
    var.dt = compute_dt(param, var);
    return dsr_get_state(h, s, DES_F_ALL);
}

int dsr_update_temperature(dsr *h)
{
    update_temperature(h->param, h->var, *h->var.temperature, *h->var.ntmp, *h->var.tmp_result);
    return 0;
}
int dsr_update_strain_rate(dsr *h) { update_strain_rate(h->var, *h->var.strain_rate); return 0; }
int dsr_compute_dvoldt(dsr *h) { compute_dvoldt(h->var, *h->var.ntmp, *h->var.tmp_result_sg); return 0; }
int dsr_compute_edvoldt(dsr *h) { compute_edvoldt(h->var, *h->var.ntmp, *h->var.edvoldt); return 0; }
int dsr_update_stress(dsr *h)
{
    Variables &var = h->var;
    update_stress(var, *var.stress, *var.stressyy, *var.dpressure, *var.strain, *var.plstrain,
                  *var.delta_plstrain, *var.strain_rate);
    return 0;
}
int dsr_NMD_stress(dsr *h) { NMD_stress(h->var, *h->var.ntmp, *h->var.stress, *h->var.tmp_result_sg); return 0; }
int dsr_update_force(dsr *h) { update_force(h->param, h->var, *h->var.force, *h->var.tmp_result); return 0; }
int dsr_update_velocity(dsr *h) { update_velocity(h->var, *h->var.vel); return 0; }
int dsr_apply_vbcs(dsr *h) { apply_vbcs(h->param, h->var, *h->var.vel); return 0; }
int dsr_update_coordinate(dsr *h) { update_coordinate(h->var, *h->var.coord); return 0; }
int dsr_compute_volume(dsr *h) { compute_volume(*h->var.coord, *h->var.connectivity, *h->var.volume); return 0; }
int dsr_compute_mass(dsr *h)
{
    Variables &var = h->var;
    compute_mass(h->param, var, *var.connectivity, *var.volume, *var.mat, var.max_vbc_val, *var.volume_n,
                 *var.mass, *var.tmass, *var.tmp_result, *var.support);
    return 0;
}
int dsr_compute_shape_fn(dsr *h)
{
    Variables &var = h->var;
    compute_shape_fn(var, *var.coord, *var.connectivity, *var.volume, *var.shpdx, *var.shpdy, *var.shpdz);
    return 0;
}
int dsr_update_mesh(dsr *h)
{
    Param &param = h->param;
    Variables &var = h->var;
    // dynearthsol.cxx:237-261
    update_coordinate(var, *var.coord);
    surface_processes(param, var, *var.coord);
    var.volume->swap(*var.volume_old);
    compute_volume(*var.coord, *var.connectivity, *var.volume);
    compute_mass(param, var, *var.connectivity, *var.volume, *var.mat, var.max_vbc_val, *var.volume_n,
                 *var.mass, *var.tmass, *var.tmp_result, *var.support);
    compute_shape_fn(var, *var.coord, *var.connectivity, *var.volume, *var.shpdx, *var.shpdy, *var.shpdz);
    return 0;
}
int dsr_rotate_stress(dsr *h) { rotate_stress(h->var, *h->var.stress, *h->var.strain); return 0; }
double dsr_compute_dt(dsr *h) { return compute_dt(h->param, h->var); }

// dynearthsol.cxx:358-394 without output, remeshing and hydration
int dsr_step(dsr *h, int nsteps)
{
    Param &param = h->param;
    Variables &var = h->var;
    for (int it = 0; it < nsteps; ++it) {
        var.steps++;
        var.time += var.dt;
        if (param.control.has_thermal_diffusion)
            update_temperature(param, var, *var.temperature, *var.ntmp, *var.tmp_result);
        update_strain_rate(var, *var.strain_rate);
        compute_dvoldt(var, *var.ntmp, *var.tmp_result_sg);
        compute_edvoldt(var, *var.ntmp, *var.edvoldt);
        update_stress(var, *var.stress, *var.stressyy, *var.dpressure, *var.strain, *var.plstrain,
                      *var.delta_plstrain, *var.strain_rate);
        NMD_stress(var, *var.ntmp, *var.stress, *var.tmp_result_sg);
        update_force(param, var, *var.force, *var.tmp_result);
        update_velocity(var, *var.vel);
        apply_vbcs(param, var, *var.vel);
        dsr_update_mesh(h);
        if (var.mat->rheol_type & MatProps::rh_elastic) rotate_stress(var, *var.stress, *var.strain);
        if (var.steps % 10 == 0) var.dt = compute_dt(param, var);
        if (h->out && param.sim.is_outputting_averaged_fields) h->out->average_fields(var);   // dynearthsol.cxx:395-396
    }
    return 0;
}

int dsr_dsyevh3(const double a[9], double q[9], double w[3])
{
    double A[3][3], Q[3][3];
    for (int i = 0; i < 9; ++i) A[i / 3][i % 3] = a[i];
    int rc = dsyevh3(A, Q, w);
    for (int i = 0; i < 9; ++i) q[i] = Q[i / 3][i % 3];
    return rc;
}

// geometry.cxx:472-526 on the harness's current state
int dsr_elem_quality(const dsr *h, double *quality)
{
    for (int e = 0; e < h->var.nelem; ++e)
        quality[e] = elem_quality(*h->var.coord, *h->var.connectivity, *h->var.volume, e);
    return 0;
}
double dsr_worst_elem_quality(const dsr *h, int *worst)
{
    return worst_elem_quality(*h->var.coord, *h->var.connectivity, *h->var.volume, *worst);
}

// Output (output.cxx) for frame `frame` of model `modelname`, averaging over
// `interval` steps when averaged != 0 (then dsr_step calls average_fields)
int dsr_output_begin(dsr *h, const char *modelname, int frame, int averaged, int interval)
{
    delete h->out;
    h->param.sim.modelname = modelname;
    h->param.sim.is_outputting_averaged_fields = averaged != 0;
    h->param.sim.has_marker_output = h->marker_output;
    h->param.mesh.quality_check_step_interval = interval;
    h->out = new Output(h->param, 0.0, frame);
    return 0;
}
// Output::write_checkpoint of the current state: <modelname>.chkpt.<frame>
int dsr_output_checkpoint(dsr *h)
{
    if (!h->out) return 1;
    h->out->write_checkpoint(h->param, h->var);
    return 0;
}

// Output::write (or write_exact) of the current state: <modelname>.save.<frame>
int dsr_output_write(dsr *h, int exact)
{
    if (!h->out) return 1;
    if (exact)
        h->out->write_exact(h->var);
    else
        h->out->write(h->var);
    return 0;
}

// a marker set named `name` in var.markersets, built by the reference's own
// MarkerSet::append_marker from the given markers (ids 0..n-1, last id n);
// with marker_output the next output_begin turns sim.has_marker_output on
int dsr_add_markers(dsr *h, const char *name, int n, const double *eta, const int *elem,
                    const int *mattype, int marker_output)
{
    MarkerSet *ms = new MarkerSet(std::string(name));
    for (int i = 0; i < n; ++i) ms->append_marker(eta + 4 * (size_t)i, elem[i], mattype[i]);
    h->var.markersets.push_back(ms);
    h->marker_output = marker_output != 0;
    return 0;
}

void dsr_destroy(dsr *h) { (void)h; /* the reference's arrays are never freed by its own code */ }

}  // extern "C"
