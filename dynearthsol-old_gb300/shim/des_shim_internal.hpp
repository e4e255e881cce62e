// Conversions shared by the loop-level shim (des_shim.cpp) and the
// reference-symbol shim (des_shim_functions.cpp): des_params, des_state_view
// and the flat marker counts from the reference's Param / Variables
// (parameters.hpp:36-287).  Every pointer handed to the library points into
// the reference's own Array2D / std::vector storage.  Compiled inside the
// reference's build, against its headers.
#pragma once

#include <vector>

#include "constants.hpp"
#include "parameters.hpp"
#include "matprops.hpp"
#include "des_gpu.h"

namespace des_shim_detail {

inline void put(des_matvec &dst, const double_vec &src)
{
    dst.len = static_cast<int>(src.size());
    for (int i = 0; i < dst.len && i < DES_MAX_MAT; ++i) dst.v[i] = src[i];
}

inline des_params make_params(const Param &p, const Variables &var)
{
    des_params q = {};
    q.gravity = p.control.gravity;
    q.inertial_scaling = p.control.inertial_scaling;
    q.dt_fraction = p.control.dt_fraction;
    q.fixed_dt = p.control.fixed_dt;
    q.damping_factor = p.control.damping_factor;
    q.surface_diffusivity = p.control.surface_diffusivity;
    q.damping_option = p.control.damping_option;
    q.ref_pressure_option = p.control.ref_pressure_option;
    q.surface_process_option = p.control.surface_process_option;
    q.is_quasi_static = p.control.is_quasi_static;
    q.has_thermal_diffusion = p.control.has_thermal_diffusion;
    q.surface_temperature = p.bc.surface_temperature;
    q.winkler_delta_rho = p.bc.winkler_delta_rho;
    q.elastic_foundation_constant = p.bc.elastic_foundation_constant;
    q.has_winkler_foundation = p.bc.has_winkler_foundation;
    q.has_elastic_foundation = p.bc.has_elastic_foundation;
    q.has_water_loading = p.bc.has_water_loading;
    q.zlength = p.mesh.zlength;
    q.rheol_type = p.mat.rheol_type;
    q.nmat = p.mat.nmat;
    q.is_plane_strain = p.mat.is_plane_strain;
    q.visc_min = p.mat.visc_min;
    q.visc_max = p.mat.visc_max;
    q.tension_max = p.mat.tension_max;
    q.therm_diff_max = p.mat.therm_diff_max;
    put(q.rho0, p.mat.rho0);
    put(q.alpha, p.mat.alpha);
    put(q.bulk_modulus, p.mat.bulk_modulus);
    put(q.shear_modulus, p.mat.shear_modulus);
    put(q.visc_exponent, p.mat.visc_exponent);
    put(q.visc_coefficient, p.mat.visc_coefficient);
    put(q.visc_activation_energy, p.mat.visc_activation_energy);
    put(q.heat_capacity, p.mat.heat_capacity);
    put(q.therm_cond, p.mat.therm_cond);
    put(q.pls0, p.mat.pls0);
    put(q.pls1, p.mat.pls1);
    put(q.cohesion0, p.mat.cohesion0);
    put(q.cohesion1, p.mat.cohesion1);
    put(q.friction_angle0, p.mat.friction_angle0);
    put(q.friction_angle1, p.mat.friction_angle1);
    put(q.dilation_angle0, p.mat.dilation_angle0);
    put(q.dilation_angle1, p.mat.dilation_angle1);
    for (int i = 0; i < nbdrytypes; ++i) {
        q.vbc_types[i] = var.vbc_types[i];
        q.vbc_values[i] = var.vbc_values[i];
        for (int d = 0; d < NDIMS; ++d) q.bnormals[i][d] = var.bnormals[i][d];
    }
    for (const auto &kv : var.edge_vectors)
        for (int d = 0; d < NDIMS; ++d) q.edge_vectors[kv.first.first][kv.first.second][d] = kv.second[d];
    q.max_vbc_val = var.max_vbc_val;
    q.compensation_pressure = var.compensation_pressure;
    q.precision = DES_PREC_FP64;
    return q;
}

inline des_state_view make_state(const Variables &v)
{
    des_state_view s = {};
    s.nnode = v.nnode;
    s.nelem = v.nelem;
    s.coord = v.coord->data();
    s.vel = v.vel->data();
    s.force = v.force->data();
    s.coord0 = v.coord0->data();
    s.temperature = v.temperature->data();
    s.mass = v.mass->data();
    s.tmass = v.tmass->data();
    s.volume_n = v.volume_n->data();
    s.ntmp = v.ntmp->data();
    s.volume = v.volume->data();
    s.volume_old = v.volume_old->data();
    s.edvoldt = v.edvoldt->data();
    s.plstrain = v.plstrain->data();
    s.delta_plstrain = v.delta_plstrain->data();
    s.dpressure = v.dpressure->data();
    s.tmp_result_sg = v.tmp_result_sg->data();
    s.stress = v.stress->data();
    s.strain = v.strain->data();
    s.strain_rate = v.strain_rate->data();
    s.shpdx = v.shpdx->data();
    s.shpdy = v.shpdy->data();
    s.shpdz = v.shpdz->data();
    s.tmp_result = v.tmp_result->data();
    s.time = v.time;
    s.dt = v.dt;
    s.steps = v.steps;
    return s;
}

// int_vec2D rows of marker counts, one after the other
inline std::vector<int> flat_markers(const Param &param, const Variables &var)
{
    std::vector<int> markers(static_cast<size_t>(var.nelem) * param.mat.nmat);
    for (int e = 0; e < var.nelem; ++e)
        for (int m = 0; m < param.mat.nmat; ++m) markers[static_cast<size_t>(e) * param.mat.nmat + m] = (*var.elemmarkers)[e][m];
    return markers;
}

}  // namespace des_shim_detail
