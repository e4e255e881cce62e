// The reference's hot-path functions under their own names and signatures
// (fields.hpp:6-12, geometry.hpp:5-27, rheology.hpp:4-6, bc.hpp:8), defined on
// the C ABI of libdes_gb300.so.  Linked in place of the reference's own
// definitions (the reference replaces functions at link time: its loop calls
// free functions), dynearthsol.cxx runs unchanged -- init, restart, remesh,
// isostasy_adjustment and the loop body 358-394 -- with every one of these
// functions computed on the GPU.
//
// Each call uploads the fields the function reads from the host Variables,
// runs the function's entry point on the device, and downloads the fields it
// writes: the host arrays stay authoritative, as in the reference, and results
// are those of the device entry points (bit-identical to the reference's
// functions in FP64; the eigen-solver's transcendentals within 1e-12).  This is
// the per-function mode, for moving one function at a time and for
// debugging; the loop-level drop-in (des_shim_step, des_shim.hpp) keeps the
// state on the device and runs the whole step as one graph.
//
// One device state per process, for the Variables and mesh of the last call:
// a call on another mesh (after remesh's reallocate_variables) creates a new
// one, from the Param of the last call that took a Param (compute_mass, which
// init, restart and remesh call before any Param-less function).  Errors end
// the program as the reference does: exit(11) for dt <= 0, exit(12) for
// inconsistent topology, exit(1) otherwise, with a message on stderr.
// compute_volume takes any arrays (the reference calls it on marker and
// remesh-candidate meshes too) and runs without the device state.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "des_shim_internal.hpp"
#include "fields.hpp"
#include "geometry.hpp"
#include "rheology.hpp"
#include "bc.hpp"

using namespace des_shim_detail;

namespace {

struct Bound {
    des_gpu *g = nullptr;
    const Variables *var = nullptr;
    const int *conn = nullptr;
    int nnode = -1, nelem = -1, nseg = -1;
    const Param *param = nullptr;
};
Bound B;

[[noreturn]] void fail(const char *fn, const char *what, int rc)
{
    std::fprintf(stderr, "Error: %s on the GPU: %s: %s\n", fn, what, des_gpu_error_string(rc));
    std::exit(rc == DES_ERR_DT || rc == DES_ERR_TOPOLOGY || rc == DES_ERR_OPTION ? rc : 1);
}

void check(const char *fn, const char *what, int rc)
{
    if (rc) fail(fn, what, rc);
}

// The per-function mode works on the loop's own arrays; other arrays have no
// device copy.
void require(bool same, const char *fn)
{
    if (same) return;
    std::fprintf(stderr, "Error: %s on the GPU needs the arrays of Variables (var.*)\n", fn);
    std::exit(1);
}

// The device state for var's mesh (created, or created anew after a remesh).
des_gpu *bind(const char *fn, const Variables &var, const Param *param)
{
    if (param) B.param = param;
    const bool same = B.g && B.var == &var && B.conn == var.connectivity->data() &&
                      B.nnode == var.nnode && B.nelem == var.nelem && B.nseg == var.nseg;
    if (same) return B.g;
    if (!B.param) {
        std::fprintf(stderr, "Error: %s on the GPU before any call with a Param\n", fn);
        std::exit(1);
    }
    if (B.g) des_gpu_destroy(B.g);
    B.g = nullptr;
    des_params q = make_params(*B.param, var);
    std::vector<int> markers = flat_markers(*B.param, var);
    des_mesh_view mesh = {var.nnode, var.nelem, var.nseg, B.param->mat.nmat, var.connectivity->data(),
                          var.segment->data(), var.segflag->data(), markers.data()};
    check(fn, "des_gpu_create", des_gpu_create(&mesh, &q, -1, &B.g));
    B.var = &var;
    B.conn = var.connectivity->data();
    B.nnode = var.nnode;
    B.nelem = var.nelem;
    B.nseg = var.nseg;
    return B.g;
}

// Param and Variables scalars (boundary normals, velocity boundary values,
// compensation pressure), which init sets between the first calls.
void sync_params(const char *fn, const Param &param, const Variables &var)
{
    des_params q = make_params(param, var);
    check(fn, "des_gpu_set_params", des_gpu_set_params(B.g, &q));
}

// Marker counts, which phase_changes and remeshing change in var.elemmarkers
// (MatProps reads them through a reference, matprops.cxx:165).
void sync_markers(const char *fn, const Variables &var)
{
    std::vector<int> markers = flat_markers(*B.param, var);
    check(fn, "des_gpu_set_elemmarkers", des_gpu_set_elemmarkers(B.g, markers.data()));
}

void up(const char *fn, const Variables &var, unsigned mask)
{
    des_state_view s = make_state(var);
    check(fn, "des_gpu_upload", des_gpu_upload(B.g, &s, mask));
}

void down(const char *fn, const Variables &var, unsigned mask)
{
    des_state_view s = make_state(var);
    check(fn, "des_gpu_download", des_gpu_download(B.g, &s, mask));
}

}  // namespace

// fields.cxx:108-172
void update_temperature(const Param &param, const Variables &var, double_vec &temperature,
                        double_vec &tdot, elem_cache &tmp_result)
{
    const char *fn = "update_temperature";
    require(&temperature == var.temperature && &tdot == var.ntmp && &tmp_result == var.tmp_result, fn);
    bind(fn, var, &param);
    sync_params(fn, param, var);
    sync_markers(fn, var);
    up(fn, var, DES_F_TEMPERATURE | DES_F_SHAPE | DES_F_VOLUME | DES_F_MASS | DES_F_SCALARS);
    check(fn, "des_gpu_update_temperature", des_gpu_update_temperature(B.g));
    down(fn, var, DES_F_TEMPERATURE | DES_F_NTMP | DES_F_TMP_RESULT);
}

// fields.cxx:175-247
void update_strain_rate(const Variables &var, tensor_t &strain_rate)
{
    const char *fn = "update_strain_rate";
    require(&strain_rate == var.strain_rate, fn);
    bind(fn, var, nullptr);
    up(fn, var, DES_F_VEL | DES_F_SHAPE);
    check(fn, "des_gpu_update_strain_rate", des_gpu_update_strain_rate(B.g));
    down(fn, var, DES_F_STRAIN_RATE);
}

// geometry.cxx:117-151
void compute_dvoldt(const Variables &var, double_vec &dvoldt, double_vec &tmp_result_sg)
{
    const char *fn = "compute_dvoldt";
    require(&dvoldt == var.ntmp && &tmp_result_sg == var.tmp_result_sg, fn);
    bind(fn, var, nullptr);
    up(fn, var, DES_F_STRAIN_RATE | DES_F_VOLUME | DES_F_MASS);
    check(fn, "des_gpu_compute_dvoldt", des_gpu_compute_dvoldt(B.g));
    down(fn, var, DES_F_NTMP | DES_F_TMP_RESULT);
}

// geometry.cxx:154-182
void compute_edvoldt(const Variables &var, double_vec &dvoldt, double_vec &edvoldt)
{
    const char *fn = "compute_edvoldt";
    require(&dvoldt == var.ntmp && &edvoldt == var.edvoldt, fn);
    bind(fn, var, nullptr);
    up(fn, var, DES_F_NTMP);
    check(fn, "des_gpu_compute_edvoldt", des_gpu_compute_edvoldt(B.g));
    down(fn, var, DES_F_EDVOLDT);
}

// rheology.cxx:513-654 (stressyy is the 2D plane-strain field, untouched in 3D)
void update_stress(const Variables &var, tensor_t &stress, double_vec &stressyy,
                   double_vec &dpressure, tensor_t &strain, double_vec &plstrain,
                   double_vec &delta_plstrain, tensor_t &strain_rate)
{
    const char *fn = "update_stress";
    (void)stressyy;
    require(&stress == var.stress && &dpressure == var.dpressure && &strain == var.strain &&
                &plstrain == var.plstrain && &delta_plstrain == var.delta_plstrain &&
                &strain_rate == var.strain_rate, fn);
    bind(fn, var, nullptr);
    sync_markers(fn, var);
    up(fn, var, DES_F_STRESS | DES_F_STRAIN | DES_F_STRAIN_RATE | DES_F_EDVOLDT | DES_F_PLSTRAIN |
                    DES_F_TEMPERATURE | DES_F_VOLUME | DES_F_SCALARS);
    check(fn, "des_gpu_update_stress", des_gpu_update_stress(B.g));
    down(fn, var, DES_F_STRESS | DES_F_STRAIN | DES_F_STRAIN_RATE | DES_F_PLSTRAIN | DES_F_DPRESSURE);
}

// geometry.cxx:185-254
void NMD_stress(const Variables &var, double_vec &dp_nd, tensor_t &stress, double_vec &tmp_result_sg)
{
    const char *fn = "NMD_stress";
    require(&dp_nd == var.ntmp && &stress == var.stress && &tmp_result_sg == var.tmp_result_sg, fn);
    bind(fn, var, nullptr);
    up(fn, var, DES_F_DPRESSURE | DES_F_VOLUME | DES_F_MASS | DES_F_STRESS);
    check(fn, "des_gpu_NMD_stress", des_gpu_NMD_stress(B.g));
    down(fn, var, DES_F_NTMP | DES_F_STRESS | DES_F_TMP_RESULT);
}

// fields.cxx:312-375, with apply_stress_bcs (bc.cxx:503-595) and apply_damping
// (fields.cxx:250-309) as update_force calls them
void update_force(const Param &param, const Variables &var, array_t &force, elem_cache &tmp_result)
{
    const char *fn = "update_force";
    require(&force == var.force && &tmp_result == var.tmp_result, fn);
    bind(fn, var, &param);
    sync_params(fn, param, var);
    sync_markers(fn, var);
    up(fn, var, DES_F_STRESS | DES_F_SHAPE | DES_F_VOLUME | DES_F_TEMPERATURE | DES_F_COORD |
                    DES_F_VEL | DES_F_MASS);
    check(fn, "des_gpu_update_force", des_gpu_update_force(B.g));
    down(fn, var, DES_F_FORCE | DES_F_TMP_RESULT);
}

// fields.cxx:378-393
void update_velocity(const Variables &var, array_t &vel)
{
    const char *fn = "update_velocity";
    require(&vel == var.vel, fn);
    bind(fn, var, nullptr);
    up(fn, var, DES_F_VEL | DES_F_FORCE | DES_F_MASS | DES_F_SCALARS);
    check(fn, "des_gpu_update_velocity", des_gpu_update_velocity(B.g));
    down(fn, var, DES_F_VEL);
}

// bc.cxx:182-500
void apply_vbcs(const Param &param, const Variables &var, array_t &vel)
{
    const char *fn = "apply_vbcs";
    require(&vel == var.vel, fn);
    bind(fn, var, &param);
    sync_params(fn, param, var);
    up(fn, var, DES_F_VEL | DES_F_COORD);
    check(fn, "des_gpu_apply_vbcs", des_gpu_apply_vbcs(B.g));
    down(fn, var, DES_F_VEL);
}

// fields.cxx:396-412
void update_coordinate(const Variables &var, array_t &coord)
{
    const char *fn = "update_coordinate";
    require(&coord == var.coord, fn);
    bind(fn, var, nullptr);
    up(fn, var, DES_F_COORD | DES_F_VEL | DES_F_SCALARS);
    check(fn, "des_gpu_update_coordinate", des_gpu_update_coordinate(B.g));
    down(fn, var, DES_F_COORD);
}

// geometry.cxx:86-114, on any mesh
void compute_volume(const array_t &coord, const conn_t &connectivity, double_vec &volume)
{
    if (volume.size() < connectivity.size()) volume.resize(connectivity.size());
    check("compute_volume", "des_compute_volume",
          des_compute_volume(static_cast<int>(coord.size()), static_cast<int>(connectivity.size()),
                             coord.data(), connectivity.data(), volume.data()));
}

// geometry.cxx:333-385
void compute_mass(const Param &param, const Variables &var, const conn_t &connectivity,
                  const double_vec &volume, const MatProps &mat, double max_vbc_val,
                  double_vec &volume_n, double_vec &mass, double_vec &tmass, elem_cache &tmp_result,
                  int_vec2D &support)
{
    const char *fn = "compute_mass";
    (void)mat;
    (void)support;
    require(&connectivity == var.connectivity && &volume == var.volume && &volume_n == var.volume_n &&
                &mass == var.mass && &tmass == var.tmass && &tmp_result == var.tmp_result &&
                max_vbc_val == var.max_vbc_val, fn);
    bind(fn, var, &param);
    sync_params(fn, param, var);
    sync_markers(fn, var);
    up(fn, var, DES_F_VOLUME | DES_F_TEMPERATURE);
    check(fn, "des_gpu_compute_mass", des_gpu_compute_mass(B.g));
    down(fn, var, DES_F_MASS | DES_F_TMP_RESULT);
}

// geometry.cxx:388-470
void compute_shape_fn(const Variables &var, const array_t &coord, const conn_t &connectivity,
                      const double_vec &volume, shapefn &shpdx, shapefn &shpdy, shapefn &shpdz)
{
    const char *fn = "compute_shape_fn";
    require(&coord == var.coord && &connectivity == var.connectivity && &volume == var.volume &&
                &shpdx == var.shpdx && &shpdy == var.shpdy && &shpdz == var.shpdz, fn);
    bind(fn, var, nullptr);
    up(fn, var, DES_F_COORD | DES_F_VOLUME);
    check(fn, "des_gpu_compute_shape_fn", des_gpu_compute_shape_fn(B.g));
    down(fn, var, DES_F_SHAPE);
}

// fields.cxx:455-533
void rotate_stress(const Variables &var, tensor_t &stress, tensor_t &strain)
{
    const char *fn = "rotate_stress";
    require(&stress == var.stress && &strain == var.strain, fn);
    bind(fn, var, nullptr);
    up(fn, var, DES_F_STRESS | DES_F_STRAIN | DES_F_VEL | DES_F_SHAPE | DES_F_SCALARS);
    check(fn, "des_gpu_rotate_stress", des_gpu_rotate_stress(B.g));
    down(fn, var, DES_F_STRESS | DES_F_STRAIN);
}

// geometry.cxx:257-330 (exit(11) on dt <= 0, as the reference)
double compute_dt(const Param &param, const Variables &var)
{
    const char *fn = "compute_dt";
    bind(fn, var, &param);
    sync_params(fn, param, var);
    sync_markers(fn, var);
    up(fn, var, DES_F_COORD | DES_F_VOLUME | DES_F_TEMPERATURE);
    double dt = 0;
    int rc = des_gpu_compute_dt(B.g, &dt);
    if (rc == DES_ERR_DT) {
        std::fprintf(stderr, "Error: dt <= 0!  %g\n", dt);
        std::exit(11);
    }
    check(fn, "des_gpu_compute_dt", rc);
    return dt;
}
