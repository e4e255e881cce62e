// See des_shim.hpp.  Builds des_params / des_mesh_view / des_state_view from
// the reference's structures (parameters.hpp:36-287); every pointer handed to
// the library points into the reference's own Array2D / std::vector storage.
#include "des_shim.hpp"

#include <cstdio>
#include <vector>

#include "des_shim_internal.hpp"

using namespace des_shim_detail;

des_gpu *des_shim_attach(const Param &param, Variables &var)
{
    des_params q = make_params(param, var);
    std::vector<int> markers = flat_markers(param, var);
    des_mesh_view mesh = {var.nnode, var.nelem, var.nseg, param.mat.nmat, var.connectivity->data(),
                          var.segment->data(), var.segflag->data(), markers.data()};
    des_gpu *g = nullptr;
    int rc = des_gpu_create(&mesh, &q, -1, &g);
    if (rc) {
        std::fprintf(stderr, "des_gpu_create: %s\n", des_gpu_error_string(rc));
        return nullptr;
    }
    des_state_view s = make_state(var);
    rc = des_gpu_upload(g, &s, DES_F_STEP_STATE | DES_F_COORD0);
    if (rc) {
        std::fprintf(stderr, "des_gpu_upload: %s\n", des_gpu_error_string(rc));
        des_gpu_destroy(g);
        return nullptr;
    }
    return g;
}

int des_shim_step(des_gpu *g, Variables &var, int nsteps)
{
    des_step_report r;
    int rc = des_gpu_step(g, nsteps, &r);
    var.steps = r.steps;
    var.time = r.time;
    var.dt = r.dt;
    return rc;
}

int des_shim_download(des_gpu *g, Variables &var, unsigned mask)
{
    des_state_view s = make_state(var);
    int rc = des_gpu_download(g, &s, mask);
    if (mask & DES_F_SCALARS) {
        var.time = s.time;
        var.dt = s.dt;
        var.steps = s.steps;
    }
    return rc;
}

int des_shim_phase_changes(des_gpu *g, const Param &param, Variables &var)
{
    std::vector<int> markers = flat_markers(param, var);
    int rc = des_gpu_set_elemmarkers(g, markers.data());
    if (rc) return rc;
    return des_gpu_compute_dt(g, &var.dt);
}

int des_shim_remeshed(des_gpu *g, const Param &param, Variables &var)
{
    std::vector<int> markers = flat_markers(param, var);
    des_mesh_view mesh = {var.nnode, var.nelem, var.nseg, param.mat.nmat, var.connectivity->data(),
                          var.segment->data(), var.segflag->data(), markers.data()};
    des_state_view s = make_state(var);
    const int opt = param.mesh.remeshing_option;
    return des_gpu_remesh(g, &mesh, &s, opt == 1 || opt == 2 || opt == 11);
}
