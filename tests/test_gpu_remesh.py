"""The remesh round trip: the host builds a new mesh and interpolates the
fields (a stand-in here for TetGen and the reference's interpolations), the
device takes them through des_gpu_remesh (support lists, boundary flags and
material tables rebuilt; compute_volume, volume_old, compute_mass,
compute_shape_fn and the bottom coord0 reset on the device), and the steps go
on, against the oracle doing the same on the new mesh."""
import numpy as np
import pytest

import des_gb300 as D
from des_gb300 import abi, workload as W
from helpers import (Case, COMPARED, diff_fields, phase_config, post_remesh, rel_l2,
                     remesh_standin)
from oracle.oracle import PortOracle

pytestmark = pytest.mark.gpu

FIELDS = COMPARED + ["coord0"]


def new_cfg(cfg, nx=9, ny=7, nz=5):
    n = W.scaled(cfg, nx, ny, nz)
    n.mesh_seed += 17
    return n


def fresh_device(c, params):
    dev = D.Device(c.mesh, params, device=0)
    s = W.new_state(c.mesh, c.T, c.pls)
    dev.upload(s, abi.F_COORD | abi.F_TEMPERATURE | abi.F_PLSTRAIN)
    dev.init_fields()
    return dev


def new_oracle(c, mesh2):
    p2 = abi.Params.from_buffer_copy(c.params)
    p2.compensation_pressure = c.params.rho0.v[0] * c.params.gravity * c.cfg.zlength
    return PortOracle(mesh2, p2)


@pytest.mark.parametrize("reset", [True, False])
def test_remesh_then_steps_bit_identical(reset):
    cfg = phase_config()
    c = Case(cfg)
    want = c.initial_state()
    dev = fresh_device(c, c.params)
    c.oracle.step(want, 20)
    dev.step(20)
    mesh2, s = remesh_standin(c.mesh, want, c.mesh.elemmarkers, new_cfg(cfg))
    assert mesh2.nelem != c.mesh.nelem
    dev.remesh(mesh2, s, reset_bottom_coord0=reset)
    o2 = new_oracle(c, mesh2)
    want2 = s.copy()
    post_remesh(o2, want2, cfg.zlength, reset)
    got = dev.download(abi.State(mesh2.nnode, mesh2.nelem), abi.F_ALL)
    assert not diff_fields(got, want2, FIELDS)
    assert (got.time, got.dt, got.steps) == (want2.time, want2.dt, want2.steps)
    o2.step(want2, 20)
    rep = dev.step(20)
    got = dev.download(abi.State(mesh2.nnode, mesh2.nelem), abi.F_ALL)
    dev.close()
    assert rep.status == 0 and rep.steps == 40
    assert not diff_fields(got, want2, FIELDS)
    assert (got.time, got.dt, got.steps) == (want2.time, want2.dt, want2.steps)


def test_fp32_form_remesh_then_one_step():
    cfg = phase_config()
    c = Case(cfg)
    s0 = c.state_after(20)
    mesh2, s = remesh_standin(c.mesh, s0, c.mesh.elemmarkers, new_cfg(cfg))
    o2 = new_oracle(c, mesh2)
    want = s.copy()
    post_remesh(o2, want, cfg.zlength, True)
    p = abi.Params.from_buffer_copy(c.params)
    p.precision = abi.PREC_FP32
    dev = fresh_device(c, p)
    dev.remesh(mesh2, s, reset_bottom_coord0=True)
    dev.upload(s, abi.F_SCALARS)          # the clock of the oracle's run
    got0 = dev.download(abi.State(mesh2.nnode, mesh2.nelem), abi.F_ALL)
    o2.step(want, 1)
    dev.step(1)
    got = dev.download(abi.State(mesh2.nnode, mesh2.nelem), abi.F_ALL)
    dev.close()
    for f in ["coord", "coord0", "temperature", "plstrain"]:
        assert np.array_equal(getattr(got0, f), getattr(s if f != "coord0" else want, f)), f
    errs = {f: rel_l2(getattr(got, f), getattr(want, f)) for f in ["vel", "force", "stress", "temperature"]}
    # the FP32 form's one-step bars on a layered model
    assert errs["force"] <= 1e-5 and errs["stress"] <= 1e-5, errs
    assert errs["vel"] <= 1e-3 and errs["temperature"] <= 1e-12, errs


def test_remesh_keeps_closure_and_averaging():
    from des_gb300 import closure
    cfg = W.CONFIGS["tiny"]
    c = Case(cfg)
    p = abi.Params.from_buffer_copy(c.params)
    p.precision = abi.PREC_FP32
    dev = fresh_device(c, p)
    dev.set_closure(closure.new_net(3, tol=1e-3))
    dev.set_averaging(5)
    dev.step(5)
    s0 = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    mesh2, s = remesh_standin(c.mesh, s0, c.mesh.elemmarkers, new_cfg(cfg, 5, 4, 2))
    # marker counts that change the closure's material are refused; the
    # handle is unchanged
    orig = mesh2.elemmarkers.copy()
    mesh2.elemmarkers[0, 0] += 1
    with pytest.raises(RuntimeError, match=f"error {abi.DES_ERR_UNSUPPORTED}"):
        dev.remesh(mesh2, s)
    assert dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL).steps == 5
    mesh2.elemmarkers[:] = orig
    dev.remesh(mesh2, s)
    # the closure is still set: changing the counts is refused
    em = mesh2.elemmarkers.copy()
    em[0, 0] += 1
    with pytest.raises(RuntimeError, match=f"error {abi.DES_ERR_UNSUPPORTED}"):
        dev.set_elemmarkers(em)
    rep = dev.step(5)
    assert rep.status == 0 and rep.steps == 10
    avg = dev.download_averages(5)        # sized for the new mesh
    assert avg.interval == 5 and avg.time0 > 0
    dev.close()


def assert_support_equal(dev, mesh, oracle=None):
    topo = D.Topology(mesh)                   # des_topology_build on the host
    off, el, sl = dev.support()
    assert np.array_equal(off, topo.support_offsets)
    assert np.array_equal(el, topo.support_elems)
    assert np.array_equal(sl, topo.support_slots)
    if oracle is not None:                    # create_support as the oracle restates it
        o_off, o_el = oracle.support()
        assert np.array_equal(off, o_off) and np.array_equal(el, o_el)


def test_support_lists_built_on_the_device_after_create_and_remesh():
    """create_support (mesh.cxx:1703-1717) on the device, in des_gpu_create and
    again in des_gpu_remesh for the new mesh (remeshing.cxx:2011-2012): the
    same CSR, element for element, as the host build and the oracle's."""
    cfg = phase_config()
    c = Case(cfg)
    dev = fresh_device(c, c.params)
    assert_support_equal(dev, c.mesh, c.oracle)
    want = c.initial_state()
    c.oracle.step(want, 5)
    dev.step(5)
    mesh2, s = remesh_standin(c.mesh, want, c.mesh.elemmarkers, new_cfg(cfg, 11, 8, 6))
    dev.remesh(mesh2, s, reset_bottom_coord0=True)
    assert_support_equal(dev, mesh2, new_oracle(c, mesh2))
    dev.close()


def test_support_lists_on_the_device_config2_size():
    """The same on config 2's mesh (9.6M tets, 1.66M nodes: 1,618 scan blocks)."""
    c = W.CONFIGS["2"]
    mesh, p, T, pls, topo = D.setup_case(c)
    dev = D.Device(mesh, p, device=0)
    off, el, sl = dev.support()
    dev.close()
    assert np.array_equal(off, topo.support_offsets)
    assert np.array_equal(el, topo.support_elems)
    assert np.array_equal(sl, topo.support_slots)
