"""The remesh trigger on the device: elem_quality and bad_mesh_quality
(geometry.cxx:472-526, remeshing.cxx:1893-1960) against the oracle, and the
step unaffected by a check between steps."""
import numpy as np
import pytest

import des_gb300 as D
from des_gb300 import abi
from helpers import Case, plastic_config, diff_fields, COMPARED
from test_remesh_check import check

pytestmark = pytest.mark.gpu

_case = {}


def case():
    if "c" not in _case:
        _case["c"] = Case(plastic_config())
    return _case["c"]


def device(c, state, precision):
    p = abi.Params.from_buffer_copy(c.params)
    p.precision = precision
    dev = D.Device(c.mesh, p, device=0)
    dev.upload(state, abi.F_ALL)
    return dev


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_FP32])
def test_quality_matches_the_oracle(gpu, precision):
    c = case()
    dev = device(c, c.state_after(5), precision)
    dev.step(20)
    s = dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL)
    q = dev.elem_quality()
    assert np.array_equal(q, c.oracle.elem_quality(s))
    dx = float(np.ptp(s.coord[:, 0])) / 6
    base = dict(resolution=dx, zlength=float(-c.mesh.coord[:, 2].min()))
    for kw in (dict(), dict(min_quality=2.0), dict(min_quality=0.0, remeshing_option=0)):
        chk = check(**base, **kw)
        assert dev.bad_mesh_quality(chk) == c.oracle.bad_mesh_quality(s, chk), kw
    dev.close()


def test_each_check_in_order(gpu):
    c = case()
    s = c.state_after(5)
    dx = float(np.ptp(s.coord[:, 0])) / 6
    base = dict(resolution=dx, zlength=float(-s.coord[:, 2].min()))
    t = s.copy()
    bottom = np.nonzero(c.oracle.bcflag() & 16)[0]
    t.coord[bottom[5], 2] -= 0.3 * dx
    dev = device(c, t, abi.PREC_FP64)
    assert dev.bad_mesh_quality(check(min_quality=2.0, **base))[:2] == (2, int(bottom[5]))
    t.volume[11] *= 1e-6
    dev.upload(t, abi.F_VOLUME)
    assert dev.bad_mesh_quality(check(min_quality=2.0, **base))[:2] == (3, 11)
    assert dev.bad_mesh_quality(check(min_quality=2.0, **base)) == \
        c.oracle.bad_mesh_quality(t, check(min_quality=2.0, **base))
    dev.close()


def test_a_check_between_steps_changes_nothing(gpu):
    c = case()
    s0 = c.state_after(5)
    out = []
    for with_check in (False, True):
        dev = device(c, s0, abi.PREC_FP64)
        dev.step(3)
        if with_check:
            dev.bad_mesh_quality(check(resolution=1e4, zlength=1e4))
            dev.elem_quality()
        dev.step(3)
        out.append(dev.download(abi.State(c.mesh.nnode, c.mesh.nelem), abi.F_ALL))
        dev.close()
    assert not diff_fields(out[0], out[1], [f for f in COMPARED if f != "ntmp"])
