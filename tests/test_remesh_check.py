"""The oracle's restatement of bad_mesh_quality (remeshing.cxx:1893-1960) on
crafted states: each of the three checks, in the reference's order."""
import numpy as np

from des_gb300 import abi
from helpers import Case, plastic_config


def check(**kw):
    c = abi.RemeshCheck(smallest_size=0.01, resolution=1.0, zlength=1.0, max_boundary_distortion=0.25,
                        min_quality=0.4, remeshing_option=1)
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def test_restated_checks_and_their_order():
    case = Case(plastic_config())
    s = case.state_after(5)
    dx = float(np.ptp(s.coord[:, 0])) / 6
    zl = float(-s.coord[:, 2].min())
    base = dict(resolution=dx, zlength=zl)
    code, _, q = case.oracle.bad_mesh_quality(s, check(**base))
    assert code == 0 and 0 < q <= 1
    # a quality bar above the worst element: code 1 at the first worst element
    qe = case.oracle.elem_quality(s)
    code, idx, q = case.oracle.bad_mesh_quality(s, check(min_quality=q + 1e-9, **base))
    assert code == 1 and idx == int(np.argmin(qe)) and q == min(1.0, qe.min()) ** (1 / 3)
    # a bottom node pushed down: code 2 takes precedence over code 1
    t = s.copy()
    bottom = np.nonzero(case.oracle.bcflag() & 16)[0]
    t.coord[bottom[3], 2] -= 0.3 * dx
    code, idx, _ = case.oracle.bad_mesh_quality(t, check(min_quality=2.0, **base))
    assert (code, idx) == (2, int(bottom[3]))
    # the bottom check only runs for remeshing options 1, 2 and 11
    code, _, _ = case.oracle.bad_mesh_quality(t, check(remeshing_option=0, **base))
    assert code == 0
    # a tiny element: code 3 first
    t.volume[7] = 1e-6 * t.volume[7]
    code, idx, _ = case.oracle.bad_mesh_quality(t, check(min_quality=2.0, **base))
    assert (code, idx) == (3, 7)
