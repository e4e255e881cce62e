"""The .save writer (des_write_save) against the reference's own Output
(output.cxx compiled from its sources), byte for byte, and its averaged form
against the restated Output::average_fields."""
import numpy as np
import pytest

import des_gb300 as D
from des_gb300 import workload as W
from helpers import Case
from oracle.oracle import RefOracle, Averages

needs_ref = pytest.mark.skipif(not RefOracle.available(), reason="reference build absent")


def run(case, s, nsteps, avg=None):
    for _ in range(nsteps):
        case.oracle.step(s, 1)
        if avg is not None:
            avg.update(s)
    return s


@needs_ref
@pytest.mark.parametrize("exact", [False, True])
def test_save_file_matches_the_reference(tmp_path, exact):
    c = Case(W.CONFIGS["1"])
    s = run(c, c.initial_state(), 25)
    r = RefOracle(c.mesh, c.params)
    r.output_begin(tmp_path / "ref", frame=4, averaged=False, interval=10)
    r.output_write(s, exact=exact)
    D.write_save(tmp_path / "ours.save", c.mesh, c.params, c.oracle.bcflag(), s)
    a = (tmp_path / "ref.save.000004").read_bytes()
    b = (tmp_path / "ours.save").read_bytes()
    assert len(a) == len(b) and a == b


@needs_ref
def test_averaged_save_file_matches_the_reference(tmp_path):
    """Averaging over an interval of 10 steps (the reference averages inside
    its loop; ours from the restated average_fields), written after step 30."""
    c = Case(W.CONFIGS["1"])
    interval = 10
    s0 = c.initial_state()
    r = RefOracle(c.mesh, c.params)
    r.output_begin(tmp_path / "ref", frame=2, averaged=True, interval=interval)
    rs = s0.copy()
    r.step(rs, 30)                    # averages in every step
    avg = Averages(interval)
    s = run(c, s0.copy(), 30, avg)
    r.output_write(s, exact=False)
    D.write_save(tmp_path / "ours.save", c.mesh, c.params, c.oracle.bcflag(), s,
                 D.save_averages(avg.coord0, avg.strain0, avg.stress_sum, avg.dpls_sum, avg.time0,
                                 interval))
    a = (tmp_path / "ref.save.000002").read_bytes()
    b = (tmp_path / "ours.save").read_bytes()
    assert a[:4096] == b[:4096]
    assert a == b


def test_save_header_and_layout(tmp_path):
    """Without the reference: the header names the arrays at their offsets."""
    c = Case(W.CONFIGS["tiny"])
    s = run(c, c.initial_state(), 3)
    D.write_save(tmp_path / "x.save", c.mesh, c.params, c.oracle.bcflag(), s)
    raw = (tmp_path / "x.save").read_bytes()
    head = raw[:4096].split(b"\0")[0].decode().splitlines()
    assert head[0] == "# DynEarthSol ndims=3 revision=3"
    names = [h.split("\t")[0] for h in head[1:]]
    assert names == ["coordinate", "connectivity", "velocity", "temperature", "plastic strain",
                     "plastic strain-rate", "strain-rate", "strain", "stress", "density", "mesh quality",
                     "viscosity", "material", "force", "coord0", "bcflag"]
    pos = {h.split("\t")[0]: int(h.split("\t")[1]) for h in head[1:]}
    stress = np.frombuffer(raw[pos["stress"]:pos["density"]], dtype=np.float64).reshape(-1, 6)
    assert np.array_equal(stress, s.stress)


@needs_ref
def test_checkpoint_file_matches_the_reference(tmp_path):
    c = Case(W.CONFIGS["1"])
    s = run(c, c.initial_state(), 12)
    r = RefOracle(c.mesh, c.params)
    r.output_begin(tmp_path / "ref", frame=1, averaged=False, interval=10)
    r.output_checkpoint(s)
    D.write_checkpoint(tmp_path / "ours.chkpt", c.mesh, s, r.compensation_pressure())
    assert (tmp_path / "ref.chkpt.000001").read_bytes() == (tmp_path / "ours.chkpt").read_bytes()
