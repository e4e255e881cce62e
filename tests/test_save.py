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


def marker_sets(mesh, seed, sizes=(("markerset", 300), ("hydrous-markerset", 5000))):
    """Marker sets with random barycentric positions in random elements; ids
    0..n-1 and last id n, as MarkerSet::append_marker numbers them."""
    rng = np.random.default_rng(seed)
    sets = []
    for name, n in sizes:
        eta = rng.dirichlet(np.ones(4), size=n)
        elem = rng.integers(0, mesh.nelem, n).astype(np.int32)
        mattype = rng.integers(0, 3, n).astype(np.int32)
        sets.append((name, eta, elem, mattype, np.arange(n, dtype=np.int32), n))
    return sets


def ref_with_markers(c, sets, marker_output):
    r = RefOracle(c.mesh, c.params)
    for name, eta, elem, mattype, _, _ in sets:
        r.add_markers(name, eta, elem, mattype, marker_output)
    return r


@needs_ref
def test_save_file_with_marker_sets_matches_the_reference(tmp_path):
    """Two marker sets (the second one past MarkerSet's 4096 preallocated
    markers) written into the .save file: marker coordinates summed from the
    element's nodes as MarkerSet::write_save_file does."""
    c = Case(W.CONFIGS["1"])
    s = run(c, c.initial_state(), 15)
    sets = marker_sets(c.mesh, 7)
    r = ref_with_markers(c, sets, True)
    r.output_begin(tmp_path / "ref", frame=3, averaged=False, interval=10)
    r.output_write(s, exact=False)
    D.write_save(tmp_path / "ours.save", c.mesh, c.params, c.oracle.bcflag(), s, markers=sets)
    a = (tmp_path / "ref.save.000003").read_bytes()
    b = (tmp_path / "ours.save").read_bytes()
    assert a[:4096] == b[:4096]
    assert a == b


@needs_ref
def test_checkpoint_file_with_marker_sets_matches_the_reference(tmp_path):
    """The checkpoint always carries the marker sets (sizes with the last id,
    barycentric coordinates, elements, material types, ids)."""
    c = Case(W.CONFIGS["1"])
    s = run(c, c.initial_state(), 6)
    sets = marker_sets(c.mesh, 11)
    r = ref_with_markers(c, sets, False)
    r.output_begin(tmp_path / "ref", frame=1, averaged=False, interval=10)
    r.output_checkpoint(s)
    D.write_checkpoint(tmp_path / "ours.chkpt", c.mesh, s, r.compensation_pressure(), markers=sets)
    a = (tmp_path / "ref.chkpt.000001").read_bytes()
    b = (tmp_path / "ours.chkpt").read_bytes()
    assert a[:4096] == b[:4096]
    assert a == b


def test_marker_set_layout_and_coordinates(tmp_path):
    """Without the reference: the marker arrays follow bcflag under the set's
    name, and each marker's coordinate is sum_k eta_k x(conn_k)."""
    c = Case(W.CONFIGS["tiny"])
    s = run(c, c.initial_state(), 2)
    sets = marker_sets(c.mesh, 3, (("markerset", 40), ("empty-set", 0)))
    D.write_save(tmp_path / "x.save", c.mesh, c.params, c.oracle.bcflag(), s, markers=sets)
    raw = (tmp_path / "x.save").read_bytes()
    head = raw[:4096].split(b"\0")[0].decode().splitlines()[1:]
    names = [h.split("\t")[0] for h in head]
    assert names[names.index("bcflag") + 1:] == [
        "markerset size", "markerset.coord", "markerset.elem", "markerset.mattype", "markerset.id",
        "empty-set size", "empty-set.coord", "empty-set.elem", "empty-set.mattype", "empty-set.id"]
    pos = {h.split("\t")[0]: int(h.split("\t")[1]) for h in head}
    _, eta, elem, mattype, ids, _ = sets[0]
    assert np.frombuffer(raw[pos["markerset size"]:pos["markerset size"] + 4], np.int32)[0] == 40
    xyz = np.frombuffer(raw[pos["markerset.coord"]:pos["markerset.elem"]], np.float64).reshape(-1, 3)
    want = np.einsum("mk,mkj->mj", eta, s.coord[c.mesh.connectivity[elem]])
    assert np.allclose(xyz, want, rtol=0, atol=1e-12 * np.abs(s.coord).max())
    assert np.array_equal(np.frombuffer(raw[pos["markerset.elem"]:pos["markerset.mattype"]], np.int32), elem)
    assert np.array_equal(np.frombuffer(raw[pos["markerset.mattype"]:pos["markerset.id"]], np.int32), mattype)
    assert np.array_equal(np.frombuffer(raw[pos["markerset.id"]:pos["empty-set size"]], np.int32), ids)
    assert pos["empty-set.id"] == len(raw)


def test_marker_sets_out_of_range_are_refused(tmp_path):
    c = Case(W.CONFIGS["tiny"])
    s = c.initial_state()
    name, eta, elem, mattype, ids, n = marker_sets(c.mesh, 5, (("markerset", 8),))[0]
    bad = elem.copy()
    bad[3] = c.mesh.nelem
    with pytest.raises(Exception):
        D.write_save(tmp_path / "x.save", c.mesh, c.params, c.oracle.bcflag(), s,
                     markers=[(name, eta, bad, mattype, ids, n)])
    with pytest.raises(Exception):
        D.write_checkpoint(tmp_path / "x.chkpt", c.mesh, s, 0.0, markers=[(name, eta[:4], elem, mattype, ids, n)])
