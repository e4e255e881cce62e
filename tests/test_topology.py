"""Mesh, boundary flags, support lists, boundary nodes and facets: the
library's host builder against the oracle (and the reference where present),
bit for bit."""
import numpy as np
import pytest

import des_gb300 as D
from des_gb300 import abi, workload as W
from helpers import layered_config
from oracle.oracle import PortOracle, RefOracle


@pytest.mark.parametrize("key", ["tiny", "1", "layered"])
def test_topology_matches_oracle_and_reference(key):
    cfg = layered_config() if key == "layered" else W.CONFIGS[key]
    mesh, p, T, pls, topo = D.setup_case(cfg)
    checkers = [PortOracle(mesh, p)] + ([RefOracle(mesh, p)] if RefOracle.available() else [])
    for o in checkers:
        assert np.array_equal(topo.bcflag, o.bcflag())
        off, el = o.support()
        assert np.array_equal(topo.support_offsets, off)
        assert np.array_equal(topo.support_elems, el)
        for b in range(abi.DES_NBDRY):
            assert np.array_equal(topo.bnodes[b], o.bnodes(b)), b
            assert np.array_equal(topo.bfacets[b], o.bfacets(b)), b
    # support slot is the node's position in the element
    conn = mesh.connectivity
    n_of = np.repeat(np.arange(mesh.nnode), np.diff(topo.support_offsets))
    assert np.array_equal(conn[topo.support_elems, topo.support_slots], n_of)


def test_boundary_normals_match_reference():
    if not RefOracle.available():
        pytest.skip("reference build absent")
    cfg = W.CONFIGS["1"]
    mesh, p, T, pls, topo = D.setup_case(cfg)
    r = RefOracle(mesh, p)
    s = W.new_state(mesh, T, pls)
    r.init_fields(s)
    bn, ev = r.normals()
    assert np.array_equal(np.array(p.bnormals), bn)
    got = np.array(p.edge_vectors)
    for i in range(10):
        for j in range(i + 1, 10):
            if len(topo.bfacets[i]) and len(topo.bfacets[j]):
                assert np.array_equal(got[i, j], ev[i, j])


@pytest.mark.parametrize("key", ["tiny", "1"])
def test_box_mesh_properties(key):
    cfg = W.CONFIGS[key]
    L = D.lib()
    m = W.Mesh(cfg, L)
    assert m.nnode == cfg.nnode and m.nelem == cfg.nelem
    assert m.nseg == 4 * (cfg.ny * cfg.nz + cfg.nx * cfg.nz + cfg.nx * cfg.ny)
    x = m.coord[m.connectivity]
    d1, d2, d3 = x[:, 1] - x[:, 0], x[:, 2] - x[:, 0], x[:, 3] - x[:, 0]
    vol = np.einsum("ij,ij->i", np.cross(d1, d2), d3)
    assert (np.abs(vol) > 0).all()
    # walls stay planar under jitter
    assert np.isin(m.coord[:, 0].round(9), m.coord[:, 0].round(9)).all()
    top = m.coord[:, 2] >= 0
    assert np.all(m.coord[top, 2] == 0)
    assert np.isclose(m.coord[:, 2].min(), -cfg.zlength)
    # every segment flag is a single wall bit
    assert all(bin(f).count("1") == 1 for f in m.segflag)
    # determinism of the seeded generator
    m2 = W.Mesh(cfg, L)
    assert np.array_equal(m.coord, m2.coord) and np.array_equal(m.connectivity, m2.connectivity)


def test_layered_markers_and_temperature_profile():
    cfg = layered_config()
    L = D.lib()
    m = W.Mesh(cfg, L)
    assert (m.elemmarkers.sum(axis=1) == 4).all()
    assert m.elemmarkers.shape[1] == 3 and (m.elemmarkers[:, 2] > 0).any()
    T, pls = W.initial_inputs(cfg, m, L)
    top = m.coord[:, 2] >= 0
    assert np.all(T[top] == 273.0)
    assert 273.0 + 1330 - 150 < T[~top].max() < 273.0 + 1330 + 150
