"""TEST INFRASTRUCTURE -- the seeded synthetic workloads restated in numpy.

The CPU arm of the benchmark must build its case without loading the product
library, so this file restates the box-mesh generator of the product's
csrc/workload.cpp (the contract is in include/des_workload.h) operation by
operation in IEEE double: the same node jitter from the same counter-based
splitmix64 stream, the same Kuhn split and orientation, the same boundary
segments and flags (constants.hpp:39-44, facet table constants.hpp:61-67), the
same marker counts and temperatures.  tests/test_workload_np.py checks that
both give identical arrays.  The boundary flags, support lists and normals
then come from the oracle itself (PortOracle), as the reference derives them
from the mesh (mesh.cxx:1529-1717, bc.cxx:90-179).
"""
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "dynearthsol-old_gb300"))
from des_gb300 import abi  # noqa: E402  (ctypes structs only; loads no library)

_M = np.uint64
_FACET = np.array([[1, 2, 3], [0, 3, 2], [0, 1, 3], [0, 2, 1]])


def _mix64(z):
    """splitmix64 finaliser (Steele, Lea & Flood 2014) on uint64 arrays."""
    with np.errstate(over="ignore"):
        z = z + _M(0x9E3779B97F4A7C15)
        z = (z ^ (z >> _M(30))) * _M(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> _M(27))) * _M(0x94D049BB133111EB)
        return z ^ (z >> _M(31))


def u01(seed, stream, index):
    """Uniform doubles in [0, 1) from the counter (seed, stream, index)."""
    with np.errstate(over="ignore"):
        key = _mix64(np.asarray(_M(seed) ^ (_M(stream) * _M(0xD1B54A32D192ED03)), dtype=_M))
        r = _mix64(key + np.asarray(index, dtype=_M))
    return (r >> _M(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def _signed_volume(p):
    d01, d12, d23 = p[0] - p[1], p[1] - p[2], p[2] - p[3]
    return (d01[0] * (d23[1] * d12[2] - d12[1] * d23[2]) + d12[0] * (d01[1] * d23[2] - d23[1] * d01[2]) +
            d23[0] * (d12[1] * d01[2] - d01[1] * d12[2])) / 6


def _kuhn():
    """Corner (a + 2b + 4c of the unit cube) of each vertex of the six tets."""
    out = []
    for perm in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
        s0 = 1 << perm[0]
        s1 = s0 | (1 << perm[1])
        c = [0, s0, s1, 7]
        p = np.array([[(cc >> d) & 1 for d in range(3)] for cc in c], np.float64)
        if _signed_volume(p) < 0:
            c[1], c[2] = c[2], c[1]
        out.append(c)
    return np.array(out)


def box(nx, ny, nz, xlength, ylength, zlength, jitter, seed):
    """coord [nnode,3], connectivity [nelem,4], segment [nseg,3], segflag [nseg]."""
    i, j, k = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), np.arange(nz + 1), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    n = ((i * (ny + 1) + j) * (nz + 1) + k).astype(np.uint64)
    x = (xlength * i.astype(np.float64)) / nx
    y = (ylength * j.astype(np.float64)) / ny
    z = np.where(k == nz, 0.0, -((zlength * (nz - k).astype(np.float64)) / nz))
    if jitter != 0:
        hx, hy, hz = xlength / nx, ylength / ny, zlength / nz
        for arr, idx, h, lim, d in ((x, i, hx, nx, 0), (y, j, hy, ny, 1), (z, k, hz, nz, 2)):
            inner = (idx > 0) & (idx < lim)
            u = u01(seed, 1, _M(3) * n[inner] + _M(d))
            arr[inner] = arr[inner] + jitter * h * (2 * u - 1)
    coord = np.stack([x, y, z], axis=1)

    kuhn = _kuhn()
    hi, hj, hk = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    hi, hj, hk = hi.ravel(), hj.ravel(), hk.ravel()
    ci = hi[:, None, None] + (kuhn[None] & 1)
    cj = hj[:, None, None] + ((kuhn[None] >> 1) & 1)
    ck = hk[:, None, None] + ((kuhn[None] >> 2) & 1)
    conn = ((ci * (ny + 1) + cj) * (nz + 1) + ck).reshape(-1, 4).astype(np.int32)

    def face_flag(node):
        kk = node % (nz + 1)
        jj = (node // (nz + 1)) % (ny + 1)
        ii = node // ((nz + 1) * (ny + 1))
        return ((ii == 0) * 1 | (ii == nx) * 2 | (jj == 0) * 4 | (jj == ny) * 8 |
                (kk == 0) * 16 | (kk == nz) * 32)

    fl = face_flag(conn.astype(np.int64))
    tri = conn[:, _FACET]                                   # [nelem, 4, 3]
    common = fl[:, _FACET[:, 0]] & fl[:, _FACET[:, 1]] & fl[:, _FACET[:, 2]]
    e, f = np.nonzero(common)                               # ascending (element, facet)
    segment = tri[e, f].astype(np.int32)
    segflag = common[e, f].astype(np.int32)
    return coord, conn, segment, segflag


def markers_layered(coord, conn, nmat, mpe, zlength, layer_mattypes, layer_depths, seed):
    """Marker counts per element: mpe markers at seeded barycentric points,
    each taking the material of its depth layer (markerset.cxx:328-341)."""
    nelem = conn.shape[0]
    em = np.zeros((nelem, nmat), np.int32)
    nl = len(layer_mattypes)
    if nl == 1:
        em[:, layer_mattypes[0]] = mpe
        return em
    e = np.arange(nelem, dtype=np.uint64)
    zc = coord[conn, 2]                                      # [nelem, 4]
    for q in range(mpe):
        u = np.stack([u01(seed, 2, _M(4 * mpe) * e + _M(4 * q + r)) for r in range(3)], axis=1)
        u.sort(axis=1)
        eta = [u[:, 0], u[:, 1] - u[:, 0], u[:, 2] - u[:, 1], 1 - u[:, 2]]
        z = np.zeros(nelem)
        for v in range(4):
            z = z + zc[:, v] * eta[v]
        mt = np.full(nelem, layer_mattypes[nl - 1])
        done = np.zeros(nelem, bool)
        for layer in range(nl - 1):
            hit = ~done & (z >= -zlength * layer_depths[layer])
            mt[hit] = layer_mattypes[layer]
            done |= hit
        np.add.at(em, (np.arange(nelem), mt), 1)
    return em


def temperature_linear(coord, zlength, t_top, t_bottom, sigma, seed):
    """Kelvin; linear in depth plus, when sigma > 0, an Irwin-Hall N(0, sigma)."""
    z = coord[:, 2]
    t = t_top + (t_bottom - t_top) * (-z / zlength)
    if sigma > 0:
        n = np.arange(coord.shape[0], dtype=np.uint64)
        g = np.full(coord.shape[0], -6.0)
        for r in range(12):
            g = g + u01(seed, 3, _M(12) * n + _M(r))
        t = t + sigma * g
    return np.where(z >= 0, t_top, t)


class Mesh:
    """The same fields and view() as the product's workload.Mesh."""

    def __init__(self, cfg):
        self.coord, self.connectivity, self.segment, self.segflag = box(
            cfg.nx, cfg.ny, cfg.nz, cfg.xlength, cfg.ylength, cfg.zlength, cfg.jitter, cfg.mesh_seed)
        shear = cfg.extra.get("shear_xz", 0.0)
        if shear:
            self.coord[:, 0] += shear * self.coord[:, 2]
            self.segflag[self.segflag == 1] = 1 << 6
            self.segflag[self.segflag == 2] = 1 << 7
        self.nnode, self.nelem, self.nseg = len(self.coord), len(self.connectivity), len(self.segment)
        self.nmat = cfg.nlayers
        depths = list(cfg.layer_depths) if cfg.nlayers > 1 else [0.0]
        self.elemmarkers = markers_layered(self.coord, self.connectivity, self.nmat, 4, cfg.zlength,
                                           list(range(cfg.nlayers)), depths, cfg.mesh_seed + 1)

    def view(self):
        v = abi.MeshView()
        v.nnode, v.nelem, v.nseg, v.nmat = self.nnode, self.nelem, self.nseg, self.nmat
        v.connectivity = abi.iptr(self.connectivity)
        v.segment = abi.iptr(self.segment)
        v.segflag = abi.iptr(self.segflag)
        v.elemmarkers = abi.iptr(self.elemmarkers)
        self._v = v
        return v


def initial_inputs(cfg, mesh):
    """Initial temperature (K) and plastic strain (the weak-seed row of hexes
    along y at mid x and mid depth carries pls1 = 0.1)."""
    T = temperature_linear(mesh.coord, cfg.zlength, 273.0, 273.0 + cfg.t_bottom_c, cfg.t_sigma,
                           cfg.t_seed)
    pls = np.zeros(mesh.nelem)
    if cfg.weak_seed_row:
        i, k = cfg.nx // 2, cfg.nz // 2
        hexes = (i * cfg.ny + np.arange(cfg.ny)) * cfg.nz + k
        pls[(6 * hexes[:, None] + np.arange(6)[None, :]).ravel()] = 0.1
    return T, pls


def setup_case(cfg):
    """Mesh, params (boundary normals from the oracle), T, plastic strain and
    the PortOracle holding the topology, built without the product library."""
    from des_gb300 import workload as W          # pure Python: configs and params
    from oracle.oracle import PortOracle
    mesh = Mesh(cfg)
    T, pls = initial_inputs(cfg, mesh)
    p = W.make_params(cfg)
    o = PortOracle(mesh, p)
    o.boundary_normals(mesh.coord, p)
    o.set_params(p)
    return mesh, p, T, pls, o
