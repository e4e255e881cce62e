"""The benchmark workloads as seeded synthetic inputs.

Configs (sizes, physics, steps, seeds):
  1  20x20x4 hexes x6   =     9,600 tets, elasto-plastic, 2,000 steps (CPU-runnable)
  2  200x200x40 x6      = 9,600,000 tets, as 1 plus a weak-seed element row
  3  150x150x40 x6      = 5,400,000 tets, elasto-visco-plastic + diffusion, T noise
  4  config-2 mesh with config-3 rheology (the learned-closure case)
  5  400x400x80 x6      = 76,800,000 tets, 3 material layers
  "tiny" 4x3x2 x6 = 144 tets with the config-2 physics (golden fixtures)
  "yield" the config-2 mesh with a weak elasto-plastic material (cohesion
        4 -> 1 MPa, friction 30 -> 15 deg, dilation 0 -> 5 deg over plastic
        strain 0 -> 0.01), inertial scaling 100 and visc_min 1e22: yielding
        spreads from the weak-seed row (1-4% of the elements return each step
        over the first 100 steps at 200x200x40, about half of them on a
        24x24x8 box), the workload of the learned closure (configs 1-3 do not
        yield within 2,000 steps)

Parameters not named by a config keep the reference defaults of input.cxx:15-456;
the two defaults that would put quadratic host loops in the step
(has_water_loading, has_winkler_foundation) are switched off, which also keeps
the bottom free-slip (input.cxx:589-592 would otherwise force vbc_z0 = 0).
Temperatures are in Kelvin (input.cxx:234).
"""
import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import abi

YEAR2SEC = 365.2422 * 86400.0


def find_max_vbc(types, values):
    """bc.cxx:62-87"""
    m = 0.0
    for t, v in zip(types, values):
        if t % 2 == 1:
            m = max(m, abs(v))
    return m


@dataclass
class Config:
    name: str
    nx: int
    ny: int
    nz: int
    xlength: float = 100e3
    ylength: float = 100e3
    zlength: float = 10e3
    jitter: float = 0.05
    mesh_seed: int = 20260101
    rheology: str = "ep"          # ep | evp
    t_bottom_c: float = 600.0     # degC at z = -zlength
    t_sigma: float = 0.0
    t_seed: int = 0
    weak_seed_row: bool = False
    nlayers: int = 1
    layer_rho0: tuple = (3000.0,)
    layer_depths: tuple = ()
    steps: int = 2000
    extra: dict = field(default_factory=dict)

    @property
    def nelem(self):
        return 6 * self.nx * self.ny * self.nz

    @property
    def nnode(self):
        return (self.nx + 1) * (self.ny + 1) * (self.nz + 1)


CONFIGS = {
    "1": Config("config1_ep_20x20x4", 20, 20, 4, mesh_seed=20260101),
    "2": Config("config2_ep_200x200x40", 200, 200, 40, mesh_seed=20260102, weak_seed_row=True),
    "3": Config("config3_evp_150x150x40", 150, 150, 40, mesh_seed=20260103, rheology="evp",
                t_bottom_c=1330.0, t_sigma=20.0, t_seed=20260203, steps=5000),
    "4": Config("config4_evp_200x200x40", 200, 200, 40, mesh_seed=20260102, rheology="evp",
                t_bottom_c=1330.0, t_sigma=20.0, t_seed=20260203, weak_seed_row=True),
    "5": Config("config5_evp3_400x400x80", 400, 400, 80, mesh_seed=20260105, rheology="evp",
                t_bottom_c=1330.0, t_sigma=20.0, t_seed=20260205, nlayers=3,
                layer_rho0=(2800.0, 3000.0, 3300.0), layer_depths=(0.3, 0.6), steps=1000),
    "tiny": Config("tiny_ep_4x3x2", 4, 3, 2, mesh_seed=7, weak_seed_row=True, steps=50),
    "yield": Config("yield_ep_200x200x40", 200, 200, 40, mesh_seed=20260106, weak_seed_row=True,
                    extra=dict(mats=dict(cohesion0=[4e6], cohesion1=[1e6], friction_angle1=[15.0],
                                         dilation_angle1=[5.0], pls1=[0.01]),
                               params=dict(inertial_scaling=100.0, visc_min=1e22))),
}


def scaled(base, nx, ny, nz, name=None):
    """Same physics as `base` on another box size."""
    d = dict(base.__dict__)
    d.update(nx=nx, ny=ny, nz=nz, name=name or f"{base.name}_{nx}x{ny}x{nz}")
    return Config(**d)


def _mv(values):
    m = abi.MatVec()
    m.len = len(values)
    for i, v in enumerate(values):
        m.v[i] = v
    return m


def make_params(cfg, precision=abi.PREC_FP64):
    p = abi.Params()
    p.gravity = 10.0
    p.inertial_scaling = 1e5
    p.dt_fraction = 1.0
    p.fixed_dt = 0.0
    p.damping_factor = 0.8
    p.damping_option = 1
    p.ref_pressure_option = 0
    p.surface_process_option = 0
    p.is_quasi_static = 1
    p.has_thermal_diffusion = 1
    p.surface_temperature = 273.0
    p.winkler_delta_rho = 0.0
    p.elastic_foundation_constant = 1e11
    p.has_winkler_foundation = 0
    p.has_elastic_foundation = 0
    p.has_water_loading = 0
    p.zlength = cfg.zlength
    p.rheol_type = abi.RH_EP if cfg.rheology == "ep" else abi.RH_EVP
    p.nmat = cfg.nlayers
    p.is_plane_strain = 0
    p.visc_min = 1e18
    p.visc_max = 1e24
    p.tension_max = 1e9
    p.therm_diff_max = 5e-6
    mats = dict(rho0=list(cfg.layer_rho0), alpha=[3e-5], bulk_modulus=[128e9],
                shear_modulus=[30e9], visc_exponent=[3.05], visc_coefficient=[1.25e-1],
                visc_activation_energy=[3.76e5], heat_capacity=[1000.0], therm_cond=[3.0],
                pls0=[0.0], pls1=[0.1], cohesion0=[44e6], cohesion1=[4e6],
                friction_angle0=[30.0], friction_angle1=[30.0], dilation_angle0=[0.0],
                dilation_angle1=[0.0])
    if cfg.rheology == "evp":
        mats.update(visc_exponent=[3.5], visc_coefficient=[7e4], visc_activation_energy=[5.3e5],
                    therm_cond=[3.3], heat_capacity=[1000.0])
    mats.update(cfg.extra.get("mats", {}))
    for n in abi.MATVEC_NAMES:
        setattr(p, n, _mv(mats[n]))
    types = [1, 1, 1, 1, 1, 0, 1, 1, 1, 1]           # x0 x1 y0 y1 z0 z1 n0..n3
    vals = [-0.01 / YEAR2SEC, 0.01 / YEAR2SEC] + [0.0] * 8
    types = cfg.extra.get("vbc_types", types)
    vals = cfg.extra.get("vbc_values", vals)
    for i in range(abi.DES_NBDRY):
        p.vbc_types[i] = types[i]
        p.vbc_values[i] = vals[i]
    p.max_vbc_val = find_max_vbc(types, vals)
    for k, v in cfg.extra.get("params", {}).items():
        setattr(p, k, v)
    # Variables::compensation_pressure as init() sets it (ic.cxx:131,
    # ref_pressure of the bottom), for a device given a state without init
    p.compensation_pressure = p.rho0.v[0] * p.gravity * p.zlength if p.gravity != 0 else 0.0
    p.precision = precision
    return p


class Mesh:
    """Box mesh + per-element marker counts, as numpy arrays."""

    def __init__(self, cfg, lib):
        spec = abi.BoxSpec(cfg.nx, cfg.ny, cfg.nz, cfg.xlength, cfg.ylength, cfg.zlength,
                           cfg.jitter, cfg.mesh_seed)
        nn, ne, ns = C.c_int(), C.c_int(), C.c_int()
        abi.check(lib.des_box_sizes(C.byref(spec), C.byref(nn), C.byref(ne), C.byref(ns)),
                  "des_box_sizes")
        self.nnode, self.nelem, self.nseg = nn.value, ne.value, ns.value
        self.coord = np.zeros((self.nnode, 3))
        self.connectivity = np.zeros((self.nelem, 4), np.int32)
        self.segment = np.zeros((self.nseg, 3), np.int32)
        self.segflag = np.zeros(self.nseg, np.int32)
        abi.check(lib.des_box_fill(C.byref(spec), abi.dptr(self.coord), abi.iptr(self.connectivity),
                                   abi.iptr(self.segment), abi.iptr(self.segflag)), "des_box_fill")
        # inclined x sides: the box sheared in x along z, its x faces flagged as
        # the inclined boundaries n0 and n1 (bcflag bits 6 and 7)
        shear = cfg.extra.get("shear_xz", 0.0)
        if shear:
            self.coord[:, 0] += shear * self.coord[:, 2]
            self.segflag[self.segflag == 1] = 1 << 6
            self.segflag[self.segflag == 2] = 1 << 7
        self.nmat = cfg.nlayers
        self.elemmarkers = np.zeros((self.nelem, self.nmat), np.int32)
        mattypes = np.arange(cfg.nlayers, dtype=np.int32)
        depths = np.array(cfg.layer_depths if cfg.nlayers > 1 else [0.0], np.float64)
        abi.check(lib.des_markers_layered(self.nelem, self.nmat, abi.dptr(self.coord),
                                          abi.iptr(self.connectivity), 4, C.c_double(cfg.zlength),
                                          cfg.nlayers, abi.iptr(mattypes), abi.dptr(depths),
                                          C.c_ulonglong(cfg.mesh_seed + 1),
                                          abi.iptr(self.elemmarkers)), "des_markers_layered")

    def view(self):
        v = abi.MeshView()
        v.nnode, v.nelem, v.nseg, v.nmat = self.nnode, self.nelem, self.nseg, self.nmat
        v.connectivity = abi.iptr(self.connectivity)
        v.segment = abi.iptr(self.segment)
        v.segflag = abi.iptr(self.segflag)
        v.elemmarkers = abi.iptr(self.elemmarkers)
        self._v = v
        return v


def initial_inputs(cfg, mesh, lib):
    """Injected initial fields: temperature (K) and plastic strain."""
    T = np.zeros(mesh.nnode)
    abi.check(lib.des_temperature_linear(mesh.nnode, abi.dptr(mesh.coord), C.c_double(cfg.zlength),
                                         C.c_double(273.0), C.c_double(273.0 + cfg.t_bottom_c),
                                         C.c_double(cfg.t_sigma), C.c_ulonglong(cfg.t_seed),
                                         abi.dptr(T)), "des_temperature_linear")
    pls = np.zeros(mesh.nelem)
    if cfg.weak_seed_row:
        # one row of hexes along y at mid x and mid depth, fully weakened
        # (plstrain = pls1, so plastic_weakening gives cohesion1 = 4 MPa)
        i, k = cfg.nx // 2, cfg.nz // 2
        hexes = (i * cfg.ny + np.arange(cfg.ny)) * cfg.nz + k
        elems = (6 * hexes[:, None] + np.arange(6)[None, :]).ravel()
        pls[elems] = 0.1
    return T, pls


def new_state(mesh, T, pls):
    s = abi.State(mesh.nnode, mesh.nelem)
    s.coord[:] = mesh.coord
    s.temperature[:] = T
    s.plstrain[:] = pls
    return s
