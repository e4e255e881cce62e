"""Shared set-up for the parity tests: workloads, loop-consistent states and
comparisons."""
import numpy as np

import des_gb300 as D
from des_gb300 import abi, workload as W
from oracle.oracle import PortOracle

# order of the reference loop body (dynearthsol.cxx:358-394); update_mesh is
# update_coordinate, volume swap, compute_volume, compute_mass, compute_shape_fn
LOOP = ["update_temperature", "update_strain_rate", "compute_dvoldt", "compute_edvoldt",
        "update_stress", "NMD_stress", "update_force", "update_velocity", "apply_vbcs",
        "update_mesh", "rotate_stress"]
MESH_PARTS = ["update_coordinate", "compute_volume", "compute_mass", "compute_shape_fn"]
COMPARED = ["coord", "vel", "force", "temperature", "mass", "tmass", "volume_n", "ntmp",
            "volume", "volume_old", "edvoldt", "plstrain", "delta_plstrain", "dpressure",
            "stress", "strain", "strain_rate", "shpdx", "shpdy", "shpdz"]


def plastic_config(nx=6, ny=5, nz=3):
    """A box that yields within tens of steps: low cohesion with friction and
    dilation weakening, small inertial scaling, and visc_min raised so that
    dt is not capped by dt_maxwell."""
    cfg = W.scaled(W.CONFIGS["tiny"], nx, ny, nz, name=f"plastic_{nx}x{ny}x{nz}")
    cfg.extra = dict(mats=dict(cohesion0=[4e6], cohesion1=[1e6], friction_angle1=[15.0],
                               dilation_angle1=[5.0], pls1=[0.01]),
                     params=dict(inertial_scaling=100.0, visc_min=1e22))
    return cfg


def evp_config(nx=6, ny=5, nz=3):
    cfg = W.scaled(W.CONFIGS["3"], nx, ny, nz, name=f"evp_{nx}x{ny}x{nz}")
    return cfg


def layered_config(nx=6, ny=5, nz=6):
    cfg = W.scaled(W.CONFIGS["5"], nx, ny, nz, name=f"layered_{nx}x{ny}x{nz}")
    return cfg


def _variant(name, nx=6, ny=5, nz=3, base="1", rheology=None, params=None, mats=None, vbc=None,
             shear_xz=0.0, **cfg_kw):
    cfg = W.scaled(W.CONFIGS[base], nx, ny, nz, name=f"opt_{name}_{nx}x{ny}x{nz}")
    if rheology:
        cfg.rheology = rheology
    for k, v in cfg_kw.items():
        setattr(cfg, k, v)
    extra = dict(cfg.extra)
    if params:
        extra["params"] = dict(extra.get("params", {}), **params)
    if mats:
        extra["mats"] = dict(extra.get("mats", {}), **mats)
    if vbc:
        extra["vbc_types"], extra["vbc_values"] = vbc
    if shear_xz:
        extra["shear_xz"] = shear_xz
    cfg.extra = extra
    return cfg


_YR = 365.2425 * 86400
# Options of the loop that the five workloads do not exercise (each on a small
# box of config 1's physics unless stated): the other rheologies, damping
# options, a fixed dt, the dynamic (not quasi-static) mode, no thermal
# diffusion, no gravity, the other velocity boundary types of the x, y and z
# sides (bc.cxx:182-500), the largest material count and a one-hex mesh.
OPTION_VARIANTS = {
    "elastic": _variant("elastic", params=dict(rheol_type=1)),
    # a viscosity the explicit step can carry (eta / dt near the shear modulus)
    "viscous": _variant("viscous", base="3", params=dict(rheol_type=2, visc_min=1e17, visc_max=3e17)),
    "maxwell": _variant("maxwell", base="3", params=dict(rheol_type=3)),
    "damping0": _variant("damping0", params=dict(damping_option=0)),
    "damping2": _variant("damping2", params=dict(damping_option=2)),
    "damping3": _variant("damping3", params=dict(damping_option=3)),
    "fixed_dt": _variant("fixed_dt", params=dict(fixed_dt=1e7)),
    "dynamic": _variant("dynamic", params=dict(is_quasi_static=0)),
    "no_thermal": _variant("no_thermal", params=dict(has_thermal_diffusion=0)),
    "no_gravity": _variant("no_gravity", params=dict(gravity=0.0)),
    "vbc_a": _variant("vbc_a", vbc=([3, 5, 2, 4, 1, 0, 0, 0, 0, 0],
                                    [-0.01 / _YR, 0.02 / _YR, 0.0, 0.005 / _YR, 0.0, 0.0, 0, 0, 0, 0])),
    "vbc_b": _variant("vbc_b", vbc=([7, 7, 7, 3, 3, 2, 0, 0, 0, 0],
                                    [-0.01 / _YR, 0.01 / _YR, 0.003 / _YR, -0.002 / _YR, 0.0, 0.0, 0, 0, 0, 0])),
    # apply_stress_bcs (bc.cxx:503-595): lithostatic tractions on sides whose
    # normal velocity is free, the Winkler foundation under a free bottom, water
    # loading on the surface, the elastic foundation
    "free_x0": _variant("free_x0", vbc=([0, 1, 1, 1, 1, 0, 0, 0, 0, 0],
                                        [0.0, 0.01 / _YR, 0.0, 0.0, 0.0, 0.0, 0, 0, 0, 0])),
    "winkler": _variant("winkler", params=dict(has_winkler_foundation=1, winkler_delta_rho=100.0),
                        vbc=([1, 1, 1, 1, 0, 0, 0, 0, 0, 0],
                             [-0.01 / _YR, 0.01 / _YR, 0.0, 0.0, 0.0, 0.0, 0, 0, 0, 0])),
    "water": _variant("water", params=dict(has_water_loading=1)),
    # (cohesion high enough that nothing yields: the reference's fast-math
    # eigen-solver and the strict restatement differ by rounding on returns)
    "elastic_fnd": _variant("elastic_fnd", params=dict(has_elastic_foundation=1,
                                                        elastic_foundation_constant=1e11),
                            mats=dict(cohesion0=[1e9], cohesion1=[1e9]),
                            vbc=([1, 1, 1, 1, 2, 0, 0, 0, 0, 0],
                                 [-0.01 / _YR, 0.01 / _YR, 0.0, 0.0, 0.0, 0.0, 0, 0, 0, 0])),
    # surface processes inside update_mesh (bc.cxx:760-782): diffusion of the
    # top surface, and the custom-rule template
    "surface": _variant("surface", params=dict(surface_process_option=1, surface_diffusivity=1.0)),
    "surface_custom": _variant("surface_custom", params=dict(surface_process_option=101)),
    # PREM reference pressure (matprops.cxx:20-108, 523-535) in the initial
    # stress, the compensation pressure and the tractions of a free side wall
    "prem": _variant("prem", params=dict(ref_pressure_option=1),
                     vbc=([0, 1, 1, 1, 1, 0, 0, 0, 0, 0], [0.0, 0.01 / _YR, 0.0, 0.0, 0.0, 0.0, 0, 0, 0, 0])),
    "prem_crust": _variant("prem_crust", nlayers=3, layer_rho0=(2800.0, 3000.0, 3300.0),
                           layer_depths=(0.3, 0.6), params=dict(ref_pressure_option=2),
                           mats=dict(bulk_modulus=[100e9, 128e9, 150e9]),
                           vbc=([0, 1, 1, 1, 1, 0, 0, 0, 0, 0], [0.0, 0.01 / _YR, 0.0, 0.0, 0.0, 0.0, 0, 0, 0, 0])),
    # inclined sides n0, n1 (the box sheared, its x faces flagged inclined):
    # normal velocity (type 1, with the edge rule where they meet y and z
    # sides), velocity along the normal (3), horizontal normal velocity (11),
    # horizontal velocity along the normal (13)
    "inclined_1": _variant("inclined_1", shear_xz=0.3, vbc=([0, 0, 1, 1, 1, 0, 1, 1, 0, 0],
                                              [0.0, 0.0, 0.0, 0.0, 0.0, 0.0, -0.01 / _YR, 0.01 / _YR, 0, 0])),
    "inclined_3_11": _variant("inclined_3_11", shear_xz=0.3, vbc=([0, 0, 1, 1, 1, 0, 3, 11, 0, 0],
                                                    [0.0, 0.0, 0.0, 0.0, 0.0, 0.0, -0.01 / _YR, 0.01 / _YR, 0, 0])),
    "inclined_13": _variant("inclined_13", shear_xz=0.3, vbc=([0, 0, 1, 1, 1, 0, 13, 1, 0, 0],
                                                [0.0, 0.0, 0.0, 0.0, 0.0, 0.0, -0.01 / _YR, 0.01 / _YR, 0, 0])),
    "mats16": _variant("mats16", nz=6, nlayers=16,
                       layer_rho0=tuple(2700.0 + 40.0 * k for k in range(16)),
                       layer_depths=tuple((k + 1) / 16 for k in range(15)),
                       mats=dict(shear_modulus=[25e9 + 1e9 * k for k in range(16)],
                                 bulk_modulus=[100e9 + 3e9 * k for k in range(16)],
                                 therm_cond=[2.5 + 0.1 * k for k in range(16)],
                                 cohesion0=[30e6 + 2e6 * k for k in range(16)])),
    "one_hex": _variant("one_hex", nx=1, ny=1, nz=1),
}
# variants whose arithmetic includes pow/exp (CUDA's differ from the host
# libm by an ulp): a per-step tolerance instead of bit-identity
OPTION_TRANSCENDENTAL = {"viscous", "maxwell"}


def phase_config(nx=8, ny=6, nz=6):
    """Three layers whose materials differ in density, moduli, conductivity,
    heat capacity and cohesion, so a phase change moves every mixed property;
    elasto-plastic (no viscosity, whose pow/exp differ from the host's libm by
    an ulp), so the FP64 form stays bit-identical."""
    cfg = W.scaled(W.CONFIGS["5"], nx, ny, nz, name=f"phase_{nx}x{ny}x{nz}")
    cfg.rheology = "ep"
    cfg.extra = dict(mats=dict(shear_modulus=[30e9, 25e9, 40e9], bulk_modulus=[128e9, 100e9, 150e9],
                               therm_cond=[3.3, 2.5, 4.0], heat_capacity=[1000.0, 900.0, 1200.0],
                               cohesion0=[44e6, 30e6, 60e6]))
    return cfg


def phase_change(mesh, state, em):
    """A deterministic stand-in for a PhaseChange rule (phasechanges.cxx:
    232-258 moves one marker's count from its old to its new material): in
    the hotter half of the elements holding material 0, one marker of
    material 0 becomes material 2; in the deeper half of those holding
    material 1, one marker of material 1 becomes material 0."""
    conn = mesh.connectivity
    T = state.temperature[conn].mean(axis=1)
    z = state.coord[conn, 2].mean(axis=1)
    em = em.copy()
    c0, c1 = em[:, 0] > 0, em[:, 1] > 0
    hot = c0 & (T > np.median(T[c0])) if c0.any() else c0
    deep = c1 & (z < np.median(z[c1])) if c1.any() else c1
    em[hot, 0] -= 1
    em[hot, 2] += 1
    em[deep, 1] -= 1
    em[deep, 0] += 1
    return em


def remesh_standin(mesh, state, elemmarkers, cfg):
    """A stand-in for the host half of remesh (remeshing.cxx:1970-2013, TetGen
    and the interpolations): a new box mesh of cfg's resolution; node fields
    from the nearest old node, element fields and marker counts from the
    element with the nearest centroid.  Returns the new mesh and its fields."""
    from scipy.spatial import cKDTree
    new = W.Mesh(cfg, D.lib())
    s = abi.State(new.nnode, new.nelem)
    s.coord[:] = new.coord
    jn = cKDTree(state.coord).query(new.coord)[1]
    for f in ("vel", "temperature", "coord0"):
        getattr(s, f)[:] = getattr(state, f)[jn]
    old_c = state.coord[mesh.connectivity].mean(axis=1)
    new_c = new.coord[new.connectivity].mean(axis=1)
    je = cKDTree(old_c).query(new_c)[1]
    for f in ("plstrain", "delta_plstrain", "strain", "stress"):
        getattr(s, f)[:] = getattr(state, f)[je]
    new.elemmarkers[:] = elemmarkers[je]
    s.time, s.dt, s.steps = state.time, state.dt, state.steps
    return new, s


def post_remesh(oracle, s, zlength, reset_bottom_coord0):
    """What remesh does after reallocate_variables (remeshing.cxx:2037-2054),
    through the oracle's functions."""
    oracle.call("compute_volume", s)
    s.volume_old[:] = s.volume
    oracle.call("compute_mass", s)
    oracle.call("compute_shape_fn", s)
    if reset_bottom_coord0:
        s.coord0[(oracle.bcflag() & 16) != 0, 2] = -zlength


class Case:
    def __init__(self, cfg):
        self.cfg = cfg
        self.mesh, self.params, self.T, self.pls, self.topo = D.setup_case(cfg)
        self.oracle = PortOracle(self.mesh, self.params)

    def initial_state(self):
        s = W.new_state(self.mesh, self.T, self.pls)
        self.oracle.init_fields(s)
        return s

    def state_after(self, nsteps):
        s = self.initial_state()
        if nsteps:
            self.oracle.step(s, nsteps)
        return s

    def state_before(self, fn, nsteps):
        """Oracle state after nsteps full steps and then the loop functions
        that precede fn in the next step."""
        s = self.state_after(nsteps)
        s.steps += 1
        s.time += s.dt
        for f in LOOP:
            if f == fn:
                return s
            if f == "update_mesh" and fn in MESH_PARTS:
                for g in MESH_PARTS:
                    if g == fn:
                        return s
                    if g == "compute_volume":
                        s.volume_old[:] = s.volume
                    self.oracle.call(g, s)
                return s
            if f == "update_temperature" and not self.params.has_thermal_diffusion:
                continue
            self.oracle.call(f, s)
        if fn == "compute_dt":
            return s
        raise KeyError(fn)

    def device(self):
        return D.Device(self.mesh, self.params, device=0)


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def diff_fields(a, b, fields=COMPARED):
    return [f for f in fields if not np.array_equal(getattr(a, f), getattr(b, f))]
