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
