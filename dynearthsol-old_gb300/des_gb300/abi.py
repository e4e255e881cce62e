"""ctypes mirror of include/des_gpu.h and include/des_workload.h.

The structs here must match the C headers field for field; tests/test_abi.py
checks the sizes against the compiled library.
"""
import ctypes as C

import numpy as np

DES_MAX_MAT = 16
DES_NBDRY = 10

DES_OK = 0
DES_ERR_OPTION = 1
DES_ERR_ARG = 2
DES_ERR_CUDA = 3
DES_ERR_NOMEM = 4
DES_ERR_UNSUPPORTED = 5
DES_ERR_SIZE = 6
DES_ERR_DT = 11
DES_ERR_TOPOLOGY = 12

DES_STATUS_DT_NONPOSITIVE = 0x1
DES_STATUS_NONFINITE = 0x2
DES_STATUS_NEG_VOLUME = 0x4
DES_STATUS_QL_NOCONV = 0x8

RH_ELASTIC, RH_VISCOUS, RH_PLASTIC = 1, 2, 4
RH_MAXWELL, RH_EP, RH_EVP = 3, 5, 7

PREC_FP64, PREC_FP32 = 0, 1

F_COORD = 1 << 0
F_VEL = 1 << 1
F_FORCE = 1 << 2
F_TEMPERATURE = 1 << 3
F_MASS = 1 << 4
F_NTMP = 1 << 5
F_VOLUME = 1 << 6
F_STRESS = 1 << 7
F_STRAIN = 1 << 8
F_STRAIN_RATE = 1 << 9
F_PLSTRAIN = 1 << 10
F_DPRESSURE = 1 << 11
F_EDVOLDT = 1 << 12
F_SHAPE = 1 << 13
F_TMP_RESULT = 1 << 14
F_SCALARS = 1 << 15
F_COORD0 = 1 << 16
F_ALL = 0x1FFFF
F_STEP_STATE = (F_COORD | F_VEL | F_FORCE | F_TEMPERATURE | F_MASS | F_NTMP | F_VOLUME |
                F_STRESS | F_STRAIN | F_STRAIN_RATE | F_PLSTRAIN | F_DPRESSURE | F_EDVOLDT |
                F_SHAPE | F_SCALARS)

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_up = C.POINTER(C.c_uint)


class MatVec(C.Structure):
    _fields_ = [("len", C.c_int), ("v", C.c_double * DES_MAX_MAT)]


MATVEC_NAMES = ["rho0", "alpha", "bulk_modulus", "shear_modulus", "visc_exponent",
                "visc_coefficient", "visc_activation_energy", "heat_capacity", "therm_cond",
                "pls0", "pls1", "cohesion0", "cohesion1", "friction_angle0", "friction_angle1",
                "dilation_angle0", "dilation_angle1"]


class Params(C.Structure):
    _fields_ = [
        ("gravity", C.c_double), ("inertial_scaling", C.c_double), ("dt_fraction", C.c_double),
        ("fixed_dt", C.c_double), ("damping_factor", C.c_double),
        ("surface_diffusivity", C.c_double), ("damping_option", C.c_int), ("ref_pressure_option", C.c_int),
        ("surface_process_option", C.c_int), ("is_quasi_static", C.c_int),
        ("has_thermal_diffusion", C.c_int),
        ("surface_temperature", C.c_double), ("winkler_delta_rho", C.c_double),
        ("elastic_foundation_constant", C.c_double),
        ("has_winkler_foundation", C.c_int), ("has_elastic_foundation", C.c_int),
        ("has_water_loading", C.c_int),
        ("zlength", C.c_double),
        ("rheol_type", C.c_int), ("nmat", C.c_int), ("is_plane_strain", C.c_int),
        ("visc_min", C.c_double), ("visc_max", C.c_double), ("tension_max", C.c_double),
        ("therm_diff_max", C.c_double),
    ] + [(n, MatVec) for n in MATVEC_NAMES] + [
        ("vbc_types", C.c_int * DES_NBDRY), ("vbc_values", C.c_double * DES_NBDRY),
        ("max_vbc_val", C.c_double), ("compensation_pressure", C.c_double),
        ("bnormals", (C.c_double * 3) * DES_NBDRY),
        ("edge_vectors", ((C.c_double * 3) * DES_NBDRY) * DES_NBDRY),
        ("precision", C.c_int),
    ]


class MeshView(C.Structure):
    _fields_ = [("nnode", C.c_int), ("nelem", C.c_int), ("nseg", C.c_int), ("nmat", C.c_int),
                ("connectivity", _ip), ("segment", _ip), ("segflag", _ip), ("elemmarkers", _ip)]


STATE_NODE3 = ["coord", "vel", "force", "coord0"]
STATE_NODE1 = ["temperature", "mass", "tmass", "volume_n", "ntmp"]
STATE_ELEM1 = ["volume", "volume_old", "edvoldt", "plstrain", "delta_plstrain", "dpressure",
               "tmp_result_sg"]
STATE_ELEM6 = ["stress", "strain", "strain_rate"]
STATE_ELEM4 = ["shpdx", "shpdy", "shpdz"]


class StateView(C.Structure):
    _fields_ = ([("nnode", C.c_int), ("nelem", C.c_int)] +
                [(n, _dp) for n in ["coord", "vel", "force", "coord0",
                                    "temperature", "mass", "tmass", "volume_n", "ntmp",
                                    "volume", "volume_old", "edvoldt",
                                    "plstrain", "delta_plstrain", "dpressure", "tmp_result_sg",
                                    "stress", "strain", "strain_rate",
                                    "shpdx", "shpdy", "shpdz", "tmp_result"]] +
                [("time", C.c_double), ("dt", C.c_double), ("steps", C.c_int)])


class Topology(C.Structure):
    _fields_ = [("nnode", C.c_int), ("nelem", C.c_int), ("bcflag", _up),
                ("support_offsets", _ip), ("support_elems", _ip), ("support_slots", _ip),
                ("bnodes_count", C.c_int * DES_NBDRY), ("bnodes", _ip * DES_NBDRY),
                ("bfacets_count", C.c_int * DES_NBDRY), ("bfacets", _ip * DES_NBDRY)]


class StepReport(C.Structure):
    _fields_ = [("steps", C.c_int), ("time", C.c_double), ("dt", C.c_double),
                ("status", C.c_uint), ("ql_fallbacks", C.c_longlong),
                ("eigen_solves", C.c_longlong), ("closure_candidates", C.c_longlong),
                ("closure_accepted", C.c_longlong), ("exact_returns", C.c_longlong)]


class MarkerSet(C.Structure):
    """des_marker_set: one marker set as the output files hold it."""
    _fields_ = [("name", C.c_char_p), ("nmarkers", C.c_int), ("last_id", C.c_int),
                ("eta", _dp), ("elem", _ip), ("mattype", _ip), ("id", _ip)]


class SaveAverages(C.Structure):
    """des_save_averages: the averaging state of Output::average_fields."""
    _fields_ = [("coord0", _dp), ("strain0", _dp), ("stress_sum", _dp), ("dpls_sum", _dp),
                ("time0", C.c_double), ("interval", C.c_int)]


class RemeshCheck(C.Structure):
    """des_remesh_check: the mesh.* parameters of bad_mesh_quality."""
    _fields_ = [("smallest_size", C.c_double), ("resolution", C.c_double), ("zlength", C.c_double),
                ("max_boundary_distortion", C.c_double), ("min_quality", C.c_double),
                ("remeshing_option", C.c_int)]


MLP_IN, MLP_HID, MLP_OUT = 16, 64, 8
RET_RECORD = 24      # floats per record of des_gpu_log_returns


class Mlp(C.Structure):
    """des_mlp: the learned closure's weights ([out][in]), normalisation,
    training envelope and acceptance tolerance."""
    _fields_ = [("w1", C.c_float * MLP_IN * MLP_HID), ("b1", C.c_float * MLP_HID),
                ("w2", C.c_float * MLP_HID * MLP_HID), ("b2", C.c_float * MLP_HID),
                ("w3", C.c_float * MLP_HID * MLP_OUT), ("b3", C.c_float * MLP_OUT),
                ("in_mean", C.c_float * MLP_IN), ("in_scale", C.c_float * MLP_IN),
                ("out_scale", C.c_float * MLP_OUT),
                ("env_lo", C.c_float * MLP_IN), ("env_hi", C.c_float * MLP_IN),
                ("tol", C.c_float)]

    def arr(self, name):
        """numpy view (float32) of one field."""
        return np.ctypeslib.as_array(getattr(self, name))


class DtInputs(C.Structure):
    _fields_ = [("visc_min", C.c_double), ("therm_diff_max", C.c_double),
                ("max_vbc_val", C.c_double), ("inertial_scaling", C.c_double),
                ("dt_fraction", C.c_double), ("fixed_dt", C.c_double),
                ("shear_modulus", C.c_double), ("bulkm0", C.c_double), ("rho0", C.c_double),
                ("is_quasi_static", C.c_int), ("has_thermal_diffusion", C.c_int)]


class BoxSpec(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("xlength", C.c_double), ("ylength", C.c_double), ("zlength", C.c_double),
                ("jitter", C.c_double), ("seed", C.c_ulonglong)]


def dptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def iptr(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


def uptr(a):
    assert a.dtype == np.uint32 and a.flags.c_contiguous
    return a.ctypes.data_as(_up)


class State:
    """Host copy of the Variables arrays of the loop, in the reference layout
    (Array2D rows of N components; parameters.hpp:270-280)."""

    def __init__(self, nnode, nelem):
        self.nnode, self.nelem = nnode, nelem
        for n in STATE_NODE3:
            setattr(self, n, np.zeros((nnode, 3)))
        for n in STATE_NODE1:
            setattr(self, n, np.zeros(nnode))
        for n in STATE_ELEM1:
            setattr(self, n, np.zeros(nelem))
        for n in STATE_ELEM6:
            setattr(self, n, np.zeros((nelem, 6)))
        for n in STATE_ELEM4:
            setattr(self, n, np.zeros((nelem, 4)))
        self.tmp_result = np.zeros((nelem, 12))
        self.time, self.dt, self.steps = 0.0, 0.0, 0
        self._view = None

    ARRAYS = STATE_NODE3 + STATE_NODE1 + STATE_ELEM1 + STATE_ELEM6 + STATE_ELEM4 + ["tmp_result"]

    def view(self):
        v = StateView()
        v.nnode, v.nelem = self.nnode, self.nelem
        for n in self.ARRAYS:
            setattr(v, n, dptr(getattr(self, n)))
        v.time, v.dt, v.steps = self.time, self.dt, self.steps
        self._view = v
        return v

    def sync_scalars(self, v=None):
        v = v or self._view
        self.time, self.dt, self.steps = v.time, v.dt, v.steps

    def copy(self):
        s = State(self.nnode, self.nelem)
        for n in self.ARRAYS:
            setattr(s, n, getattr(self, n).copy())
        s.time, s.dt, s.steps = self.time, self.dt, self.steps
        return s


def check(rc, what="call"):
    if rc != DES_OK:
        raise RuntimeError(f"{what} failed with code {rc}")
    return rc
