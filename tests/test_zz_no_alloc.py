"""des_compute_dt_noalloc against the handle's des_gpu_compute_dt.

The no-alloc entry point serves callers that cannot let a library call
cudaMalloc: they own all device memory (their own pool or budget), or must
not trigger the device-wide synchronisation cudaMalloc/cudaFree can cause.
It takes device arrays the caller already holds and keeps its scratch in a
fixed array inside the library.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

import des_gb300 as D
from des_gb300 import abi, workload as W
from helpers import Case

MAX_ELEMS = 256 * 65536


def dt_inputs(p):
    return abi.DtInputs(visc_min=p.visc_min, therm_diff_max=p.therm_diff_max,
                        max_vbc_val=p.max_vbc_val, inertial_scaling=p.inertial_scaling,
                        dt_fraction=p.dt_fraction, fixed_dt=p.fixed_dt,
                        shear_modulus=p.shear_modulus.v[0], bulkm0=p.bulk_modulus.v[0],
                        rho0=p.rho0.v[0], is_quasi_static=p.is_quasi_static,
                        has_thermal_diffusion=p.has_thermal_diffusion)


@pytest.mark.gpu
def test_noalloc_dt_equals_handle_dt_on_two_calls_in_a_row(gpu):
    torch = pytest.importorskip("torch")
    L = D.lib()
    c = Case(W.CONFIGS["1"])
    inp = dt_inputs(c.params)
    conn = torch.from_numpy(c.mesh.connectivity).cuda()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for nsteps in (3, 17):          # two consecutive calls on different states
        s = c.state_after(nsteps)
        dev = c.device()
        dev.upload(s, abi.F_ALL)
        want = dev.call("compute_dt")   # existing entry point (des_gpu_compute_dt)
        dev.close()
        coord = torch.from_numpy(s.coord).cuda()
        vol = torch.from_numpy(s.volume).cuda()
        out.fill_(-1.0)
        torch.cuda.synchronize()
        rc = L.des_compute_dt_noalloc(c.mesh.nelem, coord.data_ptr(), conn.data_ptr(),
                                      vol.data_ptr(), None, C.byref(inp), out.data_ptr(), None)
        assert rc == abi.DES_OK
        torch.cuda.synchronize()
        got = float(out.item())
        assert got == want, (nsteps, got, want)
        assert got == c.oracle.call("compute_dt", s.copy())


@pytest.mark.gpu
def test_noalloc_rejects_sizes_above_its_limit(gpu):
    L = D.lib()
    inp = abi.DtInputs(max_vbc_val=1.0, dt_fraction=1.0, shear_modulus=1.0, visc_min=1.0,
                       therm_diff_max=1.0, inertial_scaling=1.0, is_quasi_static=1)
    dummy = C.c_double()
    big = (C.c_int * 4)()
    rc = L.des_compute_dt_noalloc(MAX_ELEMS + 1, C.addressof(dummy), C.addressof(big),
                                  C.addressof(dummy), None, C.byref(inp), C.addressof(dummy), None)
    assert rc == abi.DES_ERR_SIZE
