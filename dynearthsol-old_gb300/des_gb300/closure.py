"""The learned return-map closure: training data, features and training.

Records come from Device.log_returns, the FP64 form's own shear returns
(rheology.cxx:180-240 reached from update_stress, :578-640).  Features and
targets are formed here as the FP32 stress pass forms them on the device
(csrc/des_closure.cuh); the network is trained on the GPU by des_mlp_train
(csrc/des_mlp.cu) and installed with Device.set_closure.
"""
import ctypes as C

import numpy as np

from . import abi

NIN, NOUT = 14, 7
USED_IN, USED_OUT = 4, 4     # quantities in and out that the closure uses (the rest are zero)
_FP = C.POINTER(C.c_float)


def _lib():
    from . import lib
    return lib()


def _ck(rc, what):
    from . import _ck as ck
    ck(rc, what)


def _fptr(a):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_FP)


def single_material(params):
    """(bulk modulus, shear modulus, largest pls1) of a one-material model."""
    if params.nmat != 1:
        raise ValueError("the closure is trained for one material")
    return (params.bulk_modulus.v[0], params.shear_modulus.v[0], params.pls1.v[0])


def _dev(a):
    d = a.copy()
    d[:, :3] -= a[:, :3].mean(axis=1, keepdims=True)
    return d


def _j2(d):
    return 0.5 * (d[:, :3] ** 2).sum(1) + (d[:, 3:] ** 2).sum(1)


def trial_stress(rec, bulkm, shearm):
    """Elastic trial s_old + C:de of each record (rheology.cxx:20-35)."""
    s = rec[:, 0:6].astype(np.float64)
    de = rec[:, 6:12].astype(np.float64)
    lam = bulkm - 2.0 / 3.0 * shearm
    t = s + 2.0 * shearm * de
    t[:, :3] += (lam * de[:, :3].sum(1))[:, None]
    return t


def _mat(a):
    M = np.zeros((len(a), 3, 3))
    for k, (i, j) in enumerate(((0, 0), (1, 1), (2, 2), (0, 1), (0, 2), (1, 2))):
        M[:, i, j] = M[:, j, i] = a[:, k]
    return M


def _inner(a, b):
    """Frobenius inner product of symmetric tensors in (xx yy zz xy xz yz)."""
    return (a[:, :3] * b[:, :3]).sum(1) + 2 * (a[:, 3:] * b[:, 3:]).sum(1)


def basis(trial):
    """The unit deviator n of each trial, dev(n n), the eigenvalues of n
    (ascending) and a mask of rows with a nonzero deviator."""
    d = _dev(trial)
    j2 = _j2(d)
    ok = j2 > 0
    n = d / np.sqrt(np.where(ok, j2, 1.0))[:, None]
    N = _mat(n)
    NN = N @ N
    q = _dev(np.stack([NN[:, 0, 0], NN[:, 1, 1], NN[:, 2, 2], NN[:, 0, 1], NN[:, 0, 2], NN[:, 1, 2]], 1))
    lam = np.zeros((len(trial), 3))
    lam[ok] = np.linalg.eigvalsh(N[ok])
    return n, q, lam, ok


def pole(lam):
    """(3 l_min^2 - 1)(3 l_max^2 - 1): zero where the least or the most
    compressive principal direction of the trial is not unique."""
    return (3 * lam[:, 0] ** 2 - 1) * (3 * lam[:, 2] ** 2 - 1)


def features(trial, T, pls, pls_sat):
    """The raw network inputs (padded to 16): the principal values of the
    unit trial deviator and the plastic strain capped at pls_sat.  The
    temperature T is part of the record but does not enter the shear return
    (it acts through the viscosity, outside the network), so it is not an
    input: a network that saw it would pick up the geotherm of its training
    box."""
    n, q, lam, ok = basis(trial)
    raw = np.zeros((len(trial), abi.MLP_IN))
    raw[:, 0:3] = lam
    raw[:, 3] = np.minimum(pls, pls_sat)
    return raw, ok


def targets(rec, trial, shearm):
    """Network targets from the logged returns.  The return per unit plastic
    multiplier R = (trial - new stress) / (2 G alam) is an isotropic function
    of the trial, so R = a I + b n + c dev(n n) (Cayley-Hamilton); b and c
    have poles where two principal values meet, so the targets are a,
    b D, c D with D = pole(eigenvalues of n), and depls / |alam|."""
    depls = rec[:, 20].astype(np.float64)
    anpsi = rec[:, 23].astype(np.float64)
    cdep = np.sqrt((7 + 4 * anpsi + 7 * anpsi * anpsi) / 18)
    alam = -depls / cdep            # a shear return has fs < 0, so alam < 0
    R = (trial - rec[:, 14:20]) / (2.0 * shearm * np.where(alam != 0, alam, 1.0))[:, None]
    n, q, lam, ok = basis(trial)
    a = R[:, :3].mean(1)
    Rd = _dev(R)
    g11, g12, g22 = _inner(n, n), _inner(n, q), _inner(q, q)
    r1, r2 = _inner(Rd, n), _inner(Rd, q)
    det = g11 * g22 - g12 * g12
    good = ok & (depls > 0) & (det > 1e-12)
    det = np.where(good, det, 1.0)
    b = (r1 * g22 - r2 * g12) / det
    c = (r2 * g11 - r1 * g12) / det
    rebuilt = a[:, None] * np.array([1, 1, 1, 0, 0, 0]) + b[:, None] * n + c[:, None] * q
    good &= np.linalg.norm(rebuilt - R, axis=1) <= 1e-4 * np.linalg.norm(R, axis=1)
    D = pole(lam)
    y = np.zeros((len(rec), abi.MLP_OUT))
    y[:, 0] = a
    y[:, 1] = b * D
    y[:, 2] = c * D
    y[:, 3] = cdep
    return y, good


def rebuild(y, trial):
    """The return per unit multiplier from (unscaled) network outputs."""
    n, q, lam, ok = basis(trial)
    D = pole(lam)
    return y[:, 0:1] * np.array([1, 1, 1, 0, 0, 0]) + (y[:, 1] / D)[:, None] * n + (y[:, 2] / D)[:, None] * q


def collect(device, nsteps, every=10, capacity=4_000_000):
    """Training records from an FP64 device: the returns of one step in every
    `every` over nsteps steps (the others run without logging), at most
    `capacity` in all, so that the data span the run rather than its start."""
    parts, kept = [], 0
    per = max(1, capacity // max(1, nsteps // every))
    for _ in range(nsteps // every):
        rec, _ = device.log_returns(1, per)
        parts.append(rec)
        kept += len(rec)
        if every > 1:
            device.step(every - 1)
    return np.concatenate(parts) if parts else np.zeros((0, abi.RET_RECORD), np.float32)


def dataset(rec, params):
    """(raw inputs, targets) of the usable records."""
    bulkm, shearm, pls_sat = single_material(params)
    trial = trial_stress(rec, bulkm, shearm)
    raw, ok1 = features(trial, rec[:, 12].astype(np.float64), rec[:, 13].astype(np.float64), pls_sat)
    y, ok2 = targets(rec, trial, shearm)
    ok = ok1 & ok2 & np.isfinite(y).all(1)
    return raw[ok], y[ok]


def new_net(seed, tol=1e-3):
    """He-initialised network (zero padding rows and columns, unused inputs)."""
    rng = np.random.default_rng(seed)
    net = abi.Mlp()
    w1 = net.arr("w1")
    w1[:, :2 * USED_IN:2] = rng.normal(0, np.sqrt(2.0 / USED_IN), (abi.MLP_HID, USED_IN))
    # the low half of each input pair starts with the weight that reassembles x
    w1[:, 1:2 * USED_IN:2] = w1[:, :2 * USED_IN:2] / 256.0
    net.arr("w2")[:] = rng.normal(0, np.sqrt(2.0 / abi.MLP_HID), (abi.MLP_HID, abi.MLP_HID))
    net.arr("w3")[:NOUT] = rng.normal(0, np.sqrt(1.0 / abi.MLP_HID), (NOUT, abi.MLP_HID))
    net.arr("in_scale")[:] = 1.0
    net.arr("out_scale")[:] = 1.0
    net.tol = tol
    return net


def fit_normalisation(net, raw, y, margin=0.02):
    """Input mean/scale, output scales and the training envelope of the
    normalised inputs, widened by `margin` of its range."""
    mean = np.zeros(abi.MLP_IN)
    scale = np.ones(abi.MLP_IN)
    for i in range(USED_IN):
        mean[i] = raw[:, i].mean()
        sd = raw[:, i].std()
        scale[i] = 1.0 / sd if sd > 0 else 1.0
    x = (raw - mean) * scale
    lo, hi = x.min(0), x.max(0)
    pad = margin * np.maximum(hi - lo, 1e-3)
    osc = np.ones(abi.MLP_OUT)
    # outputs that hardly vary (the isotropic part, depls/|alam| once the
    # dilation has weakened) are scaled by their size instead of their spread
    osc[:NOUT] = np.maximum(np.maximum(y[:, :NOUT].std(0), 0.1 * np.abs(y[:, :NOUT].mean(0))), 1e-6)
    net.arr("in_mean")[:] = mean
    net.arr("in_scale")[:] = scale
    net.arr("env_lo")[:] = lo - pad
    net.arr("env_hi")[:] = hi + pad
    net.arr("out_scale")[:] = osc
    return net


def _bf16(a):
    """float32 values rounded to the nearest bfloat16 (ties to even)."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def normalise(net, raw, y=None):
    """Network inputs: the normalised quantities, each as a BF16 pair
    (x = hi + lo / 256, as the stress pass forms them), and scaled targets."""
    z = ((raw - net.arr("in_mean")) * net.arr("in_scale")).astype(np.float32)
    x = np.zeros_like(z)
    for i in range(USED_IN):
        hi = _bf16(z[:, i])
        x[:, 2 * i] = hi
        x[:, 2 * i + 1] = (z[:, i] - hi) * np.float32(256)
    if y is None:
        return np.ascontiguousarray(x)
    t = (y / net.arr("out_scale")).astype(np.float32)
    t[:, NOUT:] = 0
    return np.ascontiguousarray(x), np.ascontiguousarray(t)


def train(net, x, t, epochs=20, batch=1024, lr=2e-3, seed=1):
    """Adam on the GPU over normalised (x, t); returns the mini-batch losses."""
    n = len(x)
    steps = max(1, int(epochs * n // batch))
    trace = np.zeros(steps, np.float32)
    _ck(_lib().des_mlp_train(C.byref(net), _fptr(x), _fptr(t), n, steps, batch, lr, seed,
                             _fptr(trace)), "des_mlp_train")
    return trace


def forward(net, x):
    """Network outputs (normalised) of normalised inputs, on the GPU."""
    y = np.zeros((len(x), abi.MLP_OUT), np.float32)
    _ck(_lib().des_mlp_forward(C.byref(net), _fptr(x), len(x), _fptr(y)), "des_mlp_forward")
    return y


def loss_grad(net, x, t):
    """Loss and gradient (an abi.Mlp holding d loss / d weights) on the GPU."""
    g = abi.Mlp()
    loss = C.c_double()
    _ck(_lib().des_mlp_loss_grad(C.byref(net), _fptr(x), _fptr(t), len(x), C.byref(loss),
                                 C.byref(g)), "des_mlp_loss_grad")
    return loss.value, g


def fit(records, params, seed=1, epochs=20, batch=1024, lr=2e-3, tol=1e-3):
    """Records -> trained closure (abi.Mlp) and the training losses."""
    raw, y = dataset(records, params)
    net = fit_normalisation(new_net(seed, tol), raw, y)
    x, t = normalise(net, raw, y)
    trace = train(net, x, t, epochs=epochs, batch=batch, lr=lr, seed=seed)
    return net, trace
