"""Benchmark of the DynEarthSol3D explicit time step on one GB300.

A "step" is one iteration of the reference's loop body (dynearthsol.cxx:358-394)
over the whole mesh.  The workload is config 2: 200x200x40 hexes x 6 =
9,600,000 tetrahedra (1,656,441 nodes), elasto-plastic, FP64 plain form.  The
state (about 4.8 GB) is far larger than the 129 MB L2, so no flush is needed
between timed steps.

  python bench.py [--gpus 1] [--steps K] [--warmup W] [--config 2] [--impl ours|reference]

--impl reference times the CPU implementation of the same loop on the same
workload, with the same --steps and --warmup (median of 3 timings of the
steps): the oracle restatement with OpenMP on every host thread, its case
built by the oracle alone (no product library is loaded).  The reference's own
functions need its sources, which exist only where it is checked out; their
speed against the restatement, measured there on the same threads
(oracle/ref_speed.json), is reported beside the number.
"""
import argparse
import gc
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "dynearthsol-old_gb300"))
sys.path.insert(0, str(ROOT))

METRIC = "element-steps/s on 1 GB300: FP64 plain vs FP32+MLP closure at stated error, %HBM"
UNIT = "element-steps/s"
# compulsory bytes per element-step of the FP64 elasto-plastic step: stress,
# strain (6 x 8 B read + write each), plastic strain (read + write), connectivity;
# nodal coord, vel (read + write), T (read + write), bcflag, scaled by nodes/elements
B_ELEM = 6 * 8 * 2 * 2 + 8 * 2 + 4 * 4
B_NODE = 3 * 8 * 2 * 2 + 8 * 2 + 4


# DRAM bytes (read + written) per element of each FP64 pass from one ncu
# capture of the pass alone on a 100x100x40 box of config 2's physics
TRAFFIC_PER_ELEM = {"N-A": 95.0, "E-B": 438.9, "N-B": 26.3, "E-C": 310.6, "N-C": 136.7, "E-A": 607.2}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index=0):
        self.samples, self.proc, self.index = [], None, index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = sorted(float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit())
        mx = max(float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4)
                          if len(s) > 4 + i and s[4 + i].lower().startswith("active")})
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(self.samples)}


def replica_throughput(ms, nelem, steps, world, reduce_max=None):
    """Whole-job element-steps/s of `world` independent replicas: every rank
    processed nelem * steps element-steps; the job took the slowest rank's time."""
    if reduce_max is not None:
        ms = reduce_max(ms)
    return world * nelem * steps / (ms / 1e3), ms


def torch_reduce_max(device):
    import torch
    import torch.distributed as tdist

    def f(ms):
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        return float(t.item())
    return f


def build_case(cfg_key, box=None):
    import des_gb300 as D
    from des_gb300 import workload as W
    cfg = W.CONFIGS[cfg_key]
    if box:
        nx, ny, nz = (int(v) for v in box.lower().split("x"))
        cfg = W.scaled(cfg, nx, ny, nz)
    mesh, p, T, pls, topo = D.setup_case(cfg)
    return cfg, mesh, p, T, pls


def cpu_baseline(cfg_key, steps=5, warmup=3, repeats=3):
    """The CPU restatement of the loop (OpenMP, every host thread) on the same
    workload, built by the oracle alone (oracle/workload_np.py: no product
    library is loaded): `warmup` steps, then the median of `repeats` timings
    of `steps` steps.  Beside it, the restatement's speed over the
    reference's own functions measured on the same host, threads and case
    where the reference's sources are (oracle/ref_speed.json)."""
    import statistics
    from des_gb300 import workload as W
    from oracle import workload_np as WN
    from oracle.oracle import PortOracle
    cfg = W.CONFIGS[cfg_key]
    t0 = time.perf_counter()
    mesh, p, T, pls, o = WN.setup_case(cfg)
    s = W.new_state(mesh, T, pls)
    o.init_fields(s)
    setup_s = time.perf_counter() - t0
    if warmup:
        o.step(s, warmup)
    times = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        o.step(s, steps)
        times.append(time.perf_counter() - t0)
    dt = statistics.median(times)
    threads = int(PortOracle.lib().dso_num_threads())
    out = {"value": mesh.nelem * steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
           "sample": f"{cfg.name} ({mesh.nelem} tets): {warmup} warm-up steps, then the median of "
                     f"{repeats} timings of {steps} steps ({', '.join(f'{x:.2f}' for x in times)} s); "
                     f"case built in {setup_s:.1f} s by the oracle alone"}
    f = ROOT / "oracle" / "ref_speed.json"
    if f.exists():
        r = json.loads(f.read_text())
        out["reference_functions"] = {
            "port_over_reference": r["port_over_reference"],
            "estimate": out["value"] / r["port_over_reference"],
            "measured": f"{r['case']}, {r['threads']} threads on {r['host']}: restatement "
                        f"{r['port_elem_steps_per_s']:.3e}, reference's own functions "
                        f"{r['reference_elem_steps_per_s']:.3e} element-steps/s",
            "why": "the reference's sources are not on this host; the restatement is timed and "
                   "the reference's own functions were timed against it where the sources are"}
    return out


def _fresh_form(cfg, precision, local, params=None):
    """A device with the initial state of cfg in the given precision."""
    import des_gb300 as D
    from des_gb300 import abi, workload as W
    mesh, p, T, pls, topo = D.setup_case(cfg)
    q = abi.Params.from_buffer_copy(params if params is not None else p)
    q.precision = precision
    dv = D.Device(mesh, q, device=local)
    s0 = W.new_state(mesh, T, pls)
    dv.upload(s0, abi.F_COORD | abi.F_TEMPERATURE | abi.F_PLSTRAIN)
    dv.init_fields()
    return dv, mesh, q


def e2e_rate(dev, mesh, steps, barrier, world):
    """element-steps/s through des_gpu_step_host with page-locked host arrays
    (the loop state up and down every step), and the bytes up and down."""
    import numpy as np
    import des_gb300 as D
    from des_gb300 import abi
    host = abi.State(mesh.nnode, mesh.nelem)
    dev.download(host, abi.F_ALL)
    D.pin(host)
    mask = abi.F_STEP_STATE
    nb = {abi.F_COORD: 24 * mesh.nnode, abi.F_VEL: 24 * mesh.nnode, abi.F_FORCE: 24 * mesh.nnode,
          abi.F_TEMPERATURE: 8 * mesh.nnode, abi.F_MASS: 24 * mesh.nnode,
          abi.F_NTMP: 8 * mesh.nnode, abi.F_VOLUME: 16 * mesh.nelem,
          abi.F_STRESS: 48 * mesh.nelem, abi.F_STRAIN: 48 * mesh.nelem,
          abi.F_STRAIN_RATE: 48 * mesh.nelem, abi.F_PLSTRAIN: 16 * mesh.nelem,
          abi.F_DPRESSURE: 8 * mesh.nelem, abi.F_EDVOLDT: 8 * mesh.nelem,
          abi.F_SHAPE: 96 * mesh.nelem, abi.F_SCALARS: 0}
    io_bytes = sum(v for k, v in nb.items() if mask & k)
    # des_gpu_step_host uploads only what the loop reads and recomputes volume,
    # shape derivatives and masses from coordinates and temperature
    h2d = (24 + 24 + 8) * mesh.nnode + (48 + 48 + 16 + 8) * mesh.nelem
    for _ in range(2):                          # warm-up of the host path
        dev.step_host(host, 1, mask)
    barrier()
    per_step = []
    # no garbage collection inside the timed host loop (as timeit does)
    gc.collect()
    gc.disable()
    try:
        t0 = time.perf_counter()
        for _ in range(steps):
            t1 = time.perf_counter()
            dev.step_host(host, 1, mask)
            per_step.append(time.perf_counter() - t1)
        e2e_s = time.perf_counter() - t0
    finally:
        gc.enable()
    D.unpin(host)
    e2e_rate.last_ms = {"min": 1e3 * min(per_step), "median": 1e3 * float(np.median(per_step)),
                        "max": 1e3 * max(per_step), "slowest_step": int(np.argmax(per_step))}
    return world * mesh.nelem * steps / e2e_s, h2d, io_bytes


def train_closure(base, local, box=(60, 60, 12), nsteps=300, epochs=20):
    """The closure for base's material: nsteps FP64 steps of a smaller box of
    it logged (at most 4M returns kept), then Adam on the GPU."""
    from des_gb300 import abi, closure, workload as W
    t0 = time.perf_counter()
    dv, tmesh, tp = _fresh_form(W.scaled(base, *box), abi.PREC_FP64, local)
    rec = closure.collect(dv, nsteps, every=5)
    nrec = len(rec)
    dv.close()
    net, trace = closure.fit(rec, tp, epochs=epochs, seed=1)
    net.tol = 1e-3
    info = {"records": int(nrec), "kept": int(len(rec)),
            "box": f"{box[0]}x{box[1]}x{box[2]} x6 = {tmesh.nelem} tets, {nsteps} FP64 steps",
            "seconds": time.perf_counter() - t0, "loss_first": float(trace[:100].mean()),
            "loss_last": float(trace[-100:].mean()), "tol": net.tol}
    return net, info


def profile_mlp_grad(args):
    """The closure network's loss and gradient (k_mlp_grad) over a seeded
    batch, `warmup` + `steps` calls, for ncu captures of the training kernel."""
    import numpy as np
    import des_gb300 as D
    from des_gb300 import abi, closure
    D.build()
    rng = np.random.default_rng(3)
    net = abi.Mlp()
    for k in ("w1", "b1", "w2", "b2", "w3", "b3"):
        a = net.arr(k)
        a[...] = rng.normal(0, 0.3, a.shape)
    net.arr("w1")[:, 14:] = 0
    net.arr("w3")[7] = 0
    net.arr("b3")[7] = 0
    net.arr("in_scale")[:] = 1
    net.arr("out_scale")[:] = 1
    n = args.samples
    x = np.zeros((n, 16), np.float32)
    x[:, :14] = rng.normal(0, 1, (n, 14))
    t = np.zeros((n, 8), np.float32)
    t[:, :7] = rng.normal(0, 1, (n, 7))
    for _ in range(args.warmup):
        closure.loss_grad(net, x, t)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        loss, _ = closure.loss_grad(net, x, t)
    print(json.dumps({"profile_form": "mlp_grad", "samples": n, "tiles": (n + 127) // 128, "loss": loss,
                      "seconds_per_call_with_copies": (time.perf_counter() - t0) / args.steps}))


def profile_form(args):
    """One form alone (for ncu captures): warm-up, then the timed steps."""
    import des_gb300 as D
    from des_gb300 import abi, workload as W
    if args.profile_form == "mlp_grad":
        return profile_mlp_grad(args)
    D.build()
    base = W.CONFIGS[args.config]
    cfg = base
    if args.box:
        nx, ny, nz = (int(v) for v in args.box.lower().split("x"))
        cfg = W.scaled(base, nx, ny, nz)
    net = None
    if args.profile_form == "fp32_closure":
        net, _ = train_closure(base, 0)
    prec = abi.PREC_FP64 if args.profile_form == "fp64" else abi.PREC_FP32
    dv, mesh, _ = _fresh_form(cfg, prec, 0)
    if net is not None:
        dv.set_closure(net)
    dv.step(args.warmup)
    ms = dv.time_steps(args.steps)
    r = dv.report()
    dv.close()
    print(json.dumps({"profile_form": args.profile_form, "workload": cfg.name, "nelem": mesh.nelem,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                      "value": mesh.nelem * args.steps / (ms / 1e3), "unit": UNIT,
                      "closure_candidates": r.closure_candidates, "closure_accepted": r.closure_accepted,
                      "exact_returns": r.exact_returns}))


def yielding_forms(args, local, world, barrier, reduce, compare):
    """The three forms on the yielding workload, where the learned closure has
    returns to replace: FP64 plain, FP32 mixed (exact FP64 returns) and FP32
    with the closure.  The closure is trained first, on the GPU, from the
    FP64 form's own returns on a small box of the same material."""
    import des_gb300 as D
    from des_gb300 import abi, closure, workload as W
    base = W.CONFIGS["yield"]
    cfg = base
    if args.box:
        nx, ny, nz = (int(v) for v in args.box.lower().split("x"))
        cfg = W.scaled(base, nx, ny, nz)
    net, training = train_closure(base, local)
    out = {"workload": f"{cfg.name}: weak Mohr-Coulomb material yielding from a weak-seed "
                       "row (1-4% of the elements return each step over the timed steps)",
           "closure_training": training}
    warm = max(args.warmup, 100)      # let the yielding spread from the weak row
    prof = max(2, min(args.steps, 5))
    names = ["N-A", "E-B", "N-B", "E-C", "N-C", "E-A"]
    d64 = S = None
    loose = abi.Mlp.from_buffer_copy(net)
    loose.tol = 1e-2
    for name, prec, use in (("fp64_plain", abi.PREC_FP64, None), ("fp32_mixed", abi.PREC_FP32, None),
                            ("fp32_closure", abi.PREC_FP32, net),
                            ("fp32_closure_tol_1e-2", abi.PREC_FP32, loose)):
        dv, mesh, _ = _fresh_form(cfg, prec, local)
        if use is not None:
            dv.set_closure(use)
        dv.step(warm)
        r0 = dv.report()
        barrier()
        ms = dv.time_steps(args.steps)
        barrier()
        v, ms = replica_throughput(ms, mesh.nelem, args.steps, world, reduce)
        r1 = dv.report()
        passes = dv.profile_steps(prof)
        k = args.steps
        e = {"value": v, "ms_per_step": ms / k,
             "passes_ms_per_step": {n: x / prof for n, x in zip(names, passes)},
             "principal_stress_solves_per_step": (r1.eigen_solves - r0.eigen_solves) / k}
        if use is not None:
            e["tol"] = use.tol
            cand = r1.closure_candidates - r0.closure_candidates
            acc = r1.closure_accepted - r0.closure_accepted
            exact = r1.exact_returns - r0.exact_returns
            e.update(network_candidates_per_step=cand / k, network_accepted_per_step=acc / k,
                     exact_fp64_returns_per_step=exact / k,
                     acceptance=acc / cand if cand else None,
                     fallback_rate=(exact / (exact + acc)) if exact + acc else None)
        if name == "fp64_plain":
            d64 = dv
            S = dv.download(abi.State(mesh.nnode, mesh.nelem), abi.F_ALL)
            fp64_value = v
        else:
            errs = {}
            for nsteps in (1, 100):
                d64.upload(S, abi.F_ALL)
                d64.step(nsteps)
                a = d64.download(abi.State(mesh.nnode, mesh.nelem), abi.F_ALL)
                dv.upload(S, abi.F_ALL)
                dv.step(nsteps)
                b = dv.download(abi.State(mesh.nnode, mesh.nelem), abi.F_ALL)
                errs[f"after_{nsteps}_steps"] = compare(b, a)
            e["rel_l2_vs_fp64_from_the_same_state"] = errs
            e["speedup_vs_fp64"] = v / fp64_value
            dv.close()
        out[name] = e
    # the FP64 loop's own sensitivity on this workload: the same state with
    # its stress perturbed by 1e-12 (relative), 1 and 100 steps, against the
    # unperturbed FP64 loop -- the yardstick for the errors above
    sens = {}
    for nsteps in (1, 100):
        d64.upload(S, abi.F_ALL)
        d64.step(nsteps)
        a = d64.download(abi.State(mesh.nnode, mesh.nelem), abi.F_ALL)
        P = S.copy()
        P.stress *= 1 + 1e-12
        d64.upload(P, abi.F_ALL)
        d64.step(nsteps)
        b = d64.download(abi.State(mesh.nnode, mesh.nelem), abi.F_ALL)
        sens[f"after_{nsteps}_steps"] = compare(b, a)
    out["fp64_perturbed_1e-12_vs_fp64_from_the_same_state"] = sens
    d64.close()
    for k in ("fp32_closure", "fp32_closure_tol_1e-2"):
        out[k]["speedup_vs_fp32_mixed"] = out[k]["value"] / out["fp32_mixed"]["value"]
    return out


def accuracy_2000(cfg_key, box, local, compare):
    """FP32 form against FP64 form after 500, 1,000 and 2,000 steps from init on
    the bench workload with damping option 2 (smooth: a 1e-12 perturbation of
    the FP64 loop stays bounded), each form timed as it runs."""
    import des_gb300 as D
    from des_gb300 import abi, workload as W
    base = W.CONFIGS[cfg_key]
    if box:
        nx, ny, nz = (int(v) for v in box.lower().split("x"))
        base = W.scaled(base, nx, ny, nz)
    d = dict(base.__dict__)
    d["extra"] = dict(base.extra, params=dict(base.extra.get("params", {}), damping_option=2))
    cfg = W.Config(**d)
    mesh, p, T, pls, _ = D.setup_case(cfg)
    states, secs = {}, {}
    for name, prec in (("fp64", abi.PREC_FP64), ("fp32", abi.PREC_FP32)):
        q = abi.Params.from_buffer_copy(p)
        q.precision = prec
        dev = D.Device(mesh, q, device=local)
        s = W.new_state(mesh, T, pls)
        dev.upload(s, abi.F_COORD | abi.F_TEMPERATURE | abi.F_PLSTRAIN)
        dev.init_fields()
        done, t = 0, 0.0
        for k in (500, 1000, 2000):
            t -= time.perf_counter()
            dev.step(k - done)
            dev.report()
            t += time.perf_counter()
            done = k
            states[(name, k)] = dev.download(abi.State(mesh.nnode, mesh.nelem), abi.F_ALL)
        secs[name] = t
        dev.close()
    out = {"workload": f"{cfg.name} with damping option 2", "seconds_for_2000_steps": secs}
    for k in (500, 1000, 2000):
        out[f"fp32_vs_fp64_after_{k}_steps"] = compare(states[("fp32", k)], states[("fp64", k)])
    return out


ACC_FIELDS = (("vel", "F_VEL"), ("stress", "F_STRESS"), ("temperature", "F_TEMPERATURE"),
              ("strain", "F_STRAIN"), ("force", "F_FORCE"), ("coord", "F_COORD"),
              ("plstrain", "F_PLSTRAIN"))


def _field(dev, mesh, name, mask):
    """One field of a device state (the other host arrays stay untouched)."""
    from des_gb300 import abi
    st = abi.State(mesh.nnode, mesh.nelem)
    dev.download(st, mask)
    return getattr(st, name)


def long_run(cfg_key, checkpoints, local, world, reduce, rate_steps=10, sensitivity=True):
    """Configs at their stated sizes over their stated step counts: the FP32
    form and the FP64 form with its initial stress perturbed by 1e-12
    (relative) -- the FP64 loop's own sensitivity, the yardstick for the
    FP32 error -- against the FP64 form from the same initial state.  The
    three run in lockstep on the device; at each checkpoint (steps from
    init) the relative L2 of every compared field is formed field by field.
    Each form's rate is timed with CUDA events over `rate_steps` steps after
    3 warm-up steps (those steps count towards the checkpoints).  Without
    `sensitivity` the perturbed FP64 form is left out."""
    import numpy as np
    import des_gb300 as D
    from des_gb300 import abi, workload as W
    cfg = W.CONFIGS[cfg_key]
    t0 = time.perf_counter()
    mesh, p, T, pls, _ = D.setup_case(cfg)
    out = {"workload": f"{cfg.name}: {mesh.nelem} tets / {mesh.nnode} nodes, "
                       f"{'elasto-visco-plastic' if cfg.rheology == 'evp' else 'elasto-plastic'}"
                       f"{', %d material layers' % cfg.nlayers if cfg.nlayers > 1 else ''}"
                       f"{', T noise sigma %g K' % cfg.t_sigma if cfg.t_sigma else ''}",
           "host_setup_s": time.perf_counter() - t0}
    devs = {}
    names = [("fp64_plain", abi.PREC_FP64), ("fp32_mixed", abi.PREC_FP32)]
    if sensitivity:
        names.append(("fp64_perturbed", abi.PREC_FP64))
    for name, prec in names:
        q = abi.Params.from_buffer_copy(p)
        q.precision = prec
        dv = D.Device(mesh, q, device=local)
        dv.upload(W.new_state(mesh, T, pls), abi.F_COORD | abi.F_TEMPERATURE | abi.F_PLSTRAIN)
        dv.init_fields()
        if name == "fp64_perturbed":
            st = abi.State(mesh.nnode, mesh.nelem)
            dv.download(st, abi.F_STRESS)
            st.stress *= 1 + 1e-12
            dv.upload(st, abi.F_STRESS)
        devs[name] = dv
    secs = {n: 0.0 for n in devs}
    done = 0
    for name, dv in devs.items():
        if name == "fp64_perturbed":
            dv.step(3 + rate_steps)
            continue
        dv.step(3)
        ms = dv.time_steps(rate_steps)
        v, ms = replica_throughput(ms, mesh.nelem, rate_steps, world, reduce)
        out[name] = {"value": v, "ms_per_step": ms / rate_steps, "device_gb": dv.device_bytes / 1e9}
    done = 3 + rate_steps
    reports = {}
    for k in checkpoints:
        for name, dv in devs.items():
            t1 = time.perf_counter()
            reports[name] = dv.step(k - done)
            secs[name] += time.perf_counter() - t1
        done = k
        pairs = [("fp32_mixed", "fp32_vs_fp64")]
        if sensitivity:
            pairs.append(("fp64_perturbed", "fp64_perturbed_vs_fp64"))
        errs = {key: {} for _, key in pairs}
        for f, m in ACC_FIELDS:
            ref = _field(devs["fp64_plain"], mesh, f, getattr(abi, m))
            nb = float(np.linalg.norm(ref)) or 1.0
            for name, key in pairs:
                x = _field(devs[name], mesh, f, getattr(abi, m))
                errs[key][f] = float(np.linalg.norm(x - ref)) / nb
                del x
            del ref
        out[f"after_{k}_steps"] = errs
    out["seconds_for_the_checkpointed_steps"] = secs
    out["status"] = {n: r.status for n, r in reports.items()}
    out["eigen_solves"] = {n: r.eigen_solves for n, r in reports.items()}
    out["exact_returns_fp32"] = reports["fp32_mixed"].exact_returns
    pls_end = _field(devs["fp64_plain"], mesh, "plstrain", abi.F_PLSTRAIN)
    out["elements_whose_plastic_strain_grew_fp64"] = int(np.count_nonzero(pls_end > pls))
    for dv in devs.values():
        dv.close()
    out["fp32_mixed"]["speedup_vs_fp64"] = out["fp32_mixed"]["value"] / out["fp64_plain"]["value"]
    return out


def config4_returns(local, nsteps=2000):
    """Config 4 as stated (the config-2 mesh, 9.6M tets, with config 3's
    elasto-visco-plastic rheology): how many shear returns the FP64 form makes
    over its 2,000 steps, i.e. how much work the learned closure would have."""
    import numpy as np
    import des_gb300 as D
    from des_gb300 import abi, workload as W
    cfg = W.CONFIGS["4"]
    mesh, p, T, pls, _ = D.setup_case(cfg)
    dv = D.Device(mesh, p, device=local)
    dv.upload(W.new_state(mesh, T, pls), abi.F_COORD | abi.F_TEMPERATURE | abi.F_PLSTRAIN)
    dv.init_fields()
    t0 = time.perf_counter()
    _, nret = dv.log_returns(nsteps, 1)
    secs = time.perf_counter() - t0
    r = dv.report()
    grew = int(np.count_nonzero(_field(dv, mesh, "plstrain", abi.F_PLSTRAIN) > pls))
    dv.close()
    return {"workload": f"{cfg.name}: {mesh.nelem} tets / {mesh.nnode} nodes, config 3's "
                        "elasto-visco-plastic rheology on the config-2 mesh with its weak-seed row",
            "steps": nsteps, "shear_returns_fp64": int(nret), "eigen_solves_fp64": r.eigen_solves,
            "elements_whose_plastic_strain_grew": grew, "status": r.status,
            "seconds": secs}


def workload_name(cfg):
    """The bench workload as both arms name it."""
    nelem = 6 * cfg.nx * cfg.ny * cfg.nz
    nnode = (cfg.nx + 1) * (cfg.ny + 1) * (cfg.nz + 1)
    return f"{cfg.name}: {nelem} tets / {nnode} nodes, elasto-plastic, FP64 plain form"


def line_config(cfg, world):
    """The line's config, identical in both arms."""
    return {"workload": workload_name(cfg), "parallelism": f"replicas{world}",
            "l2": "state 4.8 GB >> 129 MB L2, no flush"}


def run_reference(args):
    """The CPU implementation of the loop on the same workload, steps and
    warm-up as the GPU arm (rank 0 only under torchrun)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from des_gb300 import workload as W
    cfg = W.CONFIGS[args.config]
    cb = cpu_baseline(args.config, steps=args.steps, warmup=args.warmup, repeats=3)
    nelem = 6 * cfg.nx * cfg.ny * cfg.nz
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": nelem / cb["value"] * 1e3,
            "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": line_config(cfg, args.gpus),
            "cpu_baseline": cb,
            "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args):
    import numpy as np
    import des_gb300 as D
    from des_gb300 import abi, workload as W

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = world > 1
    if dist:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")

    D.build()
    cfg, mesh, p, T, pls = build_case(args.config, args.box)

    def barrier():
        if dist:
            tdist.barrier()

    def make_form(precision):
        q = abi.Params.from_buffer_copy(p)
        q.precision = precision
        dv = D.Device(mesh, q, device=local)
        s0 = W.new_state(mesh, T, pls)
        dv.upload(s0, abi.F_COORD | abi.F_TEMPERATURE | abi.F_PLSTRAIN)
        dv.init_fields()
        dv.step(args.warmup)                       # warm-up (also captures the graph)
        return dv

    # FP64 plain form: the headline
    dev = make_form(abi.PREC_FP64)
    barrier()
    with ClockSampler(local) as clk:
        ms = dev.time_steps(args.steps)
    barrier()
    value, ms = replica_throughput(ms, mesh.nelem, args.steps, world,
                                   torch_reduce_max(f"cuda:{local}") if dist else None)
    rep = dev.report()
    S = dev.download(abi.State(mesh.nnode, mesh.nelem), abi.F_ALL)

    def rel(a, b):
        nb = float(np.linalg.norm(b))
        return float(np.linalg.norm(a - b) / (nb if nb else 1.0))

    def compare(x, y):
        return {f: rel(getattr(x, f), getattr(y, f))
                for f in ("vel", "force", "stress", "strain", "temperature", "coord")}

    # FP32 mixed form: timed on the same workload, then checked from the FP64
    # state S (one step, and 100 steps) against the FP64 form
    forms = {"fp64_plain": {"value": value, "ms_per_step": ms / args.steps}}
    dev32 = make_form(abi.PREC_FP32)
    barrier()
    with ClockSampler(local) as clk32:
        ms32 = dev32.time_steps(args.steps)
    barrier()
    v32, ms32 = replica_throughput(ms32, mesh.nelem, args.steps, world,
                                   torch_reduce_max(f"cuda:{local}") if dist else None)
    prof32 = max(2, min(args.steps, 5))
    passes32 = dev32.profile_steps(prof32)
    rep32 = dev32.report()
    errs = {}
    for nsteps in (1, 100):
        dev.upload(S, abi.F_ALL)
        dev.step(nsteps)
        a = dev.download(abi.State(mesh.nnode, mesh.nelem), abi.F_ALL)
        dev32.upload(S, abi.F_ALL)
        dev32.step(nsteps)
        b = dev32.download(abi.State(mesh.nnode, mesh.nelem), abi.F_ALL)
        errs[f"after_{nsteps}_steps"] = compare(b, a)
    e2e32, _, _ = e2e_rate(dev32, mesh, max(1, min(args.steps, 20)), barrier, world)
    e2e32_ms = e2e_rate.last_ms
    dev32.close()
    dev.upload(S, abi.F_ALL)
    forms["fp32_mixed"] = {
        "value": v32, "ms_per_step": ms32 / args.steps, "speedup_vs_fp64": v32 / value,
        "rel_l2_vs_fp64_from_the_same_state": errs,
        "passes_ms_per_step": dict(zip(["N-A", "E-B", "N-B", "E-C", "N-C", "E-A"],
                                       [t / prof32 for t in passes32])),
        "eigen_solves": rep32.eigen_solves, "clocks": clk32.summary(),
        "e2e": {"value": e2e32, "unit": UNIT, "ms_per_step": e2e32_ms,
                "note": "same host-buffer path as the line's e2e"}}

    if not args.no_yielding:
        forms["yielding"] = yielding_forms(args, local, world, barrier,
                                           torch_reduce_max(f"cuda:{local}") if dist else None, compare)
    if not args.no_accuracy and world == 1:
        forms["fp32_accuracy_2000_steps"] = accuracy_2000(args.config, args.box, local, compare)
    red = torch_reduce_max(f"cuda:{local}") if dist else None
    if not args.no_large:
        forms["config3"] = long_run("3", (100, 1000, 5000), local, world, red)
        forms["config4"] = config4_returns(local)
        forms["config5"] = long_run("5", (100, 1000), local, world, red, sensitivity=False)

    # per-pass device times over extra steps (same arithmetic, launched one by one)
    prof_steps = max(2, min(args.steps, 5))
    per_pass = dev.profile_steps(prof_steps)
    names = ["N-A", "E-B", "N-B", "E-C", "N-C", "E-A"]
    top = int(np.argmax(per_pass))
    # algorithmic bytes per element of each pass: every array the pass reads
    # or writes, once (element arrays per element, nodal arrays scaled by
    # nodes/elements r); CSR topology excluded.  The same list, array by
    # array, is the pass table of the design notes.
    r = mesh.nnode / mesh.nelem
    alg = {
        # vol_n, tmass, T (r+w), ntmp, bcflag per node; conduction (4) and dvoldt contributions
        "N-A": r * 44 + 40,
        # conn, mix, stress/strain (r+w), next strain rate, strain rate, pls/dpls (r+w),
        # edvoldt, dp, dp*V, volume; ntmp gathered
        "E-B": 16 + 1 + 96 + 96 + 48 + 48 + 16 + 16 + 8 + 8 + 8 + 8 + r * 8,
        # dp*V; vol_n, ntmp per node
        "N-B": r * 16 + 8,
        # conn, mix, dp, stress (6 read, 3 written), shape derivatives, volume, force
        # vectors; ntmp, T gathered
        "E-C": 16 + 1 + 8 + 72 + 96 + 8 + 96 + r * 16,
        # force vectors; force, vel (r+w), mass, coord (r+w), bcflag per node
        "N-C": r * 132 + 96,
        # conn, mix, volume (r), volume_old, volume, shape derivatives, masses (2),
        # stress/strain (r+w), next strain rate, dvoldt and conduction contributions;
        # coord, vel, T gathered
        "E-A": 16 + 1 + 8 + 8 + 8 + 96 + 16 + 96 + 96 + 48 + 8 + 32 + r * 56,
    }
    hbm, hbm_kind = peaks()
    t_top = per_pass[top] / prof_steps / 1e3
    achieved = alg[names[top]] * mesh.nelem / t_top / 1e9
    step_alg = (B_ELEM + B_NODE * r) * mesh.nelem
    step_gbs = step_alg / (ms / args.steps / 1e3) / 1e9
    # FP64 pipe: thread instructions on the FP64 pipe per element of each pass
    # in a step without the dt reduction (ncu instruction counters of the same
    # passes on a 100x100x40 box of this physics), against GB300's 2 FP64
    # instructions per clock per SM.  Part of each pass's multiplies run as
    # exactly rounded integer-pipe products (sf::mul) instead, which is what
    # lets the step beat this pipe's bound for the reference's arithmetic
    # (604 FP64 instructions per element-step when every product is on it).
    fp64_ops = {"N-A": 23.1, "E-B": 44.0, "N-B": 5.4, "E-C": 44.1, "N-C": 19.7, "E-A": 260.0}
    fp64_ops_all_on_pipe = 604.2
    import torch
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    sm_hz = (clk.summary().get("sm_mhz") or 2070.0) * 1e6
    fp64_peak = 2.0 * sms * sm_hz
    fp64_top = fp64_ops[names[top]] * mesh.nelem / t_top
    fp64_step = sum(fp64_ops.values()) * mesh.nelem / (ms / args.steps / 1e3)

    # the remesh trigger (bad_mesh_quality on the device), timed on the same state
    chk = abi.RemeshCheck(smallest_size=0.01, resolution=cfg.xlength / cfg.nx, zlength=cfg.zlength,
                          max_boundary_distortion=0.25, min_quality=0.4, remeshing_option=1)
    dev.bad_mesh_quality(chk)
    t0 = time.perf_counter()
    for _ in range(3):
        qcode = dev.bad_mesh_quality(chk)
    remesh_ms = (time.perf_counter() - t0) / 3 * 1e3

    # output frames: a device snapshot of the output fields, downloaded into
    # page-locked host arrays on a second stream while 5 steps run
    out_host = abi.State(mesh.nnode, mesh.nelem)
    D.pin(out_host)
    out_bytes = (4 * 24 + 8) * mesh.nnode + (16 + 3 * 48 + 16) * mesh.nelem
    dev.output_snapshot()
    dev.output_fetch(out_host)
    dev.output_wait(out_host)                  # warm-up
    dev.report()
    t_plain = t_overlap = t_alone = float("inf")
    for _ in range(3):                          # the best of three of each
        t0 = time.perf_counter()
        dev.step(5)
        t_plain = min(t_plain, time.perf_counter() - t0)
        t0 = time.perf_counter()
        dev.output_snapshot()
        dev.output_fetch(out_host)
        dev.step(5)
        dev.output_wait(out_host)
        dev.report()
        t_overlap = min(t_overlap, time.perf_counter() - t0)
        t0 = time.perf_counter()
        dev.output_snapshot()
        dev.output_fetch(out_host)
        dev.output_wait(out_host)
        t_alone = min(t_alone, time.perf_counter() - t0)
    D.unpin(out_host)
    output = {"bytes": out_bytes, "download_alone_ms": t_alone * 1e3,
              "five_steps_ms": t_plain * 1e3, "five_steps_with_download_ms": t_overlap * 1e3}

    # end to end through the drop-in entry point with page-locked host buffers:
    # every step uploads the loop's state from the host and downloads it back
    e2e, h2d_bytes, d2h_bytes = e2e_rate(dev, mesh, max(1, min(args.steps, 20)), barrier, world)
    e2e_ms = e2e_rate.last_ms

    cb = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(args.config, steps=5, warmup=3, repeats=3)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": line_config(cfg, world),
        "gpu_launches": dev.kernels_per_step * args.steps,
        "roofline": {"bound": "hbm", "kernel": names[top],
                     "limiter": "the FP64 pipe, not HBM: fp64_pipe below is the bound that applies; "
                                "achieved/frac are the pass's algorithmic bytes over its time",
                     "fp64_pipe": {"kernel": names[top], "achieved": fp64_top, "peak": fp64_peak,
                                   "unit": "FP64 inst/s", "frac": fp64_top / fp64_peak,
                                   "ops_per_element": fp64_ops[names[top]],
                                   "step_ops_per_element": sum(fp64_ops.values()),
                                   "step_frac": fp64_step / fp64_peak,
                                   "step_ops_per_element_all_on_fp64_pipe": fp64_ops_all_on_pipe,
                                   "step_time_bound_all_on_fp64_pipe_ms":
                                       fp64_ops_all_on_pipe * mesh.nelem / fp64_peak * 1e3,
                                   "peak_kind": f"nominal: 2 per clock per SM x {sms} SMs at the sampled SM clock"},
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "alg_bytes_per_element": alg[names[top]],
                     # DRAM bytes per launch from an ncu capture of the pass on a
                     # 100x100x40 box (traffic grows with the element count), scaled
                     # to this launch
                     "traffic": TRAFFIC_PER_ELEM.get(names[top], None) and
                                TRAFFIC_PER_ELEM[names[top]] * mesh.nelem,
                     "peak_kind": hbm_kind,
                     "step_alg_bytes_per_elem": B_ELEM + B_NODE * r,
                     "step_achieved_gbs": step_gbs, "step_frac": step_gbs / hbm},
        "passes_ms_per_step": {n: t / prof_steps for n, t in zip(names, per_pass)},
        "forms": forms,
        "output_frame": output,
        "remesh_check": {"ms_per_call": remesh_ms, "result": list(qcode),
                         "what": "bad_mesh_quality on the device (elem_quality of every element, "
                                 "tiny-element and bottom checks), host wall time incl. the read-back"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d_bytes,
                "d2h_bytes_per_step": d2h_bytes, "ms_per_step": e2e_ms},
        "clocks": clk.summary(),
        "status": rep.status, "eigen_solves": rep.eigen_solves,
        "device_gb": dev.device_bytes / 1e9,
    }
    if cb:
        line["cpu_baseline"] = cb
    dev.close()
    if rank == 0:
        print(json.dumps(line))
    if dist:
        tdist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--config", default="2")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-yielding", action="store_true",
                    help="skip the forms on the yielding workload")
    ap.add_argument("--no-large", action="store_true",
                    help="skip configs 3, 4 and 5 at their stated sizes and step counts")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the 2,000-step FP32-against-FP64 accuracy run")
    ap.add_argument("--profile-form", choices=["fp64", "fp32", "fp32_closure", "mlp_grad"], default=None,
                    help="run one form alone on --config/--box (for profiling); mlp_grad: the "
                    "closure network's loss and gradient over --samples seeded samples, --steps times")
    ap.add_argument("--samples", type=int, default=152 * 8 * 128,
                    help="samples of --profile-form mlp_grad")
    ap.add_argument("--box", default=None, help="NXxNYxNZ hexes instead of the config's box "
                    "(profiling of smaller cases)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.profile_form:
        profile_form(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
