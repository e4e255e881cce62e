"""TEST INFRASTRUCTURE -- how fast the CPU restatement runs against the
reference's own functions on the same host, threads and case.

The reference's sources exist only where it is checked out, so the CPU arm
of the benchmark on a host without them times the restatement (PortOracle)
and reports, beside it, the factor measured here:

    python oracle/ref_speed.py [--box 60x60x12] [--steps 20] [--warmup 5] [--repeats 3]

writes oracle/ref_speed.json.  Both sides run the loop of config 2's physics
(elasto-plastic, weak-seed row) on the same mesh and initial state, with
OpenMP on every host thread; the reference is oracle/_ref/libdesref.so built
by oracle/ref.mk with the reference's default flags (-O2 -fopenmp).  Each
side: warm-up steps, then the median of `repeats` timings of `steps` steps.
"""
import argparse
import json
import os
import platform
import statistics
import sys
import time
from pathlib import Path

ORACLE = Path(__file__).resolve().parent
ROOT = ORACLE.parent
sys.path[:] = [x for x in sys.path if Path(x or ".").resolve() != ORACLE]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "dynearthsol-old_gb300"))

from des_gb300 import workload as W  # noqa: E402
from oracle import oracle as O, workload_np as WN  # noqa: E402


def _median_rate(step, nelem, steps, warmup, repeats):
    step(warmup)
    times = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        step(steps)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    return nelem * steps / t, times


def measure(box=(60, 60, 12), steps=20, warmup=5, repeats=3):
    if O.build_ref() is None:
        raise SystemExit("the reference tree is absent: set DES_REFERENCE")
    cfg = W.scaled(W.CONFIGS["2"], *box)
    mesh, p, T, pls, port = WN.setup_case(cfg)
    ref = O.RefOracle(mesh, p)
    s_port = W.new_state(mesh, T, pls)
    s_ref = W.new_state(mesh, T, pls)
    port.init_fields(s_port)
    ref.init_fields(s_ref)
    ref._in(s_ref)
    r_port, t_port = _median_rate(lambda n: port.step(s_port, n), mesh.nelem, steps, warmup, repeats)
    r_ref, t_ref = _median_rate(lambda n: ref.L.dsr_step(ref.h, n), mesh.nelem, steps, warmup, repeats)
    threads = int(O.PortOracle.lib().dso_num_threads())
    return {"case": f"{cfg.name}: {mesh.nelem} tets / {mesh.nnode} nodes, config 2's physics",
            "steps": steps, "warmup": warmup, "repeats": repeats, "threads": threads,
            "host": f"{platform.machine()}, {os.cpu_count()} logical CPUs",
            "port_elem_steps_per_s": r_port, "reference_elem_steps_per_s": r_ref,
            "port_over_reference": r_port / r_ref,
            "port_seconds": t_port, "reference_seconds": t_ref}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--box", default="60x60x12")
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--repeats", type=int, default=3)
    a = ap.parse_args()
    box = tuple(int(v) for v in a.box.lower().split("x"))
    out = measure(box, a.steps, a.warmup, a.repeats)
    (ORACLE / "ref_speed.json").write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out))


if __name__ == "__main__":
    main()
