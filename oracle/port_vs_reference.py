"""Times the oracle port (oracle/hobak_oracle.cpp) against the reference
built from its own sources (oracle/_ref/hobak_ref, oracle/ref/Makefile) on
the same scenes, side by side on this host, and writes
oracle/port_vs_reference.json.

Test infrastructure: the reference build exists only where the reference
sources do (an x86 host), so the GPU host's CPU baseline, which has to use
the port, reports this ratio beside its own figure.

    python oracle/port_vs_reference.py [--steps 20] [--threads 0]

Scenes: the 10^3 Kuhn cube (SNH E = 1e3, hanging under gravity) and the
16^3 compressed and twisted cube (SNH E = 1e4), BACKWARD_EULER_VELOCITY,
Jacobi PCG to 1e-8 (the reference's own preconditioner); per step the
reference's time is std::chrono around solve() in its harness and the port's
is the wall time of one oracle step.  The same number of OpenMP threads for
both."""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from hobakv1_gb300 import scenes  # noqa: E402
from oracle import oracle, refrun  # noqa: E402


def cpu_model() -> str:
    with open("/proc/cpuinfo") as f:
        for line in f:
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    return platform.machine()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--threads", type=int, default=0, help="0 = every core")
    args = ap.parse_args()
    if not refrun.available():
        sys.exit("reference build missing: make -C oracle/ref REF=<reference checkout>")
    threads = oracle.set_threads(args.threads)
    cases = [scenes.config1_scene(10), scenes.config2_scene(16, "snh")]
    rows = []
    for s in cases:
        r = refrun.run(s, args.steps, threads=threads)
        ref_ms = statistics.median(r["step_ms"].tolist())
        sim = oracle.Sim(s, precond=0)
        port = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            sim.step(1)
            port.append(1e3 * (time.perf_counter() - t0))
        x, _ = sim.state()
        xr = r["x"][-1]
        err = float(((x - xr) ** 2).sum() ** 0.5 / ((xr ** 2).sum() ** 0.5))
        rows.append({"scene": s.name, "tets": s.nt, "steps": args.steps, "reference_ms_per_step_p50": ref_ms,
                     "port_ms_per_step_p50": statistics.median(port), "speedup": ref_ms / statistics.median(port),
                     "rel_position_difference": err})
        print(rows[-1])
    out = {"host": cpu_model(), "threads": threads, "cases": rows,
           "port_speed_vs_reference": statistics.median(r["speedup"] for r in rows),
           "how": f"median over the cases of reference ms/step over port ms/step (p50 of {args.steps} steps each, "
                  f"{threads} OpenMP threads, Jacobi PCG to 1e-8), measured on {cpu_model()} by "
                  "oracle/port_vs_reference.py"}
    with open(os.path.join(HERE, "port_vs_reference.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
