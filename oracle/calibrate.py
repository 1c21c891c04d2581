"""Speed of the oracle's C restatement against the reference's own solvers, both built
here (``make -C oracle port ref``), on the same grid and steps.

The timed CPU baseline of the benchmark is the restatement (the reference's sources do
not travel to the GPU machine); this script states how fast the restatement is relative
to the reference's own -O3 build of HPC_solver (one thread) and omp_solver (all host
threads), by the difference of two runs (so that set-up is not counted).

    python oracle/calibrate.py [N] [steps]
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from oracle import port, ref  # noqa: E402


def hump(N):
    x = (np.arange(-2, N + 2) + 0.5) / N
    X, Y = np.meshgrid(x, x, indexing="ij")
    h = 1.0 + 0.1 * np.exp(-((X - 0.5) ** 2 + (Y - 0.5) ** 2) / 0.01)
    z = np.zeros_like(h)
    return h, z, z.copy(), z.copy()


def seconds(fn, steps):
    t0 = time.perf_counter()
    fn(1)
    t1 = time.perf_counter()
    fn(1 + steps)
    t2 = time.perf_counter()
    return (t2 - t1) - (t1 - t0)


def case(N, steps, one_thread):
    """One configuration, in a process whose OpenMP runtime started with the thread count
    (OMP_NUM_THREADS is read once, when the runtime starts)."""
    h, hu, hv, B = hump(N)
    dt = 0.5 * port.stable_dt(port.grid(N, N), h, hu, hv)
    solver = ref.SOLVER_HPC if one_thread else ref.SOLVER_OMP
    p = port.grid(N, N, threads=1 if one_thread else 0)
    t_port = seconds(lambda k: port.run(p, h, hu, hv, B, k, dt), steps)
    t_ref = seconds(lambda k: ref.run(N, N, h, hu, hv, B, k, dt, solver=solver), steps)
    a = port.run(p, h, hu, hv, B, 2, dt)
    b = ref.run(N, N, h, hu, hv, B, 2, dt, solver=solver)
    same = all(np.array_equal(x.view(np.uint64), y.view(np.uint64)) for x, y in zip(a[:3], b[:3]))
    return {"reference_solver": "HPC_solver" if one_thread else "omp_solver",
            "threads": int(os.environ.get("OMP_NUM_THREADS", "0")),
            "port_gcups": N * N * steps / t_port / 1e9,
            "reference_gcups": N * N * steps / t_ref / 1e9,
            "port_over_reference": t_ref / t_port, "bitwise_equal": same}


def main():
    N = int(sys.argv[1]) if len(sys.argv) > 1 else 1024
    steps = int(sys.argv[2]) if len(sys.argv) > 2 else 5
    if len(sys.argv) > 3:  # one case, in a child process
        print(json.dumps(case(N, steps, sys.argv[3] == "one")))
        return
    if not ref.available():
        print(json.dumps({"unavailable": "oracle/_ref not built (reference sources absent)"}))
        return
    cores = len(os.sched_getaffinity(0))
    out = {"grid": [N, N], "steps": steps, "host_threads": cores}
    for name, threads in (("one_thread", 1), ("all_threads", cores)):
        env = dict(os.environ, OMP_NUM_THREADS=str(threads), OMP_PROC_BIND="true",
                   OMP_PLACES="cores")
        r = subprocess.run([sys.executable, os.path.abspath(__file__), str(N), str(steps),
                            "one" if threads == 1 else "all"], env=env, capture_output=True,
                           text=True, check=True)
        out[name] = json.loads(r.stdout.strip().splitlines()[-1])
    print(json.dumps(out))


if __name__ == "__main__":
    main()
