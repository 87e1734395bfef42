"""Measures the shared-memory staging of the FP32 record-streamed evaluation kernel on the current
GPU and writes the table lagrbf_gb300/csrc/lgb_eval_tune.h (then rebuild).

The kernel streams a cell's record blocks through a ring of EVR_NB shared-memory stages of
`budget` floats each (TMA bulk copies, mbarrier completion).  For each stage count (a compile-time
constant: the library is rebuilt with -DEVR_NB=n) and each stage size (the LAGRBF_TMA_BUDGET
override, read at run time), the 3D RK4 workload (128^3 jittered lattice, ABC flow, 32^3 PU,
Wendland C2, FP32 evaluation) with `--np` uniform particles is advanced a few steps from a fresh
process and the event-timed evaluation launches are averaged; the fastest pair goes into the table.

    python -m lagrbf_gb300.tune_eval [--np N] [--out PATH]

The library is left built with the measured table's values when the tuner ends (it rebuilds with
no extra flags after writing the table).
"""
import argparse
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
TABLE = os.path.join(HERE, "csrc", "lgb_eval_tune.h")
STAGES = (2, 3, 4)
BUDGETS = (1024, 1536, 2048, 2560, 3072)

MEASURE = r"""
import json, sys
import numpy as np
sys.path.insert(0, %(root)r)
import lagrbf_gb300 as L
from lagrbf_gb300 import workloads as W
xd, fd, xp, opts = W.config_abc_3d(nlat=128, npu=32, np_=%(np)d, seed=3)
c = L.LagRBFCtx(**opts, advection=True, advection_scheme=2, advection_cfl=0.3, dt=5e-4, solve_method=1,
                eval_precision="fp32")
c.fill_data(xd, fd); c.fill_points(xp); c.interpolate_c()
t = 0.0
for _ in range(2):
    c.advect_resident(t, t + 5e-4); t += 5e-4
c.reset_stats(); c.set_profiling(True)
for _ in range(3):
    c.advect_resident(t, t + 5e-4); t += 5e-4
c.synchronize()
st = c.stats()
print(json.dumps({"eval_ms": st["eval_ms"] / max(st["eval_launches"], 1), "np": int(st["np_alive"])}))
"""


def build(flags):
    env = dict(os.environ, LAGRBF_NVCC_FLAGS=flags)
    subprocess.run([sys.executable, "-c", "import sys; sys.path.insert(0, %r); from lagrbf_gb300 import build; "
                    "build.build(force=True)" % ROOT], check=True, env=env, stdout=subprocess.DEVNULL)


def measure(budget, np_):
    env = dict(os.environ, LAGRBF_TMA_BUDGET=str(budget))
    out = subprocess.run([sys.executable, "-c", MEASURE % {"root": ROOT, "np": np_}], check=True, env=env,
                         stdout=subprocess.PIPE, text=True).stdout
    return json.loads(out.strip().splitlines()[-1])["eval_ms"]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--np", type=int, default=16_777_216)
    ap.add_argument("--out", default=TABLE)
    args = ap.parse_args()
    times = {}
    for nb in STAGES:
        build("-DEVR_NB=%d" % nb)
        for b in BUDGETS:
            times[(nb, b)] = measure(b, args.np)
            print(json.dumps({"stages": nb, "budget_floats": b, "eval_ms_per_launch": times[(nb, b)]}), flush=True)
    nb, b = min(times, key=times.get)
    lines = ["/*",
             " * lgb_eval_tune.h -- shared-memory staging of the FP32 record-streamed evaluation kernel,",
             " * measured by",
             " *     python -m lagrbf_gb300.tune_eval --np %d" % args.np,
             " * (event-timed evaluation launches of the 3D RK4 workload: 128^3 jittered lattice, ABC flow,",
             " * 32^3 PU, Wendland C2, %d uniform particles; ms per launch by stages x floats per stage):" % args.np]
    for s in STAGES:
        lines.append(" *   %d stages: %s" % (s, ", ".join("%d: %.2f" % (bb, times[(s, bb)]) for bb in BUDGETS)))
    lines += [" */",
              "#ifndef LGB_EVAL_TUNE_H",
              "#define LGB_EVAL_TUNE_H",
              "#define LGB_EVR_NB_TUNED %d" % nb,
              "#define LGB_TMA_BUDGET_TUNED %d" % b,
              "#endif", ""]
    with open(args.out, "w") as f:
        f.write("\n".join(lines))
    print("wrote %s (%d stages of %d floats)" % (args.out, nb, b))
    build("")


if __name__ == "__main__":
    main()
