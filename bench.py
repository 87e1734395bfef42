"""Benchmark: 3D RK4 RBF-PU advection throughput (particle-steps/s) on GB300.

Workload (default): 2,097,152 source nodes on a 128^3 jittered lattice in [0,1]^3 carrying the ABC
flow (A=B=C=1, X = 2 pi x), 32^3 PU patches (overlap 1.5 x spacing), Wendland C2 kernel, 16,777,216
uniform particles, RK4 with dt = 5e-4.  One step = one internal RK4 step of the reference's
interpolated advection loop over [t, t+dt] (3 stage evaluations + the "fields" evaluation, 4 particle
re-binnings, lazy patch set-up check, CFL reduction).  Inputs are seeded synthetic data (no dataset).

Legs:
  value      FP32-evaluation path, data/binning/factors resident in HBM (lagrbf_gpu_advect_resident)
  fp64       the plain FP64 path on the same context, and the FP32-vs-FP64 error after one step
  e2e        through the reference-facing C-ABI with host buffers, per step: fill_swarm(data),
             lagrbf_interpolation, lagrbf_output(coords, fields, pids), lagrbf_advect_interpolate
             (A_KSP: factors kept, coefficients re-solved each step, as the reference's reset implies)
  roofline   the evaluation kernel: algorithmic flops (counted on the device) / event-timed duration
  cpu_baseline / --impl reference: the reference algorithm on the host cores (oracle/cpu_baseline.py)

Run: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--np NP]
"""
import argparse
import faulthandler
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

T_START = time.perf_counter()


def log(msg):
    """Progress on stderr (the JSON result line alone goes to stdout)."""
    print("[bench %7.1fs] %s" % (time.perf_counter() - T_START, msg), file=sys.stderr, flush=True)


METRIC = "3D RK4 particle-steps/s (FP32 eval <=1e-6 vs FP64; plain FP64 alongside)"
DT = 5e-4


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--np", type=int, default=16_777_216, help="particles per GPU")
    ap.add_argument("--nlat", type=int, default=128)
    ap.add_argument("--npu", type=int, default=32)
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=0, help="0: same as --steps")
    ap.add_argument("--cpu-sample", type=int, default=256, help="particles per emulated rank")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--profile-only", action="store_true", help="setup + a few steps, for ncu")
    ap.add_argument("--quick", action="store_true", help="only the FP32 timed loop and the roofline pass")
    ap.add_argument("--profile-solve", action="store_true",
                    help="setup, reset_coefficients, one re-solve of every patch (kept factors), for ncu")
    ap.add_argument("--serve-jobs", type=int, default=60, help="jobs of the serving leg (0: skip it)")
    ap.add_argument("--uneven", type=int, default=1, help="run the uneven-mixture leg (0: skip it)")
    ap.add_argument("--uneven-only", default="", help="comma-separated schemes of the uneven leg (rk4, dopri, "
                    "dopri_per_particle) to run alone, printing that leg's JSON (for profiling it)")
    ap.add_argument("--eval-precision", default="fp32", choices=["fp32", "fp64"],
                    help="evaluation precision of the main context (fp64: the plain path, for profiling it)")
    ap.add_argument("--device-loop", type=int, default=1,
                    help="0: one graph launch per internal step instead of the device-side step loop "
                         "(ncu does not profile kernels inside graphs with conditional nodes)")
    ap.add_argument("--solve-method", type=int, default=1,
                    help="1: A_KSP (factors resident), 2: A_KSP_ASMB (re-factor, no factor storage)")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.samples = []
        self.proc = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 3 + i and "Active" in s[3 + i]
                          and "Not" not in s[3 + i]})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def eval_traffic_per_particle():
    """DRAM bytes (read + write) per particle of one evaluation launch, from the committed ncu
    capture of the evaluation kernel (profiles/k_eval_traffic.txt), or None."""
    p = os.path.join(ROOT, "profiles", "k_eval_traffic.txt")
    if not os.path.exists(p):
        return None, None
    with open(p) as f:
        for line in f:
            if line.startswith("dram_bytes_per_particle:"):
                return float(line.split(":", 1)[1]), "profiles/k_eval_traffic.txt"
    return None, None


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def workload(args, rank):
    from lagrbf_gb300 import workloads as W
    xd, fd, xp, opts = W.config_abc_3d(nlat=args.nlat, npu=args.npu, np_=args.np, seed=3)
    if rank:
        xp = W.uniform_points(args.np, 3, np.random.default_rng(4 + 1000 * rank))
    return xd, fd, xp, opts


def cpu_baseline(xd, fd, opts, args, nsteps=1):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import cpu_baseline as CB
    P = os.cpu_count() or 1
    r = CB.time_reference(xd, fd, args.npu, dict(opts, advection_scheme=2), P, args.cpu_sample, nsteps, DT)
    return r, P


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    xd, fd, _, opts = workload(args, 0)
    total_ps, total_s = 0, 0.0
    for _ in range(args.warmup if args.warmup < 2 else 1):
        cpu_baseline(xd, fd, opts, args, 1)
    for _ in range(args.steps):
        r, P = cpu_baseline(xd, fd, opts, args, 1)
        total_ps += r["particle_steps"]
        total_s += r["step_s"]
    v = total_ps / total_s
    sample = ("%d emulated MPI ranks (DMDA split of the 32^3 PU mesh, one-cell halo, rank-local data) x %d "
              "particles each, 1 RK4 step per bench step; oracle port compiled with the reference's flags"
              % (P, args.cpu_sample))
    line = {"metric": METRIC, "value": v, "unit": "particle-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total_s / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "abc3d: 128^3 lattice, ABC flow, 32^3 PU, Wendland C2, RK4 dt=5e-4",
                       "particles_per_rank_sample": args.cpu_sample, "ranks": P},
            "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": P, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_serving(njobs, workers=8, budget=150e9, sweep=(5.0, 10.0, 20.0, 40.0), sweep_jobs=30):
    """The serving leg: a seeded Poisson stream (200 jobs/s offered) of advection jobs on six
    datasets of 10K-2M nodes (30 % naming an already sent dataset), particle sets lognormal
    around 100K, 1-50 steps of RK1/RK2/RK4/DP45, served under a 150 GB budget; latency from
    submission to completion split into queue wait and service, aggregate particle-steps/s over the
    whole stream.  Then, with the datasets resident, streams of the same jobs (without their data)
    at lower offered rates: the highest rate whose median queue wait stays under 100 ms is reported
    as the sustainable rate."""
    from lagrbf_gb300 import workloads as W
    from lagrbf_gb300.serving import Server
    stream = W.serving_stream(np.random.default_rng(9), njobs=njobs, nd_range=(1e4, 2e6))
    srv = Server(hbm_budget_bytes=budget, nworkers=workers)

    def play(jobs):
        t0 = time.perf_counter()
        ids = []
        for when, job in jobs:
            while time.perf_counter() - t0 < when:
                time.sleep(0.0002)
            ids.append(srv.submit(**job))
        for i in ids:
            srv.wait(i)
        return time.perf_counter() - t0

    wall = play(stream)
    st = srv.stats()
    out = {"p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"],
           "queue_p50_ms": st["queue_p50_ms"], "queue_p99_ms": st["queue_p99_ms"],
           "service_p50_ms": st["service_p50_ms"], "service_p99_ms": st["service_p99_ms"],
           "jobs": st["completed"], "failed": st["failed"], "particle_steps_per_s": st["particle_steps"] / wall,
           "wall_s": wall, "offered_jobs_per_s": 200.0, "workers": workers, "hbm_budget_gb": budget / 1e9,
           "workload": "Poisson 200 jobs/s; 6 datasets 10K-2M nodes log-uniform (jittered lattice, 16-mode Fourier "
                       "field, ~70 nodes per PU cell), 30% reuse; particles lognormal median 100K in [1K, 4M]; "
                       "1-50 steps; RK1/RK2/RK4/DP45; FP32 evaluation; latency from submission"}
    resident = [dict((k, v) for k, v in job.items() if k not in ("data_coords", "data_values"))
                for _, job in stream[:sweep_jobs]]
    rates = []
    sustainable = None
    log("serving: stream done, rate sweep")
    for rate in sweep:
        log("serving: %g jobs/s" % rate)
        arr = np.cumsum(np.random.default_rng(11).exponential(1.0 / rate, size=len(resident)))
        srv.reset_stats()
        w = play(list(zip(arr.tolist(), resident)))
        s2 = srv.stats()
        rates.append({"offered_jobs_per_s": rate, "queue_p50_ms": s2["queue_p50_ms"],
                      "queue_p99_ms": s2["queue_p99_ms"], "service_p50_ms": s2["service_p50_ms"],
                      "p50_ms": s2["p50_ms"], "p99_ms": s2["p99_ms"],
                      "particle_steps_per_s": s2["particle_steps"] / w})
        if s2["queue_p50_ms"] < 100.0:
            sustainable = rate
    srv.close()
    out.update(rate_sweep=rates, sustainable_jobs_per_s=sustainable,
               rate_sweep_workload="the first %d jobs of the stream on their resident datasets, Poisson "
                                   "arrivals at each offered rate" % sweep_jobs)
    return out


def run_uneven(rk4_steps=3, dopri_steps=5, t_end=0.1, pp_budget_s=90.0, schemes=("rk4", "dopri", "dopri_per_particle"),
               device_loop=True):
    """The uneven configuration: 1M points (90 % from 8 Gaussians of widths 0.02-0.2, 10 % uniform),
    ABC flow, 8M particles from the same mixture, Wendland C2 on a uniform 160^3 PU mesh (largest
    patch 1,713 points, 2.3M non-empty patches).  Set-up time, then FP32-evaluation RK4 steps at
    the CFL step, Dormand-Prince steps (rtol 1e-6, atol 1e-9, the reference's global adapted step)
    over an interval of about `dopri_steps` of the step adapted by a first call, and per-particle
    adaptive Dormand-Prince (same tolerances) run towards t_end in intervals of t_end / 10 until
    t_end or pp_budget_s of wall time: accepted particle steps per second, sweeps, time reached."""
    import lagrbf_gb300 as L
    from lagrbf_gb300 import workloads as W
    xd, fd, xp, opts = W.config_uneven_3d()
    out = {"workload": "uneven: 1M-point Gaussian mixture + 10% uniform, ABC flow, 160^3 PU, Wendland C2, "
                       "8M particles from the mixture, FP32 evaluation"}
    for scheme, name in ((2, "rk4"), (3, "dopri"), (3, "dopri_per_particle")):
        if name not in schemes:
            continue
        pp = name == "dopri_per_particle"
        log("uneven: %s" % name)
        c = L.LagRBFCtx(**opts, advection=True, advection_scheme=scheme, advection_cfl=0.3, solve_method=1,
                        eval_precision="fp32", dt=DT, device_loop=device_loop,
                        petsc_options={"dopri_rtol": 1e-6, "dopri_atol": 1e-9, "dopri_per_particle": pp})
        c.synchronize()
        ts = time.perf_counter()
        c.fill_data(xd, fd); c.fill_points(xp); c.interpolate_c(); c.synchronize()
        if scheme == 2:
            st = c.stats()
            out.update(setup_s=time.perf_counter() - ts, max_patch=st["max_patch"],
                       patches_factored=st["patches_factored"])
        if pp:
            c.reset_stats()
            ts = time.perf_counter()
            t = 0.0
            while t < t_end - 1e-15 and time.perf_counter() - ts < pp_budget_s:
                c.advect_resident(t, t + t_end / 10)
                t += t_end / 10
            c.synchronize()
            el = time.perf_counter() - ts
            st = c.stats()
            out[name] = {"value": st["particle_steps"] / el, "unit": "accepted particle-steps/s",
                         "sweeps": st["steps"], "accepted_particle_steps": st["particle_steps"],
                         "t_reached": t, "t_end": t_end, "seconds": el, "np_alive": st["np_alive"]}
            del c
            continue
        t = 0.0
        c.advect_resident(t, t + 1e-5); t += 1e-5  # warm-up (and the first adapted step for DOPRI)
        c.synchronize()
        span = rk4_steps * DT if scheme == 2 else dopri_steps * c.stats()["dt"]
        c.reset_stats()
        ts = time.perf_counter()
        c.advect_resident(t, t + span)
        c.synchronize()
        el = time.perf_counter() - ts
        st = c.stats()
        out[name] = {"value": st["particle_steps"] / el, "unit": "particle-steps/s", "steps": st["steps"],
                     "dt_last": st["dt"], "seconds": el}
        del c
    return out


def run_precision_stress(np_=4_000_000, eps_h=1.0, steps=20):
    """The precision-stress configuration: 80^3 jittered lattice, Gaussian kernel with eps_r = eps_h/h
    (h the lattice spacing; eps_h = 1 is the configuration as stated), 16 seeded Fourier modes with
    amplitudes ~N(0,1)/k^2, 32^3 PU nodes, np_ uniform particles; the FP32-evaluation path against
    the all-FP64 path on the same data: max / RMS / pointwise relative error per component of the
    interpolated field, then (steps > 0) of the positions and fields after `steps` RK4 steps of
    dt = 5e-4; the patches' 1-norm condition estimates beside them, plus the FP64 interpolant
    against the exact field."""
    import lagrbf_gb300 as L
    from lagrbf_gb300 import workloads as W
    xd, fd, xp, opts = W.config_precision_3d(np_=np_)
    opts = dict(opts, shape_factor=opts["shape_factor"] * eps_h)
    res, kap = {}, None
    for prec in ("fp64", "fp32"):
        log("precision stress: eps_h %g, %s" % (eps_h, prec))
        c = L.LagRBFCtx(**opts, solve_method=1, eval_precision=prec, advection=steps > 0, advection_scheme=2,
                        advection_cfl=0.3, dt=DT)
        if prec == "fp64":
            c.set_condition_estimates(True)
        c.fill_data(xd, fd)
        c.fill_points(xp)
        c.interpolate_c()
        f = np.zeros((np_, 3))
        c.output(fvals=f)
        out = {"f0": f}
        if prec == "fp64":
            kap = c.condition()[1]
        if steps > 0:
            ts = time.perf_counter()
            for k in range(steps):
                c.advect_resident(k * DT, (k + 1) * DT)
            c.synchronize()
            out["seconds"] = time.perf_counter() - ts
            x = np.zeros((np_, 3)); f = np.zeros((np_, 3)); pid = np.zeros(np_, dtype=np.int64)
            c.output(coords=x, fvals=f, pidx=pid)
            out.update(x=x, f=f, alive=pid > 0)
        res[prec] = out
        del c
    mx, rms = relerr_stats(res["fp32"]["f0"], res["fp64"]["f0"])
    exact = W.fourier_field(xp, np.random.default_rng(7))
    ex_mx, ex_rms = relerr_stats(res["fp64"]["f0"], exact)
    line = {"workload": "80^3 jittered lattice, Gaussian eps_r = %g/h, 16 Fourier modes, 32^3 PU, %d particles"
                        % (eps_h, np_),
            "kappa1_max": kap["max"], "kappa1_median": kap["median"], "patches": kap["count"],
            "fp32_vs_fp64_max_rel_err": mx, "fp32_vs_fp64_rms_rel_err": rms,
            "fp32_vs_fp64_pointwise_rel_err": pointwise_relerr(res["fp32"]["f0"], res["fp64"]["f0"]),
            "fp64_vs_exact_max_rel_err": ex_mx, "fp64_vs_exact_rms_rel_err": ex_rms}
    if steps > 0:
        a, b = res["fp32"], res["fp64"]
        both = a["alive"] & b["alive"]
        travel = np.abs(b["x"][both] - xp[both]).max()
        dx = np.abs(a["x"][both] - b["x"][both])
        fmx, frms = relerr_stats(a["f"][both], b["f"][both])
        line["rk4_steps"] = {"steps": steps, "dt": DT, "same_alive": bool(np.array_equal(a["alive"], b["alive"])),
                             "alive_both": int(both.sum()), "pos_max_abs_diff": float(dx.max()),
                             "pos_rms_abs_diff": float(np.sqrt((dx ** 2).mean())),
                             "pos_max_diff_rel_to_max_travel": float(dx.max() / travel) if travel > 0 else None,
                             "field_max_rel_err": fmx, "field_rms_rel_err": frms,
                             "fp64_seconds": b["seconds"], "fp32_seconds": a["seconds"]}
    return line


def run_trajectory(xd, fd, xp, opts, nsteps=50):
    """FP32-evaluation vs plain FP64 trajectories: the same particles advanced nsteps RK4 steps
    (dt = 5e-4) by each path from the same start; position differences against the distance
    travelled, and the velocity (field) difference at the end."""
    import lagrbf_gb300 as L
    n = len(xp)
    pid = np.arange(1, n + 1, dtype=np.int64)
    c = L.LagRBFCtx(**opts, advection=True, advection_scheme=2, advection_cfl=0.3, dt=DT, solve_method=1,
                    eval_precision="fp32")
    c.fill_data(xd, fd)
    out = {}
    for prec in ("fp32", "fp64"):
        c.set_precision(prec == "fp32")
        c.fill_points(xp, pidx=pid)
        c.interpolate_c()
        t = 0.0
        for _ in range(nsteps):
            c.advect_resident(t, t + DT)
            t += DT
        x = np.zeros((n, 3)); f = np.zeros((n, 3)); p = np.zeros(n, dtype=np.int64)
        c.output(coords=x, fvals=f, pidx=p)
        out[prec] = (x, f, p)
    (x32, f32, p32), (x64, f64, p64) = out["fp32"], out["fp64"]
    alive = (p32 > 0) & (p64 > 0)
    dx = np.abs(x32[alive] - x64[alive])
    travel = np.linalg.norm(x64[alive] - xp[alive], axis=1)
    fmx, frms = relerr_stats(f32[alive], f64[alive])
    return {"particles": n, "steps": nsteps, "alive_both": int(alive.sum()), "same_alive": bool((p32 == p64).all()),
            "pos_max_abs_diff": float(dx.max()), "pos_rms_abs_diff": float(np.sqrt((dx ** 2).mean())),
            "pos_max_diff_rel_to_max_travel": float(dx.max() / travel.max()),
            "vel_max_rel_err": fmx, "vel_rms_rel_err": frms,
            "vel_pointwise_rel_err": pointwise_relerr(f32[alive], f64[alive])}


def pointwise_relerr(a, b, floor=1e-3):
    """max_p |a - b| / max(|b|, floor * max|b|), per component (floor keeps zeros of b finite)."""
    den = np.maximum(np.abs(b), floor * np.abs(b).max(axis=0))
    den[den == 0] = 1.0
    return [float(x) for x in (np.abs(a - b) / den).max(axis=0)]


def relerr_stats(a, b):
    den = np.abs(b).max(axis=0)
    den[den == 0] = 1.0
    mx = (np.abs(a - b).max(axis=0) / den)
    rms = np.sqrt(((a - b) ** 2).mean(axis=0)) / np.maximum(np.sqrt((b ** 2).mean(axis=0)), 1e-300)
    return [float(x) for x in mx], [float(x) for x in rms]


def main():
    faulthandler.enable()
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.uneven_only:
        print(json.dumps(run_uneven(schemes=tuple(args.uneven_only.split(",")), device_loop=bool(args.device_loop))))
        return 0
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as tdist
        torch.cuda.set_device(local)
        tdist.init_process_group("nccl")
        dist = tdist

    def barrier():
        if dist:
            dist.barrier()

    def allmax(x):
        if not dist:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def allsum(x):
        if not dist:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        return float(t.item())

    import lagrbf_gb300 as L
    cf = L.load_cfuncs()
    log("workload")
    xd, fd, xp, opts = workload(args, rank)
    npart = len(xp)
    log("set-up: %d nodes, %d particles" % (len(xd), npart))
    ctx = L.LagRBFCtx(**opts, advection=True, advection_scheme=2, advection_cfl=0.3, dt=DT,
                      solve_method=args.solve_method,
                      eval_precision=args.eval_precision, cuda_device=local, device_loop=bool(args.device_loop))
    # ---------------- setup (not timed in `value`) ----------------
    t0 = time.perf_counter()
    ctx.fill_data(xd, fd)
    ctx.fill_points(xp)
    ctx.interpolate_c()
    ctx.synchronize()
    setup_s = time.perf_counter() - t0
    st0 = ctx.stats()
    if args.profile_solve:
        ctx.reset_coefficients()
        ctx.set_profiling(True)
        ctx.reset_stats()
        ctx.interpolate_c()
        ctx.synchronize()
        sp = ctx.stats()
        print(json.dumps({"profile_solve": True, "setup_s": setup_s, "solve_ms": sp["factor_ms"],
                          "solve_fp64_tflops": sp["factor_flops"] / (sp["factor_ms"] * 1e-3) / 1e12,
                          "max_patch": sp["max_patch"], "patches": sp["npatch_setup"]}))
        return 0
    if args.profile_only:
        for s in range(max(args.steps, 1)):
            ctx.advect_resident(s * DT, (s + 1) * DT)
        ctx.synchronize()
        print(json.dumps({"profile_only": True, "setup_s": setup_s, "stats": ctx.stats()}))
        return 0
    log("set-up done in %.1f s; warm-up" % setup_s)
    t = 0.0
    for _ in range(args.warmup):
        ctx.advect_resident(t, t + DT)
        t += DT
    ctx.synchronize()
    # ---------------- timed FP32 loop ----------------
    ctx.reset_stats()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    ctx.synchronize()
    ts = time.perf_counter()
    for _ in range(args.steps):
        ctx.advect_resident(t, t + DT)
        t += DT
    ctx.synchronize()
    barrier()
    el = time.perf_counter() - ts
    clk = clocks.stop()
    st = ctx.stats()
    el_max = allmax(el)
    ps_total = allsum(st["particle_steps"])
    value = ps_total / el_max
    launches = st["launches"]
    log("timed loop: %.3g particle-steps/s" % value)
    # ---------------- roofline of the evaluation kernel (event-timed launches) ----------------
    ctx.reset_stats()
    ctx.set_profiling(True)
    nprof = min(3, args.steps)
    for _ in range(nprof):
        ctx.advect_resident(t, t + DT)
        t += DT
    ctx.synchronize()
    sp = ctx.stats()
    ctx.set_profiling(False)
    pk, pk_kind = peaks()
    fp32_peak = cf["lagrbf_gpu_fp32_peak_tflops"]()
    eval_tflops = sp["eval_flops"] / (sp["eval_ms"] * 1e-3) / 1e12 if sp["eval_ms"] > 0 else 0.0
    eval_gbs = sp["eval_bytes"] / (sp["eval_ms"] * 1e-3) / 1e9 if sp["eval_ms"] > 0 else 0.0
    tpp, tsrc = eval_traffic_per_particle()
    traffic = tpp * sp["np_alive"] if tpp else None
    roofline = {"bound": "fp32", "achieved": eval_tflops, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": eval_tflops / fp32_peak if fp32_peak > 0 else None, "traffic": traffic,
                "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch on a smaller "
                                   "case with the same per-cell densities, per particle, times this launch's "
                                   "particles (%s)" % tsrc) if tsrc else None,
                "kernel": "k_eval_rec<3,3,KER_C2> (PU evaluation from TMA-streamed record blocks)",
                "peak_source": "measured: FFMA-chain probe on this GPU in this run (lagrbf_gpu_fp32_peak_tflops)",
                "per_launch_ms": sp["eval_ms"] / max(sp["eval_launches"], 1),
                "flops_per_launch": sp["eval_flops"] / max(sp["eval_launches"], 1),
                "bytes_per_launch": sp["eval_bytes"] / max(sp["eval_launches"], 1),
                "hbm_achieved_gbs": eval_gbs, "hbm_peak_gbs": pk.get("hbm_gbs"),
                "hbm_frac": eval_gbs / pk["hbm_gbs"] if pk.get("hbm_gbs") else None, "hbm_peak_kind": pk_kind,
                "eval_share_of_step": (sp["eval_ms"] / nprof) / (1e3 * el / args.steps)}
    if args.quick:
        print(json.dumps({"quick": True, "value": value, "ms_per_step": 1e3 * el_max / args.steps,
                          "eval_ms_per_launch": roofline["per_launch_ms"], "frac": roofline["frac"],
                          "chunk_cap": st["chunk_cap"], "records": st["records"], "np": npart}))
        return 0
    log("FP32 vs FP64")
    # ---------------- FP32 vs FP64 error after one step from the same state ----------------
    def snapshot():
        x = np.zeros((npart, 3)); f = np.zeros((npart, 3)); p = np.zeros(npart, dtype=np.int64)
        ctx.output(coords=x, fvals=f, pidx=p)
        return x, f, p

    x_start, f_start, p_start = snapshot()
    alive = p_start > 0
    ctx.set_precision(False)
    ctx.fill_points(x_start[alive], values=f_start[alive], pidx=p_start[alive])
    ctx.advect_resident(t, t + DT)
    x64, f64, _ = snapshot()
    ctx.set_precision(True)
    ctx.fill_points(x_start[alive], values=f_start[alive], pidx=p_start[alive])
    ctx.advect_resident(t, t + DT)
    x32, f32, _ = snapshot()
    err_max, err_rms = relerr_stats(f32, f64)
    err_pw = pointwise_relerr(f32, f64)
    pos_err = float(np.abs(x32 - x64).max())
    log("FP64 steps")
    # ---------------- plain FP64 path throughput ----------------
    ctx.set_precision(False)
    ctx.reset_stats()
    ctx.synchronize()
    ts = time.perf_counter()
    for _ in range(args.fp64_steps):
        ctx.advect_resident(t, t + DT)
        t += DT
    ctx.synchronize()
    el64 = allmax(time.perf_counter() - ts)
    value64 = allsum(ctx.stats()["particle_steps"]) / el64
    # the FP64 evaluation kernel against the FP64 pipe (event-timed launches of one profiled step)
    ctx.reset_stats()
    ctx.set_profiling(True)
    ctx.advect_resident(t, t + DT)
    t += DT
    ctx.synchronize()
    sp64 = ctx.stats()
    ctx.set_profiling(False)
    fp64_peak = cf["lagrbf_gpu_fp64_peak_tflops"]()
    e64 = sp64["eval_flops"] / (sp64["eval_ms"] * 1e-3) / 1e12 if sp64["eval_ms"] > 0 else 0.0
    roofline64 = {"bound": "fp64", "achieved": e64, "peak": fp64_peak, "unit": "TFLOP/s",
                  "frac": e64 / fp64_peak if fp64_peak > 0 else None,
                  "kernel": "k_eval<double,3,3,1,KER_GENERIC> (PU evaluation, FP64 gather path)",
                  "peak_source": "measured: DFMA-chain probe on this GPU in this run (lagrbf_gpu_fp64_peak_tflops)",
                  "per_launch_ms": sp64["eval_ms"] / max(sp64["eval_launches"], 1),
                  "flops_per_launch": sp64["eval_flops"] / max(sp64["eval_launches"], 1)}
    ctx.set_precision(True)
    log("end to end")
    # ---------------- end to end through the reference-facing C-ABI, host buffers ----------------
    ke = args.e2e_steps or args.steps
    xo = np.zeros((npart, 3)); fo = np.zeros((npart, 3)); po = np.zeros(npart, dtype=np.int64)
    ctx.fill_points(x_start[alive], values=f_start[alive], pidx=p_start[alive])
    h2d = fd.nbytes  # the coordinates are the same every step: compared on the host, not sent again
    d2h = xo.nbytes + fo.nbytes + po.nbytes
    fd_alt = (fd, fd * (1.0 + 1e-6))  # the nodal field changes every step, as in a coupled run
    for k in range(args.warmup):  # untimed warm-up steps (first touch of the caller's output arrays)
        ctx.fill_data(xd, fd_alt[k % 2])
        ctx.interpolate_c()
        ctx.output(coords=xo, fvals=fo, pidx=po)
        ctx.advect_interpolate_c(t, t + DT)
        t += DT
    ctx.reset_stats()
    barrier()
    ts = time.perf_counter()
    phase = {"fill_swarm": 0.0, "interpolation": 0.0, "output": 0.0, "advect_interpolate": 0.0}
    for k in range(ke):
        # every call returns after its stream has drained, so the host clock splits the step
        t0 = time.perf_counter()
        ctx.fill_data(xd, fd_alt[k % 2])
        t1 = time.perf_counter()
        ctx.interpolate_c()
        t2 = time.perf_counter()
        ctx.output(coords=xo, fvals=fo, pidx=po)
        t3 = time.perf_counter()
        ctx.advect_interpolate_c(t, t + DT)
        t4 = time.perf_counter()
        phase["fill_swarm"] += t1 - t0
        phase["interpolation"] += t2 - t1
        phase["output"] += t3 - t2
        phase["advect_interpolate"] += t4 - t3
        t += DT
    ctx.synchronize()
    barrier()
    ele = allmax(time.perf_counter() - ts)
    phase_ms = {kk: 1e3 * v / max(ke, 1) for kk, v in phase.items()}
    e2e = allsum(ctx.stats()["particle_steps"]) / ele
    # ---------------- FP32 vs FP64 trajectories over 50 steps (1M-particle sample) ----------------
    trajectory = None
    if rank == 0 and world == 1 and args.serve_jobs > 0:
        log("trajectories")
        trajectory = run_trajectory(xd, fd, xp[:1 << 20], opts)
    # ---------------- precision stress (Gaussian, small shape parameter) ----------------
    precision = None
    if rank == 0 and world == 1 and args.serve_jobs > 0:
        log("precision stress")
        precision = run_precision_stress()
        precision["flattened"] = run_precision_stress(np_=250_000, eps_h=0.35, steps=0)
    # ---------------- serving loop: Poisson stream of mixed advection jobs ----------------
    uneven = None
    if rank == 0 and world == 1 and args.uneven:
        log("uneven")
        uneven = run_uneven()
    serve = None
    if rank == 0 and world == 1 and args.serve_jobs > 0:
        log("serving")
        serve = run_serving(args.serve_jobs)
    # ---------------- CPU baseline on the host cores ----------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        log("CPU baseline")
        try:
            r, P = cpu_baseline(xd, fd, opts, args, 1)
            cpu = {"value": r["particle_steps"] / r["step_s"], "unit": "particle-steps/s", "cores": P, "kind": "port",
                   "sample": "%d emulated MPI ranks x %d particles, 1 RK4 step, rank-local data (~%d points) and "
                             "patches; oracle port with the reference's compiler flags" % (P, args.cpu_sample,
                                                                                            r["local_data"])}
        except Exception as e:  # the baseline is reported, not required
            cpu = {"value": None, "error": str(e)[:200]}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": "abc3d: %d^3 jittered lattice (%d nodes), ABC flow, %d^3 PU patches, Wendland C2, "
                                   "%d particles/GPU, RK4 dt=%g" % (args.nlat, len(xd), args.npu, args.np, DT),
                       "eval": "FP32 evaluation, FP64 factorisation and weight normalisation",
                       "solve_method": {1: "A_KSP (factors resident)", 2: "A_KSP_ASMB (re-factor per solve)"}
                       .get(args.solve_method, str(args.solve_method)),
                       "l2": "inputs larger than L2 (particle state %.1f GB)" % (npart * 8 * 3 * 12 / 1e9),
                       "parallelism": "replicas x%d (particles sharded, data replicated)" % world,
                       "setup_s": setup_s, "patches_factored": st0["patches_factored"],
                       "max_patch": st0["max_patch"], "work_unit": st["chunk_cap"],
                       "staging": "TMA bulk copies of precomputed record blocks" if st["records"] else "gather"},
            "fp64": {"value": value64, "unit": "particle-steps/s", "steps": args.fp64_steps, "roofline": roofline64,
                     "fp32_speedup": value / value64 if value64 > 0 else None,
                     "fp32_vs_fp64_max_rel_err": err_max, "fp32_vs_fp64_rms_rel_err": err_rms,
                     "fp32_vs_fp64_pointwise_rel_err": err_pw, "fp32_vs_fp64_max_abs_pos_err": pos_err,
                     "trajectory_50_steps": trajectory,
                     "err_definition": "per component: max_p|a-b| / max_p|b|, RMS(a-b)/RMS(b), and pointwise "
                                       "max_p |a-b| / max(|b|, 1e-3 max|b|); fields after 1 step"},
            "e2e": {"value": e2e, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": ke, "phase_ms_per_step": phase_ms,
                    "path": "fill_swarm(data: same coordinates, compared word for word on the host and not "
                                         "sent again; nodal values changing every step) + lagrbf_interpolation "
                                         "(all patch coefficients re-solved) + lagrbf_output + "
                                         "lagrbf_advect_interpolate, host numpy buffers"},
            "with_setup": {"value": ps_total / el_max * (50 * el_max / args.steps) /
                           (setup_s + 50 * el_max / args.steps), "unit": "particle-steps/s", "steps": 50,
                           "definition": "50 RK4 steps including the one-time set-up (binning, factorisation, "
                                         "first solve): particles x 50 / (setup_s + 50 x the timed step)"},
            "roofline": roofline, "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches, "serve": serve,
            "precision_stress": precision, "uneven": uneven,
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
