#!/usr/bin/env python
"""Benchmark: ms per design iteration of spline topology optimisation.

Workload: half-MBB beam on a 256x128x128 voxel grid (~12.7M DOFs), E = 1e6,
nu = 0.4, SIMP p = 3, rho_min = 1e-3, B-spline lattice 65x33x33 (order 3),
coefficients start at 0.4, volume fraction 0.4, filter radius 2, OC damp 0.5 /
move 0.03; each step is one full design iteration (Galerkin operator update,
solve to FP64 relative residual 1e-6 warm-started from the previous step,
compliance, sensitivity, filter, spline adjoint, OC bisection).  Synthetic
boundary conditions (see topoptspline3d_gb300/workloads.py).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

N > 1 runs one independent replica per GPU (the path has no cross-GPU exchange).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "ms/design-iter @256x128x128, rel-res 1e-6: mixed vs FP64 MG-PCG, 1 GB300"
# the same design iterations with the trained network correcting every V-cycle
METRIC_LEARNED = "ms/design-iter @256x128x128, rel-res 1e-6: mixed+learned vs FP64 MG-PCG, 1 GB300"


def metric_for(args):
    if args.case == "mbb" and args.size == "256x128x128":
        return METRIC
    return f"ms/design-iter @{args.size} ({args.case}), rel-res 1e-6: mixed vs FP64 MG-PCG, 1 GB300"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--size", default=None, help="grid, e.g. 256x128x128 (default per case)")
    ap.add_argument("--case", default="mbb", choices=["mbb", "ellipsoids", "loads", "designs", "robust"],
                    help="mbb: half-MBB beam (headline); ellipsoids: large union-of-ellipsoids design; "
                         "loads: 16 load cases in one multi-right-hand-side solve; designs: 32 independent "
                         "designs of uneven size at once; robust: worst-case-load design iterations")
    ap.add_argument("--smoother", default="chebyshev", choices=["chebyshev", "gs"])
    ap.add_argument("--fp64-steps", type=int, default=2, help="FP64 MG-PCG comparison steps")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default solver schedule and tiles")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-preconditioner ablation")
    ap.add_argument("--retune-every", type=int, default=None,
                    help="every N timed design iterations, try the FP32 inner caps 1, 2, 4, 6 on the next four and "
                         "keep the fastest (default: 25 for --case ellipsoids, off otherwise)")
    ap.add_argument("--profile-iteration", action="store_true",
                    help="run exactly one mixed design iteration and exit (for ncu captures)")
    ap.add_argument("--schedule", default=None,
                    help="inner,pre,degree,tz32,tz64[,lo[,inner_rtol]]: use this mixed-solver schedule (lo: lower "
                         "end of the Chebyshev interval, a fraction of lambda_max; inner_rtol: tolerance of the FP32 "
                         "inner CG) and these tiles instead of autotuning (e.g. the values an earlier run's autotune "
                         "chose)")
    ap.add_argument("--profile-solve-steps", type=int, default=0,
                    help="with --profile-iteration: stop the solve after this many outer CG steps")
    ap.add_argument("--coarse-every", type=int, default=1,
                    help="recompute the coarsest dense inverse at every K-th operator update only "
                         "(topo_set_coarse_refresh; 1, the default, is each update as in the reference)")
    ap.add_argument("--no-graphs", action="store_true",
                    help="launch every kernel on its own (no CUDA graphs); with --profile-iteration this lists the "
                         "kernels the device-side loops run inside graphs")
    ap.add_argument("--profile-fp64", action="store_true",
                    help="with --profile-iteration: the design iterations run plain FP64 MG-PCG (FP64 operators, "
                         "native FP64 fine operator), the comparison path, instead of the mixed solve")
    ap.add_argument("--profile-warmup", type=int, default=0,
                    help="with --profile-iteration: run this many design iterations first and open the profiler's "
                         "capture range (cudaProfilerStart) only around the last one, for ncu --profile-from-start off")
    return ap.parse_args()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=ws)
        pg = dist
    return ws, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allmax(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for k, n in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(case, nx, ny, nz):
    from topoptspline3d_gb300 import workloads
    if case == "ellipsoids":
        return workloads.large_ellipsoids(nx, ny, nz)
    return workloads.half_mbb(nx, ny, nz, lattice=(nx // 4 + 1, ny // 4 + 1, nz // 4 + 1))


def make_problem(nx, ny, nz, device, op_precision, case="mbb"):
    from topoptspline3d_gb300 import capi
    wl = make_workload(case, nx, ny, nz)
    p = capi.Problem(nx, ny, nz, device=device, eactive=wl.eactive)
    p.set_bc(wl.fixed, wl.loads)
    bmin, bmax = wl.spline_box()
    p.set_spline(wl.order, wl.partition, bmin, bmax)
    p.put("coeff", np.full(p.num_coeffs(), wl.coeff0))
    p.coeff_to_density()
    p.set_operator_precision(op_precision)
    return wl, p


class InnerTuner:
    """Online choice of the FP32 inner-iteration cap over a long run.  The
    autotuner picks the schedule on an early design; as the design sharpens,
    the best number of FP32 CG iterations per outer step grows.  Every `every`
    design iterations the next four run with inner caps 1, 2, 4 and 6 (the other
    schedule fields as tuned), and the cap of the fastest solve is kept.  These
    are ordinary design iterations of the run, timed with the rest.  The chosen
    schedule per step is recorded so that a second pass can replay it."""

    CAPS = (1, 2, 4, 6)

    def __init__(self, opts, every):
        self.opts, self.every = dict(opts), every
        self.trial = {}
        self.used = []

    def opts_for(self, k):
        ph = k % self.every if self.every else -1
        if self.every and k >= self.every and ph < len(self.CAPS):
            o = dict(self.opts, inner_max=self.CAPS[ph])
        else:
            o = dict(self.opts)
        self.used.append(o)
        return o

    def report(self, k, st):
        ph = k % self.every if self.every else -1
        if not (self.every and k >= self.every and ph < len(self.CAPS)):
            return
        self.trial[self.CAPS[ph]] = st["solve_ms"]
        if ph == len(self.CAPS) - 1:
            self.opts["inner_max"] = min(self.trial, key=self.trial.get)
            self.trial = {}


def solve_opts(mode, smoother):
    from topoptspline3d_gb300 import capi
    return dict(mode=mode, smoother=capi.SMOOTH_CHEBYSHEV if smoother == "chebyshev" else capi.SMOOTH_GS,
                pre=2, post=2, rtol=1e-6, max_iter=300, inner_max=4, inner_rtol=0.1, cheb_degree=2)


def load_traffic():
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


def cpu_baseline(nx, ny, nz, threads_note=""):
    """One oracle design iteration (FP64 MG-PCG, GS V(2,2), rel-res 1e-6) on the host cores."""
    from oracle.oracle import Oracle, build_oracle
    from topoptspline3d_gb300 import workloads
    build_oracle()
    wl = workloads.half_mbb(nx, ny, nz, lattice=(nx // 4 + 1, ny // 4 + 1, nz // 4 + 1))
    o = Oracle(nx, ny, nz)
    o.set_bc(wl.fixed, wl.loads)
    bmin, bmax = wl.spline_box()
    o.set_spline(wl.order, wl.partition, bmin, bmax)
    o.put("coeff", np.full(o.num_coeffs(), wl.coeff0))
    o.coeff_to_density()
    t0 = time.perf_counter()
    o.update_operators()
    it, rr = o.pcg(2, 2, 1e-6, 300, 0)
    c = o.compliance()
    o.sensitivity()
    o.filter(2.0)
    o.spline_adjoint()
    o.oc_update(wl.vgoal)
    dt = (time.perf_counter() - t0) * 1e3
    return dt, it, rr, c


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-300))


def compliance_vs_oracle(p, wl, opts):
    """The GPU mixed solve against the FP64 CPU oracle solved to 1e-10 on the same
    final design (operators rebuilt on both sides): compliance, displacements,
    filtered sensitivities and coefficient sensitivities, as relative errors
    (2-norm for the fields).  The GPU solve stops at FP64 rel-res 1e-6, so U
    and the sensitivities carry that solve's error; the compliance target is
    1e-6."""
    from oracle.oracle import Oracle, build_oracle
    from topoptspline3d_gb300 import capi
    build_oracle()
    coeff = p.get("coeff")
    p.coeff_to_density()
    p.update_operators()
    p.put("u", np.zeros(3 * p.nv))
    s = p.solve(**opts)
    c_gpu = p.compliance()
    o = Oracle(wl.nx, wl.ny, wl.nz, eactive=wl.eactive)
    o.set_bc(wl.fixed, wl.loads)
    bmin, bmax = wl.spline_box()
    o.set_spline(wl.order, wl.partition, bmin, bmax)
    o.put("coeff", coeff)
    o.coeff_to_density()
    o.update_operators()
    t0 = time.perf_counter()
    it, rr = o.pcg(2, 2, 1e-10, 400, 0)
    c_o = o.compliance()
    solve_s = time.perf_counter() - t0
    u_err = _rel(p.get("u"), o.get("u"))
    fields = {}
    for q in (p, o):
        q.sensitivity()
        q.filter(wl.filter_radius)
    fields["sens_filtered"] = _rel(p.get("sens"), o.get("sens"))
    for q in (p, o):
        q.spline_adjoint()
    fields["csens"] = _rel(p.get("csens"), o.get("csens"))
    rel_err = abs(c_gpu - c_o) / abs(c_o)
    return {"compliance_gpu_mixed": c_gpu, "compliance_oracle_fp64": c_o, "rel_err": rel_err,
            "u_rel_err": u_err, "sens_filtered_rel_err": fields["sens_filtered"],
            "csens_rel_err": fields["csens"], "compliance_within_1e-6": bool(rel_err <= 1e-6),
            "gpu_relres": s["relres"], "oracle_relres": rr, "oracle_pcg_its": it, "oracle_solve_s": solve_s}


def learned_ablation(p, wl, opts):
    """Learned preconditioner at this grid: harvest 20k residual -> error crops
    (32^3; 128 from each of 8 iterates per solve) from mixed solves on 20 seeded
    smoothed random densities, 1000 Adam steps, then the same solve (one FP32
    V-cycle per outer step) with and without the network on an unseen density.
    Restores the design state afterwards."""
    from topoptspline3d_gb300 import capi, workloads
    rho0 = p.get("rho")
    u0 = p.get("u")
    nx, ny, nz = wl.nx, wl.ny, wl.nz
    p.unet_enable(11)
    p.unet_dataset_reserve(20480, crop=32, crops_per_iterate=128)
    base = dict(opts)
    base.update(inner_max=1, learned=0)
    t0 = time.perf_counter()
    for i in range(20):
        p.put("rho", workloads.random_density(nx, ny, nz, 3000 + i))
        p.update_operators()
        p.put("u", np.zeros(3 * p.nv))
        p.solve(**dict(base, learned=2, rtol=1e-8, max_iter=400), check=False)
    harvest_s = time.perf_counter() - t0
    n = p.unet_dataset_size()
    split = int(0.85 * n)
    t0 = time.perf_counter()
    fit0 = p.unet_train(20, batch=8, lo=0, hi=split, update=False, seed=7)
    p.unet_train(1000, batch=8, lr=1e-3, lo=0, hi=split, seed=6)
    train_s = time.perf_counter() - t0
    fit = p.unet_train(20, batch=8, lo=0, hi=split, update=False, seed=7)
    held = p.unet_train(20, batch=8, lo=split, hi=n, update=False, seed=5)
    p.put("rho", workloads.random_density(nx, ny, nz, 3999))
    p.update_operators()
    res = {}
    for name, lr in (("plain", 0), ("learned", 1)):
        p.put("u", np.zeros(3 * p.nv))
        st = p.solve(**dict(base, learned=lr), check=False)
        res[name] = {"iterations": st["iterations"], "ms": st["ms"], "relres": st["relres"],
                     "applied": st["learned_applied"], "fallback": st["learned_fallback"]}
    # the network's 3x3x3 convolutions on each kernel, same weights: 200 training
    # steps (forward, backward, Adam; one host synchronisation per step), 200
    # forward-only evaluations, and the learned solve above
    conv = {}
    prm = p.unet_params()
    for kname, kind in (("tcgen05", capi.CONV_TCGEN05), ("mma_sync", capi.CONV_MMA_SYNC)):
        p.unet_set_conv_kernel(kind)
        p.unet_set_params(prm)
        t0 = time.perf_counter()
        p.unet_train(200, batch=8, lr=1e-4, lo=0, hi=split, seed=3)
        t_train = time.perf_counter() - t0
        t0 = time.perf_counter()
        p.unet_train(200, batch=8, lo=0, hi=split, update=False, seed=3)
        t_eval = time.perf_counter() - t0
        p.unet_set_params(prm)
        p.put("u", np.zeros(3 * p.nv))
        st = p.solve(**dict(base, learned=1), check=False)
        conv[kname] = {"train_ms_per_step": 1e3 * t_train / 200, "forward_ms_per_batch": 1e3 * t_eval / 200,
                       "learned_solve_ms": st["ms"], "learned_solve_iterations": st["iterations"]}
    p.unet_set_conv_kernel(capi.CONV_TCGEN05)
    p.unet_set_params(prm)
    p.put("rho", rho0)
    p.update_operators()
    p.put("u", u0)
    return {"crops": n, "harvest_s": harvest_s, "train_steps": 1000, "train_s": train_s,
            "loss_train_crops": [fit0, fit], "loss_heldout_density": held, "solve_unseen_density": res,
            "conv_kernels": conv}


def mixed_learned_steps(p, ckpt, schedules, oc, ms_mixed, ms_fp64):
    """The timed region's design iterations once more from its start state (the
    checkpoint), with the trained network correcting every FP32 V-cycle of the
    mixed solve (learned = 1: energy-optimal amount, stagnation fallback, FP64
    residual judging every solve): the mixed + learned configuration of the
    headline comparison, measured and reported beside the mixed solve without
    the network."""
    p.checkpoint_load(ckpt)
    p.timer_start()
    st = [p.design_iteration(solve=dict(o, learned=1), oc=oc) for o in schedules]
    ms = p.timer_stop() / len(schedules)
    p.checkpoint_load(ckpt)
    return {"metric": METRIC_LEARNED, "ms_per_step": ms, "unit": "ms/design-iter",
            "outer_iterations": [s["iterations"] for s in st], "relres": max(s["relres"] for s in st),
            "vcycles_corrected": [s["learned_applied"] for s in st],
            "fallback": [s["learned_fallback"] for s in st],
            "speedup_vs_fp64_mgpcg": (ms_fp64 / ms) if ms_fp64 else None, "vs_mixed": ms / ms_mixed,
            "note": "same design iterations and schedules as the timed region, network applied after every "
                    "FP32 V-cycle; the headline value runs them without the network, which is faster"}


def run_reference(args, nx, ny, nz, ws, rank):
    if rank != 0:
        return
    from oracle.oracle import Oracle, build_oracle
    from topoptspline3d_gb300 import workloads
    build_oracle()
    wl = workloads.half_mbb(nx, ny, nz, lattice=(nx // 4 + 1, ny // 4 + 1, nz // 4 + 1))
    o = Oracle(nx, ny, nz)
    o.set_bc(wl.fixed, wl.loads)
    bmin, bmax = wl.spline_box()
    o.set_spline(wl.order, wl.partition, bmin, bmax)
    o.put("coeff", np.full(o.num_coeffs(), wl.coeff0))
    o.coeff_to_density()

    def step():
        o.update_operators()
        o.pcg(2, 2, 1e-6, 300, 0)
        o.compliance()
        o.sensitivity(); o.filter(2.0); o.spline_adjoint(); o.oc_update(wl.vgoal)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    ms = (time.perf_counter() - t0) * 1e3 / args.steps
    cores = os.cpu_count()
    out = {"impl": "reference", "metric": METRIC, "value": ms, "unit": "ms/design-iter", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"half-MBB {nx}x{ny}x{nz} spline OC design iteration", "grid": [nx, ny, nz],
                      "solver": "FP64 MG-PCG (GS V(2,2)) rel-res 1e-6", "parallelism": "host cores"},
           "cpu_baseline": {"value": ms, "unit": "ms/design-iter", "cores": cores, "kind": "port",
                            "sample": f"{args.steps} full design iterations of the FP64 CPU restatement "
                                      f"(the reference has no CPU path; its GPU code needs CUDA 11 and "
                                      f"unavailable libraries)"},
           "e2e": {"value": ms, "unit": "ms/design-iter", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_loads(args, rank):
    """16 load cases on the 192x96x96 cantilever: one multi-right-hand-side solve
    (every V-cycle launch serves all loads) against 16 single solves."""
    from topoptspline3d_gb300 import capi, workloads
    nx, ny, nz = (int(v) for v in args.size.lower().split("x"))
    nrhs = 16
    wl = workloads.cantilever(nx, ny, nz, lattice=(nx // 4 + 1, ny // 4 + 1, nz // 4 + 1))
    p = capi.Problem(nx, ny, nz)
    p.set_bc(wl.fixed, wl.loads)
    bmin, bmax = wl.spline_box()
    p.set_spline(wl.order, wl.partition, bmin, bmax)
    p.put("coeff", np.full(p.num_coeffs(), wl.coeff0))
    p.coeff_to_density()
    p.set_operator_precision(2)
    p.update_operators()
    F = workloads.patch_loads(nx, ny, nz, nrhs, seed0=1000, patch=8)
    p.multi_reserve(nrhs)
    kw = dict(pre=1, post=1, rtol=1e-6, max_iter=300, inner_rtol=0.05)
    # schedule: one V-cycle or 4 / 6 batched FP32 CG iterations per outer step,
    # lower end of the Chebyshev interval 0.3 or 0.1 lambda_max: the fastest on
    # one solve of the batch each (untimed set-up), for both forms below
    trial = {}
    for inner in (1, 4, 6):
        for lo in (0.3, 0.1):
            trial[(inner, lo)] = p.solve_multi(F, cheb_lo=lo, inner_max=inner, **kw)[1]["ms"]
    kw["inner_max"], kw["cheb_lo"] = min(trial, key=trial.get)
    for _ in range(args.warmup):
        p.solve_multi(F, **kw)
    ms_multi, its = [], []
    for _ in range(args.steps):
        U, st, rr = p.solve_multi(F, **kw)
        ms_multi.append(st["ms"])
        its.append(st["iterations"])
    single = dict(mode=capi.SOLVE_MIXED, smoother=capi.SMOOTH_CHEBYSHEV, pre=1, post=1, rtol=1e-6, max_iter=300,
                  inner_max=kw["inner_max"], inner_rtol=kw["inner_rtol"], cheb_lo=kw["cheb_lo"])
    ms_single = []
    for k in range(nrhs):
        p.put("f", F[k])
        p.put("u", np.zeros(3 * p.nv))
        ms_single.append(p.solve(**single)["ms"])
    comp = [float(F[k] @ U[k]) for k in range(nrhs)]
    ms = statistics.median(ms_multi)
    out = {"metric": f"ms per {nrhs}-load solve @{nx}x{ny}x{nz}, rel-res 1e-6 (multi-RHS V-cycle), 1 GB300",
           "value": ms, "unit": "ms", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32 multigrid / f64 CG",
           "data": "synthetic",
           "config": {"workload": f"cantilever {nx}x{ny}x{nz}, {nrhs} seeded 8x8 patch loads",
                      "solver": f"per-load FP64 flexible CG + {kw['inner_max']} batched FP32 CG its (to "
                                f"{kw['inner_rtol']:g}) with a Chebyshev V(1,1) degree 2 on [{kw['cheb_lo']:g}, 1.1] "
                                f"lambda_max",
                      "schedule_trials_ms": {f"inner {k[0]}, lo {k[1]:g}": v for k, v in trial.items()}},
           "sequential_single_solves_ms": sum(ms_single), "speedup_vs_sequential": sum(ms_single) / ms,
           "iterations": its, "max_relres": float(max(rr)), "worst_case_compliance": max(comp),
           "worst_case_load": int(np.argmax(comp))}
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_robust(args, rank):
    """Worst-case (robust) compliance design iterations, the reference's default
    optimisation (optimization/optimization.cpp:673-767): each step rebuilds the
    operators, finds the worst unit load on the x = nx face (any direction) by
    block Rayleigh-Ritz over multi-RHS solves, then runs sensitivity, filter,
    spline adjoint and OC on that load.  The same steps with a single load
    vector (block 1, the reference's power method with full solves) are timed
    after it."""
    from topoptspline3d_gb300 import capi, workloads
    nx, ny, nz = (int(v) for v in args.size.lower().split("x"))
    wl = workloads.cantilever(nx, ny, nz, lattice=(nx // 4 + 1, ny // 4 + 1, nz // 4 + 1))
    p = capi.Problem(nx, ny, nz)
    p.set_bc(wl.fixed, wl.loads)
    bmin, bmax = wl.spline_box()
    p.set_spline(wl.order, wl.partition, bmin, bmax)
    p.put("coeff", np.full(p.num_coeffs(), wl.coeff0))
    p.coeff_to_density()
    vid = np.array([nx + (nx + 1) * (y + (ny + 1) * z) for z in range(nz + 1) for y in range(ny + 1)])
    p.set_load_region(vid, np.tile([1.0, 0.0, 0.0], (len(vid), 1)))
    kw = dict(free_direction=True, tol=1e-4, rtol=1e-6, max_iter=200, seed=7, cheb_lo=0.1)

    def step(block):
        p.update_operators()
        st = p.worst_compliance(block=block, **kw)
        p.sensitivity()
        p.filter(wl.filter_radius)
        p.spline_adjoint()
        p.oc_update(wl.vgoal)
        return st

    for _ in range(args.warmup):
        step(16)
    state = (p.get("coeff"), p.get("rho"))
    p.sync()
    p.timer_start()
    sts = [step(16) for _ in range(args.steps)]
    ms = p.timer_stop() / args.steps
    p.put("coeff", state[0])
    p.coeff_to_density()
    p.timer_start()
    st1 = [step(1) for _ in range(min(args.steps, 3))]
    ms1 = p.timer_stop() / len(st1)
    out = {"metric": f"ms per robust design iteration @{nx}x{ny}x{nz} (worst unit load on the x={nx} face), "
                     f"1 GB300",
           "value": ms, "unit": "ms/design-iter", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32 multigrid / f64 CG", "data": "synthetic",
           "config": {"workload": f"cantilever {nx}x{ny}x{nz}, load region x={nx} face ({len(vid)} vertices, "
                                  f"any direction: {3 * len(vid)} load coordinates)",
                      "method": "block Rayleigh-Ritz, 16 load vectors, multi-RHS mixed solves warm-started, "
                                "change 1e-4, final rel-res 1e-6"},
           "worst_compliance": [s["compliance"] for s in sts], "second": [s["second"] for s in sts],
           "block_iterations": [s["iterations"] for s in sts],
           "solve_iterations": [s["solve_iterations"] for s in sts],
           "single_vector": {"ms_per_step": ms1, "block_iterations": [s["iterations"] for s in st1],
                             "worst_compliance": [s["compliance"] for s in st1]}}
    if rank == 0:
        print(json.dumps(out), flush=True)
    p.close()


def run_designs(args, rank):
    """32 independent cantilever designs of uneven size: all at once (one host
    thread per design, CUDA-graph V-cycles) against one after another."""
    from topoptspline3d_gb300 import capi, workloads
    wls = workloads.batch_cantilevers(32, seed0=2000)
    solve = dict(mode=capi.SOLVE_MIXED, smoother=capi.SMOOTH_CHEBYSHEV, pre=1, post=1, rtol=1e-6, max_iter=300,
                 inner_max=4)
    ocs = [dict(vgoal=w.vgoal) for w in wls]

    def build():
        ps = []
        for w in wls:
            q = capi.Problem(w.nx, w.ny, w.nz)
            q.set_bc(w.fixed, w.loads)
            bmin, bmax = w.spline_box()
            q.set_spline(w.order, w.partition, bmin, bmax)
            q.put("coeff", np.full(q.num_coeffs(), w.coeff0))
            q.coeff_to_density()
            q.set_operator_precision(2)
            q.set_coarse_refresh(args.coarse_every)
            ps.append(q)
        return ps

    ps = build()
    capi.design_batch(ps, args.warmup, threads=len(ps), solve=solve, ocs=ocs)
    # per-design tiles (z-march depth) and solver schedules from the autotuner, untimed
    tz, solves = [], []
    for q in ps:
        q.update_operators()
        best, rep = q.autotune(solve)
        tz.append(rep["tz32"])
        solves.append(best)
    _, conc = capi.design_batch(ps, args.steps, threads=len(ps), solve=solves, ocs=ocs)
    _, seq = capi.design_batch(ps, args.steps, threads=1, solve=solves, ocs=ocs)
    units = len(ps) * args.steps
    out = {"metric": "design iterations per second, 32 independent cantilevers 32^3..96x48x48, 1 GB300",
           "value": units / (conc["wall_ms"] / 1e3), "unit": "design-iter/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": conc["wall_ms"] / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32 multigrid / f64 CG", "data": "synthetic",
           "config": {"workload": "32 cantilevers, sizes and volume fractions from default_rng(2000 + d)",
                      "designs": [w.name for w in wls], "threads": len(ps), "autotuned_tz32": tz,
                      "coarse_refresh_every": args.coarse_every},
           "sequential_design_iter_per_s": units / (seq["wall_ms"] / 1e3),
           "speedup_vs_sequential": seq["wall_ms"] / conc["wall_ms"]}
    if rank == 0:
        print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.size is None:
        args.size = {"ellipsoids": "511x256x256", "loads": "192x96x96", "robust": "192x96x96"}.get(
            args.case, "256x128x128")
    nx, ny, nz = (int(v) for v in args.size.lower().split("x"))
    if args.retune_every is None:
        args.retune_every = 25 if args.case == "ellipsoids" else 0
    ws, rank, local, pg = dist_setup()
    if args.impl == "reference":
        run_reference(args, nx, ny, nz, ws, rank)
        return
    if args.case == "loads":
        run_loads(args, rank)
        return
    if args.case == "designs":
        run_designs(args, rank)
        return
    if args.case == "robust":
        run_robust(args, rank)
        return
    from topoptspline3d_gb300 import capi
    device = local
    wl, p = make_problem(nx, ny, nz, device, op_precision=2, case=args.case)
    opts = solve_opts(capi.SOLVE_MIXED, args.smoother)
    oc = dict(vgoal=wl.vgoal, damp=0.5, step=0.03, cmin=0.0, cmax=1.0)
    if args.no_graphs:
        p.set_graphs(0)
    p.set_coarse_refresh(args.coarse_every)
    if args.schedule:
        sched = args.schedule.split(",")
        inner, pre, deg, tz32, tz64 = (int(v) for v in sched[:5])
        opts.update(inner_max=inner, pre=pre, post=pre, cheb_degree=deg)
        if len(sched) > 5:
            opts["cheb_lo"] = float(sched[5])
        if len(sched) > 6:
            opts["inner_rtol"] = float(sched[6])
        p.set_tiles(tz32, tz64)
        args.no_autotune = True
    if args.profile_iteration:
        if args.profile_fp64:
            p.set_operator_precision(1)
            p.set_fine_arithmetic(0)
            opts = solve_opts(capi.SOLVE_PCG64, args.smoother)
        if args.profile_solve_steps > 0:
            opts["max_iter"] = args.profile_solve_steps
        for _ in range(args.profile_warmup):
            p.design_iteration(solve=opts, oc=oc)
        if args.profile_warmup > 0:
            p.sync()
            capi.profiler_range(True)
        s = p.design_iteration(solve=opts, oc=oc)
        if args.profile_warmup > 0:
            p.sync()
            capi.profiler_range(False)
        print(json.dumps({"profile_iteration": s}), flush=True)
        p.close()
        return
    for _ in range(args.warmup):
        p.design_iteration(solve=opts, oc=oc)
    # kernel tiles and solver schedule for this problem (untimed set-up)
    tune = None
    if not args.no_autotune and args.smoother == "chebyshev":
        p.update_operators()  # operators of the current design (the last OC step changed it)
        opts, tune = p.autotune(opts)
        # one more untimed iteration on the tuned schedule: captures its graphs
        p.design_iteration(solve=opts, oc=oc)
    # design state at the start of the timed region (untimed copies): the e2e
    # run below starts from it again, so both runs do the same design
    # iterations (the solver is deterministic) and differ only by the host
    # copies and the density evaluation from the uploaded coefficients
    coeff_start = p.get("coeff")
    # the whole solver state too (spectral-bound warm starts, tiles), so the
    # replays below repeat the timed iterations exactly
    import tempfile
    ckpt_dir = tempfile.mkdtemp(prefix="topo_bench_")
    ckpt = os.path.join(ckpt_dir, f"start_{rank}.ckpt")
    p.checkpoint_save(ckpt)
    # ---- timed region: K design iterations, device-resident inputs
    sampler = ClockSampler(device)
    barrier(pg)
    p.sync()
    sampler.start()
    launches0 = p.launch_count()
    p.timer_start()
    stats = []
    tuner = InnerTuner(opts, args.retune_every)
    for k in range(args.steps):
        stats.append(p.design_iteration(solve=tuner.opts_for(k), oc=oc))
        tuner.report(k, stats[-1])
    ms_total = p.timer_stop()
    launches = p.launch_count() - launches0
    clocks = sampler.stop()
    barrier(pg)
    ms_total = allmax(pg, ms_total)
    ms_step = ms_total / args.steps
    # ---- e2e: same steps through the C ABI with pinned host buffers
    nc = p.num_coeffs()
    hbuf = capi.PinnedBuffer(nc)
    hbuf.array[:] = coeff_start
    p.checkpoint_load(ckpt)
    barrier(pg)
    p.sync()
    p.timer_start()
    comp, e2e_its = [], []
    for k in range(args.steps):
        p.put_from("coeff", hbuf.ptr, nc)
        p.coeff_to_density()
        s = p.design_iteration(solve=tuner.used[k], oc=oc)
        p.get_into("coeff", hbuf.ptr, nc)
        comp.append(s["compliance"])
        e2e_its.append(s["iterations"])
    e2e_ms = allmax(pg, p.timer_stop() / args.steps)
    e2e_same_work = e2e_its == [s["iterations"] for s in stats]
    # ---- the same steps once more in reference precision (rho, coefficients and
    # sensitivities at FP32 values, rho^p by powf): the FP32-storage gap
    refp = None
    if args.case == "mbb":
        p.checkpoint_load(ckpt)
        p.set_reference_precision(1)
        p.coeff_to_density()
        ref_comp = [p.design_iteration(solve=tuner.used[k], oc=oc)["compliance"] for k in range(args.steps)]
        p.set_reference_precision(0)
        p.coeff_to_density()
        refp = {"compliance_rel_gap": [abs(a - b) / abs(b) for a, b in zip(ref_comp, comp)],
                "note": "same design iterations from the same state with the reference's FP32 storage of rho, "
                        "coefficients and sensitivities and powf for rho^p, against the FP64 path"}
    # ---- FP64 MG-PCG comparison on the same GPU (same design state)
    fp64 = None
    if args.fp64_steps > 0:
        # plain FP64 MG-PCG: FP64 operators and V-cycle, native FP64 fine matvec
        p.set_operator_precision(1)
        p.set_fine_arithmetic(0)
        o64 = solve_opts(capi.SOLVE_PCG64, args.smoother)
        p.timer_start()
        s64 = [p.design_iteration(solve=o64, oc=oc) for _ in range(args.fp64_steps)]
        fp64 = {"ms_per_step": p.timer_stop() / args.fp64_steps,
                "pcg_iterations": [s["iterations"] for s in s64], "relres": max(s["relres"] for s in s64),
                "fine_arithmetic": "native FP64"}
        p.set_operator_precision(2)
        p.set_fine_arithmetic(1)
    # ---- roofline of the dominant kernel family: per-family kernel times from
    # CUDA events around each launch, over min(K, 10) more design iterations (untimed;
    # with the events on, the inner CG runs its host loop, the same kernels)
    p.profile_enable(True)
    for _ in range(min(args.steps, 10)):
        p.design_iteration(solve=tuner.opts, oc=oc)
    prof = {k: p.profile_read(k) for k in range(4)}
    p.profile_enable(False)
    d0 = p.level_dims(0)[0]
    nv, ne = (d0[0] + 1) * (d0[1] + 1) * (d0[2] + 1), d0[0] * d0[1] * d0[2]
    fams = {capi.K_FINE_APPLY64: ("k_fine_modal_df (FP64 K.u in double-float, outer CG)",
                                  nv * (24 + 24 + 1) + ne * 8, ne * 240.0),
            # u in, f in, d out, u out (FP32 x3 each), vertex mask, the stored 3x3
            # block-Jacobi inverse (FP32, 6 of the symmetric 3x3), rho^p; d is read by one step in three
            # (a V(1,1) degree-2 cycle's pre-smoothing second step takes d from u,
            # the post-smoothing first step starts it)
            capi.K_FINE_SMOOTH32: ("k_fine_modal32<8,2|3> (FP32 Chebyshev step)",
                                   nv * (12 + 12 + 12 + 12 + 12 / 3 + 1 + 24) + ne * 4, ne * 240.0 + nv * 30.0),
            capi.K_FINE_APPLY32: ("k_fine_modal32<8,0|1> (FP32 K.u, residual)", nv * (12 + 12 + 1) + ne * 4,
                                  ne * 240.0),
            capi.K_FINE_SMOOTH64: ("k_fine_gs<double>", nv * (24 + 24 + 24 + 1) + ne * 8, nv * 1170.0)}
    dom = max(prof, key=lambda k: prof[k][1])
    name, bytes_per, flops_per = fams[dom]
    nl, tms = prof[dom]
    avg_s = (tms / max(nl, 1)) / 1e3
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    hbm_peak = peaks.get("hbm_gbs")
    peak_note = "measured (MEASURED_PEAKS.json hbm_gbs)" if hbm_peak else "fallback 6800 GB/s"
    hbm_peak = hbm_peak or 6800.0
    achieved = bytes_per / avg_s / 1e9
    # (the ncu traffic figure is for the 256x128x128 half-MBB launch)
    traffic = (load_traffic().get(name.split(" ")[0])
               if args.case == "mbb" and args.size == "256x128x128" else None)
    roof = {"bound": "hbm", "kernel": name, "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved / hbm_peak, "peak_source": peak_note,
            "traffic": traffic, "launches": nl, "avg_launch_ms": avg_s * 1e3,
            "algorithmic_bytes_per_launch": bytes_per, "flops_per_launch": flops_per,
            "achieved_tflops": flops_per / avg_s / 1e12,
            "family_ms": {fams[k][0]: prof[k][1] for k in prof if prof[k][0]}}
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline and args.case == "mbb":
        try:
            cms, cit, crr, cc = cpu_baseline(nx, ny, nz)
            cpu = {"value": cms, "unit": "ms/design-iter", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"1 design iteration (first of the run: {cit} PCG its, rel-res {crr:.1e}) of "
                             f"the FP64 CPU restatement, OpenMP on all host cores"}
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "ms/design-iter", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {e}"}
    extra = {}
    if rank == 0 and ws == 1 and args.case == "mbb" and not args.no_cpu_baseline:
        try:
            extra["compliance_vs_oracle"] = compliance_vs_oracle(p, wl, opts)
        except Exception as e:
            extra["compliance_vs_oracle"] = {"failed": str(e)}
    if args.case == "mbb" and not args.no_learned:
        try:
            extra["learned"] = learned_ablation(p, wl, opts)
        except Exception as e:
            extra["learned"] = {"failed": str(e)}
        try:
            extra["mixed_learned"] = mixed_learned_steps(p, ckpt, tuner.used, oc, ms_step,
                                                         fp64["ms_per_step"] if fp64 else None)
        except Exception as e:
            extra["mixed_learned"] = {"metric": METRIC_LEARNED, "failed": str(e)}
    h2d = 8 * nc
    d2h = 8 * nc + 8  # coefficients and the compliance scalar
    out = {"metric": metric_for(args), "value": ms_step, "unit": "ms/design-iter", "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": False, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32 multigrid / f64 CG", "data": "synthetic",
           "config": {"workload": f"{wl.name} spline OC design iteration", "grid": [nx, ny, nz],
                      "dofs": 3 * nv, "active_fraction": float(np.mean(wl.eactive)) if wl.eactive is not None else 1.0,
                      "lattice": [q + wl.order for q in wl.partition],
                      "solver": f"FP64 flexible CG (fine matvec in double-float, ~1e-14 of FP64) + "
                                f"{opts['inner_max']} FP32 CG its (to {opts.get('inner_rtol', 0.1):g}) with "
                                f"{args.smoother} V({opts['pre']},"
                                f"{opts['post']}) degree-{opts['cheb_degree']} on "
                                f"[{opts.get('cheb_lo', 0.3):g}, {opts.get('cheb_hi', 1.1):g}] lambda_max multigrid, "
                                f"rel-res 1e-6",
                      "autotune": tune,
                      "inner_cap_retune_every": args.retune_every,
                      "inner_caps_used": sorted(set(o["inner_max"] for o in tuner.used)),
                      "l2": "working set (>2 GB) larger than L2; no flush",
                      "coarse_refresh_every": args.coarse_every,
                      "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU"},
           "cg_iterations": [s["iterations"] for s in stats], "relres": max(s["relres"] for s in stats),
           "oc_trials": [s["oc_trials"] for s in stats], "compliance": [s["compliance"] for s in stats],
           "fp64_mgpcg": fp64,
           "reference_precision": refp,
           "speedup_vs_fp64_mgpcg": (fp64["ms_per_step"] / ms_step) if fp64 else None,
           "e2e": {"value": e2e_ms, "unit": "ms/design-iter", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                   "same_iterations_as_timed_region": e2e_same_work},
           "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu, "clocks": clocks}
    out.update(extra)
    if rank == 0:
        print(json.dumps(out), flush=True)
    p.close()
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
