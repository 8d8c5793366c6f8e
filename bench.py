"""PD step benchmark: tet-iterations/s of the GB300 engine.

Workload (default): 1 m cube, 64^3 hex cells split 5 tets each (274,625
verts / 1,310,720 tets), vertices jittered +-0.1 cell (seed 2024), E=1e6,
nu=0.45, rho=1000 kg/m^3 lumped, top face pinned (weight 1e6), dt=1/120,
Chebyshev-accelerated Jacobi (rho=0.9995), 20 local/global iterations per
step.  One bench step = one PD time step = 20 iterations over all tets.

  value  device time of the step graph, inputs resident in HBM, L2 flushed
         (256 MB write) between timed steps.
  e2e    the same metric through the C ABI with pinned host buffers: every
         step uploads X, V, runs the step and downloads X, V.
  roofline  local-step kernel: algorithmic bytes per launch / average launch
         time (CUDA events around every launch inside the step graph).

The default run (no --workload) adds, under "workloads", a leg for each of
the other workloads, each with its own step count: the 10^3 Cholesky cube
(c1), the 40^3 heterogeneous Cholesky cube with its factor times and the
refinement sweep (c3), the batch of 512 bodies with the plain drop-in on the
same bodies and their ratio (c4), and an 8-second window of the Cholesky
request stream with p50/p99 latency (c5).  --workload X runs X alone.

`--impl reference` times the CPU implementation of the same iteration (the
reference's kernels compiled for the CPU when present, else the project's
float restatement) on all host cores, one PD step of the workload per bench
step.
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "soft-body-simulation-cuda_gb300"))

WORKLOADS = {
    "c2": {
        "workload": "pd_jacobi_cube64",
        "desc": "64^3 hex grid x5 tets (274625 v / 1310720 t), jitter 0.1 cell seed 2024, E=1e6 nu=0.45 rho=1000, "
                "top face pinned, dt=1/120, Jacobi+Chebyshev rho=0.9995, 20 iterations/step",
        "grid": 64, "iterations": 20, "rho": 0.9995, "solver": "jacobi", "episode_steps": 50,
        "state": "50-step runs from rest, repeated: the rest state is restored on the device between runs, "
                 "outside the step events (past ~25 steps this iteration diverges, in FP64 as in FP32)",
    },
    "c1": {
        "workload": "pd_cholesky_cube10",
        "desc": "10^3 hex grid x5 tets (1331 v / 5000 t), E=1e5 nu=0.4 rho=1000, top face pinned, dt=1/120, "
                "prefactored sparse Cholesky (AMD), 10 iterations/step",
        "grid": 10, "iterations": 10, "solver": "cholesky",
    },
    "c4": {
        "workload": "pd_cholesky_batch512",
        "desc": "512 independent hex-grid bodies, dims uniform 4..24 per axis (seed 4), cells 1/16 m, E log-uniform "
                "1e4..1e7, nu U[0.3,0.45], rho U[800,1200], top faces pinned, dt=1/120, per-body prefactored sparse "
                "Cholesky (AMD), 10 iterations/step, one engine: per iteration 1 local launch over every body's tiles, "
                "the solve (autotuned schedule: per-level launches over all bodies, or one CTA per body) and 1 "
                "vertex launch, CUDA graph per step",
        "nbodies": 512, "iterations": 10, "solver": "cholesky",
    },
    "c5": {
        "workload": "pd_serving_poisson200",
        "desc": "request stream: Poisson arrivals 200 req/s over the arrival window, each a near-cubic hex-grid body "
                "with tets log-uniform 1e3..3e5 (drawn from a seeded pool of 48 bodies), material as the batch "
                "workload, K steps uniform 10..200, dt=1/120, 10 iterations of the prefactored sparse Cholesky solve "
                "(each request's FP64 factor computed on the GPU at admission and resident with its mesh and state); "
                "continuous batching, admission by an 8 GiB HBM budget",
        "rate": 200.0, "iterations": 10, "solver": "cholesky",
    },
    "c3": {
        "workload": "pd_cholesky_hetero40",
        "desc": "40^3 hex grid x5 tets (68921 v / 320000 t), per-tet E log-uniform 1e4..1e7 (seed 3), nu U[0.3,0.45], "
                "rho=1000, top face pinned, dt=1/120, prefactored sparse Cholesky (AMD, FP64 factor, FP32 solves), "
                "10 iterations/step",
        "grid": 40, "iterations": 10, "solver": "cholesky",
    },
}
WORKLOAD = None
METRIC = "PD tet-iterations/s"
UNIT = "tet-iter/s"


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def init_dist(world):
    if world <= 1:
        return None
    import torch.distributed as dist

    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group("gloo")
    return dist


def reduce_max(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic_per_launch(workload: str):
    """DRAM bytes per local-step launch from the committed ncu summary, if any."""
    p = ROOT / "profiles" / f"k_local_{workload}.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["dram_bytes_per_launch"])
        except (KeyError, ValueError):
            return None
    return None


def cpu_baseline(body, params, steps: int):
    """The float CPU restatement of the same iteration (OpenMP, all cores)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O

    cores = os.cpu_count() or 1
    r = O.Runner(body, params, precision=32, nthreads=cores)
    secs = r.run(steps)
    r.close()
    return {"value": body.num_tets * params.num_iterations * steps / secs, "unit": UNIT, "cores": cores,
            "kind": "port", "seconds": secs,
            "sample": f"{steps} PD step(s) of the full workload ({steps * params.num_iterations} iterations x "
                      f"{body.num_tets} tets), float arithmetic, OpenMP over {cores} host threads"}


def run_reference_arm(args, body, params, scale=1.0):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O

    cores = os.cpu_count() or 1
    use_ref = O.reference_available() and not args.port
    kind = "reference" if use_ref else "port"
    # Each bench step is one PD step of the workload; when K full steps would
    # take longer than the time budget, each bench step runs fewer iterations
    # (same per-iteration work: every tet, every vertex), so that the whole
    # run stays within a few minutes.
    budget_s = 120.0
    if use_ref:
        # the reference kernels compiled for the CPU (serial), one call per
        # step, set-up outside the timed region excluded by timing only the
        # step call of a one-step run is not possible: time the whole call
        X, V = body.X.copy(), np.zeros_like(body.X)
        its = params.num_iterations
        t_total = 0.0
        for k in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            X, V, _ = O.reference_simulate(body, params, 1, X=X, V=V)
            dt = time.perf_counter() - t0
            if k >= args.warmup:
                t_total += dt
    else:
        r = O.Runner(body, params, precision=32, nthreads=cores)
        t_it = r.run(1, 1)  # one iteration: the per-iteration cost
        its = max(1, min(params.num_iterations, int(budget_s / max(args.steps * t_it, 1e-9))))
        r.run(args.warmup, its)
        t_total = r.run(args.steps, its)
        r.close()
    value = body.num_tets * its * args.steps / t_total
    sample = (f"one PD step of {its} iteration(s) x {body.num_tets} tets per bench step (workload: "
              f"{params.num_iterations} iterations per step), "
              f"{'reference kernels compiled for the CPU (serial)' if use_ref else f'float CPU restatement, OpenMP over {cores} threads'}")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(WORKLOAD, parallelism=f"replicas{world}" if world > 1 else "single"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1 if use_ref else cores, "kind": kind,
                         "sample": sample, "seconds": t_total},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def accuracy_vs_fp64(body, params, steps: int, refine_sweep: bool = False, ref_gpu: bool = False) -> dict:
    """Engine vs the FP64 oracle from the rest state, `steps` steps of the
    workload (a bounded sample); relative L2 errors of positions and of
    displacements.  With refine_sweep: one entry per refinement count 0..3.
    With ref_gpu: the restated reference GPU path as well."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle as O
    from pdgb import PdSolver
    from pdgb.engine import SolverParams

    Xo, _, _ = O.simulate(body, params, steps, precision=64, nthreads=os.cpu_count() or 1)
    X0 = body.X.astype(np.float64)
    out = {"steps": steps, "oracle": "fp64"}
    counts = range(4) if refine_sweep else [params.refine_steps]
    X_engine = None
    for r in counts:
        p = SolverParams(**{**params.__dict__, "refine_steps": r})
        with PdSolver(body, p) as e:
            e.update(steps)
            X, _ = e.download_state()
        X = X.astype(np.float64)
        if X_engine is None:
            X_engine = X
        key = f"refine{r}" if refine_sweep else "engine"
        out[key] = {"rel_err_x": float(np.linalg.norm(X - Xo) / np.linalg.norm(Xo)),
                    "rel_err_disp": float(np.linalg.norm(X - Xo) / max(np.linalg.norm(Xo - X0), 1e-30))}
    if ref_gpu:
        sys.path.insert(0, str(ROOT / "baseline"))
        import refgpu

        with refgpu.ReferenceGpuPath(body, params) as r:
            r.step(steps)
            X, _ = r.state()
        X = X.astype(np.float64)
        out["reference_gpu"] = {"rel_err_x": float(np.linalg.norm(X - Xo) / np.linalg.norm(Xo)),
                                "rel_err_disp": float(np.linalg.norm(X - Xo) / max(np.linalg.norm(Xo - X0), 1e-30))}
        # the engine (first entry above) against the reference GPU path itself
        out["engine_vs_reference_gpu"] = {
            "rel_err_x": float(np.linalg.norm(X_engine - X) / np.linalg.norm(X)),
            "rel_err_disp": float(np.linalg.norm(X_engine - X) / max(np.linalg.norm(X - X0), 1e-30))}
    return out


def reference_gpu(body, params, nsteps: int, episode: int, sample: str) -> dict:
    """The reference's GPU PD step restated with cuSOLVER's FP32 sparse
    Cholesky (baseline/refgpu.cu), timed on this GPU with CUDA events on the
    default stream around `nsteps` steps (inputs resident, set-up and factor
    outside); Jacobi workloads run from rest in runs of `episode` steps.  Its
    Cholesky branch reads the error on the host every iteration, as the
    reference does."""
    sys.path.insert(0, str(ROOT / "baseline"))
    import refgpu

    t0 = time.perf_counter()
    r = refgpu.ReferenceGpuPath(body, params)
    setup_s = time.perf_counter() - t0
    try:
        r.step(3)  # warm-up
        r.reset()
        ms, its, done = 0.0, 0, 0
        while done < nsteps:
            k = min(nsteps - done, episode) if episode else nsteps - done
            if episode:
                r.reset()
            m, i = r.step(k)
            ms, its, done = ms + m, its + i, done + k
        X, _ = r.state()
        nnz = r.system_nnz()
    finally:
        r.close()
    return {"value": body.num_tets * its / (ms / 1e3), "unit": UNIT, "kind": "port",
            "what": "the reference's PdSolver::SolverStep kernels restated (per-tet threads, 12 float atomics per "
                    "tet, 4-sweep SVD) with cuSOLVER's low-level FP32 sparse Cholesky (symamd ordering) on the "
                    "3n x 3n system, or Jacobi + Chebyshev; legacy default stream, 128 threads per block",
            "steps": nsteps, "iterations": its, "ms_per_step": ms / nsteps, "setup_s": setup_s,
            "system_nnz": nnz, "finite": bool(np.isfinite(X).all()), "sample": sample}


def plain_drop_in(bodies, params, steps: int, flush) -> dict:
    """The plain drop-in on the batch's bodies: one engine per body, run one
    body at a time (the engine as a single-scene PdSolver replacement), the
    same step timing as the batch (CUDA events around every step graph, L2
    flushed between steps outside the events)."""
    from pdgb import PdSolver
    from pdgb import _native as N

    import torch

    tet_iters, ms = 0.0, 0.0
    for b in bodies:
        with PdSolver(b, params) as e:
            stream = torch.cuda.ExternalStream(e._lib.pdgb_stream(e.handle))

            def flush_l2():
                with torch.cuda.stream(stream):
                    flush.add_(1.0)

            e.enable_kernel_timing(N.PDGB_TIMING_STEPS)
            e.prepare()
            for _ in range(3):
                e.update(1)
            e.synchronize()
            e.read_timing()
            for _ in range(steps):
                e.update(1)
                flush_l2()
            e.synchronize()
            tm = e.read_timing()
        ms += tm["step_ms"]
        tet_iters += float(b.num_tets * params.num_iterations * steps)
    return {"value": tet_iters / (ms / 1e3), "unit": UNIT, "bodies": len(bodies), "steps": steps,
            "ms_per_body_step": ms / (len(bodies) * steps),
            "sample": f"every 8th body of the batch ({len(bodies)} bodies), one engine each, run one after another"}


def run_serving(args, window: float, rate: float = 0.0, solver: str = "", cache: bool = True,
                print_line: bool = True) -> dict:
    """Serving workload: wall-clock request arrivals into the server."""
    import math

    from pdgb import PdServer, PdSolver, mesh
    from pdgb.engine import SolverParams

    rank, world, local = dist_info()
    import torch

    torch.cuda.set_device(local)
    wl = dict(WORKLOADS["c5"])
    if rate > 0 and rate != wl["rate"]:
        wl["rate"] = rate
        wl["workload"] += f"_rate{rate:g}"
        wl["desc"] = wl["desc"].replace("200 req/s", f"{rate:g} req/s", 1)
    if solver and solver != wl["solver"]:
        wl["solver"] = solver
        wl["workload"] += f"_{solver}"
        wl["desc"] = wl["desc"].replace(
            "10 iterations of the prefactored sparse Cholesky solve (each request's FP64 factor computed on the GPU "
            "at admission and resident with its mesh and state)", "10 Jacobi+Chebyshev iterations (rho=0.9995)")
    if not cache:
        wl["workload"] += "_nocache"
        wl["cache"] = "off: every request builds its layout and factor"
    else:
        wl["cache"] = "layouts and factors of the 48 pool meshes kept after their first request"
    rng = np.random.default_rng(5)
    pool = [mesh.request_body(math.exp(rng.uniform(math.log(1e3), math.log(3e5))), rng) for _ in range(48)]
    n_req = int(rng.poisson(wl["rate"] * window))
    arrivals = np.sort(rng.uniform(0.0, window, size=n_req))
    picks = rng.integers(0, len(pool), size=n_req)
    ksteps = rng.integers(10, 201, size=n_req)
    params = SolverParams(num_iterations=wl["iterations"], rho=0.9995, solver=1 if wl["solver"] == "cholesky" else 0)
    offered = float(sum(pool[p].num_tets * int(k) for p, k in zip(picks, ksteps)) * params.num_iterations / window)
    srv = PdServer(params, hbm_budget_bytes=8 << 30, cache_entries=0 if cache else -1)
    # warm-up: a few requests through the server (graph capture, pool growth)
    for p in range(4):
        srv.submit(pool[p], 2)
    deadline = time.monotonic() + 300.0
    while srv.stats()["completed"] + srv.stats()["failed"] < 4 and time.monotonic() < deadline:
        if srv.tick()[0] == 0:
            time.sleep(0.002)
    base_completed = srv.stats()["completed"]
    base_failed = srv.stats()["failed"]
    base_lat = len(srv.latencies_ms())
    give_up_s = 20.0 * window + 600.0
    base_ti = srv.stats()["tet_iterations"]
    base_busy = srv.stats()["busy_ms"]
    ids = []
    t0 = time.perf_counter()
    nxt = 0
    trace, next_trace = [], 0.0
    with ClockSampler(local) as clocks:
        while True:
            now = time.perf_counter() - t0
            if now >= next_trace:  # queue state once a second
                sn = srv.stats()
                trace.append([round(now, 1), sn["active"], sn["waiting"], sn["ready"],
                              int(sn["completed"] - base_completed)])
                next_trace += 1.0
            while nxt < n_req and arrivals[nxt] <= now:
                ids.append((srv.submit(pool[picks[nxt]], int(ksteps[nxt])), int(picks[nxt]), int(ksteps[nxt])))
                nxt += 1
            st = srv.stats()
            if nxt >= n_req and st["completed"] + st["failed"] - base_completed - base_failed >= n_req:
                break
            if now > give_up_s:
                raise RuntimeError(f"serving: requests unfinished after {give_up_s:.0f} s")
            if st["active"] == 0 and st["waiting"] == 0 and st["finishing"] == 0:
                time.sleep(0.0005)
                continue
            srv.tick()  # a tick hands out the requests the previous tick's step finished
        wall = time.perf_counter() - t0
    st = srv.stats()
    lat = srv.latencies_ms()[base_lat:]
    value = (st["tet_iterations"] - base_ti) / wall
    # Same alone vs in the mix on a 1 % seeded sample across sizes, plus the
    # largest and a mid-size request of the stream.
    from pdgb import PdgbError

    srng = np.random.default_rng(11)
    by_size = sorted(range(len(ids)), key=lambda i: pool[ids[i][1]].num_tets)
    sample = sorted(set(srng.choice(len(ids), size=max(1, len(ids) // 100), replace=False).tolist()
                        + [by_size[-1], by_size[len(by_size) // 2]])) if ids else []
    results = {}
    failed_results = 0
    for i, (rid, p, k) in enumerate(ids):
        try:
            X = srv.result(rid)[0]
        except PdgbError:
            failed_results += 1
            continue
        if i in sample:
            results[i] = X
    worst_alone, alone_sizes = 0.0, []
    for i in sample:
        if i not in results:
            continue
        rid, p, k = ids[i]
        with PdSolver(pool[p], params) as e:
            e.update(k)
            Xa, _ = e.download_state()
        worst_alone = max(worst_alone, float(np.linalg.norm(results[i] - Xa) / np.linalg.norm(Xa)))
        alone_sizes.append(pool[p].num_tets)
    acc = None
    if not args.no_accuracy and results:
        sys.path.insert(0, str(ROOT / "oracle"))
        import oracle as O

        acc = []
        for i in [by_size[len(by_size) // 2]] + [j for j in sample if pool[ids[j][1]].num_tets < 2e4][:2]:
            if i not in results:
                continue
            rid, p, k = ids[i]
            Xo, _, _ = O.simulate(pool[p], params, k, precision=64, nthreads=os.cpu_count() or 1)
            acc.append({"request_tets": pool[p].num_tets, "steps": k,
                        "rel_err_x_vs_fp64": float(np.linalg.norm(results[i] - Xo) / np.linalg.norm(Xo))})
    srv.close()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": int(ksteps.sum()),
        "warmup": 4, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": dict(wl, window_s=window, requests=n_req, offered_tet_iter_per_s=offered),
        "latency_ms": {"p50": float(np.percentile(lat, 50)) if len(lat) else None,
                       "p99": float(np.percentile(lat, 99)) if len(lat) else None,
                       "mean": float(np.mean(lat)) if len(lat) else None},
        "wall_s": wall, "completed": int(st["completed"] - base_completed), "failed": int(st["failed"] - base_failed),
        "failed_results": failed_results,
        "alone_vs_mix_max_rel_err": worst_alone, "alone_vs_mix_sample": len(alone_sizes),
        "alone_vs_mix_tets": {"min": min(alone_sizes) if alone_sizes else None,
                              "max": max(alone_sizes) if alone_sizes else None},
        "nonfinite_results": int(st["nonfinite"]),
        "accuracy": acc, "clocks": clocks.summary(),
        "busy_frac": float(st["busy_ms"] - base_busy) / 1e3 / wall,
        "server_ms": {"admit": st["admit_ms"], "step": st["step_ms"], "ticks": st["ticks"]},
        "layout_cache_hits": st["layout_cache_hits"],
        "factors": {"gpu_factorisations": int(st["factors"]), "cache_hits": int(st["factor_cache_hits"]),
                    "gpu_ms": float(st["factor_ms"])} if params.solver == 1 else None,
        "queue_trace": {"fields": ["t_s", "active", "waiting", "ready", "completed"], "rows": trace[::5]},
        "e2e": {"value": value, "unit": UNIT,
                "h2d_bytes_per_request": float(np.mean([48 * pool[p].num_verts + 28 * pool[p].num_tets
                                                        for _, p, _ in ids])) if ids else 0.0,
                "d2h_bytes_per_request": float(np.mean([24 * pool[p].num_verts for _, p, _ in ids])) if ids else 0.0,
                "note": "requests enter as host meshes and leave as host arrays: the serving value is end to end"},
    }
    if rank == 0 and print_line:
        print(json.dumps(line), flush=True)
    return line


def launches_per_step(info, params) -> int:
    """Kernels of one step graph: prologue, per iteration local + global
    (Jacobi: 1 vertex kernel; Cholesky: 2 per solve level + 1 vertex kernel),
    Cholesky epilogue."""
    if params.solver == 0:
        return 1 + 2 * params.num_iterations
    return 2 + params.num_iterations * (2 + info["solve_launches"])


# Default timed steps per workload: about 1.5 s of device time, so that the
# clock sampler (200 ms period) sees the GPU under load.
DEFAULT_STEPS = {"c1": 1200, "c2": 1200, "c3": 300, "c4": 60}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0,
                    help="timed steps (default: about 1.5 s of device time for the workload)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="pdgb", choices=["pdgb", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--grid", type=int, default=0, help="override cells per axis (profiling of smaller cases)")
    ap.add_argument("--bodies", type=int, default=0, help="override the number of bodies of the batch workload")
    ap.add_argument("--cpu-steps", type=int, default=4, help="PD steps in the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--solve-mode", type=int, default=0, help="Cholesky solve schedule (PDGB_SOLVE_*), 0 = auto")
    ap.add_argument("--no-autotune", action="store_true", help="skip the engine's autotuner (tile size, solve "
                    "schedule), which runs before the timed region")
    ap.add_argument("--port", action="store_true", help="reference arm: time the oracle port even where the "
                    "reference harness is built")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP64-oracle error report")
    ap.add_argument("--window", type=float, default=20.0, help="arrival window of the serving workload, seconds")
    ap.add_argument("--rate", type=float, default=0.0, help="serving: mean arrivals per second (0 = the workload's)")
    ap.add_argument("--no-plain", action="store_true", help="batch workload: skip the plain drop-in leg (the same "
                    "bodies one engine each, one at a time)")
    ap.add_argument("--no-ref-gpu", action="store_true", help="skip the restated reference GPU path "
                    "(cuSOLVER Cholesky / Jacobi) timed beside the engine")
    ap.add_argument("--collision", action="store_true", help="run continuous collision between bodies after every "
                    "step (inside the timed region)")
    ap.add_argument("--ordering", default="", choices=["", "amd", "nd", "dense"],
                    help="Cholesky factor ordering (default: AMD, or the autotuner's choice)")
    ap.add_argument("--tile", type=int, default=0, help="most tets per local-step tile (0: default / autotuned)")
    ap.add_argument("--local-kernel", choices=["", "tile", "pipelined"], default="",
                    help="form of the local step (default: one CTA per tile, or the autotuner's choice; "
                         "the autotuner tries both, so fix it together with --no-autotune)")
    ap.add_argument("--no-legs", action="store_true", help="default run: report the 64^3 Jacobi workload only, "
                    "without the legs of the other workloads")
    ap.add_argument("--solver", default="", choices=["", "jacobi", "cholesky"],
                    help="serving workload: global solve of the requests (default: the workload's, Cholesky)")
    ap.add_argument("--no-cache", action="store_true", help="serving workload: no mesh cache (every request builds "
                    "its layout and factor)")
    args = ap.parse_args()
    explicit = "--workload" in sys.argv[1:] or any(a.startswith("--workload=") for a in sys.argv[1:])
    if args.warmup < 3 and args.impl == "pdgb":
        args.warmup = 3
    if args.steps <= 0:
        args.steps = DEFAULT_STEPS.get(args.workload, 20) if args.impl == "pdgb" else 2

    if args.workload == "c5" and args.impl != "reference":
        run_serving(args, args.window, args.rate, args.solver, not args.no_cache)
        return
    if args.impl == "reference":
        run_engine(args, args.workload, args.steps, args.warmup)
        return
    rank, world, _ = dist_info()
    line = run_engine(args, args.workload, args.steps, args.warmup)
    if line is None:
        return
    if not explicit and not args.no_legs and world == 1:
        # The default run also reports the other workloads of the benchmark,
        # each with its own (shorter) step count: the plain Cholesky cube, the
        # heterogeneous Cholesky cube, the batch of 512 bodies (with the plain
        # drop-in on the same bodies) and the Cholesky request stream.
        legs = {}
        for wl, steps in (("c1", 200), ("c3", 30), ("c4", 20)):
            legs[wl] = compact_leg(run_engine(args, wl, steps, 3, leg=True))
        legs["c5"] = compact_serving(run_serving(args, 8.0, 0.0, "", True, print_line=False))
        line["workloads"] = legs
    print(json.dumps(line), flush=True)


def compact_leg(line: dict) -> dict:
    """The fields of a workload's line that the default run reports as a leg."""
    keep = ("metric", "value", "unit", "steps", "warmup", "ms_per_step", "config", "e2e", "roofline", "kernels",
            "accuracy", "reference_gpu", "plain_drop_in", "batched_vs_plain", "factor", "cpu_baseline",
            "gpu_launches", "clocks", "finite", "autotune", "local_kernel")
    return {k: line[k] for k in keep if k in line}


def compact_serving(line: dict) -> dict:
    keep = ("metric", "value", "unit", "config", "latency_ms", "wall_s", "completed", "failed", "failed_results",
            "nonfinite_results", "alone_vs_mix_max_rel_err", "alone_vs_mix_sample", "alone_vs_mix_tets", "accuracy",
            "busy_frac", "server_ms", "layout_cache_hits", "factors", "clocks", "e2e")
    return {k: line[k] for k in keep if k in line}


def run_engine(args, workload_name: str, nsteps: int, nwarmup: int, leg: bool = False):
    """One engine workload (c1-c4): the timed steps, the kernel pass, the
    end-to-end pass and the reports.  Returns the JSON line (rank 0), or
    None on other ranks and for the reference arm (which prints its own)."""
    from pdgb import mesh
    from pdgb.engine import SolverParams

    global WORKLOAD
    WORKLOAD = dict(WORKLOADS[workload_name])
    WORKLOAD["l2"] = "flushed between timed steps (256 MB write)"
    if args.grid and not leg:
        WORKLOAD["grid"] = args.grid
        WORKLOAD["workload"] += f"_grid{args.grid}"
    n = WORKLOAD.get("grid", 0)
    bodies = None
    if workload_name == "c4":
        bodies = mesh.batch_c4(nbodies=(args.bodies if not leg else 0) or WORKLOAD["nbodies"])
        WORKLOAD["nbodies"] = len(bodies)
        body = mesh.concat(bodies)
        WORKLOAD["tets"], WORKLOAD["verts"] = body.num_tets, body.num_verts
        params = SolverParams(num_iterations=WORKLOAD["iterations"], solver=1)
    elif workload_name == "c2":
        body = mesh.cube_c2(n=n)
        params = SolverParams(num_iterations=WORKLOAD["iterations"], rho=WORKLOAD["rho"], solver=0)
    elif workload_name == "c1":
        body = mesh.make_grid_body(n, n, n, young=1e5, poisson=0.4, density=1000.0)
        params = SolverParams(num_iterations=WORKLOAD["iterations"], solver=1)
    else:
        body = mesh.cube_c3(n=n)
        params = SolverParams(num_iterations=WORKLOAD["iterations"], solver=1)

    cpu_body = body if bodies is None else mesh.concat(bodies[:16])  # bounded CPU sample of the batch
    if args.impl == "reference":
        run_reference_arm(args, cpu_body, params, scale=1.0)
        return None

    rank, world, local = dist_info()
    import torch

    torch.cuda.set_device(local)
    dist = init_dist(world) if not leg else None
    from pdgb import PdSolver

    from pdgb import _native as N

    eng = PdSolver(body if bodies is None else bodies, params)
    if args.solve_mode and not leg:
        eng.set_solve_mode(args.solve_mode)
    if args.ordering and not leg:
        eng.set_ordering({"amd": N.PDGB_ORDER_AMD, "nd": N.PDGB_ORDER_ND, "dense": N.PDGB_ORDER_DENSE}[args.ordering])
    if args.tile and not leg:
        eng.set_tile_size(args.tile)
    if args.local_kernel and not leg:
        eng.set_local_kernel({"tile": N.PDGB_LOCAL_TILE, "pipelined": N.PDGB_LOCAL_PIPELINED}[args.local_kernel])
    stream = torch.cuda.ExternalStream(eng._lib.pdgb_stream(eng.handle))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MB > L2

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.add_(1.0)

    eng.prepare()
    collision = None
    if args.collision:
        # continuous collision between bodies after every step (the
        # reference's PdSolver::Update with collision handling on)
        from pdgb.meshio import surface_triangles

        parts, off = [], 0
        for b in (bodies if bodies is not None else [body]):
            parts.append(surface_triangles(b.tets) + np.uint32(off))
            off += b.num_verts
        ctris = np.concatenate(parts)
        eng.set_collision_surface(ctris)
        eng.enable_collision(True)
        collision = {"surface_tris": int(ctris.shape[0])}
        WORKLOAD["collision"] = "continuous collision between bodies after every step"
    tune = None
    if not args.no_autotune:
        tune = eng.autotune(steps=3)  # set-up, outside the timed region; the state is restored
    local_kernel = "pipelined" if eng.local_kernel() == N.PDGB_LOCAL_PIPELINED else "tile"
    # Workloads timed as repeated runs of a fixed length from rest: the rest
    # state is uploaded from device memory (one gather launch) at the start
    # of every run, between step graphs.
    episode = int(WORKLOAD.get("episode_steps", 0))
    X0d = torch.from_numpy(np.ascontiguousarray(body.X, dtype=np.float32)).cuda()
    V0d = torch.zeros_like(X0d)
    torch.cuda.synchronize()

    def start_episode(k):
        if episode and k % episode == 0:
            N.check(eng._lib.pdgb_upload_state(eng.handle, X0d.data_ptr(), V0d.data_ptr(), N.PDGB_MEM_DEVICE),
                    "pdgb_upload_state")

    eng.enable_kernel_timing(N.PDGB_TIMING_STEPS)
    eng.prepare()
    start_episode(0)
    for _ in range(nwarmup):
        eng.update(1)
        flush_l2()
    eng.synchronize()
    eng.read_timing()  # clear the accumulators
    barrier(dist)
    torch.cuda.synchronize()
    # Timed region: every step graph is bracketed by a pair of CUDA events on
    # the engine's stream (no host wait between steps); the L2 flush runs
    # between steps, outside the events.
    with ClockSampler(local) as clocks:
        for k in range(nsteps):
            start_episode(k)
            eng.update(1)
            flush_l2()
        torch.cuda.synchronize()
    barrier(dist)
    tm = eng.read_timing()
    Xt, _ = eng.download_state()
    finite_timed = bool(np.isfinite(Xt).all())
    assert tm["steps"] == nsteps
    if collision is not None:
        _, _, cinfo = eng.collision()
        collision.update(candidate_pairs=cinfo["candidate_pairs"], vertices_hit=cinfo["vertices_hit"],
                         detect_ms_last_step=cinfo["detect_ms"])
    t_local = tm["step_ms"] / 1e3
    # Kernel pass (not part of the value): the same steps with every
    # local-step launch bracketed by events inside the graph, for the
    # roofline of the dominant kernel.
    eng.enable_kernel_timing(N.PDGB_TIMING_KERNELS)
    eng.prepare()
    start_episode(0)
    eng.update(1)
    eng.read_timing()
    for k in range(nsteps):
        start_episode(k)
        eng.update(1)
        flush_l2()
    eng.synchronize()
    tk = eng.read_timing()
    local_ms, local_launches = tk["local_ms"], tk["local_launches"]
    solve_ms, solves = tk["solve_ms"], tk["solves"]
    step_ms_kernel_pass = tk["step_ms"]
    t_max = reduce_max(dist, t_local)
    tet_iters = reduce_sum(dist, float(body.num_tets * params.num_iterations * nsteps))
    value = tet_iters / t_max

    # ---- e2e through the C ABI with pinned host buffers
    eng.enable_kernel_timing(N.PDGB_TIMING_OFF)
    eng.prepare()
    nv = body.num_verts
    X0h = torch.from_numpy(body.X.copy())
    Xh = X0h.clone().pin_memory()
    Vh = torch.zeros((nv, 3), dtype=torch.float32).pin_memory()
    lib, h = eng._lib, eng.handle
    for _ in range(2):
        N.check(lib.pdgb_upload_state(h, Xh.data_ptr(), Vh.data_ptr(), N.PDGB_MEM_HOST), "upload")
        N.check(lib.pdgb_step(h, 1), "step")
        N.check(lib.pdgb_download_state(h, Xh.data_ptr(), Vh.data_ptr(), N.PDGB_MEM_HOST), "download")
    e2e_s = 0.0
    for k in range(nsteps):
        if k == 0 or (episode and k % episode == 0):
            Xh.copy_(X0h)  # the caller starts a new run from rest
            Vh.zero_()
        flush_l2()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        N.check(lib.pdgb_upload_state(h, Xh.data_ptr(), Vh.data_ptr(), N.PDGB_MEM_HOST), "upload")
        N.check(lib.pdgb_step(h, 1), "step")
        N.check(lib.pdgb_download_state(h, Xh.data_ptr(), Vh.data_ptr(), N.PDGB_MEM_HOST), "download")
        e2e_s += time.perf_counter() - t0
    e2e_max = reduce_max(dist, e2e_s)
    e2e_value = tet_iters / e2e_max
    plain = None
    if bodies is not None and not args.no_plain:
        plain = plain_drop_in(bodies[::8], params, 10, flush)
    finite = bool(torch.isfinite(Xh).all().item())
    eng_info = eng.get_performance_data()
    eng_info["levels"] = eng.solve_levels() if params.solver == 1 else 0
    eng_info["solve_mode"] = eng.solve_mode() if params.solver == 1 else 0
    eng_info["solve_launches"] = eng.factor_info()["solve_launches"] if params.solver == 1 else 0
    factor = None
    if params.solver == 1:
        fi = eng.factor_info()
        factor = {"numeric_device": "gpu" if fi["numeric_device"] == N.PDGB_FACTOR_GPU else "host",
                  "numeric_ms": fi["numeric_ms"], "total_ms": fi["factor_ms"], "flops": fi["flops"],
                  "nnz_L": fi["nnz_L"], "m_entries": fi["m_entries"], "pool_bytes": fi["pool_bytes"],
                  "levels": fi["num_levels"],
                  "what": "total_ms: ordering + symbolic analysis (host) + FP64 numeric factorisation "
                          "(numeric_ms, device time on the GPU), once per system matrix"}
    solve_bytes = eng.solve_bytes()
    # the local step alone, back to back (CUDA events around 200 launches on
    # the engine's stream, after the timed region): no event nodes between
    # launches inflate it, unlike the in-graph pairs above
    if episode:
        # averaged over the states of one run from rest (the rotation's cost
        # depends on the deformation)
        start_episode(0)
        b2b = []
        for _ in range(episode):
            b2b.append(eng.time_local(50))
            eng.update(1)
        local_b2b_ms = sum(b2b) / len(b2b)
    else:
        local_b2b_ms = min(eng.time_local(200) for _ in range(3))
    eng.close()

    if rank != 0:
        return None
    peak, peak_kind = measured_peak_hbm()
    bytes_per_launch = 56.0 * body.num_tets + 36.0 * body.num_verts
    avg_local_s = (local_ms / 1e3) / max(local_launches, 1)
    achieved = bytes_per_launch / avg_local_s / 1e9
    traffic = ncu_traffic_per_launch(WORKLOAD["workload"])
    local_roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                  "traffic": traffic, "peak_kind": peak_kind,
                  "kernel": "k_local<jacobi_form=%d>" % (1 if params.solver == 0 else 0),
                  "bytes_per_launch": bytes_per_launch, "avg_launch_us": avg_local_s * 1e6,
                  "launches": local_launches,
                  "share_of_step": (local_ms / step_ms_kernel_pass) if step_ms_kernel_pass > 0 else None,
                  "back_to_back": {"avg_launch_us": local_b2b_ms * 1e3,
                                   "sample": ("50 launches at each of the %d states of a run from rest, mean" % episode
                                              if episode else "3 x 200 launches on the final state, min"),
                                   "achieved": bytes_per_launch / (local_b2b_ms / 1e3) / 1e9,
                                   "frac": bytes_per_launch / (local_b2b_ms / 1e3) / 1e9 / peak}}
    roofline, kernels = local_roof, {"local": local_roof}
    if params.solver == 1 and solves > 0 and solve_bytes > 0:
        avg_solve_s = (solve_ms / 1e3) / solves
        s_ach = solve_bytes / avg_solve_s / 1e9
        solve_roof = {"bound": "hbm", "achieved": s_ach, "peak": peak, "unit": "GB/s", "frac": s_ach / peak,
                      "traffic": None, "peak_kind": peak_kind,
                      "kernel": {1: "k_chol_solve_cta", 2: "k_chol_solve_cluster", 4: "k_chol_solve_dsm",
                                 3: "k_chol_fwd_level + k_chol_bwd_level",
                                 5: "k_chol_solve_persistent"}.get(eng_info.get("solve_mode"), "solve"),
                      "bytes_per_launch": solve_bytes, "avg_launch_us": avg_solve_s * 1e6, "launches": solves,
                      "share_of_step": solve_ms / step_ms_kernel_pass if step_ms_kernel_pass > 0 else None,
                      "note": "one solve = forward + backward over the supernodal tree; bytes per the scalar "
                              "factor (8 B per nonzero) plus column pointers and right-hand sides"}
        kernels["solve"] = solve_roof
        if solve_ms > local_ms:
            roofline = solve_roof  # the dominant kernel of the Cholesky step
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline(cpu_body, params, 1 if leg else args.cpu_steps)
        if bodies is not None:
            cpu["sample"] += f"; the first 16 of the {len(bodies)} bodies"
    clk = clocks.summary()
    ref_gpu = None
    if not args.no_ref_gpu:
        ref_steps = {"c1": 20, "c2": 50, "c3": 3, "c4": 5}[workload_name]
        ref_sample = (f"{ref_steps} steps of the workload" if bodies is None else
                      f"{ref_steps} steps of the first 16 of the {len(bodies)} bodies concatenated into one system "
                      "(the reference's multi-body mode)")
        ref_gpu = reference_gpu(cpu_body, params, ref_steps, episode, ref_sample)
    acc = None
    if not args.no_accuracy:
        acc_steps = {"c1": 20, "c2": 20, "c3": 3, "c4": 5}[workload_name]
        acc = accuracy_vs_fp64(cpu_body, params, acc_steps, refine_sweep=workload_name == "c3",
                               ref_gpu=not args.no_ref_gpu)
        if bodies is not None:
            acc["sample"] = "first 16 bodies of the batch"
    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": nsteps,
        "warmup": nwarmup,
        "ms_per_step": t_max * 1e3 / nsteps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": dict(WORKLOAD, parallelism=f"replicas{world}" if world > 1 else "single"),
        "local_kernel": local_kernel,
        "roofline": roofline,
        "kernels": kernels,
        "autotune": tune,
        "collision": collision,
        "cpu_baseline": cpu,
        "reference_gpu": ref_gpu,
        "plain_drop_in": plain,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * 3 * 4 * nv,
                "d2h_bytes_per_step": 2 * 3 * 4 * nv},
        "gpu_launches": nsteps * launches_per_step(eng_info, params)
                        + (-(-nsteps // episode) if episode else 0),  # + the rest-state upload of every run
        "clocks": clk,
        "finite": finite and finite_timed,
        "accuracy": acc,
        "factor": factor,
    }
    if plain is not None:
        line["batched_vs_plain"] = {"ratio": value / plain["value"], "target": 5.0,
                                    "what": "batched value over the plain drop-in's on the same bodies"}
    return line


if __name__ == "__main__":
    main()
