#!/usr/bin/env python
"""Throughput of the SIMP hot path on one GB300: 64^3 SIMP iterations per second.

Workload (64^3 SIMP, the single-GPU configuration of the headline metric): 64x64x64
unit hex-8 voxels (262,144 elements, 823,875 DOFs), E0 = 1, Emin = 1e-9, nu = 0.3,
penal 3, rmin 2.0 (33-point filter), volfrac 0.25, z = 0 face clamped, uniform -z traction
of total 1 on the central 16x16 element patch of the top face (consistent nodal loads),
inner FP32 Jacobi-PCG with FP64 outer defect correction to rtol 1e-8, warm-started from the
previous displacement. One step = one OC iteration (solve, sensitivity, filter chain rule,
OC bisection) of that trajectory, all on the device.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs one independent replica per GPU (launched by torch.distributed.run); the line
reports the whole-job rate N*K / max-over-ranks time. --impl reference times the FP64 CPU
oracle (a C/OpenMP restatement of the reference solver, on all host threads) on the same
workload.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "64^3 SIMP iters/s & FEM solves/s, served vs plain (1×GB300, rel err ≤1e-6); p50/p99"
UNIT = "SIMP iterations/s"
WORKLOADS = {
    # the bench line: 64^3 SIMP (262,144 elements, 823,875 DOFs)
    "simp64": {"workload": "simp_64cube_top_patch", "grid": [64, 64, 64], "rmin": 2.0, "volfrac": 0.25,
               "load": "top_patch",
               "load_text": "z=0 clamped, -z traction (total 1) on the central 16x16 top-face patch"},
    # 32x16x16 cantilever (8,192 elements, 28,611 DOFs), for profiling and comparison
    "c0": {"workload": "simp_32x16x16_cantilever", "grid": [32, 16, 16], "rmin": 1.5, "volfrac": 0.3,
           "load": "cantilever", "load_text": "x=0 clamped, unit -z point load at node (32, 8, 0)"},
    # the serving stream (run_serve): Poisson arrivals, edges 24..96, three load cases
    "serve": {"workload": "fem_serving_stream", "grid": [64, 64, 64], "rmin": 2.0, "volfrac": 0.25,
              "load": "top_patch", "load_text": "per request: cantilever tip, top patch or torsion couple"},
    # 192x96x96 (1,769,472 elements, 5,447,811 DOFs): the PCG vectors no longer fit in L2
    "c4": {"workload": "simp_192x96x96_edge_line", "grid": [192, 96, 96], "rmin": 3.0, "volfrac": 0.2,
           "load": "edge_line",
           "load_text": "x=0 clamped, -z line load (total 1) along the bottom edge of the x=192 face"},
}
COMMON = {"penal": 3.0, "law": "E = 1e-9 + x^3 (1 - 1e-9)",
          "solver": "FP32 Jacobi-PCG inner, defect correction to rtol 1e-8 (double-float residual, FP64 u), warm start u_{k-1} + 0.5 (u_{k-1} - u_{k-2})",
          "oc": "bisection l1=0 l2=1e9 tol 1e-4 move 0.2 (SIMPSolver._oc_update)"}


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["apply"], default="simp64",
                    help="simp64 (the bench line), c0, c4, serve, or apply (the bare stiffness apply)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-steps", type=int, default=3,
                    help="OC iterations of the CPU oracle sample (the line reports their median)")
    ap.add_argument("--serve-requests", type=int, default=2000, help="requests of --workload serve")
    ap.add_argument("--line-serve-requests", type=int, default=300,
                    help="requests of the serving stream inside the default line (0: skip it)")
    ap.add_argument("--no-c4", action="store_true", help="skip the 192x96x96 kernel timings of the default line")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip timing the reference's own GPU FEM solve (from baseline/_ref) in the default line")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched FEM (served vs plain) measurement")
    ap.add_argument("--no-rows", action="store_true",
                    help="skip the evaluator / STL / generator measurements")
    ap.add_argument("--host-loop", action="store_true",
                    help="launch PCG iterations from the host (for kernel profilers) instead of the graph loop")
    return ap.parse_args()


def _wl(a):
    w = WORKLOADS[a.workload]
    g = tuple(w["grid"])
    cfg = {"workload": w["workload"], "grid": list(g), "elements": g[0] * g[1] * g[2],
           "dofs": 3 * (g[0] + 1) * (g[1] + 1) * (g[2] + 1), "rmin": w["rmin"], "volfrac": w["volfrac"],
           "load": w["load_text"], **COMMON}
    return w, g, cfg


def _line_keys(world: int) -> dict:
    """Config keys both arms report (their config dicts differ only in `solver`)."""
    return {"l2": "the GPU arm flushes L2 (256 MB write) before every timed step; inside a step the PCG "
                  "vectors stay in L2 when they fit (64^3: ~36 MB)",
            "parallelism": f"replicas x{world}" if world > 1 else "one replica"}


def _spec(w):
    from genpipeline_gb300.simp import SolveSpec

    return SolveSpec(grid=tuple(w["grid"]), penal=3.0, rmin=w["rmin"], volfrac=w["volfrac"], law="modified",
                     rtol=1e-8)


def _load_case(w):
    from genpipeline_gb300 import bcs

    return bcs.LOAD_CASES[w["load"]](*w["grid"])


# ---- clocks ------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples (every 50 ms) while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, mx, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
                pw.append(float(parts[3]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "power_w_max": max(pw) if pw else None, "reasons": sorted(reasons)}


# ---- distributed helpers -----------------------------------------------------------------
def _dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(t: float, world: int, device) -> float:
    """The slowest rank's time (all ranks get it): replicas report N * K / max time."""
    if world <= 1:
        return t
    import torch
    import torch.distributed as dist

    tt = torch.tensor([t], device=device, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def whole_job_rate(world: int, steps: int, t_max: float) -> float:
    """Units of all replicas (world x steps) over the slowest rank's time."""
    return world * steps / t_max


def _measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _profiled_traffic(workload="simp64"):
    """DRAM bytes per launch of the one-kernel PCG iteration from the committed ncu summary of the
    workload."""
    name = {"simp64": "cg_iteration__simp_64cube.md", "c4": "cg_iteration__simp_192x96x96.md"}.get(workload)
    if name is None:
        return None
    path = os.path.join(ROOT, "profiles", name)
    try:
        txt = open(path).read()
    except OSError:
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", txt)
    return float(m.group(1)) if m else None


def _cpu_threads():
    from oracle import oracle as O

    return O.num_threads()


# ---- batched FEM evaluation: 8 designs (4 x 64^3 + 4 x 32^3), served vs plain --------------
def batch_designs():
    from genpipeline_gb300 import designs as D
    from genpipeline_gb300.batch import FEMDesign

    out = []
    for k, n in enumerate((64, 64, 64, 64, 32, 32, 32, 32)):
        f, fixed = D.cantilever_case(n)
        out.append(FEMDesign((n, n, n), D.grf_density((n, n, n), k), f, fixed))
    return out


def measure_batch(repeats=2):
    """FEM solves/s of the 8-design batch: plain = one solve per design (graph-loop PCG, one
    design on the GPU at a time); served = the designs together in gbsimp_batch_round with the
    configuration the autotuner chose for this grid class (timed once per candidate during the
    warm-up, then cached); served_rule = the untuned default (one persistent launch, SMs in
    proportion to element counts). Cold starts (u0 = 0) everywhere."""
    import torch

    from genpipeline_gb300 import autotune as A
    from genpipeline_gb300.batch import BatchFEM, solve_plain

    solve_plain(batch_designs())  # warm-up: graphs, code paths
    tuner = A.default_tuner()
    BatchFEM(tuner=tuner).solve_all(batch_designs())  # tunes this grid class (cached afterwards)
    res = {}
    for name in ("plain", "served", "served_rule"):
        best = None
        for _ in range(repeats):
            ds = batch_designs()
            bf = BatchFEM(tuner=tuner) if name == "served" else BatchFEM()
            for d in ds:
                bf.upload(d)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            out = solve_plain(ds) if name == "plain" else bf.solve_all(ds)
            torch.cuda.synchronize()
            t = time.perf_counter() - t0
            if best is None or t < best[0]:
                best = (t, {d.grid + (i,): d for i, d in enumerate(out)}, out)
        res[name] = best
    cp = sorted(d.compliance for d in res["plain"][2])
    cs = sorted(d.compliance for d in res["served"][2])
    diff = max(abs(a - b) / abs(a) for a, b in zip(cp, cs))
    return {"workload": "8 designs: 4 x 64^3 + 4 x 32^3, GRF densities (length 6, mean U(0.2,0.5)), cantilever, "
                        "FP32 PCG + FP64 correction to rtol 1e-8, cold start",
            "plain": 8 / res["plain"][0], "served": 8 / res["served"][0],
            "served_over_plain": res["plain"][0] / res["served"][0],
            "served_rule": 8 / res["served_rule"][0],
            "autotune": A.summary(tuner, [d.grid for d in batch_designs()]),
            "max_compliance_rel_diff": diff,
            "pcg_iterations": sum(d.stats["iterations"] for d in res["served"][2]),
            "unit": "FEM solves/s"}


# ---- the rows next to the path: evaluator input step, evaluator, STL export, generator -----
def _cuda_time(fn, reps=5):
    import torch

    fn()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    e.synchronize()
    return s.elapsed_time(e) * 1e-3 / reps


def measure_rows(xphys64=None):
    """Short measurements of the evaluator input step, the served evaluator, the STL surface and
    the batched data generator (each a few seconds)."""
    import numpy as np
    import torch

    from genpipeline_gb300.designs import LatentFieldDecoder
    from genpipeline_gb300.engine import get_engine
    from genpipeline_gb300.fem.voxel_fem import VoxelFEMEvaluator
    from genpipeline_gb300.schema import DesignParameters

    eng = get_engine()
    rows = {}
    # evaluator input step: 16 x 64^3 -> 32^3 (zoom 0.5 + smooth_voxels)
    vols = torch.rand((16, 64, 64, 64), device="cuda")
    t = _cuda_time(lambda: eng.voxel_prep(vols, (32, 32, 32)))
    nbytes = 4 * (16 * 64 ** 3 + 16 * 32 ** 3)
    cpu = None
    try:
        from scipy.ndimage import gaussian_filter, zoom

        v0 = vols[0].cpu().numpy()
        c0 = time.perf_counter()
        z = zoom(v0, 0.5, order=1)
        _ = 1.0 / (1.0 + np.exp(-15.0 * (gaussian_filter(z, sigma=0.5) - 0.5)))
        cpu = {"value": 1.0 / (time.perf_counter() - c0), "unit": "grids/s", "cores": 1,
               "kind": "reference", "sample": "one 64^3 grid: scipy zoom(order=1) + the smooth_voxels steps"}
    except ImportError:
        pass
    rows["voxel_prep"] = {"workload": "16 x 64^3 -> 32^3 (zoom 0.5, Gaussian 0.5, logistic 15)",
                          "value": 16 / t, "unit": "grids/s", "ms_per_batch": t * 1e3,
                          "algorithmic_GBs": nbytes / t / 1e9, "cpu_baseline": cpu}
    # served evaluator vs one evaluation at a time (stand-in decoder, 16 latents)
    dec = LatentFieldDecoder(latent_dim=16, size=64, seed=3)
    rng = np.random.Generator(np.random.PCG64(4))
    params = [DesignParameters(h_mm=10.0, r_mm=2.0, latent_z=list(rng.standard_normal(16))) for _ in range(16)]
    ev = VoxelFEMEvaluator(use_gpu=True, vae_model=dec)
    ev.evaluate_batch(params[:2])
    torch.cuda.synchronize()
    c0 = time.perf_counter()
    served = ev.evaluate_batch(params)
    torch.cuda.synchronize()
    ts = time.perf_counter() - c0
    c0 = time.perf_counter()
    plain = [ev.evaluate(np.asarray(p.latent_z), dec) for p in params]
    torch.cuda.synchronize()
    tp = time.perf_counter() - c0
    diff = max(abs(s.compliance - p["compliance"]) / abs(p["compliance"]) for s, p in zip(served, plain))
    rows["evaluator"] = {"workload": "16 latents: decode (stand-in) + 64^3->32^3 prep + GPUVoxelFEM solve "
                                     "(penal 1, x_min clamped, 1000 N on x_max) to rtol 1e-8",
                         "served": 16 / ts, "plain": 16 / tp, "served_over_plain": tp / ts, "unit": "evaluations/s",
                         "max_compliance_rel_diff": diff}
    # STL surface of the benchmark's 64^3 design
    x = xphys64 if xphys64 is not None else torch.rand((64, 64, 64), device="cuda")
    x = x.reshape(64, 64, 64).contiguous()
    ntri = eng.marching_cubes(x, 0.5).shape[0]
    t = _cuda_time(lambda: eng.marching_cubes(x, 0.5))
    rows["stl_surface"] = {"workload": "isosurface at 0.5 of the 64^3 design (marching cubes, count + emit)",
                           "value": 63 ** 3 / t / 1e9, "unit": "Gcells/s", "ms": t * 1e3, "triangles": ntri}
    # batched SIMP generator vs one solver per sample
    from genpipeline_gb300 import bcs as B
    from genpipeline_gb300.topology.batch_simp import BatchSIMP
    from genpipeline_gb300.topology.simp_solver_gpu import SIMPSolverGPU
    from genpipeline_gb300.topology.topo_data_gen import TopoDataGenerator

    np.random.seed(11)
    gen = TopoDataGenerator(output_dir=os.path.join("/tmp", "gb_rows_gen"), n_iters=10)
    cases = [gen._draw() for _ in range(16)]
    BatchSIMP(cases[:2], bc_fn=B.generator).run(2)
    torch.cuda.synchronize()
    c0 = time.perf_counter()
    BatchSIMP(cases, bc_fn=B.generator).run(10)
    torch.cuda.synchronize()
    tb = time.perf_counter() - c0
    simple = [c for c in cases if not isinstance(c.bcs.get("load_dof"), list)
              and not isinstance(c.bcs.get("fixed_face"), list)][:4]
    c0 = time.perf_counter()
    for c in simple:
        SIMPSolverGPU(nx=c.grid[0], ny=c.grid[1], nz=c.grid[2], penal=c.penal, rmin=c.rmin,
                      boundary_conditions=c.bcs).run(volfrac=c.volfrac, n_iters=10, force_mag=c.force_mag)
    torch.cuda.synchronize()
    tsq = (time.perf_counter() - c0) / max(len(simple), 1)
    rows["generator"] = {"workload": "16 generator samples (medium grids, GEOM_BCS), 10 SIMP iterations each",
                         "batched": 16 / tb, "one_solver_per_sample": 1.0 / tsq,
                         "batched_over_one": (16 / tb) * tsq, "unit": "samples/s"}
    return rows


def run_apply(a):
    """The bare stiffness apply y = D K(x) D p (`apply_modal_kernel<PLAIN>`, no masks) at 64^3
    and 192x96x96 on seeded densities U(0.1, 1) and a seeded N(0, 1) vector. Warm: 20
    back-to-back launches, median of 5 groups. Cold: single launches after a 256 MB L2 flush,
    median of `--steps` (at least 5). Algorithmic bytes are 4*(2 n_dof + n_elem): p in, y out,
    the densities in."""
    import torch

    from genpipeline_gb300 import _lib as L
    from genpipeline_gb300.engine import Engine, n_dof, n_elem

    lib = L.load()
    eng = Engine()
    law = L.make_law("modified", 3.0)
    flush = torch.empty(256 * 2**20, dtype=torch.uint8, device="cuda")
    peak, peak_src = _measured_peak()
    n_cold = max(5, a.steps)

    def timed(fn):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) * 1e-3

    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    l0 = lib.gbsimp_launch_count()
    grids = {}
    for grid in [(64, 64, 64), (192, 96, 96)]:
        ne, nd = n_elem(grid), n_dof(grid)
        gen = torch.Generator(device="cuda").manual_seed(0)
        x = torch.rand(ne, device="cuda", generator=gen) * 0.9 + 0.1
        p = torch.randn(nd, device="cuda", generator=gen)
        y = torch.empty_like(p)
        for _ in range(max(3, a.warmup)):
            eng.apply(grid, law, x, p, None, y)
        torch.cuda.synchronize()

        def burst():
            for _ in range(20):
                eng.apply(grid, law, x, p, None, y)

        warm = statistics.median(timed(burst) / 20 for _ in range(5))
        cold = []
        for _ in range(n_cold):
            flush.zero_()
            cold.append(timed(lambda: eng.apply(grid, law, x, p, None, y)))
        cold = statistics.median(cold)
        alg = 4 * (2 * nd + ne)
        grids["x".join(map(str, grid))] = {
            "path": eng.apply_path(grid[2]), "alg_bytes": alg, "warm_us": warm * 1e6, "cold_us": cold * 1e6,
            "cold_GBs": alg / cold / 1e9, "cold_frac": alg / cold / 1e9 / peak,
            "dense_equiv_tflops": 1152 * ne / cold / 1e12}
    launches = lib.gbsimp_launch_count() - l0
    clk = clocks.stop()
    c4 = grids["192x96x96"]
    line = {"metric": "stiffness apply y = K(x) p, algorithmic GB/s (192x96x96, L2 flushed)",
            "value": c4["cold_GBs"], "unit": "GB/s", "n_gpus": 1, "steps": n_cold, "warmup": max(3, a.warmup),
            "ms_per_step": c4["cold_us"] * 1e-3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "ours",
            "config": {"workload": "stiffness_apply", "grids": list(grids), "densities": "U(0.1, 1), seed 0",
                       "law": COMMON["law"], "l2": "flushed (256 MB write) before each cold launch"},
            "roofline": {"bound": "hbm", "kernel": "apply_modal_kernel<PLAIN>", "achieved": c4["cold_GBs"],
                         "peak": peak, "peak_source": peak_src, "unit": "GB/s", "frac": c4["cold_frac"],
                         "traffic": None},
            "grids": grids, "gpu_launches": int(launches), "clocks": clk}
    print(json.dumps(line), flush=True)


SERVE_ROUND_ITERS = 256  # inner PCG iterations per round: admissions every few milliseconds


def measure_serving(n_requests: int, n_plain: int, clocks=None):
    """The serving stream: Poisson arrivals at 200/s, edge U{24,32,48,64,96}, three load cases,
    ~10% repeated designs, densities drawn by the client before the clock starts (they arrive
    with the requests); continuous batching (24 slots, rounds of SERVE_ROUND_ITERS inner
    iterations) with admission by free HBM. Beside it the plain form: one slot, one solve at a
    time, on the first `n_plain` of the same requests with the same payloads, all queued at
    t = 0 (its throughput is not limited by arrivals)."""
    import numpy as np

    from genpipeline_gb300 import _lib as L
    from genpipeline_gb300.serve import FEMServer, attach_payloads, request_stream

    lib = L.load()
    warm = FEMServer(max_slots=8, round_iters=SERVE_ROUND_ITERS)
    warm.run(attach_payloads(request_stream(40, rate=1000.0, seed=99)), realtime=False)
    reqs = attach_payloads(request_stream(n_requests, rate=200.0))
    if clocks is not None:
        clocks.start()
    l0 = lib.gbsimp_launch_count()
    srv = FEMServer(max_slots=24, round_iters=SERVE_ROUND_ITERS)
    summ = srv.run(reqs, realtime=True)
    launches = lib.gbsimp_launch_count() - l0
    clk = clocks.stop() if clocks is not None else None
    plain_reqs = request_stream(n_requests, rate=200.0)[:n_plain]
    for p_req, req in zip(plain_reqs, reqs):  # the same requests with the same payloads
        p_req.density = req.density
    plain = FEMServer(max_slots=1, round_iters=0).run(plain_reqs, realtime=False)
    # the served rate over the same first requests, for a like-for-like ratio
    first = sorted(reqs, key=lambda r: r.arrival)[:n_plain]
    plain_rate = plain["solves_per_s"]
    return {"workload": f"{n_requests} requests, Poisson arrivals at 200/s, edges U{{24,32,48,64,96}} (cubic), "
                        "loads U{cantilever tip, top patch, torsion}, ~10% repeats, GRF densities as payload, "
                        "FP32 PCG + FP64 correction to rtol 1e-8",
            "unit": "FEM solves/s", "served": summ, "served_solves_per_s": summ["solves_per_s"],
            "plain_solves_per_s": plain_rate, "served_over_plain": summ["solves_per_s"] / plain_rate,
            "plain": {"requests": plain["requests"], "note": "first requests of the same stream, one slot, "
                                                             "all queued at t=0"},
            "served_first_mean_ms": float(np.mean([r.latency for r in first]) * 1e3),
            "round_iters": SERVE_ROUND_ITERS, "max_slots": 24, "gpu_launches": int(launches), "clocks": clk}


def measure_c4(peak: float):
    """192x96x96 (1,769,472 elements, 5,447,811 DOFs) on seeded densities U(0.1, 1) with the
    line-load case's Dirichlet mask: the one-kernel PCG iteration (gbsimp_time_pcg_apply: 50
    graph-replayed launches, CUDA events on the stream, frozen scalars) and the bare stiffness
    apply y = D K(x) D p (apply_modal_kernel<PLAIN>), warm (20 back-to-back launches, median of
    5) and cold (one launch after a 256 MB L2 flush, median of 5). The PCG vectors (about
    218 MB) do not fit in the 129 MB L2."""
    import torch

    from genpipeline_gb300 import _lib as L
    from genpipeline_gb300 import bcs
    from genpipeline_gb300.engine import get_engine, n_dof, n_elem

    eng = get_engine()
    grid = (192, 96, 96)
    law = L.make_law("modified", 3.0)
    ne, nd = n_elem(grid), n_dof(grid)
    gen = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand(ne, device="cuda", generator=gen) * 0.9 + 0.1
    p = torch.randn(nd, device="cuda", generator=gen)
    y = torch.empty_like(p)
    _, fixed = bcs.edge_line_load(*grid)
    mask = torch.as_tensor(bcs.node_mask(*grid, fixed), device="cuda")
    flush = torch.empty(256 * 2**20, dtype=torch.uint8, device="cuda")
    per_launch = eng.time_pcg_apply(grid, law, x, mask, reps=50)
    pcg_bytes = 4 * (10 * nd + ne)

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1) * 1e-3

    for _ in range(3):
        eng.apply(grid, law, x, p, mask, y)
    torch.cuda.synchronize()
    warm = statistics.median(timed(lambda: [eng.apply(grid, law, x, p, mask, y) for _ in range(20)]) / 20
                             for _ in range(5))
    cold = []
    for _ in range(5):
        flush.zero_()
        cold.append(timed(lambda: eng.apply(grid, law, x, p, mask, y)))
    cold = statistics.median(cold)
    apply_bytes = 4 * (2 * nd + ne)
    return {"workload": "192x96x96, densities U(0.1,1) seed 0, x=0 clamped (line-load case's mask)",
            "pcg_iteration": {"kernel": "apply_modal_kernel<CG>", "launch_us": per_launch * 1e6,
                              "alg_bytes_per_launch": pcg_bytes, "achieved_GBs": pcg_bytes / per_launch / 1e9,
                              "frac": pcg_bytes / per_launch / 1e9 / peak, "traffic": _profiled_traffic("c4")},
            "bare_apply": {"kernel": "apply_modal_kernel<PLAIN>", "warm_us": warm * 1e6, "cold_us": cold * 1e6,
                           "alg_bytes_per_launch": apply_bytes, "cold_GBs": apply_bytes / cold / 1e9,
                           "cold_frac": apply_bytes / cold / 1e9 / peak, "warm_frac": apply_bytes / warm / 1e9 / peak},
            "peak_GBs": peak}


# The reference's own GPU path, run unmodified from its installed copy (baseline/_ref) in a
# child process: GPUVoxelFEM(voxels).solve() (gpu_fem_solver.py:76-133), i.e. COO -> CSR
# assembly, boundary conditions and SIMPSolverGPU._solve (torch sparse PCG, tol 1e-3, 200
# iterations) on the same voxel grid as ours.
_REF_GPU_CHILD = r"""
import json, sys, time
import numpy as np, torch
sys.path.insert(0, sys.argv[1])
from genpipeline.fem.gpu_fem_solver import GPUVoxelFEM
vox = np.load(sys.argv[2])
reps = int(sys.argv[3])
if len(sys.argv) > 4:  # the SPD element injected in place of the literal table (one method)
    from genpipeline.topology.simp_solver_gpu import SIMPSolverGPU
    ke = np.load(sys.argv[4])
    SIMPSolverGPU._get_Ke = staticmethod(lambda nu=0.3: ke)
r = GPUVoxelFEM(vox, device="cuda").solve()
torch.cuda.synchronize()
ts = []
for _ in range(reps):
    fem = GPUVoxelFEM(vox, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = fem.solve()
    torch.cuda.synchronize()
    ts.append(time.perf_counter() - t0)
print("REFGPU " + json.dumps({"seconds": ts, "result": {k: float(v) for k, v in r.items()}}))
"""


def measure_reference_gpu(n: int = 32, reps: int = 5, timeout: float = 240.0):
    """Per-solve time of the reference's GPUVoxelFEM.solve and of this library's drop-in on one
    n^3 voxel grid (GRF densities, seed 5; x_min clamped, 1000 N in -z spread over x_max; tol
    1e-3 / 200 PCG iterations on both sides, as gpu_fem_solver.py:96 asks). The reference runs
    twice: as shipped, and with the SPD element injected (SIMPSolverGPU._get_Ke only), since
    as shipped it assembles its literal element table, which is not symmetric positive
    definite. Unavailable when the reference copy is absent (it is installed into
    baseline/_ref, not committed)."""
    import tempfile

    import numpy as np
    import torch

    from genpipeline_gb300 import designs as D
    from genpipeline_gb300.engine import Engine
    from genpipeline_gb300.fem import GPUVoxelFEM

    ref_dir = os.path.join(ROOT, "baseline", "_ref")
    if not os.path.isdir(os.path.join(ref_dir, "genpipeline")):
        return {"unavailable": "the reference is not installed in baseline/_ref"}
    vox = D.grf_density((n, n, n), 5).reshape(n, n, n).astype(np.float32)
    runs = {}
    with tempfile.TemporaryDirectory() as td:
        path, kpath = os.path.join(td, "vox.npy"), os.path.join(td, "ke.npy")
        np.save(path, vox)
        np.save(kpath, Engine.ke_quadrature(0.3, 1.0))
        for name, extra in (("as_shipped", []), ("spd_element", [kpath])):
            try:
                out = subprocess.run([sys.executable, "-c", _REF_GPU_CHILD, ref_dir, path, str(reps), *extra],
                                     capture_output=True, text=True, timeout=timeout)
            except subprocess.TimeoutExpired:
                return {"unavailable": f"the reference's solve did not finish within {timeout:.0f} s"}
            line = [ln for ln in out.stdout.splitlines() if ln.startswith("REFGPU ")]
            if out.returncode != 0 or not line:
                return {"unavailable": f"reference run failed (rc {out.returncode}): {out.stderr.strip()[-300:]}"}
            runs[name] = json.loads(line[-1][7:])
    GPUVoxelFEM(vox).solve()
    torch.cuda.synchronize()
    ours_t = []
    for _ in range(reps):
        fem = GPUVoxelFEM(vox)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fem.solve()
        torch.cuda.synchronize()
        ours_t.append(time.perf_counter() - t0)
    ref = runs["as_shipped"]
    tr, to = statistics.median(ref["seconds"]), statistics.median(ours_t)
    return {"workload": f"GPUVoxelFEM.solve, {n}^3 GRF voxels (seed 5), {3 * (n + 1) ** 3} DOFs, x_min clamped, "
                        "1000 N -z over x_max, tol 1e-3 / 200 iterations",
            "reference": "genpipeline GPUVoxelFEM (torch sparse COO->CSR assembly + SIMPSolverGPU._solve), "
                         "unmodified, in a child process",
            "reference_s_per_solve": tr, "ours_s_per_solve": to, "speedup": tr / to,
            "reference_result": ref["result"], "ours_result": {k: float(v) for k, v in r.items()},
            "reference_spd_element": {"s_per_solve": statistics.median(runs["spd_element"]["seconds"]),
                                      "result": runs["spd_element"]["result"]},
            "note": "as shipped, the reference assembles its literal element table, which is not symmetric "
                    "positive definite, so its CG result is not a solution of an elasticity problem; with the "
                    "SPD element injected both sides solve the same system to 1e-3 (FP64 oracle compliance "
                    "680056.7 at rtol 1e-10)",
            "reps": reps}


def run_serve(a):
    """The serving stream alone (--workload serve), with its own JSON line."""
    import torch

    clocks = ClockSampler(torch.cuda.current_device())
    res = measure_serving(a.serve_requests, max(50, a.serve_requests // 10), clocks)
    summ, clk, launches = res["served"], res["clocks"], res["gpu_launches"]
    plain = {"requests": res["plain"]["requests"], "solves_per_s": res["plain_solves_per_s"]}
    line = {"metric": METRIC, "value": summ["solves_per_s"], "unit": "FEM solves/s", "n_gpus": 1,
            "steps": summ["requests"], "warmup": 40, "ms_per_step": 1e3 / summ["solves_per_s"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (outer residual in double-float FP32 pairs with FP64 u; compensated FP32 dots; FP64 compliance)", "data": "synthetic", "impl": "ours",
            "config": {"workload": "fem_serving_stream", "requests": summ["requests"], "rate_per_s": 200.0,
                       "edges": [24, 32, 48, 64, 96], "loads": ["cantilever", "top_patch", "torsion"],
                       "repeat_fraction": 0.1, "rtol": 1e-8, "max_slots": 24, "round_iters": SERVE_ROUND_ITERS,
                       "payload": "densities arrive with the requests (drawn by the client before the run); "
                                  "the server builds each (edge, load) case once"},
            "serving": summ, "plain_one_at_a_time": {"requests": plain["requests"], "solves_per_s": plain["solves_per_s"],
                                                     "note": "same stream, all requests queued at t=0, one slot"},
            "gpu_launches": int(launches), "clocks": clk,
            "e2e": {"value": summ["solves_per_s"], "unit": "FEM solves/s",
                    "h2d_bytes_per_step": None, "d2h_bytes_per_step": 8}}
    print(json.dumps(line), flush=True)


# ---- our arm -----------------------------------------------------------------------------
def run_ours(a):
    import numpy as np
    import torch
    import torch.distributed as dist

    from genpipeline_gb300 import _lib as L
    from genpipeline_gb300.simp import SimpProblem

    world, rank, local = _dist()
    if world > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", init_method="env://")
    dev = torch.device("cuda", torch.cuda.current_device())
    lib = L.load()
    w, GRID, WORKLOAD = _wl(a)
    spec = _spec(w)
    f, fixed = _load_case(w)
    prob = SimpProblem(spec, f, fixed, device=dev)
    prob.profile = bool(a.host_loop)
    nd, ne = prob.f.numel(), prob.x.numel()
    flush = torch.empty(256 * 2**20, dtype=torch.uint8, device=dev)  # > L2 (129 MB)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(a.warmup):
        prob.step()
    # the state the timed steps start from; the e2e steps below repeat the same iterations
    snap = prob.state()
    barrier()
    clocks = ClockSampler(dev.index if dev.index is not None else 0)
    clocks.start()
    launches0 = lib.gbsimp_launch_count()
    st0 = torch.cuda.Event(enable_timing=True)
    st1 = torch.cuda.Event(enable_timing=True)
    barrier()
    st0.record()
    stats = []
    for _ in range(a.steps):
        flush.zero_()
        stats.append(prob.step())
    st1.record()
    barrier()
    launches = lib.gbsimp_launch_count() - launches0  # our kernels only (the L2 flush is torch)
    t = st0.elapsed_time(st1) * 1e-3
    tmax = max_over_ranks(t, world, dev)
    value = whole_job_rate(world, a.steps, tmax)
    pcg_iters = sum(s["iterations"] for s in stats)
    # The dominant kernel, timed live on the final density field of the timed region:
    # 50 back-to-back launches replayed from a CUDA graph, CUDA events on this stream.
    per_launch = prob.eng.time_pcg_apply(GRID, prob.law, prob.xphys, prob.mask, reps=50)

    # ---- e2e: through the public API with host buffers --------------------------------
    # The same SIMP iterations as the timed region (state restored to its start). Each step
    # takes the design x from pinned host memory and returns the updated design and xPhys to
    # host memory (the displacement warm start stays on the device).
    prob.restore(snap)
    x_host = torch.empty(ne, dtype=torch.float32, pin_memory=True)
    xn_host = torch.empty(ne, dtype=torch.float32, pin_memory=True)
    xp_host = torch.empty(ne, dtype=torch.float32, pin_memory=True)
    x_host.copy_(snap[0])
    barrier()
    e0 = time.perf_counter()
    for _ in range(a.steps):
        prob.x.copy_(x_host, non_blocking=True)
        prob.step()
        xn_host.copy_(prob.x, non_blocking=True)
        xp_host.copy_(prob.xphys, non_blocking=True)
        torch.cuda.current_stream().synchronize()
        x_host, xn_host = xn_host, x_host
    barrier()
    te = max_over_ranks(time.perf_counter() - e0, world, dev)
    # the sampler spans the timed steps, the kernel timing and the e2e repeat of the same steps
    # (the timed region alone can be shorter than a few sampling periods)
    clk = clocks.stop()
    clk["window"] = "timed steps, kernel timing and their e2e repeat"
    e2e = {"value": whole_job_rate(world, a.steps, te), "unit": UNIT, "h2d_bytes_per_step": 4 * ne,
           "d2h_bytes_per_step": 8 * ne}

    # ---- the same timed steps with the outer residual's element products in FP64 ----------
    # (the default forms them in double-float FP32 pairs, FP64 u and norms; GB300's FP64 pipe
    # makes the FP64 form the slower one)
    state_after = prob.state()
    prob.restore(snap)
    prob.spec.residual_fp64 = True
    barrier()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record()
    its64 = 0
    for _ in range(a.steps):
        flush.zero_()
        its64 += prob.step()["iterations"]
    f1.record()
    barrier()
    prob.spec.residual_fp64 = False
    t64 = max_over_ranks(f0.elapsed_time(f1) * 1e-3, world, dev)
    fp64_residual = {"value": whole_job_rate(world, a.steps, t64), "unit": UNIT, "ms_per_step": t64 / a.steps * 1e3,
                     "pcg_iterations_per_step": its64 / a.steps,
                     "note": "the timed steps again with gbsimp_solve_opts.residual_fp64 = 1"}
    prob.restore(state_after)

    # ---- roofline of the dominant kernel (the one-kernel PCG iteration) -----------------
    path = prob.eng.apply_path(GRID[2])
    if path == "modal":
        # r_i, w_i, s_{i-1}, 1/diag, p_{i-1} and the densities in; s_i, r_{i+1}, p_i, w_{i+1}
        # out; x read and written every other iteration (two-step update): 10 words per DOF
        # on average, the basis of one standard Jacobi-PCG iteration
        alg_bytes = 4 * (10 * nd + ne)
        kname = "apply_modal_kernel<CG> (one single-reduction PCG iteration: s, r, u staging, w = DKDu, p, x)"
    else:
        alg_bytes = 4 * (7 * nd + ne)  # r, dinv, p_old, x_u, x in; p_new, Ap, x_u out
        kname = "apply_tile_kernel<PCG> (K(x)p fused with p = z + beta p, x update, p.Ap)"
    peak, peak_src = _measured_peak()
    achieved = alg_bytes / per_launch / 1e9
    roof = {"bound": "hbm", "kernel": kname,
            "achieved": achieved, "peak": peak, "peak_source": peak_src, "unit": "GB/s", "frac": achieved / peak,
            "traffic": _profiled_traffic(a.workload), "alg_bytes_per_launch": alg_bytes, "launch_us": per_launch * 1e6,
            "fp32_flops_per_launch_dense_equiv": 1152 * ne,
            "est_share_of_step": pcg_iters * per_launch / t}

    # ---- CPU baseline: the oracle on the same trajectory, from the GPU's state ----------
    cpu = None
    rel_err = None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        from genpipeline_gb300 import bcs
        from oracle import oracle as O

        mat = O.Material("modified", 3.0, emin=1e-9)
        ost = O.SimpState(GRID, O.ke_quadrature(), mat, w["rmin"], f, bcs.dof_mask(*GRID, fixed), w["volfrac"],
                          tol=1e-8)
        ost.x = prob.x.double().cpu().numpy().copy()
        ost.xphys = prob.xphys.double().cpu().numpy().copy()
        ost.u = prob.u.cpu().numpy().copy()
        # GPU compliance of the same xPhys (solve to 1e-8 from the same warm start)
        gpu_u0 = prob.u.clone()
        prob.solve()
        c_gpu = prob.compliance()
        prob.u.copy_(gpu_u0)
        n_cpu = max(1, a.cpu_sample_steps)
        per_step = []
        for k in range(n_cpu):
            c0 = time.perf_counter()
            ost.step()
            per_step.append(time.perf_counter() - c0)
            if k == 0:
                c_cpu = ost.compliance
        tc = statistics.median(per_step)
        rel_err = abs(c_gpu - c_cpu) / abs(c_cpu)
        cpu = {"value": 1.0 / tc, "unit": UNIT, "cores": _cpu_threads(), "kind": "port",
               "sample": f"median of {n_cpu} OC iterations of the same trajectory, started from the "
                         f"GPU state after {a.warmup + a.steps} iterations (FP64 C/OpenMP oracle)",
               "seconds_per_step": per_step}

    fem = None
    rows = None
    c4 = None
    serving = None
    if rank == 0 and a.workload == "simp64" and not a.no_batch:
        fem = measure_batch()
    if rank == 0 and a.workload == "simp64" and not a.no_rows:
        rows = measure_rows(prob.xphys)
    if rank == 0 and a.workload == "simp64" and not a.no_c4:
        c4 = measure_c4(_measured_peak()[0])
    if rank == 0 and a.workload == "simp64" and a.line_serve_requests > 0:
        serving = measure_serving(a.line_serve_requests, 50, ClockSampler(dev.index if dev.index is not None else 0))
    ref_gpu = None
    if rank == 0 and a.workload == "simp64" and not a.no_reference_gpu:
        ref_gpu = measure_reference_gpu()

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": tmax / a.steps * 1e3, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 (outer residual in double-float FP32 pairs with FP64 u; compensated FP32 dots; FP64 compliance)",
                "data": "synthetic", "impl": "ours",
                "config": dict(WORKLOAD, **_line_keys(world)),
                "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": int(launches),
                "clocks": clk, "pcg_iterations_per_step": pcg_iters / a.steps, "fp64_residual": fp64_residual,
                "compliance_rel_err_vs_fp64_oracle": rel_err, "fem_solves_per_s": fem, "c4": c4,
                "serving": serving, "reference_gpu_path": ref_gpu, "next_rows": rows}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


# ---- reference arm: the FP64 CPU oracle -------------------------------------------------
def run_reference(a):
    world, rank, _ = _dist()
    if rank != 0:
        return
    from genpipeline_gb300 import bcs
    from oracle import oracle as O

    w, GRID, WORKLOAD = _wl(a)
    f, fixed = _load_case(w)
    mat = O.Material("modified", 3.0, emin=1e-9)
    st = O.SimpState(GRID, O.ke_quadrature(), mat, w["rmin"], f, bcs.dof_mask(*GRID, fixed), w["volfrac"],
                     tol=1e-8)
    for _ in range(a.warmup):
        st.step()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        st.step()
    t = time.perf_counter() - t0
    value = a.steps / t
    cores = O.num_threads()
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": t / a.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": dict(WORKLOAD, **_line_keys(world), solver="FP64 Jacobi-PCG to rtol 1e-8, warm start (oracle port)"),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"OC iterations {a.warmup}..{a.warmup + a.steps - 1} of the trajectory "
                                       "(FP64 C/OpenMP restatement of SIMPSolver, all host threads)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    a = _args()
    if a.workload == "apply" and a.impl == "reference":
        sys.exit("bench.py: --workload apply has no reference arm (the reference times whole SIMP iterations)")
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "serve":
        run_serve(a)
    elif a.workload == "apply":
        run_apply(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
