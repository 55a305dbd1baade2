"""Benchmark: steps/s of the per-step grid hot path on one GB300 (or N replicas).

Workload (one "step" = one pass of the hot path): a 256^3 unit-cube MAC grid, FP32 fields, the
spheres-over-pool scene (pool y < 0.3, three seeded spheres r in [0.08, 0.2], room walls and a
seeded solid box holding 5-10 % of the cells); each step extrapolates velocity and level set,
advects the level set (WENO6 sampling, RK2 backtrace) and the velocity (trilinear, RK3),
adds gravity (9.8), rebuilds the valid masks and solves the ghost-fluid pressure to relative
residual 1e-6, then updates the velocity -- update_second_order of the reference without
reinitialisation.  dt = min(CFL 1.0 step, 1/60 s).

value      steps/s with the mixed solver (FP32 multigrid PCG inside FP64 refinement), inputs
           resident in HBM, CUDA events on the library's stream.
plain_fp64 the same workload with plain FP64 PCG (Jacobi); mg_fp64: FP64 multigrid PCG.
e2e        steps/s through the C ABI with host buffers: every step uploads phi, u, v, w from
           pinned host memory and downloads phi, u, v, w and the pressure (asynchronous copies
           pipelined field by field on two streams).
roofline   the dominant kernel class, algorithmic bytes / device time over the timed region.
cpu_baseline  the CPU oracle (OpenMP restatement with MIC(0)-PCG) on one step of the workload.

--impl reference times the reference's CPU path for the same workload: the oracle port (the
reference's own sources compile only against a stand-in Eigen from the reference tree, which
is not present where the benchmark runs).  Under torchrun rank 0 alone runs it.
"""

import argparse
import importlib.util
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
METRIC = "steps/s at 256^3, mixed vs plain FP64 GPU PCG, same GB300, rel. resid 1e-6"
KC_NAMES = ["advect_phi", "advect_vel", "extrapolate", "masks", "build", "dir_spmv", "update", "mg_smooth_fine",
            "mg_restrict_fine", "mg_coarse", "residual_fp64", "other"]


def load_package():
    name = "eulerian_liquid_gb300"
    if name in sys.modules:
        return sys.modules[name]
    pkg_dir = os.path.join(ROOT, "eulerian-liquid_gb300")
    spec = importlib.util.spec_from_file_location(name, os.path.join(pkg_dir, "__init__.py"),
                                                  submodule_search_locations=[pkg_dir])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (pool256: 20, batch32: 100)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="pool256", choices=["pool256", "batch32", "warmstart128", "dam64", "dam128"],
                    help="pool256: one 256^3 scene (the headline); batch32: 32 scenes in one graph per step; "
                         "warmstart128: record, train and evaluate the learned warm start at 128^3; "
                         "dam64 / dam128: the FP64 dam-break workloads at 64^3 and 128^3 (GPU vs the CPU path)")
    ap.add_argument("--ws-n", type=int, default=128, help="warmstart128: grid size")
    ap.add_argument("--ws-samples", type=int, default=4000, help="warmstart128: recorded solves (capped by memory)")
    ap.add_argument("--ws-steps-per-scene", type=int, default=20)
    ap.add_argument("--ws-epochs", type=int, default=2)
    ap.add_argument("--ws-batch", type=int, default=8)
    ap.add_argument("--ws-eval-scenes", type=int, default=6)
    ap.add_argument("--scenes", type=int, default=32, help="batch32: number of scenes")
    ap.add_argument("--no-tune", action="store_true", help="pool256 / batch32: default launch shapes, no autotuning")
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--plain-steps", type=int, default=None, help="timed steps of the plain FP64 arm")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--error-steps", type=int, default=2)
    args = ap.parse_args(argv)
    if args.steps is None:
        args.steps = {"batch32": 100, "dam64": 100, "dam128": 200}.get(args.workload, 20)
    return args


# ---- distributed plumbing (replicas: no data-path collective) -----------------------------

class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as td
            backend = "nccl" if _cuda_available() else "gloo"
            td.init_process_group(backend=backend)
            self.pg = td

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, value):
        if not self.pg:
            return value
        import torch
        dev = "cuda" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def _cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def aggregate(values_per_rank, steps, world):
    """Whole-job steps/s from each rank's elapsed ms: all ranks' steps over the slowest rank."""
    slowest = max(values_per_rank)
    return steps * world / (slowest / 1000.0), slowest / steps


# ---- clocks during the timed region --------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "100"], stdout=open(self.path, "w"),
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = [r.split(", ") for r in open(self.path).read().strip().splitlines() if r.strip()]
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[q] for r in rows if len(r) >= 9 for q in range(4) if r[5 + q].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---- our arm -------------------------------------------------------------------------------

def workload(el, n, seed):
    return el.scenes.spheres_pool(n, seed)


def step_params(el, solver, tol):
    return el.step_params(trace_phi=el.TRACE_RK2, sample_phi=el.SAMPLE_WENO6, trace_vel=el.TRACE_RK3,
                          sample_vel=el.SAMPLE_TRILINEAR, gravity=9.8, extrapolation_layers=10, solver=solver,
                          tol=tol, max_iter=20000, check_every=4 if solver == el.SOLVER_MIXED else 16)


def next_dt(sim, cfl=1.0, frame=1.0 / 60.0):
    return min(sim.calc_time_step(cfl), frame)


def make_sim(el, torch, n, seed):
    sim = el.Simulator(n, n, n, dtype=el.EL_F32, device=torch.cuda.current_device())
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    sim.init_scene(workload(el, n, seed))
    return sim, stream


def timed_steps(el, torch, sim, stream, params, steps, dist, profile_mask=0, sampler=None):
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    stats = []
    dist.barrier()
    torch.cuda.synchronize()
    if profile_mask:
        sim._check(sim.lib.el_ctx_profile_begin(sim.h, profile_mask), "profile_begin")
    launches0 = sim.kernel_launches()
    if sampler:
        sampler.start()
    ev0.record(stream)
    for _ in range(steps):
        dt = next_dt(sim)
        stats.append(sim.step(dt, params))
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop() if sampler else None
    dist.barrier()
    launches = sim.kernel_launches() - launches0
    prof = None
    if profile_mask:
        prof = read_profile(el, sim)
    return ev0.elapsed_time(ev1), stats, launches, prof, clocks


def read_profile(el, sim):
    import ctypes as C

    class Entry(C.Structure):
        _fields_ = [("launches", C.c_int64), ("ms", C.c_double), ("bytes", C.c_double)]

    out = (Entry * 12)()
    sim.lib.el_ctx_profile_end.argtypes = [C.c_void_p, C.c_void_p]
    sim._check(sim.lib.el_ctx_profile_end(sim.h, C.cast(out, C.c_void_p)), "profile_end")
    return {KC_NAMES[c]: {"launches": int(out[c].launches), "ms": out[c].ms, "bytes": out[c].bytes}
            for c in range(12) if out[c].launches}


def pressure_error(el, sim, params_mixed, n_steps):
    """Mixed-solver pressure vs this GPU's FP64 multigrid PCG solve to 1e-12 from the same step
    input (the CPU oracle is not run here; its comparison is a GPU test at 128^3)."""
    import numpy as np
    ref_params = step_params(el, el.SOLVER_MG_FP64, 1e-12)
    fields = ["phi", "u", "v", "w", "valid_u", "valid_v", "valid_w"]
    errs = []
    for _ in range(n_steps):
        saved = {f: sim.download(f) for f in fields}
        dt = next_dt(sim)
        sim.step(dt, ref_params)
        p_ref = sim.download("pressure").astype(np.float64)
        for f in fields:
            sim.upload(f, saved[f])
        sim.step(dt, params_mixed)
        p = sim.download("pressure").astype(np.float64)
        errs.append(float(np.linalg.norm(p - p_ref) / max(np.linalg.norm(p_ref), 1e-300)))
    return errs


def e2e_batch_steps(el, torch, sims, batch, steps):
    """Steps through the C ABI with pinned host buffers: every step uploads each scene's inputs
    (phi, u, v, w) from host memory, runs one batch step and downloads its results (phi, u, v, w,
    pressure).  The transfers are pipelined field by field with el_download_async /
    el_upload_async on two streams: the downloads start when the step is done, and each field's
    upload for the next step starts as soon as that field's download has landed, so downloads
    and uploads of different fields share the full-duplex host link."""
    ins = ("u", "v", "w", "phi")
    outs = ins + ("pressure",)
    host = []
    for sim in sims:
        h = {}
        for f in outs:
            h[f] = torch.empty(sim.shape(f), dtype=torch.float32, pin_memory=True).numpy()
            sim.download(f, out=h[f])
        host.append(h)
    h2d = sum(h[f].nbytes for h in host for f in ins)
    d2h = sum(h[f].nbytes for h in host for f in outs)
    s_down, s_up = torch.cuda.Stream(), torch.cuda.Stream()
    scene_streams = [torch.cuda.ExternalStream(sim.stream_handle) for sim in sims]
    ev_step = [torch.cuda.Event() for _ in sims]
    ev_field = [{f: torch.cuda.Event() for f in outs} for _ in sims]
    ev_up = torch.cuda.Event()

    def uploads(wait_downloads):
        for q, sim in enumerate(sims):
            for f in ins:
                if wait_downloads:
                    s_up.wait_event(ev_field[q][f])
                sim.upload_async(f, host[q][f], s_up.cuda_stream)
        ev_up.record(s_up)
        for st in scene_streams:
            st.wait_event(ev_up)

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    uploads(False)  # the first step's inputs
    for step in range(steps):
        batch.step(1)
        for q, sim in enumerate(sims):
            ev_step[q].record(scene_streams[q])
            s_down.wait_event(ev_step[q])
            for f in outs:
                sim.download_async(f, host[q][f], s_down.cuda_stream)
                ev_field[q][f].record(s_down)
        if step + 1 < steps:
            uploads(True)  # the next step's inputs, from the host buffers just filled
    torch.cuda.synchronize()
    return steps / (time.perf_counter() - t0), h2d, d2h


def e2e_steps(el, torch, sim, stream, params, steps, dtype=None):
    """Steps through the C ABI with host buffers: inputs up, results down, every step."""
    host = {}
    for f in ("phi", "u", "v", "w", "pressure"):
        t = torch.empty(sim.shape(f), dtype=dtype or torch.float32, pin_memory=True)
        host[f] = t.numpy()
        host[f][...] = sim.download(f)
    h2d = sum(host[f].nbytes for f in ("phi", "u", "v", "w"))
    d2h = sum(host[f].nbytes for f in ("phi", "u", "v", "w", "pressure"))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        for f in ("phi", "u", "v", "w"):
            sim.upload(f, host[f])
        dt = next_dt(sim)
        sim.step(dt, params)
        for f in ("phi", "u", "v", "w", "pressure"):
            sim.download(f, out=host[f])
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t0
    return steps / elapsed, h2d, d2h


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# Launches shorter than this are timed mostly as the CUDA events around them: a class of such
# launches (the coarse multigrid levels, kernels of a few microseconds) is listed in the
# breakdown but not taken as the roofline's kernel.
ROOFLINE_MIN_LAUNCH_US = 20.0
# Classes whose profiled records each time exactly one kernel launch (the roofline is per
# launch); extrapolate, masks, build and other time groups of kernels and memsets.
SINGLE_KERNEL_CLASSES = ("advect_phi", "advect_vel", "dir_spmv", "update", "mg_smooth_fine", "mg_restrict_fine",
                         "mg_coarse", "residual_fp64")
# The finest level of the mixed solver: where the grid allows, every launch of these four classes
# is the one z-marching tile kernel (march_kernel, csrc/el_march.cu) in one of its six modes
# (direction + A p, update fused with the pre-smoother, the sweeps, restriction), so they are
# taken together as one kernel: bytes and time summed over the modes.
FINE_SOLVER = "finest_level_solver"
FINE_SOLVER_CLASSES = ("dir_spmv", "update", "mg_smooth_fine", "mg_restrict_fine")
# What bounds each class (from ncu): the HBM fraction is the roofline of the stencil and copy
# classes; the advection kernels issue far more instructions than their bytes need (WENO6
# weights, RK backtraces) and are bound by instruction issue, so their HBM fraction is listed
# for completeness only.
CLASS_BOUND = {"advect_phi": "issue", "advect_vel": "issue", "extrapolate": "latency"}

# DRAM traffic per launch of a kernel class, from ncu captures of the 256^3 workload
# (dram__bytes_read.sum + dram__bytes_write.sum; for the finest-level solver the six tile-kernel
# modes of one PCG iteration and V-cycle, weighted by their launches per iteration).
NCU_TRAFFIC_PER_LAUNCH = {"finest_level_solver": 163.4e6}


def with_fine_solver(breakdown):
    """The breakdown with the finest-level solver classes also summed into FINE_SOLVER."""
    parts = [breakdown[k] for k in FINE_SOLVER_CLASSES if k in breakdown]
    out = dict(breakdown)
    if parts:
        out[FINE_SOLVER] = {"launches": sum(p["launches"] for p in parts), "ms": sum(p["ms"] for p in parts),
                            "bytes": sum(p["bytes"] for p in parts)}
    return out


def class_mask(name):
    names = FINE_SOLVER_CLASSES if name == FINE_SOLVER else (name,)
    m = 0
    for k in names:
        m |= 1 << KC_NAMES.index(k)
    return m


def dominant_class(breakdown, fine_solver_on=True):
    """The single-kernel class with the most device time among those whose launches average at
    least ROOFLINE_MIN_LAUNCH_US (all classes if none does); with the finest-level tile kernels
    on, their four classes compete as the one kernel FINE_SOLVER."""
    b = with_fine_solver(breakdown) if fine_solver_on else dict(breakdown)
    singles = set(SINGLE_KERNEL_CLASSES)
    if fine_solver_on and FINE_SOLVER in b:
        singles = (singles - set(FINE_SOLVER_CLASSES)) | {FINE_SOLVER}
    big = {k: v for k, v in b.items()
           if k in singles and v["launches"] and v["ms"] * 1e3 / v["launches"] >= ROOFLINE_MIN_LAUNCH_US}
    pool = big or breakdown
    return max(pool, key=lambda k: pool[k]["ms"])


def class_fractions(breakdown, hbm):
    """Per class of the breakdown: algorithmic GB/s, its fraction of the HBM peak, and the bound."""
    out = {}
    for k, v in with_fine_solver(breakdown).items():
        if v["ms"] > 0:
            gbs = v["bytes"] / (v["ms"] / 1e3) / 1e9
            out[k] = {"gbs": gbs, "hbm_frac": gbs / hbm, "bound": CLASS_BOUND.get(k, "hbm"),
                      "us_per_launch": v["ms"] * 1e3 / max(1, v["launches"])}
    return out


def headline_workload_name(n, seed, tol):
    """The headline workload, named the same in both arms."""
    return (f"spheres_pool {n}^3 seed {seed}: pool y<0.3 + 3 seeded spheres r in [0.08,0.2], room walls, "
            f"seeded solid box 5-10% of cells; phi WENO6/RK2, velocity trilinear/RK3, g 9.8, CFL 1.0, "
            f"pressure to rel. resid {tol}")


def run_ours(args, dist):
    import torch

    el = load_package()
    el.load()
    torch.cuda.set_device(dist.local_rank)
    n, K, W = args.n, args.steps, max(3, args.warmup)
    params = step_params(el, el.SOLVER_MIXED, args.tol)

    sim, stream = make_sim(el, torch, n, args.seed)
    # launch shapes tuned on the scene itself (a batch of one; untimed, the scene restored after)
    tuned = None
    if not args.no_tune:
        t0 = time.perf_counter()
        tuned = el.autotune.tune_batch(el, [sim], params, 1.0, 1.0 / 60.0, device_name=torch.cuda.get_device_name(),
                                       steps=5)
        tuned["seconds"] = time.perf_counter() - t0
    for _ in range(W):
        sim.step(next_dt(sim), params)
    # class breakdown on two untimed, profiled steps (eager launches with CUDA events around each),
    # to pick the dominant kernel class
    _, _, _, breakdown, _ = timed_steps(el, torch, sim, stream, params, 2, dist, profile_mask=(1 << 12) - 1)
    fine_on = sim.march_on()
    dominant = dominant_class(breakdown, fine_on)
    # the timed region: one CUDA graph launch per step (the scene as a batch of one: dt, the
    # step and the solver's loops all decided on the device)
    batch = el.Batch([sim], params=params, cfl=1.0, dt_frame=1.0 / 60.0)
    bstream = torch.cuda.ExternalStream(batch.stream)
    batch.step(W)
    batch.sync()
    batch.reset_stats()
    sampler = ClockSampler(dist.local_rank) if dist.rank == 0 else None
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    dist.barrier()
    torch.cuda.synchronize()
    if sampler:
        sampler.start()
    ev0.record(bstream)
    batch.step(K)
    ev1.record(bstream)
    torch.cuda.synchronize()
    clocks = sampler.stop() if sampler else None
    dist.barrier()
    elapsed = dist.max(ev0.elapsed_time(ev1))
    value, ms_per_step = aggregate([elapsed], K, dist.world)
    bst = batch.stats()[0]
    launches = bst["kernels"]
    ok = bst["unconverged_steps"] == 0 and bst["bad_steps"] == 0 and bst["no_fluid_steps"] == 0
    e2e = None
    if not args.no_e2e:
        e2e_value, h2d, d2h = e2e_batch_steps(el, torch, [sim], batch, max(3, K // 2))
        slowest_step_s = dist.max(1.0 / e2e_value)
        e2e = {"value": dist.world / slowest_step_s, "unit": "steps/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h,
               "path": "el_upload_async, el_batch_step, el_download_async (pinned host buffers, two copy streams)"}
    batch.close()
    # roofline: the dominant class's launches over K eager steps, CUDA events around each launch
    _, stats, _, prof, _ = timed_steps(el, torch, sim, stream, params, K, dist,
                                       profile_mask=class_mask(dominant))
    err = pressure_error(el, sim, params, args.error_steps) if args.error_steps else []
    sim.close()
    iters_mean = bst["iterations"] / max(1, bst["steps"])
    relres = bst["max_relres"]

    plain = mgd = None
    if not args.no_plain:
        Kp = args.plain_steps or max(3, K // 4)
        for solver, key in ((el.SOLVER_JACOBI_FP64, "plain"), (el.SOLVER_MG_FP64, "mg")):
            p = step_params(el, solver, args.tol)
            s2, st2 = make_sim(el, torch, n, args.seed)
            for _ in range(W):
                s2.step(next_dt(s2), p)
            el_ms, stats2, _, _, _ = timed_steps(el, torch, s2, st2, p, Kp, dist)
            el_ms = dist.max(el_ms)
            v2, ms2 = aggregate([el_ms], Kp, dist.world)
            rec = {"value": v2, "ms_per_step": ms2, "steps": Kp,
                   "pcg_iterations_mean": statistics.mean(s["iterations"] for s in stats2),
                   "relres_max": max(s["relres"] for s in stats2)}
            if key == "plain":
                plain = rec
            else:
                mgd = rec
            s2.close()

    hbm, peak_kind = peaks()
    d = with_fine_solver(prof)[dominant]
    achieved = d["bytes"] / (d["ms"] / 1e3) / 1e9
    traffic = NCU_TRAFFIC_PER_LAUNCH.get(dominant) if n == 256 else None
    roofline = {"kernel": dominant, "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_kind": peak_kind, "traffic": traffic,
                "traffic_source": "ncu capture of this workload (per launch)" if traffic else None,
                "launches": d["launches"], "avg_launch_us": d["ms"] * 1e3 / max(1, d["launches"]),
                "bytes_per_launch": d["bytes"] / max(1, d["launches"])}
    out = {
        "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": dist.world, "steps": K, "warmup": W,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 fields; pressure solve f32 inner / f64 refinement", "data": "synthetic",
        "config": {"workload": headline_workload_name(n, args.seed, args.tol),
                   "n": n, "seed": args.seed, "parallelism": f"replicas x{dist.world}",
                   "l2": "inputs larger than L2 (fields + solver vectors > 2 GB), no flush",
                   "tuning": tuned},
        "mixed": {"pcg_iterations_mean": iters_mean, "relres_max": relres, "all_converged": ok,
                  "pressure_rel_err_vs_gpu_mg_fp64_1e-12": err,
                  "pressure_vs_cpu_oracle": "the mixed solve against a CPU oracle FP64 PCG solve to 1e-12 of the "
                                            "same system is a GPU test at 128^3 "
                                            "(tests/test_gpu_configs.py::test_mixed_solver_128_pressure_vs_fp64_oracle_solve); "
                                            "here the reference solve is this GPU's FP64 multigrid PCG to 1e-12",
                  "timed_path": "one CUDA graph launch per step (el_batch of one scene)"},
        "plain_fp64": plain, "mg_fp64": mgd,
        "mixed_over_plain": (value / plain["value"]) if plain else None,
        "roofline": roofline, "kernel_breakdown_2_steps": breakdown,
        "class_rooflines_2_steps": class_fractions(breakdown, hbm), "gpu_launches": launches,
        "clocks": clocks, "e2e": e2e,
    }
    if dist.rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(n, args.seed, args.tol, steps=1)
    return out


# ---- batched scenes ---------------------------------------------------------------------------

BATCH_METRIC = "aggregate cell-updates/s, batched scenes (one CUDA graph launch per step)"


def batch_specs(el, args):
    return el.scenes.batch_scenes(args.scenes, args.seed)


def batch_workload_name(args):
    return (f"batch of {args.scenes} scenes, seed {args.seed}: sizes U{{48..160}} per axis, fill 0.2-0.6, "
            f"dam break or sphere drop, room walls; FP32 fields, mixed PCG (FP64 refinement) to rel. resid "
            f"{args.tol}; phi WENO6/RK2, velocity trilinear/RK3, g 9.8, CFL 1.0 sub-steps of 1/60 s frames")


def step_bytes(el, sim, params):
    """Algorithmic bytes of one step of a scene, summed over the kernel classes (one profiled step)."""
    sim._check(sim.lib.el_ctx_profile_begin(sim.h, (1 << 12) - 1), "profile_begin")
    sim.step(next_dt(sim), params)
    prof = read_profile(el, sim)
    return sum(v["bytes"] for v in prof.values())


def run_batch(args, dist):
    import numpy as np
    import torch

    el = load_package()
    el.load()
    torch.cuda.set_device(dist.local_rank)
    K, W = args.steps, max(3, args.warmup)
    params = step_params(el, el.SOLVER_MIXED, args.tol)
    specs = batch_specs(el, args)
    dev = torch.cuda.current_device()
    sims = []
    for spec in specs:
        sim = el.Simulator(*spec["shape"], dtype=el.EL_F32, device=dev)
        sim.init_scene(spec)
        sims.append(sim)
    cells = sum(s.ni * s.nj * s.nk for s in sims)
    # algorithmic bytes of a step of every scene, from one profiled step of a copy of each
    total_bytes = 0.0
    for spec in specs:
        with el.Simulator(*spec["shape"], dtype=el.EL_F32, device=dev) as c:
            c.init_scene(spec)
            total_bytes += step_bytes(el, c, params)
    tuned = None
    if not args.no_tune:
        t0 = time.perf_counter()
        tuned = el.autotune.tune_batch(el, sims, params, 1.0, 1.0 / 60.0, device_name=torch.cuda.get_device_name())
        tuned["seconds"] = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    batch = el.Batch(sims, params=params, cfl=1.0, dt_frame=1.0 / 60.0)
    capture_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(batch.stream)
    batch.step(W)
    batch.sync()
    batch.reset_stats()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(dist.local_rank) if dist.rank == 0 else None
    dist.barrier()
    torch.cuda.synchronize()
    if sampler:
        sampler.start()
    ev0.record(stream)
    batch.step(K)
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop() if sampler else None
    dist.barrier()
    elapsed = dist.max(ev0.elapsed_time(ev1))
    stats = batch.stats()
    launches = sum(s["kernels"] for s in stats)
    ms_per_step = elapsed / K
    value = cells * K * dist.world / (elapsed / 1e3)

    e2e = None
    if not args.no_e2e:
        Ke = max(3, min(K, 10))
        e2e_steps_s, h2d, d2h = e2e_batch_steps(el, torch, sims, batch, Ke)
        e2e_s = dist.max(1.0 / e2e_steps_s)
        e2e = {"value": cells * dist.world / e2e_s, "unit": "cell-updates/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "steps": Ke}
    batch.close()
    for s in sims:
        s.close()

    hbm, peak_kind = peaks()
    achieved = total_bytes / (ms_per_step / 1e3) / 1e9
    roofline = {"kernel": "whole step, all scenes (every kernel class)", "bound": "hbm", "achieved": achieved,
                "peak": hbm, "unit": "GB/s", "frac": achieved / hbm, "peak_kind": peak_kind, "traffic": None,
                "bytes_per_launch": total_bytes}
    iters = [s["iterations"] / max(1, s["steps"]) for s in stats]
    out = {
        "metric": BATCH_METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": dist.world, "steps": K,
        "warmup": W, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 fields; pressure solve f32 inner / f64 refinement", "data": "synthetic",
        "config": {"workload": batch_workload_name(args), "scenes": args.scenes, "seed": args.seed,
                   "cells": cells, "sizes": [list(s["shape"]) for s in specs],
                   "parallelism": f"replicas x{dist.world}",
                   "l2": f"inputs larger than L2 ({cells} cells, > 1 GB of fields), no flush"},
        "batch": {"graph_capture_s": capture_s, "tuning": tuned, "pcg_iterations_per_step_mean": statistics.mean(iters),
                  "unconverged_steps": sum(s["unconverged_steps"] for s in stats),
                  "no_fluid_steps": sum(s["no_fluid_steps"] for s in stats),
                  "bad_steps": sum(s["bad_steps"] for s in stats),
                  "max_relres": max(s["max_relres"] for s in stats),
                  "simulated_time_s": [round(s["time"], 6) for s in stats]},
        "roofline": roofline, "gpu_launches": launches, "graph_launches": K, "clocks": clocks, "e2e": e2e,
    }
    if dist.rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_batch(specs, args.tol)
    return out


def cpu_baseline_batch(specs, tol, which=0):
    """One step of one scene of the batch on the CPU oracle, as cell-updates/s."""
    import numpy as np

    sys.path.insert(0, ROOT)
    import oracle as O
    from oracle import step as S

    spec = specs[which]
    ni, nj, nk = spec["shape"]
    phi, solid = O.rasterise(spec, np.float32)
    wts = O.compute_weights(solid)
    st = S.initial_state(phi, wts, O.cell_solid_phi(solid), O.float_dx(ni, np.float32))
    t0 = time.perf_counter()
    dt = min(O.calc_time_step(st["u"], st["v"], st["w"], st["dx"], 1.0), 1.0 / 60.0)
    st, _ = S.step(st, dt, 0, 1, 1, 0, 9.8, tol=tol, maxit=20000)
    elapsed = time.perf_counter() - t0
    return {"value": ni * nj * nk / elapsed, "unit": "cell-updates/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"1 step of scene {which} ({ni}x{nj}x{nk}) of the batch on the CPU oracle (OpenMP, FP32 "
                      f"fields, MIC(0)-PCG FP64 to {tol}; {st['pcg_iterations']} iterations), {elapsed:.2f} s"}


# ---- FP64 dam-break workloads (64^3 trilinear RK2; 128^3 WENO6/RK3 with a seeded velocity) ----------

DAM_METRIC = "steps/s, FP64 dam break, plain FP64 GPU PCG to 1e-6"


def dam_setup(args):
    n = 64 if args.workload == "dam64" else 128
    weno = args.workload == "dam128"
    return n, weno


def dam_state(el, n, weno, seed):
    """Initial fields: the dam break scene; at 128^3 a seeded velocity U(-1e-3, 1e-3) on every face."""
    import numpy as np
    spec = el.scenes.dam_break(n)
    fields = {}
    if weno:
        rng = np.random.default_rng(seed)
        for f, shape in (("u", (n, n, n + 1)), ("v", (n, n + 1, n)), ("w", (n + 1, n, n))):
            fields[f] = rng.uniform(-1e-3, 1e-3, shape)
    return spec, fields


def dam_params(el, weno, tol):
    if weno:
        return el.step_params(trace_phi=el.TRACE_RK2, sample_phi=el.SAMPLE_WENO6, trace_vel=el.TRACE_RK3,
                              sample_vel=el.SAMPLE_TRILINEAR, gravity=9.8, extrapolation_layers=10,
                              solver=el.SOLVER_JACOBI_FP64, tol=tol, max_iter=20000, check_every=16)
    return el.step_params(trace_phi=el.TRACE_RK2, sample_phi=el.SAMPLE_TRILINEAR, trace_vel=el.TRACE_RK2,
                          sample_vel=el.SAMPLE_TRILINEAR, gravity=9.8, extrapolation_layers=10,
                          solver=el.SOLVER_JACOBI_FP64, tol=tol, max_iter=20000, check_every=16)


def dam_workload_name(n, weno, tol, seed):
    if weno:
        return (f"dam break {n}^3 FP64 (box x<0.4,y<0.5 + sphere c=(0.7,0.75,0.5) r=0.12, room walls), seeded "
                f"velocity U(-1e-3,1e-3) (seed {seed}), phi WENO6/RK2, velocity trilinear/RK3, g 9.8, CFL 1.0, "
                f"plain FP64 PCG to {tol}")
    return (f"dam break {n}^3 FP64 (box x<0.4,y<0.5 + sphere c=(0.7,0.75,0.5) r=0.12, room walls), u=0, "
            f"trilinear RK2, g 9.8, CFL 1.0, plain FP64 PCG to {tol}")


def run_dam(args, dist):
    import numpy as np
    import torch

    el = load_package()
    el.load()
    torch.cuda.set_device(dist.local_rank)
    n, weno = dam_setup(args)
    K, W = args.steps, max(3, args.warmup)
    params = dam_params(el, weno, args.tol)
    spec, fields = dam_state(el, n, weno, args.seed)
    sim = el.Simulator(n, n, n, dtype=el.EL_F64, device=torch.cuda.current_device())
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    sim.init_scene(spec)
    for f, a in fields.items():
        sim.upload(f, a)
    # parity of the advected fields against the FP64 oracle, on the state after the warm-up steps
    for _ in range(W):
        sim.step(next_dt(sim), params)
    parity = advect_parity(el, sim, weno)
    sampler = ClockSampler(dist.local_rank) if dist.rank == 0 else None
    elapsed, stats, launches, _, clocks = timed_steps(el, torch, sim, stream, params, K, dist, sampler=sampler)
    elapsed = dist.max(elapsed)
    value, ms_per_step = aggregate([elapsed], K, dist.world)
    e2e = None
    if not args.no_e2e:
        ev, h2d, d2h = e2e_steps(el, torch, sim, stream, params, max(3, min(K, 20)), dtype=torch.float64)
        e2e = {"value": dist.world / dist.max(1.0 / ev), "unit": "steps/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h}
    sim.close()
    out = {
        "metric": DAM_METRIC, "value": value, "unit": "steps/s", "n_gpus": dist.world, "steps": K, "warmup": W,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": dam_workload_name(n, weno, args.tol, args.seed), "n": n, "seed": args.seed,
                   "parallelism": f"replicas x{dist.world}", "l2": "no flush: fields re-read every step"},
        "pcg": {"iterations_mean": statistics.mean(s["iterations"] for s in stats),
                "relres_max": max(s["relres"] for s in stats), "all_converged": all(s["status"] == 0 for s in stats)},
        "advected_parity_vs_fp64_oracle": parity, "gpu_launches": launches, "clocks": clocks, "e2e": e2e,
        "roofline": None,
    }
    if dist.rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_dam(args, steps=3 if n == 128 else 10)
    return out


def advect_parity(el, sim, weno):
    """Max relative error of the GPU's advected phi, u, v, w against the FP64 oracle's, from the
    scene's current state and the next CFL time step."""
    import numpy as np
    sys.path.insert(0, ROOT)
    import oracle as O

    st = {f: sim.download(f) for f in ("phi", "u", "v", "w")}
    dt = next_dt(sim)
    tp, sp = (O.TRACE_RK2, O.SAMPLE_WENO6) if weno else (O.TRACE_RK2, O.SAMPLE_TRILINEAR)
    tv = O.TRACE_RK3 if weno else O.TRACE_RK2
    ref_phi = O.advect_collocated(st["phi"], st["u"], st["v"], st["w"], sim.dx, dt, tp, sp)
    ref_u, ref_v, ref_w = O.advect_staggered(st["u"], st["v"], st["w"], sim.dx, dt, tv, O.SAMPLE_TRILINEAR)
    sim.advect_level_set(dt, tp, sp)
    sim.advect_velocity(dt, tv, el.SAMPLE_TRILINEAR)
    out = {}
    for f, ref in (("phi", ref_phi), ("u", ref_u), ("v", ref_v), ("w", ref_w)):
        got = sim.download(f)
        den = max(float(np.max(np.abs(ref))), 1e-300)
        out[f] = float(np.max(np.abs(got - ref))) / den
    for f, a in st.items():  # put the state back
        sim.upload(f, a)
    return out


def cpu_baseline_dam(args, steps):
    import numpy as np
    sys.path.insert(0, ROOT)
    import oracle as O
    from oracle import step as S

    el_scenes = _scenes_module()
    n, weno = dam_setup(args)
    spec = el_scenes.dam_break(n)
    phi, solid = O.rasterise(spec, np.float64)
    wts = O.compute_weights(solid)
    st = S.initial_state(phi, wts, O.cell_solid_phi(solid), O.float_dx(n, np.float64))
    if weno:
        rng = np.random.default_rng(args.seed)
        for f in ("u", "v", "w"):
            st[f] = rng.uniform(-1e-3, 1e-3, st[f].shape)
    tp, sp, tv = (0, 1, 1) if weno else (0, 0, 0)
    t0 = time.perf_counter()
    its = []
    for _ in range(steps):
        dt = min(O.calc_time_step(st["u"], st["v"], st["w"], st["dx"], 1.0), 1.0 / 60.0)
        st, _ = S.step(st, dt, tp, sp, tv, 0, 9.8, tol=args.tol, maxit=20000)
        its.append(st["pcg_iterations"])
    elapsed = time.perf_counter() - t0
    return {"value": steps / elapsed, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"{steps} full steps of the {n}^3 FP64 dam break from the initial state on the CPU oracle "
                      f"(OpenMP, MIC(0)-PCG FP64 to {args.tol}; iterations {its}), {elapsed:.1f} s"}


# ---- learned warm start ------------------------------------------------------------------------

WS_METRIC = "pressure-solve speed-up from the learned warm start at 128^3 (zero-guess time / learned time, to 1e-6)"


def conv_flops(n):
    """FLOPs of one forward pass of the network's 3x3x3 convolutions on an n^3 grid."""
    el = load_package()
    f = 0
    for name, _, _, _, cin, cout, level in el.warmstart.CONVS:
        f += 2 * 27 * cin * cout * (n >> level) ** 3
    return f


def run_warmstart(args, dist):
    import numpy as np
    import torch

    el = load_package()
    el.load()
    torch.cuda.set_device(dist.local_rank)
    W = el.warmstart
    n = args.ws_n
    params = step_params(el, el.SOLVER_MIXED, args.tol)
    # memory: 4 + 4 bf16 channels, FP32 target, mask per cell and tuple
    per = n ** 3 * (8 + 8 + 4 + 1)
    free, _ = torch.cuda.mem_get_info()
    samples = int(min(args.ws_samples, 0.6 * free // per))
    spp = args.ws_steps_per_scene
    specs = [el.scenes.spheres_pool(n, 1000 + s) for s in range((samples + spp - 1) // spp)]
    t0 = time.perf_counter()
    ds = W.record(el, torch, specs, spp, (n, n, n), params, capacity=samples)
    record_s = time.perf_counter() - t0
    net = W.WarmStartNet(torch, seed=args.seed, lr=1e-3)
    # training: one timed step first (CUDA events around forward + backward + Adam of one batch)
    x = net.input_buffer(n, n, n)
    x.zero_()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    stream = torch.cuda.current_stream()
    for warm in range(2):
        x[..., :4].copy_(ds.x[0])
        net.forward(n, n, n)
        net.backward(n, n, n, ds.t[0], ds.f[0], 1.0 / ds.energy[0], couplings=ds.c[0])
    net.grads.zero_()
    net.take_loss(n, n, n)
    torch.cuda.synchronize()
    reps = 5
    ev[0].record(stream)
    for _ in range(reps):
        net.forward(n, n, n)
    ev[1].record(stream)
    for _ in range(reps):
        net.backward(n, n, n, ds.t[0], ds.f[0], 1.0 / ds.energy[0], couplings=ds.c[0])
    ev[2].record(stream)
    torch.cuda.synchronize()
    fwd_ms = ev[0].elapsed_time(ev[1]) / reps
    bwd_ms = ev[1].elapsed_time(ev[2]) / reps
    net.grads.zero_()
    net.take_loss(n, n, n)
    F = conv_flops(n)
    first = 2 * 27 * 16 * 16 * n ** 3  # the first layer has no backward-data pass
    t0 = time.perf_counter()
    tr = W.train(net, ds, epochs=args.ws_epochs, batch=args.ws_batch, log=max(1, len(ds) // args.ws_batch // 10))
    train_s = time.perf_counter() - t0
    # evaluation on held-out scenes: every step's projection solved from zero and from the guess
    res = {s: {"zero_it": [], "warm_it": [], "zero_ms": [], "warm_ms": [], "infer_ms": []}
           for s in ("mixed", "plain_fp64")}
    solvers = {"mixed": el.SOLVER_MIXED, "plain_fp64": el.SOLVER_JACOBI_FP64}
    fields = ("phi", "u", "v", "w", "valid_u", "valid_v", "valid_w")
    for seed in range(args.ws_eval_scenes):
        sim = el.Simulator(n, n, n, dtype=el.EL_F32)
        sim.set_stream(stream.cuda_stream)
        sim.init_scene(el.scenes.spheres_pool(n, 90000 + seed))
        for k in range(4):
            dt = min(sim.calc_time_step(1.0), 1 / 60)
            saved = {f: sim.download(f) for f in fields}
            for key, solver in solvers.items():
                for guess in (0, 1):
                    for f, a in saved.items():
                        sim.upload(f, a)
                    sim.extrapolate_velocity(10)
                    sim.extrapolate_level_set(10)
                    sim.advect_level_set(dt, el.TRACE_RK2, el.SAMPLE_WENO6)
                    sim.advect_velocity(dt, el.TRACE_RK3, el.SAMPLE_TRILINEAR)
                    sim.add_gravity(dt, 9.8)
                    sim.find_valid_velocity()
                    sim.set_invalid_velocity_zero()
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    if guess:
                        W.predict_guess(net, sim, dt)
                        torch.cuda.synchronize()
                        res[key]["infer_ms"].append((time.perf_counter() - t0) * 1e3)
                    st = sim.solve_pressure(dt, solver=solver, tol=args.tol, max_iter=20000,
                                            check_every=4 if key == "mixed" else 16, initial_guess=guess)
                    torch.cuda.synchronize()
                    ms = (time.perf_counter() - t0) * 1e3
                    res[key]["warm_it" if guess else "zero_it"].append(st["iterations"])
                    res[key]["warm_ms" if guess else "zero_ms"].append(ms)
            # advance the scene with the last (warm, plain) step
        sim.close()
    summary = {}
    for key, r in res.items():
        summary[key] = {"iterations_zero_guess": statistics.mean(r["zero_it"]),
                        "iterations_learned_guess": statistics.mean(r["warm_it"]),
                        "ms_zero_guess": statistics.mean(r["zero_ms"]),
                        "ms_learned_guess_incl_inference": statistics.mean(r["warm_ms"]),
                        "ms_inference": statistics.mean(r["infer_ms"]),
                        "speedup": statistics.mean(r["zero_ms"]) / statistics.mean(r["warm_ms"])}
    hbm, _ = peaks()
    tflops_peak, peak_kind = bf16_peak()
    achieved = F / (fwd_ms / 1e3) / 1e12
    out = {
        "metric": WS_METRIC, "value": summary["mixed"]["speedup"], "unit": "x", "n_gpus": dist.world,
        "steps": len(res["mixed"]["zero_it"]), "warmup": 0, "ms_per_step": summary["mixed"]["ms_learned_guess_incl_inference"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "bf16 network (FP32 accumulation); f32 fields, pressure f32 inner / f64 refinement",
        "data": "synthetic: recorded from seeded spheres_pool scenes",
        "config": {"workload": f"learned warm start at {n}^3: {len(ds)} solves recorded from {len(specs)} "
                               f"spheres_pool scenes (seeds 1000+, {spp} steps each), 4-level encoder-decoder "
                               f"16/32/64/64 trained {args.ws_epochs} epochs (batch {args.ws_batch}, Adam, energy-norm "
                               f"loss); evaluated on {args.ws_eval_scenes} held-out scenes x 4 steps, solves to "
                               f"{args.tol}", "n": n, "samples": len(ds), "parallelism": "single GPU"},
        "warmstart": {"solvers": summary, "record_s": record_s, "train_s": train_s, "train_steps": tr["steps"],
                      "loss_history": tr["history"][-5:], "fwd_ms": fwd_ms, "bwd_ms": bwd_ms},
        "roofline": {"kernel": "network forward (the 3x3x3 convolutions: tcgen05 on the small-cin layers, mma.sync on the rest)", "bound": "tensor",
                     "achieved": achieved, "peak": tflops_peak, "unit": "TFLOP/s", "frac": achieved / tflops_peak,
                     "peak_kind": peak_kind, "traffic": None, "flops_per_launch": F,
                     "backward_tflops": (2 * F - first) / (bwd_ms / 1e3) / 1e12},
        "gpu_launches": None,
    }
    return out


def bf16_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        for k in ("bf16_tflops", "bf16_dense_tflops"):
            if k in d:
                return float(d[k]), "measured"
    return 1900.0, "fallback"


# ---- the reference's CPU path (the oracle port) ------------------------------------------

# How the CPU arm's sample differs from the GPU arm's timed region.
REFERENCE_ARM_DIFFERENCES = (
    "code: the oracle's C++ restatement of the reference's loops (bit-identical to the reference's own "
    "sources compiled here, which cannot be built on the Arm GPU host), not the reference binary; "
    "start: the initial scene at rest (the GPU arm times steps after warm-up steps); "
    "steps: 1-2 (the GPU arm: 20); "
    "solver: MIC(0)-PCG in FP64 to the same relative residual as the GPU arm, not the reference's own "
    "1e-4 (Eigen IncompleteCholesky CG, simulator.cpp:102-107)")


def cpu_baseline(n, seed, tol, steps):
    import numpy as np

    sys.path.insert(0, ROOT)
    import oracle as O
    from oracle import step as S

    spec = _scenes_module().spheres_pool(n, seed)
    phi, solid = O.rasterise(spec, np.float32)
    wts = O.compute_weights(solid)
    st = S.initial_state(phi, wts, O.cell_solid_phi(solid), O.float_dx(n, np.float32))
    cores = os.cpu_count()
    t0 = time.perf_counter()
    its = []
    for _ in range(steps):
        dt = min(O.calc_time_step(st["u"], st["v"], st["w"], st["dx"], 1.0), 1.0 / 60.0)
        st, _ = S.step(st, dt, 0, 1, 1, 0, 9.8, tol=tol, maxit=20000)
        its.append(st["pcg_iterations"])
    elapsed = time.perf_counter() - t0
    return {"value": steps / elapsed, "unit": "steps/s", "cores": cores, "kind": "port",
            "sample": f"{steps} full step(s) of the {n}^3 workload from the initial scene at rest on the CPU "
                      f"oracle (a restatement of the reference's loops, OpenMP, FP32 fields, MIC(0)-PCG FP64 "
                      f"to {tol}, not the reference's 1e-4; {its} iterations), {elapsed:.1f} s"}


def _scenes_module():
    spec = importlib.util.spec_from_file_location("el_scenes", os.path.join(ROOT, "eulerian-liquid_gb300", "scenes.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def run_reference_batch(args, dist):
    scenes = _scenes_module()
    specs = scenes.batch_scenes(args.scenes, args.seed)
    # a bounded sample: one step of each of the first scenes until about 10 s of CPU work
    t0 = time.perf_counter()
    cells = 0
    samples = []
    for q in range(len(specs)):
        b = cpu_baseline_batch(specs, args.tol, q)
        cells += specs[q]["shape"][0] * specs[q]["shape"][1] * specs[q]["shape"][2]
        samples.append(q)
        if time.perf_counter() - t0 > 10.0:
            break
    elapsed = time.perf_counter() - t0
    value = cells / elapsed
    return {"metric": BATCH_METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": dist.world, "steps": 1,
            "warmup": 0, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 fields; pressure f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": batch_workload_name(args) + " (same as our arm)", "scenes": args.scenes,
                       "seed": args.seed, "parallelism": "host cores"},
            "cpu_baseline": {"kind": "port", "cores": b["cores"], "value": value, "unit": "cell-updates/s",
                             "sample": f"1 step each of scenes {samples} on the CPU oracle (OpenMP), "
                                       f"{cells} cell-updates in {elapsed:.1f} s"},
            "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_reference_warmstart(args, dist):
    """The reference solves from zero only (Eigen's solve(), simulator.cpp:102-109): its speed-up
    from a learned guess is 1 by definition; the line carries the CPU path's solve rate on the same
    128^3 scenes (one step of a held-out spheres_pool scene, MIC(0)-PCG to the same tolerance)."""
    import numpy as np
    sys.path.insert(0, ROOT)
    import oracle as O
    from oracle import step as S

    n = args.ws_n
    spec = _scenes_module().spheres_pool(n, 90000)
    phi, solid = O.rasterise(spec, np.float32)
    wts = O.compute_weights(solid)
    st = S.initial_state(phi, wts, O.cell_solid_phi(solid), O.float_dx(n, np.float32))
    dt = min(O.calc_time_step(st["u"], st["v"], st["w"], st["dx"], 1.0), 1.0 / 60.0)
    t0 = time.perf_counter()
    st, _ = S.step(st, dt, 0, 1, 1, 0, 9.8, tol=args.tol, maxit=20000)
    elapsed = time.perf_counter() - t0
    rate = 1.0 / elapsed
    return {"metric": WS_METRIC, "value": 1.0, "unit": "x", "n_gpus": dist.world, "steps": 1, "warmup": 0,
            "ms_per_step": elapsed * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 fields; pressure f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": f"learned warm start at {n}^3 (the reference solves from zero: speed-up 1)",
                       "n": n, "parallelism": "host cores"},
            "cpu_baseline": {"kind": "port", "cores": os.cpu_count(), "value": rate, "unit": "steps/s",
                             "sample": f"one full {n}^3 step (held-out spheres_pool scene) on the CPU oracle, "
                                       f"MIC(0)-PCG from zero to {args.tol} ({st['pcg_iterations']} iterations), "
                                       f"{elapsed:.1f} s"},
            "e2e": {"value": 1.0, "unit": "x", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def run_reference(args, dist):
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count()))
    os.environ.setdefault("OMP_PROC_BIND", "close")
    if args.workload == "batch32":
        return run_reference_batch(args, dist)
    if args.workload == "warmstart128":
        return run_reference_warmstart(args, dist)
    if args.workload in ("dam64", "dam128"):
        n, weno = dam_setup(args)
        base = cpu_baseline_dam(args, steps=max(1, min(args.steps, 3 if n == 128 else 10)))
        return {"metric": DAM_METRIC, "value": base["value"], "unit": "steps/s", "n_gpus": dist.world,
                "steps": None, "warmup": 0, "ms_per_step": 1e3 / base["value"], "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
                "config": {"workload": dam_workload_name(n, weno, args.tol, args.seed) + " (same as our arm)",
                           "n": n, "seed": args.seed, "parallelism": "host cores"},
                "cpu_baseline": {"kind": base["kind"], "cores": base["cores"], "sample": base["sample"],
                                 "value": base["value"], "unit": "steps/s"},
                "e2e": {"value": base["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    steps = max(1, min(args.steps, 2))
    base = cpu_baseline(args.n, args.seed, args.tol, steps)
    return {"metric": METRIC, "value": base["value"], "unit": "steps/s", "n_gpus": dist.world, "steps": steps,
            "warmup": 0, "ms_per_step": 1e3 / base["value"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 fields; pressure f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": headline_workload_name(args.n, args.seed, args.tol),
                       "n": args.n, "seed": args.seed, "parallelism": "host cores",
                       "differences_from_our_arm": REFERENCE_ARM_DIFFERENCES},
            "cpu_baseline": {"kind": base["kind"], "cores": base["cores"], "sample": base["sample"],
                             "value": base["value"], "unit": "steps/s"},
            "e2e": {"value": base["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main(argv=None):
    args = parse_args(argv)
    dist = Dist()
    try:
        if args.impl == "reference":
            if dist.rank == 0:
                print(json.dumps(run_reference(args, dist)), flush=True)
            return 0
        if args.workload == "batch32":
            out = run_batch(args, dist)
        elif args.workload == "warmstart128":
            out = run_warmstart(args, dist)
        elif args.workload in ("dam64", "dam128"):
            out = run_dam(args, dist)
        else:
            out = run_ours(args, dist)
        if dist.rank == 0:
            print(json.dumps(out), flush=True)
        return 0
    finally:
        dist.close()


if __name__ == "__main__":
    sys.exit(main())
