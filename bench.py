#!/usr/bin/env python
"""Benchmark of the GB300 FDFD solve path; prints ONE JSON line.

Workload (one "step"): the 800 x 480 TM design-guide problem — input and
output guide arms (ϵᵣ = 12.25, 10 cells wide) around a 200 x 200 design
region of seeded i.i.d. ϵᵣ ~ U[1, 12.25], Gaussian line source (waist 8
cells) across the input guide, λ = 1.55 µm, dl = λ/20, 20 PML cells per side
(m = 4, R = 1e-8).  A step assembles the operator from the resident ϵᵣ,
factors it (complex FP32 block cyclic reduction with 3xTF32 tcgen05 GEMMs),
solves to ||b - A x||/||b|| <= 1e-10 with FP64 FGMRES refinement and
recovers Hx, Hy.  value = solves/s with inputs resident in HBM; e2e = the
same through the host-buffer C ABI (ϵᵣ and source copied in, three fields
copied out, every step).

--impl reference times the CPU restatement of the reference path (scipy
SuperLU FP64 on the same problem) on the host cores, one process per core.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "TM solves/s at 1e-10 residual: mixed-prec vs FP64 on one GB300; adjoint grads/s"
WORKLOAD = ("design_guide 800x480 TM: guide arms + 200x200 random design (seed 2), Gaussian line source "
            "(waist 8), lambda 1.55um, dl lambda/20, 20-cell PML m=4 R=1e-8, tol 1e-10")


def args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the adjoint / eigenfrequency / frequency-sweep measurements")
    ap.add_argument("--seed", type=int, default=2, help="seed of the random design region (2: the benchmark's)")
    ap.add_argument("--autotune", type=int, default=1, choices=[0, 1],
                    help="1: run the launch-shape autotuner on the timed handles first (outside the timed region)")
    ap.add_argument("--size", default=None,
                    help="NXxNY: same problem family at another size (profiling runs); design region = "
                         "a quarter of the smaller side squared")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def max_over_ranks(t: float, world: int, device: str = "cuda") -> float:
    """The slowest rank's time: the job of N independent replicas ends with its last one.
    `device` is where the process group's backend reduces ("cuda" for NCCL, "cpu" for gloo)."""
    if world <= 1:
        return t
    import torch
    import torch.distributed as dist
    tt = torch.tensor([t], device=device, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def job_rate(world: int, steps: int, t: float) -> float:
    """Whole-job throughput: every rank ran `steps` steps of its own replica in at most t seconds."""
    return world * steps / t


# ---------------------------------------------------------------------------
# clocks sampler (nvidia-smi during the timed region)
# ---------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu, self.lines, self.proc = gpu, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.gpu), "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU reference path (scipy SuperLU restatement of the reference solve)
# ---------------------------------------------------------------------------
def _cpu_solve(kind, seed=2, want_fields=False):
    """One oracle solve (assembly + SuperLU factor + solve + H recovery) of the workload
    ("full") or of a small warm-up problem; returns (seconds, relative residual[, fields])."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import __graft_entry__ as G
    G.load_package()
    import fdfd_oracle as O
    from fdfd_gb300 import workloads as W
    p = W.design_guide(seed=seed) if kind == "full" else W.point_source_guide(120, 80)
    g = O.Grid((p.Nx, p.Ny), p.npml, ((0.0, 0.0), (p.Nx * p.dx, p.Ny * p.dy)))
    t0 = time.perf_counter()
    f, A, b = O.solve(g, p.eps, p.src, p.omega, O.TM, p.pml_m, p.pml_lnR, return_system=True)
    t = time.perf_counter() - t0
    res = float(O.relative_residual(A, O.vec(f[0]), b))
    return (t, res, f) if want_fields else (t, res)


_BLAS_THREAD_VARS = ("OPENBLAS_NUM_THREADS", "OMP_NUM_THREADS", "MKL_NUM_THREADS")


class _single_threaded_children:
    """Spawned worker processes inherit one BLAS thread each (scipy's BLAS is multithreaded by
    default: concurrent workers would oversubscribe the host, and a single 'one core' solve
    would not be one core)."""

    def __enter__(self):
        self.saved = {k: os.environ.get(k) for k in _BLAS_THREAD_VARS}
        for k in _BLAS_THREAD_VARS:
            os.environ[k] = "1"

    def __exit__(self, *exc):
        for k, v in self.saved.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def host_threads():
    """What the host offers this process and what the BLAS would use, reported with every CPU number."""
    try:
        usable = len(os.sched_getaffinity(0))
    except Exception:
        usable = os.cpu_count() or 1
    return {"nproc": os.cpu_count(), "usable_cores": usable,
            "OMP_NUM_THREADS": os.environ.get("OMP_NUM_THREADS"),
            "OPENBLAS_NUM_THREADS": os.environ.get("OPENBLAS_NUM_THREADS")}


def mem_available_bytes():
    try:
        with open("/proc/meminfo") as f:
            for line in f:
                if line.startswith("MemAvailable:"):
                    return int(line.split()[1]) * 1024
    except Exception:
        pass
    return None


def cpu_baseline_single(seed=2):
    """One full solve on one host thread, in a spawned process whose BLAS runs one thread
    (SuperLU itself factors sequentially).  Returns (cpu_baseline block, oracle fields)."""
    import concurrent.futures as cf
    import multiprocessing as mp
    env = host_threads()
    with _single_threaded_children():
        with cf.ProcessPoolExecutor(max_workers=1, mp_context=mp.get_context("spawn")) as ex:
            t, res, f = ex.submit(_cpu_solve, "full", seed, True).result()
    return {"value": 1.0 / t, "unit": "solves/s", "cores": 1, "kind": "port", **env,
            "worker_blas_threads": 1,
            "sample": f"1 full solve of the workload with the scipy/SuperLU FP64 oracle, one thread "
                      f"({t:.1f} s, rel. residual {res:.1e})"}, f


# host memory one concurrent SuperLU solve of the workload may take at its peak (measured ~2.5 GB)
_SOLVE_BYTES = 4 << 30


def run_reference(a):
    """Whole-host throughput of the CPU reference path: one worker process per usable host core
    (one BLAS thread each; SuperLU factors sequentially), bounded by host memory.  A full solve
    takes tens of seconds, so the K steps share one pipelined batch of waves x workers solves
    (about three waves, the jobs spread evenly over the steps): every core stays busy and the
    whole run stays within a few minutes whatever K is.  value = solves completed / wall time."""
    import concurrent.futures as cf
    import multiprocessing as mp
    env = host_threads()
    mem = mem_available_bytes()
    workers = env["usable_cores"]
    mem_cap = None
    if mem:
        mem_cap = max(1, int(0.8 * mem // _SOLVE_BYTES))
        workers = min(workers, mem_cap)
    waves = 3
    total = workers * waves
    ctx = mp.get_context("spawn")
    with _single_threaded_children(), cf.ProcessPoolExecutor(max_workers=workers, mp_context=ctx) as ex:
        for _ in range(max(1, a.warmup)):   # warm the workers: small solve each
            list(ex.map(_cpu_solve, ["small"] * workers))
        t0 = time.perf_counter()
        futs = [ex.submit(_cpu_solve, "full", a.seed) for _ in range(total)]
        res = [f.result() for f in futs]
        wall = time.perf_counter() - t0
    value = total / wall
    per_solve = sorted(r[0] for r in res)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * wall / a.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": WORKLOAD.replace("(seed 2)", f"(seed {a.seed})"),
                       "solver": "scipy SuperLU FP64 (restatement of lu(A)\\b)",
                       "step": f"{total} full solves on {workers} worker processes (one per usable host core"
                               f"{', memory-capped' if mem_cap is not None and mem_cap < env['usable_cores'] else ''}"
                               f"), {waves} waves, grouped into the {a.steps} steps"},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": workers, "kind": "port", **env,
                             "worker_blas_threads": 1, "mem_available_gb": round(mem / 2**30, 1) if mem else None,
                             "sample": f"{total} concurrent full solves ({waves} per worker); one solve took "
                                       f"{per_solve[0]:.1f}-{per_solve[-1]:.1f} s (median "
                                       f"{per_solve[len(per_solve) // 2]:.1f} s), max rel. residual "
                                       f"{max(r[1] for r in res):.1e}"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU path
# ---------------------------------------------------------------------------
def tf32_cublas_tflops(torch):
    """cuBLAS TF32 GEMM throughput (context only; the roofline peak comes from MEASURED_PEAKS.json)."""
    try:
        torch.backends.cuda.matmul.allow_tf32 = True
        n = 8192
        x = torch.randn(n, n, device="cuda", dtype=torch.float32)
        y = torch.randn(n, n, device="cuda", dtype=torch.float32)
        for _ in range(2):
            x @ y
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            x @ y
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / 5
        del x, y
        return 2 * n ** 3 / t / 1e12
    except Exception:
        return None


def run_extras(L, pkg, W, a):
    """The other benchmark problems, each timed with host-buffer calls after one warm-up:
    adjoint gradients/s on the 1000x600 adjoint problem (300x300 design, Gaussian overlap
    objective), eigenfrequency time on the 12x12 rod-lattice cavity (280x280, 6 modes nearest
    ωa/2πc = 0.38), the 400x400 frequency sweep (all 64 wavelengths x 8 Gaussian sources, batched
    factorizations in CUDA graphs), coupled-sideband solves/s of the reference notebook's
    modulated waveguide (1500x200, three frequencies) and problems/s of the 32-problem mixed-size
    batch."""
    out = {}
    try:
        p = W.adjoint_problem()
        h = L.Handle(p.Nx, p.Ny, p.npml[0], p.npml[1], p.dx, p.dy, 1e-6, p.pml_m, p.pml_lnR, pkg.TM,
                     L.FDFD_PREC_MIXED)
        h.set_refinement(1e-10, 80)
        h.set_eps(p.eps)
        h.factor(p.omega)
        h.adjoint(p.src, p.extra["mvec"])
        t0 = time.perf_counter()
        n = 5
        for _ in range(n):
            h.set_eps(p.eps)
            h.factor(p.omega)
            _, _, _, st = h.adjoint(p.src, p.extra["mvec"])
        t = time.perf_counter() - t0
        h.close()
        out["adjoint_grads_per_s"] = {"value": n / t, "workload": "adjoint 1000x600, 300x300 design, mixed",
                                      "rel_residual": st.rel_residual, "iterations": st.iterations}
    except Exception as e:   # reported, not hidden
        out["adjoint_grads_per_s"] = {"error": str(e)}
    try:
        p, w0 = W.phc_cavity()
        h = L.Handle(p.Nx, p.Ny, p.npml[0], p.npml[1], p.dx, p.dy, 1e-6, p.pml_m, p.pml_lnR, pkg.TM,
                     L.FDFD_PREC_MIXED)
        h.set_refinement(1e-10, 80)
        h.set_eps(p.eps)
        h.eigfreq(w0, 6)
        t0 = time.perf_counter()
        om, lam, _, st = h.eigfreq(w0, 6)
        t = time.perf_counter() - t0
        h.close()
        out["eigfreq"] = {"seconds": t, "workload": "phc cavity 280x280, 6 modes, mixed",
                          "omega_a_over_2pi_c": [float(x.real * 1e-6 / (2 * math.pi * W.C0)) for x in om],
                          "operator_solves": st.iterations, "ritz_residual": st.rel_residual}
    except Exception as e:
        out["eigfreq"] = {"error": str(e)}
    try:
        out["sweep"] = run_sweep(L, pkg, W)
    except Exception as e:   # reported, not hidden
        out["sweep"] = {"error": str(e)}
    try:
        p = W.modulated_notebook()
        e = p.extra
        h = L.ModulatedHandle(p.Nx, p.Ny, p.npml[0], p.npml[1], p.dx, p.dy, e["nsidebands"], 1e-6, p.pml_m,
                              p.pml_lnR, e["sharedpml"], L.FDFD_PREC_MIXED)
        h.set_refinement(1e-10, 80)
        h.set_eps(p.eps)
        h.set_deps(e["deps"])
        h.factor(p.omega, e["Omega"])
        h.solve(p.src)
        t0 = time.perf_counter()
        n = 3
        for _ in range(n):
            h.set_eps(p.eps)
            h.factor(p.omega, e["Omega"])
            _, _, _, st = h.solve(p.src)
        t = time.perf_counter() - t0
        h.close()
        out["modulated"] = {"solves_per_s": n / t, "workload": "modulated waveguide 1500x200, 1 sideband each side "
                            "(3 coupled frequencies), host buffers, mixed", "rel_residual": st.rel_residual,
                            "iterations": st.iterations, "t_factor_ms": st.t_factor_ms, "t_solve_ms": st.t_solve_ms}
    except Exception as e:   # reported, not hidden
        out["modulated"] = {"error": str(e)}
    try:
        out["checkpoint"] = run_checkpoint(L, pkg, W)
    except Exception as e:   # reported, not hidden
        out["checkpoint"] = {"error": str(e)}
    try:
        out["mode_sources"] = run_mode_sources(L, pkg, W)
    except Exception as e:   # reported, not hidden
        out["mode_sources"] = {"error": str(e)}
    try:
        out["mixed_batch"] = run_mixed_batch(L, pkg, W)
    except Exception as e:
        out["mixed_batch"] = {"error": str(e)}
    return out


def run_checkpoint(L, pkg, W):
    """The benchmark workload (800x480) with its block factors checkpointed to pinned host memory
    (fdfd_set_checkpoint(1)) next to the resident layout: solves/s, device bytes, host bytes and
    the bytes moved over the host link per solve.  Three timed solves each after one warm-up."""
    import numpy as np
    p = W.design_guide()
    out = {}
    for mode, name in ((-1, "resident"), (1, "checkpointed")):
        h = L.Handle(p.Nx, p.Ny, p.npml[0], p.npml[1], p.dx, p.dy, 1e-6, p.pml_m, p.pml_lnR, pkg.TM,
                     L.FDFD_PREC_MIXED)
        h.set_refinement(1e-10, 80)
        h.set_checkpoint(mode)
        h.set_eps(p.eps)
        h.factor(p.omega)
        f = h.solve(p.src)
        c0 = h.checkpoint_info()["copied_bytes"]
        n = 3
        t0 = time.perf_counter()
        for _ in range(n):
            h.factor(p.omega)
            f = h.solve(p.src)
        t = time.perf_counter() - t0
        info = h.checkpoint_info()
        out[name] = {"solves_per_s": n / t, "device_bytes": f[3].device_bytes, "host_bytes": info["host_bytes"],
                     "host_link_bytes_per_solve": (info["copied_bytes"] - c0) / n,
                     "rel_residual": f[3].rel_residual, "ez": f[0]}
        h.close()
    out["field_diff"] = float(np.linalg.norm(out["checkpointed"].pop("ez") - out["resident"]["ez"]) /
                              np.linalg.norm(out["resident"].pop("ez")))
    out["workload"] = "design_guide 800x480, mixed, block factors resident vs checkpointed to pinned host memory"
    return out


def run_mode_sources(L, pkg, W):
    """Mode sources for the 64 wavelengths of the sweep band (λ ∈ [1.45, 1.65] µm) on the reference's
    waveguide test grid (500x100 at dh = 0.02 µm, guide ϵᵣ = 12 of 0.3 µm): one TM mode (slice width
    0.8 µm, n_eff 3.5) per wavelength, all 64 mode problems and source arrays in one call; the same
    64 mode problems with the oracle (scipy ARPACK shift-invert) on one host core beside it."""
    import numpy as np
    Nx, Ny, dh = 500, 100, 0.02
    yc = -1.0 + dh * (np.arange(Ny) + 0.5)
    eps = np.ones((Nx, Ny), dtype=np.complex128)
    eps[:, np.abs(yc) <= 0.15] = 12.0
    lams = np.linspace(1.45, 1.65, 64)
    omegas = np.array([W.omega_of(l) for l in lams])
    mode = (L.FDFD_TM, L.FDFD_X, 50, Ny // 2, 0.8, 3.5)
    h = L.Handle(Nx, Ny, 15, 15, dh, dh, 1e-6, 3.5, -12.0, pkg.TM, L.FDFD_PREC_MIXED)
    h.set_eps(eps)
    h.mode_sources(omegas, [mode])
    n = 5
    t0 = time.perf_counter()
    for _ in range(n):
        h.mode_sources(omegas, [mode])
    t = (time.perf_counter() - t0) / n
    h.close()
    res = {"modes_per_s": len(omegas) / t, "ms_per_call": 1e3 * t, "modes_per_call": len(omegas),
           "workload": "64 TM modes (41-cell slices) of the 500x100 waveguide test grid, sources in and out of "
                       "host memory, one call"}
    try:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import fdfd_oracle as O
        g = O.Grid((Nx, Ny), (15, 15), ((0.0, -1.0), (Nx * dh, 1.0)))
        t0 = time.perf_counter()
        for w in omegas[:16]:
            O.get_modes(g, eps, 1, w, 3.5, 1, 50, Ny // 2, O.X, 0.8)
        tc = (time.perf_counter() - t0) / 16
        res["cpu_oracle_modes_per_s"] = 1.0 / tc
    except Exception as e:   # reported, not hidden
        res["cpu_oracle_modes_per_s"] = {"error": str(e)}
    return res


def tuning_summary(logs):
    """Autotuner choices across handles: per product role, how often each launch shape won."""
    out = {}
    for log in logs:
        for line in log.splitlines():
            f = line.split()
            if len(f) < 4 or "->" not in f:
                continue
            role = f"{f[0]} {f[1]}"
            choice = f[f.index("->") + 1]
            d = out.setdefault(role, {})
            d[choice] = d.get(choice, 0) + 1
    return out


def run_sweep(L, pkg, W, width=8):
    """The batched frequency sweep: 400x400 with a 160x160 seeded random design, all 64 wavelengths
    (uniform in [1.45, 1.65] um, seeded), each with its 8 Gaussian line sources.  `width` handles of
    the same problem (each autotuned) are factored together, one wavelength each, by one CUDA-graph
    launch (fdfd_batch_factor); their 8-source solves (host buffers, refined to 1e-10) then run
    concurrently, one host thread per handle.  64 wavelengths = 64/width launches.  Timed after one
    untimed pass (which captures the graph); handle creation and tuning are outside the timed region."""
    import concurrent.futures as cf
    import numpy as np
    p, lams = W.frequency_sweep()
    hs = []
    for _ in range(width):
        h = L.Handle(p.Nx, p.Ny, p.npml[0], p.npml[1], p.dx, p.dy, 1e-6, p.pml_m, p.pml_lnR, pkg.TM,
                     L.FDFD_PREC_MIXED)
        h.set_refinement(1e-10, 80)
        h.set_eps(p.eps)
        hs.append(h)
    logs = [h.autotune() for h in hs]
    batch = L.Batch(hs)
    omegas = np.array([W.omega_of(l) for l in lams])

    def one_pass():
        res = []
        with cf.ThreadPoolExecutor(max_workers=width) as ex:
            for w0 in range(0, len(omegas), width):
                batch.factor(omegas[w0:w0 + width])
                res += list(ex.map(lambda h: h.solve(p.src)[3], hs))
        return res

    one_pass()
    t0 = time.perf_counter()
    res = one_pass()
    t = time.perf_counter() - t0
    st = batch.stats()
    batch.close()
    for h in hs:
        h.close()
    nsrc = p.src.shape[0]
    return {"wavelengths_per_s": len(omegas) / t, "rhs_solves_per_s": len(omegas) * nsrc / t, "seconds": t,
            "wavelengths": len(omegas), "sources_per_wavelength": nsrc,
            "rel_residual_max": max(r.rel_residual for r in res), "iterations_max": max(r.iterations for r in res),
            "fp64_fallbacks": sum(r.fp64_fallback for r in res),
            "graph": {"handles_per_launch": width, "graph_launches_timed": len(omegas) // width,
                      "kernels_per_graph": st["graph_kernels"], "last_graph_ms": st["last_graph_ms"]},
            "tuned_shapes": tuning_summary(logs),
            "workload": f"frequency sweep 400x400, 64 of 64 wavelengths x {nsrc} sources, {width} frequencies per "
                        f"CUDA-graph launch, autotuned launch shapes, host buffers, mixed"}


def run_mixed_batch(L, pkg, W):
    """The 32-problem mixed-size batch (square sides drawn from 128, 256, 512, 1024 with a fixed
    seed; split guide with a centred random design of half the side).  One autotuned handle per side
    class; the batch runs in waves, each wave taking the next problem of every class that has one:
    the wave's permittivities are copied in, all its factorizations run as one CUDA-graph launch
    (fdfd_batch_factor over that wave's handles), then its solves run concurrently, one host thread
    per handle (host buffers, refined to 1e-10).  All 32 factor sets at once would not fit in HBM
    (nine 1024^2 problems hold ~32 GB each), hence the waves.  Timed after one untimed pass (which
    captures the graphs); handle creation and tuning are outside the timed region."""
    import concurrent.futures as cf
    probs = W.mixed_size_batch()
    classes = {}
    for p in probs:
        classes.setdefault(p.Nx, []).append(p)
    sides = sorted(classes)
    handles = {}
    for sd in sides:
        p = classes[sd][0]
        h = L.Handle(p.Nx, p.Ny, p.npml[0], p.npml[1], p.dx, p.dy, 1e-6, p.pml_m, p.pml_lnR, pkg.TM,
                     L.FDFD_PREC_MIXED)
        h.set_refinement(1e-10, 80)
        handles[sd] = h
    logs = [h.autotune() for h in handles.values()]
    nwaves = max(len(v) for v in classes.values())
    waves = [[sd for sd in sides if w < len(classes[sd])] for w in range(nwaves)]
    batches = {}
    for wv in waves:
        key = tuple(wv)
        if key not in batches:
            batches[key] = L.Batch([handles[sd] for sd in wv])

    def one_pass():
        res = []
        with cf.ThreadPoolExecutor(max_workers=len(sides)) as ex:
            for w, wv in enumerate(waves):
                ps = [classes[sd][w] for sd in wv]
                for sd, p in zip(wv, ps):
                    handles[sd].set_eps(p.eps)
                batches[tuple(wv)].factor([p.omega for p in ps])
                res += list(ex.map(lambda a: handles[a[0]].solve(a[1].src)[3], zip(wv, ps)))
        return res

    one_pass()
    t0 = time.perf_counter()
    res = one_pass()
    t = time.perf_counter() - t0
    kernels = sum(b.stats()["graph_kernels"] for b in batches.values())
    for b in batches.values():
        b.close()
    for h in handles.values():
        h.close()
    return {"problems_per_s": len(probs) / t, "seconds": t, "problems": len(probs),
            "sides": {int(sd): len(classes[sd]) for sd in sides},
            "rel_residual_max": max(r.rel_residual for r in res), "iterations_max": max(r.iterations for r in res),
            "iterations_sum": sum(r.iterations for r in res), "fp64_fallbacks": sum(r.fp64_fallback for r in res),
            "graph": {"waves": len(waves), "graph_launches_timed": len(waves), "distinct_graphs": len(batches),
                      "kernels_in_graphs": kernels},
            "tuned_shapes": tuning_summary(logs),
            "workload": "32 square problems, sides from {128, 256, 512, 1024} (seed 5), one autotuned handle per side "
                        "class, one CUDA-graph launch factoring each wave, concurrent solves, host buffers, mixed"}


def gemm_traffic_bytes():
    """DRAM bytes per launch of the tensor-core GEMM from the committed ncu summary
    (profiles/gemm_tc_traffic.json: read + write of one captured launch and the units it processed),
    or None when no capture exists."""
    try:
        with open(os.path.join(ROOT, "profiles", "gemm_tc_traffic.json")) as f:
            return json.load(f)
    except Exception:
        return None


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "MEASURED_PEAKS.json"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def main():
    a = args()
    rank, local, world = dist_env()
    if a.impl == "reference":
        if rank == 0:
            run_reference(a)
        return
    import numpy as np
    import torch
    import __graft_entry__ as G

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    pkg = G.load_package()
    from fdfd_gb300 import workloads as W
    L = pkg._lib
    workload = WORKLOAD.replace("(seed 2)", f"(seed {a.seed})")
    if a.size:
        nx, ny = (int(v) for v in a.size.lower().split("x"))
        dsz = min(nx, ny) // 4
        p = W.design_guide(nx, ny, design=(dsz, dsz), seed=a.seed)
        workload = f"design_guide {nx}x{ny} (profiling size), {dsz}x{dsz} design (seed {a.seed})"
    else:
        p = W.design_guide(seed=a.seed)
    N = p.Nx * p.Ny

    def make(prec):
        h = L.Handle(p.Nx, p.Ny, p.npml[0], p.npml[1], p.dx, p.dy, 1e-6, p.pml_m, p.pml_lnR, pkg.TM, prec)
        h.set_refinement(1e-10, 80)
        h.set_eps(p.eps)
        return h

    # device-resident source and fields (x fastest, interleaved complex128)
    src_nat = L.natural(p.src).reshape(-1)
    d_src = torch.from_numpy(src_nat).to("cuda")
    d_f = [torch.empty(N, dtype=torch.complex128, device="cuda") for _ in range(3)]

    def step_device(h):
        h.factor(p.omega)
        return h.solve_device(d_src.data_ptr(), 1, d_f[0].data_ptr(), d_f[1].data_ptr(), d_f[2].data_ptr())

    h = make(L.FDFD_PREC_MIXED)
    tuned = h.autotune() if a.autotune else None
    for _ in range(a.warmup):
        step_device(h)
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    stats = []
    for _ in range(a.steps):
        stats.append(step_device(h).as_dict())
    e1.record()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    t = max_over_ranks(e0.elapsed_time(e1) / 1e3, world)
    value = job_rate(world, a.steps, t)
    # per-class device times for the rooflines: separate steps with profiling on (the library then
    # brackets every launch with events and runs the Gauss-Jordan updates on one stream)
    prof_steps = min(a.steps, 3)
    h.set_profiling(True)
    for _ in range(prof_steps):
        step_device(h)
    prof = h.profile()
    h.set_profiling(False)
    maxres = max(s["rel_residual"] for s in stats)
    launches = sum(s["gpu_launches"] for s in stats)
    iters = [s["iterations"] for s in stats]

    # fields of the last mixed solve, for the check against the FP64 oracle below
    fields_mixed = [f.cpu().numpy() for f in d_f]

    # the plain FP64 form on the GPU: timing (after one warm-up) and its fields
    fp64 = None
    fields_fp64 = None
    if not a.no_fp64:
        hf = make(L.FDFD_PREC_FP64)
        step_device(hf)                      # warm-up
        torch.cuda.synchronize()
        n64 = 3
        t0 = time.perf_counter()
        for _ in range(n64):
            st64 = step_device(hf)
        torch.cuda.synchronize()
        t64 = (time.perf_counter() - t0) / n64
        fields_fp64 = [f.cpu().numpy() for f in d_f]
        hf.close()
        fp64 = {"solves_per_s": 1.0 / t64, "timed_solves": n64, "rel_residual": st64.rel_residual,
                "t_factor_ms": st64.t_factor_ms, "mixed_over_fp64": (value / world) * t64,
                "mixed_vs_fp64_field_err": float(np.linalg.norm(fields_mixed[0] - fields_fp64[0]) /
                                                 np.linalg.norm(fields_fp64[0]))}

    # end-to-end through the host-buffer C ABI: ϵᵣ and source in, three fields out, every step.  The
    # host arrays are laid out as a Julia caller passes them (column-major, x fastest) before the
    # timed region, so the loop times fdfd_set_eps + fdfd_factor + fdfd_solve and nothing else.
    e2e = None
    if not a.no_e2e:
        import ctypes
        he = make(L.FDFD_PREC_MIXED)
        if a.autotune:
            he.autotune()
        h2d = N * 16 * 2
        d2h = N * 16 * 3
        eps_c, src_c = L.natural(p.eps), L.natural(p.src)
        outs = [np.empty_like(src_c) for _ in range(3)]
        st = L.Stats()
        lib = he.lib

        def e2e_step():
            he._check(lib.fdfd_set_eps(he.h, L.cptr(eps_c)))
            he._check(lib.fdfd_factor(he.h, float(p.omega)))
            he._check(lib.fdfd_solve(he.h, L.cptr(src_c), 1, *[L.cptr(o) for o in outs], ctypes.byref(st)))

        for _ in range(max(1, a.warmup)):   # untimed, as the device-resident leg (graph capture happens here)
            e2e_step()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        t0 = time.perf_counter()
        for _ in range(a.steps):
            e2e_step()
        torch.cuda.synchronize()
        te = max_over_ranks(time.perf_counter() - t0, world)
        he.close()
        e2e = {"value": job_rate(world, a.steps, te), "unit": "solves/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h}

    # rooflines: the factorization's tensor-core GEMM (tensor-bound) and the solve sweeps (HBM-bound),
    # from the profiled steps; class_ms_per_solve shows every kernel class, dominant_class the largest
    peaks, peak_src = measured_peaks()
    gk = "gemm_tc" if prof["gemm_tc"]["launches"] else "gemm_simt"
    d = prof[gk]
    achieved = d["work"] / (d["ms"] / 1e3) / 1e12 if d["ms"] else None
    # 3xTF32: three TF32 MMAs per real product; TF32 tensor rate = half the BF16 rate
    peak = peaks["bf16_tflops"] / 2 / 3
    roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak if achieved else None, "kernel": gk,
            "traffic": (gemm_traffic_bytes() or {}).get("bytes"),
            "traffic_note": (gemm_traffic_bytes() or {}).get("note"),
            "peak_note": f"bf16 burst from {peak_src} /2 (TF32 rate) /3 (3xTF32 split), of measured",
            "work_unit": "8*M*N*K algorithmic complex-GEMM flops per launch",
            "launches_profiled": d["launches"], "avg_launch_ms": d["ms"] / max(d["launches"], 1),
            "profiled_steps": prof_steps,
            "class_ms_per_solve": {k: round(v["ms"] / prof_steps, 3) for k, v in prof.items()},
            "dominant_class": max(prof, key=lambda k: prof[k]["ms"])}
    # HBM-bound classes: achieved = algorithmic bytes / device time
    hbm_units = {"sweep": "dense factor blocks each product references (re, im planes) and the first step's "
                          "tridiagonal factors (8b complex + b pivots per node), read once per sweep, + node vectors",
                 "gj_update": "each matrix read and written once per Gauss-Jordan panel (re, im planes)",
                 "level1": "first-step inverses written; two inverses read, three blocks written per survivor",
                 "residual": "matrix-free 5-point stencil residual r = b - A x: 80 B of stencil planes + x, b, r "
                             "(16 B each) per unknown; FP64-issue bound before HBM"}
    roof_hbm = {}
    for k, unit in hbm_units.items():
        c = prof[k]
        ach = c["work"] / (c["ms"] / 1e3) / 1e9 if c["ms"] else None
        roof_hbm[k] = {"bound": "hbm", "unit": "GB/s", "peak": peaks["hbm_gbs"], "achieved": ach,
                       "frac": ach / peaks["hbm_gbs"] if ach else None,
                       "ms_per_solve": round(c["ms"] / prof_steps, 3),
                       "launches_per_solve": c["launches"] // prof_steps, "work_unit": unit}
    roof_hbm["peak_note"] = f"hbm_gbs from {peak_src}, of measured"

    extras = {} if (a.no_extras or rank != 0) else run_extras(L, pkg, W, a)

    # CPU baseline: the FP64 oracle (scipy SuperLU) solves the same problem on one host thread;
    # its fields are also the reference of the per-solve field error of both GPU forms
    cpu = None
    vs_oracle = None
    if rank == 0 and not a.no_cpu_baseline:
        cpu, f_ref = cpu_baseline_single(a.seed)
        ref_nat = [L.natural(f).reshape(-1) for f in f_ref]

        def errs(fields):
            return {k: float(np.linalg.norm(f - r) / np.linalg.norm(r))
                    for k, f, r in zip(("Ez", "Hx", "Hy"), fields, ref_nat)}
        vs_oracle = {"mixed": errs(fields_mixed), "bound_mixed": 1e-8,
                     "note": "relative 2-norm error of each field against the FP64 oracle solve (SuperLU) of the "
                             "same problem"}
        if fields_fp64 is not None:
            vs_oracle["fp64"] = errs(fields_fp64)
            vs_oracle["bound_fp64"] = 1e-10
    tf32 = tf32_cublas_tflops(torch) if rank == 0 else None
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": a.steps,
                "warmup": a.warmup, "ms_per_step": 1e3 * t / a.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "c64(3xTF32)+c128", "data": "synthetic",
                "config": {"workload": workload, "precision": "mixed: FP32 factors, 3xTF32 tcgen05 products, "
                                                            "FP64 FGMRES refinement",
                           "l2": "inputs larger than L2 (factor storage ~6 GB per solve, no flush needed)",
                           "parallelism": f"replicas x{world}",
                           "launch_shapes": ("autotuned (fdfd_autotune, before the warm-up): " +
                                             json.dumps(tuning_summary([tuned])) if tuned else
                                             "the library's rule (widest tile that fills the GPU)")},
                "e2e": e2e, "gpu_launches": launches, "roofline": roof, "roofline_hbm": roof_hbm,
                "cpu_baseline": cpu, "clocks": clk,
                "rel_residual_max": maxres, "refine_iterations": iters, "field_err_vs_oracle": vs_oracle,
                "fp64": fp64,
                "tf32_cublas_tflops_live": tf32, "factor_flops": stats[-1]["factor_flops"],
                "t_factor_ms": stats[-1]["t_factor_ms"], "t_solve_ms": stats[-1]["t_solve_ms"], **extras}
        print(json.dumps(line), flush=True)
    h.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
