"""Benchmark of the GB300 FDTD engine (prints one JSON line on rank 0).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload plain3d|plain2d]

Metric: Gcell-updates/s, one cell-update = one cell of the PML-extended grid advanced one full
time step (velocity + pressure + memory variables). A bench step is one pass of the time loop
over ``steps_per_bench_step`` time steps of the workload:
* plain2d: the 2D forward workload (944 x 688 extended cells, 4000 time steps = one full solve);
  its 60 MB working set fits in L2, so L2 is flushed (a 256 MB write) before every bench step.
* plain3d: the 3D forward workload (512^3 + PML 32 + transition 32 -> 656^3 extended cells,
  nT = 3000), bench step = 100 time steps; its ~30 GB working set is far larger than L2.

``value`` is device-timed (CUDA events on the engine's stream) with the medium and wavefield
resident in HBM. ``e2e`` is the same metric through the public C ABI with host buffers: each e2e
step uploads that step's inputs from pinned host memory (plain2d: every map and the source
signals, i.e. a full ``fw_set_fields``; plain3d: the source-signal columns of the step's 100
time steps) and reads the step's sensor traces back to host memory.

The default line (plain3d, one GPU) also carries ``extra``: secondary workloads measured in the
same run, each with its own CUDA-event timing and its own check against the FP64 oracle or the
one-by-one path: ``plain2d`` (full solves, rel-L2 of a full solve against the FP64 C oracle,
e2e), ``batched`` (64 simulations: group engine vs one by one on the device, vs one by one
through ``Solver.run()`` and through the host-side NumPy pre-processing on 16 instances each),
``serving_short`` (10 s of the Poisson stream at half size: continuous batching vs FIFO) and
``solver_config0`` (host-to-host ``Solver.run()`` of the plain 2D problem, GPU and NumPy
pre-processing), ``solver_config1`` (the same for the plain 3D workload: host arrays of the 512^3
medium in, 65,536 traces back, against the device-built workload's solve) and ``adjoint`` (gradient evaluations of the 1024^2, nt 6000 misfit through the
autograd API). ``--no-extra`` (or FWGB_BENCH_EXTRA=0) leaves them out.

Multi-GPU (torchrun): every rank runs an independent replica of the workload (the engine does
not shard a single solve); ``value`` = cell-updates of all ranks / max rank time ("weak").
``--impl reference`` times the reference path's CPU implementation: the reference ships no
CPU engine and its GPU executables are x86-64 binaries that cannot run on the aarch64 GB300
host, so the FP64 oracle restatement of the same time loop runs on the host cores.
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
sys.path.insert(0, str(ROOT))

METRIC = "Gcell-updates/s"
L2_BYTES = 126 * 1024 * 1024


# --------------------------------------------------------------------------------- utilities
def dist_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    QUERY = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[3:7]):
                if flag.lower() in ("active", "1"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def traffic_from_profiles(workload: str):
    """DRAM bytes per cell-update recorded from an ncu capture, if a summary is committed."""
    path = ROOT / "profiles" / f"traffic_{workload}.txt"
    if not path.exists():
        return None
    for ln in path.read_text().splitlines():
        if ln.startswith("dram_bytes_per_cell_update:"):
            return float(ln.split(":", 1)[1])
    return None


# --------------------------------------------------------------------------------- workloads
PHYSICS_TEXT = {
    "isotropic": "2 relaxation mechanisms (isotropic relaxation engine)",
    "aniso": "2 relaxation mechanisms, one map set per derivative direction (anisotropic "
             "relaxation engine)",
    "exp": "exponential attenuation from alpha0 (exponential-attenuation engine)",
}


def workload_desc(name: str, grid: int = 0, physics: str = "isotropic") -> dict:
    """The ``config`` description of a workload (shared by the GPU arm and the reference arm)."""
    if name == "plain2d":
        pad = "PML 40 (864x608)" if physics == "exp" else "PML 40 + transition 40 (944x688)"
        return {"workload": f"plain 2D forward, 768x512 + {pad}, nt 4000, 8 random ellipses, "
                            + PHYSICS_TEXT[physics],
                "grid": [864, 608] if physics == "exp" else [944, 688], "nt": 4000,
                "physics": physics, "steps_per_bench_step": 4000,
                "l2": "flushed (256 MB write) before every bench step; working set 60 MB"}
    if name == "plain3d":
        edge = grid or 512
        return {"workload": f"plain 3D forward, {edge}^3 + PML 32 + transition 32 "
                            f"({edge + 144}^3), nt 3000, "
                            "layered fat/muscle/liver with perturbed interfaces and 0.5% scatterers,"
                            " 64-element plane-wave source, 256x256 sensor plane, "
                            + PHYSICS_TEXT[physics],
                "grid": [edge + 144] * 3, "nt": 3000, "physics": physics,
                "steps_per_bench_step": 100,
                "l2": "inputs larger than L2 (working set ~30 GB)"}
    raise ValueError(f"unknown workload {name}")


def make_workload(name: str, rank: int, grid: int = 0, physics: str = "isotropic"):
    """Return (inputs-or-builder, steps_per_bench_step, description dict).

    ``grid`` > 0 replaces the 3D workload's 512^3 cells by grid^3 (small profiling cases)."""
    desc = workload_desc(name, grid, physics)
    if name == "plain2d":
        from fullwave25_gb300.workloads import plain_2d_inputs

        inp = plain_2d_inputs(physics=physics, seed=rank)
        assert list(inp.shape) == desc["grid"] and inp.nt == desc["nt"]
        return inp, inp.nt, desc
    from fullwave25_gb300.workloads3d import plain_3d_device_inputs

    edge = grid or 512
    dinp = plain_3d_device_inputs(seed=rank, shape=(edge, edge, edge), physics=physics)
    assert list(dinp.shape) == desc["grid"] and dinp.nt == desc["nt"]
    return dinp, 100, desc


# --------------------------------------------------------------------------------- CPU baseline
def time_oracle(workload: str, budget_s: float, physics: str = "isotropic"):
    """FP64 C oracle (OpenMP, all host cores) on a bounded sample of the workload: the 2D grid,
    or a 96^3 block of the 3D medium, for as many time steps as fit in ``budget_s``."""
    sys.path.insert(0, str(ROOT / "oracle"))
    from fdtd_oracle_c import OracleC

    if workload == "plain2d":
        from fullwave25_gb300.workloads import plain_2d_inputs

        inp = plain_2d_inputs(physics=physics)
        label = f"plain 2D grid {inp.shape[0]}x{inp.shape[1]}"
    else:
        from fullwave25_gb300.workloads3d import plain_3d_host_sample

        inp = plain_3d_host_sample(physics=physics)
        label = f"plain 3D medium, {inp.shape[0]}x{inp.shape[1]}x{inp.shape[2]} sub-block"
    o = OracleC(inp)
    o.run(1)  # warm-up
    steps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < budget_s and steps + 10 < inp.nt:
        traces = o.run(10)
        steps += 10
    el = time.perf_counter() - t0
    o.close()
    cells = int(np.prod(inp.shape))
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    out = {"value": cells * steps / el / 1e9, "unit": METRIC, "cores": cores, "kind": "port",
           "sample": f"FP64 C oracle (OpenMP, {cores} threads), {label}, {steps} time steps in "
                     f"{el:.1f} s"}
    # kept for the parity statement (not part of the JSON line)
    time_oracle.last = (inp, traces, steps + 1, label)
    return out


def time_numpy_oracle(workload: str, budget_s: float):
    """The FP64 NumPy transcription of the scheme (``oracle/fdtd_oracle.py``) on the same bounded
    sample as :func:`time_oracle`, for as many steps as fit in ``budget_s``; NumPy runs its
    element-wise arrays on one host thread."""
    sys.path.insert(0, str(ROOT / "oracle"))
    from fdtd_oracle import Oracle

    inp, _, _, label = time_oracle.last
    o = Oracle(inp)
    o.step(None)  # warm-up (no recording: the timed loop is the time step itself)
    steps, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < budget_s and steps + 2 < inp.nt:
        o.step(None)
        steps += 1
    el = time.perf_counter() - t0
    cells = int(np.prod(inp.shape))
    return {"value": cells * steps / el / 1e9, "unit": METRIC, "cores": 1, "kind": "port",
            "sample": f"FP64 NumPy oracle (one thread), {label}, {steps} time steps in {el:.1f} s"}


def parity_vs_oracle():
    """rel-L2 of the GPU engine's traces against the FP64 oracle on the CPU-baseline sample."""
    from fullwave25_gb300.engine import Engine

    inp, ref, n_steps, label = time_oracle.last
    rows = (n_steps + inp.mod_t - 1) // inp.mod_t
    with Engine(inp) as eng:
        eng.advance(n_steps)
        got = eng.read_traces(0, rows)
    ref = ref[:rows]
    err = float(np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-300))
    return {"rel_l2_vs_fp64_oracle": err, "tolerance": 1e-4,
            "sample": f"{label}, first {n_steps} time steps, {inp.outc.shape[0]} sensors"}


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    if args.workload not in ("plain2d", "plain3d"):
        # the reference runs one closed executable per simulation and has neither a CPU engine
        # nor batching, serving or gradients: the FP64 oracle stands in for its time loop on the
        # plain workloads only
        print(json.dumps({"impl": "reference", "unavailable":
                          f"no reference counterpart for the {args.workload} workload (the "
                          "reference arm times the FP64 oracle on plain2d / plain3d)"}),
              flush=True)
        return
    per_step_budget = float(os.environ.get("FWGB_REF_SAMPLE_S", "8"))
    vals = []
    for i in range(args.warmup + args.steps):
        r = time_oracle(args.workload, per_step_budget, args.physics)
        if i >= args.warmup:
            vals.append(r["value"])
    v = statistics.mean(vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {**workload_desc(args.workload, args.grid, args.physics),
                       "parallelism": "single GPU" if world == 1 else f"replicas x{world}",
                       "engine": "FP64 C oracle restatement on the host cores (the reference "
                                 "engine is a closed x86-64 CUDA executable; it has no CPU "
                                 "engine)"},
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": r["cores"], "kind": "port",
                             "sample": r["sample"]},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------------- GPU arm
def measure_forward(workload, physics="isotropic", grid=0, steps=10, warmup=3, *,
                    cpu_baseline=True, full_parity=False):
    """The plain 2D / 3D forward workload on this rank's GPU; returns the bench line (rank 0) or
    None (other ranks). ``full_parity``: rel-L2 of one full solve against the FP64 C oracle
    (plain2d only) instead of the CPU-sample parity that comes with ``cpu_baseline``."""
    import torch

    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.workloads import algorithmic_bytes_per_cell

    rank, world, local = dist_info()
    dev = torch.device("cuda", local)
    inputs, chunk, desc = make_workload(workload, rank, grid, physics)
    engine = Engine(inputs) if workload == "plain2d" else inputs.make_engine()
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream
    nt = inputs.nt
    cells = int(np.prod(inputs.shape))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    do_flush = workload == "plain2d"

    def bench_step(i):
        # plain2d: one full solve; plain3d: `chunk` steps continuing a solve
        if workload == "plain2d":
            engine.reset(sptr)
            engine.advance(nt, sptr)
        else:
            if engine.current_step + chunk > nt:
                engine.reset(sptr)
            engine.advance(chunk, sptr)

    def barrier():
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()

    for i in range(warmup):
        bench_step(i)
    barrier()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    with ClockSampler(local) as clocks:
        barrier()
        t0 = time.perf_counter()
        for i in range(steps):
            if do_flush:
                flush.fill_(float(i))
            starts[i].record(stream)
            bench_step(i)
            ends[i].record(stream)
        barrier()
        wall = time.perf_counter() - t0
    dev_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    from fullwave25_gb300.replicas import aggregate_throughput

    _, t_max, units_per_s = aggregate_throughput(cells * chunk * steps, dev_ms / 1e3)
    value = units_per_s / 1e9
    ms_per_step = t_max * 1e3 / steps

    # roofline: one time step (velocity + pressure kernels) over the whole grid
    step_s = (dev_ms / 1e3) / (chunk * steps)
    bpc = algorithmic_bytes_per_cell(len(inputs.shape), physics=physics)
    alg_bytes = bpc * cells
    achieved = alg_bytes / step_s / 1e9
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (
        ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    tr = traffic_from_profiles(workload) if physics == "isotropic" else None

    # e2e through the C ABI with host buffers
    e2e = run_e2e(workload, steps, engine, inputs, chunk, sptr, dev, world)
    clk = clocks.summary()
    parity = None
    if full_parity and rank == 0:
        sys.path.insert(0, str(ROOT / "oracle"))
        from fdtd_oracle_c import run_oracle_c

        engine.reset(sptr)
        got = engine.run(sptr)
        t0 = time.perf_counter()
        ref = run_oracle_c(inputs)
        parity = {"rel_l2_vs_fp64_oracle": float(np.linalg.norm(got - ref) / np.linalg.norm(ref)),
                  "tolerance": 1e-4,
                  "sample": f"one full solve ({inputs.shape[0]}x{inputs.shape[1]}, {nt} steps, "
                            f"{inputs.outc.shape[0]} sensors) against the FP64 C oracle "
                            f"({time.perf_counter() - t0:.1f} s on the host cores)"}
    kernels, tile, launches = engine.kernel_variant, list(engine.block_tile), engine.launches_per_step
    engine.close()
    del engine, flush
    if rank != 0:
        return None
    cpu = cpu_numpy = None
    if cpu_baseline and world == 1:
        cpu = time_oracle(workload, float(os.environ.get("FWGB_CPU_SAMPLE_S", "15")), physics)
        parity = parity_vs_oracle()
        cpu_numpy = time_numpy_oracle(workload, float(os.environ.get("FWGB_NUMPY_SAMPLE_S", "5")))
    return {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": steps,
        "warmup": warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {**desc, "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "wall_s_timed": wall, "kernels": kernels, "block_tile_xyz": tile},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak,
                     "traffic": (tr * cells if tr is not None else None),
                     "kernel": "time step = velocity + pressure kernels",
                     "algorithmic_bytes_per_cell_update": bpc,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks
                     else "fallback 6800 GB/s"},
        "cpu_baseline": cpu,
        "cpu_baseline_numpy": cpu_numpy,
        "parity": parity,
        "e2e": e2e,
        "gpu_launches": int(launches * chunk * steps),
        "clocks": clk,
    }


def run_gpu(args):
    import torch

    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    line = measure_forward(args.workload, args.physics, args.grid, args.steps, args.warmup,
                           cpu_baseline=not args.no_cpu_baseline)
    if line is None:
        return
    if (world == 1 and args.workload == "plain3d" and args.physics == "isotropic" and not args.grid
            and not args.no_extra and os.environ.get("FWGB_BENCH_EXTRA", "1") != "0"):
        torch.cuda.empty_cache()
        line["extra"] = collect_extras()
        line["extra_keys"] = sorted(line["extra"])
    print(json.dumps(line), flush=True)


def collect_extras() -> dict:
    """Secondary workloads of the default run (one GPU), each timed and checked on its own."""
    import torch

    out = {}
    t0 = time.perf_counter()
    p2 = measure_forward("plain2d", steps=3, warmup=3, cpu_baseline=False, full_parity=True)
    out["plain2d"] = {k: p2[k] for k in ("value", "unit", "ms_per_step", "parity", "e2e", "clocks")}
    out["plain2d"].update(workload=p2["config"]["workload"], kernels=p2["config"]["kernels"],
                          l2=p2["config"]["l2"],
                          roofline={k: p2["roofline"][k] for k in ("achieved", "peak", "frac",
                                                                   "unit")})
    torch.cuda.empty_cache()
    b = measure_batch(64, steps=1, warmup=1, host_sample=16, solver_sample=16)
    out["batched"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "sims_per_s", "e2e",
                                        "one_by_one_host_api", "one_by_one_solver_run",
                                        "one_by_one_latency_ms", "batched_latency_ms", "parity",
                                        "clocks")}
    out["batched"]["workload"] = b["config"]["workload"]
    out["batched"]["roofline"] = {k: b["roofline"][k] for k in ("achieved", "peak", "frac", "unit")}
    torch.cuda.empty_cache()
    sv = measure_serve(rate=20.0, duration=10.0, scale=0.5, budget_gb=150, max_active_mcells=16.0,
                       grad_frac=0.2, host_sample=8)
    out["serving_short"] = {"sims_per_s": sv["value"], "unit": "sims/s",
                            "workload": sv["config"]["workload"],
                            "continuous": sv["continuous"], "fifo_one_at_a_time": sv["fifo_one_at_a_time"],
                            "continuous_over_fifo": sv["sims_per_s_ratio"],
                            "one_by_one_host_api_forward_sample": sv["one_by_one_host_api_forward_sample"],
                            "clocks": sv["clocks"]}
    torch.cuda.empty_cache()
    out["solver_config0"] = solver_host_to_host(engine_solve_ms=p2["ms_per_step"])
    torch.cuda.empty_cache()
    out["solver_config1"] = measure_solver3d(512)
    torch.cuda.empty_cache()
    ad = measure_adjoint(1024, 0, 200, steps=2, warmup=1)
    out["adjoint"] = {k: ad[k] for k in ("value", "unit", "ms_per_step", "gradient_check",
                                         "equivalent_Gcell_updates_per_s", "grad_norms", "clocks")}
    out["adjoint"]["workload"] = ad["config"]["workload"]
    out["wall_s"] = time.perf_counter() - t0
    return out


def solver_host_to_host(engine_solve_ms=None) -> dict:
    """``Solver.run()`` of the plain 2D problem (768 x 512 + PML 40 + transition 40, nt 4000),
    host arrays in, traces [512, 4000] back on the host: GPU pre-processing (default) and the
    NumPy pre-processing path; the medium arrays are built before the timed call."""
    import tempfile

    import torch

    from fullwave25_gb300.solver import Solver
    from fullwave25_gb300.workloads import plain_2d_problem

    grid, medium, source, sensor, (n_pml, n_tr) = plain_2d_problem()
    res = {"workload": "plain 2D problem through Solver.run(): 768x512 + PML 40 + transition 40 "
                       "(944x688), nt 4000, 512 sources, 512 sensors"}
    traces = {}
    for on_device in (True, False):
        kw = dict(pml_layer_thickness_px=n_pml, n_transition_layer=n_tr,
                  preprocess_on_device=on_device)
        Solver(tempfile.gettempdir(), grid, medium, source, sensor, **kw).run()   # warm-up
        torch.cuda.synchronize()
        runs = []
        for _ in range(2):
            t0 = time.perf_counter()
            s = Solver(tempfile.gettempdir(), grid, medium, source, sensor, **kw)
            traces[on_device] = s.run()
            runs.append((time.perf_counter() - t0, dict(s.last_timing)))
        best = min(runs, key=lambda r: r[0])
        res["gpu_preprocessing" if on_device else "numpy_preprocessing"] = {
            "host_to_host_s": best[0],
            **{k: best[1][k] for k in ("preprocess_s", "upload_s", "engine_s")}}
    a, b = traces[True], traces[False]
    res["rel_l2_gpu_vs_numpy_preprocessing"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    if engine_solve_ms is not None:
        res["engine_solve_ms_device_timed"] = engine_solve_ms
    return res


def run_e2e(workload, steps, engine, inputs, chunk, sptr, dev, world):
    import torch

    n_e2e = max(1, min(steps, 5))
    if workload == "plain2d":
        # pinned host copies of every input array
        pinned = {}

        def pin(a):
            t = torch.empty(a.shape, dtype=torch.float32 if a.dtype != np.int32 else torch.int32,
                            pin_memory=True)
            t.numpy()[...] = a
            pinned[id(t)] = t
            return t.numpy()

        import copy

        host = copy.copy(inputs)
        host.maps = {k: pin(v) for k, v in inputs.maps.items()}
        host.dcmap = pin(inputs.dcmap)
        host.icmat = pin(inputs.icmat)
        out = torch.empty((inputs.n_out, inputs.outc.shape[0]), dtype=torch.float32,
                          pin_memory=True).numpy()
        h2d = sum(v.nbytes for v in host.maps.values()) + host.dcmap.nbytes + host.icmat.nbytes
        d2h = out.nbytes
        import ctypes as C

        from fullwave25_gb300.engine import _FP

        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(n_e2e):
            engine.set_fields(host)
            engine._call("fw_run", C.c_void_p(sptr), out.ctypes.data_as(_FP), 0)
        torch.cuda.synchronize(dev)
        el = time.perf_counter() - t0
        cells = int(np.prod(inputs.shape))
        return {"value": cells * inputs.nt * n_e2e * world / el / 1e9, "unit": METRIC,
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "steps": n_e2e, "api": "fw_set_fields(host) + fw_run(host traces)"}
    return inputs.run_e2e(engine, chunk, n_e2e, sptr, dev, world)


def run_batch(args):
    """Batched 2D workload: the group engine vs the same simulations one by one."""
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    line = measure_batch(args.batch, args.steps, args.warmup, args.host_sample, args.solver_sample)
    if rank == 0:
        print(json.dumps(line), flush=True)


def measure_batch(n_batch, steps, warmup, host_sample, solver_sample):
    """The group engine on this rank's share of the batched workload, against the same
    simulations one by one: device-resident, through ``Solver.run()`` (GPU pre-processing) on
    ``solver_sample`` instances, and through the host-side NumPy pre-processing on
    ``host_sample`` instances; parity of the smallest member against the FP64 C oracle."""
    import tempfile

    import torch

    from fullwave25_gb300.engine import EngineGroup
    from fullwave25_gb300.replicas import rank_instances
    from fullwave25_gb300.workloads_batch import batch_instance

    rank, world, local = dist_info()
    dev = torch.device("cuda", local)
    ids = rank_instances(rank, world, n_batch)
    torch.zeros(1, device=dev)  # context creation outside the timed build
    # process warm-up outside the timed build: the first use of every builder and engine kernel
    # (module loading), on a small instance that is not part of the batch
    batch_instance(ids[0], scale=0.1).make_engine().close()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    insts = [batch_instance(i) for i in ids]
    engines = [d.make_engine() for d in insts]
    torch.cuda.synchronize(dev)
    build_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream
    units = sum(int(np.prod(d.shape)) * d.nt for d in insts)
    grp = EngineGroup(engines)
    for _ in range(warmup):
        grp.run(sptr)
    torch.cuda.synchronize(dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * steps)]
    with ClockSampler(local) as clocks:
        for i in range(steps):
            ev[2 * i].record(stream)
            grp.run(sptr)
            ev[2 * i + 1].record(stream)
        torch.cuda.synchronize(dev)
    group_ms = sum(ev[2 * i].elapsed_time(ev[2 * i + 1]) for i in range(steps)) / steps
    # end to end, batched: device build (timed above) + group solve + every trace to the host
    t0 = time.perf_counter()
    traces = grp.traces()
    readback_s = time.perf_counter() - t0
    # the same simulations one by one (each a full solve on the same device-resident inputs);
    # one untimed advance first, so that each grid size's kernel-shape autotuning is not timed
    for e in engines:
        e.reset(sptr)
        e.advance(1, sptr)
    torch.cuda.synchronize(dev)
    lat = []
    for e in engines:
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        e.reset(sptr)
        e.advance(e.inputs.nt, sptr)
        b.record(stream)
        torch.cuda.synchronize(dev)
        lat.append(a.elapsed_time(b))
    serial_ms = sum(lat)
    batched_e2e_s = build_s + group_ms / 1e3 + readback_s
    # the smallest member against the FP64 C oracle (full nt)
    parity = None
    if rank == 0:
        sys.path.insert(0, str(ROOT / "oracle"))
        from fdtd_oracle_c import run_oracle_c

        from fullwave25_gb300.workloads3d import to_host_inputs

        k = int(np.argmin([np.prod(d.shape) * d.nt for d in insts]))
        t0 = time.perf_counter()
        ref = run_oracle_c(to_host_inputs(insts[k]))
        parity = {"rel_l2_vs_fp64_oracle": float(np.linalg.norm(traces[k] - ref)
                                                 / np.linalg.norm(ref)),
                  "tolerance": 1e-4,
                  "sample": f"batch member {ids[k]} ({insts[k].shape[0]}x{insts[k].shape[1]}, "
                            f"nt {insts[k].nt}) from the group run, against the FP64 C oracle "
                            f"({time.perf_counter() - t0:.1f} s on the host cores)"}
    # one by one through the reference-facing API: Solver.run() (GPU pre-processing), on a
    # sample of instances; the scenario objects (Grid, medium maps, Source, Sensor) are built
    # before each timed call
    from fullwave25_gb300.solver import Solver
    from fullwave25_gb300.workloads_batch import batch_problem_host

    solver_ids = list(ids[:solver_sample])
    solver_s, solver_err, scenario_s = [], [], []
    for n, i in enumerate(solver_ids):
        t0 = time.perf_counter()
        grid, medium, source, sensor, (n_pml, n_tr) = batch_problem_host(i)
        t1 = time.perf_counter()
        out = Solver(tempfile.gettempdir(), grid, medium, source, sensor,
                     pml_layer_thickness_px=n_pml, n_transition_layer=n_tr).run()
        solver_s.append(time.perf_counter() - t1)
        scenario_s.append(t1 - t0)
        ref = traces[n].T
        solver_err.append(float(np.linalg.norm(out - ref) / max(np.linalg.norm(ref), 1e-30)))
    grp_solver_s = None
    if solver_ids:
        with EngineGroup(engines[:len(solver_ids)]) as gs:
            gs.run(sptr)  # untimed: shape autotuning of this group
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            gs.run(sptr)
            b.record(stream)
            torch.cuda.synchronize(dev)
            grp_solver_s = a.elapsed_time(b) / 1e3
    # end to end, one by one through the host-side NumPy pre-processing (the reference's call
    # sequence: NumPy pre-processing, engine creation and upload, solve, traces back)
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.workloads_batch import batch_inputs_host

    sample = list(ids[:host_sample])
    host_s, host_err = [], []
    for n, i in enumerate(sample):
        t0 = time.perf_counter()
        with Engine(batch_inputs_host(i), validate=False) as e:
            tr = e.run(sptr)
        host_s.append(time.perf_counter() - t0)
        ref = traces[n]
        host_err.append(float(np.linalg.norm(tr - ref) / max(np.linalg.norm(ref), 1e-30)))
    dev_sample_s = sum(lat[:len(sample)]) / 1e3
    # the sample's own batched throughput (same simulations as the host-API runs)
    grp_sample_s = None
    if sample:
        with EngineGroup(engines[:len(sample)]) as gs:
            gs.run(sptr)  # untimed: shape autotuning of this group
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            gs.run(sptr)
            b.record(stream)
            torch.cuda.synchronize(dev)
            grp_sample_s = a.elapsed_time(b) / 1e3
    from fullwave25_gb300.workloads import algorithmic_bytes_per_cell

    achieved = units * algorithmic_bytes_per_cell(2) / (group_ms / 1e3) / 1e9
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (
        ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    tr = traffic_from_profiles("batch2d")
    cells_all = sum(int(np.prod(d.shape)) for d in insts)
    line = {"metric": METRIC, "value": units / (group_ms / 1e3) / 1e9, "unit": METRIC,
            "n_gpus": world, "steps": steps, "warmup": warmup,
            "ms_per_step": group_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"batched 2D forward, {len(insts)} simulations of uneven "
                                   "size (512-2048 x 512-1536 + PML 40 + transition 40), "
                                   "nt 3000-8000, 128-element transmits",
                       "bench_step": "one group run = every simulation to its own nt",
                       "device_build_s": build_s,
                       "group_block_tile_xyz": list(grp.block_tile),
                       "one_by_one_block_tiles": sorted({str(e.block_tile) for e in engines})},
            "sims_per_s": {"batched": len(insts) / (group_ms / 1e3),
                           "one_by_one": len(insts) / (serial_ms / 1e3),
                           "batched_over_one_by_one": serial_ms / group_ms},
            "batched_latency_ms": {"max": group_ms,
                                   "note": "every member's traces are ready when the group run "
                                           "ends, so each member's latency is at most this"},
            "parity": parity,
            "e2e": {"value": units / batched_e2e_s / 1e9, "unit": METRIC,
                    "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": int(sum(t.nbytes for t in traces)),
                    "sims_per_s": len(insts) / batched_e2e_s,
                    "api": "device-side build of every instance + fw_group_run + "
                           "fw_read_traces of every member (media built on the GPU)"},
            "one_by_one_solver_run": {
                "sample_instances": solver_ids,
                "sims_per_s": len(solver_ids) / sum(solver_s) if solver_ids else None,
                "scenario_build_s_mean": float(np.mean(scenario_s)) if scenario_s else None,
                "batched_sims_per_s_same_sample":
                    len(solver_ids) / grp_solver_s if grp_solver_s else None,
                "batched_over_solver_run_same_sample":
                    sum(solver_s) / grp_solver_s if grp_solver_s else None,
                "rel_l2_vs_batched_traces_max": max(solver_err) if solver_err else None,
                "api": "Solver(grid, medium, source, sensor).run() per instance (GPU "
                       "pre-processing, engine creation, solve, traces to the host); the "
                       "scenario objects are built before the timed call"},
            "one_by_one_host_api": {
                "sample_instances": sample,
                "sims_per_s": len(sample) / sum(host_s) if sample else None,
                "device_resident_sims_per_s_same_sample":
                    len(sample) / dev_sample_s if sample else None,
                "batched_sims_per_s_same_sample":
                    len(sample) / grp_sample_s if grp_sample_s else None,
                "batched_over_host_api_same_sample":
                    sum(host_s) / grp_sample_s if grp_sample_s else None,
                "rel_l2_vs_batched_traces_max": max(host_err) if host_err else None,
                "api": "NumPy pre-processing (relaxation lookup, PML builder) + Engine "
                       "(fw_create, fw_set_fields host) + fw_run with host traces, per instance"},
            "one_by_one_latency_ms": {"p50": float(np.percentile(lat, 50)),
                                      "p99": float(np.percentile(lat, 99)),
                                      "max": float(max(lat))},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": (tr * cells_all if tr is not None else None),
                         "kernel": "group time step = velocity + pressure group kernels, "
                                   "every member active",
                         "algorithmic_bytes_per_cell_update": algorithmic_bytes_per_cell(2),
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks
                         else "fallback 6800 GB/s"},
            "gpu_launches": 2 * max(d.nt for d in insts) * steps,
            "clocks": clocks.summary()}
    grp.close()
    for e in engines:
        e.close()
    return line


def run_serve(args):
    """Serving stream: Poisson arrivals of forward and gradient solves, continuous batching vs
    FIFO one at a time."""
    import torch

    torch.cuda.set_device(0)
    line = measure_serve(args.rate, args.duration, args.scale, args.budget_gb,
                         args.max_active_mcells, args.grad_frac, args.host_sample)
    print(json.dumps(line), flush=True)


def measure_serve(rate, duration, scale, budget_gb, max_active_mcells, grad_frac, host_sample):
    """The serving stream on GPU 0; returns its line."""
    import torch

    from fullwave25_gb300.server import (Request, engine_bytes, poisson_arrivals,
                                         serve_continuous, serve_fifo)
    from fullwave25_gb300.workloads_batch import batch_instance, gradient_job

    arrivals = poisson_arrivals(rate, duration, seed=0)
    kinds = np.where(np.random.default_rng(1).random(len(arrivals)) < grad_frac,
                     "gradient", "forward")

    reqs = []
    for i, (t, kind) in enumerate(zip(arrivals, kinds)):
        if kind == "gradient":
            # the request's input data (starting medium, observed traces) exists before it arrives
            job = gradient_job(i, scale=scale)
            reqs.append(Request(rid=i, arrival=float(t), build=(lambda j=job: j), kind="gradient",
                                bytes_needed=job.bytes_needed()))
        else:
            r = Request(rid=i, arrival=float(t), build=lambda i=i: batch_instance(i, scale=scale))
            d = r.build()  # memory need from the instance geometry (built once to measure)
            r.bytes_needed = engine_bytes(d.shape, d.nt, d.outc.shape[0])
            r.cells = int(np.prod(d.shape))
            del d
            reqs.append(r)
    torch.cuda.synchronize()
    # warm-up: one small continuous run so that graphs and kernels are loaded
    warm = [r for r in reqs if r.kind == "forward"][:3] + [r for r in reqs if r.kind == "gradient"][:1]
    serve_continuous(warm, budget_bytes=budget_gb << 30)
    for r in warm:
        r.admitted = r.finished = -1.0
        r.traces = r.result = None
    cap = int(max_active_mcells * 1e6) if max_active_mcells > 0 else None
    with ClockSampler(0) as clocks:
        cont = serve_continuous(reqs, budget_bytes=budget_gb << 30, chunk_steps=256,
                                max_active_cells=cap)
    for r in reqs:
        r.result = None
    # the FIFO baseline runs every request on its own handle: tune the kernel shape of each
    # forward grid size first (untimed; cached per size, as in a long-running server), so that
    # the baseline does not pay autotuning trials inside its timed stream
    from fullwave25_gb300.engine import Engine

    tuned = set()
    for r in reqs:
        if r.kind == "forward":
            d = r.build()
            if tuple(d.shape) not in tuned:
                tuned.add(tuple(d.shape))
                with Engine(d, validate=False) as e:
                    e.advance(1)   # the first advance from step 0 runs the trials
            del d
    torch.cuda.synchronize()
    fifo = serve_fifo(reqs)
    for r in reqs:
        r.result = None
    # one at a time through the host-side API (the reference's call sequence: NumPy
    # pre-processing, engine creation and upload, solve, traces back) on the stream's first
    # forward requests; gradient requests have no host-side path and are left out, so the ratio
    # against the whole mixed stream understates the served advantage
    from fullwave25_gb300.workloads_batch import batch_inputs_host

    host_reqs = [r for r in reqs if r.kind == "forward"][:host_sample]
    host_s, host_err = [], []
    for r in host_reqs:
        t0 = time.perf_counter()
        with Engine(batch_inputs_host(r.rid, scale=scale), validate=False) as e:
            tr = e.run()
        host_s.append(time.perf_counter() - t0)
        host_err.append(float(np.linalg.norm(tr - r.traces) / max(np.linalg.norm(r.traces), 1e-30)))
    host_api = ({"requests": [r.rid for r in host_reqs],
                 "sims_per_s": len(host_s) / sum(host_s),
                 "continuous_over_host_api": cont["sims_per_s"] / (len(host_s) / sum(host_s)),
                 "rel_l2_vs_served_traces_max": max(host_err),
                 "api": "NumPy pre-processing (relaxation lookup, PML builder) + Engine "
                        "(fw_create, fw_set_fields host) + fw_run with host traces, per request"}
                if host_s else None)
    n_grad = int((kinds == "gradient").sum())
    line = {"metric": "simulations/s (serving stream)", "value": cont["sims_per_s"],
            "unit": "sims/s", "n_gpus": 1, "steps": 1, "warmup": 1,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": f"Poisson {rate} req/s for {duration} s: 2D forward "
                                   f"solves (batched-workload instances) and "
                                   f"{grad_frac:.0%} gradient solves (512-1024 square "
                                   f"grids, nt 6000 at 1024), sizes scaled by {scale}; device "
                                   f"budget {budget_gb} GB, blocks of 256 steps, "
                                   "2 gradient worker streams; FIFO after the kernel shape of "
                                   "every forward grid size was tuned (untimed)",
                       "requests": len(reqs), "gradient_requests": n_grad,
                       "max_active_cells": cap},
            "continuous": cont, "fifo_one_at_a_time": fifo,
            "one_by_one_host_api_forward_sample": host_api,
            "sims_per_s_ratio": cont["sims_per_s"] / fifo["sims_per_s"],
            "clocks": clocks.summary()}
    return line


def run_adjoint(args):
    """Adjoint gradient: 1024^2 grid, nt 6000, 512-sensor row, checkpoints every 200 steps."""
    line = measure_adjoint(args.grid or 1024, args.nt, args.checkpoint_every, args.steps,
                           args.warmup)
    print(json.dumps(line), flush=True)


def directional_gradient_check(prob, start, observed, grad_c, amplitude=4.0, sigma=120.0):
    """The adjoint's derivative of J along a smooth perturbation of c against a central finite
    difference of J itself: a Gaussian bump of ``amplitude`` m/s and ``sigma`` cells at the grid
    centre, J(c +- bump) from plain forward solves (J = 1/2 sum (traces - observed)^2 in FP64).
    The bump is wide and strong enough that J's change dominates the float32 rounding of the
    perturbed maps (narrow or weak bumps move K = c^2 rho by less than its float32 resolution in
    most cells) and of the forward traces; J is summed from float32 traces, so at 1024^2 its
    rounding still leaves about 1e-2 of noise in the difference (the FP64 oracle's central
    difference agrees with the adjoint to 3e-3 there, 2e-5 at 256^2)."""
    import torch

    from fullwave25_gb300.engine import Engine

    nx, ny = prob.shape
    dev = start[0].device
    x = torch.arange(nx, dtype=torch.float64, device=dev)[:, None] - (nx - 1) / 2
    y = torch.arange(ny, dtype=torch.float64, device=dev)[None, :] - (ny - 1) / 2
    bump = amplitude * torch.exp(-(x * x + y * y) / (2 * sigma * sigma))
    obs = observed.double()

    def J(c):
        with Engine(prob.build(c, *start[1:]), validate=False) as e:
            tr = torch.as_tensor(e.run(), device=dev).double()
        return 0.5 * float(((tr - obs) ** 2).sum())

    fd = (J(start[0] + bump) - J(start[0] - bump)) / 2.0
    ad = float((grad_c.double() * bump).sum())
    return {"adjoint_directional_derivative": ad, "central_difference": fd,
            "rel_diff": abs(ad - fd) / max(abs(fd), 1e-300),
            "perturbation": f"Gaussian bump of {amplitude} m/s in c, sigma {sigma} cells, at the "
                            "grid centre; J(c +- bump) from float32 forward solves"}


def measure_adjoint(n=1024, nt=0, every=200, steps=3, warmup=3):
    """Gradient evaluations through the public autograd API on GPU 0; returns the line."""
    import torch
    from scipy.ndimage import gaussian_filter

    from fullwave25_gb300.adjoint import AdjointProblem
    from fullwave25_gb300.engine import Engine
    from fullwave25_gb300.workloads import ellipse_medium_2d

    torch.cuda.set_device(0)
    dev = torch.device("cuda", 0)
    nt = nt or (6000 if n == 1024 else int(6000 * n / 1024))
    dx = 1540 / 3e6 / 12
    c, rho, a0, gam = ellipse_medium_2d((n, n), dx, seed=0)
    sig = 2e-3 / dx
    blur = lambda a: gaussian_filter(a, sig, mode="nearest")  # noqa: E731
    t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=dev)  # noqa: E731
    true = (t(c), t(rho), t(a0), t(gam))
    start = (t(blur(c)), t(blur(rho)), t(blur(a0)), t(gam))
    prob = AdjointProblem((n, n), nt=nt, n_pml=40, n_transition=40, c_ref=start[0], device=dev,
                          sensor_step=max(1, n // 512), sensor_row=5)
    with Engine(prob.build(*true), validate=False) as e:
        observed = torch.as_tensor(e.run(), device=dev)

    def evaluate():
        cc, rr, aa = [x.clone().requires_grad_(True) for x in start[:3]]
        J = prob.misfit(cc, rr, aa, start[3], observed, checkpoint_every=every)
        J.backward()
        return float(J.detach()), cc.grad, rr.grad, aa.grad

    for _ in range(warmup):
        evaluate()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    with ClockSampler(0) as clocks:
        for _ in range(steps):
            J, gc, gr, ga = evaluate()
        torch.cuda.synchronize(dev)
    el = (time.perf_counter() - t0) / steps
    ext = prob.build(*start).shape
    check = directional_gradient_check(prob, start, observed, gc)
    cells = int(np.prod(ext))
    line = {"metric": "gradient evaluations/s (adjoint)", "value": 1.0 / el, "unit": "grad/s",
            "n_gpus": 1, "steps": steps, "warmup": warmup, "ms_per_step": el * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 wavefields, f64 gradient accumulation", "data": "synthetic",
            "config": {"workload": f"adjoint gradient, {n}x{n} + PML 40 + transition 40 "
                                   f"({ext[0]}x{ext[1]}), nt {nt}, {observed.shape[1]}-sensor "
                                   "row, true medium vs Gaussian-blurred (sigma 2 mm) start, "
                                   f"gradient w.r.t. c, rho, alpha0, checkpoints every {every} steps",
                       "misfit": J,
                       "time_steps_per_evaluation": "3 nt (forward, recompute, adjoint)"},
            "equivalent_Gcell_updates_per_s": 3 * nt * cells / el / 1e9,
            "grad_norms": {"c": float(gc.norm()), "rho": float(gr.norm()),
                           "alpha0": float(ga.norm())},
            "gradient_check": check,
            "clocks": clocks.summary()}
    return line


def measure_adjoint3d(edge=160, nt=600, every=60, steps=3, warmup=3, physics="isotropic"):
    """The 3D discrete adjoint through the engine's C ABI on a block of the plain 3D medium
    (``edge``^3 + PML 16 + transition 16): per evaluation one ``fw_adjoint_forward`` (forward
    solve with checkpoints) and one ``fw_adjoint_backward`` (recomputation + reverse pass) of the
    misfit against traces scaled by 0.9, each timed with CUDA events."""
    import torch

    from fullwave25_gb300.engine import Engine, adjoint_gradient_maps
    from fullwave25_gb300.workloads3d import plain_3d_device_inputs

    torch.cuda.set_device(0)
    d = plain_3d_device_inputs(shape=(edge,) * 3, nt=nt, n_pml=16, n_transition=16,
                               sensor_plane=min(256, edge // 2), element_height=8,
                               physics=physics)
    cells = int(np.prod(d.shape))
    names = adjoint_gradient_maps(d)
    s = torch.cuda.current_stream()
    fw, bw = [], []
    with Engine(d, validate=False) as eng:
        for i in range(warmup + steps):
            e0, e1, e2, e3 = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            e0.record(s)
            eng.adjoint_forward(every, s.cuda_stream)
            e1.record(s)
            tr = torch.empty((d.n_out, d.outc.shape[0]), device="cuda")
            eng.read_traces_into(0, d.n_out, tr.data_ptr(), s.cuda_stream)
            res = (0.1 * tr).contiguous()
            g = torch.zeros((len(names),) + tuple(d.shape), dtype=torch.float64, device="cuda")
            e2.record(s)
            eng.adjoint_backward(res.data_ptr(), g.data_ptr(), s.cuda_stream)
            e3.record(s)
            torch.cuda.synchronize()
            if i >= warmup:
                fw.append(e0.elapsed_time(e1))
                bw.append(e2.elapsed_time(e3))
        dev_gb = eng.device_bytes / 1e9
    ms = float(np.mean(fw) + np.mean(bw))
    return {"metric": "gradient evaluations/s (3D adjoint)", "value": 1e3 / ms, "unit": "grad/s",
            "n_gpus": 1, "steps": steps, "warmup": warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 wavefields, f64 gradient accumulation", "data": "synthetic",
            "config": {"workload": f"3D adjoint ({physics}), plain 3D medium {edge}^3 + PML 16 + "
                                   f"transition 16 ({d.shape[0]}^3 = {cells / 1e6:.1f} M cells), "
                                   f"nt {nt}, checkpoints every {every} steps, "
                                   f"{d.outc.shape[0]} sensors",
                       "gradient_maps": len(names)},
            "forward_ms": float(np.mean(fw)), "backward_ms": float(np.mean(bw)),
            "forward_gcell_updates_per_s": cells * nt / float(np.mean(fw)) / 1e6,
            "backward_gcell_steps_per_s": cells * nt / float(np.mean(bw)) / 1e6,
            "device_gb": dev_gb, "gradient_finite": bool(torch.isfinite(g).all()),
            "gradient_nonzero": bool((g != 0).any())}


def run_adjoint3d(args):
    line = measure_adjoint3d(args.grid or 160, args.nt or 600, args.checkpoint_every
                             if args.checkpoint_every != 200 else 60, args.steps, args.warmup,
                             args.physics)
    print(json.dumps(line), flush=True)


def plain_3d_problem(edge=512, seed=0, nt=3000, f0=2e6, ppw=10, cfl=0.2, element_height=32,
                     sensor_plane=256):
    """The plain 3D workload as a user of the reference API holds it: host arrays of the
    original 512^3 grid (sound speed, density, beta, the per-cell relaxation parameters of each
    layer's table entry) in a MediumRelaxationMaps, and Source / Sensor masks (64 x 1 element
    plane wave on depth row 0, a 256 x 256 sensor plane on depth row 4). The arrays are generated
    on the GPU (same seeded layers and scatterers as the device-built workload) and copied to
    the host."""
    import torch

    from fullwave25_gb300.grid import Grid
    from fullwave25_gb300.medium import MediumRelaxationMaps, relaxation_param_keys
    from fullwave25_gb300.pulse import gaussian_modulated_sinusoidal_signal
    from fullwave25_gb300.relaxation import default_table
    from fullwave25_gb300.source import Sensor, Source
    from fullwave25_gb300.workloads3d import LAYERS, layered_medium_3d

    shape = (edge, edge, edge)
    grid = Grid.from_cells(shape, f0=f0, nt=nt, ppw=ppw, cfl=cfl)
    dev = torch.device("cuda", torch.cuda.current_device())
    c, rho, layer = layered_medium_3d(shape, grid.dx, seed, dev, n_boundary=0)
    table = default_table()
    keys = relaxation_param_keys(2)
    per_layer = np.stack([np.array([table.lookup(np.array([[lay[3]]]), np.array([[lay[4]]]))[k][0, 0]
                                    for k in keys]) for lay in LAYERS])
    lid = layer.cpu().numpy().astype(np.intp)
    relax = {k: per_layer[:, i][lid] for i, k in enumerate(keys)}
    del lid, layer
    medium = MediumRelaxationMaps(grid, c.cpu().numpy(), rho.cpu().numpy(), np.zeros(shape), relax)
    del c, rho, relax
    ny, nz = shape[1], shape[2]
    z0 = nz // 2 - element_height // 2
    mask = np.zeros(shape, dtype=bool)
    mask[0, :, z0:z0 + element_height] = True
    sig = gaussian_modulated_sinusoidal_signal(nt=nt, duration=grid.duration, ncycles=2,
                                               drop_off=2, f0=f0, p0=1e6)
    source = Source(np.broadcast_to(sig, (int(mask.sum()), nt)), mask)
    smask = np.zeros(shape, dtype=bool)
    y0, zs0 = ny // 2 - sensor_plane // 2, nz // 2 - sensor_plane // 2
    smask[4, y0:y0 + sensor_plane, zs0:zs0 + sensor_plane] = True
    return grid, medium, source, Sensor(smask)


def measure_solver3d(edge=512, parity=True) -> dict:
    """Host-to-host ``Solver.run()`` of the plain 3D workload (GPU pre-processing): host arrays
    in, traces [65536, 3000] back on the host, against the engine's own device-timed solve of
    the device-built workload (the same maps, built directly on the extended grid: the traces
    must agree to rounding)."""
    import tempfile

    import torch

    from fullwave25_gb300.solver import Solver
    from fullwave25_gb300.workloads3d import plain_3d_device_inputs

    sp, eh = min(256, edge // 2), min(32, edge // 2)
    t0 = time.perf_counter()
    grid, medium, source, sensor = plain_3d_problem(edge, element_height=eh, sensor_plane=sp)
    scenario_s = time.perf_counter() - t0
    torch.cuda.empty_cache()
    solver = Solver(tempfile.gettempdir(), grid, medium, source, sensor, pml_layer_thickness_px=32,
                    n_transition_layer=32)
    t0 = time.perf_counter()
    out = solver.run()
    host_to_host_s = time.perf_counter() - t0
    timing = dict(solver.last_timing)
    del solver, medium
    torch.cuda.empty_cache()
    ext = [edge + 144] * 3
    res = {"workload": f"plain 3D problem through Solver.run(): {edge}^3 + PML 32 + transition 32 "
                       f"({ext[0]}^3), nt {grid.nt}, {source.n_sources} sources, "
                       f"{sensor.n_sensors} sensors",
           "host_to_host_s": host_to_host_s,
           **{k: timing[k] for k in ("preprocess_s", "upload_s", "engine_s")},
           "scenario_build_s": scenario_s,
           "gcell_updates_per_s_host_to_host": float(np.prod(ext)) * grid.nt / host_to_host_s / 1e9,
           "trace_shape": list(out.shape)}
    if parity:
        d = plain_3d_device_inputs(shape=(edge,) * 3, sensor_plane=sp, element_height=eh)
        eng = d.make_engine()
        stream = torch.cuda.current_stream()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        eng.reset(stream.cuda_stream)
        a.record(stream)
        eng.advance(d.nt, stream.cuda_stream)
        b.record(stream)
        torch.cuda.synchronize()
        ref = eng.read_traces().T
        eng.close()
        res["engine_solve_s_device_timed"] = a.elapsed_time(b) / 1e3
        res["rel_l2_vs_device_built_workload"] = float(np.linalg.norm(out - ref)
                                                       / np.linalg.norm(ref))
    return res


def run_solver3d(args):
    import torch

    torch.cuda.set_device(0)
    with ClockSampler(0) as clocks:
        res = measure_solver3d(args.grid or 512)
    line = {"metric": "host-to-host Solver.run() time", "value": res["host_to_host_s"], "unit": "s",
            "n_gpus": 1, "steps": 1, "warmup": 0, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": res,
            "clocks": clocks.summary()}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=os.environ.get("FWGB_WORKLOAD", "plain3d"),
                    choices=["plain2d", "plain3d", "batch2d", "serve2d", "adjoint2d", "adjoint3d",
                             "solver3d"])
    ap.add_argument("--physics", default="isotropic", choices=["isotropic", "aniso", "exp"],
                    help="plain2d/plain3d/adjoint3d: cell physics (relaxation engine, "
                         "anisotropic relaxation, exponential attenuation)")
    ap.add_argument("--rate", type=float, default=20.0, help="serve2d: arrivals per second")
    ap.add_argument("--duration", type=float, default=10.0, help="serve2d: stream length [s]")
    ap.add_argument("--scale", type=float, default=0.5, help="serve2d: instance size scale")
    ap.add_argument("--budget-gb", type=int, default=150, help="serve2d: device memory budget")
    ap.add_argument("--max-active-mcells", type=float, default=16.0,
                    help="serve2d: cap on the grid cells (millions) of the forward requests "
                         "stepping together (0: memory budget only)")
    ap.add_argument("--grad-frac", type=float, default=0.2,
                    help="serve2d: fraction of gradient requests")
    ap.add_argument("--batch", type=int, default=64, help="simulations per rank (batch2d)")
    ap.add_argument("--host-sample", type=int, default=16,
                    help="batch2d / serve2d: instances (forward requests) also run one by one "
                         "through the host-side API")
    ap.add_argument("--solver-sample", type=int, default=16,
                    help="batch2d: instances also run one by one through Solver.run()")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="plain3d: leave out the secondary workloads of the default line")
    ap.add_argument("--grid", type=int, default=0,
                    help="3D workload edge in cells (default 512; smaller for profiling); "
                         "adjoint2d: grid edge (default 1024); adjoint3d: medium edge "
                         "(default 160)")
    ap.add_argument("--nt", type=int, default=0,
                    help="adjoint2d: time steps (default 6000 at 1024, scaled with the grid); "
                         "adjoint3d: default 600")
    ap.add_argument("--checkpoint-every", type=int, default=200,
                    help="adjoint2d: steps between wavefield checkpoints (adjoint3d: 60 unless "
                         "given)")
    args = ap.parse_args()
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps requested; using 3", file=sys.stderr)
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch2d":
        run_batch(args)
    elif args.workload == "serve2d":
        run_serve(args)
    elif args.workload == "adjoint2d":
        run_adjoint(args)
    elif args.workload == "adjoint3d":
        run_adjoint3d(args)
    elif args.workload == "solver3d":
        run_solver3d(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
