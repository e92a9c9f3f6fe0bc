"""Benchmark of the isoneutral mixing step (cells/s) on GB300.

Workload: the 1-degree global domain, 360 x 180 x 60 interior cells, nonlinear
equation of state (eq type 3), FP64, seeded synthetic state (no dataset). One
step = new time level + zeroed tendencies, isoneutral_diffusion_pre, diffusion
of temp, diffusion of salt, time-level rotation.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line. Under torchrun each rank runs its own replica of the
workload (the path has no exchange step inside one isoneutral step), timing
is the maximum over ranks and ``value`` the cells of all ranks per second.

``--impl reference`` times the CPU implementation of the same step on the host
cores (the NumPy restatement of the reference algorithm that the tests pin to
the reference's own outputs) on a bounded y-band sample of the workload.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

WORKLOAD = dict(name="global_1deg_360x180x60_eos3", nx=360, ny=180, nz=60)
# algorithmic bytes per interior cell per call, float64 fields read/written once
PRE_BYTES_PER_CELL = 180
STEP_BYTES_PER_CELL = 582


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    return rank, world


def _init_pg(world, backend):
    import torch.distributed as dist

    if world > 1 and not dist.is_initialized():
        dist.init_process_group(backend=backend)
    return dist if world > 1 else None


def aggregate_over_ranks(units, seconds, dist=None, device=None):
    """Whole-job throughput of replicas: the units of all ranks over the slowest
    rank's time. Returns ``(total_units, max_seconds)``; single-process when
    ``dist`` is None."""
    if dist is None:
        return units, seconds
    import torch

    t = torch.tensor([float(units), float(seconds)], dtype=torch.float64, device=device)
    u = t[:1].clone()
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    m = t[1:].clone()
    dist.all_reduce(m, op=dist.ReduceOp.MAX)
    return float(u.item()), float(m.item())


class ClockSampler:
    """nvidia-smi clock/throttle sampling (every 50 ms) while the timed region
    runs: the sampler starts half a second before the region, and only the
    samples whose timestamps fall inside the region (``mark_start`` to
    ``mark_stop``) are summarised."""

    QUERY = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.t0 = self.t1 = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.5)
        except OSError:
            self.proc = None
        return self

    def mark_start(self):
        self.t0 = time.time()

    def mark_stop(self):
        self.t1 = time.time()

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [ln for ln in out.splitlines() if ln.strip()]

    def _in_window(self, ln):
        if self.t0 is None or self.t1 is None:
            return True
        import datetime

        try:
            stamp = datetime.datetime.strptime(ln.split(",")[0].strip(), "%Y/%m/%d %H:%M:%S.%f").timestamp()
        except ValueError:
            return False
        return self.t0 - 0.05 <= stamp <= self.t1 + 0.05

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        window = [ln for ln in self.lines if self._in_window(ln)]
        for ln in window or self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 10:
                continue
            try:
                sm.append(float(parts[2]))
                smax = float(parts[3])
            except ValueError:
                continue
            for n, val in zip(names, parts[6:10]):
                if val.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm), "in_timed_region": bool(window),
                "interval_ms": 50}


def _peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return p.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def _profiled(name, key):
    """A figure from a committed ncu summary (``key: value`` line), if any."""
    path = os.path.join(REPO, "profiles", name)
    if not os.path.exists(path):
        return None
    with open(path) as f:
        for line in f:
            if line.startswith(key + ":"):
                return float(line.split(":")[1])
    return None


def _profiled_traffic(name):
    """dram read+write bytes per launch from the committed ncu summary, if any."""
    v = _profiled(name, "traffic_bytes_per_launch")
    return int(v) if v is not None else None


def _fp64_roofline(step_ms):
    """The step against the FP64 pipe, its binding resource: FP64 warp
    instructions per step and the pipe's peak rate from the committed ncu
    summary, the floor they imply, and the measured step's fraction of it."""
    name = "fp64_pipe_roofline_global1deg.md"
    n, peak = _profiled(name, "fp64_warp_instr_per_step"), _profiled(name, "fp64_peak_warp_instr_per_s")
    if not n or not peak:
        return None
    floor_ms = n / peak * 1e3
    return {"fp64_warp_instr_per_step": n, "peak_warp_instr_per_s": peak, "floor_ms": floor_ms,
            "frac": floor_ms / step_ms, "source": f"profiles/{name}"}


def cpu_baseline_sample(nz_band=None, steps=1):
    """Time the oracle step on one host core on a y-band sample of the workload."""
    from oracle import isoneutral_oracle as orc
    from veros_gb300 import synthetic

    ny_band = 24
    host = synthetic.make_state(WORKLOAD["nx"], ny_band, WORKLOAD["nz"], seed=0, y_origin=-30.0, dz_top=10.0,
                                dz_bottom=250.0, land_fraction=0.30, eq_of_state_type=3)
    vs = orc.OracleState({k: v.copy() for k, v in host.arrays.items()})
    orc.isoneutral_step(vs, host.settings)  # warm-up
    t0 = time.perf_counter()
    for _ in range(steps):
        orc.isoneutral_step(vs, host.settings)
    dt = time.perf_counter() - t0
    cells = WORKLOAD["nx"] * ny_band * WORKLOAD["nz"] * steps
    return {"value": cells / dt, "unit": "cells/s", "cores": 1, "kind": "port",
            "sample": f"{steps} step(s) of {WORKLOAD['nx']}x{ny_band}x{WORKLOAD['nz']} (a y-band of the workload), "
                      f"NumPy restatement of the reference NumPy backend, {dt:.2f} s"}


def _band_worker(job):
    """One host core: the oracle step on its own y-band sample (seeded by the core index)."""
    idx, warmup, steps, ny_band = job
    from oracle import isoneutral_oracle as orc
    from veros_gb300 import synthetic

    host = synthetic.make_state(WORKLOAD["nx"], ny_band, WORKLOAD["nz"], seed=idx, y_origin=-30.0, dz_top=10.0,
                                dz_bottom=250.0, land_fraction=0.30, eq_of_state_type=3)
    vs = orc.OracleState({k: v.copy() for k, v in host.arrays.items()})
    for _ in range(warmup):
        orc.isoneutral_step(vs, host.settings)
    t0 = time.perf_counter()
    for _ in range(steps):
        orc.isoneutral_step(vs, host.settings)
    return time.perf_counter() - t0


def run_reference(args):
    """The reference algorithm (NumPy, single-threaded per process) on every host core.

    Each core steps its own 360 x 24 x 60 y-band of the workload, as the
    reference's MPI decomposition would run one sub-domain per core; the rate
    is all cores' cells over the slowest core's time."""
    rank, world = _dist()
    if rank != 0:
        return 0
    import multiprocessing as mp

    cores = int(os.environ.get("VG_REFERENCE_CORES", "0")) or (os.cpu_count() or 1)
    ny_band = 24
    with mp.get_context("spawn").Pool(cores) as pool:
        times = pool.map(_band_worker, [(i, args.warmup, args.steps, ny_band) for i in range(cores)])
    cells = WORKLOAD["nx"] * ny_band * WORKLOAD["nz"] * cores
    dt = max(times)
    value = cells * args.steps / dt
    sample = (f"{cores} processes x {args.steps} steps of a {WORKLOAD['nx']}x{ny_band}x{WORKLOAD['nz']} y-band "
              f"each (the NumPy restatement of the reference NumPy backend; NumPy is single-threaded per process)")
    line = {
        "impl": "reference", "metric": "isoneutral step cells/s (FP64)", "value": value, "unit": "cells/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD["name"], "sample": f"{cores} y-bands {WORKLOAD['nx']}x{ny_band}x{WORKLOAD['nz']}",
                   "eq_of_state_type": 3},
        "cpu_baseline": {"value": value, "unit": "cells/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if not args.no_kernel_ab:
        line["kernel_ab"] = _reference_kernel_ab_line()
    print(json.dumps(line))
    return 0


def _reference_kernel_ab_line():
    try:
        import torch
    except ImportError:
        return {"unavailable": "torch not importable"}
    if not torch.cuda.is_available():
        return {"unavailable": "no CUDA device"}
    device = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(device)
    try:
        return reference_kernel_ab(device)
    except (RuntimeError, OSError) as e:
        return {"unavailable": (str(e).splitlines() or ["error"])[0]}


def _dropin_loop(states, nloop):
    """Cells/s of looping the drop-in functions over the members as Veros's
    thermodynamics calls them (thermodynamics.py:226-241 with zero advection,
    :425-432): new level and zeroed tendencies by tensor operations, then
    isoneutral_diffusion_pre and isoneutral_diffusion for temp and salt on the
    device-resident state. Wall clock over ``nloop`` sweeps after one warm-up
    sweep; the members advance by those steps."""
    import torch

    import veros_gb300 as vg

    def one(dev):
        v = dev.variables
        v.temp[..., v.taup1] = v.temp[..., v.tau] * v.maskT
        v.salt[..., v.taup1] = v.salt[..., v.tau] * v.maskT
        v.dtemp_iso.zero_()
        v.dsalt_iso.zero_()
        v.update(vg.isoneutral_diffusion_pre(dev))
        vg.isoneutral_diffusion(dev, v.temp, True)
        vg.isoneutral_diffusion(dev, v.salt, False)
        v.taum1, v.tau, v.taup1 = v.tau, v.taup1, v.taum1

    for dev in states:
        one(dev)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(nloop):
        for dev in states:
            one(dev)
    torch.cuda.synchronize()
    return sum(d.nx * d.ny * d.nz for d in states) * nloop / (time.perf_counter() - t0)


def run_ensemble(device, steps=20):
    """48 members of uneven extents: looping the single-domain step versus the
    batched persistent launches replayed from a CUDA graph of ``steps`` steps,
    in FP64 and in the split form. Returns the report dict."""
    import torch

    from veros_gb300 import synthetic
    from veros_gb300.ensemble import Ensemble
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    hosts = synthetic.ensemble_states(48)
    cells = sum(h.nx * h.ny * h.nz for h in hosts)
    out = {"members": len(hosts), "cells": cells, "graph_steps": steps}
    for precision in ("f64", "f32split"):
        states = [DeviceState.from_host(h, device=device, precision=precision) for h in hosts]
        steppers = [IsoneutralStepper(st) for st in states]
        for st in steppers:
            st.step(1)
        torch.cuda.synchronize()
        nloop = 3
        t0 = time.perf_counter()
        for _ in range(nloop):
            for st in steppers:
                st.step(1)
        torch.cuda.synchronize()
        loop_value = cells * nloop / (time.perf_counter() - t0)
        dropin_value = _dropin_loop(states, nloop) if precision == "f64" else None
        ens = Ensemble(states)
        tuning, timings = ens.autotune(steps=1)
        ens.replay(steps)  # records the graph for this phase and warms it
        ens.capture(steps)  # records the graph for the phase the timed replay starts from
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        ens.replay(steps)
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        out[precision] = {"batched_graph_cells_per_s": cells * steps / (ms / 1e3),
                          "ms_per_step": ms / steps,
                          "looped_single_domain_cells_per_s": loop_value,
                          "speedup_vs_loop": cells * steps / (ms / 1e3) / loop_value,
                          "looped_dropin_cells_per_s": dropin_value,
                          "speedup_vs_dropin_loop": (cells * steps / (ms / 1e3) / dropin_value
                                                     if dropin_value else None),
                          "tuning": tuning, "candidates_timed": len(timings)}
        ens.close()
        del ens, steppers, states
        torch.cuda.empty_cache()
    return out


def run_adjoint(device, reps=5):
    """Adjoint of an 8-step FP64 rollout at 360 x 180 x 30 (nonlinear EOS,
    lognormal K_iso with sigma 0.3): loss = sum over wet cells of
    (temp after 8 steps - target)^2 with target = initial temp + N(0, 0.05),
    gradients with respect to the initial temp, salt and K_iso through the
    autograd Function with per-step checkpoints. Returns the report dict."""
    import torch

    from veros_gb300 import synthetic
    from veros_gb300.adjoint import IsoneutralAdjoint
    from veros_gb300.state import DeviceState

    nsteps = 8
    host = synthetic.global_1deg_state(seed=0, nz=30, k_iso_lognormal_sigma=0.3)
    rng = np.random.default_rng(4)
    T0 = host.arrays["temp"][..., 1]
    wet = np.zeros_like(T0)
    wet[2:-2, 2:-2] = host.arrays["maskT"][2:-2, 2:-2]
    target = T0 + rng.normal(0.0, 0.05, T0.shape) * wet
    model = IsoneutralAdjoint(DeviceState.from_host(host, device=device))
    T0d, S0d, Kd = (model.field(x) for x in (T0, host.arrays["salt"][..., 1], host.arrays["K_iso"]))
    tgt, w = model.field(target), model.field(wet)

    def once():
        leaves = [model.field(x).requires_grad_() for x in (T0d, S0d, Kd)]
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        T, _ = model.rollout(*leaves, nsteps)
        loss = ((T - tgt) ** 2 * w).sum()
        e[1].record()
        loss.backward()
        e[2].record()
        torch.cuda.synchronize()
        return e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])

    for _ in range(2):
        once()
    torch.cuda.synchronize()
    torch.cuda.reset_peak_memory_stats(device)
    before = torch.cuda.memory_allocated(device)
    times = np.array([once() for _ in range(reps)])
    peak = torch.cuda.max_memory_allocated(device) - before
    fwd, bwd = (float(np.median(times[:, n])) for n in range(2))
    field_mib = model.dev.plane * model.dev.Z * 8 / 2**20
    cells = host.nx * host.ny * host.nz
    return {"workload": f"adjoint of an {nsteps}-step FP64 rollout, {host.nx}x{host.ny}x{host.nz}, eq 3, "
                        "lognormal K_iso (sigma 0.3)",
            "forward_ms": fwd, "backward_ms": bwd, "adjoint_over_forward": bwd / fwd,
            "forward_plus_backward_over_forward": (fwd + bwd) / fwd,
            "backward_cells_per_s": cells * nsteps / (bwd / 1e3),
            "peak_extra_mib": peak / 2**20, "checkpoint_mib_per_step": 2 * field_mib,
            "workspace_mib": model._work.numel() * 8 / 2**20,
            "gpu_launches_per_rollout": nsteps * (model.forward_launches + model.backward_launches),
            "timing": "CUDA events, median of 5 after 2 warm-up rollouts"}


def run_quarter_degree(device, steps=100):
    """The FP32/FP64-split form at 0.25 degree (1440 x 720 x 60, nonlinear
    EOS): ``steps`` steps of the FP64 drop-in and of the split form from the
    same state, cells/s of each, and per-field max and RMS errors of the split
    form against the FP64 run (the FP64 drop-in equals the FP64 oracle to
    1e-12) over the interior wet cells."""
    import torch

    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = synthetic.global_quarter_deg_state(seed=0, lean=True)
    cells = host.nx * host.ny * host.nz
    out = {"workload": f"{host.nx}x{host.ny}x{host.nz} at 0.25 degree, eq 3, {steps} steps", "steps": steps}
    states = {}
    for precision in ("f64", "f32split"):
        dev = DeviceState.from_host(host, device=device, precision=precision)
        stepper = IsoneutralStepper(dev)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        stepper.step(steps)
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        out[precision] = {"cells_per_s": cells * steps / (ms / 1e3), "ms_per_step": ms / steps}
        states[precision] = dev
    out["split_speedup"] = out["f32split"]["cells_per_s"] / out["f64"]["cells_per_s"]
    ref, got = states["f64"], states["f32split"]
    wet = ref.variables.maskT[2:-2, 2:-2].to(torch.float64)
    errs = {}
    for name in ("temp", "salt", "dtemp_iso", "dsalt_iso", "K_11", "K_22", "K_33", "Ai_ez", "Ai_nz", "Ai_bx",
                 "Ai_by"):
        r = getattr(ref.variables, name)
        g = getattr(got.variables, name)
        if name in ("temp", "salt"):
            r, g = r[..., ref.variables.tau], g[..., got.variables.tau]
        r = r[2:-2, 2:-2].to(torch.float64)
        g = g[2:-2, 2:-2].to(torch.float64)
        w = wet.reshape(wet.shape + (1,) * (r.dim() - 3))
        d = (g - r) * w
        rr = r * w
        n = float(w.expand_as(d).sum())
        errs[name] = {"max_rel": float(d.abs().max() / rr.abs().max()),
                      "rms_rel": float((d.pow(2).sum() / n).sqrt() / (rr.pow(2).sum() / n).sqrt())}
    out["split_error_vs_f64"] = errs
    del states, ref, got
    torch.cuda.empty_cache()
    return out


def run_dropin_host(device, steps=3, warmup=1):
    """The drop-in as a plugin-installed NumPy Veros calls it: the tracer part
    of thermodynamics (veros/core/thermodynamics.py:425-432: zeroed
    tendencies, isoneutral_diffusion_pre, isoneutral_diffusion of temp and of
    salt, each result applied with vs.update) on host arrays of the 1-degree
    workload. Every call uploads the fields it reads and downloads the ones it
    returns, so the host<->device copies are inside the timed region; wall
    clock per step (the calls return host arrays, so each one ends with the
    host waiting)."""
    import torch

    sys.path.insert(0, os.path.join(REPO, "tests"))
    from veros_like import VerosLikeState
    from veros_gb300 import isoneutral, synthetic
    from veros_gb300.state import DeviceState

    host = synthetic.global_1deg_state(seed=0)
    settings = dict(host.settings, nx=host.nx, ny=host.ny, nz=host.nz)
    state = VerosLikeState(settings, host.arrays, host.tau, host.taup1, host.taum1)
    vs = state.variables
    cells = host.nx * host.ny * host.nz

    def step():
        vs.P_diss_iso = np.zeros_like(vs.P_diss_iso)
        vs.dtemp_iso = np.zeros_like(vs.dtemp_iso)
        vs.dsalt_iso = np.zeros_like(vs.dsalt_iso)
        vs.update(isoneutral.isoneutral_diffusion_pre(state))
        vs.update(isoneutral.isoneutral_diffusion(state, tr=vs.temp, istemp=True))
        vs.update(isoneutral.isoneutral_diffusion(state, tr=vs.salt, istemp=False))

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    b0 = dict(DeviceState.transfer_bytes)
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    dt = time.perf_counter() - t0
    h2d = (DeviceState.transfer_bytes["h2d"] - b0["h2d"]) // steps
    d2h = (DeviceState.transfer_bytes["d2h"] - b0["d2h"]) // steps
    return {"value": cells * steps / dt, "unit": "cells/s", "ms_per_step": dt / steps * 1e3, "steps": steps,
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "api": "isoneutral_diffusion_pre / isoneutral_diffusion (the functions plugin.install() binds) on a "
                   "NumPy-backend VerosState stand-in, thermodynamics.py:425-432 call sequence, host arrays in "
                   "the reference layout",
            "timing": f"wall clock, {steps} steps after {warmup} warm-up"}


# The tridiagonal A/B workload: one system per column of the 1-degree domain
# (364 x 184 with the halo) and its 60 levels
TDMA_NSYS, TDMA_DEPTH = (WORKLOAD["nx"] + 4) * (WORKLOAD["ny"] + 4), WORKLOAD["nz"]


def tridiag_inputs(device, ncols, nz):
    """Seeded diagonally dominant systems, (columns, levels) row-major: a, b, c, d."""
    import torch

    g = torch.Generator(device="cpu").manual_seed(5)
    shp = (ncols, nz)
    a = -torch.rand(shp, generator=g, dtype=torch.float64)
    c = -torch.rand(shp, generator=g, dtype=torch.float64)
    b = 3.0 + torch.rand(shp, generator=g, dtype=torch.float64)
    d = torch.randn(shp, generator=g, dtype=torch.float64)
    return tuple(x.to(device) for x in (a, b, c, d))


def time_call(fn, flush, reps=20):
    """Median of ``reps`` single-call CUDA-event timings (ms) on torch's current
    stream, each after a write of ``flush`` (larger than L2) and after 3 warm-up calls."""
    import torch

    for _ in range(3):
        fn()
    ms = []
    for _ in range(reps):
        flush.fill_(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        ms.append(a.elapsed_time(b))
    return float(np.median(ms))


def reference_kernel_ab(device, reps=20):
    """The reference's own CUDA TDMA kernel (TridiagKernel<double>, built from
    its source for sm_103a, launched with its launcher's configuration) on the
    tridiagonal A/B workload, timed like the aux kernels."""
    import torch

    from oracle import ref_tdma

    if not ref_tdma.available():
        return {"unavailable": "reference TDMA cubin or launcher not built (oracle/_ref)"}
    kern = ref_tdma.ReferenceTdma()
    av, bv, cv, dv = tridiag_inputs(device, TDMA_NSYS, TDMA_DEPTH)
    bufs = [x.t().contiguous() for x in (av, bv, cv, dv)]
    bufs += [torch.empty_like(bufs[3]), torch.empty_like(bufs[3])]  # out, workspace (c')
    ptrs = [t.data_ptr() for t in bufs]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)
    stream = torch.cuda.current_stream(device).cuda_stream
    ms = time_call(lambda: kern(stream, ptrs, TDMA_NSYS, TDMA_DEPTH, True), flush, reps)
    nbytes = 40 * TDMA_NSYS * TDMA_DEPTH
    return {"kernel": "TridiagKernel<double> (veros/core/special/cuda_tdma_kernels.cu:19-63)",
            "launch": "128 threads, min(1024, ceil(nsys/128)) blocks (cuda_tdma_kernels.cu:96-98)",
            "systems": TDMA_NSYS, "depth": TDMA_DEPTH, "ms": ms,
            "achieved_gbs": nbytes / (ms / 1e3) / 1e9,
            "bytes": "a, b, c, d 32, solution 8 per cell (its c' workspace round trip not counted)",
            "timing": "median of per-call CUDA events, L2 evicted before each call"}


def run_aux(device, reps=20):
    """The path's neighbouring kernels, each timed alone on the 1-degree
    workload (360 x 180 x 60): vertical mixing of temp and salt
    (vertmix_kernel), the streamfunction diagnostics (streamfunction_kernel),
    the generic solve_implicit in the reference's (X, Y, Z) layout
    (pivoting_solve_kernel), the XLA TDMA custom-call target in its
    system-fastest layout (xla_thomas_kernel), and the energy branch of the
    step (one energy_kernel launch for temp and salt plus the flux stores
    it reads, as the difference between the energy and the plain diffusion
    stage).

    Each call runs after a 256 MiB write that evicts the 129 MB L2, and is
    timed alone with CUDA events on torch's current stream; ms is the median
    over ``reps`` calls. GB/s = algorithmic bytes of the call (bytes per cell
    below x cells) / ms."""
    import ctypes

    import torch

    from veros_gb300 import _capi, isoneutral, synthetic, thermodynamics
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    peak, peak_kind = _peaks()
    host = synthetic.global_1deg_state(seed=0)
    dev = DeviceState.from_host(host, device=device)
    IsoneutralStepper(dev).step(1)  # Ai_ez / Ai_nz for the streamfunction
    torch.cuda.synchronize()
    lib = _capi.load()
    cells_pad = dev.plane * dev.Z
    kb = host.arrays["kbot"].reshape(-1)  # one column per (i, j), halo included
    ncols, nz = kb.size, host.nz
    assert (ncols, nz) == (TDMA_NSYS, TDMA_DEPTH)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)

    def timed(fn):
        return time_call(fn, flush, reps)

    out = {"workload": f"{host.nx}x{host.ny}x{host.nz} at 1 degree, eq 3", "reps": reps,
           "timing": "median of per-call CUDA events, L2 evicted before each call", "peak_gbs": peak,
           "peak_source": peak_kind, "kernels": {}}

    def report(name, kernel, ms, nbytes, cells, note):
        gbs = nbytes / (ms / 1e3) / 1e9
        out["kernels"][name] = {"kernel": kernel, "ms": ms, "cells": cells, "algorithmic_bytes": nbytes,
                                "achieved_gbs": gbs, "frac": gbs / peak, "bytes": note}

    report("vertmix_tempsalt", "vertmix_kernel", timed(lambda: thermodynamics.run_vertmix(dev)), 56 * cells_pad,
           cells_pad,
           "kappaH 8, temp and salt read+write 32, dtemp_vmix and dsalt_vmix 16")
    report("isoneutral_diag_streamfunction", "streamfunction_kernel",
           timed(lambda: isoneutral._run_streamfunction(dev)), 88 * cells_pad, cells_pad,
           "K_gm 8, Ai_ez 32, Ai_nz 32, B1_gm and B2_gm 16")

    shp = (ncols, nz)
    av, bv, cv, dv = tridiag_inputs(device, ncols, nz)
    ks = torch.from_numpy(np.where(kb > 0, kb - 1, nz)).to(device)  # land columns: no water
    kk = torch.arange(nz, device=device)
    water = (kk[None, :] >= ks[:, None].long()).to(torch.uint8).contiguous()
    edge = (kk[None, :] == ks[:, None].long()).to(torch.uint8).contiguous()
    res = torch.empty(shp, dtype=torch.float64, device=device)
    bad = torch.zeros(1, dtype=torch.int32, device=device)

    def generic():
        st = lib.vg_solve_implicit_f64(ncols, 1, nz, nz, 0, 1, av.data_ptr(), bv.data_ptr(), cv.data_ptr(),
                                       dv.data_ptr(), water.data_ptr(), edge.data_ptr(), None, None, res.data_ptr(),
                                       bad.data_ptr(), torch.cuda.current_stream(device).cuda_stream)
        _capi.check(st, "solve_implicit")

    nwet = int(water.sum())
    report("solve_implicit", "pivoting_solve_kernel", timed(generic), 42 * nwet + 10 * (ncols * nz - nwet),
           ncols * nz, "water cells: a, b, c, d 32, water and edge masks 2, solution 8; other cells: masks 2, "
           "zero 8; (X, Y, Z) layout")

    at, bt, ct, dt_ = (x.t().contiguous() for x in (av, bv, cv, dv))
    outt = torch.empty_like(dt_)
    bufs = (ctypes.c_void_p * 6)(*(t.data_ptr() for t in (at, bt, ct, dt_, outt, outt)))
    desc = np.array([ncols, nz], dtype=np.int32).tobytes()

    def xla():
        lib.vg_tdma_cuda_double(ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream), bufs, desc,
                                len(desc))

    report("tdma_cuda_double", "xla_thomas_kernel", timed(xla), 40 * ncols * nz, ncols * nz,
           "a, b, c, d 32, solution 8; system-fastest layout; the same systems as the reference arm's "
           "kernel_ab (the reference's own TDMA kernel)")
    if _capi.last_error():
        raise RuntimeError(_capi.last_error())
    del av, bv, cv, dv, at, bt, ct, dt_, outt, res, water, edge

    stages = {}
    for energy in (False, True):
        h = host.copy()
        h.settings["enable_conserve_energy"] = energy
        d = DeviceState.from_host(h, device=device)
        stp = IsoneutralStepper(d)
        for _ in range(3):
            stp.step_stages()
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(reps)]
        for e in ev:
            stp.step_stages(e)
        torch.cuda.synchronize()
        stages[energy] = float(np.median([e[2].elapsed_time(e[3]) for e in ev]))
        del d, stp
    extra = stages[True] - stages[False]
    out["energy_branch"] = {"diffusion_stage_ms": stages[False], "diffusion_stage_ms_energy": stages[True],
                            "extra_ms": extra,
                            "achieved_gbs": 105 * cells_pad / (extra / 1e3) / 1e9 if extra > 0 else None,
                            "bytes": "energy_kernel per cell: per tracer int_drhodX 8, east/north/top fluxes 24, "
                                     "tracer 8; K_33 8, P_diss_iso read+write 16, mask 1"}
    del dev, flush
    torch.cuda.empty_cache()
    return out


def run_gb300(args):
    import torch

    rank, world = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if not torch.cuda.is_available():
        raise RuntimeError("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    dist = _init_pg(world, "nccl")
    device = torch.device("cuda", local)

    from veros_gb300 import synthetic
    from veros_gb300.state import DeviceState
    from veros_gb300.step import IsoneutralStepper

    host = synthetic.global_1deg_state(seed=rank)
    dev = DeviceState.from_host(host, device=device)
    stepper = IsoneutralStepper(dev)
    X, Y, Z = dev.X, dev.Y, dev.Z
    cells = host.nx * host.ny * host.nz

    for _ in range(args.warmup):
        stepper.step_stages()
    torch.cuda.synchronize()

    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        clocks.mark_start()
        start.record()
        for s in range(args.steps):
            stepper.step_stages(ev[s])
        stop.record()
        torch.cuda.synchronize()
        clocks.mark_stop()
    if dist:
        dist.barrier()
    ms = start.elapsed_time(stop)
    stage_ms = np.array([[e[n].elapsed_time(e[n + 1]) for n in range(3)] for e in ev])
    total_cells, sec = aggregate_over_ranks(cells * args.steps, ms / 1e3, dist, device)
    ms = sec * 1e3
    value = total_cells / sec

    # FP32/FP64-split form on the same workload: same number of steps from the
    # same initial state; its tracers are compared with the FP64 run's
    split = DeviceState.from_host(host, device=device, precision="f32split")
    sstep = IsoneutralStepper(split)
    for _ in range(args.warmup):
        sstep.step_stages()
    torch.cuda.synchronize()
    sev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record()
    for s in range(args.steps):
        sstep.step_stages(sev[s])
    s1.record()
    torch.cuda.synchronize()
    split_ms = s0.elapsed_time(s1)
    split_stage = np.array([[e[n].elapsed_time(e[n + 1]) for n in range(3)] for e in sev])
    split_err = {}
    for name in ("temp", "salt"):
        ref = getattr(dev.variables, name)
        got = getattr(split.variables, name)
        split_err[name] = float((got - ref).abs().max() / ref.abs().max())
    split_value = world * cells * args.steps / (split_ms / 1e3)
    del split, sstep

    # end to end through the host-buffer step API
    v = dev.variables
    pin = lambda: torch.empty((X, Y, Z), dtype=torch.float64).pin_memory()  # noqa: E731
    hT, hS = pin(), pin()
    hT.copy_(torch.from_numpy(np.ascontiguousarray(host.temp[..., 1])))
    hS.copy_(torch.from_numpy(np.ascontiguousarray(host.salt[..., 1])))
    outs = [[pin() for _ in range(4)] for _ in range(2)]  # alternate output buffers
    pipe = stepper.pipeline()
    e2e_steps = max(3, min(args.steps, 50))  # steady state: the fill and drain of the pipeline amortised
    for n in range(2):
        pipe.submit(hT, hS, *outs[n % 2])
    pipe.finish()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for n in range(e2e_steps):
        pipe.submit(hT, hS, *outs[n % 2])
    pipe.finish()
    e2e_s = time.perf_counter() - t0
    e2e_cells, e2e_s = aggregate_over_ranks(cells * e2e_steps, e2e_s, dist, device)
    e2e_value = e2e_cells / e2e_s

    launches = args.steps * stepper.launches_per_step()
    ensemble = adjoint = None
    if not (args.no_ensemble and args.no_adjoint and args.no_quarter_degree and not args.aux):
        del dev, stepper
        torch.cuda.empty_cache()
    if not args.no_ensemble:
        ensemble = run_ensemble(device)
    if not args.no_adjoint:
        adjoint = run_adjoint(device)
    quarter = None if args.no_quarter_degree else run_quarter_degree(device)
    aux = run_aux(device) if args.aux else None
    dropin = None if args.no_dropin_host else run_dropin_host(device)
    if rank != 0:
        return 0
    peak, peak_kind = _peaks()
    pre_ms = float(stage_ms[:, 1].mean())
    pre_achieved = PRE_BYTES_PER_CELL * cells / (pre_ms / 1e3) / 1e9
    step_achieved = STEP_BYTES_PER_CELL * cells * args.steps / (ms / 1e3) / 1e9
    traffic = _profiled_traffic("pre_span_kernel_global1deg.md")
    base = cpu_baseline_sample(steps=1)
    line = {
        "metric": "isoneutral step cells/s (FP64)", "value": value, "unit": "cells/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD["name"], "nx": host.nx, "ny": host.ny, "nz": host.nz,
                   "eq_of_state_type": 3, "land_fraction": host.meta["land_fraction_realised"],
                   "l2": "inputs larger than L2: one step touches ~0.9 GB of fields (Ai_* alone 0.5 GB)",
                   "parallelism": f"replicas x{world}"},
        "stage_ms": {"rim_prepare": float(stage_ms[:, 0].mean()), "pre": pre_ms,
                     "diffusion_temp_and_salt": float(stage_ms[:, 2].mean()),
                     "note": "the diffusion stage also prepares the interior cells (fused)"},
        "roofline": {"bound": "hbm", "kernel": "pre_span_kernel", "achieved": pre_achieved, "peak": peak,
                     "unit": "GB/s", "frac": pre_achieved / peak, "traffic": traffic, "peak_source": peak_kind,
                     "algorithmic_bytes_per_cell": PRE_BYTES_PER_CELL,
                     "step_achieved_gbs": step_achieved, "step_frac": step_achieved / peak,
                     "fp64_pipe_pct_ncu": _profiled("pre_span_kernel_global1deg.md", "fp64_pipe_pct"),
                     "fp64_roofline": _fp64_roofline(ms / args.steps),
                     "note": "FP64-pipe bound on GB300 (~1 TFLOP/s FP64); HBM fraction reported as asked"},
        "cpu_baseline": base,
        "e2e": {"value": e2e_value, "unit": "cells/s", "h2d_bytes_per_step": 2 * X * Y * Z * 8,
                "d2h_bytes_per_step": 4 * X * Y * Z * 8, "steps": e2e_steps,
                "api": "IsoneutralStepper.pipeline().submit per step: pinned host buffers in the reference layout, "
                       "uploads and downloads on their own streams overlapping the neighbouring steps' kernels"},
        "f32split": {"value": split_value, "unit": "cells/s", "ms_per_step": split_ms / args.steps,
                     "stage_ms": {"rim_prepare": float(split_stage[:, 0].mean()),
                                  "pre": float(split_stage[:, 1].mean()),
                                  "diffusion_temp_and_salt": float(split_stage[:, 2].mean())},
                     "speedup_vs_f64": split_value / value,
                     "tracer_rel_maxnorm_err_vs_f64": split_err,
                     "precision": "FP64 tracers, gradients, slope denominators/slopes and implicit solve; "
                                  "FP32 tensors, fluxes, taper, tendencies"},
        "gpu_launches": launches,
        "ensemble": ensemble,
        "adjoint": adjoint,
        "quarter_degree": quarter,
        "e2e_dropin_host": dropin,
        "aux": aux,
        "clocks": clocks.summary(),
    }
    print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the 48-member batched-ensemble measurement")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the 8-step rollout adjoint measurement")
    ap.add_argument("--no-quarter-degree", action="store_true",
                    help="skip the 0.25-degree split-versus-FP64 measurement (100 steps, ~25 GB of device memory)")
    ap.add_argument("--no-dropin-host", action="store_true",
                    help="skip the timing of the drop-in calls on host arrays (a plugin-installed NumPy Veros)")
    ap.add_argument("--no-kernel-ab", action="store_true",
                    help="reference arm: skip the reference's CUDA TDMA kernel timing")
    ap.add_argument("--aux", action="store_true",
                    help="add per-kernel timings of vertical mixing, streamfunction, the generic and XLA tridiagonal "
                         "solves and the energy branch (1 degree)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())
