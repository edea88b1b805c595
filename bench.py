"""Benchmark of the GB300 stencil library: T_eff of the 3-D diffusion step (ParallelStencil's
README metric, A_eff = (2*D_u + D_k) bytes per step / time per step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (headline): the 3-D diffusion step in flux form with a spatially varying conductivity
array (T, T2, Ci, lam; FP64; 512^3), memopt z-sweep kernel -- D_u = T, D_k = {lam, Ci}, so
A_eff = 4 words/cell = 4.295 GB per step. Inputs: T ~ U(0,1) (seed 2), lam = 1 + 0.5 U(0,1)
(seed 3), Ci = 1, dt = min(dx,dy,dz)^2 / max(lam) / 8.1. All arrays (4.3 GB) are far larger
than L2 (129 MB), so no L2 flush is needed between steps. Also reported: memcopy3D, the README
(T, T2, Ci) form, plain vs memopt, FP32, and 256^3.

Rank 0 prints ONE JSON line. `--impl reference` times the CPU oracle (a C/OpenMP restatement
of the reference's Threads-backend kernel) on the host cores instead.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "parallelstencil.jl_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

WORDS_FLUX_LAM = 4  # T read, T2 write, lam read, Ci read
# the headline body as a run-time compiled kernel (ps_gb300.parallel_kernel), bounds-checked and not
JIT_FLUX_LAM = """@parallel {opt}function diffusion3D_step!(T2, T, Ci, lam, dt, _dx, _dy, _dz)
    @all(qx)   = -@av_xi(lam)*@d_xi(T)*_dx
    @all(qy)   = -@av_yi(lam)*@d_yi(T)*_dy
    @all(qz)   = -@av_zi(lam)*@d_zi(T)*_dz
    @all(dTdt) = @inn(Ci)*(-@d_xa(qx)*_dx - @d_ya(qy)*_dy - @d_za(qz)*_dz)
    @inn(T2)   = @inn(T) + dt*@all(dTdt)
    return
end"""
# the @hide_communication example's step (examples/diffusion3D_multigpucpu_hidecomm_novis.jl:12-15)
JIT_DIFF_INV = """@parallel function diffusion3D_step!(T2, T, Ci, lam, dt, _dx, _dy, _dz)
    @inn(T2) = @inn(T) + dt*(lam*@inn(Ci)*(@d2_xi(T)*_dx^2 + @d2_yi(T)*_dy^2 + @d2_zi(T)*_dz^2))
    return
end"""
WORDS_README = 3  # T read, T2 write, Ci read
WORDS_MEMCOPY = 3
NT_JOB = 50  # time steps of one diffusion job (the e2e unit; the 512^3 sweep workload's step count)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(name):
    """dram bytes per launch recorded in profiles/<name>.md ('traffic_bytes_per_launch: N')."""
    p = os.path.join(ROOT, "profiles", name + ".md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons while the timed work runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        # the raw samples: PS_BENCH_CLOCKS_DIR if set, else the system's temporary directory
        import tempfile

        d = os.environ.get("PS_BENCH_CLOCKS_DIR") or tempfile.gettempdir()
        self.path = os.path.join(d, f"clocks_bench_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        load = [r for r in rows if r[2] > 300.0] or rows
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in load for i, v in enumerate(r[3]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in load), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows), "samples_under_load": len(load),
                "power_w_max": max(r[2] for r in rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def rank_ops(torch, dist, device):
    """barrier() and max_over_ranks(x) of the replica runs: every rank times its own replica and the
    job's time is the slowest rank's (NCCL between GPUs; gloo in the CPU tests of this path)."""
    def barrier():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x):
        if dist is None:
            return x
        t = torch.tensor([float(x)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    return barrier, max_over_ranks


def job_value(world, units_per_rank, seconds):
    """Whole-job throughput of `world` replicas: the units all ranks processed over the slowest
    rank's time (weak scaling: per-rank work fixed)."""
    return world * units_per_rank / seconds


def time_steps(torch, step_fn, steps, warmup, barrier, stream):
    for i in range(warmup):
        step_fn(i)
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(steps):
        step_fn(i)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3  # seconds for `steps` steps


def run_ours(a, world, rank, local):
    import torch

    import ps_gb300 as ps
    from ps_gb300 import _lib
    from ps_gb300.core import descriptor, stream_handle

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    barrier, max_over_ranks = rank_ops(torch, dist, "cuda")

    ps.init_parallel_stencil(ps.GB300, "Float64", 3, device=local)
    stream = torch.cuda.current_stream()
    n = a.n
    lx = 10.0
    dx = lx / (n - 1)
    _dx = 1.0 / dx
    dt = dx * dx / 1.5 / 8.1

    def fields(dtype, nn):
        g = torch.Generator(device="cuda")
        tdt = torch.float64 if dtype == np.float64 else torch.float32
        T = ps.empty(nn, nn, nn, dtype=dtype)
        g.manual_seed(2)
        T.copy_(torch.rand((nn, nn, nn), generator=g, device="cuda", dtype=torch.float64).to(tdt))
        T2 = ps.empty(nn, nn, nn, dtype=dtype)
        T2.copy_(T)
        lam = ps.empty(nn, nn, nn, dtype=dtype)
        g.manual_seed(3)
        lam.copy_((1 + 0.5 * torch.rand((nn, nn, nn), generator=g, device="cuda", dtype=torch.float64)).to(tdt))
        Ci = ps.ones(nn, nn, nn, dtype=dtype)
        torch.cuda.synchronize()
        return T, T2, lam, Ci

    results = {}
    launches = 0

    def bench_kernel(label, kernel, arrs, scalars, memopt, words, nn, dtype, nsteps, fp64="ieee"):
        nonlocal launches
        T, T2, lam, Ci = arrs
        bufs = [T, T2]

        def step(i):
            src, dst = bufs[i % 2], bufs[(i + 1) % 2]
            if kernel is ps.kernels.copy3D:
                ps.parallel(kernel, dst, src, Ci, memopt=memopt, sync=False)
            elif kernel is ps.kernels.diffusion3D_step_flux_lam or hasattr(kernel, "jit_launch"):
                ps.parallel(kernel, dst, src, Ci, lam, *scalars, memopt=memopt, sync=False, fp64=fp64)
            else:
                ps.parallel(kernel, dst, src, Ci, 1.0, *scalars, memopt=memopt, sync=False, fp64=fp64)

        secs = time_steps(torch, step, nsteps, a.warmup, barrier, stream)
        secs = max_over_ranks(secs)
        launches += nsteps
        bytes_step = words * nn ** 3 * np.dtype(dtype).itemsize
        t_step = secs / nsteps
        results[label] = {"t_step_ms": t_step * 1e3, "T_eff_GBs": bytes_step / t_step / 1e9,
                          "A_eff_GB": bytes_step / 1e9}
        return t_step, bytes_step

    def bench_run(label, kernel, arrs, scalars, words, nn, dtype, nsteps, fp64):
        """K steps of the time loop through one ps_diffusion3d_run call (T, T2 swapped inside)."""
        nonlocal launches
        T, T2, lam, Ci = arrs
        arg = lam if kernel is ps.kernels.diffusion3D_step_flux_lam else 1.0
        ps.kernels.run(kernel, T, T2, Ci, arg, *scalars, a.warmup, fp64=fp64, sync=False)
        torch.cuda.synchronize()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ps.kernels.run(kernel, T, T2, Ci, arg, *scalars, nsteps, fp64=fp64, sync=False)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        secs = max_over_ranks(e0.elapsed_time(e1) / 1e3)
        launches += nsteps + (3 if fp64 != "ieee" else 0)
        bytes_step = words * nn ** 3 * np.dtype(dtype).itemsize
        t_step = secs / nsteps
        results[label] = {"t_step_ms": t_step * 1e3, "T_eff_GBs": bytes_step / t_step / 1e9,
                          "A_eff_GB": bytes_step / 1e9}
        return t_step, bytes_step

    def run_errors(arrs, scalars, nt):
        """Relative max-norm error of each multi-step FP64 mode after nt steps against the IEEE run
        (bit-identical to the reference's statements) from the same initial state."""
        T, T2, lam, Ci = arrs
        T0 = T.clone()
        ps.kernels.run(ps.kernels.diffusion3D_step_flux_lam, T, T2, Ci, lam, *scalars, nt, fp64="ieee")
        ref = T.clone()
        errs = {}
        for mode in ("split", "split_state", "split_grid"):
            T.copy_(T0)
            T2.copy_(T0)
            ps.kernels.run(ps.kernels.diffusion3D_step_flux_lam, T, T2, Ci, lam, *scalars, nt, fp64=mode)
            errs[mode] = float((T - ref).abs().max() / ref.abs().max())
        T.copy_(T0)
        T2.copy_(T0)
        del T0, ref
        torch.cuda.synchronize()
        return errs

    peak, peak_kind = measured_peaks()
    with ClockSampler(local) as clk:
        arrs64 = fields(np.float64, n)
        t_head, b_head = bench_run("diffusion3d_flux_lam_f64_split_grid_run", ps.kernels.diffusion3D_step_flux_lam,
                                   arrs64, (dt, _dx, _dx, _dx), WORDS_FLUX_LAM, n, np.float64, a.steps, "split_grid")
        bench_run("diffusion3d_flux_lam_f64_split_run", ps.kernels.diffusion3D_step_flux_lam, arrs64,
                  (dt, _dx, _dx, _dx), WORDS_FLUX_LAM, n, np.float64, a.steps, "split")
        bench_run("diffusion3d_flux_lam_f64_split_state_run", ps.kernels.diffusion3D_step_flux_lam, arrs64,
                  (dt, _dx, _dx, _dx), WORDS_FLUX_LAM, n, np.float64, a.steps, "split_state")
        # the multi-step modes against the IEEE run at the timed step count and at the workload's 50
        run_err = {}
        for nt_err in sorted({a.steps, NT_JOB}):
            run_err[str(nt_err)] = run_errors(arrs64, (dt, _dx, _dx, _dx), nt_err)
            launches += 4 * nt_err
        bench_kernel("diffusion3d_flux_lam_f64_split_memopt_step", ps.kernels.diffusion3D_step_flux_lam, arrs64,
                     (dt, _dx, _dx, _dx), True, WORDS_FLUX_LAM, n, np.float64, a.steps, fp64="split")
        # accuracy of the split-FP32 arithmetic: one step against the bit-exact IEEE kernel
        T, T2, lam, Ci = arrs64
        ref = torch.empty_like(T2)
        ps.parallel(ps.kernels.diffusion3D_step_flux_lam, T2, T, Ci, lam, dt, _dx, _dx, _dx, memopt=True,
                    fp64="ieee")
        ref.copy_(T2)
        ps.parallel(ps.kernels.diffusion3D_step_flux_lam, T2, T, Ci, lam, dt, _dx, _dx, _dx, memopt=True,
                    fp64="split")
        split_err = float((T2 - ref).abs().max() / ref.abs().max())
        del ref
        launches += 2
        # e2e: diffusion jobs (NT_JOB steps each) through the C ABI from pinned host buffers: every
        # job copies its inputs T, Ci, lam host -> device, runs NT_JOB steps (T2 <- T on the device:
        # the run reads only T's boundary values from it) and copies T device -> host, all inside
        # the timed region. The runs go back to back on one compute stream; the copies run on a
        # host-to-device and a device-to-host stream, ordered by events, and jobs alternate between
        # two device buffer sets, so one job's copies overlap the neighbouring jobs' runs.
        lib = _lib.load()
        T, T2, lam, Ci = arrs64
        sets = [(T, T2, Ci, lam), tuple(ps.empty(n, n, n) for _ in range(4))]
        hostbufs = [torch.empty((n, n, n), dtype=torch.float64, pin_memory=True) for _ in range(5)]
        hT, hCi, hlam, hout0, hout1 = hostbufs
        hT.copy_(T.cpu().permute(2, 1, 0))  # column-major device layout == C order of (nz, ny, nx)
        hCi.fill_(1.0)
        hlam.copy_(lam.cpu().permute(2, 1, 0))
        hout = (hout0, hout1)
        s_h2d, s_run, s_d2h = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
        cfg = _lib.PSLaunch()
        cfg.memopt = 1
        cfg.fp64_mode = 3  # state on the fixed grid, as the headline
        P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731

        # where a job's time goes: CUDA events around its copies and its run, on their streams
        phases = {"h2d": [], "d2h": [], "run": []}

        def timed(kind, stream, fn):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            phases[kind].append((e0, e1))
            return e1

        def jobs_run(jobs):
            d2h_done = {}
            for j in range(jobs):
                k = j % 2
                dT, dT2, dCi, dlam = (descriptor(x) for x in sets[k])
                if j >= 2:
                    s_h2d.wait_event(d2h_done[j - 2])  # the set's previous job has been read out

                def copies(dT=dT, dCi=dCi, dlam=dlam):
                    for d, h in ((dT, hT), (dCi, hCi), (dlam, hlam)):
                        _lib.check(lib.ps_copy_h2d_async(d, P(h), stream_handle(s_h2d)))
                h2d_done = timed("h2d", s_h2d, copies)
                s_run.wait_event(h2d_done)
                sr = stream_handle(s_run)
                _lib.check(lib.ps_copy_d2d_async(dT2, dT, sr))
                run_done = timed("run", s_run, lambda: _lib.check(lib.ps_diffusion3d_run(
                    3, dT, dT2, dCi, dlam, 0.0, dt, _dx, _dx, _dx, NT_JOB, ctypes.byref(cfg), sr)))
                s_d2h.wait_event(run_done)
                d2h_done[j] = timed("d2h", s_d2h,
                                    lambda: _lib.check(lib.ps_copy_d2h_async(P(hout[k]), dT, stream_handle(s_d2h))))
            for st_ in (s_h2d, s_run, s_d2h):
                st_.synchronize()

        torch.cuda.synchronize()
        jobs_run(1)  # warm-up, and one job alone: its latency (median of 3, with its phases)
        barrier()
        alone, alone_phases = [], []
        for _ in range(3):
            for v in phases.values():
                v.clear()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            jobs_run(1)
            alone.append(time.perf_counter() - t0)
            alone_phases.append({kind: round(phases[kind][0][0].elapsed_time(phases[kind][0][1]), 3)
                                 for kind in ("h2d", "run", "d2h")})
        t_job1 = float(np.median(alone))
        jobs = max(1, a.e2e_jobs)
        # three pipelined batches of `jobs` jobs; the median batch is the value (the host link's
        # bandwidth on a shared box has dropped ~10x for some tens of ms at a time), all three reported
        batches = []
        for _ in range(3):
            torch.cuda.synchronize()
            for v in phases.values():
                v.clear()
            t0 = time.perf_counter()
            jobs_run(jobs)
            tb = (time.perf_counter() - t0) / jobs
            ph = {f"{kind}_ms_median": round(float(np.median([e0.elapsed_time(e1) for e0, e1 in phases[kind]])), 3)
                  for kind in ("h2d", "d2h", "run")}
            ph["h2d_ms_max"] = round(float(max(e0.elapsed_time(e1) for e0, e1 in phases["h2d"])), 3)
            run_ms = sorted(e0.elapsed_time(e1) for e0, e1 in phases["run"])
            ph["run_ms_max"] = round(float(run_ms[-1]), 3)
            batches.append((tb, ph))
        batches.sort(key=lambda b: b[0])
        t_e2e = max_over_ranks(batches[1][0])
        e2e_phases = batches[1][1]
        e2e_batches_s = [round(b[0], 5) for b in batches]
        launches += (3 * jobs + 4) * NT_JOB
        del hostbufs, hT, hCi, hlam, hout, sets
        # the other 512^3 FP64 variants run after the e2e jobs, so that --quick measures the jobs in the
        # same state of the process as the full run
        if not a.quick:
            ieee_steps = max(3, a.steps // 10)
            bench_kernel("diffusion3d_flux_lam_f64_ieee_memopt", ps.kernels.diffusion3D_step_flux_lam, arrs64,
                         (dt, _dx, _dx, _dx), True, WORDS_FLUX_LAM, n, np.float64, ieee_steps)
            bench_kernel("diffusion3d_flux_lam_f64_ieee_plain", ps.kernels.diffusion3D_step_flux_lam, arrs64,
                         (dt, _dx, _dx, _dx), False, WORDS_FLUX_LAM, n, np.float64, ieee_steps)
            bench_kernel("diffusion3d_readme_f64_split_memopt", ps.kernels.diffusion3D_step, arrs64, (dt, dx, dx, dx),
                         True, WORDS_README, n, np.float64, a.steps, fp64="split")
            bench_kernel("diffusion3d_readme_f64_ieee_memopt", ps.kernels.diffusion3D_step, arrs64, (dt, dx, dx, dx),
                         True, WORDS_README, n, np.float64, ieee_steps)
            bench_kernel("memcopy3d_f64", ps.kernels.copy3D, arrs64, (), False, WORDS_MEMCOPY, n, np.float64, a.steps)
            for opt, tag in (("", "jit"), ("inbounds=true ", "jit_inbounds")):  # run-time compiled, IEEE FP64
                bench_kernel(f"diffusion3d_flux_lam_f64_{tag}", ps.parallel_kernel(JIT_FLUX_LAM.format(opt=opt)),
                             arrs64, (dt, _dx, _dx, _dx), False, WORDS_FLUX_LAM, n, np.float64, ieee_steps)
            # the same run-time compiled body with its arithmetic on FP32 pairs (z sweep, default)
            bench_kernel("diffusion3d_flux_lam_f64_jit_split", ps.parallel_kernel(JIT_FLUX_LAM.format(opt="")),
                         arrs64, (dt, _dx, _dx, _dx), None, WORDS_FLUX_LAM, n, np.float64, a.steps, fp64="split")
        if not a.quick:
            del arrs64, T, T2, lam, Ci
            torch.cuda.empty_cache()
            arrs32 = fields(np.float32, n)
            bench_kernel("diffusion3d_flux_lam_f32_memopt", ps.kernels.diffusion3D_step_flux_lam, arrs32,
                         (dt, _dx, _dx, _dx), True, WORDS_FLUX_LAM, n, np.float32, a.steps)
            bench_kernel("diffusion3d_flux_lam_f32_plain", ps.kernels.diffusion3D_step_flux_lam, arrs32,
                         (dt, _dx, _dx, _dx), False, WORDS_FLUX_LAM, n, np.float32, a.steps)
            bench_kernel("memcopy3d_f32", ps.kernels.copy3D, arrs32, (), False, WORDS_MEMCOPY, n, np.float32, a.steps)
            for memopt, tag in ((False, "plain"), (True, "memopt")):
                bench_kernel(f"diffusion3d_flux_lam_f32_jit_{tag}", ps.parallel_kernel(JIT_FLUX_LAM.format(opt="")),
                             arrs32, (dt, _dx, _dx, _dx), memopt, WORDS_FLUX_LAM, n, np.float32, a.steps)
            del arrs32
            torch.cuda.empty_cache()
            n2 = 256
            arrs256 = fields(np.float64, n2)
            bench_kernel("diffusion3d_flux_lam_f64_split_memopt_256", ps.kernels.diffusion3D_step_flux_lam, arrs256,
                         (dt, _dx, _dx, _dx), True, WORDS_FLUX_LAM, n2, np.float64, a.steps, fp64="split")
            bench_kernel("memcopy3d_f64_256", ps.kernels.copy3D, arrs256, (), False, WORDS_MEMCOPY, n2, np.float64,
                         a.steps)
            dx2 = 10.0 / (n2 - 1)
            sc2 = (dx2 * dx2 / 1.5 / 8.1, 1 / dx2, 1 / dx2, 1 / dx2)
            bench_run("diffusion3d_flux_lam_f64_split_grid_run_256", ps.kernels.diffusion3D_step_flux_lam, arrs256,
                      sc2, WORDS_FLUX_LAM, n2, np.float64, a.steps, "split_grid")
            bench_kernel("diffusion3d_flux_lam_f64_ieee_memopt_256", ps.kernels.diffusion3D_step_flux_lam, arrs256,
                         sc2, True, WORDS_FLUX_LAM, n2, np.float64, ieee_steps)
            bench_kernel("diffusion3d_flux_lam_f64_ieee_plain_256", ps.kernels.diffusion3D_step_flux_lam, arrs256,
                         sc2, False, WORDS_FLUX_LAM, n2, np.float64, ieee_steps)
            # FP32 fields: error after 50 steps against the IEEE FP64 run (bit-identical to the oracle)
            # from the same initial state
            T, T2, lam, Ci = fields(np.float64, n2)
            ps.kernels.run(ps.kernels.diffusion3D_step_flux_lam, T, T2, Ci, lam, *sc2, 50, fp64="ieee")
            ref = T.clone()
            del T, T2, lam, Ci
            arrs256_32 = fields(np.float32, n2)
            T, T2, lam, Ci = arrs256_32
            ps.kernels.run(ps.kernels.diffusion3D_step_flux_lam, T, T2, Ci, lam, *sc2, 50)
            fp32_err = float((T.double() - ref).abs().max() / ref.abs().max())
            launches += 100
            del ref
            arrs256_32 = fields(np.float32, n2)
            bench_kernel("diffusion3d_flux_lam_f32_memopt_256", ps.kernels.diffusion3D_step_flux_lam, arrs256_32,
                         sc2, True, WORDS_FLUX_LAM, n2, np.float32, a.steps)
            bench_kernel("diffusion3d_flux_lam_f32_plain_256", ps.kernels.diffusion3D_step_flux_lam, arrs256_32,
                         sc2, False, WORDS_FLUX_LAM, n2, np.float32, a.steps)
            bench_kernel("memcopy3d_f32_256", ps.kernels.copy3D, arrs256_32, (), False, WORDS_MEMCOPY, n2, np.float32,
                         a.steps)
            results["fp32_rel_err_vs_fp64_50_steps_256"] = fp32_err
            del arrs256, arrs256_32
        if not a.quick:
            gemm = bench_gemm(torch)
            results["nn_gemm_bf16_8192"] = gemm
            launches += gemm["launches"]
        stokes = None if a.quick else bench_stokes2d(ps, torch)
        if stokes:
            launches += stokes.pop("launches")
        warm = None if a.quick else bench_warm_start(a.warm_seeds)
        if warm:
            for r in (warm["fp64"], warm["mixed"]):
                launches += int(r["seeds"] * (r["iters_zero_mean"] + r["iters_warm_mean"]))
        adj = None if a.quick else bench_adjoint(ps, torch)
        if adj:
            launches += adj.pop("launches")
        mini = None if a.quick else bench_miniapps(ps, torch, peak)
        if mini:
            launches += mini.pop("launches")
        s3solve = None if a.quick else bench_stokes3d_solve(ps)
        if s3solve:
            launches += s3solve.pop("launches")
        fdm = None if a.quick else bench_fd_macros(ps, torch)
        if fdm:
            launches += fdm.pop("launches")
        hide = None if a.quick else bench_hide_communication(ps, torch)
        if hide:
            launches += hide.pop("launches")
        sweep2d = None if a.quick else bench_sweep_2d(ps, torch)
        if sweep2d:
            launches += sweep2d.pop("launches")
        adg = None if a.quick else bench_ad(ps, torch)
        if adg:
            launches += adg.pop("launches")
    clocks = clk.summary()

    value = job_value(world, b_head, t_head) / 1e9
    e2e_bytes = NT_JOB * b_head
    out = {
        "metric": "T_eff", "value": round(value, 2), "unit": "GB/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": round(t_head * 1e3, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded U(0,1) T, 1+0.5U(0,1) lam, Ci=1)",
        "config": {"workload": f"diffusion3D flux form with lam array, memopt z-sweep, {n}^3 FP64 fields",
                   "arithmetic": "FP64 fields; run state on a fixed power-of-two grid as FP32 pairs (integer-valued "
                                 "high part <= 2^23 grid units + low part), exact differences; rounding <= "
                                 "1.5*2^-47 of max|T| per step (measured error vs the IEEE run below)",
                   "global_batch": world * n ** 3, "cells_per_gpu": n ** 3, "parallelism": f"replicas{world}",
                   "l2": "inputs 4.3 GB >> 129 MB L2 (no flush needed)"},
        "pct_of_hbm_peak": round(100 * (value / world) / peak, 2),
        "err_vs_ieee_fp64_one_step": split_err,
        "err_vs_ieee_fp64_run": {"by_steps": run_err, "timed_steps": a.steps,
                                 "headline_mode": "split_grid", "tolerance": 1e-12},
        "roofline": {"bound": "hbm", "achieved": round(b_head / t_head / 1e9, 2), "peak": peak, "unit": "GB/s",
                     "frac": round((b_head / t_head / 1e9) / peak, 4), "peak_kind": f"{peak_kind} hbm_gbs (burst)",
                     "traffic": ncu_traffic("diffusion3d_grid_flux_lam_f64_512"),
                     "kernel": "diff3d_grid_tma<LAM,ISO>", "algorithmic_bytes_per_launch": b_head},
        "e2e": {"value": round(job_value(world, e2e_bytes, t_e2e) / 1e9, 2), "unit": "GB/s",
                # an e2e step is one job of NT_JOB diffusion steps: the byte counts are per job
                "h2d_bytes_per_step": 3 * n ** 3 * 8, "d2h_bytes_per_step": n ** 3 * 8,
                "e2e_step": f"one {NT_JOB}-step diffusion job", "steps_per_job": NT_JOB,
                "h2d_bytes_per_job": 3 * n ** 3 * 8, "d2h_bytes_per_job": n ** 3 * 8,
                "step": f"one {NT_JOB}-step diffusion job through the C ABI: T, Ci, lam host -> device from pinned "
                        f"buffers, {NT_JOB} steps, T device -> host; batches of {max(1, a.e2e_jobs)} jobs, runs "
                        f"back to back on one stream, copies on a host-to-device and a device-to-host stream (events "
                        f"order them; two device buffer sets); the median of three batches",
                "amortised": f"the copies are paid once per {NT_JOB}-step job and the run's setup once per job "
                             f"(the device-timed value pays its setup once per {a.steps} steps); pipelined jobs "
                             f"hide one job's copies behind the other job's steps, so this value can exceed the "
                             f"device-timed one. one_job_alone_GBs is the same job with nothing overlapped",
                "seconds_per_job": round(t_e2e, 5), "seconds_one_job_alone": round(t_job1, 5),
                "one_job_alone_GBs": round(e2e_bytes / t_job1 / 1e9, 2), "phases": e2e_phases,
                "one_job_alone_s": [round(x, 5) for x in alone], "one_job_alone_phases_ms": alone_phases,
                "seconds_per_job_batches": e2e_batches_s},
        "gpu_launches": launches,
        "stokes2d_time_to_tol": stokes,
        "warm_start_time_to_tol": warm,
        "adjoint_gradient": adj,
        "miniapps": mini,
        "stokes3d_time_to_tol": s3solve,
        "fd_macros_512": fdm,
        "hide_communication_512": hide,
        "memopt_2d_8192": sweep2d,
        "ad_kernels_256": adg,
        "clocks": clocks,
        "variants": results,
    }
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(a, n)
        if not a.quick:
            out["cpu_baseline"]["miniapps"] = cpu_miniapps()
    if rank == 0:
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def bench_stokes2d(ps, torch, n=1023, tol=1e-8):
    """The Stokes2D PT workload: wall time to max(mean|Rx|, mean|Ry|, mean|divV|) < tol for the FP64
    PT solver and the FP32 PT + FP64 defect-correction solver on 1023^2 cells, unit box, one
    inclusion r = 0.1 with viscosity ratio 1e-3, rho*g = 1 inside, free slip. At that contrast the
    miniapp's damped iteration diverges, so the solves use the accelerated PT iteration with
    pseudo-time steps from @maxloc(Mus) (ps_stokes2d_apt_solve; FP64 residual checked every nout
    iterations). The miniapp's own iteration is timed beside it at its viscosity ratio 0.1."""
    from ps_gb300.stokes import Stokes2D, Stokes2DAPT, Stokes2DAPTParams, Stokes2DParams, inclusion_setup

    Mus, Rog = inclusion_setup(n, n, 1.0, 1.0, musi=1e-3, radius=0.1)
    out = {"config": f"{n}x{n} cells, unit box, inclusion r=0.1, viscosity ratio 1e-3, rho*g=1 inside, "
                     f"free slip, FP64 residual max(mean|Rx|, mean|Ry|, mean|divV|) < {tol}",
           "scheme": "accelerated PT (stresses relaxed in pseudo-time), pseudo-time steps from @maxloc(Mus), "
                     "Re = 16 pi, r = 1, CFL 0.9/sqrt(2)"}
    iters = 0
    for name, mode in (("fp64", 0), ("mixed", 1)):
        g = Stokes2DAPT(Stokes2DAPTParams(n, n, 1.0, 1.0), Mus, Rog)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = g.solve(tol=tol, mode=mode, max_iter=5_000_000, nout=200)
        torch.cuda.synchronize()
        out[name] = {"seconds": round(time.perf_counter() - t0, 4), "iterations": int(st.iters),
                     "outer": int(st.outer), "err": float(st.err), "converged": bool(st.converged)}
        iters += int(st.iters)
        del g
    out["mixed_over_fp64"] = round(out["mixed"]["seconds"] / out["fp64"]["seconds"], 4)
    Mus, Rog = inclusion_setup(n, n, 1.0, 1.0, musi=0.1)
    m = {"config": f"{n}x{n} cells, unit box, inclusion r=0.1, viscosity ratio 0.1 (the miniapp's ratio; at "
                   f"1e-3 its damped iteration diverges), the miniapp's iteration (Stokes2D.jl:11-55)"}
    for name, mode in (("fp64", 0), ("mixed", 1)):
        g = Stokes2D(Stokes2DParams(n, n, 1.0, 1.0), Mus, Rog)
        g.compute_timesteps()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = g.solve(tol=tol, mode=mode, max_iter=5_000_000)
        torch.cuda.synchronize()
        m[name] = {"seconds": round(time.perf_counter() - t0, 4), "iterations": int(st.iters),
                   "outer": int(st.outer), "err": float(st.err), "converged": bool(st.converged)}
        iters += int(st.iters)
        del g
    m["mixed_over_fp64"] = round(m["mixed"]["seconds"] / m["fp64"]["seconds"], 4)
    out["miniapp_iteration_ratio_0.1"] = m
    out["launches"] = 2 * iters
    return out


def bench_gemm(torch, n=8192, reps=5):
    """The warm start's tcgen05 BF16 GEMM (C = A B^T, FP32 accumulation) on an n^3 problem, against
    the measured dense bf16 peak (burst): 2 n^3 flops per call, CUDA events around each call."""
    from ps_gb300 import nn

    g = torch.Generator(device="cuda").manual_seed(0)
    A = torch.randn(n, n, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(n, n, device="cuda", generator=g).to(torch.bfloat16)
    C = torch.empty(n, n, device="cuda")
    for _ in range(2):
        nn.gemm_bf16(A, B, C)
    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        nn.gemm_bf16(A, B, C)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    t = min(times)
    tf = 2.0 * n ** 3 / t / 1e12
    peak = None
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            peak = float(json.load(fh)["bf16_tflops"])
    del A, B, C
    torch.cuda.empty_cache()
    return {"shape": f"{n}x{n}x{n}", "ms": round(t * 1e3, 4), "TFLOPs": round(tf, 1),
            "frac_of_measured_bf16_peak": round(tf / peak, 4) if peak else None, "launches": reps + 2}


def bench_warm_start(seeds, n=1023, tol=1e-8):
    """The learned warm start on unseen random setups at 1023^2 (1-5 inclusions): wall time and PT
    iterations to max residual < tol from the zero start and from the network's prediction
    (inference + interpolation inside the warm time), for the FP64 and the mixed-precision solver."""
    from ps_gb300 import warm_start as W

    net = W.load_default()
    out = {"config": f"{seeds} unseen setups at {n}^2, 1-5 inclusions r~U(0.05,0.2), viscosity 10^U(-0.5,0.5), "
                     f"rho*g=+-1, tol {tol}; network trained at 255^2 on PT solutions generated by the library"}
    for mode, name in ((0, "fp64"), (1, "mixed")):
        r = W.evaluate(net, seeds, n=n, tol=tol, mode=mode)
        r.pop("rows")
        out[name] = r
    out["mixed_warm_over_fp64_zero"] = round(out["mixed"]["seconds_warm"] / out["fp64"]["seconds_zero"], 4)
    net.close()
    return out


# the acoustic3D update statements as kernel definitions (the bodies `from_source` recognises)
ACOUSTIC_V = """@parallel function compute_V!(Vx, Vy, Vz, P, dt, ρ, dx, dy, dz)
    @inn(Vx) = @inn(Vx) - dt/ρ*@d_xi(P)/dx
    @inn(Vy) = @inn(Vy) - dt/ρ*@d_yi(P)/dy
    @inn(Vz) = @inn(Vz) - dt/ρ*@d_zi(P)/dz
    return
end"""
ACOUSTIC_P = """@parallel function compute_P!(P, Vx, Vy, Vz, dt, k, dx, dy, dz)
    @all(P) = @all(P) - dt*k*(@d_xa(Vx)/dx + @d_ya(Vy)/dy + @d_za(Vz)/dz)
    return
end"""


def _events(torch, fn, reps):
    """Seconds per call of fn() over `reps` calls (CUDA events on the current stream, after 3 warm-ups)."""
    for _ in range(3):
        fn()
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(reps):
        fn()
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3 / reps


def acoustic_fields(ps, n, dt, seed=3):
    """Vx, Vy, Vz, P of the acoustic3D miniapp at n^3 on a 40^3 box: its Gaussian pressure
    (acoustic3D.jl:39) plus seeded noise of 1e-3 on every array, so that no difference is zero
    (a zero quotient takes a shorter path in the divisions)."""
    h, lx = 40.0 / (n - 1), 40.0
    c = (np.arange(n) * h - 0.5 * lx) ** 2
    P0 = np.exp(-(c[:, None, None] + c[None, :, None] + c[None, None, :]))
    rng = np.random.default_rng(seed)
    P = ps.from_host(np.asfortranarray((P0 + 1e-3 * rng.random((n, n, n))).astype(dt)))
    V = [ps.from_host(np.asfortranarray((1e-3 * rng.standard_normal(sh)).astype(dt)))
         for sh in ((n + 1, n, n), (n, n + 1, n), (n, n, n + 1))]
    return V[0], V[1], V[2], P


def bench_miniapps(ps, torch, peak):
    """T_eff of the miniapp iterations with each miniapp's own A_eff (words per cell per iteration):
    Stokes2D 6 (Stokes2D.jl:128) at 1023^2, Stokes3D 8 (Stokes3D.jl:154) at 127^3 (the miniapp's
    default) and 255^3, acoustic3D 8 (acoustic3D.jl:62) at 255^3 (its default); FP64 IEEE and FP32.
    Fused iterations (one launch for Stokes2D, three for Stokes3D) and the miniapp's own launch
    sequence with a synchronisation after each launch, as `@parallel` does (6 / 10 / 2 launches)."""
    from ps_gb300 import stokes, stokes3d

    out, launches = {}, 0
    for dt, tag in ((np.float64, "f64"), (np.float32, "f32")):
        es = np.dtype(dt).itemsize
        n = 1023
        Mus, Rog = stokes.inclusion_setup(n, n, 1.0, 1.0, musi=0.1, radius=0.1, dtype=dt)
        g = stokes.Stokes2D(stokes.Stokes2DParams(n, n, 1.0, 1.0), Mus, Rog, dtype=dt)
        g.compute_timesteps()
        t = _events(torch, lambda: g.iterate(20), 5) / 20
        t1 = _events(torch, g.step_reference_sequence, 20)
        out[f"stokes2d_{n}_{tag}"] = {"fused_ms": round(t * 1e3, 4), "T_eff_GBs": round(6 * es * n * n / t / 1e9, 1),
                                      "six_kernels_ms": round(t1 * 1e3, 4),
                                      "six_kernels_T_eff_GBs": round(6 * es * n * n / t1 / 1e9, 1)}
        launches += 8 * 20 + 23 * 6
        del g
        for n in (127, 255):
            Mus, Rog = stokes3d.inclusion_setup(n, n, n, dtype=dt)
            g = stokes3d.Stokes3D(stokes3d.Stokes3DParams(n, n, n), Mus, Rog, dtype=dt)
            g.compute_timesteps()
            t = _events(torch, lambda: g.iterate(10), 3) / 10
            t1 = _events(torch, g.step_reference_sequence, 10)
            out[f"stokes3d_{n}_{tag}"] = {"fused_ms": round(t * 1e3, 4),
                                          "T_eff_GBs": round(8 * es * n ** 3 / t / 1e9, 1),
                                          "miniapp_sequence_ms": round(t1 * 1e3, 4),
                                          "miniapp_sequence_T_eff_GBs": round(8 * es * n ** 3 / t1 / 1e9, 1)}
            launches += 6 * 10 * 3 + 13 * 10
            del g
        n = 255
        h = 40.0 / (n - 1)
        Vx, Vy, Vz, P = acoustic_fields(ps, n, dt)
        dts = h / 6.1

        def acoustic_step():
            ps.parallel(ps.kernels.acoustic3D_compute_V, Vx, Vy, Vz, P, dts, 1.0, h, h, h, sync=False)
            ps.parallel(ps.kernels.acoustic3D_compute_P, P, Vx, Vy, Vz, dts, 1.0, h, h, h, sync=False)

        t = _events(torch, acoustic_step, 50)
        out[f"acoustic3d_{n}_{tag}"] = {"ms": round(t * 1e3, 4), "T_eff_GBs": round(8 * es * n ** 3 / t / 1e9, 1)}
        launches += 2 * 53
        # the same step as one kernel (ps_acoustic3d_step), alternating between two state sets
        sets = [[Vx, Vy, Vz, P], [ps.zeros(n + 1, n, n, dtype=dt), ps.zeros(n, n + 1, n, dtype=dt),
                                  ps.zeros(n, n, n + 1, dtype=dt), ps.zeros(n, n, n, dtype=dt)]]
        for fp64 in (("ieee", "split") if dt == np.float64 else ("ieee",)):
            flip = [0]

            def fused_step():
                i = flip[0]
                ps.kernels.acoustic3d_step(*sets[i], *sets[1 - i], dts, 1.0, 1.0, h, h, h, fp64=fp64, sync=False)
                flip[0] = 1 - i

            tf = _events(torch, fused_step, 50)
            key = f"acoustic3d_{n}_{tag}_fused" + ("_split" if fp64 == "split" else "")
            out[key] = {"ms": round(tf * 1e3, 4), "T_eff_GBs": round(8 * es * n ** 3 / tf / 1e9, 1),
                        "frac_of_measured_hbm": round(8 * es * n ** 3 / tf / 1e9 / peak, 3)}
            launches += 53
        del sets
        if dt == np.float64:  # the same two statements run-time compiled, IEEE and split FP64 arithmetic
            kv = ps.parallel_kernel(ACOUSTIC_V)
            kp = ps.parallel_kernel(ACOUSTIC_P)
            for fp64 in ("ieee", "split"):
                def jit_step():
                    ps.parallel(kv, Vx, Vy, Vz, P, dts, 1.0, h, h, h, sync=False, fp64=fp64)
                    ps.parallel(kp, P, Vx, Vy, Vz, dts, 1.0, h, h, h, sync=False, fp64=fp64)

                tj = _events(torch, jit_step, 20)
                out[f"acoustic3d_{n}_{tag}_jit_{fp64}"] = {"ms": round(tj * 1e3, 4),
                                                           "T_eff_GBs": round(8 * es * n ** 3 / tj / 1e9, 1)}
                launches += 2 * 23
        del P, Vx, Vy, Vz
    torch.cuda.empty_cache()
    out["peak_hbm_gbs"] = peak
    out["launches"] = launches
    return out


# statement -> extent of R relative to A (n^3)
FD_STATEMENTS = {"@all(R) = @d_xa(A)": (-1, 0, 0), "@inn(R) = @d2_zi(A)": (0, 0, 0), "@all(R) = @av(A)": (-1, -1, -1),
                 "@all(R) = @harm_xya(A)": (-1, -1, 0), "@inn(R) = @maxloc(A)": (0, 0, 0),
                 "@inn(R) = @av_yzi(A)": (0, 0, 0)}


def bench_fd_macros(ps, torch, n=512):
    """One-statement FiniteDifferences kernels (`@parallel f!(R, A) = (@<sel>(R) = @<op>(A))`) on
    n^3 arrays through ps_fd_apply: T_eff with 2 words per cell (A read, R written), FP64 and FP32,
    and the same statement as a run-time compiled kernel, one point per thread and as a z sweep."""
    out, launches = {}, 0
    for dt, tag in ((np.float64, "f64"), (np.float32, "f32")):
        A = ps.rand(n, n, n, dtype=dt, seed=4)
        es = np.dtype(dt).itemsize
        for stmt, off in FD_STATEMENTS.items():
            R = ps.zeros(*(n + o for o in off), dtype=dt)
            k = ps.fd_kernel(stmt)
            t = _events(torch, lambda: ps.parallel(k, R, A, sync=False), 10)
            j = ps.parallel_kernel(f"@parallel function f!(R, A)\n    {stmt}\n    return\nend")
            tj = _events(torch, lambda: ps.parallel(j, R, A, sync=False, memopt=False), 10)
            tm = _events(torch, lambda: ps.parallel(j, R, A, sync=False, memopt=True), 10)
            out[f"{stmt} {tag}"] = {"ms": round(t * 1e3, 4), "T_eff_GBs": round(2 * es * n ** 3 / t / 1e9, 1),
                                    "jit_ms": round(tj * 1e3, 4), "jit_T_eff_GBs": round(2 * es * n ** 3 / tj / 1e9, 1),
                                    "jit_memopt_T_eff_GBs": round(2 * es * n ** 3 / tm / 1e9, 1)}
            launches += 3 * 13
            if dt == np.float64:  # FP64 arrays, arithmetic on FP32 pairs
                tsp = _events(torch, lambda: ps.parallel(k, R, A, sync=False, fp64="split"), 10)
                out[f"{stmt} {tag}"]["split_T_eff_GBs"] = round(2 * es * n ** 3 / tsp / 1e9, 1)
                launches += 13
            del R
        del A
    torch.cuda.empty_cache()
    out["launches"] = launches
    return out


def bench_ad(ps, torch, n=256):
    """`@parallel ∇` of the flux-lam step (JIT_FLUX_LAM, IEEE) at n^3: the generated reverse kernel
    (∇=(T2->T2̄, T->T̄, lam->lam̄): the primal step, T2̄ taken, T̄ and lam̄ gathered with atomic
    additions) and forward kernel (tangents of T and lam) against the hand-written adjoint step
    (ps_diffusion3d_adjoint_step); FP64, plus the reverse kernel in FP32. Bytes: reverse 8 words per
    cell at least (T, Ci, lam, T2̄ read, T2 written, T2̄ zeroed, T̄ and lam̄ updated), forward 7
    (T, Ci, lam, T̄, lam̄ read; T2, T2̄ written), hand-written adjoint 6."""
    out, launches = {}, 0
    k = ps.parallel_kernel(JIT_FLUX_LAM.format(opt=""))
    h = (n - 1) / 10.0
    for dt, tag in ((np.float64, "f64"), (np.float32, "f32")):
        T = ps.rand(n, n, n, dtype=dt, seed=2)
        lam = ps.rand(n, n, n, dtype=dt, seed=3)
        lam.mul_(0.5).add_(1.0)
        Ci, T2 = ps.ones(n, n, n, dtype=dt), ps.zeros(n, n, n, dtype=dt)
        T2b, Tb, lamb = ps.rand(n, n, n, dtype=dt, seed=4), ps.zeros(n, n, n, dtype=dt), ps.zeros(n, n, n, dtype=dt)
        args = (T2, T, Ci, lam, 1e-4 / h ** 2, h, h, h)
        es = np.dtype(dt).itemsize
        row = {}
        t = _events(torch, lambda: ps.parallel(k, *args, sync=False, grad=((T2, T2b), (T, Tb), (lam, lamb))), 10)
        row["reverse_ms"] = round(t * 1e3, 4)
        row["reverse_GBs_8_words"] = round(8 * es * n ** 3 / t / 1e9, 1)
        launches += 13
        if dt == np.float64:
            t = _events(torch, lambda: ps.parallel(k, *args, sync=False, grad=((T, Tb), (lam, lamb)),
                                                   ad_mode="forward"), 10)
            row["forward_ms"] = round(t * 1e3, 4)
            row["forward_GBs_7_words"] = round(7 * es * n ** 3 / t / 1e9, 1)
            t = _events(torch, lambda: ps.adjoint.adjoint_step(Tb, T2b, T, Ci, lam, lamb, 1e-4 / h ** 2, h, h, h,
                                                               sync=False), 10)
            row["hand_written_adjoint_ms"] = round(t * 1e3, 4)
            row["hand_written_adjoint_GBs_6_words"] = round(6 * es * n ** 3 / t / 1e9, 1)
            launches += 26
        out[tag] = row
        del T, lam, Ci, T2, T2b, Tb, lamb
    torch.cuda.empty_cache()
    out["config"] = (f"{n}^3, flux form with a conductivity array run-time compiled, one point per thread; "
                     "events around 10 launches after 3 warm-up launches")
    out["launches"] = launches
    return out


HEAT2D = """@parallel function heat2d!(T2, T, Ci, lam, dt, _dx, _dy)
    @inn(T2) = @inn(T) + dt*(lam*@inn(Ci)*(@d2_xi(T)*_dx*_dx + @d2_yi(T)*_dy*_dy))
    return
end"""


def bench_sweep_2d(ps, torch, n=8192):
    """A 2-D `@parallel` diffusion step (FiniteDifferences2D, n^2, FP64 and FP32) run-time compiled:
    one point per thread (memopt=false) against the y sweep (memopt=true, src/memopt.jl's loopdim 2);
    T_eff with 3 words per cell (T and Ci read, T2 written)."""
    out = {}
    k = ps.parallel_kernel(HEAT2D)
    for dt, tag in ((np.float64, "f64"), (np.float32, "f32")):
        T = ps.rand(n, n, dtype=dt, seed=5)
        T2, Ci = ps.zeros(n, n, dtype=dt), ps.ones(n, n, dtype=dt)
        h = (n - 1) / 10.0
        args = (T2, T, Ci, 1.0, 1e-4 / h ** 2, h, h)
        b = 3 * np.dtype(dt).itemsize * n * n
        row = {}
        for name, memopt in (("plain", False), ("y_sweep", True)):
            t = _events(torch, lambda: ps.parallel(k, *args, memopt=memopt, sync=False), 20)
            row[f"{name}_ms"] = round(t * 1e3, 4)
            row[f"{name}_T_eff_GBs"] = round(b / t / 1e9, 1)
        out[f"heat2d_{n}_{tag}"] = row
        del T, T2, Ci
    torch.cuda.empty_cache()
    out["launches"] = 2 * 2 * 23
    return out


def bench_hide_communication(ps, torch, n=512, bw=(16, 2, 2)):
    """`@hide_communication bw begin @parallel diffusion3D_step!(...); comm() end` at n^3 FP64
    (memopt; IEEE and fp64="split"). The diffusion kernels run it as one boundary-first launch
    (boundary tiles counted in host-mapped memory, `comm` called as soon as they are done); the
    run-time compiled kernel as the reference's seven launches on two streams. Each is timed
    against the same step in one launch, without (`*_one_launch_ms`) and with a host
    synchronisation per step (`*_one_launch_sync_ms`, what `@parallel` does), with an empty
    `comm` and with a halo payload: the six planes a halo exchange sends (cells 1 and n-2 of each
    axis, 12.6 MB) packed and copied device -> host on a copy stream, inside `comm`. `*_seq_ms` is
    the step followed by the same copies, `payload_ms` the copies alone."""
    T = ps.rand(n, n, n, seed=2)
    T2, Ci = ps.zeros(n, n, n), ps.ones(n, n, n)
    h = (n - 1) / 10.0
    args = (T2, T, Ci, 1.0, 1e-4, h, h, h)
    k = ps.kernels.diffusion3D_step_inv
    cs = torch.cuda.Stream(priority=-1)  # high priority: the packing kernels go ahead of waiting inner tiles
    planes = [(d, i) for d in range(3) for i in (1, n - 2)]
    host = [torch.empty(tuple(m for a, m in enumerate(T2.shape) if a != d), dtype=T2.dtype, pin_memory=True)
            for d, _ in planes]

    def payload():
        with torch.cuda.stream(cs):
            for (d, i), hb in zip(planes, host):
                hb.copy_(T2.select(d, i), non_blocking=True)
        cs.synchronize()

    out = {"boundary_width": list(bw), "payload_bytes": int(sum(hb.numel() for hb in host) * 8)}
    out["payload_ms"] = round(_events(torch, payload, 10) * 1e3, 4)
    launches = 0
    for fp64, tag in (("ieee", ""), ("split", "fp64_split_")):
        one = lambda: ps.parallel(k, *args, memopt=True, sync=False, fp64=fp64)  # noqa: E731
        one_sync = lambda: ps.parallel(k, *args, memopt=True, sync=True, fp64=fp64)  # noqa: E731
        out[tag + "one_launch_ms"] = round(_events(torch, one, 10) * 1e3, 4)
        out[tag + "one_launch_sync_ms"] = round(_events(torch, one_sync, 10) * 1e3, 4)
        out[tag + "split_ms"] = round(_events(torch, lambda: ps.hide_communication(
            bw, k, args, comm=lambda: None, memopt=True, fp64=fp64), 10) * 1e3, 4)
        out[tag + "payload_split_ms"] = round(_events(torch, lambda: ps.hide_communication(
            bw, k, args, comm=payload, memopt=True, fp64=fp64), 10) * 1e3, 4)
        out[tag + "seq_ms"] = round(_events(torch, lambda: (one_sync(), payload()), 10) * 1e3, 4)
        launches += 5 * 13
    b = 3 * 8 * n ** 3
    out["one_launch_T_eff_GBs"] = round(b / out["one_launch_ms"] / 1e6, 1)
    out["split_T_eff_GBs"] = round(b / out["split_ms"] / 1e6, 1)
    # the same step as a run-time compiled kernel (split FP64 arithmetic), one launch and split
    j = ps.parallel_kernel(JIT_DIFF_INV)
    out["jit_fp64_split_one_launch_ms"] = round(_events(torch, lambda: ps.parallel(j, *args, sync=False,
                                                                                   fp64="split"), 5) * 1e3, 4)
    out["jit_fp64_split_one_launch_sync_ms"] = round(_events(torch, lambda: ps.parallel(j, *args, sync=True,
                                                                                        fp64="split"), 5) * 1e3, 4)
    out["jit_fp64_split_split_ms"] = round(_events(torch, lambda: ps.hide_communication(
        bw, j, args, comm=lambda: None, fp64="split"), 5) * 1e3, 4)
    out["jit_fp64_split_payload_split_ms"] = round(_events(torch, lambda: ps.hide_communication(
        bw, j, args, comm=payload, fp64="split"), 5) * 1e3, 4)
    launches += 8 * 8 + 8
    del T, T2, Ci, host
    out["launches"] = launches
    return out


def bench_stokes3d_solve(ps, n=127, tol=1e-6):
    """The Stokes3D miniapp's solve (127^3, its inclusion, ε = 1e-6, Stokes3D.jl:73-84): wall time
    to err < tol for the FP64 PT solver and for FP32 sweeps with FP64 defect correction."""
    from ps_gb300 import stokes3d

    out = {"config": f"{n}^3, the miniapp's setup (lx = 10, inclusion r = 1, viscosity 0.1, rho*g = 1), "
                     f"err = max(mean|Rx|, mean|Ry|, mean|Rz|, mean|divV|) < {tol}, nout 500"}
    for mode, name in ((0, "fp64"), (1, "mixed")):
        Mus, Rog = stokes3d.inclusion_setup(n, n, n)
        g = stokes3d.Stokes3D(stokes3d.Stokes3DParams(n, n, n), Mus, Rog)
        g.compute_timesteps()
        st = g.solve(tol=tol, nout=500, max_iter=400_000, max_seconds=120, mode=mode)
        out[name] = {"seconds": round(st.seconds, 4), "iterations": int(st.iters), "outer": int(st.outer),
                     "err": float(st.err), "converged": bool(st.converged)}
        del g
    out["mixed_over_fp64"] = round(out["mixed"]["seconds"] / out["fp64"]["seconds"], 4)
    out["launches"] = 3 * (out["fp64"]["iterations"] + out["mixed"]["iterations"])
    return out


def bench_adjoint(ps, torch, n=256, nt=200, every=20):
    """The inverse-conductivity gradient: dL/dlam of L = 0.5||T_nt - T_obs||^2 through nt flux-lam
    diffusion steps (n^3 FP64), checkpoints every `every` steps, reverse sweep with the hand-written
    adjoint. lam = exp(0.3 g), g a seeded Gaussian random field (white noise, seed 4, convolved with
    a Gaussian of sigma = 8 cells, unit variance); T_obs = the forward run with lam (1 + 0.05 h), h a
    second field (seed 5); T0 = 1.7 exp(-|x - 5|^2) on [0, 10]^3."""
    from ps_gb300 import adjoint

    def grf(seed):
        gen = torch.Generator(device="cuda").manual_seed(seed)
        w = torch.randn((n, n, n), generator=gen, device="cuda", dtype=torch.float64)
        k = torch.fft.fftfreq(n, device="cuda", dtype=torch.float64)
        kx, ky, kz = torch.meshgrid(k, k, k, indexing="ij")
        filt = torch.exp(-2 * (torch.pi * 8.0) ** 2 * (kx ** 2 + ky ** 2 + kz ** 2))  # Gaussian, sigma 8 cells
        f = torch.fft.ifftn(torch.fft.fftn(w) * filt).real
        return (f - f.mean()) / f.std()

    def dev(t):  # torch (x, y, z) -> column-major device array
        A = ps.empty(n, n, n)
        A.copy_(t)
        return A

    x = torch.linspace(0, 10, n, device="cuda", dtype=torch.float64)
    X, Y, Z = torch.meshgrid(x, x, x, indexing="ij")
    T0 = dev(1.7 * torch.exp(-((X - 5) ** 2 + (Y - 5) ** 2 + (Z - 5) ** 2)))
    del X, Y, Z
    lam = dev(torch.exp(0.3 * grf(4)))
    lam_obs = dev(torch.exp(0.3 * grf(4)) * (1 + 0.05 * grf(5)))
    Ci = ps.ones(n, n, n)
    h = ((n - 1) / 10.0,) * 3  # 1/dx
    dt = (10.0 / (n - 1)) ** 2 / float(lam_obs.max()) / 8.1
    torch.cuda.synchronize()
    _, _, T_obs, _ = adjoint.misfit_gradient(T0, T0, Ci, lam_obs, dt, h, nt, return_final=True)
    out = {"config": f"{n}^3 FP64, {nt} flux-lam steps, checkpoint every {every}, lam = exp(0.3 g) (Gaussian random "
                     f"field, sigma 8 cells), T_obs from lam (1 + 0.05 h)", "launches": 0}
    for fp64 in ("ieee", "split", "split_grid"):
        adjoint.misfit_gradient(T0, T_obs, Ci, lam, dt, h, 2 * every, checkpoint_every=every, fp64=fp64)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        loss, g, st = adjoint.misfit_gradient(T0, T_obs, Ci, lam, dt, h, nt, checkpoint_every=every, fp64=fp64)
        torch.cuda.synchronize()
        t_grad = time.perf_counter() - t0
        T, T2 = T0.clone(), T0.clone()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ps.kernels.run(ps.kernels.diffusion3D_step_flux_lam, T, T2, Ci, lam, dt, *h, nt, fp64=fp64, sync=False)
        torch.cuda.synchronize()
        t_fwd = time.perf_counter() - t0
        out[fp64] = {"seconds_gradient": round(t_grad, 4), "seconds_forward": round(t_fwd, 4),
                     "gradient_over_forward": round(t_grad / t_fwd, 3), "loss": loss,
                     "checkpoints": st.checkpoints, "recomputed_steps": st.recomputed_steps,
                     "grad_norm": float(g.norm())}
        if fp64 == "ieee":
            g_ieee = g.clone()
        else:
            out[fp64]["gradient_err_vs_ieee"] = float((g - g_ieee).abs().max() / g_ieee.abs().max())
        # forward and recomputed steps, adjoint steps (split: a pair pass before each; grid: the glam
        # kernel and the adjoint state's step), misfit
        out["launches"] += 2 * nt + st.recomputed_steps + nt * (1 if fp64 == "ieee" else 2) + 2
        del T, T2, g
    del g_ieee
    return out


def _oracle_slab_steps(n, slab, steps, warmup):
    """Time the oracle's flux-lam diffusion step over a z-slab of an n^3 FP64 job; `slab` = 0 times
    the whole n^3 job (every cell counted, as the GPU lines count them)."""
    import oracle

    oracle.build()
    rng2, rng3 = np.random.default_rng(2), np.random.default_rng(3)
    nz = n if slab <= 0 else slab + 2
    shape = (n, n, nz)
    T = np.asfortranarray(rng2.random(shape))
    lam = np.asfortranarray(1 + 0.5 * rng3.random(shape))
    Ci = np.asfortranarray(np.ones(shape))
    T2 = T.copy(order="F")
    dx = 10.0 / (n - 1)
    _dx = 1 / dx
    dt = dx * dx / 1.5 / 8.1
    for _ in range(warmup):
        oracle.diffusion3d_step(3, T2, T, Ci, lam, 0.0, dt, _dx, _dx, _dx)
    t0 = time.perf_counter()
    for _ in range(steps):
        oracle.diffusion3d_step(3, T2, T, Ci, lam, 0.0, dt, _dx, _dx, _dx)
        T, T2 = T2, T
    secs = (time.perf_counter() - t0) / steps
    cells = n * n * (n if slab <= 0 else slab)  # the whole box, or the slab's updated planes
    return WORDS_FLUX_LAM * cells * 8 / secs / 1e9, secs


def cpu_baseline(a, n):
    import oracle

    oracle.build()
    teff, secs = _oracle_slab_steps(n, 0, a.cpu_steps, 1)
    return {"value": round(teff, 3), "unit": "GB/s", "cores": oracle.num_threads(), "kind": "port",
            "sample": f"{a.cpu_steps} steps of the oracle (C/OpenMP, -O3) over the whole {n}^3 FP64 flux-lam "
                      f"job ({secs * 1e3:.1f} ms/step)"}


def cpu_miniapps(iters=10):
    """The oracle's loop bodies of the miniapps timed on the host cores (FP64, the GPU lines' sizes
    and A_eff): Stokes2D 1023^2, Stokes3D 127^3, acoustic3D 255^3; `iters` iterations each after one
    untimed iteration."""
    import oracle

    from ps_gb300 import stokes, stokes3d

    def timed(step):
        step()
        t0 = time.perf_counter()
        for _ in range(iters):
            step()
        return (time.perf_counter() - t0) / iters

    out = {}
    n = 1023
    Mus, Rog = stokes.inclusion_setup(n, n, 1.0, 1.0, musi=0.1, radius=0.1)
    p = stokes.Stokes2DParams(n, n, 1.0, 1.0)
    o = oracle.Stokes2D(n, n, p.dx, p.dy, Mus, Rog)
    o.compute_timesteps()
    t = timed(o.step)
    out[f"stokes2d_{n}_f64"] = {"ms": round(t * 1e3, 3), "T_eff_GBs": round(6 * 8 * n * n / t / 1e9, 2)}
    del o
    n = 127
    Mus, Rog = stokes3d.inclusion_setup(n, n, n)
    p3 = stokes3d.Stokes3DParams(n, n, n)
    o = oracle.Stokes3D(n, n, n, *p3.h, Mus, Rog)
    o.compute_timesteps()
    t = timed(o.step)
    out[f"stokes3d_{n}_f64"] = {"ms": round(t * 1e3, 3), "T_eff_GBs": round(8 * 8 * n ** 3 / t / 1e9, 2)}
    del o
    n = 255
    h = 40.0 / (n - 1)
    P = np.asfortranarray(np.ones((n, n, n)))
    Vx, Vy, Vz = (np.asfortranarray(np.zeros(s)) for s in ((n + 1, n, n), (n, n + 1, n), (n, n, n + 1)))
    dts = h / 6.1

    def acoustic_step():
        oracle.acoustic3d_v(Vx, Vy, Vz, P, dts, 1.0, h, h, h)
        oracle.acoustic3d_p(P, Vx, Vy, Vz, dts, 1.0, h, h, h)

    t = timed(acoustic_step)
    out[f"acoustic3d_{n}_f64"] = {"ms": round(t * 1e3, 3), "T_eff_GBs": round(8 * 8 * n ** 3 / t / 1e9, 2)}
    out["cores"] = oracle.num_threads()
    out["sample"] = f"{iters} iterations of each miniapp's loop body (C/OpenMP oracle, FP64)"
    return out


def run_reference(a, world, rank):
    """CPU oracle of the reference's Threads-backend kernel, timed on the host cores."""
    if rank != 0:
        return
    import oracle

    oracle.build()
    slab = a.ref_slab
    teff, secs = _oracle_slab_steps(a.n, slab, a.steps, a.warmup)
    what = (f"one diffusion step of the whole {a.n}^3 job" if slab <= 0 else
            f"one diffusion step over a {a.n}x{a.n}x{slab} z-slab of the {a.n}^3 job")
    out = {
        "metric": "T_eff", "value": round(teff, 3), "unit": "GB/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": round(secs * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded U(0,1) T, 1+0.5U(0,1) lam, Ci=1)",
        "impl": "reference",
        "config": {"workload": f"diffusion3D flux form with lam array, {a.n}^3 FP64 (CPU"
                               f"{'' if slab <= 0 else ', z-slab sample'})",
                   "global_batch": a.n ** 3, "parallelism": "host threads"},
        "cpu_baseline": {"value": round(teff, 3), "unit": "GB/s", "cores": oracle.num_threads(), "kind": "port",
                         "sample": f"each step: {what} (C/OpenMP restatement of the reference kernel)"},
        "e2e": {"value": round(teff, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def only_run(a):
    """A short run of the headline workload (for ncu captures of one kernel)."""
    import torch

    import ps_gb300 as ps

    ps.init_parallel_stencil(ps.GB300, "Float64", 3)
    n = a.n
    if a.only_run == "gemm":  # the warm start's tcgen05 GEMM on an n^3 bf16 problem, --steps calls
        from ps_gb300 import nn

        g = torch.Generator(device="cuda").manual_seed(0)
        A = torch.randn(n, n, device="cuda", generator=g).to(torch.bfloat16)
        B = torch.randn(n, n, device="cuda", generator=g).to(torch.bfloat16)
        C = torch.empty(n, n, device="cuda")
        for _ in range(a.steps):
            nn.gemm_bf16(A, B, C)
        torch.cuda.synchronize()
        print(json.dumps({"only_run": "gemm", "n": n, "steps": a.steps}))
        return
    if a.only_run in ("fd", "fd32"):  # the FD-macro kernel of one statement, FP64 / FP32, n^3, --steps calls
        dt = np.float32 if a.only_run == "fd32" else np.float64
        A, R = ps.rand(n, n, n, dtype=dt, seed=4), ps.zeros(n, n, n, dtype=dt)
        k = ps.fd_kernel("@inn(R) = @d2_zi(A)")
        for _ in range(a.steps):
            ps.parallel(k, R, A, sync=False)
        torch.cuda.synchronize()
        print(json.dumps({"only_run": a.only_run, "n": n, "steps": a.steps}))
        return
    if a.only_run == "adjoint_grid":  # the misfit gradient on fixed grids, n^3, --steps steps, 2 segments
        from ps_gb300 import adjoint

        x = torch.linspace(0, 10, n, device="cuda", dtype=torch.float64)
        T0 = ps.empty(n, n, n)
        T0.copy_(1.7 * torch.exp(-((x[:, None, None] - 5) ** 2 + (x[None, :, None] - 5) ** 2 +
                                   (x[None, None, :] - 5) ** 2)))
        lam = ps.fill(1.2, n, n, n)
        Ci = ps.ones(n, n, n)
        h = ((n - 1) / 10.0,) * 3
        dt = (10.0 / (n - 1)) ** 2 / 1.2 / 8.1
        T_obs = ps.empty(n, n, n)
        T_obs.copy_(T0 * 0.9)
        adjoint.misfit_gradient(T0, T_obs, Ci, lam, dt, h, a.steps, checkpoint_every=max(1, a.steps // 2),
                                fp64="split_grid")
        torch.cuda.synchronize()
        print(json.dumps({"only_run": a.only_run, "n": n, "steps": a.steps}))
        return
    if a.only_run in ("stokes2d_apt", "stokes2d_apt32"):  # --steps accelerated PT iterations, n^2, ratio 1e-3
        from ps_gb300 import stokes

        Mus, Rog = stokes.inclusion_setup(n, n, 1.0, 1.0, musi=1e-3, radius=0.1)
        g = stokes.Stokes2DAPT(stokes.Stokes2DAPTParams(n, n, 1.0, 1.0), Mus, Rog,
                               dtype=np.float32 if a.only_run.endswith("32") else np.float64)
        g.coefficients()
        g.iterate(a.steps)
        torch.cuda.synchronize()
        print(json.dumps({"only_run": a.only_run, "n": n, "steps": a.steps}))
        return
    if a.only_run in ("stokes2d", "stokes2d32", "stokes3d", "stokes3d_fused32", "acoustic3d", "memcopy", "adjoint",
                      "acoustic3d_fused", "acoustic3d_fused32", "acoustic3d_fused_split"):  # --steps calls, size --n
        from ps_gb300 import adjoint, stokes, stokes3d

        if a.only_run in ("stokes2d", "stokes2d32"):  # fused PT iterations, FP64 / FP32, n^2
            dtp = np.float32 if a.only_run.endswith("32") else np.float64
            Mus, Rog = stokes.inclusion_setup(n, n, 1.0, 1.0, musi=0.1, radius=0.1, dtype=dtp)
            g = stokes.Stokes2D(stokes.Stokes2DParams(n, n, 1.0, 1.0), Mus, Rog, dtype=dtp)
            g.compute_timesteps()
            g.iterate(a.steps)
        elif a.only_run in ("stokes3d", "stokes3d_fused32"):  # PT iterations, FP64 three launches / FP32 one
            dtp = np.float32 if a.only_run.endswith("32") else np.float64
            Mus, Rog = stokes3d.inclusion_setup(n, n, n, dtype=dtp)
            g = stokes3d.Stokes3D(stokes3d.Stokes3DParams(n, n, n), Mus, Rog, dtype=dtp)
            g.compute_timesteps()
            g.iterate(a.steps, one_launch=a.only_run.endswith("32"))
        elif a.only_run == "acoustic3d":
            h = 40.0 / (n - 1)
            P = ps.ones(n, n, n)
            Vx, Vy, Vz = ps.zeros(n + 1, n, n), ps.zeros(n, n + 1, n), ps.zeros(n, n, n + 1)
            for _ in range(a.steps):
                ps.parallel(ps.kernels.acoustic3D_compute_V, Vx, Vy, Vz, P, h / 6.1, 1.0, h, h, h, sync=False)
                ps.parallel(ps.kernels.acoustic3D_compute_P, P, Vx, Vy, Vz, h / 6.1, 1.0, h, h, h, sync=False)
        elif a.only_run.startswith("acoustic3d_fused"):  # the one-kernel step, ping-pong between two sets
            dtp = np.float32 if a.only_run.endswith("32") else np.float64
            fp64 = "split" if a.only_run.endswith("split") else "ieee"
            h = 40.0 / (n - 1)
            sets = [list(acoustic_fields(ps, n, dtp, seed=3 + i)) for i in range(2)]
            for it in range(a.steps):
                ps.kernels.acoustic3d_step(*sets[it % 2], *sets[1 - it % 2], h / 6.1, 1.0, 1.0, h, h, h, fp64=fp64,
                                           sync=False)
        elif a.only_run == "memcopy":
            T, Ci, T2 = ps.ones(n, n, n), ps.ones(n, n, n), ps.zeros(n, n, n)
            for _ in range(a.steps):
                ps.parallel(ps.kernels.copy3D, T2, T, Ci, sync=False)
        else:  # one adjoint step of the flux-lam diffusion step, FP64, n^3
            T, Ci, lam = ps.ones(n, n, n), ps.ones(n, n, n), ps.fill(1.5, n, n, n)
            lt, lt2, gl = ps.zeros(n, n, n), ps.ones(n, n, n), ps.zeros(n, n, n)
            for _ in range(a.steps):
                adjoint.adjoint_step(lt, lt2, T, Ci, lam, gl, 1e-4, 1.0, 1.0, 1.0, sync=False)
        torch.cuda.synchronize()
        print(json.dumps({"only_run": a.only_run, "n": n, "steps": a.steps}))
        return
    if a.only_run in ("ad", "ad32"):  # the generated reverse kernel of the flux-lam body, n^3, --steps launches
        dt_np = np.float32 if a.only_run == "ad32" else np.float64
        k = ps.parallel_kernel(JIT_FLUX_LAM.format(opt=""))
        T, lam = ps.rand(n, n, n, dtype=dt_np, seed=2), ps.rand(n, n, n, dtype=dt_np, seed=3)
        lam.mul_(0.5).add_(1.0)
        Ci, T2 = ps.ones(n, n, n, dtype=dt_np), ps.zeros(n, n, n, dtype=dt_np)
        T2b, Tb, lamb = ps.rand(n, n, n, dtype=dt_np, seed=4), ps.zeros(n, n, n, dtype=dt_np), ps.zeros(n, n, n, dtype=dt_np)
        h = (n - 1) / 10.0
        for _ in range(a.steps):
            ps.parallel(k, T2, T, Ci, lam, 1e-4 / h ** 2, h, h, h, sync=False, grad=((T2, T2b), (T, Tb), (lam, lamb)))
        torch.cuda.synchronize()
        print(json.dumps({"only_run": a.only_run, "n": n, "steps": a.steps}))
        return
    if a.only_run == "hide":  # the @hide_communication measurement alone, at --n
        print(json.dumps(bench_hide_communication(ps, torch, n=n)))
        return
    if a.only_run == "miniapps":  # the miniapp measurement alone
        print(json.dumps(bench_miniapps(ps, torch, json.load(open("MEASURED_PEAKS.json"))["hbm_gbs"]
                                        if os.path.exists("MEASURED_PEAKS.json") else 6782.0)))
        return
    if a.only_run in ("jit", "jit32"):  # the headline body, run-time compiled (IEEE, bounds-checked), --steps steps
        dt_np = np.float32 if a.only_run == "jit32" else np.float64
        tdt = torch.float32 if a.only_run == "jit32" else torch.float64
        k = ps.parallel_kernel(JIT_FLUX_LAM.format(opt=""))
        g = torch.Generator(device="cuda").manual_seed(2)
        T = ps.empty(n, n, n, dtype=dt_np)
        T.copy_(torch.rand((n, n, n), generator=g, device="cuda", dtype=torch.float64).to(tdt))
        T2, lam, Ci = T.clone(), ps.empty(n, n, n, dtype=dt_np), ps.ones(n, n, n, dtype=dt_np)
        lam.copy_((1 + 0.5 * torch.rand((n, n, n), generator=g, device="cuda", dtype=torch.float64)).to(tdt))
        dx = 10.0 / (n - 1)
        stream = torch.cuda.current_stream()
        res = {"only_run": a.only_run, "n": n, "steps": a.steps}
        for memopt in (False, True):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            for i in range(a.steps + 1):
                if i == 1:
                    e0.record(stream)
                src, dst = (T, T2) if i % 2 == 0 else (T2, T)
                ps.parallel(k, dst, src, Ci, lam, dx * dx / 1.5 / 8.1, 1 / dx, 1 / dx, 1 / dx, sync=False,
                            memopt=memopt, loopsize=a.loopsize)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / max(1, a.steps)
            res["memopt" if memopt else "plain"] = {
                "ms_per_step": round(ms, 4),
                "T_eff_GBs": round(WORDS_FLUX_LAM * n ** 3 * np.dtype(dt_np).itemsize / ms / 1e6, 1)}
        print(json.dumps(res))
        return
    g = torch.Generator(device="cuda")
    g.manual_seed(2)
    T = ps.empty(n, n, n)
    T.copy_(torch.rand((n, n, n), generator=g, device="cuda", dtype=torch.float64))
    T2 = ps.empty(n, n, n)
    T2.copy_(T)
    g.manual_seed(3)
    lam = ps.empty(n, n, n)
    lam.copy_(1 + 0.5 * torch.rand((n, n, n), generator=g, device="cuda", dtype=torch.float64))
    Ci = ps.ones(n, n, n)
    dx = 10.0 / (n - 1)
    ps.kernels.run(ps.kernels.diffusion3D_step_flux_lam, T, T2, Ci, lam, dx * dx / 1.5 / 8.1, 1 / dx, 1 / dx, 1 / dx,
                   a.steps, fp64=a.only_run)
    torch.cuda.synchronize()
    print(json.dumps({"only_run": a.only_run, "n": n, "steps": a.steps}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--quick", action="store_true", help="headline + e2e only")
    ap.add_argument("--e2e-jobs", type=int, default=16, help="diffusion jobs of the e2e measurement (pipelined)")
    ap.add_argument("--cpu-steps", type=int, default=5)
    ap.add_argument("--ref-slab", type=int, default=0, help="z planes timed by --impl reference (0: the whole job)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--loopsize", type=int, default=0, help="z indices per thread of memopt run-time compiled kernels")
    ap.add_argument("--warm-seeds", type=int, default=2, help="unseen setups of the warm-start comparison")
    ap.add_argument("--only-run", choices=["ieee", "split", "split_state", "split_grid", "gemm", "jit", "jit32",
                                                 "stokes2d", "stokes2d32", "stokes3d", "acoustic3d", "memcopy", "adjoint",
                                                 "fd", "fd32",
                                                 "stokes2d_apt", "stokes2d_apt32", "adjoint_grid", "acoustic3d_fused",
                                                 "acoustic3d_fused32", "acoustic3d_fused_split", "hide", "miniapps", "stokes3d_fused32",
                                                 "ad", "ad32"],
                    default=None,
                    help="profiling aid: run --steps steps of the headline workload in this fp64 mode (or as a "
                         "run-time compiled kernel: jit; or --steps calls of the tcgen05 GEMM on an --n cubed bf16 "
                         "problem) and exit")
    a = ap.parse_args()
    if a.only_run:
        only_run(a)
        return
    if a.warmup < 3:
        a.warmup = 3
    world, rank, local = dist_setup()
    if a.impl == "reference":
        run_reference(a, world, rank)
        return
    run_ours(a, world, rank, local)


if __name__ == "__main__":
    main()
