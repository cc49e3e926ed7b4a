#!/usr/bin/env python
"""Benchmark: 3D cartesian acoustic forward modelling (the 512^3 workload).

One bench step = one complete forward run of the workload: 512 x 512 x 512
model at 5 m (576^3 with the nb=32 padding), 8th-order Laplacian, nt = 3000
steps of 0.005 us, Gaussian sponge + one-way ABC (dabc=y), one Ricker source
(5 MHz) and a 128 x 128 receiver grid at z = 50 m.  The model is the seeded
layered vacuum / ice (5 dust layers) / basalt model with 2D Gaussian-random
interfaces.

  value : padded cell-updates/s with model, wavelet and trace buffers
          already resident in HBM (awe_forward_device), all ranks
  e2e   : the same metric through awe_set_model + awe_set_geometry +
          awe_forward with pinned host buffers (H2D of the model and
          wavelet, D2H of the traces inside the timed region)

After the headline (rank 0, one GPU) two more legs go on the same line:
  batched_gradient  : FWI gradients of the 256-shot survey, batched against
                      the per-shot loop (the second half of the metric)
  spherical_forward : the spherical-shell configuration's 16-source track
and cpu_baseline.gradient times the FP64 adjoint oracle on one survey shot
and states the engine's gradient error against it.  --no-extras skips them.

--impl reference times the reference CPU implementation of the same update
(the oracle port of ts_kernel.c step_forward_3d, OpenMP over all host cores)
on a bounded sample of time steps of the same padded grid.

Multi-GPU: shots are independent, so N ranks run N replicas (weak scaling,
no collective on the data path); value = all ranks' cell-updates / max time.
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

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s & %HBM peak (3D acoustic)"
UNIT = "cell-updates/s"
BYTES_PER_CELL = 16  # read u_cur, read u_prev, read v^2dt^2, write u_next
# spherical adjoint step: read z_{j+1}, v, A_j, z_{j+2} and the gradient pair
# (8 B); write z_j and the pair
ADJ_BYTES_PER_CELL = 36


def workload(nt=3000, n=512):
    return dict(name="3D cartesian acoustic forward, %d^3 at 5 m (%d^3 padded, nb=32), 8th order, "
                     "nt=%d, dabc=y, 1 Ricker source, 128x128 receivers" % (n, n + 64, nt),
                n=(n, n, n), d=(5.0, 5.0, 5.0), o=(0.0, 0.0, 0.0), nt=nt, dt=0.005, nb=32, fdorder=8,
                dabc=1, f0=5.0, seed=3)


def gaussian_field(rng, shape, corr_cells):
    """Zero-mean unit-std 2D Gaussian random field with a Gaussian
    correlation of length corr_cells (FFT filter)."""
    w = rng.standard_normal(shape)
    ky = np.fft.fftfreq(shape[0])[:, None]
    kx = np.fft.fftfreq(shape[1])[None, :]
    filt = np.exp(-0.5 * (2 * np.pi) ** 2 * (kx ** 2 + ky ** 2) * corr_cells ** 2 / 2.0)
    f = np.real(np.fft.ifft2(np.fft.fft2(w) * filt))
    return (f - f.mean()) / (f.std() + 1e-12)


def layered_model_3d(w):
    """Vacuum 300 m/us down to a Gaussian-random surface (mean 200 m, std 30 m,
    correlation 200 m); ice 168 m/us with 5 dust layers (+-5 %, 10-20 m);
    basalt 110 m/us below a second random interface (mean 1800 m).
    Returns [ny][nx][nz] float32 (axis 1 = z fastest)."""
    rng = np.random.default_rng(w["seed"])
    nz, nx, ny = w["n"]
    dz, dx = w["d"][0], w["d"][1]
    surf = 200.0 + 30.0 * gaussian_field(rng, (ny, nx), 200.0 / dx)
    base = 1800.0 + 30.0 * gaussian_field(rng, (ny, nx), 200.0 / dx)
    z = (np.arange(nz, dtype=np.float32) * dz)[None, None, :]
    vel = np.full((ny, nx, nz), 168.0, np.float32)
    for _ in range(5):
        zd = rng.uniform(400.0, 1600.0)
        th = rng.uniform(10.0, 20.0)
        amp = rng.choice([0.95, 1.05])
        depth = surf + (zd - 200.0)
        band = np.abs(z - depth[:, :, None]) < 0.5 * th
        vel[band] = 168.0 * amp
    vel[z < surf[:, :, None].astype(np.float32)] = 300.0
    vel[z >= base[:, :, None].astype(np.float32)] = 110.0
    return vel


def geometry(w):
    nz, nx, ny = w["n"]
    dx = w["d"][1]
    xc, yc = 0.5 * (nx - 1) * dx, 0.5 * (ny - 1) * dx
    sou = np.array([[xc, yc, 50.0]], np.float32)
    gx = np.linspace(0.05, 0.95, 128) * (nx - 1) * dx
    gy = np.linspace(0.05, 0.95, 128) * (ny - 1) * dx
    X, Y = np.meshgrid(gx, gy, indexing="ij")
    rec = np.stack([X.ravel(), Y.ravel(), np.full(X.size, 50.0)], 1).astype(np.float32)
    return sou, rec


def ricker(nt, dt, f0):
    t = np.arange(nt) * dt - 1.5 / f0
    a = (np.pi * f0 * t) ** 2
    r = (1 - 2 * a) * np.exp(-a)
    return (r / np.abs(r).max()).astype(np.float32)


def padded_cells(w):
    return int(np.prod([n + 2 * w["nb"] for n in w["n"]]))


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) >= 8:
                rows.append(parts)
        if not rows:
            return None
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, name in enumerate(names):
                if r[4 + k].lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": float(rows[0][1]) if rows[0][1].replace(".", "").isdigit() else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# DRAM bytes per cell of one step-kernel launch (k_stepB3_o8, AWE_FAST),
# from the ncu capture of a 384^3-padded launch: 895.2 MB read + written
# over 56.62 M padded cells (profiles/k_stepB3_o8_tma_n320.md).  A full
# 576^3 launch is too large for a capture; DRAM traffic scales with the cells
# a launch processes.
STEP_DRAM_BYTES_PER_CELL = 15.810


def profiled_traffic(cells):
    """DRAM bytes of one step-kernel launch over `cells` padded cells."""
    return STEP_DRAM_BYTES_PER_CELL * cells


def cpu_baseline(w, target_s=10.0):
    """Oracle port of the reference CPU update (OpenMP, all host cores) on
    the padded grid: returns (cell-updates/s, cores, sample description)."""
    from oracle import oracle

    oracle.build(with_reference=False)
    cores = os.cpu_count() or 1
    npad = [n + 2 * w["nb"] for n in w["n"]]
    t1 = oracle.cart3d_steps_seconds(npad[0], npad[1], npad[2], w["fdorder"], 1, cores)
    nsteps = int(max(1, min(20, target_s / max(t1, 1e-3))))
    t = oracle.cart3d_steps_seconds(npad[0], npad[1], npad[2], w["fdorder"], nsteps, cores)
    cells = float(np.prod(npad))
    sample = "%d time steps of the %dx%dx%d padded grid (8th-order update of ts_kernel.c step_forward_3d, %d threads)" % (
        nsteps, npad[0], npad[1], npad[2], cores)
    return cells * nsteps / t, cores, sample, nsteps


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
        return dist, rank, world, local
    return None, rank, world, local


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, x):
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# the reference's own sfAWEFDcart3Dcpu, built from its sources by
# oracle/ref/Makefile.cpu (absent: the oracle port is timed instead)
REF_CPU_PROGRAM = os.path.join(ROOT, "oracle", "_ref", "sfAWEFDcart3Dcpu_ref")


def _time_reference_program(args, w, cores, extra_steps=40):
    """The reference CPU program on the workload: vel, sources and receivers
    as RSF files, run with 2 and with 2 + extra_steps time steps; the wall-time
    difference per step excludes reading the inputs and setting up.  Returns
    (seconds per time step of each timed pair, sample text)."""
    import shutil
    import subprocess
    import tempfile

    from wavefield_imaging_gb300 import rsf

    tmp = tempfile.mkdtemp(dir="/dev/shm" if os.path.isdir("/dev/shm") else None)
    try:
        vel = layered_model_3d(w)
        sou, rec = geometry(w)
        rsf.write(os.path.join(tmp, "vel.rsf"), vel, [(n, o, d) for n, o, d in zip(w["n"], w["o"], w["d"])])
        rsf.write(os.path.join(tmp, "sou.rsf"), sou, [(3, 0.0, 1.0), (sou.shape[0], 0.0, 1.0)])
        rsf.write(os.path.join(tmp, "rec.rsf"), rec, [(3, 0.0, 1.0), (rec.shape[0], 0.0, 1.0)])
        del vel

        def run(nt):
            wpath = os.path.join(tmp, "wav_%d.rsf" % nt)
            if not os.path.exists(wpath):
                rsf.write(wpath, ricker(nt, w["dt"], w["f0"]).reshape(nt, 1), [(1, 0.0, 1.0), (nt, 0.0, w["dt"])])
            cmd = [REF_CPU_PROGRAM, "vel=vel.rsf", "sou=sou.rsf", "rec=rec.rsf", "fdorder=%d" % w["fdorder"],
                   "dabc=y", "free=n", "expl=y", "cden=y", "snap=n", "nb=%d" % w["nb"], "ompnth=%d" % cores,
                   "verb=n"]
            with open(wpath, "rb") as fin, open(os.path.join(tmp, "dat.rsf"), "wb") as fout:
                t0 = time.perf_counter()
                r = subprocess.run(cmd, stdin=fin, stdout=fout, stderr=subprocess.PIPE, cwd=tmp, timeout=600)
                t1 = time.perf_counter()
            if r.returncode != 0:
                raise RuntimeError("reference program failed: %s" % r.stderr.decode()[-300:])
            return t1 - t0

        for _ in range(args.warmup):
            run(2)
        per_step = [(run(2 + extra_steps) - run(2)) / extra_steps for _ in range(args.steps)]
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    sample = ("%d-step difference of the reference's sfAWEFDcart3Dcpu (built from its sources, -O3 -fopenmp, "
              "%d OpenMP threads) on the workload's %dx%dx%d padded grid, runs of 2 and %d steps per timed pair, "
              "input reading and set-up cancelled" % (extra_steps, cores, w["n"][0] + 2 * w["nb"],
                                                      w["n"][1] + 2 * w["nb"], w["n"][2] + 2 * w["nb"],
                                                      2 + extra_steps))
    return per_step, sample


def host_baseline(w):
    """The engine line's host-core baseline: one 2- and 42-step pair of the
    reference's own sfAWEFDcart3Dcpu (about 13 s on 16 Grace cores), else
    the oracle port of its update."""
    from types import SimpleNamespace

    cores = os.cpu_count() or 1
    note = None
    if os.access(REF_CPU_PROGRAM, os.X_OK):
        try:
            per_step, sample = _time_reference_program(SimpleNamespace(steps=1, warmup=0), w, cores)
            cells = float(np.prod([n + 2 * w["nb"] for n in w["n"]]))
            return {"value": cells / per_step[0], "unit": UNIT, "cores": cores, "kind": "reference",
                    "sample": sample}
        except Exception as e:  # noqa: BLE001 - the port is timed instead
            note = "reference program not timed (%s: %s)" % (type(e).__name__, e)
    v, cores, sample, _ = cpu_baseline(w)
    out = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}
    if note:
        out["note"] = note
    return out


def run_reference(args):
    dist, rank, world, local = dist_init()
    if rank != 0:
        return
    w = workload()
    from oracle import oracle

    oracle.build(with_reference=False)
    cores = os.cpu_count() or 1
    if os.access(REF_CPU_PROGRAM, os.X_OK):
        try:
            # a pair costs about two set-ups (2.8 s each on 16 Grace cores) plus
            # the extra steps (0.17 s each): 40 extra steps up to 8 bench steps,
            # 20 beyond, so that --steps 20 still ends within about 3 minutes
            per_step, sample = _time_reference_program(args, w, cores, extra_steps=40 if args.steps <= 8 else 20)
            cells = float(np.prod([n + 2 * w["nb"] for n in w["n"]]))
            value = cells * len(per_step) / sum(per_step)
            out = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
                   "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(per_step) / len(per_step),
                   "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
                   "data": "synthetic", "config": {"workload": w["name"], "sample": sample,
                                                   "ms_per_step": "one time step of the reference program"},
                   "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "reference",
                                    "sample": sample},
                   "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
            print(json.dumps(out))
            return
        except Exception as e:  # noqa: BLE001 - the port is timed instead
            print("reference program not timed (%s); timing the oracle port" % e, file=sys.stderr)
    npad = [n + 2 * w["nb"] for n in w["n"]]
    cells = float(np.prod(npad))
    t1 = oracle.cart3d_steps_seconds(npad[0], npad[1], npad[2], w["fdorder"], 1, cores)
    per_step = int(max(1, min(10, 8.0 / max(t1, 1e-3))))
    for _ in range(args.warmup):
        oracle.cart3d_steps_seconds(npad[0], npad[1], npad[2], w["fdorder"], per_step, cores)
    times = [oracle.cart3d_steps_seconds(npad[0], npad[1], npad[2], w["fdorder"], per_step, cores)
             for _ in range(args.steps)]
    total = sum(times)
    value = cells * per_step * args.steps / total
    sample = "%d time steps per bench step of the %dx%dx%d padded grid (oracle port of ts_kernel.c step_forward_3d, %d OpenMP threads)" % (
        per_step, npad[0], npad[1], npad[2], cores)
    out = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
           "data": "synthetic", "config": {"workload": w["name"], "sample": sample},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def run_ours(args):
    import torch

    import wavefield_imaging_gb300 as awe

    dist, rank, world, local = dist_init()
    torch.cuda.set_device(local)
    w = workload(args.nt, args.n)
    vel = layered_model_3d(w)
    sou, rec = geometry(w)
    if world > 1:  # a survey: every rank models its own source position (shot `rank`)
        sou = sou + np.array([[10.0 * rank, 0.0, 0.0]], np.float32)
    wav = ricker(w["nt"], w["dt"], w["f0"])
    prec = awe.EXACT if args.precision == "exact" else awe.FAST
    desc = awe.make_desc(3, w["n"], w["d"], w["o"], w["nt"], w["dt"], nb=w["nb"], fdorder=w["fdorder"],
                         dabc=w["dabc"], expl=1, precision=prec)
    plan = awe.Plan(desc, device=local)
    plan.set_model(vel)
    plan.set_geometry(sou, rec)
    nr = rec.shape[0]
    d_wav = torch.from_numpy(wav).cuda()
    d_dat = torch.zeros((plan.nsmp, nr), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    cells = padded_cells(w)

    def step():
        plan.forward_device(d_wav.data_ptr(), 1, d_dat.data_ptr(), 0, stream.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    plan.profile(True)
    barrier(dist)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    launches = 0
    for _ in range(args.steps):
        step()
        launches += plan.last_launch_count()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(dist)
    clocks = sampler.stop()
    ms = ev0.elapsed_time(ev1)
    kern_ms, kern_n = plan.profile_read()
    plan.profile(False)
    ms_max = allmax(dist, ms)
    value = cells * w["nt"] * args.steps * world / (ms_max / 1e3)

    # end to end through the public API with pinned host buffers
    h_vel = torch.from_numpy(vel).pin_memory()
    h_wav = torch.from_numpy(wav).pin_memory()
    h_dat = torch.zeros((plan.nsmp, nr), dtype=torch.float32).pin_memory()
    vel_np, wav_np, dat_np = h_vel.numpy(), h_wav.numpy(), h_dat.numpy()

    def e2e_step():
        plan.set_model(vel_np)
        plan.set_geometry(sou, rec)
        lib = awe.lib()
        import ctypes as C
        st = lib.awe_forward(plan.handle, wav_np.ctypes.data_as(C.POINTER(C.c_float)), 1,
                             dat_np.ctypes.data_as(C.POINTER(C.c_float)), None)
        if st != 0:
            raise RuntimeError(lib.awe_last_error().decode())

    e2e_step()
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    t1 = time.perf_counter()
    e2e_s = allmax(dist, t1 - t0)
    e2e_value = cells * w["nt"] * args.steps * world / e2e_s
    check = float(np.abs(dat_np).max())
    sharded = None
    if args.extras and world > 1:
        try:
            sharded = extra_sharded_gradient(dist, rank, world, local)
        except Exception as e:  # noqa: BLE001 - reported in the JSON line
            sharded = {"error": "%s: %s" % (type(e).__name__, e)}

    if rank != 0:
        return
    peak, peak_kind = measured_peak()
    avg_kernel_s = (kern_ms / 1e3) / max(kern_n, 1)
    achieved = BYTES_PER_CELL * cells / avg_kernel_s / 1e9
    traffic = profiled_traffic(cells) if args.precision == "fast" else None
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
           "config": {"workload": w["name"], "padded_cells": cells, "interior_cells": int(np.prod(w["n"])),
                      "precision": args.precision,
                      "l2": "no flush: every step streams 3 fields of %d MB (> 129 MB L2)" % (cells * 4 // 10**6),
                      "parallelism": ("shots: one source position per rank, no collective on the data path"
                                      if world > 1 else "single"), "seed": w["seed"]},
           "e2e": {"value": e2e_value, "unit": UNIT,
                   "h2d_bytes_per_step": int(vel.nbytes + wav.nbytes + sou.nbytes + rec.nbytes),
                   "d2h_bytes_per_step": int(plan.nsmp * nr * 4)},
           "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "traffic": traffic,
                        "traffic_source": ("ncu DRAM bytes per cell of a 384^3-padded launch of the same kernel "
                                           "(profiles/k_stepB3_o8_tma_n320.md) x this launch's cells"
                                           if traffic else None),
                        "kernel": ("k_stepB3_o8 (TMA-staged, 3D 8th order)" if plan.step_kernel == "tma3d"
                                   else "k_stepB (one thread per cell, 3D 8th order)"),
                        "peak_source": peak_kind, "avg_launch_us": avg_kernel_s * 1e6,
                        "kernel_share": (kern_ms / ms) if ms > 0 else None},
           "gpu_launches": int(launches), "clocks": clocks, "trace_max_abs": check}
    plan.close()
    if sharded is not None:
        out["batched_gradient"] = sharded
    grad_check = None
    if args.extras and world == 1:
        # the second half of the metric and the spherical configuration, on the
        # same GPU after the headline (each leg reports its own failure)
        for key, fn in (("batched_gradient", extra_batched_gradient), ("spherical_forward", extra_spherical_forward),
                        ("gradients_3d", extra_gradients_3d)):
            try:
                res = fn(args, local, peak, peak_kind)
                if key == "batched_gradient":
                    grad_check = res.pop("_check")
                out[key] = res
            except Exception as e:  # noqa: BLE001 - reported in the JSON line
                out[key] = {"error": "%s: %s" % (type(e).__name__, e)}
            torch.cuda.empty_cache()
    if args.cpu_baseline and world == 1:  # the host-core baseline belongs to the one-GPU line
        out["cpu_baseline"] = host_baseline(w)
        if grad_check is not None:
            try:
                out["cpu_baseline"]["gradient"] = oracle_gradient_check(grad_check)
            except Exception as e:  # noqa: BLE001
                out["cpu_baseline"]["gradient"] = {"error": "%s: %s" % (type(e).__name__, e)}
    print(json.dumps(out))


def extra_batched_gradient(args, local, peak, peak_kind):
    """FWI gradients of the 256-shot survey (the survey's geometry, the 2D gradient's physics: true
    model vs the same smoothed 100 m, BFP16 checkpoints, compensated sums):
    the batched gradient (all shots per launch) against the plain per-shot
    loop (awe_gradient shot after shot), the latter timed on 16 evenly spaced
    shots.  Both from host buffers, host wall clock around the synchronous
    calls; one untimed call each first."""
    import torch

    import wavefield_imaging_gb300 as awe

    nt, nz, nshots = 4000, 512, 256
    vtrue, shots = batch_survey(nshots=nshots, nz=nz)
    v0 = smooth(vtrue, 100.0 / 5.0)
    wav = ricker(nt, 0.005, 5.0)
    desc = awe.make_desc(2, (nz, vtrue.shape[0]), (5.0, 5.0), (0.0, 0.0), nt, 0.005, nb=40, fdorder=8, dabc=1, expl=1,
                         precision=awe.FAST)
    with awe.Batch(desc, shots, device=local) as b:
        b.set_model(vtrue)
        b.select(4, chunk=64)
        dobs = b.forward(wav)
        b.set_model(v0)
        b.gradient(wav, dobs)
        torch.cuda.synchronize()
        reps = 2
        t0 = time.perf_counter()
        for _ in range(reps):
            gb, Jb = b.gradient(wav, dobs)
        batch_s = (time.perf_counter() - t0) / reps
    sample = [int(k) for k in np.linspace(0, nshots - 1, 16)]
    plans = []
    for k in sample:
        x0, nx, sou, rec = shots[k]
        dk = awe.make_desc(2, (nz, nx), (5.0, 5.0), (0.0, x0 * 5.0), nt, 0.005, nb=40, fdorder=8, dabc=1, expl=1,
                           precision=awe.FAST)
        p = awe.Plan(dk, device=local)
        p.set_model(v0[x0:x0 + nx])
        p.set_geometry(sou, rec)
        plans.append(p)
    plans[0].gradient(wav, dobs[sample[0]])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    grads = [p.gradient(wav, dobs[k]) for p, k in zip(plans, sample)]
    plain_s = (time.perf_counter() - t0) / len(sample)
    for p in plans:
        p.close()
    # the smallest window of the sample, for the FP64 oracle check on the host
    kmin = min(sample, key=lambda k: shots[k][1])
    x0, nx, sou, rec = shots[kmin]
    check = dict(shot=kmin, x0=x0, nx=nx, nz=nz, nt=nt, vel=v0[x0:x0 + nx], wav=wav, sou=sou, rec=rec,
                 dobs=dobs[kmin], grad=grads[sample.index(kmin)][0])
    return {"workload": "%d shots on windows nx in [300, 700] x nz 512 of a 6000-column model, 8th order, nt=%d, "
                        "nb=40, dabc=y; start model = true model smoothed 100 m; BFP16 checkpoints" % (nshots, nt),
            "batched_shot_gradients_per_s": nshots / batch_s, "batched_s": batch_s,
            "plain_shot_gradients_per_s": 1.0 / plain_s, "plain_s_per_shot": plain_s,
            "plain_sample": "16 evenly spaced shots of the survey, awe_gradient one after the other",
            "speedup_batched_vs_plain": plain_s * nshots / batch_s, "misfit": Jb,
            "timing": "host wall clock around synchronous calls from host buffers", "_check": check}


def extra_sharded_gradient(dist, rank, world, local):
    """N ranks: the 256-shot survey's gradient with the shots split across
    ranks (every world-th shot, replicas.survey_gradient: each rank's batched
    gradient, one FP64 sum over the process group).  One untimed call, then
    one timed between barriers; whole-job shot gradients/s over the slowest
    rank."""
    import wavefield_imaging_gb300 as awe
    from wavefield_imaging_gb300.replicas import survey_gradient

    nt, nz, nshots = 4000, 512, 256
    vtrue, shots = batch_survey(nshots=nshots, nz=nz)
    v0 = smooth(vtrue, 100.0 / 5.0)
    wav = ricker(nt, 0.005, 5.0)
    desc = awe.make_desc(2, (nz, vtrue.shape[0]), (5.0, 5.0), (0.0, 0.0), nt, 0.005, nb=40, fdorder=8, dabc=1, expl=1,
                         precision=awe.FAST)
    mine = set(range(nshots)[rank::world])
    dobs = [None] * nshots
    with awe.Batch(desc, [shots[i] for i in sorted(mine)], device=local) as b:
        b.set_model(vtrue)
        b.select(4, chunk=64)
        for i, d in zip(sorted(mine), b.forward(wav)):
            dobs[i] = d
    zero = [np.zeros((nt, s[3].shape[0]), np.float32) for s in shots]  # other ranks' shots are not read
    dobs = [d if d is not None else z for d, z in zip(dobs, zero)]
    survey_gradient(desc, shots, v0, wav, dobs, dist=dist, device=local)
    barrier(dist)
    t0 = time.perf_counter()
    _, J = survey_gradient(desc, shots, v0, wav, dobs, dist=dist, device=local)
    secs = allmax(dist, time.perf_counter() - t0)
    return {"workload": "%d shots split across %d ranks (every %d-th shot per rank), nt=%d, BFP16 checkpoints"
                        % (nshots, world, world, nt),
            "shot_gradients_per_s": nshots / secs, "s": secs, "misfit": J,
            "timing": "host wall clock between barriers, the slowest rank, including the FP64 sum"}


def oracle_gradient_check(c):
    """The FP64 adjoint oracle (all forward levels kept in host memory, one
    thread) on one survey shot: its time is the CPU baseline of the gradient
    half of the metric, its gradient the reference for the engine's
    (rel-L2 over the shot's window)."""
    from oracle import oracle

    nz, nx = c["nz"], c["nx"]
    npad = (nz + 80) * (nx + 80)
    try:
        mem = os.sysconf("SC_PAGE_SIZE") * os.sysconf("SC_PHYS_PAGES")
    except (ValueError, OSError):
        mem = 64 << 30
    nt = c["nt"]
    need = (nt + 1) * npad * 8 * 1.1
    if need > 0.25 * mem:
        return {"skipped": "needs %.1f GB of host memory, more than a quarter of %.1f GB" % (need / 1e9, mem / 1e9)}
    par = dict(n=[nz, nx], d=[5.0, 5.0], o=[0.0, c["x0"] * 5.0], nb=40, nt=nt, dt=0.005, fdorder=8, dabc=1, expl=1)
    t0 = time.perf_counter()
    g64, J64, _ = oracle.misfit_gradient(par, c["vel"], c["wav"], c["sou"], c["rec"], c["dobs"])
    secs = time.perf_counter() - t0
    g = np.asarray(c["grad"], np.float64)
    err = float(np.linalg.norm(g - g64) / max(np.linalg.norm(g64), 1e-300))
    return {"value": 1.0 / secs, "unit": "shot gradients/s", "cores": 1, "kind": "port",
            "sample": "shot %d of the survey (window of %d columns, nt=%d): FP64 adjoint oracle" % (
                c["shot"], nx, nt),
            "rel_l2_engine_bfp16_vs_fp64": err}


def extra_spherical_forward(args, local, peak, peak_kind):
    """The spherical-shell configuration (764 x 576 x 576 padded, scheme of
    sfAWEFDspher3Dgpu): the 16-source track advancing in one launch per step,
    200 of its 3000 steps, device-resident; cell-updates/s and the step
    kernel's HBM roofline."""
    import torch

    import wavefield_imaging_gb300 as awe

    nt, nshots = 200, 16
    w = spher_workload(nt)
    vel = spher_model(w)
    shots = spher_shots(w, nshots)
    wav = ricker(nt, w["dt"], w["f0"])
    desc = awe.make_desc(3, w["n"], w["d"], w["o"], nt, w["dt"], coords=awe.SPHER, scheme=awe.SCHEME_GPU,
                         nb=w["nb"], expl=0, precision=awe.FAST)
    with awe.Plan(desc, device=local) as plan:
        plan.set_model(vel)
        plan.set_shots(shots)
        nrec = sum(r.shape[0] for _, r in shots)
        d_wav = torch.from_numpy(wav).cuda()
        d_dat = torch.zeros((plan.nsmp, nrec), dtype=torch.float32, device="cuda")
        stream = torch.cuda.Stream()
        plan.forward_device(d_wav.data_ptr(), 1, d_dat.data_ptr(), 0, stream.cuda_stream)
        torch.cuda.synchronize()
        plan.profile(True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.forward_device(d_wav.data_ptr(), 1, d_dat.data_ptr(), 0, stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        kern_ms, kern_n = plan.profile_read()
        plan.profile(False)
        kernel = SPHER_KERNEL[plan.step_kernel]
    cells = nshots * int(np.prod([n + 2 * w["nb"] for n in w["n"]]))
    avg = kern_ms / 1e3 / max(kern_n, 1)
    achieved = BYTES_PER_CELL * cells / avg / 1e9
    return {"workload": w["name"].replace("1 source", "%d sources along the track, one launch per step" % nshots)
                        + " (%d of 3000 steps)" % nt,
            "value": cells * nt / (ms / 1e3), "unit": "cell-updates/s", "ms_per_run": ms,
            "roofline": {"kernel": kernel, "avg_launch_us": avg * 1e6, "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind}}


def _timed_gradient(plan, wav, dobs, nt, cells, peak, peak_kind, step_bytes, adj_bytes, names):
    """One untimed and one timed device-resident gradient (BFP16
    checkpoints) of a plan whose model and geometry are set; the step and
    adjoint kernels timed with CUDA events on their stream."""
    import torch

    import wavefield_imaging_gb300 as awe

    d_wav = torch.from_numpy(wav).cuda()
    d_dobs = torch.from_numpy(np.ascontiguousarray(dobs, np.float32)).cuda()
    d_grad = torch.zeros(int(plan.desc.n[0]) * int(plan.desc.n[1]) * int(plan.desc.n[2]), dtype=torch.float64,
                         device="cuda")
    stream = torch.cuda.Stream()

    def step():
        return plan.gradient_device(d_wav.data_ptr(), 1, d_dobs.data_ptr(), d_grad.data_ptr(),
                                    ckpt_format=awe.CKPT_BFP16, stream=stream.cuda_stream)

    step()
    torch.cuda.synchronize()
    plan.profile(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    J = step()
    e1.record(stream)
    torch.cuda.synchronize()
    kinds = plan.profile_read_kinds()
    plan.profile(False)
    ms = e0.elapsed_time(e1)
    out = {"gradient_ms": ms, "misfit": J, "kernels": {}}
    for kind, nbytes in (("step", step_bytes), ("adjoint", adj_bytes)):
        kms, kn = kinds[kind]
        if kn:
            avg = kms / 1e3 / kn
            k = {"kernel": names[kind], "launches": kn, "avg_launch_us": avg * 1e6, "share_of_gradient": kms / ms}
            if nbytes:
                k.update(bytes_per_cell=nbytes, achieved=nbytes * cells / avg / 1e9, unit="GB/s",
                         frac=nbytes * cells / avg / 1e9 / peak, peak=peak, peak_source=peak_kind)
            out["kernels"][kind] = k
    return out


def extra_gradients_3d(args, local, peak, peak_kind):
    """The 512^3 cartesian and the spherical-shell gradients, each on its full grid for 300 of its 3000
    steps (one shot, BFP16 checkpoints, start model smoothed 100 m along z or
    r): gradient time and the step and adjoint kernels' HBM fractions."""
    from scipy.ndimage import gaussian_filter1d

    import wavefield_imaging_gb300 as awe

    nt = 300
    res = {}
    # the 512^3 cube, 8th order (forward steps 16 B per cell; the
    # recompute steps also store L(V_k), 20 B; adjoint step 36 B)
    w = workload(nt, args.n)
    vtrue = layered_model_3d(w)
    v0 = gaussian_filter1d(vtrue, 100.0 / 5.0, axis=2, mode="nearest").astype(np.float32)
    sou, rec = geometry(w)
    wav = ricker(nt, w["dt"], w["f0"])
    desc = awe.make_desc(3, w["n"], w["d"], w["o"], nt, w["dt"], nb=w["nb"], fdorder=w["fdorder"], dabc=w["dabc"],
                         expl=1, precision=awe.FAST)
    with awe.Plan(desc, device=local) as plan:
        plan.set_geometry(sou, rec)
        plan.set_model(vtrue)
        dobs = plan.forward(wav)
        plan.set_model(v0)
        r = _timed_gradient(plan, wav, dobs, nt, padded_cells(w), peak, peak_kind, None, 36,
                            {"step": "k_stepB3_o8 (forward 16 B, recompute 20 B per cell)",
                             "adjoint": "k_stepB3_o8 adjoint step"})
    r["workload"] = w["name"].replace("nt=%d" % nt, "nt=%d of 3000" % nt) + ", gradient, BFP16 checkpoints"
    res["cartesian"] = r
    # the spherical shell, one source
    w = spher_workload(nt)
    vtrue = spher_model(w)
    v0 = gaussian_filter1d(vtrue, 100.0 / 5.0, axis=2, mode="nearest").astype(np.float32)
    sou, rec = spher_shots(w, 1)[0]
    wav = ricker(nt, w["dt"], w["f0"])
    desc = awe.make_desc(3, w["n"], w["d"], w["o"], nt, w["dt"], coords=awe.SPHER, scheme=awe.SCHEME_GPU,
                         nb=w["nb"], expl=0, precision=awe.FAST)
    cells = int(np.prod([n + 2 * w["nb"] for n in w["n"]]))
    with awe.Plan(desc, device=local) as plan:
        plan.set_geometry(sou, rec)
        plan.set_model(vtrue)
        dobs = plan.forward(wav)
        plan.set_model(v0)
        tma = plan.step_kernel == "tma_sph"
        r = _timed_gradient(plan, wav, dobs, nt, cells, peak, peak_kind, BYTES_PER_CELL, ADJ_BYTES_PER_CELL,
                            {"step": SPHER_KERNEL[plan.step_kernel],
                             "adjoint": "k_adjA_sph_tma" if tma else "k_adjA_sph2"})
    r["workload"] = w["name"].replace("nt=%d" % nt, "nt=%d of 3000" % nt) + ", gradient, BFP16 checkpoints"
    res["spherical"] = r
    return res


GRAD_METRIC = "FWI gradients/s (misfit gradient, checkpointed fwd + adjoint)"


def grad_workload(kind, nt, n):
    if kind == "grad3d":
        w = workload(nt, n)
        w["name"] = ("3D misfit gradient d(0.5||d-dobs||^2)/d(1/v^2), %d^3 at 5 m (%d^3 padded), 8th order, nt=%d, "
                     "dabc=y, 1 source, 128x128 receivers" % (n, n + 64, nt))
        return w
    # 2D: 512 x 512 at 5 m, nb=40, nt=4000, 512 receivers at z = 50 m, source at x = centre, z = 50 m
    return dict(name="2D misfit gradient, %d^2 at 5 m (%d^2 padded, nb=40), 8th order, nt=%d, dabc=y, 1 source, "
                     "512 receivers" % (n, n + 80, nt),
                n=(n, n), d=(5.0, 5.0), o=(0.0, 0.0), nt=nt, dt=0.005, nb=40, fdorder=8, dabc=1, f0=5.0, seed=1)


def smooth(vel, sigma_cells):
    """Gaussian smoothing (FFT, periodic) of a model, for the starting model."""
    out = vel.astype(np.float64)
    for ax in range(vel.ndim):
        k = np.fft.fftfreq(vel.shape[ax])
        shape = [1] * vel.ndim
        shape[ax] = -1
        filt = np.exp(-0.5 * (2 * np.pi * k * sigma_cells) ** 2).reshape(shape)
        out = np.real(np.fft.ifft(np.fft.fft(out, axis=ax) * filt, axis=ax))
    return out.astype(np.float32)


def run_grad(args):
    """--workload grad3d | grad2d: time whole misfit gradients (forward with
    checkpoints + segment recompute + adjoint) of the true-vs-smoothed model
    problem.  One bench step = one gradient."""
    import torch

    import wavefield_imaging_gb300 as awe

    dist, rank, world, local = dist_init()
    torch.cuda.set_device(local)
    nt = args.nt if args.nt != 3000 or args.workload == "grad3d" else 4000
    w = grad_workload(args.workload, nt, args.n)
    nd = len(w["n"])
    if nd == 3:
        vtrue = layered_model_3d(w)
        sou, rec = geometry(w)
    else:
        w3 = dict(w, n=(w["n"][0], w["n"][1], 1))
        vtrue = layered_model_3d(w3)[0]
        nx = w["n"][1]
        sou = np.array([[0.5 * (nx - 1) * 5.0, 50.0]], np.float32)
        rec = np.stack([np.arange(nx) * 5.0, np.full(nx, 50.0)], 1).astype(np.float32)
    v0 = smooth(vtrue, 100.0 / 5.0)
    wav = ricker(w["nt"], w["dt"], w["f0"])
    desc = awe.make_desc(nd, w["n"], w["d"], w["o"], w["nt"], w["dt"], nb=w["nb"], fdorder=w["fdorder"],
                         dabc=w["dabc"], expl=1, precision=awe.FAST)
    plan = awe.Plan(desc, device=local)
    plan.set_geometry(sou, rec)
    plan.set_model(vtrue)
    dobs = plan.forward(wav)
    plan.set_model(v0)
    fmt = {"bfp16": awe.CKPT_BFP16, "bf16": awe.CKPT_BF16, "fp16": awe.CKPT_FP16, "fp32": awe.CKPT_FP32}[args.ckpt]
    d_wav = torch.from_numpy(wav).cuda()
    d_dobs = torch.from_numpy(dobs).cuda()
    ngrad = int(np.prod(w["n"]))
    d_grad = torch.zeros(ngrad, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()

    def step():
        return plan.gradient_device(d_wav.data_ptr(), 1, d_dobs.data_ptr(), d_grad.data_ptr(), ckpt_format=fmt,
                                    stream=stream.cuda_stream)

    for _ in range(args.warmup):
        J = step()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    barrier(dist)
    plan.profile(True)  # events around every step and adjoint kernel launch
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    launches = 0
    for _ in range(args.steps):
        J = step()
        launches += plan.last_launch_count()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(dist)
    clocks = sampler.stop()
    kinds = plan.profile_read_kinds()
    plan.profile(False)
    ms = allmax(dist, ev0.elapsed_time(ev1))
    # the forward alone, for the split
    d_dat = torch.zeros((plan.nsmp, rec.shape[0]), dtype=torch.float32, device="cuda")
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    plan.forward_device(d_wav.data_ptr(), 1, d_dat.data_ptr(), 0, stream.cuda_stream)
    f1.record(stream)
    torch.cuda.synchronize()
    fwd_ms = f0.elapsed_time(f1)
    if rank != 0:
        return
    cells = padded_cells(w)
    g_s = ms / 1e3 / args.steps
    peak, peak_kind = measured_peak()
    kernels = {}
    # 3D: forward steps 16 B per cell, recompute steps (which also store
    # L(V_k)) 20 B; the adjoint step 36 B (halo of I vel2 nu, nu_{k+1}, nu_k,
    # L(V_k), the 8-byte gradient pair read and written, mu written)
    for kind, nbytes in (("step", None), ("adjoint", 36 if nd == 3 else None)):
        kms, kn = kinds[kind]
        if kn:
            avg = kms / 1e3 / kn
            k = {"launches": kn, "ms": kms, "avg_launch_us": avg * 1e6, "share_of_gradient": kms / args.steps / ms}
            if nbytes:
                k.update(bytes_per_cell=nbytes, achieved=nbytes * cells / avg / 1e9, unit="GB/s",
                         frac=nbytes * cells / avg / 1e9 / peak, peak=peak, peak_source=peak_kind)
            kernels[kind] = k
    out = {"metric": GRAD_METRIC, "value": args.steps * world / (ms / 1e3), "unit": "gradients/s",
           "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32 fields, compensated fp32 sums",
           "data": "synthetic",
           "config": {"workload": w["name"], "checkpoint": args.ckpt, "padded_cells": cells,
                      "ckpt_every": int(np.ceil(np.sqrt(w["nt"]))), "start_model": "true model smoothed, 100 m",
                      "device_bytes": plan.device_bytes(), "seed": w["seed"]},
           "split": {"forward_ms": fwd_ms, "gradient_ms": ms / args.steps,
                     "gradient_over_forward": (ms / args.steps) / fwd_ms,
                     "cell_steps_per_s": cells * w["nt"] / g_s,
                     "algorithmic_GBps": 48.0 * cells * w["nt"] / g_s / 1e9},
           "kernels": kernels,
           "misfit": J, "gpu_launches": int(launches), "clocks": clocks}
    print(json.dumps(out))
    plan.close()


BATCH_METRIC = "batched 2D forward shots/s (uneven windows, one graph-replayed launch per step)"


def batch_survey(nshots=256, nxm=6000, nz=512, seed=5):
    """The 256-shot survey: a seeded layered model 6000 columns wide, shots
    every 20 m (4 columns) along a straight track, each on its own window of
    nx in [300, 700] columns centred on the source, 128 receivers centred on
    the source at z = 50 m, source at z = 50 m."""
    rng = np.random.default_rng(seed)
    w3 = dict(n=(nz, nxm, 1), d=(5.0, 5.0, 5.0), seed=seed)
    vel = layered_model_3d(w3)[0]  # [nxm][nz]
    shots = []
    first = nxm // 2 - 2 * nshots
    for i in range(nshots):
        xs = first + 4 * i
        nx = int(rng.integers(300, 701))
        x0 = max(0, min(nxm - nx, xs - nx // 2))
        sou = np.array([[xs * 5.0, 50.0]], np.float32)
        rec = np.stack([(xs - 64 + np.arange(128)) * 5.0, np.full(128, 50.0)], 1).astype(np.float32)
        shots.append((x0, nx, sou, rec))
    return vel, shots


def run_batch(args):
    """--workload batch2d: all shots in one batched, graph-replayed forward
    (autotuned tiles) against the same shots run one by one through the
    single-shot path (each a plain launch sequence of its own)."""
    import torch

    import wavefield_imaging_gb300 as awe

    dist, rank, world, local = dist_init()
    torch.cuda.set_device(local)
    nt = 4000 if args.nt == 3000 else args.nt
    nshots, nz = args.shots or 256, 512
    vel, shots = batch_survey(nshots=nshots, nz=nz)
    nxm = vel.shape[0]
    wav = ricker(nt, 0.005, 5.0)
    desc = awe.make_desc(2, (nz, nxm), (5.0, 5.0), (0.0, 0.0), nt, 0.005, nb=40, fdorder=8, dabc=1, expl=1,
                         precision=awe.FAST)
    batch = awe.Batch(desc, shots, device=local)
    batch.set_model(vel)
    tile, grid = batch.tune(steps=20)
    d_wav = torch.from_numpy(wav).cuda()
    d_dat = torch.zeros(batch.info.total_samples, dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()

    def step():
        batch.forward_device(d_wav.data_ptr(), d_dat.data_ptr(), stream.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    barrier(dist)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = allmax(dist, e0.elapsed_time(e1)) / args.steps
    cells = batch.info.cells

    # plain loop: one single-shot plan per shot, run one after the other
    plans = []
    for (x0, nx, sou, rec) in shots:
        dsc = awe.make_desc(2, (nz, nx), (5.0, 5.0), (0.0, x0 * 5.0), nt, 0.005, nb=40, fdorder=8, dabc=1, expl=1,
                            precision=awe.FAST)
        p = awe.Plan(dsc, device=local)
        p.set_model(vel[x0:x0 + nx])
        p.set_geometry(sou, rec)
        plans.append(p)
    d_pd = [torch.zeros((p.nsmp, 128), dtype=torch.float32, device="cuda") for p in plans]
    for p, dd in zip(plans[:4], d_pd):
        p.forward_device(d_wav.data_ptr(), 1, dd.data_ptr(), 0, stream.cuda_stream)
    torch.cuda.synchronize()
    p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    plain_launches = 0
    for p, dd in zip(plans, d_pd):
        p.forward_device(d_wav.data_ptr(), 1, dd.data_ptr(), 0, stream.cuda_stream)
        plain_launches += p.last_launch_count()
    p1.record(stream)
    torch.cuda.synchronize()
    plain_ms = p0.elapsed_time(p1)
    # the batch's traces against the plain runs
    dat = d_dat.cpu().numpy()
    worst, off = 0.0, 0
    for p, dd in zip(plans, d_pd):
        a = dat[off:off + dd.numel()]
        b_ = dd.cpu().numpy().ravel()
        worst = max(worst, float(np.linalg.norm(a - b_) / max(np.linalg.norm(b_), 1e-30)))
        off += dd.numel()
    for p in plans:
        p.close()
    if rank != 0:
        return
    out = {"metric": BATCH_METRIC, "value": nshots * world / (ms / 1e3), "unit": "shots/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
           "config": {"workload": "%d shots, 20 m apart, windows nx in [300, 700] x nz 512 of a 6000-column model, "
                                  "8th order, nt=%d, nb=40, dabc=y, 128 receivers per shot" % (nshots, nt),
                      "padded_cells": cells, "tile": list(tile), "grid": grid,
                      "work_items_per_launch": batch.info.work_items},
           "cell_updates_per_s": cells * nt / (ms / 1e3),
           "achieved_GBps": 16.0 * cells * nt / (ms / 1e3) / 1e9,
           "plain": {"ms": plain_ms, "shots_per_s": nshots / (plain_ms / 1e3), "launches": plain_launches},
           "speedup_vs_plain": plain_ms / ms, "max_rel_l2_vs_plain": worst,
           "gpu_launches": nt * args.steps, "clocks": clocks}
    print(json.dumps(out))
    batch.close()


def run_batch_grad(args):
    """--workload batchgrad2d: misfit gradient of the whole survey in one
    batched, checkpointed fwd + adjoint run, against the plain per-shot loop
    (awe_gradient shot after shot on the same GPU).  Value: shot gradients/s."""
    import torch

    import wavefield_imaging_gb300 as awe

    dist, rank, world, local = dist_init()
    torch.cuda.set_device(local)
    nt = 4000 if args.nt == 3000 else args.nt
    nshots, nz = args.shots or 256, 512
    vtrue, shots = batch_survey(nshots=nshots, nz=nz)
    v0 = smooth(vtrue, 100.0 / 5.0)
    nxm = vtrue.shape[0]
    wav = ricker(nt, 0.005, 5.0)
    fmt = {"bfp16": awe.CKPT_BFP16, "bf16": awe.CKPT_BF16, "fp16": awe.CKPT_FP16, "fp32": awe.CKPT_FP32}[args.ckpt]
    desc = awe.make_desc(2, (nz, nxm), (5.0, 5.0), (0.0, 0.0), nt, 0.005, nb=40, fdorder=8, dabc=1, expl=1,
                         precision=awe.FAST)
    batch = awe.Batch(desc, shots, device=local)
    batch.set_model(vtrue)
    batch.tune(steps=20)
    dobs = batch.forward(wav)
    batch.set_model(v0)
    for _ in range(args.warmup):
        batch.gradient(wav, dobs, ckpt_format=fmt)
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        gb, Jb = batch.gradient(wav, dobs, ckpt_format=fmt)
    t1 = time.perf_counter()
    clocks = sampler.stop()
    batch_s = allmax(dist, (t1 - t0) / args.steps)
    info = batch.info
    batch.close()
    # plain: one plan per shot, awe_gradient one shot after the other
    plans = []
    for (x0, nx, sou, rec) in shots:
        dsc = awe.make_desc(2, (nz, nx), (5.0, 5.0), (0.0, x0 * 5.0), nt, 0.005, nb=40, fdorder=8, dabc=1, expl=1,
                            precision=awe.FAST)
        p = awe.Plan(dsc, device=local)
        p.set_model(v0[x0:x0 + nx])
        p.set_geometry(sou, rec)
        plans.append(p)
    gp = np.zeros_like(gb)
    plans[0].gradient(wav, dobs[0], ckpt_format=fmt)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    Jp = 0.0
    for (x0, nx, _, _), p, d in zip(shots, plans, dobs):
        g, J = p.gradient(wav, d, ckpt_format=fmt)
        gp[x0:x0 + nx] += g
        Jp += J
    t1 = time.perf_counter()
    plain_s = t1 - t0
    for p in plans:
        p.close()
    if rank != 0:
        return
    out = {"metric": "batched FWI gradients/s (2D survey, checkpointed fwd + adjoint)",
           "value": nshots * world / batch_s, "unit": "shot gradients/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 1e3 * batch_s, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "fp32 fields, compensated fp32 sums", "data": "synthetic",
           "config": {"workload": "%d shots, windows nx in [300, 700] x nz 512 of a 6000-column model, 8th order, "
                                  "nt=%d, nb=40, dabc=y; start model = true model smoothed 100 m" % (nshots, nt),
                      "checkpoint": args.ckpt, "padded_cells": info.cells,
                      "tile": [info.tile_z, info.tile_x], "grid": info.grid,
                      "timing": "host wall clock around the synchronous gradient call (inputs from host)"},
           "plain": {"s": plain_s, "shot_gradients_per_s": nshots / plain_s},
           "speedup_vs_plain": plain_s / batch_s,
           "rel_l2_batch_vs_plain": float(np.linalg.norm(gb - gp) / max(np.linalg.norm(gp), 1e-300)),
           "misfit": {"batch": Jb, "plain": Jp},
           "cell_steps_per_s": info.cells * nt / batch_s, "clocks": clocks}
    print(json.dumps(out))


# the spherical step kernel a plan runs (Plan.step_kernel)
SPHER_KERNEL = {"tma_sph": "k_stepA_sph_tma", "simple": "k_stepA_sph_march2"}


def spher_workload(nt, nr=700, nang=512):
    return dict(name="3D spherical shell (GPU-program scheme, metric terms), r in [3387.0, 3390.5] km at 5 m, "
                     "theta and phi %d x 0.04/%d rad at the equator, nb=32, nt=%d, 1 source, 64x64 receivers"
                     % (nang, nang, nt),
                n=(nr, nang, nang), d=(0.005, 0.04 / nang, 0.04 / nang),
                o=(3387.0, np.pi / 2 - 0.02, -0.02), nt=nt, dt=0.005, nb=32, f0=5.0, seed=11)


def spher_model(w):
    """Vacuum / ice (5 dust layers) / basalt as a function of depth below
    r = 3389.5 km (surface at 200 m depth with 30 m random topography, basalt
    below 1800 m), velocities in km/us.  Returns [nphi][ntheta][nr]."""
    rng = np.random.default_rng(w["seed"])
    nr, nth, nph = w["n"]
    r = w["o"][0] + np.arange(nr) * w["d"][0]
    depth = (3389.5 - r)[None, None, :]
    topo = 0.2 + 0.03 * gaussian_field(rng, (nph, nth), 40.0)[:, :, None]
    vel = np.full((nph, nth, nr), 0.168, np.float32)
    for _ in range(5):
        zd = rng.uniform(0.4, 1.6)
        th = rng.uniform(0.010, 0.020)
        vel[np.broadcast_to(np.abs(depth - (topo + zd - 0.2)) < 0.5 * th, vel.shape)] = 0.168 * rng.choice([0.95, 1.05])
    vel[np.broadcast_to(depth < topo, vel.shape)] = 0.3
    vel[np.broadcast_to(depth >= 1.8, vel.shape)] = 0.110
    return vel


def spher_shots(w, nshots):
    """Sources along the equator (a great circle) at 50 m altitude above the
    mean surface, 64 x 64 receivers around each: [(sou, rec)] in (r, phi, theta)."""
    nr_, nth, nph = w["n"]
    rs = 3389.5 - 0.2 + 0.05
    th0 = w["o"][1] + 0.5 * (nth - 1) * w["d"][1]
    shots = []
    for k in range(nshots):
        ph_s = w["o"][2] + (0.5 if nshots == 1 else 0.3 + 0.4 * k / (nshots - 1)) * (nph - 1) * w["d"][2]
        sou = np.array([[rs, ph_s, th0]], np.float32)
        gth = th0 + np.linspace(-0.25, 0.25, 64) * (nth - 1) * w["d"][1]
        gph = ph_s + np.linspace(-0.25, 0.25, 64) * (nph - 1) * w["d"][2]
        P, T = np.meshgrid(gph, gth, indexing="ij")
        rec = np.stack([np.full(P.size, rs), P.ravel(), T.ravel()], 1).astype(np.float32)
        shots.append((sou, rec))
    return shots


def run_sphergrad(args):
    """--workload sphergrad3d: misfit gradient of the spherical shell (700 x 512 x 512
    grid and scheme; --shots sources along the track, default 1): forward
    with checkpoints, segment recompute, adjoint of the spherical step, shot
    after shot.  Start model: the true model smoothed along r (100 m).  One
    bench step = one gradient of all shots; the forward of all shots (one
    launch per step) is timed beside it."""
    import torch
    from scipy.ndimage import gaussian_filter1d

    import wavefield_imaging_gb300 as awe

    torch.cuda.set_device(0)
    nt = args.nt
    w = spher_workload(nt, nr=args.n + 188 if args.n != 512 else 700, nang=args.n)
    vtrue = spher_model(w)
    v0 = gaussian_filter1d(vtrue, 100.0 / 5.0, axis=2, mode="nearest").astype(np.float32)
    nshots = args.shots or 1
    shots = spher_shots(w, nshots)
    rec = np.concatenate([r for _, r in shots])
    wav = ricker(nt, w["dt"], w["f0"])
    desc = awe.make_desc(3, w["n"], w["d"], w["o"], nt, w["dt"], coords=awe.SPHER, scheme=awe.SCHEME_GPU,
                         nb=w["nb"], expl=0, precision=awe.FAST)
    plan = awe.Plan(desc)
    if nshots == 1:
        plan.set_geometry(*shots[0])
    else:  # the track: one launch per step for the forward, shot after shot for the gradient
        plan.set_shots(shots)
    plan.set_model(vtrue)
    dobs = plan.forward(wav)
    plan.set_model(v0)
    fmt = {"bfp16": awe.CKPT_BFP16, "bf16": awe.CKPT_BF16, "fp16": awe.CKPT_FP16, "fp32": awe.CKPT_FP32}[args.ckpt]
    d_wav = torch.from_numpy(wav).cuda()
    d_dobs = torch.from_numpy(dobs).cuda()
    d_grad = torch.zeros(int(np.prod(w["n"])), dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()

    def step():
        return plan.gradient_device(d_wav.data_ptr(), 1, d_dobs.data_ptr(), d_grad.data_ptr(), ckpt_format=fmt,
                                    stream=stream.cuda_stream)

    for _ in range(args.warmup):
        J = step()
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    plan.profile(True)  # events around every step and adjoint kernel launch
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    launches = 0
    for _ in range(args.steps):
        J = step()
        launches += plan.last_launch_count()
    ev1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    kinds = plan.profile_read_kinds()
    plan.profile(False)
    ms = ev0.elapsed_time(ev1) / args.steps
    peak, peak_kind = measured_peak()
    cells_pad = int(np.prod([n + 2 * w["nb"] for n in w["n"]]))
    kernels = {}
    for kind, nbytes, name in (("step", BYTES_PER_CELL, "k_stepA_sph_tma" if plan.step_kernel == "tma_sph"
                                else "k_stepA_sph_march2"),
                               ("adjoint", ADJ_BYTES_PER_CELL, "k_adjA_sph_tma" if plan.step_kernel == "tma_sph"
                                else "k_adjA_sph2")):
        kms, kn = kinds[kind]
        if kn:
            avg = kms / 1e3 / kn
            kernels[kind] = {"kernel": name, "launches": kn, "ms": kms, "avg_launch_us": avg * 1e6,
                             "bytes_per_cell": nbytes, "achieved": nbytes * cells_pad / avg / 1e9, "unit": "GB/s",
                             "frac": nbytes * cells_pad / avg / 1e9 / peak, "peak": peak, "peak_source": peak_kind,
                             "share_of_gradient": kms / args.steps / ms}
    d_dat = torch.zeros((plan.nsmp, rec.shape[0]), dtype=torch.float32, device="cuda")
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    plan.forward_device(d_wav.data_ptr(), 1, d_dat.data_ptr(), 0, stream.cuda_stream)
    f1.record(stream)
    torch.cuda.synchronize()
    fwd_ms = f0.elapsed_time(f1)
    cells = int(np.prod([n + 2 * w["nb"] for n in w["n"]]))
    g = d_grad.cpu().numpy()
    out = {"metric": "FWI gradients/s (spherical shell, checkpointed fwd + adjoint)", "value": nshots * 1e3 / ms,
           "unit": "shot gradients/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "fp32 fields, compensated fp32 sums", "data": "synthetic",
           "config": {"workload": w["name"] + ", %d shot%s, start model smoothed 100 m along r"
                      % (nshots, "s" if nshots > 1 else ""), "checkpoint": args.ckpt, "shots": nshots,
                      "padded_cells": cells, "ckpt_every": int(np.ceil(np.sqrt(nt))),
                      "device_bytes": plan.device_bytes()},
           "split": {"forward_ms": fwd_ms, "gradient_ms": ms, "gradient_over_forward": ms / fwd_ms,
                     "cell_steps_per_s": nshots * cells * nt / (ms / 1e3)},
           "kernels": kernels,
           "misfit": J, "grad_finite": bool(np.isfinite(g).all()), "grad_max_abs": float(np.abs(g).max()),
           "gpu_launches": int(launches), "clocks": clocks}
    print(json.dumps(out))
    plan.close()


def run_spher(args):
    """--workload spher3d: one shot of the spherical-shell forward (scheme of
    sfAWEFDspher3Dgpu) on the 700 x 512 x 512 shell."""
    import torch

    import wavefield_imaging_gb300 as awe

    torch.cuda.set_device(0)
    nt = args.nt
    nshots = args.shots or 1
    w = spher_workload(nt, nr=args.n + 188 if args.n != 512 else 700, nang=args.n)
    vel = spher_model(w)
    shots = spher_shots(w, nshots)
    wav = ricker(nt, w["dt"], w["f0"])
    desc = awe.make_desc(3, w["n"], w["d"], w["o"], nt, w["dt"], coords=awe.SPHER, scheme=awe.SCHEME_GPU,
                         nb=w["nb"], expl=0, precision=awe.FAST)
    plan = awe.Plan(desc)
    plan.set_model(vel)
    if nshots == 1:
        plan.set_geometry(*shots[0])
    else:
        plan.set_shots(shots)
    rec = np.concatenate([r for _, r in shots])
    d_wav = torch.from_numpy(wav).cuda()
    d_dat = torch.zeros((plan.nsmp, rec.shape[0]), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()
    for _ in range(args.warmup):
        plan.forward_device(d_wav.data_ptr(), 1, d_dat.data_ptr(), 0, stream.cuda_stream)
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    plan.profile(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        plan.forward_device(d_wav.data_ptr(), 1, d_dat.data_ptr(), 0, stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
    kern_ms, kern_n = plan.profile_read()
    cells = nshots * int(np.prod([n + 2 * w["nb"] for n in w["n"]]))
    peak, peak_kind = measured_peak()
    avg = kern_ms / 1e3 / max(kern_n, 1)
    plain = None
    if nshots > 1:  # the same shots one after the other through the single-shot path
        single = awe.Plan(desc)
        single.set_model(vel)
        d1 = torch.zeros((single.nsmp, 4096), dtype=torch.float32, device="cuda")
        q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        q0.record(stream)
        for sou, r in shots:
            single.set_geometry(sou, r)
            single.forward_device(d_wav.data_ptr(), 1, d1.data_ptr(), 0, stream.cuda_stream)
        q1.record(stream)
        torch.cuda.synchronize()
        plain = {"ms": q0.elapsed_time(q1), "speedup_batched_vs_plain": q0.elapsed_time(q1) / ms}
        single.close()
    out = {"metric": "cell-updates/s (3D spherical shell, GPU-program scheme)", "value": cells * nt / (ms / 1e3),
           "unit": "cell-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
           "config": {"workload": w["name"] + (", %d shots in one launch per step" % nshots if nshots > 1 else ""),
                      "padded_cells": cells, "shots": nshots},
           "plain_sequential": plain,
           "roofline": {"bound": "hbm", "kernel": SPHER_KERNEL[plan.step_kernel], "avg_launch_us": avg * 1e6,
                        "achieved": BYTES_PER_CELL * cells / avg / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": BYTES_PER_CELL * cells / avg / 1e9 / peak, "peak_source": peak_kind,
                        "kernel_share": kern_ms / args.steps / ms},
           "gpu_launches": plan.last_launch_count() * args.steps, "clocks": clocks,
           "trace_max_abs": float(d_dat.abs().max())}
    print(json.dumps(out))
    plan.close()


def run_fwd2d(args):
    """--workload fwd2d: the 2D single-shot forward (512^2 at 5 m, nb=40,
    nt=4000, 8th order, dabc, 512 receivers at z = 50 m): the time loop runs as
    a captured CUDA graph; a second, profiled pass gives the step kernel's time."""
    import torch

    import wavefield_imaging_gb300 as awe

    torch.cuda.set_device(0)
    nz = nx = args.n
    nt = 4000 if args.nt == 3000 else args.nt
    vel = layered_model_3d(dict(n=(nz, nx, 1), d=(5.0, 5.0, 5.0), seed=1))[0]
    wav = ricker(nt, 0.005, 5.0)
    sou = np.array([[0.5 * (nx - 1) * 5.0, 50.0]], np.float32)
    rec = np.stack([np.arange(nx) * 5.0, np.full(nx, 50.0)], 1).astype(np.float32)
    desc = awe.make_desc(2, (nz, nx), (5.0, 5.0), (0.0, 0.0), nt, 0.005, nb=40, fdorder=8, dabc=1, expl=1,
                         precision=awe.FAST)
    plan = awe.Plan(desc)
    plan.set_model(vel)
    plan.set_geometry(sou, rec)
    d_wav = torch.from_numpy(wav).cuda()
    d_dat = torch.zeros((plan.nsmp, nx), dtype=torch.float32, device="cuda")
    stream = torch.cuda.Stream()

    def step():
        plan.forward_device(d_wav.data_ptr(), 1, d_dat.data_ptr(), 0, stream.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    sampler.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    ms = e0.elapsed_time(e1) / args.steps
    plan.profile(True)
    step()
    torch.cuda.synchronize()
    kern_ms, kern_n = plan.profile_read()
    plan.profile(False)
    cells = (nz + 80) * (nx + 80)
    avg = kern_ms / 1e3 / max(kern_n, 1)
    out = {"metric": "cell-updates/s (2D single-shot forward)", "value": cells * nt / (ms / 1e3),
           "unit": "cell-updates/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
           "config": {"workload": "2D %dx%d at 5 m (nb=40), 8th order, nt=%d, dabc=y, 1 source, %d receivers; "
                                  "time loop as one CUDA graph" % (nz, nx, nt, nx), "padded_cells": cells,
                      "l2": "the 1.4 MB fields stay in L2: launch- and latency-bound, no HBM claim"},
           "step_kernel_us_directly_launched": avg * 1e6, "us_per_time_step": 1e3 * ms / nt,
           "gpu_launches": plan.last_launch_count(), "clocks": clocks}
    print(json.dumps(out))
    plan.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fast", choices=["fast", "exact"])
    ap.add_argument("--nt", type=int, default=3000, help="time steps (the workload is nt=3000)")
    ap.add_argument("--n", type=int, default=512, help="model edge (the workload is 512; smaller for profiling)")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-extras", dest="extras", action="store_false",
                    help="skip the batched-gradient and spherical legs that follow the headline")
    ap.add_argument("--workload", default="fwd3d", choices=["fwd3d", "fwd2d", "grad3d", "grad2d", "batch2d", "batchgrad2d", "spher3d", "sphergrad3d"],
                    help="fwd3d: the headline forward workload; grad3d/grad2d: misfit gradients; "
                         "batch2d: the batched 2D survey")
    ap.add_argument("--shots", type=int, default=0,
                    help="shots: batch2d/batchgrad2d (default 256), spher3d (default 1; 16 on the survey track)")
    ap.add_argument("--ckpt", default="bfp16", choices=["bfp16", "bf16", "fp16", "fp32"],
                    help="checkpoint storage (grad*): bfp16 = 16-bit block floating point")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch2d":
        run_batch(args)
    elif args.workload == "batchgrad2d":
        run_batch_grad(args)
    elif args.workload == "sphergrad3d":
        run_sphergrad(args)
    elif args.workload == "spher3d":
        run_spher(args)
    elif args.workload == "fwd2d":
        run_fwd2d(args)
    elif args.workload != "fwd3d":
        run_grad(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
