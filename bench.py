#!/usr/bin/env python3
"""Benchmark of the 3D pure-qP VTI forward modeling loop on GB300.

Workload (one bench "step" = one whole shot): layered VTI model 400x400x300
cells + 30-cell PML (460x460x360 padded, 76.2 M cells), 10 m spacing, 3000
time steps of 0.5 ms, 20 Hz Ricker source at the surface centre, receivers on
the full surface, xz/yz wavefield slices every 100 steps.  Synthetic, seeded
(no field data is available); the working set (~4.8 GB) is far larger than
the 129 MB L2, so no flush is needed between steps.

Metric: Gcell-updates/s = padded cells x time steps / seconds.
  value      device time (CUDA events on the library's stream) of K shots with
             the model resident in HBM: reset + 3000 steps + slice snapshots
  e2e        the same shots through qp3d_forward (the modeling3d replacement)
             from pinned host buffers: model upload, time loop, record download
  roofline   the fused step kernel: algorithmic bytes per launch
             (24 B per interior cell + 64 B per PML cell) / its mean duration
             (CUDA events around every launch of one more shot, outside the
             timed shots), against the measured HBM copy bandwidth
  reference_arithmetic  one shot in the reference-arithmetic mode (arith=0),
             whose records equal the reference CPU operators' bit for bit
  batch, adjoint  one timed pass of the batched and gradient workloads below
             (default line, one GPU)
  cpu_baseline  the reference CPU arithmetic (oracle port of CPU_function.c,
             bit-exact to it) on all host cores, on a bounded sample

--impl reference runs only that CPU implementation, a few time steps of the
same workload per bench step.

--workload batch measures the batched path instead (one bench step = one
qp3d_batch call): 64 shots on uneven windows (hx, hy uniform in [128, 256],
Nz0 in [128, 200], 20-cell PML, 10.8 M padded cells on average) cut from one
512x512x200 layered model, 2000 steps, 15-30 Hz sources, surface receivers.
  value      batched shots/s, device time of the time loop (all groups)
  e2e        shots/s of the whole qp3d_batch call from pageable host buffers
             (model upload, time loop, record download)
  single_shot_form  the same shots one qp3d call each: device time of the
             resident time loop and wall time of qp3d_forward
Under torchrun with N ranks the shots are split into N contiguous blocks
balanced by cells x steps (shard.py), one qp3d_batch call per rank; value =
all shots / the slowest rank's time ("strong" scaling).

--workload adjoint measures the misfit gradient (qp3d_adjoint): a 12-layer
200x200x150 true model (+20-cell PML, 240x240x190 padded) and a start model
smoothed by a 3D Gaussian of 5 cells, 16 shots on a 4x4 surface grid, 2000
steps, sqrt(nt) checkpoints in FP32 (and with BF16 PML levels beside it);
value = seconds per shot of the gradient (forward, residual, checkpointed
backward), the records of the true model made first.  Beside it, the schedule
that keeps every u^k in device memory (88 GB here, no recomputation; the
library's default when it fits), whose gradient is identical.  Two library
contexts (--adj-contexts) on the GPU run two shots at a time; under torchrun
the shots are split into contiguous blocks across ranks; either way the FP64
gradient is summed on the host in shot order, bit-equal to one process
(shard.py).

--workload large measures the large mixed-precision configuration (one bench
step = one shot): 800x800x400 cells + 40-cell PML (880x880x480 padded, 372 M
cells), 20 dipping layers and 30 Gaussian velocity anomalies, 5000 steps,
with vp/eps/delta stored as FP32 and as FP16 (param_fp16), wavefields FP32.
The two full-size records are compared on every 10th step (rel-L2 and max
abs / peak of FP16 against FP32).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "gpu-c_3dqmodeling_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

WORKLOAD = dict(hx=400, hy=400, nz0=300, pml=30, nt=3000, dt=5e-4, dx=10.0, fm=20.0,
                seed=2, snap_every=100)
WORKLOAD_NAME = ("layered VTI 400x400x300 + 30-cell PML (460x460x360 padded), 12 dipping "
                 "layers seed 2, 3000 steps x 0.5 ms, 20 Hz Ricker at surface centre, "
                 "full-surface receivers, xz/yz slices every 100 steps")
REF_SAMPLE_STEPS = 2      # time steps per reference-arm bench step
CPU_SAMPLE_STEPS = 6      # time steps of the in-line CPU baseline


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="qp3d", choices=["qp3d", "reference"])
    ap.add_argument("--nt", type=int, default=None, help="override time steps (testing)")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="scale the horizontal/vertical extent (testing only)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-sub", action="store_true",
                    help="skip the batched and gradient measurements of the default line")
    ap.add_argument("--no-ref-arith", action="store_true",
                    help="skip the timed shot in the reference-arithmetic mode")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="reference arm: skip the reference GPU kernels' sample")
    ap.add_argument("--workload", default="single",
                    choices=["single", "batch", "large", "adjoint"])
    ap.add_argument("--shots", type=int, default=64,
                    help="batch workload: shots; adjoint workload: up to 16 (a square grid)")
    ap.add_argument("--adj-contexts", type=int, default=2,
                    help="adjoint workload: library contexts per GPU running shots at once")
    ap.add_argument("--spec-delta-ppm", type=int, default=None,
                    help="smallest half-width of the predicted max window (ppm)")
    return ap.parse_args()


def workload(args):
    w = dict(WORKLOAD)
    if args.nt is not None:
        w["nt"] = args.nt
    if args.scale != 1.0:
        for k in ("hx", "hy", "nz0"):
            w[k] = max(16, int(round(w[k] * args.scale)))
    return w


def make_shot(w):
    import synthetic
    return synthetic.layered_vti(hx=w["hx"], hy=w["hy"], nz0=w["nz0"], pml=w["pml"],
                                 nt=w["nt"], dx=w["dx"], dt=w["dt"], fm=w["fm"],
                                 seed=w["seed"])


def algorithmic_bytes(shot, param_bytes=4):
    """See below; param_bytes = bytes of each of vp, eps, delta per cell."""
    b, ni, npml = _algorithmic_bytes(shot)
    d = 3 * (4 - param_bytes)
    return b - d * shot.N, ni, npml


def _algorithmic_bytes(shot):
    """24 B per interior cell (read u(k), u(k-1), vp, eps, delta; write u(k+1))
    + 64 B per PML cell (u(k), vp, eps, delta, 7 state reads, 4 state writes,
    u(k+1)), over the updated box as the reference defines the layers."""
    n = shot.N
    ni = (shot.nx - 2 * shot.pml) * (shot.ny - 2 * shot.pml) * (shot.nz - 2 * shot.pml)
    return 24 * ni + 64 * (n - ni), ni, n - ni


# ---------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            backend = "nccl" if os.environ.get("QP3D_BENCH_BACKEND", "gloo") == "nccl" else "gloo"
            dist.init_process_group(backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v):
        if not self.pg:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class Clocks:
    """nvidia-smi samples (200 ms) during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, gpu_index):
        self.rows = []
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], None, set()
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
            except ValueError:
                continue
            for name, flag in zip(self.NAMES, r[3:]):
                if flag.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "samples": len(sm),
                "reasons": sorted(reasons)}


def hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_ratio():
    """DRAM bytes / algorithmic bytes of one step-kernel launch from the
    committed ncu summary (profiles/traffic.json), or None."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["qp3d_step_kernel"]["traffic_over_algorithmic"]), d["qp3d_step_kernel"].get("case")
    except Exception:
        return None, None


# ---------------------------------------------------------------------------
def cpu_sample(shot, nsteps, k0=1500, seed=0):
    """Reference CPU arithmetic (oracle REF32 port, all host threads) for
    nsteps from a dense random state; returns (seconds, threads)."""
    from oracle import oracle as O
    import synthetic
    prob = shot.to_oracle(O)
    u_prev, u_cur, pml = synthetic.random_state(shot, seed=seed)
    st = O.State(prob)
    st.u1[:] = u_prev
    st.u2[:] = u_cur
    st.pml[:] = pml
    threads = os.cpu_count() or 1
    k0 = max(0, min(k0, shot.nt - nsteps))   # the wavelet has nt samples
    t0 = time.perf_counter()
    O.run(O.REF32, prob, k0=k0, nsteps=nsteps, state=st, nthreads=threads, want_record=False)
    return time.perf_counter() - t0, threads


def repo_native_libs():
    """Shared objects of this repository mapped into the process (Linux)."""
    out = set()
    try:
        with open("/proc/self/maps") as f:
            for line in f:
                path = line.split()[-1] if line.strip() else ""
                if path.endswith(".so") and path.startswith(ROOT):
                    out.add(os.path.relpath(path, ROOT))
    except OSError:
        pass
    return sorted(out)


def reference_gpu_sample(shot, steps_dev=10, steps_host=3, seed=0):
    """The reference's own GPU kernels (GPU_kernel.cu compiled for sm_103a)
    in its driver's step sequence on cuda:0, from a dense random state: Gcell/s
    with the step max taken on the device, and as the reference's driver does
    it (full D2H copies of ux, uy, uz and u2 every step, host scan)."""
    from oracle import oracle as O
    import synthetic
    if not O.ref_gpu_available():
        return {"unavailable": "reference GPU kernels were not compiled (no checkout)"}
    try:
        prob = shot.to_oracle(O)
        u_prev, u_cur, pml = synthetic.random_state(shot, seed=seed)
        out = {"kind": "reference", "source": "GPU_kernel.cu unmodified, nvcc -cubin sm_103a",
               "unit": "Gcell/s", "workload": WORKLOAD_NAME}
        for key, n, host in (("device_max", steps_dev, False), ("host_max", steps_host, True)):
            st = O.State(prob)
            st.u1[:] = u_prev
            st.u2[:] = u_cur
            st.u3[:] = u_cur
            st.pml[:] = pml
            k0 = max(0, min(1500, shot.nt - n))
            O.run_reference_gpu(prob, k0=k0, nsteps=1, state=st.copy(), host_max=host,
                                want_record=False)   # warm-up (module load, first launches)
            _, _, _, ms = O.run_reference_gpu(prob, k0=k0, nsteps=n, state=st, host_max=host,
                                              want_record=False)
            out[key] = {"value": round(shot.N * n / (ms * 1e-3) / 1e9, 4), "steps": n,
                        "ms_per_step": round(ms / n, 3)}
        out["device_max"]["form"] = ("grad, scalar_operator, wavefield_update, addsource, "
                                     "exchange per step; max by a device reduction; record "
                                     "plane copied to the host")
        out["host_max"]["form"] = ("as 3dPureqPModeling_single_shot.cu:282-337: ux, uy, uz "
                                   "and u2 copied to the host every step, max scanned there")
        return out
    except Exception as e:   # no usable GPU in this process
        return {"unavailable": str(e).splitlines()[0][:200]}


def run_reference_arm(args, dist):
    if dist.rank != 0:
        return 0
    import synthetic
    # inputs from the oracle's restatements of the host utilities: this
    # process must not load the library it is compared with
    synthetic.set_backend("oracle")
    w = workload(args)
    shot = make_shot(w)
    cells = shot.N
    times = []
    threads = os.cpu_count() or 1
    for i in range(args.warmup + args.steps):
        dt, threads = cpu_sample(shot, REF_SAMPLE_STEPS, k0=1500 + i, seed=i)
        if i >= args.warmup:
            times.append(dt)
    total = sum(times)
    value = cells * REF_SAMPLE_STEPS * args.steps / total / 1e9
    sample = ("%d time steps of the %dx%dx%d padded grid per bench step, from a dense random "
              "state, oracle port of CPU_function.c (bit-exact to it), OpenMP %d threads" %
              (REF_SAMPLE_STEPS, shot.nx, shot.ny, shot.nz, threads))
    line = {
        "impl": "reference", "metric": "Gcell-updates/s", "value": round(value, 6),
        "unit": "Gcell/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * total / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD_NAME, "step": "bounded sample: %d time steps" %
                   REF_SAMPLE_STEPS, "cells": cells, "parallelism": "host threads"},
        "cpu_baseline": {"value": round(value, 6), "unit": "Gcell/s", "cores": threads,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 6), "unit": "Gcell/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "native_libs": repo_native_libs(),
    }
    if not args.no_reference_gpu:
        line["reference_gpu"] = reference_gpu_sample(shot)
        line["native_libs"] = repo_native_libs()
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
def run_gpu_arm(args, dist):
    import qp3d
    w = workload(args)
    shot = make_shot(w)
    nt = shot.nt
    cells = shot.N
    dev = dist.local
    ctx = qp3d.Context(dev)
    snap = qp3d.make_snap(lambda step, kind, arr: 0, w["snap_every"], [qp3d.SNAP_XZ, qp3d.SNAP_YZ])
    every = w["snap_every"]
    snaps_per_shot = len(range(0, nt, every))

    def one_shot(per_kernel):
        """reset + nt steps + slices; returns (ms_step_kernel, ms_gradmax) sums."""
        ctx.reset()
        k, ms_s, ms_g = 0, 0.0, 0.0
        while k < nt:
            nxt = k if k % every == 0 else (k // every + 1) * every
            n = min(nt - k, nxt - k + 1)
            if per_kernel:
                _, a, b = ctx.time(n, per_kernel=True)
                ms_s += a
                ms_g += b
            else:
                ctx.advance(n)
            k += n
            if (k - 1) % every == 0:
                ctx.snapshot(snap)
        return ms_s, ms_g

    ctx.load(shot)
    for _ in range(args.warmup):
        one_shot(False)
    ctx.sync()
    dist.barrier()
    gpu_index = (os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[dev]
                 if os.environ.get("CUDA_VISIBLE_DEVICES") else dev)
    clocks = Clocks(gpu_index)
    launches0 = ctx.launch_count()
    ctx.event(0)
    for _ in range(args.steps):
        one_shot(False)
    ctx.event(1)
    ctx.sync()
    ms = ctx.elapsed(0, 1)
    clk = clocks.stop()
    dist.barrier()
    ms = dist.max(ms)
    value = dist.world * cells * nt * args.steps / (ms / 1e3) / 1e9
    gpu_launches = ctx.launch_count() - launches0
    redo, alt = ctx.stats(0, nt)
    # the step kernel's own duration: one more shot with events around every
    # launch (kept out of the timed shots, whose loop it would slow)
    ms_step, ms_grad = one_shot(True)

    # roofline of the fused step kernel (one launch = one time step)
    bstep, ni, np_ = algorithmic_bytes(shot)
    n_launch = nt
    t_step = ms_step / n_launch / 1e3
    achieved = bstep / t_step / 1e9
    peak, peak_kind = hbm_peak()
    tratio, tcase = traffic_ratio()
    roofline = {"bound": "hbm", "kernel": "qp3d_step_kernel", "achieved": round(achieved, 1),
                "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "peak_kind": peak_kind + " copy bandwidth (MEASURED_PEAKS.json hbm_gbs)"
                if peak_kind == "measured" else "fallback 6.8 TB/s",
                "algorithmic_bytes_per_launch": bstep,
                "traffic": (round(tratio * bstep) if tratio else None),
                "traffic_note": ("ncu dram read+write of one launch on %s, scaled to this grid by "
                                 "its algorithmic bytes" % tcase) if tratio else
                                "no ncu capture committed",
                "step_kernel_ms": round(ms_step / n_launch, 5),
                "threshold_overhead_ms": round(ms_grad / n_launch, 5),
                "threshold_note": "per step: gradmax pre-pass for the first 3 steps, then the "
                                  "resolution and deferred-cell compaction kernel and the "
                                  "fix-up (or, when the max left the window, the exact re-run) "
                                  "of the speculative step; last shot: "
                                  "%d re-runs in %d steps, max %d deferred cells per step" %
                                  (int(redo.sum()), nt, int(alt.max()))}

    # end to end through the C ABI from pinned host memory
    pin = {}
    for key in ("vp", "eps", "delta", "src", "wavelet"):
        a = getattr(shot, key)
        pa = qp3d.PinnedArray(a.shape)
        pa.array[:] = a
        pin[key] = pa
    rec = qp3d.PinnedArray((nt, shot.hx, shot.hy))
    pshot = qp3d.Shot(shot.nx, shot.ny, shot.nz, shot.pml, shot.sz, shot.dx, shot.dy, shot.dz,
                      shot.dt, pin["vp"].array, pin["eps"].array, pin["delta"].array,
                      pin["src"].array, pin["wavelet"].array, shot.prof, shot.c, shot.c2)
    ctx.forward(pshot, snap=snap, record=rec.array)     # warm-up
    dist.barrier()
    clocks_e2e = Clocks(gpu_index)
    per_shot = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t1 = time.perf_counter()
        ctx.forward(pshot, snap=snap, record=rec.array)
        per_shot.append(round((time.perf_counter() - t1) * 1e3, 1))
    e2e_s = dist.max(time.perf_counter() - t0)
    clk_e2e = clocks_e2e.stop()
    # its parts: the upload and set-up of the model (qp3d_shot_load from the
    # same page-locked buffers), after which the time loop and the record run
    load_ms = []
    for _ in range(3):
        t1 = time.perf_counter()
        ctx.load(pshot)
        ctx.sync()
        load_ms.append((time.perf_counter() - t1) * 1e3)
    e2e = dist.world * cells * nt * args.steps / e2e_s / 1e9
    h2d = 3 * cells * 4 + nt * 4 + 6 * shot.pml * 4 + 2 * 36 * 4
    d2h = nt * shot.hx * shot.hy * 4 + snaps_per_shot * (shot.nz - 2 * shot.pml) * (shot.hx + shot.hy) * 4

    # the same shot in the reference-arithmetic mode (bit-identical to the
    # reference CPU operators), one timed shot after one untimed
    ref_arith = None
    if not args.no_ref_arith:
        ctx.tune(arith=0)
        one_shot(False)
        ctx.sync()
        ctx.event(2)
        ms_rs, _ = one_shot(True)
        ctx.event(3)
        ctx.sync()
        ms_r = ctx.elapsed(2, 3)
        ctx.tune(arith=1)
        ref_arith = {"value": round(cells * nt / (ms_r / 1e3) / 1e9, 3), "unit": "Gcell/s",
                     "ms_per_shot": round(ms_r, 2),
                     "step_kernel_ms": round(ms_rs / nt, 5),
                     "step_kernel_frac_of_peak": round(bstep / (ms_rs / nt / 1e3) / 1e9 / peak, 4),
                     "note": "the reference CPU operators' roundings operation by operation "
                             "(tuning key arith=0): records equal CPU_function.c's bit for bit"}

    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        secs, threads = cpu_sample(shot, CPU_SAMPLE_STEPS)
        cpu = {"value": round(cells * CPU_SAMPLE_STEPS / secs / 1e9, 6), "unit": "Gcell/s",
               "cores": threads, "kind": "port",
               "sample": "%d time steps of this grid from a dense random state; oracle port of "
                         "CPU_function.c (bit-exact to it), OpenMP" % CPU_SAMPLE_STEPS}

    subs = {}
    if dist.world == 1 and not args.no_sub:
        subs["batch"] = batch_summary(ctx)
        subs["adjoint"] = adjoint_summary(ctx)

    if dist.rank == 0:
        line = {
            "metric": "Gcell-updates/s", "value": round(value, 3), "unit": "Gcell/s",
            "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD_NAME, "step": "one shot of %d time steps" % nt,
                       "grid": [shot.nx, shot.ny, shot.nz], "cells": cells,
                       "interior_cells": ni, "pml_cells": np_, "nt": nt,
                       "l2": "inputs larger than L2 (working set %.1f GB)" %
                             (15 * cells * 4 / 1e9),
                       "parallelism": "replicas" if dist.world > 1 else "single"},
            "roofline": roofline,
            "reference_arithmetic": ref_arith,
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e, 3), "unit": "Gcell/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": round(1000 * e2e_s / args.steps, 2),
                    "ms_per_shot": per_shot, "load_ms": round(min(load_ms), 1),
                    "clocks": clk_e2e,
                    "note": "qp3d_forward from page-locked host buffers, every step: the "
                            "parameter volumes to the device, the time loop, the record "
                            "streamed back during the loop and the xz/yz slices"},
            "gpu_launches": gpu_launches,
            "clocks": clk,
        }
        line.update(subs)
        print(json.dumps(line), flush=True)
    for p in list(pin.values()) + [rec]:
        p.free()
    ctx.close()
    return 0


BATCH_NAME = ("%d shots, windows hx,hy U[128,256], Nz0 U[128,200] (+20-cell PML) cut from a "
              "512x512x200 layered VTI model (12 dipping layers, seed 3), %d steps x 0.5 ms, "
              "15-30 Hz Ricker at each window's surface centre, surface receivers")


def run_batch_arm(args, dist):
    import qp3d
    import synthetic
    import shard
    nt = args.nt if args.nt is not None else 2000
    all_shots = synthetic.batch_shots(nshots=args.shots, nt=nt)
    # ranks take contiguous blocks of the shot list, balanced by cells x steps
    blocks = shard.partition([shard.shot_cost(s) for s in all_shots], dist.world)
    blk_a, blk_b = blocks[dist.rank]
    shots = all_shots[blk_a:blk_b]
    cells = [s.N for s in all_shots]
    work = sum(c * nt for c in cells)
    ctx = qp3d.Context(dist.local)
    if args.spec_delta_ppm is not None:
        ctx.tune(spec_delta_ppm=args.spec_delta_ppm)
    records = [np.empty((s.nt, s.hx, s.hy), np.float32) for s in shots]
    for _ in range(args.warmup):
        if shots:
            ctx.batch(shots, records)
    dist.barrier()
    gpu_index = (os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[dist.local]
                 if os.environ.get("CUDA_VISIBLE_DEVICES") else dist.local)
    clocks = Clocks(gpu_index)
    launches0 = ctx.launch_count()
    run_ms, wall = 0.0, 0.0
    st = {}
    for _ in range(args.steps):
        t0 = time.perf_counter()
        if shots:
            ctx.batch(shots, records)
            st = ctx.batch_stats()
            run_ms += st["run_ms"]
        wall += time.perf_counter() - t0
    clk = clocks.stop()
    gpu_launches = ctx.launch_count() - launches0
    run_ms = dist.max(run_ms)
    wall = dist.max(wall)
    n = len(all_shots) * args.steps
    value = n / (run_ms / 1e3)
    e2e = n / wall

    # the same shots one call each
    ms_single, wall_single = 0.0, 0.0
    for s in shots:
        ctx.load(s)
        ms_single += ctx.time(s.nt, per_kernel=False)[0]
    t0 = time.perf_counter()
    for s, r in zip(shots, records):
        ctx.forward(s, record=r)
    wall_single = time.perf_counter() - t0
    ms_single = dist.max(ms_single)
    wall_single = dist.max(wall_single)

    # whole-step HBM rate of the batched time loop (algorithmic bytes of all
    # shots per step / device time per step)
    bsum = sum(algorithmic_bytes(s)[0] for s in all_shots)
    peak, peak_kind = hbm_peak()
    achieved = bsum / (run_ms / args.steps / nt / 1e3) / 1e9
    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        secs, threads = cpu_sample(all_shots[0], CPU_SAMPLE_STEPS, k0=nt // 2)
        rate = all_shots[0].N * CPU_SAMPLE_STEPS / secs
        cpu = {"value": round(rate / (work / len(all_shots)), 6), "unit": "shots/s",
               "cores": threads,
               "kind": "port",
               "sample": "%d time steps of shot 0 (%dx%dx%d) from a dense random state, oracle "
                         "port of CPU_function.c, OpenMP; shots/s = cell rate / mean cells x nt"
                         % (CPU_SAMPLE_STEPS, all_shots[0].nx, all_shots[0].ny,
                            all_shots[0].nz)}
    if dist.rank == 0:
        line = {
            "metric": "batched shots/s", "value": round(value, 4), "unit": "shots/s",
            "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(run_ms / args.steps, 2), "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": BATCH_NAME % (len(all_shots), nt),
                       "step": "one qp3d_batch call per rank over its block of the shots",
                       "shots": len(all_shots), "nt": nt, "cells_total": sum(cells),
                       "cells_mean": round(sum(cells) / len(cells)),
                       "l2": "inputs larger than L2 (working set %.0f GB)" %
                             (sum(17 * c * 4 for c in cells) / 1e9),
                       "parallelism": ("shots split into %d contiguous blocks balanced by "
                                       "cells x steps, one per rank, no exchange"
                                       % dist.world) if dist.world > 1 else "single",
                       "blocks": blocks},
            "gcell_per_s": round(work * args.steps / (run_ms / 1e3) / 1e9, 3),
            "step_roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                              "unit": "GB/s", "frac": round(achieved / peak, 4),
                              "note": "algorithmic bytes of all shots per time step / device "
                                      "time per step (all kernels of the step)"},
            "batch": st,
            "single_shot_form": {
                "value": round(len(all_shots) / (ms_single / 1e3), 4), "unit": "shots/s",
                "e2e": round(len(all_shots) / wall_single, 4),
                "note": "same shots, one call each: device time of the resident time loop "
                        "(qp3d_shot_load + nt steps), and wall time of qp3d_forward"},
            "cpu_baseline": cpu,
            "e2e": {"value": round(e2e, 4), "unit": "shots/s",
                    "h2d_bytes_per_step": sum(4 * (3 * c) + 4 * nt for c in cells),
                    "d2h_bytes_per_step": sum(4 * nt * s.hx * s.hy for s in all_shots),
                    "note": "pageable host buffers"},
            "gpu_launches": gpu_launches,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def batch_summary(ctx, nshots=64, nt=2000):
    """One timed qp3d_batch pass of the batched workload (after one untimed
    pass, which also tunes the tile shape), beside the same shots as one
    qp3d_shot_load + nt steps each (the one-shot-per-launch form); records of
    both forms compared bit for bit on the first shots."""
    import synthetic
    shots = synthetic.batch_shots(nshots=nshots, nt=nt)
    records = [np.empty((s.nt, s.hx, s.hy), np.float32) for s in shots]
    ctx.batch(shots, records)
    ctx.batch(shots, records)
    st = ctx.batch_stats()
    run_ms = st["run_ms"]
    ms_single = 0.0
    for s in shots:
        ctx.load(s)
        ms_single += ctx.time(s.nt, per_kernel=False)[0]
    same = all(np.array_equal(ctx.forward(s).view(np.uint32), r.view(np.uint32))
               for s, r in zip(shots[:4], records[:4]))
    bsum = sum(algorithmic_bytes(s)[0] for s in shots)
    peak, _ = hbm_peak()
    achieved = bsum / (run_ms / nt / 1e3) / 1e9
    return {"metric": "batched shots/s", "value": round(len(shots) / (run_ms / 1e3), 4),
            "unit": "shots/s", "workload": BATCH_NAME % (len(shots), nt),
            "one_shot_per_launch": round(len(shots) / (ms_single / 1e3), 4),
            "speedup": round(ms_single / run_ms, 3),
            "step_roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                              "unit": "GB/s", "frac": round(achieved / peak, 4)},
            "records_bit_identical_to_qp3d_forward": same,
            "tuned_shape": {"tile_rows": st["tile_rows"], "zblocks": st["zblocks"]},
            "note": "device time of the time loop (CUDA events) for both forms; the batched "
                    "records equal the one-call records bit for bit (checked on 4 shots)"}


ADJ_CONTEXTS = 2   # library contexts (streams) per GPU running gradient shots at once


def gradient_contexts(device, n):
    import qp3d
    return [qp3d.Context(device) for _ in range(n)]


def timed_gradient(ctxs, start, d_obs, keep):
    """Gradient of all shots through shard.gradient with one shot per
    context at a time (the FP64 sum in shot order); (s per shot, J, grads)."""
    import shard
    fns = []
    for c in ctxs:
        c.tune(adj_keep_all=keep)
        fns.append(lambda i, s, out, c=c: c.adjoint(s, d_obs[i], out)[0])
    for c in ctxs:   # first call of each context: buffers and schedule
        c.adjoint(start[0], d_obs[0])
    t0 = time.perf_counter()
    J, grads = shard.gradient(start, fns if len(fns) > 1 else fns[0],
                              group=shard.Group())
    return (time.perf_counter() - t0) / len(start), J, grads


def adjoint_summary(ctx, grid=4, nt=2000):
    """Misfit gradient of the 16-shot gradient workload with the library's
    default schedule (every u^k kept when they fit in device memory), and
    with the sqrt(nt) checkpoint schedule in its default storage (BF16 PML
    levels, the forward's threshold decisions replayed), beside the forward
    alone of the same shots; the checkpointed gradient's cosine against the
    kept one (FP32 checkpoints give the kept gradient bit for bit).  Two
    library contexts run two shots at a time (the adjoint passes are
    latency-bound: one context per GPU measured 1.23 s per shot, two 1.07)."""
    import synthetic
    true, start = synthetic.adjoint_case(nt=nt, grid=grid)
    d_obs = [ctx.forward(s).copy() for s in true]
    ctxs = gradient_contexts(ctx.device, ADJ_CONTEXTS)
    try:
        sec, J, g_keep = timed_gradient(ctxs, start, d_obs, -1)
        sec_ck, J_ck, g_ck = timed_gradient(ctxs, start, d_obs, 0)
    finally:
        for c in ctxs:
            c.close()
    cos = [float(np.dot(a, b) / (np.linalg.norm(a) * np.linalg.norm(b)))
           for a, b in zip(g_ck, g_keep)]
    ctx.load(start[0])
    t_fwd = ctx.time(nt, per_kernel=False)[0] / 1e3
    return {"metric": "adjoint grad s/shot", "value": round(sec, 4), "unit": "s/shot",
            "higher_is_better": False, "workload": ADJ_NAME % (len(start), nt),
            "forward_only_s_per_shot": round(t_fwd, 4),
            "schedule": "default (every u^k kept when nt wavefields fit in device memory); "
                        "%d library contexts on the GPU, one shot each at a time" % ADJ_CONTEXTS,
            "misfit": J,
            "checkpointed": {"s_per_shot": round(sec_ck, 4), "misfit": J_ck,
                             "schedule": "ceil(sqrt(nt)) checkpoints, PML levels in BF16, "
                                         "threshold decisions of the forward replayed",
                             "cosine_vs_kept": {"vp": round(cos[0], 6), "eps": round(cos[1], 6),
                                                "delta": round(cos[2], 6)}},
            "operator": "live (S's dependence on grad u differentiated; threshold decisions "
                        "held)",
            "accuracy": "gradient cosine against the FP64 CPU adjoint 1.000000 for vp, eps and "
                        "delta on the test case; vp directional derivative within 1.4e-5 of "
                        "converged FP64 central differences of the live forward "
                        "(tests/test_adjoint.py)"}


LARGE_NAME = ("anomalous layered VTI 800x800x400 + 40-cell PML (880x880x480 padded), 20 dipping "
              "layers + 30 Gaussian vp anomalies (+-15%%, sigma 10-40 cells) seed 5, %d steps x "
              "0.5 ms, 20 Hz Ricker at surface centre, full-surface receivers")


def run_large_arm(args, dist):
    import qp3d
    import synthetic
    nt = args.nt if args.nt is not None else 5000
    shot = synthetic.large_vti(nt=nt)
    cells = shot.N
    ctx = qp3d.Context(dist.local)
    gpu_index = (os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[dist.local]
                 if os.environ.get("CUDA_VISIBLE_DEVICES") else dist.local)
    peak, peak_kind = hbm_peak()
    runs = {}
    rec_sample = {}
    launches0 = ctx.launch_count()
    clocks = Clocks(gpu_index)
    for name, fp16 in (("fp32_params", 0), ("fp16_params", 1)):
        ctx.tune(param_fp16=fp16)
        ctx.load(shot)
        for _ in range(args.warmup):
            ctx.reset()
            ctx.advance(nt)
        ctx.sync()
        tot = ms_s = 0.0
        for _ in range(args.steps):
            ctx.reset()
            t, s, _ = ctx.time(nt)
            tot += t
            ms_s += s
        # every 10th record step of the full-size run, for the FP16 vs FP32
        # comparison (outside the timed region)
        rec_sample[name] = np.stack([ctx.record(k, 1)[0] for k in range(0, nt, 10)])
        bstep = algorithmic_bytes(shot, 2 if fp16 else 4)[0]
        t_step = ms_s / (nt * args.steps) / 1e3
        runs[name] = {"value": round(cells * nt * args.steps / (tot / 1e3) / 1e9, 3),
                      "ms_per_step": round(tot / args.steps, 2),
                      "step_kernel_ms": round(ms_s / (nt * args.steps), 5),
                      "roofline": {"bound": "hbm", "achieved": round(bstep / t_step / 1e9, 1),
                                   "peak": peak, "unit": "GB/s",
                                   "frac": round(bstep / t_step / 1e9 / peak, 4),
                                   "algorithmic_bytes_per_launch": bstep}}
    clk = clocks.stop()
    gpu_launches = ctx.launch_count() - launches0
    a32, a16 = rec_sample["fp32_params"], rec_sample["fp16_params"]
    num = den = 0.0
    dmax = pmax = 0.0
    for p32, p16 in zip(a32, a16):
        d = p16.astype(np.float64) - p32
        num += float(np.sum(d * d))
        den += float(np.sum(p32.astype(np.float64) ** 2))
        dmax = max(dmax, float(np.max(np.abs(d))))
        pmax = max(pmax, float(np.max(np.abs(p32))))
    fp16_vs_fp32 = {
        "rel_l2": (num / den) ** 0.5 if den > 0 else None,
        "max_abs_over_peak": dmax / pmax if pmax > 0 else None,
        "sampled": "record planes of every 10th step (%d of %d), full %dx%d surface"
                   % (a32.shape[0], nt, a32.shape[1], a32.shape[2])}
    if dist.rank == 0:
        line = {
            "metric": "Gcell-updates/s", "value": runs["fp16_params"]["value"], "unit": "Gcell/s",
            "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": runs["fp16_params"]["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 (params f16)",
            "data": "synthetic",
            "config": {"workload": LARGE_NAME % nt, "step": "one shot of %d time steps" % nt,
                       "grid": [shot.nx, shot.ny, shot.nz], "cells": cells, "nt": nt,
                       "l2": "inputs larger than L2", "parallelism": "single"},
            "runs": runs,
            "fp16_vs_fp32_record": fp16_vs_fp32,
            "gpu_launches": gpu_launches,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    return 0


ADJ_NAME = ("misfit gradient: 12-layer 200x200x150 true model (+20-cell PML), start model "
            "smoothed by a 3D Gaussian (sigma 5 cells), %d shots on a 4x4 surface grid, %d "
            "steps x 0.5 ms, 20 Hz, surface receivers, sqrt(nt) checkpoints")


def run_adjoint_arm(args, dist):
    import qp3d
    import synthetic
    nt = args.nt if args.nt is not None else 2000
    grid = 4 if args.shots >= 16 else max(1, int(round(args.shots ** 0.5)))   # grid x grid shots
    import shard
    true, start = synthetic.adjoint_case(nt=nt, grid=grid)
    # ranks take contiguous blocks of the shots; the FP64 gradient is summed
    # across them in shot order (bit-equal to one process)
    blocks = shard.partition([shard.shot_cost(s) for s in start], dist.world)
    blk_a, blk_b = blocks[dist.rank]
    ctx = qp3d.Context(dist.local)
    d_obs = {i: ctx.forward(true[i]).copy() for i in range(blk_a, blk_b)}
    res = {}
    gpu_index = (os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[dist.local]
                 if os.environ.get("CUDA_VISIBLE_DEVICES") else dist.local)

    # contexts (streams) on this rank's GPU running gradient shots at once
    ctxs = [ctx] + gradient_contexts(dist.local, max(1, args.adj_contexts) - 1)
    fns = [lambda i, s, out, c=c: c.adjoint(s, d_obs[i], out)[0] for c in ctxs]

    clocks = Clocks(gpu_index)
    launches0 = sum(c.launch_count() for c in ctxs)
    for name, bf16, keep in (("fp32_checkpoints", 0, 0), ("bf16_pml_checkpoints", 1, 0),
                             ("keep_all", 0, 1)):
        for c in ctxs:
            c.tune(adj_ckpt_bf16=bf16, adj_keep_all=keep)
        for _ in range(args.warmup):
            if blk_b > blk_a:
                for c in ctxs:
                    c.adjoint(start[blk_a], d_obs[blk_a])
        dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            J, grads = shard.gradient(start, fns if len(fns) > 1 else fns[0])
        sec = dist.max(time.perf_counter() - t0)
        res[name] = {"s_per_shot": round(sec / (args.steps * len(start)), 4),
                     "misfit": J, "grads": grads}
    clk = clocks.stop()
    gpu_launches = sum(c.launch_count() for c in ctxs) - launches0
    for c in ctxs[1:]:
        c.close()
    cos = {}
    for i, p in enumerate(("vp", "eps", "delta")):
        a, b = res["bf16_pml_checkpoints"]["grads"][i], res["fp32_checkpoints"]["grads"][i]
        cos[p] = round(float(np.dot(a, b) / (np.linalg.norm(a) * np.linalg.norm(b))), 6)
    keep_same = all(np.array_equal(a, b) for a, b in zip(res["keep_all"]["grads"],
                                                          res["fp32_checkpoints"]["grads"]))
    ctx.load(start[blk_a] if blk_b > blk_a else start[0])
    tot, _, _ = ctx.time(nt, per_kernel=False)
    t_fwd = tot / 1e3
    if dist.rank == 0:
        line = {
            "metric": "adjoint grad s/shot", "value": res["fp32_checkpoints"]["s_per_shot"],
            "unit": "s/shot", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * res["fp32_checkpoints"]["s_per_shot"]
                                                        * len(start), 1),
            "higher_is_better": False, "scaling": "strong", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": ADJ_NAME % (len(start), nt),
                       "step": "gradient of all %d shots" % len(start),
                       "grid": [start[0].nx, start[0].ny, start[0].nz], "nt": nt,
                       "parallelism": ("shots split into %d contiguous blocks, one per rank; "
                                       "FP64 gradient summed across ranks on the host in shot "
                                       "order (gloo)" % dist.world) if dist.world > 1
                       else "single",
                       "contexts_per_gpu": len(ctxs),
                       "blocks": blocks},
            "bf16_pml_checkpoints_s_per_shot": res["bf16_pml_checkpoints"]["s_per_shot"],
            "keep_all_s_per_shot": res["keep_all"]["s_per_shot"],
            "keep_all_gradient_identical": keep_same,
            "forward_only_s_per_shot": round(t_fwd, 4),
            "misfit": res["fp32_checkpoints"]["misfit"],
            "cosine_bf16_pml_vs_fp32_checkpoints": cos,
            "e2e": {"value": res["fp32_checkpoints"]["s_per_shot"], "unit": "s/shot",
                    "note": "host model in, host FP64 gradient out"},
            "gpu_launches": gpu_launches,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def main():
    args = parse()
    dist = Dist()
    try:
        if args.impl == "reference":
            return run_reference_arm(args, dist)
        if args.workload == "batch":
            return run_batch_arm(args, dist)
        if args.workload == "large":
            return run_large_arm(args, dist)
        if args.workload == "adjoint":
            return run_adjoint_arm(args, dist)
        return run_gpu_arm(args, dist)
    finally:
        dist.close()


if __name__ == "__main__":
    sys.exit(main())
