#!/usr/bin/env python3
"""Benchmark: NU points*coils/s for forward+adjoint SENSE NUFFT on one GB300.

Workload (the metric's configuration): 2D SENSE, batch 4, 16 coils, image
320x320 complex64 N(0,1), grid 640x640, numpoints 6, table_oversamp 1024,
golden-angle radial trajectory 404 spokes x 640 samples (258,560 points),
smooth Gaussian-bump coil maps normalised to sum_c |s_c|^2 = 1. Synthetic,
seeded data (no dataset involved).

A step is one forward NUFFT of the batch followed by one adjoint NUFFT of the
forward's output; the work of a step is B*C*M points*coils (counted once per
forward+adjoint pair). Every step touches > 129 MB (the L2 size), so no L2
flush is inserted between steps.

  value : device-resident inputs, timed with CUDA events around K steps.
  e2e   : the public API (KbNufft / KbNufftAdjoint modules) with the image in
          pinned host memory: H2D copy of the image, forward, adjoint, D2H copy
          of the result image, every step.
  roofline: algorithmic bytes of the dominant hand-written kernel / its
          CUDA-event duration, against the measured HBM copy bandwidth.
  cpu_baseline: the CPU port of the reference table path on a bounded sample.

``--impl reference`` times the CPU port of the reference path on the host
cores on the same workload definition and prints the same line with
``"impl": "reference"``. ``--impl reference-gpu`` times the unmodified
reference (installed in baseline/_ref) through its own modules on the GPU, a
second comparator.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

B, C, N, SPOKES, READ = 4, 16, 320, 404, 640
# kernels of this library per timed step: forward FFT (row pass + column
# pass), gather, adjoint (split-tile zeroing + register scatter + exact pass
# for the linear-phase form's left-out points; the per-point factor pre-pass
# runs once per layout and tables, before the timed steps), inverse FFT
# (column pass + row pass)
LAUNCHES_PER_STEP = 8
METRIC = "NU points*coils/s (forward+adjoint SENSE NUFFT, 2D 320^2, 16 coils, batch 4)"
UNIT = "points*coils/s"


# ---------------------------------------------------------------- workload


def golden_angle_traj(spokes: int, readout: int) -> np.ndarray:
    """(2, spokes*readout) float32, rows (ky, kx), readout endpoint excluded."""
    ga = np.deg2rad(180.0 / ((1 + np.sqrt(5.0)) / 2))
    r = np.linspace(-np.pi, np.pi, readout + 1)[:-1]
    theta = np.arange(spokes) * ga
    ky = np.sin(theta)[:, None] * r[None, :]
    kx = np.cos(theta)[:, None] * r[None, :]
    return np.stack((ky.reshape(-1), kx.reshape(-1))).astype(np.float32)


def ring_smaps(ncoil: int, n: int, batch: int, seed: int) -> np.ndarray:
    """Complex Gaussian bumps centred on a ring (radius 0.35 n, width 0.4 n),
    a linear phase per coil, normalised so that sum_c |s_c|^2 = 1."""
    rng = np.random.default_rng(seed)
    y, x = np.meshgrid(np.arange(n) - n / 2, np.arange(n) - n / 2, indexing="ij")
    out = np.empty((batch, ncoil, n, n), dtype=np.complex64)
    for b in range(batch):
        rot = rng.uniform(0, 2 * np.pi)
        maps = []
        for c in range(ncoil):
            ang = rot + 2 * np.pi * c / ncoil
            cx, cy = 0.35 * n * np.cos(ang), 0.35 * n * np.sin(ang)
            mag = np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * (0.4 * n) ** 2))
            ph = np.exp(1j * (np.pi / n) * (np.cos(ang) * x + np.sin(ang) * y) + 1j * ang)
            maps.append(mag * ph)
        maps = np.stack(maps)
        maps /= np.sqrt(np.sum(np.abs(maps) ** 2, axis=0, keepdims=True))
        out[b] = maps
    return out


def make_inputs(seed: int = 1002):
    rng = np.random.default_rng(seed)
    image = (rng.standard_normal((B, 1, N, N)) + 1j * rng.standard_normal((B, 1, N, N))).astype(np.complex64)
    return image, ring_smaps(C, N, B, seed + 1), golden_angle_traj(SPOKES, READ)


def algorithmic_bytes(M: int):
    G = 2 * N
    cb = 8
    gather = B * C * G * G * cb + B * C * M * cb + 2 * M * 4 + M * 4
    scatter = B * C * M * cb + B * C * G * G * cb + 2 * M * 4 + M * 4
    fwd = cb * (B * N * N + B * C * N * N + B * C * G * G + 2 * B * C * G * G + B * C * G * G + B * C * M) + 4 * 2 * M
    adj = cb * (B * C * M + B * C * G * G + 2 * B * C * G * G + B * C * N * N + B * C * N * N + B * N * N) + 4 * 2 * M
    return {"gather": gather, "scatter": scatter, "forward": fwd, "adjoint": adj}


# ---------------------------------------------------------------- helpers


def measured_peak_gbs():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kernel: str):
    """Per-launch DRAM bytes for `kernel` at this workload, from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "dram_traffic_2d_sense_320.json")
    try:
        with open(path) as f:
            return json.load(f).get(kernel)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clock / throttle-reason sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join("/tmp", f"tkbn_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[4], parts[5:9]))
                except ValueError:
                    continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        smax = max(r[1] for r in rows)
        loaded = [r for r in rows if r[2] > 200.0] or rows
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in loaded for i, v in enumerate(r[4]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in loaded), "sm_max_mhz": smax, "reasons": reasons,
                "samples": len(rows), "samples_under_load": len(loaded)}


def dist_setup():
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 and not dist.is_initialized():
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int, device) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- CPU baseline (port of the reference path)


def rel_l2(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def cpu_full_step(image, smaps, omega):
    """One forward+adjoint of the reference table path (CPU port) on the full
    workload: all B images, all C coils, the full trajectory. Returns
    (k-space data, adjoint image)."""
    from oracle import cpu_baseline

    return cpu_baseline.forward_adjoint(image, smaps, omega)


def cpu_baseline_leg(image, smaps, omega, reps: int = 2):
    """Times the CPU port on the full workload (min of ``reps`` steps after
    one untimed step); returns the cpu_baseline object and the untimed step's
    outputs (the parity reference)."""
    from oracle import cpu_baseline

    ref = cpu_full_step(image, smaps, omega)
    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        cpu_full_step(image, smaps, omega)
        times.append(time.perf_counter() - t0)
    t = min(times)
    M = omega.shape[1]
    work = image.shape[0] * smaps.shape[1] * M
    return {"value": work / t, "unit": UNIT, "cores": cpu_baseline.threads(), "kind": "port",
            "sample": f"the full workload (batch {image.shape[0]}, {smaps.shape[1]} coils, {M} points) per step; "
                      f"min of {reps} forward+adjoint steps ({t:.3f} s each) after one untimed; "
                      f"{cpu_baseline.describe()}"}, ref


# ---------------------------------------------------------------- arms


def run_reference(args):
    world, rank, local = dist_setup()
    if rank != 0:
        return
    image, smaps, omega = make_inputs()
    from oracle import cpu_baseline

    M = omega.shape[1]
    for _ in range(args.warmup):
        cpu_full_step(image, smaps, omega)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_full_step(image, smaps, omega)
    dt = (time.perf_counter() - t0) / args.steps
    work = B * C * M
    value = work / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": {"workload": "2D SENSE NUFFT fwd+adj, image 320x320, grid 640x640, J=6, L=1024, 16 coils, "
                               "batch 4, golden-angle 404x640 (258560 points)", "same_config": True,
                   "work_per_step": work},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cpu_baseline.threads(), "kind": "port",
                         "sample": f"the full workload (batch {B}, {C} coils, {M} points) every step; "
                                   f"{cpu_baseline.describe()}"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def run_gpu(args):
    import torch

    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import torchkbnufft_gb300 as tkbn
    from torchkbnufft_gb300 import _runtime as R

    image_np, smaps_np, omega_np = make_inputs()
    M = omega_np.shape[1]
    image = torch.tensor(image_np, device=dev)
    smaps = torch.tensor(smaps_np, device=dev)
    omega = torch.tensor(omega_np, device=dev)
    fwd = tkbn.KbNufft(im_size=(N, N), dtype=torch.complex64, device=dev)
    adj = tkbn.KbNufftAdjoint(im_size=(N, N), dtype=torch.complex64, device=dev)
    geom = fwd._geom(torch.complex64)
    tables = fwd._tables()
    scaling = fwd.scaling_coef
    lay = R.points_layout(geom, omega)

    def step_staged(ev=None):
        if ev is not None:
            ev[0].record()
        grid = R.fft_and_scale(geom, image, smaps, scaling, None)
        if ev is not None:
            ev[1].record()
        kdata = R.interp_fwd(geom, lay, tables, grid)
        if ev is not None:
            ev[2].record()
        grid2 = R.interp_adj(geom, lay, tables, kdata)
        if ev is not None:
            ev[3].record()
        out = R.ifft_and_scale(geom, grid2, smaps, scaling, None, overwrite=True)
        if ev is not None:
            ev[4].record()
        return out

    # correctness gate on the bench inputs: staged path == module path
    with torch.no_grad():
        ref_out = adj(fwd(image, omega, smaps=smaps), omega, smaps=smaps)
        st_out = step_staged()
        torch.cuda.synchronize()
        gate = float((torch.linalg.vector_norm(ref_out - st_out) / torch.linalg.vector_norm(ref_out)).item())

    for _ in range(args.warmup):
        step_staged()
    torch.cuda.synchronize()
    barrier(world)

    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(args.steps)]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        start.record()
        for k in range(args.steps):
            step_staged(evs[k])
        end.record()
        torch.cuda.synchronize()
    barrier(world)
    ms = start.elapsed_time(end) / args.steps
    ms = max_over_ranks(ms, world, dev)
    stage = {name: statistics.mean(e[i].elapsed_time(e[i + 1]) for e in evs)
             for i, name in enumerate(["fft_and_scale", "interp_fwd", "interp_adj", "ifft_and_scale"])}

    # e2e through the public modules with pinned host buffers: every step
    # copies its image in (H2D) and its result out (D2H); the copies run on
    # their own streams, double-buffered, so step k+1's upload and step k's
    # download overlap step k+1's compute
    x_host = torch.tensor(image_np).pin_memory()
    out_host = [torch.empty((B, 1, N, N), dtype=torch.complex64).pin_memory() for _ in range(2)]
    x_dev = [torch.empty_like(image) for _ in range(2)]
    comp = torch.cuda.current_stream()
    up, down = torch.cuda.Stream(), torch.cuda.Stream()
    free = [torch.cuda.Event() for _ in range(2)]
    loaded = [torch.cuda.Event() for _ in range(2)]
    done = [torch.cuda.Event() for _ in range(2)]

    def upload(k):
        with torch.cuda.stream(up):
            up.wait_event(free[k % 2])
            x_dev[k % 2].copy_(x_host, non_blocking=True)
            loaded[k % 2].record(up)

    def e2e_steps(n):
        for ev in free:
            ev.record(comp)
        upload(0)
        for k in range(n):
            if k + 1 < n:
                upload(k + 1)
            comp.wait_event(loaded[k % 2])
            y = adj(fwd(x_dev[k % 2], omega, smaps=smaps), omega, smaps=smaps)
            free[k % 2].record(comp)
            done[k % 2].record(comp)
            with torch.cuda.stream(down):
                down.wait_event(done[k % 2])
                out_host[k % 2].copy_(y, non_blocking=True)
                y.record_stream(down)
        comp.wait_stream(down)

    with torch.no_grad():
        e2e_steps(args.warmup)
        torch.cuda.synchronize()
        barrier(world)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        e2e_steps(args.steps)
        e1.record()
        torch.cuda.synchronize()
    e2e_ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, world, dev)

    # Toeplitz normal operator (ToepNufft) on the same workload, reported beside the metric
    with torch.no_grad():
        kern = tkbn.calc_toeplitz_kernel(omega, (N, N))
        toep = tkbn.ToepNufft()
        for _ in range(args.warmup):
            toep(image, kern, smaps=smaps)
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(args.steps):
            toep(image, kern, smaps=smaps)
        t1.record()
        torch.cuda.synchronize()
    toep_ms = max_over_ranks(t0.elapsed_time(t1) / args.steps, world, dev)

    work = B * C * M
    value = world * work / (ms * 1e-3)
    byts = algorithmic_bytes(M)
    kernel = "interp_fwd" if stage["interp_fwd"] >= stage["interp_adj"] else "interp_adj"
    kbytes = byts["gather"] if kernel == "interp_fwd" else byts["scatter"]
    peak, peak_src = measured_peak_gbs()
    achieved = kbytes / (stage[kernel] * 1e-3) / 1e9
    pipeline_gbs = (byts["forward"] + byts["adjoint"]) / (ms * 1e-3) / 1e9

    if rank != 0:
        return
    # the CPU port on the full workload: its timing is the cpu_baseline leg
    # (N=1 only) and its outputs are the parity reference of this line
    cpu = None
    if world == 1 and not args.no_cpu_baseline:
        cpu, (k_ref, x_ref) = cpu_baseline_leg(image_np, smaps_np, omega_np)
    else:
        k_ref, x_ref = cpu_full_step(image_np, smaps_np, omega_np)
    with torch.no_grad():
        k_gpu = fwd(image, omega, smaps=smaps)
        x_gpu = adj(torch.tensor(k_ref, device=dev), omega, smaps=smaps)
        st_gpu = step_staged()
        parity = {"forward": rel_l2(k_gpu.cpu().numpy(), k_ref), "adjoint": rel_l2(x_gpu.cpu().numpy(), x_ref),
                  "forward_adjoint_step": rel_l2(st_gpu.cpu().numpy(), x_ref)}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": {
            "workload": "2D SENSE NUFFT fwd+adj, image 320x320, grid 640x640, J=6, L=1024, 16 coils, batch 4, "
                        "golden-angle 404x640 (258560 points)",
            "global_batch": B * world, "parallelism": f"replicas{world}", "l2": "inputs larger than L2 (no flush)",
            "work_per_step": f"{work} points*coils per GPU (B*C*M, once per fwd+adj pair)",
            "stage_ms": {k: round(v, 4) for k, v in stage.items()},
            "toep_nufft_ms": round(toep_ms, 4),
            "pipeline_gbs": round(pipeline_gbs, 1),
            "pipeline_algorithmic_bytes": byts["forward"] + byts["adjoint"],
            "parity_gate_rel_l2_staged_vs_module": gate,
            "parity_oracle": "CPU port of the reference table path (oracle/cpu_baseline.py), same inputs, "
                             "full workload; adjoint of the port's k-space data",
        },
        "rel_l2_vs_oracle": parity,
        "roofline": {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": f"{peak_src} hbm_gbs",
                     "algorithmic_bytes_per_launch": kbytes, "traffic": ncu_traffic(kernel)},
        "cpu_baseline": cpu,
        "e2e": {"value": world * work / (e2e_ms * 1e-3), "unit": UNIT, "ms_per_step": e2e_ms,
                "h2d_bytes_per_step": int(x_host.numel() * 8), "d2h_bytes_per_step": int(out_host[0].numel() * 8)},
        "gpu_launches": LAUNCHES_PER_STEP * args.steps,
        "clocks": clk.summary(),
    }
    print(json.dumps(line))


# ---------------------------------------------------------------- ragged batch (64 independent problems)


def ragged_spec(seed: int = 1005, nprob: int = 64):
    """64 problems: image 128/192/256/320 squared (grid 2x), 20k-400k points
    (uniform random in [-pi, pi)^2 or a variable-density spiral), 1-16 coils."""
    rng = np.random.default_rng(seed)
    spec = []
    for _ in range(nprob):
        n = int(rng.choice([128, 192, 256, 320]))
        M = int(rng.integers(20000, 400001))
        C = int(rng.integers(1, 17))
        if rng.random() < 0.5:
            om = rng.uniform(-np.pi, np.pi, size=(2, M))
        else:
            nil = max(1, M // 2048)
            t = (np.arange(-(-M // nil)) / (-(-M // nil)))
            ks = [np.pi * t ** 1.5 * np.exp(1j * (2 * np.pi * 16 * t + 2 * np.pi * j / nil)) for j in range(nil)]
            k = np.concatenate(ks)[:M]
            om = np.stack([k.imag, k.real])
        spec.append(((n, n), om.astype(np.float32), C))
    return spec


def run_ragged(args):
    import torch

    import torchkbnufft_gb300 as tkbn

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    spec = ragged_spec()
    rng = np.random.default_rng(7)
    probs, images = [], []
    for im, om, C in spec:
        probs.append((im, torch.tensor(om, device=dev), C))
        x = (rng.standard_normal((1, C) + im) + 1j * rng.standard_normal((1, C) + im)).astype(np.complex64)
        images.append(torch.tensor(x, device=dev))
    work = sum(C * om.shape[1] for _, om, C in spec)
    rn = tkbn.RaggedNufft(probs, autotune_layout=True)
    rn.set_images(images)
    # plain: one module call per problem and direction (the reference's way)
    mods = {}
    for im, _, _ in spec:
        if im not in mods:
            mods[im] = (tkbn.KbNufft(im_size=im, device=dev), tkbn.KbNufftAdjoint(im_size=im, device=dev))

    def plain_step():
        for (im, om, _), x in zip(probs, images):
            f, a = mods[im]
            a(f(x, om), om)

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    with torch.no_grad():
        # parity gate: ragged vs per-problem calls on three problems
        rn.forward_adjoint()
        gate = 0.0
        for p in range(3):
            im, om, _ = probs[p]
            f, a = mods[im]
            ref = a(f(images[p], om), om)
            out = rn.output_view(p)
            gate = max(gate, float((torch.linalg.vector_norm(out - ref) / torch.linalg.vector_norm(ref)).item()))
        plain_ms = timed(plain_step, args.steps, args.warmup)
        # the same per-problem module calls captured as one CUDA graph: the
        # plain path's GPU time without host launch gaps (its kernel floor)
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            plain_step()
        torch.cuda.current_stream().wait_stream(side)
        pg = torch.cuda.CUDAGraph()
        with torch.cuda.graph(pg):
            plain_step()
        plain_graph_ms = timed(pg.replay, args.steps, args.warmup)
        eager_ms = timed(rn.forward_adjoint, args.steps, args.warmup)
        rn.capture()
        graph_ms = timed(rn.replay, args.steps, args.warmup)
        # every problem against the CPU port of the reference path: the
        # forward of its image, the adjoint of the port's k-space data
        from oracle import cpu_baseline as P

        xs_np = [x.cpu().numpy() for x in images]
        ks = rn.forward(images)
        want_k = [P.nufft_forward(xn, om, None) for xn, (_, om, _) in zip(xs_np, spec)]
        e_fwd = max(rel_l2(a.cpu().numpy(), b) for a, b in zip(ks, want_k))
        xs = rn.adjoint([torch.tensor(k, device=dev) for k in want_k])
        e_adj = max(rel_l2(a.cpu().numpy(), P.nufft_adjoint(k, om, im, None))
                    for a, k, (im, om, _) in zip(xs, want_k, spec))
    line = {
        "metric": "NU points*coils/s (ragged batch fwd+adj, 64 problems, graph-captured)", "value": work / (graph_ms * 1e-3),
        "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": graph_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": {"workload": "ragged batch: 64 problems, image 128/192/256/320 squared, grid 2x, 20k-400k points "
                               "(uniform random or variable-density spiral), 1-16 coil images, J=6, L=1024",
                   "work_per_step": work, "plain_ms_per_step": plain_ms,
                   "plain_loop_graph_ms_per_step": plain_graph_ms, "eager_ms_per_step": eager_ms,
                   "graph_ms_per_step": graph_ms, "speedup_graph_vs_plain": plain_ms / graph_ms,
                   "tiles": {f"{k[0]}x{k[1]}": v for k, v in rn.tiles.items()},
                   "parity_gate_rel_l2_vs_per_problem": gate},
        "rel_l2_vs_oracle": {"forward_max_over_problems": e_fwd, "adjoint_max_over_problems": e_adj,
                             "problems_compared": len(spec)},
        "gpu_launches": None,
    }
    print(json.dumps(line))


# ---------------------------------------------------------------- other configurations (reported beside the metric)


def radial_traj(spokes: int, readout: int) -> np.ndarray:
    """(2, spokes*readout): angles k*pi/spokes, readout linspace(-pi, pi, readout+1)[:-1]."""
    r = np.linspace(-np.pi, np.pi, readout + 1)[:-1]
    th = np.arange(spokes) * np.pi / spokes
    return np.stack([(np.sin(th)[:, None] * r).reshape(-1), (np.cos(th)[:, None] * r).reshape(-1)]).astype(np.float32)


def kooshball_traj(spokes: int, readout: int) -> np.ndarray:
    """(3, spokes*readout): Fibonacci-sphere directions times linspace(-pi, pi, readout+1)[:-1]."""
    i = np.arange(spokes)
    z = 1 - 2 * (i + 0.5) / spokes
    phi = i * np.pi * (3 - np.sqrt(5))
    rxy = np.sqrt(1 - z * z)
    d = np.stack([z, rxy * np.sin(phi), rxy * np.cos(phi)])
    r = np.linspace(-np.pi, np.pi, readout + 1)[:-1]
    return (d[:, :, None] * r[None, None, :]).reshape(3, -1).astype(np.float32)


def spiral_traj(interleaves: int, samples: int) -> np.ndarray:
    """(2, interleaves*samples): k_j(t) = pi t^1.5 exp(i (2 pi 16 t + 2 pi j / interleaves))."""
    t = np.arange(samples) / samples
    k = np.concatenate([np.pi * t ** 1.5 * np.exp(1j * (2 * np.pi * 16 * t + 2 * np.pi * j / interleaves))
                        for j in range(interleaves)])
    return np.stack([k.imag, k.real]).astype(np.float32)


def smooth_maps_3d(ncoil: int, n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    g = np.arange(n) - n / 2
    z, y, x = np.meshgrid(g, g, g, indexing="ij")
    maps = []
    for c in range(ncoil):
        ang = 2 * np.pi * c / ncoil + rng.uniform(0, 0.3)
        cz, cy, cx = 0.2 * n * np.cos(2 * ang), 0.35 * n * np.sin(ang), 0.35 * n * np.cos(ang)
        mag = np.exp(-((x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2) / (2 * (0.4 * n) ** 2))
        maps.append(mag * np.exp(1j * ang))
    maps = np.stack(maps)
    maps /= np.sqrt(np.sum(np.abs(maps) ** 2, axis=0, keepdims=True))
    return maps[None].astype(np.complex64)


def stage_times(fwd, omega, x, smaps, steps, warmup):
    """Mean time (ms) of each stage of forward + adjoint, timed on the stream."""
    import torch

    from torchkbnufft_gb300 import _runtime as R

    cd = x.dtype
    geom = fwd._geom(cd)
    tables = fwd._tables()
    scaling = fwd.scaling_coef.to(cd)
    lay = R.points_layout(geom, omega)
    names = ["fft_and_scale", "interp_fwd", "interp_adj", "ifft_and_scale"]

    def staged(ev=None):
        rec = (lambda i: ev[i].record()) if ev is not None else (lambda i: None)
        rec(0)
        grid = R.fft_and_scale(geom, x, smaps, scaling, None)
        rec(1)
        kdata = R.interp_fwd(geom, lay, tables, grid)
        rec(2)
        grid2 = R.interp_adj(geom, lay, tables, kdata)
        rec(3)
        R.ifft_and_scale(geom, grid2, smaps, scaling, None, overwrite=True)
        rec(4)

    for _ in range(warmup):
        staged()
    torch.cuda.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(steps)]
    for k in range(steps):
        staged(evs[k])
    torch.cuda.synchronize()
    return {n: round(statistics.mean(e[i].elapsed_time(e[i + 1]) for e in evs), 4) for i, n in enumerate(names)}


def run_config(args):
    """Forward+adjoint (or, for spiral-grad, loss + backward) throughput at the
    other configurations; one JSON line each, not the headline metric."""
    import torch

    import torchkbnufft_gb300 as tkbn

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(1000)
    w = args.workload

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    cdt = torch.complex64
    if w == "single":
        n, om, Bc, Cc, smaps = 256, radial_traj(402, 512), 1, 1, None
        desc = "2D single-coil radial, image 256^2, grid 512^2, 402x512 (205824 points), batch 1"
    elif w == "sense-c128":
        cdt = torch.complex128
        image_np, smaps_np, om = make_inputs()
        n, Bc, Cc = N, B, C
        smaps = torch.tensor(smaps_np.astype(np.complex128), device=dev)
        desc = ("2D SENSE NUFFT fwd+adj in complex128, image 320x320, grid 640x640, J=6, L=1024, 16 coils, "
                "batch 4, golden-angle 404x640 (258560 points)")
    elif w == "kooshball":
        sp = args.kooshball_spokes
        n, om, Bc, Cc = 128, kooshball_traj(sp, 256), 1, 8
        smaps = torch.tensor(smooth_maps_3d(8, 128, 3), device=dev)
        desc = f"3D kooshball, image 128^3, grid 256^3, 8 coils, {sp}x256 ({sp * 256} points), batch 1"
    else:
        n, om, Bc, Cc = 256, spiral_traj(32, 2048), 8, 16
        smaps = torch.tensor(ring_smaps(16, 256, 1, 4)[:1], device=dev)
        desc = ("2D spiral 32x2048 (65536 points), image 256^2, grid 512^2, 16 coils, batch 8; loss "
                "||A^H A x - x||^2, gradients w.r.t. x and ktraj")
    nd = om.shape[0]
    im = (n,) * nd
    M = om.shape[1]
    x = torch.tensor((rng.standard_normal((Bc, 1 if smaps is not None else Cc) + im)
                      + 1j * rng.standard_normal((Bc, 1 if smaps is not None else Cc) + im)),
                     device=dev).to(cdt)
    omega = torch.tensor(om, device=dev)
    if cdt == torch.complex128:
        omega = omega.double()
    fwd = tkbn.KbNufft(im_size=im, dtype=cdt, device=dev)
    adj = tkbn.KbNufftAdjoint(im_size=im, dtype=cdt, device=dev)
    work = Bc * Cc * M
    extra = {}
    if w == "spiral-grad":
        xr = x.clone().requires_grad_(True)
        om_r = omega.clone().requires_grad_(True)

        def move_trajectory():
            # a trajectory-optimisation step changes ktraj in place (here a
            # sign step of 1e-5 rad, no host sync), so the next call rebuilds
            # the bin-sorted layout and the adjoint's per-point factors
            with torch.no_grad():
                g = om_r.grad if om_r.grad is not None else torch.ones_like(om_r)
                om_r.sub_(1e-5 * torch.sign(g))

        def fwd_step():
            move_trajectory()
            with torch.no_grad():
                adj(fwd(x, om_r, smaps=smaps), om_r, smaps=smaps)

        def grad_step():
            move_trajectory()
            xr.grad = None
            om_r.grad = None
            y = adj(fwd(xr, om_r, smaps=smaps), om_r, smaps=smaps)
            loss = (y - xr).abs().pow(2).sum()
            loss.backward()

        fwd_ms = timed(fwd_step, args.steps, args.warmup)
        ms = timed(grad_step, args.steps, args.warmup)
        from torchkbnufft_gb300 import _runtime as R

        extra = {"forward_AHA_ms": fwd_ms, "grad_step_ms": ms, "backward_over_forward": (ms - fwd_ms) / fwd_ms,
                 "trajectory": "updated in place every step (layout rebuild and factor pre-pass timed)",
                 "layout_cache_entries_after": R.layout_cache_info()[0],
                 "note": "a step is the ktraj update, the forward A^H A x, the loss and its backward "
                         "(x and ktraj gradients); the forward-only step is the update and A^H A x"}
    else:
        with torch.no_grad():
            ms = timed(lambda: adj(fwd(x, omega, smaps=smaps), omega, smaps=smaps), args.steps, args.warmup)
            extra = {"stage_ms": stage_times(fwd, omega, x, smaps, args.steps, args.warmup)}
            if w == "kooshball":
                # the Toeplitz normal operator (ToepNufft) on the same image, maps and trajectory
                kern = tkbn.calc_toeplitz_kernel(omega, im)
                toep = tkbn.ToepNufft()
                extra["toep_nufft_ms"] = round(timed(lambda: toep(x, kern, smaps=smaps), args.steps, args.warmup), 4)
                del kern
    parity = config_parity(w, fwd, adj, x, omega, smaps, om, im)
    line = {
        "metric": f"NU points*coils/s ({w})", "value": work / (ms * 1e-3), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128" if cdt == torch.complex128 else "c64", "data": "synthetic",
        "config": {"workload": desc, "work_per_step": work, **extra},
        "rel_l2_vs_oracle": parity,
    }
    print(json.dumps(line))


def config_parity(w, fwd, adj, x, omega, smaps, om, im):
    """Forward and adjoint of the workload's inputs against the CPU port of the
    reference path (oracle/cpu_baseline.py): the full workload, except the
    kooshball, whose port side runs at a seeded 4096-point subset (forward at
    those points; adjoint of k-space data that is zero elsewhere)."""
    import torch

    from oracle import cpu_baseline as P

    xn = x.detach().cpu().numpy()
    sn = None if smaps is None else smaps.detach().cpu().numpy().astype(xn.dtype)
    omn = om.astype(np.float64) if xn.dtype == np.complex128 else om
    with torch.no_grad():
        y = fwd(x, omega, smaps=smaps)
        if w == "kooshball":
            sub = np.sort(np.random.default_rng(1003).choice(om.shape[1], 4096, replace=False))
            subd = torch.tensor(sub, device=y.device)
            k_ref = P.nufft_forward(xn, omn[:, sub], sn)
            e_fwd = rel_l2(y[..., subd].cpu().numpy(), k_ref)
            kfull = torch.zeros_like(y)
            kfull[..., subd] = torch.tensor(k_ref, device=y.device)
            del y
            e_adj = rel_l2(adj(kfull, omega, smaps=smaps).cpu().numpy(), P.nufft_adjoint(k_ref, omn[:, sub], im, sn))
            return {"forward": e_fwd, "adjoint": e_adj, "points_compared": 4096}
        k_ref = P.nufft_forward(xn, omn, sn)
        e_fwd = rel_l2(y.cpu().numpy(), k_ref)
        del y
        x_ref = P.nufft_adjoint(k_ref, omn, im, sn)
        e_adj = rel_l2(adj(torch.tensor(k_ref, device=x.device), omega, smaps=smaps).cpu().numpy(), x_ref)
    return {"forward": e_fwd, "adjoint": e_adj}


# ---------------------------------------------------------------- second comparator: the reference on the GPU


def run_reference_gpu(args):
    """The unmodified reference, installed in baseline/_ref, through its own
    public API (KbNufft forward and KbNufftAdjoint with the maps) on the same
    device and workload as the GPU arm. Inputs are resident on the device. On a
    GPU it is timed with CUDA events on the current stream. Runs on rank 0 only.
    ``--device`` overrides the device (cpu for a check without a GPU)."""
    world, rank, local = dist_setup()
    if rank != 0:
        return
    ref_dir = os.path.join(ROOT, "baseline", "_ref")
    if not os.path.isfile(os.path.join(ref_dir, "torchkbnufft", "__init__.py")):
        print(json.dumps({"impl": "reference-gpu", "unavailable": "the reference is not installed in baseline/_ref"}))
        return
    import warnings

    import torch

    sys.path.insert(0, ref_dir)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        import torchkbnufft as ref
    dev = torch.device(args.device or "cuda")
    image_np, smaps_np, omega_np = make_inputs()
    x, s, om = (torch.tensor(a, device=dev) for a in (image_np, smaps_np, omega_np))
    fwd = ref.KbNufft(im_size=(N, N), device=dev)
    adj = ref.KbNufftAdjoint(im_size=(N, N), device=dev)

    def step():
        with torch.no_grad():
            return adj(fwd(x, om, smaps=s), om, smaps=s)

    for _ in range(args.warmup):
        step()
    if dev.type == "cuda":
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.steps):
            step()
        e1.record()
        torch.cuda.synchronize(dev)
        ms = e0.elapsed_time(e1) / args.steps
    else:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        ms = (time.perf_counter() - t0) * 1e3 / args.steps
    work = B * C * omega_np.shape[1]
    print(json.dumps({
        "impl": "reference-gpu", "metric": METRIC, "value": work / (ms * 1e-3), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c64", "data": "synthetic",
        "config": {"workload": "2D SENSE NUFFT fwd+adj, image 320x320, grid 640x640, J=6, L=1024, 16 coils, "
                               "batch 4, golden-angle 404x640 (258560 points)",
                   "device": str(dev), "path": "the reference's own table path, unmodified (baseline/_ref)",
                   "work_per_step": work},
    }))


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference", "reference-gpu"],
                   help="reference: the reference path on the host cores; reference-gpu: the reference's "
                        "own PyTorch path on the GPU (a second comparator)")
    p.add_argument("--device", default=None, help="device of the reference-gpu arm (default cuda)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--kooshball-spokes", type=int, default=20000,
                   help="spokes of the kooshball workload (20000 is the configuration; fewer for a small profiling case)")
    p.add_argument("--workload", default="sense", choices=["sense", "ragged", "single", "kooshball", "spiral-grad", "sense-c128"],
                   help="sense: the metric's workload (default); the others are reported beside it")
    args = p.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.impl == "reference-gpu":
        run_reference_gpu(args)
    elif args.workload == "ragged":
        run_ragged(args)
    elif args.workload != "sense":
        run_config(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
