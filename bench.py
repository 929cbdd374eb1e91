#!/usr/bin/env python
"""Benchmark: Psi-propagation steps/s of the electron-hole propagator.

Workload (default): the 1,200-atom disordered C/H/O cluster (60/30/10 %, 1.4 A
jittered cubic lattice, N = 3,720 AO), moving nuclei (fresh N(0, 0.02 A^2)
perturbation of every coordinate each step), dt = 0.5 fs, Chebyshev propagation
of electron and hole (bra and ket), S, h, the Cholesky factor of S and the
propagation operator rebuilt on the device every step.  One step = one nuclear
step of both particles.  Default precision OZ64: FP64 results, with every
operator product computed exactly on the tensor cores from BF16 slices and
rounded once to FP64; the same line carries the FP64-pipe run (fp64_variant)
and the DF64 run (df64_variant) of the same workload.  `--method taylor` times
the reference's adaptive-tau Taylor step instead.

Synthetic, seeded data (no external dataset).  Lines:
  value  device-resident: all steps' coordinates uploaded before the timed
         region, populations left on the device (elhl_traj_step_device);
  e2e    through the C ABI with host buffers: pinned host coordinates in and
         populations out every step (elhl_traj_step).
Timing: CUDA events on the library's launch stream (set to torch's stream),
W untimed warm-up steps, L2 flushed (512 MB write) between timed steps.

`--impl reference` times the reference algorithm on the host cores instead:
the oracle port (the reference itself needs Fortran/MKL/MPI and cannot be
built), all host threads, bounded sample.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

H_BAR = 6.58264e-4


def workload(name: str):
    from dynemol_gb300 import systems
    if name == "ehrenfest":   # 1,200-atom C/H/O cluster, moving nuclei, dt 0.5 fs
        return systems.cubic_cluster(n_atoms=1200, seed=2), 5.0e-4, True
    if name == "flake":       # C100H50 flake, fixed nuclei, dt 0.1 fs
        return systems.honeycomb_flake(), 1.0e-4, False
    if name == "small":       # quick check: 300-atom cluster, moving nuclei
        return systems.cubic_cluster(n_atoms=300, seed=2), 5.0e-4, True
    if name == "medium":      # profiling case: 900-atom cluster (N = 2790), G + h + G^T above L2
        return systems.cubic_cluster(n_atoms=900, seed=2), 5.0e-4, True
    raise ValueError(name)


WORKLOAD_DESC = {
    "ehrenfest": "C/H/O cluster 1200 atoms (60/30/10%), jittered 1.4 A cubic lattice, moving nuclei "
                 "(sigma 0.02 A per step), dt 0.5 fs, S, h and the propagation operator rebuilt every step, el+hl bra/ket",
    "flake": "C100H50 honeycomb flake (sigma 0.03 A), fixed nuclei, dt 0.1 fs, el+hl bra/ket",
    "small": "C/H/O cluster 300 atoms, moving nuclei, dt 0.5 fs, el+hl bra/ket",
    "medium": "C/H/O cluster 900 atoms, moving nuclei, dt 0.5 fs, el+hl bra/ket",
}


def step_coords(sysm, moving, nsteps, offset=0):
    from dynemol_gb300 import systems
    if not moving:
        return None
    return np.stack([systems.perturbed_coords(sysm.coords, offset + i, sigma=0.02, seed=2) for i in range(nsteps)])


# ----------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", os.environ.get("LOCAL_RANK", "0")],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clock sampling unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------- replicas
def max_over_ranks(t_local: float, world: int) -> float:
    """Slowest rank's time (replicas: every rank propagates its own trajectory)."""
    if world <= 1:
        return t_local
    import torch
    import torch.distributed as dist
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([t_local], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(steps: int, world: int, t_max: float) -> float:
    """Whole-job steps/s: all ranks' steps over the slowest rank's time."""
    return world * steps / t_max


# ----------------------------------------------------------------- our arm
def run_ours(args, rank, world):
    import torch
    from dynemol_gb300 import api, build, systems

    build.build()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    api.load()
    # a dedicated (non-default) stream: the library launches on it and the CUDA
    # events below are recorded on it
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    api.set_stream(stream.cuda_stream)

    sysm, dt, moving = workload(args.workload)
    homo = systems.fermi_state(sysm, np.arange(20))
    W, K = args.warmup, args.steps
    coords = step_coords(sysm, moving, W + K + 1, offset=1000 * rank)
    method = api.METHOD_CHEBYSHEV if args.method == "chebyshev" else api.METHOD_TAYLOR_REF
    prec = {"fp64": api.PREC_FP64, "fp32": api.PREC_FP32, "bf16x3": api.PREC_BF16X3,
            "df64": api.PREC_DF64, "oz64": api.PREC_OZ64}[args.precision]
    tr = api.Trajectory(sysm, coords=None if coords is None else coords[0], dt=dt, method=method, precision=prec,
                        ncols=4 if moving else 2, cheb_tol=1e-12)
    tr.init_fmo(homo + 1, homo)

    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    nf1 = sysm.nfrag + 1
    d_pops = torch.zeros((W + K) * 2 * nf1, dtype=torch.float64, device=dev)
    d_coords = None if coords is None else torch.from_numpy(coords[1:]).to(dev).contiguous()
    nc = sysm.natoms * 3

    def dev_step(i):
        cptr = 0 if d_coords is None else d_coords.data_ptr() + i * nc * 8
        if d_coords is None:
            tr.step(None, nsteps=1, want_pops=False)
        else:
            tr.step_device(cptr, 1, d_pops.data_ptr() + i * 2 * nf1 * 8)

    # warm-up
    for i in range(W):
        dev_step(i)
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()

    # ---- value: device-resident, per-step CUDA events, L2 flush between steps
    clocks = ClockSampler()
    clocks.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    prop_ms = rebuild_ms = sh_ms = factor_ms = inverse_ms = 0.0
    orders = launches = 0
    torch.cuda.synchronize(dev)
    for i in range(K):
        flush.fill_(float(i))
        n0 = api.kernel_launches()
        ev[i][0].record(stream)
        dev_step(W + i)
        ev[i][1].record(stream)
        launches += api.kernel_launches() - n0  # this library's kernels in the timed region
        st = tr.stats()
        prop_ms += st.prop_ms
        rebuild_ms += st.rebuild_ms
        sh_ms += st.sh_ms
        factor_ms += st.factor_ms
        inverse_ms += st.inverse_ms
        orders += st.orders
    tile = {"tile_cols": st.tile_cols, "phases": st.phases} if method == api.METHOD_CHEBYSHEV else {}
    torch.cuda.synchronize(dev)
    clk = clocks.stop()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    t_dev = max_over_ranks(ms / 1e3, world)

    # ---- e2e: host buffers through the C ABI (H2D coords + D2H populations each step)
    Ke = K
    e_coords = step_coords(sysm, moving, Ke, offset=5000 + 1000 * rank)
    h_pops = np.zeros((1, 2, nf1))
    if e_coords is not None:
        pinned = torch.from_numpy(e_coords).pin_memory()
        host_coords = pinned.numpy()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(Ke):
        if e_coords is None:
            h_pops = tr.step(None, nsteps=1)
        else:
            h_pops = tr.step(host_coords[i], nsteps=1)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    t_e2e = max_over_ranks(e0.elapsed_time(e1) / 1e3, world)
    api.set_stream(None)
    tr.close()

    N = sysm.nao
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    FP64_PEAK = 1.20  # TFLOP/s: FP64 FMA throughput of a GB300 measured by a DFMA loop
    prop_launch_ms = prop_ms / K
    traffic_per_launch = None
    if args.method == "taylor":
        # dominant kernel: taylor_kernel.  Unit = one expansion order of one
        # particle: H' read twice, by rows for the ket (H') and by columns for the
        # bra (H'^T), 2 complex columns: bytes = 16 N^2 + 160 N, flops = 8 N^2
        kernel = "taylor_kernel"
        per_launch_orders = orders / max(1, K)
        bytes_per_launch = per_launch_orders * (16.0 * N * N + 160.0 * N)
        flops_per_launch = per_launch_orders * 8.0 * N * N
    else:
        # dominant kernel: cheb_kernel (oz_cheb_kernel for OZ64).  Unit = one Chebyshev
        # order over m complex columns.  Explicit Hs: Hs read once (b_H N^2) + 5 x 16 N m
        # vector bytes, flops 4 N^2 m.  Implicit G (h/b) G^T (moving nuclei, three
        # phases): N^2/2 + N^2 + N^2/2 matrix elements (b_H 2 N^2) + 9 x 16 N m vector
        # bytes, flops 8 N^2 m
        kernel = "oz_cheb_kernel" if args.precision == "oz64" else "cheb_kernel"
        m = 4 if moving else 2
        # bytes per matrix element: FP64 / DF64 pairs 8, FP32 4, OZ64 seven BF16 slices 14
        bH = {"fp64": 8.0, "df64": 8.0, "oz64": 14.0}.get(args.precision, 4.0)
        # the implicit operator (three grid phases) reads 2 N^2 elements per order, an
        # explicit H~ (one phase: fixed nuclei, and OZ64 moving nuclei) N^2
        implicit = st.phases == 3 if method == api.METHOD_CHEBYSHEV else False
        elems, vec = (2.0 * N * N, 144.0) if implicit else (1.0 * N * N, 80.0)
        per_launch_orders = orders / max(1, K) / m
        bytes_per_launch = per_launch_orders * (bH * elems + vec * N * m)
        flops_per_launch = per_launch_orders * 4.0 * elems * m
        if args.precision == "oz64" and not implicit and N == 3720:
            # DRAM traffic per matrix element and order measured by ncu on the same kernel
            # and workload (N = 3720: 18.77 GB read + 0.61 GB written in one launch of
            # 143.4 orders of N^2 elements, 9.77 B: the backward walk serves about 31 % of
            # the 14 B of slices from L2); scaled to this launch's orders.  At other sizes
            # the L2's share differs (N = 2790 fits in it), so no figure is claimed there
            traffic_per_launch = 9.77 * elems * per_launch_orders
        if implicit and args.precision in ("fp64", "df64"):
            # DRAM traffic per matrix element and order measured by ncu on the same
            # kernel at N = 2790 (18.68 GB read + 0.11 GB written over 149 orders of
            # 2 N^2 elements); traffic grows with N^2 and the orders, so it is scaled
            # to this launch
            traffic_per_launch = 8.10 * elems * per_launch_orders
    achieved_gbs = bytes_per_launch / (prop_launch_ms * 1e-3) / 1e9
    # ALU bound: FP64 FMA pipe; FP32 FMA pipe; DF64 = FP32 pipe at 12 FP32
    # instructions per FP64-equivalent FMA (peak 70.1 / 12 FP64-equivalent TFLOP/s)
    alu_peak, alu_pipe = {"fp64": (FP64_PEAK, "fp64 FMA"),
                          "df64": (70.1 / 12.0, "fp32 FMA, 12 instructions per df64 FMA")}.get(
        args.precision, (70.1, "fp32 FMA"))
    alu_src = "of measured (FP64/FP32 FMA probe on a GB300)"
    if args.precision == "oz64":
        # tensor pipe: per matrix element and order, 2 x 256 BF16 MMA flops (the 7 slice
        # products against 8, 6, 6, 4, 4, 2, 2 vector slice columns of 8 real columns)
        flops_per_launch = per_launch_orders * 512.0 * elems
        alu_peak, alu_pipe = peaks.get("bf16_tflops", 1900.0), "bf16 tensor (tcgen05.mma, FP32 accumulation)"
        alu_src = "of measured (MEASURED_PEAKS.json bf16_tflops)"
    tflops = flops_per_launch / (prop_launch_ms * 1e-3) / 1e12

    line = {
        "metric": "psi_propagation_steps_per_s",
        "value": replica_value(K, world, t_dev),
        "unit": "steps/s",
        "n_gpus": world,
        "steps": K,
        "warmup": W,
        "ms_per_step": 1e3 * t_dev / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": {"fp64": "f64", "df64": "f64-accurate FP32 pairs (df64), f64 recurrence",
                  "oz64": "f64 (operator products exact on bf16 tensor cores from 8-bit slices, "
                          "rounded once to f64; f64 vectors and recurrence)"}.get(
            args.precision, "f32 products, f64 accumulation"),
        "data": "synthetic (seeded geometry, no external dataset)",
        "config": {"workload": WORKLOAD_DESC[args.workload], "N_ao": N, "natoms": sysm.natoms,
                   "dt_ps": dt, "particles": 2, "method": args.method, "precision": args.precision,
                   "moving_nuclei": moving, "l2": "flushed (512 MB write) between timed steps", **tile,
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": replica_value(Ke, world, t_e2e), "unit": "steps/s",
                "h2d_bytes_per_step": (nc * 8) if moving else 0, "d2h_bytes_per_step": 2 * nf1 * 8},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved_gbs / hbm_peak, "traffic": traffic_per_launch,
                     "kernel": kernel, "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)",
                     "alu": {"achieved_tflops": tflops,
                             "peak_tflops": alu_peak,
                             "frac": tflops / alu_peak,
                             "pipe": alu_pipe,
                             "peak_source": alu_src},
                     "orders_per_launch": per_launch_orders, "launch_ms": prop_launch_ms},
        "breakdown_ms_per_step": {"propagation": prop_ms / K, "rebuild_S_h_operator": rebuild_ms / K,
                                  "rebuild_parts": {"S_h_build": sh_ms / K, "cholesky": factor_ms / K,
                                                    "operator_form": inverse_ms / K,
                                                    "bounds_columns_other": (rebuild_ms - sh_ms - factor_ms
                                                                             - inverse_ms) / K}},
        "clocks": clk,
    }
    return line


def run_variant(args, precision_name: str):
    """The same workload and coordinates with another precision (device-resident
    steps, CUDA events on the library's stream, L2 flushed between steps): the
    FP64-pipe, DF64 and OZ64 variants of the default run."""
    import torch
    from dynemol_gb300 import api, systems
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    api.set_stream(stream.cuda_stream)
    sysm, dt, moving = workload(args.workload)
    homo = systems.fermi_state(sysm, np.arange(20))
    W, K = args.warmup, args.steps
    coords = step_coords(sysm, moving, W + K + 1)
    prec = {"fp64": api.PREC_FP64, "fp32": api.PREC_FP32, "df64": api.PREC_DF64, "oz64": api.PREC_OZ64}[
        precision_name]
    tr = api.Trajectory(sysm, coords=None if coords is None else coords[0], dt=dt, method=api.METHOD_CHEBYSHEV,
                        precision=prec, ncols=4 if moving else 2, cheb_tol=1e-12)
    tr.init_fmo(homo + 1, homo)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    d_coords = None if coords is None else torch.from_numpy(coords[1:]).to(dev).contiguous()
    nf1 = sysm.nfrag + 1
    d_pops = torch.zeros((W + K) * 2 * nf1, dtype=torch.float64, device=dev)
    nc = sysm.natoms * 3

    def dev_step(i):
        if d_coords is None:
            tr.step(None, nsteps=1, want_pops=False)
        else:
            tr.step_device(d_coords.data_ptr() + i * nc * 8, 1, d_pops.data_ptr() + i * 2 * nf1 * 8)

    for i in range(W):
        dev_step(i)
    torch.cuda.synchronize(dev)
    ms = prop = rebuild = sh = factor = 0.0
    for i in range(K):
        flush.fill_(float(i))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        dev_step(W + i)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms += e0.elapsed_time(e1)
        st = tr.stats()
        prop += st.prop_ms
        rebuild += st.rebuild_ms
        sh += st.sh_ms
        factor += st.factor_ms + st.inverse_ms
    tr.close()
    api.set_stream(None)
    return {"precision": precision_name, "value": K / (ms / 1e3), "unit": "steps/s", "ms_per_step": ms / K,
            "propagation_ms_per_step": prop / K,
            "rebuild_parts_ms_per_step": {"S_h_build": sh / K, "cholesky_and_inverse": factor / K,
                                          "bounds_columns_other": (rebuild - sh - factor) / K}}


def run_dropin(args, steps: int = 2):
    """The reference-semantics FP64 Taylor path (the propagationelhl_gpucaller_
    algorithm) on the same workload and coordinates, device-resident, CUDA events."""
    import torch
    from dynemol_gb300 import api, systems
    sysm, dt, moving = workload(args.workload)
    homo = systems.fermi_state(sysm, np.arange(20))
    coords = step_coords(sysm, moving, 4 + steps)
    tr = api.Trajectory(sysm, coords=None if coords is None else coords[0], dt=dt)
    tr.init_fmo(homo + 1, homo)
    stream = torch.cuda.current_stream()
    api.set_stream(stream.cuda_stream if stream.cuda_stream else None)
    tr.step(None if coords is None else coords[1:3], nsteps=2, want_pops=False)  # warm-up
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    tr.step(None if coords is None else coords[3:3 + steps], nsteps=steps, want_pops=True)
    e1.record(stream)
    torch.cuda.synchronize()
    st = tr.stats()
    tr.close()
    api.set_stream(None)
    t = e0.elapsed_time(e1) / 1e3
    return {"steps_per_s": steps / t, "steps": steps, "orders_per_step": st.orders / steps,
            "propagation_ms_per_step": st.prop_ms / steps, "rebuild_ms_per_step": st.rebuild_ms / steps}


def run_dropin_host(args, steps: int = 3):
    """The drop-in as the reference's Fortran host calls it: per nuclear step one
    propagationelhl_gpucaller_ call per particle (electron, hole) with host S, h
    (column-major N x N), H' out and Psi in/out (Taylor_gpu.cpp:634-736;
    ElHl_Chebyshev_GPU.f:269-272), on the workload's geometries.  S and h of each
    step come from the library's own device build at that geometry, outside the
    timed region, as the reference builds them on the host before the call."""
    from dynemol_gb300 import api, systems
    sysm, dt, moving = workload(args.workload)
    homo = systems.fermi_state(sysm, np.arange(20))
    coords = step_coords(sysm, moving, steps + 2)
    tr = api.Trajectory(sysm, coords=None if coords is None else coords[0], dt=dt, method=api.METHOD_CHEBYSHEV,
                        precision=api.PREC_FP64, ncols=4, cheb_tol=1e-12)
    tr.init_fmo(homo + 1, homo)
    bra, ket = tr.get_psi()
    mats = []
    for i in range(steps + 1):
        if coords is not None:
            tr.step(coords[1 + i: 2 + i], nsteps=1, want_pops=False)
        S, h, _ = tr.matrices()
        mats.append((np.asfortranarray(S), np.asfortranarray(h)))
    tr.close()
    N = sysm.nao
    bra = [np.ascontiguousarray(bra[:, p]) for p in range(2)]
    ket = [np.ascontiguousarray(ket[:, p]) for p in range(2)]
    tau_max = dt / H_BAR
    save = [tau_max, tau_max]
    t_timed = 0.0
    for s in range(steps + 1):  # one untimed step, then `steps` timed
        S, h = mats[s]
        t0 = time.perf_counter()
        for p in range(2):
            tau = tau_max if s == 0 else min(1.15 * save[p], tau_max)
            *_, save[p] = api.propagationelhl_gpucaller(S, h, bra[p], ket[p], s * dt, (s + 1) * dt, tau)
        if s:
            t_timed += time.perf_counter() - t0
    return {"steps_per_s": steps / t_timed, "steps": steps, "N_ao": N,
            "h2d_bytes_per_step": 2 * (2 * N * N * 8 + 2 * N * 16),
            "d2h_bytes_per_step": 2 * (N * N * 8 + 3 * N * 16),
            "path": "propagationelhl_gpucaller_ with host buffers, electron and hole one call each per step "
                    "(S^-1 h by the library's FP64 Cholesky with inverse, adaptive-tau Taylor)"}


# ----------------------------------------------------------------- CPU sample
def cpu_sample(args, sysm, dt, moving, nsteps, nthreads):
    """Oracle port timed on the host cores: `nsteps` nuclear steps after one untimed step."""
    from dynemol_gb300 import systems
    from oracle import oracle
    oracle.build()
    homo = systems.fermi_state(sysm, np.arange(20))
    coords = step_coords(sysm, moving, nsteps + 2)
    c0 = sysm.coords if coords is None else coords[0]
    S = oracle.overlap(sysm, c0, nthreads=nthreads)
    bra, ket = oracle.initial_states(sysm, S, homo + 1, homo)
    ref = oracle.ReferenceStep(sysm, bra, ket, dt, nthreads=nthreads)
    ref.step(None if coords is None else coords[1])
    t0 = time.perf_counter()
    for i in range(nsteps):
        ref.step(None if coords is None else coords[2 + i])
    el = time.perf_counter() - t0
    return nsteps / el, el


def run_reference(args, rank, world):
    if rank != 0:
        return None
    sysm, dt, moving = workload(args.workload)
    nthreads = os.cpu_count() or 1
    nsteps = max(1, args.steps // 5) if args.workload == "ehrenfest" else args.steps
    rate, el = cpu_sample(args, sysm, dt, moving, nsteps, nthreads)
    sample = f"{nsteps} nuclear steps of the workload after 1 untimed step ({el:.1f} s)"
    return {
        "impl": "reference",
        "metric": "psi_propagation_steps_per_s", "value": rate, "unit": "steps/s", "n_gpus": world,
        "steps": nsteps, "warmup": 1, "ms_per_step": 1e3 / rate, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded geometry, no external dataset)",
        "config": {"workload": WORKLOAD_DESC[args.workload], "N_ao": sysm.nao, "natoms": sysm.natoms,
                   "dt_ps": dt, "particles": 2, "method": "taylor_ref", "precision": "fp64"},
        "cpu_baseline": {"value": rate, "unit": "steps/s", "cores": nthreads, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# ----------------------------------------------------------------- trajectory mix
def trajectory_mix(ntraj: int, nmin: int = 200, nmax: int = 3000, seed: int = 4):
    """Uneven C/H/O systems: N drawn uniformly in [nmin, nmax] AOs (seed), each its
    own jittered cubic cluster (60/30/10 %) -- the batching workload."""
    from dynemol_gb300 import systems
    rng = systems.SplitMix64(seed)
    out = []
    for i in range(ntraj):
        target = nmin + (rng.next_u64() % (nmax - nmin + 1))
        n_atoms = max(8, int(round(target / 3.1)))  # 3.1 AO per atom at 60/30/10 % C/H/O
        out.append(systems.cubic_cluster(n_atoms=n_atoms, seed=seed + i))
    return out


def run_mix(args, ntraj, steps, warm, precision, dropin_sample):
    """Batched Chebyshev (one launch per step for the whole mix) vs the plain
    FP64 drop-in (propagationelhl_gpucaller_ semantics: Taylor, one trajectory
    per call) on the same mix.  Returns a dict of results."""
    import torch
    from dynemol_gb300 import api, systems
    mix = trajectory_mix(ntraj)
    dt = 1e-4
    res = {"ntraj": ntraj, "N_range": [min(s.nao for s in mix), max(s.nao for s in mix)],
           "N_mean": float(np.mean([s.nao for s in mix])), "dt_ps": dt}
    out = {}
    for prec in (api.PREC_FP64, precision):
        b = api.Batch(mix, dt=dt, precision=prec, ncols=2, cheb_tol=1e-12)
        b.init_fmo()
        b.compact()
        b.step(warm, want_pops=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pops = b.step(steps)
        el = time.perf_counter() - t0
        st = b.stats()
        out[prec] = (pops, el, st)
        b.close()
    p64, el64, st64 = out[api.PREC_FP64]
    pmx, elmx, stmx = out[precision]
    res["batched_fp64_steps_per_s"] = ntraj * steps / el64
    res["batched_mixed_steps_per_s"] = ntraj * steps / elmx
    res["mixed_precision"] = {api.PREC_FP32: "fp32", api.PREC_BF16X3: "bf16x3"}.get(precision, "fp64")
    res["mixed_pop_err_vs_fp64"] = float(np.abs(pmx - p64).max())
    res["kernel_ms_per_step_mixed"] = stmx.prop_ms / steps
    # plain FP64 drop-in on a uniform sample of the same mix
    sample = mix[:: max(1, ntraj // dropin_sample)][:dropin_sample]
    t_drop, n_drop = 0.0, 0
    for sysm in sample:
        tr = api.Trajectory(sysm, dt=dt)
        homo = systems.fermi_state(sysm, sysm.fragment_atoms("E"))
        tr.init_fmo(homo + 1, homo)
        tr.step(None, nsteps=1, want_pops=False)  # warm-up (first step starts at tau_max)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tr.step(None, nsteps=2, want_pops=True)
        t_drop += time.perf_counter() - t0
        n_drop += 2
        tr.close()
    # the sample's mean cost per trajectory-step, scaled to the mix by sum N^2
    scale = np.mean([s.nao ** 2 for s in mix]) / np.mean([s.nao ** 2 for s in sample])
    res["dropin_fp64_steps_per_s"] = n_drop / (t_drop * scale)
    res["dropin_sample"] = f"{len(sample)} trajectories x 2 steps, cost scaled to the mix by mean N^2 ({scale:.2f})"
    res["speedup_batched_mixed_vs_dropin_fp64"] = res["batched_mixed_steps_per_s"] / res["dropin_fp64_steps_per_s"]
    return res


def serve_all(sv_factory, mix, steps, submit_at=None):
    """Submit every system of `mix` (fragment LUMO/HOMO pair, `steps` steps) to a
    fresh server and step it until all are done.  submit_at: per-request arrival
    offsets in seconds (None: all at t = 0).  Returns (wall s, populations
    [request][P][nfrag+1], latencies s, statuses)."""
    from dynemol_gb300 import systems
    sv = sv_factory()
    n = len(mix)
    order = list(range(n)) if submit_at is None else sorted(range(n), key=lambda i: submit_at[i])
    ids, pops, lat, status = {}, [None] * n, [0.0] * n, [0] * n
    t0 = time.perf_counter()
    nxt, done = 0, 0
    while done < n:
        now = time.perf_counter() - t0
        while nxt < n and (submit_at is None or submit_at[order[nxt]] <= now):
            i = order[nxt]
            sysm = mix[i]
            homo = systems.fermi_state(sysm, sysm.fragment_atoms("E"))
            ids[sv.submit(sysm, steps if np.isscalar(steps) else steps[i], [homo + 1, homo])] = i
            nxt += 1
        active, pending = sv.step()
        for rid in sv.poll():
            i = ids.pop(rid)
            try:
                p, _, times = sv.result(rid)
                pops[i] = p
                lat[i] = times[2] - times[0]
            except Exception as e:  # a failed request keeps its status; the caller reports it
                status[i] = getattr(e, "status", -1)
            done += 1
        if active == 0 and pending == 0 and nxt < n and submit_at is not None:
            time.sleep(max(0.0, submit_at[order[nxt]] - (time.perf_counter() - t0)))
    wall = time.perf_counter() - t0
    sv.close()
    return wall, pops, np.array(lat), status


def run_served_mix(args, ntraj=512, steps=200, sample=32):
    """The batching workload through the continuous-batching server: every
    trajectory of the uneven mix (N uniform in [200, 3000], dt 0.1 fs, electron
    and hole) submitted at t = 0, served in FP32 and, on the same path, in FP64
    (the reference for the population error of every member).  The plain FP64
    drop-in (propagationelhl_gpucaller_ with host S, h, H', Psi buffers, one
    particle per call, the reference's Taylor semantics) and the solo FP64
    Chebyshev trajectory are timed on a stratified sample of the mix (every
    (ntraj/sample)-th member by N), whose mean cost per trajectory-step stands
    for the mix's.  The speed-up splits into method (Taylor drop-in -> solo
    Chebyshev), batching (solo -> served, FP64) and precision (FP64 -> FP32)."""
    import torch
    from dynemol_gb300 import api, systems
    mix = trajectory_mix(ntraj)
    dt = 1e-4
    res = {"ntraj": ntraj, "steps": steps, "dt_ps": dt, "N_range": [min(s.nao for s in mix), max(s.nao for s in mix)],
           "N_mean": float(np.mean([s.nao for s in mix])), "hbm_budget_GB": 150.0,
           "arrivals": "all requests submitted at t = 0"}
    out = {}
    for name, prec in (("fp32", api.PREC_FP32), ("fp64", api.PREC_FP64)):
        wall, pops, lat, status = serve_all(lambda: api.Server(150e9, dt=dt, precision=prec, cheb_tol=1e-12),
                                            mix, steps)
        out[name] = (wall, pops, lat, status)
        res[f"served_{name}"] = {"trajectory_steps_per_s": ntraj * steps / wall, "wall_s": wall,
                                 "latency_p50_s": float(np.percentile(lat, 50)),
                                 "latency_p99_s": float(np.percentile(lat, 99)),
                                 "failed": int(sum(1 for x in status if x))}
    ok = [i for i in range(ntraj) if not out["fp32"][3][i] and not out["fp64"][3][i]]
    err = [float(np.abs(out["fp32"][1][i] - out["fp64"][1][i]).max()) for i in ok]
    res["pop_err_vs_fp64"] = {"max": max(err), "members_compared": len(ok),
                              "note": "every member's final populations (fragments and totals), FP32 served vs "
                                      "FP64 served"}
    # stratified sample by N: drop-in (host buffers) and solo Chebyshev FP64 (device resident)
    by_n = sorted(range(ntraj), key=lambda i: mix[i].nao)
    stride = max(1, ntraj // sample)
    picks = [by_n[stride // 2 + k * stride] for k in range(min(sample, ntraj // stride))]
    t_drop = t_solo = 0.0
    nstep_s = 2
    for i in picks:
        sysm = mix[i]
        homo = systems.fermi_state(sysm, sysm.fragment_atoms("E"))
        tr = api.Trajectory(sysm, dt=dt)  # host S and h for the drop-in calls
        tr.init_fmo(homo + 1, homo)
        S, h, _ = tr.matrices()
        bra, ket = tr.get_psi()
        tr.close()
        bra = [np.ascontiguousarray(bra[:, p]) for p in range(2)]
        ket = [np.ascontiguousarray(ket[:, p]) for p in range(2)]
        save = [dt / H_BAR, dt / H_BAR]
        for s in range(1 + nstep_s):  # one untimed step, then nstep_s timed ones; el and hl one call each
            t0 = time.perf_counter()
            for p in range(2):
                tau = dt / H_BAR if s == 0 else min(1.15 * save[p], dt / H_BAR)
                *_, save[p] = api.propagationelhl_gpucaller(S, h, bra[p], ket[p], s * dt, (s + 1) * dt, tau)
            if s:
                t_drop += time.perf_counter() - t0
        tr = api.Trajectory(sysm, dt=dt, method=api.METHOD_CHEBYSHEV, precision=api.PREC_FP64, ncols=2,
                            cheb_tol=1e-12)
        tr.init_fmo(homo + 1, homo)
        tr.step(None, nsteps=1, want_pops=False)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        tr.step(None, nsteps=nstep_s, want_pops=True)
        t_solo += time.perf_counter() - t0
        tr.close()
    n_s = len(picks) * nstep_s
    r_drop, r_solo = n_s / t_drop, n_s / t_solo
    r64, r32 = res["served_fp64"]["trajectory_steps_per_s"], res["served_fp32"]["trajectory_steps_per_s"]
    res["dropin_fp64"] = {"trajectory_steps_per_s": r_drop,
                          "sample": f"{len(picks)} members, every {stride}th by N (N {mix[picks[0]].nao}-"
                                    f"{mix[picks[-1]].nao}), {nstep_s} timed steps each after one untimed; "
                                    "two propagationelhl_gpucaller_ calls (electron, hole) per step, host buffers"}
    res["solo_chebyshev_fp64"] = {"trajectory_steps_per_s": r_solo, "sample": "the same members and steps"}
    res["speedup_served_fp32_vs_dropin_fp64"] = r32 / r_drop
    res["speedup_factors"] = {"method": r_solo / r_drop, "batching": r64 / r_solo, "precision": r32 / r64}
    return res


def run_config5(args, nreq=12, rate=200.0, nmax=16384, precision=None):
    """Bounded sample of the serving workload at its stated ranges: Poisson
    arrivals (200 / s), N log-uniform in [256, 16384], 50-5,000 steps, 2-32
    even complex columns, 150 GB budget; fewer requests than a long stream."""
    from dynemol_gb300 import api, systems
    precision = api.PREC_FP32 if precision is None else precision
    rng = systems.SplitMix64(5)
    mix, steps, cols, arrive = [], [], [], []
    t = 0.0
    for i in range(nreq):
        u = ((rng.next_u64() >> 11) + 0.5) / 9007199254740992.0
        t += -np.log(u) / rate
        u = ((rng.next_u64() >> 11) + 0.5) / 9007199254740992.0
        N = 256.0 * (nmax / 256.0) ** u
        mix.append(systems.cubic_cluster(n_atoms=max(8, int(round(N / 3.1))), seed=500 + i))
        steps.append(int(50 + rng.next_u64() % 4951))
        cols.append(2 * (1 + int(rng.next_u64() % 16)))
        arrive.append(t)
    sv = api.Server(150e9, dt=1e-4, precision=precision, cheb_tol=1e-12)
    t0 = time.perf_counter()
    ids, lat, done, nxt = {}, [], 0, 0
    while done < nreq:
        now = time.perf_counter() - t0
        while nxt < nreq and arrive[nxt] <= now:
            sysm = mix[nxt]
            homo = systems.fermi_state(sysm, sysm.fragment_atoms("E"))
            nf = int(sum(sysm.atom_nao[a] for a in sysm.fragment_atoms("E")))
            states = [int(1 + (homo - cols[nxt] // 2 + c) % nf) for c in range(cols[nxt])]
            ids[sv.submit(sysm, steps[nxt], states)] = nxt
            nxt += 1
        active, pending = sv.step()
        for rid in sv.poll():
            ids.pop(rid)
            _, _, times = sv.result(rid)
            lat.append(times[2] - times[0])
            done += 1
        if active == 0 and pending == 0 and nxt < nreq:
            time.sleep(max(0.0, arrive[nxt] - (time.perf_counter() - t0)))
    wall = time.perf_counter() - t0
    sv.close()
    lat = np.array(lat)
    col_steps = sum(s * c for s, c in zip(steps, cols))
    return {"requests": nreq, "arrival_rate_per_s": rate, "N": sorted(s.nao for s in mix), "steps": steps,
            "columns": cols, "hbm_budget_GB": 150.0, "precision": "fp32", "wall_s": wall,
            "request_steps_per_s": sum(steps) / wall, "column_steps_per_s": col_steps / wall,
            "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99))}


def run_precision_study(args, steps=5, ncols=64, nao=8192):
    """Config 3: C/H honeycomb sheet with N = 8192 AOs, 64 complex columns
    (seeded random fragment MOs), fixed nuclei, dt 0.1 fs.  FP32 runs H.Psi as
    FP32 GEMMs on the FP32 pipes, BF16X3 as tensor-core GEMMs (three BF16 terms
    per operand); FP64 runs the GEMV kernel.  Reports steps/s of the 64-column
    block and the population error per step against FP64."""
    import torch
    from dynemol_gb300 import api, systems
    sysm = systems.honeycomb_sheet(nao)
    nf = int(sum(sysm.atom_nao[a] for a in sysm.fragment_atoms("E")))
    states = (systems.SplitMix64(3).permutation(nf)[:ncols] + 1).tolist()
    res = {"N_ao": sysm.nao, "columns": ncols, "dt_ps": 1e-4, "steps": steps}
    pops = {}
    variants = ((api.PREC_FP64, "fp64"), (api.PREC_FP32, "fp32_gemm"), (api.PREC_BF16X3, "bf16x3_tensor_gemm"))
    for prec, name in variants:
        tr = api.Trajectory(sysm, dt=1e-4, method=api.METHOD_CHEBYSHEV, precision=prec, ncols=ncols,
                            nparticles=ncols, cheb_tol=1e-12)
        tr.init_fmo_states(states)
        tr.step(None, nsteps=1, want_pops=False)
        tr.init_fmo_states(states)  # same start for both precisions
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pops[name] = tr.step(None, nsteps=steps)
        el = time.perf_counter() - t0
        st = tr.stats()
        res[name] = {"steps_per_s": steps / el, "kernel_ms_per_step": st.prop_ms / steps,
                     "orders_per_step": st.orders / steps / ncols}
        tr.close()
    for _, name in variants[1:]:
        err = np.abs(pops[name] - pops["fp64"])
        res[name]["pop_err_per_step_vs_fp64"] = [float(x) for x in err[:, :, :-1].max(axis=(1, 2))]
        res[name]["norm_err_per_step_vs_fp64"] = [float(x) for x in err[:, :, -1].max(axis=1)]
        res[name]["speedup_vs_fp64"] = res[name]["steps_per_s"] / res["fp64"]["steps_per_s"]
    return res


def run_serve(args, nreq, rate, steps_scale, nmax, precision, budget):
    """Poisson stream of propagation requests against an HBM budget (continuous
    batching).  Returns latency percentiles and aggregate steps/s."""
    from dynemol_gb300 import api, systems
    rng = systems.SplitMix64(5)
    reqs = []
    t = 0.0
    for i in range(nreq):
        u = ((rng.next_u64() >> 11) + 0.5) / 9007199254740992.0
        t += -np.log(u) / rate
        u = ((rng.next_u64() >> 11) + 0.5) / 9007199254740992.0
        N = 256.0 * (nmax / 256.0) ** u  # log-uniform
        n_atoms = max(8, int(round(N / 3.1)))
        nsteps = max(1, int((50 + rng.next_u64() % 4951) * steps_scale))
        cols = 2 * (1 + int(rng.next_u64() % 16))  # even 2..32
        sysm = systems.cubic_cluster(n_atoms=n_atoms, seed=500 + i)
        homo = systems.fermi_state(sysm, sysm.fragment_atoms("E"))
        nf = int(sum(sysm.atom_nao[a] for a in sysm.fragment_atoms("E")))
        states = [int(1 + (homo - cols // 2 + c) % nf) for c in range(cols)]
        reqs.append((t, sysm, nsteps, states))
    sv = api.Server(budget, dt=1e-4, precision=precision, cheb_tol=1e-12)
    t0 = time.perf_counter()
    nxt, done, lat, total_steps = 0, 0, [], 0
    while done < nreq:
        now = time.perf_counter() - t0
        while nxt < nreq and reqs[nxt][0] <= now:
            sv.submit(reqs[nxt][1], reqs[nxt][2], reqs[nxt][3])
            nxt += 1
        active, pending = sv.step()
        for rid in sv.poll():
            pops, psi, times = sv.result(rid)
            lat.append(times[2] - times[0])
            done += 1
        if active == 0 and pending == 0 and nxt < nreq:
            time.sleep(max(0.0, reqs[nxt][0] - (time.perf_counter() - t0)))
    wall = time.perf_counter() - t0
    total_steps = sum(r[2] for r in reqs)
    sv.close()
    lat = np.array(lat)
    return {"requests": nreq, "arrival_rate_per_s": rate, "N_logrange": [256, nmax], "steps_scale": steps_scale,
            "columns": "even 2..32", "hbm_budget_GB": budget / 1e9, "wall_s": wall,
            "aggregate_steps_per_s": total_steps / wall, "latency_p50_s": float(np.percentile(lat, 50)),
            "latency_p99_s": float(np.percentile(lat, 99))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ehrenfest", choices=sorted(WORKLOAD_DESC))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--method", default="chebyshev", choices=["taylor", "chebyshev"])
    ap.add_argument("--precision", default="oz64", choices=["fp64", "fp32", "bf16x3", "df64", "oz64"])
    ap.add_argument("--mix", type=int, default=0, help="also run the batched-vs-drop-in comparison on a mix "
                    "of this many trajectories (0 = skip)")
    ap.add_argument("--served-mix", type=int, default=512, help="trajectories of the served mix (0 = skip)")
    ap.add_argument("--served-steps", type=int, default=200, help="steps of each served-mix trajectory")
    ap.add_argument("--config5", type=int, default=6, help="requests of the bounded serving sample (0 = skip)")
    ap.add_argument("--no-dropin", action="store_true", help="skip the Taylor drop-in measurement")
    ap.add_argument("--serve", type=int, default=0, help="also run a serving stream of this many requests")
    ap.add_argument("--no-precision-study", action="store_true", help="skip the N = 8192, 64-column study")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        line = run_reference(args, rank, world)
        if line is not None:
            print(json.dumps(line), flush=True)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    line = run_ours(args, rank, world)
    if rank == 0 and args.method == "chebyshev" and args.precision in ("fp64", "oz64") and args.workload != "flake":
        # the same moving-nuclei workload with the other FP64-level operators: OZ64 (every
        # operator product exact on the tensor cores), FP64 on the FP64 pipe, DF64 (FP32
        # pairs; populations tested to 1e-9 against the oracle)
        for p in ("oz64", "fp64", "df64"):
            if p != args.precision:
                line[p + "_variant"] = run_variant(args, p)
    if rank == 0 and args.method == "chebyshev" and not args.no_dropin:
        line["dropin_taylor_fp64"] = run_dropin(args)
        line["dropin_host_fp64"] = run_dropin_host(args)
    if rank == 0 and args.mix:
        from dynemol_gb300 import api
        line["trajectory_mix"] = run_mix(args, args.mix, steps=5, warm=2, precision=api.PREC_FP32,
                                         dropin_sample=4)
    if rank == 0 and args.served_mix:
        line["served_mix"] = run_served_mix(args, args.served_mix, args.served_steps)
    if rank == 0 and args.config5:
        line["serving_config5"] = run_config5(args, args.config5)
    if rank == 0 and not args.no_precision_study:
        line["precision_study"] = run_precision_study(args)
    if rank == 0 and args.serve:
        from dynemol_gb300 import api
        line["serving"] = run_serve(args, args.serve, rate=200.0, steps_scale=0.02, nmax=4096,
                                    precision=api.PREC_FP32, budget=150e9)
    if rank == 0:
        if not args.no_cpu_baseline:
            sysm, dt, moving = workload(args.workload)
            nthreads = os.cpu_count() or 1
            nsteps = 2 if args.workload == "ehrenfest" else 20
            rate, el = cpu_sample(args, sysm, dt, moving, nsteps, nthreads)
            line["cpu_baseline"] = {"value": rate, "unit": "steps/s", "cores": nthreads, "kind": "port",
                                    "sample": f"{nsteps} nuclear steps of the workload after 1 untimed step "
                                              f"({el:.1f} s), oracle port with OpenMP + OpenBLAS"}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
