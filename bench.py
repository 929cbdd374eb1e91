#!/usr/bin/env python
"""Benchmark: Psi-propagation steps/s of the electron-hole propagator.

Workload (default): the 1,200-atom disordered C/H/O cluster (60/30/10 %, 1.4 A
jittered cubic lattice, N = 3,720 AO), moving nuclei (fresh N(0, 0.02 A^2)
perturbation of every coordinate each step), dt = 0.5 fs, FP64 reference Taylor
propagation of electron and hole (bra and ket), S, h and H' = S^-1 h rebuilt on
the device every step.  One step = one nuclear step of both particles.

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
    raise ValueError(name)


WORKLOAD_DESC = {
    "ehrenfest": "C/H/O cluster 1200 atoms (60/30/10%), jittered 1.4 A cubic lattice, moving nuclei "
                 "(sigma 0.02 A per step), dt 0.5 fs, FP64 Taylor (reference semantics), el+hl bra/ket",
    "flake": "C100H50 honeycomb flake (sigma 0.03 A), fixed nuclei, dt 0.1 fs, FP64 Taylor, el+hl bra/ket",
    "small": "C/H/O cluster 300 atoms, moving nuclei, dt 0.5 fs, FP64 Taylor",
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


# ----------------------------------------------------------------- our arm
def run_ours(args, rank, world):
    import torch
    from dynemol_gb300 import api, build, systems

    build.build()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    api.load()
    stream = torch.cuda.current_stream(dev)
    api.set_stream(stream.cuda_stream)

    sysm, dt, moving = workload(args.workload)
    homo = systems.fermi_state(sysm, np.arange(20))
    W, K = args.warmup, args.steps
    coords = step_coords(sysm, moving, W + K + 1, offset=1000 * rank)
    tr = api.Trajectory(sysm, coords=None if coords is None else coords[0], dt=dt)
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
    prop_ms = rebuild_ms = 0.0
    orders = launches = 0
    torch.cuda.synchronize(dev)
    for i in range(K):
        flush.fill_(float(i))
        ev[i][0].record(stream)
        dev_step(W + i)
        ev[i][1].record(stream)
        st = tr.stats()
        prop_ms += st.prop_ms
        rebuild_ms += st.rebuild_ms
        orders += st.orders
        launches += st.prop_launches + st.rebuild_count
    torch.cuda.synchronize(dev)
    clk = clocks.stop()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    t_dev = ms / 1e3
    if world > 1:
        t = torch.tensor([t_dev], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_dev = float(t.item())

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
    t_e2e = e0.elapsed_time(e1) / 1e3
    if world > 1:
        t = torch.tensor([t_e2e], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_e2e = float(t.item())
    api.set_stream(None)
    tr.close()

    N = sysm.nao
    # roofline of the dominant kernel (the propagation kernel): per executed
    # expansion order of one particle, H' read once for bra (H'^T) and ket (H'):
    # bytes = 8 N^2 + 160 N, flops = 8 N^2 (real x complex, 2 columns)
    per_launch_orders = orders / max(1, K)
    bytes_per_launch = per_launch_orders * (8.0 * N * N + 160.0 * N)
    flops_per_launch = per_launch_orders * 8.0 * N * N
    prop_launch_ms = prop_ms / K
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    achieved_gbs = bytes_per_launch / (prop_launch_ms * 1e-3) / 1e9
    fp64_tflops = flops_per_launch / (prop_launch_ms * 1e-3) / 1e12
    FP64_PEAK = 1.20  # TFLOP/s, FMA probe measured on this machine's GB300 (profiles/gb300_peaks_probe.md)

    line = {
        "metric": "psi_propagation_steps_per_s",
        "value": world * K / t_dev,
        "unit": "steps/s",
        "n_gpus": world,
        "steps": K,
        "warmup": W,
        "ms_per_step": 1e3 * t_dev / K,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded geometry, no external dataset)",
        "config": {"workload": WORKLOAD_DESC[args.workload], "N_ao": N, "natoms": sysm.natoms,
                   "dt_ps": dt, "particles": 2, "method": "taylor_ref", "precision": "fp64",
                   "moving_nuclei": moving, "l2": "flushed (512 MB write) between timed steps",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": world * Ke / t_e2e, "unit": "steps/s",
                "h2d_bytes_per_step": (nc * 8) if moving else 0, "d2h_bytes_per_step": 2 * nf1 * 8},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                     "frac": achieved_gbs / hbm_peak, "traffic": None,
                     "kernel": "taylor_kernel", "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)",
                     "fp64_alu": {"achieved_tflops": fp64_tflops, "peak_tflops": FP64_PEAK,
                                  "frac": fp64_tflops / FP64_PEAK, "peak_source": "of measured (FMA probe)"},
                     "orders_per_launch": per_launch_orders, "launch_ms": prop_launch_ms},
        "breakdown_ms_per_step": {"propagation": prop_ms / K, "rebuild_S_h_Hprime": rebuild_ms / K},
        "clocks": clk,
    }
    return line


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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ehrenfest", choices=sorted(WORKLOAD_DESC))
    ap.add_argument("--no-cpu-baseline", action="store_true")
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
