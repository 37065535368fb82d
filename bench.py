#!/usr/bin/env python
"""Benchmark of the direct two-electron Fock build on the 32-water 6-31G cluster.

One step = one Fock build G(P) (RHF, packed P in, packed G out) of a cluster of 32 rigid waters in
6-31G (416 basis functions; oxygens uniform in a 10 A cube with O-O >= 2.7 A, random orientations,
numpy default_rng(0)), the precision workload of the reference's headline metric.  Synthetic data:
the geometry is generated, the density is a fixed synthetic symmetric matrix (RHF form P = C C^T of
random orthonormal occupied orbitals, 160 doubly occupied), since the reference measures on no public
dataset.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--form fp64|mixed] [--impl ours|reference]

value: Fock builds/s with P and G resident in HBM (device entry point), device time from CUDA events
on the build's stream, L2 flushed (256 MiB write) between timed builds.  e2e: the same metric through
the host entry point (unomol_gpu_fock_rhf: pinned host P in, host G out, copies inside the timing).
roofline: the ERI + J/K kernels (every class instance of the launch) against the FP64 FMA peak measured
by the library's own microbenchmark (the kernels are bound by the FP64 pipe, not by HBM or tensor
cores).  cpu_baseline: the C restatement of the reference algorithm (oracle/) on the host cores, on a
strided sample of the shell quartets.  --impl reference: that CPU implementation as the reference arm.
Multi-GPU: replicas only (every rank builds its own Fock matrix; value sums over ranks).
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

METRIC = "Fock builds/sec (32-water 6-31G RHF Fock build)"
UNIT = "Fock builds/s"
WORKLOAD = "32-water cluster, 6-31G, RHF Fock build G(P), 416 basis functions (seed 0)"
CPU_STRIDE = 64


def workload():
    from unomol_gb300 import molecules
    from unomol_gb300.basis import Basis
    b = Basis(text=molecules.patin_text(molecules.water_cluster(32, 0), "6-31G"))
    n, nocc = b.norb, b.nelec // 2
    rng = np.random.default_rng(1234)
    q, _ = np.linalg.qr(rng.normal(size=(n, nocc)))
    C = q * 0.9
    P = C @ C.T
    return b, np.ascontiguousarray(P[np.tril_indices(n)])


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index: int):
        self.p = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv")
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--id={index}", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_port_rate(b, P, stride, threads):
    """Fock builds/s of the C restatement on a 1/stride sample (extrapolated)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import orc
    t0 = time.perf_counter()
    orc.fock(b, P, stride=stride, offset=0, threads=threads)
    dt = time.perf_counter() - t0
    return 1.0 / (dt * stride), dt


def ensure_oracle():
    lib = os.path.join(ROOT, "oracle", "_build", "libunomol_oracle.so")
    if not os.path.exists(lib):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    ensure_oracle()
    b, P = workload()
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_port_rate(b, P, CPU_STRIDE * 4, threads)
    times = []
    for _ in range(args.steps):
        r, dt = cpu_port_rate(b, P, CPU_STRIDE, threads)
        times.append(dt * CPU_STRIDE)
    value = len(times) / sum(times)
    sample = f"every {CPU_STRIDE}th canonical shell quartet per step ({100.0 / CPU_STRIDE:.2f}% of the build), extrapolated"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 / value, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "form": "reference algorithm (C restatement), FP64"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def profile_traffic(form):
    """dram bytes per launch of the dominant kernel from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", f"fock_{form}_water32_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f).get("traffic_bytes_per_build")
    return None


def run_ours(args):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from unomol_gb300 import native
    b, P = workload()
    ctx = native.TwoElectronInts(b)
    if args.form == "mixed":
        ctx.set_precision(native.PREC_MIXED, args.fp32_cutoff)
    # a dedicated stream: the library maps a NULL stream handle to its own context stream, so the
    # builds and the timing events must share a non-default torch stream
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    sp = stream.cuda_stream
    assert sp != 0
    dP = torch.from_numpy(P).to(dev)
    dG = torch.zeros_like(dP)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        dG.zero_()
        ctx.fock_device(dP.data_ptr(), dG.data_ptr(), sp)
    if args.profile:
        # profiling mode (for ncu): `steps` device builds after the warm-up, nothing else
        for _ in range(args.steps):
            dG.zero_()
            ctx.fock_device(dP.data_ptr(), dG.data_ptr(), sp)
        torch.cuda.synchronize(dev)
        print(json.dumps({"profile_builds": args.steps, "form": args.form}), flush=True)
        return 0
    # one counted build (untimed) for the algorithmic flops of the ERI kernels
    ctx.set_counting(True)
    dG.zero_()
    ctx.fock_device(dP.data_ptr(), dG.data_ptr(), sp)
    torch.cuda.synchronize(dev)
    st = ctx.stats()
    ctx.set_counting(False)
    launches_per_build = st["kernel_launches"]
    # timed region: K builds, L2 flushed before each
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    clocks = Clocks(local)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    eri_ms = []
    for k in range(args.steps):
        flush.fill_(k & 0xFF)
        dG.zero_()
        ev[k][0].record(stream)
        ctx.fock_device(dP.data_ptr(), dG.data_ptr(), sp)
        ev[k][1].record(stream)
        eri_ms.append(ctx.last_build_ms()[0])
    torch.cuda.synchronize(dev)
    if ws > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b_) for a, b_ in ev]
    total_s = sum(step_ms) / 1e3
    if ws > 1:
        t = torch.tensor([total_s], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_s = float(t.item())
    value = ws * args.steps / total_s
    # end to end through the host entry point, pinned host buffers
    Ph = torch.from_numpy(P).pin_memory()
    Gh = torch.zeros(len(P), dtype=torch.float64).pin_memory()
    Pn, Gn = Ph.numpy(), Gh.numpy()
    for _ in range(max(1, args.warmup // 2)):
        Gn[:] = 0.0
        ctx.formGmatrix(Pn, Gn)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        Gn[:] = 0.0
        ctx.formGmatrix(Pn, Gn)
    torch.cuda.synchronize(dev)
    e2e_s = time.perf_counter() - t0
    if ws > 1:
        t = torch.tensor([e2e_s], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = ws * args.steps / e2e_s
    # roofline of the ERI + J/K kernels
    peak64 = native.fma_peak(True)
    peak32 = native.fma_peak(False)
    eri_s = statistics.mean(eri_ms) / 1e3
    flops = st["eri_flops"]
    achieved = flops / eri_s / 1e12
    if args.form == "mixed":
        # FP32 and FP64 parts share the launch: time-weighted peak is not separable; report against FP64
        pass
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.form == "fp64" else "f64+f32",
            "data": "synthetic (generated 32-water geometry, synthetic RHF density)",
            "config": {"workload": WORKLOAD, "form": args.form, "rys_mode": "reference-compatible",
                       "schwarz_cutoff": 1e-14, "l2": "flushed: 256 MiB write before every timed build",
                       "nbf": b.norb, "shell_quartets": st["shell_quartets"],
                       "shell_quartets_unscreened": st["shell_quartets_total"],
                       "primitive_quartets_computed": st["primitive_quartets_computed"],
                       "parallelism": f"replicas x{ws}"},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 2 * 8 * len(P), "d2h_bytes_per_step": 8 * len(P)},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak64, "unit": "TFLOP/s",
                         "frac": achieved / peak64, "traffic": profile_traffic(args.form),
                         "kernel": "fock_jk_kernel (all class instances of one build)",
                         "flops_per_launch": flops, "kernel_ms": eri_s * 1e3,
                         "peak_source": "FP64 FMA microbenchmark of this library (unomol_gpu_fma_peak), measured in this run",
                         "fp32_peak": peak32},
            "clocks": clk, "gpu_launches": launches_per_build * args.steps,
            "eri_flops_per_build": flops}
    if rank == 0 and ws == 1:
        ensure_oracle()
        threads = os.cpu_count() or 1
        rate, dt = cpu_port_rate(b, P, CPU_STRIDE, threads)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"C restatement of the reference algorithm, every {CPU_STRIDE}th canonical "
                                          f"shell quartet ({dt:.1f} s), extrapolated to one build"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--form", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--fp32-cutoff", type=float, default=1e-9)
    ap.add_argument("--profile", action="store_true", help="device builds only (for ncu captures)")
    args = ap.parse_args()
    if args.impl == "ours" and not args.profile:
        args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
