#!/usr/bin/env python
"""Benchmark of the direct two-electron Fock build on the 32-water 6-31G cluster.

Workload: 32 rigid waters in 6-31G (416 basis functions; oxygens uniform in a 10 A cube with O-O >= 2.7 A,
random orientations, numpy default_rng(0)), RHF -- the precision workload on which the reference's
headline metric is quoted.  Synthetic data: the geometry is generated (there is no public dataset).

Untimed set-up: one-electron integrals, the superposition-of-fragments guess, and two SCFs to
convergence (DIIS, 1e-10 Eh): the plain FP64 path (full FP64 builds) and the precision form
(incremental builds G(P_k) = G(P_k-1) + G(P_k - P_k-1), FP32 for quartets with Schwarz bound x max|dP|
below the cutoff, full rebuild every 8 builds).  Their energy difference is |dE|.

One step = one Fock build of the precision form's own SCF sequence (the k-th build: full density at
k = 0, 8, ..., else the density change), cycled for K steps.
  value    Fock builds/s, P and G resident in HBM, device time from CUDA events on the build's stream,
           L2 flushed (256 MiB write) before every timed build;
  e2e      the same builds through the host entry point (unomol_gpu_fock_rhf: pinned host P and G in,
           G out, copies inside the timing);
  plain_fp64   the plain FP64 path on the same densities (full builds), device-timed the same way;
  roofline the ERI + J/K kernels of one build against the FP64 and FP32 FMA peaks measured by the
           library's own microbenchmark (scalar work: no tensor-core ceiling applies, and the data
           stays in L2): peak = flops / max(flops64/peak64, flops32/peak32), the two pipes busy at
           once (peak_one_after_other = flops / (flops64/peak64 + flops32/peak32) beside it); flops
           of each part booked to the pipe that does them, at the quartets of the build's own lists;
  fp64_incremental  the same incremental sequence with the FP32 part off (density-screened FP64
           builds): value / fp64_incremental is the gain of FP32, fp64_incremental / plain_fp64 that of
           the incremental build;
  stored_form  the conventional build (the reference's own scheme: every integral computed once, then
           streamed per build): the stored matrix of P -> G in HBM, FP64, builds of the plain SCF's
           densities, its SCF, and the streaming kernel against the measured HBM bandwidth;
  batched_form the batching workload (256 molecules, alkanes C1-C8 and 1-6 water clusters, STO-3G or
           6-31G): batched FP64 and precision-form builds of the converged densities, and the batched
           SCF of both forms (|dE| per molecule);
  cpu_baseline the C restatement of the reference algorithm (oracle/) on the host cores, on a
           pseudo-random third of the canonical shell quartets of one full build (hashed sample).
--impl reference: that CPU implementation as the reference arm (same metric and workload): its K steps
           are the K hashed slices of ONE full FP64 build (slice s = the quartets with hash(q) % K == s),
           so the timed region covers exactly one whole build; one slice is timed again on one core.
--form fp64: the plain FP64 path as the measured form.
Multi-GPU: replicas only (every rank runs the whole workload; value sums over ranks).
"""
from __future__ import annotations

import argparse
import atexit
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Fock builds/sec (32-water 6-31G RHF SCF Fock builds)"
UNIT = "Fock builds/s"
WORKLOAD = "32-water cluster, 6-31G, RHF, 416 basis functions (seed 0): Fock builds of the converging SCF"
CPU_BASELINE_STRIDE = 3  # the cpu_baseline of the measured line: a hashed third, ~10 s on 16 Grace cores
FP32_CUTOFF = 1e-3  # swept 1e-7..1e0 in profiles/fp32_cutoff_sweep_water32.md; |dE| stays ~1e-9 Eh here
# quartets with Schwarz bound x max|dP| below this are skipped in a build: at 1e-12 the skipped parts of
# ~1e8 quartets left 1e-9..1e-8 Eh of energy noise per incremental build, which stalled the 1e-10 Eh
# test at FP32 cutoffs of 1e-6 and below; at 1e-13 every cutoff of the sweep converges in 11-12
# iterations, for 1 % more build time at 1e-3
SKIP_CUTOFF = 1e-13
REBUILD = 8


def basis():
    from unomol_gb300 import molecules
    from unomol_gb300.basis import Basis
    return Basis(text=molecules.patin_text(molecules.water_cluster(32, 0), "6-31G", eps=1e-10))


def dist_env():
    from unomol_gb300.replicas import env
    return env()


class Clocks:
    """nvidia-smi sampling of the timed region.

    The sampler is started before the warm-up, so that it is live when the timed region opens
    (start()); it is stopped only after a sample taken at or after the region's end, so that even a
    region shorter than the sampling period has a sample.  The reported figures use the samples taken
    after start(): those inside the region and the first one after it, while the clocks of the load
    still hold."""

    PERIOD_MS = 100
    FIELDS = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, index: int, exe: str = "nvidia-smi"):
        self.p = None
        self.first = 0
        self.path = os.path.join(os.environ.get("UNOMOL_CLOCKS_DIR", tempfile.gettempdir()), f"clocks_{os.getpid()}.csv")
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(
                [exe, f"--id={index}", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", str(self.PERIOD_MS)], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
            return
        atexit.register(self._end)  # no sampler outlives the process, whatever path it leaves by

    def _end(self):
        if self.p is not None and self.p.poll() is None:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()

    def _lines(self):
        try:
            with open(self.path) as f:
                return [l for l in f.read().splitlines() if l.count(",") >= 8]
        except OSError:
            return []

    def _wait_for(self, n: int, timeout_s: float):
        t_end = time.monotonic() + timeout_s
        while len(self._lines()) < n and time.monotonic() < t_end and self.p.poll() is None:
            time.sleep(0.01)

    def start(self):
        """Marks the opening of the timed region (call right before it)."""
        if self.p is not None:
            self._wait_for(1, 3.0)  # the sampler is live
            self.first = len(self._lines())

    def stop(self):
        """Ends sampling after the timed region and summarises the samples taken since start()."""
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self._wait_for(len(self._lines()) + 1, 2.0)  # one sample at or after the region's end
        self._end()
        self.f.close()
        sm, smax, reasons = [], [], set()
        for line in self._lines()[self.first:]:
            parts = [x.strip() for x in line.split(",")]
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(self.FIELDS, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "period_ms": self.PERIOD_MS}


def ensure_oracle():
    if not os.path.exists(os.path.join(ROOT, "oracle", "_build", "libunomol_oracle.so")):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)


def cpu_slice(b, P, stride, offset, threads):
    """Seconds and counts of the C restatement on the hashed slice `offset` of `stride` (a
    pseudo-random 1/stride of the canonical shell quartets of one full build; the stride slices
    partition the build)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import orc
    t0 = time.perf_counter()
    _, cnt = orc.fock(b, P, stride=stride, offset=offset, threads=threads, hashed=True)
    return time.perf_counter() - t0, cnt


def synthetic_density(b):
    n, nocc = b.norb, b.nelec // 2
    q, _ = np.linalg.qr(np.random.default_rng(1234).normal(size=(n, nocc)))
    P = 0.81 * q @ q.T
    return np.ascontiguousarray(P[np.tril_indices(n)])


def run_reference(args):
    """The reference algorithm on the host cores: the K = --steps steps are the K hashed slices of
    one full FP64 build of the workload, so the timed region is exactly one whole build (measured, not
    extrapolated); value = 1 build / the summed step times.  The reference's work does not depend on
    the density (it computes every canonical quartet and keeps |v| > 1e-14), so a synthetic density
    of the cluster's trace stands in for the SCF's densities.  Then slice 0 once more on one core
    (the reference is a serial program): the one-core figure is that slice's time x K."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    ensure_oracle()
    b = basis()
    P = synthetic_density(b)
    threads = os.cpu_count() or 1
    K = max(1, args.steps)
    for w in range(args.warmup):  # warm-up: tiny hashed samples (1/(64 K) of a build each)
        cpu_slice(b, P, 64 * K, w, threads)
    times, counts = [], np.zeros(4, np.int64)
    for s in range(K):
        dt, cnt = cpu_slice(b, P, K, s, threads)
        times.append(dt)
        counts += cnt
    total = sum(times)
    value = 1.0 / total
    t1, cnt1 = cpu_slice(b, P, K, 0, 1)
    single = 1.0 / (t1 * K)
    sample = (f"C restatement of the reference algorithm, full FP64 build of the workload split into {K} hashed slices "
              f"(one per step; together exactly one build: {int(counts[0])} shell quartets, {int(counts[1])} function "
              f"quartets), {threads} threads")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (generated geometry, synthetic density)",
            "impl": "reference",
            "config": {"workload": WORKLOAD, "form": "reference algorithm (CPU), full FP64 build",
                       "step": f"1/{K} of one full build (hashed slice); the {K} steps are one whole build",
                       "extrapolated": False},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
            "single_core": {"value": single, "unit": UNIT, "cores": 1, "kind": "port", "extrapolated": True,
                            "sample": f"hashed slice 0 of {K} ({int(cnt1[1])} function quartets) on one thread: "
                                      f"{t1:.1f} s, x {K}"},
            "slice_s": [round(x, 3) for x in times],
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def measured_hbm():
    """HBM copy bandwidth (GB/s) from MEASURED_PEAKS.json, None when the file is absent."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
    except (OSError, ValueError):
        return None
    for k in ("hbm_gbs", "hbm_GBps", "hbm"):
        v = d.get(k)
        if isinstance(v, (int, float)):
            return float(v)
        if isinstance(v, dict):
            for kk in ("value", "gbs", "burst"):
                if isinstance(v.get(kk), (int, float)):
                    return float(v[kk])
    return None


def profile_traffic(form):
    p = os.path.join(ROOT, "profiles", f"fock_{form}_water32_traffic.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f).get("traffic_bytes_per_build")
    return None


def two_pipe_ceiling(fl64, fl32, peak64, peak32):
    """Ceiling rates (same unit as the peaks) of fl64 FP64 and fl32 FP32 flops: the two parts run
    concurrently on their own pipes, so the work needs at least the longer of the two pipe times; the
    second figure is the ceiling of running them one after the other (the sum of the times)."""
    if fl64 + fl32 <= 0:
        return peak64, peak64
    return ((fl64 + fl32) / max(fl64 / peak64, fl32 / peak32),
            (fl64 + fl32) / (fl64 / peak64 + fl32 / peak32))


def step_inputs(dens):
    """Per build of the sequence: (is_full, density or density change), rebuilding every REBUILD builds."""
    out = []
    for k, D in enumerate(dens):
        if k % REBUILD == 0:
            out.append((True, D))
        else:
            out.append((False, D - dens[k - 1]))
    return out


def timed_builds(ctx, inputs, steps, dev, stream, flush):
    """Device-resident builds: per step an L2 flush, then the build between two events."""
    import torch
    sp = stream.cuda_stream
    dIn = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for _, x in inputs]
    dG = torch.zeros_like(dIn[0])
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    eri = []
    for k in range(steps):
        full, _ = inputs[k % len(inputs)]
        flush.fill_(k & 0xFF)
        if full:
            dG.zero_()
        ev[k][0].record(stream)
        ctx.fock_device(dIn[k % len(inputs)].data_ptr(), dG.data_ptr(), sp)
        ev[k][1].record(stream)
        eri.append(ctx.last_build_ms()[0])
    torch.cuda.synchronize(dev)
    return [a.elapsed_time(b_) for a, b_ in ev], eri


def timed_batch_builds(bat, inputs, steps, dev, stream, flush):
    """The same builds through the batched path (one-molecule batch: persistent kernels, CUDA graph):
    per step an L2 flush, the input copied into the batch's density buffer, the graph replayed."""
    import torch
    from unomol_gb300 import native
    sp = stream.cuda_stream
    dIn = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for _, x in inputs]
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for k in range(steps):
        flush.fill_(k & 0xFF)
        ev[k][0].record(stream)
        bat.fock_device(dIn[k % len(inputs)].data_ptr(), 0, native.BATCH_GRAPH, sp)
        ev[k][1].record(stream)
    torch.cuda.synchronize(dev)
    return [a.elapsed_time(b_) for a, b_ in ev]


def batch_form(args, dev, stream, flush):
    """The batching workload (molecules.batch_workload(0): 256 molecules, 7-108 functions).
    SCF builds: the batched SCF (DIIS, every iteration one CUDA graph) of the plain form (full FP64
    builds) and of the precision form (incremental builds, FP32 below the value's cutoff, full rebuild
    every 8), the device time of each SCF's builds (events around every build), and |dE| per molecule.
    Converged-density builds: batched builds of the FP64 SCF's converged densities in FP64 and in the
    precision form (full builds, autotuned, CUDA graph per build, L2 flushed per build)."""
    from unomol_gb300 import molecules, native
    from unomol_gb300.basis import Basis
    bases = [Basis(text=t) for _, t in molecules.batch_workload(0)]
    out = {"molecules": len(bases), "nbf_total": int(sum(x.norb for x in bases)),
           "nbf_max": int(max(x.norb for x in bases))}
    bat = native.Batch(bases)
    SH = [native.one_electron_gpu(x) for x in bases]
    S, H = [x[0] for x in SH], [x[1] for x in SH]
    bat.scf(S=S, H=H, maxits=4)  # warm-up of the batched SCF (first-use costs)
    r64 = bat.scf(S=S, H=H)
    bat.set_precision(native.PREC_MIXED, args.fp32_cutoff, SKIP_CUTOFF)
    bat.scf(S=S, H=H, maxits=4, incremental=True)  # warm-up of the precision form's capture
    rm = bat.scf(S=S, H=H, incremental=True)
    # the same SCFs with pseudo-diagonalisation steps after the first two iterations
    bat.scf(S=S, H=H, maxits=4, incremental=True, density=native.DENSITY_PSEUDO)  # warm-up of its capture
    rmp = bat.scf(S=S, H=H, incremental=True, density=native.DENSITY_PSEUDO)
    bat.set_precision(native.PREC_FP64, 0.0, SKIP_CUTOFF)
    r64p = bat.scf(S=S, H=H, density=native.DENSITY_PSEUDO)
    bat.set_precision(native.PREC_MIXED, args.fp32_cutoff, SKIP_CUTOFF)
    dE = np.abs(rm["energy"] - r64["energy"])
    rate64 = r64["builds"] / (r64["fock_ms"] / 1e3)
    ratem = rm["builds"] / (rm["fock_ms"] / 1e3)
    # builds of the converged densities (full builds), FP64 and precision form
    Pcat = np.concatenate(r64["P"])
    conv_rates = {}
    for form in ("fp64", "mixed"):
        if form == "fp64":
            bat.set_precision(native.PREC_FP64, 0.0, SKIP_CUTOFF)
        else:
            bat.set_precision(native.PREC_MIXED, args.fp32_cutoff, SKIP_CUTOFF)
        bat.set_densities(r64["P"])
        bat.autotune(2)
        inp = [(True, Pcat)]
        timed_batch_builds(bat, inp, 3, dev, stream, flush)
        ms = timed_batch_builds(bat, inp, args.steps, dev, stream, flush)
        conv_rates[form] = (len(ms) / (sum(ms) / 1e3), statistics.mean(ms))
    bat.close()
    out.update({"value": ratem, "unit": "batch Fock builds/s (256 molecules each), builds of the batched SCF",
                "ms_per_build": 1e3 / ratem, "fp64_value": rate64, "fp64_ms_per_build": 1e3 / rate64,
                "speedup_vs_fp64_batch": ratem / rate64, "molecule_builds_per_s": len(bases) * ratem,
                "builds": rm["builds"], "fp64_builds": r64["builds"],
                "scf_max_abs_dE": float(dE.max()), "scf_mean_abs_dE": float(dE.mean()),
                "scf_converged": int(np.sum(r64["converged"] & rm["converged"])),
                "scf_wall_s_fp64": r64["seconds"], "scf_wall_s_form": rm["seconds"],
                "graph_used": bool(r64["graph_used"] and rm["graph_used"]),
                "scf_pseudo_diag": {"scf_wall_s_fp64": r64p["seconds"], "scf_wall_s_form": rmp["seconds"],
                                    "speedup_of_form": r64p["seconds"] / rmp["seconds"],
                                    "builds_fp64": r64p["builds"], "builds_form": rmp["builds"],
                                    "pseudo_steps_form": rmp["pseudo_steps"], "pseudo_refused_form": rmp["pseudo_refused"],
                                    "max_abs_dE_vs_fp64_eigen_solve": float(np.abs(rmp["energy"] - r64["energy"]).max()),
                                    "scf_converged": int(np.sum(r64p["converged"] & rmp["converged"])),
                                    "graph_used": bool(r64p["graph_used"] and rmp["graph_used"]),
                                    "note": "density=UNOMOL_DENSITY_PSEUDO: batched eigen-solve for two iterations, then "
                                            "pseudo-diagonalisation steps (grouped matrix products) where every molecule "
                                            "passes the step check, the batched eigen-solve where one does not"},
                "converged_density_builds": {"fp64_ms": conv_rates["fp64"][1], "form_ms": conv_rates["mixed"][1],
                                             "speedup": conv_rates["mixed"][0] / conv_rates["fp64"][0],
                                             "note": "full builds of the FP64 SCF's converged densities, L2 flushed per build"},
                "note": "value: the builds of the precision form's batched SCF (incremental, FP32 below the value's "
                        "cutoff, density skip as the value's) over their device time; fp64_value: the builds of the "
                        "plain batched SCF (full FP64 builds); |dE| per molecule between the two SCFs; builds "
                        "timed inside the SCF's replayed graphs (no L2 flush between them)"})
    return out


def stored_form(b, kw, r64, plain, dens, dev, stream, flush, steps):
    """The conventional build (unomol_gpu_store_integrals): every canonical integral computed once into
    the sparse matrix of P -> G kept in HBM, each build one stream of that matrix (FP64).  Timed on the
    same full densities as plain_fp64; the SCF through the store against the plain SCF; the roofline of
    the streaming kernel against the measured HBM copy bandwidth (algorithmic bytes per build = the
    store's values, columns and row offsets, each read once)."""
    import torch
    from unomol_gb300 import native
    st = native.TwoElectronInts(b)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    st.store_integrals(native.STORE_RHF)
    torch.cuda.synchronize(dev)
    t_store = time.perf_counter() - t0
    info = st.store_info()
    full = [(True, D) for D in dens]
    timed_builds(st, full, 3, dev, stream, flush)
    s_ms, _ = timed_builds(st, full, steps, dev, stream, flush)
    rate = len(s_ms) / (sum(s_ms) / 1e3)
    max_dF = float(np.max(np.abs(st.form_g(r64["P"]) - plain.form_g(r64["P"]))))
    rs = native.scf(st, b, **kw)
    hbm = measured_hbm()
    gbs = info["bytes"] / (statistics.mean(s_ms) * 1e-3) / 1e9
    st.close()
    return {"value": rate, "unit": UNIT, "ms_per_build": statistics.mean(s_ms),
            "store_build_s": t_store, "store_ms_records": info["ms_records"], "store_ms_assemble": info["ms_assemble"],
            "records": info["records"], "nonzeros": info["nonzeros"], "bytes": info["bytes"], "slabs": info["slabs"],
            "abs_dE": abs(rs["energy"] - r64["energy"]), "max_abs_dF": max_dF, "iterations": rs["iterations"],
            "scf_wall_s": rs["seconds"], "scf_wall_s_with_store_build": rs["seconds"] + t_store,
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s",
                         "frac": gbs / hbm if hbm else None, "kernel": "store_spmv",
                         "algorithmic_bytes_per_build": info["bytes"]},
            "note": "dtype f64; builds of the plain SCF's densities (full builds), L2 flushed per build; "
                    "store_build_s = integral pass + assembly, once per geometry"}


def counted_flops(ctx, inputs, dev, stream):
    """Algorithmic flops (FP64, FP32) and launches of every build of the sequence (untimed)."""
    import torch
    ctx.set_counting(True)
    dG = None
    f64, f32, launches, q32, q, fq, pq, scr, dem = [], [], [], [], [], [], [], [], []
    for full, x in inputs:
        dx = torch.from_numpy(np.ascontiguousarray(x)).to(dev)
        if full or dG is None:
            dG = torch.zeros_like(dx)
        ctx.fock_device(dx.data_ptr(), dG.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize(dev)
        st = ctx.stats()
        f64.append(st["eri_flops"] - st["eri_flops_fp32"])
        f32.append(st["eri_flops_fp32"])
        launches.append(st["kernel_launches"])
        q.append(st["shell_quartets"])
        q32.append(st["shell_quartets_fp32"])
        fq.append(st["function_quartets_computed"])
        pq.append(st["primitive_quartets_computed"])
        scr.append(st["shell_quartets_screened"])
        dem.append(st["shell_quartets_demoted"])
    ctx.set_counting(False)
    return f64, f32, launches, q, q32, fq, pq, scr, dem


def run_ours(args):
    import torch

    from unomol_gb300 import guess, native, replicas
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(dev)  # non-default: a NULL handle would mean the library's own stream
    torch.cuda.set_stream(stream)
    b = basis()
    S, T, H = native.one_electron(b)
    t0 = time.perf_counter()
    P0 = guess.fragment_density(b)
    t_guess = time.perf_counter() - t0
    kw = dict(S=S, H=H, accel=native.SCF_DIIS, maxits=100, eps=1e-10, diis_tol=1e-7, guess_P=P0, keep_densities=64)
    plain = native.TwoElectronInts(b)
    r64 = None
    if not (args.profile and args.form == "mixed"):
        native.scf(plain, b, **kw)  # warm-up: first-use costs (module loading, library set-up) stay out of the SCF times
        r64 = native.scf(plain, b, **kw)
    mixed = native.TwoElectronInts(b)
    if args.form == "mixed":
        mixed.set_precision(native.PREC_MIXED, args.fp32_cutoff)
        mixed.set_density_screening(SKIP_CUTOFF)
        rm = native.scf(mixed, b, incremental=True, rebuild_every=REBUILD, **kw)
        inputs = step_inputs(rm["densities"])
    else:
        rm = r64
        inputs = [(True, D) for D in r64["densities"]]
    if args.profile:
        # profiling mode (for ncu with --profile-from-start off): only the `steps` builds after the
        # warm-up sit between cudaProfilerStart and cudaProfilerStop
        dG = torch.zeros(b.no2, dtype=torch.float64, device=dev)
        dins = [torch.from_numpy(np.ascontiguousarray(x)).to(dev) for _, x in inputs]
        for k in range(args.warmup + args.steps):
            if k == args.warmup:
                torch.cuda.synchronize(dev)
                torch.cuda.profiler.start()
            full, _ = inputs[k % len(inputs)]
            if full:
                dG.zero_()
            mixed.fock_device(dins[k % len(inputs)].data_ptr(), dG.data_ptr(), stream.cuda_stream)
        torch.cuda.synchronize(dev)
        torch.cuda.profiler.stop()
        print(json.dumps({"profile_builds": args.steps, "form": args.form}), flush=True)
        return 0
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    clocks = Clocks(local)
    # warm-up, then the counted (untimed) pass for the algorithmic flops
    timed_builds(mixed, inputs, max(args.warmup, 3), dev, stream, flush)
    f64, f32, launches, nq, nq32, nfq, npq, nscr, ndem = counted_flops(mixed, inputs, dev, stream)
    # timed region
    replicas.barrier(ws)
    torch.cuda.synchronize(dev)
    clocks.start()
    step_ms, eri_ms = timed_builds(mixed, inputs, args.steps, dev, stream, flush)
    torch.cuda.synchronize(dev)
    replicas.barrier(ws)
    clk = clocks.stop()
    total_s = replicas.max_over_ranks(sum(step_ms) / 1e3, ws, dev)
    value = ws * args.steps / total_s
    # max |dF|: the form's full build and the plain build of the converged plain-FP64 density
    max_dF = float(np.max(np.abs(mixed.form_g(r64["P"]) - plain.form_g(r64["P"]))))
    # the plain FP64 path on the same densities (full builds)
    plain_inputs = [(True, D) for D in rm["densities"]]
    timed_builds(plain, plain_inputs, 2, dev, stream, flush)
    p_ms, p_eri = timed_builds(plain, plain_inputs, min(args.steps, len(plain_inputs)), dev, stream, flush)
    plain_rate = len(p_ms) / (sum(p_ms) / 1e3)
    # the same incremental sequence with the FP32 part off: density-screened FP64 builds
    # (fp32 cutoff <= skip cutoff), to read the gains of the incremental build and of FP32 apart
    inc64 = native.TwoElectronInts(b)
    inc64.set_precision(native.PREC_MIXED, 0.0)
    inc64.set_density_screening(SKIP_CUTOFF)
    timed_builds(inc64, inputs, 2, dev, stream, flush)
    i_ms, _ = timed_builds(inc64, inputs, args.steps, dev, stream, flush)
    inc_rate = len(i_ms) / (sum(i_ms) / 1e3)
    fp64_incremental = {"value": inc_rate, "unit": UNIT, "ms_per_build": statistics.mean(i_ms),
                        "incremental_gain": inc_rate / plain_rate, "fp32_gain": value / inc_rate,
                        "note": "the value's build sequence, density skip cutoff as the value's, FP32 off: "
                                "fp32_gain = value / this, incremental_gain = this / plain_fp64"}
    inc64.close()
    # the same SCFs with pseudo-diagonalisation steps in place of most eigen-solves (the eigen-solve of
    # cuSOLVER takes ~12 ms at this size, more than a mixed Fock build)
    p64 = native.scf(plain, b, density=native.DENSITY_PSEUDO, **kw)
    pm = (native.scf(mixed, b, incremental=True, rebuild_every=REBUILD, density=native.DENSITY_PSEUDO, **kw)
          if args.form == "mixed" else p64)
    scf_pseudo = {"energy_plain_fp64": p64["energy"], "energy_form": pm["energy"],
                  "abs_dE_vs_plain_fp64_eigen_solve": abs(pm["energy"] - r64["energy"]),
                  "iterations_plain": p64["iterations"], "iterations_form": pm["iterations"],
                  "pseudo_steps_plain": p64["pseudo_steps"], "pseudo_steps_form": pm["pseudo_steps"],
                  "converged": bool(p64["converged"] and pm["converged"]),
                  "scf_wall_s_plain_fp64": p64["seconds"], "scf_wall_s_form": pm["seconds"],
                  "speedup_of_form": p64["seconds"] / pm["seconds"],
                  "phases_s_form": {k: pm["seconds_" + k] for k in ("setup", "fock", "diis", "diag")},
                  "note": "UNOMOL_DENSITY_PSEUDO: first density of each spin, large rotations and the final "
                          "orbital energies by the eigen-solve, every other density by a pseudo-diagonalisation step"}
    stored = None
    if args.form == "mixed" and not args.no_store:
        stored = stored_form(b, kw, r64, plain, rm["densities"], dev, stream, flush, args.steps)
    batched = batch_form(args, dev, stream, flush) if args.form == "mixed" and not args.no_batch else None
    # end to end through the host entry point, pinned host buffers
    pin_in = [torch.from_numpy(np.ascontiguousarray(x)).pin_memory() for _, x in inputs]
    Gh = torch.zeros(b.no2, dtype=torch.float64).pin_memory()
    Gn = Gh.numpy()

    def e2e_steps(n):
        for k in range(n):
            full, _ = inputs[k % len(inputs)]
            if full:
                Gn[:] = 0.0
            mixed.formGmatrix(pin_in[k % len(inputs)].numpy(), Gn)

    e2e_steps(3)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    e2e_steps(args.steps)
    torch.cuda.synchronize(dev)
    e2e = replicas.job_rate(args.steps, time.perf_counter() - t0, ws, dev)
    # roofline of the ERI + J/K kernels over the timed steps
    peak64 = native.fma_peak(True)
    peak32 = native.fma_peak(False)
    fl64 = sum(f64[k % len(inputs)] for k in range(args.steps))
    fl32 = sum(f32[k % len(inputs)] for k in range(args.steps))
    eri_s = sum(eri_ms) / 1e3
    achieved = (fl64 + fl32) / eri_s / 1e12
    peak, peak_serial = two_pipe_ceiling(fl64, fl32, peak64, peak32)
    launches_total = sum(launches[k % len(inputs)] for k in range(args.steps))
    # J/K scatter: 144 algorithmic bytes per computed function quartet (6 density reads and 6 Fock
    # read-modify-writes of 8 bytes), fused into the ERI kernels, against HBM and the L2 figures
    l2_read, l2_atom = native.l2_peak()
    fq_steps = sum(nfq[k % len(inputs)] for k in range(args.steps))
    pq_steps = sum(npq[k % len(inputs)] for k in range(args.steps))
    scatter_bytes = 144.0 * fq_steps
    scatter_gbs = scatter_bytes / eri_s / 1e9
    hbm = measured_hbm()
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": statistics.mean(step_ms), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32" if args.form == "mixed" else "f64",
            "data": "synthetic (generated 32-water geometry; densities of its own SCF)",
            "config": {"workload": WORKLOAD, "form": args.form, "fp32_cutoff": args.fp32_cutoff if args.form == "mixed" else None,
                       "density_skip_cutoff": SKIP_CUTOFF if args.form == "mixed" else None, "rebuild_every": REBUILD,
                       "rys_mode": "reference-compatible", "schwarz_cutoff": 1e-14,
                       "l2": "flushed: 256 MiB write before every timed build", "nbf": b.norb,
                       "builds_in_sequence": len(inputs), "parallelism": f"replicas x{ws}",
                       "shell_quartets_per_build": [int(x) for x in nq], "fp32_shell_quartets_per_build": [int(x) for x in nq32],
                       "screened_shell_quartets_per_build": [int(x) for x in nscr],
                       "fp32_shell_quartets_of_fp64_lists_per_build": [int(x) for x in ndem]},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 2 * 8 * b.no2, "d2h_bytes_per_step": 8 * b.no2,
                    "note": "formGmatrix on pinned host P and G, called back to back as an SCF calls it: no L2 "
                            "flush between calls (the value's device-timed builds each follow a 256 MiB flush)"},
            "roofline": {"bound": "fp64+fp32 pipes", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": profile_traffic(args.form),
                         "kernel": "fock_jk_kernel (all class instances and both precisions of a build)",
                         "flops_fp64": fl64 / args.steps, "flops_fp32": fl32 / args.steps, "kernel_ms": 1e3 * eri_s / args.steps,
                         "peak_fp64": peak64, "peak_fp32": peak32,
                         "peak_note": "peak = (flops64 + flops32) / max(flops64 / peak64, flops32 / peak32): both pipes busy at once",
                         "peak_one_after_other": peak_serial,
                         "peak_source": "FMA microbenchmark of this library (unomol_gpu_fma_peak), this run",
                         "flops_note": "per primitive quartet from device counters per class and precision; "
                                       "per shell quartet (density contraction) at the FP64 and FP32 parts of "
                                       "each build's own work lists"},
            "batched_form": batched,
            "stored_form": stored,
            "plain_fp64": {"value": plain_rate, "unit": UNIT, "ms_per_build": statistics.mean(p_ms),
                           "kernel_ms": statistics.mean(p_eri), "speedup_of_value": value / plain_rate},
            "fp64_incremental": fp64_incremental,
            "scf": {"energy_plain_fp64": r64["energy"], "energy_form": rm["energy"],
                    "abs_dE": abs(rm["energy"] - r64["energy"]), "max_abs_dF": max_dF,
                    "max_abs_dF_note": "G of the converged plain-FP64 density: full build of the form against the plain build",
                    "iterations_plain": r64["iterations"],
                    "iterations_form": rm["iterations"], "converged": bool(r64["converged"] and rm["converged"]),
                    "scf_wall_s_plain_fp64": r64["seconds"], "scf_wall_s_form": rm["seconds"],
                    "fock_ms_plain_fp64": r64["fock_ms"], "fock_ms_form": rm["fock_ms"], "guess_s": t_guess,
                    "phases_s_plain_fp64": {k: r64["seconds_" + k] for k in ("setup", "fock", "diis", "diag")},
                    "phases_s_form": {k: rm["seconds_" + k] for k in ("setup", "fock", "diis", "diag")}},
            "scf_pseudo_diag": scf_pseudo,
            "scatter": {"algorithmic_bytes_per_build": scatter_bytes / args.steps, "achieved_gbs": scatter_gbs,
                        "hbm_gbs": hbm, "frac_of_hbm": scatter_gbs / hbm if hbm else None,
                        "l2_read_gbs": l2_read, "frac_of_l2_read": scatter_gbs / l2_read,
                        "l2_fp64_atomics_per_s": l2_atom * 1e9,
                        "note": "fused into the ERI kernels (the J/K epilogue); time = ERI kernel time"},
            "eri_rate": {"function_quartets_per_s": fq_steps / eri_s, "primitive_quartets_per_s": pq_steps / eri_s,
                         "function_quartets_per_build": fq_steps / args.steps,
                         "primitive_quartets_per_build": pq_steps / args.steps,
                         "note": "unique canonical quartets of each build's work lists (FP64 and FP32 parts), primitive "
                                 "quartets past the 1e-12 prefactor cut, over the ERI kernel time"},
            "clocks": clk, "gpu_launches": launches_total}
    if rank == 0 and ws == 1:
        ensure_oracle()
        threads = os.cpu_count() or 1
        dt, cnt = cpu_slice(b, synthetic_density(b), CPU_BASELINE_STRIDE, 0, threads)
        line["cpu_baseline"] = {"value": 1.0 / (dt * CPU_BASELINE_STRIDE), "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"C restatement of the reference algorithm, full FP64 build: a hashed 1/{CPU_BASELINE_STRIDE} "
                                          f"of the canonical shell quartets ({int(cnt[1])} function quartets, {dt:.1f} s), x "
                                          f"{CPU_BASELINE_STRIDE}"}
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
    ap.add_argument("--form", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--fp32-cutoff", type=float, default=FP32_CUTOFF)
    ap.add_argument("--profile", action="store_true", help="device builds only (for ncu captures)")
    ap.add_argument("--no-batch", action="store_true", help="leave out the 256-molecule batched form")
    ap.add_argument("--no-store", action="store_true", help="leave out the stored-integral (conventional) form")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
