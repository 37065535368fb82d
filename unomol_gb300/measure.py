"""Measurements behind the committed summaries of the batching and precision forms.

    python -m unomol_gb300.measure batch [--reps 5] [--out batch.json]
        The batching workload (molecules.batch_workload(seed=0): 256 molecules, half all-trans alkanes
        C_kH_2k+2 with k in 1..8, half water clusters of 1..6 monomers, STO-3G or 6-31G by a seeded coin
        flip).  Densities: 0.9 x the projector onto nocc random orthonormal vectors (numpy default_rng(0)).
        Device time per build of all 256 molecules (CUDA events on one stream, mean of `reps` after one
        warm-up) for one molecule at a time, the batched persistent launches, the batched CUDA graph,
        and both again after the autotuner; max |G(batch) - G(one at a time)|.  Then the RHF SCF of all
        256 molecules (core-Hamiltonian guess, DIIS, 1e-10 Eh): batched with every iteration as one CUDA
        graph, batched with plain launches, and one molecule at a time through the single-molecule
        driver (wall times; contexts created outside the timing), with the energy differences.

    python -m unomol_gb300.measure gemm [--reps 20] [--out gemm.json]
        The tcgen05 GEMM of the learned guess at the network's shapes (13 856 rows = 16 decane molecules)
        and one 8192^3 square, device time by CUDA events (mean of reps after a warm-up), TFLOP/s against
        the measured BF16 peak of MEASURED_PEAKS.json, with cuBLAS (torch.matmul) beside it.

    python -m unomol_gb300.measure dpm [--points 64] [--out dpm.json]
        DPM polarisation potential of water/6-31G with a 2s1p positron basis on 64 positron positions:
        the grid point after point (one context recalculated per point) against all points as one
        batched SCF whose iterations replay as a CUDA graph.

    python -m unomol_gb300.measure setup [--reps 5] [--out setup.json]
        Wall time of the device set-up (shell pairs, primitive pairs, sorts, Schwarz diagonal, staircase
        work lists): create and the best of `reps` recalculates of one context for n-decane, 32 and 64
        waters (6-31G), and the creation of the 256-molecule batch.

    python -m unomol_gb300.measure store [--system water32|decane] [--reps 5] [--out store.json]
        The conventional build from stored integrals (RHF and UHF stores): construction time, matrix size,
        device time per build against the direct FP64 build, and the agreement of G.

    python -m unomol_gb300.measure sweep [--out sweep.json]
        FP32 cutoff sweep of the precision form on the 32-water 6-31G cluster (molecules.water_cluster(32, 0),
        superposition-of-fragments guess, DIIS, 1e-10 Eh): the incremental mixed-precision SCF against the
        plain FP64 SCF for every cutoff, with dE, max |dF| (G of the final FP64 density built by both
        paths, full builds), iterations, device ms per build and SCF wall time.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import guess, molecules, native
from .basis import Basis


def _batch(reps: int, scf: bool = True) -> dict:
    import torch
    work = molecules.batch_workload(seed=0)
    bases = [Basis(text=t) for _, t in work]
    rng = np.random.default_rng(0)
    Ps = []
    for b in bases:
        q, _ = np.linalg.qr(rng.normal(size=(b.norb, b.nelec // 2)))
        Ps.append(np.ascontiguousarray((0.9 * q @ q.T)[np.tril_indices(b.norb)]))
    bat = native.Batch(bases)
    bat.set_densities(Ps)
    s = torch.cuda.Stream()

    def timeit(mode):
        bat.fock(mode, s.cuda_stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            bat.fock(mode, s.cuda_stream)
        e1.record(s)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    out = {"molecules": len(bases), "basis_functions_total": int(sum(b.norb for b in bases)),
           "nbf_min": int(min(b.norb for b in bases)), "nbf_max": int(max(b.norb for b in bases)), "modes": {}}
    for name, mode in (("sequential", native.BATCH_SEQUENTIAL), ("batched_launches", native.BATCH_LAUNCHES),
                       ("batched_graph", native.BATCH_GRAPH)):
        out["modes"][name] = timeit(mode)
    out["autotune_choice"] = [list(map(int, c)) for c in bat.autotune(2)]
    for name, mode in (("tuned_launches", native.BATCH_LAUNCHES), ("tuned_graph", native.BATCH_GRAPH)):
        out["modes"][name] = timeit(mode)
    Gb = bat.get_focks()
    bat.fock(native.BATCH_SEQUENTIAL)
    Gq = bat.get_focks()
    out["max_abs_dG_batch_vs_sequential"] = float(max(np.abs(a - c).max() for a, c in zip(Gb, Gq)))
    # the precision form in the batched build (FP32 cutoff 1e-3, density skip 1e-13), same densities
    bat.set_precision(native.PREC_MIXED, 1e-3, 1e-13)
    out["modes"]["mixed_graph"] = timeit(native.BATCH_GRAPH)
    Gm = bat.get_focks()
    out["mixed_max_abs_dG_vs_fp64"] = float(max(np.abs(a - c).max() for a, c in zip(Gm, Gb)))
    out["mixed_max_rel_dG_vs_fp64"] = float(max(np.abs(a - c).max() / np.abs(c).max() for a, c in zip(Gm, Gb)))
    bat.set_precision(native.PREC_FP64)
    out["builds_per_s"] = {k: len(bases) / v * 1e3 for k, v in out["modes"].items()}
    # algorithmic FP64 flops of one build of every molecule (the single-molecule contexts' counters, same
    # screening), against the batched build time and the library's FP64 FMA peak
    flops = 0.0
    for b, P in zip(bases, Ps):
        t = native.TwoElectronInts(b)
        t.set_counting(True)
        t.form_g(P)
        flops += t.stats()["eri_flops"]
        t.close()
    best = min(v for k, v in out["modes"].items() if k not in ("sequential", "mixed_graph"))
    out["eri_flops_per_batch_build"] = flops
    out["achieved_tflops"] = flops / best / 1e9
    out["fp64_peak_tflops"] = native.fma_peak(True)
    out["frac_of_fp64_peak"] = out["achieved_tflops"] / out["fp64_peak_tflops"]
    out["speedup_vs_sequential"] = out["modes"]["sequential"] / min(
        v for k, v in out["modes"].items() if k not in ("sequential", "mixed_graph"))
    if scf:
        out["scf"] = _batch_scf(bat, bases)
    return out


def _batch_scf(bat, bases) -> dict:
    """SCF of all molecules: batched (graph, plain launches) against one molecule at a time."""
    import time
    SH = [native.one_electron_gpu(b) for b in bases]
    S, H = [x[0] for x in SH], [x[1] for x in SH]
    kw = dict(eps=1e-10, diis_tol=1e-6, maxits=200)
    bat.scf(S=S, H=H, graph=True, eps=1e-10, diis_tol=1e-6, maxits=2)  # warm-up: first-use set-up stays out
    rg = bat.scf(S=S, H=H, graph=True, **kw)
    rl = bat.scf(S=S, H=H, graph=False, **kw)
    ctxs = [native.TwoElectronInts(b) for b in bases]  # set-up outside the timing, as for the batch
    native.scf(ctxs[0], bases[0], S=S[0], H=H[0], accel=native.SCF_DIIS, conv_type=0, **kw)  # warm-up
    t0 = time.perf_counter()
    seq = [native.scf(c, b, S=s, H=h, accel=native.SCF_DIIS, conv_type=0, **kw)
           for c, b, s, h in zip(ctxs, bases, S, H)]
    t_seq = time.perf_counter() - t0
    for c in ctxs:
        c.close()
    e_seq = np.array([q["energy"] for q in seq])
    return {"molecules": len(bases), "options": kw,
            "batched_graph_s": rg["seconds"], "graph_used": rg["graph_used"], "capture_note": rg["capture_note"],
            "batched_launches_s": rl["seconds"], "one_at_a_time_s": t_seq,
            "speedup_graph_vs_one_at_a_time": t_seq / rg["seconds"],
            "iterations_batched_max": int(rg["iterations"].max()),
            "iterations_one_at_a_time_sum": int(sum(q["iterations"] for q in seq)),
            "converged_batched": int(rg["converged"].sum()), "converged_one_at_a_time": int(sum(q["converged"] for q in seq)),
            "max_abs_dE_batched_vs_one_at_a_time": float(np.max(np.abs(rg["energy"] - e_seq))),
            "max_abs_dE_graph_vs_launches": float(np.max(np.abs(rg["energy"] - rl["energy"])))}


def _sweep() -> dict:
    b = Basis(text=molecules.patin_text(molecules.water_cluster(32, 0), "6-31G", eps=1e-10))
    S, _, H = native.one_electron(b)
    P0 = guess.fragment_density(b)
    kw = dict(S=S, H=H, accel=native.SCF_DIIS, maxits=100, eps=1e-10, diis_tol=1e-7, guess_P=P0)
    t64 = native.TwoElectronInts(b)
    native.scf(t64, b, **kw)  # warm-up: first-use costs (module loading, library set-up) stay out of the times
    r64 = native.scf(t64, b, **kw)
    G64 = t64.form_g(r64["P"])
    ms64 = r64["fock_ms"] / r64["fock_builds"]
    out = {"fp64": {"energy": r64["energy"], "iterations": r64["iterations"], "ms_per_build": ms64,
                    "scf_wall_s": r64["seconds"]}, "rows": []}
    for cut in (1e0, 1e-1, 1e-2, 1e-3, 1e-4, 1e-5, 1e-6, 1e-7):
        tm = native.TwoElectronInts(b)
        tm.set_precision(native.PREC_MIXED, cut)
        tm.set_density_screening(1e-13)
        rm = native.scf(tm, b, incremental=True, **kw)
        Gm = tm.form_g(r64["P"])
        ms = rm["fock_ms"] / rm["fock_builds"]
        out["rows"].append({"fp32_cutoff": cut, "dE": rm["energy"] - r64["energy"],
                            "max_abs_dF": float(np.max(np.abs(Gm - G64))), "iterations": rm["iterations"],
                            "converged": bool(rm["converged"]), "ms_per_build": ms, "speedup": ms64 / ms,
                            "scf_wall_s": rm["seconds"]})
        tm.close()
    return out


def _gemm(reps: int) -> dict:
    """The tensor-core GEMM of the learned guess (unomol_tc_gemm_bf16, C = A B^T, BF16 in, FP32 out)
    against cuBLAS (torch.matmul, BF16 in and out) at the network's shapes and one large square."""
    import ctypes as C

    import torch
    from .learned import _lib
    L = _lib()
    dev = torch.device("cuda", 0)
    st = torch.zeros(1, dtype=torch.int32, device=dev)
    s = torch.cuda.current_stream()
    peak = None
    try:
        with open(__import__("os").path.join(__import__("os").path.dirname(__file__), "..", "MEASURED_PEAKS.json")) as f:
            peak = json.load(f).get("bf16_tflops")
    except (OSError, ValueError):
        pass
    shapes = [("hidden layer, 16 decane molecules", 13856, 256, 256), ("first layer", 13856, 256, 24),
              ("output layer", 13856, 48, 256), ("dH backward", 13856, 256, 48), ("square 8192", 8192, 8192, 8192)]
    out = {"bf16_peak_tflops": peak, "rows": []}
    for name, M, N, K in shapes:
        g = torch.Generator(device="cpu").manual_seed(M + N + K)
        A = torch.randn(M, K, generator=g).to(torch.bfloat16).to(dev)
        B = torch.randn(N, K, generator=g).to(torch.bfloat16).to(dev)
        Cm = torch.empty(M, N, dtype=torch.float32, device=dev)

        def ours():
            rc = L.unomol_tc_gemm_bf16(A.data_ptr(), B.data_ptr(), M, N, K, Cm.data_ptr(), st.data_ptr(),
                                       C.c_void_p(s.cuda_stream))
            assert rc == 0

        def timed(fn):
            fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s)
            for _ in range(reps):
                fn()
            e1.record(s)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / reps

        ms = timed(ours)
        ms_cublas = timed(lambda: A @ B.T)
        err = float((Cm - (A.float() @ B.float().T)).abs().max())
        fl = 2.0 * M * N * K
        byt = 2.0 * (M * K + N * K) + 4.0 * M * N
        out["rows"].append({"shape": name, "M": M, "N": N, "K": K, "ms": ms, "tflops": fl / ms / 1e9,
                            "frac_of_bf16_peak": fl / ms / 1e9 / peak if peak else None,
                            "gbs": byt / ms / 1e6, "ms_cublas_bf16_out": ms_cublas, "max_abs_err": err,
                            "status_flag": int(st.item())})
    return out


def _dpm(npts: int) -> dict:
    """DPM polarisation potential of water/6-31G with the two-s-one-p positron basis on `npts` positron
    positions (radii 3, 4, 5, 6 bohr, directions from a Fibonacci sphere): the points one after the
    other against all points as one batched SCF (CUDA-graph iterations), with their differences."""
    import time
    from . import dpm
    b = Basis(text=molecules.patin_text(molecules.water(), "6-31G", int_flags=(1, 0), scf_flags=(2, 1, 0)))
    posin = molecules.posin_text()
    ndir = max(1, npts // 4)
    k = np.arange(ndir) + 0.5
    th, ph = np.arccos(1 - 2 * k / ndir), np.pi * (1 + 5 ** 0.5) * k
    dirs = np.stack([np.cos(ph) * np.sin(th), np.sin(ph) * np.sin(th), np.cos(th)], 1)
    pts = np.concatenate([r * dirs for r in (3.0, 4.0, 5.0, 6.0)])[:npts]
    gs = dpm.ground_state(b)
    dpm.polarization_potential(b, posin, pts[:1], gs=gs)  # warm-up
    t0 = time.perf_counter()
    seq = dpm.polarization_potential(b, posin, pts, gs=gs)
    t_seq = time.perf_counter() - t0
    t0 = time.perf_counter()
    bat, info = dpm.polarization_potential_batched(b, posin, pts, gs=gs)
    t_bat = time.perf_counter() - t0
    dv = max(abs(x["vpol"] - y["vpol"]) for x, y in zip(seq, bat))
    return {"workload": f"water/6-31G + positron basis (2s1p), {len(pts)} positions", "points": len(pts),
            "one_at_a_time_s": t_seq, "batched_s": t_bat, "batched_parts": info, "speedup": t_seq / t_bat,
            "max_abs_dvpol_batched_vs_sequential": dv,
            "iterations_one_at_a_time": [int(x["iterations"]) for x in seq],
            "iterations_batched_max": max(int(x["iterations"]) for x in bat),
            "converged": [bool(x["converged"]) for x in bat],
            "vpol_range": [float(min(x["vpol"] for x in seq)), float(max(x["vpol"] for x in seq))]}


def _setup(reps: int) -> dict:
    """Wall time of the device set-up (create, recalculate) on three clusters and of the batch create."""
    import time
    cases = [("n-decane/6-31G", molecules.patin_text(molecules.alkane(10), "6-31G")),
             ("32 waters/6-31G", molecules.patin_text(molecules.water_cluster(32, 0), "6-31G")),
             ("64 waters/6-31G (13 A box)", molecules.patin_text(molecules.water_cluster(64, 0, box=13.0), "6-31G"))]
    native.TwoElectronInts(Basis(text=cases[0][1])).close()  # first use: module loading stays out
    out = {"contexts": []}
    for name, text in cases:
        b = Basis(text=text)
        t0 = time.perf_counter()
        t = native.TwoElectronInts(b)
        create = time.perf_counter() - t0
        rec = []
        for _ in range(reps):
            t0 = time.perf_counter()
            t.recalculate(b)
            rec.append(time.perf_counter() - t0)
        st = t.stats()
        t.close()
        out["contexts"].append({"system": name, "nbf": b.norb, "shell_pairs": st["npairs"],
                                "create_ms": 1e3 * create, "recalculate_ms": 1e3 * min(rec)})
    bases = [Basis(text=x) for _, x in molecules.batch_workload(seed=0)]
    t0 = time.perf_counter()
    bat = native.Batch(bases)
    out["batch_create_ms"] = 1e3 * (time.perf_counter() - t0)
    out["batch_molecules"] = len(bases)
    bat.close()
    return out


def _store(reps: int, system: str) -> dict:
    """The conventional build (unomol_gpu_store_integrals, RHF and UHF stores) of n-decane or the 32-water
    cluster (6-31G): construction time (integral pass, assembly), matrix size, device time per build
    (events on one stream, L2 flushed by a 256 MiB write before each build, mean of `reps` after three
    warm-ups) against the direct FP64 build of the same density, and max |G(store) - G(direct)|."""
    import time

    import torch
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    atoms = molecules.alkane(10) if system == "decane" else molecules.water_cluster(32, 0)
    b = Basis(text=molecules.patin_text(atoms, "6-31G"))
    rng = np.random.default_rng(0)
    q, _ = np.linalg.qr(rng.normal(size=(b.norb, b.nelec // 2)))
    P = np.ascontiguousarray((q @ q.T)[np.tril_indices(b.norb)])
    dP = torch.from_numpy(P).to(dev)
    dG = torch.zeros_like(dP)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def timeit(ctx, n):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
        for k in range(n + 3):
            flush.fill_(k & 0xFF)
            if k >= 3:
                ev[k - 3][0].record(stream)
            ctx.fock_device(dP.data_ptr(), dG.data_ptr(), stream.cuda_stream)
            if k >= 3:
                ev[k - 3][1].record(stream)
        torch.cuda.synchronize(dev)
        return sum(a.elapsed_time(c) for a, c in ev) / n

    direct = native.TwoElectronInts(b)
    out = {"system": system + "/6-31G", "nbf": b.norb, "direct_fp64_ms": timeit(direct, max(2, reps // 4))}
    G_direct = direct.form_g(P)
    for kind, name in ((native.STORE_RHF, "rhf"), (native.STORE_UHF, "uhf")):
        t = native.TwoElectronInts(b)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        t.store_integrals(kind)
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t0
        info = t.store_info()
        ms = timeit(t, reps)
        out[name + "_store"] = dict(info, construction_wall_s=wall, ms_per_build=ms,
                                    stream_gbs=info["bytes"] / (ms * 1e-3) / 1e9,
                                    max_abs_dG_vs_direct=float(np.abs(t.form_g(P) - G_direct).max()))
        t.close()
    return out


def main():
    ap = argparse.ArgumentParser(description="batching / precision-form / tensor-core GEMM / DPM / set-up / "
                                             "stored-integral measurements")
    ap.add_argument("what", choices=["batch", "sweep", "gemm", "dpm", "setup", "store"])
    ap.add_argument("--points", type=int, default=64)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--system", default="water32", choices=["water32", "decane"])
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    rep = (_batch(a.reps) if a.what == "batch" else _sweep() if a.what == "sweep" else
           _gemm(max(a.reps, 10)) if a.what == "gemm" else _setup(a.reps) if a.what == "setup" else
           _store(a.reps, a.system) if a.what == "store" else _dpm(a.points))
    print(json.dumps(rep, indent=1))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(rep, f, indent=1)


if __name__ == "__main__":
    main()
