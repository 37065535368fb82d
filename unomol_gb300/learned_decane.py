"""The learned-guess workload: n-decane geometries, RHF/6-31G, core-Hamiltonian guess vs learned guess.

Geometries: the all-trans C10H22 of molecules.alkane(10) (C-C 1.54, C-H 1.09 A, 109.47 deg), every
atom displaced by an isotropic Gaussian (sigma = 0.05 A per Cartesian component) from
numpy.random.default_rng(seed * 1_000_003 + k) for geometry k.  The first n_train geometries train the
network on the converged densities of the plain SCF (core-Hamiltonian guess); on the held-out ones
the plain SCF and the learned-guess SCF run back to back with the same options, and the report gives
their iterations, wall times and energy differences.

The plain and learned SCF share everything but the starting density: DIIS on the GPU, convergence at
|dE| < eps and max |X^T (FPS - SPF) X| < diis_tol.  The learned run's wall time includes the network's
prediction and the purification.

    python -m unomol_gb300.learned_decane --geometries 2000 --train 1600 --out report.json
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import molecules, native
from .basis import Basis
from .learned import LearnedGuess


def geometries(n: int, sigma: float = 0.05, seed: int = 0, carbons: int = 10):
    base = molecules.alkane(carbons)
    return [molecules.perturb(base, sigma, seed * 1_000_003 + k) for k in range(n)]


def _scf(ctx, b, S, H, opts, guess=None):
    return native.scf(ctx, b, S=S, H=H, accel=native.SCF_DIIS, guess_P=guess, purify=guess is not None, **opts)


def run(n_geom: int = 2000, n_train: int = 1600, sigma: float = 0.05, seed: int = 0, epochs: int = 150,
        batch: int = 16, lr: float = 1e-3, lr_final: float = 1e-5, eps: float = 1e-10, diis_tol: float = 1e-6,
        maxits: int = 200, basis: str = "6-31G", carbons: int = 10, log=None) -> dict:
    say = log or (lambda *a: None)
    t_all = time.perf_counter()
    geoms = geometries(n_geom, sigma, seed, carbons)
    bases = [Basis(text=molecules.patin_text(a, basis, maxits=maxits, eps=eps)) for a in geoms]
    opts = dict(eps=eps, diis_tol=diis_tol, maxits=maxits, conv_type=0)
    ctx = native.TwoElectronInts(bases[0])
    # one-electron integrals of every geometry in one GPU launch
    t0 = time.perf_counter()
    S_all, H_all = native.one_electron_gpu(bases[0], centers=np.stack([b.centers for b in bases]))
    t_one = time.perf_counter() - t0
    one = [(S_all[k], H_all[k]) for k in range(n_geom)]
    # warm-up (first launches, cuBLAS/cuSOLVER handles)
    _scf(ctx, bases[0], *one[0], opts)
    # plain SCF on the training geometries: the training targets
    t0 = time.perf_counter()
    train = []
    for k in range(n_train):
        ctx.recalculate(bases[k])
        r = _scf(ctx, bases[k], *one[k], opts)
        train.append(r)
    t_data = time.perf_counter() - t0
    ok = [k for k in range(n_train) if train[k]["converged"]]
    say(f"data: {len(ok)}/{n_train} converged, {t_data:.1f} s")
    model = LearnedGuess(bases[0], seed=seed)
    for k in ok:
        model.add(bases[k], train[k]["P"])
    t0 = time.perf_counter()
    hist = model.train(0, len(ok), epochs, batch_molecules=batch, lr=lr, lr_final=lr_final, seed=seed)
    t_train = time.perf_counter() - t0
    say(f"train: {epochs} epochs, {t_train:.1f} s, loss {hist[0]:.4g} -> {hist[-1]:.4g}")
    # held-out: plain and learned back to back
    rows = []
    for k in range(n_train, n_geom):
        b = bases[k]
        ctx.recalculate(b)
        p = _scf(ctx, b, *one[k], opts)
        t0 = time.perf_counter()
        Pg = model.predict(b)
        t_pred = time.perf_counter() - t0
        q = _scf(ctx, b, *one[k], opts, guess=Pg)
        rows.append(dict(k=k, plain_its=p["iterations"], plain_s=p["seconds"], plain_E=p["energy"],
                         plain_conv=p["converged"], plain_fock_ms=p["fock_ms"], learned_its=q["iterations"],
                         learned_s=q["seconds"] + t_pred, learned_E=q["energy"], learned_conv=q["converged"],
                         learned_fock_ms=q["fock_ms"], guess_used=q["guess_used"],
                         purify_iterations=q["purify_iterations"], predict_s=t_pred))
    # held-out loss of the trained network against the plain densities
    both = [r for r in rows if r["plain_conv"] and r["learned_conv"]]
    dE = [abs(r["learned_E"] - r["plain_E"]) for r in both]
    pi = np.array([r["plain_its"] for r in rows], float)
    li = np.array([r["learned_its"] for r in rows], float)
    ps = np.array([r["plain_s"] for r in rows])
    ls = np.array([r["learned_s"] for r in rows])
    rep = {
        "workload": f"C{carbons}H{2 * carbons + 2}/{basis} RHF, {n_geom} geometries (sigma {sigma} A, seed {seed}), "
                    f"{n_train} train / {n_geom - n_train} held out",
        "network": {"hidden": model.hidden, "layers": model.layers, "n_rbf": model.n_rbf, "r_cut_bohr": model.r_cut,
                    "n_in": model.n_in, "n_out": model.n_out, "params": model.n_params},
        "training": {"molecules": len(ok), "epochs": epochs, "batch_molecules": batch, "lr": lr, "lr_final": lr_final,
                     "seconds": t_train, "loss_first_epoch": float(hist[0]), "loss_last_epoch": float(hist[-1]),
                     "data_seconds": t_data, "train_not_converged": n_train - len(ok)},
        "held_out": {
            "n": len(rows),
            "plain_mean_iterations": float(pi.mean()), "learned_mean_iterations": float(li.mean()),
            "iteration_reduction": float(1.0 - li.mean() / pi.mean()),
            "plain_mean_seconds": float(ps.mean()), "learned_mean_seconds": float(ls.mean()),
            "wall_reduction": float(1.0 - ls.mean() / ps.mean()),
            "max_abs_dE": float(max(dE)) if dE else None,
            "both_converged": len(both),
            "fallbacks": sum(r["guess_used"] != "purified" for r in rows),
            "mean_predict_seconds": float(np.mean([r["predict_s"] for r in rows])),
            "plain_mean_fock_ms_per_scf": float(np.mean([r["plain_fock_ms"] for r in rows])),
            "learned_mean_fock_ms_per_scf": float(np.mean([r["learned_fock_ms"] for r in rows])),
        },
        "one_electron_gpu_seconds_all_geometries": t_one,
        "scf": {"accel": "DIIS", "eps": eps, "diis_tol": diis_tol, "maxits": maxits},
        "loss_history": [float(x) for x in hist],
        "rows": rows,
        "seconds_total": time.perf_counter() - t_all,
    }
    model.close()
    ctx.close()
    return rep


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--geometries", type=int, default=2000)
    ap.add_argument("--train", type=int, default=1600)
    ap.add_argument("--epochs", type=int, default=150)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    rep = run(a.geometries, a.train, epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.seed,
              log=lambda *x: print(*x, flush=True))
    h = rep["held_out"]
    print(json.dumps({k: v for k, v in rep.items() if k not in ("rows", "loss_history")}, indent=1))
    if a.out:
        with open(a.out, "w") as f:
            json.dump(rep, f, indent=1)
    print(f"iterations {h['plain_mean_iterations']:.2f} -> {h['learned_mean_iterations']:.2f} "
          f"({100 * h['iteration_reduction']:.1f}% fewer), max |dE| {h['max_abs_dE']:.2e} Eh, fallbacks {h['fallbacks']}")


if __name__ == "__main__":
    main()
