"""Molecular properties after the SCF: multipole moments (MomentInts / AnalyzeMoments, Moments.cpp:98-271)
and the finite-field analysis (RestrictedHartreeFock::FiniteFieldAnalysis, RHF.hpp:235-271;
FiniteFieldMatrix, FField.cpp:6-20), on the GPU.

  * moment integrals: dx, dy, dz, qxx, qxy, qxz, qyy, qyz, qzz about the origin (unomol_gpu_moment_ints);
  * moments: electronic = sum over packed elements of w P m (w = 4 off the diagonal, 2 on it: the weights
    MOMINTS.DAT carries, so electronic = 2 tr(P M) for the RHF half density and tr((Pa + Pb) M) for UHF),
    nuclear = sum_c Z_c r_c (r_c r_c), total = nuclear - electronic; "dipole moment" = total dz and
    "quadrupole moment" = total qzz - (qxx + qyy) / 2, as moments.out prints them;
  * finite field: for a field of magnitude F (5e-3, Basis.hpp FiniteFieldValue) along x, y and z, H - F d_k,
    the SCF restarted from the ground-state density with the loop update / (converger, update, test),
    polnrg_k = E_k - E_gs and alfa_k = -2 polnrg_k / F^2 (which, as in the reference, keeps the
    permanent-dipole term), alfa_iso = mean, alfa_aniso = (2 alfa_z - alfa_x - alfa_y) / 3.  The three
    SCFs run as one batch (unomol_gpu_batch_scf, RHF), or one after the other (also UHF).
"""
from __future__ import annotations

import numpy as np

from . import native
from .basis import Basis

MOMENTS = ("dx", "dy", "dz", "qxx", "qxy", "qxz", "qyy", "qyz", "qzz")
FIELD = 5.0e-3


def packed_weights(n: int) -> np.ndarray:
    w = np.full(n * (n + 1) // 2, 4.0)
    w[np.arange(n) * (np.arange(n) + 3) // 2] = 2.0
    return w


def analyze_moments(b: Basis, P, Pb=None, M=None) -> dict:
    M = native.moment_ints(b) if M is None else M
    dens = np.asarray(P, float) if Pb is None else 0.5 * (np.asarray(P, float) + np.asarray(Pb, float))
    electronic = M @ (packed_weights(b.norb) * dens)
    r, q = np.asarray(b.centers, float), np.asarray(b.charges, float)
    x, y, z = r[:, 0], r[:, 1], r[:, 2]
    nuclear = np.array([q @ x, q @ y, q @ z, q @ (x * x), q @ (x * y), q @ (x * z), q @ (y * y), q @ (y * z), q @ (z * z)])
    total = nuclear - electronic
    return {"total": total, "electronic": electronic, "nuclear": nuclear, "dipole_moment": float(total[2]),
            "quadrupole_moment": float(total[8] - 0.5 * (total[3] + total[6]))}


def finite_field(b: Basis, gs: dict, field: float = FIELD, batched: bool = True, graph: bool = True) -> dict:
    """gs: the ground-state SCF result (native.scf: "energy", "P")."""
    S, _, H = native.one_electron(b)
    M = native.moment_ints(b)
    Hs = [H - field * M[k] for k in range(3)]
    kw = dict(accel=b.scf_flag[1], conv_type=b.scf_flag[0], eps=b.eps, maxits=b.maxits, loop=native.SCF_LOOP_DPM)
    if batched and b.nelec % 2 == 0:
        bat = native.Batch([b, b, b])
        r = bat.scf(S=[S] * 3, H=Hs, guess_P=[gs["P"]] * 3, graph=graph, **kw)
        energies, conv, its = r["energy"], r["converged"], r["iterations"]
        bat.close()
    else:
        ctx = native.TwoElectronInts(b)
        rr = [native.scf(ctx, b, S=S, H=Hk, guess_P=gs["P"], **kw) for Hk in Hs]
        energies = np.array([x["energy"] for x in rr])
        conv = np.array([x["converged"] for x in rr])
        its = np.array([x["iterations"] for x in rr])
        ctx.close()
    polnrg = np.asarray(energies) - gs["energy"]
    alfa = -polnrg * 2.0 / field / field
    return {"field": field, "polnrg": polnrg, "alfa": alfa, "alfa_iso": float(alfa.mean()),
            "alfa_aniso": float((2.0 * alfa[2] - alfa[1] - alfa[0]) / 3.0), "converged": np.asarray(conv),
            "iterations": np.asarray(its)}
