"""DPM polarisation potential on a grid of positron positions (RestrictedHartreeFock::
findPolarizationPotential, RHF.hpp:292-388), on the GPU.

For the molecule's ground state (the SCF of the plain basis: its density P_gs and energy E_gs), and for
every grid point q:
  * the basis is augmented with the posin.bas shells on a +1 centre at q (Basis.hpp:341-348);
  * H = T + V over all centres (the positron a point charge) minus the DPM potential integrals of the
    positron's six-Gaussian charge (GDPMInts.cpp:86-143; unomol_gpu_gdpm on the GPU);
  * the SCF restarts from P_gs padded with zeros (RHF.hpp:318, PmatGs) with eps = 1e-12 (RHF.hpp:302),
    the loop of findPolarizationPotential (one update, then converger / update / test; RHF.hpp:323-329)
    and the patin flags' accelerator and convergence test;
  * vpol = E_final - E_init, vstat = E_init - E_gs, alfa = -2 vpol r^4, as vpol.out and spol.out write
    them (RHF.hpp:333-347, 362-375).  The reference's first point adds the nuclear repulsion to vstat a
    second time (RHF.hpp:332 against :365); the same forms are kept so that the outputs compare line
    by line.
The molecule's centres stay fixed, so each point changes only the shell pairs that involve the
positron shells; the direct Fock build recomputes all of them (there is no integral file to reuse).

polarization_potential runs the points one after the other (one context, recalculated per point);
polarization_potential_batched runs every point's SCF in lockstep as one batch: the one-electron
integrals of all points in one launch, one batched Fock build per iteration for all points, the
iteration replayed as a CUDA graph (unomol_gpu_batch_scf with the reference's damping and tests).
"""
from __future__ import annotations

import time

import numpy as np

from . import native
from .basis import Basis, dpm_augment


def ground_state(b: Basis, ctx=None, **scf_kw):
    """The molecule's SCF (findEnergy, RHF.hpp:114-176) with the patin flags: P_gs, E_gs."""
    ctx = ctx or native.TwoElectronInts(b)
    S, _, H = native.one_electron(b)
    kw = dict(accel=b.scf_flag[1])
    kw.update(scf_kw)
    r = native.scf(ctx, b, S=S, H=H, **kw)
    return r


def polarization_potential(b: Basis, posin: str, points, gs=None, **scf_kw):
    """Rows of vpol.out / spol.out for every point: dict(q, vpol, alfa, vstat, vsum, e_gs, e_init,
    e_final, ediff, iterations, converged, seconds)."""
    points = np.asarray(points, float).reshape(-1, 3)
    if gs is None:
        gs = ground_state(b)
    e_gs, P_gs = gs["energy"], gs["P"]
    a = dpm_augment(b, posin, points[0])
    ctx = native.TwoElectronInts(a)
    P0 = np.zeros(a.no2)
    P0[:b.no2] = P_gs  # packed storage is prefix-stable: the molecule's block comes first
    kw = dict(accel=b.scf_flag[1], conv_type=b.scf_flag[0], eps=1e-12, maxits=b.maxits, loop=native.SCF_LOOP_DPM)
    kw.update(scf_kw)
    rows = []
    for i, q in enumerate(points):
        a.centers[a.skip_center] = q
        ctx.recalculate(a)
        S, _, H = native.one_electron(a)
        ctx.gdpm(q, H)
        nucrep = a.nuclear_repulsion()
        r = native.scf(ctx, a, S=S, H=H, guess_P=P0, **kw)
        e_init, e_final = r["init_energy"], r["energy"]
        vpol = e_final - e_init
        vstat = e_init - e_gs + (nucrep if i == 0 else 0.0)
        r2 = float(q @ q)
        rows.append(dict(q=q.copy(), vpol=vpol, alfa=-2.0 * vpol * r2 * r2, vstat=vstat, vsum=vstat + vpol,
                         e_gs=e_gs, e_init=e_init, e_final=e_final, ediff=r["ediff"], iterations=r["iterations"],
                         converged=bool(r["converged"]), seconds=r["seconds"]))
    ctx.close()
    return rows


def _row(i, q, e_gs, e_init, e_final, nucrep, **extra):
    vpol = e_final - e_init
    vstat = e_init - e_gs + (nucrep if i == 0 else 0.0)
    r2 = float(q @ q)
    out = dict(q=np.array(q, float), vpol=vpol, alfa=-2.0 * vpol * r2 * r2, vstat=vstat, vsum=vstat + vpol, e_gs=e_gs,
               e_init=e_init, e_final=e_final)
    out.update(extra)
    return out


def polarization_potential_batched(b: Basis, posin: str, points, gs=None, graph: bool = True, **scf_kw):
    """The same rows as polarization_potential, all points in one batched SCF.  Returns (rows, info)."""
    points = np.asarray(points, float).reshape(-1, 3)
    if gs is None:
        gs = ground_state(b)
    e_gs, P_gs = gs["energy"], gs["P"]
    t0 = time.perf_counter()
    bases = [dpm_augment(b, posin, q) for q in points]
    bat = native.Batch(bases)
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    S, H = native.one_electron_gpu(bases[0], centers=np.stack([a.centers for a in bases]))
    scratch = native.TwoElectronInts(bases[0])
    for k, (a, q) in enumerate(zip(bases, points)):
        if k:
            scratch.recalculate(a)
        scratch.gdpm(q, H[k])
    scratch.close()
    t_one = time.perf_counter() - t0
    P0 = np.zeros(bases[0].no2)
    P0[:b.no2] = P_gs
    kw = dict(accel=b.scf_flag[1], conv_type=b.scf_flag[0], eps=1e-12, maxits=b.maxits, loop=native.SCF_LOOP_DPM)
    kw.update(scf_kw)
    r = bat.scf(S=list(S), H=list(H), guess_P=[P0] * len(points), graph=graph, **kw)
    rows = [_row(i, q, e_gs, r["init_energy"][i], r["energy"][i], a.nuclear_repulsion(), ediff=r["ediff"][i],
                 iterations=int(r["iterations"][i]), converged=bool(r["converged"][i]))
            for i, (q, a) in enumerate(zip(points, bases))]
    info = dict(setup_s=t_setup, one_electron_s=t_one, scf_s=r["seconds"], graph_used=r["graph_used"],
                capture_note=r["capture_note"])
    bat.close()
    return rows, info
