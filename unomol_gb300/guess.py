"""Initial densities for the SCF driver.

core_hamiltonian: the reference's guess (RHF.hpp:205-211) -- the SCF driver's default.
fragments:        superposition of fragment densities.  The molecule is split into covalently bonded
                  fragments (distance < 1.2 x the sum of covalent radii); every closed-shell fragment
                  gets its own small SCF on the GPU, and its density fills the fragment's diagonal
                  block of P.  For clusters of molecules (the water clusters of the benchmark) this
                  starts the SCF next to its solution, where the core-Hamiltonian guess of a large
                  cluster leaves a near-zero HOMO-LUMO gap and the SCF wanders.  The guess changes the
                  starting point only; the converged energy is that of the SCF equations.
"""
from __future__ import annotations

import numpy as np

from .basis import Basis, full_to_packed
from .molecules import BOHR, Z

# covalent radii in Angstrom
_RCOV = {1: 0.31, 2: 0.28, 3: 1.28, 4: 0.96, 5: 0.84, 6: 0.76, 7: 0.71, 8: 0.66, 9: 0.57, 10: 0.58}


def fragments(b: Basis) -> list[list[int]]:
    """Connected components of the covalent-bond graph (centre indices)."""
    n = b.ncen
    r = np.array([_RCOV.get(int(round(q)), 0.8) for q in b.charges]) / BOHR
    d = np.linalg.norm(b.centers[:, None] - b.centers[None], axis=2)
    bonded = d < 1.2 * (r[:, None] + r[None])
    seen = np.zeros(n, bool)
    out = []
    for s in range(n):
        if seen[s]:
            continue
        comp, stack = [], [s]
        seen[s] = True
        while stack:
            i = stack.pop()
            comp.append(i)
            for j in np.nonzero(bonded[i] & ~seen)[0]:
                seen[j] = True
                stack.append(int(j))
        out.append(sorted(comp))
    return out


def _sub_basis(b: Basis, cens: list[int]):
    """Basis of the shells on `cens` (patin text) and the AO indices of the full basis it maps to."""
    cmap = {c: k for k, c in enumerate(cens)}
    lines_c, lines_s, aos = [], [], []
    nelec = 0
    nsh = norb = maxl = 0
    for c in cens:
        lines_c.append(f"{b.charges[c]:15.10f}" + "".join(f"{v:20.12f}" for v in b.centers[c]))
        nelec += int(round(b.charges[c]))
    for s in range(b.nshell):
        c = b.shell_center[s]
        if c not in cmap:
            continue
        l = b.shell_l[s]
        a, k = b.shell_prims(s)
        # the stored coefficients are normalised; divide the primitive factor back out so that the
        # fragment Basis re-normalises to the same values
        raw = _unnormalize(l, a, k)
        lines_s.append(f"{len(a):4d}{l:4d}{cmap[c]:6d}")
        for ai, ki in zip(a, raw):
            lines_s.append(f"{ai:.17g} {ki:.17g}")
        nc = (l + 1) * (l + 2) // 2
        aos.extend(range(b.shell_offset[s], b.shell_offset[s] + nc))
        nsh += 1
        norb += nc
        maxl = max(maxl, l)
    head = [f"{nsh:7d}{norb:7d}{len(cens):7d}{maxl:3d}", f"{nelec:7d}{200:7d}", f"{1e-10:24.16e}", " 0 0", " 2 1 0",
            " 0 0 0"]
    return Basis(text="\n".join(head + lines_c + lines_s) + "\n"), np.array(aos)


def _unnormalize(l, a, k):
    """Inverse of Shell::normalize up to a common factor (which the re-normalisation removes)."""
    piterm = 5.568327996831707
    lpow = 1.5 + l
    return [ki / np.sqrt((2 * ai) ** lpow / piterm) for ai, ki in zip(a, k)]


def fragment_density(b: Basis, *, eps: float = 1e-8) -> np.ndarray | None:
    """Packed superposition-of-fragments density (RHF normalisation, P = C_occ C_occ^T), or None when
    the molecule is one fragment or a fragment is open-shell."""
    from . import native
    frags = fragments(b)
    if len(frags) < 2:
        return None
    n = b.norb
    P = np.zeros((n, n))
    cache: dict = {}
    for cens in frags:
        fb, aos = _sub_basis(b, cens)
        if fb.nelec % 2:
            return None
        t = native.TwoElectronInts(fb)
        r = native.scf(t, fb, accel=native.SCF_DIIS, eps=eps, diis_tol=1e-5, maxits=60)
        t.close()
        Pf = np.zeros((fb.norb, fb.norb))
        Pf[np.tril_indices(fb.norb)] = r["P"]
        Pf = Pf + Pf.T - np.diag(np.diag(Pf))
        P[np.ix_(aos, aos)] = Pf
        cache[len(cache)] = r["energy"]
    return full_to_packed(P)
