"""Synthetic molecules for the benchmark workloads, written in unomol's patin.dat format.

Geometries (Angstrom in, bohr out with BOHR = 0.5291772083, the constant of input.cc:18):
  * water: O (0, 0, 0.1173), H (0, +-0.7572, -0.4692);
  * all-trans alkane C_nH_{2n+2}: C-C 1.54, C-H 1.09, every bond angle 109.47 deg; carbon zig-zag in
    the xy plane, the two H of an inner carbon above and below that plane, each terminal CH3 with
    one H in the plane on the zig-zag continuation (anti to the chain) and two out of plane;
  * water cluster: oxygen positions uniform in a cube (10 A edge) with a minimum O-O distance
    (2.7 A) by rejection sampling, then each monomer rotated by a uniform random unit quaternion,
    all from numpy.random.default_rng(seed).

patin.dat layout (Basis.hpp:181-255): "nshell norb ncen maxl", "nelec maxits", "eps",
"int_flag[0] int_flag[1]", "scf_flag[0..2]", "prt_flag[0..2]", centres (charge x y z in bohr), then
for every shell "npr L centre" followed by npr lines "alpha coef".
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

BOHR = 0.5291772083
Z = {"H": 1, "HE": 2, "LI": 3, "BE": 4, "B": 5, "C": 6, "N": 7, "O": 8, "F": 9, "NE": 10}
_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "basis_sets.json")
_BASIS = None

WATER = [("O", (0.0, 0.0, 0.1173)), ("H", (0.0, 0.7572, -0.4692)), ("H", (0.0, -0.7572, -0.4692))]


def basis_sets() -> dict:
    global _BASIS
    if _BASIS is None:
        with open(_DATA) as f:
            _BASIS = json.load(f)
    return _BASIS


def water():
    return [(e, tuple(x)) for e, x in WATER]


def alkane(n: int, cc: float = 1.54, ch: float = 1.09, angle_deg: float = 109.47):
    """All-trans C_nH_{2n+2} (Angstrom)."""
    th = math.radians(angle_deg)
    dx = cc * math.sin(th / 2)
    dy = cc * math.cos(th / 2)

    def cpos(i):  # zig-zag, also for the virtual neighbours i = -1 and i = n
        return np.array([i * dx, (dy / 2) * (1 if i % 2 == 0 else -1), 0.0])

    C = [cpos(i) for i in range(n)]
    atoms = [("C", tuple(c)) for c in C]
    zhat = np.array([0.0, 0.0, 1.0])
    for i, c in enumerate(C):
        if n == 1:
            dirs = [np.array(v) / math.sqrt(3.0) for v in ((1, 1, 1), (1, -1, -1), (-1, 1, -1), (-1, -1, 1))]
        elif 0 < i < n - 1:
            u1 = (C[i - 1] - c) / cc
            u2 = (C[i + 1] - c) / cc
            b = -(u1 + u2)
            b /= np.linalg.norm(b)
            dirs = [math.cos(th / 2) * b + s * math.sin(th / 2) * zhat for s in (1.0, -1.0)]
        else:
            nb = i + 1 if i == 0 else i - 1
            virt = -1 if i == 0 else n
            u = (C[nb] - c) / cc
            h0 = (cpos(virt) - c) / cc
            mid = -(u + h0) / 2.0
            s = math.sqrt(max(0.0, 1.0 - float(mid @ mid)))
            dirs = [h0, mid + s * zhat, mid - s * zhat]
        for d in dirs:
            atoms.append(("H", tuple(c + ch * d / np.linalg.norm(d))))
    return atoms


def water_cluster(nw: int, seed: int, box: float = 10.0, dmin: float = 2.7):
    rng = np.random.default_rng(seed)
    mono = np.array([x for _, x in WATER])
    mono = mono - mono[0]
    O = []
    tries = 0
    while len(O) < nw:
        p = rng.uniform(0.0, box, 3)
        tries += 1
        if tries > 1_000_000:
            raise RuntimeError("water cluster: cannot place oxygens")
        if all(np.linalg.norm(p - q) >= dmin for q in O):
            O.append(p)
    atoms = []
    for p in O:
        q = rng.normal(size=4)
        a, b, c, d = q / np.linalg.norm(q)
        R = np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                      [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                      [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])
        for e, x in zip(("O", "H", "H"), mono):
            atoms.append((e, tuple(p + R @ x)))
    return atoms


def batch_workload(seed: int = 0, n: int = 256):
    """The batching workload: n molecules, half all-trans alkanes C_kH_{2k+2} with k uniform in 1..8,
    half water clusters of 1..6 monomers (as water_cluster), each in STO-3G or 6-31G by a coin flip;
    everything from numpy.random.default_rng(seed).  Returns [(label, patin text)]."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        basis = "STO-3G" if rng.integers(2) == 0 else "6-31G"
        if i < n // 2:
            k = int(rng.integers(1, 9))
            out.append((f"C{k}H{2 * k + 2}/{basis}", patin_text(alkane(k), basis)))
        else:
            nw = int(rng.integers(1, 7))
            out.append((f"(H2O){nw}/{basis}", patin_text(water_cluster(nw, int(rng.integers(1 << 30))), basis)))
    return out


# A small positron basis for the DPM path (posin.bas: "nshell norb maxl", then per shell "npr L" and
# npr lines "alpha coef"; the shells sit on the positron centre): two s and one p Gaussian.
POSITRON_BASIS = [(0, [(2.0, 1.0)]), (0, [(0.4, 1.0)]), (1, [(0.5, 1.0)])]


def posin_text(shells=POSITRON_BASIS) -> str:
    norb = sum((l + 1) * (l + 2) // 2 for l, _ in shells)
    out = [f"{len(shells)} {norb} {max(l for l, _ in shells)}"]
    for l, prims in shells:
        out.append(f"{len(prims)} {l}")
        out += [f"{a:20.10f}{c:20.10f}" for a, c in prims]
    return "\n".join(out) + "\n"


def grid_text(points) -> str:
    """pos.grid.dat: the number of points, then x y z (bohr) per point (RHF.hpp:308-313)."""
    return "\n".join([str(len(points))] + [f"{x:.10f} {y:.10f} {z:.10f}" for x, y, z in points]) + "\n"


def perturb(atoms, sigma: float, seed: int):
    """Isotropic Gaussian displacement of every atom (Angstrom)."""
    rng = np.random.default_rng(seed)
    return [(e, tuple(np.array(x) + rng.normal(scale=sigma, size=3))) for e, x in atoms]


def patin_text(atoms, basis: str, charge: int = 0, maxits: int = 300, eps: float = 1e-10,
               scf_flags=(2, 1, 0), int_flags=(0, 0)) -> str:
    """patin.dat text for `atoms` (Angstrom) in `basis`, shells atom after atom.  int_flags[0] = 1
    asks for the DPM polarisation potential (positron basis in posin.bas, positions in pos.grid.dat)."""
    lib = basis_sets()
    shells = []
    for c, (e, _) in enumerate(atoms):
        for sh in lib[e.upper()][basis]:
            shells.append((sh["l"], sh["prims"], c))
    norb = sum((l + 1) * (l + 2) // 2 for l, _, _ in shells)
    maxl = max(l for l, _, _ in shells)
    nelec = sum(Z[e.upper()] for e, _ in atoms) - charge
    out = [f"{len(shells):7d}{norb:7d}{len(atoms):7d}{maxl:3d}", f"{nelec:7d}{maxits:7d}", f"{eps:24.16e}",
           " " + " ".join(str(v) for v in int_flags), " " + " ".join(str(v) for v in scf_flags), " 0 0 0"]
    for e, x in atoms:
        out.append(f"{float(Z[e.upper()]):15.10f}" + "".join(f"{v / BOHR:20.12f}" for v in x))
    for l, prims, c in shells:
        out.append(f"{len(prims):4d}{l:4d}{c:6d}")  # whitespace separated for any centre index
        for a, cc in prims:
            out.append(f"{a:20.10f}{cc:20.10f}")
    return "\n".join(out) + "\n"
