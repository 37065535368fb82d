"""Host mirror of unomol's Basis (Basis.hpp:17-352): reads patin.dat and normalises the shells.

Only the input side of the reference is mirrored: the header and flags, centres, shells, AO
offsets (Basis.hpp:226-232), the primitive normalisation folded into the coefficients
(Shell::normalize, Basis.hpp:56-75) and the eps clamp (Basis.hpp:249-254).  The positron basis of the
DPM path (posin.bas, Basis.hpp:207-245) is read by read_posin and appended by dpm_augment.
"""
from __future__ import annotations

import math
import sys

import numpy as np

DBL_EPSILON = sys.float_info.epsilon


class Basis:
    def __init__(self, path: str | None = None, text: str | None = None):
        if text is None:
            with open(path) as f:
                text = f.read()
        tok = text.split()
        pos = 0

        def nxt():
            nonlocal pos
            v = tok[pos]
            pos += 1
            return v

        self.nshell = int(nxt())
        self.norb = int(nxt())
        self.ncen = int(nxt())
        self.maxl = int(nxt())
        self.nelec = int(nxt())
        self.maxits = int(nxt())
        self.eps = float(nxt())
        self.int_flag = [int(nxt()), int(nxt())]
        self.scf_flag = [int(nxt()), int(nxt()), int(nxt())]
        self.prt_flag = [int(nxt()), int(nxt()), int(nxt())]
        if self.maxl > 4:
            raise ValueError("Angular Momentum is too large for present program")
        self.charges = np.zeros(self.ncen)
        self.centers = np.zeros((self.ncen, 3))
        for i in range(self.ncen):
            self.charges[i] = float(nxt())
            self.centers[i] = [float(nxt()), float(nxt()), float(nxt())]
        self.shell_l, self.shell_nprim, self.shell_center, self.shell_offset = [], [], [], []
        alpha, coef = [], []
        off = 0
        for _ in range(self.nshell):
            npr, l, cen = int(nxt()), int(nxt()), int(nxt())
            a = [0.0] * npr
            c = [0.0] * npr
            for k in range(npr):
                a[k] = float(nxt())
                c[k] = float(nxt())
            c = _normalize(l, a, c)
            self.shell_l.append(l)
            self.shell_nprim.append(npr)
            self.shell_center.append(cen)
            self.shell_offset.append(off)
            off += (l + 1) * (l + 2) // 2
            alpha += a
            coef += c
        if off != self.norb:
            raise ValueError(f"patin.dat declares {self.norb} orbitals, shells give {off}")
        self.alpha = np.array(alpha)
        self.coef = np.array(coef)
        xeps = DBL_EPSILON * self.norb * self.norb * 0.5
        if self.eps < xeps:
            self.eps = xeps
        self.no2 = self.norb * (self.norb + 1) // 2

    @property
    def nocc(self) -> int:
        return self.nelec // 2

    def shell_prims(self, i: int):
        b = int(sum(self.shell_nprim[:i]))
        return self.alpha[b:b + self.shell_nprim[i]], self.coef[b:b + self.shell_nprim[i]]

    def nuclear_repulsion(self) -> float:
        """RHF.hpp:273-289."""
        s = 0.0
        for i in range(self.ncen):
            for j in range(i + 1, self.ncen):
                s += self.charges[i] * self.charges[j] / math.sqrt(float(((self.centers[i] - self.centers[j]) ** 2).sum()))
        return s


def read_posin(text: str):
    """posin.bas (Basis.hpp:207-245): "nshell norb maxl", then per shell "npr L" and npr lines
    "alpha coef" (the shells sit on the positron centre).  Returns [(L, alphas, normalised coefs)]."""
    tok = text.split()
    nsh, norb, _maxl = int(tok[0]), int(tok[1]), int(tok[2])
    pos, out, nf = 3, [], 0
    for _ in range(nsh):
        npr, l = int(tok[pos]), int(tok[pos + 1])
        pos += 2
        a = [float(tok[pos + 2 * k]) for k in range(npr)]
        c = [float(tok[pos + 2 * k + 1]) for k in range(npr)]
        pos += 2 * npr
        out.append((l, a, _normalize(l, a, c)))
        nf += (l + 1) * (l + 2) // 2
    if nf != norb:
        raise ValueError(f"posin.bas declares {norb} orbitals, shells give {nf}")
    return out


def dpm_augment(b: "Basis", posin: str, position) -> "Basis":
    """The positron-augmented basis of the DPM path (Basis.hpp:229-245, 341-348): a centre of charge +1
    at `position` (bohr) appended after the molecule's centres, carrying the posin.bas shells, whose
    functions follow the molecule's.  The electron count does not change."""
    import copy
    a = copy.copy(b)
    shells = read_posin(posin)
    a.skip_center = b.ncen
    a.ncen = b.ncen + 1
    a.charges = np.append(np.asarray(b.charges, float), 1.0)
    a.centers = np.vstack([np.asarray(b.centers, float), np.asarray(position, float).reshape(1, 3)])
    a.shell_l, a.shell_nprim = list(b.shell_l), list(b.shell_nprim)
    a.shell_center, a.shell_offset = list(b.shell_center), list(b.shell_offset)
    alpha, coef = list(b.alpha), list(b.coef)
    off = b.norb
    for l, al, co in shells:
        a.shell_l.append(l)
        a.shell_nprim.append(len(al))
        a.shell_center.append(b.ncen)
        a.shell_offset.append(off)
        off += (l + 1) * (l + 2) // 2
        alpha += al
        coef += co
    a.alpha, a.coef = np.array(alpha), np.array(coef)
    a.nshell = len(a.shell_l)
    a.norb = off
    a.no2 = off * (off + 1) // 2
    a.maxl = max(b.maxl, max(l for l, _, _ in shells))
    return a


def _normalize(l: int, a, c):
    """Shell::normalize (Basis.hpp:56-75): contracted normalisation folded into the coefficients."""
    twofact = 2.8284271247461903
    piterm = 5.568327996831707
    lpow = 1.5 + l
    s = 0.0
    for i in range(len(a)):
        for j in range(len(a)):
            s += c[i] * c[j] * math.pow(math.sqrt(a[i] * a[j]) / (a[i] + a[j]), lpow)
    s *= twofact
    s = 1.0 / math.sqrt(s)
    return [c[i] * s * math.sqrt(math.pow(2 * a[i], lpow) / piterm) for i in range(len(a))]


def packed_to_full(p: np.ndarray, n: int) -> np.ndarray:
    m = np.zeros((n, n))
    il = np.tril_indices(n)
    m[il] = p
    m = m + m.T - np.diag(np.diag(m))
    return m


def full_to_packed(m: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(m[np.tril_indices(m.shape[0])])
