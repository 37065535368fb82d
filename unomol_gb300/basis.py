"""Host mirror of unomol's Basis (Basis.hpp:17-352): reads patin.dat and normalises the shells.

Only the input side of the reference is mirrored: the header and flags, centres, shells, AO
offsets (Basis.hpp:226-232), the primitive normalisation folded into the coefficients
(Shell::normalize, Basis.hpp:56-75) and the eps clamp (Basis.hpp:249-254).  The positron basis of
the DPM path (posin.bas) is not read.
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
