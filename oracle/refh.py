"""Test infrastructure: ctypes view of the reference's own objects (oracle/_ref/*.so).

The libraries are compiled, unchanged, from the reference sources by ``oracle/Makefile``; the C ABI is
``oracle/ref_harness.cpp``.  Only tests and the golden-fixture generator use this module, and only in a
container where the reference sources exist (the libraries are not shipped to other machines).
"""
from __future__ import annotations

import ctypes as C
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
# Where the reference sources lie (the fixture generators read its inputs and pbas.lib there):
# $UNOMOL_REFERENCE, else the container's read-only copy that oracle/Makefile also defaults to.
REFERENCE = os.environ.get("UNOMOL_REFERENCE", "/root/reference")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


# Variants: False / "" = stock reference (Rys for lvt <= 8, MD above); True / "md" = -DUNOMOL_MD_INTS;
# "exact" = stock reference with Rys::root2 replaced by exact quadrature (oracle/exact_root2.cpp).
_NAMES = {False: "libunomol_ref.so", "": "libunomol_ref.so", True: "libunomol_ref_md.so",
          "md": "libunomol_ref_md.so", "exact": "libunomol_ref_exact.so"}


def available(md=False) -> bool:
    return os.path.exists(_libpath(md))


def _libpath(md) -> str:
    return os.path.join(REF_DIR, _NAMES[md])


_LIBS: dict = {}


def lib(md=False) -> C.CDLL:
    name = _NAMES[md]
    if name in _LIBS:
        return _LIBS[name]
    L = C.CDLL(os.path.join(REF_DIR, name))
    L.refh_basis_new.restype = C.c_void_p
    L.refh_basis_new.argtypes = [C.c_char_p]
    L.refh_basis_free.argtypes = [C.c_void_p]
    L.refh_basis_dims.argtypes = [C.c_void_p, _ip]
    L.refh_basis_export.restype = C.c_int
    L.refh_basis_export.argtypes = [C.c_void_p, _ip, _dp, _dp, _dp]
    L.refh_tints_new.restype = C.c_void_p
    L.refh_tints_new.argtypes = [C.c_void_p, C.c_int, C.c_char_p]
    L.refh_tints_free.argtypes = [C.c_void_p]
    L.refh_tints_count.restype = C.c_longlong
    L.refh_tints_count.argtypes = [C.c_void_p]
    L.refh_tints_dump.restype = C.c_longlong
    L.refh_tints_dump.argtypes = [C.c_void_p, _dp, _ip, C.c_longlong]
    L.refh_form_g.argtypes = [C.c_void_p, _dp, _dp]
    L.refh_form_g_uhf.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
    L.refh_one_electron.argtypes = [C.c_void_p, _dp, _dp, _dp]
    L.refh_scf.restype = C.c_int
    L.refh_scf.argtypes = [C.c_char_p, C.c_char_p, _dp, C.c_void_p]
    L.refh_dpm_h.restype = C.c_int
    L.refh_dpm_h.argtypes = [C.c_char_p, _dp, C.c_void_p, C.c_void_p, C.c_void_p, _ip]
    L.refh_scf_trace.restype = C.c_int
    L.refh_scf_trace.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p, C.c_int, _dp, C.c_double]
    L.refh_scf_diis.restype = C.c_int
    L.refh_scf_diis.argtypes = [C.c_void_p, C.c_void_p, C.c_char_p, C.c_void_p, C.c_int, C.c_int, C.c_double,
                                C.c_double, _dp, _dp]
    _LIBS[name] = L
    return L


def dpm_h(workdir: str, q):
    """S, T + V, and T + V minus the DPM potential integrals of the reference (GDPMInts.cpp:86-143) over
    the positron-augmented basis of workdir/patin.dat + workdir/posin.bas, positron at q (bohr)."""
    L = lib()
    dims = np.zeros(3, np.int32)
    qq = np.ascontiguousarray(q, np.float64)
    rc = L.refh_dpm_h(os.path.abspath(workdir).encode(), qq, None, None, None, dims)
    if rc:
        raise RuntimeError(f"refh_dpm_h: {rc}")
    no2 = int(dims[1]) * (int(dims[1]) + 1) // 2
    S, Hp, Hd = np.zeros(no2), np.zeros(no2), np.zeros(no2)
    rc = L.refh_dpm_h(os.path.abspath(workdir).encode(), qq, S.ctypes.data, Hp.ctypes.data, Hd.ctypes.data, dims)
    if rc:
        raise RuntimeError(f"refh_dpm_h: {rc}")
    return S, Hp, Hd


class RefBasis:
    """The reference Basis (Basis.hpp:181-255) read from a patin.dat file."""

    def __init__(self, patin_path: str, md: bool = False):
        self.L = lib(md)
        self.h = self.L.refh_basis_new(patin_path.encode())
        d = np.zeros(6, np.int32)
        self.L.refh_basis_dims(self.h, d)
        self.nshell, self.norb, self.ncen, self.maxl, self.nelec, self.maxits = map(int, d)
        self.no2 = self.norb * (self.norb + 1) // 2

    def export(self):
        info = np.zeros(4 * self.nshell, np.int32)
        cap = 64 * self.nshell
        alpha = np.zeros(cap)
        coef = np.zeros(cap)
        cen = np.zeros(4 * self.ncen)
        n = self.L.refh_basis_export(self.h, info, alpha, coef, cen)
        return info.reshape(-1, 4), alpha[:n].copy(), coef[:n].copy(), cen.reshape(-1, 4)

    def one_electron(self):
        S = np.zeros(self.no2)
        T = np.zeros(self.no2)
        H = np.zeros(self.no2)
        self.L.refh_one_electron(self.h, S, T, H)
        return S, T, H

    def __del__(self):
        try:
            self.L.refh_basis_free(self.h)
        except Exception:
            pass


class RefTwoElectronInts:
    """The reference TwoElectronInts (TwoElectronInts.hpp:79-110): integral pass at construction."""

    def __init__(self, basis: RefBasis, start_shell: int = 0):
        self.basis = basis
        self.L = basis.L
        self._tmp = tempfile.mkdtemp(prefix="unomol_ref_")
        self.h = self.L.refh_tints_new(basis.h, start_shell, os.path.join(self._tmp, "MINTS.DAT").encode())

    def records(self):
        n = self.L.refh_tints_count(self.h)
        vals = np.zeros(n)
        ijkl = np.zeros(4 * n, np.int32)
        self.L.refh_tints_dump(self.h, vals, ijkl, n)
        return vals, ijkl.reshape(-1, 4)

    def form_g(self, P):
        G = np.zeros(self.basis.no2)
        self.L.refh_form_g(self.h, np.ascontiguousarray(P, np.float64), G)
        return G

    def form_g_uhf(self, Pa, Pb):
        Ga = np.zeros(self.basis.no2)
        Gb = np.zeros(self.basis.no2)
        self.L.refh_form_g_uhf(self.h, np.ascontiguousarray(Pa, np.float64),
                               np.ascontiguousarray(Pb, np.float64), Ga, Gb)
        return Ga, Gb

    def __del__(self):
        try:
            self.L.refh_tints_free(self.h)
        except Exception:
            pass


def run_scf(patin_path: str, md: bool = False):
    """Stock reference SCF (Unomol.cc:8-26).  Returns a dict with energies, iterations and final P."""
    L = lib(md)
    b = RefBasis(patin_path, md)
    nP = b.no2 * (2 if b.nelec % 2 else 1)
    out = np.zeros(8)
    P = np.zeros(nP)
    with tempfile.TemporaryDirectory(prefix="unomol_scf_") as wd:
        rc = L.refh_scf(os.path.abspath(patin_path).encode(), wd.encode(), out, P.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"refh_scf failed: {rc}")
    return {"energy": out[0], "init_energy": out[1], "iterations": int(out[2]), "ediff": out[3],
            "pdiff": out[4], "nucrep": out[5], "t_ints": out[6], "t_scf": out[7], "P": P}


def scf_trace(basis: RefBasis, tints: RefTwoElectronInts, kmax: int, perturb: float = 0.0) -> np.ndarray:
    """The first kmax total energies of the stock damped SCF loop (RHF.hpp:140-166 / UHF.hpp:150-163,
    core-Hamiltonian guess) of `basis`, with the integrals of `tints` (same shells).  perturb: the
    starting density scaled by (1 + perturb), to measure how the trajectory amplifies a difference."""
    e = np.zeros(kmax)
    with tempfile.TemporaryDirectory(prefix="unomol_trace_") as wd:
        k = basis.L.refh_scf_trace(basis.h, tints.h, wd.encode(), kmax, e, float(perturb))
    if k < 0:
        raise RuntimeError(f"refh_scf_trace failed: {k}")
    return e[:k].copy()


def scf_diis(basis: RefBasis, tints: RefTwoElectronInts, P0=None, maxits: int = 200, nkeep: int = 8,
             eps_e: float = 1e-12, eps_err: float = 1e-9):
    """Pulay DIIS SCF on the reference's own formGmatrix, one-electron integrals and eigen-solver
    (oracle/ref_harness.cpp: diis_loop).  P0: starting density (RHF packed, UHF Pa then Pb) or None for
    the core-Hamiltonian guess.  Returns energy, iterations, converged, max error, last |dE|, P."""
    nP = basis.no2 * (2 if basis.nelec % 2 else 1)
    out = np.zeros(8)
    P = np.zeros(nP)
    p0 = None
    if P0 is not None:
        p0 = np.ascontiguousarray(P0, np.float64)
        assert p0.size == nP
    with tempfile.TemporaryDirectory(prefix="unomol_diis_") as wd:
        rc = basis.L.refh_scf_diis(basis.h, tints.h, wd.encode(), None if p0 is None else p0.ctypes.data,
                                   maxits, nkeep, eps_e, eps_err, out, P)
    if rc != 0:
        raise RuntimeError(f"refh_scf_diis failed: {rc}")
    return {"energy": out[0], "iterations": int(out[1]), "converged": bool(out[2]), "error": out[3],
            "de": out[4], "nucrep": out[5], "seconds": out[6], "x_orthonormality": out[7], "P": P}
