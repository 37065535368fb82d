"""Test infrastructure: ctypes view of the C restatement (oracle/unomol_oracle.c).

Built by `make -C oracle port` (also from __graft_entry__.build()).  Only tests, smoke() and bench.py's
CPU legs use it.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libunomol_oracle.so")


class _Basis(C.Structure):
    _fields_ = [("nshell", C.c_int), ("norb", C.c_int), ("ncen", C.c_int),
                ("shell_l", C.POINTER(C.c_int)), ("shell_nprim", C.POINTER(C.c_int)),
                ("shell_center", C.POINTER(C.c_int)), ("shell_offset", C.POINTER(C.c_int)),
                ("alpha", C.POINTER(C.c_double)), ("coef", C.POINTER(C.c_double)),
                ("centers", C.POINTER(C.c_double))]


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} missing: run `make -C oracle port`")
        L = C.CDLL(LIB_PATH)
        L.orc_fock.restype = C.c_int
        L.orc_fock.argtypes = [C.POINTER(_Basis), C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_int, C.c_longlong, C.c_longlong, C.c_int, C.c_void_p]
        L.orc_records.restype = C.c_longlong
        L.orc_records.argtypes = [C.POINTER(_Basis), C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_longlong]
        _LIB = L
    return _LIB


def _desc(b):
    keep = [np.ascontiguousarray(b.shell_l, np.int32), np.ascontiguousarray(b.shell_nprim, np.int32),
            np.ascontiguousarray(b.shell_center, np.int32), np.ascontiguousarray(b.shell_offset, np.int32),
            np.ascontiguousarray(b.alpha, np.float64), np.ascontiguousarray(b.coef, np.float64),
            np.ascontiguousarray(b.centers, np.float64).reshape(-1)]
    ip, dp = C.POINTER(C.c_int), C.POINTER(C.c_double)
    d = _Basis(b.nshell, b.norb, b.ncen, *(k.ctypes.data_as(ip) for k in keep[:4]),
               *(k.ctypes.data_as(dp) for k in keep[4:]))
    return d, keep


def fock(b, Pa, Pb=None, exact=False, stride=1, offset=0, threads=0, start=0, hashed=False):
    """G(P) (RHF, Pb None) or (Ga, Gb) (UHF), plus counts [shell quartets, function quartets,
    primitive quartets, stored integrals].  stride > 1: only the canonical quartets q with
    q % stride == offset; with hashed, those with hash(q) % stride == offset (a pseudo-random
    1/stride of every class; the stride offsets partition the build)."""
    if hashed and stride > 1:
        stride = -stride
    d, keep = _desc(b)
    Pa = np.ascontiguousarray(Pa, np.float64)
    Ga = np.zeros(b.no2)
    Gb = np.zeros(b.no2) if Pb is not None else None
    if Pb is not None:
        Pb = np.ascontiguousarray(Pb, np.float64)
    cnt = np.zeros(4, np.int64)
    rc = lib().orc_fock(C.byref(d), int(start), Pa.ctypes.data, None if Pb is None else Pb.ctypes.data,
                        Ga.ctypes.data, None if Gb is None else Gb.ctypes.data, 1 if exact else 0,
                        int(stride), int(offset), int(threads), cnt.ctypes.data)
    if rc != 0:
        raise RuntimeError(f"orc_fock failed ({rc})")
    return (Ga if Pb is None else (Ga, Gb)), cnt


def records(b, exact=False, start=0):
    """The stored integrals of the reference's integral pass (TwoElectronInts.cpp:622-671): values and
    canonical labels (i, j, k, l) of every function quartet with |v| > 1e-14, in its loop order."""
    d, keep = _desc(b)
    n = lib().orc_records(C.byref(d), int(start), 1 if exact else 0, None, None, 0)
    if n < 0:
        raise RuntimeError("orc_records: unsupported basis")
    val = np.zeros(max(n, 1))
    ijkl = np.zeros((max(n, 1), 4), np.int32)
    m = lib().orc_records(C.byref(d), int(start), 1 if exact else 0, val.ctypes.data, ijkl.ctypes.data, int(n))
    assert m == n
    return val[:n], ijkl[:n]


def scatter_records(val, ijkl, nbf, Pa, Pb=None):
    """G from stored integral records, by the six-term form of the conventional build: for a record
    v = (ij|kl), with d = 1/2 per coincidence (i = j, k = l, (ij) = (kl)), T_ij += c d v P_kl,
    T_kl += c d v P_ij (c = 4 RHF, 2 UHF with P = Pa + Pb) and T_ik, T_jk, T_il, T_jl -= d v P_jl, P_il,
    P_jk, P_ik (the spin's own density in UHF); G = T + T^T, packed.  Summed over each record's
    permutations this is the reference's scatter (TwoElectronInts.cpp:699-820)."""
    def full(p):
        m = np.zeros((nbf, nbf))
        m[np.tril_indices(nbf)] = p
        return m + np.tril(m, -1).T
    i, j, k, l = (ijkl[:, t].astype(np.int64) for t in range(4))
    d = np.where(i == j, 0.5, 1.0) * np.where(k == l, 0.5, 1.0) * np.where((i == k) & (j == l), 0.5, 1.0)
    dv = d * val
    uhf = Pb is not None
    Pj = full(Pa) + (full(Pb) if uhf else 0.0)
    out = []
    for P in ([full(Pa), full(Pb)] if uhf else [full(Pa)]):
        T = np.zeros((nbf, nbf))
        c = 2.0 if uhf else 4.0
        np.add.at(T, (i, j), c * dv * Pj[k, l])
        np.add.at(T, (k, l), c * dv * Pj[i, j])
        np.add.at(T, (i, k), -dv * P[j, l])
        np.add.at(T, (j, k), -dv * P[i, l])
        np.add.at(T, (i, l), -dv * P[j, k])
        np.add.at(T, (j, l), -dv * P[i, k])
        G = T + T.T
        out.append(G[np.tril_indices(nbf)])
    return (out[0], out[1]) if uhf else out[0]
