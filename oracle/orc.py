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
