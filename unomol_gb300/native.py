"""ctypes binding of the C ABI (include/unomol_gb300.h) and the Python mirror of TwoElectronInts.

The library libunomol_gb300.so is built in-tree by unomol_gb300.build.  There is no CPU fallback:
loading fails loudly when the library is missing, and every call raises on a non-zero status.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .basis import Basis

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libunomol_gb300.so")

PREC_FP64 = 0
PREC_MIXED = 1

# Exported symbols of include/unomol_gb300.h (checked by the CPU tests).
EXPORTS = [
    "unomol_gpu_create", "unomol_gpu_recalculate", "unomol_gpu_fock_rhf", "unomol_gpu_fock_uhf",
    "unomol_gpu_fock_rhf_device", "unomol_gpu_fock_uhf_device", "unomol_gpu_set_precision",
    "unomol_gpu_set_screening", "unomol_gpu_set_rys_mode", "unomol_gpu_get_stats", "unomol_gpu_destroy",
    "unomol_gpu_last_error", "unomol_gpu_version", "unomol_gpu_set_counting", "unomol_gpu_fma_peak",
    "unomol_gpu_last_build_ms", "unomol_gpu_set_density_screening", "unomol_gpu_fock_rhf_noalloc",
    "unomol_one_electron", "unomol_scf", "unomol_gpu_set_eri_method", "unomol_gpu_batch_create",
    "unomol_gpu_batch_buffers", "unomol_gpu_batch_fock", "unomol_gpu_batch_autotune", "unomol_gpu_batch_set_density",
    "unomol_gpu_batch_get_fock", "unomol_gpu_batch_destroy", "unomol_gpu_batch_last_error", "unomol_tc_gemm_bf16",
    "unomol_mlp_create", "unomol_mlp_num_params", "unomol_mlp_get_params", "unomol_mlp_set_params",
    "unomol_mlp_forward", "unomol_mlp_backward", "unomol_mlp_get_grads", "unomol_mlp_adam", "unomol_mlp_destroy",
    "unomol_mlp_last_error", "unomol_guess_create", "unomol_guess_info", "unomol_guess_add_molecule",
    "unomol_guess_num_molecules", "unomol_guess_train", "unomol_guess_loss", "unomol_guess_predict",
    "unomol_guess_get_params", "unomol_guess_set_params", "unomol_guess_destroy", "unomol_guess_last_error",
    "unomol_gpu_one_electron", "unomol_gpu_one_electron_last_error", "unomol_gpu_l2_peak", "unomol_gpu_batch_scf",
    "unomol_gpu_batch_scf_last_error", "unomol_gpu_batch_size", "unomol_gpu_gdpm", "unomol_gpu_gdpm_last_error",
    "unomol_gpu_moment_ints", "unomol_gpu_batch_set_precision", "unomol_gpu_batch_fock_device",
    "unomol_tc_set_wait_polls", "unomol_gpu_set_launch_order", "unomol_gpu_batch_scf_last_builds",
    "unomol_gpu_batch_scf_last_pseudo",
    "unomol_gpu_store_integrals", "unomol_gpu_store_records", "unomol_gpu_drop_store", "unomol_gpu_store_info",
    "unomol_gpu_write_records",
]
STORE_RHF = 1
STORE_UHF = 2
# TwoInts (TwoElectronInts.hpp:20-23): the 24-byte records of the reference's integral file
RECORD_DTYPE = np.dtype([("val", "<f8"), ("i", "<i4"), ("j", "<i4"), ("k", "<i4"), ("l", "<i4")])
RYS_REFERENCE = 0
RYS_EXACT = 1
ERI_REFERENCE = 0
ERI_MD = 1


class BasisDesc(C.Structure):
    _fields_ = [("nshell", C.c_int), ("norb", C.c_int), ("ncen", C.c_int),
                ("shell_l", C.POINTER(C.c_int)), ("shell_nprim", C.POINTER(C.c_int)),
                ("shell_center", C.POINTER(C.c_int)), ("shell_offset", C.POINTER(C.c_int)),
                ("alpha", C.POINTER(C.c_double)), ("coef", C.POINTER(C.c_double)),
                ("centers", C.POINTER(C.c_double))]


class Stats(C.Structure):
    _fields_ = [("shell_quartets", C.c_int64), ("shell_quartets_fp32", C.c_int64),
                ("shell_quartets_total", C.c_int64), ("function_quartets", C.c_int64),
                ("primitive_quartets", C.c_int64), ("ms_eri", C.c_double), ("ms_total", C.c_double),
                ("nbf", C.c_int), ("npairs", C.c_int), ("kernel_launches", C.c_int), ("pad_", C.c_int),
                ("primitive_quartets_computed", C.c_int64), ("eri_flops", C.c_double),
                ("eri_flops_fp32", C.c_double), ("function_quartets_computed", C.c_int64),
                ("shell_quartets_screened", C.c_int64), ("shell_quartets_demoted", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class StoreInfo(C.Structure):
    _fields_ = [("kind", C.c_int), ("slabs", C.c_int), ("records", C.c_int64), ("nonzeros", C.c_int64),
                ("bytes", C.c_int64), ("ms_records", C.c_double), ("ms_assemble", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class UnomolError(RuntimeError):
    pass


_LIB = None
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def lib() -> C.CDLL:
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise UnomolError(f"{LIB_PATH} is missing: build it with `python -m unomol_gb300.build` "
                          "(the Fock build has no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    L.unomol_gpu_create.argtypes = [C.POINTER(BasisDesc), C.c_int, C.POINTER(C.c_void_p)]
    L.unomol_gpu_recalculate.argtypes = [C.c_void_p, _dp]
    L.unomol_gpu_fock_rhf.argtypes = [C.c_void_p, _dp, _dp]
    L.unomol_gpu_fock_uhf.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
    L.unomol_gpu_fock_rhf_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.unomol_gpu_fock_uhf_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.unomol_gpu_set_precision.argtypes = [C.c_void_p, C.c_int, C.c_double]
    L.unomol_gpu_set_screening.argtypes = [C.c_void_p, C.c_double]
    L.unomol_gpu_set_rys_mode.argtypes = [C.c_void_p, C.c_int]
    L.unomol_gpu_set_counting.argtypes = [C.c_void_p, C.c_int]
    L.unomol_gpu_set_launch_order.argtypes = [C.c_void_p, C.c_int]
    L.unomol_tc_set_wait_polls.argtypes = [C.c_int]
    L.unomol_gpu_last_build_ms.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.unomol_gpu_fma_peak.argtypes = [C.c_int, C.POINTER(C.c_double)]
    L.unomol_gpu_get_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
    L.unomol_gpu_destroy.argtypes = [C.c_void_p]
    L.unomol_gpu_destroy.restype = None
    L.unomol_gpu_last_error.argtypes = [C.c_void_p]
    L.unomol_gpu_last_error.restype = C.c_char_p
    L.unomol_gpu_version.restype = C.c_char_p
    _LIB = L
    return L


def _check(rc: int, h=None):
    if rc != 0:
        msg = lib().unomol_gpu_last_error(h).decode(errors="replace")
        raise UnomolError(f"unomol_gb300 error {rc}: {msg}")


def basis_desc(b: Basis):
    """Keeps the arrays alive together with the descriptor."""
    keep = {
        "l": np.ascontiguousarray(b.shell_l, np.int32), "np": np.ascontiguousarray(b.shell_nprim, np.int32),
        "c": np.ascontiguousarray(b.shell_center, np.int32), "o": np.ascontiguousarray(b.shell_offset, np.int32),
        "a": np.ascontiguousarray(b.alpha, np.float64), "k": np.ascontiguousarray(b.coef, np.float64),
        "x": np.ascontiguousarray(b.centers, np.float64).reshape(-1),
    }
    ip = C.POINTER(C.c_int)
    dp = C.POINTER(C.c_double)
    d = BasisDesc(b.nshell, b.norb, b.ncen, keep["l"].ctypes.data_as(ip), keep["np"].ctypes.data_as(ip),
                  keep["c"].ctypes.data_as(ip), keep["o"].ctypes.data_as(ip), keep["a"].ctypes.data_as(dp),
                  keep["k"].ctypes.data_as(dp), keep["x"].ctypes.data_as(dp))
    return d, keep


class TwoElectronInts:
    """GPU drop-in for unomol::TwoElectronInts (TwoElectronInts.hpp:79-110).

    The constructor sets up shell pairs and Schwarz bounds on the GPU (the reference computes and
    stores every integral there); formGmatrix recomputes the integrals and contracts them into G,
    adding into the caller's array as the reference does.
    """

    def __init__(self, basis: Basis, start_shell: int = 0, label: str = "MINTS.DAT"):
        self.basis = basis
        self.start = start_shell
        self.label = label  # kept for interface parity; nothing is stored
        self._h = C.c_void_p()
        d, self._keep = basis_desc(basis)
        _check(lib().unomol_gpu_create(C.byref(d), int(start_shell), C.byref(self._h)))

    def recalculate(self, basis: Basis):
        """TwoElectronInts::recalculate (centre moved)."""
        self.basis = basis
        _check(lib().unomol_gpu_recalculate(self._h, np.ascontiguousarray(basis.centers, np.float64).reshape(-1)), self._h)

    def formGmatrix(self, *args):
        """formGmatrix(P, G) (RHF) or formGmatrix(Pa, Pb, Ga, Gb) (UHF); G arrays are added into."""
        if len(args) == 2:
            P, G = args
            _check(lib().unomol_gpu_fock_rhf(self._h, _c(P), _out(G)), self._h)
        elif len(args) == 4:
            Pa, Pb, Ga, Gb = args
            _check(lib().unomol_gpu_fock_uhf(self._h, _c(Pa), _c(Pb), _out(Ga), _out(Gb)), self._h)
        else:
            raise TypeError("formGmatrix(P, G) or formGmatrix(Pa, Pb, Ga, Gb)")

    def directFormGMatrix(self, P, G, basis: Basis | None = None):
        """The reference's direct variant (TwoElectronInts.cpp:871-1055) has a lossy pair cut; here it
        is the same exact direct build as formGmatrix."""
        self.formGmatrix(P, G)

    def form_g(self, P) -> np.ndarray:
        G = np.zeros(self.basis.no2)
        self.formGmatrix(np.ascontiguousarray(P, np.float64), G)
        return G

    def form_g_uhf(self, Pa, Pb):
        Ga = np.zeros(self.basis.no2)
        Gb = np.zeros(self.basis.no2)
        self.formGmatrix(np.ascontiguousarray(Pa, np.float64), np.ascontiguousarray(Pb, np.float64), Ga, Gb)
        return Ga, Gb

    def fock_device(self, dP_ptr: int, dG_ptr: int, stream: int = 0):
        _check(lib().unomol_gpu_fock_rhf_device(self._h, C.c_void_p(dP_ptr), C.c_void_p(dG_ptr), C.c_void_p(stream)), self._h)

    def fock_device_uhf(self, dPa, dPb, dGa, dGb, stream: int = 0):
        _check(lib().unomol_gpu_fock_uhf_device(self._h, C.c_void_p(dPa), C.c_void_p(dPb), C.c_void_p(dGa),
                                                C.c_void_p(dGb), C.c_void_p(stream)), self._h)

    def gdpm(self, q, H):
        """H -= the DPM potential integrals of a positron at q (unomol_gpu_gdpm, GDPMInts.cpp:86-143)."""
        L = lib()
        L.unomol_gpu_gdpm.argtypes = [C.c_void_p, _dp, _dp]
        L.unomol_gpu_gdpm_last_error.restype = C.c_char_p
        rc = L.unomol_gpu_gdpm(self._h, np.ascontiguousarray(q, np.float64), H)
        if rc != 0:
            raise UnomolError(f"unomol_gpu_gdpm error {rc}: {L.unomol_gpu_gdpm_last_error().decode()}")
        return H

    def set_precision(self, mode: int, fp32_cutoff: float = 1e-10):
        _check(lib().unomol_gpu_set_precision(self._h, int(mode), float(fp32_cutoff)), self._h)

    def set_rys_mode(self, mode: int):
        """RYS_REFERENCE (default, the reference's two-root fit) or RYS_EXACT (exact quadrature)."""
        _check(lib().unomol_gpu_set_rys_mode(self._h, int(mode)), self._h)

    def last_build_ms(self):
        """(ms of the ERI + J/K kernels, ms of the whole build) of the last build, device events."""
        a, b = C.c_double(), C.c_double()
        _check(lib().unomol_gpu_last_build_ms(self._h, C.byref(a), C.byref(b)), self._h)
        return a.value, b.value

    def set_eri_method(self, method: int):
        """ERI_REFERENCE (Rys for la+lb+lc+ld <= 8, MD above; default) or ERI_MD (MD everywhere)."""
        lib().unomol_gpu_set_eri_method.argtypes = [C.c_void_p, C.c_int]
        _check(lib().unomol_gpu_set_eri_method(self._h, int(method)), self._h)

    def set_density_screening(self, skip_cut: float):
        lib().unomol_gpu_set_density_screening.argtypes = [C.c_void_p, C.c_double]
        _check(lib().unomol_gpu_set_density_screening(self._h, float(skip_cut)), self._h)

    def set_counting(self, on: bool):
        _check(lib().unomol_gpu_set_counting(self._h, 1 if on else 0), self._h)

    def set_launch_order(self, reversed_: bool):
        _check(lib().unomol_gpu_set_launch_order(self._h, 1 if reversed_ else 0), self._h)

    def set_screening(self, cutoff: float):
        _check(lib().unomol_gpu_set_screening(self._h, float(cutoff)), self._h)

    def store_integrals(self, kind: int = STORE_RHF, max_gib: float = 0.0):
        """Conventional build: compute every canonical integral once on the GPU and keep the matrix of
        P -> G in device memory; later builds stream it (unomol_gpu_store_integrals)."""
        lib().unomol_gpu_store_integrals.argtypes = [C.c_void_p, C.c_int, C.c_double]
        _check(lib().unomol_gpu_store_integrals(self._h, int(kind), float(max_gib)), self._h)

    def store_records(self, path: str, kind: int = STORE_RHF, max_gib: float = 0.0):
        """The same store from a file of 24-byte TwoInts records (unomol_gpu_store_records)."""
        lib().unomol_gpu_store_records.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.c_double]
        _check(lib().unomol_gpu_store_records(self._h, os.fsencode(path), int(kind), float(max_gib)), self._h)

    def drop_store(self):
        lib().unomol_gpu_drop_store.argtypes = [C.c_void_p]
        _check(lib().unomol_gpu_drop_store(self._h), self._h)

    def store_info(self) -> dict:
        s = StoreInfo()
        lib().unomol_gpu_store_info.argtypes = [C.c_void_p, C.POINTER(StoreInfo)]
        _check(lib().unomol_gpu_store_info(self._h, C.byref(s)), self._h)
        return s.as_dict()

    def write_records(self, path: str) -> int:
        """Write the canonical integral records (|v| > 1e-14) to `path` as raw TwoInts records; returns
        their count.  np.fromfile(path, RECORD_DTYPE) reads them back."""
        n = C.c_int64()
        lib().unomol_gpu_write_records.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_int64)]
        _check(lib().unomol_gpu_write_records(self._h, os.fsencode(path), C.byref(n)), self._h)
        return int(n.value)

    def stats(self) -> dict:
        s = Stats()
        _check(lib().unomol_gpu_get_stats(self._h, C.byref(s)), self._h)
        return s.as_dict()

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().unomol_gpu_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ScfInput(C.Structure):
    _fields_ = [("norb", C.c_int), ("nelec", C.c_int), ("nucrep", C.c_double),
                ("S", C.POINTER(C.c_double)), ("H", C.POINTER(C.c_double))]


class ScfOptions(C.Structure):
    _fields_ = [("maxits", C.c_int), ("eps", C.c_double), ("conv_type", C.c_int), ("accel", C.c_int),
                ("guess", C.c_int), ("diis_size", C.c_int), ("diis_tol", C.c_double),
                ("diis_start", C.c_double), ("level_shift", C.c_double), ("level_shift_until", C.c_double),
                ("incremental", C.c_int), ("rebuild_every", C.c_int), ("loop", C.c_int), ("density", C.c_int)]


class ScfResult(C.Structure):
    _fields_ = [("status", C.c_int), ("message", C.c_char * 256), ("energy", C.c_double),
                ("e_electronic", C.c_double), ("init_energy", C.c_double), ("ediff", C.c_double),
                ("pdiff", C.c_double), ("diis_error", C.c_double), ("seconds", C.c_double),
                ("iterations", C.c_int), ("converged", C.c_int), ("fock_builds", C.c_int),
                ("energies", C.POINTER(C.c_double)), ("energies_cap", C.c_int), ("fock_ms", C.c_double),
                ("densities", C.POINTER(C.c_double)), ("densities_cap", C.c_int), ("guess_used", C.c_int),
                ("purify_iterations", C.c_int), ("purify_error", C.c_double), ("guess_trace", C.c_double),
                ("seconds_setup", C.c_double), ("seconds_fock", C.c_double), ("seconds_diis", C.c_double),
                ("seconds_diag", C.c_double), ("sp2_steps", C.c_int), ("sp2_fallbacks", C.c_int),
                ("pseudo_steps", C.c_int)]


class BatchScfResult(C.Structure):
    _fields_ = [("energy", C.c_double), ("e_electronic", C.c_double), ("diis_error", C.c_double),
                ("iterations", C.c_int), ("converged", C.c_int), ("init_energy", C.c_double),
                ("ediff", C.c_double), ("pdiff", C.c_double)]


DENSITY_DIAG = 0
DENSITY_SP2 = 1
DENSITY_PSEUDO = 2
SCF_DAMPED = 0
SCF_DIIS = 2
SCF_LOOP_GROUND, SCF_LOOP_DPM = 0, 1
GUESS_CORE, GUESS_GIVEN, GUESS_PURIFY = 0, 1, 2
GUESS_USED = {0: "core", 1: "given", 2: "purified", 3: "fallback"}


def attracting_charges(b: Basis):
    """Charges of the nuclear attraction: every centre's, except the positron centre of a DPM basis,
    which the reference skips there (OneElectronInts.cpp:43; its attraction is the DPM potential)."""
    q = np.array(b.charges, np.float64)
    skip = getattr(b, "skip_center", None)
    if skip is not None and skip < len(q):
        q[skip] = 0.0
    return q


def one_electron(b: Basis, charges=None):
    """S, T, H (packed) of the basis: unomol_one_electron (host code of the library)."""
    L = lib()
    L.unomol_one_electron.argtypes = [C.POINTER(BasisDesc), _dp, _dp, _dp, _dp]
    d, keep = basis_desc(b)
    S, T, H = np.zeros(b.no2), np.zeros(b.no2), np.zeros(b.no2)
    q = attracting_charges(b) if charges is None else charges
    _check(L.unomol_one_electron(C.byref(d), np.ascontiguousarray(q, np.float64), S, T, H))
    return S, T, H


def one_electron_gpu(b: Basis, centers=None, with_t: bool = False):
    """S, H (and T) packed on the GPU (unomol_gpu_one_electron); centers: None (the basis's geometry) or
    an array [ngeom, ncen, 3] in bohr, giving arrays [ngeom, no2]."""
    L = lib()
    L.unomol_gpu_one_electron.argtypes = [C.POINTER(BasisDesc), _dp, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p]
    L.unomol_gpu_one_electron_last_error.restype = C.c_char_p
    d, keep = basis_desc(b)
    many = centers is not None
    cen = np.ascontiguousarray(b.centers if centers is None else centers, np.float64).reshape(-1, b.ncen, 3)
    ng = cen.shape[0]
    S, H = np.zeros((ng, b.no2)), np.zeros((ng, b.no2))
    T = np.zeros((ng, b.no2)) if with_t else None
    rc = L.unomol_gpu_one_electron(C.byref(d), np.ascontiguousarray(attracting_charges(b), np.float64), ng, cen.ctypes.data,
                                   S.ctypes.data, T.ctypes.data if with_t else None, H.ctypes.data)
    if rc != 0:
        raise UnomolError(f"unomol_gpu_one_electron error {rc}: {L.unomol_gpu_one_electron_last_error().decode()}")
    if not many:
        S, H = S[0], H[0]
        T = T[0] if with_t else None
    return (S, T, H) if with_t else (S, H)


def moment_ints(b: Basis) -> np.ndarray:
    """[9, no2]: dx, dy, dz, qxx, qxy, qxz, qyy, qyz, qzz integrals (unomol_gpu_moment_ints)."""
    L = lib()
    L.unomol_gpu_moment_ints.argtypes = [C.POINTER(BasisDesc), C.c_void_p]
    L.unomol_gpu_one_electron_last_error.restype = C.c_char_p
    d, keep = basis_desc(b)
    M = np.zeros((9, b.no2))
    rc = L.unomol_gpu_moment_ints(C.byref(d), M.ctypes.data)
    if rc != 0:
        raise UnomolError(f"unomol_gpu_moment_ints error {rc}: {L.unomol_gpu_one_electron_last_error().decode()}")
    return M


def scf(ctx: "TwoElectronInts", b: Basis, S=None, H=None, accel: int = SCF_DAMPED, guess_P=None,
        maxits: int | None = None, eps: float | None = None, conv_type: int | None = None,
        diis_size: int = 8, diis_tol: float = 1e-6, record: int = 0, diis_start: float = 0.0,
        level_shift: float = 0.0, level_shift_until: float = 0.05, incremental: bool = False,
        rebuild_every: int = 8, keep_densities: int = 0, purify: bool = False, loop: int = 0, density: int = 0):
    """SCF on the GPU (unomol_scf).  Returns a dict: energy, init_energy, iterations, converged, P, ...
    purify: start from guess_P after McWeeny purification and a trace check, or from the core
    Hamiltonian when it fails them (out["guess_used"] says which).  density: DENSITY_DIAG (eigen-solve),
    DENSITY_SP2 (second-order spectral projection, eigen-solve where it finds no gap) or DENSITY_PSEUDO
    (pseudo-diagonalisation steps on the last orbitals, eigen-solve for the first density, large steps
    and small gaps; out["pseudo_steps"] counts the steps)."""
    L = lib()
    L.unomol_scf.argtypes = [C.c_void_p, C.POINTER(ScfInput), C.POINTER(ScfOptions), C.POINTER(ScfResult),
                             _dp, C.c_void_p]
    if S is None or H is None:
        S, _, H = one_electron(b)
    S = np.ascontiguousarray(S, np.float64)
    H = np.ascontiguousarray(H, np.float64)
    dp = C.POINTER(C.c_double)
    inp = ScfInput(b.norb, b.nelec, b.nuclear_repulsion(), S.ctypes.data_as(dp), H.ctypes.data_as(dp))
    opt = ScfOptions(maxits if maxits is not None else b.maxits, eps if eps is not None else b.eps,
                     conv_type if conv_type is not None else b.scf_flag[0], accel,
                     GUESS_CORE if guess_P is None else (GUESS_PURIFY if purify else GUESS_GIVEN),
                     diis_size, diis_tol, diis_start, level_shift, level_shift_until, 1 if incremental else 0,
                     rebuild_every, loop, int(density))
    uhf = b.nelec % 2 == 1
    P = np.zeros(b.no2 * (2 if uhf else 1))
    if guess_P is not None:
        P[:] = guess_P
    eps_orb = np.zeros(b.norb * (2 if uhf else 1))
    res = ScfResult()
    energies = np.zeros(max(record, 1))
    if record:
        res.energies = energies.ctypes.data_as(dp)
        res.energies_cap = record
    dens = np.zeros((max(keep_densities, 1), len(P)))
    if keep_densities:
        res.densities = dens.ctypes.data_as(dp)
        res.densities_cap = keep_densities
    rc = L.unomol_scf(ctx._h, C.byref(inp), C.byref(opt), C.byref(res), P, eps_orb.ctypes.data)
    if rc != 0:
        raise UnomolError(f"unomol_scf error {rc}: {res.message.decode(errors='replace')}")
    out = {k: getattr(res, k) for k in ("energy", "e_electronic", "init_energy", "ediff", "pdiff", "diis_error",
                                        "seconds", "iterations", "converged", "fock_builds", "fock_ms",
                                        "purify_iterations", "purify_error", "guess_trace", "seconds_setup",
                                        "seconds_fock", "seconds_diis", "seconds_diag", "sp2_steps",
                                        "sp2_fallbacks", "pseudo_steps")}
    out["guess_used"] = GUESS_USED.get(res.guess_used, str(res.guess_used))
    out["P"] = P
    out["orbital_energies"] = eps_orb
    if record:
        out["energies"] = energies[:min(record, res.iterations)].copy()
    if keep_densities:
        out["densities"] = dens[:min(keep_densities, res.fock_builds)].copy()
    return out


BATCH_GRAPH = 0
BATCH_LAUNCHES = 1
BATCH_SEQUENTIAL = 2


class Batch:
    """Many molecules in one batched Fock build (unomol_gpu_batch_*): merged work lists, persistent
    kernels per quartet class, CUDA-graph replay, autotuned launch shapes."""

    def __init__(self, bases: list):
        L = lib()
        L.unomol_gpu_batch_create.argtypes = [C.POINTER(BasisDesc), C.c_int, C.POINTER(C.c_void_p)]
        L.unomol_gpu_batch_buffers.argtypes = [C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
                                               C.POINTER(C.c_void_p), C.POINTER(C.c_int64)]
        L.unomol_gpu_batch_fock.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.unomol_gpu_batch_autotune.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
        L.unomol_gpu_batch_set_precision.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double]
        L.unomol_gpu_batch_fock_device.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        L.unomol_gpu_batch_set_density.argtypes = [C.c_void_p, _dp]
        L.unomol_gpu_batch_get_fock.argtypes = [C.c_void_p, _dp]
        L.unomol_gpu_batch_destroy.argtypes = [C.c_void_p]
        L.unomol_gpu_batch_destroy.restype = None
        L.unomol_gpu_batch_last_error.argtypes = [C.c_void_p]
        L.unomol_gpu_batch_last_error.restype = C.c_char_p
        self.bases = bases
        descs, self._keep = [], []
        for b in bases:
            d, k = basis_desc(b)
            descs.append(d)
            self._keep.append(k)
        arr = (BasisDesc * len(descs))(*descs)
        self._h = C.c_void_p()
        self._chk(L.unomol_gpu_batch_create(arr, len(descs), C.byref(self._h)))
        dP, dG, off, tot = C.c_void_p(), C.c_void_p(), C.c_void_p(), C.c_int64()
        self._chk(L.unomol_gpu_batch_buffers(self._h, C.byref(dP), C.byref(dG), C.byref(off), C.byref(tot)))
        self.dP, self.dG, self.total = dP.value, dG.value, tot.value
        self.offsets = [0]
        for b in bases[:-1]:
            self.offsets.append(self.offsets[-1] + b.no2)

    def _chk(self, rc):
        if rc < 0:
            msg = lib().unomol_gpu_batch_last_error(getattr(self, "_h", None) or None).decode(errors="replace")
            raise UnomolError(f"unomol_gb300 batch error {rc}: {msg}")
        return rc

    def set_precision(self, mode: int, fp32_cutoff: float = 1e-10, skip_cutoff: float = 1e-13):
        """Precision form of the batched build (PREC_FP64 or PREC_MIXED with the FP32 and density-skip
        cutoffs), as set_precision + set_density_screening of one context."""
        self._chk(lib().unomol_gpu_batch_set_precision(self._h, int(mode), float(fp32_cutoff), float(skip_cutoff)))

    def set_densities(self, Ps):
        self._chk(lib().unomol_gpu_batch_set_density(self._h, np.ascontiguousarray(np.concatenate(Ps), np.float64)))

    def fock(self, mode: int = BATCH_GRAPH, stream: int = 0):
        self._chk(lib().unomol_gpu_batch_fock(self._h, int(mode), C.c_void_p(stream)))

    def fock_device(self, dP_ptr: int = 0, dG_ptr: int = 0, mode: int = BATCH_GRAPH, stream: int = 0):
        """Batched build on device buffers (packed P of all molecules in, packed G out; 0: the batch's own)."""
        self._chk(lib().unomol_gpu_batch_fock_device(self._h, C.c_void_p(dP_ptr or None), C.c_void_p(dG_ptr or None),
                                                     int(mode), C.c_void_p(stream)))

    def get_focks(self):
        G = np.zeros(self.total)
        self._chk(lib().unomol_gpu_batch_get_fock(self._h, G))
        return [G[o:o + b.no2].copy() for o, b in zip(self.offsets, self.bases)]

    def autotune(self, reps: int = 2):
        chosen = np.zeros(3 * 64, np.int32)
        n = self._chk(lib().unomol_gpu_batch_autotune(self._h, int(reps), chosen.ctypes.data))
        return [tuple(int(x) for x in chosen[3 * k:3 * k + 3]) for k in range(n)]

    def scf(self, S=None, H=None, eps: float = 1e-10, diis_tol: float = 1e-6, maxits: int = 200,
            diis_size: int = 8, graph: bool = True, accel: int = SCF_DIIS, conv_type: int = 0, guess_P=None,
            loop: int = SCF_LOOP_GROUND, incremental: bool = False, rebuild_every: int = 8, density: int = 0):
        """RHF SCF of every molecule at once (unomol_gpu_batch_scf).  S, H: lists of packed matrices
        (default: the GPU one-electron integrals of each basis); guess_P: list of packed starting
        densities (default: core Hamiltonian); accel / conv_type / loop as for scf(); density:
        DENSITY_DIAG, or DENSITY_PSEUDO (DIIS loop: pseudo-diagonalisation steps after the first two
        iterations where every active molecule passes the step check, else the eigen-solve; the counts
        come back as pseudo_steps / pseudo_refused).  Returns a dict
        with per-molecule energies, iterations and convergence, the packed densities, the wall time
        and whether the iteration ran as a CUDA graph."""
        L = lib()
        L.unomol_gpu_batch_scf.argtypes = [C.c_void_p, C.POINTER(ScfInput), C.c_int, C.POINTER(ScfOptions), C.c_int,
                                           C.POINTER(BatchScfResult), _dp, C.POINTER(C.c_double), C.POINTER(C.c_int)]
        L.unomol_gpu_batch_scf_last_error.restype = C.c_char_p
        n = len(self.bases)
        if S is None or H is None:
            SH = [one_electron_gpu(b) for b in self.bases]
            S, H = [x[0] for x in SH], [x[1] for x in SH]
        S = [np.ascontiguousarray(x, np.float64) for x in S]
        H = [np.ascontiguousarray(x, np.float64) for x in H]
        dp = C.POINTER(C.c_double)
        inp = (ScfInput * n)(*[ScfInput(b.norb, b.nelec, b.nuclear_repulsion(), s.ctypes.data_as(dp), h.ctypes.data_as(dp))
                               for b, s, h in zip(self.bases, S, H)])
        opt = ScfOptions(maxits, eps, conv_type, accel, GUESS_CORE if guess_P is None else GUESS_GIVEN, diis_size,
                         diis_tol, 0.0, 0.0, 0.0, 1 if incremental else 0, rebuild_every, loop, density)
        res = (BatchScfResult * n)()
        P = np.zeros(self.total)
        if guess_P is not None:
            P[:] = np.concatenate([np.asarray(x, np.float64) for x in guess_P])
        sec, used = C.c_double(), C.c_int()
        rc = L.unomol_gpu_batch_scf(self._h, inp, n, C.byref(opt), 1 if graph else 0, res, P, C.byref(sec), C.byref(used))
        note = L.unomol_gpu_batch_scf_last_error().decode(errors="replace")
        if rc != 0:
            raise UnomolError(f"unomol_gpu_batch_scf error {rc}: {note}")
        L.unomol_gpu_batch_scf_last_builds.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_int)]
        fms, nb = C.c_double(), C.c_int()
        L.unomol_gpu_batch_scf_last_builds(C.byref(fms), C.byref(nb))
        L.unomol_gpu_batch_scf_last_pseudo.argtypes = [C.POINTER(C.c_int), C.POINTER(C.c_int)]
        ps, pr = C.c_int(), C.c_int()
        L.unomol_gpu_batch_scf_last_pseudo(C.byref(ps), C.byref(pr))
        return {"fock_ms": fms.value, "builds": nb.value, "pseudo_steps": ps.value, "pseudo_refused": pr.value,"energy": np.array([r.energy for r in res]), "iterations": np.array([r.iterations for r in res]),
                "init_energy": np.array([r.init_energy for r in res]), "ediff": np.array([r.ediff for r in res]),
                "pdiff": np.array([r.pdiff for r in res]),
                "converged": np.array([bool(r.converged) for r in res]),
                "diis_error": np.array([r.diis_error for r in res]),
                "P": [P[o:o + b.no2].copy() for o, b in zip(self.offsets, self.bases)],
                "seconds": sec.value, "graph_used": bool(used.value), "capture_note": note}

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            lib().unomol_gpu_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def l2_peak():
    """(L2 read GB/s, FP64 atomic adds 1e9/s) of the current device (unomol_gpu_l2_peak)."""
    L = lib()
    L.unomol_gpu_l2_peak.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double)]
    r, a = C.c_double(), C.c_double()
    _check(L.unomol_gpu_l2_peak(C.byref(r), C.byref(a)))
    return r.value, a.value


def fma_peak(fp64: bool = True) -> float:
    """TFLOP/s of the FP64 (or FP32) FMA pipe of the current device (library microbenchmark)."""
    v = C.c_double()
    _check(lib().unomol_gpu_fma_peak(1 if fp64 else 0, C.byref(v)))
    return v.value


def _c(a):
    a = np.asarray(a)
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous float64 array")
    return a


def _out(a):
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("G must be a C-contiguous float64 numpy array (it is added into)")
    return a
