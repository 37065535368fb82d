"""Learned initial density (ctypes mirror of the unomol_guess_* / unomol_mlp_* C ABI).

No reference counterpart: the reference starts its SCF from the core Hamiltonian (RHF.hpp:205-211) or
from a PMATRIX.DAT density (RHF.hpp:120-123).  LearnedGuess.predict() writes a density in that
PMATRIX.DAT form (the RHF half density, trace(PS) = nocc); native.scf(..., purify=True) then purifies
and trace-checks it on the GPU and falls back to the core Hamiltonian when it fails.

Training and inference run in the library: BF16 GEMMs on the tensor cores with FP32 accumulation,
FP32 master weights, Adam, the density assembly and the loss on the GPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native
from .basis import Basis

_fp = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


class GuessConfig(C.Structure):
    _fields_ = [("hidden", C.c_int), ("layers", C.c_int), ("n_rbf", C.c_int), ("r_cut", C.c_double),
                ("seed", C.c_ulonglong)]


class TrainOptions(C.Structure):
    _fields_ = [("first", C.c_int), ("count", C.c_int), ("epochs", C.c_int), ("batch_molecules", C.c_int),
                ("lr", C.c_float), ("lr_final", C.c_float), ("weight_decay", C.c_float), ("seed", C.c_ulonglong)]


_BOUND = False


def _lib():
    global _BOUND
    L = native.lib()
    if not _BOUND:
        vp = C.c_void_p
        L.unomol_tc_gemm_bf16.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, vp, vp, vp]
        L.unomol_mlp_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.POINTER(vp)]
        L.unomol_mlp_num_params.argtypes = [vp]
        L.unomol_mlp_num_params.restype = C.c_longlong
        L.unomol_mlp_get_params.argtypes = [vp, _fp]
        L.unomol_mlp_set_params.argtypes = [vp, _fp]
        L.unomol_mlp_get_grads.argtypes = [vp, _fp]
        L.unomol_mlp_forward.argtypes = [vp, vp, C.c_int, vp, vp]
        L.unomol_mlp_backward.argtypes = [vp, vp, vp]
        L.unomol_mlp_adam.argtypes = [vp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, vp]
        L.unomol_mlp_destroy.argtypes = [vp]
        L.unomol_mlp_destroy.restype = None
        L.unomol_mlp_last_error.argtypes = [vp]
        L.unomol_mlp_last_error.restype = C.c_char_p
        L.unomol_guess_create.argtypes = [C.POINTER(GuessConfig), C.POINTER(native.BasisDesc), _ip, C.POINTER(vp)]
        L.unomol_guess_info.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_longlong),
                                        C.POINTER(C.c_int)]
        L.unomol_guess_add_molecule.argtypes = [vp, C.POINTER(native.BasisDesc), _ip, _dp]
        L.unomol_guess_num_molecules.argtypes = [vp]
        L.unomol_guess_train.argtypes = [vp, C.POINTER(TrainOptions), vp]
        L.unomol_guess_loss.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double), vp]
        L.unomol_guess_predict.argtypes = [vp, C.POINTER(native.BasisDesc), _ip, _dp]
        L.unomol_guess_get_params.argtypes = [vp, _fp]
        L.unomol_guess_set_params.argtypes = [vp, _fp]
        L.unomol_guess_destroy.argtypes = [vp]
        L.unomol_guess_destroy.restype = None
        L.unomol_guess_last_error.argtypes = [vp]
        L.unomol_guess_last_error.restype = C.c_char_p
        _BOUND = True
    return L


def charges_of(b: Basis) -> np.ndarray:
    return np.ascontiguousarray(np.rint(b.charges), np.int32)


class Mlp:
    """The network alone (unomol_mlp_*): forward/backward on device buffers (torch tensors here)."""

    def __init__(self, n_in: int, hidden: int, layers: int, n_out: int, seed: int = 0):
        L = _lib()
        self._h = C.c_void_p()
        self._check(L.unomol_mlp_create(n_in, hidden, layers, n_out, seed, C.byref(self._h)))
        self.n_in, self.hidden, self.layers, self.n_out = n_in, hidden, layers, n_out
        self.n_params = int(L.unomol_mlp_num_params(self._h))

    def _check(self, rc):
        if rc != 0:
            msg = _lib().unomol_mlp_last_error(self._h if getattr(self, "_h", None) else None)
            raise native.UnomolError(f"unomol_mlp error {rc}: {msg.decode(errors='replace')}")

    def params(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        self._check(_lib().unomol_mlp_get_params(self._h, out))
        return out

    def set_params(self, p):
        self._check(_lib().unomol_mlp_set_params(self._h, np.ascontiguousarray(p, np.float32)))

    def grads(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        self._check(_lib().unomol_mlp_get_grads(self._h, out))
        return out

    def forward(self, x, y, stream=None):
        """x, y: contiguous fp32 CUDA tensors [rows x n_in], [rows x n_out]."""
        self._check(_lib().unomol_mlp_forward(self._h, x.data_ptr(), x.shape[0], y.data_ptr(), stream))

    def backward(self, dy, stream=None):
        self._check(_lib().unomol_mlp_backward(self._h, dy.data_ptr(), stream))

    def adam(self, lr, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0, stream=None):
        self._check(_lib().unomol_mlp_adam(self._h, lr, beta1, beta2, eps, weight_decay, stream))

    def unpack(self, p=None):
        """[(W, b)] per linear map from a flat parameter vector (host order)."""
        p = self.params() if p is None else p
        dims = [self.n_in] + [self.hidden] * self.layers + [self.n_out]
        out, k = [], 0
        for din, dout in zip(dims[:-1], dims[1:]):
            W = p[k:k + din * dout].reshape(dout, din)
            k += din * dout
            out.append((W, p[k:k + dout]))
            k += dout
        return out

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib().unomol_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LearnedGuess:
    """Per-atom-pair density model (unomol_guess_*).  The example basis fixes the elements and their
    shell lists (s and p shells)."""

    def __init__(self, example: Basis, hidden: int = 256, layers: int = 3, n_rbf: int = 16, r_cut: float = 15.0,
                 seed: int = 0):
        L = _lib()
        self._h = C.c_void_p()
        cfg = GuessConfig(hidden, layers, n_rbf, r_cut, seed)
        d, keep = native.basis_desc(example)
        self._check(L.unomol_guess_create(C.byref(cfg), C.byref(d), charges_of(example), C.byref(self._h)))
        n_in, n_out, n_el = C.c_int(), C.c_int(), C.c_int()
        npar = C.c_longlong()
        self._check(L.unomol_guess_info(self._h, C.byref(n_in), C.byref(n_out), C.byref(npar), C.byref(n_el)))
        self.n_in, self.n_out, self.n_params, self.n_elements = n_in.value, n_out.value, npar.value, n_el.value
        self.hidden, self.layers, self.n_rbf, self.r_cut = hidden, layers, n_rbf, r_cut

    def _check(self, rc):
        if rc != 0:
            msg = _lib().unomol_guess_last_error(self._h if getattr(self, "_h", None) else None)
            raise native.UnomolError(f"unomol_guess error {rc}: {msg.decode(errors='replace')}")

    def add(self, b: Basis, P):
        d, keep = native.basis_desc(b)
        self._check(_lib().unomol_guess_add_molecule(self._h, C.byref(d), charges_of(b),
                                                      np.ascontiguousarray(P, np.float64)))

    def __len__(self):
        return int(_lib().unomol_guess_num_molecules(self._h))

    def train(self, first: int, count: int, epochs: int, batch_molecules: int = 16, lr: float = 1e-3,
              lr_final: float = 1e-5, weight_decay: float = 0.0, seed: int = 0) -> np.ndarray:
        opt = TrainOptions(first, count, epochs, batch_molecules, lr, lr_final, weight_decay, seed)
        hist = np.zeros(epochs, np.float64)
        self._check(_lib().unomol_guess_train(self._h, C.byref(opt), hist.ctypes.data))
        return hist

    def loss(self, first: int, count: int, grads: bool = False, batch_molecules: int = 16):
        l = C.c_double()
        g = np.zeros(self.n_params, np.float32) if grads else None
        self._check(_lib().unomol_guess_loss(self._h, first, count, batch_molecules, C.byref(l),
                                             g.ctypes.data if grads else None))
        return (l.value, g) if grads else l.value

    def predict(self, b: Basis) -> np.ndarray:
        d, keep = native.basis_desc(b)
        P = np.zeros(b.no2, np.float64)
        self._check(_lib().unomol_guess_predict(self._h, C.byref(d), charges_of(b), P))
        return P

    def params(self) -> np.ndarray:
        out = np.zeros(self.n_params, np.float32)
        self._check(_lib().unomol_guess_get_params(self._h, out))
        return out

    def set_params(self, p):
        self._check(_lib().unomol_guess_set_params(self._h, np.ascontiguousarray(p, np.float32)))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            _lib().unomol_guess_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
