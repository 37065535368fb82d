"""GPU test of the allocation-free Fock build (unomol_gpu_fock_rhf_noalloc), through the C ABI.

That entry point serves callers that must not trigger cudaMalloc once they are running (a host
framework that owns all device memory after start-up, or a loop that must not take cudaMalloc's
implicit synchronisation): its scratch is a static device array of the library.  Its output must equal
the regular device entry point's (unomol_gpu_fock_rhf_device) within the G tolerance of the other
parity tests, on two calls in a row (the array keeps the previous call's contents), for every
integral method the regular build dispatches (templated Rys, runtime-L Rys, MD); a basis larger than
the array and counting mode are rejected with an error instead of running.

This file is collected last (test_zz_*), so a run that stops at the first failure has run every other
test before it.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import basis_of, load_golden

TOL_G = 1e-10


def _noalloc_fn():
    from unomol_gb300 import native
    L = native.lib()
    f = L.unomol_gpu_fock_rhf_noalloc
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return L, f


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["h2o_631g", "ethane_631g", "ref_dh95_co2", "ref_tzp_ch4", "he_ccpvqz", "h2o_631g_md"])
def test_noalloc_matches_device_entry_point(gpu, name):
    """s/p bases; d shells (templated Rys classes); He cc-pVQZ with f shells (runtime-L Rys up to
    la+lb+lc+ld = 8, MD above); and a context in MD mode against the -DUNOMOL_MD_INTS reference."""
    import torch
    from unomol_gb300.native import ERI_MD, TwoElectronInts
    L, noalloc = _noalloc_fn()
    g = load_golden(name)
    t = TwoElectronInts(basis_of(g))
    if name.endswith("_md"):
        t.set_eri_method(ERI_MD)
    dP = torch.from_numpy(np.ascontiguousarray(g["P_rand"])).to(gpu)
    ref = torch.zeros_like(dP)
    t.fock_device(dP.data_ptr(), ref.data_ptr(), 0)  # existing entry point, context stream
    torch.cuda.synchronize()
    ref_h = ref.cpu().numpy()
    for call in range(2):  # two calls in a row share the static scratch
        out = torch.zeros_like(dP)
        rc = noalloc(t._h, C.c_void_p(dP.data_ptr()), C.c_void_p(out.data_ptr()), None)
        assert rc == 0, L.unomol_gpu_last_error(t._h).decode()
        torch.cuda.synchronize()
        err = float(np.abs(out.cpu().numpy() - ref_h).max())
        assert err <= TOL_G, f"call {call}: max|dG| = {err:.3e}"
    # and the golden G of the reference itself
    assert float(np.abs(ref_h - g["G_rand"]).max()) <= TOL_G


@pytest.mark.gpu
def test_noalloc_adds_into_g(gpu):
    import torch
    from unomol_gb300.native import TwoElectronInts
    L, noalloc = _noalloc_fn()
    g = load_golden("h2o_631g")
    t = TwoElectronInts(basis_of(g))
    dP = torch.from_numpy(np.ascontiguousarray(g["P_rand"])).to(gpu)
    out = torch.full_like(dP, 0.25)
    assert noalloc(t._h, C.c_void_p(dP.data_ptr()), C.c_void_p(out.data_ptr()), None) == 0
    torch.cuda.synchronize()
    assert float(np.abs(out.cpu().numpy() - 0.25 - g["G_rand"]).max()) <= TOL_G


@pytest.mark.gpu
def test_noalloc_rejects_basis_beyond_scratch(gpu):
    import torch
    from unomol_gb300 import molecules
    from unomol_gb300.basis import Basis
    from unomol_gb300.native import TwoElectronInts
    L, noalloc = _noalloc_fn()
    b = Basis(text=molecules.patin_text(molecules.water_cluster(80, 3, box=20.0), "6-31G"))
    assert b.norb > 1024
    t = TwoElectronInts(b)
    dP = torch.zeros(b.no2, dtype=torch.float64, device=gpu)
    dG = torch.zeros_like(dP)
    rc = noalloc(t._h, C.c_void_p(dP.data_ptr()), C.c_void_p(dG.data_ptr()), None)
    assert rc == -1  # UNOMOL_EINVAL
    assert "1024" in L.unomol_gpu_last_error(t._h).decode()


@pytest.mark.gpu
def test_noalloc_rejects_counting_mode(gpu):
    """Counting needs a counter buffer of its own; the allocation-free build refuses it with a message
    instead of leaving the previous build's counts in place."""
    import torch
    from unomol_gb300.native import TwoElectronInts
    L, noalloc = _noalloc_fn()
    g = load_golden("h2o_631g")
    t = TwoElectronInts(basis_of(g))
    t.set_counting(True)
    dP = torch.from_numpy(np.ascontiguousarray(g["P_rand"])).to(gpu)
    dG = torch.zeros_like(dP)
    assert noalloc(t._h, C.c_void_p(dP.data_ptr()), C.c_void_p(dG.data_ptr()), None) == -1
    assert "counting" in L.unomol_gpu_last_error(t._h).decode()
    t.set_counting(False)
    assert noalloc(t._h, C.c_void_p(dP.data_ptr()), C.c_void_p(dG.data_ptr()), None) == 0
    torch.cuda.synchronize()
    assert float(np.abs(dG.cpu().numpy() - g["G_rand"]).max()) <= TOL_G
    assert t.stats()["kernel_launches"] >= 3  # expand, the class launches, fold: this build's count
