"""Run-to-run and launch-order independence of the Fock build (the J/K contributions meet in FP64
atomics, in an order that changes from run to run).

On the 32-water 6-31G cluster (416 functions) with a physical density (the superposition of monomer
densities): the same build twice, and once with the class launches in reverse order
(unomol_gpu_set_launch_order), for the plain FP64 build and the mixed-precision build.  Only the
rounding of the additions may differ: max|dG| within 1e-11 (about 1e-13 of max|G|), and the
two-electron energy Tr(PG) within 1e-10 Eh.
"""
import numpy as np
import pytest

from conftest import load_golden

TOL_G = 1e-11
TOL_E = 1e-10


def _trace(P, G, n):
    from unomol_gb300.basis import packed_to_full
    return float(np.sum(packed_to_full(P, n) * packed_to_full(G, n)))


@pytest.mark.gpu
@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
def test_build_independent_of_atomic_order(gpu, mixed):
    from unomol_gb300 import guess, native
    from unomol_gb300.basis import Basis
    g = load_golden("water32_631g")
    b = Basis(text=str(g["patin"]))
    P = guess.fragment_density(b)
    t = native.TwoElectronInts(b)
    if mixed:
        t.set_precision(native.PREC_MIXED, 1e-3)
    G1 = t.form_g(P)
    G2 = t.form_g(P)
    t.set_launch_order(True)
    G3 = t.form_g(P)
    t.set_launch_order(False)
    scale = float(np.abs(G1).max())
    d12 = float(np.abs(G1 - G2).max())
    d13 = float(np.abs(G1 - G3).max())
    print(f"max|G| {scale:.3e}  run-to-run {d12:.3e}  reversed launches {d13:.3e}")
    assert d12 <= TOL_G and d13 <= TOL_G, (d12, d13, scale)
    e1, e3 = _trace(P, G1, b.norb), _trace(P, G3, b.norb)
    assert abs(e1 - e3) <= TOL_E, (e1, e3)
