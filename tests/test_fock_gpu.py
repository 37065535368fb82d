"""G(P) parity of the GPU Fock build against the reference's own formGmatrix (golden fixtures).

Two reference builds pin the two Rys modes of the GPU path:
  * reference-compatible mode (default)  vs the stock reference (G_rand, Ga, Gb);
  * exact mode                           vs the reference with Rys::root2 made exact (G_rand_exact, ...).
Tolerance: 1e-10 absolute on every packed element of G (the bar for Fock elements is 1e-8; FP64
rounding and the independent Rys fits leave ~1e-13).
"""
import numpy as np
import pytest

from conftest import basis_of, golden_cases, load_golden

TOL_G = 1e-10

CASES = golden_cases()


def _ctx(g, exact):
    from unomol_gb300.native import RYS_EXACT, TwoElectronInts
    t = TwoElectronInts(basis_of(g))
    if exact:
        t.set_rys_mode(RYS_EXACT)
    return t


@pytest.mark.gpu
@pytest.mark.parametrize("exact", [False, True], ids=["refmode", "exact"])
@pytest.mark.parametrize("name", CASES)
def test_rhf_g_parity(gpu, name, exact):
    g = load_golden(name)
    t = _ctx(g, exact)
    G = t.form_g(g["P_rand"])
    want = g["G_rand_exact"] if exact else g["G_rand"]
    err = np.abs(G - want).max()
    assert err <= TOL_G, f"{name}: max|dG| = {err:.3e}"


@pytest.mark.gpu
@pytest.mark.parametrize("exact", [False, True], ids=["refmode", "exact"])
@pytest.mark.parametrize("name", CASES)
def test_uhf_g_parity(gpu, name, exact):
    g = load_golden(name)
    t = _ctx(g, exact)
    Ga, Gb = t.form_g_uhf(g["Pa"], g["Pb"])
    wa, wb = (g["Ga_exact"], g["Gb_exact"]) if exact else (g["Ga"], g["Gb"])
    err = max(np.abs(Ga - wa).max(), np.abs(Gb - wb).max())
    assert err <= TOL_G, f"{name}: max|dG| = {err:.3e}"


@pytest.mark.gpu
def test_g_adds_into_caller_array(gpu):
    """formGmatrix adds into G (RHF.hpp:89-90 zeroes it first)."""
    from unomol_gb300.native import TwoElectronInts
    g = load_golden("h2o_631g")
    t = TwoElectronInts(basis_of(g))
    G = np.full(len(g["G_rand"]), 1.5)
    t.formGmatrix(g["P_rand"], G)
    assert np.abs(G - 1.5 - g["G_rand"]).max() <= TOL_G


MD_CASES = golden_cases("*_md.npz", exclude_md=False)


@pytest.mark.gpu
@pytest.mark.parametrize("name", MD_CASES)
def test_md_mode_matches_md_reference(gpu, name):
    """MD for every quartet against the reference built with -DUNOMOL_MD_INTS (f-shell cases included)."""
    from unomol_gb300.native import ERI_MD, TwoElectronInts
    g = load_golden(name)
    t = TwoElectronInts(basis_of(g))
    t.set_eri_method(ERI_MD)
    G = t.form_g(g["P_rand"])
    err = np.abs(G - g["G_rand"]).max()
    assert err <= TOL_G, f"{name}: max|dG| = {err:.3e}"
    Ga, Gb = t.form_g_uhf(g["Pa"], g["Pb"])
    assert max(np.abs(Ga - g["Ga"]).max(), np.abs(Gb - g["Gb"]).max()) <= TOL_G


@pytest.mark.gpu
def test_s_integrals_match_closed_form(gpu):
    """G(P) of a basis of s functions only against the closed form of (ss|ss) (F0 through erf),
    independent of the reference: within the G tolerance."""
    from conftest import closed_form_s_basis
    from unomol_gb300 import native
    b, P, G = closed_form_s_basis()
    t = native.TwoElectronInts(b)
    assert np.abs(t.form_g(P) - G).max() <= 1e-10
    t.set_rys_mode(native.RYS_EXACT)
    assert np.abs(t.form_g(P) - G).max() <= 1e-10
