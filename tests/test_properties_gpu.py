"""Moments and finite-field analysis on the GPU against the reference program's moments.out and
finitefield.out on its own test inputs (fixtures from tests/golden/make_property_golden.py)."""
import numpy as np
import pytest

from conftest import load_golden

CASES = [f"prop_{b}_{m}" for b in ("3g", "431", "631") for m in ("co", "h2o", "hf", "nh3")]


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_moments_match_reference(gpu, name):
    from unomol_gb300 import properties
    from unomol_gb300.basis import Basis
    g = load_golden(name)
    b = Basis(text=str(g["patin"]))
    m = properties.analyze_moments(b, g["P"])
    table = np.stack([m["total"], m["electronic"], m["nuclear"]], 1)
    # moments.out prints 8 significant digits
    assert np.all(np.abs(table - g["moments"]) <= 6e-8 * np.abs(g["moments"]) + 1e-12), np.abs(table - g["moments"]).max()
    assert abs(m["dipole_moment"] - float(g["dipole"])) < 1e-10
    assert abs(m["quadrupole_moment"] - float(g["quadrupole"])) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["prop_3g_h2o", "prop_631_co", "prop_431_nh3", "prop_631_hf"])
@pytest.mark.parametrize("batched", [True, False])
def test_finite_field_matches_reference(gpu, name, batched):
    from unomol_gb300 import native, properties
    from unomol_gb300.basis import Basis
    g = load_golden(name)
    b = Basis(text=str(g["patin"]))
    t = native.TwoElectronInts(b)
    gs = native.scf(t, b)  # the reference's own loop and flags
    t.close()
    ff = properties.finite_field(b, gs, field=float(g["field"]), batched=batched)
    assert ff["converged"].all()
    assert np.abs(ff["polnrg"] - g["ff_polnrg"]).max() < 1e-9
    tol = 2e-9 / float(g["field"]) ** 2
    assert np.abs(ff["alfa"] - g["ff_alfa"]).max() < tol
    assert abs(ff["alfa_iso"] - float(g["ff_iso"])) < tol and abs(ff["alfa_aniso"] - float(g["ff_aniso"])) < tol
