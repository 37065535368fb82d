"""The C restatement (oracle/unomol_oracle.c) pinned against the golden fixtures of the reference itself.

The stock reference (G_rand, Ga/Gb) pins the reference-compatible Rys mode; the reference with an
exact two-root quadrature (G_rand_exact, ...) pins the exact mode.  Tolerance 1e-10 on packed G.
Also checks that the fixtures reproduce the reference's published energies (test/scfout.dat.*).
"""
import numpy as np
import pytest

from conftest import ROOT, basis_of, golden_cases, load_golden

import sys
sys.path.insert(0, ROOT + "/oracle")

TOL_G = 1e-10
# d-shell and large cases are slow for the single-pass C oracle; they are covered on the GPU
FAST = [c for c in golden_cases() if not any(s in c for s in ("tzp", "dh95_co2", "dh95_h2", "ccpvqz"))]


@pytest.mark.parametrize("name", FAST)
def test_oracle_rhf_matches_reference(name):
    import orc
    g = load_golden(name)
    b = basis_of(g)
    G, cnt = orc.fock(b, g["P_rand"])
    assert np.abs(G - g["G_rand"]).max() <= TOL_G
    assert cnt[3] == int(g["n_stored"]) or abs(cnt[3] - int(g["n_stored"])) <= 2  # |v| > 1e-14 count
    Ge, _ = orc.fock(b, g["P_rand"], exact=True)
    assert np.abs(Ge - g["G_rand_exact"]).max() <= TOL_G


@pytest.mark.parametrize("name", ["h2o_631g", "ref_b_dhdz", "h2o_cation_631g", "ref_631_co"])
def test_oracle_uhf_matches_reference(name):
    import orc
    g = load_golden(name)
    (Ga, Gb), _ = orc.fock(basis_of(g), g["Pa"], g["Pb"])
    assert max(np.abs(Ga - g["Ga"]).max(), np.abs(Gb - g["Gb"]).max()) <= TOL_G


def test_oracle_strided_sample_sums_to_full():
    import orc
    g = load_golden("h2o_631g")
    b = basis_of(g)
    full, c_full = orc.fock(b, g["P_rand"])
    parts = [orc.fock(b, g["P_rand"], stride=5, offset=o) for o in range(5)]
    assert np.abs(sum(p[0] for p in parts) - full).max() < 1e-12
    assert sum(p[1][0] for p in parts) == c_full[0]


@pytest.mark.parametrize("name", [c for c in golden_cases() if c.startswith("ref_") and "dhdz" not in c
                                  and "dh95" not in c and "tzp" not in c and "d6s3p" not in c])
def test_fixture_energy_matches_published(name):
    """The stock reference run here reproduces the published golden energy (test/scfout.dat.*)."""
    g = load_golden(name)
    assert abs(float(g["scf_energy"]) - float(g["golden_energy"])) < 1e-10


@pytest.mark.parametrize("exact", [False, True])
def test_oracle_matches_closed_form_s_integrals(exact):
    """An independent pin of the restatement: G(P) of a basis of s functions only, against the closed
    form of (ss|ss) (one Rys root, the Boys function F0 through erf)."""
    import orc
    from conftest import closed_form_s_basis
    b, P, G = closed_form_s_basis()
    Go, _ = orc.fock(b, P, exact=exact)
    assert np.abs(Go - G).max() <= 1e-13 * np.abs(G).max()


def test_reference_damped_trajectory_amplifies_input_differences():
    """Why the scale tests hold the damped loop's energies to 1e-8 Eh for three iterations only: on
    n-decane the reference's own stock loop (core-H guess) moves by more than 1e-9 Eh at its fourth
    energy and by more than 1e-7 Eh at its fifth when its starting density is scaled by 1 + 1e-13,
    while its first three energies move by less than 1e-9 Eh (oracle/ref_harness.cpp: refh_scf_trace)."""
    import os
    import tempfile
    import refh
    if not refh.available():
        pytest.skip("reference build not present (oracle/_ref)")
    g = load_golden("decane_631g")
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "patin.dat")
        with open(p, "w") as f:
            f.write(str(g["patin"]))
        b = refh.RefBasis(p)
        t = refh.RefTwoElectronInts(b)
        e0 = refh.scf_trace(b, t, 5)
        e1 = refh.scf_trace(b, t, 5, 1e-13)
    assert np.abs(e0 - g["trace"]).max() == 0.0  # the fixture is this trajectory
    d = np.abs(e1 - e0)
    assert d[:3].max() < 1e-9 and d[3] > 1e-9 and d[4] > 1e-7, d


@pytest.mark.parametrize("name", ["h2o_631g", "h2o_sto3g_c0"])
def test_oracle_records_are_the_reference_records(name):
    """orc_records (the stored integrals of the integral pass, TwoElectronInts.cpp:622-671) against the
    records the reference itself stored: the same labels (the oracle's threads split the outer shell
    loop, so the order differs), values within 1e-12."""
    import orc
    g = load_golden(name)
    val, ijkl = orc.records(basis_of(g))

    def by_label(v, q):
        q = q.astype(np.int64)
        o = np.lexsort((q[:, 3], q[:, 2], q[:, 1], q[:, 0]))
        return v[o], q[o]
    v1, q1 = by_label(val, ijkl)
    v2, q2 = by_label(g["ints_val"], g["ints_ijkl"])
    assert np.array_equal(q1, q2)
    assert np.abs(v1 - v2).max() <= 1e-12


@pytest.mark.parametrize("name", ["h2o_631g", "h2o_sto3g_c0"])
def test_six_term_scatter_of_the_reference_records(name):
    """The record -> G map of the conventional build (six terms per record with the coincidence factors,
    G = T + T^T) applied to the reference's own records gives the reference's G, RHF and UHF."""
    import orc
    g = load_golden(name)
    n = basis_of(g).norb
    G = orc.scatter_records(g["ints_val"], g["ints_ijkl"], n, g["P_rand"])
    assert np.abs(G - g["G_rand"]).max() <= 1e-12
    Ga, Gb = orc.scatter_records(g["ints_val"], g["ints_ijkl"], n, g["Pa"], g["Pb"])
    assert max(np.abs(Ga - g["Ga"]).max(), np.abs(Gb - g["Gb"]).max()) <= 1e-12


@pytest.mark.parametrize("name", [c for c in FAST if not c.startswith("he")][:12])
def test_six_term_scatter_of_oracle_records(name):
    """The same map on the C restatement's records, for fixtures without a record dump."""
    import orc
    g = load_golden(name)
    b = basis_of(g)
    val, ijkl = orc.records(b)
    assert abs(len(val) - int(g["n_stored"])) <= 2
    assert np.abs(orc.scatter_records(val, ijkl, b.norb, g["P_rand"]) - g["G_rand"]).max() <= TOL_G
