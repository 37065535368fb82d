"""DPM polarisation-potential path (RHF.hpp:292-388) against the reference's own runs (golden fixtures
from tests/golden/make_dpm_golden.py): the positron-augmented basis and its one-electron matrices on
the host, the DPM potential integrals and the whole grid of SCFs on the GPU."""
import numpy as np
import pytest

from conftest import load_golden

CASES = ["dpm_h2o_sto3g", "dpm_h2o_631g", "dpm_ch4_sto3g"]


def _bases(g):
    from unomol_gb300.basis import Basis, dpm_augment
    b = Basis(text=str(g["patin"]))
    return b, dpm_augment(b, str(g["posin"]), g["points"][0])


@pytest.mark.parametrize("name", CASES)
def test_augmented_basis_one_electron_matches_reference(name):
    from unomol_gb300 import native
    g = load_golden(name)
    b, a = _bases(g)
    assert b.int_flag[0] == 1
    assert a.norb == b.norb + 5 and a.ncen == b.ncen + 1 and a.charges[-1] == 1.0
    S, _, H = native.one_electron(a)
    assert np.abs(S - g["S"]).max() < 1e-12
    assert np.abs(H - g["H_plain"]).max() < 1e-11


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_dpm_integrals_match_reference(gpu, name):
    from unomol_gb300 import native
    g = load_golden(name)
    _, a = _bases(g)
    t = native.TwoElectronInts(a)
    H = np.array(g["H_plain"], float)
    t.gdpm(g["points"][0], H)
    ref = g["H_dpm"] - g["H_plain"]
    assert np.abs((H - g["H_plain"]) - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max())
    t.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_gpu_polarization_potential_matches_reference(gpu, name):
    from unomol_gb300 import dpm
    from unomol_gb300.basis import Basis
    g = load_golden(name)
    b = Basis(text=str(g["patin"]))
    rows = dpm.polarization_potential(b, str(g["posin"]), g["points"])
    vpol, spol = g["vpol"], g["spol"]
    for r, v, sp in zip(rows, vpol, spol):
        assert r["converged"]
        np.testing.assert_allclose(r["q"], v[:3], atol=1e-9)
        assert abs(r["e_gs"] - sp[1]) < 1e-9          # spol.out prints 10 decimals
        assert abs(r["e_init"] - sp[2]) < 1e-9
        assert abs(r["e_final"] - sp[3]) < 1e-9
        assert abs(r["vpol"] - v[3]) < 1e-10, (r["vpol"], v[3])
        r4 = float(np.dot(v[:3], v[:3])) ** 2
        assert abs(r["alfa"] - v[4]) < 2.0 * r4 * 1e-10 + 1e-12  # alfa = -2 vpol r^4 carries vpol's error
        assert abs(r["vstat"] - v[5]) < 1e-10, (r["vstat"], v[5])
        assert abs(r["vsum"] - v[6]) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [True, False])
def test_gpu_batched_polarization_potential_matches_reference(gpu, graph):
    from unomol_gb300 import dpm
    from unomol_gb300.basis import Basis
    g = load_golden("dpm_h2o_sto3g")
    b = Basis(text=str(g["patin"]))
    rows, info = dpm.polarization_potential_batched(b, str(g["posin"]), g["points"], graph=graph)
    assert info["graph_used"] == graph, info
    for r, v, sp in zip(rows, g["vpol"], g["spol"]):
        assert r["converged"]
        assert abs(r["e_init"] - sp[2]) < 1e-9 and abs(r["e_final"] - sp[3]) < 1e-9
        assert abs(r["vpol"] - v[3]) < 1e-10, (r["vpol"], v[3])
        assert abs(r["vstat"] - v[5]) < 1e-10
