"""GPU one-electron integrals (unomol_gpu_one_electron) against the reference's S, T, H (golden
fixtures exported from OneElectronInts) and against the host version on many geometries at once."""
import numpy as np
import pytest

from conftest import basis_of, golden_cases, load_golden


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_cases())
def test_gpu_one_electron_matches_reference(gpu, name):
    from unomol_gb300 import native
    g = load_golden(name)
    S, T, H = native.one_electron_gpu(basis_of(g), with_t=True)
    for got, ref in ((S, g["S"]), (T, g["T"]), (H, g["H"])):
        assert np.abs(got - ref).max() <= 1e-12 * max(1.0, np.abs(ref).max()), np.abs(got - ref).max()


@pytest.mark.gpu
def test_gpu_one_electron_many_geometries(gpu):
    from unomol_gb300 import molecules, native
    from unomol_gb300.basis import Basis
    base = molecules.alkane(4)
    geoms = [molecules.perturb(base, 0.05, k) for k in range(6)]
    bases = [Basis(text=molecules.patin_text(a, "6-31G")) for a in geoms]
    cen = np.stack([b.centers for b in bases])
    S, H = native.one_electron_gpu(bases[0], centers=cen)
    assert S.shape == (6, bases[0].no2)
    for k, b in enumerate(bases):
        Sh, _, Hh = native.one_electron(b)
        assert np.abs(S[k] - Sh).max() < 1e-12
        assert np.abs(H[k] - Hh).max() < 1e-11
