"""Density-screened and mixed-precision Fock builds (UNOMOL_PREC_MIXED) on the GPU.

* with the FP32 cutoff at or below the skip cutoff the build is FP64 with density screening: it must
  equal the plain FP64 build within the G tolerance (1e-10) when the skip cutoff is tiny;
* with every quartet in FP32 the result must stay within FP32 accuracy of the FP64 build (relative
  1e-5 of max|G|) and differ from it (the FP32 kernels really ran);
* an incremental mixed-precision SCF reaches the FP64 SCF energy within 1e-6 Eh (the accuracy bar of
  the precision form), for RHF and UHF.
"""
import numpy as np
import pytest

from conftest import basis_of, load_golden


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["water3_631g", "ethane_631g", "ref_dh95_h2"])
def test_density_screened_fp64_equals_plain(gpu, name):
    from unomol_gb300 import native
    g = load_golden(name)
    t = native.TwoElectronInts(basis_of(g))
    G0 = t.form_g(g["P_rand"])
    t.set_precision(native.PREC_MIXED, 0.0)
    t.set_density_screening(1e-20)
    G1 = t.form_g(g["P_rand"])
    assert np.abs(G1 - G0).max() <= 1e-10
    Ga0, Gb0 = native.TwoElectronInts(basis_of(g)).form_g_uhf(g["Pa"], g["Pb"])
    Ga1, Gb1 = t.form_g_uhf(g["Pa"], g["Pb"])
    assert max(np.abs(Ga1 - Ga0).max(), np.abs(Gb1 - Gb0).max()) <= 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["water3_631g", "ethane_631g", "ref_dh95_h2"])
def test_all_fp32_within_fp32_accuracy(gpu, name):
    from unomol_gb300 import native
    g = load_golden(name)
    t = native.TwoElectronInts(basis_of(g))
    G0 = t.form_g(g["P_rand"])
    t.set_precision(native.PREC_MIXED, 1e30)
    t.set_density_screening(1e-20)
    t.set_counting(True)
    G1 = t.form_g(g["P_rand"])
    st = t.stats()
    assert st["shell_quartets_fp32"] > 0 and st["shell_quartets_fp32"] == st["shell_quartets"]
    err = np.abs(G1 - G0).max()
    assert err <= 1e-5 * np.abs(G0).max()
    assert err > 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["water3_631g", "ref_dh95_h2"])
def test_counted_work_belongs_to_the_part_that_does_it(gpu, name):
    """The counting mode's algorithmic flops and function quartets: the quartet-level work
    (normalisation and density contraction) is booked to the precision of the kernel that does it and
    to the quartets of the build's own work lists, so a build with every quartet in FP32 books no FP64
    work, and a density-screened FP64 build that keeps every quartet books what the plain build does."""
    from unomol_gb300 import native
    g = load_golden(name)
    t = native.TwoElectronInts(basis_of(g))
    t.set_counting(True)
    t.form_g(g["P_rand"])
    plain = t.stats()
    assert plain["eri_flops"] > 0 and plain["eri_flops_fp32"] == 0
    assert plain["function_quartets_computed"] == plain["function_quartets"]
    t.set_precision(native.PREC_MIXED, 0.0)
    t.set_density_screening(1e-20)
    t.form_g(g["P_rand"])
    st = t.stats()
    assert st["eri_flops_fp32"] == 0
    assert st["function_quartets_computed"] == plain["function_quartets"]
    assert abs(st["eri_flops"] - plain["eri_flops"]) <= 1e-12 * plain["eri_flops"]
    t.set_precision(native.PREC_MIXED, 1e30)
    t.form_g(g["P_rand"])
    st = t.stats()
    assert st["eri_flops_fp32"] > 0 and st["eri_flops"] - st["eri_flops_fp32"] == 0
    assert st["function_quartets_computed"] == plain["function_quartets"]
    assert st["shell_quartets_fp32"] == st["shell_quartets"] == plain["shell_quartets"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["h2o_631g", "water3_631g", "ethane_631g", "propane_cation_sto3g"])
def test_incremental_mixed_scf_energy(gpu, name):
    from unomol_gb300 import native
    g = load_golden(name)
    b = basis_of(g)
    t = native.TwoElectronInts(b)
    r64 = native.scf(t, b, S=g["S"], H=g["H"], accel=native.SCF_DIIS, eps=1e-10, diis_tol=1e-7, maxits=100)
    tm = native.TwoElectronInts(b)
    tm.set_precision(native.PREC_MIXED, 1e-7)
    tm.set_density_screening(1e-12)
    rm = native.scf(tm, b, S=g["S"], H=g["H"], accel=native.SCF_DIIS, eps=1e-10, diis_tol=1e-7, maxits=100,
                    incremental=True)
    assert r64["converged"] and rm["converged"]
    assert abs(rm["energy"] - r64["energy"]) <= 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("cut", [1e-3, 1e-5, 1e-7])
def test_incremental_mixed_scf_converges_across_fp32_cutoffs(gpu, cut):
    """An 8-water cluster (6-31G, 104 functions) with the default density skip cutoff: the incremental
    mixed SCF reaches the 1e-10 Eh test at every FP32 cutoff, in about the plain SCF's iterations, and its
    energy stays within 1e-6 Eh of the plain FP64 SCF."""
    from unomol_gb300 import guess, molecules, native
    from unomol_gb300.basis import Basis
    b = Basis(text=molecules.patin_text(molecules.water_cluster(8, 1, box=7.0), "6-31G", eps=1e-10))
    S, _, H = native.one_electron(b)
    P0 = guess.fragment_density(b)
    kw = dict(S=S, H=H, accel=native.SCF_DIIS, maxits=60, eps=1e-10, diis_tol=1e-7, guess_P=P0)
    r64 = native.scf(native.TwoElectronInts(b), b, **kw)
    tm = native.TwoElectronInts(b)
    tm.set_precision(native.PREC_MIXED, cut)  # density skip cutoff: the library default
    rm = native.scf(tm, b, incremental=True, **kw)
    assert r64["converged"] and rm["converged"], (r64["iterations"], rm["iterations"])
    assert rm["iterations"] <= r64["iterations"] + 4
    assert abs(rm["energy"] - r64["energy"]) <= 1e-6


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["water3_631g", "ethane_631g"])
def test_fp64_part_runs_low_density_quartets_in_fp32(gpu, name):
    """The work lists put a quartet in the FP64 part when its Schwarz bound times the largest |P| of the
    whole density reaches the FP32 cutoff; the fused mixed kernel runs it in FP32 when its bound times
    the largest |P| of its own six blocks is below the cutoff.  Over a range of cutoffs some quartets
    move, the counts add up (moved quartets are FP32 quartets and stay in the build), and G stays within
    FP32 accuracy of the plain FP64 build."""
    from unomol_gb300 import native
    g = load_golden(name)
    t = native.TwoElectronInts(basis_of(g))
    G0 = t.form_g(g["P_rand"])
    t.set_counting(True)
    t.form_g(g["P_rand"])
    nq = t.stats()["shell_quartets"]
    moved = []
    for cut in (1e-1, 1e-2, 1e-3, 1e-4, 1e-5):
        t.set_precision(native.PREC_MIXED, cut)
        t.set_density_screening(1e-20)
        G1 = t.form_g(g["P_rand"])
        st = t.stats()
        assert st["shell_quartets"] == nq
        assert 0 <= st["shell_quartets_demoted"] <= st["shell_quartets_fp32"] <= st["shell_quartets"]
        assert np.abs(G1 - G0).max() <= 1e-5 * np.abs(G0).max()
        moved.append(st["shell_quartets_demoted"])
    assert max(moved) > 0, moved


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["water3_631g", "h2o_cation_631g", "ref_631_co"])
@pytest.mark.parametrize("cut", [1e-2, 1e-4])
def test_mixed_uhf_both_parts(gpu, name, cut):
    """UHF through both parts of the mixed build (the fused (ss|ss) launch, and the other classes' FP64
    part on four lanes per quartet beside their FP32 kernel): Ga and Gb within FP32 accuracy of the
    plain FP64 build, with the FP32 and FP64 parts both non-empty."""
    from unomol_gb300 import native
    g = load_golden(name)
    t = native.TwoElectronInts(basis_of(g))
    Ga0, Gb0 = t.form_g_uhf(g["Pa"], g["Pb"])
    t.set_precision(native.PREC_MIXED, cut)
    t.set_density_screening(1e-20)
    t.set_counting(True)
    Ga1, Gb1 = t.form_g_uhf(g["Pa"], g["Pb"])
    st = t.stats()
    assert st["shell_quartets_fp32"] < st["shell_quartets"]
    if cut >= 1e-2:
        assert st["shell_quartets_fp32"] > 0
    scale = max(np.abs(Ga0).max(), np.abs(Gb0).max())
    err = max(np.abs(Ga1 - Ga0).max(), np.abs(Gb1 - Gb0).max())
    assert err <= 1e-5 * scale, err
