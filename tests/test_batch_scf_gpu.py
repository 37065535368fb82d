"""Batched RHF SCF (unomol_gpu_batch_scf): every molecule of a batch in lockstep, one batched Fock build
and one set of batched linear algebra per iteration, against the single-molecule SCF driver."""
import numpy as np
import pytest

from unomol_gb300 import molecules


def _batch_molecules():
    out = [(molecules.water(), "STO-3G"), (molecules.water(), "6-31G"), (molecules.alkane(1), "6-31G"),
           (molecules.alkane(2), "STO-3G"), (molecules.water_cluster(2, 3), "6-31G"),
           (molecules.perturb(molecules.water(), 0.05, 4), "STO-3G"), (molecules.alkane(3), "6-31G")]
    from unomol_gb300.basis import Basis
    return [Basis(text=molecules.patin_text(a, bs)) for a, bs in out]


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [True, False])
def test_batched_scf_matches_single_molecule_scf(gpu, graph):
    from unomol_gb300 import native
    bases = _batch_molecules()
    bat = native.Batch(bases)
    SH = [native.one_electron_gpu(b) for b in bases]
    r = bat.scf(S=[x[0] for x in SH], H=[x[1] for x in SH], eps=1e-10, diis_tol=1e-7, graph=graph)
    assert r["converged"].all(), r
    for k, b in enumerate(bases):
        t = native.TwoElectronInts(b)
        q = native.scf(t, b, S=SH[k][0], H=SH[k][1], accel=native.SCF_DIIS, eps=1e-10, diis_tol=1e-7, conv_type=0)
        assert q["converged"]
        assert abs(r["energy"][k] - q["energy"]) < 1e-9, (k, r["energy"][k], q["energy"])
        assert abs(int(r["iterations"][k]) - q["iterations"]) <= 1, (k, r["iterations"][k], q["iterations"])
        assert np.abs(r["P"][k] - q["P"]).max() < 1e-5
        t.close()
    bat.close()


@pytest.mark.gpu
def test_batched_scf_iteration_is_one_cuda_graph(gpu):
    from unomol_gb300 import native
    bases = _batch_molecules()[:3]
    bat = native.Batch(bases)
    r = bat.scf(graph=True)
    assert r["graph_used"], r["capture_note"]
    assert r["converged"].all()


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [True, False])
def test_batched_scf_incremental_builds(gpu, graph):
    """Incremental builds in the batched SCF (G(P_prev) + G(P - P_prev), a full build every 8): in FP64
    the energies are those of full builds within 1e-9 Eh; in the precision form (FP32 cutoff 1e-3,
    density skip 1e-13) within the form's 1e-6 Eh bar, at the same iteration counts to within one.  The
    build timings come back (unomol_gpu_batch_scf_last_builds), also from a replayed graph."""
    from unomol_gb300 import native
    bases = _batch_molecules()
    SH = [native.one_electron_gpu(b) for b in bases]
    S, H = [x[0] for x in SH], [x[1] for x in SH]
    bat = native.Batch(bases)
    full = bat.scf(S=S, H=H, eps=1e-10, diis_tol=1e-7, graph=graph)
    inc = bat.scf(S=S, H=H, eps=1e-10, diis_tol=1e-7, graph=graph, incremental=True)
    assert full["converged"].all() and inc["converged"].all()
    assert np.abs(inc["energy"] - full["energy"]).max() < 1e-9
    assert abs(inc["builds"] - int(inc["iterations"].max())) <= 1 and inc["fock_ms"] > 0.0
    if graph:
        assert inc["graph_used"], inc["capture_note"]
    bat.set_precision(native.PREC_MIXED, 1e-3, 1e-13)
    mix = bat.scf(S=S, H=H, eps=1e-10, diis_tol=1e-7, graph=graph, incremental=True)
    assert mix["converged"].all()
    assert np.abs(mix["energy"] - full["energy"]).max() < 1e-6
    assert np.abs(mix["iterations"] - full["iterations"]).max() <= 1
    bat.close()


@pytest.mark.gpu
@pytest.mark.parametrize("graph", [True, False])
def test_batched_scf_pseudo_diagonalisation(gpu, graph):
    """Pseudo-diagonalisation steps in the batched DIIS SCF (UNOMOL_DENSITY_PSEUDO: the batched eigen-solve
    for the first two iterations, then first-order rotations by grouped matrix products wherever every
    molecule's step passes the check, the eigen-solve tail otherwise): every molecule converges to the
    energy and density of the eigen-solve SCF (1e-9 Eh), with plain launches and with the iteration's
    parts captured as graphs; in the precision form with incremental builds too."""
    from unomol_gb300 import native
    bases = _batch_molecules()
    SH = [native.one_electron_gpu(b) for b in bases]
    S, H = [x[0] for x in SH], [x[1] for x in SH]
    bat = native.Batch(bases)
    ref = bat.scf(S=S, H=H, eps=1e-10, diis_tol=1e-7, graph=graph)
    r = bat.scf(S=S, H=H, eps=1e-10, diis_tol=1e-7, graph=graph, density=native.DENSITY_PSEUDO)
    assert r["converged"].all(), r["iterations"]
    assert r["graph_used"] == graph, r["capture_note"]
    assert np.abs(r["energy"] - ref["energy"]).max() < 1e-9, np.abs(r["energy"] - ref["energy"])
    assert (r["iterations"] <= ref["iterations"] + 6).all(), (r["iterations"], ref["iterations"])
    assert r["pseudo_steps"] > 0 and r["pseudo_steps"] + r["pseudo_refused"] + 2 >= r["builds"] - 1, r
    for k in range(len(bases)):
        assert np.abs(r["P"][k] - ref["P"][k]).max() < 1e-5
    bat.set_precision(native.PREC_MIXED, 1e-3, 1e-13)
    m = bat.scf(S=S, H=H, eps=1e-10, diis_tol=1e-7, graph=graph, incremental=True, density=native.DENSITY_PSEUDO)
    assert m["converged"].all()
    assert np.abs(m["energy"] - ref["energy"]).max() < 1e-6
    bat.close()
