"""Batched Fock build over many molecules (the batching form) against the single-molecule path.

Every molecule's G from the batch (CUDA-graph replay, plain launches, and after the autotuner) must equal
the reference's G (golden fixtures, 1e-10) and the single-molecule build's G.
"""
import numpy as np
import pytest

from conftest import basis_of, load_golden

NAMES = ["h2o_sto3g_c0", "h2o_631g", "ethane_631g", "ref_3g_co", "ref_631_nh3", "water3_631g", "ref_dh95_h2",
         "propane_cation_sto3g"]


@pytest.mark.gpu
def test_batch_matches_reference_all_modes(gpu):
    from unomol_gb300 import native
    gs = [load_golden(n) for n in NAMES]
    bat = native.Batch([basis_of(g) for g in gs])
    bat.set_densities([g["P_rand"] for g in gs])
    for mode in (native.BATCH_LAUNCHES, native.BATCH_GRAPH, native.BATCH_GRAPH, native.BATCH_SEQUENTIAL):
        bat.fock(mode)
        for name, g, G in zip(NAMES, gs, bat.get_focks()):
            assert np.abs(G - g["G_rand"]).max() <= 1e-10, (mode, name)
    chosen = bat.autotune(1)
    assert len(chosen) > 0 and all(c[1] in (64, 128, 256) and c[2] in (1, 2, 4, 8) for c in chosen)
    bat.fock(native.BATCH_GRAPH)
    for name, g, G in zip(NAMES, gs, bat.get_focks()):
        assert np.abs(G - g["G_rand"]).max() <= 1e-10, ("tuned", name)


@pytest.mark.gpu
def test_batch_workload_matches_single_molecule(gpu):
    from unomol_gb300 import molecules, native
    from unomol_gb300.basis import Basis
    work = molecules.batch_workload(seed=3, n=24)
    bases = [Basis(text=t) for _, t in work]
    rng = np.random.default_rng(0)
    Ps = []
    for b in bases:
        m = rng.uniform(-0.1, 0.1, (b.norb, b.norb))
        m = 0.5 * (m + m.T) + np.eye(b.norb) * 0.5
        Ps.append(np.ascontiguousarray(m[np.tril_indices(b.norb)]))
    bat = native.Batch(bases)
    bat.set_densities(Ps)
    bat.fock(native.BATCH_GRAPH)
    Gb = bat.get_focks()
    for b, P, G in zip(bases, Ps, Gb):
        G1 = native.TwoElectronInts(b).form_g(P)
        assert np.abs(G - G1).max() <= 1e-10
