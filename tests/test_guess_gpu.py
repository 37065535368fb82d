"""Learned initial density on the GPU: the tensor-core network and the density model against the CPU
oracle (oracle/guess_oracle.py), the purification / trace check / core-Hamiltonian fallback of the SCF,
and the gain of the trained network over the core-Hamiltonian guess."""
import sys

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, ROOT + "/oracle")
import guess_oracle as go  # noqa: E402

from unomol_gb300 import molecules, native  # noqa: E402
from unomol_gb300.basis import Basis  # noqa: E402


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, float) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.gpu
def test_mlp_forward_backward_match_oracle(gpu):
    import torch
    from unomol_gb300.learned import Mlp
    n_in, hidden, layers, n_out, rows = 20, 256, 3, 48, 777
    m = Mlp(n_in, hidden, layers, n_out, seed=5)
    rng = np.random.default_rng(0)
    p = m.params()
    p = (p + rng.normal(scale=0.02, size=p.shape)).astype(np.float32)  # non-zero biases too
    m.set_params(p)
    np.testing.assert_array_equal(m.params(), p)
    x = rng.normal(size=(rows, n_in)).astype(np.float32)
    dy = rng.normal(size=(rows, n_out)).astype(np.float32)
    xd = torch.from_numpy(x).to(gpu)
    yd = torch.zeros(rows, n_out, dtype=torch.float32, device=gpu)
    dyd = torch.from_numpy(dy).to(gpu)
    m.forward(xd, yd)
    m.backward(dyd)
    torch.cuda.synchronize()
    y = yd.cpu().numpy()
    g = m.grads()
    params = go.unpack(p, n_in, hidden, layers, n_out)
    yo, cache = go.mlp_forward(params, x, bf=True)
    go_ = go.pack(go.mlp_backward(params, cache, dy, bf=True))
    # BF16 operands with FP32 accumulation against the same roundings in FP64
    assert np.max(np.abs(y - yo)) <= 2e-3 * np.max(np.abs(yo)), np.max(np.abs(y - yo))
    assert _rel(g, go_) < 5e-3, _rel(g, go_)
    # and against plain FP64 (no BF16 rounding anywhere): the BF16 error budget
    y64, c64 = go.mlp_forward(params, x)
    g64 = go.pack(go.mlp_backward(params, c64, dy))
    assert _rel(y, y64) < 3e-2 and _rel(g, g64) < 5e-2, (_rel(y, y64), _rel(g, g64))


def _propanes(n, seed=11):
    bs = [Basis(text=molecules.patin_text(molecules.perturb(molecules.alkane(3), 0.05, seed + k), "6-31G"))
          for k in range(n)]
    return bs


def _oracle_mol(b, elements, r_cut=15.0):
    return go.Molecule(b.shell_l, b.shell_offset, b.shell_center, b.centers, b.charges, b.norb, elements, 16, r_cut)


@pytest.mark.gpu
def test_guess_loss_gradient_and_prediction_match_oracle(gpu):
    from unomol_gb300.learned import LearnedGuess
    bs = _propanes(3)
    model = LearnedGuess(bs[0], seed=3)
    elements = [1, 6]
    assert (model.n_in, model.n_out, model.n_elements) == (20, 48, 2)
    rng = np.random.default_rng(1)
    targets = []
    for b in bs:
        T = 0.2 * rng.normal(size=(b.norb, b.norb))
        T = 0.5 * (T + T.T)
        targets.append(T)
        model.add(b, T[np.tril_indices(b.norb)])  # packed row by row: (i, j <= i)
    p = model.params()
    loss, g = model.loss(0, 3, grads=True, batch_molecules=2)
    params = go.unpack(p, model.n_in, model.hidden, model.layers, model.n_out)
    mols = [_oracle_mol(b, elements) for b in bs]
    lo, gor = go.loss_and_grad(params, mols, targets, model.n_out, bf=True)
    assert abs(loss - lo) <= 1e-4 * lo, (loss, lo)
    assert _rel(g, gor) < 1e-2, _rel(g, gor)
    # prediction = oracle assembly of the oracle network outputs
    Y, _ = go.mlp_forward(params, mols[0].X, bf=True)
    Po = mols[0].assemble(Y)
    Pg = go.packed_to_full(model.predict(bs[0]), bs[0].norb)
    assert np.max(np.abs(Pg - Po)) <= 2e-3 * np.max(np.abs(Po)), np.max(np.abs(Pg - Po))


@pytest.mark.gpu
def test_training_lowers_the_loss(gpu):
    from unomol_gb300.learned import LearnedGuess
    bs = _propanes(8, seed=40)
    ctx = native.TwoElectronInts(bs[0])
    model = LearnedGuess(bs[0], seed=1)
    for b in bs:
        ctx.recalculate(b)
        r = native.scf(ctx, b, accel=native.SCF_DIIS, eps=1e-10)
        assert r["converged"]
        model.add(b, r["P"])
    l0 = model.loss(0, 8)
    hist = model.train(0, 8, epochs=40, batch_molecules=4, lr=1e-3)
    l1 = model.loss(0, 8)
    assert l1 < 0.05 * l0 and hist[-1] < hist[0], (l0, l1, hist[:3], hist[-3:])


@pytest.mark.gpu
@pytest.mark.parametrize("corrupt", ["noise", "nan", "double", "zero"])
def test_purified_guess_and_core_hamiltonian_fallback(gpu, corrupt):
    """Host-side fault injection: a guess that fails purification or the trace check must give the
    core-Hamiltonian SCF; a noisy guess is purified and reaches the same energy."""
    b = Basis(text=molecules.patin_text(molecules.perturb(molecules.alkane(2), 0.05, 7), "6-31G"))
    ctx = native.TwoElectronInts(b)
    S, _, H = native.one_electron(b)
    ref = native.scf(ctx, b, S=S, H=H, accel=native.SCF_DIIS, eps=1e-10)
    assert ref["converged"] and ref["guess_used"] == "core"
    P = ref["P"].copy()
    rng = np.random.default_rng(2)
    guess = {"noise": P + 0.02 * rng.normal(size=P.shape), "nan": np.full_like(P, np.nan), "double": 2.0 * P,
             "zero": np.zeros_like(P)}[corrupt]
    r = native.scf(ctx, b, S=S, H=H, accel=native.SCF_DIIS, eps=1e-10, guess_P=guess, purify=True)
    assert r["converged"]
    assert abs(r["energy"] - ref["energy"]) < 1e-8
    if corrupt == "noise":
        assert r["guess_used"] == "purified"
        assert abs(r["guess_trace"] - b.nelec // 2) < 1e-6
        assert r["iterations"] < ref["iterations"]
    else:
        assert r["guess_used"] == "fallback"
        assert r["iterations"] == ref["iterations"]


@pytest.mark.gpu
def test_learned_guess_cuts_scf_iterations(gpu):
    """The trained network against the core-Hamiltonian guess on held-out n-decane geometries (a
    reduced version of the 2000-geometry workload): >= 30% fewer SCF iterations, energies within
    1e-8 Eh of the plain SCF, no fallback."""
    from unomol_gb300 import learned_decane
    rep = learned_decane.run(n_geom=104, n_train=96, epochs=60, batch=8, seed=7)
    h = rep["held_out"]
    assert h["both_converged"] == h["n"] == 8
    assert h["fallbacks"] == 0
    assert h["max_abs_dE"] <= 1e-8, h
    assert h["iteration_reduction"] >= 0.30, h
