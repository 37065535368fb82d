"""CPU checks of the learned-guess oracle (oracle/guess_oracle.py): its FP64 gradient against finite
differences of its own loss, the rotation covariance of the density assembly, and its BF16 rounding
against torch's."""
import sys

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, ROOT + "/oracle")
import guess_oracle as go  # noqa: E402

from unomol_gb300 import molecules  # noqa: E402
from unomol_gb300.basis import Basis  # noqa: E402


def _mol(atoms, basis="6-31G", n_rbf=16, r_cut=15.0):
    b = Basis(text=molecules.patin_text(atoms, basis))
    elements = sorted({int(round(q)) for q in b.charges})
    return b, go.Molecule(b.shell_l, b.shell_offset, b.shell_center, b.centers, b.charges, b.norb, elements,
                          n_rbf, r_cut)


def _params(n_in, hidden, layers, n_out, seed):
    rng = np.random.default_rng(seed)
    dims = [n_in] + [hidden] * layers + [n_out]
    p = []
    for din, dout in zip(dims[:-1], dims[1:]):
        p.append(rng.normal(scale=1.0 / np.sqrt(din), size=(dout, din)).ravel())
        p.append(rng.normal(scale=0.1, size=dout))
    return np.concatenate(p)


def test_oracle_gradient_matches_finite_differences():
    _, m1 = _mol(molecules.perturb(molecules.water(), 0.05, 1))
    n_in, hidden, layers, n_out = m1.X.shape[1], 8, 2, 48
    rng = np.random.default_rng(3)
    mols = [m1]
    tg = [0.3 * rng.normal(size=(m1.norb, m1.norb))]
    tg = [0.5 * (t + t.T) for t in tg]
    p = _params(n_in, hidden, layers, n_out, 4)
    f = lambda q: go.loss_and_grad(go.unpack(q, n_in, hidden, layers, n_out), mols, tg, n_out)[0]
    _, g = go.loss_and_grad(go.unpack(p, n_in, hidden, layers, n_out), mols, tg, n_out)
    idx = rng.choice(len(p), 60, replace=False)
    h = 1e-6
    for k in idx:
        e = np.zeros_like(p)
        e[k] = h
        fd = (f(p + e) - f(p - e)) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])


def _ao_rotation(b, R):
    """AO transformation of a rotation: identity on s functions, R on every p shell (x, y, z order)."""
    U = np.eye(b.norb)
    for s in range(b.nshell):
        if b.shell_l[s] == 1:
            o = b.shell_offset[s]
            U[o:o + 3, o:o + 3] = R
    return U


def test_assembly_is_rotation_covariant():
    atoms = molecules.perturb(molecules.alkane(3), 0.05, 5)
    b, m = _mol(atoms)
    rng = np.random.default_rng(6)
    q = rng.normal(size=4)
    a, bb, c, d = q / np.linalg.norm(q)
    R = np.array([[a * a + bb * bb - c * c - d * d, 2 * (bb * c - a * d), 2 * (bb * d + a * c)],
                  [2 * (bb * c + a * d), a * a - bb * bb + c * c - d * d, 2 * (c * d - a * bb)],
                  [2 * (bb * d - a * c), 2 * (c * d + a * bb), a * a - bb * bb - c * c + d * d]])
    rot = [(e, tuple(R @ np.array(x))) for e, x in atoms]
    b2, m2 = _mol(rot)
    np.testing.assert_allclose(m.X, m2.X, atol=1e-9)  # invariant features
    Y = rng.normal(size=(len(m.rows), 48))
    P = m.assemble(Y)
    P2 = m2.assemble(Y)
    U = _ao_rotation(b, R)
    np.testing.assert_allclose(P2, U @ P @ U.T, atol=1e-10)
    np.testing.assert_allclose(P, P.T, atol=1e-12)


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    x = np.random.default_rng(7).normal(size=10000).astype(np.float32) * np.float32(3.0)
    x[:4] = [0.0, 1.0, -2.5, 1e-30]
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float64).numpy()
    np.testing.assert_array_equal(go.bf16(x), ref)
