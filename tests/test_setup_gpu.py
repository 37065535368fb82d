"""Device set-up of the Fock build: shell pairs and primitive pairs built on the GPU, sorted into blocks
by (class, new/old, primitive-pair count) and by Schwarz bound, and the staircase work lists.

* With the Schwarz cutoff at 0 every canonical shell quartet is kept, so the set-up's quartet,
  function-quartet and primitive-quartet counts equal those of the canonical enumeration of
  TwoElectronInts::calculate (TwoElectronInts.cpp:511-697, primitive loops :439-460), counted here on
  the host from the basis alone.
* With start_shell only the quartets whose largest shell index reaches start_shell are kept
  (TwoElectronInts.cpp:541).
* The default cutoff keeps a subset, and G with the cutoff at 0 equals G with the default cutoff within
  the G tolerance (the dropped quartets are below 1e-14).
* recalculate at a moved geometry gives the same G as a new context built there.
"""
import numpy as np
import pytest

from conftest import basis_of, load_golden

G_TOL = 1e-10


def canonical_counts(b, start_shell=0):
    """(shell quartets, function quartets, primitive quartets) of the canonical enumeration."""
    L = np.array(b.shell_l)
    K = np.array(b.shell_nprim)
    nf = (L + 1) * (L + 2) // 2
    i, j = np.tril_indices(b.nshell)
    same = i == j
    kp = np.where(same, K[i] * (K[i] + 1) // 2, K[i] * K[j]).astype(np.int64)
    fp = (nf[i] * nf[j]).astype(np.int64)
    new = i >= start_shell

    def pair_pairs(x, keep):
        # sum over unordered pairs of pairs (p >= q) of x_p x_q, at least one of them new
        tot = (x.sum() ** 2 + (x ** 2).sum()) // 2
        xo = x[~keep]
        return int(tot - (xo.sum() ** 2 + (xo ** 2).sum()) // 2)

    one = np.ones_like(kp)
    return pair_pairs(one, new), pair_pairs(fp, new), pair_pairs(kp, new)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["water3_631g", "ethane_631g", "ref_dh95_h2"])
def test_unscreened_counts_match_canonical_enumeration(gpu, name):
    from unomol_gb300 import native
    g = load_golden(name)
    b = basis_of(g)
    t = native.TwoElectronInts(b)
    st0 = t.stats()
    t.set_screening(0.0)
    st = t.stats()
    nsq, nfq, npq = canonical_counts(b)
    assert st["npairs"] == b.nshell * (b.nshell + 1) // 2
    assert st["shell_quartets_total"] == nsq
    assert st["shell_quartets"] == nsq
    assert st["function_quartets"] == nfq
    assert st["primitive_quartets"] == npq
    # the default cutoff keeps a subset, whose G is the same within the tolerance
    assert 0 < st0["shell_quartets"] <= nsq
    G_all = t.form_g(g["P_rand"])
    t.set_screening(1e-14)
    G_cut = t.form_g(g["P_rand"])
    assert np.abs(G_all - G_cut).max() <= G_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("start", [1, 3])
def test_start_shell_keeps_quartets_reaching_it(gpu, start):
    from unomol_gb300 import native
    g = load_golden("water3_631g")
    b = basis_of(g)
    t = native.TwoElectronInts(b, start_shell=start)
    t.set_screening(0.0)
    st = t.stats()
    nsq, nfq, npq = canonical_counts(b, start)
    assert st["shell_quartets"] == nsq
    assert st["function_quartets"] == nfq
    assert st["primitive_quartets"] == npq


@pytest.mark.gpu
def test_recalculate_equals_new_context(gpu):
    from unomol_gb300 import molecules, native
    from unomol_gb300.basis import Basis
    atoms = molecules.water_cluster(4, 3)
    rng = np.random.default_rng(7)
    moved = [(e, tuple(np.asarray(x) + rng.normal(scale=0.1, size=3))) for e, x in atoms]
    b0 = Basis(text=molecules.patin_text(atoms, "6-31G"))
    b1 = Basis(text=molecules.patin_text(moved, "6-31G"))
    n = b0.norb
    m = rng.uniform(-0.1, 0.1, (n, n))
    P = np.ascontiguousarray((0.5 * (m + m.T) + 0.5 * np.eye(n))[np.tril_indices(n)])
    t = native.TwoElectronInts(b0)
    G0 = t.form_g(P)
    t.recalculate(b1)
    G1 = t.form_g(P)
    ref = native.TwoElectronInts(b1).form_g(P)
    assert np.abs(G1 - ref).max() <= 1e-12
    assert np.abs(G1 - G0).max() > 1e-6  # the geometry really moved
    t.recalculate(b0)
    assert np.abs(t.form_g(P) - G0).max() <= 1e-12
