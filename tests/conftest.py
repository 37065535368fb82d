import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


# Scale fixtures (n-decane and the 32-water cluster, tests/golden/make_golden.py --big): no stored
# densities or one-electron matrices, their own tests (tests/test_scale_parity_gpu.py)
BIG_CASES = ("decane_631g", "water32_631g")


def golden_cases(pattern="*.npz", exclude_md=True):
    out = []
    for p in sorted(glob.glob(os.path.join(GOLDEN, pattern))):
        name = os.path.basename(p)[:-4]
        if exclude_md and name.endswith("_md"):
            continue
        if name.startswith(("dpm_", "prop_")):  # DPM grids, moments / finite field: their own tests
            continue
        if name in BIG_CASES:
            continue
        out.append(name)
    return out


def rand_density(n: int, seed: int, scale: float = 0.3) -> np.ndarray:
    """The seeded random symmetric density of the fixture generator (tests/golden/make_golden.py):
    packed, off-diagonal uniform in (-scale, scale), diagonal uniform in (0, 1)."""
    rng = np.random.default_rng(seed)
    m = rng.uniform(-scale, scale, (n, n))
    m = 0.5 * (m + m.T) + np.diag(rng.uniform(0.0, 1.0, n))
    return np.ascontiguousarray(m[np.tril_indices(n)])


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def basis_of(g):
    from unomol_gb300.basis import Basis
    return Basis(text=str(g["patin"]))


@pytest.fixture(scope="session")
def gpu():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from unomol_gb300 import native
    native.lib()  # fails loudly when the extension is missing
    return torch.device("cuda:0")


def closed_form_s_basis():
    """Four hydrogens in 6-31G (8 contracted s functions) at fixed positions, with the closed-form
    G(P) of a random symmetric density: (ij|kl) over s Gaussians is
    sum c c c c 2 pi^(5/2) / (p q sqrt(p+q)) exp(-ab/p |AB|^2) exp(-cd/q |CD|^2) F0(pq/(p+q) |PQ|^2)
    with F0(T) = sqrt(pi/T) erf(sqrt(T)) / 2, and G = 2 J(P) - K(P) with P the half density, as the
    reference's RHF scatter forms it.  Returns (basis, packed P, packed G)."""
    import math

    from scipy.special import erf

    from unomol_gb300 import molecules
    from unomol_gb300.basis import Basis, full_to_packed

    atoms = [("H", (0, 0, 0)), ("H", (0, 0, 0.74)), ("H", (1.1, 0.3, 0.2)), ("H", (1.0, 0.9, 1.3))]
    b = Basis(text=molecules.patin_text(atoms, "6-31G"))
    n = b.norb
    funcs = []
    for i in range(b.nshell):
        assert b.shell_l[i] == 0
        a, c = b.shell_prims(i)
        funcs.append((a, c, b.centers[b.shell_center[i]]))

    def pair(i, j):
        (ai, ci, A), (aj, cj, B) = funcs[i], funcs[j]
        return [(x + y, (x * A + y * B) / (x + y), cx * cy * math.exp(-x * y / (x + y) * ((A - B) ** 2).sum()))
                for x, cx in zip(ai, ci) for y, cy in zip(aj, cj)]

    def f0(t):
        return 1.0 if t < 1e-15 else 0.5 * math.sqrt(math.pi / t) * float(erf(math.sqrt(t)))

    prs = {(i, j): pair(i, j) for i in range(n) for j in range(i + 1)}
    E = np.zeros((n, n, n, n))
    for (i, j), bra in prs.items():
        for (k, l), ket in prs.items():
            v = sum(kp * kq * 2 * math.pi ** 2.5 / (p * q * math.sqrt(p + q)) * f0(p * q / (p + q) * ((P - Q) ** 2).sum())
                    for p, P, kp in bra for q, Q, kq in ket)
            for a1, b1 in ((i, j), (j, i)):
                for c1, d1 in ((k, l), (l, k)):
                    E[a1, b1, c1, d1] = v
    m = np.random.default_rng(3).uniform(-0.5, 0.5, (n, n))
    P = 0.5 * (m + m.T)
    G = 2 * np.einsum("ijkl,kl->ij", E, P) - np.einsum("ikjl,kl->ij", E, P)
    return b, full_to_packed(P), full_to_packed(G)
