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


def golden_cases(pattern="*.npz", exclude_md=True):
    out = []
    for p in sorted(glob.glob(os.path.join(GOLDEN, pattern))):
        name = os.path.basename(p)[:-4]
        if exclude_md and name.endswith("_md"):
            continue
        if name.startswith(("dpm_", "prop_")):  # DPM grids, moments / finite field: their own tests
            continue
        out.append(name)
    return out


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
