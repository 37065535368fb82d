"""The precision form inside the batched build (unomol_gpu_batch_set_precision): per build, every
molecule's quartets split into FP64, FP32 and skipped parts by Schwarz bound x max|P| of the quartet's
density blocks (max|P| of its own molecule), both parts run by the persistent kernels.

* FP32 cutoff at 0 with a tiny skip cutoff: the density-screened FP64 build, equal to the reference's G
  (golden fixtures) within the G tolerance 1e-10;
* the mixed split of one molecule in the batch is the split of the single-molecule context with the
  same cutoffs, so G agrees with that context's mixed build to FP64 summation order (1e-12), in CUDA
  graph and plain-launch modes;
* every quartet in FP32: within FP32 accuracy of the FP64 build (1e-5 of max|G|) and different from it.
"""
import numpy as np
import pytest

from conftest import basis_of, load_golden

NAMES = ["h2o_631g", "ethane_631g", "ref_631_nh3", "water3_631g", "ref_dh95_h2", "propane_cation_sto3g"]


@pytest.fixture(scope="module")
def batch_case():
    gs = [load_golden(n) for n in NAMES]
    return gs, [basis_of(g) for g in gs]


@pytest.mark.gpu
def test_batch_screened_fp64_equals_reference(gpu, batch_case):
    from unomol_gb300 import native
    gs, bases = batch_case
    bat = native.Batch(bases)
    bat.set_densities([g["P_rand"] for g in gs])
    bat.set_precision(native.PREC_MIXED, 0.0, 1e-20)
    for mode in (native.BATCH_LAUNCHES, native.BATCH_GRAPH):
        bat.fock(mode)
        for name, g, G in zip(NAMES, gs, bat.get_focks()):
            assert np.abs(G - g["G_rand"]).max() <= 1e-10, (mode, name)


@pytest.mark.gpu
@pytest.mark.parametrize("cut", [1e-3, 1e-6])
def test_batch_mixed_equals_single_context_mixed(gpu, batch_case, cut):
    from unomol_gb300 import native
    gs, bases = batch_case
    bat = native.Batch(bases)
    bat.set_densities([g["P_rand"] for g in gs])
    bat.set_precision(native.PREC_MIXED, cut, 1e-12)
    for mode in (native.BATCH_GRAPH, native.BATCH_LAUNCHES):
        bat.fock(mode)
        for name, g, b, G in zip(NAMES, gs, bases, bat.get_focks()):
            t = native.TwoElectronInts(b)
            t.set_precision(native.PREC_MIXED, cut)
            t.set_density_screening(1e-12)
            G1 = t.form_g(g["P_rand"])
            t.close()
            assert np.abs(G - G1).max() <= 1e-12 * max(1.0, np.abs(G1).max()), (mode, name)
            assert np.abs(G - g["G_rand"]).max() <= 1e-4 * np.abs(g["G_rand"]).max(), (mode, name)


@pytest.mark.gpu
def test_batch_all_fp32_within_fp32_accuracy(gpu, batch_case):
    from unomol_gb300 import native
    gs, bases = batch_case
    bat = native.Batch(bases)
    bat.set_densities([g["P_rand"] for g in gs])
    bat.set_precision(native.PREC_MIXED, 1e30, 1e-20)
    bat.fock(native.BATCH_GRAPH)
    for name, g, G in zip(NAMES, gs, bat.get_focks()):
        err = np.abs(G - g["G_rand"]).max()
        scale = np.abs(g["G_rand"]).max()
        assert err <= 1e-5 * scale, name
        assert err > 0.0, name  # the FP32 kernels really ran
    # back to the plain FP64 build
    bat.set_precision(native.PREC_FP64)
    bat.fock(native.BATCH_GRAPH)
    for name, g, G in zip(NAMES, gs, bat.get_focks()):
        assert np.abs(G - g["G_rand"]).max() <= 1e-10, name


@pytest.mark.gpu
def test_batch_build_on_device_buffers(gpu, batch_case):
    """unomol_gpu_batch_fock_device: the caller's packed densities in and packed G out, on the caller's
    stream, equal to the build on the batch's own buffers."""
    import torch
    from unomol_gb300 import native
    gs, bases = batch_case
    bat = native.Batch(bases)
    Ps = [g["P_rand"] for g in gs]
    bat.set_precision(native.PREC_MIXED, 1e-3, 1e-13)
    bat.set_densities(Ps)
    bat.fock(native.BATCH_GRAPH)
    G_own = bat.get_focks()
    dev = torch.device("cuda", 0)
    dP = torch.from_numpy(np.concatenate(Ps)).to(dev)
    dG = torch.zeros_like(dP)
    s = torch.cuda.Stream(dev)
    bat.set_densities([np.zeros_like(P) for P in Ps])  # the batch's own buffer no longer holds the input
    for mode in (native.BATCH_GRAPH, native.BATCH_LAUNCHES):
        dG.zero_()
        torch.cuda.synchronize(dev)
        bat.fock_device(dP.data_ptr(), dG.data_ptr(), mode, s.cuda_stream)
        torch.cuda.synchronize(dev)
        G = dG.cpu().numpy()
        for o, b, Go in zip(bat.offsets, bases, G_own):
            assert np.abs(G[o:o + b.no2] - Go).max() <= 1e-12 * max(1.0, np.abs(Go).max()), mode
