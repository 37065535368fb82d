"""The C++ drop-in (include/unomol_gb300/TwoElectronInts.hpp).

* CPU (where the reference sources exist): the reference's unchanged Unomol.cc compiles and links
  against the drop-in and libunomol_gb300.so, and without a GPU it stops at the constructor with the
  library's error instead of falling back to the CPU.
* GPU: a C++ driver of the drop-in class reproduces the reference's G(P) (RHF and UHF) on golden cases.
"""
import os
import sys
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import ROOT, load_golden

INC = os.path.join(ROOT, "include")
LIBDIR = os.path.join(ROOT, "unomol_gb300")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import refh  # noqa: E402

REF = refh.REFERENCE


def _build_driver(tmp):
    exe = os.path.join(tmp, "dropin_main")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I" + INC, "-I" + os.path.join(ROOT, "tests", "cpp"),
                        os.path.join(ROOT, "tests", "cpp", "dropin_main.cpp"), "-o", exe, "-L" + LIBDIR,
                        "-lunomol_gb300", "-Wl,-rpath," + LIBDIR], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_dropin_driver_compiles():
    with tempfile.TemporaryDirectory() as tmp:
        _build_driver(tmp)


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference sources not present")
def test_unchanged_unomol_builds_against_dropin():
    objs = [os.path.join(ROOT, "oracle", "_ref", f + ".o") for f in
            ("Util", "SymmPack", "Rys", "Moments", "OneElectronInts", "FField", "GDPMInts", "putils_c")]
    if not all(os.path.exists(o) for o in objs):
        pytest.skip("oracle/_ref not built")
    with tempfile.TemporaryDirectory() as tmp:
        obj = os.path.join(tmp, "Unomol.o")
        exe = os.path.join(tmp, "Unomol_gb300")
        r = subprocess.run(["g++", "-std=c++17", "-O2", "-w", "-include",
                            os.path.join(INC, "unomol_gb300", "TwoElectronInts.hpp"), "-I" + REF, "-c",
                            os.path.join(REF, "Unomol.cc"), "-o", obj], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        r = subprocess.run(["g++", "-o", exe, obj, *objs, "-L" + LIBDIR, "-lunomol_gb300", "-Wl,-rpath," + LIBDIR],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        import torch
        if not torch.cuda.is_available():
            wd = os.path.join(tmp, "run")
            os.makedirs(wd)
            with open(os.path.join(REF, "test", "patin.dat.3g.h2o")) as f, open(os.path.join(wd, "patin.dat"), "w") as g:
                g.write(f.read())
            r = subprocess.run([exe], cwd=wd, capture_output=True, text=True, timeout=60)
            assert r.returncode != 0 and "no CUDA device" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["h2o_631g", "ref_631_co", "ref_dh95_h2", "h2o_cation_631g"])
def test_dropin_matches_reference(gpu, name):
    g = load_golden(name)
    with tempfile.TemporaryDirectory() as tmp:
        exe = _build_driver(tmp)
        patin = os.path.join(tmp, "patin.dat")
        with open(patin, "w") as f:
            f.write(str(g["patin"]))
        for k in ("P_rand", "Pa", "Pb"):
            g[k].astype(np.float64).tofile(os.path.join(tmp, k))
        r = subprocess.run([exe, patin, os.path.join(tmp, "P_rand"), os.path.join(tmp, "G")], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        G = np.fromfile(os.path.join(tmp, "G"))
        assert np.abs(G - g["G_rand"]).max() <= 1e-10
        r = subprocess.run([exe, patin, os.path.join(tmp, "Pa"), os.path.join(tmp, "Pb"), os.path.join(tmp, "Ga"),
                            os.path.join(tmp, "Gb")], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        assert np.abs(np.fromfile(os.path.join(tmp, "Ga")) - g["Ga"]).max() <= 1e-10
        assert np.abs(np.fromfile(os.path.join(tmp, "Gb")) - g["Gb"]).max() <= 1e-10
