"""CPU tests of the host side: library exports, basis reader, one-electron integrals, molecules."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, basis_of, golden_cases, load_golden


def _header_symbols():
    txt = open(os.path.join(ROOT, "include", "unomol_gb300.h")).read()
    return sorted(set(re.findall(r"\b(unomol_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from unomol_gb300 import native
    L = native.lib()
    syms = _header_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(L, s), f"{s} declared in include/unomol_gb300.h but not exported"
    for s in native.EXPORTS:
        assert s in syms


def test_version_string():
    from unomol_gb300 import native
    assert b"sm_103a" in native.lib().unomol_gpu_version()


def test_create_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from unomol_gb300 import native
    g = load_golden("h2o_sto3g_c0")
    with pytest.raises(native.UnomolError, match="no CUDA device"):
        native.TwoElectronInts(basis_of(g))


def _private_handle():
    """A CDLL object of its own, so that argument types set by a test leave the bindings' untouched."""
    from unomol_gb300 import native
    native.lib()
    return C.CDLL(native.LIB_PATH)


def test_missing_library_fails_loudly(monkeypatch):
    """Without the built library every binding raises: there is no CPU fallback."""
    from unomol_gb300 import native
    monkeypatch.setattr(native, "_LIB", None)
    monkeypatch.setattr(native, "LIB_PATH", os.path.join(ROOT, "no_such_dir", "libunomol_gb300.so"))
    with pytest.raises(native.UnomolError, match="no CPU fallback"):
        native.lib()
    with pytest.raises(native.UnomolError, match="is missing"):
        native.TwoElectronInts(basis_of(load_golden("h2o_sto3g_c0")))


def test_bad_basis_rejected_before_device_use():
    L = _private_handle()
    L.unomol_gpu_create.argtypes = [C.c_void_p, C.c_int, C.c_void_p]
    h = C.c_void_p()
    assert L.unomol_gpu_create(None, 0, C.byref(h)) == -1


def _header_declarations():
    txt = open(os.path.join(ROOT, "include", "unomol_gb300.h")).read()
    out = []
    for ret, name, params in re.findall(r"^(int|long long|void|const char\*)\s+(unomol_\w+)\(([^;]*?)\);", txt, re.M | re.S):
        out.append((ret, name, len([p for p in params.split(",") if p.strip() and p.strip() != "void"])))
    return out


def test_every_entry_point_rejects_null_arguments():
    """Every entry point called with null handles and pointers (zero sizes) returns UNOMOL_EINVAL
    (-1), destroys are no-ops and the error-string getters return a string: nothing dereferences a
    null argument or reaches the device first."""
    L = _private_handle()
    decls = _header_declarations()
    assert sorted(n for _, n, _ in decls) == _header_symbols()  # every declared entry point is called
    for ret, name, n in decls:
        f = getattr(L, name)
        f.argtypes = [C.c_void_p] * n
        if ret in ("int", "long long"):
            f.restype = C.c_int if ret == "int" else C.c_longlong
            if name in ("unomol_gpu_batch_size", "unomol_guess_num_molecules", "unomol_mlp_num_params"):
                assert f(*([None] * n)) < 0, name
            elif name == "unomol_tc_set_wait_polls":  # its one argument is a number: 0 = the default limit
                assert f(*([None] * n)) == 0, name
            else:
                assert f(*([None] * n)) == -1, name
        elif ret == "void":
            f.restype = None
            f(*([None] * n))
        else:
            f.restype = C.c_char_p
            assert isinstance(f(*([None] * n)), bytes), name


@pytest.mark.parametrize("field,index,value,message", [
    ("l", 0, 5, "angular momentum above 4"),
    ("np", 0, 0, "no primitives"),
    ("np", 1, 256, "more than 255 primitives"),
    ("c", 0, 99, "centre out of range"),
    ("o", 1, 0, "offsets must follow shell order"),
])
def test_malformed_basis_is_reported_on_any_machine(field, index, value, message):
    """A malformed basis description is rejected (UNOMOL_EINVAL, with the reason) before any device use."""
    from unomol_gb300 import native
    L = native.lib()
    g = load_golden("h2o_631g")
    d, keep = native.basis_desc(basis_of(g))
    keep[field][index] = value
    h = C.c_void_p()
    L.unomol_gpu_create.argtypes = [C.POINTER(native.BasisDesc), C.c_int, C.POINTER(C.c_void_p)]
    assert L.unomol_gpu_create(C.byref(d), 0, C.byref(h)) == -1
    assert message in L.unomol_gpu_last_error(None).decode()
    assert not h.value


@pytest.mark.parametrize("name", golden_cases())
def test_one_electron_matches_reference(name):
    from unomol_gb300 import native
    g = load_golden(name)
    S, T, H = native.one_electron(basis_of(g))
    assert np.abs(S - g["S"]).max() < 1e-12
    assert np.abs(T - g["T"]).max() < 1e-12
    assert np.abs(H - g["H"]).max() < 1e-12


def test_basis_reader_normalisation_matches_reference_export():
    """Shell::normalize restated (Basis.hpp:56-75): coefficients within 2 ulp of the reference's."""
    import sys
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import refh
    if not refh.available():
        pytest.skip("reference build not present (oracle/_ref)")
    from unomol_gb300.basis import Basis
    for tag in ("631.h2o", "dh95.co2", "3g.ch4"):
        path = os.path.join(refh.REFERENCE, "test", f"patin.dat.{tag}")
        rb = refh.RefBasis(path)
        info, a, c, cen = rb.export()
        b = Basis(path)
        assert np.abs(b.coef - c).max() <= 4 * np.finfo(float).eps * np.abs(c).max()
        assert (np.array(b.shell_offset) == info[:, 3]).all()


def test_molecule_generators():
    from unomol_gb300 import molecules
    from unomol_gb300.basis import Basis
    dec = molecules.alkane(10)
    assert len(dec) == 32
    C = np.array([x for e, x in dec if e == "C"])
    H = np.array([x for e, x in dec if e == "H"])
    d = np.linalg.norm(C[1:] - C[:-1], axis=1)
    assert np.allclose(d, 1.54)
    # every H at 1.09 A from its nearest carbon, every angle at a carbon 109.47 deg
    for h in H:
        assert abs(np.min(np.linalg.norm(C - h, axis=1)) - 1.09) < 1e-9
    for i, c in enumerate(C):
        nb = [x for x in np.vstack([C, H]) if 0.1 < np.linalg.norm(x - c) < 1.6]
        assert len(nb) == 4
        for a in range(4):
            for bb in range(a):
                u, v = nb[a] - c, nb[bb] - c
                ang = np.degrees(np.arccos(u @ v / np.linalg.norm(u) / np.linalg.norm(v)))
                assert abs(ang - 109.47) < 0.01  # a tetrahedron's angle is 109.4712 deg
    b = Basis(text=molecules.patin_text(dec, "6-31G"))
    assert b.norb == 134 and b.nshell == 94
    w = molecules.water_cluster(32, 0)
    O = np.array([x for e, x in w if e == "O"])
    dm = np.linalg.norm(O[:, None] - O[None], axis=2) + np.eye(32) * 10
    assert dm.min() >= 2.7 and O.min() >= 0 and O.max() <= 10.0 + 1.0
    b = Basis(text=molecules.patin_text(w, "6-31G"))
    assert b.norb == 416 and b.nshell == 288


def test_oracle_port_builds_without_reference():
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_batch_workload_generator():
    """The 256-molecule batching workload: half alkanes C1-C8, half clusters of 1-6 waters, STO-3G or
    6-31G per molecule, reproducible from its seed; 7 to 108 basis functions (C8H18/6-31G is the
    largest molecule the rules allow)."""
    from unomol_gb300 import molecules
    from unomol_gb300.basis import Basis
    work = molecules.batch_workload(seed=0)
    assert len(work) == 256
    labels = [l for l, _ in work]
    assert all(l.startswith("C") for l in labels[:128]) and all(l.startswith("(H2O)") for l in labels[128:])
    assert {l.split("/")[1] for l in labels} == {"STO-3G", "6-31G"}
    nbf = [Basis(text=t).norb for _, t in work]
    assert min(nbf) >= 7 and max(nbf) <= 108 and sum(nbf) == 11246
    assert [l for l, _ in molecules.batch_workload(seed=0)] == labels


def test_record_layout_is_the_reference_twoints():
    """The integral records of the conventional build are the reference's TwoInts (TwoElectronInts.hpp:20-23):
    a double and four ints, 24 bytes, the header's UnomolRecord."""
    from unomol_gb300 import native
    assert native.RECORD_DTYPE.itemsize == 24
    assert [native.RECORD_DTYPE.fields[k][1] for k in ("val", "i", "j", "k", "l")] == [0, 8, 12, 16, 20]
    txt = open(os.path.join(ROOT, "include", "unomol_gb300.h")).read()
    assert "double val;\n    int32_t i, j, k, l;\n} UnomolRecord;" in txt


def test_python_structures_match_the_c_header(tmp_path):
    """Every ctypes mirror of a structure of include/unomol_gb300.h has the C layout: the same size and the
    same offset for every field, as gcc lays out the header (the C ABI the bindings call through)."""
    import ctypes
    import subprocess
    from unomol_gb300 import learned, native
    structs = {"UnomolBasisDesc": native.BasisDesc, "UnomolStats": native.Stats, "UnomolStoreInfo": native.StoreInfo,
               "UnomolScfInput": native.ScfInput, "UnomolScfOptions": native.ScfOptions,
               "UnomolScfResult": native.ScfResult, "UnomolBatchScfResult": native.BatchScfResult,
               "UnomolGuessConfig": learned.GuessConfig, "UnomolGuessTrainOptions": learned.TrainOptions}
    src = ["#include <stdio.h>", "#include <stddef.h>", '#include "unomol_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        src.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            src.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    src += ["return 0;", "}"]
    c = tmp_path / "layout.c"
    c.write_text("\n".join(src) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                      text=True).stdout.splitlines())
    for cname, py in structs.items():
        assert int(got[cname]) == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(py, fname).offset, (cname, fname)
