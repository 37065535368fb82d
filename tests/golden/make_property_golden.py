"""Generates the moment / finite-field golden fixtures (prop_<case>.npz) from the reference's own
program (oracle/_ref/unomol, built from the reference sources by oracle/Makefile), run on the
reference's test inputs that ship moments.dat files.  Run in a container that has the reference tree:

    make -C oracle ref && python tests/golden/make_property_golden.py

Per case: the input (patin.dat; its int_flag[1] = 1 asks for the finite-field analysis), the final RHF
density (PMATRIX.DAT, RHF.hpp:172-174), the moments.out table (total / electronic / nuclear for dx,
dy, dz, qxx, qxy, qxz, qyy, qyz, qzz; Moments.cpp:184-271) with its two full-precision lines, and
finitefield.out (field, per-axis alfa and polarisation energy, isotropic and anisotropic alfa;
RHF.hpp:235-271).
"""
from __future__ import annotations

import os
import re
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
import sys  # noqa: E402

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))), "oracle"))
import refh  # noqa: E402

REF = refh.REFERENCE
CASES = [f"{b}.{m}" for b in ("3g", "431", "631") for m in ("co", "h2o", "hf", "nh3")]
NUM = r"[-+]?\d+\.\d+(?:[eE][-+]?\d+)?"


def parse_moments(text):
    rows = {}
    for line in text.splitlines():
        m = re.match(r"\s*(x|y|z|xx|xy|xz|yy|yz|zz)\s+(" + NUM + r")\s+(" + NUM + r")\s+(" + NUM + r")", line)
        if m:
            rows[m.group(1)] = [float(m.group(k)) for k in (2, 3, 4)]
    order = ("x", "y", "z", "xx", "xy", "xz", "yy", "yz", "zz")
    table = np.array([rows[k] for k in order])
    dip = float(re.search(r"Dipole moment\s*=\s*(" + NUM + ")", text).group(1))
    quad = float(re.search(r"Quadrupole moment\s*=\s*(" + NUM + ")", text).group(1))
    return table, dip, quad


def parse_ff(text):
    field = float(re.search(r"magnitude\s*=\s*(" + NUM + ")", text).group(1))
    ax = []
    for k in ("x", "y", "z"):
        m = re.search(r"^\s*" + k + r"\s+(" + NUM + r")\s+(" + NUM + ")", text, re.M)
        ax.append([float(m.group(1)), float(m.group(2))])
    iso = float(re.search(r"isotropic\s*=\s*(" + NUM + ")", text).group(1))
    aniso = float(re.search(r"aniso\s*=\s*(" + NUM + ")", text).group(1))
    return field, np.array(ax), iso, aniso


def main():
    for case in CASES:
        with open(os.path.join(REF, "test", f"patin.dat.{case}")) as f:
            patin = f.read()
        with tempfile.TemporaryDirectory(prefix="unomol_prop_") as wd:
            with open(os.path.join(wd, "patin.dat"), "w") as f:
                f.write(patin)
            subprocess.run([os.path.join(ROOT, "oracle", "_ref", "unomol")], cwd=wd, check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, timeout=600)
            with open(os.path.join(wd, "moments.out")) as f:
                table, dip, quad = parse_moments(f.read())
            with open(os.path.join(wd, "finitefield.out")) as f:
                field, ax, iso, aniso = parse_ff(f.read())
            P = np.fromfile(os.path.join(wd, "PMATRIX.DAT"), dtype=np.float64)
        name = "prop_" + case.replace(".", "_")
        np.savez_compressed(os.path.join(HERE, name + ".npz"), patin=patin, P=P, moments=table, dipole=dip,
                            quadrupole=quad, field=field, ff_alfa=ax[:, 0], ff_polnrg=ax[:, 1], ff_iso=iso,
                            ff_aniso=aniso)
        print(name, "dipole", dip, "alfa", ax[:, 0])


if __name__ == "__main__":
    main()
