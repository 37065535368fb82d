"""Generates the DPM golden fixtures (dpm_<name>.npz) from the reference's own program and harness
(oracle/_ref/unomol and oracle/_ref/libunomol_ref.so, built from the reference sources by
oracle/Makefile).  Run in a container that has the reference tree:

    make -C oracle ref && python tests/golden/make_dpm_golden.py

Per case: the inputs (patin.dat with int_flag[0] = 1, posin.bas, the positron positions of
pos.grid.dat), the reference's vpol.out rows (q, vpol, alfa, vstat, vstat + vpol) and spol.out rows
(point, E_gs, E_init, E_final, vstat, ediff) of RestrictedHartreeFock::findPolarizationPotential
(RHF.hpp:292-388), and for the first position the reference's S, T + V and T + V - DPM over the
augmented basis (OneElectronInts.cpp, GDPMInts.cpp:86-143).
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import refh  # noqa: E402

from unomol_gb300 import molecules  # noqa: E402

CASES = {
    "dpm_h2o_sto3g": (molecules.water(), "STO-3G", [(0, 0, 4.0), (0, 0, 5.0), (0, 3.0, -3.0), (6.0, 0, 0)]),
    "dpm_h2o_631g": (molecules.water(), "6-31G", [(0, 0, 4.5), (3.0, 3.0, 3.0), (0, -5.0, 0)]),
    "dpm_ch4_sto3g": (molecules.alkane(1), "STO-3G", [(4.0, 4.0, 4.0), (0, 0, 6.0)]),
}


def run_case(name, atoms, basis, points):
    patin = molecules.patin_text(atoms, basis, int_flags=(1, 0), scf_flags=(2, 1, 0))
    posin = molecules.posin_text()
    grid = molecules.grid_text(points)
    with tempfile.TemporaryDirectory(prefix="unomol_dpm_") as wd:
        for fn, txt in (("patin.dat", patin), ("posin.bas", posin), ("pos.grid.dat", grid)):
            with open(os.path.join(wd, fn), "w") as f:
                f.write(txt)
        subprocess.run([os.path.join(ROOT, "oracle", "_ref", "unomol")], cwd=wd, check=True,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL, timeout=600)
        vpol = np.loadtxt(os.path.join(wd, "vpol.out"), ndmin=2)
        spol = np.loadtxt(os.path.join(wd, "spol.out"), ndmin=2)
        S, Hp, Hd = refh.dpm_h(wd, points[0])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), patin=patin, posin=posin,
                        points=np.array(points, float), vpol=vpol, spol=spol, S=S, H_plain=Hp, H_dpm=Hd)
    print(name, "vpol", vpol[:, 3])


def main():
    for name, (atoms, basis, pts) in CASES.items():
        run_case(name, atoms, basis, pts)


if __name__ == "__main__":
    main()
