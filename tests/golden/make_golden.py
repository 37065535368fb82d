"""Generates the golden fixtures in this folder from the reference itself (oracle/_ref, built from the
reference sources by oracle/Makefile).  Run in a container that has the reference tree:

    make -C oracle && python tests/golden/make_golden.py [--big]

Per case (<name>.npz):
  patin            the input text (patin.dat format)
  S, T, H          one-electron matrices (OneElectronInts.cpp), packed
  P_rand, G_rand   a seeded random symmetric density and the reference's G(P) (TwoElectronInts.cpp:822-844)
  Pa, Pb, Ga, Gb   seeded random alpha/beta densities and the reference's UHF G (TwoElectronInts.cpp:846-869)
  n_stored         number of integral records the reference stored (|v| > 1e-14)
  scf_*            (SCF cases) final / initial energy, iterations and final P of the stock SCF
  golden_energy    (reference test inputs) the published energy of test/scfout.dat.*
  ints_*           (small cases) the reference's stored integral records (val, i, j, k, l)

--big writes the scale fixtures (make_big_case): n-decane 6-31G (RHF and the UHF doublet cation) and
the 32-water 6-31G cluster (seed 0).  The reference's own damped SCF does not converge on either, so
their energies come from the test-only DIIS loop over the reference's formGmatrix (oracle/ref_harness.cpp
diis_loop); the first iterations of the stock damped loop are recorded as well.  About 2 minutes for
decane and 15 minutes for the cluster (its reference integral pass alone takes 10).
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

import refh  # noqa: E402

from unomol_gb300 import molecules  # noqa: E402

REF = refh.REFERENCE


def rand_density(n: int, seed: int, scale: float = 0.3) -> np.ndarray:
    rng = np.random.default_rng(seed)
    m = rng.uniform(-scale, scale, (n, n))
    m = 0.5 * (m + m.T) + np.diag(rng.uniform(0.0, 1.0, n))
    return np.ascontiguousarray(m[np.tril_indices(n)])


def make_case(name: str, patin: str, scf: bool, golden_energy: float | None, dump_ints: bool, md: bool = False):
    path = os.path.join(HERE, f"_{name}.patin")
    with open(path, "w") as f:
        f.write(patin)
    b = refh.RefBasis(path, md)
    S, T, H = b.one_electron()
    t = refh.RefTwoElectronInts(b)
    n = b.norb
    out = {"patin": np.array(patin), "S": S, "T": T, "H": H}
    seed = abs(hash(name)) % (2 ** 31)
    seed = sum(ord(c) * 131 ** i for i, c in enumerate(name)) % (2 ** 31)
    P = rand_density(n, seed)
    out["P_rand"], out["G_rand"] = P, t.form_g(P)
    Pa, Pb = rand_density(n, seed + 1), rand_density(n, seed + 2)
    Ga, Gb = t.form_g_uhf(Pa, Pb)
    out.update(Pa=Pa, Pb=Pb, Ga=Ga, Gb=Gb)
    vals, ijkl = t.records()
    out["n_stored"] = np.array(len(vals))
    if dump_ints:
        out["ints_val"], out["ints_ijkl"] = vals, ijkl
    del t
    if not md:
        # the same reference with its two-root Rys fit replaced by exact quadrature
        be = refh.RefBasis(path, "exact")
        te = refh.RefTwoElectronInts(be)
        out["G_rand_exact"] = te.form_g(P)
        out["Ga_exact"], out["Gb_exact"] = te.form_g_uhf(Pa, Pb)
        del te
    if scf:
        r = refh.run_scf(path, md)
        out.update(scf_energy=np.array(r["energy"]), scf_init_energy=np.array(r["init_energy"]),
                   scf_iterations=np.array(r["iterations"]), scf_P=r["P"], scf_nucrep=np.array(r["nucrep"]))
        if not md:
            re = refh.run_scf(path, "exact")
            out.update(scf_energy_exact=np.array(re["energy"]), scf_iterations_exact=np.array(re["iterations"]))
    if golden_energy is not None:
        out["golden_energy"] = np.array(golden_energy)
    os.remove(path)
    np.savez_compressed(os.path.join(HERE, f"{name}{'_md' if md else ''}.npz"), **out)
    print(name, "nbf", n, "stored", len(vals), "E" if scf else "", out.get("scf_energy", ""), file=sys.stderr)


def make_big_case(name: str, patin: str, cation_patin: str | None, fragments: list | None, seed: int,
                   keep_conv: bool):
    """A scale fixture (<name>.npz), arrays kept to what the GPU tests read:
      patin, seed           the input and the seed of rand_density(n, seed) (P is rebuilt by the tests)
      G_rand                the reference's G(P_rand) (TwoElectronInts.cpp:822-844)
      n_stored              integral records the reference stored
      diis_energy, diis_iterations, diis_error
                            the DIIS SCF of the reference's pieces (RHF), from the core-H guess or, with
                            `fragments`, from the superposition of the fragments' own DIIS densities
      trace                 the first 5 total energies of the stock damped loop (core-H guess)
      P_conv, G_conv        (keep_conv) the DIIS density and the reference's G of it
      patin_cation, Pa/Pb seeds, Ga, Gb, uhf_diis_*, trace_uhf
                            (cation_patin) the same basis with one electron less: UHF G of seeded
                            densities (TwoElectronInts.cpp:846-869), its DIIS energy and stock trace
    """
    import time
    t0 = time.time()
    path = os.path.join(HERE, f"_{name}.patin")
    with open(path, "w") as f:
        f.write(patin)
    b = refh.RefBasis(path)
    t = refh.RefTwoElectronInts(b)
    n = b.norb
    out = {"patin": np.array(patin), "seed": np.array(seed)}
    P = rand_density(n, seed)
    out["G_rand"] = t.form_g(P)
    vals, _ = t.records()
    out["n_stored"] = np.array(len(vals))
    del vals
    print(name, "integrals + G", f"{time.time() - t0:.1f} s", file=sys.stderr)
    P0 = None
    if fragments:
        P0 = np.zeros((n, n))
        for k, (ftext, aos) in enumerate(fragments):
            fp = os.path.join(HERE, f"_{name}_frag.patin")
            with open(fp, "w") as f:
                f.write(ftext)
            fb = refh.RefBasis(fp)
            ft = refh.RefTwoElectronInts(fb)
            r = refh.scf_diis(fb, ft, eps_e=1e-8, eps_err=1e-5, maxits=60)
            Pf = np.zeros((fb.norb, fb.norb))
            Pf[np.tril_indices(fb.norb)] = r["P"]
            Pf = Pf + Pf.T - np.diag(np.diag(Pf))
            P0[np.ix_(aos, aos)] = Pf
            del ft, fb
            os.remove(fp)
        P0 = np.ascontiguousarray(P0[np.tril_indices(n)])
    r = refh.scf_diis(b, t, P0=P0, maxits=200, eps_e=1e-12, eps_err=1e-9)
    assert r["converged"], (name, r)
    out.update(diis_energy=np.array(r["energy"]), diis_iterations=np.array(r["iterations"]),
               diis_error=np.array(r["error"]))
    print(name, "DIIS", r["energy"], r["iterations"], f"{time.time() - t0:.1f} s", file=sys.stderr)
    if keep_conv:
        out["P_conv"] = r["P"]
        out["G_conv"] = t.form_g(r["P"])
    out["trace"] = refh.scf_trace(b, t, 5)
    print(name, "trace", out["trace"], file=sys.stderr)
    if cation_patin is not None:
        cpath = os.path.join(HERE, f"_{name}_cation.patin")
        with open(cpath, "w") as f:
            f.write(cation_patin)
        cb = refh.RefBasis(cpath)
        assert cb.nelec % 2 == 1 and cb.norb == n
        out["patin_cation"] = np.array(cation_patin)
        Pa, Pb = rand_density(n, seed + 1), rand_density(n, seed + 2)
        out["Ga"], out["Gb"] = t.form_g_uhf(Pa, Pb)
        ru = refh.scf_diis(cb, t, maxits=300, eps_e=1e-12, eps_err=1e-9)
        assert ru["converged"], (name, ru)
        out.update(uhf_diis_energy=np.array(ru["energy"]), uhf_diis_iterations=np.array(ru["iterations"]),
                   uhf_diis_error=np.array(ru["error"]))
        out["trace_uhf"] = refh.scf_trace(cb, t, 5)
        print(name, "UHF DIIS", ru["energy"], ru["iterations"], out["trace_uhf"], file=sys.stderr)
        del cb
        os.remove(cpath)
    del t
    os.remove(path)
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(name, "nbf", n, "stored", out["n_stored"], f"{time.time() - t0:.1f} s", file=sys.stderr)


def water_fragments(nw: int, seed: int, basis: str):
    """Per monomer of molecules.water_cluster(nw, seed): its patin text and its AO indices in the
    cluster's basis (shells atom after atom, 13 functions per water in 6-31G)."""
    atoms = molecules.water_cluster(nw, seed)
    out, off = [], 0
    for m in range(nw):
        mono = atoms[3 * m:3 * m + 3]
        txt = molecules.patin_text(mono, basis, eps=1e-8)
        nbf = int(txt.split()[1])
        out.append((txt, list(range(off, off + nbf))))
        off += nbf
    return out


def pbas_patin(atoms_bohr, key: str, nelec: int, eps: float = 1e-10) -> str:
    """patin.dat text for atoms [(Z, (x, y, z) bohr)] with basis `key` of the reference's pbas.lib
    (used for the f-shell cases: the basis_sets.json of the package holds the light bases only)."""
    lines = open(os.path.join(REF, "pbas.lib")).read().split("\n")
    i = lines.index(key)
    nsh = int(lines[i + 1].split()[0])
    j = i + 2
    shells = []
    for _ in range(nsh):
        npr, l = map(int, lines[j].split()[:2])
        shells.append((l, [lines[j + 1 + k].split()[:2] for k in range(npr)]))
        j += npr + 1
    out_s, norb, maxl = [], 0, 0
    for c in range(len(atoms_bohr)):
        for l, prims in shells:
            out_s.append(f"{len(prims):4d}{l:4d}{c:6d}")
            out_s += [f"{a} {k}" for a, k in prims]
            norb += (l + 1) * (l + 2) // 2
            maxl = max(maxl, l)
    head = [f"{len(shells) * len(atoms_bohr):7d}{norb:7d}{len(atoms_bohr):7d}{maxl:3d}", f"{nelec:7d}{299:7d}",
            f"{eps:24.16e}", " 0 0", " 2 1 0", " 0 0 0"]
    cen = [f"{float(z):15.10f}" + "".join(f"{v:20.12f}" for v in x) for z, x in atoms_bohr]
    return "\n".join(head + cen + out_s) + "\n"


def published_energy(tag: str) -> float:
    with open(os.path.join(REF, "test", f"scfout.dat.{tag}")) as f:
        for line in f:
            if line.startswith("Hartree Fock Energy"):
                return float(line.split("=")[1].split()[0])
    raise ValueError(tag)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--big", action="store_true")
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    cases = []
    # the configuration-0 water (STO-3G, eps 1e-10, flags 2 1 0)
    cases.append(("h2o_sto3g_c0", molecules.patin_text(molecules.water(), "STO-3G", eps=1e-10), True, None, True))
    cases.append(("h2o_631g", molecules.patin_text(molecules.water(), "6-31G", eps=1e-10), True, None, True))
    # the reference's own test inputs with published energies (test/scfout.dat.*)
    for bas in ("3g", "431", "631"):
        for mol in ("h2", "n2", "co", "hf", "h2o", "nh3", "ch4"):
            tag = f"{bas}.{mol}"
            with open(os.path.join(REF, "test", f"patin.dat.{tag}")) as f:
                txt = f.read()
            cases.append((f"ref_{bas}_{mol}", txt, True, published_energy(tag), False))
    # inputs without published outputs: open shells (UHF) and d shells
    for tag in ("b.dhdz", "n.dhdz", "f.dhdz", "dh95.h2", "dh95.co2", "d6s3p.h2", "tzp.ch4"):
        with open(os.path.join(REF, "test", f"patin.dat.{tag}")) as f:
            txt = f.read()
        cases.append((f"ref_{tag.replace('.', '_')}", txt, True, None, False))
    # small UHF radicals and small alkanes
    cases.append(("h2o_cation_631g", molecules.patin_text(molecules.water(), "6-31G", charge=1, eps=1e-10), True, None, False))
    cases.append(("ethane_631g", molecules.patin_text(molecules.alkane(2), "6-31G", eps=1e-10), True, None, False))
    cases.append(("propane_cation_sto3g", molecules.patin_text(molecules.alkane(3), "STO-3G", charge=1, eps=1e-10), True, None, False))
    cases.append(("water3_631g", molecules.patin_text(molecules.water_cluster(3, 7), "6-31G", eps=1e-10), True, None, False))
    # f shells (He cc-pVQZ of pbas.lib): classes with la+lb+lc+ld > 8 run the reference's MD path
    fcases = [("he_ccpvqz", pbas_patin([(2, (0.0, 0.0, 0.0))], "HE:CC-PVQZU", 2), True, None, False),
              ("he2_ccpvqz", pbas_patin([(2, (0.0, 0.0, 0.0)), (2, (0.0, 0.0, 3.0))], "HE:CC-PVQZU", 4), False, None, False)]
    cases += fcases
    if a.big:
        big = [("decane_631g", molecules.patin_text(molecules.alkane(10), "6-31G", eps=1e-10),
                molecules.patin_text(molecules.alkane(10), "6-31G", charge=1, eps=1e-10), None, 1010, True),
               ("water32_631g", molecules.patin_text(molecules.water_cluster(32, 0), "6-31G", eps=1e-10), None,
                water_fragments(32, 0, "6-31G"), 3232, False)]
        for c in big:
            if a.only and a.only not in c[0]:
                continue
            make_big_case(*c)
        return
    for c in cases:
        if a.only and a.only not in c[0]:
            continue
        make_case(*c)
    # MD-only reference build on a few cases (parity target of the MD mode)
    for c in cases[:2] + fcases:
        if a.only and a.only not in c[0]:
            continue
        make_case(c[0], c[1], False, None, False, md=True)


if __name__ == "__main__":
    main()
