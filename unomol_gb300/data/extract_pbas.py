"""Writes basis_sets.json from the reference's basis library file (pbas.lib).

The published STO-3G / 3-21G / 4-31G / 6-31G parameters of the light elements are copied as data
(exponent, contraction coefficient per primitive; s and p shells listed separately, as pbas.lib
lists them) so that molecules can be built without the reference tree.

    python unomol_gb300/data/extract_pbas.py /path/to/pbas.lib
"""
import json
import os
import sys

ELEMENTS = ["H", "HE", "LI", "BE", "B", "C", "N", "O", "F", "NE"]
BASES = ["STO-3G", "3-21G", "4-31G", "6-31G"]


def parse(path):
    lines = open(path).read().split("\n")
    out = {}
    i = 0
    while i < len(lines):
        tok = lines[i].strip()
        if ":" in tok:
            elem, name = tok.split(":", 1)
            if elem in ELEMENTS and name in BASES:
                nsh = int(lines[i + 1].split()[0])
                j = i + 2
                shells = []
                for _ in range(nsh):
                    npr, l = map(int, lines[j].split()[:2])
                    prims = [list(map(float, lines[j + 1 + k].split()[:2])) for k in range(npr)]
                    shells.append({"l": l, "prims": prims})
                    j += npr + 1
                out.setdefault(elem, {})[name] = shells
                i = j
                continue
        i += 1
    return out


if __name__ == "__main__":
    data = parse(sys.argv[1])
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "basis_sets.json")
    with open(dst, "w") as f:
        json.dump(data, f, indent=0)
    print("wrote", dst, {k: sorted(v) for k, v in data.items()})
