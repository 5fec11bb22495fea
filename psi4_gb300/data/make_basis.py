"""Extract the Gaussian basis sets this engine's workloads use into compact JSON.

The basis-set data are the published correlation-consistent sets (Dunning 1989 for
cc-pVXZ on H/C/O; Weigend 2002 for the cc-pVXZ-JKFIT fitting sets) as distributed
with psi4 in ``psi4/share/psi4/basis/*.gbs`` (Gaussian94 format).  Only the elements
the seeded workloads and the reference's stored test values need (H, C, O, Ar) are kept.  The files are data, not code; each
JSON records the source file and the element list.

Usage (in a checkout with the psi4 sources available)::

    python psi4_gb300/data/make_basis.py /path/to/psi4/share/psi4/basis

The JSON layout is ``{"name", "puream", "source", "elements": {sym: [shell, ...]}}``
with ``shell = {"l": int, "exps": [...], "coefs": [...]}`` (raw, unnormalised
contraction coefficients exactly as printed in the .gbs file).
"""
import json
import os
import sys

AM = {"S": 0, "P": 1, "D": 2, "F": 3, "G": 4, "H": 5, "I": 6}
BASES = ["cc-pvdz", "cc-pvdz-jkfit", "cc-pvtz", "cc-pvtz-jkfit", "cc-pv5z", "cc-pv5z-jkfit"]
ELEMENTS = ["H", "C", "O", "Ar"]


def _num(tok):
    return float(tok.replace("D", "E").replace("d", "e"))


def parse_gbs(path, keep):
    puream = None
    elements = {}
    with open(path) as fh:
        lines = [ln.strip() for ln in fh]
    i = 0
    n = len(lines)
    while i < n:
        ln = lines[i]
        if not ln or ln.startswith("!"):
            i += 1
            continue
        low = ln.lower()
        if low in ("spherical", "cartesian"):
            puream = low == "spherical"
            i += 1
            continue
        if ln.startswith("****"):
            i += 1
            continue
        toks = ln.split()
        if len(toks) == 2 and toks[1] == "0" and toks[0].isalpha():
            sym = toks[0].capitalize()
            shells = []
            i += 1
            while i < n and not lines[i].startswith("****"):
                st = lines[i].split()
                if not st or st[0].startswith("!"):
                    i += 1
                    continue
                kind, nprim = st[0].upper(), int(st[1])
                rows = [lines[i + 1 + k].split() for k in range(nprim)]
                i += 1 + nprim
                if kind == "SP":
                    shells.append({"l": 0, "exps": [_num(r[0]) for r in rows], "coefs": [_num(r[1]) for r in rows]})
                    shells.append({"l": 1, "exps": [_num(r[0]) for r in rows], "coefs": [_num(r[2]) for r in rows]})
                else:
                    shells.append({"l": AM[kind], "exps": [_num(r[0]) for r in rows], "coefs": [_num(r[1]) for r in rows]})
            if sym in keep:
                elements[sym] = shells
            continue
        i += 1
    return puream, elements


def main(src):
    out_dir = os.path.join(os.path.dirname(os.path.abspath(__file__)), "basis")
    os.makedirs(out_dir, exist_ok=True)
    for name in BASES:
        puream, elements = parse_gbs(os.path.join(src, name + ".gbs"), ELEMENTS)
        missing = [e for e in ELEMENTS if e not in elements]
        if missing:
            raise SystemExit(f"{name}: elements {missing} not found")
        doc = {"name": name, "puream": bool(puream), "source": f"psi4/share/psi4/basis/{name}.gbs",
               "elements": elements}
        with open(os.path.join(out_dir, name + ".json"), "w") as fh:
            json.dump(doc, fh, indent=0, separators=(",", ":"))
        print(name, {e: len(s) for e, s in elements.items()}, "puream" if puream else "cartesian")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: make_basis.py <psi4 source tree>/psi4/share/psi4/basis")
    main(sys.argv[1])
