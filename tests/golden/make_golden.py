"""Writes tests/golden/eam_setfl_lattice.json from exaStamp's own setfl
fixtures (data/potentials/*.eam.alloy of the exaStamp tree).

Run here, where the exaStamp sources are readable:

    python tests/golden/make_golden.py /path/to/exaStamp

For each potential it keeps the file header and only the table entries a
perfect-lattice known-answer test reads: windows of +-24 knots around every
neighbour-shell distance (r < rcut) of the element's lattice at a0 - 0.01,
..., a0 + 0.01 Angstrom, and around the embedding densities of those lattices.
The spline of data/potentials files is local (each knot's coefficients use
the four neighbouring values), so lookups inside a window are the same, bit
for bit, as with the full table.  The known answers themselves are the
header's lattice constant (zero pressure there) and, for the Ravelo Ta
models, their fitted cohesive energy of 8.1 eV per atom (PRB 88, 134101).
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

from exastamp_gb300 import setfl  # noqa: E402
from oracle import oracle as O  # noqa: E402

WIN = 24
SPAN = np.linspace(-0.01, 0.01, 5)
BASIS = {"bcc": np.array([[0, 0, 0], [.5, .5, .5]]),
         "fcc": np.array([[0, 0, 0], [.5, .5, 0], [.5, 0, .5], [0, .5, .5]])}
# (file, element index, cohesive energy in eV per atom or None)
CASES = [("Ta1_Ravelo_2013", 0, -8.1), ("Ta2_Ravelo_2013", 0, -8.1), ("AlCu", 0, None), ("AlCu", 1, None)]


def shells(struct, a, rcut):
    """Distinct neighbour distances (< rcut) and their counts around one site."""
    b = BASIS[struct]
    n = int(np.ceil(rcut / a)) + 1
    g = np.stack(np.meshgrid(*[np.arange(-n, n + 1)] * 3, indexing="ij"), -1).reshape(-1, 3)
    pts = ((g[:, None, :] + b[None, :, :]).reshape(-1, 3)) * a
    r = np.sqrt((pts ** 2).sum(1))
    r = r[(r > 0) & (r < rcut)]
    d, cnt = np.unique(np.round(r, 9), return_counts=True)
    return d, cnt


def windows(idx, n):
    """Merged [start, stop) index ranges of +-WIN around each 0-based index."""
    out = []
    for k in sorted(set(int(i) for i in idx)):
        lo, hi = max(0, k - WIN), min(n, k + WIN + 1)
        if out and lo <= out[-1][1]:
            out[-1][1] = max(out[-1][1], hi)
        else:
            out.append([lo, hi])
    return out


def main(ref_root):
    out = {"source": "exaStamp data/potentials/*.eam.alloy (setfl); generated by tests/golden/make_golden.py",
           "window": WIN, "potentials": {}, "cases": []}
    for fname, el, ecoh in CASES:
        path = os.path.join(ref_root, "data", "potentials", fname + ".eam.alloy")
        sf = setfl.read_setfl(path)
        pot = out["potentials"].setdefault(fname, {
            "elements": sf.elements, "Z": sf.Z, "masses": sf.masses, "a0": sf.a0, "structs": sf.structs,
            "nrho": sf.nrho, "drho": sf.drho, "nr": sf.nr, "dr": sf.dr, "rcut": sf.rcut,
            "frho": {}, "rhor": {}, "z2r": {}})
        struct = sf.structs[el].lower()
        a0 = sf.a0[el]
        kz = el * (el + 1) // 2 + el  # z2r index of the (el, el) pair, i >= j order
        ridx, rhoidx = [], []
        tab = O.EamOracleTables.from_setfl(sf, 1.0, 1.0)
        for da in SPAN:
            d, cnt = shells(struct, a0 + da, sf.rcut)
            ridx += [int(r / sf.dr) for r in d]
            rho = sum(c * O.eam_rho(tab, r, el, el) for r, c in zip(d, cnt))
            rhoidx.append(int(rho / sf.drho))
        for key, tab, idx, k in (("rhor", sf.rhor[el], ridx, el), ("z2r", sf.z2r[kz], ridx, kz),
                                 ("frho", sf.frho[el], rhoidx, el)):
            wl = pot[key].setdefault(str(k), [])
            for lo, hi in windows(idx, len(tab)):
                wl.append([lo, [float(v) for v in tab[lo:hi]]])
        out["cases"].append({"file": fname, "element": el, "struct": struct, "a0": a0, "z2r_index": kz,
                             "cohesive_energy_eV": ecoh, "lattice_offsets": [float(x) for x in SPAN]})
    # merge overlapping windows per table
    for pot in out["potentials"].values():
        for key in ("rhor", "z2r", "frho"):
            for k, wl in pot[key].items():
                wl.sort(key=lambda w: w[0])
                merged = []
                for lo, vals in wl:
                    if merged and lo <= merged[-1][0] + len(merged[-1][1]):
                        mlo, mv = merged[-1]
                        end = max(mlo + len(mv), lo + len(vals))
                        full = mv + [None] * (end - mlo - len(mv))
                        for i, v in enumerate(vals):
                            full[lo - mlo + i] = v
                        merged[-1] = [mlo, full]
                    else:
                        merged.append([lo, list(vals)])
                pot[key][k] = merged
    dst = os.path.join(HERE, "eam_setfl_lattice.json")
    with open(dst, "w") as fh:
        json.dump(out, fh, indent=0)
    print("wrote", dst, os.path.getsize(dst), "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("EXASTAMP_ROOT", ""))
