"""Writes tests/golden/ref_pin_vectors.json: outputs of the reference's own
per-pair code (oracle/_ref/libref.so, compiled from the exaStamp sources by
oracle/ref_pin/build_ref.py) on seeded inputs, so the oracle stays pinned to
the reference where the exaStamp sources are not readable.

Run where they are:

    python tests/golden/make_ref_pin.py

Contents (every double as its exact hex form):
  lj_pair     (eps, sigma, r) -> (e, de)                 lennard_jones.h L41-50
  lj_atom     pair buffers (drx, dry, drz, d2) of one atom and (eps, sigma,
              ecut) -> (ep, fx, fy, fz, virial[9])      force_op_impl2.hxx L22-78
  eam         for the build's copper-like analytic table written as a setfl
              file (5,000-point grids): the sha256 of that file's text, the
              sha256 of the reference reader's three spline arrays
              (eam_alloy.cpp L29-278), and samples of eam_alloy_rho_noderiv,
              eam_alloy_mm_force and eam_alloy_fEmbed (eam_alloy.h L198-313)
"""
import hashlib
import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from exastamp_gb300 import setfl as SF  # noqa: E402

import ref_pin_lib as R  # noqa: E402

OUT = os.path.join(HERE, "ref_pin_vectors.json")


def hx(v):
    return [float(x).hex() for x in np.ravel(v)]


def cu_setfl_text(path):
    SF.write_setfl(SF.tabulate(SF.load_cu_params()), path)
    with open(path, "rb") as fh:
        return hashlib.sha256(fh.read()).hexdigest()


def main():
    L = R.load()
    if L is None:
        sys.exit("the pin library cannot be built here (exaStamp sources not readable)")
    rng = np.random.default_rng(2024)
    out = {"generator": "tests/golden/make_ref_pin.py", "lj_pair": [], "lj_atom": []}
    for _ in range(200):
        eps, sig = rng.uniform(0.1, 3.0), rng.uniform(0.5, 2.0)
        r = rng.uniform(0.6, 3.2) * sig
        out["lj_pair"].append(hx([eps, sig, r]) + hx(R.lj_pair(L, eps, sig, r)))
    for n in (1, 13, 30, 54):
        eps, sig = rng.uniform(0.5, 2.0), rng.uniform(0.8, 1.2)
        rc = 2.5 * sig
        # ecut = e(rcut) as the reference's operator computes it (pair_potential_impl.hxx L489-498)
        ecut = R.lj_pair(L, eps, sig, rc)[0]
        u = rng.normal(size=(n, 3))
        u /= np.linalg.norm(u, axis=1)[:, None]
        d = u * rng.uniform(0.85, rc, n)[:, None]
        d2 = d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2]
        res = R.lj_force_atom(L, eps, sig, ecut, d[:, 0], d[:, 1], d[:, 2], d2)
        out["lj_atom"].append({"params": hx([eps, sig, ecut]), "drx": hx(d[:, 0]), "dry": hx(d[:, 1]),
                               "drz": hx(d[:, 2]), "d2": hx(d2), "out": hx(res)})
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "cu_analytic.eam.alloy")
        text_sha = cu_setfl_text(path)
        nel, nr, nrho = R.eam_load(L, path)
        sf = SF.read_setfl(path)
    spl = [hashlib.sha256(np.ascontiguousarray(R.eam_spline(L, w), "<f8").tobytes()).hexdigest() for w in range(3)]
    cz, cf = R.eam_conversions(L)
    rhomax = (sf.nrho - 1) * sf.drho
    samples = []
    for _ in range(250):
        r = rng.uniform(0.5, sf.rcut * 1.08)
        fpi, fpj = rng.normal(0.0, 2.0, 2)
        dr = rng.normal(0.0, 1.0, 3)
        rho = rng.uniform(0.0, 1.3 * rhomax)
        v, phi = R.eam_mm_force(L, r, fpi, fpj, 0, 0, dr)
        fphi, fp = R.eam_fembed(L, rho, 0)
        samples.append(hx([r, fpi, fpj, dr[0], dr[1], dr[2], rho, L.ref_eam_rho(r, 0, 0), v[0], v[1], v[2], phi,
                           fphi, fp]))
    out["eam"] = {"setfl_text_sha256": text_sha, "nelements": nel, "nr": nr, "nrho": nrho,
                  "spline_sha256": {"frho": spl[0], "rhor": spl[1], "z2r": spl[2]},
                  "conversions": hx([cz, cf]),
                  "samples_columns": ["r", "fpi", "fpj", "dx", "dy", "dz", "rho", "rho_of_r", "fx", "fy", "fz",
                                      "phi", "F", "Fprime"],
                  "samples": samples}
    with open(OUT, "w") as fh:
        json.dump(out, fh, separators=(",", ":"))
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
