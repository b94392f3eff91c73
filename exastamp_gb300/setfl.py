"""setfl (``.eam.alloy``) files: reader, writer and analytic tabulation.

The reader follows the reference's ``eam_alloy_init`` parser
(src/potential/eam_potentials/eam_alloy/eam_alloy.cpp L86-201): three comment
lines, ``N el1 el2 ...``, ``nrho drho nr dr rcut``, then per element
``Z mass a0 structure`` followed by nrho F(rho) values and nr rho(r) values,
then the nel*(nel+1)/2 tables of z2r = r*phi(r) (eV*angstrom) in the order
1-1, 2-1, 2-2, 3-1, ... .  Knot k of a table sits at k*dr (or k*drho).

The tabulator restates the analytic-to-setfl step of the reference's
scripts/python/pytab-eam-alloy/pytab-eam-alloy-sutton-chen.py L39-100 for
the copper-like analytic form used by the benchmark (data/cu_analytic.json).
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass, field
from typing import List

import numpy as np

PARAM_NAMES = ("fe", "beta", "re", "A", "B", "alpha", "kappa", "F0", "F1")


@dataclass
class Setfl:
    elements: List[str]
    Z: List[int]
    masses: List[float]
    a0: List[float]
    structs: List[str]
    nrho: int
    drho: float
    nr: int
    dr: float
    rcut: float
    frho: List[np.ndarray]          # nel x nrho (eV)
    rhor: List[np.ndarray]          # nel x nr
    z2r: List[np.ndarray]           # nel*(nel+1)/2 x nr (eV*angstrom)
    comments: List[str] = field(default_factory=lambda: ["", "", ""])

    @property
    def nelements(self) -> int:
        return len(self.elements)


def read_setfl(path: str) -> Setfl:
    with open(path) as fh:
        lines = fh.read().split("\n")
    comments = lines[:3]
    toks = " ".join(lines[3:]).split()
    pos = 0

    def take(k=1):
        nonlocal pos
        v = toks[pos:pos + k]
        pos += k
        return v

    nel = int(take()[0])
    elements = take(nel)
    nrho, drho, nr, dr, rcut = take(5)
    nrho, nr = int(nrho), int(nr)
    drho, dr, rcut = float(drho), float(dr), float(rcut)
    Z, masses, a0, structs, frho, rhor = [], [], [], [], [], []
    for _ in range(nel):
        z, m, a, s = take(4)
        Z.append(int(z)); masses.append(float(m)); a0.append(float(a)); structs.append(s)
        frho.append(np.array(take(nrho), dtype=np.float64))
        rhor.append(np.array(take(nr), dtype=np.float64))
    z2r = [np.array(take(nr), dtype=np.float64) for _ in range(nel * (nel + 1) // 2)]
    return Setfl(elements, Z, masses, a0, structs, nrho, drho, nr, dr, rcut, frho, rhor, z2r, comments)


def write_setfl(sf: Setfl, path: str) -> None:
    def block(vals):
        out = []
        for k in range(0, len(vals), 5):
            out.append(" ".join("%.16e" % v for v in vals[k:k + 5]))
        return "\n".join(out)

    with open(path, "w") as fh:
        for c in (sf.comments + ["", "", ""])[:3]:
            fh.write(c + "\n")
        fh.write("%d %s\n" % (sf.nelements, " ".join(sf.elements)))
        fh.write("%d %.16e %d %.16e %.16e\n" % (sf.nrho, sf.drho, sf.nr, sf.dr, sf.rcut))
        for e in range(sf.nelements):
            fh.write("%d %.10g %.10g %s\n" % (sf.Z[e], sf.masses[e], sf.a0[e], sf.structs[e]))
            fh.write(block(sf.frho[e]) + "\n")
            fh.write(block(sf.rhor[e]) + "\n")
        for t in sf.z2r:
            fh.write(block(t) + "\n")


# --------------------------------------------------------------------------
# analytic copper-like EAM
# --------------------------------------------------------------------------

DATA = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "data")


def load_cu_params(path: str | None = None) -> dict:
    with open(path or os.path.join(DATA, "cu_analytic.json")) as fh:
        return json.load(fh)


def analytic_functions(p: dict, rho_e: float):
    """Return (f(r), phi(r), F(rho)) closures for parameter dict p."""
    fe, beta, re, A, B, alpha, kappa, F0, F1 = (p[k] for k in PARAM_NAMES)

    def f(r):
        return fe * np.exp(-beta * (r / re - 1.0))

    def phi(r):
        return A * np.exp(-alpha * (r / re - 1.0)) - B * np.exp(-kappa * (r / re - 1.0))

    def F(rho):
        return -F0 * np.sqrt(np.maximum(rho, 0.0) / rho_e) + F1 * (rho / rho_e)

    return f, phi, F


def table_grids(cfg: dict):
    nr, nrho = int(cfg["nr"]), int(cfg["nrho"])
    rcut = float(cfg["rcut"])
    dr = rcut / (nr - 1)
    drho = float(cfg["rhomax_over_rho_e"]) * float(cfg["rho_e"]) / (nrho - 1)
    r = np.arange(nr, dtype=np.float64) * dr
    rho = np.arange(nrho, dtype=np.float64) * drho
    return r, rho, dr, drho


def tabulate(cfg: dict, params: dict | None = None) -> Setfl:
    """Tabulate the analytic form onto setfl knots (r = k*dr, rho = k*drho)."""
    p = dict(cfg["params"])
    if params:
        p.update(params)
    r, rho, dr, drho = table_grids(cfg)
    f, phi, F = analytic_functions(p, float(cfg["rho_e"]))
    return Setfl([cfg["element"]], [int(cfg["Z"])], [float(cfg["mass"])], [float(cfg["lattice_constant"])],
                 [cfg["lattice"]], len(rho), drho, len(r), dr, float(cfg["rcut"]),
                 [F(rho)], [f(r)], [r * phi(r)],
                 ["analytic copper-like EAM (see data/cu_analytic.json)", "tabulated by exastamp_gb300.setfl",
                  "units: eV, angstrom"])


def table_param_jacobian(cfg: dict, params: dict | None = None):
    """d(table knot values)/d(parameter) for the 9 analytic parameters.

    Returns three arrays (frho, rhor, z2r) of shape (9, n) with the partial
    derivative of every tabulated knot value with respect to fe, beta, re, A,
    B, alpha, kappa, F0, F1 (in PARAM_NAMES order).  The spline coefficients
    are linear in the knot values, so this is the last link of the adjoint."""
    p = dict(cfg["params"])
    if params:
        p.update(params)
    fe, beta, re, A, B, alpha, kappa, F0, F1 = (p[k] for k in PARAM_NAMES)
    rho_e = float(cfg["rho_e"])
    r, rho, _, _ = table_grids(cfg)
    x = r / re - 1.0
    g = np.exp(-beta * x)
    ea, ek = np.exp(-alpha * x), np.exp(-kappa * x)
    s = rho / rho_e
    J_f = np.zeros((9, len(r)))
    J_f[0] = g
    J_f[1] = -fe * x * g
    J_f[2] = fe * g * beta * r / re ** 2
    J_z = np.zeros((9, len(r)))           # z2r = r * phi
    J_z[2] = r * (A * ea * alpha * r / re ** 2 - B * ek * kappa * r / re ** 2)
    J_z[3] = r * ea
    J_z[4] = -r * ek
    J_z[5] = -r * A * x * ea
    J_z[6] = r * B * x * ek
    J_F = np.zeros((9, len(rho)))
    J_F[7] = -np.sqrt(np.maximum(s, 0.0))
    J_F[8] = s
    return J_F, J_f, J_z


def write_cu_setfl(path: str, cfg: dict | None = None) -> Setfl:
    cfg = cfg or load_cu_params()
    sf = tabulate(cfg)
    write_setfl(sf, path)
    return sf
