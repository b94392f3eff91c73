"""Setfl tables rebuilt from tests/golden/eam_setfl_lattice.json (windows of
exaStamp's own data/potentials/*.eam.alloy fixtures) and the perfect-lattice
known-answer cases that go with them."""
import json
import os

import numpy as np

from exastamp_gb300 import setfl, systems as S

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "eam_setfl_lattice.json")
BASIS = {"bcc": S.BCC_BASIS, "fcc": S.FCC_BASIS}


def load():
    with open(FIXTURE) as fh:
        return json.load(fh)


def _table(windows, n):
    """Full-length table: window values exactly, linear in between (never read
    by a perfect-lattice evaluation)."""
    idx, val = [], []
    for lo, vals in windows:
        idx += list(range(lo, lo + len(vals)))
        val += vals
    idx, val = np.array(idx), np.array(val, dtype=np.float64)
    t = np.interp(np.arange(n), idx, val)
    t[idx] = val
    return t


def setfl_for(case, fx):
    """One-element Setfl of the case's element (tables of that element only)."""
    p = fx["potentials"][case["file"]]
    e = case["element"]
    frho = _table(p["frho"][str(e)], p["nrho"])
    rhor = _table(p["rhor"][str(e)], p["nr"])
    z2r = _table(p["z2r"][str(case["z2r_index"])], p["nr"])
    return setfl.Setfl([p["elements"][e]], [p["Z"][e]], [p["masses"][e]], [p["a0"][e]], [p["structs"][e]],
                       p["nrho"], p["drho"], p["nr"], p["dr"], p["rcut"], [frho], [rhor], [z2r])


def lattice_system(case, a, ncell=6, mass=1.0):
    pos, lo, hi = S.lattice(ncell, ncell, ncell, a, BASIS[case["struct"]])
    return S._make(pos, lo, hi, np.zeros(len(pos)), np.array([mass]), np.zeros_like(pos), {})
