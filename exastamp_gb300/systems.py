"""Seeded synthetic systems for the MD hot path (input generation only).

These restate the reference's setup operators as plain numpy generators:
``lattice`` (src/setup_system/region_lattice.cpp L29) for FCC/BCC crystals and
``init_temperature_new`` (src/setup_system/init_temperature_new.cpp
L277-283, L335, L361, L401-410) for Maxwell-Boltzmann velocities: unit
Gaussian draws, centre-of-mass velocity removed, then scaled so the
centre-of-mass-corrected temperature equals T.

Units: the reference's internal units are angstrom, dalton, picosecond
(energy Da*A^2/ps^2).  Lennard-Jones workloads use reduced units (k_B = 1).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List

import numpy as np

# CODATA 2018: internal energy unit Da*A^2/ps^2 in joules = 1.66053906660e-27 * 1e4
_DA_A2_PS2_J = 1.66053906660e-23
EV = 1.602176634e-19 / _DA_A2_PS2_J            # 1 eV in Da*A^2/ps^2
KB_METAL = 1.380649e-23 / _DA_A2_PS2_J         # Boltzmann constant in Da*A^2/ps^2/K


@dataclass
class System:
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    vx: np.ndarray
    vy: np.ndarray
    vz: np.ndarray
    type: np.ndarray          # uint8
    id: np.ndarray            # uint64
    lo: np.ndarray            # (3,)
    hi: np.ndarray            # (3,)
    masses: np.ndarray        # per type
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.x)

    @property
    def L(self) -> np.ndarray:
        return self.hi - self.lo

    def copy(self) -> "System":
        return System(*(np.array(getattr(self, k)) for k in
                        ("x", "y", "z", "vx", "vy", "vz", "type", "id", "lo", "hi", "masses")),
                      meta=dict(self.meta))

    def state(self) -> dict:
        """Mutable dict of contiguous arrays in the layout the oracle runner uses."""
        n = self.n
        return {"x": self.x.copy(), "y": self.y.copy(), "z": self.z.copy(),
                "vx": self.vx.copy(), "vy": self.vy.copy(), "vz": self.vz.copy(),
                "ax": np.zeros(n), "ay": np.zeros(n), "az": np.zeros(n), "ep": np.zeros(n),
                "type": np.ascontiguousarray(self.type, np.uint8),
                "id": np.ascontiguousarray(self.id, np.uint64)}


FCC_BASIS = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
BCC_BASIS = np.array([[0, 0, 0], [0.5, 0.5, 0.5]])


def lattice(nx: int, ny: int, nz: int, a, basis: np.ndarray):
    a = np.broadcast_to(np.asarray(a, dtype=np.float64), (3,))
    g = np.stack(np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij"), -1).reshape(-1, 3)
    pos = (g[:, None, :] + basis[None, :, :]).reshape(-1, 3) * a
    hi = np.array([nx, ny, nz], dtype=np.float64) * a
    return pos, np.zeros(3), hi


def grid_order(s: System, R: float) -> System:
    """The same atoms stored cell by cell in cells at least R wide, cell
    index (k ny + j) nx + i (z slowest), as an exaNBody grid holds them: a
    contiguous chunk of the arrays is then a slab of the box along z."""
    L = s.hi - s.lo
    nc = np.maximum(np.floor(L / R), 1).astype(np.int64)
    c = [np.clip(((a - lo) * (m / Ld)).astype(np.int64), 0, m - 1)
         for a, lo, Ld, m in zip((s.x, s.y, s.z), s.lo, L, nc)]
    perm = np.argsort((c[2] * nc[1] + c[1]) * nc[0] + c[0], kind="stable")
    for k in ("x", "y", "z", "vx", "vy", "vz", "type", "id"):
        setattr(s, k, np.ascontiguousarray(getattr(s, k)[perm]))
    s.meta = dict(s.meta, order="grid cells of %g, z slowest" % R)
    return s


def maxwell_boltzmann(masses_per_atom: np.ndarray, T: float, kB: float, rng: np.random.Generator):
    """init_temperature_new restated: Gaussian draws, remove v_cm, scale to T."""
    n = len(masses_per_atom)
    v = rng.standard_normal((n, 3))
    m = masses_per_atom[:, None]
    M = masses_per_atom.sum()
    vcm = (v * m).sum(0) / M
    ke = 0.5 * (m * v * v).sum(0) - 0.5 * M * vcm * vcm
    t_cur = 2.0 * ke.sum() / (3.0 * n * kB)
    scale = np.sqrt(T / t_cur) if t_cur > 0 else 0.0
    v = (v - vcm) * scale
    return v


def _make(pos, lo, hi, types, masses, v, meta):
    n = len(pos)
    return System(np.ascontiguousarray(pos[:, 0]), np.ascontiguousarray(pos[:, 1]),
                  np.ascontiguousarray(pos[:, 2]), np.ascontiguousarray(v[:, 0]),
                  np.ascontiguousarray(v[:, 1]), np.ascontiguousarray(v[:, 2]),
                  np.ascontiguousarray(types, np.uint8), np.arange(n, dtype=np.uint64),
                  np.asarray(lo, np.float64), np.asarray(hi, np.float64),
                  np.asarray(masses, np.float64), meta)


def lj_fcc(ncell: int = 20, density: float = 0.8442, T: float = 1.0, seed: int = 1) -> System:
    """LJ FCC crystal, reduced units: 4*ncell^3 atoms at reduced density rho*.

    ncell=20 is the 32,000-atom plain-FP64 case (a = (4/rho*)^(1/3))."""
    a = (4.0 / density) ** (1.0 / 3.0)
    pos, lo, hi = lattice(ncell, ncell, ncell, a, FCC_BASIS)
    masses = np.array([1.0])
    rng = np.random.default_rng(seed)
    v = maxwell_boltzmann(np.ones(len(pos)), T, 1.0, rng)
    return _make(pos, lo, hi, np.zeros(len(pos)), masses, v,
                 {"kind": "lj_fcc", "ncell": ncell, "a": a, "T": T, "seed": seed})


def eam_cu_fcc(ncell: int = 100, a: float = 3.615, T: float = 300.0, seed: int = 2,
               mass: float = 63.546, displace: float = 0.0) -> System:
    """Copper-like FCC crystal in metal units; ncell=100 gives 4,000,000 atoms."""
    pos, lo, hi = lattice(ncell, ncell, ncell, a, FCC_BASIS)
    rng = np.random.default_rng(seed)
    if displace > 0:
        pos = pos + rng.normal(0.0, displace, pos.shape)
        pos = lo + np.mod(pos - lo, hi - lo)
    v = maxwell_boltzmann(np.full(len(pos), mass), T, KB_METAL, rng)
    return _make(pos, lo, hi, np.zeros(len(pos)), np.array([mass]), v,
                 {"kind": "eam_cu_fcc", "ncell": ncell, "a": a, "T": T, "seed": seed})


# johnson_force parameter order (EamJohnsonParameters, johnson.h L28-49)
JOHNSON_PARAM_NAMES = ("re", "fe", "rhoe", "alpha", "beta", "A", "B", "kappa", "lambda", "Fn0", "Fn1", "Fn2",
                       "Fn3", "F0", "F1", "F2", "F3", "Fo", "eta")


def johnson_ta_params(conv: float = EV) -> np.ndarray:
    """The Ta parameter set of the reference's johnson_force regression case
    (data/regression_new/potentials/eam/eam_johnson/single_specy.msp L6-27),
    as the 19-vector of gbmd_set_eam_johnson: re in angstrom, energies (A, B,
    Fn*, F*, Fo) and fe, rhoe (eV/angstrom there) multiplied by `conv`; alpha,
    beta, kappa, lambda and eta dimensionless (the run file tags eta with eV,
    but it is an exponent)."""
    v = dict(re=2.860082, fe=3.08634, rhoe=33.787168, alpha=8.489528, beta=4.527748, A=0.611679, B=1.032101,
             kappa=0.176977, lambda_=0.353954, Fn0=-5.103845, Fn1=-0.405524, Fn2=1.112997, Fn3=-3.585325,
             F0=-5.14, F1=0.0, F2=1.640098, F3=0.221375, Fo=-5.141526, eta=0.848843)
    v["lambda"] = v.pop("lambda_")
    scaled = {"fe", "rhoe", "A", "B", "Fn0", "Fn1", "Fn2", "Fn3", "F0", "F1", "F2", "F3", "Fo"}
    return np.array([v[k] * (conv if k in scaled else 1.0) for k in JOHNSON_PARAM_NAMES])


# sutton_chen_force parameter order (EamSuttonChenParameters, sutton_chen.h L30-37)
SUTTON_CHEN_PARAM_NAMES = ("c", "epsilon", "a0", "n", "m")


def sutton_chen_cu_params() -> np.ndarray:
    """The Cu parameter set of the reference's sutton_chen_force regression
    case (data/regression_new/potentials/eam/eam_sutton_chen/single_specy.msp
    L8-13) in internal units: c, epsilon (3.605e-21 J), a0 (0.327 nm), n, m."""
    return np.array([3.317e+01, 3.605e-21 / _DA_A2_PS2_J, 3.27, 9.050, 5.005])


def ta_bcc(ncell: int = 20, a: float = 3.3, T: float = 300.0, noise: float = 0.05, seed: int = 7,
           mass: float = 180.95) -> System:
    """BCC tantalum as in the johnson_force regression case (20^3 cells of
    3.3 angstrom, positions shifted 0.01 angstrom, Gaussian noise 0.05
    angstrom; seeded here)."""
    pos, lo, hi = lattice(ncell, ncell, ncell, a, BCC_BASIS)
    rng = np.random.default_rng(seed)
    pos = pos + 0.01 + rng.normal(0.0, noise, pos.shape)
    pos = lo + np.mod(pos - lo, hi - lo)
    v = maxwell_boltzmann(np.full(len(pos), mass), T, KB_METAL, rng)
    return _make(pos, lo, hi, np.zeros(len(pos)), np.array([mass]), v,
                 {"kind": "ta_bcc", "ncell": ncell, "a": a, "T": T, "seed": seed})


def lj_binary_voids(n: int = 16_777_216, density: float = 1.2, frac_a: float = 0.8, nvoids: int = 64,
                    void_r: float = 8.0, T: float = 1.0, seed: int = 3, min_dist: float = 0.0) -> System:
    """Uneven-density LJ A/B mixture: uniform random positions at `density`
    outside `nvoids` spherical voids.  Types: 0 = A, 1 = B."""
    L = (n / density) ** (1.0 / 3.0)
    rng = np.random.default_rng(seed)
    centers = rng.uniform(0.0, L, (nvoids, 3))
    out = []
    need = n
    while need > 0:
        cand = rng.uniform(0.0, L, (int(need * 1.1) + 16, 3))
        keep = np.ones(len(cand), bool)
        # only the periodic slab |x - cx| < void_r can hit a void: candidates
        # sorted by x, each slab is one or two index ranges
        order = np.argsort(cand[:, 0], kind="stable")
        xs = cand[order, 0]
        for c in centers:
            parts = []
            for a, b in ((c[0] - void_r, c[0] + void_r), (c[0] - void_r + L, c[0] + void_r + L),
                         (c[0] - void_r - L, c[0] + void_r - L)):
                a, b = max(a, 0.0), min(b, L)
                if a < b:
                    parts.append(order[np.searchsorted(xs, a):np.searchsorted(xs, b, side="right")])
            sel = np.concatenate(parts)
            d = cand[sel] - c
            d -= L * np.round(d / L)
            keep[sel[(d * d).sum(1) <= void_r * void_r]] = False
        cand = cand[keep][:need]
        out.append(cand)
        need -= len(cand)
    pos = np.concatenate(out)
    na = int(round(frac_a * n))
    types = np.zeros(n, np.uint8)
    types[rng.permutation(n)[: n - na]] = 1
    v = maxwell_boltzmann(np.ones(n), T, 1.0, rng)
    return _make(pos, np.zeros(3), np.full(3, L), types, np.array([1.0, 1.0]), v,
                 {"kind": "lj_binary_voids", "n": n, "L": L, "seed": seed})


def kob_andersen_tables():
    """Per-type-pair (eps, sigma, rcut) of the binary mixture: eps AA 1, AB 1.5,
    BB 0.5; sigma AA 1, AB 0.8, BB 0.88; cutoff 2.5*sigma_pair."""
    eps = np.array([[1.0, 1.5], [1.5, 0.5]])
    sig = np.array([[1.0, 0.8], [0.8, 0.88]])
    rc = 2.5 * sig
    return eps, sig, rc


def adjoint_training_set(nconf: int = 256, ncell: int = 4, seed: int = 4, vac_frac: float = 0.05):
    """Small FCC copper-like training configurations (256 sites, 5% vacancies,
    a in [3.5, 3.75] A, Gaussian displacements sigma in [0.05, 0.15] A)."""
    rng = np.random.default_rng(seed)
    confs: List[System] = []
    for c in range(nconf):
        a = rng.uniform(3.5, 3.75)
        pos, lo, hi = lattice(ncell, ncell, ncell, a, FCC_BASIS)
        nvac = int(round(vac_frac * len(pos)))
        keep = np.sort(rng.permutation(len(pos))[nvac:])
        pos = pos[keep]
        sig = rng.uniform(0.05, 0.15)
        pos = pos + rng.normal(0.0, sig, pos.shape)
        pos = lo + np.mod(pos - lo, hi - lo)
        v = np.zeros_like(pos)
        confs.append(_make(pos, lo, hi, np.zeros(len(pos)), np.array([63.546]), v,
                           {"a": a, "sigma": sig}))
    return confs


def replica_set(nrep: int = 4096, nmin: int = 32, nmax: int = 2048, seed: int = 6,
                rmin_box: float = 5.3):
    """Independent periodic copper-like replicas with log-uniform atom counts.

    FCC or BCC, random strain up to 3% per axis, thermal displacements for
    300-1200 K.  Every box edge is kept >= rmin_box (the neighbour radius)."""
    rng = np.random.default_rng(seed)
    out: List[System] = []
    for r in range(nrep):
        target = float(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))
        fcc = rng.random() < 0.5
        basis = FCC_BASIS if fcc else BCC_BASIS
        a = 3.615 if fcc else 2.87
        per = len(basis)
        cells = max(1, target / per)
        k = max(1, int(round(cells ** (1.0 / 3.0))))
        dims = [k, k, max(1, int(round(cells / (k * k))))]
        for d in range(3):
            while dims[d] * a < rmin_box * 1.001:
                dims[d] += 1
        strain = 1.0 + rng.uniform(-0.03, 0.03, 3)
        pos, lo, hi = lattice(dims[0], dims[1], dims[2], a * strain, basis)
        T = rng.uniform(300.0, 1200.0)
        sig = np.sqrt(KB_METAL * T / (63.546 * 4.0e3))   # ~0.05-0.1 A
        pos = pos + rng.normal(0.0, sig, pos.shape)
        pos = lo + np.mod(pos - lo, hi - lo)
        out.append(_make(pos, lo, hi, np.zeros(len(pos)), np.array([63.546]), np.zeros_like(pos),
                         {"T": T, "fcc": fcc}))
    return out
