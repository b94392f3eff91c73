"""ctypes binding of the CPU FP64 oracle (oracle/gbmd_oracle.c).

TEST INFRASTRUCTURE ONLY.  This module is the correctness checker for the
GB300 kernels and the timed CPU baseline; only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its CPU-baseline leg and its
reference arm) may import it.  The product package never does.

Every function here forwards to the C restatement, which cites the exaStamp
file:line it follows.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "gbmd_oracle.c")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "liboracle.so")


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (-O3 -fopenmp -ffp-contract=off)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                             os.path.getmtime(os.path.join(HERE, "gbmd_oracle.h")))):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11",
           "-o", tmp, SRC, "-lm"]
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


class EamTables(C.Structure):
    _fields_ = [("nelements", C.c_int), ("nr", C.c_int), ("nrho", C.c_int), ("pad_", C.c_int),
                ("rdr", C.c_double), ("rdrho", C.c_double), ("rhomax", C.c_double),
                ("conv_z2r", C.c_double), ("conv_frho", C.c_double),
                ("frho", C.c_void_p), ("rhor", C.c_void_p), ("z2r", C.c_void_p)]


class EamPot(C.Structure):
    _fields_ = [("t", EamTables), ("rcut", C.c_double)]


class LJParams(C.Structure):
    _fields_ = [("epsilon", C.c_double), ("sigma", C.c_double), ("rcut", C.c_double)]


class LJMultiParams(C.Structure):
    _fields_ = [("ntypes", C.c_int), ("pad_", C.c_int), ("epsilon", C.c_void_p),
                ("sigma", C.c_void_p), ("rcut", C.c_void_p), ("rcut_max", C.c_double)]


POT_LJ, POT_LJ_MULTI, POT_EAM, POT_EAM_JOHNSON, POT_EAM_SUTTON_CHEN = 0, 1, 2, 3, 4


class JohnsonParams(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("re", "fe", "rhoe", "alpha", "beta", "A", "B", "kappa", "lambda_",
                                          "Fn0", "Fn1", "Fn2", "Fn3", "F0", "F1", "F2", "F3", "Fo", "eta")]


class JohnsonPot(C.Structure):
    _fields_ = [("p", JohnsonParams), ("rcut", C.c_double)]


class Johnson:
    """johnson_force parameters (19-vector, EamJohnsonParameters order) + rcut."""

    def __init__(self, params, rcut):
        self.pot = JohnsonPot(JohnsonParams(*[float(v) for v in params]), float(rcut))


class SuttonChenParams(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("c", "epsilon", "a0", "n", "m")]


class SuttonChenPot(C.Structure):
    _fields_ = [("p", SuttonChenParams), ("rcut", C.c_double)]


class SuttonChen:
    """sutton_chen_force parameters (c, epsilon, a0, n, m) + rcut."""

    def __init__(self, params, rcut):
        self.pot = SuttonChenPot(SuttonChenParams(*[float(v) for v in params]), float(rcut))

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        L = _lib
        vp, i64, dbl, i32 = C.c_void_p, C.c_int64, C.c_double, C.c_int
        L.orc_grid_dims.argtypes = [vp, vp, dbl, vp]
        L.orc_wrap.restype = i64
        L.orc_wrap.argtypes = [i64, vp, vp, vp, vp, vp]
        L.orc_build_neighbors.restype = i64
        L.orc_build_neighbors.argtypes = [i64, vp, vp, vp, vp, vp, vp, dbl, vp, i64, vp, vp]
        L.orc_build_neighbors_first.restype = i64
        L.orc_build_neighbors_first.argtypes = [i64, i64, vp, vp, vp, vp, vp, vp, dbl, vp, i64, vp, vp]
        L.orc_brute_pairs.restype = i64
        L.orc_brute_pairs.argtypes = [i64, vp, vp, vp, vp, vp, dbl, i64, vp, vp, vp]
        L.orc_lj_energy_cut.restype = dbl
        L.orc_lj_energy_cut.argtypes = [dbl, dbl, dbl]
        L.orc_lj_pair.argtypes = [dbl, dbl, dbl, vp, vp]
        L.orc_lj_atom_buffer.argtypes = [dbl, dbl, dbl, i32, vp, vp, vp, vp, vp]
        L.orc_lj_force.argtypes = [i64, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        L.orc_lj_multi_force.argtypes = [i64, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        L.orc_lj_direct.restype = dbl
        L.orc_lj_direct.argtypes = [i64, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        L.orc_eam_spline.argtypes = [i32, dbl, vp, vp]
        L.orc_eam_rho.restype = dbl
        L.orc_eam_rho.argtypes = [vp, dbl, i32, i32]
        L.orc_eam_embed_one.argtypes = [vp, dbl, i32, vp, vp]
        L.orc_eam_pair_force.argtypes = [vp, dbl, dbl, dbl, i32, i32, vp, vp]
        L.orc_eam_density.argtypes = [i64, vp, vp, vp, vp, vp, vp, vp, vp, vp, dbl, vp]
        L.orc_eam_embed.argtypes = [i64, vp, vp, vp, vp]
        L.orc_eam_force.argtypes = [i64, vp, vp, vp, vp, vp, vp, vp, vp, vp, dbl, vp, vp, vp, vp,
                                    vp, vp]
        L.orc_push_f_v_r.argtypes = [i64, vp, vp, vp, vp, vp, vp, vp, vp, vp, dbl, dbl]
        L.orc_push_f_v.argtypes = [i64, vp, vp, vp, vp, vp, vp, dbl, dbl]
        L.orc_push_min.argtypes = [i64, vp, vp, vp, vp, vp, vp, vp, vp, dbl, dbl, dbl]
        L.orc_force_to_accel.argtypes = [i64, vp, vp, vp, vp, vp]
        L.orc_thermo.argtypes = [i64, vp, vp, vp, vp, vp, vp, vp, vp]
        L.orc_run_nve.restype = i32
        L.orc_run_nve.argtypes = [i64] + [vp] * 15 + [i32, vp, dbl, dbl, i32, i32, vp]
        L.orc_run_nve_from.restype = i32
        L.orc_run_nve_from.argtypes = [i64] + [vp] * 15 + [i32, vp, dbl, dbl, i32, i32, vp]
        L.orc_run_minimize.restype = i32
        L.orc_run_minimize.argtypes = [i64] + [vp] * 12 + [i32, vp, dbl, dbl, dbl, i32, i32]
        L.orc_last_list_builds.restype = i64
        L.orc_lj_loss_grad.restype = dbl
        L.orc_lj_loss_grad.argtypes = [i64] + [vp] * 7 + [vp] + [vp] * 4 + [dbl, dbl, vp]
        L.orc_ej_forces.restype = None
        L.orc_ej_forces.argtypes = [i64] + [vp] * 7 + [vp, dbl] + [vp] * 6
        L.orc_sc_forces.restype = None
        L.orc_sc_forces.argtypes = [i64] + [vp] * 7 + [vp, dbl] + [vp] * 6
        for f in ("orc_ej_phi", "orc_ej_rho", "orc_ej_embed", "orc_sc_phi", "orc_sc_rho", "orc_sc_embed"):
            getattr(L, f).restype = None
            getattr(L, f).argtypes = [vp, dbl, vp, vp]
        L.orc_num_threads.restype = i32
        L.orc_eam_loss_grad.restype = dbl
        L.orc_eam_loss_grad.argtypes = [i64, vp, vp, vp, vp, vp, vp, vp, vp, dbl, vp, vp, vp, dbl, dbl, vp, vp, vp]
    return _lib


def _p(a):
    if a is None:
        return None
    assert a.flags.c_contiguous, "oracle arrays must be C-contiguous"
    return a.ctypes.data


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def num_threads() -> int:
    return int(lib().orc_num_threads())


def grid_dims(lo, hi, R):
    nc = np.zeros(3, dtype=np.int32)
    rc = lib().orc_grid_dims(_p(_f64(lo)), _p(_f64(hi)), float(R), _p(nc))
    if rc != 0:
        raise ValueError("box too small for neighbour radius %g" % R)
    return nc


def wrap(x, y, z, lo, hi):
    lo, hi = _f64(lo), _f64(hi)
    return int(lib().orc_wrap(len(x), _p(x), _p(y), _p(z), _p(lo), _p(hi)))


class NeighborList:
    """CSR full neighbour list (offsets, j, image shift) in canonical order."""

    def __init__(self, off, nbr, img):
        self.off, self.nbr, self.img = off, nbr, img

    @property
    def npairs(self):
        return int(self.off[-1])

    def pairs_with_ids(self, ids):
        """(id_i, id_j, nx, ny, nz) rows in list order."""
        n = len(self.off) - 1
        counts = np.diff(self.off)
        ii = np.repeat(np.arange(n), counts)
        return np.column_stack([ids[ii].astype(np.int64), ids[self.nbr].astype(np.int64),
                                self.img.astype(np.int64)])


def build_neighbors(x, y, z, ids, lo, hi, R) -> NeighborList:
    n = len(x)
    lo, hi = _f64(lo), _f64(hi)
    ids = np.ascontiguousarray(ids, dtype=np.uint64)
    off = np.zeros(n + 1, dtype=np.int64)
    tot = lib().orc_build_neighbors(n, _p(x), _p(y), _p(z), _p(ids), _p(lo), _p(hi), float(R),
                                    _p(off), 0, None, None)
    if tot < 0:
        raise ValueError("neighbour build failed (box thinner than radius?)")
    nbr = np.zeros(max(tot, 1), dtype=np.int32)
    img = np.zeros((max(tot, 1), 3), dtype=np.int8)
    tot2 = lib().orc_build_neighbors(n, _p(x), _p(y), _p(z), _p(ids), _p(lo), _p(hi), float(R),
                                     _p(off), tot, _p(nbr), _p(img))
    assert tot2 == tot
    return NeighborList(off, nbr[:tot], img[:tot])


def build_neighbors_first(x, y, z, ids, lo, hi, R, nlist) -> NeighborList:
    """The lists of the first nlist atoms only (neighbours among all atoms):
    a bounded sample of a large system's pair set."""
    n = len(x)
    lo, hi = _f64(lo), _f64(hi)
    ids = np.ascontiguousarray(ids, dtype=np.uint64)
    off = np.zeros(nlist + 1, dtype=np.int64)
    tot = lib().orc_build_neighbors_first(n, nlist, _p(x), _p(y), _p(z), _p(ids), _p(lo), _p(hi), float(R),
                                          _p(off), 0, None, None)
    if tot < 0:
        raise ValueError("neighbour build failed (box thinner than radius?)")
    nbr = np.zeros(max(tot, 1), dtype=np.int32)
    img = np.zeros((max(tot, 1), 3), dtype=np.int8)
    tot2 = lib().orc_build_neighbors_first(n, nlist, _p(x), _p(y), _p(z), _p(ids), _p(lo), _p(hi), float(R),
                                           _p(off), tot, _p(nbr), _p(img))
    assert tot2 == tot
    return NeighborList(off, nbr[:tot], img[:tot])


def brute_pairs(x, y, z, lo, hi, R):
    n = len(x)
    lo, hi = _f64(lo), _f64(hi)
    cnt = lib().orc_brute_pairs(n, _p(x), _p(y), _p(z), _p(lo), _p(hi), float(R), 0, None, None, None)
    pi = np.zeros(max(cnt, 1), np.int32)
    pj = np.zeros(max(cnt, 1), np.int32)
    img = np.zeros((max(cnt, 1), 3), np.int8)
    lib().orc_brute_pairs(n, _p(x), _p(y), _p(z), _p(lo), _p(hi), float(R), cnt, _p(pi), _p(pj), _p(img))
    return pi[:cnt], pj[:cnt], img[:cnt]


def lj_pair(eps, sigma, r):
    e, de = C.c_double(), C.c_double()
    lib().orc_lj_pair(float(eps), float(sigma), float(r), C.addressof(e), C.addressof(de))
    return e.value, de.value


def lj_energy_cut(eps, sigma, rcut):
    return float(lib().orc_lj_energy_cut(float(eps), float(sigma), float(rcut)))


def lj_atom_buffer(eps, sigma, ecut, drx, dry, drz, d2):
    """One atom of lj_compute_force over its pair buffer (in-cutoff pairs):
    {ep, fx, fy, fz, vir[9]} (force_op_impl2.hxx L22-78)."""
    arrs = [_f64(a) for a in (drx, dry, drz, d2)]
    out = np.zeros(13)
    lib().orc_lj_atom_buffer(float(eps), float(sigma), float(ecut), len(arrs[0]), *[_p(a) for a in arrs], _p(out))
    return out


def _outs(n, vir):
    fx, fy, fz, ep = (np.zeros(n) for _ in range(4))
    v = np.zeros((n, 9)) if vir else None
    return fx, fy, fz, ep, v


def lj_force(x, y, z, nl, L, eps, sigma, rcut, virial=True):
    n = len(nl.off) - 1
    fx, fy, fz, ep, v = _outs(n, virial)
    prm = LJParams(eps, sigma, rcut)
    lib().orc_lj_force(n, _p(x), _p(y), _p(z), _p(nl.off), _p(nl.nbr), _p(nl.img), _p(_f64(L)),
                       C.addressof(prm), _p(fx), _p(fy), _p(fz), _p(ep), _p(v))
    return fx, fy, fz, ep, v


class _Multi:
    def __init__(self, eps, sig, rc, rcut_max):
        self.eps, self.sig, self.rc = _f64(eps), _f64(sig), _f64(rc)
        self.s = LJMultiParams(self.eps.shape[0], 0, _p(self.eps), _p(self.sig), _p(self.rc),
                               float(rcut_max))


def lj_loss_grad(x, y, z, nl, L, eps, sigma, rcut, ft, et, wF, wE):
    """lj_compute_force force-matching + energy loss and its gradient with
    respect to (epsilon, sigma); ft (n, 3) target forces, et (n,) energies."""
    n = len(x)
    prm = LJParams(eps, sigma, rcut)
    ft = np.ascontiguousarray(ft, dtype=np.float64)
    fx, fy, fz = (np.ascontiguousarray(ft[:, d]) for d in range(3))
    g = np.zeros(2)
    loss = lib().orc_lj_loss_grad(n, _p(x), _p(y), _p(z), _p(nl.off), _p(nl.nbr), _p(nl.img), _p(_f64(L)),
                                  C.addressof(prm), _p(fx), _p(fy), _p(fz), _p(_f64(et)), float(wF), float(wE),
                                  _p(g))
    return loss, g


def ej_function(name, pot, arg):
    """(value, derivative) of orc_ej_phi / orc_ej_rho / orc_ej_embed."""
    a, b = C.c_double(), C.c_double()
    getattr(lib(), "orc_ej_" + name)(C.addressof(pot.pot.p), float(arg), C.addressof(a), C.addressof(b))
    return a.value, b.value


def ej_forces(x, y, z, nl, L, pot, virial=True):
    """johnson_force, both passes: returns (fx, fy, fz, ep, vir, F')."""
    n = len(x)
    fx, fy, fz, ep, v = _outs(n, virial)
    fp = np.zeros(n)
    lib().orc_ej_forces(n, _p(x), _p(y), _p(z), _p(nl.off), _p(nl.nbr), _p(nl.img), _p(_f64(L)),
                        C.addressof(pot.pot.p), pot.pot.rcut, _p(fp), _p(fx), _p(fy), _p(fz), _p(ep), _p(v))
    return fx, fy, fz, ep, v, fp


def sc_function(name, pot, arg):
    """(value, derivative) of orc_sc_phi / orc_sc_rho / orc_sc_embed."""
    a, b = C.c_double(), C.c_double()
    getattr(lib(), "orc_sc_" + name)(C.addressof(pot.pot.p), float(arg), C.addressof(a), C.addressof(b))
    return a.value, b.value


def sc_forces(x, y, z, nl, L, pot, virial=True):
    """sutton_chen_force, both passes: returns (fx, fy, fz, ep, vir, F')."""
    n = len(x)
    fx, fy, fz, ep, v = _outs(n, virial)
    fp = np.zeros(n)
    lib().orc_sc_forces(n, _p(x), _p(y), _p(z), _p(nl.off), _p(nl.nbr), _p(nl.img), _p(_f64(L)),
                        C.addressof(pot.pot.p), pot.pot.rcut, _p(fp), _p(fx), _p(fy), _p(fz), _p(ep), _p(v))
    return fx, fy, fz, ep, v, fp


def lj_multi_force(x, y, z, types, nl, L, eps, sig, rc, rcut_max, virial=True):
    """Forces of the atoms the list covers: all of them, or the first
    len(nl.off) - 1 for a build_neighbors_first list."""
    n = len(nl.off) - 1
    m = _Multi(eps, sig, rc, rcut_max)
    fx, fy, fz, ep, v = _outs(n, virial)
    types = np.ascontiguousarray(types, dtype=np.uint8)
    lib().orc_lj_multi_force(n, _p(x), _p(y), _p(z), _p(types), _p(nl.off), _p(nl.nbr), _p(nl.img),
                             _p(_f64(L)), C.addressof(m.s), _p(fx), _p(fy), _p(fz), _p(ep), _p(v))
    return fx, fy, fz, ep, v


def lj_direct(x, y, z, lo, hi, eps, sigma, rcut):
    n = len(x)
    fx, fy, fz = np.zeros(n), np.zeros(n), np.zeros(n)
    prm = LJParams(eps, sigma, rcut)
    e = lib().orc_lj_direct(n, _p(x), _p(y), _p(z), _p(_f64(lo)), _p(_f64(hi)), C.addressof(prm),
                            _p(fx), _p(fy), _p(fz))
    return float(e), fx, fy, fz


def eam_spline(f, delta):
    """f indexed 1..n (f[0] ignored) -> (n+1, 8) coefficient array."""
    f = _f64(f)
    n = len(f) - 1
    out = np.zeros((n + 1, 8))
    lib().orc_eam_spline(n, float(delta), _p(f), _p(out))
    return out


class EamOracleTables:
    """Holds flattened spline arrays alive and exposes the C struct."""

    def __init__(self, frho, rhor, z2r, nr, nrho, dr, drho, conv_z2r, conv_frho, rcut):
        self.frho, self.rhor, self.z2r = _f64(frho), _f64(rhor), _f64(z2r)
        nel = self.frho.shape[0]
        self.pot = EamPot(EamTables(nel, nr, nrho, 0, 1.0 / dr, 1.0 / drho, (nrho - 1) * drho,
                                    conv_z2r, conv_frho, _p(self.frho), _p(self.rhor), _p(self.z2r)),
                          float(rcut))

    @property
    def tp(self):
        return C.addressof(self.pot.t)

    @classmethod
    def from_setfl(cls, sf, conv_z2r, conv_frho, rcut=None):
        """sf: exastamp_gb300.setfl.Setfl (raw tabulated values)."""
        frho = np.stack([eam_spline(np.concatenate([[0.0], t]), sf.drho) for t in sf.frho])
        rhor = np.stack([eam_spline(np.concatenate([[0.0], t]), sf.dr) for t in sf.rhor])
        z2r = np.stack([eam_spline(np.concatenate([[0.0], t]), sf.dr) for t in sf.z2r])
        return cls(frho, rhor, z2r, sf.nr, sf.nrho, sf.dr, sf.drho, conv_z2r, conv_frho,
                   sf.rcut if rcut is None else rcut)


def eam_rho(tab, r, itype=0, jtype=0):
    return float(lib().orc_eam_rho(tab.tp, float(r), itype, jtype))


def eam_embed_one(tab, rho, itype=0):
    phi, fp = C.c_double(), C.c_double()
    lib().orc_eam_embed_one(tab.tp, float(rho), itype, C.addressof(phi), C.addressof(fp))
    return phi.value, fp.value


def eam_pair_force(tab, r, fpi, fpj, itype=0, jtype=0):
    fpair, phi = C.c_double(), C.c_double()
    lib().orc_eam_pair_force(tab.tp, float(r), float(fpi), float(fpj), itype, jtype,
                             C.addressof(fpair), C.addressof(phi))
    return fpair.value, phi.value


def eam_forces(x, y, z, types, nl, L, tab, rcut, virial=True, energy=True):
    """All three EAM passes: returns (fx, fy, fz, ep, vir, fp)."""
    n = len(x)
    types = np.ascontiguousarray(types, dtype=np.uint8)
    rho = np.zeros(n)
    Lp = _f64(L)
    lib().orc_eam_density(n, _p(x), _p(y), _p(z), _p(types), _p(nl.off), _p(nl.nbr), _p(nl.img), _p(Lp),
                          tab.tp, float(rcut), _p(rho))
    rho_copy = rho.copy()
    ep = np.zeros(n)
    lib().orc_eam_embed(n, _p(types), tab.tp, _p(rho), _p(ep) if energy else None)
    fx, fy, fz = np.zeros(n), np.zeros(n), np.zeros(n)
    v = np.zeros((n, 9)) if virial else None
    lib().orc_eam_force(n, _p(x), _p(y), _p(z), _p(types), _p(nl.off), _p(nl.nbr), _p(nl.img), _p(Lp),
                        tab.tp, float(rcut), _p(rho), _p(fx), _p(fy), _p(fz),
                        _p(ep) if energy else None, _p(v))
    return fx, fy, fz, ep, v, rho, rho_copy


def push_f_v_r(x, y, z, vx, vy, vz, ax, ay, az, dt, dt_scale=1.0):
    lib().orc_push_f_v_r(len(x), _p(x), _p(y), _p(z), _p(vx), _p(vy), _p(vz), _p(ax), _p(ay), _p(az),
                         float(dt), float(dt_scale))


def push_f_v(vx, vy, vz, ax, ay, az, dt, dt_scale=0.5):
    lib().orc_push_f_v(len(vx), _p(vx), _p(vy), _p(vz), _p(ax), _p(ay), _p(az), float(dt), float(dt_scale))


def push_min(x, y, z, ax, ay, az, dt, dt_scale=1.0, tolF=0.0):
    lib().orc_push_min(len(x), _p(x), _p(y), _p(z), _p(ax), _p(ay), _p(az), None, None, float(dt),
                       float(dt_scale), float(tolF))


def force_to_accel(fx, fy, fz, types, masses):
    types = np.ascontiguousarray(types, dtype=np.uint8)
    lib().orc_force_to_accel(len(fx), _p(fx), _p(fy), _p(fz), _p(types), _p(_f64(masses)))


def thermo(vx, vy, vz, ep, vir, types, masses):
    out = np.zeros(27)
    types = np.ascontiguousarray(types, dtype=np.uint8)
    lib().orc_thermo(len(vx), _p(vx), _p(vy), _p(vz), _p(ep), _p(vir), _p(types), _p(_f64(masses)),
                     _p(out))
    return out


def run_nve(state, masses, lo, hi, pot_kind, pot, skin, dt, nsteps, rebuild_every, thermo=True,
            initial_forces=True):
    """Run the verlet_nve graph in place on `state` (dict of numpy arrays).

    pot: LJParams / _Multi / EamOracleTables (its .pot is used).
    initial_forces=False: continue from the state's ax, ay, az (orc_run_nve_from)."""
    n = len(state["x"])
    th = np.zeros((nsteps + 1, 27)) if thermo else None
    if pot_kind == POT_LJ:
        pp = C.addressof(pot)
    elif pot_kind == POT_LJ_MULTI:
        pp = C.addressof(pot.s)
    else:
        pp = C.addressof(pot.pot)
    s = state
    run = lib().orc_run_nve if initial_forces else lib().orc_run_nve_from
    rc = run(n, _p(s["x"]), _p(s["y"]), _p(s["z"]), _p(s["vx"]), _p(s["vy"]), _p(s["vz"]),
             _p(s["ax"]), _p(s["ay"]), _p(s["az"]), _p(s["ep"]), _p(s["type"]), _p(s["id"]),
             _p(_f64(masses)), _p(_f64(lo)), _p(_f64(hi)), pot_kind, pp, float(skin),
             float(dt), int(nsteps), int(rebuild_every), _p(th))
    if rc != 0:
        raise RuntimeError("oracle run_nve failed with code %d" % rc)
    return th


def _pot_ptr(pot_kind, pot):
    if pot_kind == POT_LJ:
        return C.addressof(pot)
    if pot_kind == POT_LJ_MULTI:
        return C.addressof(pot.s)
    return C.addressof(pot.pot)


def run_minimize(state, masses, lo, hi, pot_kind, pot, skin, dt, tolF, nsteps, rebuild_every):
    """Clipped minimiser (forces, r += a*dt^2/2, rebuild every
    `rebuild_every`) in place on `state`."""
    n = len(state["x"])
    s = state
    rc = lib().orc_run_minimize(n, _p(s["x"]), _p(s["y"]), _p(s["z"]), _p(s["ax"]), _p(s["ay"]), _p(s["az"]),
                                _p(s["ep"]), _p(s["type"]), _p(s["id"]), _p(_f64(masses)), _p(_f64(lo)),
                                _p(_f64(hi)), pot_kind, _pot_ptr(pot_kind, pot), float(skin), float(dt),
                                float(tolF), int(nsteps), int(rebuild_every))
    if rc != 0:
        raise RuntimeError("oracle run_minimize failed with code %d" % rc)


def last_list_builds():
    """List builds of the last run_nve / run_minimize (initial build included)."""
    return int(lib().orc_last_list_builds())


def multi_params(eps, sig, rc, rcut_max):
    return _Multi(eps, sig, rc, rcut_max)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))


# --------------------------------------------------------------------------
# parameter adjoint (single-element analytic EAM, eV units)
# --------------------------------------------------------------------------
class EamDTables(C.Structure):
    _fields_ = [("nparam", C.c_int), ("pad_", C.c_int), ("dfrho", C.c_void_p), ("drhor", C.c_void_p),
                ("dz2r", C.c_void_p)]


class EamDerivativeSplines:
    """Splines of d(knot values)/d(parameter) for every analytic parameter;
    the spline map is linear, so these are d(spline coefficients)/d(param)."""

    def __init__(self, cfg, params=None):
        from exastamp_gb300 import setfl as SF
        J_F, J_f, J_z = SF.table_param_jacobian(cfg, params)
        _, _, dr, drho = SF.table_grids(cfg)
        pad = lambda row: np.concatenate([[0.0], row])  # noqa: E731
        self.dfrho = np.ascontiguousarray(np.stack([eam_spline(pad(r), drho) for r in J_F]))
        self.drhor = np.ascontiguousarray(np.stack([eam_spline(pad(r), dr) for r in J_f]))
        self.dz2r = np.ascontiguousarray(np.stack([eam_spline(pad(r), dr) for r in J_z]))
        self.s = EamDTables(J_F.shape[0], 0, _p(self.dfrho), _p(self.drhor), _p(self.dz2r))


def eam_loss_grad(x, y, z, nl, L, tab, rcut, dsp, Ft, Et, wF, wE):
    """(loss, grad[9], F (n,3), E (n)) for one configuration."""
    n = len(x)
    grad = np.zeros(dsp.s.nparam)
    F = np.zeros((n, 3))
    E = np.zeros(n)
    Ft = np.ascontiguousarray(Ft, np.float64).reshape(n, 3)
    Et = np.ascontiguousarray(Et, np.float64)
    loss = lib().orc_eam_loss_grad(n, _p(x), _p(y), _p(z), _p(nl.off), _p(nl.nbr), _p(nl.img), _p(_f64(L)),
                                   tab.tp, float(rcut), C.addressof(dsp.s), _p(Ft), _p(Et), float(wF), float(wE),
                                   _p(grad), _p(F), _p(E))
    return float(loss), grad, F, E
