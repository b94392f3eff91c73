"""ctypes binding of oracle/_ref/libref.so, the reference's own per-pair code
compiled from the exaStamp sources by oracle/ref_pin/build_ref.py (test
infrastructure; absent where the exaStamp sources are not readable)."""
import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle", "ref_pin"))
import build_ref  # noqa: E402

_lib = None


def load():
    """The pin library, built if the exaStamp sources are readable; None otherwise."""
    global _lib
    if _lib is not None:
        return _lib
    path = build_ref.build()
    if not path:
        return None
    L = C.CDLL(path)
    vp, dbl, i32, i64 = C.c_void_p, C.c_double, C.c_int, C.c_int64
    L.ref_lj_compute_energy.argtypes = [dbl, dbl, dbl, vp, vp]
    L.ref_lj_force_atom.argtypes = [dbl, dbl, dbl, i32, vp, vp, vp, vp, vp]
    L.ref_eam_load.restype = i32
    L.ref_eam_load.argtypes = [C.c_char_p, vp, vp]
    L.ref_eam_spline.restype = i64
    L.ref_eam_spline.argtypes = [i32, vp]
    L.ref_eam_conversions.argtypes = [vp, vp]
    L.ref_eam_rho.restype = dbl
    L.ref_eam_rho.argtypes = [dbl, i32, i32]
    L.ref_eam_mm_force.argtypes = [dbl, dbl, dbl, i32, i32, vp, vp]
    L.ref_eam_fembed.argtypes = [dbl, i32, vp, vp]
    _lib = L
    return L


def exastamp_file(*parts):
    """A file of the exaStamp tree the pin library was built from."""
    return os.path.join(build_ref.reference_root(), *parts)


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def lj_pair(L, eps, sig, r):
    e, de = C.c_double(), C.c_double()
    L.ref_lj_compute_energy(eps, sig, r, C.byref(e), C.byref(de))
    return e.value, de.value


def lj_force_atom(L, eps, sig, ecut, drx, dry, drz, d2):
    out = np.zeros(13)
    arrs = [np.ascontiguousarray(a, np.float64) for a in (drx, dry, drz, d2)]
    L.ref_lj_force_atom(eps, sig, ecut, len(arrs[0]), *[_p(a) for a in arrs], _p(out))
    return out


def eam_load(L, path):
    nr, nrho = C.c_int(), C.c_int()
    nel = L.ref_eam_load(path.encode(), C.byref(nr), C.byref(nrho))
    if nel <= 0:
        raise RuntimeError("reference setfl reader failed on %s" % path)
    return nel, nr.value, nrho.value


def eam_spline(L, which):
    k = L.ref_eam_spline(which, None)
    out = np.zeros(8 * k)
    L.ref_eam_spline(which, _p(out))
    return out


def eam_conversions(L):
    a, b = C.c_double(), C.c_double()
    L.ref_eam_conversions(C.byref(a), C.byref(b))
    return a.value, b.value


def eam_mm_force(L, r, fpi, fpj, it, jt, dr):
    v = np.ascontiguousarray(dr, np.float64).copy()
    phi = C.c_double()
    L.ref_eam_mm_force(r, fpi, fpj, it, jt, _p(v), C.byref(phi))
    return v, phi.value


def eam_fembed(L, rho, it):
    phi, fp = C.c_double(), C.c_double()
    L.ref_eam_fembed(rho, it, C.byref(phi), C.byref(fp))
    return phi.value, fp.value
