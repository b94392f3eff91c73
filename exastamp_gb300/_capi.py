"""ctypes binding of libgbmd.so (include/gbmd.h).

There is no fallback: if the library is missing or no GPU is present, the
calls raise.  `Context` is a thin RAII wrapper that turns status codes into
exceptions and numpy arrays into pointers.
"""
from __future__ import annotations

import ctypes as C
import os
import re

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB_PATH = os.path.join(PKG, "libgbmd.so")
HEADER = os.path.join(ROOT, "include", "gbmd.h")

OK = 0
REBUILD_ON_DISPLACEMENT = -1  # rebuild_every value of the displacement trigger
ERR_NAMES = {1: "INVALID", 2: "CUDA", 3: "NO_DEVICE", 4: "NEIGHBOR_OVERFLOW", 5: "LOST_ATOM",
             6: "NONFINITE", 7: "IO", 8: "UNSUPPORTED", 9: "TOO_LARGE"}
PRECISION_FP64, PRECISION_MIXED = 0, 1
POT_NONE, POT_LJ, POT_LJ_MULTI, POT_EAM_ALLOY = 0, 1, 2, 3
FORCE_ENERGY, FORCE_VIRIAL = 1, 2
FORCE_PASS_DENSITY, FORCE_PASS_FORCE = 4, 8  # split EAM passes (eam_rho + eam_rho2emb / eam_force)


class GbmdError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("gbmd error %d (%s): %s" % (code, ERR_NAMES.get(code, "?"), msg))
        self.code = code


def declared_symbols(header: str = HEADER):
    """Function names declared in include/gbmd.h."""
    txt = open(header).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gbmd_[a-z0-9_]+)\s*\(", txt)))


_lib = None


def lib(path: str = LIB_PATH):
    """Load libgbmd.so (raises OSError if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise OSError("libgbmd.so not built (run __graft_entry__.build())")
        L = C.CDLL(path)
        vp, i64, i32, dbl = C.c_void_p, C.c_int64, C.c_int, C.c_double
        P = C.POINTER
        sig = {
            "gbmd_abi_version": ([], i32),
            "gbmd_last_error": ([vp], C.c_char_p),
            "gbmd_create": ([P(vp), i32, vp], i32),
            "gbmd_destroy": ([vp], i32),
            "gbmd_synchronize": ([vp], i32),
            "gbmd_set_box": ([vp, vp, vp, vp], i32),
            "gbmd_set_species": ([vp, i32, vp], i32),
            "gbmd_upload_atoms": ([vp, i64, vp, vp, vp, vp, vp, vp, vp, vp], i32),
            "gbmd_upload_positions": ([vp, vp, vp, vp, vp, vp, vp], i32),
            "gbmd_upload_state": ([vp] + [vp] * 9, i32),
            "gbmd_download": ([vp] + [vp] * 11, i32),
            "gbmd_profile_step": ([vp, i32, vp], i32),
            "gbmd_num_atoms": ([vp, P(i64)], i32),
            "gbmd_set_lj": ([vp, dbl, dbl, dbl], i32),
            "gbmd_set_lj_multi": ([vp, i32, vp, vp, vp, dbl], i32),
            "gbmd_set_eam_alloy": ([vp, i32, i32, dbl, i32, dbl, vp, vp, vp, dbl, dbl, dbl], i32),
            "gbmd_load_setfl": ([vp, C.c_char_p, dbl, dbl, dbl], i32),
            "gbmd_set_precision": ([vp, i32], i32),
            "gbmd_set_launch": ([vp, i32, i32], i32),
            "gbmd_get_launch": ([vp, P(i32), P(i32)], i32),
            "gbmd_set_launch_ex": ([vp, i32, i32, i32], i32),
            "gbmd_set_neighbor_staging": ([vp, i32], i32),
            "gbmd_set_newton3": ([vp, i32], i32),
            "gbmd_check_errors": ([vp], i32),
            "gbmd_get_newton3": ([vp, P(i32)], i32),
            "gbmd_set_density_block": ([vp, i32], i32),
            "gbmd_get_density_block": ([vp, P(i32)], i32),
            "gbmd_get_neighbor_staging": ([vp, P(i32)], i32),
            "gbmd_get_launch_ex": ([vp, P(i32), P(i32), P(i32)], i32),
            "gbmd_set_skin": ([vp, dbl], i32),
            "gbmd_set_list_buffer": ([vp, dbl], i32),
            "gbmd_get_list_buffer": ([vp, P(dbl), P(i64)], i32),
            "gbmd_build_neighbors": ([vp], i32),
            "gbmd_update_neighbors": ([vp, P(i32)], i32),
            "gbmd_export_pairs": ([vp, i64, vp, vp, vp, P(i64)], i32),
            "gbmd_neighbor_stats": ([vp, P(i64), P(i32), vp], i32),
            "gbmd_compute_forces": ([vp, i32], i32),
            "gbmd_push_f_v_r": ([vp, dbl, dbl], i32),
            "gbmd_push_f_v": ([vp, dbl, dbl], i32),
            "gbmd_push_min": ([vp, dbl, dbl, dbl], i32),
            "gbmd_run_nve": ([vp, i32, dbl, i32, i32, vp, i32], i32),
            "gbmd_run_nve_host": ([vp, i32, dbl, i32] + [vp] * 9, i32),
            "gbmd_run_minimize": ([vp, i32, dbl, dbl, i32], i32),
            "gbmd_set_eam_johnson": ([vp, vp, dbl], i32),
            "gbmd_set_eam_sutton_chen": ([vp, vp, dbl], i32),
            "gbmd_lj_loss_grad": ([vp, vp, vp, vp, vp, dbl, dbl, P(dbl), vp], i32),
            "gbmd_lj_multi_loss_grad": ([vp, vp, vp, vp, vp, dbl, dbl, P(dbl), vp, vp], i32),
            "gbmd_list_builds": ([vp, P(i64)], i32),
            "gbmd_set_host_pipeline": ([vp, i32], i32),
            "gbmd_set_host_pipeline_link": ([vp, i32, i32, i32], i32),
            "gbmd_set_host_pipeline_trace": ([vp, i32], i32),
            "gbmd_get_host_pipeline_trace": ([vp, i32, vp, vp, vp, P(i32)], i32),
            "gbmd_get_host_pipeline": ([vp, P(i32), P(i64), P(i64)], i32),
            "gbmd_thermo": ([vp, vp], i32),
            "gbmd_device_state": ([vp] + [vp] * 11, i32),
            "gbmd_thermo_reduce_noalloc": ([i64, vp, vp, vp, vp, vp, vp, vp, i32, vp, vp], i32),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _p(a):
    if a is None:
        return None
    if not a.flags.c_contiguous:
        raise ValueError("arrays must be C-contiguous")
    return a.ctypes.data


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


class Context:
    """One device context of the hot path (see include/gbmd.h)."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self._L = lib()
        h = C.c_void_p()
        rc = self._L.gbmd_create(C.byref(h), device, stream)
        if rc != OK:
            raise GbmdError(rc, "gbmd_create failed")
        self.h = h

    # -- plumbing --------------------------------------------------------
    def _chk(self, rc):
        if rc != OK:
            raise GbmdError(rc, self._L.gbmd_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self._L.gbmd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- set-up -----------------------------------------------------------
    def set_box(self, lo, hi):
        lo, hi = _f64(lo), _f64(hi)
        per = np.ones(3, dtype=np.int32)
        self._chk(self._L.gbmd_set_box(self.h, _p(lo), _p(hi), _p(per)))

    def set_species(self, masses):
        m = _f64(masses)
        self._chk(self._L.gbmd_set_species(self.h, len(m), _p(m)))

    def upload(self, x, y, z, vx=None, vy=None, vz=None, types=None, ids=None):
        x, y, z, vx, vy, vz = (_f64(a) for a in (x, y, z, vx, vy, vz))
        t = None if types is None else np.ascontiguousarray(types, np.uint8)
        i = None if ids is None else np.ascontiguousarray(ids, np.uint64)
        self._keep = (x, y, z, vx, vy, vz, t, i)
        self._chk(self._L.gbmd_upload_atoms(self.h, len(x), _p(x), _p(y), _p(z), _p(vx), _p(vy), _p(vz),
                                            _p(t), _p(i)))

    def upload_system(self, s):
        self.set_box(s.lo, s.hi)
        self.set_species(s.masses)
        self.upload(s.x, s.y, s.z, s.vx, s.vy, s.vz, s.type, s.id)

    def upload_positions(self, x, y, z, vx=None, vy=None, vz=None):
        x, y, z, vx, vy, vz = (_f64(a) for a in (x, y, z, vx, vy, vz))
        self._chk(self._L.gbmd_upload_positions(self.h, _p(x), _p(y), _p(z), _p(vx), _p(vy), _p(vz)))

    def upload_state(self, x, y, z, vx, vy, vz, ax, ay, az):
        arrs = [_f64(a) for a in (x, y, z, vx, vy, vz, ax, ay, az)]
        self._chk(self._L.gbmd_upload_state(self.h, *[_p(a) for a in arrs]))

    def profile_step(self, reps=10):
        ms = np.zeros(5)
        self._chk(self._L.gbmd_profile_step(self.h, int(reps), _p(ms)))
        return dict(zip(("rebuild", "density", "pair", "first_half", "thermo"), ms.tolist()))

    @property
    def n(self) -> int:
        v = C.c_int64()
        self._chk(self._L.gbmd_num_atoms(self.h, C.byref(v)))
        return v.value

    def download(self, fields=("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "ep"), virial=False):
        n = self.n
        names = ["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "ep"]
        out = {k: np.empty(n) for k in names if k in fields}
        vir = np.empty((n, 9)) if virial else None
        self._chk(self._L.gbmd_download(self.h, *[_p(out.get(k)) for k in names], _p(vir)))
        if virial:
            out["vir"] = vir
        return out

    def set_lj(self, epsilon, sigma, rcut):
        self._chk(self._L.gbmd_set_lj(self.h, float(epsilon), float(sigma), float(rcut)))

    def set_lj_multi(self, eps, sig, rc, rcut_common=0.0):
        eps, sig, rc = _f64(eps), _f64(sig), _f64(rc)
        self._chk(self._L.gbmd_set_lj_multi(self.h, eps.shape[0], _p(eps), _p(sig), _p(rc), float(rcut_common)))
        self._lj_ntypes = int(eps.shape[0])

    def set_eam_alloy(self, sf, rcut, conv_z2r, conv_frho):
        frho = np.ascontiguousarray(np.stack(sf.frho), np.float64)
        rhor = np.ascontiguousarray(np.stack(sf.rhor), np.float64)
        z2r = np.ascontiguousarray(np.stack(sf.z2r), np.float64)
        self._chk(self._L.gbmd_set_eam_alloy(self.h, sf.nelements, sf.nrho, sf.drho, sf.nr, sf.dr, _p(frho),
                                             _p(rhor), _p(z2r), float(rcut), float(conv_z2r), float(conv_frho)))

    def load_setfl(self, path, rcut, conv_z2r, conv_frho):
        self._chk(self._L.gbmd_load_setfl(self.h, path.encode(), float(rcut), float(conv_z2r), float(conv_frho)))

    def set_precision(self, mixed: bool):
        self._chk(self._L.gbmd_set_precision(self.h, PRECISION_MIXED if mixed else PRECISION_FP64))

    def set_launch(self, lanes_per_atom, block, entries_per_load=1):
        self._chk(self._L.gbmd_set_launch_ex(self.h, int(lanes_per_atom), int(entries_per_load), int(block)))

    def get_launch(self):
        """(lanes per atom, threads per block)."""
        t, b = C.c_int(), C.c_int()
        self._chk(self._L.gbmd_get_launch(self.h, C.byref(t), C.byref(b)))
        return t.value, b.value

    def set_density_block(self, block):
        """Threads per block of the EAM density kernels (0 = the pair kernels')."""
        self._chk(self._L.gbmd_set_density_block(self.h, int(block)))

    def get_density_block(self):
        b = C.c_int()
        self._chk(self._L.gbmd_get_density_block(self.h, C.byref(b)))
        return b.value

    def set_neighbor_staging(self, enable):
        self._chk(self._L.gbmd_set_neighbor_staging(self.h, 1 if enable else 0))

    def get_neighbor_staging(self):
        e = C.c_int()
        self._chk(self._L.gbmd_get_neighbor_staging(self.h, C.byref(e)))
        return bool(e.value)

    def check_errors(self):
        """Wait for the stream and raise on the device error word
        (gbmd_check_errors)."""
        self._chk(self._L.gbmd_check_errors(self.h))

    def set_newton3(self, enable):
        """Half list + scattered reaction forces (LJ, mixed precision)."""
        self._chk(self._L.gbmd_set_newton3(self.h, 1 if enable else 0))

    def get_newton3(self):
        e = C.c_int()
        self._chk(self._L.gbmd_get_newton3(self.h, C.byref(e)))
        return bool(e.value)

    def get_launch_ex(self):
        """(lanes per atom, list entries per load, threads per block)."""
        t, v, b = C.c_int(), C.c_int(), C.c_int()
        self._chk(self._L.gbmd_get_launch_ex(self.h, C.byref(t), C.byref(v), C.byref(b)))
        return t.value, v.value, b.value

    def set_skin(self, skin):
        self._chk(self._L.gbmd_set_skin(self.h, float(skin)))

    # -- operators --------------------------------------------------------
    def set_list_buffer(self, buffer):
        """Two-level list: an outer list of radius rcut + skin + buffer, the
        list filtered from it at each rebuild (gbmd_set_list_buffer)."""
        self._chk(self._L.gbmd_set_list_buffer(self.h, float(buffer)))

    def list_buffer(self):
        """(buffer, outer list builds so far)."""
        b = C.c_double()
        k = C.c_int64()
        self._chk(self._L.gbmd_get_list_buffer(self.h, C.byref(b), C.byref(k)))
        return b.value, k.value

    def build_neighbors(self):
        self._chk(self._L.gbmd_build_neighbors(self.h))

    def export_pairs(self):
        cnt = C.c_int64()
        self._chk(self._L.gbmd_export_pairs(self.h, 0, None, None, None, C.byref(cnt)))
        n = cnt.value
        a = np.empty(max(n, 1), np.uint64)
        b = np.empty(max(n, 1), np.uint64)
        img = np.empty((max(n, 1), 3), np.int8)
        self._chk(self._L.gbmd_export_pairs(self.h, n, _p(a), _p(b), _p(img), C.byref(cnt)))
        return np.column_stack([a[:n].astype(np.int64), b[:n].astype(np.int64), img[:n].astype(np.int64)])

    def update_neighbors(self) -> bool:
        """check_and_update_particles: rebuild when some atom moved more than
        skin/2 since the last rebuild; returns whether it rebuilt."""
        r = C.c_int()
        self._chk(self._L.gbmd_update_neighbors(self.h, C.byref(r)))
        return bool(r.value)

    def export_pairs_raw(self):
        """The exported pair set as three arrays (id_i, id_j: uint64; image:
        n x 3 int8), without the int64 stacking of export_pairs (for lists of
        hundreds of millions of pairs)."""
        cnt = C.c_int64()
        self._chk(self._L.gbmd_export_pairs(self.h, 0, None, None, None, C.byref(cnt)))
        n = cnt.value
        a = np.empty(max(n, 1), np.uint64)
        b = np.empty(max(n, 1), np.uint64)
        img = np.empty((max(n, 1), 3), np.int8)
        self._chk(self._L.gbmd_export_pairs(self.h, n, _p(a), _p(b), _p(img), C.byref(cnt)))
        return a[:n], b[:n], img[:n]

    def neighbor_stats(self):
        npairs, maxnb = C.c_int64(), C.c_int()
        nc = np.zeros(3, np.int32)
        self._chk(self._L.gbmd_neighbor_stats(self.h, C.byref(npairs), C.byref(maxnb), _p(nc)))
        return npairs.value, maxnb.value, nc

    def compute_forces(self, energy=True, virial=False, passes="all"):
        """passes: "all", "density" (EAM density + embedding only) or "force"
        (the final pair pass from the kept F'(rho))."""
        flags = (FORCE_ENERGY if energy else 0) | (FORCE_VIRIAL if virial else 0)
        flags |= {"all": 0, "density": FORCE_PASS_DENSITY, "force": FORCE_PASS_FORCE}[passes]
        self._chk(self._L.gbmd_compute_forces(self.h, flags))

    def push_f_v_r(self, dt, dt_scale=1.0):
        self._chk(self._L.gbmd_push_f_v_r(self.h, float(dt), float(dt_scale)))

    def push_f_v(self, dt, dt_scale=0.5):
        self._chk(self._L.gbmd_push_f_v(self.h, float(dt), float(dt_scale)))

    def push_min(self, dt, dt_scale=1.0, tolF=0.0):
        self._chk(self._L.gbmd_push_min(self.h, float(dt), float(dt_scale), float(tolF)))

    def run_nve(self, nsteps, dt, rebuild_every=10, thermo_every=0, use_graph=False):
        rows = (nsteps // thermo_every + 1) if thermo_every > 0 else 0
        out = np.zeros((max(rows, 1), 27))
        self._chk(self._L.gbmd_run_nve(self.h, int(nsteps), float(dt), int(rebuild_every), int(thermo_every),
                                       _p(out) if rows else None, 1 if use_graph else 0))
        return out[:rows] if rows else None

    def run_nve_host(self, state, nsteps, dt, rebuild_every=10):
        """gbmd_run_nve_host on a dict of 9 contiguous float64 arrays (x, y, z,
        vx, vy, vz, ax, ay, az), updated in place."""
        keys = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")
        for k in keys:
            a = state[k]
            if a.dtype != np.float64 or not a.flags.c_contiguous or len(a) != self.n:
                raise ValueError("%s: need a contiguous float64 array of n atoms" % k)
        self._chk(self._L.gbmd_run_nve_host(self.h, int(nsteps), float(dt), int(rebuild_every),
                                            *[state[k].ctypes.data for k in keys]))

    def run_minimize(self, nsteps, dt, tolF=0.0, rebuild_every=10):
        self._chk(self._L.gbmd_run_minimize(self.h, int(nsteps), float(dt), float(tolF), int(rebuild_every)))

    def set_eam_johnson(self, params, rcut):
        """johnson_force: params = 19 values in EamJohnsonParameters order."""
        p = _f64(params)
        if p.shape != (19,):
            raise ValueError("johnson_force takes 19 parameters")
        self._chk(self._L.gbmd_set_eam_johnson(self.h, _p(p), float(rcut)))

    def set_eam_sutton_chen(self, params, rcut):
        """sutton_chen_force: params = (c, epsilon, a0, n, m), EamSuttonChenParameters order."""
        p = _f64(params)
        if p.shape != (5,):
            raise ValueError("sutton_chen_force takes 5 parameters")
        self._chk(self._L.gbmd_set_eam_sutton_chen(self.h, _p(p), float(rcut)))

    def lj_loss_grad(self, f_target, e_target, w_force, w_energy):
        """Force-matching + energy loss of lj_compute_force and its gradient
        with respect to (epsilon, sigma); f_target (n, 3) forces, e_target (n,)
        per-atom energies, both in upload order."""
        ft = np.asarray(f_target, dtype=np.float64)
        fx, fy, fz = (np.ascontiguousarray(ft[:, d]) for d in range(3))
        et = _f64(e_target)
        loss, g = C.c_double(), np.zeros(2)
        self._chk(self._L.gbmd_lj_loss_grad(self.h, _p(fx), _p(fy), _p(fz), _p(et), float(w_force), float(w_energy),
                                            C.byref(loss), _p(g)))
        return loss.value, g

    def lj_multi_loss_grad(self, f_target, e_target, w_force, w_energy):
        """The same loss for lj_multi_force; returns (loss, dL/deps, dL/dsigma)
        with the gradients as symmetric ntypes x ntypes arrays (one parameter
        per unordered species pair)."""
        ft = np.asarray(f_target, dtype=np.float64)
        fx, fy, fz = (np.ascontiguousarray(ft[:, d]) for d in range(3))
        et = _f64(e_target)
        nt = getattr(self, "_lj_ntypes", 0)
        if not nt:
            raise GbmdError(1, "set_lj_multi first")
        loss, ge, gs = C.c_double(), np.zeros((nt, nt)), np.zeros((nt, nt))
        self._chk(self._L.gbmd_lj_multi_loss_grad(self.h, _p(fx), _p(fy), _p(fz), _p(et), float(w_force),
                                                  float(w_energy), C.byref(loss), _p(ge), _p(gs)))
        return loss.value, ge, gs

    def set_host_pipeline(self, slabs):
        """gbmd_set_host_pipeline: -1 automatic, 0 off, 4..64 slabs."""
        self._chk(self._L.gbmd_set_host_pipeline(self.h, int(slabs)))

    def set_host_pipeline_link(self, mode, blocks=40, threads=512):
        """gbmd_set_host_pipeline_link: 0 copy engines, 1 kernels on the page-locked arrays."""
        self._chk(self._L.gbmd_set_host_pipeline_link(self.h, int(mode), int(blocks), int(threads)))

    def set_host_pipeline_trace(self, on):
        self._chk(self._L.gbmd_set_host_pipeline_trace(self.h, 1 if on else 0))

    def host_pipeline_trace(self):
        """Marks of the last pipelined host step: list of (ms, kind, index),
        kind one of start, in, density, force, out, end."""
        cnt = C.c_int(0)
        self._chk(self._L.gbmd_get_host_pipeline_trace(self.h, 0, None, None, None, C.byref(cnt)))
        n = cnt.value
        t, k, i = np.zeros(n), np.zeros(n, np.int32), np.zeros(n, np.int32)
        self._chk(self._L.gbmd_get_host_pipeline_trace(self.h, n, _p(t), _p(k), _p(i), C.byref(cnt)))
        names = ("start", "in", "density", "force", "out", "end")
        return [(float(t[q]), names[k[q]], int(i[q])) for q in range(n)]

    def host_pipeline(self):
        """(slabs the next host step would use, steps that stood as
        pipelined, pipelined steps discarded for an unpredicted rebuild)."""
        sl, st, rd = C.c_int(0), C.c_int64(0), C.c_int64(0)
        self._chk(self._L.gbmd_get_host_pipeline(self.h, C.byref(sl), C.byref(st), C.byref(rd)))
        return sl.value, st.value, rd.value

    def list_builds(self):
        n = C.c_int64(0)
        self._chk(self._L.gbmd_list_builds(self.h, C.byref(n)))
        return n.value

    def thermo(self):
        out = np.zeros(27)
        self._chk(self._L.gbmd_thermo(self.h, _p(out)))
        return out

    def synchronize(self):
        self._chk(self._L.gbmd_synchronize(self.h))


# --------------------------------------------------------------------------
# batched replicas (gbmd_batch_*)
# --------------------------------------------------------------------------
_BATCH_SIG = {
    "gbmd_batch_create": (["P(vp)", "i32", "vp"], "i32"),
    "gbmd_batch_destroy": (["vp"], "i32"),
    "gbmd_batch_last_error": (["vp"], "cp"),
    "gbmd_batch_set_eam_alloy": (["vp", "i32", "dbl", "i32", "dbl", "vp", "vp", "vp", "dbl", "dbl", "dbl"], "i32"),
    "gbmd_batch_set_param_derivatives": (["vp", "i32", "vp", "vp", "vp", "dbl", "dbl"], "i32"),
    "gbmd_batch_upload": (["vp", "i32", "vp", "vp", "vp", "vp", "vp", "vp"], "i32"),
    "gbmd_batch_set_targets": (["vp", "vp", "vp", "vp", "vp", "dbl", "dbl"], "i32"),
    "gbmd_batch_set_launch": (["vp", "i32", "i32"], "i32"),
    "gbmd_batch_set_small_block": (["vp", "i32"], "i32"),
    "gbmd_batch_run": (["vp", "i32", "i32", "i32"], "i32"),
    "gbmd_batch_synchronize": (["vp"], "i32"),
    "gbmd_batch_download": (["vp", "vp", "vp", "vp", "vp", "vp", "vp", "vp", "vp"], "i32"),
}


def _batch_lib():
    L = lib()
    if not getattr(L, "_batch_ready", False):
        T = {"vp": C.c_void_p, "i32": C.c_int, "dbl": C.c_double, "cp": C.c_char_p,
             "P(vp)": C.POINTER(C.c_void_p)}
        for name, (args, res) in _BATCH_SIG.items():
            fn = getattr(L, name)
            fn.argtypes = [T[a] for a in args]
            fn.restype = T[res]
        L._batch_ready = True
    return L


class Batch:
    """Many independent periodic eam_alloy replicas, one persistent launch."""

    def __init__(self, device: int = 0, stream: int | None = None):
        self._L = _batch_lib()
        h = C.c_void_p()
        rc = self._L.gbmd_batch_create(C.byref(h), device, stream)
        if rc != OK:
            raise GbmdError(rc, "gbmd_batch_create failed")
        self.h = h
        self.nrep = 0
        self.n = 0

    def _chk(self, rc):
        if rc != OK:
            raise GbmdError(rc, self._L.gbmd_batch_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self._L.gbmd_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_eam_alloy(self, sf, rcut, conv_z2r=1.0, conv_frho=1.0):
        frho, rhor, z2r = (np.ascontiguousarray(t[0], np.float64) for t in (sf.frho, sf.rhor, sf.z2r))
        self._keep_tab = (frho, rhor, z2r)
        self._chk(self._L.gbmd_batch_set_eam_alloy(self.h, sf.nrho, sf.drho, sf.nr, sf.dr, _p(frho), _p(rhor),
                                                   _p(z2r), float(rcut), float(conv_z2r), float(conv_frho)))

    def set_param_derivatives(self, J_F, J_f, J_z, conv_z2r=1.0, conv_frho=1.0):
        J_F, J_f, J_z = (np.ascontiguousarray(a, np.float64) for a in (J_F, J_f, J_z))
        self._chk(self._L.gbmd_batch_set_param_derivatives(self.h, J_F.shape[0], _p(J_F), _p(J_f), _p(J_z),
                                                           float(conv_z2r), float(conv_frho)))

    def upload(self, systems):
        off = np.zeros(len(systems) + 1, np.int64)
        off[1:] = np.cumsum([s.n for s in systems])
        lo = np.ascontiguousarray(np.stack([s.lo for s in systems]), np.float64)
        hi = np.ascontiguousarray(np.stack([s.hi for s in systems]), np.float64)
        x, y, z = (np.ascontiguousarray(np.concatenate([getattr(s, k) for s in systems]), np.float64)
                   for k in ("x", "y", "z"))
        self._chk(self._L.gbmd_batch_upload(self.h, len(systems), _p(off), _p(lo), _p(hi), _p(x), _p(y), _p(z)))
        self.nrep, self.n, self.offsets = len(systems), int(off[-1]), off

    def set_targets(self, F, E, wF, wE):
        F = np.ascontiguousarray(F, np.float64).reshape(-1, 3)
        fx, fy, fz = (np.ascontiguousarray(F[:, k]) for k in range(3))
        E = np.ascontiguousarray(E, np.float64)
        self._chk(self._L.gbmd_batch_set_targets(self.h, _p(fx), _p(fy), _p(fz), _p(E), float(wF), float(wE)))

    def set_launch(self, block, stencil):
        self._chk(self._L.gbmd_batch_set_launch(self.h, int(block), int(stencil)))

    def set_small_block(self, block):
        """Threads per block of the kernel for replicas of at most 512 atoms."""
        self._chk(self._L.gbmd_batch_set_small_block(self.h, int(block)))

    def run(self, adjoint=False, per_replica=False, use_graph=False):
        self._chk(self._L.gbmd_batch_run(self.h, 1 if adjoint else 0, 1 if per_replica else 0,
                                         1 if use_graph else 0))

    def synchronize(self):
        self._chk(self._L.gbmd_batch_synchronize(self.h))

    def download(self):
        n, r = self.n, self.nrep
        fx, fy, fz, ep = (np.empty(n) for _ in range(4))
        e_rep, vir = np.empty(r), np.empty((r, 9))
        loss, grad = C.c_double(), np.empty(9)
        self._chk(self._L.gbmd_batch_download(self.h, _p(fx), _p(fy), _p(fz), _p(ep), _p(e_rep), _p(vir),
                                              C.addressof(loss), _p(grad)))
        return {"F": np.stack([fx, fy, fz], 1), "ep": ep, "e_rep": e_rep, "vir_rep": vir, "loss": loss.value,
                "grad": grad}
