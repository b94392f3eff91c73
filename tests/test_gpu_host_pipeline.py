"""gbmd_run_nve_host one step at a time with the host link pipelined
(gbmd_set_host_pipeline) against the same steps unpipelined.

The pipelined step reads the caller's page-locked r, v, a in chunks of the
caller order, runs the pair passes slab by slab (whole z layers of the cell
grid) as their neighbourhoods arrive and writes v, a back chunk by chunk;
every atom goes through the same kernels on the same data, so the caller's
arrays after every step must equal the unpipelined step's bit for bit.  The
skin is small enough that the displacement trigger fires every few steps:
those steps are finished after a rebuild without the pipeline, from the
pushed state, and must give the same arrays too.

Caller orders: atoms sorted cell by cell with z slowest (as exaNBody's
grids store them; the schedule overlaps), the generator's lattice order, and
a random permutation (every slab then waits for the last chunk).
"""
import numpy as np
import pytest

from exastamp_gb300 import setfl as SF
from exastamp_gb300 import systems as S

pytestmark = pytest.mark.gpu

KEYS = ("x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az")
NSTEPS = 40


def _reorder(s, order, R, seed):
    n = s.n
    if order == "lattice":
        perm = np.arange(n)
    elif order == "random":
        perm = np.random.default_rng(seed).permutation(n)
    else:
        return S.grid_order(s, R)
    for k in ("x", "y", "z", "vx", "vy", "vz", "type", "id"):
        setattr(s, k, np.ascontiguousarray(getattr(s, k)[perm]))
    return s


def _case(kind):
    """(system, potential setter, rcut, skin, dt, mixed)"""
    if kind == "lj":
        return S.lj_fcc(ncell=8, seed=41), (lambda c: c.set_lj(1.0, 1.0, 2.5)), 2.5, 0.08, 0.005, True
    if kind == "lj_multi_fp64":
        # an 80:20 mixture of two species on the FCC lattice
        s = S.lj_fcc(ncell=8, seed=42)
        s.type = (np.random.default_rng(42).random(s.n) < 0.2).astype(np.uint8)
        s.masses = np.array([1.0, 1.0])
        eps, sig, rc = S.kob_andersen_tables()
        return s, (lambda c: c.set_lj_multi(eps, sig, rc, 0.0)), float(rc.max()), 0.08, 0.005, False
    if kind in ("eam", "eam_fp64"):
        sf = SF.tabulate(SF.load_cu_params())
        s = S.eam_cu_fcc(ncell=12, seed=43)
        return s, (lambda c: c.set_eam_alloy(sf, 5.0, S.EV, S.EV)), 5.0, 0.1, 2e-3, kind == "eam"
    if kind == "johnson":
        params = S.johnson_ta_params()
        return S.ta_bcc(ncell=12, seed=44), (lambda c: c.set_eam_johnson(params, 6.1)), 6.1, 0.1, 2e-3, True
    raise ValueError(kind)


def _host_steps(gpu, s, setpot, skin, dt, mixed, slabs, link=1, buffer=0.0):
    torch = pytest.importorskip("torch")
    hist = []
    with gpu.Context(0) as ctx:
        ctx.upload_system(s)
        setpot(ctx)
        ctx.set_skin(skin)
        ctx.set_list_buffer(buffer)
        ctx.set_precision(mixed)
        ctx.set_host_pipeline(slabs)
        ctx.set_host_pipeline_link(link)
        ctx.compute_forces()
        start = ctx.download(KEYS)
        st = {}
        for k in KEYS:
            st[k] = torch.empty(s.n, dtype=torch.float64, pin_memory=True).numpy()
            st[k][:] = start[k]
        ctx.build_neighbors()
        used = ctx.host_pipeline()[0]
        for _ in range(NSTEPS):
            ctx.run_nve_host(st, 1, dt, rebuild_every=10)
            hist.append({k: st[k].copy() for k in KEYS})
        steps, redone = ctx.host_pipeline()[1:]
        builds = ctx.list_builds()
    return hist, used, steps, builds, redone


@pytest.mark.parametrize("kind,order,link,buffer", [
    ("lj", "cells", 1, 0.0), ("lj", "random", 1, 0.0), ("eam", "cells", 1, 0.0), ("eam", "lattice", 1, 0.0),
    ("eam_fp64", "cells", 1, 0.0), ("johnson", "cells", 1, 0.0), ("lj_multi_fp64", "cells", 1, 0.0),
    ("eam", "cells", 0, 0.0), ("lj", "random", 0, 0.0), ("eam", "cells", 1, 0.3), ("lj", "cells", 1, 0.2)])
def test_pipelined_host_steps_equal_unpipelined(gpu, kind, order, link, buffer):
    """link 0: chunks carried by the copy engines through HBM staging;
    link 1: kernels reading and writing the page-locked arrays.  buffer > 0:
    both runs rebuild through a two-level list (gbmd_set_list_buffer)."""
    s, setpot, rcut, skin, dt, mixed = _case(kind)
    s = _reorder(s, order, rcut + skin, 7)
    ref, used0, steps0, builds0, _ = _host_steps(gpu, s, setpot, skin, dt, mixed, 0, buffer=buffer)
    got, used, steps, builds, redone = _host_steps(gpu, s, setpot, skin, dt, mixed, 64, link, buffer=buffer)
    assert used0 == 0 and steps0 == 0
    assert used >= 4
    # the trigger fired on some steps, not on most; each was predicted by
    # the step before it (the arrays go back unchanged) and run unpipelined,
    # except when that step was itself unpipelined (the first step, or the
    # step right after a rebuild)
    assert builds == builds0 and builds >= 3
    assert steps == NSTEPS - (builds - 2)
    assert redone <= 1
    for t, (a, b) in enumerate(zip(ref, got)):
        for k in KEYS:
            assert np.array_equal(a[k], b[k]), (t, k)


def test_pipeline_settings(gpu):
    s, setpot, rcut, skin, dt, mixed = _case("lj")
    with gpu.Context(0) as ctx:
        ctx.upload_system(s)
        setpot(ctx)
        ctx.set_skin(skin)
        ctx.build_neighbors()
        assert ctx.host_pipeline() == (0, 0, 0)        # automatic: off below 262,144 atoms
        ctx.set_host_pipeline(4)
        assert ctx.host_pipeline()[0] == 4
        ctx.set_host_pipeline(64)
        assert ctx.host_pipeline()[0] == 5             # one slab per z layer of the 5^3 cells
        ctx.set_newton3(True)
        assert ctx.host_pipeline()[0] == 0             # half lists scatter into other slabs
        for bad in (-2, 1, 3, 65):
            with pytest.raises(gpu.GbmdError):
                ctx.set_host_pipeline(bad)
        for bad in ((2, 40, 512), (1, 0, 512), (1, 40, 48), (1, 40, 2048)):
            with pytest.raises(gpu.GbmdError):
                ctx.set_host_pipeline_link(*bad)


def test_pipeline_timeline(gpu):
    """gbmd_get_host_pipeline_trace: one mark per chunk read, per density and
    force piece and per chunk written back, in dependency order."""
    s, setpot, rcut, skin, dt, mixed = _case("eam")
    s = S.grid_order(s, rcut + skin)
    torch = pytest.importorskip("torch")
    with gpu.Context(0) as ctx:
        ctx.upload_system(s)
        setpot(ctx)
        ctx.set_skin(0.3)
        ctx.set_precision(True)
        ctx.compute_forces()
        start = ctx.download(KEYS)
        st = {k: torch.empty(s.n, dtype=torch.float64, pin_memory=True).numpy() for k in KEYS}
        for k in KEYS:
            st[k][:] = start[k]
        ctx.build_neighbors()
        ctx.set_host_pipeline(8)
        ctx.set_host_pipeline_trace(True)
        ctx.run_nve_host(st, 1, 1e-3, rebuild_every=10)
        marks = ctx.host_pipeline_trace()
        assert ctx.host_pipeline()[1] == 1
    S8 = 8
    kinds = [m[1] for m in marks]
    assert kinds[0] == "start" and kinds[-1] == "end"
    for kind in ("in", "density", "force", "out"):
        assert sorted(m[2] for m in marks if m[1] == kind) == list(range(S8)), kind
    t = {(m[1], m[2]): m[0] for m in marks}
    ins = [t[("in", k)] for k in range(S8)]
    assert ins == sorted(ins)
    end = t[("end", -1)]
    assert all(m[0] <= end for m in marks)
    for q in range(S8):
        for d in (-1, 0, 1):
            assert t[("force", q)] >= t[("density", (q + d) % S8)]
