"""The allocation-free thermodynamic reduction, called through the C ABI.

Callers that may not allocate device memory (a plugin living on its host
framework's memory pool, code running during a stream capture, latency-
critical loops) use gbmd_thermo_reduce_noalloc, which keeps its scratch in a
fixed array of the library.  This checks its output against gbmd_thermo (the
context-owned reduction) on two calls in a row -- the second call finds the
scratch holding the first call's partial sums -- with the tolerance of the
other thermo tests (1e-12 relative).  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_thermo_reduce_noalloc_matches_context_reduction(gpu):
    import torch
    from exastamp_gb300 import systems as S

    s = S.lj_fcc(ncell=7, seed=21)
    rng = np.random.default_rng(21)
    for a in (s.x, s.y, s.z):
        a += rng.normal(0.0, 0.03, s.n)
    s.type = (rng.random(s.n) < 0.3).astype(np.uint8)
    s.masses = np.array([1.0, 2.5])
    with gpu.Context(0) as ctx:
        ctx.upload_system(s)
        ctx.set_lj(1.0, 1.0, 2.5)
        ctx.set_skin(0.3)
        ctx.compute_forces(energy=True, virial=True)
        ref = ctx.thermo()
        d = ctx.download(virial=True)

    dev = torch.device("cuda:0")
    arrays = {k: torch.tensor(d[k], dtype=torch.float64, device=dev) for k in ("vx", "vy", "vz", "ep")}
    vir = torch.tensor(d["vir"], dtype=torch.float64, device=dev).contiguous()
    types = torch.tensor(s.type, dtype=torch.uint8, device=dev)
    masses = np.ascontiguousarray(s.masses, dtype=np.float64)
    out = torch.empty(27, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    fn = gpu.lib().gbmd_thermo_reduce_noalloc
    for _ in range(2):
        out.fill_(float("nan"))
        rc = fn(s.n, arrays["vx"].data_ptr(), arrays["vy"].data_ptr(), arrays["vz"].data_ptr(),
                arrays["ep"].data_ptr(), vir.data_ptr(), types.data_ptr(), masses.ctypes.data, len(masses),
                out.data_ptr(), ctypes.c_void_p(stream))
        assert rc == 0
        torch.cuda.synchronize(dev)
        got = out.cpu().numpy()
        assert np.allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())

    # sizes beyond the stated maximum are refused before anything is launched
    rc = fn((1 << 26) + 1, arrays["vx"].data_ptr(), arrays["vy"].data_ptr(), arrays["vz"].data_ptr(), None, None,
            types.data_ptr(), masses.ctypes.data, len(masses), out.data_ptr(), ctypes.c_void_p(stream))
    assert rc == 9
