"""Cell grid of a batched replica, checked on the CPU.

The batch kernel sizes each replica's cell grid with gbmd::batch_grid_dims
(exastamp_gb300/csrc/gbmd_batch_grid.h), and gbmd_batch_upload refuses boxes
that gbmd::batch_box_ok rejects.  Both are plain C++, so this compiles them
with g++ and checks that huge and infinite boxes neither overflow the cell
count nor leave the shared-memory limit, and that ordinary boxes keep cells
of at least rcut / S.
"""
import math
import shutil
import subprocess

import pytest

DRIVER = r"""
#include <cstdio>
#include <cstdlib>
#include "gbmd_batch_grid.h"
int main(int argc, char** argv) {
  const double L[3] = {atof(argv[1]), atof(argv[2]), atof(argv[3])};
  const double rcut = atof(argv[4]);
  const int S = atoi(argv[5]), maxc = atoi(argv[6]);
  int nc[3];
  const int n = gbmd::batch_grid_dims(L, rcut, S, maxc, nc);
  const double lo[3] = {0, 0, 0};
  printf("%d %d %d %d %d\n", n, nc[0], nc[1], nc[2], (int)gbmd::batch_box_ok(lo, L));
  return 0;
}
"""


@pytest.fixture(scope="module")
def grid_exe(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    import os
    d = tmp_path_factory.mktemp("batch_grid")
    src = d / "drv.cpp"
    src.write_text(DRIVER)
    exe = d / "drv"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "exastamp_gb300", "csrc")
    subprocess.run([gxx, "-O1", "-std=c++17", "-I", inc, str(src), "-o", str(exe)], check=True)

    def run(L, rcut=5.0, S=1, maxc=1024):
        out = subprocess.run([str(exe)] + [repr(float(x)) for x in L] + [repr(rcut), str(S), str(maxc)],
                             capture_output=True, text=True, check=True, timeout=20).stdout.split()
        n, a, b, c, ok = map(int, out)
        return n, (a, b, c), bool(ok)
    return run


@pytest.mark.parametrize("L", [(1e300, 1e300, 1e300), (1e7, 1e7, 1e7), (1e12, 20.0, 20.0),
                               (float("inf"), 30.0, 30.0)])
@pytest.mark.parametrize("S,maxc", [(1, 1024), (2, 1024), (2, 512)])
def test_huge_boxes_stay_within_the_cell_limit(grid_exe, L, S, maxc):
    n, nc, ok = grid_exe(L, 5.0, S, maxc)
    assert 0 < n <= maxc and n == nc[0] * nc[1] * nc[2]
    assert all(c >= S for c in nc)
    assert ok == all(math.isfinite(x) for x in L)


@pytest.mark.parametrize("L", [(10.85, 10.85, 10.85), (28.9, 28.9, 28.9), (14.5, 21.7, 36.2), (5.01, 5.01, 5.01)])
@pytest.mark.parametrize("S", [1, 2])
def test_ordinary_boxes_keep_cells_of_at_least_rcut_over_s(grid_exe, L, S):
    rcut = 5.0
    n, nc, ok = grid_exe(L, rcut, S, 1024)
    assert ok and n <= 1024
    for Ld, c in zip(L, nc):
        assert c >= S
        if Ld >= rcut:
            assert Ld / c >= rcut / S * (1 - 1e-12)


def test_empty_box_rejected(grid_exe):
    assert grid_exe((0.0, 10.0, 10.0))[2] is False
    assert grid_exe((-1.0, 10.0, 10.0))[2] is False
