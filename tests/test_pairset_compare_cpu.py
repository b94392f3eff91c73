"""The large-list pair-set comparison used by the headline-size GPU tests
fails on a planted difference (planted in the oracle's list, on the CPU)."""
import numpy as np
import pytest

from exastamp_gb300 import systems as S

from pairset_compare import assert_same_pair_sets


def test_pair_set_comparison_detects_a_changed_pair(oracle):
    """A GPU-like export built from the oracle list passes; one changed
    neighbour id fails."""
    s = S.lj_fcc(ncell=4, seed=5)
    rng = np.random.default_rng(5)
    for arr in (s.x, s.y, s.z):
        arr += rng.normal(0.0, 0.05, s.n)
    ids = rng.permutation(s.n).astype(np.uint64)
    x, y, z = s.x.copy(), s.y.copy(), s.z.copy()
    oracle.wrap(x, y, z, s.lo, s.hi)
    nl = oracle.build_neighbors(x, y, z, ids, s.lo, s.hi, 2.8)
    # a GPU-like export: atoms in a shuffled order, rows in list order
    perm = rng.permutation(s.n)
    cnt = np.diff(nl.off)
    rows_i = np.concatenate([np.full(cnt[k], ids[k], np.uint64) for k in perm])
    rows_j = np.concatenate([ids[nl.nbr[nl.off[k]:nl.off[k + 1]]] for k in perm])
    rows_img = np.concatenate([nl.img[nl.off[k]:nl.off[k + 1]] for k in perm])
    assert_same_pair_sets((rows_i, rows_j, rows_img), nl, ids)
    bad = rows_j.copy()
    bad[len(bad) // 2] = bad[len(bad) // 2 + 1]
    with pytest.raises(AssertionError):
        assert_same_pair_sets((rows_i, bad, rows_img), nl, ids)
