"""Element-for-element comparison of a GPU pair export with the oracle's
neighbour list, for lists of hundreds of millions of pairs (vectorised, no
per-pair Python objects)."""
import numpy as np


def assert_same_pair_sets(gpu_rows, nl, ids):
    """GPU export (id_i, id_j, image) -- atoms in the library's cell order,
    each atom's rows in list order -- against the oracle's CSR list (atoms
    in input order), compared element for element after reordering the
    oracle's rows into the GPU's atom order."""
    a, b, img = gpu_rows
    n = len(ids)
    order = np.argsort(ids, kind="stable")          # id -> oracle index (ids may be any permutation)
    sorted_ids = ids[order]
    counts_o = np.diff(nl.off)
    assert len(a) == int(nl.off[-1]), (len(a), int(nl.off[-1]))
    # per-atom counts, by id
    ka = order[np.searchsorted(sorted_ids, a)]
    assert np.array_equal(sorted_ids[np.searchsorted(sorted_ids, a)], a), "unknown id_i"
    cnt_gpu = np.bincount(ka, minlength=n)
    assert np.array_equal(cnt_gpu, counts_o), "per-atom neighbour counts differ"
    del cnt_gpu
    # atom sequence of the export (each atom's rows are contiguous)
    starts = np.flatnonzero(np.r_[True, ka[1:] != ka[:-1]])
    seq = ka[starts]
    assert len(np.unique(seq)) == len(seq), "an atom's rows are not contiguous"
    del ka
    lens = counts_o[seq]
    # oracle row index of every GPU row
    pos = np.repeat(nl.off[seq] - (np.cumsum(lens) - lens), lens) + np.arange(len(a), dtype=np.int64)
    del lens, seq, starts
    assert np.array_equal(ids[nl.nbr[pos]], b), "neighbour ids differ"
    assert np.array_equal(nl.img[pos], img), "image shifts differ"
