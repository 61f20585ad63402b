"""Work partition of the split GEMM's stream-K schedule, on the CPU.

itg_split_partition runs the same partition code as k_split_gemm (compiled for
the host as well) and returns each cluster's tile segments.  The kernel's
correctness rests on these properties, checked here without a GPU:

* every unit (tile, level) belongs to exactly one cluster;
* whole tiles run in waves: cluster g's first q segments are the whole tiles
  g, g + G, ..., g + (q - 1) G, q = tiles // G;
* a shared tile is cut only at level boundaries, its contributor count is the
  number of clusters that own one of its levels and the reported first
  contributor is the lowest of them (the kernel's last-arrival test and the
  shared accumulator slot depend on both);
* shared accumulator slots (first contributors of shared tiles) are distinct;
* the work (units weighted by level cost L + 1) is balanced: each end of a
  cluster's range lies less than one unit (cost <= S) from its even share.
"""
import ctypes as C

import pytest

S = 6  # digit levels of the split GEMM (base-2^8 digits per operand)
T = S * (S + 1) // 2


def _segments(lib, nct, G, g):
    cap = 4
    while True:
        buf = (C.c_int32 * (5 * cap))()
        n = C.c_int()
        st = lib.itg_split_partition(nct, G, g, buf, cap, C.byref(n))
        if st == 0:
            return [tuple(buf[5 * i:5 * i + 5]) for i in range(n.value)]
        assert st == 2 and n.value > cap  # ITG_ERR_SHAPE: buffer too small
        cap = n.value


def _check(lib, nct, G):
    q = nct // G
    owner = {}
    reported = {}
    work = [0] * G
    for g in range(G):
        segs = _segments(lib, nct, G, g)
        for i, (ct, L0, Le, contrib, first) in enumerate(segs):
            assert 0 <= ct < nct and 0 <= L0 < Le <= S
            if i < q:
                assert (ct, L0, Le) == (g + i * G, 0, S)
            for L in range(L0, Le):
                assert (ct, L) not in owner, (nct, G, ct, L)
                owner[(ct, L)] = g
                work[g] += L + 1
            reported.setdefault(ct, set()).add((contrib, first))
    assert len(owner) == nct * S
    slots = set()
    for ct in range(nct):
        clusters = sorted({owner[(ct, L)] for L in range(S)})
        assert len(reported[ct]) == 1  # every segment of a tile reports the same
        (contrib, first), = reported[ct]
        assert contrib == len(clusters)
        if contrib > 1:
            assert first == clusters[0]
            assert clusters[0] not in slots
            slots.add(clusters[0])
            # owners are non-decreasing over the levels: cuts at level boundaries
            levels = [owner[(ct, L)] for L in range(S)]
            assert levels == sorted(levels)
    # each end of a cluster's range moves by less than one unit (cost <= S)
    assert max(work) - min(work) <= 2 * (S - 1) + 1


@pytest.mark.parametrize("G", [1, 2, 3, 7, 36, 38, 76, 151, 152])
def test_partition_covers_every_unit_once(itg_lib, G):
    for nct in [1, 2, 5, 37, 64, 75, 76, 77, 128, 151, 152, 153, 300, 320, 640, 1280]:
        _check(itg_lib, nct, G)


def test_one_cluster_per_tile_without_stream_k(itg_lib):
    """G = tiles (the one-tile-per-CTA launch): cluster g computes exactly tile g."""
    for nct in [1, 3, 64, 200]:
        for g in range(nct):
            assert _segments(itg_lib, nct, nct, g) == [(g, 0, S, 1, 0)]


def test_partition_rejects_bad_arguments(itg_lib):
    n = C.c_int()
    buf = (C.c_int32 * 5)()
    assert itg_lib.itg_split_partition(0, 4, 0, buf, 1, C.byref(n)) != 0
    assert itg_lib.itg_split_partition(10, 4, 4, buf, 1, C.byref(n)) != 0
    assert itg_lib.itg_split_partition(10, 0, 0, buf, 1, C.byref(n)) != 0
