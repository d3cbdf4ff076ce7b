"""A model of the cluster selection's arithmetic (csrc/bsj_kernels.cu, select_cluster), run on
the CPU against the order it must produce.

The selection replaces the reference's stable sort of all child slots
(cub::DeviceRadixSort::SortPairs, gpu/v1/solver.cu:255-258): the first R keys in ascending
(score bits, slot) order.  The cluster route splits the level's keys, in slot order, over C
blocks and combines per-block pieces into global positions:

  * the threshold bucket T comes from the bucket counts summed over the blocks;
  * each block compacts its own keys of buckets <= T, keeping their order;
  * dense ranks come from the union of the blocks' distinct scores;
  * each block counts its survivors per (warp, rank) in the kernel's element layout
    (p = warp * 32 * E + e * 32 + lane), and a survivor's position is
        (survivors of lower ranks in all blocks) + (its rank in lower blocks)
        + (its rank in lower warps of its block) + (its order within its warp).

This test restates those steps with numpy and checks the positions against a stable sort,
for 2 and 4 blocks, levels smaller than the block count, and tie-heavy scores.  The GPU
kernels themselves are checked against the oracle in tests/test_gpu_select_routes.py and
tests/test_gpu_k4096.py.
"""
import numpy as np
import pytest

NB = 4096          # buckets (kNB)
THREADS = 1024     # threads per block (kSelectThreads)


def bucket_params(scores):
    smin, smax = int(scores.min()), int(scores.max())
    rng = smax - smin
    nbits = rng.bit_length()
    shift = nbits - 12 if nbits > 12 else 0
    return smin, shift


def cluster_select(scores, R, C):
    """Positions 0..R-1 -> slot, as the cluster route computes them."""
    V = len(scores)
    slots = np.arange(V, dtype=np.int64)
    smin, shift = bucket_params(scores)
    bucket = np.minimum((scores.astype(np.int64) - smin) >> shift, NB - 1)
    # block r holds keys [r*V/C, (r+1)*V/C) in slot order
    bounds = [(V * r) // C for r in range(C + 1)]
    counts = np.zeros(NB, dtype=np.int64)
    for r in range(C):
        counts += np.bincount(bucket[bounds[r]:bounds[r + 1]], minlength=NB)
    cum = np.cumsum(counts)
    T = int(np.searchsorted(cum, R))        # first bucket whose running count reaches R
    lim = (T + 1) << shift
    # each block's survivors, compacted in order
    surv = []
    for r in range(C):
        lo, hi = bounds[r], bounds[r + 1]
        keep = (scores[lo:hi].astype(np.int64) - smin) < lim
        surv.append(np.nonzero(keep)[0] + lo)
    # dense ranks: the union of the blocks' distinct scores among the survivors
    distinct = np.unique(np.concatenate([scores[s] for s in surv]))
    rank_of = {int(v): i for i, v in enumerate(distinct)}
    nd = len(distinct)
    # per block: per-(warp, digit) counts in the kernel's element layout
    per_block_tot = []
    placed = []
    for r in range(C):
        s = surv[r]
        cl = len(s)
        E = (cl + THREADS - 1) // THREADS
        wh = np.zeros((32, nd), dtype=np.int64)
        off = np.zeros(cl, dtype=np.int64)
        dig = np.array([rank_of[int(scores[k])] for k in s], dtype=np.int64)
        for warp in range(32):
            for e in range(E):
                for lane in range(32):
                    p = warp * 32 * E + e * 32 + lane
                    if p < cl:
                        d = dig[p]
                        off[p] = wh[warp, d]
                        wh[warp, d] += 1
        # per digit, exclusive prefix over the warps
        wpre = np.cumsum(wh, axis=0) - wh
        tot = wh.sum(axis=0)
        per_block_tot.append(tot)
        placed.append((s, dig, off, wpre, E))
    gtot = np.sum(per_block_tot, axis=0)
    gbase = np.cumsum(gtot) - gtot
    out = np.full(R, -1, dtype=np.int64)
    for r in range(C):
        s, dig, off, wpre, E = placed[r]
        lower = np.sum(per_block_tot[:r], axis=0) if r > 0 else np.zeros_like(gtot)
        for p in range(len(s)):
            warp = p // (32 * E) if E else 0
            d = dig[p]
            pos = gbase[d] + lower[d] + wpre[warp, d] + off[p]
            if pos < R:
                assert out[pos] == -1
                out[pos] = slots[s[p]]
    return out


def reference_order(scores, R):
    return np.lexsort((np.arange(len(scores)), scores))[:R]


@pytest.mark.parametrize("C", [2, 4])
@pytest.mark.parametrize("case", range(6))
def test_cluster_positions_equal_the_stable_order(C, case):
    rng = np.random.default_rng(100 + 10 * C + case)
    V = int(rng.choice([1, 3, 7, 200, 1500, 3000]))
    # scores: float bits of positive values with few distinct levels plus a small noise
    # (as cmax / ns + noise), or heavy ties
    base = rng.integers(50, 60, size=V).astype(np.float32) / np.float32(7.0)
    noise = (rng.integers(0, 1000 if case % 2 == 0 else 3, size=V).astype(np.float32) / np.float32(1e9))
    scores = (base + noise).view(np.uint32).astype(np.uint32)
    R = int(rng.integers(1, V + 1))
    got = cluster_select(scores, R, C)
    want = reference_order(scores, R)
    assert np.array_equal(got, want), (C, V, R)


def test_more_blocks_than_keys():
    scores = np.array([1065353216, 1065353216], dtype=np.uint32)   # two equal scores
    for C in (2, 4):
        assert np.array_equal(cluster_select(scores, 2, C), np.array([0, 1]))
