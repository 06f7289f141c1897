"""The index arithmetic of the count scan and the child map (csrc/rp_trace.cu
tile_scan_kernel, child_map_kernel), restated in numpy and run on CPU for
sizes around every boundary the kernels have: warp chunks of 128-count
slices (per = ceil(n / 4096) * 128), ragged last slices and chunks past the
end.  The scan must give the exclusive prefix and the total; the map must
send the children of sub-tile q to positions offset[q] .. offset[q] +
count[q] - 1 with arena slots q * 64 + j."""
import numpy as np
import pytest

SLICE = 128  # RP_SCAN_SLICE: counts per warp step, 4 per lane
WARPS = 32   # warps of the one 1024-thread block
SUB_SLOTS = 64


def scan_like_kernel(counts):
    n = len(counts)
    per = (n + WARPS * SLICE - 1) // (WARPS * SLICE) * SLICE
    offsets = np.full(n, -1, dtype=np.int64)
    sums = []
    for w in range(WARPS):
        c0 = min(per * w, n)
        c1 = min(c0 + per, n)
        sums.append(int(counts[c0:c1].sum()))
    prefix = np.cumsum(sums)
    for w in range(WARPS):
        c0 = min(per * w, n)
        c1 = min(c0 + per, n)
        carry = int(prefix[w - 1]) if w else 0
        for base in range(c0, c1, SLICE):
            v = np.zeros((32, 4), dtype=np.int64)
            for lane in range(32):
                for j in range(4):
                    k = base + 4 * lane + j
                    if k < c1:
                        v[lane, j] = counts[k]
            lane_sum = v.sum(1)
            incl = np.cumsum(lane_sum)
            for lane in range(32):
                e = carry + incl[lane] - lane_sum[lane]
                for j in range(4):
                    k = base + 4 * lane + j
                    if k < c1:
                        offsets[k] = e
                    e += v[lane, j]
            carry += int(incl[31])
    return offsets, int(prefix[-1]) if n else 0


@pytest.mark.parametrize("n", [0, 1, 3, 127, 128, 129, 4095, 4096, 4097, 8191, 12289, 40000])
def test_scan_is_the_exclusive_prefix(n):
    counts = np.random.default_rng(n).integers(0, SUB_SLOTS + 1, n)
    offsets, total = scan_like_kernel(counts)
    ref = np.concatenate([[0], np.cumsum(counts)[:-1]]) if n else np.zeros(0, dtype=np.int64)
    assert np.array_equal(offsets, ref) and total == int(counts.sum())


def test_child_map_places_every_child_once():
    rng = np.random.default_rng(7)
    counts = rng.integers(0, SUB_SLOTS + 1, 1000)
    offsets, total = scan_like_kernel(counts)
    child_map = np.full(total, -1, dtype=np.int64)
    for q, (c, o) in enumerate(zip(counts, offsets)):
        for j in range(c):  # child_map_kernel: map[base + j] = q * RP_SUB_SLOTS + j
            assert child_map[o + j] == -1
            child_map[o + j] = q * SUB_SLOTS + j
    assert np.all(child_map >= 0)
    # children keep parent order: slots increase along the generation
    assert np.all(np.diff(child_map) > 0)
