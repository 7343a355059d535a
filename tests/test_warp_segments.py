"""CPU restatement of the run kernel's segmented warp sum (scatter_seg in
csrc/oxg_kernels.cuh): 32 lanes each hold a pair's i-side force and its i; lanes form
runs of adjacent equal keys; a suffix sum with doubling offsets, limited to the lane's
run, leaves each run's total in its first lane, which adds it once. Every particle's
force must equal the plain sum of its pairs' forces, also when its pairs are split over
runs that are not adjacent and when lanes hold no pair (key -1) or no contribution."""

import numpy as np


def seg_sums(keys, v, has):
    n = len(keys)
    v = np.where(has, v, 0.0)
    cnt = has.astype(float)
    head = np.array([l == 0 or keys[l - 1] != keys[l] for l in range(n)])
    heads = sum(1 << l for l in range(n) if head[l])
    ends = []
    for lane in range(n):
        above = heads & ~((2 << lane) - 1) & 0xFFFFFFFF
        ends.append((above & -above).bit_length() - 2 if above else 31)
    off = 1
    while off < n:
        nv, nc = v.copy(), cnt.copy()
        for lane in range(n):
            if lane + off <= ends[lane]:
                nv[lane] += v[lane + off]
                nc[lane] += cnt[lane + off]
        v, cnt = nv, nc
        off *= 2
    out = {}
    for lane in range(n):
        if head[lane] and keys[lane] >= 0 and cnt[lane] > 0:
            out[keys[lane]] = out.get(keys[lane], 0.0) + v[lane]
    return out


def test_segmented_sum_matches_plain_sum():
    rng = np.random.default_rng(7)
    for trial in range(3000):
        keys = rng.integers(-1, 6, 32)
        if trial % 2:
            keys = np.sort(keys)
        v = rng.normal(size=32)
        has = (rng.random(32) < 0.8) & (keys >= 0)
        got = seg_sums(keys, v, has)
        for k in set(keys[keys >= 0].tolist()):
            want = v[(keys == k) & has].sum()
            assert abs(got.get(k, 0.0) - want) < 1e-12, (keys, k)
        assert set(got) <= set(keys[has].tolist())


def test_run_end_from_head_mask():
    # the last lane of each run is the lane before the next head (31 for the last run)
    keys = np.array([3] * 5 + [1] * 10 + [3] * 2 + [-1] * 15)
    head = [l == 0 or keys[l - 1] != keys[l] for l in range(32)]
    heads = sum(1 << l for l in range(32) if head[l])
    for lane, want in ((0, 4), (4, 4), (5, 14), (15, 16), (17, 31), (31, 31)):
        above = heads & ~((2 << lane) - 1) & 0xFFFFFFFF
        assert ((above & -above).bit_length() - 2 if above else 31) == want
