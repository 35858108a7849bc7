"""The arithmetic facts the hash kernels rest on, checked on the CPU (the
kernels themselves are checked on the GPU against brute forces in
test_gpu_broadphase.py and test_gpu_edge_edge.py):

* the cell of a coordinate, floor((v - start) / cell) in float32, is
  monotone in v, so the cell of the low corner of two boxes' intersection is
  the larger of the two boxes' first cells (the edge pairing's reporting
  rule, csrc/pbd_edge.cu);
* the 64-bit mask of k_point_pairs: with incident cells inside a 2 x 2 x 2
  block, OR-ing 0x0000077707770777 shifted by dx + 4 dy + 16 dz gives exactly
  the union of their 27-neighbourhoods inside the 4 x 4 x 4 block around
  them (bit x + 4 y + 16 z);
* the round-robin pairing of a bucket run (k_ee_pairs): record a of m takes
  (a + d) mod m for d = 1 .. (m - 1) / 2, and d = m / 2 when m is even and
  a < m / 2; every unordered pair once, at most ceil((m - 1) / 2) steps.
"""
import itertools

import numpy as np

NEAR3 = 0x0000077707770777


def cell_of(v, start, cell):
    f32 = np.float32
    return np.floor((f32(v) - f32(start)) / f32(cell)).astype(np.int64)


def test_cell_is_monotone_so_the_corner_cell_is_the_larger_first_cell():
    rng = np.random.default_rng(0)
    for start, cell in [(0.0, 0.0089), (-2.5, 0.0157), (0.3, 0.02054875), (1e3, 0.01)]:
        v = np.sort(rng.uniform(start - 50 * cell, start + 50 * cell, 200000).astype(np.float32))
        # include exact cell boundaries and their float neighbours
        b = (start + cell * np.arange(-50, 50)).astype(np.float32)
        v = np.sort(np.concatenate([v, b, np.nextafter(b, np.float32(-np.inf)),
                                    np.nextafter(b, np.float32(np.inf))]))
        c = cell_of(v, start, cell)
        assert np.all(np.diff(c) >= 0)
        a, w = rng.choice(v, 50000), rng.choice(v, 50000)
        np.testing.assert_array_equal(cell_of(np.maximum(a, w), start, cell),
                                      np.maximum(cell_of(a, start, cell), cell_of(w, start, cell)))


def test_neighbourhood_mask_is_the_union_of_27_neighbourhoods():
    block = list(itertools.product(range(2), repeat=3))
    for k in range(1, 1 << 8):
        inc = [block[i] for i in range(8) if k >> i & 1]
        lx, ly, lz = (min(c[j] for c in inc) for j in range(3))
        mask = 0
        for (x, y, z) in inc:
            mask |= NEAR3 << ((x - lx) + 4 * (y - ly) + 16 * (z - lz))
        assert mask < 1 << 64
        for bi in range(64):
            cx, cy, cz = lx - 1 + (bi & 3), ly - 1 + (bi >> 2 & 3), lz - 1 + (bi >> 4)
            near = any(abs(cx - x) <= 1 and abs(cy - y) <= 1 and abs(cz - z) <= 1
                       for (x, y, z) in inc)
            assert bool(mask >> bi & 1) == near, (k, bi)


def test_round_robin_covers_every_pair_once():
    for m in range(1, 80):
        seen = {}
        most = 0
        for a in range(m):
            steps = (m - 1) // 2 + (1 if m % 2 == 0 and a < m // 2 else 0)
            most = max(most, steps)
            for d in range(1, steps + 1):
                b = (a + d) % m
                key = (min(a, b), max(a, b))
                seen[key] = seen.get(key, 0) + 1
        assert len(seen) == m * (m - 1) // 2
        assert all(v == 1 for v in seen.values())
        assert most == -(-(m - 1) // 2)
