"""The certified integer path of the octree keys, emulated on the CPU.

The GPU computes the high key word (levels 1..21) of a particle from the binary
digits of its fixed-point position V = (x - c)/(2 hw) + 1/2, whenever every cell
plane the particle is tested against lies farther than a certified margin; it
replays the reference's f64 centre arithmetic otherwise (gravis_gb300/csrc/bh.cu,
k_root / fast_hi / octant_path; the reference: crates/sim-core/src/octree.rs:14-79).
This test restates both in Python's IEEE f64 and checks that, wherever the fast
path claims a key, the key equals the sequential replay: on random, offset,
stretched and lattice inputs and on points placed exactly on, and one ulp beside,
cell planes.
"""
import math

import numpy as np


def root_cell(x, y, z):
    """BoundingBox::containing (octree.rs:29-43)."""
    mn = [x.min(), y.min(), z.min()]
    mx = [x.max(), y.max(), z.max()]
    c = [0.5 * (mn[d] + mx[d]) for d in range(3)]
    e = max(mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2])
    return c, (0.5 * e) * 1.001 + 1e-10


def replay(p, c, hw):
    """The reference's octant path: x >= centre, centre +- hw/2, 21 levels."""
    c = list(c)
    h = 0
    for _ in range(21):
        g = [p[d] >= c[d] for d in range(3)]
        h = (h << 3) | (g[0] | (g[1] << 1) | (g[2] << 2))
        q = hw * 0.5
        c = [c[d] + (q if g[d] else -q) for d in range(3)]
        hw = q
    return h


def fast(p, c, hw):
    """The fixed-point path with the margin of k_root; None where it defers to the replay."""
    ratio = (max(abs(c[0]), abs(c[1]), abs(c[2])) + hw) / hw
    inv = 1.0 / (2.0 * hw)
    margin = int(8192.0 + 65536.0 * math.ceil(ratio))
    W = []
    for d in range(3):
        v = (p[d] - c[d]) * inv + 0.5
        if not 0.0 < v < 1.0:
            return None
        W.append(int(math.floor(v * 2.0 ** 62)))
    h = 0
    for L in range(1, 22):
        half = 1 << (62 - L)
        mask = (half << 1) - 1
        octant = 0
        for d in range(3):
            if abs((W[d] & mask) - half) <= margin:
                return None
            octant |= ((W[d] >> (62 - L)) & 1) << d
        h = (h << 3) | octant
    return h


def inputs():
    rng = np.random.default_rng(11)
    n = 1500
    yield rng.standard_normal((n, 3))
    yield rng.standard_normal((n, 3)) * 1e-3 + np.array([1e3, -2e3, 5e2])  # far from the origin
    yield rng.standard_normal((n, 3)) * np.array([1.0, 1e-6, 1e6])        # stretched
    g = np.arange(10) * 0.5
    yield np.array([[a, b, cc] for a in g for b in g for cc in g])         # exact ties
    p = rng.standard_normal((n, 3))
    c, hw = root_cell(*p.T)
    for k in range(300):                                                   # on and beside planes
        L = int(rng.integers(1, 22))
        p[k, k % 3] = c[k % 3] + hw * (int(rng.integers(-2 ** (L - 1), 2 ** (L - 1))) * 2.0 ** -(L - 1))
        if k % 2:
            p[k, k % 3] = np.nextafter(p[k, k % 3], np.inf)
    yield p


def test_fast_keys_agree_with_the_replay():
    claimed = total = 0
    for pts in inputs():
        x, y, z = (pts[:, d].copy() for d in range(3))
        c, hw = root_cell(x, y, z)
        for i in range(len(x)):
            p = (float(x[i]), float(y[i]), float(z[i]))
            f = fast(p, c, hw)
            total += 1
            if f is not None:
                claimed += 1
                assert f == replay(p, c, hw), (p, hex(f))
    # the fast path must take the bulk of ordinary inputs
    assert claimed > 0.8 * total
