"""The stream-position algorithm of the device Plummer generator (gravis_gb300/csrc/ics_dev.cu),
restated in numpy and checked on the CPU against the oracle's sequential sampler
(orc_plummer_sample, the restatement of plummer_sphere.rs:13-58 pinned to the reference's m1
CSV): a successor map over the stream's draw offsets (where a particle starting there would
end, its rejection loop replayed), its powers 2^k by repeated squaring, and particle i's
start composed from the bits of i, give every particle the stream position the sequential
sampler reaches -- shown by sampling each particle from its start and comparing with the
oracle's particles bit for bit.  Offsets here count u64 draws (two stream words).
"""
import ctypes as C
import math
import struct

import numpy as np
import pytest

import oracle as O

TWO_PI = 2.0 * 3.14159265358979323846


def stream(seed, count):
    rng = O.Rng(seed)
    return np.array([rng.next_u64() for _ in range(count)], dtype=np.uint64)


def draw_range(u, lo, hi):
    """rand's random_range(lo..hi) for f64 from one u64 (as ics.cpp and the oracle)."""
    v = struct.unpack("<d", struct.pack("<Q", (int(u) >> 12) | (1023 << 52)))[0]
    return (v - 1.0) * (hi - lo) + lo


def draw_uniform(u):
    return (int(u) >> 11) * (1.0 / 9007199254740992.0)


def accept(qq, u):
    return u < qq * qq * math.pow(1.0 - qq * qq, 3.5) / 0.1


def successor(U):
    """succ[h]: the draw offset where a particle starting at draw h ends (len(U) when the
    stream is too short); succ[len(U)] = len(U)."""
    H = len(U)
    succ = np.full(H + 1, H, dtype=np.int64)
    for h in range(H):
        p = h + 3  # after the mass fraction, cos theta and phi
        while p + 4 <= H:  # this attempt and the final direction must fit
            qq, u = draw_range(U[p], 0.0, 1.0), draw_uniform(U[p + 1])
            p += 2
            if accept(qq, u):
                succ[h] = p + 2
                break
    return succ


def starts_by_squaring(succ, n):
    levels = [succ]
    while (1 << len(levels)) < n:
        levels.append(levels[-1][levels[-1]])
    out = np.zeros(n, dtype=np.int64)
    for i in range(n):
        h = 0
        for k, J in enumerate(levels):
            if (i >> k) & 1:
                h = J[h]
        out[i] = h
    return out


def sample(U, p, a=1.0, total_mass=1.0):
    """sample_plummer_particle from draw offset p (ics.cpp's plummer_particle)."""
    x_mass = draw_range(U[p], 0.001, 1.0)
    r = a / math.sqrt(math.pow(x_mass, -2.0 / 3.0) - 1.0)
    ct = draw_range(U[p + 1], -1.0, 1.0)
    st = math.sqrt(1.0 - ct * ct)
    phi = draw_range(U[p + 2], 0.0, TWO_PI)
    pos = (r * st * math.cos(phi), r * st * math.sin(phi), r * ct)
    v_esc = math.sqrt(2.0 * 1.0 * total_mass / math.sqrt(r * r + a * a))
    p += 3
    while True:
        qq, u = draw_range(U[p], 0.0, 1.0), draw_uniform(U[p + 1])
        p += 2
        if accept(qq, u):
            break
    v = qq * v_esc
    cv = draw_range(U[p], -1.0, 1.0)
    sv = math.sqrt(1.0 - cv * cv)
    pv = draw_range(U[p + 1], 0.0, TWO_PI)
    return pos + (v * sv * math.cos(pv), v * sv * math.sin(pv), v * cv)


@pytest.mark.parametrize("n,seed", [(1, 3), (7, 42), (300, 1), (1500, 7)])
def test_squaring_finds_every_start_of_the_sequential_sampler(n, seed):
    U = stream(seed, 12 * n + 64)  # 24 words per particle, as the device budget
    succ = successor(U)
    starts = starts_by_squaring(succ, n)
    # the sequential chain
    h, chain = 0, []
    for _ in range(n):
        chain.append(h)
        h = succ[h]
    assert np.array_equal(starts, np.array(chain))
    assert starts[-1] < len(U)
    # each particle sampled from its start equals the oracle's sequential sampler
    lib = O.lib()
    lib.orc_plummer_sample.restype = None
    lib.orc_plummer_sample.argtypes = [C.c_void_p, C.c_double, C.c_double, C.POINTER(C.c_double),
                                       C.POINTER(C.c_double)]
    rng = O.Rng(seed)
    pos, vel = (C.c_double * 3)(), (C.c_double * 3)()
    for i in range(n):
        lib.orc_plummer_sample(rng._buf, 1.0, 1.0, pos, vel)
        assert sample(U, int(starts[i])) == tuple(pos) + tuple(vel), i
