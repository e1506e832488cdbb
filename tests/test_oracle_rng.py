"""RNG restatements: the C oracle against independent pure-Python restatements.

xoroshiro128+ streams, the 2^64 jump and the int64 -> [0,1) conversion follow
lib/rngzig/rng_par_zig.f90:67-74, 253-307; the Irwin-Hall(12) "normal" follows
TrackSubCell.F90:3631-3663.  Philox4x32-10 (the GPU library's counter-based
stream) follows Salmon et al., SC'11.
"""
import struct

import numpy as np
import pytest

from oracle import oracle as O

M64 = (1 << 64) - 1
BASE = (0x1DADBEEFBAADD0D0, 0x5BADD0D0DEADBEEF)  # TrackSubCell.F90:553-555


def rotl(x, k):
    return ((x << k) | (x >> (64 - k))) & M64


def xoro_py(s):
    s1, s2 = s
    out = (s1 + s2) & M64
    s2 ^= s1
    s1 = rotl(s1, 24) ^ s2 ^ ((s2 << 16) & M64)
    s2 = rotl(s2, 37)
    return out, [s1, s2]


def jump_py(s):
    jmp = [(~0x206ffd6b270aab5a) & M64, 0x170865df4b3201fc]
    a = b = 0
    for w in jmp:
        for bit in range(64):
            if w & (1 << bit):
                a ^= s[0]
                b ^= s[1]
            _, s = xoro_py(s)
    return [a, b]


def to_unit(x):
    bits = 0x3FF0000000000000 | (x >> 12)
    return struct.unpack("<d", struct.pack("<Q", bits))[0] - 1.0


def test_xoroshiro_stream0_matches_python():
    s = O.xoro_stream(0)
    assert [int(v) for v in s] == list(BASE)
    got = O.xoro_next(s, 50)
    ps = list(BASE)
    for k in range(50):
        v, ps = xoro_py(ps)
        assert int(got[k]) == v


def test_xoroshiro_jump_streams():
    ps = list(BASE)
    for k in range(1, 4):
        ps = jump_py(ps)
        s = O.xoro_stream(k)
        assert [int(v) for v in s] == ps


def test_uniform_conversion_and_ih12_normal():
    s = O.xoro_stream(0)
    us = O.xoro_uniforms(s, 24)
    ps = list(BASE)
    for k in range(24):
        v, ps = xoro_py(ps)
        assert us[k] == to_unit(v)
        assert 0.0 <= us[k] < 1.0
    # Irwin-Hall(12): sequential sum then minus 6
    s = O.xoro_stream(0)
    L = O.lib()
    import ctypes as C
    val = L.orc_xoro_normal_ih12(s.ctypes.data_as(C.POINTER(C.c_uint64)))
    r = 0.0
    for k in range(12):
        r = r + us[k]
    assert val == r - 6.0


def philox_py(ctr, key):
    c0, c1, c2, c3 = ctr
    k0, k1 = key
    for _ in range(10):
        p0 = 0xD2511F53 * c0
        p1 = 0xCD9E8D57 * c2
        c0, c1, c2, c3 = ((p1 >> 32) ^ c1 ^ k0) & 0xFFFFFFFF, p1 & 0xFFFFFFFF, ((p0 >> 32) ^ c3 ^ k1) & 0xFFFFFFFF, \
            p0 & 0xFFFFFFFF
        k0 = (k0 + 0x9E3779B9) & 0xFFFFFFFF
        k1 = (k1 + 0xBB67AE85) & 0xFFFFFFFF
    return [c0, c1, c2, c3]


@pytest.mark.parametrize("ctr,key", [((0, 0, 0, 0), (0, 0)), ((1, 2, 3, 4), (5, 6)),
                                     ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2),
                                     ((0x12345678, 0, 77, 1), (0xCAFEBABE, 0x5EED))])
def test_philox_matches_python(ctr, key):
    assert O.philox(ctr, key) == philox_py(ctr, key)


def test_philox_ih12_normal_exact_and_counter():
    seed, pid = 0x5EED, 42
    vals, ctr = O.philox_normals(seed, pid, 5)
    assert ctr == 15
    for j in range(5):
        s = 0
        for b in range(3):
            n = 3 * j + b
            o = philox_py((n & 0xFFFFFFFF, n >> 32, pid & 0xFFFFFFFF, pid >> 32),
                          (seed & 0xFFFFFFFF, seed >> 32))
            s += sum(o)
        assert vals[j] == (s - 6 * 2 ** 32) * 2.0 ** -32


def test_ih12_moments():
    vals, _ = O.philox_normals(7, 3, 20000)
    assert abs(vals.mean()) < 0.03
    assert abs(vals.var() - 1.0) < 0.04
    assert vals.min() > -6 and vals.max() < 6


def test_xoroshiro_streams_continue_across_intervals():
    """The reference seeds its thread streams once per run (rng_init in
    pr_InitializeRandomWalk, TrackSubCell.F90:613-620) and every tracking
    interval continues them: two intervals of one run draw different numbers,
    and a single-threaded run is deterministic."""
    from mprw import workloads as W
    g, f, p, opt = W.uniform_pulse(n_particles=50)

    def run(reset_between):
        O.reset_xoroshiro()
        q, _ = O.advance(g, f, opt, p, 0.0, 5.0, rng_kind=O.RNG_XOROSHIRO, nthreads=1)
        if reset_between:
            O.reset_xoroshiro()
        q, _ = O.advance(g, f, opt, q, 5.0, 10.0, rng_kind=O.RNG_XOROSHIRO, nthreads=1)
        return q

    a, b, c = run(False), run(False), run(True)
    assert np.array_equal(a.lx, b.lx) and np.array_equal(a.cell, b.cell)
    # restarting the streams replays the first interval's draws: another trajectory
    assert not np.array_equal(a.lx, c.lx)
