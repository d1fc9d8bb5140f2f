"""thermal! (src/forcing.jl:297-320) in the oracle.

The normals come from Philox-4x32-10; its implementation is pinned to the
generator's published known-answer vectors (Random123), and the forces to the
reference's own statistical test (test/forcing.jl:141-164: at h = 1, μ = 1/6,
δ = 1 the fluctuations have mean ≈ 0 and variance 2 kbt / 11).
"""
import numpy as np
import pytest


@pytest.mark.parametrize("ctr,key,out", [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
])
def test_philox_known_answers(orc, ctr, key, out):
    assert orc.philox4x32_10(ctr, key) == out


@pytest.mark.parametrize("kb", [0.01, 0.1])
@pytest.mark.parametrize("seed,t", [(0, 1), (12345, 7)])
def test_thermal_statistics_like_reference(orc, kb, seed, t):
    # test/forcing.jl:151-162 (50x50 field of h = 1, μ = 1/6, δ = 1)
    fx, fy = orc.thermal(np.ones((50, 50)), kb, 1 / 6, 1.0, seed=seed, t=t)
    var = 2 * kb / 11
    for f in (fx, fy):
        assert np.mean(f) == pytest.approx(0.0, abs=1e-2)
        assert np.var(f, ddof=1) == pytest.approx(var, abs=var / 10)


def test_thermal_streams_differ_by_seed_and_time(orc):
    a = orc.thermal(np.ones((8, 8)), 0.1, 1 / 6, 1.0, seed=1, t=3)[0]
    b = orc.thermal(np.ones((8, 8)), 0.1, 1 / 6, 1.0, seed=2, t=3)[0]
    c = orc.thermal(np.ones((8, 8)), 0.1, 1 / 6, 1.0, seed=1, t=4)[0]
    d = orc.thermal(np.ones((8, 8)), 0.1, 1 / 6, 1.0, seed=1, t=3)[0]
    assert not np.array_equal(a, b) and not np.array_equal(a, c) and np.array_equal(a, d)


def test_thermal_sigma_depends_on_height(orc):
    # the prefactor sqrt(2 kbt μ 6 h / (2h² + 6hδ + 3δ²)) at two heights, same normals
    h = np.full((16, 16), 2.0)
    f1 = orc.thermal(np.ones((16, 16)), 0.1, 1 / 6, 1.0, seed=5, t=1)[0]
    f2 = orc.thermal(h, 0.1, 1 / 6, 1.0, seed=5, t=1)[0]
    s1 = np.sqrt(2 * 0.1 * (1 / 6) * 6 * 1 / (2 + 6 + 3))
    s2 = np.sqrt(2 * 0.1 * (1 / 6) * 6 * 2 / (8 + 12 + 3))
    assert np.allclose(f2 / f1, s2 / s1, rtol=1e-14)


def test_thermal_literal_equals_fused(orc):
    L = 24
    P = orc.params(L, L, kbt=1e-4, delta=2.0, tau=0.9)
    rng = np.random.default_rng(3)
    h0 = 1.0 + 0.05 * rng.uniform(-1, 1, (L, L))
    lit = orc.LiteralState(P)
    lit.field("height")[:] = h0
    a = lit.run(30, seed=9)
    b = lit.run(20, seed=9)  # the noise continues at iterations 31..50
    fs = orc.FusedState(P, h0)
    fs.run(30, seed=9)
    c = fs.run(20, seed=9)
    assert np.array_equal(b.height, c.height)
    assert np.array_equal(b.velx, c.velx)
    # the noise acts: a run without it differs
    fs0 = orc.FusedState(orc.params(L, L, kbt=0.0, delta=2.0, tau=0.9), h0)
    d = fs0.run(50)
    assert not np.allclose(c.height, d.height, rtol=0, atol=1e-12)
