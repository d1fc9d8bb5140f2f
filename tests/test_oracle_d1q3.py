"""The D1Q3 (one-dimensional) path of the oracle against the reference's
tests: equilibria (test/equilibrium.jl:87-150), collision and streaming
(test/collide.jl:125-226), slippage (test/forcing.jl:71-100) and the 1D
simulations (test/simulate.jl:3-94)."""
import math

import numpy as np
import pytest


def test_equilibria_1d(orc):
    assert np.all(orc.equilibrium_1d(np.zeros(30), np.zeros(30)) == 0.0)
    fe = orc.equilibrium_1d(np.ones(30), np.zeros(30))
    assert np.all(fe[:, 0] == 1.0) and np.all(fe[:, 1:] == 0.0)
    fe = orc.equilibrium_1d(np.ones(30), np.zeros(30), 0.1)
    assert np.all(fe[:, 0] == 1.0 - 0.05) and np.all(fe[:, 1:] == 0.025)
    fe = orc.equilibrium_1d(np.ones(30), np.full(30, 0.1))
    assert np.all(fe[:, 0] == 1.0 - 0.01)
    assert np.allclose(fe[:, 1], 0.5 * 0.1 + 0.5 * 0.01) and np.allclose(fe[:, 2], -0.5 * 0.1 + 0.5 * 0.01)
    fe = orc.equilibrium_1d(np.ones(30), np.full(30, 0.1), 0.1)
    assert np.all(fe[:, 0] == 1.0 - 0.5 * 0.1 - 0.01)
    assert np.allclose(fe[:, 1], 0.025 + 0.5 * 0.1 + 0.5 * 0.01)
    assert np.allclose(fe[:, 2], 0.025 - 0.5 * 0.1 + 0.5 * 0.01)


@pytest.mark.parametrize("tau,F", [(1.0, 0.0), (0.75, 0.0), (1.0, 0.1), (0.75, 0.1)])
def test_collide_and_stream_1d(orc, tau, F):
    feq = np.ones((30, 3), order="F")
    feq[0, :] = 2.0
    ftemp = np.ones((30, 3), order="F")
    fout, _ = orc.bgk_stream_1d(feq, ftemp, np.full(30, F), tau)
    omega, onebytau = 1.0 - 1.0 / tau, 1.0 / tau
    post = omega * 1.0 + onebytau * feq[:, 0] if tau != 1.0 else feq[:, 0]
    assert np.all(fout[:, 0] == post)
    assert np.all(fout[:, 1] == np.roll(post + F / 2, 1))
    assert np.all(fout[:, 2] == np.roll(post - F / 2, -1))


def test_slippage_1d(orc):
    # test/forcing.jl:71-100: zero velocity -> 0; u = 0.1, h = 1, δ = 1 -> 6μ u / 11
    assert np.all(orc.slippage_1d(np.ones(30), np.zeros(30), 1.0, 1 / 6) == 0.0)
    s = orc.slippage_1d(np.ones(30), np.full(30, 0.1), 1.0, 1 / 6)
    assert np.allclose(s, 0.1 / 11)
    s = orc.slippage_1d(np.ones(30), np.full(30, 0.1), 0.0, 1 / 6)
    assert np.allclose(s, 0.1 / 2)


def test_flat_1d(orc):
    s = orc.State1D(orc.params(25, 1, Tmax=200, tdump=100))
    s.run(200)
    assert np.all(s.h == 1.0) and np.sum(s.h) == 25


def test_random_1d_flattens(orc):
    P = orc.params(25, 1, Tmax=10000, tdump=5000)
    rng = np.random.default_rng(7)
    s = orc.State1D(P, 1.0 * (1.0 + 0.1 * rng.standard_normal(25)))
    s.run(10000, theta_field=np.full(25, 1 / 9))
    assert s.h.max() - s.h.min() < 0.02


def test_rayleigh_taylor_1d_grows(orc):
    L = 512
    P = orc.params(L, 1, Tmax=1000, tdump=500, g=-0.002)
    i = np.arange(1, L + 1)
    s = orc.State1D(P, 1.0 * (1 + 0.01 * np.sin(2 * np.pi * 4 * i / (L - 1))))
    dh = s.run(1000, record_dh=True)
    assert dh[0] < dh[-1]


def test_droplet_relax_1d(orc):
    rads, L = 35, 150
    P = orc.params(L, 1, Tmax=10000, delta=3.0)
    s = orc.State1D(P, orc.singledroplet_1d(L, rads, 1 / 6, L // 2))
    _, A = s.run(10000, wetted=True)
    h = s.h
    c0, c1 = math.cos(math.pi / 6), math.cos(math.pi / 9)
    vol = math.pi / 3 * rads ** 3 * (2 + c0) * (1 - c0) ** 2
    R1 = ((rads ** 3 * (2 + c0) * (1 - c0) ** 2) / ((2 + c1) * (1 - c1) ** 2)) ** (1 / 3)
    r1 = math.sin(math.pi / 9) * R1
    thresh = 0.05026
    drop1d = np.nonzero(h > 0.055)[0]
    droprad = len(drop1d) / 2
    droph = h.max()
    vnum = 1 / 6 * math.pi * droph * (3 * droprad ** 2 + droph ** 2)
    ar = 2 / 3 * len(drop1d) * droph
    assert vnum == pytest.approx(vol, abs=vol / 10)
    assert np.sum(np.where(h > thresh, h, 0.0)) == pytest.approx(ar, abs=ar / 10)
    assert droprad == pytest.approx(r1, abs=r1 / 10)
    assert A[0] < A[-1]
