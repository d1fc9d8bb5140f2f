"""The 1D (D1Q3) solver on the GPU against the oracle (Float64 bit for bit)
and against the reference's 1D simulation tests (test/simulate.jl:3-94)."""
import math

import numpy as np
import pytest

import oracle
import swalbe_gb300 as sw

pytestmark = pytest.mark.gpu


def s1(L, **kw):
    return sw.SysConst_1D(L, sw.Taumucs(**kw))


def opar(s):
    p = s.param
    return oracle.params(s.L, 1, Tmax=p.Tmax, tdump=p.tdump, tau=p.tau, delta=p.delta, gamma=p.gamma,
                         n=p.n, m=p.m, hmin=p.hmin, hcrit=p.hcrit, theta=p.theta, g=p.g)


def film(L, seed, amp=0.05):
    rng = np.random.default_rng(seed)
    return 1.0 + amp * rng.uniform(-1, 1, L)


CASES = [
    dict(L=97, kw=dict(tau=0.8, delta=2.0, g=0.001), theta=False, gamma=False),
    dict(L=64, kw=dict(), theta=True, gamma=False),
    dict(L=200, kw=dict(n=3, m=2, hmin=0.07), theta=False, gamma=True),
    dict(L=3, kw=dict(tau=0.9), theta=False, gamma=False),
]


@pytest.mark.parametrize("case", CASES, ids=["tau0.8_g", "theta_field", "gamma_field", "L3"])
def test_f64_bit_exact(case):
    L = case["L"]
    s = s1(L, **case["kw"])
    h0 = film(L, L)
    th = 1 / 9 + 0.05 * np.sin(2 * np.pi * np.arange(L) / L) if case["theta"] else None
    gm = 0.01 + 0.002 * np.cos(2 * np.pi * np.arange(L) / L) if case["gamma"] else None
    st = sw.Sys(s, T=np.float64)
    st.height = h0
    if th is not None:
        st.set_theta(th)
    if gm is not None:
        st.set_gamma(gm)
    ref = oracle.State1D(opar(s), h0)
    for n in (1, 50, 149):
        st.step(n)
        ref.run(n, theta_field=th, gamma_field=gm)
    st.sync()
    assert np.array_equal(st.height, ref.h)
    assert np.array_equal(st.vel, ref.u)
    assert np.array_equal(st.fout, ref.fout)


def test_batch_of_lattices_f64():
    systems = [s1(50), s1(131, tau=0.7), s1(77, g=-0.002)]
    hs = [film(s.L, k) for k, s in enumerate(systems)]
    b = sw.Batch1D(systems, T=np.float64)
    for i, h in enumerate(hs):
        b.set_height(i, h)
    b.step(300)
    b.sync()
    for i, (s, h) in enumerate(zip(systems, hs)):
        ref = oracle.State1D(opar(s), h)
        ref.run(300)
        assert np.array_equal(b.height(i), ref.h), i


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_reference_1d_simulations(T):
    # test/simulate.jl:9-13
    h = sw.run_flat(s1(25, Tmax=200, tdump=100), verbos=False, T=T)
    assert np.all(h == 1.0) and np.sum(h) == 25
    # test/simulate.jl:24-27 (seeded random interface)
    h = sw.run_random(s1(25, Tmax=10000, tdump=5000), ϵ=0.1, verbos=False, T=T,
                      rng=np.random.default_rng(7))
    assert h.max() - h.min() < 0.02
    # test/simulate.jl:38-40
    _, diff = sw.run_rayleightaylor(s1(512, Tmax=1000, tdump=500, g=-0.002), k=4, ϵ=0.01,
                                    verbos=False, T=T)
    assert len(diff) == 1000 and diff[0] < diff[-1]
    # test/simulate.jl:63-90
    rads = 35
    h, A = sw.run_dropletrelax(s1(150, Tmax=10000, delta=3.0), radius=rads, verbos=False, T=T)
    c0, c1 = math.cos(math.pi / 6), math.cos(math.pi / 9)
    vol = math.pi / 3 * rads ** 3 * (2 + c0) * (1 - c0) ** 2
    R1 = ((rads ** 3 * (2 + c0) * (1 - c0) ** 2) / ((2 + c1) * (1 - c1) ** 2)) ** (1 / 3)
    r1 = math.sin(math.pi / 9) * R1
    drop1d = np.nonzero(h > 0.055)[0]
    droprad, droph = len(drop1d) / 2, h.max()
    vnum = 1 / 6 * math.pi * droph * (3 * droprad ** 2 + droph ** 2)
    ar = 2 / 3 * len(drop1d) * droph
    assert vnum == pytest.approx(vol, abs=vol / 10)
    assert np.sum(np.where(h > 0.05026, h, 0.0)) == pytest.approx(ar, abs=ar / 10)
    assert droprad == pytest.approx(r1, abs=r1 / 10)
    assert len(A) == 10000 and A[0] < A[-1]


def test_run_gamma_conserves_mass_and_matches_oracle():
    L, Tmax = 600, 3000
    s = s1(L, Tmax=Tmax, tdump=1000)
    gamma = 0.01 * (1 + 0.1 * np.sin(2 * np.pi * np.arange(L) / L))
    fluid = sw.run_gamma(s, gamma, r1=80, r2=80, θ0=1 / 9, verbos=False, dump=500)
    assert fluid.shape == (Tmax // 500, L)
    m = fluid.sum(axis=1)
    assert np.abs(m - m[0]).max() / m[0] < 1e-12
    h0 = sw.two_droplets(s, r1=80, r2=80, θ1=1 / 9, θ2=1 / 9)
    ref = oracle.State1D(opar(s), h0)
    ref.run(Tmax, gamma_field=gamma)
    assert np.array_equal(fluid[-1], ref.h)


def test_f32_close_to_f64():
    s = s1(300, Tmax=2000, delta=2.0)
    h0 = sw.singledroplet(np.zeros(300), 60, 1 / 6, 150)
    a = sw.Sys(s, T=np.float32)
    a.height = h0
    a.step(2000)
    ref = oracle.State1D(opar(s), h0)
    ref.run(2000)
    assert np.linalg.norm(a.height - ref.h) / np.linalg.norm(ref.h) < 1e-5
