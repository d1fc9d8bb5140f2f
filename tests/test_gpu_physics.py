"""The reference's simulation tests (test/simulate.jl) on the GPU, through the
same drivers a user calls: run_flat, run_random, run_rayleightaylor,
run_dropletrelax, run_dropletpatterned, run_dropletforced with device "GB300",
in Float64 and in the FP32 / FP16-storage modes."""
import math

import numpy as np
import pytest

import swalbe_gb300 as sw

pytestmark = pytest.mark.gpu

MODES = [np.float64, np.float32, np.float16]


def sysc(L, **kw):
    return sw.SysConst(L, L, sw.Taumucs(**kw))


@pytest.mark.parametrize("T", MODES)
def test_flat_interface(T):
    # test/simulate.jl:3-7: all(h .== 1.0) and sum(h) == 625, bit for bit
    h = sw.run_flat(sysc(25, Tmax=200, tdump=100), "GB300", verbos=False, T=T)
    assert np.all(h == 1.0)
    assert np.sum(h) == 625


@pytest.mark.parametrize("T", MODES)
def test_random_interface(T):
    # test/simulate.jl:16-21
    h = sw.run_random(sysc(25, Tmax=10000, tdump=5000), "GB300", ϵ=0.1, verbos=False, T=T,
                      rng=np.random.default_rng(11))
    assert h.max() - h.min() < 0.1


@pytest.mark.parametrize("T", MODES)
def test_rayleigh_taylor(T):
    # test/simulate.jl:32-35
    _, diff = sw.run_rayleightaylor(sysc(100, Tmax=1000, tdump=500, g=-0.002), "GB300", kx=4,
                                    ky=5, ϵ=0.01, verbos=False, T=T)
    assert len(diff) == 1000
    assert diff[0] < diff[-1]


def droplet_checks(h, R=35, th0=1 / 6, th=1 / 9):
    c0, c1 = math.cos(math.pi * th0), math.cos(math.pi * th)
    vol = math.pi / 3 * R ** 3 * (2 + c0) * (1 - c0) ** 2
    R1 = ((R ** 3 * (2 + c0) * (1 - c0) ** 2) / ((2 + c1) * (1 - c1) ** 2)) ** (1 / 3)
    r1 = math.sin(math.pi * th) * R1
    drop1d = np.nonzero(h[74, :] > 0.055)[0]
    droprad = len(drop1d) / 2
    droph = h.max()
    vnum = 1 / 6 * math.pi * droph * (3 * droprad ** 2 + droph ** 2)
    assert vnum == pytest.approx(vol, abs=vol / 10)
    assert droprad == pytest.approx(r1, abs=r1 / 10)


@pytest.mark.parametrize("T", MODES)
def test_droplet_relax(T):
    # test/simulate.jl:42-60
    h, A = sw.run_dropletrelax(sysc(150, Tmax=10000, delta=3.0), "GB300", radius=35,
                               verbos=False, T=T)
    droplet_checks(h)
    assert len(A) == 10000 and A[0] < A[-1]


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_droplet_patterned(T):
    # test/simulate.jl:96-112
    h = sw.run_dropletpatterned(sysc(150, Tmax=10000, delta=3.0), "GB300", radius=35,
                                θₛ=np.full((150, 150), 1 / 9), verbos=False, T=T)
    droplet_checks(h)


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_droplet_forced(T):
    # test/simulate.jl:146-155: the maximum moves in x, not in y; |u| < 0.1
    h, u, v = sw.run_dropletforced(sysc(150, Tmax=5000, delta=2.0), "GB300", radius=35, fx=1e-4,
                                   verbos=False, T=T)
    ix, iy = np.unravel_index(np.argmax(h), h.shape)
    assert ix + 1 != 75 and iy + 1 == 75
    assert np.all(u < 0.1) and np.all(v < 0.1)


def test_plain_path_drivers_agree_with_fused():
    """The plain per-op path and the fused path give the same Float64 result."""
    s = sysc(64, Tmax=300, delta=3.0)
    a, _ = sw.run_dropletrelax(s, "GB300", radius=15, verbos=False)
    b, _ = sw.run_dropletrelax(s, "GB300-plain", radius=15, verbos=False)
    assert np.array_equal(a, b)
