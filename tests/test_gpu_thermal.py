"""Thermal fluctuations (src/forcing.jl:297-320) on the GPU.

The reference pins thermal! only statistically (test/forcing.jl:141-164);
here the GPU and the oracle share the counter-based generator, so the
Float64 mode is also compared value by value (the normals' log/cos differ by
at most an ulp between the device and the host libm)."""
import numpy as np
import pytest

import oracle
import swalbe_gb300 as sw
from swalbe_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def sysc(L_, **kw):
    return sw.SysConst(L_, L_, sw.Taumucs(**kw))


def film(L_, seed=3, amp=0.05):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(1.0 + amp * rng.uniform(-1, 1, (L_, L_)))


@pytest.mark.parametrize("T", [np.float64, np.float32, np.float16])
@pytest.mark.parametrize("kb", [0.01, 0.1])
def test_field_statistics_like_reference(T, kb):
    # test/forcing.jl:151-162: 50x50, h = 1, μ = 1/6, δ = 1
    st = sw.Sys(sysc(50, kbt=kb), "GB300", T=T, kind="thermal")
    var = 2 * kb / 11
    for t in (1, 2, 1000):
        fx, fy = st.thermal_field(t)
        for f in (fx, fy):
            assert np.mean(f) == pytest.approx(0.0, abs=1e-2)
            assert np.var(f, ddof=1) == pytest.approx(var, abs=var / 10)


def test_field_f64_matches_oracle():
    st = sw.Sys(sysc(64, kbt=0.05, delta=2.0), "GB300", T=np.float64, kind="thermal")
    st.set_thermal_seed(77)
    h = film(64, 4, 0.3)
    st.height = h
    fx, fy = st.thermal_field(123)
    ox, oy = oracle.thermal(h, 0.05, 1 / 6, 2.0, seed=77, t=123)
    assert np.allclose(fx, ox, rtol=1e-13, atol=1e-16)
    assert np.allclose(fy, oy, rtol=1e-13, atol=1e-16)
    # FP32 draws its normals from the same Philox words in single precision
    s32 = sw.Sys(sysc(64, kbt=0.05, delta=2.0), "GB300", T=np.float32, kind="thermal")
    s32.set_thermal_seed(77)
    s32.height = h
    gx, _ = s32.thermal_field(123)
    assert np.median(np.abs(gx - ox)) < 1e-5 * np.std(ox)


def test_f64_run_matches_oracle_and_plain():
    L_, n = 48, 60
    s = sysc(L_, kbt=1e-4, delta=2.0, tau=0.9)
    h0 = film(L_)
    a = sw.Sys(s, "GB300", T=np.float64, kind="thermal")
    a.set_thermal_seed(5)
    a.height = h0
    a.step(n)
    b = sw.Sys(s, "GB300-plain", T=np.float64, kind="thermal")
    b.set_thermal_seed(5)
    b.height = h0
    b.step(n)
    assert np.array_equal(a.height, b.height)  # same device arithmetic, op by op
    P = oracle.params(L_, L_, kbt=1e-4, delta=2.0, tau=0.9)
    ref = oracle.FusedState(P, h0).run(n, seed=5)
    assert np.allclose(a.height, ref.height, rtol=1e-11, atol=0)
    # and the noise matters: without it the film differs
    c = sw.Sys(sysc(L_, delta=2.0, tau=0.9), "GB300", T=np.float64)
    c.height = h0
    c.step(n)
    assert np.abs(c.height - a.height).max() > 1e-9


def test_simple_kind_ignores_kbt():
    # a "simple" State has no fluctuation fields (src/initialize.jl:491-536)
    L_ = 32
    h0 = film(L_)
    a = sw.Sys(sysc(L_, kbt=1e-3), "GB300", T=np.float64)
    b = sw.Sys(sysc(L_), "GB300", T=np.float64)
    for st in (a, b):
        st.height = h0
        st.step(20)
    assert np.array_equal(a.height, b.height)


@pytest.mark.parametrize("T", [np.float32, np.float16])
def test_thermal_forms_and_mass(T):
    L_, n = 96, 400
    s = sysc(L_, kbt=1e-5)
    h0 = film(L_, 9, 0.01)
    outs = []
    for mode in ("per_iteration", "multi"):
        st = sw.Sys(s, "GB300", T=T, kind="thermal")
        st.set_geometry(64, 8)
        st.set_step_mode(mode)
        st.set_measures(L.MEAS_MASS)
        st.height = h0
        st.step(n)
        outs.append((st.height, [r.mass for r in st.measures()]))
    assert np.array_equal(outs[0][0], outs[1][0])
    m = np.array(outs[0][1])
    assert np.abs(m - m[0]).max() / m[0] < (1e-10 if T == np.float32 else 2e-8)
    assert outs[0][0].std() > h0.std() * 0.5  # the film fluctuates


def test_batch_lattice_seed_is_its_index():
    systems = [sysc(40, kbt=1e-5), sysc(56, kbt=2e-5)]
    hs = [film(40, 1), film(56, 2)]
    b = sw.Batch(systems, T=np.float32)
    for i, h in enumerate(hs):
        b.set_height(i, h)
    b.step(77)
    b.sync()
    for i, (s, h) in enumerate(zip(systems, hs)):
        st = sw.Sys(s, "GB300", T=np.float32, kind="thermal")
        st.set_thermal_seed(i)
        st.height = h
        st.step(77)
        assert np.array_equal(b.get_height(i), st.height)
    b.close()
