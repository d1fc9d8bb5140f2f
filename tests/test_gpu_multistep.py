"""The multi-step (cooperative) launch form against one launch per iteration.

Both forms run the same step code with the same strip geometry, so heights,
velocities and every per-step measure must agree bit for bit, in FP32 and in
FP16 storage (whose FP64 mass correction is fed by the per-step reductions).
"""
import numpy as np
import pytest

import swalbe_gb300 as sw
from swalbe_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def sysc(Lx, Ly, **kw):
    return sw.SysConst(Lx, Ly, sw.Taumucs(**kw))


def film(Lx, Ly, seed=7, amp=0.1):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(1.0 + amp * rng.uniform(-1, 1, (Lx, Ly)))


def run(s, h0, mode, geometry, chunks, T, meas=L.MEAS_ALL, wave=None, edit=None):
    st = sw.Sys(s, "GB300", T=T)
    st.set_geometry(*geometry)
    st.set_step_mode(mode)
    assert st.step_mode() == mode
    st.set_measures(meas)
    if wave:
        st.set_theta_wave(*wave)
    st.height = h0
    for i, n in enumerate(chunks):
        st.step(n)
        if edit is not None and i == 0:
            h = st.height
            h[: h.shape[0] // 4, :] += 0.01
            st.height = h
    st.sync()
    recs = st.measures()
    return st.height, st.velx, st.vely, recs


def same(a, b):
    ha, ua, va, ra = a
    hb, ub, vb, rb = b
    assert np.array_equal(ha, hb)
    assert np.array_equal(ua, ub)
    assert np.array_equal(va, vb)
    assert len(ra) == len(rb)
    for x, y in zip(ra, rb):
        assert (x.t, x.mass, x.wetted, x.hmax, x.hmin, x.area, x.energy) == \
               (y.t, y.mass, y.wetted, y.hmax, y.hmin, y.area, y.energy)


@pytest.mark.parametrize("T", [np.float32, np.float16])
@pytest.mark.parametrize("geometry", [(64, 4), (128, 16), (32, 16)])
def test_multi_equals_per_iteration(T, geometry):
    # 1500 iterations cross the 1024-iteration launch boundary; the chunks
    # exercise resumption and a partial graph
    s = sysc(150, 97, tau=0.9, delta=2.0)
    h0 = film(150, 97)
    chunks = (1, 700, 799)
    a = run(s, h0, "multi", geometry, chunks, T)
    b = run(s, h0, "per_iteration", geometry, chunks, T)
    same(a, b)
    assert len(a[3]) == sum(chunks)


@pytest.mark.parametrize("T", [np.float32, np.float16])
def test_multi_equals_per_iteration_wave_and_edit(T):
    s = sysc(128, 64, Tmax=400, g=-0.0005)
    h0 = film(128, 64, seed=9)
    wave = (1 / 9, 1 / 36, 1 / 98)
    for geo in ((64, 8), (32, 16)):
        a = run(s, h0, "multi", geo, (200, 200), T, wave=wave, edit=True)
        b = run(s, h0, "per_iteration", geo, (200, 200), T, wave=wave, edit=True)
        same(a, b)


def test_multi_more_strips_than_resident_ctas():
    # 1024² at strips of 60x4: 18 x 256 = 4608 strips, more than the GPU
    # holds at once, so each CTA walks several strips per iteration
    s = sysc(1024, 1024)
    h0 = film(1024, 1024, seed=11)
    a = run(s, h0, "multi", (64, 4), (40,), np.float32, meas=L.MEAS_MASS | L.MEAS_MAXMIN)
    b = run(s, h0, "per_iteration", (64, 4), (40,), np.float32, meas=L.MEAS_MASS | L.MEAS_MAXMIN)
    same(a, b)


def test_step_mode_rules():
    s = sysc(64, 64)
    st = sw.Sys(s, "GB300", T=np.float64)
    with pytest.raises(sw.SwbError):
        st.set_step_mode("multi")
    assert st.step_mode() == "per_iteration"
    st32 = sw.Sys(s, "GB300", T=np.float32)
    assert st32.step_mode() == "per_iteration"  # default without the tuner
    st32.set_step_mode("per_iteration")
    assert st32.step_mode() == "per_iteration"
    st32.set_step_mode("multi")
    with pytest.raises(sw.SwbError):
        st32.set_geometry(256, 16)
    st32.set_geometry(32, 0)  # 2D tiles of 32 x 16 cells
    assert st32.geometry() == (32, 16)
    with pytest.raises(sw.SwbError):
        st.set_geometry(32, 16)  # Float64: strips only
    st32.set_step_mode("auto")
    assert st32.step_mode() == "per_iteration"


@pytest.mark.parametrize("T", [np.float32, np.float16])
def test_tiles_equal_strips(T):
    """2D tiles and strips run the same per-cell code: FP32 heights and
    velocities agree bit for bit (only the order of the mass partial sums
    differs, which in FP16 storage feeds the mass correction)."""
    s = sysc(150, 97, tau=0.8, delta=2.0, g=-0.0002)
    h0 = film(150, 97, seed=5)
    wave = (1 / 9, 1 / 36, 1 / 98)
    a = run(s, h0, "per_iteration", (32, 16), (300,), T, wave=wave)
    b = run(s, h0, "per_iteration", (64, 8), (300,), T, wave=wave)
    if T == np.float32:
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        assert [r.wetted for r in a[3]] == [r.wetted for r in b[3]]
        ma = np.array([r.mass for r in a[3]]); mb = np.array([r.mass for r in b[3]])
        assert np.abs(ma - mb).max() <= 1e-12 * ma.max()
    else:
        assert np.abs(a[0] - b[0]).max() < 1e-5


@pytest.mark.parametrize("L", [(1, 24), (24, 2), (33, 17), (5, 5)])
def test_tiles_small_and_ragged(L):
    """Lattices thinner than a tile (wrapping halos) and ragged edges."""
    Lx, Ly = L
    s = sysc(Lx, Ly, tau=0.9)
    h0 = film(Lx, Ly, seed=2, amp=0.05)
    a = run(s, h0, "multi", (32, 16), (37,), np.float32)
    b = run(s, h0, "per_iteration", (64, 4), (37,), np.float32)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


# ------------------------------------------------------------------ resident tiles
def _run_form(s, h0, steps, T, geo, chunks=3, wave=None):
    st = sw.Sys(s, "GB300", T=T)
    st.set_geometry(*geo)
    st.set_measures(L.MEAS_ALL)
    if wave:
        st.set_theta_wave(*wave)
    st.height = h0
    done = 0
    for c in range(chunks):
        n = (steps - done) if c == chunks - 1 else steps // chunks
        st.step(n)
        done += n
    st.sync()
    return st, st.height, st.measures_array(cap=steps)


@pytest.mark.parametrize("T", [np.float32, np.float16])
def test_resident_tiles_equal_strips(T):
    """Resident tiles (populations kept in shared memory across iterations of
    one cooperative launch, a 3-cell ring exchanged through L2) give the bits
    of the strips: heights and every per-step measure, on lattices with full
    and partial tiles, narrower than a tile, and more iterations than one
    launch takes."""
    cases = [(512, 512, 300), (96, 64, 200), (48, 40, 1500), (130, 34, 200), (256, 256, 120)]
    for Lx, Ly, steps in cases:
        s = sw.SysConst(Lx, Ly, sw.Taumucs(delta=2.0))
        h0 = np.asfortranarray(1.0 + 0.1 * np.random.default_rng(Lx + Ly).uniform(-1, 1, (Lx, Ly)))
        _, h_ref, r_ref = _run_form(s, h0, steps, T, (64, 8))
        for geo in (33, 34):  # one CTA of 512 threads per SM, or two of 256
            st, h, r = _run_form(s, h0, steps, T, (geo, 0))
            assert st.geometry()[0] == geo and st.step_mode() == "multi", (Lx, Ly)
            assert np.array_equal(h, h_ref), (Lx, Ly, geo)
            for f in ("t", "mass", "wetted", "hmax", "hmin", "area", "energy"):
                assert np.array_equal(r[f], r_ref[f]), (Lx, Ly, geo, f)


def test_resident_tiles_fallback_and_rules():
    """A resident-tile state whose iterations need another form (a θ wave)
    runs them one launch each, on strips: same results; Float64 and lattices
    too large for the GPU's shared memory are refused."""
    s = sw.SysConst(96, 64, sw.Taumucs())
    h0 = np.asfortranarray(1.0 + 0.1 * np.random.default_rng(1).uniform(-1, 1, (96, 64)))
    wave = (1 / 9, 1 / 36, 1 / 98)
    _, h_ref, _ = _run_form(s, h0, 100, np.float32, (64, 8), wave=wave)
    _, h, _ = _run_form(s, h0, 100, np.float32, (33, 0), wave=wave)
    assert np.array_equal(h, h_ref)
    with pytest.raises(sw.SwbError):
        sw.Sys(s, "GB300", T=np.float64).set_geometry(33, 0)
    with pytest.raises(sw.SwbError):
        sw.Sys(sw.SysConst(2048, 2048, sw.Taumucs()), "GB300", T=np.float32).set_geometry(33, 0)
