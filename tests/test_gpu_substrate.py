"""Patterned and moving substrates on the GPU: a θ field from the pattern
generators (src/initialvalues.jl:423-581) and move_substrate!
(scripts/Moving_wettability_structs.jl:139-152), against the oracle."""
import numpy as np
import pytest

import oracle
import swalbe_gb300 as sw

pytestmark = pytest.mark.gpu


def film(Lx, Ly, seed=3, amp=0.05):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(1.0 + amp * rng.uniform(-1, 1, (Lx, Ly)))


@pytest.mark.parametrize("device", ["GB300", "GB300-plain"])
@pytest.mark.parametrize("direction,dxy", [("diagonal", (1, 1)), ("x", (1, 0)), ("y", (0, 1))])
def test_moving_field_f64_bit_exact(device, direction, dxy):
    # the reference's pattern generators index θ[j, i]: square lattices only
    Lx, Ly = 36, 36
    th, _ = sw.boxpattern(np.ones((Lx, Ly)), 1 / 9, side=10, δa=1 / 18)
    h0 = film(Lx, Ly)
    s = sw.SysConst(Lx, Ly, sw.Taumucs())
    st = sw.Sys(s, device, T=np.float64)
    st.set_theta(th)
    st.move_substrate(7, direction)
    st.height = h0
    lit = oracle.LiteralState(oracle.params(Lx, Ly))
    lit.field("height")[:] = h0
    for n in (1, 20, 29):
        st.step(n)
        ref = lit.run(n, theta_field=th, motion=(7,) + dxy)
    assert np.array_equal(st.height, ref.height)
    # the motion matters
    still = oracle.FusedState(oracle.params(Lx, Ly), h0).run(50, theta_field=th)
    assert not np.array_equal(st.height, still.height)


def test_moving_field_forms_agree_f32():
    Lx, Ly = 96, 96
    th, _ = sw.trianglepattern(np.ones((Lx, Ly)), 1 / 9, side=30)
    h0 = film(Lx, Ly, 5)
    s = sw.SysConst(Lx, Ly, sw.Taumucs())
    out = []
    for geo, mode in (((64, 8), "per_iteration"), ((32, 16), "per_iteration"), ((64, 8), "multi")):
        st = sw.Sys(s, "GB300", T=np.float32)
        st.set_geometry(*geo)
        st.set_step_mode(mode)
        st.set_theta(th)
        st.move_substrate(11, "x")
        st.height = h0
        st.step(300)
        out.append(st.height)
    assert np.array_equal(out[0], out[1]) and np.array_equal(out[0], out[2])
    ref = oracle.FusedState(oracle.params(Lx, Ly), h0).run(300, theta_field=th, motion=(11, 1, 0))
    assert np.linalg.norm(out[0] - ref.height) / np.linalg.norm(ref.height) < 1e-5


def test_motion_needs_a_field():
    st = sw.Sys(sw.SysConst(16, 16, sw.Taumucs()), "GB300", T=np.float32)
    with pytest.raises(sw.SwbError):
        st.move_substrate(5)


@pytest.mark.parametrize("device", ["GB300", "GB300-plain"])
def test_device_snapshots_f64(device):
    """snapshot! every 7 iterations into the device ring, against the literal
    oracle's heights at t = 7, 14, 21, 28."""
    Lx, Ly = 30, 22
    h0 = film(Lx, Ly, 8)
    st = sw.Sys(sw.SysConst(Lx, Ly, sw.Taumucs()), device, T=np.float64)
    st.set_snapshots(7, capacity=8)
    st.height = h0
    for n in (5, 13, 12):
        st.step(n)
    times, rows = st.snapshots()
    assert times == [7, 14, 21, 28]
    lit = oracle.LiteralState(oracle.params(Lx, Ly))
    lit.field("height")[:] = h0
    for k, t in enumerate(times):
        ref = lit.run(7)
        assert np.array_equal(rows[k].reshape((Lx, Ly), order="F"), ref.height), t
    assert st.snapshots()[0] == []  # all read


def test_device_snapshot_ring_keeps_newest():
    Lx = Ly = 24
    st = sw.Sys(sw.SysConst(Lx, Ly, sw.Taumucs()), "GB300", T=np.float32)
    st.set_snapshots(5, capacity=2)
    st.height = film(Lx, Ly, 9)
    st.step(22)  # snapshots at 5, 10, 15, 20
    times, rows = st.snapshots()
    assert times == [15, 20]
    st.step(3)
    times, rows = st.snapshots()
    assert times == [25] and np.array_equal(rows[0].reshape((Lx, Ly), order="F"), st.height)
