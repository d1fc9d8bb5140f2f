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
    Lx, Ly = 40, 28
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
    Lx, Ly = 96, 64
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
