"""GPU parity of the surface measures: surfacearea!'s area and energy
(src/measures.jl:126-168 with ∇f_simple!, :175-192) as the fused step records
them every iteration, and swb_measure_now, against the oracle.

The fused step measures the height each iteration starts from: record t
holds the measures of the height after t - 1 iterations, with the θ that
iteration t uses (a moving θ field at its offset of iteration t, the θ wave
at time t).  The tests read that height back from the GPU and give it to the
oracle's surfacearea (Float64, long-double sums), so that only the measure
itself is compared:

* Float64: area and energy within 1e-12 relative (the GPU sums per CTA, the
  oracle in one long-double pass), wetted count exact;
* FP32 arithmetic (FP32 and FP16 storage): each cell's surface element and
  cos θ are FP32 values summed in fixed point (2^-32 per cell), so area and
  energy agree within 2e-6 of the area, wetted count exact.
"""
import numpy as np
import pytest

import oracle
import swalbe_gb300 as sw
from swalbe_gb300 import _lib as L

pytestmark = pytest.mark.gpu

Lx, Ly = 48, 40
TH0, DTH, V = 1 / 9, 1 / 36, 1 / 98
TOL = {np.float64: 1e-12, np.float32: 2e-6, np.float16: 2e-6}


def droplet():
    return oracle.singledroplet(Lx, Ly, 12, 1 / 6, (Lx // 2, Ly // 2))


def theta_field():
    rng = np.random.default_rng(41)
    return np.asfortranarray(1 / 9 + 0.04 * rng.uniform(-1, 1, (Lx, Ly)))


def wave_at(t):
    """θ(x, t) = θ0 + Δθ sinpi(2 (x - v t) / Lx), x the 0-based column."""
    x = np.arange(Lx, dtype=np.float64)
    th = TH0 + DTH * np.sin(np.pi * (2.0 * (x - V * t) / Lx))
    return np.asfortranarray(np.repeat(th[:, None], Ly, axis=1))


def moved(field, t, tmove, t0=0):
    """The diagonal move_substrate! offset of iteration t (1-based)."""
    k = (t - 1 - t0) // tmove if t - 1 - t0 >= tmove else 0
    return np.asfortranarray(np.roll(field, (k % Lx, k % Ly), axis=(0, 1)))


def make_state(T, mode, device="GB300"):
    s = sw.SysConst(Lx, Ly, sw.Taumucs(theta=TH0))
    st = sw.Sys(s, device, T=T)
    st.height = droplet()
    if mode in ("field", "moving"):
        st.set_theta(theta_field())
        if mode == "moving":
            st.move_substrate(3, "diagonal")
    elif mode == "wave":
        st.set_theta_wave(TH0, DTH, V)
    st.set_measures(L.MEAS_ALL)
    return st


def theta_of_record(mode, t):
    if mode == "scalar":
        return TH0
    if mode == "field":
        return theta_field()
    if mode == "moving":
        return moved(theta_field(), t, 3)
    return wave_at(t)


MODES = ["scalar", "field", "moving", "wave"]


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("T", [np.float64, np.float32, np.float16])
def test_step_records_area_energy_vs_oracle(T, mode):
    st = make_state(T, mode)
    k = 57
    st.step(k - 1)
    h = st.height  # the height iteration k starts from
    st.step(1)
    st.sync()
    rec = st.measures()[-1]
    assert rec.t == k
    area, energy = oracle.surfacearea(h, theta_of_record(mode, k))
    assert rec.wetted == oracle.wetted(h)
    tol = TOL[T]
    assert abs(rec.area - area) <= tol * area, (rec.area, area)
    assert abs(rec.energy - energy) <= tol * area, (rec.energy, energy)


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_measure_now_equals_next_record(T, mode):
    """measure_now of the current height uses the θ of the next iteration,
    so it equals that iteration's own record (moving field and wave too)."""
    st = make_state(T, mode)
    st.step(40)
    h = st.height
    m = st.measure_now()
    st.step(1)
    st.sync()
    rec = st.measures()[-1]
    assert rec.t == 41
    assert m.wetted == rec.wetted
    assert m.hmax == rec.hmax and m.hmin == rec.hmin
    # Float64: the same per-cell values summed in another order; FP32: the
    # same FP32 per-cell values, Float64 sums against fixed-point sums
    tol = 1e-13 if T == np.float64 else 1e-9
    assert abs(m.area - rec.area) <= tol * rec.area
    assert abs(m.energy - rec.energy) <= tol * rec.area
    area, energy = oracle.surfacearea(h, theta_of_record(mode, 41))
    assert abs(m.energy - energy) <= TOL[T] * area


@pytest.mark.parametrize("mode", ["scalar", "field", "moving"])
def test_plain_records_area_energy_vs_oracle(mode):
    """The per-op Float64 path records the same measures, with the θ field
    (moving or not) in the energy term."""
    st = make_state(np.float64, mode, device="GB300-plain")
    k = 23
    st.step(k - 1)
    h = st.height
    st.step(1)
    rec = st.measures()[-1]
    assert rec.t == k
    area, energy = oracle.surfacearea(h, theta_of_record(mode, k))
    assert rec.wetted == oracle.wetted(h)
    assert abs(rec.area - area) <= 1e-12 * area
    assert abs(rec.energy - energy) <= 1e-12 * area
    h2 = st.height
    m = st.measure_now()
    area2, energy2 = oracle.surfacearea(h2, theta_of_record(mode, k + 1))
    assert abs(m.energy - energy2) <= 1e-12 * area2
