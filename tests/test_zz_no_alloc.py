"""swb_measure_field_noalloc: measures of a device height field computed with
the library's fixed scratch array instead of allocated memory.

It exists for callers that must not allocate device memory (a host that has
committed its whole HBM budget, or whose own pool owns the device).  This
test checks it through the C ABI against swb_measure_now, the entry point
that uses a state's allocated scratch, on two calls in a row (the second
call reuses the array the first one left behind).  It is collected last so
that a run stopping at the first failure has run every other test already.
"""
import ctypes as C

import numpy as np
import pytest

import swalbe_gb300 as sw
from swalbe_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def _measure_noalloc(d_ptr, Lx, Ly, hthresh, cos_theta, d_cos=None, stream=None):
    m = L.Measure()
    st = sw.lib().swb_measure_field_noalloc(C.c_void_p(d_ptr), Lx, Ly, hthresh,
                                             None if d_cos is None else C.c_void_p(d_cos),
                                             cos_theta,
                                             None if stream is None else C.c_void_p(stream),
                                             C.byref(m))
    return st, m


def test_noalloc_matches_measure_now():
    torch = pytest.importorskip("torch")
    Lx, Ly, theta = 300, 211, 1 / 7
    h = sw.singledroplet(np.zeros((Lx, Ly)), 70, 1 / 5, (150, 100))
    h = np.asfortranarray(np.maximum(h, 0.05))
    st = sw.Sys(sw.SysConst(Lx, Ly, sw.Taumucs(theta=theta)), "GB300", T=np.float64)
    st.height = h
    st.set_theta(theta)
    ref = st.measure_now(0.055)
    d_h = torch.from_numpy(np.ascontiguousarray(h.ravel(order="F"))).to("cuda")
    torch.cuda.synchronize()
    for _ in range(2):
        rc, m = _measure_noalloc(d_h.data_ptr(), Lx, Ly, 0.055, sw.cospi(theta))
        assert rc == L.SWB_OK
        assert m.wetted == ref.wetted and m.hmax == ref.hmax and m.hmin == ref.hmin
        assert m.mass == pytest.approx(ref.mass, rel=1e-12)
        assert m.area == pytest.approx(ref.area, rel=1e-12)
        assert m.energy == pytest.approx(ref.energy, rel=1e-12)
    rc, _ = _measure_noalloc(d_h.data_ptr(), 20000, 20000, 0.055, 1.0)
    assert rc == L.SWB_ERR_ARG


def test_noalloc_theta_field_on_a_stream():
    """The per-cell cos θ branch, on a caller's stream: the energy of a θ
    field equals swb_measure_now's for the same field, on two calls in a row."""
    torch = pytest.importorskip("torch")
    Lx, Ly = 128, 96
    rng = np.random.default_rng(5)
    th = np.asfortranarray(1 / 9 + 0.05 * rng.uniform(-1, 1, (Lx, Ly)))
    h = np.asfortranarray(np.maximum(sw.singledroplet(np.zeros((Lx, Ly)), 40, 1 / 5, (64, 48)), 0.05))
    st = sw.Sys(sw.SysConst(Lx, Ly, sw.Taumucs()), "GB300", T=np.float64)
    st.height = h
    st.set_theta(th)
    ref = st.measure_now(0.055)
    cos = np.asfortranarray(np.vectorize(sw.cospi)(th))
    d_h = torch.from_numpy(np.ascontiguousarray(h.ravel(order="F"))).to("cuda")
    d_cos = torch.from_numpy(np.ascontiguousarray(cos.ravel(order="F"))).to("cuda")
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    for _ in range(2):
        rc, m = _measure_noalloc(d_h.data_ptr(), Lx, Ly, 0.055, 0.0, d_cos=d_cos.data_ptr(),
                                 stream=s.cuda_stream)
        assert rc == L.SWB_OK
        assert m.wetted == ref.wetted
        assert m.area == pytest.approx(ref.area, rel=1e-12)
        assert m.energy == pytest.approx(ref.energy, rel=1e-12)
    # host memory is refused before anything runs on the GPU
    rc, _ = _measure_noalloc(h.ctypes.data, Lx, Ly, 0.055, 0.0)
    assert rc == L.SWB_ERR_ARG
