"""One-dimensional thin films: the D1Q3 solver of Swalbe.jl on the GPU.

Mirrors the reference's 1D API: ``SysConst_1D`` (src/initialize.jl:96-100),
``Sys(sysc::SysConst_1D; T, kind)`` (src/initialize.jl:587-616), the 1D
``time_loop`` methods (src/simulate.jl:98-179), the 1D drivers and
``run_gamma`` (src/simulate.jl:247-560), ``two_droplets``
(src/initialvalues.jl:277-323).  A state is one lattice of a ``Batch1D``;
many 1D simulations run together, one CTA each, in one launch per call.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence

import numpy as np

from . import _lib as L
from ._lib import check, lib

FIELD_THETA, FIELD_GAMMA = 20, 21


class SysConst_1D:
    """SysConst_1D{T}(L, param) (src/initialize.jl:96-100)."""

    def __init__(self, L: int = 256, param=None):
        from .api import Taumucs
        self.L = int(L)
        self.param = param if param is not None else Taumucs()

    def c_params(self) -> L.Params:
        p = self.param
        return L.Params(self.L, 1, p.Tmax, p.tdump, p.tau, p.cs, p.mu, p.delta, p.kbt, p.gamma,
                        p.n, p.m, p.hmin, p.hcrit, p.theta, p.g)


def _prec(T) -> int:
    T = np.dtype(T).type
    if T is np.float64:
        return L.SWB_F64
    if T is np.float32:
        return L.SWB_F32
    raise ValueError("1D states: T = Float64 or Float32")


class Batch1D:
    """Many 1D lattices advanced together (one CTA per lattice)."""

    def __init__(self, systems: Sequence[SysConst_1D], T=np.float64, records: int = 0):
        self.systems = list(systems)
        arr = (L.Params * len(self.systems))(*[s.c_params() for s in self.systems])
        h = C.c_void_p()
        check(lib().swb1d_create(arr, len(self.systems), _prec(T), int(records), C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().swb1d_destroy(h)
            except Exception:
                pass
            self._h = None

    close = __del__

    def _set(self, i, field, values):
        n = self.systems[i].L
        a = None if values is None else np.ascontiguousarray(
            np.broadcast_to(np.asarray(values, dtype=np.float64), (n,)))
        check(lib().swb1d_set_field(self._h, i, field, None if a is None else a.ctypes.data))

    def _get(self, i, field, n):
        out = np.empty(n)
        check(lib().swb1d_get_field(self._h, i, field, out.ctypes.data))
        return out

    def set_height(self, i, h):
        self._set(i, L.FIELD_HEIGHT, h)

    def set_vel(self, i, u):
        self._set(i, L.FIELD_VELX, u)

    def set_theta(self, i, theta):
        """θ field (an array), a constant θ, or None (the params' θ)."""
        self._set(i, FIELD_THETA, theta)

    def set_gamma(self, i, gamma):
        """γ field: surface tension per cell, and the ∇γ force (run_gamma)."""
        self._set(i, FIELD_GAMMA, gamma)

    def height(self, i):
        return self._get(i, L.FIELD_HEIGHT, self.systems[i].L)

    def vel(self, i):
        return self._get(i, L.FIELD_VELX, self.systems[i].L)

    def pressure(self, i):
        return self._get(i, L.FIELD_PRESSURE, self.systems[i].L)

    def fout(self, i):
        n = self.systems[i].L
        return self._get(i, L.FIELD_FOUT, 3 * n).reshape((n, 3), order="F")

    def step(self, n: int) -> None:
        check(lib().swb1d_step(self._h, int(n)))

    def sync(self) -> None:
        check(lib().swb1d_sync(self._h))

    def measures(self, i, cap: int = 1 << 16):
        buf = (L.Measure * cap)()
        n = C.c_int64()
        check(lib().swb1d_get_measures(self._h, i, buf, cap, C.byref(n)))
        return list(buf[: n.value])


class State1D:
    """Sys(sysc::SysConst_1D; T, kind="simple"): one 1D lattice on the GPU.
    ``height``, ``vel`` read and write the device fields; ``fout`` is the
    reference's streamed populations (L x 3)."""

    def __init__(self, sysc: SysConst_1D, T=np.float64, records: int = 1 << 16):
        self.sys = sysc
        self.T = T
        self._b = Batch1D([sysc], T, records)
        self._records = records

    @property
    def height(self):
        return self._b.height(0)

    @height.setter
    def height(self, h):
        self._b.set_height(0, h)

    @property
    def vel(self):
        return self._b.vel(0)

    @vel.setter
    def vel(self, u):
        self._b.set_vel(0, u)

    @property
    def pressure(self):
        return self._b.pressure(0)

    @property
    def fout(self):
        return self._b.fout(0)

    def set_theta(self, theta):
        self._b.set_theta(0, theta)

    def set_gamma(self, gamma):
        self._b.set_gamma(0, gamma)

    def step(self, n: int) -> None:
        self._b.step(n)

    def sync(self) -> None:
        self._b.sync()

    def measures(self, cap: int = 1 << 16):
        return self._b.measures(0, cap)


def time_loop(sysc: SysConst_1D, state: State1D, *args, verbose: bool = False):
    """time_loop(sys::SysConst_1D, state[, θ | Δh | f, measure])
    (src/simulate.jl:98-179); ``wetted_`` is the callback that runs fused."""
    from .api import wetted_
    P = sysc.param
    dh = measure = None
    state.set_theta(None)
    if len(args) == 1 and isinstance(args[0], list):
        dh = args[0]
    elif len(args) == 1:
        state.set_theta(args[0])
    elif len(args) == 2:
        f, measure = args
        if f is not wetted_:
            raise NotImplementedError("1D states fuse the wetted_ callback only")
    elif args:
        raise TypeError("time_loop(sys, state[, θ | Δh | f, measure])")
    state.step(P.Tmax)
    state.sync()
    if dh is not None or measure is not None or verbose:
        recs = state.measures(cap=max(P.Tmax, 1))
        if len(recs) < P.Tmax and (dh is not None or measure is not None):
            raise RuntimeError("more iterations than the state's measure records hold")
        for r in recs:
            if verbose and P.tdump > 0 and r.t % P.tdump == 0:
                print(f"Time step {r.t} mass is {round(r.mass, 3)}")
            if dh is not None:
                dh.append(r.hmax - r.hmin)
            if measure is not None:
                measure.append(int(r.wetted))
    if measure is not None:
        return state, measure
    return state


def singledroplet_1d(height: np.ndarray, radius, θ, center, hcrit=0.05) -> np.ndarray:
    """singledroplet(height::Vector, radius, θ, center; hcrit) (src/initialvalues.jl:226-243)."""
    from .api import cospi
    n = height.shape[0]
    i = np.arange(1, n + 1)
    circ = np.sqrt((i - center) ** 2.0)
    cap = (np.cos(np.arcsin(np.minimum(circ / radius, 1.0))) - cospi(θ)) * radius
    h = np.where(circ <= radius, cap, hcrit)
    height[:] = np.where(h <= hcrit, hcrit, h)
    return height


def two_droplets(sysc: SysConst_1D, r1=230, r2=230, θ1=1 / 9, θ2=1 / 9, center=None):
    """two_droplets(sys; r₁, r₂, θ₁, θ₂, center) (src/initialvalues.jl:277-323)."""
    from .api import cospi
    Lx = sysc.L
    c = (Lx / 3, 2 * Lx / 3) if center is None else center
    i = np.arange(1, Lx + 1)

    def cap(cc, r, th):
        circ = np.sqrt((i - cc) ** 2.0)
        d = np.where(circ <= r, (np.cos(np.arcsin(np.minimum(circ / r, 1.0))) - cospi(th)) * r, 0.05)
        return np.where(d < 0, 0.05, d)

    h = cap(c[0], r1, θ1) + cap(c[1], r2, θ2) - 0.05
    return np.where(h < 0, 0.05, h)


# ---------------------------------------------------------------- drivers
def run_flat(sysc: SysConst_1D, verbos=True, T=np.float64):
    """run_flat(sys::SysConst_1D) (src/simulate.jl:247-256)."""
    st = State1D(sysc, T)
    st.height = np.ones(sysc.L)
    time_loop(sysc, st, verbose=verbos)
    return st.height


def run_random(sysc: SysConst_1D, h0=1.0, ϵ=0.01, verbos=True, T=np.float64, rng=None):
    """run_random(sys::SysConst_1D; h₀, ϵ) (src/simulate.jl:296-303); the
    random interface comes from a seeded numpy generator (Julia's randn
    stream cannot be reproduced)."""
    rng = np.random.default_rng(0) if rng is None else rng
    st = State1D(sysc, T)
    st.height = h0 * (1.0 + ϵ * rng.standard_normal(sysc.L))
    time_loop(sysc, st, 1 / 9, verbose=verbos)
    return st.height


def run_rayleightaylor(sysc: SysConst_1D, k=15, h0=1.0, ϵ=0.001, verbos=True, T=np.float64):
    """run_rayleightaylor(sys::SysConst_1D; k, h₀, ϵ) (src/simulate.jl:360-377)."""
    st = State1D(sysc, T)
    i = np.arange(1, sysc.L + 1)
    st.height = h0 * (1 + ϵ * np.sin(2 * np.pi * k * i / (sysc.L - 1)))
    diff: List[float] = []
    time_loop(sysc, st, diff, verbose=verbos)
    return st.height, diff


def run_dropletrelax(sysc: SysConst_1D, radius=20, θ0=1 / 6, center=None, verbos=True,
                     T=np.float64):
    """run_dropletrelax(sys::SysConst_1D; radius, θ₀, center) (src/simulate.jl:401-416)."""
    from .api import wetted_
    c = sysc.L // 2 if center is None else center
    st = State1D(sysc, T)
    st.height = singledroplet_1d(np.zeros(sysc.L), radius, θ0, c)
    area: List[int] = []
    time_loop(sysc, st, wetted_, area, verbose=verbos)
    return st.height, area


def run_gamma(sysc: SysConst_1D, gamma, r1=115, r2=115, θ0=1 / 9, verbos=True, dump=100,
              fluid=None, T=np.float64):
    """run_gamma(sys::SysConst_1D, gamma; r₁, r₂, θ₀, dump, fluid)
    (src/simulate.jl:518-556): coalescing droplets on a surface-tension
    gradient; returns the snapshots of h every `dump` iterations."""
    P = sysc.param
    fluid = np.zeros((P.Tmax // dump, sysc.L)) if fluid is None else fluid
    st = State1D(sysc, T, records=0)
    st.height = two_droplets(sysc, r1=r1, r2=r2, θ1=θ0, θ2=θ0, center=(sysc.L / 3, 2 * sysc.L / 3))
    st.set_gamma(np.asarray(gamma, dtype=np.float64))
    for row in range(P.Tmax // dump):
        st.step(dump)
        fluid[row, :] = st.height
        if verbos and ((row + 1) * dump) % P.tdump == 0:
            h = st.height
            mid = sysc.L // 2
            print(f"Time step {(row + 1) * dump} bridge height is "
                  f"{round(float(h[mid - 20:mid + 20].min()), 3)}")
    rest = P.Tmax - (P.Tmax // dump) * dump
    if rest:
        st.step(rest)
    st.sync()
    return fluid
