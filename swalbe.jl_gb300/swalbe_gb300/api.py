"""Host-side mirror of Swalbe.jl's Julia API over the C ABI.

Names, arguments and defaults follow the reference (paths relative to the
Swalbe.jl project root) so that a script written against `Swalbe` reads the
same: ``Sys(sys, "GB300")`` instead of ``Sys(sys, "GPU")``, then
``time_loop``, the ``run_*`` drivers and the per-op functions.  Julia's
``!``-suffixed mutating functions end in ``_`` here (``filmpressure_``).
"""
from __future__ import annotations

import ctypes as C
import functools
import math
from typing import Callable, Optional, Sequence

import numpy as np

from . import _lib as L
from ._lib import check, lib

_GREEK = {"τ": "tau", "cₛ": "cs", "μ": "mu", "δ": "delta", "γ": "gamma", "θ": "theta"}


class Taumucs:
    """Run-time constants (src/initialize.jl:43-60).  θ is in units of π."""

    def __init__(self, **kw):
        kw = {_GREEK.get(k, k): v for k, v in kw.items()}
        self.Tmax = int(kw.pop("Tmax", 1000))
        self.tdump = int(kw.pop("tdump", self.Tmax // 10))
        self.tau = float(kw.pop("tau", 1.0))
        self.cs = float(kw.pop("cs", 1 / math.sqrt(3.0)))
        self.mu = float(kw.pop("mu", self.cs ** 2 * (self.tau - 0.5)))
        self.delta = float(kw.pop("delta", 1.0))
        self.kbt = float(kw.pop("kbt", 0.0))
        self.gamma = float(kw.pop("gamma", 0.01))
        self.n = int(kw.pop("n", 9))
        self.m = int(kw.pop("m", 3))
        self.hmin = float(kw.pop("hmin", 0.1))
        self.hcrit = float(kw.pop("hcrit", 0.05))
        self.theta = float(kw.pop("theta", 1 / 9))
        self.g = float(kw.pop("g", 0.0))
        if kw:
            raise TypeError(f"unknown Taumucs fields {sorted(kw)}")

    # Greek aliases as in the reference
    τ = property(lambda s: s.tau)
    μ = property(lambda s: s.mu)
    δ = property(lambda s: s.delta)
    γ = property(lambda s: s.gamma)
    θ = property(lambda s: s.theta)

    def replace(self, **kw):
        d = dict(Tmax=self.Tmax, tdump=self.tdump, tau=self.tau, cs=self.cs, mu=self.mu,
                 delta=self.delta, kbt=self.kbt, gamma=self.gamma, n=self.n, m=self.m,
                 hmin=self.hmin, hcrit=self.hcrit, theta=self.theta, g=self.g)
        d.update({_GREEK.get(k, k): v for k, v in kw.items()})
        return Taumucs(**d)


class SysConst:
    """Lattice size + constants (src/initialize.jl:76-81)."""

    def __init__(self, Lx: int = 256, Ly: int = 256, param: Optional[Taumucs] = None):
        self.Lx, self.Ly = int(Lx), int(Ly)
        self.param = param if param is not None else Taumucs()

    def c_params(self) -> L.Params:
        p = self.param
        return L.Params(self.Lx, self.Ly, p.Tmax, p.tdump, p.tau, p.cs, p.mu, p.delta, p.kbt,
                        p.gamma, p.n, p.m, p.hmin, p.hcrit, p.theta, p.g)


def cospi(x: float) -> float:
    r = math.fmod(abs(float(x)), 2.0)
    if r == 0.0:
        return 1.0
    if r == 1.0:
        return -1.0
    if r in (0.5, 1.5):
        return 0.0
    return math.cos(math.pi * r)


def _precision(device: str, T) -> int:
    if device in ("GB300-plain", "GPU-plain"):
        if np.dtype(T) != np.float64:
            raise ValueError("the plain per-op path is Float64 only")
        return L.SWB_PLAIN64
    if device not in ("GB300", "GPU"):
        raise ValueError(f"device {device!r}: this package runs on 'GB300' (or 'GB300-plain')")
    dt = np.dtype(T)
    if dt == np.float64:
        return L.SWB_F64
    if dt == np.float32:
        return L.SWB_F32
    if dt == np.float16:
        return L.SWB_F16
    raise ValueError(f"unsupported element type {T}")


def _f64(a, shape) -> np.ndarray:
    a = np.asfortranarray(np.broadcast_to(np.asarray(a, dtype=np.float64), shape))
    return a


class GB300State:
    """A simulation resident on the GPU: the `State` of src/initialize.jl:149-168.

    Fields read (``state.height``) copy the current values to the host;
    assignment (``state.height = h`` or ``state.height[...] = ...`` via
    ``set``) uploads them.
    """

    def __init__(self, sysc: SysConst, precision: int):
        self.sys = sysc
        self.precision = precision
        self._p = sysc.c_params()
        h = C.c_void_p()
        check(lib().swb_create(C.byref(self._p), precision, C.byref(h)))
        self._h = h
        self.shape = (sysc.Lx, sysc.Ly)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().swb_destroy(h)
            except Exception:
                pass
            self._h = None

    close = __del__

    @property
    def handle(self):
        return self._h

    def _chk(self, st):
        return check(st, self._h)

    # ---- fields
    def get(self, name: str, out: Optional[np.ndarray] = None) -> np.ndarray:
        """Copy field `name` to the host: a new array, or into `out` (Float64,
        column-major, the field's shape; e.g. pinned host memory)."""
        shape = self.shape + ((9,) if name in ("fout", "feq") else ())
        if out is None:
            out = np.empty(shape, dtype=np.float64, order="F")
        elif out.shape != shape or out.dtype != np.float64 or not out.flags.f_contiguous:
            raise ValueError(f"out must be a column-major Float64 array of shape {shape}")
        self._chk(lib().swb_get_field(self._h, L.FIELD[name], out.ctypes.data))
        return out

    def set(self, name: str, values) -> None:
        shape = self.shape + ((9,) if name in ("fout", "feq") else ())
        a = _f64(values, shape)
        self._chk(lib().swb_set_field(self._h, L.FIELD[name], a.ctypes.data))

    height = property(lambda s: s.get("height"), lambda s, v: s.set("height", v))
    velx = property(lambda s: s.get("velx"), lambda s, v: s.set("velx", v))
    vely = property(lambda s: s.get("vely"), lambda s, v: s.set("vely", v))
    pressure = property(lambda s: s.get("pressure"), lambda s, v: s.set("pressure", v))
    fout = property(lambda s: s.get("fout"), lambda s, v: s.set("fout", v))
    feq = property(lambda s: s.get("feq"), lambda s, v: s.set("feq", v))
    Fx = property(lambda s: s.get("Fx"), lambda s, v: s.set("Fx", v))
    Fy = property(lambda s: s.get("Fy"), lambda s, v: s.set("Fy", v))
    slipx = property(lambda s: s.get("slipx"), lambda s, v: s.set("slipx", v))
    slipy = property(lambda s: s.get("slipy"), lambda s, v: s.set("slipy", v))
    h_grad_px = property(lambda s: s.get("h∇px"), lambda s, v: s.set("h∇px", v))
    h_grad_py = property(lambda s: s.get("h∇py"), lambda s, v: s.set("h∇py", v))
    vsq = property(lambda s: s.get("vsq"), lambda s, v: s.set("vsq", v))

    def set_device(self, name: str, device_ptr: int) -> None:
        """Field from a Float64 column-major device array (no host copy)."""
        self._chk(lib().swb_set_field_device(self._h, L.FIELD[name], C.c_void_p(device_ptr)))

    def set_stream(self, stream_ptr: Optional[int]) -> None:
        self._chk(lib().swb_set_stream(self._h, None if not stream_ptr else C.c_void_p(stream_ptr)))

    def stream(self) -> int:
        p = C.c_void_p()
        self._chk(lib().swb_get_stream(self._h, C.byref(p)))
        return p.value or 0

    # ---- configuration
    def set_theta(self, theta) -> None:
        if np.ndim(theta) == 0:
            self._chk(lib().swb_set_theta(self._h, float(theta)))
        else:
            t = _f64(theta, self.shape)
            self._chk(lib().swb_set_theta_field(self._h, t.ctypes.data))

    def set_theta_wave(self, theta0: float, dtheta: float, v: float) -> None:
        self._chk(lib().swb_set_theta_wave(self._h, theta0, dtheta, v))

    def move_substrate(self, tmove: int, direction: str = "diagonal") -> None:
        """move_substrate!(θ, input, t, tmove; direction) after every iteration
        (scripts/Moving_wettability_structs.jl:139-152): the θ field set by
        set_theta_field moves one cell along `direction` ("diagonal", "x",
        "y") after every `tmove` iterations from now; tmove = 0 stops it."""
        dx, dy = {"diagonal": (1, 1), "x": (1, 0), "y": (0, 1)}[direction]
        self._chk(lib().swb_set_substrate_motion(self._h, int(tmove), dx, dy))

    def set_inclination(self, alpha, t=1000, tstart=0, tsmooth=1, loop_time=False) -> None:
        self._chk(lib().swb_set_inclination(self._h, float(alpha[0]), float(alpha[1]),
                                            int(loop_time), int(t), int(tstart), int(tsmooth)))

    def set_geometry(self, nt: int = 0, h: int = 0) -> None:
        self._chk(lib().swb_set_geometry(self._h, int(nt), int(h)))

    def geometry(self):
        a, b = C.c_int(), C.c_int()
        self._chk(lib().swb_get_geometry(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_step_mode(self, mode) -> None:
        """"auto", "per_iteration" (one launch per iteration, CUDA graphs) or
        "multi" (one cooperative launch per 1024 iterations; FP32/FP16)."""
        m = {"auto": 0, "per_iteration": 1, "multi": 2}.get(mode, mode)
        self._chk(lib().swb_set_step_mode(self._h, int(m)))

    def step_mode(self) -> str:
        a = C.c_int()
        self._chk(lib().swb_get_step_mode(self._h, C.byref(a)))
        return {1: "per_iteration", 2: "multi"}[a.value]

    def set_snapshots(self, dumping: int, capacity: int = 64) -> None:
        """snapshot!(fluid, height, t; dumping) on the device: the height
        after every `dumping`-th iteration goes into a device ring of
        `capacity` fields (0 turns it off)."""
        self._chk(lib().swb_set_snapshots(self._h, int(dumping), int(capacity)))

    def snapshots(self, cap: int = 1 << 12):
        """(times, rows): the snapshots taken since the last call, oldest
        first; row k is vec(h) (column-major) as in the reference's snapshot
        matrix."""
        n = self.shape[0] * self.shape[1]
        out = []
        times = []
        while True:
            k = min(cap, 64)
            buf = np.empty((k, n))
            ts = np.empty(k, dtype=np.int64)
            cnt = C.c_int64()
            self._chk(lib().swb_get_snapshots(self._h, buf.ctypes.data, k, C.byref(cnt),
                                              ts.ctypes.data))
            out.append(buf[:cnt.value])
            times.extend(ts[:cnt.value].tolist())
            if cnt.value < k:
                break
        return times, np.concatenate(out, axis=0)

    def set_thermal_seed(self, seed: int) -> None:
        """Key of the thermal noise stream (Philox-4x32-10; counter = cell, iteration)."""
        self._chk(lib().swb_set_thermal_seed(self._h, int(seed)))

    def thermal_field(self, t: int):
        """(kbtx, kbty): thermal!'s forces on the current height for iteration t."""
        shape = self.shape
        fx = np.empty(shape, order="F")
        fy = np.empty(shape, order="F")
        self._chk(lib().swb_thermal_field(self._h, int(t), fx.ctypes.data, fy.ctypes.data))
        return fx, fy

    def set_mass_correction(self, on: bool) -> None:
        self._chk(lib().swb_set_mass_correction(self._h, int(bool(on))))

    def set_measures(self, mask: int, hthresh: float = 0.055) -> None:
        self._chk(lib().swb_set_measures(self._h, int(mask), float(hthresh)))

    # ---- stepping
    def step(self, nsteps: int) -> None:
        self._chk(lib().swb_step(self._h, int(nsteps)))

    def sync(self) -> None:
        self._chk(lib().swb_sync(self._h))

    def steps_done(self) -> int:
        t = C.c_int64()
        self._chk(lib().swb_steps_done(self._h, C.byref(t)))
        return t.value

    def measures(self, cap: int = 1 << 16):
        buf = (L.Measure * cap)()
        n = C.c_int64()
        self._chk(lib().swb_get_measures(self._h, buf, cap, C.byref(n)))
        return [buf[k] for k in range(n.value)]

    def measures_array(self, cap: int = 1 << 16) -> np.ndarray:
        """The records as a numpy structured array (fields of ``Measure``)."""
        buf = (L.Measure * cap)()
        n = C.c_int64()
        self._chk(lib().swb_get_measures(self._h, buf, cap, C.byref(n)))
        return np.ctypeslib.as_array(buf)[: n.value].copy()

    def measures_dropped(self) -> int:
        """Per-step records overwritten on the device before they were read."""
        n = C.c_int64()
        self._chk(lib().swb_measures_dropped(self._h, C.byref(n)))
        return n.value

    def measure_now(self, hthresh: float = 0.055) -> L.Measure:
        m = L.Measure()
        self._chk(lib().swb_measure_now(self._h, hthresh, C.byref(m)))
        return m


def Sys(sysc: SysConst, device: str = "GB300", T=np.float64, kind: str = "simple") -> GB300State:
    from . import d1
    if isinstance(sysc, d1.SysConst_1D):  # Sys(sysc::SysConst_1D; T, kind)
        if kind != "simple":
            raise NotImplementedError(f"kind={kind!r}: 1D states are 'simple' (use set_gamma for γ fields)")
        return d1.State1D(sysc, T)
    """Sys(sysc, device; T, kind) (src/initialize.jl:491-572): zero populations, h = 1.

    kind="thermal" adds thermal!'s fluctuating forces every iteration when
    kbt > 0 (src/forcing.jl:297-320); a "simple" state has no fluctuation
    fields in the reference, so its kbt has no effect here either."""
    if kind not in ("simple", "thermal"):
        raise NotImplementedError(f"kind={kind!r}: 'simple' and 'thermal' states run on the GB300 path")
    if kind == "simple" and sysc.param.kbt != 0.0:
        sysc = SysConst(sysc.Lx, sysc.Ly, sysc.param.replace(kbt=0.0))
    return GB300State(sysc, _precision(device, T))


def launch_count() -> int:
    """Kernel launches the library has issued since it was loaded."""
    n = C.c_uint64()
    check(lib().swb_launch_count(C.byref(n)))
    return n.value


# ------------------------------------------------------------------ per-op API
def filmpressure_(state: GB300State, sysc: SysConst, θ=None, theta=None) -> None:
    """filmpressure!(state, sys; θ) (src/pressure.jl:119-155)."""
    th = θ if θ is not None else theta
    state.set_theta(sysc.param.theta if th is None else th)
    state._chk(lib().swb_op_filmpressure(state.handle))


def thermal_(state: GB300State, t: int) -> None:
    """Fx .-= kbtx, Fy .-= kbty with thermal!'s forces of iteration t
    (src/forcing.jl:297-320), on a "GB300-plain" state after force_sum_."""
    state._chk(lib().swb_op_thermal(state.handle, int(t)))


def h_grad_p_(state: GB300State) -> None:
    """h∇p!(state) (src/forcing.jl:168-187)."""
    state._chk(lib().swb_op_hgradp(state.handle))


def slippage_(state: GB300State, sysc: SysConst) -> None:
    """slippage!(state, sys) (src/forcing.jl:48-56)."""
    state._chk(lib().swb_op_slippage(state.handle))


def force_sum_(state: GB300State) -> None:
    """state.Fx .= -state.h∇px .- state.slipx, likewise y (src/simulate.jl:18-19)."""
    state._chk(lib().swb_op_force_sum(state.handle))


def inclination_(α, state: GB300State, t: int = 1000, tstart: int = 0, tsmooth: int = 1) -> None:
    """inclination!(α, state; t, tstart, tsmooth) (src/forcing.jl:363-368)."""
    state._chk(lib().swb_op_inclination(state.handle, float(α[0]), float(α[1]), int(t),
                                        int(tstart), int(tsmooth)))


def equilibrium_(state: GB300State, sysc: SysConst) -> None:
    """equilibrium!(state, sys) (src/equilibrium.jl:118-119)."""
    state._chk(lib().swb_op_equilibrium(state.handle))


def BGKandStream_(state: GB300State, sysc: SysConst) -> None:
    """BGKandStream!(state, sys) (src/collide.jl:151-152)."""
    state._chk(lib().swb_op_bgk_stream(state.handle))


def moments_(state: GB300State) -> None:
    """moments!(state) (src/moments.jl:64)."""
    state._chk(lib().swb_op_moments(state.handle))


def wetted_(area_size: list, state: GB300State, hthresh: float = 0.055) -> None:
    """wetted!(area_size, state) (src/measures.jl:13-17)."""
    area_size.append(int(state.measure_now(hthresh).wetted))


def count_droplets(h, hthresh: float = 0.055) -> int:
    """Droplets in a height field: connected components of h > hthresh,
    8-connected and periodic (host code in the library)."""
    a = _f64(h, np.shape(h))
    n = C.c_int64()
    check(lib().swb_count_droplets(a.ctypes.data, a.shape[0], a.shape[1], float(hthresh),
                                   C.byref(n)))
    return n.value


def surfacearea_(state: GB300State, hthresh: float = 0.055):
    """(area_lv, red_energy) of surfacearea! (src/measures.jl:126-168) for the θ set."""
    m = state.measure_now(hthresh)
    return m.area, m.energy


# ------------------------------------------------------------------ time loop
def time_loop(sysc: SysConst, state: GB300State, *args, verbose: bool = False):
    """time_loop(sys, state[, θ | Δh | f, measure]) (src/simulate.jl:6-96);
    a SysConst_1D dispatches to the 1D method (src/simulate.jl:98-179).

    - ``time_loop(sys, state)``: θ = sys.param.θ;
    - ``time_loop(sys, state, θ)``: θ a number or an Lx x Ly array;
    - ``time_loop(sys, state, Δh)``: Δh a list, max(h) - min(h) pushed every step;
    - ``time_loop(sys, state, f, measure)``: the callback runs after the forces
      each step; ``wetted_`` and ``inclination_`` run fused on the device; any
      other callable runs between the reference's ops on the per-op Float64
      path (a ``"GB300-plain"`` state, or a per-op twin of a fused state that
      hands the populations back at the end).
    """
    from . import d1
    if isinstance(sysc, d1.SysConst_1D):
        return d1.time_loop(sysc, state, *args, verbose=verbose)
    P = sysc.param
    Tmax = P.Tmax
    mask = L.MEAS_MASS
    dh = None
    callback = None
    measure = None
    state.set_theta(P.theta)
    if len(args) == 1 and isinstance(args[0], list):
        dh = args[0]
        mask |= L.MEAS_MAXMIN
    elif len(args) == 1:
        state.set_theta(args[0])
    elif len(args) == 2:
        callback, measure = args
        if callback is wetted_:
            mask |= L.MEAS_WETTED
        elif callback is inclination_:
            state.set_inclination(measure)
    elif args:
        raise TypeError("time_loop(sys, state[, θ | Δh | f, measure])")
    state.set_measures(mask)
    if callback is not None and callback not in (wetted_, inclination_):
        if state.precision == L.SWB_PLAIN64:
            for _ in range(Tmax):
                _plain_iteration_with_callback(sysc, state, callback, measure)
        else:
            _callback_loop_on_plain_twin(sysc, state, callback, measure, Tmax)
        recs = state.measures_array(cap=max(Tmax, 1))
    else:
        # the device ring holds RECORD_CAPACITY per-step records: step in
        # chunks no longer than that and drain after each, so that every
        # step's Δh / wetted! entry reaches the host (src/simulate.jl:56)
        state.measures_array(cap=L.RECORD_CAPACITY)  # records of earlier calls
        dropped0 = state.measures_dropped()
        parts = []
        left = Tmax
        while left > 0:
            n = min(left, L.RECORD_CAPACITY)
            state.step(n)
            parts.append(state.measures_array(cap=n))
            left -= n
        recs = np.concatenate(parts) if parts else state.measures_array(cap=1)
        if state.measures_dropped() != dropped0:
            raise RuntimeError("per-step records were overwritten before they were read")
    if verbose and P.tdump > 0:
        for r in recs[recs["t"] % P.tdump == 0]:
            print(f"Time step {int(r['t'])} mass is {round(float(r['mass']), 3)}")
    if dh is not None:
        dh.extend((recs["hmax"] - recs["hmin"]).tolist())
    if callback is wetted_:
        measure.extend(recs["wetted"].tolist())
    if callback is inclination_:
        state.set_inclination((0.0, 0.0))
    state.sync()
    if callback is not None:
        return state, measure
    return state


def _callback_loop_on_plain_twin(sysc, state, f: Callable, measure, Tmax: int) -> None:
    """time_loop(sys, state, f, measure) with a callback the fused kernels
    cannot run (any f other than wetted!/inclination!): the reference calls
    f(measure, state) after the forces of every iteration and f may read or
    change any field (src/simulate.jl:68-96).  The loop runs on a per-op
    Float64 twin of the state (the reference's op sequence, one kernel per
    op, f between the ops) and hands the populations and fields back: the
    twin starts from the state's fout, h and u, and the state continues from
    the twin's.  θ is sys.param.θ, as filmpressure!(state, sys) takes it."""
    twin = GB300State(sysc, L.SWB_PLAIN64)
    twin.set_theta(sysc.param.theta)
    twin.set("fout", state.get("fout"))
    twin.height = state.height
    twin.velx = state.velx
    twin.vely = state.vely
    for _ in range(Tmax):
        _plain_iteration_with_callback(sysc, twin, f, measure)
    state.set("fout", twin.get("fout"))
    state.height = twin.height
    state.velx = twin.velx
    state.vely = twin.vely
    del twin


def _plain_iteration_with_callback(sysc, state, f: Callable, measure):
    filmpressure_(state, sysc)
    h_grad_p_(state)
    slippage_(state, sysc)
    force_sum_(state)
    f(measure, state)
    equilibrium_(state, sysc)
    BGKandStream_(state, sysc)
    moments_(state)


# ------------------------------------------------------------------ initial values
def singledroplet(height: np.ndarray, radius, θ, center) -> np.ndarray:
    if np.ndim(height) == 1:  # singledroplet(height::Vector, ...) (src/initialvalues.jl:226-243)
        from .d1 import singledroplet_1d
        return singledroplet_1d(np.asarray(height, dtype=np.float64), radius, θ, center)
    """singledroplet(height, radius, θ, center) (src/initialvalues.jl:203-224); 1-based center."""
    lx, ly = height.shape
    i = np.arange(1, lx + 1, dtype=np.float64)[:, None]
    j = np.arange(1, ly + 1, dtype=np.float64)[None, :]
    circ = np.sqrt((i - center[0]) ** 2 + (j - center[1]) ** 2)
    with np.errstate(invalid="ignore"):
        cap = (np.cos(np.arcsin(np.minimum(circ / radius, 1.0))) - cospi(θ)) * radius
    h = np.where(circ <= radius, cap, 0.05)
    h = np.where(h < 0, 0.05, h)
    height[...] = h
    return height


def randinterface_(height: np.ndarray, h0: float, ϵ: float, rng=None) -> None:
    """randinterface!(height, h₀, ϵ) (src/initialvalues.jl:23-33) with a seeded numpy RNG."""
    rng = np.random.default_rng(0) if rng is None else rng
    height[...] = h0 * (1.0 + ϵ * rng.standard_normal(height.shape))


def two_caps(Lx: int, Ly: int, r1, r2, θ1, θ2, c1, c2) -> np.ndarray:
    """Two spherical caps combined as two_droplets does in 1D
    (src/initialvalues.jl:277-323): h1 + h2 - 0.05, negatives clamped."""
    a = singledroplet(np.zeros((Lx, Ly)), r1, θ1, c1)
    b = singledroplet(np.zeros((Lx, Ly)), r2, θ2, c2)
    h = a + b - 0.05
    return np.asfortranarray(np.where(h < 0, 0.05, h))


# ------------------------------------------------------------------ snapshots / restart
def snapshot_(snap: np.ndarray, field, t: int, dumping: int = 1000) -> None:
    """snapshot!(snap, field, t; dumping) (src/measures.jl:99-105): row
    t ÷ dumping (1-based) of `snap` becomes vec(field) when t % dumping == 0."""
    if t % dumping == 0:
        snap[t // dumping - 1, :] = np.asarray(field).ravel(order="F")


def save_snapshots(path: str, times, rows) -> None:
    """Snapshots as an .npz archive with one vec(h) per key "h_<t>" (the key
    names restart_from_height reads, src/initialvalues.jl:358-382)."""
    np.savez(path, **{f"h_{int(t)}": np.asarray(r) for t, r in zip(times, rows)})


def restart_from_height(data, kind: str = "npz", timestep: int = 0, size=(512, 512)):
    """restart_from_height(data; kind, timestep, size) (src/initialvalues.jl:
    358-382): the height stored under "h_<timestep>", or the last stored one
    for timestep = 0, reshaped to `size` (column-major).  Archives written by
    save_snapshots (kind "npz"); the reference's JLD2 (HDF5) and BSON
    containers need readers this package does not bundle."""
    if kind != "npz":
        raise NotImplementedError(f"kind={kind!r}: only .npz snapshot archives are read here")
    with np.load(data) as f:
        keys = list(f.keys())
        key = keys[-1] if timestep == 0 else f"h_{int(timestep)}"
        return np.asfortranarray(np.asarray(f[key]).reshape(size, order="F"))


# ------------------------------------------------------------------ substrate patterns
# boxpattern / ellipsepattern / trianglepattern (src/initialvalues.jl:423-581)
# build a contact-angle field with a patch of θ0 + δa.  The reference tests
# membership of the lattice point (i, j) (1-based) in a LazySets polygon or
# ellipsoid and writes θ[j, i] (rows and columns swapped, kept here), and it
# moves vertices that fall off the lattice onto coordinate 1 (x first; y only
# when x was on the lattice).  Because of the swapped write the reference's generators need a
# square field (a rectangular one runs out of bounds there and here).
class Polygon:
    """Convex polygon (the convex hull of its vertices, closed)."""

    def __init__(self, vertices):
        pts = sorted({(float(x), float(y)) for x, y in vertices})

        def cross(o, a, b):
            return (a[0] - o[0]) * (b[1] - o[1]) - (a[1] - o[1]) * (b[0] - o[0])

        lower, upper = [], []
        for p in pts:  # Andrew's monotone chain, counter-clockwise
            while len(lower) >= 2 and cross(lower[-2], lower[-1], p) <= 0:
                lower.pop()
            lower.append(p)
        for p in reversed(pts):
            while len(upper) >= 2 and cross(upper[-2], upper[-1], p) <= 0:
                upper.pop()
            upper.append(p)
        self.vertices = lower[:-1] + upper[:-1]

    def __contains__(self, pt) -> bool:
        v = self.vertices
        x, y = float(pt[0]), float(pt[1])
        if len(v) == 1:
            return (x, y) == v[0]
        for k in range(len(v)):
            (ax, ay), (bx, by) = v[k], v[(k + 1) % len(v)]
            if (bx - ax) * (y - ay) - (by - ay) * (x - ax) < -1e-12 * max(1.0, abs(bx - ax) + abs(by - ay)):
                return False
        if len(v) == 2:  # a segment: also within its extent
            return min(v[0][0], v[1][0]) <= x <= max(v[0][0], v[1][0]) and \
                min(v[0][1], v[1][1]) <= y <= max(v[0][1], v[1][1])
        return True


class Ellipse:
    """Closed ellipse {x : (x - c)ᵀ Q⁻¹ (x - c) <= 1}, Q = diag(a², b²)."""

    def __init__(self, center, a, b):
        self.center = (float(center[0]), float(center[1]))
        self.q = (float(a) ** 2, float(b) ** 2)

    def __contains__(self, pt) -> bool:
        dx, dy = float(pt[0]) - self.center[0], float(pt[1]) - self.center[1]
        return dx * (dx / self.q[0]) + dy * (dy / self.q[1]) <= 1.0


def _clamp_vertices(xs, ys, shape):
    for k in range(len(xs)):
        if xs[k] < 1 or xs[k] > shape[0]:
            xs[k] = 1.0
        elif ys[k] < 1 or ys[k] > shape[1]:
            ys[k] = 1.0
    return list(zip(xs, ys))


def _paint(theta, theta0, da, region):
    th = np.array(theta, dtype=np.float64, order="F", copy=True)
    n1, n2 = th.shape
    for i in range(1, n1 + 1):
        for j in range(1, n2 + 1):
            th[j - 1, i - 1] = theta0 + da if (i, j) in region else theta0
    return th


def boxpattern(theta, theta0, center=None, δa=1 / 36, side=20, **kw):
    """boxpattern(θ, θ₀; center, δₐ, side) (src/initialvalues.jl:423-458): (θ, P)."""
    da = kw.get("delta_a", δa)
    sh = np.shape(theta)
    c = (sh[0] // 2, sh[1] // 2) if center is None else center
    xs = [c[0] - side / 2, c[0] - side / 2, c[0] + side / 2, c[0] + side / 2]
    ys = [c[1] - side / 2, c[1] + side / 2, c[1] - side / 2, c[1] + side / 2]
    P = Polygon(_clamp_vertices(xs, ys, sh))
    return _paint(theta, theta0, da, P), P


def ellipsepattern(theta, theta0, center=None, δa=1 / 36, a=10, b=5, **kw):
    """ellipsepattern(θ, θ₀; center, δₐ, a, b) (src/initialvalues.jl:489-510): (θ, P)."""
    da = kw.get("delta_a", δa)
    sh = np.shape(theta)
    c = (sh[0] // 2, sh[1] // 2) if center is None else center
    P = Ellipse(c, a, b)
    return _paint(theta, theta0, da, P), P


def trianglepattern(theta, theta0, center=None, δa=1 / 36, side=60, **kw):
    """trianglepattern(θ, θ₀; center, δₐ, side) (src/initialvalues.jl:552-581): (θ, P)."""
    da = kw.get("delta_a", δa)
    sh = np.shape(theta)
    c = (sh[0] // 2, sh[1] // 2) if center is None else center
    height = np.sqrt(3) / 2 * side
    xs = [c[0] - side / 2, c[0] + side / 2, c[0]]
    ys = [c[1] - height / 3, c[1] - height / 3, c[1] + 2 * height / 3]
    P = Polygon(_clamp_vertices(xs, ys, sh))
    return _paint(theta, theta0, da, P), P


# ------------------------------------------------------------------ run_* drivers
def _new(sysc, device, T):
    return Sys(sysc, device, T=T)


def _one_dim(name):
    """The reference dispatches the drivers on the system type; a
    SysConst_1D call goes to the 1D method of the same name (which, as in
    the reference, takes no device argument)."""
    def deco(fn2d):
        @functools.wraps(fn2d)
        def wrapper(sysc, *args, **kw):
            from . import d1
            if isinstance(sysc, d1.SysConst_1D):
                return getattr(d1, name)(sysc, *args, **kw)
            return fn2d(sysc, *args, **kw)
        return wrapper
    return deco


@_one_dim("run_flat")
def run_flat(sysc: SysConst, device: str = "GB300", verbos: bool = True, T=np.float64):
    """run_flat(sys, device) (src/simulate.jl:236-245)."""
    state = _new(sysc, device, T)
    state.height = np.ones(state.shape)
    time_loop(sysc, state, verbose=verbos)
    return state.height


@_one_dim("run_random")
def run_random(sysc: SysConst, device: str = "GB300", h0=1.0, ϵ=0.01, verbos=True, T=np.float64,
               rng=None):
    """run_random(sys, device; h₀, ϵ) (src/simulate.jl:286-294); θ = 1/9 as there."""
    state = _new(sysc, device, T)
    h = np.zeros(state.shape)
    randinterface_(h, h0, ϵ, rng)
    state.height = h
    time_loop(sysc, state, 1 / 9, verbose=verbos)
    return state.height


@_one_dim("run_rayleightaylor")
def run_rayleightaylor(sysc: SysConst, device: str = "GB300", kx=15, ky=18, h0=1.0, ϵ=0.001,
                       verbos=True, T=np.float64):
    """run_rayleightaylor(sys, device; kx, ky, h₀, ϵ) (src/simulate.jl:338-358)."""
    state = _new(sysc, device, T)
    i = np.arange(1, sysc.Lx + 1)[:, None]
    j = np.arange(1, sysc.Ly + 1)[None, :]
    state.height = h0 * (1 + ϵ * np.sin(2 * np.pi * kx * i / (sysc.Lx - 1)) *
                         np.sin(2 * np.pi * ky * j / (sysc.Ly - 1)))
    diff = []
    time_loop(sysc, state, diff, verbose=verbos)
    return state.height, diff


@_one_dim("run_dropletrelax")
def run_dropletrelax(sysc: SysConst, device: str = "GB300", radius=20, theta0=1 / 6, center=None,
                     verbos=True, T=np.float64):
    """run_dropletrelax(sys, device; radius, theta0, center) (src/simulate.jl:384-399)."""
    center = (sysc.Lx // 2, sysc.Ly // 2) if center is None else center
    state = _new(sysc, device, T)
    state.height = singledroplet(np.zeros(state.shape), radius, theta0, center)
    area = []
    time_loop(sysc, state, wetted_, area, verbose=verbos)
    return state.height, area


def run_dropletpatterned(sysc: SysConst, device: str = "GB300", radius=20, theta0=1 / 6, center=None,
                         θₛ=None, verbos=True, T=np.float64):
    """run_dropletpatterned(sys, device; radius, θ₀, center, θₛ) (src/simulate.jl:422-439)."""
    center = (sysc.Lx // 2, sysc.Ly // 2) if center is None else center
    θₛ = np.full((sysc.Lx, sysc.Ly), 1 / 9) if θₛ is None else θₛ
    state = _new(sysc, device, T)
    state.height = singledroplet(np.zeros(state.shape), radius, theta0, center)
    time_loop(sysc, state, θₛ, verbose=verbos)
    return state.height


def run_dropletforced(sysc: SysConst, device: str = "GB300", radius=20, theta0=1 / 6, center=None,
                      fx=0.0, fy=0.0, verbos=True, T=np.float64):
    """run_dropletforced(sys, device; radius, θ₀, center, fx, fy) (src/simulate.jl:462-484)."""
    center = (sysc.Lx // 2, sysc.Ly // 2) if center is None else center
    state = _new(sysc, device, T)
    state.height = singledroplet(np.zeros(state.shape), radius, theta0, center)
    time_loop(sysc, state, inclination_, [fx, fy], verbose=verbos)
    return state.height, state.velx, state.vely


# ------------------------------------------------------------------ batch / server
class Batch:
    """Many simulations advanced together (one launch per step, packed tiles)."""

    def __init__(self, systems: Sequence[SysConst], T=np.float32):
        self.systems = list(systems)
        prec = _precision("GB300", T)
        arr = (L.Params * len(self.systems))(*[s.c_params() for s in self.systems])
        h = C.c_void_p()
        check(lib().swb_batch_create(arr, len(self.systems), prec, C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().swb_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    close = __del__

    def set_height(self, i: int, h) -> None:
        s = self.systems[i]
        a = _f64(h, (s.Lx, s.Ly))
        check(lib().swb_batch_set_height(self._h, i, a.ctypes.data))

    def get_height(self, i: int) -> np.ndarray:
        s = self.systems[i]
        out = np.empty((s.Lx, s.Ly), order="F")
        check(lib().swb_batch_get_height(self._h, i, out.ctypes.data))
        return out

    def set_geometry(self, nt: int = 64, rows: int = 32) -> None:
        """Strips of every lattice: nt threads (nt - 4 columns) x rows, or
        pair strips of -nt threads (2|nt| - 4 columns) for nt = -32, -64, -128."""
        check(lib().swb_batch_set_geometry(self._h, int(nt), int(rows)))

    def geometry(self):
        """(nt, rows, CTAs per launch) in use; nt < 0: pair strips."""
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        check(lib().swb_batch_geometry(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def set_theta_wave(self, i: int, theta0: float, dtheta: float, v: float) -> None:
        check(lib().swb_batch_set_theta_wave(self._h, i, theta0, dtheta, v))

    def step(self, n: int) -> None:
        check(lib().swb_batch_step(self._h, int(n)))

    def sync(self) -> None:
        check(lib().swb_batch_sync(self._h))

    def tile(self):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        check(lib().swb_batch_tile(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value


class Server:
    """Request loop with HBM-footprint admission and continuous batching."""

    def __init__(self, hbm_budget: int, T=np.float32, steps_per_tick: int = 100):
        h = C.c_void_p()
        check(lib().swb_server_create(int(hbm_budget), _precision("GB300", T), int(steps_per_tick),
                                      C.byref(h)))
        self._h = h

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().swb_server_destroy(h)
            self._h = None

    __del__ = close

    def set_queue_limit(self, n: int) -> None:
        check(lib().swb_server_set_queue_limit(self._h, int(n)))

    def set_geometry(self, nt: int = 0, rows: int = 0) -> None:
        """Strips of the resident set: nt = 0 chosen per set (default), or
        pair strips of nt = -32 / -64 threads whenever every lattice allows
        them; each lattice's rows balanced up to `rows` (0 with nt = 0: 64)."""
        check(lib().swb_server_set_geometry(self._h, int(nt), int(rows)))

    def set_policy(self, policy: str = "fifo", max_resident_cells: int = 0) -> None:
        """"fifo" or "sjf" (shortest job first by Lx*Ly*nsteps, shedding the
        largest queued job when the queue is full), and an optional bound
        on the summed cells of resident requests."""
        code = {"fifo": 0, "sjf": 1}[policy]
        check(lib().swb_server_set_policy(self._h, code, int(max_resident_cells)))

    def submit(self, sysc: SysConst, h0, nsteps: int, theta0=None, dtheta=0.0, v=0.0):
        """Request id, or None when the queue is full (counted as rejected)."""
        p = sysc.c_params()
        a = _f64(h0, (sysc.Lx, sysc.Ly))
        th0 = sysc.param.theta if theta0 is None else theta0
        rid = C.c_int64()
        st = lib().swb_server_submit(self._h, C.byref(p), a.ctypes.data, float(th0), float(dtheta),
                                     float(v), int(nsteps), C.byref(rid))
        if st == L.SWB_ERR_BUSY:
            return None
        check(st)
        return rid.value

    def poll(self, rid: int, shape=None):
        """(done, height or None, info).  A failed or cancelled request is
        reported through info.status < 0, not raised."""
        info = L.RequestInfo()
        out = None if shape is None else np.empty(shape, order="F")
        st = lib().swb_server_poll(self._h, int(rid), None if out is None else out.ctypes.data,
                                   C.byref(info))
        if st in (L.SWB_ERR_ARG, L.SWB_ERR_NOT_FOUND):
            check(st)
        return st == 1, (out if st == 1 else None), info

    def cancel(self, rid: int) -> None:
        check(lib().swb_server_cancel(self._h, int(rid)))

    def stats(self) -> L.ServerStats:
        s = L.ServerStats()
        check(lib().swb_server_stats_get(self._h, C.byref(s)))
        return s

    def clock(self) -> float:
        return lib().swb_server_clock(self._h)
