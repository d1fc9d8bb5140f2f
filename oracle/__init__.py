"""CPU oracle for the thin-film LBM step -- test infrastructure only.

The product library never imports this package.  It is used by ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (CPU-baseline leg and the
``--impl reference`` arm) as the checker.

The reference (Swalbe.jl) is pure Julia and cannot run here, so
``swalbe_oracle.c`` restates its Float64 algorithm; see the header of that
file for the functions it follows.  This module builds it with gcc and binds
it with ctypes.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "swalbe_oracle.c")
_OUT_DIR = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_OUT_DIR, "liboracle.so")

# -ffp-contract=off: the reference (Julia) never contracts a*b+c into an FMA.
CFLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
          "-fno-fast-math"]


def build(force: bool = False) -> str:
    """Compile the oracle into oracle/_build/liboracle.so (seconds)."""
    os.makedirs(_OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(_SRC)):
        return _LIB_PATH
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", *CFLAGS, "-o", tmp, _SRC, "-lm"])
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


class Params(C.Structure):
    """Mirror of Taumucs + SysConst (src/initialize.jl:43-60, 76-81)."""
    _fields_ = [("Lx", C.c_int32), ("Ly", C.c_int32), ("Tmax", C.c_int32), ("tdump", C.c_int32),
                ("tau", C.c_double), ("cs", C.c_double), ("mu", C.c_double),
                ("delta", C.c_double), ("kbt", C.c_double), ("gamma", C.c_double),
                ("n", C.c_int32), ("m", C.c_int32), ("hmin", C.c_double),
                ("hcrit", C.c_double), ("theta", C.c_double), ("g", C.c_double)]


class LoopOpts(C.Structure):
    _fields_ = [("theta_field", C.c_void_p), ("theta", C.c_double), ("record_dh", C.c_int),
                ("callback", C.c_int), ("hthresh", C.c_double), ("incl_ax", C.c_double),
                ("incl_ay", C.c_double), ("incl_loop_time", C.c_int), ("incl_t", C.c_long),
                ("incl_tstart", C.c_long), ("incl_tsmooth", C.c_long),
                ("thermal_seed", C.c_uint64), ("t_offset", C.c_long),
                ("shift_tmove", C.c_long), ("shift_dx", C.c_int), ("shift_dy", C.c_int)]


class LoopOut(C.Structure):
    _fields_ = [("mass", C.c_void_p), ("dh", C.c_void_p), ("wet", C.c_void_p)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        d, i, p, sz = C.c_double, C.c_int, C.c_void_p, C.c_size_t
        sig = {
            "orc_cospi": (d, [d]),
            "orc_power_broad": (d, [d, i]),
            "orc_kappa": (d, [d, i, i, d]),
            "orc_circshift": (None, [p, p, i, i, i, i]),
            "orc_filmpressure": (None, [p, p, p, i, i, d, p, d, i, i, d, d]),
            "orc_filmpressure_raw": (i, [p, p, p, i, i, d, d, i, i, d, d]),
            "orc_laplacian": (None, [p, p, p, i, i, d]),
            "orc_gradient": (None, [p, p, p, p, i, i]),
            "orc_hgradp": (None, [p, p, p, p, p, i, i]),
            "orc_slippage": (None, [p, p, p, p, p, sz, d, d]),
            "orc_force_sum": (None, [p, p, p, p, p, p, sz]),
            "orc_incl_factor": (d, [C.c_long, C.c_long, C.c_long]),
            "orc_inclination": (None, [p, p, p, sz, d, d, C.c_long, C.c_long, C.c_long]),
            "orc_equilibrium": (None, [p, p, p, p, p, sz, d]),
            "orc_bgk_stream": (None, [p, p, p, p, p, i, i, d]),
            "orc_moments": (None, [p, p, p, p, sz]),
            "orc_sum": (d, [p, sz]),
            "orc_wetted": (C.c_int64, [p, sz, d]),
            "orc_dh": (d, [p, sz]),
            "orc_surfacearea": (None, [p, p, d, i, i, d, p, p, p]),
            "orc_singledroplet": (None, [p, i, i, d, d, d, d]),
            "orc_state_new": (p, [i, i]),
            "orc_state_free": (None, [p]),
            "orc_state_field": (p, [p, i]),
            "orc_time_loop": (None, [p, p, i, p, p]),
            "orc_fused_run": (i, [p, p, p, p, p, p, p, p, i, i, p, p, i]),
            "orc_pull_all": (None, [p, p, i, i]),
            "orc_max_threads": (i, []),
            "orc_philox4x32_10": (None, [p, p, p]),
            "orc_thermal_normals": (None, [C.c_uint64, C.c_uint64, C.c_int64, p, p]),
            "orc_thermal": (None, [p, p, p, sz, d, d, d, C.c_uint64, C.c_int64]),
            "orc1_filmpressure": (None, [p, p, i, d, p, p, d, i, i, d, d]),
            "orc1_hgradp": (None, [p, p, p, i]),
            "orc1_slippage": (None, [p, p, p, i, d, d]),
            "orc1_gradgamma": (None, [p, p, i]),
            "orc1_equilibrium": (None, [p, p, p, i, d]),
            "orc1_bgk_stream": (None, [p, p, p, p, i, d]),
            "orc1_moments": (None, [p, p, p, i]),
            "orc1_time_loop": (None, [p, p, p, p, p, i, p, p, p, p]),
            "orc1_two_droplets": (None, [p, i, d, d, d, d, d, d]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a: Optional[np.ndarray]):
    if a is None:
        return None
    assert a.flags["F_CONTIGUOUS"] or a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def _col(a) -> np.ndarray:
    """Float64 column-major copy (Julia memory order)."""
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


def params(Lx, Ly, *, Tmax=1000, tdump=None, tau=1.0, cs=None, mu=None, delta=1.0, kbt=0.0,
           gamma=0.01, n=9, m=3, hmin=0.1, hcrit=0.05, theta=1 / 9, g=0.0) -> Params:
    """Taumucs defaults (src/initialize.jl:43-60): μ = cₛ²(τ − ½)."""
    cs = 1 / np.sqrt(3.0) if cs is None else cs
    mu = cs ** 2 * (tau - 0.5) if mu is None else mu
    tdump = Tmax // 10 if tdump is None else tdump
    return Params(Lx, Ly, Tmax, tdump, tau, cs, mu, delta, kbt, gamma, n, m, hmin, hcrit, theta, g)


# ---------------------------------------------------------------- ops
def cospi(x: float) -> float:
    return lib().orc_cospi(float(x))


def circshift(src, shift):
    s = _col(src)
    out = np.empty_like(s)
    lib().orc_circshift(_p(out), _p(s), s.shape[0], s.shape[1], int(shift[0]), int(shift[1]))
    return out


def filmpressure(h, gamma, theta, n, m, hmin, hcrit, theta_field=None):
    """filmpressure!(state, sys; θ) (src/pressure.jl:119-155)."""
    h = _col(h)
    Lx, Ly = h.shape
    p = np.zeros_like(h)
    dg = np.zeros((Lx, Ly, 8), order="F")
    tf = None if theta_field is None else _col(theta_field)
    lib().orc_filmpressure(_p(p), _p(h), _p(dg), Lx, Ly, gamma, _p(tf), float(theta), n, m,
                           hmin, hcrit)
    return p


def filmpressure_raw(h, gamma, theta, n, m, hmin, hcrit):
    """filmpressure!(output, f, dgrad, γ, θ, n, m, hmin, hcrit) (src/pressure.jl:72-115)."""
    h = _col(h)
    Lx, Ly = h.shape
    p = np.zeros_like(h)
    dg = np.zeros((Lx, Ly, 8), order="F")
    rc = lib().orc_filmpressure_raw(_p(p), _p(h), _p(dg), Lx, Ly, gamma, float(theta), n, m,
                                    hmin, hcrit)
    if rc != 0:
        raise ValueError(f"exponents {(n, m)} not supported by the raw form")
    return p


def laplacian(f, gamma):
    f = _col(f)
    out = np.zeros_like(f)
    dg = np.zeros(f.shape + (8,), order="F")
    lib().orc_laplacian(_p(out), _p(f), _p(dg), f.shape[0], f.shape[1], gamma)
    return out


def gradient(f):
    f = _col(f)
    gx, gy = np.zeros_like(f), np.zeros_like(f)
    dg = np.zeros(f.shape + (8,), order="F")
    lib().orc_gradient(_p(gx), _p(gy), _p(f), _p(dg), f.shape[0], f.shape[1])
    return gx, gy


def hgradp(h, p):
    h, p = _col(h), _col(p)
    gx, gy = np.zeros_like(h), np.zeros_like(h)
    dg = np.zeros(h.shape + (8,), order="F")
    lib().orc_hgradp(_p(gx), _p(gy), _p(h), _p(p), _p(dg), h.shape[0], h.shape[1])
    return gx, gy


def slippage(h, ux, uy, delta, mu):
    h, ux, uy = _col(h), _col(ux), _col(uy)
    sx, sy = np.zeros_like(h), np.zeros_like(h)
    lib().orc_slippage(_p(sx), _p(sy), _p(h), _p(ux), _p(uy), h.size, delta, mu)
    return sx, sy


def inclination(Fx, Fy, h, alpha, t=1000, tstart=0, tsmooth=1):
    Fx, Fy, h = _col(Fx).copy(order="F"), _col(Fy).copy(order="F"), _col(h)
    lib().orc_inclination(_p(Fx), _p(Fy), _p(h), h.size, float(alpha[0]), float(alpha[1]),
                          t, tstart, tsmooth)
    return Fx, Fy


def equilibrium(h, ux, uy, g):
    h, ux, uy = _col(h), _col(ux), _col(uy)
    feq = np.zeros(h.shape + (9,), order="F")
    vsq = np.zeros_like(h)
    lib().orc_equilibrium(_p(feq), _p(h), _p(ux), _p(uy), _p(vsq), h.size, g)
    return feq


def bgk_stream(feq, ftemp, Fx, Fy, tau):
    """BGKandStream!(fout, feq, ftemp, Fx, Fy, τ); returns (fout, ftemp)."""
    feq = _col(feq)
    ftemp = _col(ftemp).copy(order="F")
    Fx, Fy = _col(Fx), _col(Fy)
    fout = np.zeros_like(feq)
    lib().orc_bgk_stream(_p(fout), _p(feq), _p(ftemp), _p(Fx), _p(Fy), feq.shape[0],
                         feq.shape[1], tau)
    return fout, ftemp


def moments(fout):
    fout = _col(fout)
    Lx, Ly = fout.shape[:2]
    h, ux, uy = (np.zeros((Lx, Ly), order="F") for _ in range(3))
    lib().orc_moments(_p(h), _p(ux), _p(uy), _p(fout), Lx * Ly)
    return h, ux, uy


def wetted(h, hthresh=0.055) -> int:
    h = _col(h)
    return int(lib().orc_wetted(_p(h), h.size, hthresh))


def surfacearea(h, theta, htresh=0.055):
    """(area_lv, red_energy) of surfacearea! (src/measures.jl:126-168)."""
    h = _col(h)
    tf = None
    th = 0.0
    if np.ndim(theta) == 0:
        th = float(theta)
    else:
        tf = _col(theta)
    dg = np.zeros(h.shape + (8,), order="F")
    a, e = C.c_double(), C.c_double()
    lib().orc_surfacearea(_p(h), _p(tf), th, h.shape[0], h.shape[1], htresh, _p(dg),
                          C.byref(a), C.byref(e))
    return a.value, e.value


def singledroplet(Lx, Ly, radius, theta, center):
    h = np.zeros((Lx, Ly), order="F")
    lib().orc_singledroplet(_p(h), Lx, Ly, float(radius), float(theta), float(center[0]),
                            float(center[1]))
    return h


# ---------------------------------------------------------------- loops
@dataclass
class LoopResult:
    height: np.ndarray
    velx: np.ndarray
    vely: np.ndarray
    mass: np.ndarray
    dh: Optional[np.ndarray]
    wet: Optional[np.ndarray]


def _opts(theta_field, theta, record_dh, callback, hthresh, incl, seed=0, t_offset=0,
          motion=None):
    tf = None if theta_field is None else _col(theta_field)
    o = LoopOpts()
    if motion:  # (tmove, dx, dy): move_substrate! after every tmove iterations
        o.shift_tmove, o.shift_dx, o.shift_dy = (int(v) for v in motion)
    o.thermal_seed = int(seed)
    o.t_offset = int(t_offset)
    o.theta_field = None if tf is None else tf.ctypes.data
    o.theta = float(theta)
    o.record_dh = int(record_dh)
    o.callback = {None: 0, "wetted": 1, "inclination": 2}[callback]
    o.hthresh = hthresh
    incl = incl or {}
    alpha = incl.get("alpha", (0.0, 0.0))
    o.incl_ax, o.incl_ay = float(alpha[0]), float(alpha[1])
    o.incl_loop_time = int(incl.get("loop_time", False))
    o.incl_t = int(incl.get("t", 1000))
    o.incl_tstart = int(incl.get("tstart", 0))
    o.incl_tsmooth = int(incl.get("tsmooth", 1))
    return o, tf


def time_loop_literal(P: Params, h0, steps, *, theta_field=None, theta=None, record_dh=False,
                      callback=None, hthresh=0.055, incl=None, ux0=None, uy0=None,
                      seed=0) -> LoopResult:
    """Literal time_loop on a fresh Sys() state with height = h0 (src/simulate.jl:6-96)."""
    L = lib()
    Lx, Ly = P.Lx, P.Ly
    s = L.orc_state_new(Lx, Ly)
    try:
        def field(i, shape):
            ptr = L.orc_state_field(s, i)
            n = int(np.prod(shape))
            return np.ctypeslib.as_array((C.c_double * n).from_address(ptr)).reshape(shape, order="F")
        field(3, (Lx, Ly))[...] = _col(h0)
        if ux0 is not None:
            field(4, (Lx, Ly))[...] = _col(ux0)
        if uy0 is not None:
            field(5, (Lx, Ly))[...] = _col(uy0)
        o, tf = _opts(theta_field, P.theta if theta is None else theta, record_dh, callback,
                      hthresh, incl, seed)
        mass = np.full(steps, np.nan)
        dh = np.zeros(steps) if record_dh else None
        wet = np.zeros(steps, dtype=np.int64) if callback == "wetted" else None
        out = LoopOut(mass.ctypes.data, None if dh is None else dh.ctypes.data,
                      None if wet is None else wet.ctypes.data)
        L.orc_time_loop(s, C.byref(P), steps, C.byref(o), C.byref(out))
        return LoopResult(field(3, (Lx, Ly)).copy(order="F"), field(4, (Lx, Ly)).copy(order="F"),
                          field(5, (Lx, Ly)).copy(order="F"), mass, dh, wet)
    finally:
        L.orc_state_free(s)


class FusedState:
    """Post-collision population buffer + macroscopic fields for orc_fused_run."""

    def __init__(self, P: Params, h0, ux0=None, uy0=None):
        self.P = P
        Lx, Ly = P.Lx, P.Ly
        self.fpost = np.zeros((Lx, Ly, 9), order="F")
        self.tmp = np.zeros_like(self.fpost)
        self.h = _col(h0).copy(order="F")
        self.ux = np.zeros((Lx, Ly), order="F") if ux0 is None else _col(ux0).copy(order="F")
        self.uy = np.zeros((Lx, Ly), order="F") if uy0 is None else _col(uy0).copy(order="F")
        self.press = np.zeros((Lx, Ly), order="F")
        self.kappa = np.zeros((Lx, Ly), order="F")
        self.fresh = True
        self.t = 0  # iterations done (index of the thermal noise)

    def run(self, steps, *, theta_field=None, theta=None, record_dh=False, callback=None,
            hthresh=0.055, incl=None, nthreads=0, seed=0, motion=None):
        P = self.P
        o, tf = _opts(theta_field, P.theta if theta is None else theta, record_dh, callback,
                      hthresh, incl, seed, self.t, motion)
        mass = np.full(steps, np.nan)
        dh = np.zeros(steps) if record_dh else None
        wet = np.zeros(steps, dtype=np.int64) if callback == "wetted" else None
        out = LoopOut(mass.ctypes.data, None if dh is None else dh.ctypes.data,
                      None if wet is None else wet.ctypes.data)
        lib().orc_fused_run(C.byref(P), _p(self.fpost), _p(self.tmp), _p(self.h), _p(self.ux),
                            _p(self.uy), _p(self.press), _p(self.kappa), int(self.fresh), steps,
                            C.byref(o), C.byref(out), int(nthreads))
        if steps > 0:
            self.fresh = False
        self.t += steps
        return LoopResult(self.h, self.ux, self.uy, mass, dh, wet)

    def fout(self):
        out = np.zeros_like(self.fpost)
        lib().orc_pull_all(_p(out), _p(self.fpost), self.P.Lx, self.P.Ly)
        return out


def max_threads() -> int:
    return int(lib().orc_max_threads())


class LiteralState:
    """A literal-oracle `State` that can be stepped in chunks and edited between
    chunks, like a Julia user script does (src/initialize.jl:491-508)."""

    _IDS = {"fout": 0, "ftemp": 1, "feq": 2, "height": 3, "velx": 4, "vely": 5, "vsq": 6,
            "pressure": 7, "Fx": 8, "Fy": 9, "slipx": 10, "slipy": 11, "h∇px": 12, "h∇py": 13}

    def __init__(self, P: Params):
        self.P = P
        self._s = lib().orc_state_new(P.Lx, P.Ly)
        self.t = 0

    def __del__(self):
        if getattr(self, "_s", None):
            lib().orc_state_free(self._s)
            self._s = None

    def field(self, name) -> np.ndarray:
        n9 = name in ("fout", "ftemp", "feq")
        shape = (self.P.Lx, self.P.Ly) + ((9,) if n9 else ())
        ptr = lib().orc_state_field(self._s, self._IDS[name])
        n = int(np.prod(shape))
        return np.ctypeslib.as_array((C.c_double * n).from_address(ptr)).reshape(shape, order="F")

    def run(self, steps, *, theta_field=None, theta=None, record_dh=False, callback=None,
            hthresh=0.055, incl=None, seed=0, motion=None) -> LoopResult:
        P = self.P
        o, tf = _opts(theta_field, P.theta if theta is None else theta, record_dh, callback,
                      hthresh, incl, seed, self.t, motion)
        self.t += steps
        mass = np.full(steps, np.nan)
        dh = np.zeros(steps) if record_dh else None
        wet = np.zeros(steps, dtype=np.int64) if callback == "wetted" else None
        out = LoopOut(mass.ctypes.data, None if dh is None else dh.ctypes.data,
                      None if wet is None else wet.ctypes.data)
        lib().orc_time_loop(self._s, C.byref(P), steps, C.byref(o), C.byref(out))
        return LoopResult(self.field("height").copy(order="F"), self.field("velx").copy(order="F"),
                          self.field("vely").copy(order="F"), mass, dh, wet)


# ---------------------------------------------------------------- thermal
def philox4x32_10(ctr, key):
    """Philox-4x32-10 block (four 32-bit words) of counter `ctr` and key `key`."""
    c = (C.c_uint32 * 4)(*[int(v) & 0xFFFFFFFF for v in ctr])
    k = (C.c_uint32 * 2)(*[int(v) & 0xFFFFFFFF for v in key])
    out = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, out)
    return list(out)


def thermal(h, kbt, mu, delta, seed=0, t=1):
    """thermal!(fx, fy, h, kbt, mu, delta) (src/forcing.jl:297-311) with the
    counter-based normals of iteration t."""
    hh = _col(h)
    fx = np.zeros_like(hh)
    fy = np.zeros_like(hh)
    lib().orc_thermal(_p(fx), _p(fy), _p(hh), hh.size, float(kbt), float(mu), float(delta),
                      int(seed), int(t))
    return fx, fy


# ---------------------------------------------------------------- D1Q3
def _v(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def equilibrium_1d(h, u, g=0.0):
    """equilibrium!(feq, height, velocity, gravity) (src/equilibrium.jl:169-181): L x 3."""
    h, u = _v(h), _v(u)
    feq = np.zeros((h.size, 3), order="F")
    lib().orc1_equilibrium(_p(feq), _p(h), _p(u), h.size, float(g))
    return feq


def bgk_stream_1d(feq, ftemp, F, tau):
    """BGKandStream!(fout, feq, ftemp, F, τ) (src/collide.jl:179-201): (fout, ftemp)."""
    fe = np.asfortranarray(feq, dtype=np.float64)
    ft = np.asfortranarray(ftemp, dtype=np.float64).copy(order="F")
    FF = _v(F)
    fout = np.zeros_like(ft)
    lib().orc1_bgk_stream(_p(fout), _p(fe), _p(ft), _p(FF), fe.shape[0], float(tau))
    return fout, ft


def slippage_1d(h, u, delta, mu):
    h, u = _v(h), _v(u)
    out = np.zeros_like(h)
    lib().orc1_slippage(_p(out), _p(h), _p(u), h.size, float(delta), float(mu))
    return out


def singledroplet_1d(L, radius, theta, center, hcrit=0.05):
    """singledroplet(height::Vector, radius, θ, center; hcrit) (src/initialvalues.jl:226-243)."""
    h = np.zeros(L)
    for i in range(1, L + 1):
        circ = np.sqrt((i - center) ** 2)
        h[i - 1] = (np.cos(np.arcsin(circ / radius)) - cospi(theta)) * radius if circ <= radius else hcrit
    return np.where(h <= hcrit, hcrit, h)


def two_droplets(L, r1=230, r2=230, th1=1 / 9, th2=1 / 9, center=None):
    """two_droplets(sys; r₁, r₂, θ₁, θ₂, center) (src/initialvalues.jl:277-323)."""
    c = (L / 3, 2 * L / 3) if center is None else center
    h = np.zeros(L)
    lib().orc1_two_droplets(_p(h), int(L), float(r1), float(r2), float(th1), float(th2),
                            float(c[0]), float(c[1]))
    return h


class State1D:
    """A D1Q3 State (src/initialize.jl:587-599): fout, ftemp, height, vel."""

    def __init__(self, P: Params, h0=None):
        self.P = P
        L = P.Lx
        self.fout = np.zeros((L, 3), order="F")
        self.ftemp = np.zeros((L, 3), order="F")
        self.h = np.ones(L) if h0 is None else _v(h0).copy()
        self.u = np.zeros(L)

    def run(self, steps, theta_field=None, gamma_field=None, record_dh=False, wetted=False):
        dh = np.zeros(steps) if record_dh else None
        wet = np.zeros(steps, dtype=np.int64) if wetted else None
        tf = None if theta_field is None else _v(theta_field)
        gf = None if gamma_field is None else _v(gamma_field)
        lib().orc1_time_loop(_p(self.fout), _p(self.ftemp), _p(self.h), _p(self.u), C.byref(self.P),
                             int(steps), _p(tf), _p(gf), _p(dh), _p(wet))
        return dh if not wetted else (dh, wet)
