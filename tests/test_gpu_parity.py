"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Float64 (SWB_F64 fused and SWB_PLAIN64 per-op) must be bit-identical to the
literal oracle: same operations, same order, no FMA contraction.  FP32 and
FP16-storage modes are compared with stated tolerances.
"""
import numpy as np
import pytest

import oracle
import swalbe_gb300 as sw
from swalbe_gb300 import _lib as L

pytestmark = pytest.mark.gpu


def sysc(Lx, Ly, **kw):
    return sw.SysConst(Lx, Ly, sw.Taumucs(**kw))


def oparams(s: sw.SysConst):
    p = s.param
    return oracle.params(s.Lx, s.Ly, Tmax=p.Tmax, tdump=p.tdump, tau=p.tau, cs=p.cs, mu=p.mu,
                         delta=p.delta, gamma=p.gamma, n=p.n, m=p.m, hmin=p.hmin, hcrit=p.hcrit,
                         theta=p.theta, g=p.g)


def rough(Lx, Ly, seed=3, amp=0.1):
    rng = np.random.default_rng(seed)
    return np.asfortranarray(1.0 + amp * rng.uniform(-1, 1, (Lx, Ly)))


def droplet(Lx, Ly, R, th0=1 / 6):
    return oracle.singledroplet(Lx, Ly, R, th0, (Lx // 2, Ly // 2))


def gpu_run(s, h0, steps, T=np.float64, device="GB300", theta_field=None, incl=None, meas=0,
            chunks=(None,)):
    st = sw.Sys(s, device, T=T)
    st.height = h0
    if theta_field is not None:
        st.set_theta(theta_field)
    if incl is not None:
        st.set_inclination(incl["alpha"], t=incl.get("t", 1000), tstart=incl.get("tstart", 0),
                           tsmooth=incl.get("tsmooth", 1), loop_time=incl.get("loop_time", False))
    if meas:
        st.set_measures(meas)
    st.step(steps)
    st.sync()
    return st


CASES = {
    # name: (Lx, Ly, params, init, steps)
    "ramp_5x5": (5, 5, {}, lambda: np.asfortranarray(np.arange(1.0, 26.0).reshape(5, 5, order="F") / 10), 60),
    "odd_7x13": (7, 13, {"g": -0.002}, lambda: rough(7, 13), 120),
    "partial_tiles_37x29": (37, 29, {"tau": 0.8}, lambda: rough(37, 29, 5), 150),
    "droplet_64x48": (64, 48, {"delta": 3.0}, lambda: droplet(64, 48, 14), 300),
    "n3m2_40x40": (40, 40, {"n": 3, "m": 2, "hmin": 0.07, "mu": 1 / 12}, lambda: rough(40, 40, 9), 200),
    "thin_1x24": (1, 24, {}, lambda: rough(1, 24, 2), 80),
    "thin_24x2": (24, 2, {"tau": 0.9}, lambda: rough(24, 2, 4), 80),
}


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("device", ["GB300", "GB300-plain"])
def test_f64_bit_exact(name, device):
    Lx, Ly, kw, init, steps = CASES[name]
    s = sysc(Lx, Ly, Tmax=steps, **kw)
    h0 = init()
    ref = oracle.time_loop_literal(oparams(s), h0, steps)
    st = gpu_run(s, h0, steps, device=device)
    assert np.array_equal(st.height, ref.height)
    assert np.array_equal(st.velx, ref.velx)
    assert np.array_equal(st.vely, ref.vely)


def test_f64_theta_field_and_measures():
    Lx, Ly, steps = 48, 40, 250
    s = sysc(Lx, Ly, Tmax=steps, tdump=50)
    rng = np.random.default_rng(12)
    th = np.asfortranarray(1 / 9 + 0.04 * rng.uniform(-1, 1, (Lx, Ly)))
    h0 = droplet(Lx, Ly, 12)
    ref = oracle.time_loop_literal(oparams(s), h0, steps, theta_field=th, record_dh=True,
                                   callback="wetted")
    st = gpu_run(s, h0, steps, theta_field=th, meas=L.MEAS_ALL)
    assert np.array_equal(st.height, ref.height)
    recs = st.measures()
    assert [r.t for r in recs] == list(range(1, steps + 1))
    assert np.array_equal([r.wetted for r in recs], ref.wet)
    assert np.array_equal([r.hmax - r.hmin for r in recs], ref.dh)
    m = np.array([r.mass for r in recs])
    sel = ~np.isnan(ref.mass)
    assert np.allclose(m[sel], ref.mass[sel], rtol=1e-13, atol=0)


def test_f64_inclination_loop_time():
    Lx, Ly, steps = 40, 32, 200
    s = sysc(Lx, Ly, Tmax=steps, delta=2.0)
    h0 = droplet(Lx, Ly, 10)
    incl = {"alpha": (2e-4, -1e-4), "loop_time": True, "tstart": 50, "tsmooth": 20}
    ref = oracle.time_loop_literal(oparams(s), h0, steps, callback="inclination", incl=incl)
    st = gpu_run(s, h0, steps, incl=incl)
    # the device tanh may differ from the host libm by an ulp
    assert np.allclose(st.height, ref.height, rtol=1e-12, atol=0)
    incl2 = {"alpha": (1e-4, 0.0)}  # the callback's default t = 1000: factor exactly 1
    ref2 = oracle.time_loop_literal(oparams(s), h0, steps, callback="inclination", incl=incl2)
    st2 = gpu_run(s, h0, steps, incl=incl2)
    assert np.array_equal(st2.height, ref2.height)


@pytest.mark.parametrize("device", ["GB300", "GB300-plain"])
def test_f64_edit_between_chunks(device):
    """state.height .= … between two time loops keeps ftemp, like the reference."""
    Lx, Ly = 33, 21
    s = sysc(Lx, Ly, tau=0.7)
    h0 = rough(Lx, Ly, 21)
    lit = oracle.LiteralState(oparams(s))
    lit.field("height")[...] = h0
    lit.run(40)
    st = sw.Sys(s, device)
    st.height = h0
    st.step(40)
    h_mid = st.height
    assert np.array_equal(h_mid, lit.field("height"))
    h_new = h_mid * 1.01
    lit.field("height")[...] = h_new
    st.height = h_new
    lit.run(60)
    st.step(60)
    assert np.array_equal(st.height, lit.field("height"))
    assert np.array_equal(st.fout, lit.field("fout"))


def test_plain_ops_match_oracle():
    """Each per-op kernel equals the reference op (src/*.jl) on the same inputs."""
    Lx, Ly = 11, 9
    s = sysc(Lx, Ly, tau=0.75, g=0.01, delta=2.0)
    rng = np.random.default_rng(5)
    h = np.asfortranarray(1 + 0.2 * rng.uniform(-1, 1, (Lx, Ly)))
    ux = np.asfortranarray(0.01 * rng.uniform(-1, 1, (Lx, Ly)))
    uy = np.asfortranarray(0.01 * rng.uniform(-1, 1, (Lx, Ly)))
    st = sw.Sys(s, "GB300-plain")
    st.height, st.velx, st.vely = h, ux, uy
    sw.filmpressure_(st, s)
    p_ref = oracle.filmpressure(h, 0.01, 1 / 9, 9, 3, 0.1, 0.05)
    assert np.array_equal(st.pressure, p_ref)
    sw.h_grad_p_(st)
    gx, gy = oracle.hgradp(h, p_ref)
    assert np.array_equal(st.h_grad_px, gx) and np.array_equal(st.h_grad_py, gy)
    sw.slippage_(st, s)
    sx, sy = oracle.slippage(h, ux, uy, 2.0, s.param.mu)
    assert np.array_equal(st.slipx, sx) and np.array_equal(st.slipy, sy)
    sw.force_sum_(st)
    assert np.array_equal(st.Fx, -gx - sx) and np.array_equal(st.Fy, -gy - sy)
    sw.inclination_([1e-3, 2e-3], st, t=3, tstart=1, tsmooth=2)
    Fx, Fy = oracle.inclination(-gx - sx, -gy - sy, h, (1e-3, 2e-3), t=3, tstart=1, tsmooth=2)
    assert np.array_equal(st.Fx, Fx) and np.array_equal(st.Fy, Fy)
    sw.equilibrium_(st, s)
    feq = oracle.equilibrium(h, ux, uy, 0.01)
    assert np.array_equal(st.feq, feq)
    ft = np.asfortranarray(rng.uniform(0, 0.2, (Lx, Ly, 9)))
    st.fout = ft
    sw.BGKandStream_(st, s)
    fout, _ = oracle.bgk_stream(feq, ft, Fx, Fy, 0.75)
    assert np.array_equal(st.fout, fout)
    sw.moments_(st)
    hh, uu, vv = oracle.moments(fout)
    assert np.array_equal(st.height, hh) and np.array_equal(st.velx, uu)


def test_fused_fout_roundtrip():
    Lx, Ly = 20, 12
    s = sysc(Lx, Ly, tau=0.6)
    h0 = rough(Lx, Ly, 8)
    st = sw.Sys(s, "GB300")
    st.height = h0
    st.step(30)
    lit = oracle.LiteralState(oparams(s))
    lit.field("height")[...] = h0
    lit.run(30)
    assert np.array_equal(st.fout, lit.field("fout"))
    f = st.fout
    st.fout = f * 1.0  # push back: the next steps must be unchanged
    lit_f = lit.field("fout").copy(order="F")
    lit.field("fout")[...] = lit_f
    lit.field("ftemp")[...] = lit_f
    st.step(10)
    lit.run(10)
    assert np.array_equal(st.height, lit.field("height"))


def test_droplet_relax_256_bit_exact():
    """The reference's CPU-runnable case: 256², R=60 cap of height 20, 10k steps,
    with its mass and wetted-area series."""
    from swalbe_gb300 import configs
    s, h0, steps = configs.droplet_relax_256()
    fs = oracle.FusedState(oparams(s), h0)
    ref = fs.run(steps, callback="wetted")
    st = gpu_run(s, h0, steps, meas=L.MEAS_MASS | L.MEAS_WETTED)
    assert np.array_equal(st.height, ref.height)
    recs = st.measures()
    assert np.array_equal([r.wetted for r in recs], ref.wet)
    assert ref.wet[0] < ref.wet[-1]


@pytest.mark.parametrize("T", [np.float64, np.float32, np.float16])
def test_geometry_does_not_change_results(T):
    """Strip width and height are a performance choice only (FP32/FP16: the
    mass sum that drives the mass correction is exact, so order-free)."""
    Lx, Ly, steps = 150, 97, 120
    s = sysc(Lx, Ly, tau=0.9, delta=2.0)
    h0 = droplet(Lx, Ly, 30)
    out = []
    geos = [(64, 2), (64, 4), (128, 16), (256, 64), (128, 512)]
    if T != np.float64:
        geos.append((32, 16))  # 2D tiles (FP32 arithmetic only)
        geos.append((-64, 8))  # pair strips; at τ = 0.9 their one-column fallback runs
    for nt, hh in geos:
        st = sw.Sys(s, "GB300", T=T)
        st.set_geometry(nt, hh)
        st.height = h0
        st.step(steps)
        out.append(st.height)
    for o in out[1:]:
        assert np.array_equal(o, out[0])
    if T == np.float64:
        ref = oracle.time_loop_literal(oparams(s), h0, steps)
        assert np.array_equal(out[0], ref.height)


def _run_geo(s, h0, steps, T, geo, theta_wave=None):
    st = sw.Sys(s, "GB300", T=T)
    st.set_geometry(*geo)
    st.set_measures(L.MEAS_ALL)
    if theta_wave:
        st.set_theta_wave(*theta_wave)
    st.height = h0
    st.step(steps // 3)
    st.step(steps - steps // 3)
    st.sync()
    return st.height, st.measures_array(cap=steps)


@pytest.mark.parametrize("T", [np.float32, np.float16])
def test_pair_strips_equal_one_column_strips(T):
    """Pair strips (two columns per thread, paired loads and stores, warp
    shuffles across x) give the bits of one-column strips: heights and every
    per-step measure, on full, ragged, tiny and multi-strip lattices."""
    cases = [(150, 97, droplet(150, 97, 30)), (64, 48, rough(64, 48, 3)),
             (2, 24, rough(2, 24, 2)), (246, 130, droplet(246, 130, 40)),
             (128, 3, rough(128, 3, 5)), (520, 40, rough(520, 40, 8))]
    steps = 150
    for Lx, Ly, h0 in cases:
        s = sysc(Lx, Ly, delta=2.0)
        h_ref, r_ref = _run_geo(s, h0, steps, T, (64, 8))
        for geo in ((-32, 4), (-64, 2), (-64, 16), (-128, 64)):
            h, r = _run_geo(s, h0, steps, T, geo)
            assert np.array_equal(h, h_ref), (Lx, Ly, geo)
            for f in ("t", "mass", "wetted", "hmax", "hmin", "area", "energy"):
                assert np.array_equal(r[f], r_ref[f]), (Lx, Ly, geo, f)


@pytest.mark.parametrize("T", [np.float32, np.float16])
def test_pair_geometry_fallback_forms(T):
    """A pair-strip state whose iterations need another form (τ != 1, a θ
    wave) runs them as one-column strips of the same rows: same results."""
    Lx, Ly = 96, 64
    h0 = droplet(Lx, Ly, 20)
    for kw, wave in (({"tau": 0.8}, None), ({}, (1 / 9, 1 / 36, 1 / 98))):
        s = sysc(Lx, Ly, **kw)
        h_ref, r_ref = _run_geo(s, h0, 120, T, (64, 16), theta_wave=wave)
        h, r = _run_geo(s, h0, 120, T, (-64, 16), theta_wave=wave)
        assert np.array_equal(h, h_ref)
        assert np.array_equal(r["mass"], r_ref["mass"]) and np.array_equal(r["area"], r_ref["area"])


def test_pair_geometry_rules():
    st = sw.Sys(sysc(33, 16), "GB300", T=np.float32)
    with pytest.raises(sw.SwbError):
        st.set_geometry(-64, 8)  # odd Lx
    st64 = sw.Sys(sysc(32, 16), "GB300", T=np.float64)
    with pytest.raises(sw.SwbError):
        st64.set_geometry(-64, 8)  # Float64


# ------------------------------------------------------------------ FP32 / FP16
def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


# Tolerances: FP32 arithmetic vs the Float64 oracle after 4000 steps of a
# relaxing droplet (measured ~3.5e-6 relative L2 for both storage modes).
@pytest.mark.parametrize("T,tol", [(np.float32, 2e-5), (np.float16, 5e-5)])
def test_low_precision_droplet(T, tol):
    Lx, Ly, steps = 96, 96, 4000
    s = sysc(Lx, Ly, Tmax=steps, delta=3.0)
    h0 = droplet(Lx, Ly, 25)
    ref = oracle.FusedState(oparams(s), h0).run(steps)
    st = gpu_run(s, h0, steps, T=T, meas=L.MEAS_MASS)
    h = st.height
    assert rel_l2(h, ref.height) < tol
    recs = st.measures()
    m = np.array([r.mass for r in recs])
    drift = np.abs(m - m[0]).max() / m[0]
    # FP32 populations: the part of f0's residue that its stochastic rounding
    # leaves out is folded into f5/f7, mass is kept to ~1e-12 without the
    # correction.  FP16 populations: f0 (FP32) is stochastically
    # rounded, each cell's storage error is ~ulp(h)/2 and unbiased; on 96² cells
    # the FP64-measured correction holds the mass at that noise floor
    # (sqrt(N) * 5e-8 / M ≈ 4e-9; measured max 5.6e-9 over 300 steps).
    assert drift < (1e-10 if T == np.float32 else 2e-8)
    assert abs(h.sum() - h0.sum()) / h0.sum() < 1e-6


@pytest.mark.parametrize("T", [np.float32, np.float16])
def test_low_precision_mass_drift_large(T):
    """Mass drift < 1e-10 (FP64-measured) on a 2048² film over 600 steps."""
    n = 2048
    s = sysc(n, n)
    st = gpu_run(s, rough(n, n, 17, amp=0.1), 600, T=T, meas=L.MEAS_MASS)
    m = np.array([r.mass for r in st.measures()])
    drift = np.abs(m - m[0]) / m[0]
    assert drift[-1] < 1e-10
    # FP16: the per-step noise floor is ~2.4e-11 on 2048² cells
    assert drift.max() < (1e-10 if T == np.float32 else 2e-10)


def test_fp32_rayleigh_taylor_short():
    # the hanging film is linearly unstable (the Float64 oracle diverges near
    # t = 2300 for this input), so compare over its finite part
    Lx, Ly, steps = 128, 128, 1500
    s = sysc(Lx, Ly, Tmax=steps, g=-0.001, gamma=0.0005)
    h0 = rough(Lx, Ly, 2, amp=0.01)
    ref = oracle.FusedState(oparams(s), h0).run(steps)
    st = gpu_run(s, h0, steps, T=np.float32)
    # the instability amplifies rounding differences like any perturbation
    assert rel_l2(st.height - 1, ref.height - 1) < 2e-3
    assert rel_l2(st.height, ref.height) < 1e-4


# ------------------------------------------------------------------ batch / server
def test_batch_matches_single():
    shapes = [(64, 64), (48, 32), (33, 17), (128, 32)]
    systems = [sysc(Lx, Ly, theta=th) for (Lx, Ly), th in zip(shapes, (1 / 9, 1 / 6, 1 / 12, 1 / 5))]
    hs = [droplet(Lx, Ly, min(Lx, Ly) // 4) for (Lx, Ly) in shapes]
    for T in (np.float64, np.float32, np.float16):
        b = sw.Batch(systems, T=T)
        for i, h in enumerate(hs):
            b.set_height(i, h)
        b.set_theta_wave(3, 1 / 5, 1 / 36, 1 / 98)
        b.step(100)
        b.step(37)
        for i, (sc, h) in enumerate(zip(systems, hs)):
            st = sw.Sys(sc, "GB300", T=T)
            st.height = h
            if i == 3:
                st.set_theta_wave(1 / 5, 1 / 36, 1 / 98)
            st.step(137)
            # exact in every mode: the FP32/FP16 mass correction is driven by
            # an exact fixed-point mass sum, whatever the strips of the batch
            # and of the single state
            assert np.array_equal(b.get_height(i), st.height), (T, i)
        if T == np.float64:
            ref = oracle.time_loop_literal(oparams(systems[0]), hs[0], 137)
            assert np.array_equal(b.get_height(0), ref.height)
        b.close()


@pytest.mark.parametrize("T", [np.float32, np.float16])
def test_batch_pair_strips_equal_single(T):
    """A batch on pair strips (set, and chosen by the batch tuner), with a
    θ-wave member, gives each lattice's result alone, bit for bit."""
    shapes = [(64, 64), (48, 32), (130, 34), (128, 32), (256, 20)]
    systems = [sysc(Lx, Ly, theta=th) for (Lx, Ly), th in zip(shapes, (1 / 9, 1 / 6, 1 / 12, 1 / 5, 1 / 8))]
    hs = [droplet(Lx, Ly, min(Lx, Ly) // 4) for (Lx, Ly) in shapes]
    singles = []
    for i, (sc, h) in enumerate(zip(systems, hs)):
        st = sw.Sys(sc, "GB300", T=T)
        st.height = h
        if i == 3:
            st.set_theta_wave(1 / 5, 1 / 36, 1 / 98)
        st.step(137)
        singles.append(st.height)
    for geo in ((-64, 16), None):
        b = sw.Batch(systems, T=T)
        if geo:
            b.set_geometry(*geo)
        for i, h in enumerate(hs):
            b.set_height(i, h)
        b.set_theta_wave(3, 1 / 5, 1 / 36, 1 / 98)
        b.step(100)
        b.step(37)
        b.sync()
        for i in range(len(shapes)):
            assert np.array_equal(b.get_height(i), singles[i]), (T, geo, i, b.geometry())
        if geo:
            assert b.geometry()[0] == geo[0]
        b.close()


def test_server_alone_equals_mixed():
    import time
    s1 = sysc(64, 64, theta=1 / 8, g=-5e-4)
    h1 = rough(64, 64, 31)
    sv = sw.Server(1 << 30, T=np.float32, steps_per_tick=50)
    rid = sv.submit(s1, h1, 330, dtheta=1 / 36, v=1 / 98)
    alone = _wait(sv, rid, (64, 64))
    others = [sv.submit(sysc(L_, L_), rough(L_, L_, k), 200 + 37 * k) for k, L_ in
              enumerate((128, 64, 192, 32))]
    time.sleep(0.01)
    rid2 = sv.submit(s1, h1, 330, dtheta=1 / 36, v=1 / 98)
    mixed = _wait(sv, rid2, (64, 64))
    outs = [_wait(sv, o, (L_, L_)) for o, L_ in zip(others, (128, 64, 192, 32))]
    assert np.array_equal(alone, mixed)
    st = sv.stats()
    assert st.completed == 6 and st.rejected == 0
    # the ticks are 50 steps, the requests 330 and 200 + 37 k: each stops
    # inside a tick, at exactly its own step count, like a solve run alone
    single = sw.Sys(s1, "GB300", T=np.float32)
    single.height = h1
    single.set_theta_wave(1 / 8, 1 / 36, 1 / 98)
    single.step(330)
    assert np.array_equal(alone, single.height)
    for k, (L_, out) in enumerate(zip((128, 64, 192, 32), outs)):
        st1 = sw.Sys(sysc(L_, L_), "GB300", T=np.float32)
        st1.height = rough(L_, L_, k)
        st1.step(200 + 37 * k)
        assert np.array_equal(out, st1.height), L_
    sv.close()


@pytest.mark.parametrize("T", [np.float32, np.float16])
def test_server_pair_and_one_column_sets(T):
    """The resident set runs as pair strips while every lattice has an even
    width, as one-column strips once an odd-width lattice joins; a lattice's
    result is the single state's either way, in FP32 and FP16 storage."""
    sv = sw.Server(1 << 30, T=T, steps_per_tick=40)
    cases = [((64, 100), 150, 3), ((128, 64), 90, 4), ((62, 130), 170, 5)]
    rids = [sv.submit(sysc(lx, ly, theta=1 / 7), rough(lx, ly, k), n, dtheta=1 / 36, v=1 / 98)
            for (lx, ly), n, k in cases]
    outs = [_wait(sv, r, shape) for r, (shape, _, _) in zip(rids, cases)]
    odd = ((63, 40), 120, 6)
    rid_odd = sv.submit(sysc(63, 40), rough(63, 40, 6), 120)
    rid_even = sv.submit(sysc(64, 100, theta=1 / 7), rough(64, 100, 3), 150, dtheta=1 / 36, v=1 / 98)
    out_odd = _wait(sv, rid_odd, (63, 40))
    out_even = _wait(sv, rid_even, (64, 100))
    sv.close()
    assert np.array_equal(out_even, outs[0])
    for ((lx, ly), n, k), out in zip(cases + [odd], outs + [out_odd]):
        st = sw.Sys(sysc(lx, ly, theta=1 / 7) if (lx, ly) != (63, 40) else sysc(63, 40), "GB300", T=T)
        st.height = rough(lx, ly, k)
        if (lx, ly) != (63, 40):
            st.set_theta_wave(1 / 7, 1 / 36, 1 / 98)
        st.step(n)
        assert np.array_equal(out, st.height), (lx, ly)


@pytest.mark.parametrize("geo", [(-64, 32), (-32, 16), (0, 48)])
def test_server_fixed_geometry_equals_single(geo):
    """swb_server_set_geometry changes the strips, not the results."""
    sv = sw.Server(1 << 30, T=np.float32, steps_per_tick=30)
    sv.set_geometry(*geo)
    cases = [((128, 100), 95, 7), ((64, 64), 70, 8)]
    rids = [sv.submit(sysc(lx, ly, theta=1 / 6), rough(lx, ly, k), n, dtheta=1 / 36, v=1 / 98)
            for (lx, ly), n, k in cases]
    outs = [_wait(sv, r, shape) for r, (shape, _, _) in zip(rids, cases)]
    sv.close()
    for ((lx, ly), n, k), out in zip(cases, outs):
        st = sw.Sys(sysc(lx, ly, theta=1 / 6), "GB300", T=np.float32)
        st.height = rough(lx, ly, k)
        st.set_theta_wave(1 / 6, 1 / 36, 1 / 98)
        st.step(n)
        assert np.array_equal(out, st.height), (geo, lx, ly)


def test_server_geometry_rejects_bad_arguments():
    sv = sw.Server(1 << 28, T=np.float32)
    for nt, rows in ((-128, 32), (64, 32), (-64, 0), (0, 1)):
        with pytest.raises(sw.SwbError):
            sv.set_geometry(nt, rows)
    sv.close()


def _wait(sv, rid, shape, timeout=60):
    import time
    t0 = time.time()
    while time.time() - t0 < timeout:
        done, out, info = sv.poll(rid, shape)
        if done:
            return out
        time.sleep(0.002)
    raise TimeoutError(rid)


def _wait_running(sv, rid, timeout=60):
    import time
    t0 = time.time()
    while time.time() - t0 < timeout:
        if sv.poll(rid)[2].status >= 1:
            return
        time.sleep(0.001)
    raise TimeoutError(rid)


def test_server_admission_by_hbm():
    sv = sw.Server(40 << 20, T=np.float32, steps_per_tick=20)
    big = sysc(1024, 1024)  # ~76 MB of state: larger than the budget
    rid = sv.submit(big, np.ones((1024, 1024)), 10)
    done, _, info = sv.poll(rid)
    assert info.status == L.SWB_ERR_OOM
    ids = [sv.submit(sysc(512, 512), rough(512, 512, k), 40) for k in range(4)]
    for i in ids:
        _wait(sv, i, None)
    st = sv.stats()
    assert st.completed == 4 and st.hbm_in_use == 0
    sv.close()


def test_server_sjf_admits_smallest_first():
    # one resident at a time (bound of 128x128 cells); while A runs, C (large)
    # and B (small) queue; shortest-job-first admits B before C
    sv = sw.Server(1 << 30, T=np.float32, steps_per_tick=100)
    sv.set_policy("sjf", 128 * 128)
    a = sv.submit(sysc(128, 128), rough(128, 128, 1), 4000)
    _wait_running(sv, a)
    c = sv.submit(sysc(128, 128), rough(128, 128, 2), 2000)
    b = sv.submit(sysc(32, 32), rough(32, 32, 3), 100)
    for rid in (a, b, c):
        _wait(sv, rid, None)
    info = {rid: sv.poll(rid)[2] for rid in (a, b, c)}
    assert info[b].t_admit < info[c].t_admit
    assert info[a].t_admit <= info[b].t_admit
    sv.close()


def test_server_sjf_sheds_largest_when_full():
    sv = sw.Server(1 << 30, T=np.float32, steps_per_tick=100)
    sv.set_policy("sjf", 128 * 128)
    sv.set_queue_limit(2)
    a = sv.submit(sysc(128, 128), rough(128, 128, 1), 6000)
    _wait_running(sv, a)  # resident: the bound keeps the others queued
    big1 = sv.submit(sysc(128, 128), rough(128, 128, 2), 3000)
    big2 = sv.submit(sysc(128, 128), rough(128, 128, 3), 2500)
    small = sv.submit(sysc(32, 32), rough(32, 32, 4), 100)  # queue full: big1 is shed
    assert small is not None
    huge = sv.submit(sysc(128, 128), rough(128, 128, 5), 9000)  # larger than all queued
    assert huge is None
    for rid in (a, big2, small):
        _wait(sv, rid, None)
    done, _, info = sv.poll(big1)
    assert not done and info.status == L.SWB_ERR_BUSY
    sv.close()


def test_server_fifo_refuses_when_full():
    sv = sw.Server(1 << 30, T=np.float32, steps_per_tick=100)
    sv.set_policy("fifo", 128 * 128)
    sv.set_queue_limit(1)
    a = sv.submit(sysc(128, 128), rough(128, 128, 1), 6000)
    _wait_running(sv, a)
    q = sv.submit(sysc(128, 128), rough(128, 128, 2), 100)
    small = sv.submit(sysc(32, 32), rough(32, 32, 4), 100)
    assert small is None  # FIFO never sheds a queued request
    for rid in (a, q):
        _wait(sv, rid, None)
    sv.close()


# ------------------------------------------------------------------ failure detection
def test_nan_detected():
    s = sysc(32, 32)
    st = sw.Sys(s, "GB300", T=np.float32)
    h = rough(32, 32)
    h[5, 7] = np.nan
    st.height = h
    st.step(3)
    with pytest.raises(sw.SwbError) as e:
        st.sync()
    assert e.value.status == L.SWB_ERR_NAN


# ------------------------------------------------------------------ first iterations
# The first iteration after the height is set runs alone (it takes h, u from
# the fields); every other iteration runs the steady kernel forms, replayed
# from CUDA graphs.  Re-setting the height after graphs exist must give what
# the same iterations give when they are issued in small chunks, without
# graphs (the stochastic rounding of FP32/FP16 depends on the iteration
# number, so both runs go through the same iterations).
@pytest.mark.parametrize("T", [np.float64, np.float32, np.float16])
@pytest.mark.parametrize("tau", [1.0, 0.8])
def test_height_reset_after_graphs(T, tau):
    s = sysc(96, 80, tau=tau, g=-1e-4)
    h_a, h_b = rough(96, 80, 11), rough(96, 80, 12)

    def run(before, after):
        st = sw.Sys(s, "GB300", T=T)
        st.set_geometry(64, 8)
        st.height = h_a
        for n in before:
            st.step(n)
        st.height = h_b  # the velocities carry on
        for n in after:
            st.step(n)
        return st.height

    graphs = run([200], [150])  # 64-iteration graphs before and after the reset
    chunks = run([1] * 5 + [13] * 15, [7] * 21 + [3])
    assert np.array_equal(graphs, chunks)
    if T == np.float64 and tau == 1.0:
        # and the literal oracle through the same sequence (τ = 1: the
        # populations before the reset drop out of the collision, so a
        # fresh oracle state with the same h and u is the same state)
        P = oparams(s)
        first = oracle.time_loop_literal(P, h_a, 200)
        ref = oracle.time_loop_literal(P, h_b, 150, ux0=first.velx, uy0=first.vely)
        assert np.array_equal(graphs, ref.height)


def test_batch_height_reset_matches_single():
    """One lattice of a batch starts over while the other carries on: both
    match single states that went through the same sequence."""
    shapes = [(64, 64), (96, 48)]
    systems = [sysc(Lx, Ly, g=-1e-4) for Lx, Ly in shapes]
    b = sw.Batch(systems, T=np.float32)
    for i, (Lx, Ly) in enumerate(shapes):
        b.set_height(i, rough(Lx, Ly, 20 + i))
    b.step(100)  # graphs of the steady batch form
    h_new = rough(96, 48, 31)
    b.set_height(1, h_new)
    b.step(70)
    single0 = sw.Sys(systems[0], "GB300", T=np.float32)
    single0.height = rough(64, 64, 20)
    single0.step(170)
    single1 = sw.Sys(systems[1], "GB300", T=np.float32)
    single1.height = rough(96, 48, 21)
    single1.step(100)
    single1.height = h_new
    single1.step(70)
    assert np.array_equal(b.get_height(0), single0.height)
    assert np.array_equal(b.get_height(1), single1.height)
    b.close()


@pytest.mark.parametrize("T", [np.float64, np.float32])
def test_time_loop_arbitrary_callback_on_fused_state(T):
    """time_loop(sys, state, f, measure) with a callback of the user's own (it
    reads the height and adds a force after the force sum every iteration,
    like the reference's callbacks, src/simulate.jl:68-96) runs on a fused
    state: bit for bit the per-op Float64 path with the same callback, from
    the same (for an FP32 state, FP32-rounded) initial film."""
    Lx, Ly, steps = 40, 32, 60
    s = sysc(Lx, Ly, Tmax=steps, delta=2.0)
    h0 = droplet(Lx, Ly, 10)

    def push(measure, state):
        measure.append(float(state.height.max()))
        state.Fx = state.Fx + 1e-5 * state.height

    ref = sw.Sys(s, "GB300-plain", T=np.float64)
    # an FP32 state holds h0 rounded to FP32: the per-op run starts from that
    ref.height = h0 if T == np.float64 else h0.astype(np.float32).astype(np.float64)
    m_ref = []
    sw.time_loop(s, ref, push, m_ref)
    st = sw.Sys(s, "GB300", T=T)
    st.height = h0
    m = []
    sw.time_loop(s, st, push, m)
    assert m == m_ref and len(m) == steps
    if T == np.float64:
        assert np.array_equal(st.height, ref.height)
    else:  # the handed-back height is stored in the state's FP32 field
        assert np.allclose(st.height, ref.height, rtol=2 ** -23, atol=0)
    # and the state goes on from there in its own precision
    st.step(10)
    assert np.isfinite(st.height).all()
