"""Pins the CPU oracle to the reference's own golden vectors.

Every case restates an assertion of the reference test-suite (test/*.jl) or
a doctest (src/*.jl) with the same inputs and the same comparison (`==` or
`≈ atol`).  Numbers come from tests/golden/reference_unit.json.
"""
import math

import numpy as np
import pytest


def M(rows):
    return np.array(rows, dtype=np.float64)


# ---------------------------------------------------------------- differences
def test_gradient_ramp(orc, golden, ramp):
    # test/differences.jl:3-32: all(outputx .== solx), all(outputy .== soly)
    gx, gy = orc.gradient(ramp)
    assert np.array_equal(gx, M(golden["grad_solx"]["rows"]))
    assert np.array_equal(gy, M(golden["grad_soly"]["rows"]))


def test_laplacian_ramp(orc, golden, ramp):
    # test/differences.jl:104-124: ∇²f!(output, f, -1.0) ≈ sol atol 1e-10
    out = orc.laplacian(ramp, -1.0)
    assert np.allclose(out, M(golden["lap_sol"]["rows"]), rtol=0, atol=1e-10)


def test_circshift_convention(orc):
    # circshift!(dst, src, (1,0)) puts src[i-1, j] at (i, j) (src/collide.jl:36-59)
    a = np.asfortranarray(np.arange(12.0).reshape(3, 4, order="F"))
    s = orc.circshift(a, (1, 0))
    assert s[1, 0] == a[0, 0] and s[0, 0] == a[2, 0]
    s = orc.circshift(a, (-1, 1))
    assert s[0, 1] == a[1, 0]


# ---------------------------------------------------------------- pressure
def test_filmpressure_no_contact_angle(orc, golden, ramp):
    # test/pressure.jl:18-34: n=3, m=2, γ=1, hmin=0.1, hcrit=0.1, θ=0 → sol, atol 1e-10
    sol = M(golden["lap_sol"]["rows"])
    p = orc.filmpressure(ramp, 1.0, 0.0, 3, 2, 0.1, 0.1)
    assert np.allclose(p, sol, rtol=0, atol=1e-10)
    praw = orc.filmpressure_raw(ramp, 1.0, 0.0, 3, 2, 0.1, 0.1)
    assert np.allclose(praw, sol, rtol=0, atol=1e-10)


def test_filmpressure_gradient_and_angle(orc, golden, ramp):
    # test/pressure.jl:35-43: hcrit=0, θ=1/2 → -1 .* (-sol .+ 20 .* ((0.1 ./ f).^3 .- (0.1 ./ f).^2))
    sol = M(golden["lap_sol"]["rows"])
    want = -1 * (-sol + 20 * ((0.1 / ramp) ** 3 - (0.1 / ramp) ** 2))
    p = orc.filmpressure(ramp, 1.0, 0.5, 3, 2, 0.1, 0.0)
    assert np.allclose(p, want, rtol=0, atol=1e-10)
    p2 = orc.filmpressure(ramp, 1.0, 0.0, 3, 2, 0.1, 0.0, theta_field=np.full((5, 5), 0.5))
    assert np.array_equal(p, p2)
    praw = orc.filmpressure_raw(ramp, 1.0, 0.5, 3, 2, 0.1, 0.0)
    assert np.allclose(praw, want, rtol=0, atol=1e-10)


def test_filmpressure_no_gradient(orc):
    # test/pressure.jl:44-53: h=1, θ=1/2, hcrit=0 → -2(0.1^2-0.1)
    p = orc.filmpressure(np.ones((5, 5)), 1.0, 0.5, 3, 2, 0.1, 0.0)
    assert np.allclose(p, -2 * (0.1 ** 2 - 0.1), rtol=0, atol=1e-10)


def test_filmpressure_doctest(orc, golden, ramp):
    # src/pressure.jl:52-62: result ≈ -100 .* pressure atol 1e-12
    g = golden["pressure_doctest"]
    a = g["args"]
    p = orc.filmpressure_raw(ramp, a["gamma"], a["theta"], a["n"], a["m"], a["hmin"], a["hcrit"])
    assert np.allclose(-100 * p, M(g["rows"]), rtol=0, atol=g["atol"])


def test_filmpressure_raw_rejects_exponents(orc, ramp):
    # src/pressure.jl:101-107: DomainError for (n, m) other than (9,3), (3,2)
    with pytest.raises(ValueError):
        orc.filmpressure_raw(ramp, 1.0, 0.0, 4, 2, 0.1, 0.1)


def test_power_broad(orc, golden):
    # test/pressure.jl:139-160
    g = golden["power_broad"]
    lib = orc.lib()
    for i, n in enumerate(g["n"]):
        assert lib.orc_power_broad(2.0, n) == g["int2"][i]
        assert lib.orc_power_broad(5.0, n) == g["five"][i]
        for j, a in enumerate(g["vec"]["args"]):
            assert lib.orc_power_broad(a, n) == g["vec"]["rows"][i][j]


# ---------------------------------------------------------------- forcing
def test_slippage(orc, golden):
    # test/forcing.jl:13-69 (h = 1, μ = 1/6)
    g = golden["slippage"]
    h = np.ones((5, 5))
    for c in g["cases"]:
        sx, sy = orc.slippage(h, np.full((5, 5), c["ux"]), np.full((5, 5), c["uy"]),
                              c["delta"], 1 / 6)
        if c.get("exact"):
            assert np.all(sx == c["sx"]) and np.all(sy == c["sy"])
        else:
            assert np.allclose(sx, c["sx"], rtol=0, atol=g["atol"])
            assert np.allclose(sy, c["sy"], rtol=0, atol=g["atol"])


def test_hgradp_ramp(orc, golden, ramp):
    # test/forcing.jl:104-139: h = 1 (Sys default), pressure = ramp; exact ==
    gx, gy = orc.hgradp(np.ones((5, 5)), ramp)
    assert np.array_equal(gx, M(golden["grad_solx"]["rows"]))
    assert np.array_equal(gy, M(golden["grad_soly"]["rows"]))


def test_hgradp_doctest(orc, golden):
    # src/forcing.jl:147-157: 10x10 ramp: h∇px[1,:] .== -4, h∇px[2,:] .== 1
    p = np.asfortranarray(np.arange(1.0, 101.0).reshape(10, 10, order="F"))
    gx, _ = orc.hgradp(np.ones((10, 10)), p)
    assert np.all(gx[0, :] == golden["hgradp_doctest"]["row1"])
    assert np.all(gx[1, :] == golden["hgradp_doctest"]["row2"])


def test_inclination(orc, golden):
    # test/forcing.jl:166-184: exact ==
    g = golden["inclination"]
    h = np.ones((5, 5))
    for c in g["cases"]:
        Fx, Fy = orc.inclination(np.zeros((5, 5)), np.zeros((5, 5)), h, g["alpha"], t=c["t"],
                                 tstart=0, tsmooth=1)
        want = c["value"] if "value" in c else 0.1 * (0.5 + 0.5 * math.tanh(1.0))
        assert np.all(Fx == want) and np.all(Fy == want)


# ---------------------------------------------------------------- equilibrium
def test_equilibrium(orc):
    # test/equilibrium.jl:6-83
    z, o = np.zeros((5, 5)), np.ones((5, 5))
    assert np.all(orc.equilibrium(z, z, z, 0.0) == 0.0)
    f = orc.equilibrium(o, z, z, 0.0)
    assert np.all(f[:, :, 0] == 1.0) and np.all(f[:, :, 1:] == 0.0)
    f = orc.equilibrium(o, z, z, 0.1)
    assert np.all(f[:, :, 0] == 1.0 - 1 / 12)
    assert np.allclose(f[:, :, 1:5], 1 / 9 * 1.5 * 0.1)
    assert np.allclose(f[:, :, 5:9], 1 / 36 * 1.5 * 0.1)
    ux, uy = np.full((5, 5), 0.1), np.full((5, 5), -0.1)
    f = orc.equilibrium(o, ux, uy, 0.0)
    assert np.all(f[:, :, 0] == 1.0 - 2 / 3 * 0.02)
    assert np.allclose(f[:, :, 1], 1 / 9 * (3 * 0.1 + 4.5 * 0.01 - 3 / 2 * 0.02))
    assert np.allclose(f[:, :, 2], 1 / 9 * (3 * -0.1 + 4.5 * 0.01 - 3 / 2 * 0.02))
    assert np.allclose(f[:, :, 3], 1 / 9 * (3 * -0.1 + 4.5 * 0.01 - 3 / 2 * 0.02))
    assert np.allclose(f[:, :, 4], 1 / 9 * (3 * 0.1 + 4.5 * 0.01 - 3 / 2 * 0.02))
    assert np.allclose(f[:, :, 5], 1 / 36 * (-3 / 2 * 0.02))
    assert np.allclose(f[:, :, 6], 1 / 36 * (3 * -0.2 + 4.5 * 0.2 ** 2 - 3 / 2 * 0.02))
    assert np.allclose(f[:, :, 7], 1 / 36 * (-3 / 2 * 0.02))
    assert np.allclose(f[:, :, 8], 1 / 36 * (3 * 0.2 + 4.5 * 0.2 ** 2 - 3 / 2 * 0.02))
    f = orc.equilibrium(o, ux, uy, 0.1)
    assert np.all(f[:, :, 0] == 1.0 - 1 / 12 - 2 / 3 * 0.02)
    assert np.allclose(f[:, :, 1], 1 / 9 * (1.5 * 0.1 + 3 * 0.1 + 4.5 * 0.01 - 3 / 2 * 0.02))
    assert np.allclose(f[:, :, 5], 1 / 36 * (1.5 * 0.1 + -3 / 2 * 0.02))
    assert np.allclose(f[:, :, 8], 1 / 36 * (1.5 * 0.1 + 3 * 0.2 + 4.5 * 0.2 ** 2 - 3 / 2 * 0.02))


def test_equilibrium_doctest(orc):
    # src/equilibrium.jl:38-53: g=0.1, ux=0.1 → f0 = 0.91 printed; g=0 → 1 - 2/3*0.01
    o, z = np.ones((5, 5)), np.zeros((5, 5))
    f = orc.equilibrium(o, np.full((5, 5), 0.1), z, 0.1)
    assert np.all(np.round(f[:, :, 0], 12) == 0.91)
    f = orc.equilibrium(o, np.full((5, 5), 0.1), z, 0.0)
    assert np.allclose(f[:, :, 0], 1 - 2 / 3 * 0.01)


# ---------------------------------------------------------------- collide
def _shift(a, s):
    return np.roll(a, s, axis=(0, 1))


SHIFTS = [(0, 0), (1, 0), (0, 1), (-1, 0), (0, -1), (1, 1), (-1, 1), (-1, -1), (1, -1)]


def test_bgk_tau1_no_forces(orc):
    # test/collide.jl:27-43 and doctest src/collide.jl:33-59
    feq = np.ones((5, 5, 9), order="F")
    feq[0, 0, :] = 2.0
    fout, _ = orc.bgk_stream(feq, np.ones((5, 5, 9)), np.zeros((5, 5)), np.zeros((5, 5)), 1.0)
    for q, s in enumerate(SHIFTS):
        assert np.array_equal(fout[:, :, q], _shift(feq[:, :, 0], s))
    assert fout[1, 1, 5] == 2.0  # "moved one down and one to the right"


def test_bgk_tau1_forces(orc):
    # test/collide.jl:44-71: ftemp = 1.2, feq = 1, Fx = 0.1, Fy = -0.1; exact ==
    feq = np.ones((5, 5, 9), order="F")
    fout, _ = orc.bgk_stream(feq, np.full((5, 5, 9), 1.2), np.full((5, 5), 0.1),
                             np.full((5, 5), -0.1), 1.0)
    e = feq[:, :, 0]
    want = [e, e + 1 / 30, e - 1 / 30, e - 1 / 30, e + 1 / 30, e, e - 1 / 24 * 0.2, e,
            e + 1 / 24 * 0.2]
    for q, s in enumerate(SHIFTS):
        assert np.array_equal(fout[:, :, q], _shift(want[q], s)), q


@pytest.mark.parametrize("forces", [False, True])
def test_bgk_tau075(orc, forces):
    # test/collide.jl:72-138: ftemp = 1 (set_dist!), feq = 1 with feq[1,1,:] = 2
    feq = np.ones((5, 5, 9), order="F")
    feq[0, 0, :] = 2.0
    ftemp = np.ones((5, 5, 9), order="F")
    F = 0.1 if forces else 0.0
    fout, _ = orc.bgk_stream(feq, ftemp, np.full((5, 5), F), np.full((5, 5), -F), 0.75)
    onebytau, omega = 1.0 / 0.75, 1.0 - 1.0 / 0.75
    base = omega * 1.0 + onebytau * feq[:, :, 0]
    if forces:
        add = [0, 1 / 30, -1 / 30, -1 / 30, 1 / 30, 0, -1 / 24 * 0.2, 0, 1 / 24 * 0.2]
    else:
        add = [0] * 9
    assert np.array_equal(fout[:, :, 0], base)
    for q in range(1, 9):
        w = _shift(base + add[q], SHIFTS[q])
        if q == 1:  # the reference compares population 2 with ≈ (test/collide.jl:88)
            assert np.allclose(fout[:, :, q], w)
        else:
            assert np.array_equal(fout[:, :, q], w), q


# ---------------------------------------------------------------- moments
def test_moments(orc, golden):
    # test/moments.jl:14-134: populations are filled cumulatively
    f = np.zeros((5, 5, 9), order="F")
    for st in golden["moments"]["steps"]:
        q, v = st["set"]
        f[:, :, q] = v
        h, ux, uy = orc.moments(f)
        if q == 0:
            assert np.all(h == 1.0)
            continue
        assert np.all(h == st["h"])
        wx, wy = eval(st["ux"]), eval(st["uy"])
        if st.get("exact"):
            assert np.all(ux == wx) and np.all(uy == wy)
        else:
            assert np.allclose(ux, wx, rtol=0, atol=1e-10)
            assert np.allclose(uy, wy, rtol=0, atol=1e-10)


def test_moments_doctest(orc):
    # src/moments.jl:18-35
    f = np.zeros((5, 5, 9), order="F")
    f[:, :, 0], f[:, :, 1] = 1.0, 0.1
    h, ux, uy = orc.moments(f)
    assert np.all(h == 1.1) and np.all(ux == 0.1 / 1.1) and np.all(uy == 0.0)


# ---------------------------------------------------------------- measures
def test_wetted(orc, golden):
    # test/measures.jl:2-24 (wetted!(area, maxheight, height, t) form)
    h = np.zeros((5, 5))
    h[1:3, 1:3] = 1.0
    assert orc.wetted(h) == golden["wetted"]["block_2_3"]
    h = np.zeros((5, 5))
    for t in range(1, 6):
        h[t - 1, t - 1] = t
        assert orc.wetted(h) == golden["wetted"]["diag_series"][t - 1]
        assert h.max() == t


def test_surfacearea(orc, golden, ramp):
    # test/measures.jl:55-115
    gx, gy = M(golden["grad_solx"]["rows"]), M(golden["grad_soly"]["rows"])
    solsurf = np.sum(np.sqrt(gx ** 2 + gy ** 2 + 1))
    th = np.full((5, 5), 0.5)
    a, e = orc.surfacearea(ramp, th)
    assert a == pytest.approx(solsurf, abs=1e-10)
    assert e == pytest.approx(solsurf - np.sum(np.cos(np.pi * th)), abs=1e-10)
    th = np.full((5, 5), 1 / 9)
    a1, e1 = orc.surfacearea(ramp, th)
    a2, e2 = orc.surfacearea(ramp, 1 / 9)
    want_e = solsurf - 25 * math.cos(math.pi / 9)
    for a_, e_ in ((a1, e1), (a2, e2)):
        assert a_ == pytest.approx(solsurf, abs=1e-10)
        assert e_ == pytest.approx(want_e, abs=1e-10)
    h = ramp.copy(order="F")
    for t in range(1, 6):
        h[t - 1, t - 1] = t
        th[t - 1, t - 1] = 0.0
        d1, d2 = orc.gradient(h)
        a, e = orc.surfacearea(h, th)
        sc = np.sum(np.sqrt(d1 ** 2 + d2 ** 2 + 1))
        assert a == pytest.approx(sc)
        assert e == pytest.approx(sc - np.sum([orc.cospi(x) for x in th.ravel()]))


def test_singledroplet(orc):
    # test/initialvalues.jl: max == rad*(1-cospi(θ)) at the centre
    h = orc.singledroplet(100, 100, 50, 1 / 3, (50, 50))
    assert h.max() == 50 * (1 - orc.cospi(1 / 3))
    assert np.unravel_index(np.argmax(h), h.shape) == (49, 49)


# ---------------------------------------------------------------- time loops
def test_flat_interface_bit_exact(orc, golden):
    # test/simulate.jl:3-7: all(h .== 1.0), sum(h) == 625
    g = golden["simulate"]["flat"]
    P = orc.params(g["L"], g["L"], Tmax=g["Tmax"], tdump=g["tdump"])
    r = orc.time_loop_literal(P, np.ones((g["L"], g["L"])), g["Tmax"])
    assert np.all(r.height == 1.0)
    assert np.sum(r.height) == 625
    fs = orc.FusedState(P, np.ones((g["L"], g["L"])))
    rf = fs.run(g["Tmax"])
    assert np.all(rf.height == 1.0)


@pytest.mark.parametrize("case", ["plain", "gravity_tau", "theta_field", "wetted", "incl"])
def test_fused_equals_literal(orc, case):
    """The fused OpenMP oracle performs the literal oracle's arithmetic."""
    rng = np.random.default_rng(7)
    Lx, Ly = 13, 9
    kw = {}
    opts = {}
    if case == "gravity_tau":
        kw = dict(g=-0.002, tau=0.8)
    P = orc.params(Lx, Ly, Tmax=40, tdump=7, **kw)
    h0 = 1.0 + 0.1 * rng.uniform(-1, 1, (Lx, Ly))
    if case == "theta_field":
        opts["theta_field"] = 1 / 9 + 0.05 * rng.uniform(-1, 1, (Lx, Ly))
    if case == "wetted":
        h0 = orc.singledroplet(Lx, Ly, 5, 1 / 4, (7, 5))
        opts["callback"] = "wetted"
    if case == "incl":
        opts["callback"] = "inclination"
        opts["incl"] = {"alpha": (1e-3, -2e-4), "loop_time": True, "tstart": 10, "tsmooth": 5}
    r = orc.time_loop_literal(P, h0, 40, record_dh=True, **opts)
    fs = orc.FusedState(P, h0)
    rf = fs.run(25, record_dh=True, **opts) if case != "incl" else fs.run(40, record_dh=True, **opts)
    if case != "incl":
        rf2 = fs.run(15, record_dh=True, **opts)  # split runs continue exactly
        rf = rf2
    assert np.array_equal(r.height, rf.height)
    assert np.array_equal(r.velx, rf.velx)
    assert np.array_equal(r.vely, rf.vely)
