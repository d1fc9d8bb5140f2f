"""Write tests/golden/reference_unit.json.

The reference (Swalbe.jl) is Julia and cannot be executed in this
environment, so its golden vectors are taken from its own test files and
doctests, read as text.  Each entry below is a transcription of the numbers
the reference asserts, with the file:line it comes from (paths relative to
the Swalbe.jl project root).  Matrices are written row by row exactly as the
Julia literals are, so ``np.array(rows)[i-1, j-1]`` is Julia's ``A[i, j]``.

Run ``python tests/golden/make_golden.py`` to regenerate the JSON.
"""
import json
import os

G = {}

# test/differences.jl:21-32 (also src/differences.jl:125-139, test/forcing.jl:119-128,
# test/measures.jl:66-79): ∇f! of reshape(1:25,5,5); `==` comparison.
G["grad_solx"] = {
    "src": "test/differences.jl:21-32",
    "rows": [[-1.5] * 5, [1.0] * 5, [1.0] * 5, [1.0] * 5, [-1.5] * 5],
}
G["grad_soly"] = {
    "src": "test/differences.jl:21-32",
    "rows": [[-7.5, 5.0, 5.0, 5.0, -7.5]] * 5,
}
# test/differences.jl:104-124: ∇²f!(output, f, -1.0) of the ramp; atol 1e-10.
# The same matrix is `sol` in test/pressure.jl:12-17 and the doctest
# src/differences.jl:39-43 / src/pressure.jl:54-58.
G["lap_sol"] = {
    "src": "test/differences.jl:117-123",
    "rows": [[-30.0, -5.0, -5.0, -5.0, 20.0],
             [-25.0, 0.0, 0.0, 0.0, 25.0],
             [-25.0, 0.0, 0.0, 0.0, 25.0],
             [-25.0, 0.0, 0.0, 0.0, 25.0],
             [-20.0, 5.0, 5.0, 5.0, 30.0]],
}
# src/pressure.jl:52-62 doctest: filmpressure!(p, h, dgrad, 0.01, 0.0, 3, 2, 0.1, 0.05);
# result ≈ -100 .* pressure, atol 1e-12.
G["pressure_doctest"] = {
    "src": "src/pressure.jl:52-62",
    "args": {"gamma": 0.01, "theta": 0.0, "n": 3, "m": 2, "hmin": 0.1, "hcrit": 0.05},
    "rows": [[30.0, 5.0, 5.0, 5.0, -20.0],
             [25.0, 0.0, 0.0, 0.0, -25.0],
             [25.0, 0.0, 0.0, 0.0, -25.0],
             [25.0, 0.0, 0.0, 0.0, -25.0],
             [20.0, -5.0, -5.0, -5.0, -30.0]],
    "atol": 1e-12,
}
# test/pressure.jl:139-160: power_broad
G["power_broad"] = {
    "src": "test/pressure.jl:139-160",
    "n": [3, 6],
    "int2": [8, 64],
    "five": [125.0, 15625.0],
    "vec": {"args": [2.0, 3.0, 4.0], "rows": [[8.0, 27.0, 64.0], [64.0, 729.0, 4096.0]]},
}
# test/forcing.jl:13-69: slippage!, h = 1, μ = 1/6
G["slippage"] = {
    "src": "test/forcing.jl:13-69",
    "cases": [
        {"ux": 0.0, "uy": 0.0, "delta": 1.0, "sx": 0.0, "sy": 0.0, "exact": True},
        {"ux": 0.1, "uy": 0.0, "delta": 1.0, "sx": 0.1 / 11, "sy": 0.0},
        {"ux": 0.0, "uy": 0.1, "delta": 1.0, "sx": 0.0, "sy": 0.1 / 11},
        {"ux": -0.1, "uy": 0.1, "delta": 1.0, "sx": -0.1 / 11, "sy": 0.1 / 11},
        {"ux": -0.1, "uy": 0.1, "delta": 0.0, "sx": -0.1 / 2, "sy": 0.1 / 2},
    ],
    "atol": 1e-10,
}
# src/forcing.jl:147-157 doctest: 10x10, pressure = reshape(1:100,10,10), h = 1:
# h∇px[1,:] == -4, h∇px[2,:] == 1 (exact).
G["hgradp_doctest"] = {"src": "src/forcing.jl:147-157", "row1": -4.0, "row2": 1.0}
# test/forcing.jl:166-184: inclination!([0.1,0.1], state, t, tstart=0, tsmooth=1), h = 1
G["inclination"] = {
    "src": "test/forcing.jl:173-183",
    "alpha": [0.1, 0.1],
    "cases": [{"t": 0, "value": 0.05}, {"t": 1, "value_formula": "0.1*(0.5+0.5*tanh(1.0))"}],
}
# test/equilibrium.jl:6-83 (values given as formulas; see the test for exact/≈)
G["equilibrium"] = {"src": "test/equilibrium.jl:6-83"}
# test/collide.jl:27-123 (τ = 1 and τ = 0.75, forces ±0.1)
G["collide"] = {"src": "test/collide.jl:27-138", "tau2": 0.75, "ftemp_fill": 1.2}
# test/moments.jl:14-134
G["moments"] = {
    "src": "test/moments.jl:14-134",
    "steps": [
        {"set": [0, 1.0], "h": 1.0},
        {"set": [1, 0.1], "h": 1.1, "ux": "0.1/1.1", "uy": "0.0", "exact": True},
        {"set": [2, 0.2], "h": 1.3, "ux": "0.1/1.3", "uy": "0.2/1.3", "exact": True},
        {"set": [3, -0.2], "h": 1.1, "ux": "0.3/1.1", "uy": "0.2/1.1"},
        {"set": [4, -0.1], "h": 1.0, "ux": "0.3/1.0", "uy": "0.3/1.0"},
        {"set": [5, 0.1], "h": 1.1, "ux": "0.4/1.1", "uy": "0.4/1.1"},
    ],
}
# test/measures.jl:2-24 wetted!; test/measures.jl:55-115 surfacearea!
G["wetted"] = {"src": "test/measures.jl:2-24", "block_2_3": 4, "diag_series": [1, 2, 3, 4, 5]}
# test/simulate.jl: integration tests (physics tolerances, not bit pins)
G["simulate"] = {
    "flat": {"src": "test/simulate.jl:3-7", "L": 25, "Tmax": 200, "tdump": 100},
    "random": {"src": "test/simulate.jl:16-21", "L": 25, "Tmax": 10000, "eps": 0.1,
               "bound": 0.1},
    "rayleigh_taylor": {"src": "test/simulate.jl:32-35", "L": 100, "Tmax": 1000, "g": -0.002,
                        "kx": 4, "ky": 5, "eps": 0.01},
    "droplet": {"src": "test/simulate.jl:42-60", "L": 150, "R": 35, "Tmax": 10000,
                "delta": 3.0, "theta0": 1 / 6, "theta": 1 / 9, "rtol": 0.10},
    "sliding": {"src": "test/simulate.jl:146-155", "L": 150, "R": 35, "Tmax": 5000,
                "delta": 2.0, "fx": 1e-4},
}

if __name__ == "__main__":
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_unit.json")
    with open(out, "w") as fh:
        json.dump(G, fh, indent=1)
    print("wrote", out)
