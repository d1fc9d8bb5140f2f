"""Contact-angle patterns (src/initialvalues.jl:423-581), host side, against
the reference's own tests (test/initialvalues.jl:104-173) and doctests."""
import numpy as np
import pytest

import swalbe_gb300 as sw

T0, D = 1 / 9, 1 / 36


def J(a, b):  # Julia 1-based indexing
    return (a - 1, b - 1)


def test_ellipse_default_offcentre_negative_larger():
    th, _ = sw.ellipsepattern(np.ones((100, 100)), T0)
    assert th.shape == (100, 100) and th[J(50, 50)] == T0 + D and th[J(1, 1)] == T0
    th, _ = sw.ellipsepattern(np.ones((100, 100)), T0, center=(20, 20))
    assert th[J(20, 20)] == T0 + D and th[J(100, 100)] == T0
    th, _ = sw.ellipsepattern(np.ones((100, 100)), T0, δa=-1 / 36)
    assert th[J(50, 50)] == T0 - D and th[J(100, 100)] == T0
    th, _ = sw.ellipsepattern(np.ones((100, 100)), T0, a=10, b=20)
    assert th[J(40, 50)] == T0 + D and th[J(70, 50)] == T0 + D and th[J(100, 100)] == T0


def test_triangle():
    lx, ly = 100, 100
    th, _ = sw.trianglepattern(np.ones((100, 100)), T0)
    assert np.all(th > 0) and th[J(1, 1)] == T0 and th[J(50, 50)] == T0 + D
    th, _ = sw.trianglepattern(np.ones((100, 100)), T0, center=(lx / 3, 2 * ly / 3))
    assert th[J(1, 1)] == T0 and th[J(round(lx / 3), round(2 * ly / 3))] == T0
    th, _ = sw.trianglepattern(np.ones((100, 100)), T0, center=(0, 2 * ly / 3))
    assert th[J(1, 1)] == T0 and th[J(round(lx / 3), round(2 * ly / 3))] == T0
    assert th[J(60, 1)] == T0 + D
    th, _ = sw.trianglepattern(np.ones((100, 100)), T0, δa=-1 / 36)
    assert th[J(1, 1)] == T0 and th[J(50, 50)] == T0 - D
    th, _ = sw.trianglepattern(np.ones((100, 100)), T0, side=30)
    assert th[J(1, 1)] == T0 and th[J(50, 50)] == T0 + D and th[J(50, 60)] == T0 + D


def test_triangle_doctest_vertices():
    # src/initialvalues.jl:530-545
    th, P = sw.trianglepattern(np.ones((50, 50)), T0, side=20)
    want = [(15.0, 19.226497308103742), (35.0, 19.226497308103742), (25.0, 36.547005383792516)]
    got = sorted(P.vertices)
    for (a, b), (c, d) in zip(got, sorted(want)):
        assert a == pytest.approx(c, abs=1e-12) and b == pytest.approx(d, abs=1e-12)
    assert th[J(25, 25)] == pytest.approx(0.1388888888888889, abs=1e-16)


def test_box():
    lx, ly = 100, 100
    th, _ = sw.boxpattern(np.ones((100, 100)), T0)
    assert np.all(th > 0) and th[J(1, 1)] == T0 and th[J(50, 50)] == T0 + D
    th, _ = sw.boxpattern(np.ones((100, 100)), T0, center=(lx / 3, 2 * ly / 3))
    assert th[J(1, 1)] == T0 and th[J(round(2 * ly / 3), round(lx / 3))] == T0 + D
    th, _ = sw.boxpattern(np.ones((100, 100)), T0, center=(0, 2 * ly / 3))
    assert th[J(20, 1)] == T0 and th[J(60, 1)] == T0 + D
    th, _ = sw.boxpattern(np.ones((100, 100)), T0, δa=-1 / 36)
    assert th[J(1, 1)] == T0 and th[J(50, 50)] == T0 - D
    th, _ = sw.boxpattern(np.ones((100, 100)), T0, side=30)
    assert th[J(1, 1)] == T0 and th[J(50, 50)] == T0 + D and th[J(65, 65)] == T0 + D
