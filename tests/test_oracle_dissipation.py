"""Known answers of the reference's dissipation tests, checked on the oracle.

  TestShockFinder     DG2D/dfr_shock_capturing_test.go:11-50   (shocked-element pattern, N = 2..4)
  TestDissipation     model_problems/Euler2D/euler_test.go:418-518 (element areas, vertex maxima)
  TestDissipation2    model_problems/Euler2D/euler_test.go:520-680 (RT gradient of polynomials, N = 4)
"""
import numpy as np
import pytest

from conftest import fixture, golden
import oracle
from gocfd_gb300 import meshes


def solver(N, name, **kw):
    m = meshes.read_mesh(fixture(name))
    return oracle.OracleSolver(N, m.VX, m.VY, m.EToV, m.bc_edges, **kw), m


@pytest.mark.parametrize("N", [2, 3, 4])
def test_shock_finder_pattern(N):
    """Mach 2 normal shock at x = 0: elements 2, 3, 7, 8 hold the jump."""
    s, _ = solver(N, "test_10tris_centered.neu")
    U1, U2 = oracle.shock_conditions(2.0)
    x = s.geo.SolX
    rho = np.where(x < 0.0, U1[0], U2[0])
    threshold = 0.0075  # ShockSigmaThreshold (dfr_shock_capturing.go:83)
    shocked = [s.shock_indicator(rho[:, k], 3.0) > threshold for k in range(s.K)]
    assert shocked == golden("shock_finder_pattern")["pattern"]


def test_element_areas_tris_9():
    s, _ = solver(1, "test_tris_9.neu")
    assert np.allclose(2.0 * s.geo.Jdet, 0.25, atol=1e-6)


def test_vertex_max_of_element_ids():
    s, _ = solver(1, "test_tris_9.neu", limiter="PerssonC0")
    v = s.vertex_max(np.arange(s.K, dtype=np.float64))
    assert v.tolist() == [1, 3, 4, 5, 7, 9, 9, 6, 8, 9]


def test_rt_gradient_of_polynomials_n4():
    """d/dx, d/dy of x+y, x^2+y^2, x^3+y^3, x^4+y^4 at every flux point, exact at N = 4."""
    s, _ = solver(4, "test_tris_5.neu", flux="average")
    X, Y = s.geo.SolX, s.geo.SolY
    Q = np.stack([X + Y, X ** 2 + Y ** 2, X ** 3 + Y ** 3, X ** 4 + Y ** 4])
    gx, gy = s.gradient(Q)
    FX, FY = s.geo.FluxX, s.geo.FluxY
    for n in range(4):
        p = n + 1
        assert np.abs(gx[n] - p * FX ** (p - 1)).max() < 1e-6
        assert np.abs(gy[n] - p * FY ** (p - 1)).max() < 1e-6


def test_dissipated_rhs_of_freestream_is_zero():
    """A uniform state has no sensor energy, no gradient and no viscous flux."""
    s, _ = solver(2, "test_tris_6_nowall.neu", limiter="PerssonC0", minf=2.0, flux="average")
    r = s.rhs(s.Q)
    assert np.abs(r).max() < 1e-9


def test_dissipation_changes_a_shocked_rhs():
    m = meshes.sod_channel(20, 2)
    a = oracle.OracleSolver(2, m.VX, m.VY, m.EToV, m.bc_edges, init="shocktube", limiter="PerssonC0")
    b = oracle.OracleSolver(2, m.VX, m.VY, m.EToV, m.bc_edges, init="shocktube")
    ra, rb = a.rhs(a.Q), b.rhs(b.Q)
    assert np.all(np.isfinite(ra))
    assert np.abs(ra - rb).max() > 1e-3 * np.abs(rb).max()
