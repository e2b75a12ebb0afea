"""Pins the oracle (CPU restatement) against the reference's own known-answer
tests for this path.  CPU only.

  TestEuler interpolation      model_problems/Euler2D/euler_test.go:55-90
  TestEuler freestream         euler_test.go:173-228
  CheckFlux0 polynomial flux   euler_test.go:229-260, 903-982
  TestEuler vortex divergence  euler_test.go:262-322
  TestFluidFunctions           euler_test.go:32-45
  TestDivergence               DG2D/dfr_startup_test.go:293-368
  TestIVortex                  model_problems/Euler2D/isentropic_vortex/analytic_vortex_test.go:11-23
"""
import math

import numpy as np
import pytest

from conftest import fixture, golden
import dfr_ops
import oracle
from gocfd_gb300 import meshes


@pytest.mark.parametrize("N", range(5))
def test_interpolation_reproduces_element_constants(N):
    m = meshes.read_mesh(fixture("test_tris_5.neu"))
    el = dfr_ops.build_element(N)
    K = m.K
    Q = np.tile(np.arange(1, K + 1, dtype=float), (el.Np, 1))
    QF = el.FluxEdgeInterp @ Q
    assert np.allclose(QF, np.arange(1, K + 1, dtype=float)[None, :], atol=1e-6, rtol=0)
    assert np.abs(QF - np.arange(1, K + 1)[None, :]).max() < 1e-12


@pytest.mark.parametrize("N", range(5))
def test_freestream_divergence_is_zero(N):
    m = meshes.read_mesh(fixture("test_tris_6_nowall.neu"))
    s = oracle.OracleSolver(N, m.VX, m.VY, m.EToV, m.bc_edges, flux="average", init="freestream",
                            minf=2.0, gamma=1.4, cfl=2.5)
    r = s.rhs(s.Q)
    assert np.abs(r).max() < 1e-6


def poly_state(x, y, gamma=1.4):
    """GetStatePoly (euler_test.go:848-875) with a = b = c = d = 1."""
    rho = np.abs(x) + np.abs(y)
    rhoU = x * rho
    rhoV = y * rho
    E = (x * x + y * y) * (rho / 2.0) + rho ** gamma / (gamma - 1.0)
    return np.stack([rho, rhoU, rhoV, E])


@pytest.mark.parametrize("N", [2, 3, 4])
@pytest.mark.parametrize("mesh", ["test_tris_1tri.neu", "test_tris_two.neu", "test_tris_twoR.neu",
                                  "test_tris_6_nowall.neu"])
def test_polynomial_flux_divergence(N, mesh):
    """CheckFlux0: momentum-only flux mock, exact face values, density divergence
    3(|x|+|y|) recovered to 1e-4 relative."""
    m = meshes.read_mesh(fixture(mesh))
    s = oracle.OracleSolver(N, m.VX, m.VY, m.EToV, m.bc_edges, flux="average", init="freestream",
                            minf=2.0, flux_mock=1)
    g, el = s.geo, s.el
    Qall = poly_state(g.FluxX, g.FluxY)
    Q = np.ascontiguousarray(Qall[:, :el.Np, :])
    faces = np.ascontiguousarray(Qall[:, 2 * el.Np:, :])
    rhs = s.rhs_faces(Q, faces)
    div = -rhs                    # RHS = -div(F)
    x, y = g.FluxX[:el.Np], g.FluxY[:el.Np]
    exact = 3.0 * (np.abs(x) + np.abs(y))
    for n in range(4):
        assert np.abs(div[n] / Q[0] - exact / Q[0]).max() < 1e-4


def _vortex_div_density(vortex, x, y, h=1e-30):
    """d(rho u)/dx + d(rho v)/dy of the exact vortex at t = 0 (complex step)."""
    qx = oracle.ivortex_state(vortex, 0.0, x + 1j * h, y + 0j)
    qy = oracle.ivortex_state(vortex, 0.0, x + 0j, y + 1j * h)
    return qx[1].imag / h + qy[2].imag / h


def test_vortex_density_divergence_n1():
    m = meshes.read_mesh(fixture("test_tris_6.neu"))
    s = oracle.OracleSolver(1, m.VX, m.VY, m.EToV, m.bc_edges, flux="average", init="ivortex")
    r = s.rhs(s.Q)
    g = s.geo
    x, y = g.FluxX[:s.el.Np], g.FluxY[:s.el.Np]
    qc = oracle.ivortex_state(s.vortex, 0.0, x, y)
    assert np.allclose(s.Q, qc, atol=1e-6)
    exact_rhs = -_vortex_div_density(s.vortex, x, y)
    assert np.abs(r[0] / qc[0] - exact_rhs / qc[0]).max() < 1e-3


def test_fluid_functions_mach2():
    fs = oracle.freestream_mach(2.0, 1.4, 0.0)
    q = fs["qinf"]
    rho, u, v = q[0], q[1] / q[0], q[2] / q[0]
    p = 0.4 * (q[3] - 0.5 * rho * (u * u + v * v))
    c = math.sqrt(abs(1.4 * p / rho))
    vals = [q[0], q[1], q[2], q[3], math.hypot(u, v) / c, p]
    g = golden("fluid_functions_mach2")
    assert np.allclose(vals, g["values"], atol=g["atol"])


def test_ivortex_exact_state():
    vortex = (5.0, 5.0, 0.0, 1.4)
    q = oracle.ivortex_state(vortex, 0.0, np.array([5.0]), np.array([0.0]))[:, 0]
    g = golden("ivortex_state_at_5_0")
    assert np.allclose(q, g["q"], atol=g["atol"])
    rho, rhoU, rhoV, E = q
    u, v = rhoU / rho, rhoV / rho
    p = 0.4 * (E - 0.5 * rho * (u * u + v * v))
    Fx = [rhoU, rhoU * u + p, rhoU * v, u * (E + p)]
    Fy = [rhoV, rhoV * u, rhoV * v + p, v * (E + p)]
    assert np.allclose(Fx, g["Fx"], atol=g["atol"])
    assert np.allclose(Fy, g["Fy"], atol=g["atol"])
    # divergence of the y-momentum flux at the centre: d(rho v)/dx (complex step)
    h = 1e-30
    qx = oracle.ivortex_state(vortex, 0.0, np.array([5.0 + 1j * h]), np.array([0.0 + 0j]))
    assert abs(qx[2, 0].imag / h - g["drhov_dx"]) < g["atol"]


def equilateral_triangle(angle_deg):
    a = math.radians(angle_deg)
    pts = np.array([[0.0, 0.0], [1.0, 0.0], [0.5, math.sqrt(3) / 2]])
    R = np.array([[math.cos(a), -math.sin(a)], [math.sin(a), math.cos(a)]])
    pts = pts @ R.T
    return pts[:, 0].copy(), pts[:, 1].copy(), np.array([[0, 1, 2]], np.int32)


def rt_divergence_check(Div, el, geo, tol_scale=1e-9):
    """DivergenceCheck (dfr_startup_test.go:293-356): (x^p, y^p) for p = 1..N
    projected on the RT DOFs (transformed interior components, ||n||-scaled
    physical normal flux on the edges), divergence recovered to 1e-9 rel."""
    Np, NE = el.Np, el.NpEdge
    for p in range(1, el.N + 1):
        for k in range(geo.K):
            x, y = geo.FluxX[:, k], geo.FluxY[:, k]
            fx, fy = x ** p, y ** p
            Jd = geo.Jdet[k]
            Ji = geo.Jinv[k]
            F = np.zeros(el.NpFlux)
            F[:Np] = (Jd * (Ji[0] * fx + Ji[1] * fy))[:Np]
            F[Np:2 * Np] = (Jd * (Ji[2] * fx + Ji[3] * fy))[Np:2 * Np]
            for e in range(3):
                sl = slice(2 * Np + e * NE, 2 * Np + (e + 1) * NE)
                F[sl] = (geo.nx[e, k] * fx[sl] + geo.ny[e, k] * fy[sl]) * geo.IInII[e, k]
            div = Div @ F / Jd
            exact = p * (x ** (p - 1) + y ** (p - 1))
            tol = tol_scale * np.abs(fx).max()
            assert np.abs(div - exact).max() <= max(tol, 1e-12), (p, k, np.abs(div - exact).max())


@pytest.mark.parametrize("angle", [0, 15, 25, 45, 90, 180, 210, 270, 310])
def test_rt_divergence_exact_rotated_triangles(angle):
    el = dfr_ops.build_element(4)
    VX, VY, EToV = equilateral_triangle(angle)
    geo = dfr_ops.build_geometry(el, VX, VY, EToV, [])
    rt_divergence_check(el.Div, el, geo)


def test_rt_divergence_exact_tris5():
    el = dfr_ops.build_element(4)
    m = meshes.read_mesh(fixture("test_tris_5.neu"))
    geo = dfr_ops.build_geometry(el, m.VX, m.VY, m.EToV, m.bc_edges)
    rt_divergence_check(el.Div, el, geo)
