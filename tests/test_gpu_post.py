"""Post-processing through the C ABI against numpy restatements on the
oracle's own operators and geometry: the solution sampled at points
(gcfd_sample_points; the Sod line samples of shock_tube.go:27-142) and the
wall data (gcfd_wall_points; OutputFinal, euler.go:251-316).

Tolerance: 1e-12 relative to the largest value (FP64 sums of Np products of
two independently built interpolation operators that agree to ~1e-14).
"""
import numpy as np
import pytest

import dfr_ops
import oracle
from conftest import fixture
from gocfd_gb300 import meshes
from gocfd_gb300.euler2d import Euler, InputParameters2D

pytestmark = pytest.mark.gpu


def oracle_sample(el, mesh, Q, x, y):
    """Brute-force containing element, reference coordinates from the affine
    map of element_utils.go:163-175, value = Vandermonde(r, s) Vinv Q."""
    V = mesh.EToV
    A = np.stack([mesh.VX[V[:, 0]], mesh.VY[V[:, 0]]], 1)
    B = np.stack([mesh.VX[V[:, 1]], mesh.VY[V[:, 1]]], 1)
    Cc = np.stack([mesh.VX[V[:, 2]], mesh.VY[V[:, 2]]], 1)
    out = np.zeros((4, len(x)))
    for p, (px, py) in enumerate(zip(x, y)):
        J = np.stack([0.5 * (B - A), 0.5 * (Cc - A)], 2)          # K x 2 x 2, columns d/dr, d/ds
        rs = np.linalg.solve(J, (np.array([px, py]) - A)[:, :, None])[:, :, 0] - 1.0
        inside = (rs[:, 0] >= -1 - 1e-12) & (rs[:, 1] >= -1 - 1e-12) & (rs.sum(1) <= 1e-12)
        k = int(np.flatnonzero(inside)[0])
        basis = dfr_ops.vandermonde2d(el.N, rs[k:k + 1, 0], rs[k:k + 1, 1]) @ el.Vinv   # 1 x Np
        out[:, p] = (basis @ Q[:, :, k].T)[0]
    return out


def _solver(mesh, N, init="shocktube", minf=0.0):
    ip = InputParameters2D(CFL=1.0, FluxType="roe", InitType=init, PolynomialOrder=N, FinalTime=1e9, Minf=minf,
                           Gamma=1.4, MaxIterations=10 ** 9)
    return Euler(ip, mesh, 1, precision="fp64")


@pytest.mark.parametrize("N", [1, 2, 3, 4])
def test_sample_points_against_oracle(N):
    mesh = meshes.structured_triangles(16, 5, 0.0, 1.0, 0.0, 0.05, jitter=0.15, seed=N,
                                       tags=("wall", "out", "wall", "in"))
    el = dfr_ops.build_element(N)
    rng = np.random.default_rng(N)
    with _solver(mesh, N) as s:
        Q = s.get_global_state() * (1.0 + 0.1 * rng.uniform(-1, 1, (4, el.Np, mesh.K)))
        s.set_global_state(Q)
        x, q = s.sod_line(41)
        ymid = 0.025
        ref = oracle_sample(el, mesh, Q, x, np.full_like(x, ymid))
        assert np.abs(q - ref).max() <= 1e-12 * np.abs(ref).max()
        # random points, and the solution points themselves (the interpolant reproduces them)
        px, py = rng.uniform(0, 1, 30), rng.uniform(0, 0.05, 30)
        q2, elem = s.sample_points(px, py)
        assert np.abs(q2 - oracle_sample(el, mesh, Q, px, py)).max() <= 1e-12 * np.abs(Q).max()
        geo = dfr_ops.build_geometry(el, mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges)
        ks = [3, 17, 40]
        sx = np.concatenate([geo.SolX[:, k] for k in ks])
        sy = np.concatenate([geo.SolY[:, k] for k in ks])
        q3, e3 = s.sample_points(sx, sy)
        want = np.concatenate([Q[:, :, k] for k in ks], axis=1)
        assert np.abs(q3 - want).max() <= 1e-12 * np.abs(want).max()


def test_sample_points_reproduce_polynomials():
    """A state that is a degree-N polynomial in (x, y) is sampled exactly anywhere."""
    N = 3
    mesh = meshes.vortex_box(6, jitter=0.2, seed=9)
    el = dfr_ops.build_element(N)
    with _solver(mesh, N, init="freestream", minf=0.3) as s:
        geo = dfr_ops.build_geometry(el, mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges)
        f = lambda X, Y, c: 1.5 + c * X - 0.3 * Y + 0.02 * X * X * Y - 0.01 * Y ** 3
        Q = np.stack([f(geo.SolX, geo.SolY, c) for c in (0.05, 0.1, -0.2, 0.3)])
        s.set_global_state(Q)
        rng = np.random.default_rng(1)
        px, py = rng.uniform(-5, 5, 200), rng.uniform(-5, 5, 200)
        q, _ = s.sample_points(px, py)
        want = np.stack([f(px, py, c) for c in (0.05, 0.1, -0.2, 0.3)])
        assert np.abs(q - want).max() <= 1e-11


def test_sample_point_outside_the_mesh_is_an_error():
    from gocfd_gb300 import _lib
    mesh = meshes.vortex_box(4)
    with _solver(mesh, 1, init="freestream", minf=0.3) as s:
        with pytest.raises(_lib.GcfdError) as e:
            s.sample_points([0.0, 7.0], [0.0, 0.0])
        assert e.value.code == -1


@pytest.mark.parametrize("N", [0, 2, 3])
def test_wall_points_against_oracle(N):
    mesh = meshes.wedge_channel(12, 6)
    el = dfr_ops.build_element(N)
    ora = oracle.OracleSolver(N, mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges, flux="roe", init="freestream",
                              minf=2.0)
    g = ora.geo
    with _solver(mesh, N, init="freestream", minf=2.0) as s:
        rng = np.random.default_rng(4)
        Q = ora.Q * (1.0 + 0.05 * rng.uniform(-1, 1, ora.Q.shape))
        s.set_global_state(Q)
        x, y, q, p = s.wall_points()
    NE = el.NpEdge
    per = 1 if N == 0 else NE
    wall = [en for en in range(len(g.kL)) if g.kR[en] < 0 and g.bc[en] in (5, 6)]
    assert len(x) == len(wall) * per
    o = 0
    for en in wall:
        k, e = g.kL[en], g.eL[en]
        for i in range(per):
            row = e * NE + i
            assert abs(x[o] - g.FluxX[2 * el.Np + row, k]) < 1e-13 and abs(y[o] - g.FluxY[2 * el.Np + row, k]) < 1e-13
            face = el.FluxEdgeInterp[row] @ Q[:, :, k].T
            assert np.abs(q[:, o] - face).max() <= 1e-12 * np.abs(face).max()
            pr = 0.4 * (face[3] - 0.5 * (face[1] ** 2 + face[2] ** 2) / face[0])
            assert abs(p[o] - pr) <= 1e-12 * abs(pr)
            o += 1
