"""Periodic boundaries (BC_Periodic / BC_PeriodicReversed): the pairing of
NewTriangulation (DG2D/triangulation.go:63-99), each periodic tag's edge list
split into halves ordered as curves, edge i of the first half shared with edge
i of the second (edges.go:436-437 leaves the second record as a no-op).

CPU: the oracle's pairing on periodic boxes, the C++ mesh reader's group bits.
GPU (through the C ABI, against the FP64 oracle with the same pairing): RHS
parity for N = 1..4, freestream preservation, 20-step trajectories on the FP64
and mixed paths.  Tolerances as in test_gpu_parity.py.
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
import dfr_ops
from gocfd_gb300 import _lib, meshes
from gocfd_gb300.euler2d import Euler, InputParameters2D


def test_oracle_pairs_every_edge_of_a_periodic_box():
    n = 5
    mesh = meshes.periodic_box(n, jitter=0.1, seed=2)
    el = dfr_ops.build_element(2)
    g = dfr_ops.build_geometry(el, mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges)
    # a torus of 2 n^2 triangles: every edge shared, 3 n^2 edges
    assert len(g.kL) == 3 * n * n
    assert np.all(g.kR >= 0)
    # every element's edge slot names an edge that has the element on one side
    for k in range(g.K):
        for e in range(3):
            en = g.EtoEdge[k, e]
            assert (g.kL[en], g.eL[en]) == (k, e) or (g.kR[en], g.eR[en]) == (k, e)
    # paired edges have equal length and opposite normals (a translation)
    for en in range(len(g.kL)):
        kl, el_, kr, er = g.kL[en], g.eL[en], g.kR[en], g.eR[en]
        assert abs(g.nx[el_, kl] + g.nx[er, kr]) < 1e-12 and abs(g.ny[el_, kl] + g.ny[er, kr]) < 1e-12


def test_oracle_pairs_the_reference_periodic_vortex_mesh():
    """The reference's own periodic vortex mesh (test_cases/Euler2D/isentropic-vortex/
    geometry/vnew-coarse.su2: far field and a PeriodicReversed pair): its 28
    periodic edges become 14 shared edges between equal, opposite faces."""
    from conftest import fixture
    mesh = meshes.read_mesh(fixture("vnew-coarse.su2"))
    assert {f & 0xFF for _, _, f in mesh.bc_edges} == {4, 11}
    el = dfr_ops.build_element(2)
    g = dfr_ops.build_geometry(el, mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges)
    nfar = sum(1 for _, _, f in mesh.bc_edges if f & 0xFF == 4)
    assert int(np.sum(g.kR < 0)) == nfar == 28
    assert len(g.kL) == (3 * mesh.K - nfar - 28) // 2 + 14 + nfar
    for en in np.nonzero(g.kR >= 0)[0]:
        kl, el_, kr, er = g.kL[en], g.eL[en], g.kR[en], g.eR[en]
        assert abs(g.nx[el_, kl] + g.nx[er, kr]) < 1e-12 and abs(g.ny[el_, kl] + g.ny[er, kr]) < 1e-12


def test_oracle_rejects_odd_periodic_lists():
    mesh = meshes.periodic_box(3)
    bc = [e for e in mesh.bc_edges if (e[2] >> 8) == 0][:-1] + [e for e in mesh.bc_edges if (e[2] >> 8) == 1]
    el = dfr_ops.build_element(1)
    with pytest.raises(ValueError):
        dfr_ops.build_geometry(el, mesh.VX, mesh.VY, mesh.EToV, bc)


def test_reader_group_bits(tmp_path):
    mesh = meshes.periodic_box(4)
    path = os.path.join(tmp_path, "pbox.neu")
    meshes.write_gambit(mesh, path)
    back = meshes.read_mesh(path)
    _, _, _, bc = _lib.read_mesh(path)
    flags = sorted(set(f for _, _, f in bc))
    assert flags == sorted(set(f for _, _, f in back.bc_edges))
    assert set(f & 0xFF for f in flags) == {10} and len(flags) == 2


def _pair(mesh, N, precision="fp64", init="ivortex", center=(0.0, 0.0), minf=0.5):
    ip = InputParameters2D(CFL=1.0, FluxType="roe", InitType=init, PolynomialOrder=N, FinalTime=1e9,
                           Minf=minf, Gamma=1.4, MaxIterations=10 ** 9)
    gpu = Euler(ip, mesh, 1, precision=precision, vortex_center=center)
    ora = oracle.OracleSolver(N, mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges, flux="roe", init=init, cfl=1.0,
                              minf=minf, gamma=1.4, vortex_center=center)
    return gpu, ora


@pytest.mark.gpu
@pytest.mark.parametrize("N", [1, 2, 3, 4])
def test_periodic_rhs_parity(N):
    mesh = meshes.periodic_box(10, jitter=0.1, seed=4)
    gpu, ora = _pair(mesh, N)
    amp = max(1.0, np.abs(_lib.host_operator(N, 1)).max() / 50.0)
    for t in (0.0, 0.3):
        r, ref = gpu.rhs_global(ora.Q, t), ora.rhs(ora.Q, t)
        assert np.abs(r - ref).max() <= 1e-9 * amp * np.abs(ref).max() + 1e-13
    gpu.close()


@pytest.mark.gpu
@pytest.mark.parametrize("N", [2, 3])
def test_reference_periodic_vortex_mesh_rhs_parity(N):
    """RHS parity on the reference's own PeriodicReversed vortex mesh
    (vnew-coarse.su2, vortex at its default centre (5, 0))."""
    from conftest import fixture
    mesh = meshes.read_mesh(fixture("vnew-coarse.su2"))
    gpu, ora = _pair(mesh, N, center=(5.0, 0.0))
    amp = max(1.0, np.abs(_lib.host_operator(N, 1)).max() / 50.0)
    for t in (0.0, 0.3):
        r, ref = gpu.rhs_global(ora.Q, t), ora.rhs(ora.Q, t)
        assert np.abs(r - ref).max() <= 1e-9 * amp * np.abs(ref).max() + 1e-13
    gpu.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_periodic_freestream_preserved(precision):
    mesh = meshes.periodic_box(8, jitter=0.1, seed=1)
    gpu, _ = _pair(mesh, 3, precision=precision, init="freestream", minf=0.7)
    q0 = gpu.get_global_state()
    info = gpu.step(10)
    assert np.abs(gpu.get_global_state() - q0).max() < (1e-12 if precision == "fp64" else 1e-6)
    assert max(info["resid_absmax"]) < (1e-12 if precision == "fp64" else 1e-6)
    gpu.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol,ttol", [("fp64", 1e-10, 1e-12), ("fp32", 1e-7, 1e-7)])
def test_periodic_step_parity(precision, tol, ttol):
    """FP64: the oracle's trajectory; mixed: its FP32 wave speeds set dt to ~1e-8 relative."""
    mesh = meshes.periodic_box(12, jitter=0.1, seed=6)
    gpu, ora = _pair(mesh, 3, precision=precision)
    info = gpu.step(20)
    t_ora, _, _ = ora.step(20)
    assert abs(info["time"] - t_ora) <= ttol * t_ora
    q = gpu.get_global_state()
    assert np.linalg.norm(q - ora.Q) / np.linalg.norm(ora.Q) <= tol
    gpu.close()


@pytest.mark.gpu
@pytest.mark.parametrize("precision,every,rtol", [("fp64", 3, 1e-6), ("fp32", 3, 1e-5), ("fp32", 6, 1e-5)])
def test_periodic_step_vjp_against_oracle_fd(precision, every, rtol):
    """The adjoint runs through the paired periodic edges like any shared edge:
    a 6-step window (checkpoint every 3, or taped while recording) against the
    oracle's central differences, on the FP64 path and the mixed path's FP32
    adjoint."""
    mesh = meshes.periodic_box(6, jitter=0.1, seed=8)
    gpu, ora = _pair(mesh, 2, precision=precision)
    rng = np.random.default_rng(21)
    Q0 = np.ascontiguousarray(ora.Q * (1.0 + 0.01 * rng.uniform(-1, 1, ora.Q.shape)))
    nsteps = 6
    gpu.set_global_state(Q0)
    gpu.time = 0.0
    gpu.record(nsteps, every)
    assert gpu.window_taped() == (every >= nsteps)
    Qbf = rng.standard_normal(Q0.shape)
    Qb0, _, _ = gpu.step_vjp(Qbf)
    d = rng.standard_normal(Q0.shape) * np.abs(Q0)
    h = 1e-6

    def J(sign):
        ora.Q = np.ascontiguousarray(Q0 + sign * h * d)
        ora.time = 0.0
        ora.step(nsteps)
        return float(np.sum(Qbf * ora.Q))
    fd = (J(1.0) - J(-1.0)) / (2 * h)
    ad = float(np.sum(Qb0 * d))
    assert abs(ad - fd) <= rtol * max(abs(ad), abs(fd)), (ad, fd)
    gpu.close()


@pytest.mark.gpu
def test_periodic_with_shock_capturing_matches_oracle():
    """PerssonC0 on a periodic box ([-1, 1]^2) holding Sod states joined by a tanh
    front inside the elements at x = 0.5 (the sensor is on there) and by a jump
    across the periodic seam at x = -1 / 1: the sensor, vertex maxima, viscous edge
    fluxes and limiter run on the paired edges; 10 FP64 steps against the oracle."""
    mesh = meshes.periodic_box(16, L=2.0, jitter=0.1, seed=9)
    ip = InputParameters2D(CFL=0.3, FluxType="roe", InitType="shocktube", PolynomialOrder=2, FinalTime=1e9,
                           Gamma=1.4, MaxIterations=10 ** 9, Limiter="PerssonC0", Kappa=5.0)
    gpu = Euler(ip, mesh, 1, precision="fp64")
    ora = oracle.OracleSolver(2, mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges, flux="roe", init="shocktube", cfl=0.3,
                              gamma=1.4, limiter="PerssonC0", kappa=5.0)
    X = ora.geo.SolX
    front = 0.5 * (1.0 + np.tanh((X - 0.5) / 0.03))
    h = np.clip(front * 0.5 * (1.0 - np.tanh((X + 0.6) / 0.03)) + front, 0.0, 1.0)
    Q = np.zeros((4,) + X.shape)
    Q[0], Q[3] = 1.0 + (0.125 - 1.0) * h, (1.0 + (0.1 - 1.0) * h) / 0.4
    Q = np.ascontiguousarray(Q)
    ora.Q = Q.copy()
    gpu.set_global_state(Q)
    _, sigma, _, _, _ = ora.sensor(ora.Q)
    assert (sigma > 0).any()  # the shock capturing is active
    gpu.step(10)
    ora.step(10)
    q = gpu.get_global_state()
    assert np.isfinite(q).all()
    assert np.linalg.norm(q - ora.Q) / np.linalg.norm(ora.Q) <= 1e-10
    gpu.close()
