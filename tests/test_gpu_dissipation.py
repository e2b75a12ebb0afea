"""GPU parity of the PerssonC0 shock capturing (sensor, C0 viscosity, RT-gradient
dissipation, modal limiter and RHS filter) on the FP64 path against the oracle.

Tolerances: RHS max |d| <= 1e-9 * amp * max|RHS| (amp as in the Euler RHS parity,
max|DivInt| / 50, >= 1); steps: rel L2 of the state <= 1e-10.  The sensor's
log10 and the ramp's sine differ from the host's by an ulp or so, which moves
the dissipation by ~1e-16 relative.
"""
import numpy as np
import pytest

from conftest import fixture
import oracle
from gocfd_gb300 import _lib, meshes
from gocfd_gb300.euler2d import Euler, InputParameters2D

pytestmark = pytest.mark.gpu


def make_pair(mesh, N, *, init="shocktube", flux="roe", kappa=0.0, local_dt=False, cfl=0.5, minf=0.5,
              precision="fp64", vortex_center=(5.0, 0.0)):
    ip = InputParameters2D(CFL=cfl, FluxType=flux, InitType=init, PolynomialOrder=N, FinalTime=1e9,
                           Minf=minf, Gamma=1.4, Alpha=0.0, LocalTimeStepping=local_dt, MaxIterations=10 ** 9,
                           Limiter="PerssonC0", Kappa=kappa)
    gpu = Euler(ip, mesh, 1, precision=precision, vortex_center=vortex_center)
    ora = oracle.OracleSolver(N, mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges, flux=flux, init=init, cfl=cfl,
                              final_time=1e9, minf=minf, gamma=1.4, alpha=0.0, local_dt=local_dt,
                              vortex_center=vortex_center, limiter="PerssonC0", kappa=kappa)
    return gpu, ora


def smooth_tube(ora, width=0.005):
    """Sod states joined by a tanh of the given width at x = 0.5, so that the
    jump lies inside elements and the sensor switches on."""
    h = 0.5 * (1.0 + np.tanh((ora.geo.SolX - 0.5) / width))
    rho, p = 1.0 + (0.125 - 1.0) * h, 1.0 + (0.1 - 1.0) * h
    Q = np.zeros((4,) + h.shape)
    Q[0], Q[3] = rho, p / 0.4
    return Q


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def assert_rhs_close(r, ref, N, rtol=1e-9):
    amp = max(1.0, np.abs(_lib.host_operator(N, 1)).max() / 50.0)
    tol = rtol * amp * np.abs(ref).max() + 1e-13
    assert np.abs(r - ref).max() <= tol, (np.abs(r - ref).max(), tol)


@pytest.mark.parametrize("N", [1, 2, 3, 4])
@pytest.mark.parametrize("kappa", [0.0, 3.0])
def test_rhs_parity_shocktube(N, kappa):
    mesh = meshes.sod_channel(25, 3)
    gpu, ora = make_pair(mesh, N, kappa=kappa)
    Q0 = gpu.get_global_state()
    assert np.array_equal(Q0, ora.Q)
    rng = np.random.default_rng(N)
    # at N = 1 a narrower jump extrapolates to negative face pressures
    Q = smooth_tube(ora, 0.02 if N == 1 else 0.005)
    Q = np.ascontiguousarray(Q * (1.0 + 0.01 * rng.uniform(-1, 1, Q.shape)))
    r = gpu.rhs_global(Q)
    ref = ora.rhs(Q)
    assert np.all(np.isfinite(ref))
    assert_rhs_close(r, ref, N)
    # the shock has switched the sensor on somewhere
    _, sig, _, _, _ = ora.sensor(Q)
    assert sig.max() > 0.0
    gpu.close()


def test_rhs_parity_bc_mesh_with_walls():
    """fstepA001 (walls, inflow, outflow) at Mach 0.5 with a perturbed state."""
    mesh = meshes.read_mesh(fixture("fstepA001.neu"))
    gpu, ora = make_pair(mesh, 2, init="freestream", kappa=3.0)
    rng = np.random.default_rng(7)
    Q = np.ascontiguousarray(ora.Q * (1.0 + 0.05 * rng.uniform(-1, 1, ora.Q.shape)))
    assert_rhs_close(gpu.rhs_global(Q), ora.rhs(Q), 2)
    gpu.close()


@pytest.mark.parametrize("N,local_dt", [(1, False), (2, False), (3, True), (4, False)])
def test_step_parity_shocktube(N, local_dt):
    mesh = meshes.sod_channel(40, 4)
    gpu, ora = make_pair(mesh, N, local_dt=local_dt)
    ora.Q = np.ascontiguousarray(smooth_tube(ora))
    gpu.set_global_state(ora.Q)
    assert ora.sensor(ora.Q)[1].max() > 0.0
    nsteps = 10
    res = gpu.step(nsteps)
    t, dt = res["time"], res["dt"]
    to, dto, _ = ora.step(nsteps)
    Q = gpu.get_global_state()
    assert np.all(np.isfinite(Q))
    assert rel_l2(Q, ora.Q) <= 1e-10, rel_l2(Q, ora.Q)
    if not local_dt:
        # the viscous limit C/max(eps/h^2) carries the dissipation's round-off
        assert abs(t - to) <= 1e-10 * max(1.0, abs(to))
        assert abs(dt - dto) <= 1e-10 * abs(dto)
    gpu.close()


def test_step_parity_limiter_state_vortex():
    """A smooth flow: the sensor is small but the rkStep-2 limiter and the RHS filter still act."""
    mesh = meshes.vortex_box(8, jitter=0.1)
    gpu, ora = make_pair(mesh, 2, init="ivortex", cfl=1.0, vortex_center=(0.0, 0.0))
    gpu.step(5)
    ora.step(5)
    assert rel_l2(gpu.get_global_state(), ora.Q) <= 1e-10
    gpu.close()


@pytest.mark.parametrize("N", [2, 3])
def test_rhs_mixed_with_dissipation(N):
    """Mixed path: FP32 delta-form Euler RHS plus the FP64 dissipation and filter."""
    mesh = meshes.sod_channel(25, 3)
    gpu, ora = make_pair(mesh, N, precision="fp32")
    rng = np.random.default_rng(N)
    Q = smooth_tube(ora, 0.005)
    Q = np.ascontiguousarray(Q * (1.0 + 0.01 * rng.uniform(-1, 1, Q.shape)))
    r = gpu.rhs_global(Q)
    ref = ora.rhs(Q)
    err = rel_l2(r, ref)
    print(f"mixed + dissipation RHS rel L2 N={N}: {err:.3e}")
    assert err <= 5e-4
    gpu.close()


@pytest.mark.parametrize("local_dt", [False, True])
def test_step_mixed_with_dissipation(local_dt):
    mesh = meshes.sod_channel(40, 4)
    gpu, ora = make_pair(mesh, 2, local_dt=local_dt, precision="fp32")
    ora.Q = np.ascontiguousarray(smooth_tube(ora))
    gpu.set_global_state(ora.Q)
    gpu.step(10)
    ora.step(10)
    Q = gpu.get_global_state()
    err = rel_l2(Q, ora.Q)
    print(f"mixed + dissipation 10-step rel L2 (local dt {local_dt}): {err:.3e}")
    assert np.all(np.isfinite(Q))
    assert err <= 1e-6
    gpu.close()
