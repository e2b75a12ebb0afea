"""GPU parity of the CUDA path (through the C ABI) against the FP64 oracle.

Tolerances, written here:
  FP64 path   RHS: max |d| <= 1e-9 * amp * max|RHS|, amp = max|DivInt| / 50 (>= 1),
              covering the two FP64 constructions of DivInt (they agree to ~1e-13
              relative to its entries); steps: rel L2 of the state <= 1e-10
  mixed path  (FP32 delta form, FP64 state): RHS rel L2 <= MIXED_RHS_TOL on the
              near-uniform BC mesh and <= MIXED_VORTEX_RHS_TOL on vortex meshes, where
              FP32 accumulation against DivInt (entries up to ~3.6e2 at N = 4) bounds
              it at ~eps32 * max|DivInt| independent of h; 100 steps: rel L2 of the
              state <= MIXED_STEP_TOL (the RK increments are small, so the state error
              stays ~1e-8)
"""
import numpy as np
import pytest

from conftest import fixture
import oracle
from gocfd_gb300 import _lib, meshes
from gocfd_gb300.euler2d import Euler, InputParameters2D

pytestmark = pytest.mark.gpu


def make_pair(mesh, N, flux="roe", init="freestream", precision="fp64", cfl=1.0, minf=0.5, alpha=0.0,
              local_dt=False, vortex_center=(5.0, 0.0), proc_limit=1, final_time=1e9):
    ip = InputParameters2D(CFL=cfl, FluxType=flux, InitType=init, PolynomialOrder=N, FinalTime=final_time,
                           Minf=minf, Gamma=1.4, Alpha=alpha, LocalTimeStepping=local_dt,
                           MaxIterations=10 ** 9)
    gpu = Euler(ip, mesh, proc_limit, precision=precision, vortex_center=vortex_center)
    ora = oracle.OracleSolver(N, mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges, flux=flux, init=init, cfl=cfl,
                              final_time=final_time, minf=minf, gamma=1.4, alpha=alpha, local_dt=local_dt,
                              vortex_center=vortex_center)
    return gpu, ora


def perturbed(Q, seed=0, amp=0.02):
    rng = np.random.default_rng(seed)
    P = Q * (1.0 + amp * rng.uniform(-1, 1, Q.shape))
    return np.ascontiguousarray(P)


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


MIXED_RHS_TOL = 2e-6
MIXED_VORTEX_RHS_TOL = 5e-4
MIXED_STEP_TOL = 1e-7


def assert_rhs_close(r, ref, rtol=1e-9, N=None):
    # Round-off scales with the divergence operator's entries: the reference's
    # N = 1 edge points (+-0.028, 0) make them ~1e3 instead of ~1e1.
    amp = 1.0 if N is None else max(1.0, np.abs(_lib.host_operator(N, 1)).max() / 50.0)
    tol = rtol * amp * np.abs(ref).max() + 1e-13
    assert np.abs(r - ref).max() <= tol, (np.abs(r - ref).max(), tol)


@pytest.mark.parametrize("N", range(5))
@pytest.mark.parametrize("flux", ["average", "lax", "roe", "roe-er"])
def test_rhs_parity_fp64_bc_mesh(N, flux):
    """fstepA001: walls plus inflow/outflow characteristic BCs."""
    mesh = meshes.read_mesh(fixture("fstepA001.neu"))
    gpu, ora = make_pair(mesh, N, flux=flux, minf=0.5, alpha=10.0)
    Q0 = gpu.get_global_state()
    # built on the device (CUDA's exp / pow against the host's: a few ulp)
    assert np.allclose(Q0, ora.Q, rtol=2e-15, atol=1e-15)
    Q = perturbed(ora.Q, seed=N)
    r = gpu.rhs_global(Q)
    ref = ora.rhs(Q)
    assert_rhs_close(r, ref, N=N)
    gpu.close()


@pytest.mark.parametrize("N", range(5))
def test_freestream_preserved_fp64(N):
    mesh = meshes.read_mesh(fixture("test_tris_6_nowall.neu"))
    gpu, _ = make_pair(mesh, N, flux="average", minf=2.0)
    r = gpu.rhs_global(gpu.get_global_state())
    assert np.abs(r).max() < 1e-6
    gpu.close()


@pytest.mark.parametrize("N", [1, 2, 4])
def test_rhs_parity_vortex_box(N):
    mesh = meshes.vortex_box(20)
    gpu, ora = make_pair(mesh, N, init="ivortex", vortex_center=(0.0, 0.0))
    Q0 = gpu.get_global_state()
    assert np.abs(Q0 - ora.Q).max() < 1e-14
    for t in (0.0, 0.37):
        assert_rhs_close(gpu.rhs_global(ora.Q, t), ora.rhs(ora.Q, t), N=N)
    gpu.close()


def test_step_parity_fp64_vortex_800_tris():
    """Configuration 1: 20x20 quads -> 800 triangles, N = 2, Roe, CFL 1, 100 steps."""
    mesh = meshes.vortex_box(20)
    gpu, ora = make_pair(mesh, 2, init="ivortex", vortex_center=(0.0, 0.0), cfl=1.0)
    info = gpu.step(100)
    t_ora, dt_ora, R = ora.step(100)
    Qg = gpu.get_global_state()
    assert abs(info["time"] - t_ora) <= 1e-12 * t_ora
    assert abs(info["dt"] - dt_ora) <= 1e-12 * dt_ora
    assert rel_l2(Qg, ora.Q) <= 1e-10
    # residual = signed max of the final increment, per variable
    assert np.allclose(info["resid_max"], R.reshape(4, -1).max(axis=1), rtol=1e-6, atol=1e-14)
    gpu.close()


def test_step_parity_fp64_bc_mesh_sharded():
    mesh = meshes.read_mesh(fixture("fstepA001.neu"))
    gpu, ora = make_pair(mesh, 2, flux="lax", minf=0.5, alpha=5.0, proc_limit=7, cfl=0.5)
    gpu.step(20)
    ora.step(20)
    assert rel_l2(gpu.get_global_state(), ora.Q) <= 1e-10
    gpu.close()


@pytest.mark.parametrize("N", [2, 4])
def test_rhs_parity_reference_wedge_mesh(N):
    """The reference's own Mach-2 wedge mesh (test_cases/Euler2D/Wedge/wedge.su2:
    walls and a supersonic far field), its input's Minf = 2, on a perturbed
    freestream state."""
    mesh = meshes.read_mesh(fixture("wedge.su2"))
    gpu, ora = make_pair(mesh, N, flux="roe", minf=2.0)
    Q = perturbed(ora.Q, seed=10 + N)
    assert_rhs_close(gpu.rhs_global(Q), ora.rhs(Q), N=N)
    gpu.close()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-7)])
def test_step_parity_reference_wedge_mesh_lts(precision, tol):
    """20 local-time-stepping steps from the freestream on the reference's wedge
    mesh (its input: Roe, LTS, Minf 2), FP64 and mixed against the oracle."""
    mesh = meshes.read_mesh(fixture("wedge.su2"))
    gpu, ora = make_pair(mesh, 2, flux="roe", minf=2.0, local_dt=True, cfl=0.5, precision=precision)
    gpu.step(20)
    ora.step(20)
    assert rel_l2(gpu.get_global_state(), ora.Q) <= tol
    gpu.close()


def test_local_time_stepping_parity():
    """Supersonic far-field (copy) branch, slip walls, local time stepping."""
    mesh = meshes.wedge_channel(24, 12)
    gpu, ora = make_pair(mesh, 1, flux="roe", minf=2.0, local_dt=True, cfl=0.5)
    gpu.step(10)
    ora.step(10)
    assert rel_l2(gpu.get_global_state(), ora.Q) <= 1e-10
    assert gpu.time == 0.0  # local time stepping never advances the global time
    gpu.close()


@pytest.mark.parametrize("N", [1, 2, 3, 4])
@pytest.mark.parametrize("precision", ["fp32", "tf32x3"])
def test_rhs_mixed_vortex(N, precision):
    mesh = meshes.vortex_box(16, jitter=0.1)
    gpu, ora = make_pair(mesh, N, init="ivortex", vortex_center=(0.0, 0.0), precision=precision)
    r = gpu.rhs_global(ora.Q, 0.1)
    ref = ora.rhs(ora.Q, 0.1)
    err = rel_l2(r, ref)
    print(f"mixed RHS rel L2 N={N}: {err:.3e}")
    assert err <= MIXED_VORTEX_RHS_TOL
    gpu.close()


@pytest.mark.parametrize("N", [2, 4])
@pytest.mark.parametrize("precision", ["fp32", "tf32x3"])
def test_rhs_mixed_resolved_vortex(N, precision):
    """64x64 jittered mesh: the vortex is resolved, deltas are small."""
    mesh = meshes.vortex_box(64, jitter=0.1, seed=2)
    gpu, ora = make_pair(mesh, N, init="ivortex", vortex_center=(0.0, 0.0), precision=precision)
    r = gpu.rhs_global(ora.Q, 0.05)
    ref = ora.rhs(ora.Q, 0.05)
    err = rel_l2(r, ref)
    print(f"mixed RHS rel L2 resolved N={N}: {err:.3e}")
    assert err <= MIXED_VORTEX_RHS_TOL
    gpu.close()


@pytest.mark.parametrize("flux", ["average", "lax", "roe", "roe-er"])
@pytest.mark.parametrize("precision", ["fp32", "tf32x3"])
def test_rhs_mixed_bc_mesh(flux, precision):
    mesh = meshes.read_mesh(fixture("fstepA001.neu"))
    gpu, ora = make_pair(mesh, 3, flux=flux, minf=0.5, alpha=10.0, precision=precision)
    Q = perturbed(ora.Q, seed=3, amp=0.01)
    err = rel_l2(gpu.rhs_global(Q), ora.rhs(Q))
    print(f"mixed RHS rel L2 {flux}: {err:.3e}")
    assert err <= MIXED_RHS_TOL
    gpu.close()


@pytest.mark.parametrize("N", range(5))
@pytest.mark.parametrize("precision", ["fp32", "tf32x3"])
def test_freestream_exact_mixed(N, precision):
    """Delta form: a uniform state has zero deltas, so the RHS is exactly zero."""
    mesh = meshes.read_mesh(fixture("test_tris_6_nowall.neu"))
    gpu, _ = make_pair(mesh, N, flux="roe", minf=2.0, precision=precision)
    r = gpu.rhs_global(gpu.get_global_state())
    assert np.abs(r).max() < 1e-12
    gpu.close()


@pytest.mark.parametrize("precision", ["fp32", "tf32x3"])
def test_step_mixed_vortex(precision):
    mesh = meshes.vortex_box(20)
    gpu, ora = make_pair(mesh, 2, init="ivortex", vortex_center=(0.0, 0.0), precision=precision)
    info = gpu.step(100)
    t, _, _ = ora.step(100)
    err = rel_l2(gpu.get_global_state(), ora.Q)
    print(f"mixed 100-step rel L2: {err:.3e}")
    assert err <= MIXED_STEP_TOL
    assert abs(info["time"] - t) <= 1e-6 * t
    gpu.close()


@pytest.mark.parametrize("precision", ["fp32", "tf32x3"])
def test_step_mixed_local_dt_and_restart(precision):
    """Local time stepping, and set_state between steps (stage-0 rebuild)."""
    mesh = meshes.wedge_channel(24, 12)
    gpu, ora = make_pair(mesh, 2, flux="roe", minf=2.0, local_dt=True, cfl=0.5, precision=precision)
    gpu.step(5)
    ora.step(5)
    gpu.set_global_state(ora.Q)
    gpu.step(5)
    ora.step(5)
    err = rel_l2(gpu.get_global_state(), ora.Q)
    print(f"mixed local-dt rel L2: {err:.3e}")
    assert err <= MIXED_STEP_TOL
    gpu.close()


def test_shard_layout_roundtrip():
    mesh = meshes.vortex_box(10)
    gpu, ora = make_pair(mesh, 3, init="ivortex", vortex_center=(0.0, 0.0), proc_limit=7)
    assert gpu.partitions.ParallelDegree == 7
    shards = gpu.Q
    assert [s[0].shape for s in shards] == [(10, gpu.partitions.bucket_dimension(i)) for i in range(7)]
    Q = perturbed(ora.Q, seed=5)
    gpu.set_global_state(Q)
    assert np.array_equal(gpu.get_global_state(), Q)
    gpu.close()


@pytest.mark.parametrize("precision", ["fp32", "tf32x3"])
def test_shard_layout_roundtrip_mixed(precision):
    """The mixed path moves the state in element chunks (copy of one chunk
    overlapping the conversion of the previous): uneven shards that straddle the
    chunk boundaries, K not a multiple of 32."""
    mesh = meshes.vortex_box(30, jitter=0.1, seed=8)  # K = 1800: 8 chunks of 256 elements, the last of 8
    gpu, ora = make_pair(mesh, 3, init="ivortex", vortex_center=(0.0, 0.0), proc_limit=7, precision=precision)
    Q = perturbed(ora.Q, seed=6)
    gpu.set_global_state(Q)
    # hi + lo holds ~48 bits: the round trip is exact to ~1e-14 relative
    assert rel_l2(gpu.get_global_state(), Q) <= 1e-13
    # state set through the chunked path, then stepped, against the oracle
    ora.Q = Q
    gpu.step(5)
    ora.step(5)
    err = rel_l2(gpu.get_global_state(), ora.Q)
    print(f"chunked set_state + 5 mixed steps on a 2%-perturbed state: rel L2 {err:.3e}")
    assert err <= 1e-6  # deltas of the perturbed state are ~100x the smooth field's
    gpu.close()


def test_errors_are_status_codes():
    mesh = meshes.vortex_box(4)
    gpu, _ = make_pair(mesh, 1, init="ivortex", vortex_center=(0.0, 0.0))
    lib = gpu.lib
    km = np.array([5, 5], np.int32)
    ptrs = gpu._ptrs([[np.zeros((gpu.Np, 5)) for _ in range(4)] for _ in range(2)])
    rc = lib.gcfd_set_state(gpu.ctx, 2, km.ctypes.data_as(_lib.PI), ptrs)
    assert rc == -2 and b"shard sizes" in lib.gcfd_last_error(gpu.ctx)
    # a non-physical state: NaN travels into the increment and is reported
    Q = gpu.get_global_state()
    Q[0, 0, 3] = np.nan
    gpu.set_global_state(Q)
    with pytest.raises(_lib.GcfdError) as ei:
        gpu.step(1)
    assert ei.value.code == -4
    gpu.close()
    ip = InputParameters2D(CFL=1, FluxType="roe", InitType="freestream", PolynomialOrder=7)
    with pytest.raises(_lib.GcfdError) as ei:
        Euler(ip, mesh)
    assert ei.value.code == -7
    bad = meshes.Mesh(mesh.VX, mesh.VY, mesh.EToV[:, [0, 2, 1]].copy(), [])
    ip = InputParameters2D(CFL=1, FluxType="roe", InitType="freestream", PolynomialOrder=1)
    with pytest.raises(_lib.GcfdError) as ei:
        Euler(ip, bad)
    assert ei.value.code == -1


def test_profile_step_counts_launches():
    mesh = meshes.vortex_box(8)
    gpu, _ = make_pair(mesh, 2, init="ivortex", vortex_center=(0.0, 0.0))
    ms, n = gpu.profile_step()
    assert n[:3] == [5, 5, 5] and all(m >= 0 for m in ms)
    gpu.close()
