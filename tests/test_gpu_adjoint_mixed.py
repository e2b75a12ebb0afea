"""The adjoint of the mixed path (gcfd_record_steps + gcfd_step_vjp on a
GCFD_PREC_FP32 / TF32X3 context): the mixed forward recomputes and tapes each
step (its own FP32 stage increments and stage RHS), and the reverse sweep runs
the adjoint kernels in FP32.

Checks, on the same inputs:
  * against the FP64 path's adjoint (itself checked against the oracle's
    central differences in test_gpu_adjoint.py): the directional derivative
    <Q0_bar, d> to 1e-5 relative, the whole Q0_bar field to the stated
    relative L2 bound, the far-field adjoint to 1e-5 and the time adjoint to
    1e-8 (final time weighted) or 1e-3 (a random final-state weight, whose
    time adjoint cancels to ~1% of its terms);
  * against the oracle's central differences directly: <Q0_bar, d> to 1e-5
    relative, the tolerance of the gradient check on the mixed path.
The mixed trajectory differs from the FP64 one by ~1e-8 relative, and FP32
Jacobians carry ~1e-7 relative rounding, so both comparisons hold with room
to spare on smooth states.
"""
import numpy as np
import pytest

from conftest import fixture
import oracle
from gocfd_gb300 import _lib, meshes
from gocfd_gb300.euler2d import Euler, InputParameters2D
from test_gpu_adjoint import far_box, perturbed, set_far, step_fd

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-5   # directional derivatives, time and far-field adjoints
FIELD_RTOL = 1e-4  # relative L2 of the whole Q0_bar field against the FP64 adjoint


def params(N, *, flux="roe", init="freestream", local_dt=False, cfl=0.8, minf=0.5, alpha=0.0):
    return InputParameters2D(CFL=cfl, FluxType=flux, InitType=init, PolynomialOrder=N, FinalTime=1e9, Minf=minf,
                             Gamma=1.4, Alpha=alpha, LocalTimeStepping=local_dt, MaxIterations=10 ** 9)


def oracle_for(mesh, N, *, flux="roe", init="freestream", local_dt=False, cfl=0.8, minf=0.5, alpha=0.0,
               vortex_center=(5.0, 0.0)):
    return oracle.OracleSolver(N, mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges, flux=flux, init=init, cfl=cfl,
                               final_time=1e9, minf=minf, gamma=1.4, alpha=alpha, local_dt=local_dt,
                               vortex_center=vortex_center)


def rel(a, b):
    return abs(a - b) / max(abs(a), abs(b), 1e-300)


def window_adjoint(mesh, ip, precision, Q0, t0, nsteps, every, Qbf, tbf=0.0, vortex_center=(5.0, 0.0)):
    with Euler(ip, mesh, 1, precision=precision, vortex_center=vortex_center) as g:
        g.set_global_state(Q0)
        g.time = t0
        t_end, _ = g.record(nsteps, every)
        Q_end = g.get_global_state()
        Qb0, qinfb, tb0 = g.step_vjp(Qbf, tbf)
        # the window's end state is back in place after the reverse sweep
        Q_back = g.get_global_state()
        assert np.array_equal(Q_back, Q_end)
        assert abs(g.time - t_end) == 0.0
    return Qb0, qinfb, tb0


@pytest.mark.parametrize("N", [1, 4])
def test_rhs_vjp_on_mixed_context_is_the_fp64_adjoint(N):
    """One RHS adjoint runs the FP64 kernels on a mixed context too: the same
    bits as an FP64 context's (the FP32 transpose of a single RHS loses up to
    ~5e-5 relative to DivInt's cancellation at N = 1 and 4)."""
    mesh = far_box(4, 4)
    ip = params(N, alpha=15.0)
    ora = oracle_for(mesh, N, alpha=15.0)
    rng = np.random.default_rng(100 + N)
    Q = perturbed(ora.Q, N, 0.02)
    Rb = rng.standard_normal(Q.shape)
    out = {}
    for prec in ("fp64", "fp32"):
        with Euler(ip, mesh, 1, precision=prec) as g:
            out[prec] = g.rhs_vjp_global(Q, Rb)
    assert np.array_equal(out["fp32"][0], out["fp64"][0])
    assert np.allclose(out["fp32"][1], out["fp64"][1], rtol=1e-13, atol=0.0)


@pytest.mark.parametrize("precision", ["fp32", "tf32x3"])
@pytest.mark.parametrize("every", [1, 4])
def test_mixed_step_vjp_vortex(precision, every):
    """10 steps of the isentropic vortex (IVortex boundaries, global dt): Q0, time
    and the window with and without the segment tape."""
    mesh = meshes.vortex_box(6, jitter=0.1)
    N, nsteps, t0 = 3, 10, 0.1
    # CFL 0.5: the oracle's differences at h = 1e-6, 5e-7, 2e-7 agree to 5e-9 (at
    # CFL 1 the h = 1e-6 pair straddles a switch of the dt-setting edge)
    ip = params(N, init="ivortex", cfl=0.5)
    ora = oracle_for(mesh, N, init="ivortex", cfl=0.5)
    rng = np.random.default_rng(7)
    Q0 = perturbed(ora.Q, 7, 0.01)
    Qbf = rng.standard_normal(Q0.shape)
    d = rng.standard_normal(Q0.shape) * np.abs(Q0)
    Qb64, _, tb64 = window_adjoint(mesh, ip, "fp64", Q0, t0, nsteps, every, Qbf)
    Qb32, _, tb32 = window_adjoint(mesh, ip, precision, Q0, t0, nsteps, every, Qbf)
    field = np.linalg.norm(Qb32 - Qb64) / np.linalg.norm(Qb64)
    g64, g32 = float(np.sum(Qb64 * d)), float(np.sum(Qb32 * d))
    print(f"mixed step adjoint ({precision}, every {every}): field rel L2 {field:.3e}, "
          f"<Qb,d> rel {rel(g32, g64):.3e}, t-bar rel {rel(tb32, tb64):.3e}")
    assert field <= FIELD_RTOL
    assert rel(g32, g64) <= GRAD_RTOL
    # the time adjoint of a random final-state weight is a sum over the boundary
    # points that cancels to ~1% of its terms' size: FP32 keeps ~1e-5 of the terms
    assert rel(tb32, tb64) <= 100 * GRAD_RTOL
    fd = step_fd(ora, Q0, t0, nsteps, Qbf, d, 1e-6)
    assert rel(g32, fd) <= GRAD_RTOL


@pytest.mark.parametrize("local_dt", [False, True])
def test_mixed_step_vjp_final_time_weight(local_dt):
    """Only the final time weighted (Qbar_final = 0, tbar_final = 1): the time
    adjoint runs back through every stage's dt and the IVortex boundary time."""
    mesh = meshes.vortex_box(6, jitter=0.1)
    N, nsteps, t0 = 3, 10, 0.1
    ip = params(N, init="ivortex", cfl=1.0, local_dt=local_dt)
    ora = oracle_for(mesh, N, init="ivortex", cfl=1.0, local_dt=local_dt)
    Q0 = perturbed(ora.Q, 7, 0.01)
    Qbf = np.zeros_like(Q0)
    Qb64, _, tb64 = window_adjoint(mesh, ip, "fp64", Q0, t0, nsteps, 1, Qbf, 1.0)
    Qb32, _, tb32 = window_adjoint(mesh, ip, "fp32", Q0, t0, nsteps, 1, Qbf, 1.0)
    scale = max(np.linalg.norm(Qb64), 1e-300)
    print(f"final-time weight (local dt {local_dt}): t-bar rel {rel(tb32, tb64):.3e}, "
          f"field rel L2 {np.linalg.norm(Qb32 - Qb64) / scale if np.linalg.norm(Qb64) > 0 else 0.0:.3e}")
    assert rel(tb32, tb64) <= 1e-8
    assert np.linalg.norm(Qb32 - Qb64) <= FIELD_RTOL * scale


def test_mixed_step_vjp_local_dt():
    """Local time stepping on the inflow / outflow / wall mesh: the dt adjoint
    runs through the taped per-element dt of every stage."""
    mesh = meshes.read_mesh(fixture("fstepA001.neu"))
    N, nsteps = 2, 5
    ip = params(N, local_dt=True, cfl=0.5, alpha=10.0)
    ora = oracle_for(mesh, N, local_dt=True, cfl=0.5, alpha=10.0)
    rng = np.random.default_rng(9)
    Q0 = perturbed(ora.Q, 9, 0.02)
    Qbf = rng.standard_normal(Q0.shape)
    d = rng.standard_normal(Q0.shape) * np.abs(Q0)
    Qb64, _, _ = window_adjoint(mesh, ip, "fp64", Q0, 0.0, nsteps, 2, Qbf)
    Qb32, _, _ = window_adjoint(mesh, ip, "fp32", Q0, 0.0, nsteps, 2, Qbf)
    field = np.linalg.norm(Qb32 - Qb64) / np.linalg.norm(Qb64)
    g64, g32 = float(np.sum(Qb64 * d)), float(np.sum(Qb32 * d))
    print(f"mixed step adjoint (local dt): field rel L2 {field:.3e}, <Qb,d> rel {rel(g32, g64):.3e}")
    assert field <= FIELD_RTOL
    assert rel(g32, g64) <= GRAD_RTOL
    fd = step_fd(ora, Q0, 0.0, nsteps, Qbf, d, 1e-7)
    assert rel(g32, fd) <= GRAD_RTOL


def test_mixed_step_vjp_farfield_state():
    """The far-field Qinf adjoint through the characteristic boundary points."""
    mesh = meshes.wedge_channel(8, 4)
    N, nsteps = 2, 5
    ip = params(N, minf=0.5, cfl=0.5)
    ora = oracle_for(mesh, N, minf=0.5, cfl=0.5)
    Q0 = perturbed(ora.Q, 11, 0.01)
    rng = np.random.default_rng(11)
    Qbf = rng.standard_normal(Q0.shape)
    _, q64, _ = window_adjoint(mesh, ip, "fp64", Q0, 0.0, nsteps, 1, Qbf)
    _, q32, _ = window_adjoint(mesh, ip, "fp32", Q0, 0.0, nsteps, 1, Qbf)
    print("far-field adjoint fp64", q64, "fp32", q32)
    assert np.all(np.abs(q32 - q64) <= GRAD_RTOL * np.abs(q64).max())


def test_mixed_field_error_functional_window():
    """J = sum (Q_final - Q_exact(t_final))^2 on the mixed path, adjoint through
    40 steps with a checkpoint every 8: against the FP64 path's adjoint."""
    mesh = meshes.vortex_box(8, jitter=0.1)
    N, nsteps = 2, 40
    ip = params(N, init="ivortex", cfl=0.5)
    ora = oracle_for(mesh, N, init="ivortex", cfl=0.5, vortex_center=(0.0, 0.0))
    Q0 = np.ascontiguousarray(ora.Q)
    d = np.random.default_rng(15).standard_normal(Q0.shape) * np.abs(Q0)
    res = {}
    for prec in ("fp64", "fp32"):
        with Euler(ip, mesh, 1, precision=prec, vortex_center=(0.0, 0.0)) as g:
            g.set_global_state(Q0)
            g.record(nsteps, 8)
            J, Qbf, tbf = g.functional("vortex_error")
            res[prec] = (J,) + g.step_vjp(Qbf, tbf)
    J64, Qb64, _, _ = res["fp64"]
    J32, Qb32, _, _ = res["fp32"]
    g64, g32 = float(np.sum(Qb64 * d)), float(np.sum(Qb32 * d))
    field = np.linalg.norm(Qb32 - Qb64) / np.linalg.norm(Qb64)
    print(f"field-error functional, 40 steps: J rel {rel(J32, J64):.3e}, field rel L2 {field:.3e}, "
          f"<Qb,d> rel {rel(g32, g64):.3e}")
    assert rel(g32, g64) <= GRAD_RTOL
    assert field <= FIELD_RTOL


def test_mixed_adjoint_rejects_dissipation():
    mesh = far_box(2, 2)
    ip = InputParameters2D(CFL=0.5, FluxType="roe", InitType="freestream", PolynomialOrder=2, FinalTime=1e9,
                           Minf=0.5, Gamma=1.4, Limiter="PerssonC0", Kappa=5.0)
    with Euler(ip, mesh, 1, precision="fp32") as gpu:
        with pytest.raises(_lib.GcfdError) as e:
            gpu.record(1)
        assert e.value.code == -7


def test_mixed_adjoint_smooth_directions_against_fp64_differences():
    """The gradient check of the vortex configurations at a small size (N = 4,
    vortex_box(48), 40 steps after 50, checkpoint every 10): the adjoint with the
    FP64 path's field-error weight, along d/dx0 and d/dbeta of the exact vortex,
    against Richardson-extrapolated FP64 central differences (GPU FP64 path): the
    FP64 adjoint to 1e-8 (the differences are clean), the mixed one to 1e-5."""
    from gocfd_gb300 import configs
    mesh = meshes.vortex_box(48, jitter=0.1)
    ip = InputParameters2D(CFL=1.0, FluxType="roe", InitType="ivortex", PolynomialOrder=4, FinalTime=1e9,
                           Minf=0.5, Gamma=1.4, MaxIterations=10 ** 9)
    steps = 40
    with Euler(ip, mesh, 1, precision="fp64", vortex_center=(0.0, 0.0)) as s:
        s.step(50)
        Q0, t0 = s.get_global_state(), s.time
        s.record(steps, 10)
        J, Qbf, tbf = s.functional("vortex_error")
        Qb64, _, _ = s.step_vjp(Qbf, tbf)
        X, Y = configs.solution_points_xy(s)

        def J_at(q):
            s.set_global_state(q)
            s.time = t0
            s.step(steps)
            return s.functional("vortex_error")[0]
        with Euler(ip, mesh, 1, precision="fp32", vortex_center=(0.0, 0.0)) as g:
            g.set_global_state(Q0)
            g.time = t0
            g.record(steps, 10)
            Qb32, _, _ = g.step_vjp(Qbf, tbf)
        for param in ("x0", "beta"):
            d = configs.exact_vortex_param_derivative(X, Y, t0, param)
            fd = {h: (J_at(Q0 + h * d) - J_at(Q0 - h * d)) / (2 * h) for h in (2e-4, 1e-4)}
            rich = (4 * fd[1e-4] - fd[2e-4]) / 3
            a64, a32 = float(np.sum(Qb64 * d)), float(np.sum(Qb32 * d))
            print(f"smooth direction {param}: FD {rich:.10e}, FP64 adjoint rel {rel(a64, rich):.3e}, "
                  f"mixed adjoint rel {rel(a32, rich):.3e}")
            assert rel(a64, rich) <= 1e-8
            assert rel(a32, rich) <= GRAD_RTOL


def test_mixed_window_taped_while_recording():
    """checkpoint_every >= nsteps on the mixed path: the recording keeps every
    step's tape and the reverse sweep recomputes nothing.  Its adjoint agrees
    with the checkpointed sweeps' (every 1, every 4) to FP32 rounding, a second
    sweep of the same window repeats it bit for bit, and stepping on between
    the two (the context's own stage arrays) leaves the window's tape alone."""
    mesh = meshes.vortex_box(6, jitter=0.1)
    N, nsteps, t0 = 3, 8, 0.1
    ip = params(N, init="ivortex", cfl=0.5)
    ora = oracle_for(mesh, N, init="ivortex", cfl=0.5)
    Q0 = perturbed(ora.Q, 7, 0.01)
    Qbf = np.random.default_rng(7).standard_normal(Q0.shape)
    res = {}
    for every in (1, 4, nsteps):
        res[every] = window_adjoint(mesh, ip, "fp32", Q0, t0, nsteps, every, Qbf)
    ref = res[1][0]
    for every in (4, nsteps):
        rel_l2 = np.linalg.norm(res[every][0] - ref) / np.linalg.norm(ref)
        print(f"taped window vs every {every}: rel L2 {rel_l2:.3e}")
        assert rel_l2 <= 1e-5
    with Euler(ip, mesh, 1, precision="fp32", vortex_center=(5.0, 0.0)) as g:
        g.set_global_state(Q0)
        g.time = t0
        g.record(nsteps, nsteps)
        assert g.window_taped()
        a1 = g.step_vjp(Qbf)[0]
        g.step(3)
        a2 = g.step_vjp(Qbf)[0]
    assert np.array_equal(a1, a2)
    assert np.linalg.norm(a1 - res[nsteps][0]) == 0.0


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_window_blocks_carried_to_the_next_window(precision):
    """A window's device blocks go to the next window (blocks of the same size
    reused, the rest held): a sequence of taped and checkpointed windows of
    different lengths on one context gives each window the adjoint a fresh
    context gives it — bit for bit on the mixed path; to 1e-13 relative on the
    FP64 path, whose global-dt adjoint sums its warps' FP64 partials by atomics
    (the order of those additions sets the last bits)."""
    mesh = meshes.vortex_box(6, jitter=0.1)
    N, t0 = 3, 0.1
    ip = params(N, init="ivortex", cfl=0.5)
    ora = oracle_for(mesh, N, init="ivortex", cfl=0.5)
    Q0 = perturbed(ora.Q, 11, 0.01)
    Qbf = np.random.default_rng(11).standard_normal(Q0.shape)
    seq = [(8, 8), (4, 4), (8, 4), (8, 8), (6, 2), (4, 4)]
    fresh = {w: window_adjoint(mesh, ip, precision, Q0, t0, w[0], w[1], Qbf)[0] for w in set(seq)}
    with Euler(ip, mesh, 1, precision=precision, vortex_center=(5.0, 0.0)) as g:
        for n, every in seq:
            g.set_global_state(Q0)
            g.time = t0
            g.record(n, every)
            assert g.window_taped() == (every >= n)
            a = g.step_vjp(Qbf)[0]
            ref = fresh[(n, every)]
            if precision == "fp32":
                assert np.array_equal(a, ref), (n, every)
            else:
                assert np.max(np.abs(a - ref)) <= 1e-13 * np.max(np.abs(ref)), (n, every)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_window_blocks_held_once_and_freed_with_the_context(precision):
    """Repeated windows of one shape take no further device memory, and
    gcfd_destroy frees the window's blocks with the pool."""
    import torch
    mesh = meshes.vortex_box(48, jitter=0.1)
    ip = params(3, init="ivortex", cfl=0.5)
    Qbf = None

    def free():
        torch.cuda.synchronize()
        return torch.cuda.mem_get_info()[0]

    def lifetime(windows):
        nonlocal Qbf
        with Euler(ip, mesh, 1, precision=precision, vortex_center=(0.0, 0.0)) as g:
            if Qbf is None:
                Qbf = np.random.default_rng(3).standard_normal(g.get_global_state().shape)
            seen = []
            for n, every in windows:
                g.record(n, every)
                g.step_vjp(Qbf)
                seen.append(free())
        return seen

    lifetime([(6, 6), (6, 2)])  # first launches (lazy module loading), then the baseline
    base = free()
    seen = lifetime([(6, 6), (6, 6), (6, 6), (6, 2), (6, 6)])
    slot = 10 * 4 * 10 * mesh.EToV.shape[0] * (4 if precision == "fp32" else 8)
    assert base - seen[0] >= 6 * slot                    # the taped window is held
    assert seen[1] == seen[0] and seen[2] == seen[0]     # the same shape again: nothing new
    assert seen[4] >= seen[3] - 2 ** 21                  # back to the taped shape: from the pool
    assert free() >= base - 2 ** 22                      # destroyed: all of it back
