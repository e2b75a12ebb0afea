"""The adjoint (gcfd_rhs_vjp, gcfd_record_steps + gcfd_step_vjp, gcfd_functional)
against central finite differences of the FP64 oracle, and torch gradchecks.

Every check is a directional one: for a random direction d,
<adjoint, d> against (J(x + h d) - J(x - h d)) / 2h with J the oracle's map
dotted with a random output weight.  Tolerance: 1e-6 relative to the larger
of the two sides (central differences at h ~ 1e-6 of the state scale are good
to ~1e-9 here; the time-step maxima stay on the same edge within +-h).
"""
import numpy as np
import pytest

from conftest import fixture
import oracle
from gocfd_gb300 import meshes
from gocfd_gb300.euler2d import Euler, InputParameters2D

pytestmark = pytest.mark.gpu

FD_RTOL = 1e-6


def make_pair(mesh, N, *, flux="roe", init="freestream", local_dt=False, cfl=0.8, minf=0.5, alpha=0.0,
              final_time=1e9, vortex_center=(5.0, 0.0)):
    ip = InputParameters2D(CFL=cfl, FluxType=flux, InitType=init, PolynomialOrder=N, FinalTime=final_time,
                           Minf=minf, Gamma=1.4, Alpha=alpha, LocalTimeStepping=local_dt, MaxIterations=10 ** 9)
    gpu = Euler(ip, mesh, 1, precision="fp64", vortex_center=vortex_center)
    ora = oracle.OracleSolver(N, mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges, flux=flux, init=init, cfl=cfl,
                              final_time=final_time, minf=minf, gamma=1.4, alpha=alpha, local_dt=local_dt,
                              vortex_center=vortex_center)
    return gpu, ora


def far_box(n=3, m=3):
    return meshes.structured_triangles(n, m, 0.0, 1.0, 0.0, 1.0, jitter=0.15, seed=3,
                                       tags=("wall", "far", "wall", "far"))


def set_far(ora, q):
    fs = oracle._fs(list(q), ora.far["gamma"], ora.far["minf"])
    f = ora.p.far
    for i in range(4):
        f.qinf[i] = fs["qinf"][i]
    f.pinf, f.cinf = fs["pinf"], fs["cinf"]


def assert_close(ad, fd, rtol=FD_RTOL, what=""):
    scale = max(abs(ad), abs(fd), 1e-300)
    assert abs(ad - fd) <= rtol * scale, (what, ad, fd, abs(ad - fd) / scale)


def perturbed(Q, seed, amp=0.05):
    rng = np.random.default_rng(seed)
    return np.ascontiguousarray(Q * (1.0 + amp * rng.uniform(-1, 1, Q.shape)))


# ----------------------------------------------------------------------------- RHS
@pytest.mark.parametrize("N", [1, 2, 3])
@pytest.mark.parametrize("flux", ["roe", "lax", "average", "roe-er"])
def test_rhs_vjp_directional_fd(N, flux):
    mesh = far_box()
    gpu, ora = make_pair(mesh, N, flux=flux, minf=0.5, alpha=15.0)
    rng = np.random.default_rng(10 * N + len(flux))
    Q = perturbed(ora.Q, N)
    Rb = rng.standard_normal(Q.shape)
    d = rng.standard_normal(Q.shape) * np.abs(Q)
    Qb, qinfb, _ = gpu.rhs_vjp_global(Q, Rb)
    h = 1e-6
    fd = (np.sum(Rb * ora.rhs(Q + h * d)) - np.sum(Rb * ora.rhs(Q - h * d))) / (2 * h)
    assert_close(float(np.sum(Qb * d)), fd, what="Q")
    # far-field Qinf (pinf and cinf follow it)
    q0 = np.array(ora.far["qinf"])
    dq = rng.standard_normal(4) * np.abs(q0).clip(0.1)
    set_far(ora, q0 + h * dq)
    jp = np.sum(Rb * ora.rhs(Q))
    set_far(ora, q0 - h * dq)
    jm = np.sum(Rb * ora.rhs(Q))
    set_far(ora, q0)
    assert_close(float(np.dot(qinfb, dq)), (jp - jm) / (2 * h), what="Qinf")
    gpu.close()


def test_rhs_vjp_inflow_outflow_mesh():
    mesh = meshes.read_mesh(fixture("fstepA001.neu"))
    gpu, ora = make_pair(mesh, 2, minf=0.5, alpha=10.0)
    rng = np.random.default_rng(5)
    Q = perturbed(ora.Q, 5)
    Rb = rng.standard_normal(Q.shape)
    d = rng.standard_normal(Q.shape) * np.abs(Q)
    Qb, _, _ = gpu.rhs_vjp_global(Q, Rb)
    h = 1e-6
    fd = (np.sum(Rb * ora.rhs(Q + h * d)) - np.sum(Rb * ora.rhs(Q - h * d))) / (2 * h)
    assert_close(float(np.sum(Qb * d)), fd)
    gpu.close()


def test_rhs_vjp_time_through_vortex_boundary():
    # the vortex centred on the boundary (the reference's (5, 0)) makes the
    # boundary state depend on time
    mesh = meshes.vortex_box(3, jitter=0.1)
    gpu, ora = make_pair(mesh, 2, init="ivortex", vortex_center=(5.0, 0.0))
    rng = np.random.default_rng(2)
    Q = perturbed(ora.Q, 2, 0.02)
    Rb = rng.standard_normal(Q.shape)
    t, h = 0.3, 1e-6
    _, _, tb = gpu.rhs_vjp_global(Q, Rb, t)
    fd = (np.sum(Rb * ora.rhs(Q, t + h)) - np.sum(Rb * ora.rhs(Q, t - h))) / (2 * h)
    assert_close(tb, fd)
    gpu.close()


def test_rhs_gradcheck_torch():
    torch = pytest.importorskip("torch")
    from gocfd_gb300.autograd import RHS
    mesh = meshes.structured_triangles(2, 2, 0.0, 1.0, 0.0, 1.0, jitter=0.1, seed=1,
                                       tags=("wall", "far", "wall", "far"))
    gpu, ora = make_pair(mesh, 2, minf=0.5, alpha=20.0)
    Q = torch.tensor(perturbed(ora.Q, 1), dtype=torch.float64, requires_grad=True)
    # Jacobian entries reach ~1e2 (DivInt / |J|); eps 1e-6 differences are good to ~1e-6 of that
    assert torch.autograd.gradcheck(lambda q: RHS.apply(q, gpu, 0.0), (Q,), eps=1e-6, atol=1e-5, rtol=1e-4)
    gpu.close()


# ----------------------------------------------------------------------------- steps
def step_fd(ora, Q0, t0, nsteps, Qbf, d, h, td=0.0):
    def J(sign):
        ora.Q = np.ascontiguousarray(Q0 + sign * h * d)
        ora.time = t0 + sign * h * td
        ora.DT[:] = 0.0
        ora.step(nsteps)
        return float(np.sum(Qbf * ora.Q))
    return (J(1.0) - J(-1.0)) / (2 * h)


@pytest.mark.parametrize("every", [1, 4])
def test_step_vjp_global_dt_vortex(every):
    """IVortex boundaries (time-dependent), global dt from the max wave speed."""
    mesh = meshes.vortex_box(4, jitter=0.1)
    gpu, ora = make_pair(mesh, 2, init="ivortex", cfl=1.0, vortex_center=(5.0, 0.0))
    rng = np.random.default_rng(7)
    Q0 = perturbed(ora.Q, 7, 0.01)
    nsteps, t0 = 6, 0.1
    gpu.set_global_state(Q0)
    gpu.time = t0
    gpu.record(nsteps, every)
    Qbf = rng.standard_normal(Q0.shape)
    Qb0, _, tb0 = gpu.step_vjp(Qbf)
    d = rng.standard_normal(Q0.shape) * np.abs(Q0)
    assert_close(float(np.sum(Qb0 * d)), step_fd(ora, Q0, t0, nsteps, Qbf, d, 1e-6), what="Q0")
    assert_close(tb0, step_fd(ora, Q0, t0, nsteps, Qbf, 0 * d, 1e-6, td=1.0), what="t0")
    gpu.close()


def test_step_vjp_final_time_clip():
    """The last steps' dt is FinalTime - t: its adjoint moves to the time."""
    mesh = meshes.vortex_box(4, jitter=0.1)
    gpu, ora = make_pair(mesh, 2, init="ivortex", cfl=1.0, vortex_center=(0.0, 0.0))
    gpu.set_global_state(ora.Q)
    t_probe, _ = gpu.record(3, 1)
    final = t_probe * 2.5 / 3.0  # reached inside the third step; the fourth has dt = 0
    gpu.close()
    gpu, ora = make_pair(mesh, 2, init="ivortex", cfl=1.0, vortex_center=(0.0, 0.0), final_time=final)
    rng = np.random.default_rng(8)
    Q0 = perturbed(ora.Q, 8, 0.01)
    gpu.set_global_state(Q0)
    t_end, _ = gpu.record(4, 2)
    assert abs(t_end - final) < 1e-12
    Qbf = rng.standard_normal(Q0.shape)
    Qb0, _, _ = gpu.step_vjp(Qbf)
    d = rng.standard_normal(Q0.shape) * np.abs(Q0)
    assert_close(float(np.sum(Qb0 * d)), step_fd(ora, Q0, 0.0, 4, Qbf, d, 1e-6))
    gpu.close()


def test_step_vjp_local_dt():
    """Local dt: every element's dt is a max over its edges' max wave speeds,
    so near-ties are common on a real mesh; h = 1e-7 keeps the differences
    clear of them on this one (checked: one-sided differences agree)."""
    mesh = meshes.read_mesh(fixture("fstepA001.neu"))
    gpu, ora = make_pair(mesh, 2, local_dt=True, cfl=0.5, minf=0.5, alpha=10.0)
    rng = np.random.default_rng(9)
    Q0 = perturbed(ora.Q, 9, 0.02)
    gpu.set_global_state(Q0)
    gpu.record(5, 2)
    Qbf = rng.standard_normal(Q0.shape)
    Qb0, _, _ = gpu.step_vjp(Qbf)
    d = rng.standard_normal(Q0.shape) * np.abs(Q0)
    assert_close(float(np.sum(Qb0 * d)), step_fd(ora, Q0, 0.0, 5, Qbf, d, 1e-7))
    gpu.close()


@pytest.mark.parametrize("minf,local_dt", [(0.5, False), (2.0, True)])
def test_step_vjp_farfield_state(minf, local_dt):
    """Gradient with respect to the far-field Qinf, initial state held fixed."""
    mesh = meshes.wedge_channel(8, 4)
    gpu, ora = make_pair(mesh, 2, minf=minf, local_dt=local_dt, cfl=0.5)
    rng = np.random.default_rng(11)
    Q0 = perturbed(ora.Q, 11, 0.01)
    nsteps = 5
    gpu.set_global_state(Q0)
    gpu.record(nsteps, 2)
    Qbf = rng.standard_normal(Q0.shape)
    _, qinfb, _ = gpu.step_vjp(Qbf)
    q0 = np.array(ora.far["qinf"])
    dq = rng.standard_normal(4) * np.abs(q0).clip(0.1)
    h = 1e-6

    def J(sign):
        set_far(ora, q0 + sign * h * dq)
        ora.Q = Q0.copy()
        ora.time = 0.0
        ora.step(nsteps)
        return float(np.sum(Qbf * ora.Q))
    fd = (J(1.0) - J(-1.0)) / (2 * h)
    set_far(ora, q0)
    assert_close(float(np.dot(qinfb, dq)), fd)
    gpu.close()


def test_step_gradcheck_torch():
    torch = pytest.importorskip("torch")
    from gocfd_gb300.autograd import Steps
    mesh = meshes.structured_triangles(2, 2, 0.0, 1.0, 0.0, 1.0, jitter=0.1, seed=2,
                                       tags=("wall", "far", "wall", "far"))
    gpu, ora = make_pair(mesh, 1, minf=0.5, alpha=20.0, cfl=0.5)
    Q = torch.tensor(perturbed(ora.Q, 3), dtype=torch.float64, requires_grad=True)
    assert torch.autograd.gradcheck(lambda q: Steps.apply(q, gpu, 2, 0.0, 1), (Q,), eps=1e-6, atol=1e-6,
                                    rtol=1e-5)
    gpu.close()


# ----------------------------------------------------------------------------- functionals
def edge_weights(el):
    t = el.R[2 * el.Np: 2 * el.Np + el.NpEdge]
    A = np.vander(t, el.NpEdge, increasing=True).T
    b = np.array([1.0 / (m + 1) if m % 2 == 0 else 0.0 for m in range(el.NpEdge)])
    return np.linalg.solve(A, b)


def wall_force_numpy(ora, mesh, Q, comp):
    el, g = ora.el, ora.geo
    NE = el.NpEdge
    w = edge_weights(el)
    faces = np.einsum("jp,npk->njk", el.FluxEdgeInterp, Q)
    J = 0.0
    for en in range(len(g.kL)):
        if g.bc[en] not in (5, 6):
            continue
        k, e = int(g.kL[en]), int(g.eL[en])
        v = mesh.EToV[k]
        a, b = v[e], v[(e + 1) % 3]
        length = np.hypot(mesh.VX[a] - mesh.VX[b], mesh.VY[a] - mesh.VY[b])
        n = g.nx[e, k] if comp == 0 else g.ny[e, k]
        for p in range(NE):
            q = faces[:, e * NE + p, k]
            pr = 0.4 * (q[3] - 0.5 * (q[1] ** 2 + q[2] ** 2) / q[0])
            J += length * w[p] * pr * n
    return J


@pytest.mark.parametrize("kind,comp", [("wall_force_x", 0), ("wall_force_y", 1)])
def test_wall_force_functional(kind, comp):
    mesh = meshes.wedge_channel(8, 4)
    gpu, ora = make_pair(mesh, 2, minf=2.0)
    Q = perturbed(ora.Q, 4, 0.05)
    gpu.set_global_state(Q)
    J, Qb, _ = gpu.functional(kind)
    ref = wall_force_numpy(ora, mesh, Q, comp)
    assert abs(J - ref) <= 1e-12 * max(1.0, abs(ref))
    rng = np.random.default_rng(4)
    d = rng.standard_normal(Q.shape) * np.abs(Q)
    h = 1e-6
    fd = (wall_force_numpy(ora, mesh, Q + h * d, comp) - wall_force_numpy(ora, mesh, Q - h * d, comp)) / (2 * h)
    assert_close(float(np.sum(Qb * d)), fd)
    gpu.close()


@pytest.mark.parametrize("kind,comp", [("wall_force_x", 0), ("wall_force_y", 1)])
def test_wall_force_on_the_reference_airfoil(kind, comp):
    """The wall force on the reference's own NACA 0012 mesh
    (test_cases/Euler2D/naca_12/mesh/naca12_2d-medium-lal.su2) at its input's
    Minf = 0.8, alpha = 1.25 (input-wall.yaml), on a perturbed freestream state:
    J against the oracle's faces, and the RHS there."""
    mesh = meshes.read_mesh(fixture("naca12_2d-medium-lal.su2"))
    gpu, ora = make_pair(mesh, 2, minf=0.8, alpha=1.25)
    Q = perturbed(ora.Q, 8, 0.05)
    gpu.set_global_state(Q)
    J, Qb, _ = gpu.functional(kind)
    ref = wall_force_numpy(ora, mesh, Q, comp)
    assert abs(J - ref) <= 1e-12 * max(1.0, abs(ref))
    r, rr = gpu.rhs_global(Q), ora.rhs(Q)
    assert np.abs(r - rr).max() <= 1e-9 * np.abs(rr).max() + 1e-13
    gpu.close()


def test_vortex_error_functional():
    mesh = meshes.vortex_box(4, jitter=0.1)
    gpu, ora = make_pair(mesh, 3, init="ivortex", vortex_center=(0.0, 0.0))
    Q = perturbed(ora.Q, 6, 0.01)
    gpu.set_global_state(Q)
    t = 0.25
    gpu.time = t
    J, Qb, tb = gpu.functional("vortex_error")
    ex = oracle.ivortex_state(ora.vortex, t, ora.geo.SolX, ora.geo.SolY)
    assert abs(J - np.sum((Q - ex) ** 2)) <= 1e-12 * np.sum((Q - ex) ** 2)
    assert np.allclose(Qb, 2 * (Q - ex), rtol=0, atol=1e-14)
    h = 1e-6
    jp = np.sum((Q - oracle.ivortex_state(ora.vortex, t + h, ora.geo.SolX, ora.geo.SolY)) ** 2)
    jm = np.sum((Q - oracle.ivortex_state(ora.vortex, t - h, ora.geo.SolX, ora.geo.SolY)) ** 2)
    assert_close(tb, (jp - jm) / (2 * h))
    gpu.close()


@pytest.mark.parametrize("precision,limiter", [("fp32", ""), ("fp64", "PerssonC0")])
def test_functional_on_mixed_and_dissipation_paths(precision, limiter):
    """The functionals on the mixed path and the PerssonC0 path, against the FP64 one."""
    mesh = meshes.wedge_channel(8, 4)
    ip = InputParameters2D(CFL=0.5, FluxType="roe", InitType="freestream", PolynomialOrder=2, FinalTime=1e9,
                           Minf=2.0, Gamma=1.4, Limiter=limiter, Kappa=6.0)
    gpu, ora = make_pair(mesh, 2, minf=2.0)
    Q = perturbed(ora.Q, 12, 0.05)
    gpu.set_global_state(Q)
    J_ref, _, _ = gpu.functional("wall_force_x")
    gpu.close()
    with Euler(ip, mesh, 1, precision=precision) as other:
        other.set_global_state(Q)
        J, Qb, _ = other.functional("wall_force_x")
    assert abs(J - J_ref) <= 1e-12 * abs(J_ref)
    assert np.all(np.isfinite(Qb))


@pytest.mark.parametrize("center", [(0.0, 0.0), (5.0, 0.0)])
def test_step_vjp_field_error_functional(center):
    """J = sum (Q_final - Q_exact(t_final))^2: the final time's adjoint enters through tfinal_bar."""
    mesh = meshes.vortex_box(4, jitter=0.1)
    gpu, ora = make_pair(mesh, 2, init="ivortex", cfl=1.0, vortex_center=center)
    Q0 = perturbed(ora.Q, 13, 0.01)
    nsteps = 6
    gpu.set_global_state(Q0)
    gpu.record(nsteps, 4)
    J, Qbf, tbf = gpu.functional("vortex_error")
    Qb0, _, _ = gpu.step_vjp(Qbf, tbf)
    rng = np.random.default_rng(14)
    d = rng.standard_normal(Q0.shape) * np.abs(Q0)
    vortex = (5.0, center[0], center[1], 1.4)
    X, Y = ora.geo.SolX, ora.geo.SolY

    def Jat(sign, h=1e-6):
        ora.Q = np.ascontiguousarray(Q0 + sign * h * d)
        ora.time = 0.0
        ora.step(nsteps)
        return float(np.sum((ora.Q - oracle.ivortex_state(vortex, ora.time, X, Y)) ** 2))
    assert abs(Jat(0.0) - J) <= 1e-10 * J
    fd = (Jat(1.0) - Jat(-1.0)) / 2e-6
    assert_close(float(np.sum(Qb0 * d)), fd)
    gpu.close()


# ----------------------------------------------------------------------------- with PerssonC0
def diss_pair(mesh, N, *, kappa=0.0, local_dt=False, cfl=0.5):
    ip = InputParameters2D(CFL=cfl, FluxType="roe", InitType="shocktube", PolynomialOrder=N, FinalTime=1e9,
                           Minf=0.5, Gamma=1.4, LocalTimeStepping=local_dt, MaxIterations=10 ** 9,
                           Limiter="PerssonC0", Kappa=kappa)
    gpu = Euler(ip, mesh, 1, precision="fp64")
    ora = oracle.OracleSolver(N, mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges, flux="roe", init="shocktube",
                              cfl=cfl, final_time=1e9, minf=0.5, local_dt=local_dt, limiter="PerssonC0",
                              kappa=kappa)
    return gpu, ora


def smooth_tube(ora, width):
    h = 0.5 * (1.0 + np.tanh((ora.geo.SolX - 0.5) / width))
    Q = np.zeros((4,) + h.shape)
    Q[0] = 1.0 + (0.125 - 1.0) * h
    Q[3] = (1.0 + (0.1 - 1.0) * h) / 0.4
    return Q


@pytest.mark.parametrize("N,kappa", [(1, 0.0), (2, 0.0), (2, 3.0), (3, 0.0)])
def test_rhs_vjp_with_dissipation(N, kappa):
    mesh = meshes.sod_channel(25, 3)
    gpu, ora = diss_pair(mesh, N, kappa=kappa)
    rng = np.random.default_rng(20 + N)
    Q = smooth_tube(ora, 0.02 if N == 1 else 0.008)
    Q = np.ascontiguousarray(Q * (1.0 + 0.01 * rng.uniform(-1, 1, Q.shape)))
    sig = ora.sensor(Q)[1]
    assert ((sig > 0) & (sig < 1)).any()  # the ramp is live somewhere
    Rb = rng.standard_normal(Q.shape)
    d = rng.standard_normal(Q.shape) * np.abs(Q)
    Qb, _, _ = gpu.rhs_vjp_global(Q, Rb)
    ad = float(np.sum(Qb * d))
    # The vertex maxima and the ramp's ends are kinks; a central difference
    # that straddles one disagrees with the one-sided adjoint, so the check
    # takes the best of three step sizes (a kink cannot sit inside all three).
    errs = []
    for h in (1e-6, 1e-7, 1e-8):
        fd = (np.sum(Rb * ora.rhs(Q + h * d)) - np.sum(Rb * ora.rhs(Q - h * d))) / (2 * h)
        errs.append(abs(ad - fd) / max(abs(ad), abs(fd)))
    assert min(errs) <= FD_RTOL, errs
    gpu.close()


@pytest.mark.parametrize("N,local_dt", [(2, False), (2, True), (3, False)])
def test_step_vjp_with_dissipation(N, local_dt):
    mesh = meshes.sod_channel(24, 3)
    gpu, ora = diss_pair(mesh, N, local_dt=local_dt)
    rng = np.random.default_rng(30 + N)
    Q0 = smooth_tube(ora, 0.01)
    Q0 = np.ascontiguousarray(Q0 * (1.0 + 0.005 * rng.uniform(-1, 1, Q0.shape)))
    nsteps = 4
    gpu.set_global_state(Q0)
    gpu.record(nsteps, 2)
    Qbf = rng.standard_normal(Q0.shape)
    Qb0, _, _ = gpu.step_vjp(Qbf)
    d = rng.standard_normal(Q0.shape) * np.abs(Q0)

    def J(sign, h=1e-7):
        ora.Q = np.ascontiguousarray(Q0 + sign * h * d)
        ora.time = 0.0
        ora.DT[:] = 0.0
        ora.DTVisc[:] = 0.0
        ora.step(nsteps)
        return float(np.sum(Qbf * ora.Q))
    fd = (J(1.0) - J(-1.0)) / 2e-7
    assert_close(float(np.sum(Qb0 * d)), fd)
    gpu.close()


@pytest.mark.parametrize("limiter,local_dt", [("", False), ("", True), ("PerssonC0", False)])
def test_segment_tape_matches_per_step_recompute(limiter, local_dt):
    """A window with several steps per checkpoint segment keeps each recomputed
    step's tape (one slot per step, faces rebuilt from the stage states); one
    step per segment tapes each step as it is reversed.  Both run the same
    kernels on the same states; they differ only where the adjoint sums over
    the mesh with atomics (the global time step's adjoint), in the order of
    those FP64 additions, so they agree to round-off (1e-12 of the largest
    entry), as two sweeps of one window do."""
    if limiter:
        mesh = meshes.sod_channel(24, 3)
        init, minf = "shocktube", 0.0
    else:
        mesh = meshes.vortex_box(6, jitter=0.1)
        init, minf = "ivortex", 0.5
    ip = InputParameters2D(CFL=0.8, FluxType="roe", InitType=init, PolynomialOrder=2, FinalTime=1e9,
                           Minf=minf, Gamma=1.4, LocalTimeStepping=local_dt, MaxIterations=10 ** 9,
                           Limiter=limiter, Kappa=5.0)
    rng = np.random.default_rng(41)
    out = []
    for every in (1, 3, 7):
        with Euler(ip, mesh, 1, precision="fp64") as gpu:
            Q0 = gpu.get_global_state()
            Q0 = np.ascontiguousarray(Q0 * (1.0 + 0.003 * np.random.default_rng(40).uniform(-1, 1, Q0.shape)))
            gpu.set_global_state(Q0)
            gpu.record(7, every)
            # every = 7 covers the window: it is taped while recording, nothing recomputed
            assert gpu.window_taped() == (every == 7)
            Qbf = np.random.default_rng(42).standard_normal(Q0.shape)
            out.append(gpu.step_vjp(Qbf, 0.3))
            # a second reverse sweep of the same window gives the same adjoint
            again = gpu.step_vjp(Qbf, 0.3)
            assert np.abs(again[0] - out[-1][0]).max() <= 1e-12 * np.abs(out[-1][0]).max()
    scale = np.abs(out[0][0]).max()
    for qb, qinf, tb in out[1:]:
        assert np.abs(qb - out[0][0]).max() <= 1e-12 * scale
        assert np.allclose(qinf, out[0][1], rtol=1e-11, atol=1e-12 * scale)
        assert abs(tb - out[0][2]) <= 1e-11 * max(abs(tb), 1e-300) + 1e-12 * scale
