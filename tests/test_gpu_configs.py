"""The validation configurations at reduced size: the vortex against its exact
solution, the Sod tube against the exact Riemann solution (and the oracle's
run of the same mesh), and the wedge's steady march with its ramp force."""
import numpy as np
import pytest

import oracle
from gocfd_gb300 import configs
from gocfd_gb300.sod import SodExact

pytestmark = pytest.mark.gpu


def test_vortex20_full_size():
    out = configs.run("vortex20")
    assert out["K"] == 800 and out["steps"] == 100
    assert out["rel_l2_vs_exact"] < 1e-2   # N=2 on 20x20 quads


def test_sod_reduced_against_exact_and_oracle():
    out = configs.run("sod2000x100", scale=0.05)          # 100 x 5 quads
    assert abs(out["time"] - 0.2) < 1e-12
    err = out["density_error"]
    cfg = configs.CONFIGS["sod2000x100"]
    mesh = configs.build_mesh(cfg, 0.05)
    ora = oracle.OracleSolver(cfg.N, mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges, init="shocktube",
                              limiter="PerssonC0", kappa=cfg.kappa, cfl=cfg.cfl, final_time=cfg.final_time)
    while ora.time < 0.2 * (1 - 1e-12):
        ora.step(100)
    ora_l1 = float(np.abs(ora.Q[0] - SodExact(ora.time).density(ora.geo.SolX)).mean())
    assert err["l1"] < 0.01
    assert abs(err["l1"] - ora_l1) <= 0.05 * ora_l1


def test_wedge_reduced_march():
    out = configs.run("wedge512x256", scale=1 / 32, max_steps=300)   # 16 x 8 quads
    assert np.isfinite(out["residual_rel_rms"])
    assert out["ramp_force_x"] > 0.0   # the ramp pushes back on the flow: +x pressure force on the wall


def test_wedge_force_sensitivities_reduced():
    """dJ/dMinf and dJ/dalpha of the ramp force (PerssonC0, local dt) by the adjoint
    against central differences of the FP64 forward."""
    out = configs.wedge_sensitivity(steps=20, every=5, scale=1 / 32, fd_h=1e-5)
    assert out["rel_diff_Minf"] <= 1e-6, out
    assert out["rel_diff_alpha"] <= 1e-6, out


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-7)])
def test_reference_vortex_benchmark_input(precision, tol):
    """The reference's isentropic-vortex benchmark input as it ships
    (test_cases/Euler2D/isentropic-vortex/input-bench.yaml: Lax flux, IVortex,
    N = 2, CFL 1, FinalTime 0.5) on its mesh (vortex-new.su2, the vortex at the
    reference's default centre (5, 0)): 40 steps through the C ABI against the
    oracle with the same parameters, and both against the exact vortex.  (Its
    MaxIterations is absent, i.e. 0, so the reference's Solve stops after one
    step; the steps here are taken directly.)"""
    from conftest import fixture
    from gocfd_gb300 import meshes
    from gocfd_gb300.euler2d import Euler, InputParameters2D
    ip = InputParameters2D.from_file(fixture("inputs/isentropic-vortex_input-bench.yaml"))
    assert (ip.FluxType, ip.InitType, ip.PolynomialOrder, ip.MaxIterations) == ("Lax", "IVortex", 2, 0)
    mesh = meshes.read_mesh(fixture("vortex-new.su2"))
    ora = oracle.OracleSolver(ip.PolynomialOrder, mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges, flux="lax",
                              init="ivortex", cfl=ip.CFL, final_time=ip.FinalTime, minf=ip.Minf, gamma=ip.Gamma,
                              vortex_center=(5.0, 0.0))
    with Euler(ip, mesh, 1, precision=precision, vortex_center=(5.0, 0.0)) as g:
        info = g.step(40)
        Q = g.get_global_state()
        t = info["time"]
    ora.step(40)
    assert abs(t - ora.time) <= (1e-12 if precision == "fp64" else 1e-7) * max(1.0, ora.time)
    assert np.linalg.norm(Q - ora.Q) <= tol * np.linalg.norm(ora.Q)
    ex = oracle.ivortex_state(ora.vortex, ora.time, ora.geo.SolX, ora.geo.SolY)
    e_gpu, e_ora = np.linalg.norm(Q - ex), np.linalg.norm(ora.Q - ex)
    assert abs(e_gpu - e_ora) <= 1e-3 * e_ora


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-7)])
def test_reference_airfoil_wall_input(precision, tol):
    """The reference's NACA 0012 input (test_cases/Euler2D/naca_12/input-wall.yaml:
    Roe, N = 0, Minf 0.8, alpha 1.25, local time stepping; its PerssonC0 limiter is
    off at N = 0, as NewEuler builds it only for N > 0) on its medium mesh: 30
    steps against the oracle."""
    from conftest import fixture
    from gocfd_gb300 import meshes
    from gocfd_gb300.euler2d import Euler, InputParameters2D
    ip = InputParameters2D.from_file(fixture("inputs/naca_12_input-wall.yaml"))
    assert (ip.PolynomialOrder, ip.LocalTimeStepping, ip.Minf, ip.Alpha) == (0, True, 0.8, 1.25)
    mesh = meshes.read_mesh(fixture("naca12_2d-medium-lal.su2"))
    ora = oracle.OracleSolver(0, mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges, flux="roe", init="freestream",
                              cfl=ip.CFL, final_time=ip.FinalTime, minf=ip.Minf, gamma=ip.Gamma, alpha=ip.Alpha,
                              local_dt=True)
    with Euler(ip, mesh, 1, precision=precision) as g:
        g.step(30)
        Q = g.get_global_state()
    ora.step(30)
    assert np.linalg.norm(Q - ora.Q) <= tol * np.linalg.norm(ora.Q)
