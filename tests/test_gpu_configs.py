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
