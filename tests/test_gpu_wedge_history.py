"""The wedge's steady march (Mach 2 over a 15 degree ramp, local time
stepping, PerssonC0 with Kappa 6: test_cases/Euler2D/Wedge/input.yaml) on a
reduced 64 x 32 mesh at N = 2: the GPU FP64 path and the FP64 oracle advance
side by side for 2,000 steps and their per-step residual histories (RMS of
the final RK increment per variable, the residual Solve prints,
euler.go:814-849) are compared.

Both histories flatten out at the same level (the increment RMS stops
decaying after ~500 steps) and agree step by step to round-off, with the two
states still equal to ~1e-12 after 2,000 steps: the plateau belongs to the
scheme the oracle restates, not to the GPU implementation.  At the end, the
largest increments sit on a few elements at the top wall downstream of the
reflected shock, where the shock sensor is off.
"""
import os

import numpy as np
import pytest

import oracle
from gocfd_gb300 import meshes
from gocfd_gb300.euler2d import Euler, InputParameters2D

pytestmark = pytest.mark.gpu

STEPS = int(os.environ.get("GCFD_WEDGE_STEPS", "2000"))


def test_wedge_residual_history_matches_oracle():
    mesh = meshes.wedge_channel(64, 32)
    N = 2
    ip = InputParameters2D(CFL=1.0, FluxType="roe", InitType="freestream", PolynomialOrder=N, FinalTime=1e9,
                           Minf=2.0, Gamma=1.4, LocalTimeStepping=True, MaxIterations=10 ** 9,
                           Limiter="PerssonC0", Kappa=6.0)
    ora = oracle.OracleSolver(N, mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges, flux="roe", init="freestream",
                              cfl=1.0, minf=2.0, gamma=1.4, local_dt=True, limiter="PerssonC0", kappa=6.0)
    hg, ho = np.zeros((STEPS, 4)), np.zeros((STEPS, 4))
    with Euler(ip, mesh, 1, precision="fp64") as gpu:
        for n in range(STEPS):
            hg[n] = gpu.step(1)["resid_rms"]
            _, _, R = ora.step(1)
            ho[n] = np.sqrt((R.reshape(4, -1) ** 2).mean(axis=1))
        q_gpu = gpu.get_global_state()
        q_prev = q_gpu.copy()
        info = gpu.step(1)
        R_gpu = gpu.get_global_state() - q_prev
    rel = np.abs(hg - ho) / np.maximum(np.abs(ho), 1e-300)
    state_diff = float(np.linalg.norm(q_gpu - ora.Q) / np.linalg.norm(ora.Q))
    # Where the residual sits at the end: element-wise max |R| of the energy.
    el_res = np.abs(R_gpu[3]).max(axis=0)
    top = np.argsort(el_res)[::-1][: max(1, mesh.K // 100)]
    share = float((el_res[top] ** 2).sum() / (el_res ** 2).sum())
    _, sigma, _, _, _ = ora.sensor(ora.Q)
    active_top = float(np.mean(sigma[top] > 0))
    cx = mesh.VX[mesh.EToV[top]].mean(axis=1)
    cy = mesh.VY[mesh.EToV[top]].mean(axis=1)
    qn = np.sqrt((q_gpu.reshape(4, -1) ** 2).mean(axis=1))
    marks = [s for s in (1, 10, 100, 500, 1000, 1500, STEPS) if s <= STEPS]
    print("\nstep  rms(R) per variable (GPU FP64)            max rel diff to the oracle")
    for s in marks:
        print(f"{s:5d}  " + " ".join(f"{v:.3e}" for v in hg[s - 1]) + f"   {rel[s - 1].max():.2e}")
    print(f"final rms(R)/rms(Q) per variable: {np.array(info['resid_rms']) / qn}")
    print(f"state rel L2 GPU vs oracle after {STEPS} steps: {state_diff:.3e}")
    print(f"top 1% elements by |R_E| carry {share:.2f} of ||R_E||^2; sensor active on {active_top:.2f} of them;"
          f" centroids x in [{cx.min():.2f}, {cx.max():.2f}], y in [{cy.min():.2f}, {cy.max():.2f}]")
    # the histories agree step by step; the states stay together; the plateau is the oracle's too
    assert rel.max() <= 1e-9, rel.max()
    assert state_diff <= 1e-10
    late = slice(STEPS // 2, STEPS)
    assert np.allclose(np.median(hg[late], axis=0), np.median(ho[late], axis=0), rtol=1e-6)
    if STEPS >= 1000:  # no decay towards a steady state after the first few hundred steps
        assert hg[-1, 3] > 0.5 * hg[STEPS // 4, 3]
