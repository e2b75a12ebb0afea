"""The exact Sod solution against TestSOD's golden vectors
(model_problems/Euler1D/sod_shock_tube/analytic_sod_test.go:16-30)."""
import numpy as np

from conftest import golden
from gocfd_gb300.sod import SodExact

def test_sod_golden_vectors_t01():
    g = golden("sod_t01")
    sod = SodExact(0.1)
    X, rho = sod.sample()
    assert np.allclose(X, g["x"], rtol=0, atol=g["atol"])
    assert np.allclose(rho, g["rho"], rtol=0, atol=g["atol"])
    assert abs(sod.x4 - g["x4"]) < g["x4_atol"]


def test_sod_shock_position_t02():
    g = golden("sod_t02")
    assert abs(SodExact(0.2).x4 - g["x4"]) < g["x4_atol"]


def test_sod_states_are_consistent():
    sod = SodExact(0.2)
    rho, p, u, E, m = sod.getx(0.5 * (sod.x3 + sod.x4))  # between contact and shock
    assert rho == sod.post[0] and p == sod.post[1]
    assert abs(E - (p / 0.4 + 0.5 * rho * u * u)) < 1e-15
