"""The exact Sod solution against TestSOD's golden vectors
(model_problems/Euler1D/sod_shock_tube/analytic_sod_test.go:16-30)."""
import numpy as np

from gocfd_gb300.sod import SodExact

X_T01 = [0, 0.3815784043380077, 0.3817784043380077, 0.39280783577858336, 0.40393726721915907, 0.4150666986597348,
         0.42619613010031043, 0.4373255615408861, 0.4484549929814618, 0.4595844244220375, 0.47071385586261316,
         0.4818432873031888, 0.49277271874376455, 0.49287271874376454, 0.4930727187437645, 0.5926452620047974,
         0.5928452620047974, 0.675115573202932, 0.675315573202932, 1]
RHO_T01 = [1, 1, 0.9992959031724784, 0.9240353444481086, 0.852758969991083, 0.7859504402212434, 0.7233963393812908,
           0.6648901587403833, 0.6102321829702019, 0.5592293765210307, 0.5116952699978237, 0.467449846536279,
           0.4270320564069276, 0.42667562327066666, 0.4263194281781805, 0.4263194281781805, 0.26557371170513905,
           0.26557371170513905, 0.125, 0.125]


def test_sod_golden_vectors_t01():
    sod = SodExact(0.1)
    X, rho = sod.sample()
    assert np.allclose(X, X_T01, rtol=0, atol=1e-3)
    assert np.allclose(rho, RHO_T01, rtol=0, atol=1e-3)
    assert abs(sod.x4 - 0.6752) < 1e-4


def test_sod_shock_position_t02():
    assert abs(SodExact(0.2).x4 - 0.8504) < 1e-4


def test_sod_states_are_consistent():
    sod = SodExact(0.2)
    rho, p, u, E, m = sod.getx(0.5 * (sod.x3 + sod.x4))  # between contact and shock
    assert rho == sod.post[0] and p == sod.post[1]
    assert abs(E - (p / 0.4 + 0.5 * rho * u * u)) < 1e-15
