"""ORACLE (test infrastructure only): builds and drives the C++ FP64 restatement
of gocfd's Euler2D RHS / SSP-RK step (euler_oracle.cpp) on operators and
geometry from the numpy restatement (dfr_ops.py).

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, as the checker; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
import sys
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import dfr_ops  # noqa: E402

LIB = os.path.join(HERE, "_build", "liboracle.so")
SRC = os.path.join(HERE, "euler_oracle.cpp")
_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """g++ -O3 -fopenmp build of the oracle into oracle/_build/ (git-ignored)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = LIB + f".{os.getpid()}.tmp"
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off", SRC, "-o", tmp]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stderr)
    os.replace(tmp, LIB)
    return LIB


class _FS(C.Structure):
    _fields_ = [("qinf", C.c_double * 4), ("pinf", C.c_double), ("cinf", C.c_double),
                ("gamma", C.c_double), ("minf", C.c_double)]


PD = C.POINTER(C.c_double)
PL = C.POINTER(C.c_int64)


class _Problem(C.Structure):
    _fields_ = [
        ("N", C.c_int32), ("K", C.c_int32), ("Np", C.c_int32), ("NpEdge", C.c_int32),
        ("NpFlux", C.c_int32), ("nEdges", C.c_int32),
        ("FluxEdgeInterp", PD), ("DivInt", PD), ("Jdet", PD), ("Jinv", PD), ("nx", PD), ("ny", PD),
        ("IInII", PD), ("hK", PD), ("FluxX", PD), ("FluxY", PD),
        ("kL", PL), ("eL", PL), ("kR", PL), ("eR", PL), ("bc", PL), ("EtoEdge", PL),
        ("flux_type", C.c_int32), ("flux_mock", C.c_int32), ("local_dt", C.c_int32), ("pad", C.c_int32),
        ("cfl", C.c_double), ("final_time", C.c_double), ("gamma", C.c_double),
        ("far", _FS), ("inn", _FS), ("out", _FS),
        ("vbeta", C.c_double), ("vx0", C.c_double), ("vy0", C.c_double), ("vgamma", C.c_double),
        ("diss", C.c_int32), ("nverts", C.c_int32), ("EtoV", PL), ("V", PD), ("Vinv", PD), ("SensD", PD),
        ("SensP", PD), ("Mass", PD), ("ModeFilter", PD), ("Div", PD), ("Bary", PD),
        ("kappa", C.c_double), ("eps0", C.c_double),
    ]


def load():
    global _lib
    with _lock:
        if _lib is None:
            lib = C.CDLL(build())
            lib.oracle_rhs.argtypes = [C.POINTER(_Problem), C.c_double, PD, PD, PD]
            lib.oracle_rhs_faces.argtypes = [C.POINTER(_Problem), C.c_double, PD, PD, PD]
            lib.oracle_step.argtypes = [C.POINTER(_Problem), C.c_int, PD, PD, PD, PD, PD, PD]
            lib.oracle_shock_indicator.argtypes = [C.POINTER(_Problem), PD, PD, C.c_double]
            lib.oracle_shock_indicator.restype = C.c_double
            lib.oracle_sensor.argtypes = [C.POINTER(_Problem), PD, PD, PD, PD, PD, PD]
            lib.oracle_vertex_max.argtypes = [C.POINTER(_Problem), PD, PD]
            lib.oracle_gradient.argtypes = [C.POINTER(_Problem), PD, PD, PD]
            lib.oracle_num_threads.restype = C.c_int
            lib.oracle_set_threads.argtypes = [C.c_int]
            _lib = lib
    return _lib


FLUX = {"average": 0, "lax": 1, "roe": 2, "roe-er": 3}
INIT = {"freestream": 0, "ivortex": 1, "shocktube": 2}


def freestream_mach(minf, gamma, alpha):
    """NewFreeStream (fluids.go:378-395)."""
    q = [1.0, minf * math.cos(alpha * math.pi / 180.0), minf * math.sin(alpha * math.pi / 180.0),
         1.0 / (gamma * (gamma - 1.0)) + 0.5 * minf * minf]
    return _fs(q, gamma, minf)


def freestream_q(gamma, q):
    """NewFreestreamFromQinf (fluids.go:397-406)."""
    return _fs(q, gamma, 0.0)


def _fs(q, gamma, minf):
    rho, u, v = q[0], q[1] / q[0], q[2] / q[0]
    p = (gamma - 1.0) * (q[3] - 0.5 * rho * (u * u + v * v))
    return dict(qinf=list(q), pinf=p, cinf=math.sqrt(abs(gamma * p / rho)), gamma=gamma, minf=minf)


class OracleSolver:
    """Euler2D on the CPU in FP64, with the reference's set-up semantics."""

    def __init__(self, N, VX, VY, EToV, bc_edges, *, flux="roe", init="freestream", cfl=1.0,
                 final_time=1e30, minf=0.1, gamma=1.4, alpha=0.0, local_dt=False,
                 vortex_center=(5.0, 0.0), flux_mock=0, limiter="", kappa=0.0):
        self.el = dfr_ops.build_element(N)
        bc_edges = list(bc_edges) if bc_edges is not None else []
        if init == "ivortex":  # Wall -> IVortex relabel (euler.go:780-790)
            bc_edges = [(a, b, 9 if f == 5 else f) for (a, b, f) in bc_edges]
        self.geo = dfr_ops.build_geometry(self.el, VX, VY, EToV, bc_edges)
        self.N, self.K = N, self.geo.K
        far = freestream_mach(minf, gamma, alpha)
        fin = fout = far
        if init == "ivortex":
            far = freestream_q(1.4, [1.0, 1.0, 0.0, 3.0])
        elif init == "shocktube":
            g = 1.4
            fin = freestream_q(g, [1.0, 0.0, 0.0, 1.0 / (g - 1.0)])
            fout = freestream_q(g, [0.125, 0.0, 0.0, 0.1 / (g - 1.0)])
        self.far, self.fin, self.fout = far, fin, fout
        self.init = init
        self.vortex = (5.0, vortex_center[0], vortex_center[1], 1.4)
        el, g = self.el, self.geo
        self._keep = dict(
            I=np.ascontiguousarray(el.FluxEdgeInterp), D=np.ascontiguousarray(el.DivInt),
            Jdet=np.ascontiguousarray(g.Jdet), Jinv=np.ascontiguousarray(g.Jinv),
            nx=np.ascontiguousarray(g.nx), ny=np.ascontiguousarray(g.ny), II=np.ascontiguousarray(g.IInII),
            hK=np.ascontiguousarray(g.hK), FX=np.ascontiguousarray(g.FluxX), FY=np.ascontiguousarray(g.FluxY),
            kL=np.ascontiguousarray(g.kL, np.int64), eL=np.ascontiguousarray(g.eL, np.int64),
            kR=np.ascontiguousarray(g.kR, np.int64), eR=np.ascontiguousarray(g.eR, np.int64),
            bc=np.ascontiguousarray(g.bc, np.int64), E2E=np.ascontiguousarray(g.EtoEdge, np.int64))
        k = self._keep
        p = _Problem()
        p.N, p.K, p.Np, p.NpEdge, p.NpFlux, p.nEdges = N, g.K, el.Np, el.NpEdge, el.NpFlux, len(g.kL)
        for name, key in (("FluxEdgeInterp", "I"), ("DivInt", "D"), ("Jdet", "Jdet"), ("Jinv", "Jinv"),
                          ("nx", "nx"), ("ny", "ny"), ("IInII", "II"), ("hK", "hK"), ("FluxX", "FX"),
                          ("FluxY", "FY")):
            setattr(p, name, k[key].ctypes.data_as(PD))
        for name, key in (("kL", "kL"), ("eL", "eL"), ("kR", "kR"), ("eR", "eR"), ("bc", "bc"),
                          ("EtoEdge", "E2E")):
            setattr(p, name, k[key].ctypes.data_as(PL))
        p.flux_type = FLUX[flux]
        p.flux_mock = flux_mock
        p.local_dt = int(local_dt)
        p.cfl, p.final_time = cfl, final_time
        p.gamma = far["gamma"]
        for fld, fs in (("far", far), ("inn", fin), ("out", fout)):
            s = getattr(p, fld)
            for i in range(4):
                s.qinf[i] = fs["qinf"][i]
            s.pinf, s.cinf, s.gamma, s.minf = fs["pinf"], fs["cinf"], fs["gamma"], fs["minf"]
        p.vbeta, p.vx0, p.vy0, p.vgamma = self.vortex
        # PerssonC0 dissipation (euler.go:107-112: only for N > 0); Eps0 = 5/1.5
        # regardless of Kappa, which only sets the sensor ramp (dissipation.go:140-147).
        self.diss = limiter.strip().lower() in ("perssonc0", "persson c0") and N != 0
        el = self.el
        k.update(EtoV=np.ascontiguousarray(np.asarray(EToV, np.int64)), V=np.ascontiguousarray(el.V),
                 Vinv=np.ascontiguousarray(el.Vinv), SD=np.ascontiguousarray(el.SensD),
                 SP=np.ascontiguousarray(el.SensP), M=np.ascontiguousarray(el.MassMatrix),
                 MF=np.ascontiguousarray(el.ModeFilter), Div=np.ascontiguousarray(el.Div),
                 Bary=np.ascontiguousarray(el.Bary), Clip=np.ascontiguousarray(el.Clipper))
        p.diss = int(self.diss)
        p.nverts = len(VX)
        p.EtoV = k["EtoV"].ctypes.data_as(PL)
        for name, key in (("V", "V"), ("Vinv", "Vinv"), ("SensD", "SD"), ("SensP", "SP"), ("Mass", "M"),
                          ("ModeFilter", "MF"), ("Div", "Div"), ("Bary", "Bary")):
            setattr(p, name, k[key].ctypes.data_as(PD))
        p.kappa = 5.0 if kappa == 0.0 else kappa
        p.eps0 = 5.0 / 1.5
        self.p = p
        self.lib = load()
        self.Q = self.initial_state()
        self.time = 0.0
        self.DT = np.zeros(self.K)
        self.DTVisc = np.zeros(self.K)

    def initial_state(self):
        """InitializeSolution (euler.go:728-794); returns 4 x Np x K."""
        el, g = self.el, self.geo
        Q = np.zeros((4, el.Np, self.K))
        if self.init == "ivortex":
            Q[:] = ivortex_state(self.vortex, 0.0, g.SolX, g.SolY)
        elif self.init == "shocktube":
            left = g.SolX < 0.5
            for n in range(4):
                Q[n] = np.where(left, self.fin["qinf"][n], self.fout["qinf"][n])
        else:
            for n in range(4):
                Q[n] = self.far["qinf"][n]
        return Q

    def rhs(self, Q, time=0.0, return_faces=False):
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        out = np.zeros_like(Q)
        faces = np.zeros((4, 3 * self.el.NpEdge, self.K)) if return_faces else None
        self.lib.oracle_rhs(C.byref(self.p), time, Q.ctypes.data_as(PD), out.ctypes.data_as(PD),
                            faces.ctypes.data_as(PD) if return_faces else None)
        return (out, faces) if return_faces else out

    def rhs_faces(self, Q, faces, time=0.0):
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        faces = np.ascontiguousarray(faces, dtype=np.float64)
        out = np.zeros_like(Q)
        self.lib.oracle_rhs_faces(C.byref(self.p), time, Q.ctypes.data_as(PD), faces.ctypes.data_as(PD),
                                  out.ctypes.data_as(PD))
        return out

    def step(self, nsteps=1):
        """Advance self.Q in place; returns (time, dt_last, R)."""
        R = np.zeros_like(self.Q)
        t = C.c_double(self.time)
        dt = C.c_double(0.0)
        self.lib.oracle_step(C.byref(self.p), nsteps, self.Q.ctypes.data_as(PD), C.byref(t), C.byref(dt),
                             R.ctypes.data_as(PD), self.DT.ctypes.data_as(PD), self.DTVisc.ctypes.data_as(PD))
        self.time = t.value
        return t.value, dt.value, R


    def shock_indicator(self, q, kappa):
        """ModeAliasShockFinder.ShockIndicator on one element's density values."""
        q = np.ascontiguousarray(q, dtype=np.float64)
        return self.lib.oracle_shock_indicator(C.byref(self.p), q.ctypes.data_as(PD),
                                               self._keep["Clip"].ctypes.data_as(PD), float(kappa))

    def vertex_max(self, elem):
        """Maximum of an element scalar over the elements at each vertex."""
        elem = np.ascontiguousarray(elem, dtype=np.float64)
        out = np.zeros(self.p.nverts)
        self.lib.oracle_vertex_max(C.byref(self.p), elem.ctypes.data_as(PD), out.ctypes.data_as(PD))
        return out

    def gradient(self, Q):
        """(d/dx, d/dy) of each variable at the NpFlux flux points, 4 x NpFlux x K each."""
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        gx = np.zeros((4, self.el.NpFlux, self.K))
        gy = np.zeros_like(gx)
        self.lib.oracle_gradient(C.byref(self.p), Q.ctypes.data_as(PD), gx.ctypes.data_as(PD),
                                 gy.ctypes.data_as(PD))
        return gx, gy

    def sensor(self, Q):
        """(Se, sigma, eps, sigma vertex-averaged, eps at vertices) for state Q."""
        Q = np.ascontiguousarray(Q, dtype=np.float64)
        out = [np.zeros(self.K) for _ in range(4)] + [np.zeros(self.p.nverts)]
        self.lib.oracle_sensor(C.byref(self.p), Q.ctypes.data_as(PD), *[o.ctypes.data_as(PD) for o in out])
        return out


def shock_conditions(M1, alpha=0.0, gamma=1.4):
    """ShockConditions (DG2D/test_functions2.go:184-240): pre/post normal-shock states."""
    a = alpha * math.pi / 180.0
    rho1, p1, u1, v1 = 1.0, 1.0, M1, 0.0
    u1n = u1 * math.cos(a) + v1 * math.sin(a)
    u1t = -u1 * math.sin(a) + v1 * math.cos(a)
    M1n = u1n / math.sqrt(gamma * p1 / rho1)
    En1 = p1 / (gamma - 1) + 0.5 * rho1 * (u1 * u1 + v1 * v1)
    U1 = [rho1, rho1 * u1, rho1 * v1, En1]
    if M1n < 1.0:
        return U1, list(U1)
    rr = ((gamma + 1) * M1n * M1n) / ((gamma - 1) * M1n * M1n + 2)
    pr = 1 + (2 * gamma / (gamma + 1)) * (M1n * M1n - 1)
    u2n = u1n * ((gamma - 1) * M1n * M1n + 2) / ((gamma + 1) * M1n * M1n)
    rho2, p2, u2t = rho1 * rr, p1 * pr, u1t
    u2 = u2n * math.cos(a) - u2t * math.sin(a)
    v2 = u2n * math.sin(a) + u2t * math.cos(a)
    En2 = p2 / (gamma - 1) + 0.5 * rho2 * (u2 * u2 + v2 * v2)
    return U1, [rho2, rho2 * u2, rho2 * v2, En2]


def ivortex_state(vortex, t, x, y):
    """IVortex.GetStateC (isentropic_vortex/analytic_vortex.go:31-82), vectorised."""
    beta, x0, y0, gamma = vortex
    x = np.asarray(x)
    y = np.asarray(y)
    if not (np.iscomplexobj(x) or np.iscomplexobj(y)):
        x, y = x.astype(np.float64), y.astype(np.float64)
    GM1 = gamma - 1.0
    fac = 16 * gamma * math.pi ** 2
    u = np.ones_like(x)
    v = np.zeros_like(x)
    xmut, ymvt = x - u * t, y - v * t
    r2 = (xmut - x0) ** 2 + (ymvt - y0) ** 2
    ex1r = np.exp(1 - r2)
    tv1 = 1.0 - (GM1 * beta * beta * np.exp(2.0 * (1.0 - r2)) / fac)
    u = u - beta * ex1r * (ymvt - y0) * (0.5 / math.pi)
    v = v + beta * ex1r * (xmut - x0) * (0.5 / math.pi)
    rho = tv1 ** (1.0 / GM1)
    p = rho ** gamma
    return np.stack([rho, rho * u, rho * v, p / GM1 + 0.5 * rho * (u * u + v * v)])
