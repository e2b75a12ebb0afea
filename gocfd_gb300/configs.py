"""The five validation / benchmark configurations of the Euler2D DFR path, with
a runner that reports each one's errors against its exact solution.

    vortex20      isentropic vortex, [-5,5]^2, 20x20 quads (800 triangles), N=2, 100 steps
    vortex256     the same on 256x256 quads (131,072 triangles), +-10% node jitter, N=4, 1000 steps
    sod2000x100   Sod shock tube, [0,1]x[0,0.05], 2000x100 quads (400,000 triangles), N=3,
                  PerssonC0 (Kappa 5), to t = 0.2, density against the exact solution
    wedge512x256  Mach 2 over a 15 degree ramp, [0,3]x[0,1], 512x256 quads (262,144 triangles), N=2,
                  local time stepping, PerssonC0 (Kappa 6), steady march, ramp pressure force
    vortex1024    the vortex on 1024x1024 quads (2,097,152 triangles), N=4, 1000 steps

Physics, BCs and inputs follow the reference's runs (InitializeSolution,
euler.go:728-794; test_cases/Euler2D/shock-tube/input-wall.yaml: CFL 5, Roe,
PerssonC0, Kappa 5; test_cases/Euler2D/Wedge/input.yaml: CFL 1, Roe, Minf 2,
local time stepping, PerssonC0, Kappa 6, 15000 iterations): vortex boundaries are Wall-tagged and
become IVortex (exact state through the characteristic BC); the vortex is
centred at (0, 0) inside the box.  Meshes are generated (gocfd_gb300.meshes);
the jitter stream is numpy's PCG64 with the stated seed.

Run one:  python -m gocfd_gb300.configs --config sod2000x100 [--precision fp64] [--scale 0.25]
(--scale shrinks the quad counts for a quick look.)  The vortex1024 adjoint
(1000 mixed-precision steps, then the field-error adjoint through 200 FP64
steps with a checkpoint every 10):
          python -m gocfd_gb300.configs --config vortex1024 --warm-steps 1000 --adjoint-steps 200
The wedge's ramp-force sensitivity to Minf and the flow angle through 500 steps:
          python -m gocfd_gb300.configs --config wedge512x256 --adjoint-steps 500 --fd-h 1e-6
"""
import argparse
import json
import math
import time
from dataclasses import dataclass, field

import numpy as np

from . import _lib, meshes
from .euler2d import Euler, InputParameters2D


@dataclass
class Config:
    name: str
    desc: str
    mesh: str                      # vortex | sod | wedge
    nx: int
    ny: int
    N: int
    init: str
    jitter: float = 0.0
    seed: int = 0
    cfl: float = 1.0
    flux: str = "roe"
    steps: int = 0                 # fixed step count (vortex)
    final_time: float = 1e9
    limiter: str = ""
    kappa: float = 0.0
    minf: float = 0.1
    local_dt: bool = False
    residual_tol: float = 0.0      # steady march stop: rms(R)/rms(Q) per variable
    max_steps: int = 0
    extra: dict = field(default_factory=dict)


CONFIGS = {
    "vortex20": Config("vortex20", "isentropic vortex [-5,5]^2, 20x20 quads -> 800 tris, N=2", "vortex", 20, 20, 2,
                       "ivortex", steps=100),
    "vortex256": Config("vortex256", "isentropic vortex [-5,5]^2, 256x256 quads -> 131072 tris, jitter 0.1h seed 0, N=4",
                        "vortex", 256, 256, 4, "ivortex", jitter=0.1, steps=1000),
    "sod2000x100": Config("sod2000x100", "Sod shock tube [0,1]x[0,0.05], 2000x100 quads -> 400000 tris, N=3, PerssonC0",
                          "sod", 2000, 100, 3, "shocktube", cfl=5.0, final_time=0.2, limiter="PerssonC0",
                          kappa=5.0),
    "wedge512x256": Config("wedge512x256", "Mach 2 wedge 15 deg, [0,3]x[0,1], 512x256 quads -> 262144 tris, N=2, "
                           "local dt, PerssonC0", "wedge", 512, 256, 2, "freestream", cfl=1.0, limiter="PerssonC0",
                           kappa=6.0, minf=2.0, local_dt=True, residual_tol=1e-10, max_steps=15000),
    "vortex1024": Config("vortex1024", "isentropic vortex [-5,5]^2, 1024x1024 quads -> 2097152 tris, jitter 0.1h "
                         "seed 0, N=4", "vortex", 1024, 1024, 4, "ivortex", jitter=0.1, steps=1000),
}


def build_mesh(cfg: Config, scale: float = 1.0):
    nx, ny = max(2, int(round(cfg.nx * scale))), max(2, int(round(cfg.ny * scale)))
    if cfg.mesh == "vortex":
        return meshes.vortex_box(nx, jitter=cfg.jitter, seed=cfg.seed)
    if cfg.mesh == "sod":
        return meshes.sod_channel(nx, ny)
    if cfg.mesh == "wedge":
        return meshes.wedge_channel(nx, ny)
    raise ValueError(cfg.mesh)


def input_params(cfg: Config) -> InputParameters2D:
    return InputParameters2D(CFL=cfg.cfl, FluxType=cfg.flux, InitType=cfg.init, PolynomialOrder=cfg.N,
                             FinalTime=cfg.final_time, Minf=cfg.minf, Gamma=1.4, Alpha=0.0,
                             LocalTimeStepping=cfg.local_dt, MaxIterations=10 ** 9, Limiter=cfg.limiter,
                             Kappa=cfg.kappa)


def solution_points_xy(solver: Euler):
    """Physical coordinates of the solution points, Np x K each."""
    rs = _lib.host_operator(solver.ip.PolynomialOrder, 4)
    v = solver.mesh.EToV
    VX, VY = solver.mesh.VX, solver.mesh.VY
    r, s = rs[:, 0:1], rs[:, 1:2]
    X = 0.5 * (-(r + s) * VX[v[:, 0]][None] + (r + 1) * VX[v[:, 1]][None] + (s + 1) * VX[v[:, 2]][None])
    Y = 0.5 * (-(r + s) * VY[v[:, 0]][None] + (r + 1) * VY[v[:, 1]][None] + (s + 1) * VY[v[:, 2]][None])
    return X, Y


def exact_vortex(X, Y, t, vortex=(5.0, 0.0, 0.0, 1.4)):
    """IVortex.GetStateC (isentropic_vortex/analytic_vortex.go:31-82) at (X, Y), 4 x shape."""
    beta, x0, y0, gamma = vortex
    GM1 = gamma - 1.0
    xm, ym = X - t, Y
    r2 = (xm - x0) ** 2 + (ym - y0) ** 2
    ex1r = np.exp(1 - r2)
    u = 1.0 - beta * ex1r * (ym - y0) / (2 * math.pi)
    v = beta * ex1r * (xm - x0) / (2 * math.pi)
    rho = (1.0 - GM1 * beta * beta * np.exp(2 * (1 - r2)) / (16 * gamma * math.pi ** 2)) ** (1 / GM1)
    p = rho ** gamma
    return np.stack([rho, rho * u, rho * v, p / GM1 + 0.5 * rho * (u * u + v * v)])


def exact_vortex_error(solver: Euler, t: float):
    """(relative L2, relative Linf) over all solution points and variables."""
    X, Y = solution_points_xy(solver)
    ex = exact_vortex(X, Y, t)
    d = solver.get_global_state() - ex
    return float(np.linalg.norm(d) / np.linalg.norm(ex)), float(np.abs(d).max() / np.abs(ex).max())


def sod_density_error(solver: Euler, t: float):
    """Density at every solution point against the exact Sod solution at its x:
    (L1 mean, L2 rms, Linf), and the same over points at least 0.02 from the waves."""
    from .sod import SodExact
    sod = SodExact(t)
    X, _ = solution_points_xy(solver)
    rho = solver.get_global_state()[0]
    ex = sod.density(X)
    d = np.abs(rho - ex)
    waves = np.array([sod.x1, sod.x2, sod.x3, sod.x4])
    far = np.min(np.abs(X[..., None] - waves), axis=-1) > 0.02
    return {"l1": float(d.mean()), "l2": float(np.sqrt((d ** 2).mean())), "linf": float(d.max()),
            "l1_smooth": float(d[far].mean()), "linf_smooth": float(d[far].max()),
            "shock_x_exact": sod.x4}


def run(name: str, precision: str = "fp64", scale: float = 1.0, device: int = 0, max_steps: int = 0,
        report_every: int = 0, stage_pipeline: bool = False):
    cfg = CONFIGS[name]
    mesh = build_mesh(cfg, scale)
    ip = input_params(cfg)
    center = (0.0, 0.0) if cfg.mesh == "vortex" else (5.0, 0.0)
    out = {"config": name, "desc": cfg.desc, "scale": scale, "precision": precision}
    with Euler(ip, mesh, 1, precision=precision, device=device, vortex_center=center) as s:
        if stage_pipeline:
            s.set_stage_pipeline(True)
            out["stage_pipeline"] = s.stage_pipeline()
        out["K"] = s.K
        t0 = time.perf_counter()
        if cfg.mesh == "vortex":
            n = min(cfg.steps, max_steps) if max_steps else cfg.steps
            info = s.step(n)
            out.update(steps=n, time=info["time"])
            out["rel_l2_vs_exact"], out["rel_linf_vs_exact"] = exact_vortex_error(s, info["time"])
        elif cfg.mesh == "sod":
            steps, t = 0, 0.0
            cap = max_steps or 10 ** 7
            while t < cfg.final_time * (1 - 1e-12) and steps < cap:
                n = min(100, cap - steps)
                info = s.step(n)
                steps += n
                t = info["time"]
            out.update(steps=steps, time=t)
            out["density_error"] = sod_density_error(s, t)
        else:  # steady march
            steps, hist = 0, []
            # per-variable RMS of the state, floored so that a variable that is zero
            # in the initial state (v-momentum at zero incidence) is measured on the others' scale
            qn = np.sqrt(np.mean(s.get_global_state() ** 2, axis=(1, 2)))
            qn = np.maximum(qn, 1e-3 * qn.max())
            cap = max_steps or cfg.max_steps
            rel = np.inf
            while steps < cap:
                info = s.step(50)
                steps += 50
                rel = float(np.max(np.array(info["resid_rms"]) / qn))
                if report_every and steps % report_every == 0:
                    # absolute increment RMS per variable, and relative to the current state's RMS
                    qc = np.sqrt(np.mean(s.get_global_state() ** 2, axis=(1, 2)))
                    hist.append({"step": steps, "rel_initial_floored": rel,
                                 "abs_rms": [float(v) for v in info["resid_rms"]],
                                 "rel_current": [float(v) for v in np.array(info["resid_rms"]) / qc]})
                if rel < cfg.residual_tol:
                    break
            out.update(steps=steps, residual_rel_rms=rel, converged=bool(rel < cfg.residual_tol), history=hist)
            out["ramp_force_x"], _, _ = s.functional("wall_force_x")
            out["ramp_force_y"], _, _ = s.functional("wall_force_y")
        out["seconds"] = time.perf_counter() - t0
    return out


def adjoint(name: str, steps: int, every: int, warm_steps: int = 0, warm_precision: str = "fp32",
            fd_h: float = 1e-8, device: int = 0, seed: int = 0, adjoint_precision: str = "fp64"):
    """The field-error adjoint of a vortex configuration: advance warm_steps in
    warm_precision, then record `steps` FP64 steps with a checkpoint every
    `every` steps, take J = sum (Q - Q_exact(t))^2 at the end and run the
    adjoint back to the window's start.  The gradient is checked along one
    random direction against central differences of the FP64 forward
    (the GPU FP64 path, which tracks the oracle to 1e-10).  adjoint_precision
    "fp32" / "tf32x3" records and reverses the window on the mixed path instead
    (its own J; no difference check)."""
    cfg = CONFIGS[name]
    assert cfg.mesh == "vortex"
    mesh = build_mesh(cfg)
    ip = input_params(cfg)
    out = {"config": name, "warm_steps": warm_steps, "warm_precision": warm_precision, "adjoint_steps": steps,
           "checkpoint_every": every}
    with Euler(ip, mesh, 1, precision="fp64", device=device, vortex_center=(0.0, 0.0)) as s:
        if warm_steps:
            with Euler(ip, mesh, 1, precision=warm_precision, device=device, vortex_center=(0.0, 0.0)) as w:
                info = w.step(warm_steps)
                s.set_global_state(w.get_global_state())
                s.time = info["time"]
        Q0, t0 = s.get_global_state(), s.time
        g = s
        if adjoint_precision != "fp64":
            g = Euler(ip, mesh, 1, precision=adjoint_precision, device=device, vortex_center=(0.0, 0.0))
            g.set_global_state(Q0)
            g.time = t0
        out["adjoint_precision"] = adjoint_precision
        t1 = time.perf_counter()
        g.record(steps, every)
        t2 = time.perf_counter()
        J, Qbf, tbf = g.functional("vortex_error")
        t3 = time.perf_counter()
        Qb0, qinfb, tb0 = g.step_vjp(Qbf, tbf)
        t4 = time.perf_counter()
        out.update(J=J, grad_norm=float(np.linalg.norm(Qb0)), time_bar0=tb0,
                   record_s=t2 - t1, vjp_s=t4 - t3, vjp_over_record=(t4 - t3) / (t2 - t1))
        if g is not s:
            g.close()
        if fd_h > 0 and g is s:
            rng = np.random.default_rng(seed)
            d = rng.standard_normal(Q0.shape) * np.abs(Q0)

            def Jat(q):
                s.set_global_state(q)
                s.time = t0
                s.step(steps)
                return s.functional("vortex_error")[0]
            ad = float(np.sum(Qb0 * d))
            out.update(directional_adjoint=ad, fd={})
            # d has norm ~ sqrt(#DOF) |Q|: the step h must keep h |d| small against the
            # error the functional measures, or the cubic term of the central
            # difference dominates; two steps show the convergence.
            for h in (fd_h, fd_h / 10):
                fd = (Jat(Q0 + h * d) - Jat(Q0 - h * d)) / (2 * h)
                out["fd"][f"{h:g}"] = {"directional_fd": fd, "rel_diff": abs(ad - fd) / max(abs(fd), 1e-300)}
    return out


def exact_vortex_param_derivative(X, Y, t, param: str, vortex=(5.0, 0.0, 0.0, 1.4), eps: float = 1e-3):
    """d Q_exact / d param at (X, Y, t) for param in {"x0", "beta"}: the state's
    change when the vortex centre moves along x, or when its strength changes
    (IVortex.GetStateC, isentropic_vortex/analytic_vortex.go:31-82).  Fourth-order
    central differences of the analytic state (truncation ~ eps^4 times the
    fifth derivative, ~1e-12 here)."""
    beta, x0, y0, gamma = vortex
    idx = {"beta": 0, "x0": 1}[param]

    def at(dv):
        v = [beta, x0, y0, gamma]
        v[idx] += dv
        return exact_vortex(X, Y, t, tuple(v))
    return (8.0 * (at(eps) - at(-eps)) - (at(2 * eps) - at(-2 * eps))) / (12.0 * eps)


def adjoint_smooth(name: str, steps: int, every: int, warm_steps: int = 0, warm_precision: str = "fp32",
                   params=("x0", "beta"), hs=(2e-4, 1e-4, 5e-5, 2.5e-5), device: int = 0,
                   adjoint_precision: str = "fp64"):
    """The field-error adjoint of a vortex configuration checked along smooth
    one-parameter directions of the window's initial state: d = dQ/d(param) of
    the exact vortex at the window's start (a shift of the vortex centre, or a
    change of its strength), against FP64 central differences
    (J(Q0 + h d) - J(Q0 - h d)) / 2h over a sweep of h and their Richardson
    extrapolation (4 FD(h/2) - FD(h)) / 3, which removes the h^2 term.

    The time step is CFL / max wave speed over all edge points, a max over
    about 10^7 candidates per stage; where the +h and -h trajectories pick a
    different maximiser the map has a kink.  Each run records its per-step dt,
    and dt_fd(h) = (dt+ - dt-) / 2h is compared with dt_fd(h/2): a step where
    they disagree by more than 1% straddles such a switch.  These counts go
    into the output beside the gradients.

    adjoint_precision "fp32" (or "tf32x3") takes the gradient from the mixed
    path's FP32 adjoint instead, over its own recorded window, with the FP64
    path's field-error weight dJ/dQ_final: the differences stay FP64, and both
    sides then differentiate the same weighted sum.  (The mixed path's own
    weight 2 (Q_final - Q_exact) is not the FP64 one: after 1000+ steps the
    discretisation error is ~3e-7 per value and the mixed path's rounding
    differs from the FP64 path's by a tenth of that.)"""
    cfg = CONFIGS[name]
    assert cfg.mesh == "vortex"
    mesh = build_mesh(cfg)
    ip = input_params(cfg)
    out = {"config": name, "warm_steps": warm_steps, "warm_precision": warm_precision, "adjoint_steps": steps,
           "checkpoint_every": every, "hs": list(hs)}
    with Euler(ip, mesh, 1, precision="fp64", device=device, vortex_center=(0.0, 0.0)) as s:
        if warm_steps:
            with Euler(ip, mesh, 1, precision=warm_precision, device=device, vortex_center=(0.0, 0.0)) as w:
                info = w.step(warm_steps)
                s.set_global_state(w.get_global_state())
                s.time = info["time"]
        Q0, t0 = s.get_global_state(), s.time
        out["K"], out["t0"] = s.K, t0
        out["adjoint_precision"] = adjoint_precision
        if adjoint_precision == "fp64":
            t1 = time.perf_counter()
            s.record(steps, every)
            t2 = time.perf_counter()
            J, Qbf, tbf = s.functional("vortex_error")
            Qb0, _, _ = s.step_vjp(Qbf, tbf)
            t3 = time.perf_counter()
        else:
            s.step(steps)
            J, Qbf, tbf = s.functional("vortex_error")
            with Euler(ip, mesh, 1, precision=adjoint_precision, device=device, vortex_center=(0.0, 0.0)) as g:
                g.set_global_state(Q0)
                g.time = t0
                t1 = time.perf_counter()
                g.record(steps, every)
                t2 = time.perf_counter()
                out["J_adjoint_path"] = g.functional("vortex_error")[0]
                Qb0, _, _ = g.step_vjp(Qbf, tbf)
                t3 = time.perf_counter()
        out.update(J=J, record_s=t2 - t1, vjp_s=t3 - t2)
        X, Y = solution_points_xy(s)

        def run_at(q):
            s.set_global_state(q)
            s.time = t0
            dts = np.empty(steps)
            for n in range(steps):
                dts[n] = s.step(1)["dt"]
            return s.functional("vortex_error")[0], dts
        for param in params:
            d = exact_vortex_param_derivative(X, Y, t0, param)
            ad = float(np.sum(Qb0 * d))
            res = {"directional_adjoint": ad, "fd": {}, "richardson": {}, "dt_switch_steps": {}}
            fds, dtfd = {}, {}
            for h in hs:
                jp, dp = run_at(Q0 + h * d)
                jm, dm = run_at(Q0 - h * d)
                fds[h] = (jp - jm) / (2 * h)
                dtfd[h] = (dp - dm) / (2 * h)
                res["fd"][f"{h:g}"] = {"directional_fd": fds[h], "rel_diff": abs(ad - fds[h]) / abs(fds[h])}
            for h in hs:
                if h / 2 in fds:
                    r = (4 * fds[h / 2] - fds[h]) / 3
                    res["richardson"][f"{h:g}"] = {"value": r, "rel_diff": abs(ad - r) / abs(r)}
                    floor = 1e-3 * np.abs(dtfd[h / 2]).max()
                    bad = np.abs(dtfd[h] - dtfd[h / 2]) > 1e-2 * np.maximum(np.abs(dtfd[h / 2]), floor)
                    res["dt_switch_steps"][f"{h:g}"] = int(bad.sum())
            out[param] = res
    return out


def wedge_sensitivity(steps: int = 500, every: int = 10, scale: float = 1.0, fd_h: float = 1e-6, device: int = 0):
    """Ramp pressure force after `steps` local-dt steps from the freestream state,
    and its derivatives with respect to the inflow Mach number and the flow
    angle by the adjoint (recorded window, checkpoint every `every` steps),
    against central differences of the FP64 forward at Minf +- h, alpha +- h.
    The freestream enters both the far-field BC (Qinf adjoint) and the initial
    state (its adjoint summed over the mesh): dQinf/dM = (0, cos a, sin a, M),
    dQinf/da = (0, -M sin a, M cos a, 0) per radian (NewFreeStream, fluids.go:245-262)."""
    cfg = CONFIGS["wedge512x256"]
    mesh = build_mesh(cfg, scale)

    def solver(minf, alpha_deg):
        ip = input_params(cfg)
        ip.Minf, ip.Alpha = minf, alpha_deg
        return Euler(ip, mesh, 1, precision="fp64", device=device)

    M, A = cfg.minf, 0.0
    out = {"config": "wedge512x256", "scale": scale, "steps": steps, "checkpoint_every": every}
    with solver(M, A) as s:
        out["K"] = s.K
        t0 = time.perf_counter()
        s.record(steps, every)
        t1 = time.perf_counter()
        J, Qbf, _ = s.functional("wall_force_x")
        Qb0, qinfb, _ = s.step_vjp(Qbf)
        t2 = time.perf_counter()
    a = math.radians(A)
    dq_dM = np.array([0.0, math.cos(a), math.sin(a), M])
    dq_da = np.array([0.0, -M * math.sin(a), M * math.cos(a), 0.0]) * (math.pi / 180.0)  # per degree
    ic = Qb0.sum(axis=(1, 2))  # the initial state is Qinf at every point
    out.update(J=J, dJ_dMinf=float(qinfb @ dq_dM + ic @ dq_dM), dJ_dalpha_deg=float(qinfb @ dq_da + ic @ dq_da),
               record_s=t1 - t0, vjp_s=t2 - t1)

    def J_at(minf, alpha_deg):
        with solver(minf, alpha_deg) as s2:
            s2.step(steps)
            return s2.functional("wall_force_x")[0]
    if fd_h > 0:
        out["fd_dJ_dMinf"] = (J_at(M + fd_h, A) - J_at(M - fd_h, A)) / (2 * fd_h)
        out["fd_dJ_dalpha_deg"] = (J_at(M, A + fd_h) - J_at(M, A - fd_h)) / (2 * fd_h)
        out["rel_diff_Minf"] = abs(out["dJ_dMinf"] - out["fd_dJ_dMinf"]) / abs(out["fd_dJ_dMinf"])
        out["rel_diff_alpha"] = abs(out["dJ_dalpha_deg"] - out["fd_dJ_dalpha_deg"]) / abs(out["fd_dJ_dalpha_deg"])
    return out


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    p.add_argument("--config", choices=sorted(CONFIGS), required=True)
    p.add_argument("--precision", choices=["fp64", "fp32", "tf32x3"], default="fp64")
    p.add_argument("--scale", type=float, default=1.0)
    p.add_argument("--max-steps", type=int, default=0)
    p.add_argument("--report-every", type=int, default=0)
    p.add_argument("--stage-pipeline", action="store_true",
                   help="mixed path: the persistent TMA-pipelined stage kernel instead of the one-block kernel")
    p.add_argument("--adjoint-steps", type=int, default=0,
                   help="vortex configs: run the field-error adjoint through this many steps instead")
    p.add_argument("--checkpoint-every", type=int, default=10)
    p.add_argument("--warm-steps", type=int, default=0)
    p.add_argument("--fd-h", type=float, default=1e-8, help="central-difference step of the adjoint check (0: skip)")
    p.add_argument("--smooth", action="store_true",
                   help="vortex adjoint: check along the smooth directions d/dx0 and d/dbeta of the exact vortex "
                        "with an h sweep and Richardson extrapolation instead of a random direction")
    p.add_argument("--adjoint-precision", choices=["fp64", "fp32", "tf32x3"], default="fp64",
                   help="vortex adjoint: the path whose adjoint runs the window (fp32: the mixed path)")
    a = p.parse_args(argv)
    if a.adjoint_steps and a.config.startswith("wedge"):
        res = wedge_sensitivity(a.adjoint_steps, a.checkpoint_every, a.scale, fd_h=a.fd_h)
    elif a.adjoint_steps and a.smooth:
        res = adjoint_smooth(a.config, a.adjoint_steps, a.checkpoint_every, a.warm_steps,
                             a.precision if a.precision != "fp64" else "fp32",
                             adjoint_precision=a.adjoint_precision)
    elif a.adjoint_steps:
        res = adjoint(a.config, a.adjoint_steps, a.checkpoint_every, a.warm_steps,
                      a.precision if a.precision != "fp64" else "fp32", fd_h=a.fd_h,
                      adjoint_precision=a.adjoint_precision)
    else:
        res = run(a.config, a.precision, a.scale, max_steps=a.max_steps, report_every=a.report_every,
                  stage_pipeline=a.stage_pipeline)
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
