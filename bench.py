#!/usr/bin/env python3
"""Benchmark: RK-stage DOF-updates/s of the 2D Euler DFR right-hand side +
SSP(5,4) step on GB300, against the CPU restatement timed on the host cores.

One "step" is one 5-stage SSP-RK step over the whole mesh.  DOF-updates per
step = K * Np * 4 * 5.  Default workload: isentropic vortex on [-5,5]^2,
1024 x 1024 quads split into 2,097,152 triangles with +-10% h interior jitter
(seed 0), N = 4 (Np = 15), Roe flux, CFL 1, far-field exact-state BCs
(--workload vortex256: 256 x 256 quads, 131,072 triangles).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) each rank runs an independent replica on its own GPU
(the path has no exchange step on one-GPU deployments), the timed region is
bracketed by barriers and the max over ranks is reported; value is the
whole-job aggregate.  Prints ONE JSON line on rank 0.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RK-stage DOF-updates/s: FP64 plain vs mixed form at equal L2 err; adjoint/fwd"
UNIT = "DOF-updates/s"

WORKLOADS = {
    "vortex256": dict(n=256, N=4, jitter=0.1, seed=0,
                      desc="isentropic vortex [-5,5]^2, 256x256 quads -> 131072 tris, jitter 0.1h seed 0, N=4"),
    "vortex1024": dict(n=1024, N=4, jitter=0.1, seed=0,
                       desc="isentropic vortex [-5,5]^2, 1024x1024 quads -> 2097152 tris, jitter 0.1h seed 0, N=4"),
    "vortex20": dict(n=20, N=2, jitter=0.0, seed=0,
                     desc="isentropic vortex [-5,5]^2, 20x20 quads -> 800 tris, N=2"),
}


def args_parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--precision", choices=["fp32", "tf32x3", "fp64"], default="fp32")
    p.add_argument("--workload", choices=sorted(WORKLOADS), default="vortex1024")
    p.add_argument("--fp64-steps", type=int, default=100)
    p.add_argument("--adj-steps", type=int, default=20, help="steps of the adjoint timings, FP64 and mixed (0: skip)")
    p.add_argument("--e2e-steps", type=int, default=50)
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--accuracy", type=int, default=0,
                   help="instead of timing: run this many steps in FP64 and FP32 and report the "
                        "relative L2 differences and the errors against the exact vortex")
    p.add_argument("--acc-steps", type=int, default=1000,
                   help="after the timed region: steps of the accuracy leg on vortex256 (0: skip)")
    p.add_argument("--acc-steps-large", type=int, default=100,
                   help="after the timed region: steps of the accuracy leg on the benchmarked workload (0: skip)")
    p.add_argument("--adj-acc-steps", type=int, default=200,
                   help="after the timed region: window of the adjoint gradient check on vortex256 (0: skip)")
    return p.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def make_mesh(wl):
    from gocfd_gb300 import meshes
    return meshes.vortex_box(wl["n"], jitter=wl["jitter"], seed=wl["seed"])


def workload_config(name, K, Np):
    """The workload description both arms print (the same dict, key for key)."""
    wl = WORKLOADS[name]
    return {"workload": name, "description": wl["desc"], "K": K, "N": wl["N"], "Np": Np,
            "dof_updates_per_step": K * Np * 4 * 5, "flux": "roe", "cfl": 1.0,
            "l2": "state of %.3g GB per FP64 copy against a 129 MB L2; the GPU arm also writes 256 MB "
                  "between timed steps" % (K * Np * 4 * 8 / 1e9)}


def input_params(N, final_time=1e9):
    from gocfd_gb300.euler2d import InputParameters2D
    return InputParameters2D(CFL=1.0, FluxType="roe", InitType="ivortex", PolynomialOrder=N,
                             FinalTime=final_time, MaxIterations=10 ** 9)


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.samples = []
        self.proc = None
        self.thread = None
        self.marks = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.monotonic(), line.strip()))

    def mark(self):
        self.marks.append(time.monotonic())

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0, t1):
        rows = [s for (t, s) in self.samples if t0 - 0.15 <= t <= t1 + 0.15]
        if not rows:
            rows = [s for (_, s) in self.samples]
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            f = [x.strip() for x in r.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for name, val in zip(names[1:], f[4:8]):
                if val.lower() in ("active", "1", "yes"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------- roofline
def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def algorithmic_bytes(family, K, nInt, nBC, Np, NE, precision):
    """Algorithmic DRAM bytes per launch of each kernel family, every array
    touched once.  FP64 path: state S8 = 4*Np*8 B per element, faces and edge
    DOFs per element F8 = 4*3*NpEdge*8 B.  Mixed path: FP32 stage increments
    S4 = 4*Np*4, edge-major faces/fluxes in FP32; the 5 stage launches are
    averaged (their traffic differs by stage)."""
    S8, S4 = 4 * Np * 8, 4 * Np * 4
    if precision == "fp64":
        F = 4 * 3 * NE * 8
        if family == 0:   # k_interp: read state, write faces
            return K * (S8 + F)
        if family == 1:   # k_edge_flux: both sides' faces in, both sides' DOFs out, edge data
            return nInt * (4 * (4 * NE * 8) + 60) + nBC * (2 * (4 * NE * 8) + 60 + 2 * NE * 8)
        if family == 2:   # k_div_update: 19 state passes over the 5 stages + FE + geometry
            return K * (19 * S8 + 5 * (F + 40)) / 5.0
        return 0.0
    F = 3 * 4 * NE * 4      # one element's faces (or fluxes) over its 3 edges
    G = 112                 # slots, IInII, Jacobian, reference state in/out
    if family == 0:         # k_mixed_prepare: Q0 in, dQ0 + faces + reference state out
        return K * (S8 + S4 + F + 32)
    if family == 1:         # interior edges: 2 sides' faces + 2 reference states in, fhat + corr + speed out
        per_int = 2 * 4 * NE * 4 + 64 + 20 + 4 * NE * 4 + 16 + 8
        per_bc = 4 * NE * 4 + 32 + 20 + 2 * NE * 8 + 4 * NE * 4 + 8
        return nInt * per_int + nBC * per_bc
    if family == 2:         # k_mixed_stage over the 5 stages: 18 S4 + 2 S8 + 10 F + 5 (G + corr)
        return K * (18 * S4 + 2 * S8 + 10 * F + 5 * (G + 48)) / 5.0
    return 0.0


def ncu_traffic_per_element(kernel, precision, N):
    """Per-element DRAM bytes of one launch, measured by ncu and recorded in
    profiles/*.md as 'traffic_bytes_per_element <kernel> <precision> N=<N>: <v>'."""
    pat = re.compile(rf"traffic_bytes_per_element\s+{kernel}\s+{precision}\s+N={N}:\s*([0-9.eE+]+)")
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    for name in sorted(os.listdir(d)):
        if not name.endswith((".md", ".txt")):
            continue
        with open(os.path.join(d, name)) as f:
            m = pat.search(f.read())
        if m:
            return float(m.group(1))
    return None


# --------------------------------------------------------------------------- CPU oracle
def cpu_baseline(wl, mesh, seconds, steps=None, warmup=0, max_steps=200):
    """The oracle (C++ FP64, OpenMP on all host cores) on the same workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    ora = oracle.OracleSolver(wl["N"], mesh.VX, mesh.VY, mesh.EToV, mesh.bc_edges, flux="roe",
                              init="ivortex", cfl=1.0, vortex_center=(0.0, 0.0))
    threads = ora.lib.oracle_num_threads()
    if warmup:
        ora.step(warmup)
    t0 = time.perf_counter()
    ora.step(1)
    t1 = time.perf_counter()
    done, el = 1, t1 - t0
    target = steps if steps is not None else max(1, min(max_steps, int(seconds / max(el, 1e-6))))
    while done < target:
        ora.step(1)
        done += 1
    el = time.perf_counter() - t0
    dof = ora.K * ora.el.Np * 4 * 5
    return dict(value=dof * done / el, unit=UNIT, cores=threads, kind="port", steps=done, seconds=el,
                K=ora.K, Np=ora.el.Np,
                sample=f"{done} full SSP-RK steps of the same {ora.K}-element N={wl['N']} workload")


# --------------------------------------------------------------------------- ranks
def max_over_ranks(x: float, world: int, device: str = "cpu") -> float:
    """The slowest rank's time: all-reduce(max) of x over the process group."""
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(world: int, units_per_rank: float, seconds: float) -> float:
    """Whole-job rate of independent replicas: every rank processed units_per_rank
    in at most `seconds` (the max over ranks)."""
    return world * units_per_rank / seconds


# --------------------------------------------------------------------------- GPU arm
def run_ours(a, world, rank, local):
    import torch
    import torch.distributed as dist
    from gocfd_gb300.euler2d import Euler
    from gocfd_gb300 import _lib

    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    wl = WORKLOADS[a.workload]
    mesh = make_mesh(wl)
    ip = input_params(wl["N"])
    solver = Euler(ip, mesh, 1, precision=a.precision, device=local, vortex_center=(0.0, 0.0))
    K, Np, NE = solver.K, solver.Np, solver.NpEdge
    dof_per_step = K * Np * 4 * 5
    stream = torch.cuda.ExternalStream(solver.stream_handle(), device=torch.device("cuda", local))
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")  # 256 MB > L2

    def barrier():
        if world > 1:
            dist.barrier()

    solver.enqueue_steps(a.warmup)
    torch.cuda.synchronize()
    solver.step(0)
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(a.steps)]
    t_wall0 = time.monotonic()
    with torch.cuda.stream(stream):
        for i, (s, e) in enumerate(evs):
            flush.fill_(float(i & 7))       # L2 flushed between timed steps (not timed)
            s.record(stream)
            solver.enqueue_steps(1)
            e.record(stream)
    torch.cuda.synchronize()
    t_wall1 = time.monotonic()
    barrier()
    ms = float(sum(s.elapsed_time(e) for s, e in evs))
    info = solver.step(0)  # raises on a non-finite state
    clocks.stop()  # samples cover the timed region; nvidia-smi's queries would perturb the host-API timings below
    clk = clocks.summary(t_wall0, t_wall1)
    ms = max_over_ranks(ms, world, f"cuda:{local}")
    value = aggregate_rate(world, dof_per_step * a.steps, ms / 1e3)
    nBC_mesh = 4 * wl["n"]
    launches_per_step = 2 + 5 * (3 if a.precision == "fp64" else (2 + (nBC_mesh > 0)))

    # Per-kernel attribution for the roofline (eager launches with events).
    fam_ms, fam_n = [0.0] * 4, [0] * 4
    for _ in range(5):
        m, n = solver.profile_step()
        fam_ms = [x + y for x, y in zip(fam_ms, m)]
        fam_n = [x + y for x, y in zip(fam_n, n)]
    if a.precision != "fp64":  # the preparation is not part of a graph step
        fam_ms[0], fam_n[0] = 0.0, 0
    if a.precision == "fp32":
        names = ["k_mixed_prepare", "k_mixed_edge", "k_mixed_stage", "k_step"]
    elif a.precision == "tf32x3":
        names = ["k_mixed_prepare", "k_mixed_edge", "k_mixed_stage_tc", "k_step"]
    else:
        names = ["k_interp", "k_edge_flux", "k_div_update", "k_step"]
    dom = max(range(3), key=lambda i: fam_ms[i])
    per_launch_ms = fam_ms[dom] / max(fam_n[dom], 1)
    nE = solver.nEdges
    nBC = 4 * WORKLOADS[a.workload]["n"]
    nInt = nE - nBC
    alg = algorithmic_bytes(dom, K, nInt, nBC, Np, NE, a.precision)
    peak, peak_kind = measured_peaks()
    achieved = alg / (per_launch_ms / 1e3) / 1e9
    tpe = ncu_traffic_per_element(names[dom], a.precision, wl["N"])
    roofline = {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": (tpe * K if tpe is not None else None),
                "algorithmic_bytes": alg, "peak_source": peak_kind,
                "avg_launch_us": per_launch_ms * 1e3,
                "kernel_share": {names[i]: fam_ms[i] / max(sum(fam_ms), 1e-12) for i in range(4)}}

    # The other mixed variant (FMA or tensor-core divergence) on the same workload.
    other = None
    if a.precision in ("fp32", "tf32x3") and a.fp64_steps > 0:
        oprec = "tf32x3" if a.precision == "fp32" else "fp32"
        so = Euler(ip, mesh, 1, precision=oprec, device=local, vortex_center=(0.0, 0.0))
        sto = torch.cuda.ExternalStream(so.stream_handle(), device=torch.device("cuda", local))
        so.enqueue_steps(3)
        torch.cuda.synchronize()
        evo = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(20)]
        with torch.cuda.stream(sto):
            for i, (s0, s1) in enumerate(evo):
                flush.fill_(float(i & 7))
                s0.record(sto)
                so.enqueue_steps(1)
                s1.record(sto)
        torch.cuda.synchronize()
        mso = float(sum(s0.elapsed_time(s1) for s0, s1 in evo)) / len(evo)
        so.step(0)
        other = {"precision": oprec, "value": world * dof_per_step / (mso / 1e3), "ms_per_step": mso,
                 "steps": len(evo)}
        so.close()

    # FP64 drop-in path on the same workload (device-timed, no flush).
    fp64 = None
    if a.precision != "fp64" and a.fp64_steps > 0:
        s64 = Euler(ip, mesh, 1, precision="fp64", device=local, vortex_center=(0.0, 0.0))
        st64 = torch.cuda.ExternalStream(s64.stream_handle(), device=torch.device("cuda", local))
        s64.enqueue_steps(2)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(st64):
            e0.record(st64)
            s64.enqueue_steps(a.fp64_steps)
            e1.record(st64)
        torch.cuda.synchronize()
        ms64 = e0.elapsed_time(e1)
        s64.step(0)
        fp64 = {"value": world * dof_per_step * a.fp64_steps / (ms64 / 1e3),
                "ms_per_step": ms64 / a.fp64_steps, "steps": a.fp64_steps}
        # Compute roofline of the FP64 path's dominant kernel (k_div_update: the
        # DivInt GEMM, 2 Np NpFlux flops per variable and element, on the FP64
        # FMA pipe) against the device's measured FP64 FMA rate.
        m64, n64 = [0.0] * 4, [0] * 4
        for _ in range(2):
            m, n = s64.profile_step()
            m64 = [x + y for x, y in zip(m64, m)]
            n64 = [x + y for x, y in zip(n64, n)]
        peak64 = _lib.device_fma_peaks(local)[0]
        NF = s64.NpFlux
        div_flops = K * 4.0 * (2.0 * Np * NF + Np)
        div_ms = m64[2] / max(n64[2], 1)
        ach = div_flops / (div_ms / 1e3) / 1e12
        fp64["roofline"] = {"bound": "fp64 fma", "kernel": "k_div_update", "achieved": ach, "peak": peak64,
                            "unit": "TFLOP/s", "frac": ach / peak64, "flops_per_launch": div_flops,
                            "avg_launch_us": div_ms * 1e3,
                            "peak_source": "measured (gcfd_device_fma_peaks: FP64 FMA chains on every SM)",
                            "kernel_share": {k: m64[i] / max(sum(m64), 1e-12)
                                             for i, k in enumerate(["k_interp", "k_edge_flux", "k_div_update",
                                                                    "k_step"])}}
        s64.close()

    # Adjoint cost: the reverse sweep of a recorded window against the forward
    # step of the same path (FP64, and the mixed path's FP32 adjoint).  With a
    # checkpoint every 10 steps (what the vortex1024 adjoint runs) each segment
    # is recomputed once with its per-step tape kept, then reversed; with a
    # checkpoint every step each reverse step recomputes its forward step once
    # with the tape.
    def adjoint_cost(precision):
        sa = Euler(ip, mesh, 1, precision=precision, device=local, vortex_center=(0.0, 0.0))
        sta = torch.cuda.ExternalStream(sa.stream_handle(), device=torch.device("cuda", local))
        sa.enqueue_steps(2)
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(sta):
            f0.record(sta)
            sa.enqueue_steps(a.adj_steps)
            f1.record(sta)
        torch.cuda.synchronize()
        fwd_ms = f0.elapsed_time(f1) / a.adj_steps
        # the adjoint in and out through the C ABI from pinned host shards (as the
        # e2e leg moves the state), so the window's fixed cost is two ~1 GB copies
        # at link speed rather than pageable copies and Python-side array work
        hin = [torch.ones((Np, K), dtype=torch.float64, pin_memory=True) for _ in range(4)]
        hout = [torch.empty((Np, K), dtype=torch.float64, pin_memory=True) for _ in range(4)]
        pin_in = (_lib.PD * 4)(*[h.numpy().ctypes.data_as(_lib.PD) for h in hin])
        pin_out = (_lib.PD * 4)(*[h.numpy().ctypes.data_as(_lib.PD) for h in hout])
        kmv = np.array([K], np.int32)
        qinf_b, t_b = (C.c_double * 4)(), C.c_double()

        def vjp():
            _lib.check(sa.lib, sa.ctx, sa.lib.gcfd_step_vjp(sa.ctx, 1, kmv.ctypes.data_as(_lib.PI), pin_in, 0.0,
                                                            pin_out, qinf_b, C.byref(t_b)))
        legs = {}
        # the window's fixed costs still vary by a few ms from call to call: the mixed
        # path's short reverse steps take the best of two calls per window length
        reps = 1 if precision == "fp64" else 2
        for every in (10, 1):
            sa.record(2 * every if every > 1 else 2, every)
            vjp()  # warm-up (allocations, first launches)

            def sweep(n):
                best = float("inf")
                for _ in range(reps):
                    sa.record(n, every)
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    vjp()
                    best = min(best, (time.perf_counter() - t0) * 1e3)
                return best
            # windows of two segments or more, so both are checkpointed (a window of one
            # segment is taped while recording: the third leg below)
            n1 = max(2 * every, a.adj_steps // 2)
            n2 = n1 + max(every, a.adj_steps)
            n1, n2 = every * ((n1 + every - 1) // every), every * ((n2 + every - 1) // every)
            t1, t2 = sweep(n1), sweep(n2)
            adj_ms = (t2 - t1) / (n2 - n1)  # per reverse step, without the window's fixed costs
            legs[every] = {"ms_per_step": adj_ms, "ratio": adj_ms / fwd_ms, "window_ms": {str(n1): t1, str(n2): t2}}
        if precision != "fp64":
            # the whole window taped while recording (checkpoint_every >= nsteps,
            # when a tape slot per step fits): the reverse sweep recomputes nothing;
            # the cost is the reverse plus the taping's extra over the plain forward.
            # On a fresh context: the checkpointed windows' blocks, held for reuse,
            # would otherwise be freed and re-allocated around the taped slots
            # (~160 GB here), which leaves the later slots' mappings fragmented.
            sa.close()
            sa = Euler(ip, mesh, 1, precision=precision, device=local, vortex_center=(0.0, 0.0))

            def taped(n, reps=1):
                r = v = float("inf")
                for _ in range(reps):
                    torch.cuda.synchronize()
                    t0 = time.perf_counter()
                    sa.record(n, n)
                    torch.cuda.synchronize()
                    t1 = time.perf_counter()
                    tapedOK.append(sa.window_taped())
                    vjp()
                    r, v = min(r, (t1 - t0) * 1e3), min(v, (time.perf_counter() - t1) * 1e3)
                return r, v
            tapedOK = []
            n1 = max(10, a.adj_steps // 2)
            n2 = n1 + max(10, a.adj_steps)
            # the first window of n2 steps allocates its tape slots (a window's device
            # blocks are kept for the next window); the timed windows reuse them
            r0, _ = taped(n2)
            (r1, v1), (r2, v2) = taped(n1, reps), taped(n2, reps)
            vjp_ms = (v2 - v1) / (n2 - n1)
            rec_extra = (r2 - r1) / (n2 - n1) - fwd_ms
            legs["taped"] = {"ms_per_step": vjp_ms, "record_extra_ms_per_step": rec_extra,
                             "ratio": (vjp_ms + max(rec_extra, 0.0)) / fwd_ms,
                             "window_ms": {str(n1): [r1, v1], str(n2): [r2, v2]},
                             "first_record_ms": {str(n2): r0},
                             "taped": all(tapedOK),
                             "note": "ratio = (reverse per step + taping's extra per recorded step) / forward; "
                                     "first_record_ms: the first window's recording, which allocates its tape"}
        sa.close()
        return {"ms_per_step": legs[10]["ms_per_step"], "forward_ms_per_step": fwd_ms,
                "ratio": legs[10]["ratio"], "checkpoint_every": 10, "path": precision,
                "window_ms": legs[10]["window_ms"], "checkpoint_every_1": legs[1],
                "window_taped": legs.get("taped"),
                "timing": "host clock around gcfd_step_vjp (synchronous; adjoint in and out as pinned host shards) for two window lengths; per-step cost = "
                          "difference / difference in steps (the adjoint's host transfer and set-up are per "
                          "window); forward by CUDA events"}

    adjoint = adjoint_cost("fp64") if a.adj_steps > 0 else None
    adjoint_mixed = adjoint_cost("fp32") if a.adj_steps > 0 else None
    if adjoint_mixed is not None:
        adjoint_mixed["vs_fp64_adjoint"] = adjoint["ms_per_step"] / adjoint_mixed["ms_per_step"]

    # End to end through the public API: pinned host state in, step, state out.
    import torch as _t
    host = [_t.empty((Np, K), dtype=_t.float64, pin_memory=True) for _ in range(4)]
    hostn = [h.numpy() for h in host]
    km = np.array([K], np.int32)
    ptrs = (_lib.PD * 4)(*[h.ctypes.data_as(_lib.PD) for h in hostn])
    lib = solver.lib
    _lib.check(lib, solver.ctx, lib.gcfd_get_state(solver.ctx, 1, km.ctypes.data_as(_lib.PI), ptrs))
    for _ in range(3):
        _lib.check(lib, solver.ctx, lib.gcfd_set_state(solver.ctx, 1, km.ctypes.data_as(_lib.PI), ptrs))
        _lib.check(lib, solver.ctx, lib.gcfd_step(solver.ctx, 1, None, None, None, None, None))
        _lib.check(lib, solver.ctx, lib.gcfd_get_state(solver.ctx, 1, km.ctypes.data_as(_lib.PI), ptrs))
    barrier()
    t0 = time.perf_counter()
    for _ in range(a.e2e_steps):
        _lib.check(lib, solver.ctx, lib.gcfd_set_state(solver.ctx, 1, km.ctypes.data_as(_lib.PI), ptrs))
        _lib.check(lib, solver.ctx, lib.gcfd_step(solver.ctx, 1, None, None, None, None, None))
        _lib.check(lib, solver.ctx, lib.gcfd_get_state(solver.ctx, 1, km.ctypes.data_as(_lib.PI), ptrs))
    e2e_s = time.perf_counter() - t0
    barrier()
    e2e_s = max_over_ranks(e2e_s, world, f"cuda:{local}")
    state_bytes = 4 * Np * K * 8
    e2e = {"value": aggregate_rate(world, dof_per_step * a.e2e_steps, e2e_s), "unit": UNIT,
           "h2d_bytes_per_step": state_bytes, "d2h_bytes_per_step": state_bytes,
           "steps": a.e2e_steps, "api": "gcfd_set_state + gcfd_step + gcfd_get_state, pinned host shards"}

    # Accuracy (the "at equal L2 error" half of the metric): the mixed paths
    # against the FP64 path and both against the exact vortex, after the timed region.
    accuracy = None
    if rank == 0 and a.precision != "fp64":
        solver.close()
        solver = None
        accuracy = {}
        if a.acc_steps > 0:
            accuracy["vortex256"] = accuracy_leg("vortex256", a.acc_steps, local, ("fp64", "fp32", "tf32x3"))
        if a.acc_steps_large > 0 and a.workload != "vortex256":
            accuracy[a.workload] = accuracy_leg(a.workload, a.acc_steps_large, local, ("fp64", a.precision))
        if a.adj_acc_steps > 0:
            accuracy["adjoint_vortex256"] = adjoint_accuracy_leg("vortex256", a.adj_acc_steps, local)
        m = accuracy.get("vortex256") or accuracy.get(a.workload)
        if m:
            accuracy["mixed_vs_fp64_rel_l2"] = m.get(f"{a.precision}_vs_fp64_rel_l2")
            accuracy["mixed_vs_fp64_rel_linf"] = m.get(f"{a.precision}_vs_fp64_rel_linf")
            accuracy["mixed_vs_fp64_steps"] = m["steps"]
            accuracy["mixed_vs_fp64_workload"] = m["workload"]

    cpu = None
    if rank == 0 and world == 1 and not a.no_cpu:
        cpu = cpu_baseline(wl, mesh, a.cpu_seconds)
    if solver is not None:
        solver.close()
    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": {"fp64": "fp64", "fp32": "fp32 (compensated fp32 state)",
                                                  "tf32x3": "3xtf32 tensor-core GEMM, fp32 elsewhere (compensated fp32 state)"}[a.precision],
            "data": "synthetic (analytic isentropic-vortex initial condition on a generated mesh)",
            "config": workload_config(a.workload, K, Np),
            "parallelism": f"replicas x{world}",
            "timing": "CUDA events per graph-launched step on the solver stream",
            "accuracy": accuracy,
            "e2e": e2e,
            "gpu_launches": launches_per_step * a.steps,
            "clocks": clk,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "fp64_path": fp64,
            "other_mixed_path": other,
            "adjoint": adjoint,
            "adjoint_mixed": adjoint_mixed,
            "final_time": info["time"],
        }
        if cpu:
            out["us_per_element_step_cpu"] = 1e6 / (cpu["value"] / (Np * 4 * 5))
        out["us_per_element_step"] = 1e6 * (ms / a.steps / 1e3) / K * world
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


def accuracy_leg(workload, steps, local, precisions):
    """Run `steps` steps of `workload` in each arithmetic and report the errors
    against the exact vortex and the mixed paths' differences from FP64."""
    from gocfd_gb300.configs import exact_vortex_error
    from gocfd_gb300.euler2d import Euler
    wl = WORKLOADS[workload]
    mesh = make_mesh(wl)
    ip = input_params(wl["N"])
    res = {"workload": workload, "steps": steps}
    states = {}
    for prec in precisions:
        s = Euler(ip, mesh, 1, precision=prec, device=local, vortex_center=(0.0, 0.0))
        info = s.step(steps)
        states[prec] = s.get_global_state()
        l2, linf = exact_vortex_error(s, info["time"])
        res[prec] = {"time": info["time"], "rel_l2_vs_exact": l2, "rel_linf_vs_exact": linf}
        s.close()
    ref = states["fp64"]
    nref = np.linalg.norm(ref)
    for prec in precisions:
        if prec == "fp64":
            continue
        d = states[prec] - ref
        res[f"{prec}_vs_fp64_rel_l2"] = float(np.linalg.norm(d) / nref)
        res[f"{prec}_vs_fp64_rel_linf"] = float(np.abs(d).max() / np.abs(ref).max())
        res[f"{prec}_vs_fp64_rel_l2_per_var"] = [float(np.linalg.norm(d[n]) / np.linalg.norm(ref[n]))
                                                for n in range(4)]
    return res


def adjoint_accuracy_leg(workload, steps, local, warm_steps=1000, every=10, hs=(1e-4, 5e-5)):
    """The adjoints' gradients against FP64 central differences: after
    warm_steps mixed steps, the field-error adjoint through `steps` steps
    (checkpoint every `every`) on the FP64 path and on the mixed path (FP32
    reverse sweep, the FP64 path's weight), dotted with the smooth directions
    d/dx0 and d/dbeta of the exact vortex at the window's start, against the
    Richardson extrapolation of FP64 central differences over hs."""
    from gocfd_gb300 import configs
    from gocfd_gb300.euler2d import Euler
    wl = WORKLOADS[workload]
    mesh = make_mesh(wl)
    ip = input_params(wl["N"])
    out = {"workload": workload, "warm_steps": warm_steps, "steps": steps, "checkpoint_every": every,
           "hs": list(hs), "directions": "d Q_exact / d x0, d Q_exact / d beta at the window's start"}
    with Euler(ip, mesh, 1, precision="fp64", device=local, vortex_center=(0.0, 0.0)) as s:
        with Euler(ip, mesh, 1, precision="fp32", device=local, vortex_center=(0.0, 0.0)) as w:
            info = w.step(warm_steps)
            Q0 = w.get_global_state()
        t0 = info["time"]
        s.set_global_state(Q0)
        s.time = t0
        s.record(steps, every)
        J, Qbf, tbf = s.functional("vortex_error")
        Qb64, _, _ = s.step_vjp(Qbf, tbf)
        with Euler(ip, mesh, 1, precision="fp32", device=local, vortex_center=(0.0, 0.0)) as g:
            g.set_global_state(Q0)
            g.time = t0
            g.record(steps, every)
            Qb32, _, _ = g.step_vjp(Qbf, tbf)
        X, Y = configs.solution_points_xy(s)

        def J_at(q):
            s.set_global_state(q)
            s.time = t0
            s.step(steps)
            return s.functional("vortex_error")[0]
        for param in ("x0", "beta"):
            d = configs.exact_vortex_param_derivative(X, Y, t0, param)
            fd = {h: (J_at(Q0 + h * d) - J_at(Q0 - h * d)) / (2 * h) for h in hs}
            rich = (4 * fd[hs[1]] - fd[hs[0]]) / 3
            a64, a32 = float(np.sum(Qb64 * d)), float(np.sum(Qb32 * d))
            out[param] = {"richardson_fd": rich, "fp64_adjoint": a64, "mixed_adjoint": a32,
                          "fp64_rel_diff": abs(a64 - rich) / abs(rich), "mixed_rel_diff": abs(a32 - rich) / abs(rich)}
    return out


def run_accuracy(a, local):
    import torch
    torch.cuda.set_device(local)
    print(json.dumps(accuracy_leg(a.workload, a.accuracy, local, ("fp64", "fp32", "tf32x3"))), flush=True)


def run_reference(a, world, rank):
    """The reference's CPU path, restated in C++ (the Go reference cannot be
    built here), timed on all host cores with the same workload and metric."""
    if rank != 0:
        return
    wl = WORKLOADS[a.workload]
    mesh = make_mesh(wl)
    # A bounded sample of the workload: full steps of the whole mesh, as many as
    # fit in ~60 s of host time (at least one, at most --steps), after --warmup
    # untimed steps.
    r = cpu_baseline(wl, mesh, 60.0, warmup=a.warmup, max_steps=a.steps)
    out = {"impl": "reference", "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": world,
           "steps": r["steps"], "warmup": a.warmup, "ms_per_step": 1e3 * r["seconds"] / r["steps"],
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
           "data": "synthetic (analytic isentropic-vortex initial condition on a generated mesh)",
           "config": workload_config(a.workload, r["K"], r["Np"]),
           "parallelism": "OpenMP over host cores",
           "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": "port",
                            "sample": r["sample"]},
           "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "Go toolchain unavailable: the reference arm is the C++ FP64 restatement of its CPU path"}
    print(json.dumps(out), flush=True)


def main():
    a = args_parse()
    world, rank, local = dist_env()
    if a.accuracy:
        run_accuracy(a, local)
    elif a.impl == "reference":
        run_reference(a, world, rank)
    else:
        run_ours(a, world, rank, local)


if __name__ == "__main__":
    main()
