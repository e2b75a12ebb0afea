"""Host-side mirror of gocfd's Euler2D solver interface over libgcfd.

Names and argument meanings follow the reference so that a caller of
model_problems/Euler2D reads the same here:

  InputParameters2D  InputParameters/InputParameters.go:11-31 (YAML keys are the
                     field names, matched case-insensitively as ghodss/yaml does;
                     Gamma = 1.4 and Minf = 0.1 defaults of cmd/2D.go:84-86)
  Euler              NewEuler (model_problems/Euler2D/euler.go:61-136)
  Euler.step         RungeKutta5SSP.Step + Time += GlobalDT (euler.go:176-181,408-418)
  Euler.solve        Solve (euler.go:138-220) without plotting output
  Euler.rhs          the RHS chain used by the reference tests (euler_test.go:202-222)
  Euler.Q            the sharded state [np][4] of Np x Kmax matrices (euler.go:47)
  PartitionMap       utils/parallel_utils.go:86-192
  set_parallel_degree  SetParallelDegree (parallelism.go:100-120)

Errors from the library raise GcfdError (the reference panics).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from .meshes import Mesh, read_mesh

FLUX_TYPES = {"average": 0, "lax": 1, "roe": 2, "roe-er": 3}          # fluxes.go:25-33
INIT_TYPES = {"freestream": 0, "ivortex": 1, "shocktube": 2}          # initialization.go:22-31
LIMITERS = {"": 0, "perssonc0": 1, "persson c0": 1}                   # filter.go:29-35
PRECISIONS = {"fp64": 0, "fp32": 1, "tf32x3": 2}


@dataclass
class InputParameters2D:
    """The reference's InputParameters2D (InputParameters/InputParameters.go:11)
    with its field names and defaults; `parse` / `from_file` read its YAML inputs."""
    Title: str = ""
    CFL: float = 0.0
    FluxType: str = ""
    InitType: str = ""
    PolynomialOrder: int = 0
    FinalTime: float = 0.0
    Minf: float = 0.1
    Gamma: float = 1.4
    Alpha: float = 0.0
    BCs: dict = field(default_factory=dict)
    LocalTimeStepping: bool = False
    MaxIterations: int = 0
    ImplicitSolver: bool = False
    Limiter: str = ""
    Kappa: float = 0.0
    PlotFields: list = field(default_factory=list)

    @classmethod
    def parse(cls, text: str) -> "InputParameters2D":
        """Flat YAML subset of the reference inputs: 'Key: value' lines, '#'
        comments, inline lists; nested BCs blocks are kept as raw text maps."""
        ip = cls()
        names = {f.lower(): f for f in cls.__dataclass_fields__}
        for raw in text.splitlines():
            line = raw.split("#", 1)[0].rstrip()
            if not line.strip() or line.startswith((" ", "\t")) or ":" not in line:
                continue
            key, val = line.split(":", 1)
            key, val = key.strip(), val.strip()
            fname = names.get(key.lower())
            if fname is None:
                continue
            cur = getattr(ip, fname)
            if isinstance(cur, bool):
                setattr(ip, fname, val.lower() in ("true", "yes", "on", "1"))
            elif isinstance(cur, int):
                setattr(ip, fname, int(float(val)))
            elif isinstance(cur, float):
                setattr(ip, fname, float(val))
            elif isinstance(cur, list):
                items = val.strip("[]")
                setattr(ip, fname, [s.strip().strip("'\"") for s in items.split(",") if s.strip()])
            elif isinstance(cur, dict):
                continue
            else:
                setattr(ip, fname, val.strip("'\""))
        return ip

    @classmethod
    def from_file(cls, path: str) -> "InputParameters2D":
        """Parse a reference input file (test_cases/Euler2D/*/input*.yaml)."""
        with open(path) as f:
            return cls.parse(f.read())


class PartitionMap:
    """Contiguous split of MaxIndex items into ParallelDegree buckets with at
    most one item of imbalance, the remainder spread over the first buckets."""

    def __init__(self, parallel_degree: int, max_index: int):
        self.ParallelDegree = parallel_degree
        self.MaxIndex = max_index
        self.Partitions = [self.split1d(n) for n in range(parallel_degree)]

    def split1d(self, n: int):
        """Half-open item range of bucket n (PartitionMap.Split1D, utils/parallel_utils.go:172-192)."""
        npart = self.MaxIndex // self.ParallelDegree
        rem = self.MaxIndex % self.ParallelDegree
        start_add, end_add = 0, 0
        if rem:
            if n + 1 > rem:
                start_add, end_add = rem, 0
            else:
                start_add, end_add = n, 1
        b0 = n * npart + start_add
        return (b0, b0 + npart + end_add)

    def bucket_dimension(self, n: int) -> int:
        """Number of items in bucket n (GetBucketDimension, utils/parallel_utils.go:160)."""
        a, b = self.Partitions[n]
        return b - a


def set_parallel_degree(proc_limit: int, K: int) -> PartitionMap:
    """The shard count of Euler.SetParallelDegree (model_problems/Euler2D/parallelism.go:100-114):
    the process limit if given, else max(NumCPU, K / 185), and 1 when that exceeds K."""
    if proc_limit != 0:
        pd = proc_limit
    else:
        pd = max(os.cpu_count() or 1, K // 185)
    if pd > K:
        pd = 1
    return PartitionMap(pd, K)


class Euler:
    """A device-resident Euler2D DFR solver with the reference's interface."""

    def __init__(self, ip: InputParameters2D, mesh, proc_limit: int = 0, *, precision: str = "fp64",
                 device: int = 0, vortex_center=(5.0, 0.0), verbose: bool = False):
        self.lib = _lib.load()
        self.ip = ip
        self.mesh: Mesh = read_mesh(mesh) if isinstance(mesh, str) else mesh
        flux = ip.FluxType.strip().lower()
        if flux not in FLUX_TYPES:
            raise ValueError(f"unable to use flux named {ip.FluxType}")
        init = ip.InitType.strip().lower()
        if init not in INIT_TYPES:
            raise ValueError(f"unable to use init type named {ip.InitType}")
        lim = ip.Limiter.strip().lower()
        if lim not in LIMITERS:
            raise ValueError(f"unable to use limiter named [{lim}]")
        self.partitions = set_parallel_degree(proc_limit, self.mesh.K)
        m = self.mesh
        self._vx = np.ascontiguousarray(m.VX, dtype=np.float64)
        self._vy = np.ascontiguousarray(m.VY, dtype=np.float64)
        self._etov = np.ascontiguousarray(m.EToV, dtype=np.int32)
        b1, b2, bf = m.bc_arrays()
        self._bc = (b1, b2, bf)
        cm = _lib.Mesh(len(self._vx), self._vx.ctypes.data_as(_lib.PD), self._vy.ctypes.data_as(_lib.PD),
                       m.K, self._etov.ctypes.data_as(_lib.PI), len(b1), b1.ctypes.data_as(_lib.PI),
                       b2.ctypes.data_as(_lib.PI), bf.ctypes.data_as(_lib.PI))
        prm = _lib.Params()
        prm.N = ip.PolynomialOrder
        prm.cfl = ip.CFL
        prm.final_time = ip.FinalTime
        prm.minf = ip.Minf
        prm.gamma = ip.Gamma
        prm.alpha = ip.Alpha
        prm.kappa = ip.Kappa
        prm.max_iterations = ip.MaxIterations
        prm.flux_type = FLUX_TYPES[flux]
        prm.init_type = INIT_TYPES[init]
        prm.limiter = LIMITERS[lim]
        prm.local_time_stepping = int(ip.LocalTimeStepping)
        prm.precision = PRECISIONS[precision]
        prm.vortex_x0, prm.vortex_y0 = vortex_center
        prm.device = device
        ctx = C.c_void_p()
        _lib.check(self.lib, None, self.lib.gcfd_create(C.byref(cm), C.byref(prm), C.byref(ctx)))
        self.ctx = ctx
        dims = [C.c_int32() for _ in range(5)]
        _lib.check(self.lib, ctx, self.lib.gcfd_dims(ctx, *[C.byref(d) for d in dims]))
        self.K, self.Np, self.NpEdge, self.NpFlux, self.nEdges = (d.value for d in dims)
        self.steps = 0
        if verbose:
            print(f"Euler Equations in 2 Dimensions\nSolving {init}\nFlux Algorithm: [{flux}]\n"
                  f"CFL = {ip.CFL:8.4f}, Polynomial Degree N = {ip.PolynomialOrder}, Num Elements K = {m.K}")

    # -- lifetime --------------------------------------------------------------
    def close(self):
        """Release the device context (gcfd_destroy); idempotent."""
        if getattr(self, "ctx", None):
            self.lib.gcfd_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- sharded state ------------------------------------------------------------
    def _kmax(self):
        pm = self.partitions
        return np.array([pm.bucket_dimension(n) for n in range(pm.ParallelDegree)], dtype=np.int32)

    def _ptrs(self, shards):
        arr = (_lib.PD * (4 * len(shards)))()
        for np_, sh in enumerate(shards):
            for n in range(4):
                a = sh[n]
                if a.dtype != np.float64 or not a.flags.c_contiguous:
                    raise ValueError("state matrices must be C-contiguous float64")
                arr[np_ * 4 + n] = a.ctypes.data_as(_lib.PD)
        return arr

    def new_sharded(self):
        """Zeroed shards shaped like the reference's c.Q: per shard, 4 Np x Kmax matrices."""
        return [[np.zeros((self.Np, k)) for _ in range(4)] for k in self._kmax()]

    @property
    def Q(self):
        """The sharded state (c.Q of euler.go:47), copied from the device (gcfd_get_state)."""
        out = self.new_sharded()
        km = self._kmax()
        _lib.check(self.lib, self.ctx, self.lib.gcfd_get_state(self.ctx, len(km), km.ctypes.data_as(_lib.PI),
                                                              self._ptrs(out)))
        return out

    @Q.setter
    def Q(self, shards):
        """Copy a sharded state to the device (gcfd_set_state)."""
        km = self._kmax()
        _lib.check(self.lib, self.ctx, self.lib.gcfd_set_state(self.ctx, len(km), km.ctypes.data_as(_lib.PI),
                                                              self._ptrs(shards)))

    def shard(self, Qg: np.ndarray):
        """Split a global 4 x Np x K array into the reference's shards."""
        out = []
        for (a, b) in self.partitions.Partitions:
            out.append([np.ascontiguousarray(Qg[n][:, a:b]) for n in range(4)])
        return out

    def unshard(self, shards) -> np.ndarray:
        """Join the reference's shards into one 4 x Np x K array."""
        return np.stack([np.concatenate([sh[n] for sh in shards], axis=1) for n in range(4)])

    def get_global_state(self) -> np.ndarray:
        """The state as one 4 x Np x K array."""
        return self.unshard(self.Q)

    def set_global_state(self, Qg: np.ndarray):
        """Set the state from one 4 x Np x K array."""
        self.Q = self.shard(np.asarray(Qg, dtype=np.float64))

    # -- time ------------------------------------------------------------------------
    @property
    def time(self) -> float:
        """Solver time (RungeKutta5SSP.Time)."""
        t, s = C.c_double(), C.c_int32()
        _lib.check(self.lib, self.ctx, self.lib.gcfd_get_time(self.ctx, C.byref(t), C.byref(s)))
        return t.value

    @time.setter
    def time(self, t: float):
        """Set the solver time (the BC time of the next step)."""
        _lib.check(self.lib, self.ctx, self.lib.gcfd_set_time(self.ctx, float(t)))

    # -- the hot path ------------------------------------------------------------------
    def rhs(self, shards, time: float = 0.0):
        """One RHS evaluation of a sharded state at BC time `time` (gcfd_rhs: the chain
        SetRTFluxInternal .. RHSInternalPoints, euler.go:665-726, edges.go:325-488)."""
        out = self.new_sharded()
        km = self._kmax()
        _lib.check(self.lib, self.ctx, self.lib.gcfd_rhs(self.ctx, float(time), len(km), km.ctypes.data_as(_lib.PI),
                                                        self._ptrs(shards), self._ptrs(out)))
        return out

    def rhs_global(self, Qg: np.ndarray, time: float = 0.0) -> np.ndarray:
        """rhs() on a 4 x Np x K array."""
        return self.unshard(self.rhs(self.shard(np.asarray(Qg, dtype=np.float64)), time))

    # -- adjoint (FP64 path) --------------------------------------------------------------
    FUNCTIONALS = {"wall_force_x": 0, "wall_force_y": 1, "vortex_error": 2}

    def functional(self, kind: str):
        """(J, dJ/dQ as a global 4 x Np x K array, dJ/dtime) of the current state."""
        J, tb = C.c_double(), C.c_double()
        out = self.new_sharded()
        km = self._kmax()
        _lib.check(self.lib, self.ctx, self.lib.gcfd_functional(self.ctx, self.FUNCTIONALS[kind], C.byref(J), len(km),
                                                               km.ctypes.data_as(_lib.PI), self._ptrs(out),
                                                               C.byref(tb)))
        return J.value, self.unshard(out), tb.value

    def rhs_vjp_global(self, Qg: np.ndarray, Rbar: np.ndarray, time: float = 0.0):
        """(dRHS/dQ)^T Rbar at (Qg, time); returns (Qbar, Qinf_bar[4], time_bar)."""
        out = self.new_sharded()
        km = self._kmax()
        qinf, tb = (C.c_double * 4)(), C.c_double()
        _lib.check(self.lib, self.ctx, self.lib.gcfd_rhs_vjp(
            self.ctx, float(time), len(km), km.ctypes.data_as(_lib.PI),
            self._ptrs(self.shard(np.asarray(Qg, dtype=np.float64))),
            self._ptrs(self.shard(np.asarray(Rbar, dtype=np.float64))), self._ptrs(out), qinf, C.byref(tb)))
        return self.unshard(out), np.array(qinf[:]), tb.value

    def record(self, nsteps: int, checkpoint_every: int = 1):
        """Advance nsteps keeping checkpoints for step_vjp; returns (time, dt_last)."""
        t, dt = C.c_double(), C.c_double()
        _lib.check(self.lib, self.ctx, self.lib.gcfd_record_steps(self.ctx, int(nsteps), int(checkpoint_every),
                                                                 C.byref(t), C.byref(dt)))
        self.steps += nsteps
        return t.value, dt.value

    def step_vjp(self, Qbar_final: np.ndarray, tbar_final: float = 0.0):
        """Adjoint of the recorded window: (Q0_bar, Qinf_bar[4], t0_bar)."""
        out = self.new_sharded()
        km = self._kmax()
        qinf, tb = (C.c_double * 4)(), C.c_double()
        _lib.check(self.lib, self.ctx, self.lib.gcfd_step_vjp(
            self.ctx, len(km), km.ctypes.data_as(_lib.PI),
            self._ptrs(self.shard(np.asarray(Qbar_final, dtype=np.float64))), float(tbar_final),
            self._ptrs(out), qinf, C.byref(tb)))
        return self.unshard(out), np.array(qinf[:]), tb.value

    # -- post-processing -----------------------------------------------------------
    def sample_points(self, x, y):
        """The state interpolated at points (x, y) (gcfd_sample_points; the Sod line
        samples of shock_tube.go:27-142): (4 x npts array, containing elements)."""
        x = np.ascontiguousarray(x, dtype=np.float64).ravel()
        y = np.ascontiguousarray(y, dtype=np.float64).ravel()
        q = np.zeros((4, x.size))
        el = np.zeros(x.size, np.int32)
        _lib.check(self.lib, self.ctx, self.lib.gcfd_sample_points(
            self.ctx, x.size, x.ctypes.data_as(_lib.PD), y.ctypes.data_as(_lib.PD), q.ctypes.data_as(_lib.PD),
            el.ctypes.data_as(_lib.PI)))
        return q, el

    def sod_line(self, npts: int):
        """NewSODShockTube's samples (shock_tube.go:27-49): npts x locations equally spaced
        on [0, 1] (the ends moved 1e-5 inward) along the mesh's mid-height line; returns
        (x, 4 x npts state)."""
        x = np.arange(npts) / (npts - 1.0)
        x[0] += 1e-5
        x[-1] -= 1e-5
        ymid = 0.5 * (self.mesh.VY.max() - self.mesh.VY.min()) + self.mesh.VY.min()
        q, _ = self.sample_points(x, np.full(npts, ymid))
        return x, q

    def wall_points(self):
        """Wall data of OutputFinal (euler.go:251-316; gcfd_wall_points): x, y, state
        (4 x npts) and pressure at every Wall/Cyl edge flux point."""
        n = C.c_int32(0)
        _lib.check(self.lib, self.ctx, self.lib.gcfd_wall_points(self.ctx, C.byref(n), None, None, None, None))
        x, y, p = np.zeros(n.value), np.zeros(n.value), np.zeros(n.value)
        q = np.zeros((4, n.value))
        _lib.check(self.lib, self.ctx, self.lib.gcfd_wall_points(
            self.ctx, C.byref(n), x.ctypes.data_as(_lib.PD), y.ctypes.data_as(_lib.PD), q.ctypes.data_as(_lib.PD),
            p.ctypes.data_as(_lib.PD)))
        return x, y, q, p

    # the reference's FlowFunction names and values (fluids.go:209-222)
    FLOW_FUNCTIONS = {"Density": 0, "XMomentum": 1, "YMomentum": 2, "Energy": 3, "Mach": 4, "StaticPressure": 5,
                      "DynamicPressure": 6, "PressureCoefficient": 7, "SoundSpeed": 8, "Velocity": 9,
                      "XVelocity": 10, "YVelocity": 11, "Enthalpy": 12, "Entropy": 13}

    def graph_mesh(self):
        """The solution output's graph mesh (gcfd_graph_mesh; CreateAVSGraphMesh,
        graphics_support.go:173-230): XY as (K * len_element) x 2 float32 and the
        sub-triangles as (K * ntri) x 3 int64 global point indices."""
        L, nt = C.c_int32(), C.c_int32()
        _lib.check(self.lib, self.ctx, self.lib.gcfd_graph_mesh(self.ctx, C.byref(L), C.byref(nt), None, None))
        xy = np.zeros((self.K * L.value, 2), dtype=np.float32)
        tris = np.zeros((self.K * nt.value, 3), dtype=np.int64)
        _lib.check(self.lib, self.ctx, self.lib.gcfd_graph_mesh(
            self.ctx, None, None, xy.ctypes.data_as(C.POINTER(C.c_float)), tris.ctypes.data_as(C.POINTER(C.c_int64))))
        return xy, tris

    def graph_fields(self, names):
        """Flow functions (names of FLOW_FUNCTIONS) at the graph points, a dict of
        float32 arrays of K * len_element (gcfd_graph_fields; GetPlotField, plot.go:14-85)."""
        kinds = np.array([self.FLOW_FUNCTIONS[n] for n in names], dtype=np.int32)
        L = C.c_int32()
        _lib.check(self.lib, self.ctx, self.lib.gcfd_graph_mesh(self.ctx, C.byref(L), None, None, None))
        out = np.zeros((len(names), self.K * L.value), dtype=np.float32)
        _lib.check(self.lib, self.ctx, self.lib.gcfd_graph_fields(self.ctx, len(names), kinds.ctypes.data_as(_lib.PI),
                                                                 out.ctypes.data_as(C.POINTER(C.c_float))))
        return {n: out[i] for i, n in enumerate(names)}

    def step(self, nsteps: int = 1):
        """Advance nsteps; returns dict(time, dt, resid_max, resid_absmax, resid_rms)."""
        t, dt = C.c_double(), C.c_double()
        rmax, rabs, rrms = (C.c_double * 4)(), (C.c_double * 4)(), (C.c_double * 4)()
        _lib.check(self.lib, self.ctx, self.lib.gcfd_step(self.ctx, int(nsteps), C.byref(t), C.byref(dt),
                                                         rmax, rabs, rrms))
        self.steps += nsteps
        return dict(time=t.value, dt=dt.value, resid_max=list(rmax), resid_absmax=list(rabs),
                    resid_rms=list(rrms))

    def enqueue_steps(self, nsteps: int):
        """Queue nsteps on the context's stream without waiting."""
        _lib.check(self.lib, self.ctx, self.lib.gcfd_enqueue_steps(self.ctx, int(nsteps)))
        self.steps += nsteps

    def check_if_finished(self, time: float, steps: int) -> bool:
        """Solve's stopping test (euler.go:796-801): FinalTime reached or MaxIterations steps done."""
        return time >= self.ip.FinalTime or steps >= self.ip.MaxIterations

    def solve(self, print_every: int = 100, printer=print):
        """Solve (euler.go:138-220): step until FinalTime or MaxIterations,
        printing the reference's update line (signed max residual per variable,
        "L1" = their max, "L2" = sqrt(sum of squares)/4)."""
        steps, finished, info = 0, False, {}
        while not finished:
            info = self.step(1)
            steps += 1
            finished = self.check_if_finished(info["time"], steps)
            if finished or steps == 1 or steps % print_every == 0:
                r = info["resid_max"]
                l1 = max(0.0, *r)
                l2 = float(np.sqrt(sum(x * x for x in r))) / 4.0
                if self.ip.LocalTimeStepping:
                    head = f"{steps:10d}              "
                else:
                    head = f"{steps:8d}{info['time']:8.5f}{info['dt']:8.5f}"
                printer(head + "".join(f"{v:11.4e}" for v in r) + f"{l1:11.4e}{l2:11.4e}")
        return info

    def profile_step(self):
        """One eagerly launched step with CUDA events around each kernel family (gcfd_profile_step):
        ([ms] x 4, [launches] x 4) for preparation/interpolation, edge fluxes, stage update, bookkeeping."""
        ms, n = (C.c_double * 4)(), (C.c_int32 * 4)()
        _lib.check(self.lib, self.ctx, self.lib.gcfd_profile_step(self.ctx, ms, n))
        return list(ms), list(n)

    def stream_handle(self) -> int:
        """The context's CUDA stream (cudaStream_t) as an integer, for torch.cuda.ExternalStream."""
        s = C.c_void_p()
        _lib.check(self.lib, self.ctx, self.lib.gcfd_get_stream(self.ctx, C.byref(s)))
        return s.value or 0

    # GCFD_OPT_STAGE_PIPELINE of gcfd.h
    OPT_STAGE_PIPELINE = 1

    def set_stage_pipeline(self, on: bool) -> None:
        """Select the persistent TMA-pipelined stage kernel (True) or the one-block kernel (False, the default)."""
        _lib.check(self.lib, self.ctx, self.lib.gcfd_set_option(self.ctx, self.OPT_STAGE_PIPELINE, int(bool(on))))

    def stage_pipeline(self) -> bool:
        """True while the mixed path's stage update runs as the pipelined kernel."""
        v = C.c_int32()
        _lib.check(self.lib, self.ctx, self.lib.gcfd_get_option(self.ctx, self.OPT_STAGE_PIPELINE, C.byref(v)))
        return bool(v.value)

    # GCFD_OPT_WINDOW_TAPED of gcfd.h (read only)
    OPT_WINDOW_TAPED = 2

    def window_taped(self) -> bool:
        """True when the last record() kept every step's tape (checkpoint_every >= nsteps, and it fitted)."""
        v = C.c_int32()
        _lib.check(self.lib, self.ctx, self.lib.gcfd_get_option(self.ctx, self.OPT_WINDOW_TAPED, C.byref(v)))
        return bool(v.value)


def parse_yaml_file(path: str) -> InputParameters2D:
    """The reference's input-file reader (InputParameters2D.Parse of a YAML file)."""
    return InputParameters2D.from_file(path)

