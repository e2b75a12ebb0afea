/*
 * libgcfd - GB300 (sm_103a) implementation of gocfd's 2D Euler Direct Flux
 * Reconstruction right-hand side and 5-stage SSP Runge-Kutta step.
 *
 * Plain C ABI: pointers, sizes and int status codes only, so the Go driver
 * binds it with cgo and Python with ctypes.  Every entry point returns
 * GCFD_OK (0) or a negative GCFD_ERR_* code; gcfd_last_error() gives the
 * message for the context (or for a failed gcfd_create, with ctx == NULL).
 *
 * State layout (the drop-in contract of model_problems/Euler2D/euler.go:47):
 * the solution is sharded by contiguous element ranges; shard np holds four
 * row-major Np x Kmax[np] matrices (rho, rhoU, rhoV, E), element index
 * fastest (ind = k + i*Kmax, euler.go:513-516).  Shards cover the global
 * elements in order, as utils.PartitionMap.Split1D lays them out
 * (utils/parallel_utils.go:172-192).  Host arrays are only read or written
 * during a call; the library never keeps a caller pointer.
 *
 * Threading: one context is used by one host thread at a time.  Separate
 * contexts own separate CUDA streams and may be used concurrently.
 */
#ifndef GCFD_H_
#define GCFD_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GCFD_OK 0
#define GCFD_ERR_ARG (-1)
#define GCFD_ERR_SHAPE (-2)
#define GCFD_ERR_CUDA (-3)
#define GCFD_ERR_NAN (-4)
#define GCFD_ERR_TIMEOUT (-5)
#define GCFD_ERR_OOM (-6)
#define GCFD_ERR_UNSUPPORTED (-7)

/* Flux names of model_problems/Euler2D/fluxes.go:18-33. */
enum { GCFD_FLUX_AVERAGE = 0, GCFD_FLUX_LAX = 1, GCFD_FLUX_ROE = 2, GCFD_FLUX_ROE_ER = 3 };
/* Init names of model_problems/Euler2D/initialization.go:22-31. */
enum { GCFD_INIT_FREESTREAM = 0, GCFD_INIT_IVORTEX = 1, GCFD_INIT_SHOCKTUBE = 2 };
/* Limiter names of model_problems/Euler2D/filter.go:10-23. */
enum { GCFD_LIMITER_NONE = 0, GCFD_LIMITER_PERSSON_C0 = 1 };
/* Arithmetic of the RHS.  FP64 is the drop-in.  FP32 is the delta-form mixed
 * path (FP32 arithmetic, compensated FP32 conserved state, FP64 dt and
 * residual scalars); TF32X3 is the same path with the divergence GEMM on the
 * tensor cores as three TF32 products (hi*hi + hi*lo + lo*hi). */
enum { GCFD_PREC_FP64 = 0, GCFD_PREC_FP32 = 1, GCFD_PREC_TF32X3 = 2 };
/* BC flags, numbered as types.BCFLAG (types/cfd.go:11-26).  A periodic flag
 * carries its tag's group in bits 8 and up (flag | group << 8: one group per
 * periodic tag, e.g. "periodic-1", "periodic-2"); the edges of a group are
 * paired as NewTriangulation pairs them (DG2D/triangulation.go:63-99): the
 * first half and the second half of the group's list, each ordered as a
 * connected curve from its first edge (the second half from its last edge for
 * PERIODIC_REVERSED), edge i with edge i, each pair becoming one shared edge. */
enum {
  GCFD_BC_NONE = 0, GCFD_BC_IN = 1, GCFD_BC_FAR = 4, GCFD_BC_WALL = 5, GCFD_BC_CYL = 6,
  GCFD_BC_OUT = 8, GCFD_BC_IVORTEX = 9, GCFD_BC_PERIODIC = 10, GCFD_BC_PERIODIC_REVERSED = 11
};

/* Triangle mesh as readfiles.ReadGambit2d / ReadSU2 return it
 * (readfiles/readGambitGrid.go:21, readfiles/readSU2Grid.go:156): vertex
 * coordinates, 0-based element-to-vertex table, and the tagged boundary edges
 * flattened to (v1, v2, flag) triples. */
typedef struct {
  int32_t nverts;
  const double* vx;
  const double* vy;
  int32_t K;
  const int32_t* etov; /* K x 3 */
  int32_t nbc;
  const int32_t* bc_v1;
  const int32_t* bc_v2;
  const int32_t* bc_flag;
} gcfd_mesh;

/* The solver inputs of InputParameters.InputParameters2D
 * (InputParameters/InputParameters.go:11-28) plus the arithmetic mode. */
typedef struct {
  int32_t N;          /* PolynomialOrder, 0..4 */
  double cfl;         /* CFL */
  double final_time;  /* FinalTime */
  double minf;        /* Minf */
  double gamma;       /* Gamma */
  double alpha;       /* Alpha, degrees */
  double kappa;       /* Kappa (shock finder) */
  int32_t max_iterations;
  int32_t flux_type;  /* GCFD_FLUX_* */
  int32_t init_type;  /* GCFD_INIT_* */
  int32_t limiter;    /* GCFD_LIMITER_* */
  int32_t local_time_stepping;
  int32_t precision;  /* GCFD_PREC_* */
  double vortex_x0, vortex_y0; /* IVORTEX centre; the reference hard-codes (5,0) */
  int32_t device;     /* CUDA device ordinal */
} gcfd_params;

typedef struct gcfd_ctx gcfd_ctx;

/* Host-only (no GPU needed): reads a Gambit neutral (.neu) or SU2 (.su2) 2D
 * triangle mesh with the reference's conventions (ReadGambit2d,
 * readfiles/readGambitGrid.go:21-165,223-363; ReadSU2,
 * readfiles/readSU2Grid.go:27-177; chosen by extension as
 * getFileTypeFromExtension, DG2D/dfr_startup.go:184-204): 0-based triangles,
 * boundary edges with the BCFLAG of their tag (types/cfd.go:28-73).  The arrays
 * are owned by the library until gcfd_free_mesh.  Errors: GCFD_ERR_ARG with
 * gcfd_last_error(NULL). */
int gcfd_read_mesh(const char* path, gcfd_mesh* out);
void gcfd_free_mesh(gcfd_mesh* mesh);

/* Replaces Euler2D.NewEuler (model_problems/Euler2D/euler.go:61-136): builds
 * the DFR operators and the mesh topology on the host, the FP64 geometry and
 * the initial condition (InitializeSolution, euler.go:728-794) on the device,
 * and records the per-step CUDA graph.  An element with |J| <= 0 (not
 * counter-clockwise) is GCFD_ERR_ARG. */
int gcfd_create(const gcfd_mesh* mesh, const gcfd_params* params, gcfd_ctx** out);
int gcfd_destroy(gcfd_ctx* ctx);
const char* gcfd_last_error(const gcfd_ctx* ctx);

/* Sizes: elements, solution points, edge points, RT flux points, mesh edges. */
int gcfd_dims(const gcfd_ctx* ctx, int32_t* K, int32_t* Np, int32_t* NpEdge, int32_t* NpFlux,
              int32_t* nEdges);

/* Copy the sharded state in / out (c.Q of euler.go:47).  Q[np*4 + n] points at
 * shard np's Np x Kmax[np] matrix of variable n. */
int gcfd_set_state(gcfd_ctx* ctx, int32_t nshards, const int32_t* Kmax, const double* const* Q);
int gcfd_get_state(gcfd_ctx* ctx, int32_t nshards, const int32_t* Kmax, double* const* Q);
/* The same for a device-resident contiguous 4 x Np x K FP64 array. */
int gcfd_set_state_device(gcfd_ctx* ctx, const double* dQ);
int gcfd_get_state_device(gcfd_ctx* ctx, double* dQ);

/* Solver time (RungeKutta5SSP.Time, euler.go:332) and step counter. */
int gcfd_set_time(gcfd_ctx* ctx, double time);
int gcfd_get_time(gcfd_ctx* ctx, double* time, int32_t* steps);

/* One right-hand-side evaluation at `time` (BC time), replacing the chain
 * SetRTFluxInternal -> InterpolateSolutionToEdges -> CalculateEdgeEulerFlux ->
 * SetRTFluxOnEdges -> RHSInternalPoints (euler.go:665-726, edges.go:325-488)
 * as the reference tests compose it (euler_test.go:202-222).  Does not change
 * the solver state. */
int gcfd_rhs(gcfd_ctx* ctx, double time, int32_t nshards, const int32_t* Kmax,
             const double* const* Q, double* const* RHS);

/* Advance nsteps RK steps, replacing RungeKutta5SSP.Step (euler.go:408-418)
 * together with the Time += GlobalDT update of Solve (euler.go:180).  Returns
 * the time, the last global dt, and per variable the signed max of the final
 * stage increment R (the reference's printed residual, euler.go:814-849), its
 * max |R| and its RMS.  Any output pointer may be NULL.  GCFD_ERR_NAN when the
 * increment is not finite. */
int gcfd_step(gcfd_ctx* ctx, int32_t nsteps, double* time, double* dt_last, double* resid_max4,
              double* resid_absmax4, double* resid_rms4);

/* Enqueue nsteps RK steps on the context's stream and return without waiting
 * (the asynchronous form of gcfd_step; read results with gcfd_step(ctx, 0, ...)
 * or gcfd_get_state, which synchronise). */
int gcfd_enqueue_steps(gcfd_ctx* ctx, int32_t nsteps);

/* The CUDA stream (cudaStream_t) all work of the context is ordered on. */
int gcfd_get_stream(gcfd_ctx* ctx, void** stream);

/* Implementation choices of a context; no counterpart in the reference.
 * GCFD_OPT_STAGE_PIPELINE: 1 runs the mixed path's stage update as the
 * persistent kernel whose element inputs are double-buffered by TMA copies
 * (used when K % 4 == 0); 0 (the default) keeps the one-block-per-CTA kernel.
 * Setting an option records the per-step CUDA graph again.  Reading
 * GCFD_OPT_STAGE_PIPELINE gives 1 only while the pipelined kernel runs.
 * GCFD_OPT_WINDOW_TAPED (read only): 1 when the last gcfd_record_steps kept
 * every step's tape while recording (checkpoint_every >= nsteps and the tape
 * fitted in device memory), so gcfd_step_vjp recomputes nothing. */
#define GCFD_OPT_STAGE_PIPELINE 1
#define GCFD_OPT_WINDOW_TAPED 2
int gcfd_set_option(gcfd_ctx* ctx, int32_t option, int32_t value);
int gcfd_get_option(const gcfd_ctx* ctx, int32_t option, int32_t* value);

/* Run one step launch by launch with CUDA events around each kernel and
 * return the summed device time per kernel family (ms): [0] face
 * interpolation, [1] edge flux + BCs, [2] divergence + RK update, [3] step
 * bookkeeping.  Used to attribute time for the roofline. */
int gcfd_profile_step(gcfd_ctx* ctx, double* kernel_ms4, int32_t* launches4);

/* SIMT FMA rates of the device (TFLOP/s, FMA = 2 flops), measured by
 * independent FMA chains on every SM: the compute roofline of the FP64 path's
 * kernels and of the mixed path's FP32 arithmetic.  No counterpart in the
 * reference.  Either output may be NULL. */
int gcfd_device_fma_peaks(int32_t device, double* fp64_tflops, double* fp32_tflops);

/* Host-only (no GPU needed): the FP64 operator matrices built for order N.
 * which: 0 FluxEdgeInterp (3NpEdge x Np), 1 DivInt (Np x NpFlux),
 * 2 Div (NpFlux x NpFlux), 3 V (Np x Np), 4 solution r,s (Np x 2),
 * 5 flux-point r,s (NpFlux x 2).  With out == NULL only rows/cols are set. */
int gcfd_host_operator(int32_t N, int32_t which, double* out, int32_t* rows, int32_t* cols);

/* ---- Adjoint (vector-Jacobian products) ----
 * The reference has no adjoint; these transpose its discrete RHS and step
 * exactly, including the time step's dependence on the state (the global max
 * wave speed of calculateGlobalDT, euler.go:945-971, with the FinalTime clip;
 * the running max of CalculateLocalDT, euler.go:973-1002), the IVortex
 * boundary state's dependence on the solver time and, with the PerssonC0
 * limiter, the sensor, vertex maxima, limiter, RT gradient, viscous fluxes and
 * viscous time-step limit.
 * On a mixed-precision context (GCFD_PREC_FP32 / GCFD_PREC_TF32X3) the
 * window's steps are recomputed and taped by the mixed forward itself and the
 * reverse sweep of gcfd_step_vjp runs in FP32 (boundary points and wave-speed
 * maxima in FP64); the state adjoints agree with the FP64 path's to ~1e-6
 * relative.  gcfd_rhs_vjp runs the FP64 kernels on every context.  The mixed
 * path's adjoint covers the Euler RHS and step without the PerssonC0
 * dissipation and without GCFD_OPT_STAGE_PIPELINE; those return
 * GCFD_ERR_UNSUPPORTED. */

/* Functionals of the current state: the wall pressure force, summed over Wall
 * and Cyl boundary edges as |edge| sum_p w_p p n_x (or n_y), with the
 * interpolatory weights of the edge flux points (the integrated form of the
 * wall data OutputFinal writes, euler.go:251-316); and the squared error
 * sum (Q - Q_exact(t))^2 against the isentropic vortex at the solver time
 * (IVortex.GetStateC, isentropic_vortex/analytic_vortex.go:31-82). */
#define GCFD_FUNC_WALL_FORCE_X 0
#define GCFD_FUNC_WALL_FORCE_Y 1
#define GCFD_FUNC_VORTEX_ERROR 2
/* J and, when Qbar is given, dJ/dQ (sharded like gcfd_get_state) and dJ/dt. */
int gcfd_functional(gcfd_ctx* ctx, int32_t kind, double* J, int32_t nshards, const int32_t* Kmax,
                    double* const* Qbar, double* tbar);

/* Adjoint of gcfd_rhs at (Q, time): Qbar = (dRHS/dQ)^T RHSbar, plus the
 * far-field Qinf adjoint (4, with pinf and cinf following Qinf as FreeStream
 * derives them, fluids.go:370-406) and d/dtime (IVortex boundaries).  Replaces
 * nothing in the reference: the transpose of SetRTFluxInternal ->
 * InterpolateSolutionToEdges -> CalculateEdgeEulerFlux -> SetRTFluxOnEdges ->
 * RHSInternalPoints (euler.go:665-726, edges.go:325-488). */
int gcfd_rhs_vjp(gcfd_ctx* ctx, double time, int32_t nshards, const int32_t* Kmax, const double* const* Q,
                 const double* const* RHSbar, double* const* Qbar, double* qinf_bar4, double* time_bar);

/* Advance nsteps like gcfd_step, keeping a checkpoint of the state every
 * checkpoint_every steps for a following gcfd_step_vjp (memory: the
 * checkpoints plus checkpoint_every states, FP64; plus, when it fits, a tape
 * slot per step of a segment).  A mixed-precision context checkpoints its
 * compensated state as hi + lo in FP64, which restores it exactly; with
 * checkpoint_every >= nsteps it keeps every step's tape while recording when a
 * slot per step fits in device memory (10 FP32 state copies per step; 10 FP64
 * ones on an FP64 context), and gcfd_step_vjp then recomputes nothing.  The
 * window's device blocks are kept when the next window is recorded and reused
 * where it asks for blocks of the same size (the same shape of window asks for
 * the same blocks); what it does not reuse stays held until an allocation
 * fails (then it is freed and the allocation tried again) or gcfd_destroy. */
int gcfd_record_steps(gcfd_ctx* ctx, int32_t nsteps, int32_t checkpoint_every, double* time, double* dt_last);

/* Adjoint of the recorded window (RungeKutta5SSP.Step x nsteps, euler.go:408-418):
 * from the adjoint of the final state (and of the final time) to the adjoint
 * of the window's initial state, the far-field Qinf (4) and the initial time.
 * Each segment of checkpoint_every steps is recomputed once from its
 * checkpoint with every step's stage tape kept (a slot per step, when they fit;
 * otherwise each step is recomputed once more with its tape), then reversed; a
 * window taped while it was recorded is only reversed.  On a mixed-precision
 * context the recompute is the mixed forward and the reverse sweep runs in
 * FP32 (PerssonC0 and the pipelined stage kernel: GCFD_ERR_UNSUPPORTED there).
 * The solver state and time are the window's end again on return. */
int gcfd_step_vjp(gcfd_ctx* ctx, int32_t nshards, const int32_t* Kmax, const double* const* Qfinal_bar,
                  double tfinal_bar, double* const* Q0_bar, double* qinf_bar4, double* t0_bar);

/* ---- Post-processing of the current state ---- */

/* The solution interpolated at npts points (x[p], y[p]) by the element's own
 * polynomial (the Lagrange basis of its solution points at the point's
 * reference coordinates), replacing the sampled lines of the Sod validation
 * (NewSODShockTube / InterpolateFields,
 * model_problems/Euler2D/sod_shock_tube/shock_tube.go:27-142).  q4 receives
 * 4 x npts values (variable-major: rho, rhoU, rhoV, E); elem (may be NULL)
 * the containing element of each point, or -1.  A point on a shared edge or
 * vertex takes the element with the lowest index.  GCFD_ERR_ARG when a point
 * lies in no element.  The reference maps the barycentric coordinates of the
 * point straight to the element's (r, s) (getUVCoords, shock_tube.go:81-128),
 * which samples a different point of the element; this call samples the
 * point itself. */
int gcfd_sample_points(gcfd_ctx* ctx, int32_t npts, const double* x, const double* y, double* q4,
                       int32_t* elem);

/* The wall data of OutputFinal (model_problems/Euler2D/euler.go:251-316): for
 * every Wall or Cyl boundary edge (in the mesh's order) and each of its NpEdge
 * edge flux points (one point per edge at N = 0), the point's coordinates, the
 * state interpolated there from the wall element's solution points (4 x npts,
 * variable-major) and the pressure.  With x, y, q4 and p all NULL only *npts
 * is set (the count); otherwise *npts gives the room in each array on entry
 * and the count on return.  Any of x, y, q4, p may be NULL. */
int gcfd_wall_points(gcfd_ctx* ctx, int32_t* npts, double* x, double* y, double* q4, double* p);

/* ---- Solution output: the graph mesh and fields ----
 * What the reference streams to meshfile.gobcfd and solutionfile.gobcfd
 * (CreateAVSGraphMesh, AVSFieldWriter, DG2D/graphics_support.go:43-128,173-230;
 * GetPlotField, model_problems/Euler2D/plot.go:14-85; Solve, euler.go:190-215),
 * as arrays for the caller's writer (the Go caller keeps its gob encoder).
 * Each element has len_element = 3 (NpEdge + 1) + Np graph points: per edge
 * n = 0..2 its starting vertex then its NpEdge flux points counter-clockwise,
 * then the Np solution points; element-major (point k * len_element + p). */

/* The reference element's graph points (2 x len_element r, s pairs) and its
 * sub-triangles (3 x ntri local point indices, counter-clockwise): the Delaunay
 * triangulation of the graph points (the reference's constrained triangulation
 * with Triangle, geometry2D/triangulate.go:34-93; its constraints lie on the
 * hull).  Needs no context; NULL outputs are skipped. */
int gcfd_host_graph_element(int32_t N, int32_t* len_element, int32_t* ntri, double* rs, int32_t* tris);

/* The mesh's graph points as FP32 (x, y) pairs (2 x K x len_element; the
 * vertices are the mesh's, the edge and solution points their affine images)
 * and the sub-triangles as global point indices (3 x K x ntri_per_element,
 * int64 like the reference's TriMesh).  NULL outputs are skipped. */
int gcfd_graph_mesh(gcfd_ctx* ctx, int32_t* len_element, int32_t* ntri_per_element, float* xy, int64_t* tris);

/* Flow functions of the current state at the graph points, FP32, K x
 * len_element per field, fields one after another.  kinds are the reference's
 * FlowFunction values 0..13 (fluids.go:209-222: Density, XMomentum, YMomentum,
 * Energy, Mach, StaticPressure, DynamicPressure, PressureCoefficient,
 * SoundSpeed, Velocity, XVelocity, YVelocity, Enthalpy, Entropy), evaluated at
 * the solution points (GetFlowFunctionBase, fluids.go:289-336, with the far
 * field's Pinf and dynamic pressure), taken to the graph points by the
 * solution basis, each vertex value then the mean of the two edge points
 * beside it (AverageGraphFieldVertices, DG2D/graphics_support2.go:184-199). */
int gcfd_graph_fields(gcfd_ctx* ctx, int32_t nfields, const int32_t* kinds, float* out);

/* Residual norms of an increment array that the caller owns, computed without
 * allocating anything.  This entry point has no counterpart in the reference.
 *
 * It is for callers that cannot call cudaMalloc when they need the norms: a
 * host framework whose own allocator owns the GPU's memory and allows no
 * allocation behind its back, or a steady-state loop that must not allocate
 * (an allocation can fail mid-run, and cudaFree synchronises the device).
 * Such a caller keeps the increments of a step (for example the difference of
 * two gcfd_get_state_device snapshots) in its own memory and asks for the same
 * numbers gcfd_step reports: per variable the signed max, the max |R| and the
 * RMS over the Np x K points.
 *
 * dR: device pointer, 4 x Np x K FP64 (variable, point, element fastest), on
 * the device that is current for the calling thread.  stream: a cudaStream_t
 * (NULL for the default stream); the call enqueues its two kernels and one
 * 96-byte copy there and waits for that stream.  Any output pointer may be NULL.
 *
 * The intermediate per-block partials live in one fixed device array built
 * into the library (1.5 MiB, no per-call allocation), which caps Np x K at
 * GCFD_RESID_STATIC_MAX_POINTS; larger inputs return GCFD_ERR_SHAPE with a
 * message in gcfd_last_error(NULL).  Every part of that array that a call
 * reads is written earlier in the same call, so nothing carries over from one
 * call to the next.  All calls on a device share the array: calls that can
 * overlap on the GPU (other streams, other host threads) race and must be
 * serialised by the caller.  The call blocks on the stream (it copies the 12
 * results to the host and synchronises), so it must not be called on a
 * stream that is being captured into a CUDA graph.  The first call on each
 * device, and the first after that device's context was destroyed and
 * recreated (cudaDeviceReset), looks up the array's device address
 * (cudaGetSymbolAddress, which can load the module) and so costs more than
 * the later ones.  GCFD_ERR_NAN when an increment is not finite (the outputs
 * are still written). */
#define GCFD_RESID_STATIC_MAX_POINTS 33554432 /* 16384 blocks x 2048 points */
int gcfd_residual_norms_static(const double* dR, int32_t Np, int32_t K, void* stream, double* resid_max4,
                               double* resid_absmax4, double* resid_rms4);

#ifdef __cplusplus
}
#endif
#endif /* GCFD_H_ */
