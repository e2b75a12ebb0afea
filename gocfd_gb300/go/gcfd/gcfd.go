// Package gcfd binds libgcfd (include/gcfd.h) for the gocfd Euler2D solver.
//
// It is the thin cgo layer between model_problems/Euler2D (NewEuler,
// RungeKutta5SSP.Step, the RHS chain) and the GB300 kernels.  Every non-zero
// status becomes an error; Euler2D turns it into a panic, as the reference
// does for its own failures.
//
// Host arrays stay owned by Go: the library copies them during the call and
// keeps no pointer.  The per-shard pointer table lives in C memory and holds
// Go pointers only while they are pinned (runtime.Pinner, Go 1.21+).
package gcfd

/*
#cgo CFLAGS: -I${SRCDIR}/../../../include
#cgo LDFLAGS: -L${SRCDIR}/../.. -lgcfd -Wl,-rpath,${SRCDIR}/../..
#include <stdlib.h>
#include "gcfd.h"
*/
import "C"

import (
	"fmt"
	"runtime"
	"unsafe"
)

// Precision modes of gcfd_params.precision.
const (
	PrecFP64 = int(C.GCFD_PREC_FP64) // the drop-in
	PrecFP32 = int(C.GCFD_PREC_FP32) // delta-form FP32 arithmetic, compensated state
	PrecTF32x3 = int(C.GCFD_PREC_TF32X3) // the same with the divergence GEMM on the tensor cores
)

// Functionals for the adjoint (GCFD_FUNC_*).
const (
	FuncWallForceX  = int(C.GCFD_FUNC_WALL_FORCE_X)
	FuncWallForceY  = int(C.GCFD_FUNC_WALL_FORCE_Y)
	FuncVortexError = int(C.GCFD_FUNC_VORTEX_ERROR)
)

// Params mirrors InputParameters.InputParameters2D plus the arithmetic mode.
type Params struct {
	N                             int
	CFL, FinalTime, Minf, Gamma   float64
	Alpha, Kappa                  float64
	MaxIterations                 int
	FluxType, InitType, Limiter   int // GCFD_FLUX_*, GCFD_INIT_*, GCFD_LIMITER_*
	LocalTimeStepping             bool
	Precision                     int
	VortexX0, VortexY0            float64
	Device                        int
}

// Context is one device-resident solver.
type Context struct {
	ctx *C.gcfd_ctx
}

func status(ctx *C.gcfd_ctx, rc C.int) error {
	if rc == C.GCFD_OK {
		return nil
	}
	return fmt.Errorf("gcfd: status %d: %s", int(rc), C.GoString(C.gcfd_last_error(ctx)))
}

// New replaces Euler2D.NewEuler's set-up: vertices, 0-based element table
// (K x 3, row-major) and the boundary edges as (v1, v2, BCFLAG) triples.
func New(vx, vy []float64, etov []int32, bcV1, bcV2, bcFlag []int32, p Params) (*Context, error) {
	var pin runtime.Pinner
	defer pin.Unpin()
	m := C.gcfd_mesh{
		nverts: C.int32_t(len(vx)), vx: (*C.double)(unsafe.Pointer(&vx[0])),
		vy: (*C.double)(unsafe.Pointer(&vy[0])),
		K:  C.int32_t(len(etov) / 3), etov: (*C.int32_t)(unsafe.Pointer(&etov[0])),
		nbc: C.int32_t(len(bcFlag)),
	}
	if len(bcFlag) > 0 {
		m.bc_v1 = (*C.int32_t)(unsafe.Pointer(&bcV1[0]))
		m.bc_v2 = (*C.int32_t)(unsafe.Pointer(&bcV2[0]))
		m.bc_flag = (*C.int32_t)(unsafe.Pointer(&bcFlag[0]))
	}
	pin.Pin(&vx[0])
	pin.Pin(&vy[0])
	pin.Pin(&etov[0])
	if len(bcFlag) > 0 {
		pin.Pin(&bcV1[0])
		pin.Pin(&bcV2[0])
		pin.Pin(&bcFlag[0])
	}
	lts := 0
	if p.LocalTimeStepping {
		lts = 1
	}
	cp := C.gcfd_params{
		N: C.int32_t(p.N), cfl: C.double(p.CFL), final_time: C.double(p.FinalTime),
		minf: C.double(p.Minf), gamma: C.double(p.Gamma), alpha: C.double(p.Alpha),
		kappa: C.double(p.Kappa), max_iterations: C.int32_t(p.MaxIterations),
		flux_type: C.int32_t(p.FluxType), init_type: C.int32_t(p.InitType),
		limiter: C.int32_t(p.Limiter), local_time_stepping: C.int32_t(lts),
		precision: C.int32_t(p.Precision), vortex_x0: C.double(p.VortexX0),
		vortex_y0: C.double(p.VortexY0), device: C.int32_t(p.Device),
	}
	c := &Context{}
	if err := status(nil, C.gcfd_create(&m, &cp, &c.ctx)); err != nil {
		return nil, err
	}
	runtime.SetFinalizer(c, (*Context).Close)
	return c, nil
}

// Close releases the device context.
func (c *Context) Close() {
	if c.ctx != nil {
		C.gcfd_destroy(c.ctx)
		c.ctx = nil
	}
}

// shardTable pins the shards' Np x Kmax data and builds the C pointer table
// Q[np*4 + n] the ABI expects; free() must be called after the C call.
func shardTable(pin *runtime.Pinner, Q [][4][]float64) (**C.double, *C.int32_t, func()) {
	ns := len(Q)
	tab := (*[1 << 28]*C.double)(C.malloc(C.size_t(ns*4) * C.size_t(unsafe.Sizeof(uintptr(0)))))[: ns*4 : ns*4]
	km := (*[1 << 28]C.int32_t)(C.malloc(C.size_t(ns) * 4))[:ns:ns]
	for np := range Q {
		for n := 0; n < 4; n++ {
			pin.Pin(&Q[np][n][0])
			tab[np*4+n] = (*C.double)(unsafe.Pointer(&Q[np][n][0]))
		}
	}
	return &tab[0], &km[0], func() {
		C.free(unsafe.Pointer(&tab[0]))
		C.free(unsafe.Pointer(&km[0]))
	}
}

// SetState copies the reference's sharded c.Q (Np x Kmax[np] per variable).
func (c *Context) SetState(Q [][4][]float64, Kmax []int) error {
	var pin runtime.Pinner
	defer pin.Unpin()
	tab, km, free := shardTable(&pin, Q)
	defer free()
	kmS := unsafe.Slice(km, len(Kmax))
	for i, k := range Kmax {
		kmS[i] = C.int32_t(k)
	}
	return status(c.ctx, C.gcfd_set_state(c.ctx, C.int32_t(len(Q)), km, tab))
}

// GetState copies the device state back into the sharded c.Q.
func (c *Context) GetState(Q [][4][]float64, Kmax []int) error {
	var pin runtime.Pinner
	defer pin.Unpin()
	tab, km, free := shardTable(&pin, Q)
	defer free()
	kmS := unsafe.Slice(km, len(Kmax))
	for i, k := range Kmax {
		kmS[i] = C.int32_t(k)
	}
	return status(c.ctx, C.gcfd_get_state(c.ctx, C.int32_t(len(Q)), km, tab))
}

// Step replaces RungeKutta5SSP.Step plus Solve's Time += GlobalDT; it returns
// the time, the last global dt and the signed max of the final increment per
// variable (PrintUpdate's residuals).
func (c *Context) Step(nsteps int) (time, dt float64, resid [4]float64, err error) {
	var t, d C.double
	var r [4]C.double
	err = status(c.ctx, C.gcfd_step(c.ctx, C.int32_t(nsteps), &t, &d, &r[0], nil, nil))
	for i := range r {
		resid[i] = float64(r[i])
	}
	return float64(t), float64(d), resid, err
}

// SetTime sets the solver time (RungeKutta5SSP.Time, euler.go:332), e.g. on a
// restart; the IVortex boundaries and the FinalTime clip read it.
func (c *Context) SetTime(t float64) error {
	return status(c.ctx, C.gcfd_set_time(c.ctx, C.double(t)))
}

// Time returns the solver time and the number of steps taken.
func (c *Context) Time() (t float64, steps int, err error) {
	var tt C.double
	var n C.int32_t
	err = status(c.ctx, C.gcfd_get_time(c.ctx, &tt, &n))
	return float64(tt), int(n), err
}

// SetStagePipeline selects the mixed path's persistent TMA-pipelined stage
// kernel (true) or the one-block kernel (false, the default);
// GCFD_OPT_STAGE_PIPELINE of gcfd.h.
func (c *Context) SetStagePipeline(on bool) error {
	v := C.int32_t(0)
	if on {
		v = 1
	}
	return status(c.ctx, C.gcfd_set_option(c.ctx, C.GCFD_OPT_STAGE_PIPELINE, v))
}

// WindowTaped reports whether the last Forward (gcfd_record_steps) kept every
// step's tape while recording, so Backward recomputes nothing
// (GCFD_OPT_WINDOW_TAPED of gcfd.h).
func (c *Context) WindowTaped() (bool, error) {
	var v C.int32_t
	err := status(c.ctx, C.gcfd_get_option(c.ctx, C.GCFD_OPT_WINDOW_TAPED, &v))
	return v != 0, err
}

// RHS evaluates the right-hand side of Q at BC time t into RHS (same shards).
func (c *Context) RHS(t float64, Q, RHS [][4][]float64, Kmax []int) error {
	var pin runtime.Pinner
	defer pin.Unpin()
	tq, km, freeQ := shardTable(&pin, Q)
	defer freeQ()
	tr, _, freeR := shardTable(&pin, RHS)
	defer freeR()
	kmS := unsafe.Slice(km, len(Kmax))
	for i, k := range Kmax {
		kmS[i] = C.int32_t(k)
	}
	return status(c.ctx, C.gcfd_rhs(c.ctx, C.double(t), C.int32_t(len(Q)), km, tq, tr))
}

// kmaxTable fills the C shard-size table that shardTable allocated.
func kmaxTable(km *C.int32_t, Kmax []int) {
	kmS := unsafe.Slice(km, len(Kmax))
	for i, k := range Kmax {
		kmS[i] = C.int32_t(k)
	}
}

// Forward records nsteps steps (Step semantics) with a checkpoint every
// `every` steps, for a following Backward.
func (c *Context) Forward(nsteps, every int) (time, dt float64, err error) {
	var t, d C.double
	err = status(c.ctx, C.gcfd_record_steps(c.ctx, C.int32_t(nsteps), C.int32_t(every), &t, &d))
	return float64(t), float64(d), err
}

// Functional evaluates J on the current state and, with Qbar non-nil, writes
// dJ/dQ into the shards and returns dJ/dtime.
func (c *Context) Functional(kind int, Qbar [][4][]float64, Kmax []int) (J, tbar float64, err error) {
	var j, tb C.double
	if Qbar == nil {
		err = status(c.ctx, C.gcfd_functional(c.ctx, C.int32_t(kind), &j, 0, nil, nil, &tb))
		return float64(j), float64(tb), err
	}
	var pin runtime.Pinner
	defer pin.Unpin()
	tab, km, free := shardTable(&pin, Qbar)
	defer free()
	kmaxTable(km, Kmax)
	err = status(c.ctx, C.gcfd_functional(c.ctx, C.int32_t(kind), &j, C.int32_t(len(Qbar)), km, tab, &tb))
	return float64(j), float64(tb), err
}

// Backward runs the adjoint of the recorded window: from the adjoint of the
// final state (and time) to that of the initial state, the far-field Qinf and
// the initial time.
func (c *Context) Backward(QfinalBar [][4][]float64, tfinalBar float64, Q0Bar [][4][]float64, Kmax []int) (
	qinfBar [4]float64, t0Bar float64, err error) {
	var pin runtime.Pinner
	defer pin.Unpin()
	tf, km, freeF := shardTable(&pin, QfinalBar)
	defer freeF()
	t0, _, free0 := shardTable(&pin, Q0Bar)
	defer free0()
	kmaxTable(km, Kmax)
	var qb [4]C.double
	var tb C.double
	err = status(c.ctx, C.gcfd_step_vjp(c.ctx, C.int32_t(len(QfinalBar)), km, tf, C.double(tfinalBar), t0,
		&qb[0], &tb))
	for i := range qb {
		qinfBar[i] = float64(qb[i])
	}
	return qinfBar, float64(tb), err
}

// RHSBackward is the adjoint of RHS at (Q, t): Qbar = (dRHS/dQ)^T RHSbar.
func (c *Context) RHSBackward(t float64, Q, RHSbar, Qbar [][4][]float64, Kmax []int) (qinfBar [4]float64,
	tbar float64, err error) {
	var pin runtime.Pinner
	defer pin.Unpin()
	tq, km, freeQ := shardTable(&pin, Q)
	defer freeQ()
	tr, _, freeR := shardTable(&pin, RHSbar)
	defer freeR()
	tb, _, freeB := shardTable(&pin, Qbar)
	defer freeB()
	kmaxTable(km, Kmax)
	var qb [4]C.double
	var tt C.double
	err = status(c.ctx, C.gcfd_rhs_vjp(c.ctx, C.double(t), C.int32_t(len(Q)), km, tq, tr, tb, &qb[0], &tt))
	for i := range qb {
		qinfBar[i] = float64(qb[i])
	}
	return qinfBar, float64(tt), err
}

// Periodic boundary flags: a periodic tag's edges carry BCPeriodic (or
// BCPeriodicReversed) with the tag's group in bits 8 and up, e.g.
// PeriodicFlag(BCPeriodic, 1) for the second periodic tag of the mesh.
const (
	BCPeriodic         = int32(C.GCFD_BC_PERIODIC)
	BCPeriodicReversed = int32(C.GCFD_BC_PERIODIC_REVERSED)
)

// PeriodicFlag returns the BC flag of group g of a periodic kind.
func PeriodicFlag(kind int32, g int) int32 { return kind | int32(g)<<8 }

// SamplePoints interpolates the current state at the points (x[p], y[p]):
// q[n][p] for the four variables, and each point's element (the Sod line
// samples of sod_shock_tube.NewSODShockTube / InterpolateFields).
func (c *Context) SamplePoints(x, y []float64) (q [4][]float64, elem []int32, err error) {
	n := len(x)
	if len(y) != n {
		return q, nil, fmt.Errorf("gcfd: SamplePoints: %d x and %d y values", n, len(y))
	}
	flat := make([]float64, 4*n)
	elem = make([]int32, n)
	if n > 0 {
		err = status(c.ctx, C.gcfd_sample_points(c.ctx, C.int32_t(n), (*C.double)(unsafe.Pointer(&x[0])),
			(*C.double)(unsafe.Pointer(&y[0])), (*C.double)(unsafe.Pointer(&flat[0])),
			(*C.int32_t)(unsafe.Pointer(&elem[0]))))
	}
	for v := 0; v < 4; v++ {
		q[v] = flat[v*n : (v+1)*n]
	}
	return q, elem, err
}

// WallPoints returns the wall data OutputFinal writes: coordinates, state and
// pressure at every Wall/Cyl edge point.
func (c *Context) WallPoints() (x, y []float64, q [4][]float64, p []float64, err error) {
	var n C.int32_t
	if err = status(c.ctx, C.gcfd_wall_points(c.ctx, &n, nil, nil, nil, nil)); err != nil || n == 0 {
		return
	}
	m := int(n)
	x, y, p = make([]float64, m), make([]float64, m), make([]float64, m)
	flat := make([]float64, 4*m)
	err = status(c.ctx, C.gcfd_wall_points(c.ctx, &n, (*C.double)(unsafe.Pointer(&x[0])),
		(*C.double)(unsafe.Pointer(&y[0])), (*C.double)(unsafe.Pointer(&flat[0])), (*C.double)(unsafe.Pointer(&p[0]))))
	for v := 0; v < 4; v++ {
		q[v] = flat[v*m : (v+1)*m]
	}
	return
}

// GraphMesh returns the solution output's graph mesh (CreateAVSGraphMesh):
// XY as interleaved float32 pairs, the sub-triangles as int64 point indices
// (the avs TriMesh's XY and TriVerts), and the points per element.
func (c *Context) GraphMesh() (xy []float32, tris [][3]int64, lenElement int, err error) {
	var L, nt, k32 C.int32_t
	if err = status(c.ctx, C.gcfd_graph_mesh(c.ctx, &L, &nt, nil, nil)); err != nil {
		return
	}
	if err = status(c.ctx, C.gcfd_dims(c.ctx, &k32, nil, nil, nil, nil)); err != nil {
		return
	}
	K := int(k32)
	xy = make([]float32, 2*K*int(L))
	tris = make([][3]int64, K*int(nt))
	if K > 0 {
		err = status(c.ctx, C.gcfd_graph_mesh(c.ctx, nil, nil, (*C.float)(unsafe.Pointer(&xy[0])),
			(*C.int64_t)(unsafe.Pointer(&tris[0][0]))))
	}
	return xy, tris, int(L), err
}

// GraphFields evaluates flow functions (the reference's FlowFunction values
// 0..13) at the graph points, K x lenElement float32 per field: the fields
// map AVSFieldWriter.Save takes.
func (c *Context) GraphFields(kinds []int32, lenElement int) (out [][]float32, err error) {
	var k32 C.int32_t
	if err = status(c.ctx, C.gcfd_dims(c.ctx, &k32, nil, nil, nil, nil)); err != nil {
		return
	}
	n := int(k32) * lenElement
	flat := make([]float32, len(kinds)*n)
	if len(kinds) > 0 && n > 0 {
		err = status(c.ctx, C.gcfd_graph_fields(c.ctx, C.int32_t(len(kinds)), (*C.int32_t)(unsafe.Pointer(&kinds[0])),
			(*C.float)(unsafe.Pointer(&flat[0]))))
	}
	out = make([][]float32, len(kinds))
	for f := range kinds {
		out[f] = flat[f*n : (f+1)*n]
	}
	return out, err
}
