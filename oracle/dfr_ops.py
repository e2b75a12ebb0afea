"""ORACLE (test infrastructure only): numpy restatement of gocfd's DFR element
operators, mesh topology and FP64 geometry.

Only tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may use this module, as the checker.  It is deliberately written
independently of the product library: the RT divergence here follows the
reference's own basis (RTBasisSimplex with the Lagrange-type polynomial
multipliers) rather than the product's monomial-extended basis, so the two
constructions cross-check each other.

Reference sources restated (paths inside Notargets/gocfd):
  DG1D/elements.go:249-328                      JacobiP, GradJacobiP, Vandermonde1D
  DG2D/basis_polynomials.go:19-153,192-214,266-312  Dubiner basis, interp matrix
  DG2D/nodes2d_williams_shunn_jameson.go:151-171 barycentric -> (r,s)
  DG2D/lagrange_element.go:54-92                 solution element, mass matrix
  DG2D/raviart_thomas_element.go:192-297,377-400,429-496  RT element
  DG2D/rt_basis_simplex.go:17-273                RT basis functions
  DG2D/dfr_startup.go:43-65,89-147,256-314       DFR2D, geometry, normals, hK
  DG2D/triangulation.go:19-171,230-235           edges, IInII, orientation
  DG2D/dfr_shock_capturing.go:43-140             filter, clipper, sensor matrices
  DG2D/element_utils.go:163-175                  element-local coordinates
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from wsj_nodes import WSJ

# ----------------------------------------------------------------------------
# 1D / 2D orthonormal polynomials (DG1D/elements.go:257-328,
# DG2D/basis_polynomials.go:72-153)


def _gamma0(a, b):
    return 2.0 ** (a + b + 1) / (a + b + 1) * math.gamma(a + 1) * math.gamma(b + 1) / math.gamma(a + b + 1)


def jacobi_p(x, alpha, beta, n):
    x = np.asarray(x, dtype=np.float64)
    g0 = _gamma0(alpha, beta)
    p0 = np.full_like(x, 1.0 / math.sqrt(g0))
    if n == 0:
        return p0
    g1 = (alpha + 1) * (beta + 1) / (alpha + beta + 3) * g0
    p1 = ((alpha + beta + 2) * x / 2 + (alpha - beta) / 2) / math.sqrt(g1)
    if n == 1:
        return p1
    ab = alpha + beta
    aold = 2.0 * math.sqrt((alpha + 1) * (beta + 1) / (ab + 3.0)) / (ab + 2.0)
    for i in range(n - 1):
        ip1 = i + 1.0
        ip2 = ip1 + 1.0
        h1 = 2.0 * ip1 + ab
        anew = 2.0 / (h1 + 2.0) * math.sqrt(ip2 * (ip1 + ab + 1) * (ip1 + alpha + 1) * (ip1 + beta + 1) / (h1 + 1.0) / (h1 + 3.0))
        bnew = -(alpha * alpha - beta * beta) / h1 / (h1 + 2.0)
        p2 = (-aold * p0 + (x - bnew) * p1) / anew
        p0, p1, aold = p1, p2, anew
    return p1


def grad_jacobi_p(x, alpha, beta, n):
    x = np.asarray(x, dtype=np.float64)
    if n == 0:
        return np.zeros_like(x)
    return jacobi_p(x, alpha + 1, beta + 1, n - 1) * math.sqrt(n * (n + alpha + beta + 1))


def _rs_to_ab(r, s):
    r = np.asarray(r, dtype=np.float64)
    s = np.asarray(s, dtype=np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        a = np.where(s != 1.0, 2.0 * (1.0 + r) / (1.0 - s) - 1.0, -1.0)
    return a, s.copy()


def simplex2d_p(r, s, i, j):
    a, b = _rs_to_ab(r, s)
    h1 = jacobi_p(a, 0, 0, i)
    h2 = jacobi_p(b, 2 * i + 1, 0, j)
    return math.sqrt(2.0) * h1 * h2 * (1.0 - b) ** i


def grad_simplex2d_p(r, s, i, j):
    a, b = _rs_to_ab(r, s)
    fa = jacobi_p(a, 0, 0, i)
    dfa = grad_jacobi_p(a, 0, 0, i)
    gb = jacobi_p(b, 2 * i + 1, 0, j)
    dgb = grad_jacobi_p(b, 2 * i + 1, 0, j)
    ddr = dfa * gb
    if i > 0:
        ddr = ddr * (0.5 * (1 - b)) ** (i - 1)
    ddr = ddr * 2.0 ** (i + 0.5)
    dds = 0.5 * dfa * gb * (1 + a)
    if i > 0:
        dds = dds * (0.5 * (1 - b)) ** (i - 1)
    tmp = dgb * (0.5 * (1 - b)) ** i
    if i > 0:
        tmp = tmp - 0.5 * i * gb * (0.5 * (1 - b)) ** (i - 1)
    dds = (dds + fa * tmp) * 2.0 ** (i + 0.5)
    return ddr, dds


def mode_list(N):
    return [(i, j) for i in range(N + 1) for j in range(N - i + 1)]


def vandermonde2d(N, r, s):
    return np.stack([simplex2d_p(r, s, i, j) for (i, j) in mode_list(N)], axis=1)


def grad_vandermonde2d(N, r, s):
    cols = [grad_simplex2d_p(r, s, i, j) for (i, j) in mode_list(N)]
    return np.stack([c[0] for c in cols], axis=1), np.stack([c[1] for c in cols], axis=1)


def wsj_points(N):
    """Solution points (r, s, w) of order N (nodes2d_williams_shunn_jameson.go:151-171)."""
    t = np.array(WSJ[N], dtype=np.float64)
    r = -t[:, 0] + t[:, 1] - t[:, 2]
    s = -t[:, 0] - t[:, 1] + t[:, 2]
    return r, s, t[:, 3].copy()


OPTIMIZED_EDGE_POINTS = {  # raviart_thomas_element.go:377-400, keyed by RT order P
    1: [-0.38490018, 0.38490018],
    2: [-0.028, 0.000, 0.028],
    3: [-0.482, -0.161, 0.161, 0.482],
    4: [-0.586, -0.293, 0.000, 0.293, 0.586],
    5: [-0.634, -0.381, -0.127, 0.127, 0.381, 0.634],
    6: [-0.671, -0.452, -0.219, 0.000, 0.219, 0.452, 0.671],
    7: [-0.808, -0.578, -0.343, -0.113, 0.113, 0.343, 0.578, 0.808],
    8: [-0.692, -0.523, -0.350, -0.176, 0.000, 0.176, 0.350, 0.523, 0.692],
}


# ----------------------------------------------------------------------------
# Raviart-Thomas element with the reference's simplex RT basis


def rt_element(P):
    """Returns (R, S, Div) of NewRTElement(P, SimplexRTBasis)
    (raviart_thomas_element.go:192-249, rt_basis_simplex.go:17-194)."""
    Np = (P + 1) * (P + 3)
    NpInt = P * (P + 1) // 2
    NpEdge = P + 1
    rI, sI, _ = wsj_points(P - 1)
    gp = np.array(OPTIMIZED_EDGE_POINTS[P], dtype=np.float64)
    # ExtendGeomToRT (raviart_thomas_element.go:429-496)
    gpT = 0.5 * (gp + 1.0)
    R = np.concatenate([rI, rI, gp, 1 - 2 * gpT, -np.ones(NpEdge)])
    S = np.concatenate([sI, sI, -np.ones(NpEdge), -1 + 2 * gpT, -gp])
    oosr2 = 0.5 * math.sqrt(2.0)
    B = np.zeros((Np, 2))
    B[:NpInt] = (1, 0)
    B[NpInt:2 * NpInt] = (0, 1)
    B[2 * NpInt:2 * NpInt + NpEdge] = (0, -1)
    B[2 * NpInt + NpEdge:2 * NpInt + 2 * NpEdge] = (oosr2, oosr2)
    B[2 * NpInt + 2 * NpEdge:] = (-1, 0)

    # PKBasis: Lagrange polynomials through the interior points, degree P-1
    # (GetOrthogonalPolynomialAtJ = sum_i Simplex2DP_i * Vinv[i, j]).
    Vpk_inv = np.linalg.inv(vandermonde2d(P - 1, rI, sI))
    # PEdgeBasis: 1D Lagrange polynomials through the edge parameters, degree P.
    V1 = np.stack([jacobi_p(gp, 0, 0, j) for j in range(P + 1)], axis=1)
    V1_inv = np.linalg.inv(V1)

    def pk_eval(r, s, j):
        return vandermonde2d(P - 1, r, s) @ Vpk_inv[:, j]

    def pk_grad(r, s, j):
        Vr, Vs = grad_vandermonde2d(P - 1, r, s)
        return Vr @ Vpk_inv[:, j], Vs @ Vpk_inv[:, j]

    def e1d_eval(t, j):
        return np.stack([jacobi_p(t, 0, 0, i) for i in range(P + 1)], axis=1) @ V1_inv[:, j]

    def e1d_deriv(t, j):
        return np.stack([grad_jacobi_p(t, 0, 0, i) for i in range(P + 1)], axis=1) @ V1_inv[:, j]

    r, s = R, S
    Phi = np.zeros((Np, Np, 2))   # [point, function, component]
    Dphi = np.zeros((Np, Np))      # divergence [point, function]
    sr2 = math.sqrt(2.0)
    for j in range(Np):
        if j < 2 * NpInt:
            if j < NpInt:  # E4
                jj = j
                base = np.stack([0.5 * (s + 1) * 0.5 * (r + 1), 0.5 * (s + 1) * 0.5 * (s - 1)], axis=1)
                bdiv = (3.0 * s + 1.0) / 4.0
            else:  # E5
                jj = j - NpInt
                base = np.stack([0.5 * (r + 1) * 0.5 * (r - 1), 0.5 * (r + 1) * 0.5 * (s + 1)], axis=1)
                bdiv = (3.0 * r + 1.0) / 4.0
            pv = pk_eval(r, s, jj)
            gr, gs = pk_grad(r, s, jj)
        else:
            je = j - 2 * NpInt
            if je < NpEdge:  # E1, bottom: parameter r
                base = np.stack([0.5 * (r + 1), 0.5 * (s - 1)], axis=1)
                bdiv = np.ones_like(r)
                pv = e1d_eval(r, je)
                gr, gs = e1d_deriv(r, je), np.zeros_like(r)
            elif je < 2 * NpEdge:  # E2, hypotenuse: parameter s
                base = np.stack([sr2 * 0.5 * (r + 1), sr2 * 0.5 * (s + 1)], axis=1)
                bdiv = np.full_like(r, sr2)
                pv = e1d_eval(s, je - NpEdge)
                gr, gs = np.zeros_like(r), e1d_deriv(s, je - NpEdge)
            else:  # E3, left: parameter -s
                base = np.stack([0.5 * (r - 1), 0.5 * (s + 1)], axis=1)
                bdiv = np.ones_like(r)
                pv = e1d_eval(-s, je - 2 * NpEdge)
                gr, gs = np.zeros_like(r), -e1d_deriv(-s, je - 2 * NpEdge)
        Phi[:, j, :] = base * pv[:, None]
        Dphi[:, j] = pv * bdiv + base[:, 0] * gr + base[:, 1] * gs
    V = np.einsum("pjc,pc->pj", Phi, B)
    Div = Dphi @ np.linalg.inv(V)
    return R, S, Div


# ----------------------------------------------------------------------------


def recommended_filter(P):
    if P <= 2:
        return 4.0, 4
    if P == 3:
        return 6.0, 4
    if P == 4:
        return 8.0, 5
    if P == 5:
        return 10.0, 6
    if P == 6:
        return 14.0, 6
    if P == 7:
        return 18.0, 7
    if P == 8:
        return 24.0, 8
    return 30.0 + 2.0 * (P - 9), 8 + (P - 9) // 2


@dataclass
class Element:
    N: int
    Np: int
    NpEdge: int
    NpFlux: int
    r: np.ndarray
    s: np.ndarray
    w: np.ndarray
    R: np.ndarray          # flux-element points
    S: np.ndarray
    V: np.ndarray
    Vinv: np.ndarray
    FluxEdgeInterp: np.ndarray
    Div: np.ndarray
    DivInt: np.ndarray
    MassMatrix: np.ndarray
    Clipper: np.ndarray
    SensD: np.ndarray
    SensP: np.ndarray
    ModeFilter: np.ndarray
    Bary: np.ndarray
    mode_degree: np.ndarray = field(default_factory=lambda: np.zeros(0))


def build_element(N: int) -> Element:
    """NewDFR2D's element part (dfr_startup.go:43-65) plus the shock-finder
    matrices of NewAliasShockFinder (dfr_shock_capturing.go:71-107)."""
    r, s, w = wsj_points(N)
    Np = len(r)
    V = vandermonde2d(N, r, s)
    Vinv = np.linalg.inv(V)
    R, S, Div = rt_element(N + 1)
    NpInt = Np
    NpEdge = N + 2
    Redge, Sedge = R[2 * NpInt:], S[2 * NpInt:]
    FluxEdgeInterp = vandermonde2d(N, Redge, Sedge) @ Vinv
    degs = np.array([i + j for (i, j) in mode_list(N)])
    Mass = V.T @ np.diag(w) @ V
    cut = np.where(degs >= N, 0.0, 1.0)
    Clipper = V @ np.diag(cut) @ Vinv
    D = np.eye(Np) - Clipper
    alpha, sexp = recommended_filter(N)
    mf = np.ones(Np)
    if N > 1:
        mf = np.where(degs == 0, 1.0, np.exp(-alpha * (degs / N) ** sexp))
    # createInterpolationStencil (dissipation.go:414-449)
    RR = np.array([[1.0, 1.0, 1.0], [-1.0, 1.0, -1.0], [-1.0, -1.0, 1.0]])
    Bary = (np.linalg.inv(RR) @ np.stack([np.ones_like(R), R, S])).T
    return Element(N=N, Np=Np, NpEdge=NpEdge, NpFlux=len(R), r=r, s=s, w=w, R=R, S=S, V=V, Vinv=Vinv,
                   FluxEdgeInterp=FluxEdgeInterp, Div=Div, DivInt=Div[:Np].copy(), MassMatrix=Mass,
                   Clipper=Clipper, SensD=D, SensP=Mass @ D, ModeFilter=mf, Bary=Bary, mode_degree=degs)


# ----------------------------------------------------------------------------
# Mesh topology and geometry

BC = {"none": 0, "in": 1, "inflow": 1, "far": 4, "wall": 5, "cyl": 6, "out": 8, "outflow": 8, "ivortex": 9}


@dataclass
class Geometry:
    K: int
    kL: np.ndarray
    eL: np.ndarray
    kR: np.ndarray
    eR: np.ndarray
    bc: np.ndarray
    Jdet: np.ndarray      # K
    Jinv: np.ndarray      # K x 4  [ys, -xs, -yr, xr] / |J|
    nx: np.ndarray        # 3 x K outward unit normals
    ny: np.ndarray
    IInII: np.ndarray     # 3 x K
    EdgeLenMax: np.ndarray
    hK: np.ndarray
    FluxX: np.ndarray     # NpFlux x K
    FluxY: np.ndarray
    SolX: np.ndarray      # Np x K
    SolY: np.ndarray
    EtoEdge: np.ndarray   # K x 3


def _curve(ekeys, edges, reverse):
    """Curve.ReOrder + AssembleCurve (types/elemental.go:141-240): the edges
    as one open chain, starting from the first edge (the last with reverse)."""
    ends_of = {}
    for e in edges:
        for v in (int(ekeys[e]) & 0xFFFFFFFF, int(ekeys[e]) >> 32):
            ends_of.setdefault(v, []).append(e)
    dangling = sorted(v for v, es in ends_of.items() if len(es) == 1)
    if len(dangling) != 2 or any(len(es) > 2 for es in ends_of.values()):
        raise ValueError("periodic edges do not form one open curve")
    start = edges[-1] if reverse else edges[0]
    if all(len(ends_of[v]) == 2 for v in (int(ekeys[start]) & 0xFFFFFFFF, int(ekeys[start]) >> 32)):
        start = ends_of[dangling[0]][0]
    chain = [start]
    verts = (int(ekeys[start]) & 0xFFFFFFFF, int(ekeys[start]) >> 32)
    tip = verts[0] if len(ends_of[verts[0]]) == 2 else verts[1]
    while len(ends_of[tip]) == 2:
        nxt = [e for e in ends_of[tip] if e != chain[-1]][0]
        chain.append(nxt)
        a, b = int(ekeys[nxt]) & 0xFFFFFFFF, int(ekeys[nxt]) >> 32
        tip = b if a == tip else a
    if len(chain) != len(edges):
        raise ValueError("periodic edges do not form one open curve")
    return chain


def _pair_periodic(groups, ekeys, kL, eL, kR, eR, edge_of):
    """Periodic pairing of NewTriangulation (triangulation.go:63-99): per tag,
    the first and second halves of its edge list as curves, edge i of one
    shared with edge i of the other (second element = right side; its edge
    slot points at the shared edge).  Returns the edges that remain."""
    gone = np.zeros(len(ekeys), bool)
    for flag, lst in groups.items():
        if len(lst) % 2:
            raise ValueError("periodic boundaries must be present in pairs")
        h = len(lst) // 2
        c1 = _curve(ekeys, lst[:h], False)
        c2 = _curve(ekeys, lst[h:], (flag & 0xFF) == 11)
        for e1, e2 in zip(c1, c2):
            kR[e1], eR[e1] = kL[e2], eL[e2]
            edge_of[kL[e2] * 3 + eL[e2]] = e1
            gone[e2] = True
    return np.flatnonzero(~gone)


def build_geometry(el: Element, VX, VY, EToV, bc_edges) -> Geometry:
    """NewTriangulation + ProcessGeometry + GetEdgeLengths
    (triangulation.go:19-171, dfr_startup.go:125-175,256-314).

    bc_edges: iterable of (v1, v2, flag)."""
    VX = np.asarray(VX, dtype=np.float64)
    VY = np.asarray(VY, dtype=np.float64)
    EToV = np.asarray(EToV, dtype=np.int64)
    K = EToV.shape[0]
    a = EToV
    b = np.roll(EToV, -1, axis=1)       # edges v0v1, v1v2, v2v0
    lo, hi = np.minimum(a, b), np.maximum(a, b)
    keys = (lo + (hi << 32)).reshape(-1)  # index k*3 + ed
    uniq, first, inv, counts = np.unique(keys, return_index=True, return_inverse=True, return_counts=True)
    if counts.max() > 2:
        raise ValueError("edge shared by more than two triangles")
    # Order edges by first appearance (the left element is the first to create it).
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(len(order))
    edge_of = rank[inv]                   # edge number for each (k, ed)
    nE = len(uniq)
    slots = np.arange(3 * K)
    kL = np.empty(nE, np.int64)
    eL = np.empty(nE, np.int64)
    kR = np.full(nE, -1, np.int64)
    eR = np.full(nE, -1, np.int64)
    firstslot = first[order]
    kL[:] = firstslot // 3
    eL[:] = firstslot % 3
    second = slots[np.ones(3 * K, bool)]
    is_second = np.ones(3 * K, bool)
    is_second[firstslot] = False
    sec = second[is_second]
    kR[edge_of[sec]] = sec // 3
    eR[edge_of[sec]] = sec % 3
    ekeys = uniq[order]
    bcf = np.zeros(nE, np.int64)
    edge_of = edge_of.copy()
    if bc_edges is not None and len(bc_edges):
        lookup = {int(k): i for i, k in enumerate(ekeys)}
        groups = {}
        for (v1, v2, flag) in bc_edges:
            kk = min(v1, v2) + (max(v1, v2) << 32)
            if (flag & 0xFF) in (10, 11):      # BC_Periodic, BC_PeriodicReversed: group in bits 8..
                groups.setdefault(flag, []).append(lookup[kk])
            else:
                bcf[lookup[kk]] = flag
        if groups:
            keep = _pair_periodic(groups, ekeys, kL, eL, kR, eR, edge_of)
            ekeys, kL, eL, kR, eR, bcf = (x[keep] for x in (ekeys, kL, eL, kR, eR, bcf))
            renum = -np.ones(nE, np.int64)
            renum[keep] = np.arange(len(keep))
            edge_of = renum[edge_of]
            nE = len(keep)
    # Jacobian (dfr_startup.go:256-287)
    v1, v2, v3 = EToV[:, 0], EToV[:, 1], EToV[:, 2]
    xr, yr = 0.5 * (VX[v2] - VX[v1]), 0.5 * (VY[v2] - VY[v1])
    xs, ys = 0.5 * (VX[v3] - VX[v1]), 0.5 * (VY[v3] - VY[v1])
    Jdet = xr * ys - xs * yr
    Jinv = np.stack([ys, -xs, -yr, xr], axis=1) / Jdet[:, None]
    # Face normals / IInII per connection (dfr_startup.go:289-314, triangulation.go:149-171, 230-235)
    rev = (a > b).reshape(-1)
    lo_f, hi_f = lo.reshape(-1), hi.reshape(-1)
    pa = np.where(rev, lo_f, hi_f)
    pb = np.where(rev, hi_f, lo_f)
    dx, dy = VX[pb] - VX[pa], VY[pb] - VY[pa]
    ln = np.sqrt(dx * dx + dy * dy)
    ed = slots % 3
    kk_ = slots // 3
    nx = np.zeros((3, K))
    ny = np.zeros((3, K))
    II = np.zeros((3, K))
    nx[ed, kk_] = -dy / ln
    ny[ed, kk_] = dx / ln
    II[ed, kk_] = np.where(ed == 1, ln / (2.0 * math.sqrt(2.0)), ln / 2.0)
    EdgeLenMax = Jdet / II.max(axis=0)
    hK = EdgeLenMax / float((el.N + 1) ** 2)

    def local(R, S):  # element_utils.go:163-175
        X = 0.5 * (np.outer(-(R + S), VX[v1]) + np.outer(R + 1, VX[v2]) + np.outer(S + 1, VX[v3]))
        Y = 0.5 * (np.outer(-(R + S), VY[v1]) + np.outer(R + 1, VY[v2]) + np.outer(S + 1, VY[v3]))
        return X, Y

    FX, FY = local(el.R, el.S)
    SX, SY = local(el.r, el.s)
    return Geometry(K=K, kL=kL, eL=eL, kR=kR, eR=eR, bc=bcf, Jdet=Jdet, Jinv=Jinv, nx=nx, ny=ny, IInII=II,
                    EdgeLenMax=EdgeLenMax, hK=hK, FluxX=FX, FluxY=FY, SolX=SX, SolY=SY,
                    EtoEdge=edge_of.reshape(K, 3))
