"""Solution output (gcfd_host_graph_element, gcfd_graph_mesh, gcfd_graph_fields,
gocfd_gb300.output): the graph mesh and fields the reference streams to
meshfile.gobcfd / solutionfile.gobcfd (DG2D/graphics_support.go:43-230,
model_problems/Euler2D/plot.go:14-85).

CPU: the reference element's graph points against the oracle's flux points,
its triangulation (covers the element, Delaunay), the file layouts round trip.
GPU: the graph fields of every flow function against a numpy restatement on
the oracle's operators (FP32 output: 2e-6 relative to each field's largest
value), the graph mesh against the oracle's affine map.
"""
import os

import numpy as np
import pytest

import dfr_ops
from gocfd_gb300 import _lib, meshes, output
from gocfd_gb300.euler2d import Euler, InputParameters2D


def oracle_graph_rs(el):
    """GetRSForGraphMesh (graphics_support.go:130-159) on the oracle's element."""
    vr, vs = [-1.0, 1.0, -1.0], [-1.0, -1.0, 1.0]
    r, s = [], []
    for n in range(3):
        r.append(vr[n])
        s.append(vs[n])
        off = 2 * el.Np + n * el.NpEdge
        r.extend(el.R[off:off + el.NpEdge])
        s.extend(el.S[off:off + el.NpEdge])
    r.extend(el.R[:el.Np])
    s.extend(el.S[:el.Np])
    return np.array(r), np.array(s)


@pytest.mark.parametrize("N", [0, 1, 2, 3, 4])
def test_graph_element_points_and_triangulation(N):
    rs, tris = _lib.graph_element(N)
    el = dfr_ops.build_element(N)
    r, s = oracle_graph_rs(el)
    assert rs.shape == (3 * (el.NpEdge + 1) + el.Np, 2)
    assert np.allclose(rs[:, 0], r, atol=1e-13) and np.allclose(rs[:, 1], s, atol=1e-13)
    a = rs[tris]
    area = 0.5 * ((a[:, 1, 0] - a[:, 0, 0]) * (a[:, 2, 1] - a[:, 0, 1])
                  - (a[:, 1, 1] - a[:, 0, 1]) * (a[:, 2, 0] - a[:, 0, 0]))
    assert area.min() > 0.0                            # counter-clockwise, none degenerate
    assert abs(area.sum() - 2.0) < 1e-12               # covers the reference triangle
    assert set(tris.ravel()) == set(range(len(rs)))    # every graph point is a vertex
    nb = 3 * (el.NpEdge + 1)
    assert len(tris) == 2 * el.Np + nb - 2             # Euler's formula for a triangulated polygon
    # Delaunay: no graph point strictly inside a sub-triangle's circumcircle
    for t in tris:
        (ax, ay), (bx, by), (cx, cy) = rs[t]
        d = 2 * (ax * (by - cy) + bx * (cy - ay) + cx * (ay - by))
        ux = ((ax ** 2 + ay ** 2) * (by - cy) + (bx ** 2 + by ** 2) * (cy - ay) + (cx ** 2 + cy ** 2) * (ay - by)) / d
        uy = ((ax ** 2 + ay ** 2) * (cx - bx) + (bx ** 2 + by ** 2) * (ax - cx) + (cx ** 2 + cy ** 2) * (bx - ax)) / d
        R2 = (ax - ux) ** 2 + (ay - uy) ** 2
        dist2 = (rs[:, 0] - ux) ** 2 + (rs[:, 1] - uy) ** 2
        assert np.all(dist2 >= R2 * (1 - 1e-9))


class _FakeSolver:
    """The two graph calls of a solver, for the file round trip without a GPU."""

    def __init__(self):
        self.K, self.ip = 3, InputParameters2D(PolynomialOrder=1)
        self.mesh = meshes.structured_triangles(1, 1, 0.0, 1.0, 0.0, 1.0, tags=("wall", "far", "wall", "far"))
        rng = np.random.default_rng(0)
        self.xy = rng.standard_normal((self.K * 15, 2)).astype(np.float32)
        self.tris = rng.integers(0, self.K * 15, (self.K * 16, 3))
        self.f = {"Density": rng.standard_normal(self.K * 15).astype(np.float32),
                  "Mach": rng.standard_normal(self.K * 15).astype(np.float32)}

    def graph_mesh(self):
        return self.xy, self.tris

    def graph_fields(self, names):
        return {n: self.f[n] for n in names}


def test_output_files_round_trip(tmp_path):
    s = _FakeSolver()
    mp, sp = os.path.join(tmp_path, "meshfile.gcfd"), os.path.join(tmp_path, "solutionfile.gcfd")
    output.write_mesh(mp, s)
    m = output.read_mesh_file(mp)
    assert m["K"] == 3 and m["len_element"] == 15 and m["ntri_per_element"] == 16
    assert np.array_equal(m["xy"], s.xy) and np.array_equal(m["tris"], s.tris)
    # every boundary edge appears in its tag's runs
    nedge = sum(len(line) - 1 for lines in m["bcs"].values() for line in lines)
    assert nedge == len(s.mesh.bc_edges)
    with output.SolutionWriter(sp, s, ["Density", "Mach"], {"CFL": 1.0, "Solver": "2D Euler"}) as w:
        w.save(10, 0.5)
        w.save(20, 1.0)
    sol = output.read_solution_file(sp)
    assert sol["names"] == ["Density", "Mach"] and sol["metadata"]["CFL"] == 1.0
    assert [fr["iterations"] for fr in sol["frames"]] == [10, 20]
    assert np.array_equal(sol["frames"][1]["fields"]["Mach"], s.f["Mach"])


def oracle_flow(kind, Q, gamma, pinf, qqinf):
    """GetFlowFunctionBase (fluids.go:289-336)."""
    rho, ru, rv, E = Q
    u, v = ru / rho, rv / rho
    U2 = u * u + v * v
    q = 0.5 * rho * U2
    p = (gamma - 1) * (E - q)
    c = np.sqrt(np.abs(gamma * p / rho))
    return {0: rho, 1: ru, 2: rv, 3: E, 4: np.sqrt(U2) / c, 5: p, 6: q, 7: (p - pinf) / qqinf, 8: c,
            9: np.sqrt(U2), 10: u, 11: v, 12: (E + p) / rho, 13: np.log(p) - gamma * np.log(rho)}[kind]


@pytest.mark.gpu
@pytest.mark.parametrize("N", [1, 2, 4])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_graph_fields_against_oracle(N, precision):
    mesh = meshes.structured_triangles(4, 3, 0.0, 2.0, 0.0, 1.0, jitter=0.1, seed=5,
                                       tags=("wall", "far", "wall", "far"))
    ip = InputParameters2D(CFL=0.5, FluxType="roe", InitType="freestream", PolynomialOrder=N, FinalTime=1e9,
                           Minf=0.6, Gamma=1.4, Alpha=10.0)
    el = dfr_ops.build_element(N)
    with Euler(ip, mesh, 1, precision=precision) as g:
        Q = g.get_global_state()
        Q = np.ascontiguousarray(Q * (1.0 + 0.05 * np.random.default_rng(N).uniform(-1, 1, Q.shape)))
        g.set_global_state(Q)
        names = list(Euler.FLOW_FUNCTIONS)
        fields = g.graph_fields(names)
        xy, tris = g.graph_mesh()
        Q = g.get_global_state()
    qinf = np.array([1.0, 0.6 * np.cos(np.radians(10.0)), 0.6 * np.sin(np.radians(10.0)), 0.0])
    # the far-field state of NewFreeStream (fluids.go:245-262): rho = 1, p = 1/gamma
    gamma = 1.4
    pinf = 1.0 / gamma
    qinf[3] = pinf / (gamma - 1) + 0.5 * (qinf[1] ** 2 + qinf[2] ** 2)
    qqinf = 0.5 * (qinf[1] ** 2 + qinf[2] ** 2) / qinf[0]
    r, s = oracle_graph_rs(el)
    G = dfr_ops.vandermonde2d(N, r, s) @ el.Vinv          # GraphInterp, L x Np
    L, E1 = len(r), el.NpEdge + 1
    for name in names:
        f = oracle_flow(Euler.FLOW_FUNCTIONS[name], Q, gamma, pinf, qqinf)   # Np x K
        ref = G @ f                                                        # L x K
        for n in range(3):                                                 # AverageGraphFieldVertices
            iV = n * E1
            iVm = 3 * E1 - 1 if n == 0 else iV - 1
            ref[iV] = 0.5 * (ref[iV + 1] + ref[iVm])
        ref = ref.T.ravel()                                                # element-major
        got = fields[name].astype(np.float64)
        assert got.shape == ref.shape
        assert np.max(np.abs(got - ref)) <= 2e-6 * np.max(np.abs(ref)) + 1e-30, name
    # graph mesh: the affine image of the graph points, the mesh's own vertices
    V = mesh.EToV
    X = 0.5 * (-(r + s)[:, None] * mesh.VX[V[:, 0]][None] + (r + 1)[:, None] * mesh.VX[V[:, 1]][None]
               + (s + 1)[:, None] * mesh.VX[V[:, 2]][None])
    Y = 0.5 * (-(r + s)[:, None] * mesh.VY[V[:, 0]][None] + (r + 1)[:, None] * mesh.VY[V[:, 1]][None]
               + (s + 1)[:, None] * mesh.VY[V[:, 2]][None])
    assert np.allclose(xy[:, 0], X.T.ravel(), atol=1e-6) and np.allclose(xy[:, 1], Y.T.ravel(), atol=1e-6)
    K = mesh.EToV.shape[0]
    assert tris.shape[0] % K == 0 and tris.min() == 0 and tris.max() == K * L - 1


@pytest.mark.gpu
def test_solution_writer_on_a_solver(tmp_path):
    mesh = meshes.vortex_box(8, jitter=0.1)
    ip = InputParameters2D(CFL=0.5, FluxType="roe", InitType="ivortex", PolynomialOrder=2, FinalTime=1e9)
    mp, sp = os.path.join(tmp_path, "m.gcfd"), os.path.join(tmp_path, "s.gcfd")
    with Euler(ip, mesh, 1, precision="fp32", vortex_center=(0.0, 0.0)) as g:
        output.write_mesh(mp, g)
        with output.SolutionWriter(sp, g, ["Density", "Mach"], {"CFL": 1.0}) as w:
            for it in range(3):
                info = g.step(5)
                w.save(5 * (it + 1), info["time"])
        last = g.graph_fields(["Density"])["Density"]
    m = output.read_mesh_file(mp)
    sol = output.read_solution_file(sp)
    assert m["K"] == mesh.EToV.shape[0] and len(sol["frames"]) == 3
    assert np.array_equal(sol["frames"][-1]["fields"]["Density"], last)
    assert np.all(np.isfinite(sol["frames"][-1]["fields"]["Mach"]))
