"""CPU tests of the product's host side: the C-ABI library loads and exports
every symbol of include/gcfd.h, its FP64 operators match the oracle's
independent construction and the reference's exactness tests, and the host
mirror of the Euler2D interface (inputs, partitions, meshes) behaves as the
reference's.  No GPU compute."""
import os
import re

import numpy as np
import pytest

from conftest import ROOT, fixture
import dfr_ops
from gocfd_gb300 import _lib, meshes
from gocfd_gb300.euler2d import InputParameters2D, PartitionMap, set_parallel_degree
from test_oracle_known_answers import equilateral_triangle, rt_divergence_check


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "gcfd.h")).read()
    return sorted(set(re.findall(r"\b(gcfd_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_every_header_symbol():
    lib = _lib.load()
    syms = header_symbols()
    assert len(syms) >= 14
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(_lib.EXPORTS) == syms


def test_header_builds_as_c_and_a_c_caller_links(tmp_path):
    """include/gcfd.h is plain C (C99, pedantic, no warnings), and a C program
    links against libgcfd.so and gets the documented status codes for invalid
    arguments (checked on the host before any CUDA call)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lib = _lib.load()
    libdir = os.path.dirname(lib._name)
    src = tmp_path / "caller.c"
    src.write_text(r'''
#include "gcfd.h"
#include <stdio.h>
#include <string.h>
int main(void) {
  gcfd_ctx* ctx = NULL;
  gcfd_params p;
  memset(&p, 0, sizeof p);
  if (gcfd_create(NULL, &p, &ctx) != GCFD_ERR_ARG || ctx != NULL) return 1;
  if (strlen(gcfd_last_error(NULL)) == 0) return 2;
  double vx[3] = {0.0, 1.0, 0.0}, vy[3] = {0.0, 0.0, 1.0};
  int32_t etov[3] = {0, 1, 2};
  gcfd_mesh m;
  memset(&m, 0, sizeof m);
  m.nverts = 3; m.K = 0; m.vx = vx; m.vy = vy; m.etov = etov;
  if (gcfd_create(&m, &p, &ctx) != GCFD_ERR_ARG) return 3;       /* K = 0 */
  if (gcfd_step(NULL, 1, NULL, NULL, NULL, NULL, NULL) != GCFD_ERR_ARG) return 4;
  gcfd_destroy(NULL);
  printf("ok: %s\n", gcfd_last_error(NULL));
  return 0;
}
''')
    exe = tmp_path / "caller"
    cmd = [cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I", os.path.join(ROOT, "include"),
           str(src), "-o", str(exe), "-L", libdir, "-l:libgcfd.so", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.startswith("ok:"), (r.returncode, r.stdout, r.stderr)


def test_go_binding_calls_every_entry_a_go_caller_needs():
    """The cgo binding (gocfd_gb300/go/gcfd/gcfd.go) calls every header entry
    but the ones left to other callers (device pointers and streams, the C++
    mesh reader, the allocation-free residual norms, measurement and host
    helpers), and calls nothing the header does not declare."""
    go = open(os.path.join(ROOT, "gocfd_gb300", "go", "gcfd", "gcfd.go")).read()
    called = set(re.findall(r"C\.(gcfd_[a-z0-9_]+)\(", go))
    others = {"gcfd_set_state_device", "gcfd_get_state_device", "gcfd_get_stream", "gcfd_enqueue_steps",
              "gcfd_read_mesh", "gcfd_free_mesh", "gcfd_residual_norms_static", "gcfd_profile_step",
              "gcfd_device_fma_peaks", "gcfd_host_operator", "gcfd_host_graph_element"}
    syms = set(header_symbols())
    assert called <= syms, sorted(called - syms)
    assert syms - others <= called, sorted(syms - others - called)


@pytest.mark.parametrize("N", range(5))
def test_product_operators_match_oracle(N):
    el = dfr_ops.build_element(N)
    I = _lib.host_operator(N, 0)
    D = _lib.host_operator(N, 1)
    Div = _lib.host_operator(N, 2)
    V = _lib.host_operator(N, 3)
    rs = _lib.host_operator(N, 4)
    RS = _lib.host_operator(N, 5)
    assert I.shape == el.FluxEdgeInterp.shape and D.shape == el.DivInt.shape
    assert np.allclose(rs[:, 0], el.r, atol=1e-15) and np.allclose(rs[:, 1], el.s, atol=1e-15)
    assert np.allclose(RS[:, 0], el.R, atol=1e-15) and np.allclose(RS[:, 1], el.S, atol=1e-15)
    assert np.abs(V - el.V).max() < 1e-12
    assert np.abs(I - el.FluxEdgeInterp).max() < 1e-12
    scale = np.abs(el.Div).max()
    # Two constructions of the same RT divergence (different bases): agree to
    # round-off amplified by the conditioning of the point set.
    assert np.abs(D - el.DivInt).max() <= 1e-12 * scale * 10 ** (N == 1) * 10 ** (N == 4)
    assert np.abs(Div - el.Div).max() <= 1e-12 * scale * 10 ** (N == 1) * 10 ** (N == 4)


@pytest.mark.parametrize("angle", [0, 25, 90, 210, 310])
def test_product_rt_divergence_exact(angle):
    el = dfr_ops.build_element(4)
    Div = _lib.host_operator(4, 2)
    VX, VY, EToV = equilateral_triangle(angle)
    geo = dfr_ops.build_geometry(el, VX, VY, EToV, [])
    rt_divergence_check(Div, el, geo)


def test_unsupported_order_is_an_error():
    with pytest.raises(_lib.GcfdError):
        _lib.host_operator(9, 0)


def test_input_parameters_parse():
    txt = """Title: "Test Case"
CFL: 4.00
FluxType: Roe
InitType: IVortex # Can be "Freestream" or "IVortex"
PolynomialOrder: 2
FinalTime: 200
MaxIterations: 10000
Limiter: persson c0
Kappa: 5
LocalTimeStepping: true
PlotFields: [ "mach", "density" ]
"""
    ip = InputParameters2D.parse(txt)
    assert ip.CFL == 4.0 and ip.FluxType == "Roe" and ip.InitType == "IVortex"
    assert ip.PolynomialOrder == 2 and ip.FinalTime == 200 and ip.MaxIterations == 10000
    assert ip.Limiter == "persson c0" and ip.Kappa == 5 and ip.LocalTimeStepping is True
    assert ip.PlotFields == ["mach", "density"]
    assert ip.Gamma == 1.4 and ip.Minf == 0.1  # CLI defaults


@pytest.mark.parametrize("nb,K", [(1, 10), (3, 10), (7, 100), (16, 131072), (5, 3)])
def test_partition_map_split1d(nb, K):
    pm = PartitionMap(nb, K)
    sizes = [pm.bucket_dimension(i) for i in range(nb)]
    assert sum(sizes) == K and max(sizes) - min(sizes) <= 1
    assert pm.Partitions[0][0] == 0 and pm.Partitions[-1][1] == K
    for a, b in zip(pm.Partitions[:-1], pm.Partitions[1:]):
        assert a[1] == b[0]
    rem = K % nb
    assert all(s == K // nb + 1 for s in sizes[:rem])


def test_set_parallel_degree():
    assert set_parallel_degree(4, 100).ParallelDegree == 4
    assert set_parallel_degree(10, 5).ParallelDegree == 1
    assert set_parallel_degree(0, 185 * 1000).ParallelDegree == max(os.cpu_count(), 1000)


def test_mesh_readers_on_reference_fixtures():
    m = meshes.read_mesh(fixture("test_tris_6_nowall.neu"))
    assert m.K == 2 and len(m.VX) == 4 and list(m.EToV[1]) == [0, 2, 3]
    m = meshes.read_mesh(fixture("fstepA001.neu"))
    assert m.K == 381 and {k: len(v) for k, v in m.bc_tags.items()} == {"wall": 55, "inflow": 8, "outflow": 8}
    m = meshes.read_mesh(fixture("vortex-new.su2"))
    assert m.K == 2402 and len(m.VX) == 1267
    with pytest.raises(ValueError):
        meshes.read_mesh("mesh.msh")


@pytest.mark.parametrize("name", sorted(f for f in os.listdir(os.path.join(os.path.dirname(__file__), "fixtures"))
                                        if f.endswith((".neu", ".su2"))))
def test_native_mesh_reader_matches_python_reader(name):
    """gcfd_read_mesh (C++) against the Python readers on every fixture mesh."""
    m = meshes.read_mesh(fixture(name))
    vx, vy, etov, bc = _lib.read_mesh(fixture(name))
    assert np.array_equal(vx, m.VX) and np.array_equal(vy, m.VY)
    assert np.array_equal(etov, m.EToV)
    assert bc == [tuple(int(x) for x in e) for e in m.bc_edges]


def test_native_mesh_reader_written_meshes(tmp_path):
    """Gambit files written for the benchmark meshes (all BC groups, several
    hundred elements) and an SU2 file with dashed marker tags read the same in
    C++ and Python."""
    for name, mesh in (("sod.neu", meshes.sod_channel(20, 3)), ("wedge.neu", meshes.wedge_channel(12, 6))):
        path = str(tmp_path / name)
        meshes.write_gambit(mesh, path)
        m = meshes.read_mesh(path)
        vx, vy, etov, bc = _lib.read_mesh(path)
        assert np.array_equal(vx, m.VX) and np.array_equal(vy, m.VY) and np.array_equal(etov, m.EToV)
        assert bc == [tuple(int(x) for x in e) for e in m.bc_edges] and len(bc) == len(mesh.bc_edges)
    su2 = tmp_path / "tags.su2"
    su2.write_text("% comment\nNDIME= 2\nNELEM= 2\n5 0 1 2 0\n5 0 2 3 1\nNPOIN= 4\n0 0 0\n1 0 1\n1 1 2\n"
                   "0 1 3\nNMARK= 2\nMARKER_TAG= far-upstream\nMARKER_ELEMS= 2\n3 0 1\n3 1 2\n"
                   "MARKER_TAG= Wall-top\nMARKER_ELEMS= 2\n3 2 3\n3 3 0\n")
    vx, vy, etov, bc = _lib.read_mesh(str(su2))
    m = meshes.read_mesh(str(su2))
    assert np.array_equal(etov, m.EToV) and bc == [tuple(int(x) for x in e) for e in m.bc_edges]
    assert [f for (_, _, f) in bc] == [4, 4, 5, 5]


def test_native_mesh_reader_errors(tmp_path):
    with pytest.raises(_lib.GcfdError):
        _lib.read_mesh(str(tmp_path / "mesh.msh"))        # unsupported extension
    with pytest.raises(_lib.GcfdError):
        _lib.read_mesh(str(tmp_path / "missing.neu"))     # no such file
    src = open(fixture("fstepA001.neu")).read()
    bad = tmp_path / "badtag.neu"
    bad.write_text(src.replace("Wall  ", "nosuchbc", 1))
    with pytest.raises(_lib.GcfdError, match="nosuchbc"):
        _lib.read_mesh(str(bad))
    cut = tmp_path / "cut.neu"
    cut.write_text("\n".join(src.splitlines()[:40]))       # truncated
    with pytest.raises(_lib.GcfdError):
        _lib.read_mesh(str(cut))


def test_structured_mesh_is_ccw_and_roundtrips(tmp_path):
    m = meshes.vortex_box(6, jitter=0.1, seed=3)
    v = m.EToV
    x, y = m.VX, m.VY
    area = (x[v[:, 1]] - x[v[:, 0]]) * (y[v[:, 2]] - y[v[:, 0]]) - (x[v[:, 2]] - x[v[:, 0]]) * (y[v[:, 1]] - y[v[:, 0]])
    assert (area > 0).all() and m.K == 72 and len(m.bc_edges) == 24
    p = tmp_path / "box.neu"
    meshes.write_gambit(m, str(p))
    m2 = meshes.read_gambit(str(p))
    assert np.allclose(m.VX, m2.VX, atol=1e-10) and (m.EToV == m2.EToV).all()
    assert sorted(m.bc_edges) == sorted(m2.bc_edges)
    w = meshes.wedge_channel(16, 8)
    v = w.EToV
    area = (w.VX[v[:, 1]] - w.VX[v[:, 0]]) * (w.VY[v[:, 2]] - w.VY[v[:, 0]]) - (w.VX[v[:, 2]] - w.VX[v[:, 0]]) * (w.VY[v[:, 1]] - w.VY[v[:, 0]])
    assert (area > 0).all()


def test_bc_tag_parsing():
    assert meshes.bc_flag("Wall-top") == 5 and meshes.bc_flag("far") == 4
    assert meshes.bc_flag("inflow") == 1 and meshes.bc_flag("Outflow") == 8
    with pytest.raises(ValueError):
        meshes.bc_flag("bogus")


# The reference's own input files (test_cases/Euler2D/*/input*.yaml, copied
# into tests/fixtures/inputs/): every one parses, to the values its live lines
# set (commented alternatives ignored, Go zero values / CLI defaults elsewhere).
REFERENCE_INPUTS = {
    "SU2-naca12_input-base.yaml": dict(CFL=5.0, FluxType="Roe", InitType="Freestream", PolynomialOrder=4,
                                       FinalTime=20.0, Minf=0.8, Alpha=1.25, LocalTimeStepping=True,
                                       MaxIterations=50000, Limiter="PerssonC0", Kappa=4.5,
                                       PlotFields=["mach", "pressure coefficient"]),
    "Wedge_input.yaml": dict(CFL=1.0, FluxType="Roe", InitType="Freestream", PolynomialOrder=7, FinalTime=20.0,
                             Minf=2.0, Alpha=0.0, LocalTimeStepping=True, MaxIterations=15000, Limiter="PerssonC0",
                             Kappa=6.0, PlotFields=["mach"]),
    "isentropic-vortex_input-bench.yaml": dict(CFL=1.0, FluxType="Lax", InitType="IVortex", PolynomialOrder=2,
                                               FinalTime=0.5, LocalTimeStepping=False, MaxIterations=0),
    "isentropic-vortex_input.yaml": dict(CFL=4.0, FluxType="Roe", InitType="IVortex", PolynomialOrder=2,
                                         FinalTime=200.0, MaxIterations=10000),
    "naca_12_input-bench.yaml": dict(CFL=1.0, FluxType="Roe", InitType="Freestream", PolynomialOrder=2,
                                     FinalTime=20.0, Minf=0.3, LocalTimeStepping=True, MaxIterations=100),
    "naca_12_input-wall.yaml": dict(CFL=2.0, FluxType="Roe", InitType="Freestream", PolynomialOrder=0,
                                    FinalTime=20.0, Minf=0.8, Alpha=1.25, LocalTimeStepping=True, MaxIterations=6000,
                                    Limiter="PerssonC0", Kappa=4.5, PlotFields=["mach", "pressure coefficient"]),
    "shock-tube_input-wall.yaml": dict(CFL=5.0, FluxType="Roe", InitType="shocktube", PolynomialOrder=7,
                                       FinalTime=0.2, LocalTimeStepping=False, MaxIterations=80000,
                                       Limiter="persson c0", Kappa=5.0, PlotFields=["mach"]),
}


@pytest.mark.parametrize("name", sorted(REFERENCE_INPUTS))
def test_reference_input_files_parse(name):
    ip = InputParameters2D.from_file(os.path.join(ROOT, "tests", "fixtures", "inputs", name))
    for k, v in REFERENCE_INPUTS[name].items():
        assert getattr(ip, k) == v, (k, getattr(ip, k), v)
    assert ip.Gamma == 1.4
