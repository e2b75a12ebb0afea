"""Headless solution output: the content of the reference's meshfile.gobcfd /
solutionfile.gobcfd (WriteMesh, AVSFieldWriter: DG2D/graphics_support.go:43-128,
247-314; Solve writes a frame per reporting step, euler.go:190-215) in a
documented little-endian binary layout instead of Go's gob encoding (gob is a
Go-specific self-describing stream; the Go caller keeps its own encoder and
feeds it from gcfd_graph_mesh / gcfd_graph_fields).

Mesh file ("GCFDMESH", version 1):
    u32 version; i32 N, K, len_element, ntri_per_element
    str description                           (u32 byte length + UTF-8)
    f32 XY[K * len_element][2]                graph points (gcfd_graph_mesh)
    i64 tris[K * ntri_per_element][3]         sub-triangles, global point indices
    u32 n_bc; per boundary tag: str name, u32 n_lines, per line u32 n_pts,
        f32 xy[n_pts][2]                      contiguous runs of the tag's edges
                                              (SerializeBCs, plot.go:88-114)
Solution file ("GCFDSOL\\0", version 1):
    u32 version; u32 n_fields; str names[n_fields]; str metadata (JSON:
        CFL, Mesh, Case, Solver, FS Mach as FieldMetadata.SolutionMetadata)
    frames to the end: i32 iterations, f32 time, i32 count, i32 length,
        f32 field[count][length] in the order of names
"""
from __future__ import annotations

import json
import struct

import numpy as np

MESH_MAGIC = b"GCFDMESH"
SOL_MAGIC = b"GCFDSOL\0"
VERSION = 1


def _wstr(f, s: str):
    b = s.encode()
    f.write(struct.pack("<I", len(b)))
    f.write(b)


def _rstr(f) -> str:
    (n,) = struct.unpack("<I", f.read(4))
    return f.read(n).decode()


def bc_polylines(VX, VY, bc_edges, names=None):
    """Boundary edges grouped by tag into contiguous vertex runs (a new run where
    an edge does not start at the previous edge's end), as SerializeBCs does."""
    out = {}
    for v1, v2, flag in bc_edges:
        name = names.get(flag, str(flag)) if names else str(flag)
        runs = out.setdefault(name, [])
        if not runs or runs[-1][-1] != v1:
            runs.append([v1])
        runs[-1].append(v2)
    return {name: [np.stack([VX[r], VY[r]], 1).astype(np.float32) for r in runs] for name, runs in out.items()}


def write_mesh(path: str, solver, description="Hybrid Lagrangian / Raviart Thomas elements", bc_names=None):
    xy, tris = solver.graph_mesh()
    L = xy.shape[0] // solver.K
    nt = tris.shape[0] // solver.K
    bcs = bc_polylines(solver.mesh.VX, solver.mesh.VY, solver.mesh.bc_edges, bc_names)
    with open(path, "wb") as f:
        f.write(MESH_MAGIC)
        f.write(struct.pack("<Iiiii", VERSION, solver.ip.PolynomialOrder, solver.K, L, nt))
        _wstr(f, description)
        f.write(np.ascontiguousarray(xy, dtype="<f4").tobytes())
        f.write(np.ascontiguousarray(tris, dtype="<i8").tobytes())
        f.write(struct.pack("<I", len(bcs)))
        for name, lines in bcs.items():
            _wstr(f, name)
            f.write(struct.pack("<I", len(lines)))
            for line in lines:
                f.write(struct.pack("<I", line.shape[0]))
                f.write(np.ascontiguousarray(line, dtype="<f4").tobytes())


def read_mesh_file(path: str):
    with open(path, "rb") as f:
        assert f.read(8) == MESH_MAGIC
        version, N, K, L, nt = struct.unpack("<Iiiii", f.read(20))
        desc = _rstr(f)
        xy = np.frombuffer(f.read(8 * K * L), dtype="<f4").reshape(K * L, 2)
        tris = np.frombuffer(f.read(24 * K * nt), dtype="<i8").reshape(K * nt, 3)
        (nbc,) = struct.unpack("<I", f.read(4))
        bcs = {}
        for _ in range(nbc):
            name = _rstr(f)
            (nl,) = struct.unpack("<I", f.read(4))
            lines = []
            for _ in range(nl):
                (npts,) = struct.unpack("<I", f.read(4))
                lines.append(np.frombuffer(f.read(8 * npts), dtype="<f4").reshape(npts, 2))
            bcs[name] = lines
    return dict(version=version, N=N, K=K, len_element=L, ntri_per_element=nt, description=desc, xy=xy, tris=tris,
                bcs=bcs)


class SolutionWriter:
    """Frames of flow functions at the graph points (AVSFieldWriter.Save)."""

    def __init__(self, path: str, solver, names, metadata=None):
        self.solver, self.names = solver, list(names)
        self.f = open(path, "wb")
        self.f.write(SOL_MAGIC)
        self.f.write(struct.pack("<II", VERSION, len(self.names)))
        for n in self.names:
            _wstr(self.f, n)
        _wstr(self.f, json.dumps(metadata or {}))

    def save(self, iterations: int, time: float):
        fields = self.solver.graph_fields(self.names)
        length = next(iter(fields.values())).shape[0] if fields else 0
        self.f.write(struct.pack("<ifii", int(iterations), float(time), len(self.names), length))
        for n in self.names:
            self.f.write(np.ascontiguousarray(fields[n], dtype="<f4").tobytes())

    def close(self):
        if self.f:
            self.f.close()
            self.f = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def read_solution_file(path: str):
    with open(path, "rb") as f:
        assert f.read(8) == SOL_MAGIC
        version, nf = struct.unpack("<II", f.read(8))
        names = [_rstr(f) for _ in range(nf)]
        meta = json.loads(_rstr(f))
        frames = []
        while True:
            head = f.read(16)
            if len(head) < 16:
                break
            it, t, count, length = struct.unpack("<ifii", head)
            data = np.frombuffer(f.read(4 * count * length), dtype="<f4").reshape(count, length)
            frames.append(dict(iterations=it, time=t, fields={n: data[i] for i, n in enumerate(names)}))
    return dict(version=version, names=names, metadata=meta, frames=frames)
