"""Mesh inputs for the solver: Gambit / SU2 readers with the reference's
conventions, and the structured triangle meshes of the benchmark workloads.

Readers follow readfiles/readGambitGrid.go:21-165,223-363 (first six lines
skipped, 1-based vertices, BC faces as (element, type, face) triples) and
readfiles/readSU2Grid.go:27-177 (NDIME / NELEM / NPOIN / NMARK blocks,
0-based vertices).  BC tags map to flags as types.BCNameMap (types/cfd.go:28-73):
the part of the tag before a '-' selects the flag.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

BC_FLAGS = {
    "inflow": 1, "in": 1, "dirichlet": 2, "slip": 3, "far": 4, "wall": 5, "cyl": 6, "neuman": 7,
    "out": 8, "outflow": 8, "ivortex": 9, "periodic": 10, "periodicreversed": 11,
}


def bc_flag(tag: str) -> int:
    base = tag.strip().lower()
    if "-" in base and base.index("-") > 0:
        base = base[: base.index("-")]
    if base not in BC_FLAGS:
        raise ValueError(f"unable to find BC with base name: [{base}], full tag: [{tag}]")
    return BC_FLAGS[base]


PERIODIC_FLAGS = (10, 11)


@dataclass
class Mesh:
    VX: np.ndarray                 # Nv
    VY: np.ndarray
    EToV: np.ndarray               # K x 3, int32, 0-based
    bc_edges: list = field(default_factory=list)   # (v1, v2, flag); periodic flags | group << 8
    bc_tags: dict = field(default_factory=dict)    # tag -> list of (v1, v2)
    periodic_tags: list = field(default_factory=list)  # group -> periodic tag

    @property
    def K(self) -> int:
        return int(self.EToV.shape[0])

    def bc_arrays(self):
        if not self.bc_edges:
            z = np.zeros(0, np.int32)
            return z, z, z
        a = np.asarray(self.bc_edges, dtype=np.int32)
        return (np.ascontiguousarray(a[:, 0]), np.ascontiguousarray(a[:, 1]),
                np.ascontiguousarray(a[:, 2]))


def _add_bc(mesh: Mesh, tag: str, pairs):
    flag = bc_flag(tag)
    low = tag.strip().lower()
    if flag in PERIODIC_FLAGS:
        # one group per periodic tag (the reference's BCMAP is keyed by the full tag, types/cfd.go:43)
        if low not in mesh.periodic_tags:
            mesh.periodic_tags.append(low)
        flag |= mesh.periodic_tags.index(low) << 8
    mesh.bc_tags.setdefault(low, []).extend(pairs)
    mesh.bc_edges.extend((int(a), int(b), flag) for a, b in pairs)


def read_gambit(path: str) -> Mesh:
    with open(path) as f:
        lines = f.read().splitlines()
    pos = 6
    Nv, K, Nmats, Nbcs, Nsd = (int(v) for v in lines[pos].split()[:5])
    if Nsd != 2:
        raise ValueError("only 2D Gambit meshes are supported")
    pos += 3
    VX, VY = np.zeros(Nv), np.zeros(Nv)
    for i in range(Nv):
        t = lines[pos + i].split()
        ind = int(t[0]) - 1
        VX[ind], VY[ind] = float(t[1]), float(t[2])
    pos += Nv + 2
    EToV = np.zeros((K, 3), np.int32)
    for i in range(K):
        t = lines[pos + i].split()
        EToV[int(t[0]) - 1] = [int(t[3]) - 1, int(t[4]) - 1, int(t[5]) - 1]
    pos += K + 2
    mesh = Mesh(VX, VY, EToV)
    for _ in range(Nmats):
        nel = int(lines[pos].split("ELEMENTS:")[1].split()[0])
        pos += 3 + (nel + 9) // 10 + 2
    for b in range(Nbcs):
        if b != 0:
            pos += 1
        head = lines[pos].split()
        tag = head[0]
        nfaces = int(head[3]) if tag.lower() == "cyl" and len(head) > 3 else int(head[2])
        pos += 1
        pairs = []
        for i in range(nfaces):
            t = lines[pos + i].split()
            k, face = int(t[0]) - 1, int(t[2])
            v = EToV[k]
            pairs.append(((v[0], v[1]), (v[1], v[2]), (v[2], v[0]))[face - 1])
        pos += nfaces + 1
        _add_bc(mesh, tag, pairs)
    return mesh


def read_su2(path: str) -> Mesh:
    with open(path) as f:
        lines = [ln.strip() for ln in f.read().splitlines()]
    lines = [ln for ln in lines if ln and not ln.startswith("%")]
    pos = 0

    def token():
        nonlocal pos
        ln = lines[pos]
        pos += 1
        if "=" not in ln:
            raise ValueError(f"badly formed input line [{ln}], should have an =")
        return ln.split("=", 1)[1].strip()

    ndim = int(token())
    if ndim != 2:
        raise ValueError("only 2D SU2 meshes are supported")
    K = int(token())
    EToV = np.zeros((K, 3), np.int32)
    for k in range(K):
        t = lines[pos + k].split()
        if int(t[0]) != 5:
            raise ValueError("unable to deal with non-triangular elements right now")
        EToV[k] = [int(t[1]), int(t[2]), int(t[3])]
    pos += K
    Nv = int(token())
    VX, VY = np.zeros(Nv), np.zeros(Nv)
    for i in range(Nv):
        t = lines[pos + i].split()
        VX[i], VY[i] = float(t[0]), float(t[1])
    pos += Nv
    mesh = Mesh(VX, VY, EToV)
    nmark = int(token())
    for _ in range(nmark):
        tag = token().split()[0]
        ne = int(token())
        pairs = []
        for i in range(ne):
            t = lines[pos + i].split()
            if int(t[0]) != 3:
                raise ValueError("BCs should only contain line elements in 2D")
            pairs.append((int(t[1]), int(t[2])))
        pos += ne
        _add_bc(mesh, tag, pairs)
    return mesh


def read_mesh(path: str) -> Mesh:
    """Dispatch on the extension like getFileTypeFromExtension (dfr_startup.go:184-204)."""
    p = path.strip()
    if p.endswith(".neu"):
        return read_gambit(p)
    if p.endswith(".su2"):
        return read_su2(p)
    raise ValueError(f"unsupported file type: {path}")


def structured_triangles(nx: int, ny: int, x0: float, x1: float, y0: float, y1: float, *,
                         jitter: float = 0.0, seed: int = 0, ymap=None,
                         tags=("wall", "wall", "wall", "wall")) -> Mesh:
    """nx x ny quads on [x0,x1] x [y0,y1], each split along its lower-left to
    upper-right diagonal into two counter-clockwise triangles, numbered quad
    by quad (row-major, x fastest).  Interior nodes move by U(-jitter*h, +jitter*h)
    in x and y from numpy's PCG64 stream seeded with `seed`.  `ymap(x, eta)`
    optionally maps the unit-height column to physical y.  tags = BC tags of the
    (bottom, right, top, left) sides."""
    xs = np.linspace(x0, x1, nx + 1)
    etas = np.linspace(0.0, 1.0, ny + 1)
    X, E = np.meshgrid(xs, etas)          # (ny+1, nx+1)
    if ymap is None:
        Y = y0 + (y1 - y0) * E
    else:
        Y = ymap(X, E)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        hx, hy = (x1 - x0) / nx, (y1 - y0) / ny
        dx = rng.uniform(-1.0, 1.0, size=X.shape) * jitter * hx
        dy = rng.uniform(-1.0, 1.0, size=X.shape) * jitter * hy
        interior = np.zeros(X.shape, bool)
        interior[1:-1, 1:-1] = True
        X = np.where(interior, X + dx, X)
        Y = np.where(interior, Y + dy, Y)
    VX, VY = X.reshape(-1).copy(), Y.reshape(-1).copy()
    vid = np.arange((nx + 1) * (ny + 1), dtype=np.int64).reshape(ny + 1, nx + 1)
    a = vid[:-1, :-1].reshape(-1)
    b = vid[:-1, 1:].reshape(-1)
    c = vid[1:, 1:].reshape(-1)
    d = vid[1:, :-1].reshape(-1)
    tri = np.empty((a.size, 2, 3), np.int64)
    tri[:, 0] = np.stack([a, b, c], 1)
    tri[:, 1] = np.stack([a, c, d], 1)
    EToV = tri.reshape(-1, 3).astype(np.int32)
    mesh = Mesh(VX, VY, EToV)
    bottom = [(vid[0, i], vid[0, i + 1]) for i in range(nx)]
    right = [(vid[j, nx], vid[j + 1, nx]) for j in range(ny)]
    top = [(vid[ny, i + 1], vid[ny, i]) for i in range(nx)]
    left = [(vid[j + 1, 0], vid[j, 0]) for j in range(ny)]
    for tag, pairs in zip(tags, (bottom, right, top, left)):
        if tag:
            _add_bc(mesh, tag, pairs)
    return mesh


# --- The benchmark workloads (synthetic inputs with the named shapes) ---------

def vortex_box(n: int, *, jitter: float = 0.0, seed: int = 0) -> Mesh:
    """[-5,5]^2 with n x n quads, all sides tagged wall (-> IVortex BCs)."""
    return structured_triangles(n, n, -5.0, 5.0, -5.0, 5.0, jitter=jitter, seed=seed)


def periodic_box(n: int, *, L: float = 10.0, jitter: float = 0.0, seed: int = 0) -> Mesh:
    """[-L/2, L/2]^2 with n x n quads, periodic in x (tag periodic-1: the right
    side's edges, then the left side's, both listed bottom to top) and in y
    (periodic-2: bottom, then top, both left to right), so NewTriangulation's
    pairing matches edges at the same y (x).  Boundary nodes are not jittered."""
    return structured_triangles(n, n, -0.5 * L, 0.5 * L, -0.5 * L, 0.5 * L, jitter=jitter, seed=seed,
                                tags=("periodic-2", "periodic-1", "periodic-2", "periodic-1"))


def sod_channel(nx: int = 2000, ny: int = 100) -> Mesh:
    """[0,1] x [0,0.05]: inflow left, outflow right, walls top and bottom."""
    return structured_triangles(nx, ny, 0.0, 1.0, 0.0, 0.05, tags=("wall", "out", "wall", "in"))


def wedge_channel(nx: int = 512, ny: int = 256, angle_deg: float = 15.0, ramp_x: float = 0.5) -> Mesh:
    """[0,3] x [0,1] with a compression ramp from x = ramp_x; columns mapped to
    y_b(x) = max(0, x - ramp_x) tan(angle) .. 1.  Inflow/outflow far, walls."""
    t = math.tan(math.radians(angle_deg))

    def ymap(X, E):
        yb = np.maximum(0.0, X - ramp_x) * t
        return yb + E * (1.0 - yb)

    return structured_triangles(nx, ny, 0.0, 3.0, 0.0, 1.0, ymap=ymap, tags=("wall", "far", "wall", "far"))


def write_gambit(mesh: Mesh, path: str):
    """Gambit neutral file readable by readfiles.ReadGambit2d."""
    K, Nv = mesh.K, len(mesh.VX)
    groups = {}
    for (a, b, f) in mesh.bc_edges:
        groups.setdefault(f, []).append((a, b))
    face_of = {}
    for k in range(K):
        v = mesh.EToV[k]
        for fidx, (p, q) in enumerate(((v[0], v[1]), (v[1], v[2]), (v[2], v[0]))):
            face_of[(min(p, q), max(p, q))] = (k, fidx)
    names = {v: k for k, v in BC_FLAGS.items() if k not in ("inflow", "outflow")}
    for g, tag in enumerate(mesh.periodic_tags):
        names[bc_flag(tag) | (g << 8)] = tag
    with open(path, "w") as f:
        f.write("CONTROL INFO 2.0.0\n** GAMBIT NEUTRAL FILE\ngcfd\nPROGRAM: gcfd\nDATE\n")
        f.write("     NUMNP     NELEM     NGRPS    NBSETS     NDFCD     NDFVL\n")
        f.write(f"{Nv:10d}{K:10d}{1:10d}{len(groups):10d}{2:10d}{2:10d}\nENDOFSECTION\n")
        f.write("   NODAL COORDINATES 2.0.0\n")
        for i in range(Nv):
            f.write(f"{i + 1:10d}{mesh.VX[i]:20.11e}{mesh.VY[i]:20.11e}\n")
        f.write("ENDOFSECTION\n      ELEMENTS/CELLS 2.0.0\n")
        for k in range(K):
            v = mesh.EToV[k] + 1
            f.write(f"{k + 1:8d} {3:2d} {3:2d} {v[0]:8d}{v[1]:8d}{v[2]:8d}\n")
        f.write("ENDOFSECTION\n       ELEMENT GROUP 2.0.0\n")
        f.write(f"GROUP:{1:12d} ELEMENTS:{K:11d} MATERIAL:{1.0:11.3f} NFLAGS:{0:11d}\n")
        f.write("                  epsilon: 1.000\n       0\n")
        ids = np.arange(1, K + 1)
        for i in range(0, K, 10):
            f.write("".join(f"{v:8d}" for v in ids[i:i + 10]) + "\n")
        f.write("ENDOFSECTION\n")
        for flag, pairs in groups.items():
            f.write(" BOUNDARY CONDITIONS 2.0.0\n")
            f.write(f"{names[flag]:>32s}{1:8d}{len(pairs):8d}{0:8d}{0:8d}\n")
            for (a, b) in pairs:
                k, fidx = face_of[(min(a, b), max(a, b))]
                f.write(f"{k + 1:10d}{3:5d}{fidx + 1:5d}\n")
            f.write("ENDOFSECTION\n")
