"""Test infrastructure only (the oracle): numpy restatement of the
reference's plain full-mesh generators, so that the oracle and the CPU
baseline can build their meshes without the product library.

Follows pressio-demoapps meshing_scripts/create_full_mesh.py (dx = L / N,
info/connectivity/coordinates text written with "%.14f" / "%8d") and the
natural row ordering of meshing_scripts/_impl/one_dim_mesh.py,
natural_order_mesh_2d.py and natural_order_mesh_3d.py:

* cell id = i + Nx (j + Ny k); centre = lower bound + dx/2 + i dx;
* graph row = [cell, layer-1 neighbours, layer-2 neighbours, ...], each
  layer in the scripts' side order: 1D (left, right), 2D (left, front,
  right, back), 3D (left, front, right, back, bottom, top) with
  left/right = -x/+x, back/front = -y/+y, bottom/top = -z/+z;
* a neighbour k cells away on the minus side of index g is g - k when that
  is >= 0, else (periodic axis) g - k + N, else -1; on the plus side g + k
  when <= N - 1, else (periodic) g + k - N, else -1 (the scripts' if-chains,
  _buildGraphStencil3/5/7, spell out these cases one by one).

The mesh reader of the reference parses the text files, so coordinates and
dx are the values "%.14f" prints, read back (mesh_read_coords.hpp,
mesh_read_info.hpp); dxInv = 1 / dx.  The 3D generator is extended to
stencil 7 the same way (the reference script stops at 5).
"""
from __future__ import annotations

import os

import numpy as np

_SIDES = {1: [(0, -1), (0, +1)],
          2: [(0, -1), (1, +1), (0, +1), (1, -1)],
          3: [(0, -1), (1, +1), (0, +1), (1, -1), (2, -1), (2, +1)]}


class FullMesh:
    def __init__(self, dim, stencil, n, graph, x, y, z, dx, bounds):
        self.dim, self.stencil, self.n = dim, stencil, n
        self.graph, self.x, self.y, self.z, self.dx, self.bounds = graph, x, y, z, dx, bounds

    def oracle_mesh(self, orc):
        return orc.mesh_from_arrays(self.dim, self.stencil, self.graph, self.x, self.y, self.z, self.dx)

    def write(self, d):
        """The three files of create_full_mesh.py, byte for byte."""
        os.makedirs(d, exist_ok=True)
        N = self.graph.shape[0]
        lines = ["dim %1d\n" % self.dim]
        names = "xyz"
        for a in range(self.dim):
            lines.append("%sMin %.14f\n" % (names[a], self.bounds[2 * a]))
            lines.append("%sMax %.14f\n" % (names[a], self.bounds[2 * a + 1]))
        for a in range(self.dim):
            lines.append("d%s %.14f\n" % (names[a], self._dx_raw[a]))
        lines.append("sampleMeshSize %8d\n" % N)
        lines.append("stencilMeshSize %8d\n" % N)
        lines.append("stencilSize %2d\n" % self.stencil)
        for a in range(self.dim):
            lines.append("n%s %8d\n" % (names[a], self.n[a]))
        with open(os.path.join(d, "info.dat"), "w") as f:
            f.write("".join(lines))
        with open(os.path.join(d, "connectivity.dat"), "w") as f:
            for row in self.graph:
                f.write("".join("%8d " % v for v in row) + "\n")
        with open(os.path.join(d, "coordinates.dat"), "w") as f:
            for k in range(N):
                s = "%8d %.14f %.14f " % (k, self._raw[0][k], self._raw[1][k])
                if self.dim == 3:
                    s += "%.14f " % self._raw[2][k]
                f.write(s + "\n")


def _neighbour(g, k, sign, N, periodic):
    t = g + sign * k
    inside = (t >= 0) if sign < 0 else (t <= N - 1)
    if periodic:
        return np.where(inside, t, t + N if sign < 0 else t - N), np.ones_like(t, dtype=bool)
    return t, inside


def full_mesh(n, bounds, stencil, periodic=(False, False, False), orc=None) -> FullMesh:
    """n = (Nx,) / (Nx, Ny) / (Nx, Ny, Nz); bounds = (xL, xR[, yL, yR[, zL, zR]]).
    orc: the loaded oracle, whose C round trip of the coordinates is used for
    large meshes (the Python one is exact too, but slow)."""
    assert stencil in (3, 5, 7)
    dim = len(n)
    nn = list(n) + [1] * (3 - dim)
    Nx, Ny, Nz = nn
    per = [bool(p) for p in periodic] + [False] * (3 - len(periodic))
    bb = list(bounds) + [0.0] * (6 - len(bounds))
    dxr = [(bb[1] - bb[0]) / Nx, (bb[3] - bb[2]) / Ny, (bb[5] - bb[4]) / Nz]
    N = Nx * Ny * Nz
    ids = np.arange(N, dtype=np.int64)
    gi = ids % (Nx * Ny) % Nx
    gj = (ids % (Nx * Ny)) // Nx
    gk = ids // (Nx * Ny)
    g = [gi, gj, gk]
    raw = [bb[2 * a] + 0.5 * dxr[a] + g[a] * dxr[a] if a < dim else np.zeros(N) for a in range(3)]
    h = (stencil - 1) // 2
    cols = [ids]
    for k in range(1, h + 1):
        for axis, sign in _SIDES[dim]:
            t, ok = _neighbour(g[axis], k, sign, nn[axis], per[axis])
            idx = [gi, gj, gk]
            idx[axis] = t
            gid = idx[0] + Nx * (idx[1] + Ny * idx[2])
            cols.append(np.where(ok, gid, -1))
    graph = np.stack(cols, axis=1).astype(np.int32)
    coords = []
    for a in range(3):
        coords.append((orc.round14(raw[a]) if orc is not None else _r14(raw[a])) if a < dim else np.zeros(N))
    dx = [float("%.14f" % dxr[a]) if a < dim else 0.0 for a in range(3)]
    m = FullMesh(dim, stencil, nn[:dim], graph, coords[0], coords[1], coords[2], np.array(dx), bb[:2 * dim])
    m._raw, m._dx_raw = raw, dxr
    return m


def _r14(v):
    """The values "%.14f" prints, parsed back (np.round(v, 14) is a different
    operation: it scales by 1e14 in floating point)."""
    return np.array([float("%.14f" % x) for x in np.asarray(v, dtype=np.float64)])
