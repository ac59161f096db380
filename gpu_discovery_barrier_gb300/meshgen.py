"""Seeded synthetic meshes for Delaunay mesh refinement.

The reference refines meshes read from Triangle's .node/.ele/.poly files
(lonestar/apps/dmr/meshfiles.h:19-110): node coordinates as doubles,
triangles as three node ids, boundary segments as two node ids.  Those input
meshes are external datasets; `grid_mesh` builds one with the same layout
from a jittered anisotropic grid, which refinement has to rework
everywhere (its cells are hx x hy rectangles, so with hy/hx = 0.3 every
triangle has an angle near 17 degrees, below the 30-degree bound).

Element layout (as the reference's `elements`, shmesh.h:53): one uint32
triple per element; triangles first, then the boundary segments, whose
third node is ``SEGMENT`` (INVALIDID, dmr_common.cl:49).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

SEGMENT = 1234567890  # a segment's third node and an absent neighbour


@dataclass
class Mesh:
    x: np.ndarray         # float64 [nnodes]
    y: np.ndarray         # float64 [nnodes]
    elements: np.ndarray  # uint32 [nelements, 3]; segments carry SEGMENT third
    ntriangles: int
    nsegments: int
    name: str = ""

    @property
    def nnodes(self) -> int:
        return int(self.x.size)

    @property
    def nelements(self) -> int:
        return int(self.elements.shape[0])


def _incircle(ax, ay, bx, by, cx, cy, px, py):
    """> 0 when p is inside the circle through a, b, c (counter-clockwise)."""
    adx, ady = ax - px, ay - py
    bdx, bdy = bx - px, by - py
    cdx, cdy = cx - px, cy - py
    ad = adx * adx + ady * ady
    bd = bdx * bdx + bdy * bdy
    cd = cdx * cdx + cdy * cdy
    return ad * (bdx * cdy - cdx * bdy) + bd * (cdx * ady - adx * cdy) + cd * (adx * bdy - bdx * ady)


def grid_mesh(nx: int, ny: int, hx: float = 1.0, hy: float = 0.3, jitter: float = 0.03,
              seed: int = 1) -> Mesh:
    """Delaunay triangulation of an nx x ny jittered grid on a rectangle.

    Interior nodes move by up to `jitter` (in units of hx) in each axis,
    nodes on the border only along it, so the domain stays the rectangle
    [0, (nx-1) hx] x [0, (ny-1) hy].  Each cell is cut along the diagonal
    the incircle test picks; with jitter well inside the margin by which the
    next row's nodes clear a cell's circumcircle (hx = 1, hy = 0.3: 0.15),
    that is the Delaunay triangulation of the nodes.
    """
    if nx < 2 or ny < 2:
        raise ValueError("grid_mesh needs at least 2 x 2 nodes")
    rng = np.random.default_rng(seed)
    i = np.tile(np.arange(nx, dtype=np.float64), ny)
    j = np.repeat(np.arange(ny, dtype=np.float64), nx)
    dx = rng.uniform(-jitter, jitter, nx * ny) * hx
    dy = rng.uniform(-jitter, jitter, nx * ny) * hx
    dx[(i == 0) | (i == nx - 1)] = 0.0
    dy[(j == 0) | (j == ny - 1)] = 0.0
    x = i * hx + dx
    y = j * hy + dy
    ci, cj = np.meshgrid(np.arange(nx - 1), np.arange(ny - 1))
    ci, cj = ci.ravel(), cj.ravel()
    a = (cj * nx + ci).astype(np.int64)
    b, c, d = a + 1, a + nx + 1, a + nx  # counter-clockwise a b c d
    d_in = _incircle(x[a], y[a], x[b], y[b], x[c], y[c], x[d], y[d]) > 0
    t1 = np.where(d_in[:, None], np.stack([a, b, d], 1), np.stack([a, b, c], 1))
    t2 = np.where(d_in[:, None], np.stack([b, c, d], 1), np.stack([a, c, d], 1))
    tri = np.empty((2 * a.size, 3), dtype=np.int64)
    tri[0::2], tri[1::2] = t1, t2
    # border segments, counter-clockwise around the rectangle
    bottom = np.arange(nx - 1)
    right = (np.arange(ny - 1) * nx) + (nx - 1)
    top = (ny - 1) * nx + np.arange(nx - 1, 0, -1)
    left = np.arange(ny - 1, 0, -1) * nx
    s0 = np.concatenate([bottom, right, top, left])
    s1 = np.concatenate([bottom + 1, right + nx, top - 1, left - nx])
    seg = np.stack([s0, s1, np.full(s0.size, SEGMENT)], 1)
    elements = np.concatenate([tri, seg]).astype(np.uint32)
    return Mesh(x, y, elements, int(tri.shape[0]), int(seg.shape[0]),
                f"grid {nx}x{ny} hx {hx} hy {hy} jitter {jitter} seed {seed}")
