"""Seeded synthetic 2-D triangle meshes in the shape Triangle/meshpy hands to
``Mesher.import_meshpy`` (reference ``src/mesher.py:48-61``): ``points``
[P,2] float64, ``elements`` [N,3] int32, ``faces`` [F,2] int32 and
``point_markers`` [P] int32.

Triangle (through meshpy) is what the reference's notebooks mesh with
(``tests/porous_flow.ipynb:347``, ``tests/flow_over_cyl.ipynb``); it is not
available here, so these generators stand in for it:

* ``cavity``: a jittered n x n point grid whose quads are split along a seeded
  random diagonal (the lid-driven cavity).
* ``channel_cylinder`` / ``porous``: boundary-sampled rectangles and circles
  plus a jittered hexagonal interior point set, triangulated with
  ``scipy.spatial.Delaunay``; triangles whose centroid lies inside an obstacle
  are removed, which leaves the sampled circle polygons as hole boundaries.

Point markers follow meshpy's ``make_box`` facet order: bottom 1, right 2,
top 3, left 4, obstacles 5.  Corner points carry a wall marker.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

BOTTOM, RIGHT, TOP, LEFT, OBSTACLE = 1, 2, 3, 4, 5


@dataclass
class RawMesh:
    """A triangulation with boundary markers, before any FVDBM geometry."""

    points: np.ndarray
    elements: np.ndarray
    faces: np.ndarray
    point_markers: np.ndarray
    info: dict = field(default_factory=dict)

    @property
    def n_cells(self) -> int:
        return int(self.elements.shape[0])


def unique_edges(tris: np.ndarray, n_points: int) -> np.ndarray:
    """Unique undirected edges of ``tris`` ([N,3]); each edge keeps the
    orientation of its first occurrence in element order, and edges are
    listed in ascending (min vertex, max vertex) order."""
    e = np.stack([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]], axis=1).reshape(-1, 2)
    lo = np.minimum(e[:, 0], e[:, 1]).astype(np.int64)
    hi = np.maximum(e[:, 0], e[:, 1]).astype(np.int64)
    key = lo * np.int64(n_points) + hi
    _, first = np.unique(key, return_index=True)
    return e[first].astype(np.int32)


def _signed_area(points: np.ndarray, tris: np.ndarray) -> np.ndarray:
    p = points[tris]
    return 0.5 * ((p[:, 1, 0] - p[:, 0, 0]) * (p[:, 2, 1] - p[:, 0, 1])
                  - (p[:, 2, 0] - p[:, 0, 0]) * (p[:, 1, 1] - p[:, 0, 1]))


def cavity(n: int = 41, jitter: float = 0.2, seed: int = 0) -> RawMesh:
    """Unit square from an n x n grid; interior points jittered uniformly by
    +-jitter*h in x and y; each quad split along a seeded random diagonal.
    n=41 gives 3,200 triangles.  Lid (top, corners excluded) is marker 3."""
    rng = np.random.default_rng(seed)
    h = 1.0 / (n - 1)
    xs = np.linspace(0.0, 1.0, n)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    pts = np.stack([X.ravel(), Y.ravel()], axis=1).astype(np.float64)
    ii = np.tile(np.arange(n), n)
    jj = np.repeat(np.arange(n), n)
    interior = (ii > 0) & (ii < n - 1) & (jj > 0) & (jj < n - 1)
    pts[interior] += rng.uniform(-jitter * h, jitter * h, size=(int(interior.sum()), 2))

    qi, qj = np.meshgrid(np.arange(n - 1), np.arange(n - 1), indexing="xy")
    p00 = (qj * n + qi).ravel()
    p10, p01, p11 = p00 + 1, p00 + n, p00 + n + 1
    diag = rng.integers(0, 2, size=p00.shape[0])
    t_a = np.where(diag[:, None] == 0, np.stack([p00, p10, p11], 1), np.stack([p00, p10, p01], 1))
    t_b = np.where(diag[:, None] == 0, np.stack([p00, p11, p01], 1), np.stack([p10, p11, p01], 1))
    tris = np.stack([t_a, t_b], axis=1).reshape(-1, 3).astype(np.int32)

    mk = np.zeros(n * n, dtype=np.int32)
    mk[jj == n - 1] = TOP
    mk[ii == n - 1] = RIGHT
    mk[ii == 0] = LEFT
    mk[jj == 0] = BOTTOM
    faces = unique_edges(tris, n * n)
    return RawMesh(pts, tris, faces, mk, info={"kind": "cavity", "n": n, "h": h,
                                                "jitter": jitter, "seed": seed})


def _rect_boundary(width: float, height: float, h: float):
    nx = max(2, int(np.ceil(width / h)))
    ny = max(2, int(np.ceil(height / h)))
    xs = np.linspace(0.0, width, nx + 1)
    ys = np.linspace(0.0, height, ny + 1)
    bottom = np.stack([xs, np.zeros_like(xs)], 1)
    top = np.stack([xs, np.full_like(xs, height)], 1)
    right = np.stack([np.full(ny - 1, width), ys[1:-1]], 1)
    left = np.stack([np.zeros(ny - 1), ys[1:-1]], 1)
    pts = np.concatenate([bottom, right, top, left])
    mk = np.concatenate([np.full(len(bottom), BOTTOM), np.full(len(right), RIGHT),
                         np.full(len(top), TOP), np.full(len(left), LEFT)]).astype(np.int32)
    return pts, mk


def _delaunay_domain(width: float, height: float, circles: np.ndarray, h: float,
                     rng: np.random.Generator) -> RawMesh:
    from scipy.spatial import Delaunay, cKDTree

    bpts, bmk = _rect_boundary(width, height, h)
    cpts, cmk = [], []
    for cx, cy, r in circles:
        nc = max(12, int(np.ceil(2.0 * np.pi * r / h)))
        th = np.linspace(0.0, 2.0 * np.pi, nc, endpoint=False) + rng.uniform(0, 2 * np.pi / nc)
        cpts.append(np.stack([cx + r * np.cos(th), cy + r * np.sin(th)], 1))
        cmk.append(np.full(nc, OBSTACLE, dtype=np.int32))

    dy = h * np.sqrt(3.0) / 2.0
    rows = np.arange(1, int(height / dy) + 1)
    cols = np.arange(0, int(width / h) + 2)
    gx = cols[None, :] * h + (rows[:, None] % 2) * (h / 2.0)
    gy = np.broadcast_to(rows[:, None] * dy, gx.shape)
    ipts = np.stack([gx.ravel(), gy.ravel()], 1)
    ipts = ipts + rng.uniform(-0.15 * h, 0.15 * h, size=ipts.shape)
    m = 0.5 * h
    keep = (ipts[:, 0] > m) & (ipts[:, 0] < width - m) & (ipts[:, 1] > m) & (ipts[:, 1] < height - m)
    ipts = ipts[keep]
    if len(circles):
        tree = cKDTree(ipts)
        drop = np.zeros(len(ipts), dtype=bool)
        for cx, cy, r in circles:
            drop[tree.query_ball_point((cx, cy), r + 0.55 * h)] = True
        ipts = ipts[~drop]

    pts = np.concatenate([bpts] + cpts + [ipts])
    mk = np.concatenate([bmk] + cmk + [np.zeros(len(ipts), dtype=np.int32)]).astype(np.int32)
    tris = Delaunay(pts).simplices.astype(np.int64)
    if len(circles):
        cen = pts[tris].mean(axis=1)
        tree = cKDTree(cen)
        inside = np.zeros(len(tris), dtype=bool)
        for cx, cy, r in circles:
            inside[tree.query_ball_point((cx, cy), r)] = True
        tris = tris[~inside]
    area = np.abs(_signed_area(pts, tris))
    tris = tris[area > 1e-9 * h * h]
    used = np.zeros(len(pts), dtype=bool)
    used[tris.ravel()] = True
    remap = -np.ones(len(pts), dtype=np.int64)
    remap[used] = np.arange(int(used.sum()))
    pts, mk, tris = pts[used], mk[used], remap[tris].astype(np.int32)
    faces = unique_edges(tris, len(pts))

    # every boundary edge (one adjacent triangle) must join two marked points
    e = np.stack([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]], 1).reshape(-1, 2)
    key = np.minimum(e[:, 0], e[:, 1]).astype(np.int64) * len(pts) + np.maximum(e[:, 0], e[:, 1])
    uk, cnt = np.unique(key, return_counts=True)
    bkey = uk[cnt == 1]
    b0, b1 = bkey // len(pts), bkey % len(pts)
    if not np.all((mk[b0] != 0) & (mk[b1] != 0)):
        raise RuntimeError("mesh boundary not recovered; change seed or spacing")
    return RawMesh(pts.astype(np.float64), tris, faces, mk)


def channel_cylinder(length: float = 2.2, height: float = 0.41, center=(0.2, 0.2),
                     radius: float = 0.05, n_target: int = 60_000, seed: int = 0) -> RawMesh:
    """Channel length x height with a circular hole; spacing chosen so that
    the mesh has about ``n_target`` triangles (Triangle with max-area 2e-5
    gives a similar count)."""
    rng = np.random.default_rng(seed)
    fluid = length * height - np.pi * radius ** 2
    h = float(np.sqrt(4.0 * fluid / (np.sqrt(3.0) * n_target)))
    m = _delaunay_domain(length, height, np.array([[center[0], center[1], radius]]), h, rng)
    m.info = {"kind": "channel_cylinder", "length": length, "height": height,
              "center": tuple(center), "radius": radius, "h": h, "seed": seed}
    return m


def porous_obstacles(n_obstacles: int = 400, mu: float = float(np.log(0.012)), sigma: float = 0.3,
                     porosity: float = 0.70, gap: float = 0.0, seed: int = 0,
                     max_tries: int = 200_000) -> np.ndarray:
    """Non-overlapping circles in the unit square: centres uniform, radii
    lognormal(mu, sigma), all radii scaled by one factor so that the solid
    fraction is 1-porosity.  Circles keep ``gap`` clear of each other and of
    the square's sides.  Returns [n,3] (cx, cy, r)."""
    rng = np.random.default_rng(seed)
    r = np.exp(rng.normal(mu, sigma, size=n_obstacles))
    r *= np.sqrt((1.0 - porosity) / np.sum(np.pi * r * r))
    r = np.sort(r)[::-1]
    out = np.zeros((n_obstacles, 3))
    k = 0
    tries = 0
    while k < n_obstacles:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("could not place obstacles")
        ri = r[k]
        c = rng.uniform(ri + gap, 1.0 - ri - gap, size=2)
        if k:
            d = np.hypot(out[:k, 0] - c[0], out[:k, 1] - c[1])
            if np.any(d < out[:k, 2] + ri + gap):
                continue
        out[k] = (c[0], c[1], ri)
        k += 1
    return out


def porous(n_obstacles: int = 400, n_target: int = 1_000_000, porosity: float = 0.70,
           mu: float = float(np.log(0.012)), sigma: float = 0.3, seed: int = 0,
           gap_cells: float = 2.5) -> RawMesh:
    """Unit square holding ``n_obstacles`` circular obstacles at the given
    porosity, meshed to about ``n_target`` triangles.  Inlet is the left side
    (marker 4), outlet the right side (marker 2).  Obstacles keep
    ``gap_cells`` mesh spacings clear of each other and of the sides."""
    rng = np.random.default_rng(seed + 1)
    h = float(np.sqrt(4.0 * porosity / (np.sqrt(3.0) * n_target)))
    circles = porous_obstacles(n_obstacles, mu, sigma, porosity, gap=gap_cells * h, seed=seed)
    m = _delaunay_domain(1.0, 1.0, circles, h, rng)
    solid = float(np.sum(np.pi * circles[:, 2] ** 2))
    m.info = {"kind": "porous", "n_obstacles": n_obstacles, "porosity": 1.0 - solid,
              "h": h, "seed": seed, "circles": circles}
    return m
