"""Seeded synthetic tetrahedral meshes of the unit cube.

n^3 hexahedral cells, each split into the six Kuhn tetrahedra around its
(0,0,0)->(1,1,1) diagonal, every tetrahedron positively oriented.  Node
(i, j, k) sits at (i h, j h, k h) with id (i (n+1) + j)(n+1) + k; elements
come cell by cell (cell id (i n + j) n + k), six per cell.  Optional: a
uniform +-delta*h jitter of the interior nodes, a random element permutation,
and lognormal per-element coefficients -- all from numpy's PCG64 generator so
that the same seed gives the same mesh on every machine.

The reference has no mesh generator (its test meshes are hand-written Gmsh
files); meshes made here can be written in Gmsh 2 ASCII with `write_gmsh`
and read back through the library's Gmsh loader.
"""
from __future__ import annotations

import itertools
from dataclasses import dataclass

import numpy as np


@dataclass
class CubeMesh:
    n: int
    xyz: np.ndarray        # (N, 3) float64
    conn: np.ndarray       # (E, 4) int32, 0-based node ids
    boundary: np.ndarray   # (N,) bool, node on the cube surface
    min_det: float
    perm: np.ndarray | None  # perm[k] = original (cell-major) id of element k


def _kuhn_local():
    """Six tets of the unit cell as corner indices (corner c = 4 ci + 2 cj + ck)."""
    tets = []
    for sigma in itertools.permutations(range(3)):
        v = [0, 0, 0]
        pts = [tuple(v)]
        for ax in sigma:
            v[ax] = 1
            pts.append(tuple(v))
        det = np.linalg.det(np.array([np.subtract(pts[s], pts[0]) for s in (1, 2, 3)], dtype=float).T)
        if det < 0:  # odd permutation: swap the last two vertices
            pts[2], pts[3] = pts[3], pts[2]
        tets.append([4 * p[0] + 2 * p[1] + p[2] for p in pts])
    return np.array(tets, dtype=np.int64)


def element_dets(xyz: np.ndarray, conn: np.ndarray) -> np.ndarray:
    p0 = xyz[conn[:, 0]]
    e1, e2, e3 = xyz[conn[:, 1]] - p0, xyz[conn[:, 2]] - p0, xyz[conn[:, 3]] - p0
    return np.einsum("ij,ij->i", e1, np.cross(e2, e3))


def kuhn_cube(n: int, jitter: float = 0.0, seed: int | None = None, permute: bool = False) -> CubeMesh:
    """Kuhn-split unit cube with n^3 cells; see the module docstring."""
    m = n + 1
    h = 1.0 / n
    i, j, k = np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij")
    xyz = np.stack([i.ravel() * h, j.ravel() * h, k.ravel() * h], axis=1).astype(np.float64)
    boundary = ((i == 0) | (i == n) | (j == 0) | (j == n) | (k == 0) | (k == n)).ravel()
    ci, cj, ck = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    base = ((ci.ravel() * m + cj.ravel()) * m + ck.ravel()).astype(np.int64)
    corner = np.array([(a * m + b) * m + c for a in (0, 1) for b in (0, 1) for c in (0, 1)], dtype=np.int64)
    local = _kuhn_local()
    conn = (base[:, None, None] + corner[local][None, :, :]).reshape(-1, 4)
    rng = np.random.default_rng(seed) if (jitter > 0.0 or permute) else None
    if jitter > 0.0:
        interior = ~boundary
        d = rng.uniform(-jitter * h, jitter * h, size=xyz.shape)
        xyz = xyz + np.where(interior[:, None], d, 0.0)
        # re-draw the jitter of the nodes of any tet that came out inverted
        for _ in range(64):
            dets = element_dets(xyz, conn)
            bad = dets <= 0.0
            if not bad.any():
                break
            nodes = np.unique(conn[bad].ravel())
            nodes = nodes[interior[nodes]]
            base_xyz = np.stack([i.ravel()[nodes] * h, j.ravel()[nodes] * h, k.ravel()[nodes] * h], axis=1)
            xyz[nodes] = base_xyz + rng.uniform(-jitter * h, jitter * h, size=(len(nodes), 3))
    perm = None
    if permute:
        perm = rng.permutation(conn.shape[0])
        conn = conn[perm]
    dets = element_dets(xyz, conn)
    if not (dets > 0.0).all():
        raise ValueError("mesh generator produced an inverted tetrahedron")
    return CubeMesh(n=n, xyz=np.ascontiguousarray(xyz), conn=np.ascontiguousarray(conn.astype(np.int32)),
                    boundary=boundary, min_det=float(dets.min()), perm=perm)


def lognormal(count: int, sigma: float, seed: int) -> np.ndarray:
    """kappa_e = exp(sigma * N(0, 1)), seeded."""
    return np.exp(sigma * np.random.default_rng(seed).standard_normal(count))


def write_gmsh(path: str, xyz: np.ndarray, conn: np.ndarray, geo_id: int = 1) -> None:
    """Gmsh 2.2 ASCII: nodes labelled 1..N in order, tets as type 4 with 2 tags."""
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % len(xyz))
        for a, (x, y, z) in enumerate(xyz):
            f.write("%d %.17g %.17g %.17g\n" % (a + 1, x, y, z))
        f.write("$EndNodes\n$Elements\n%d\n" % len(conn))
        for e, c in enumerate(conn):
            f.write("%d 4 2 0 %d %d %d %d %d\n" % (e + 1, geo_id, c[0] + 1, c[1] + 1, c[2] + 1, c[3] + 1))
        f.write("$EndElements\n")


def p2_boundary(mesh_boundary: np.ndarray, edge_nodes: np.ndarray) -> np.ndarray:
    """Boundary mask of P2 dofs: vertices as given, an edge dof when both ends are."""
    eb = mesh_boundary[edge_nodes[:, 0]] & mesh_boundary[edge_nodes[:, 1]]
    return np.concatenate([mesh_boundary, eb])
