"""Capsomere templates for the synthetic workloads, written in SOUFFLE's infile format.

A SOUFFLE system is ``S`` copies of one template subunit (beads, edges, faces and
an LJ-attraction table), replicated by ``generate_lattice``
(src/initialize.cpp:295-404).  The infile the reference parses is token-counted
(src/initialize.cpp:47-128): a 9-token header ``ks_vdwr = b mass = kg sigma = m``,
then particle, edge, triangle and LJ-attraction blocks, each introduced by a
``# Number of ... = n`` line and a line of column names.  ``write_infile``
produces exactly that layout so the same file feeds the reference and this
package.

Two templates are provided:

* ``patch_n3`` -- one triangulated equilateral patch with 3 segments per side
  (10 beads, 18 edges, 9 faces); the 10-bead capsomere of the small plain run.
* ``bilayer_n5`` -- two 5-segment patches of 21 beads, 0.5 sigma apart, joined by
  one vertical spring per bead pair and one diagonal spring per in-layer edge
  (42 beads, 156 edges, 50 faces); the 42-bead capsomere of the larger runs.

Bead types: rim beads that are not corners are type 2 (LJ-attractive through the
``2 2`` attraction row), all others type 1.  Charges: interior beads +0.5 e,
rim beads -0.5 e.  Interior in-layer edges (shared by two faces of the same
layer) are bending edges (type 1), all others type 0.  The reference bending
energy has no rest angle (src/edge.cpp:51-67), so a curvature radius only
shapes the initial template: beads are lifted onto a sphere of that radius and
every edge's rest length is its template chord length.  ``with_rest_dihedral``
makes that curved shape the bending rest shape as well (every bending edge then
relaxes to its dihedral there): an option of this package, which the reference
does not have.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence, Tuple

import numpy as np


@dataclasses.dataclass
class Template:
    """One capsomere.  Indices are template-local (0..np-1)."""

    pos: np.ndarray            # (np, 3) float64
    types: np.ndarray          # (np,) int
    charge: np.ndarray         # (np,) float64
    diameter: np.ndarray       # (np,) float64  (sigma of each bead, LJ units)
    mass: np.ndarray           # (np,) float64  (LJ units)
    edges: np.ndarray          # (ne, 2) int   endpoints
    edge_type: np.ndarray      # (ne,) int     0 = spring only, != 0 = bending edge
    edge_len0: np.ndarray      # (ne,) float64 rest length
    faces: np.ndarray          # (nf, 3) int
    lj_attract: List[Tuple[int, int]]  # directed (type_i, type_j) rows
    name: str = "template"
    bend_rest: Optional[np.ndarray] = None  # (np, 3) bending rest shape; None = no rest angle

    @property
    def n_beads(self) -> int:
        return int(self.pos.shape[0])

    def radius(self) -> float:
        c = self.pos.mean(axis=0)
        return float(np.sqrt(((self.pos - c) ** 2).sum(axis=1)).max())


def _tri_lattice(n: int):
    """Vertices (i, j) with i + j <= n of a unit triangular lattice, edges, faces.

    Faces are wound counter-clockwise seen from +z so neighbouring normals agree.
    """
    idx = {}
    pts = []
    for j in range(n + 1):
        for i in range(n + 1 - j):
            idx[(i, j)] = len(pts)
            pts.append((i + 0.5 * j, j * math.sqrt(3.0) / 2.0, 0.0))
    faces = []
    for j in range(n):
        for i in range(n - j):
            faces.append((idx[(i, j)], idx[(i + 1, j)], idx[(i, j + 1)]))
            if i + j <= n - 2:
                faces.append((idx[(i + 1, j)], idx[(i + 1, j + 1)], idx[(i, j + 1)]))
    edges = set()
    for f in faces:
        for a, b in ((f[0], f[1]), (f[1], f[2]), (f[0], f[2])):
            edges.add((min(a, b), max(a, b)))
    edges = sorted(edges)
    rim = [False] * len(pts)
    corner = [False] * len(pts)
    for (i, j), k in idx.items():
        on = (i == 0) + (j == 0) + (i + j == n)
        rim[k] = on >= 1
        corner[k] = on >= 2
    return np.array(pts), edges, faces, np.array(rim), np.array(corner)


def _curve(pts: np.ndarray, radius: float) -> np.ndarray:
    """Lift a flat (z = 0) patch onto a sphere of ``radius`` about its centroid."""
    if not radius or radius <= 0:
        return pts.copy()
    c = pts.mean(axis=0)
    out = pts.copy()
    d2 = ((pts[:, :2] - c[:2]) ** 2).sum(axis=1)
    out[:, 2] = radius - np.sqrt(np.maximum(radius * radius - d2, 0.0))
    return out


def _interior_edges(faces: Sequence[Tuple[int, int, int]]) -> set:
    count = {}
    for f in faces:
        for a, b in ((f[0], f[1]), (f[1], f[2]), (f[0], f[2])):
            key = (min(a, b), max(a, b))
            count[key] = count.get(key, 0) + 1
    return {e for e, c in count.items() if c == 2}


def patch_n3(curvature_radius: float = 6.0) -> Template:
    """10-bead single-layer capsomere (3 segments per side)."""
    pts, edges, faces, rim, corner = _tri_lattice(3)
    pts = _curve(pts, curvature_radius)
    interior = _interior_edges(faces)
    e = np.array(edges, dtype=np.int64)
    etype = np.array([1 if tuple(x) in interior else 0 for x in edges], dtype=np.int64)
    len0 = np.sqrt(((pts[e[:, 0]] - pts[e[:, 1]]) ** 2).sum(axis=1))
    types = np.where(rim & ~corner, 2, 1)
    charge = np.where(rim, -0.5, 0.5)
    n = pts.shape[0]
    return Template(pts, types, charge, np.ones(n), np.ones(n), e, etype, len0,
                    np.array(faces, dtype=np.int64), [(2, 2)], name="patch_n3")


def bilayer_n5(curvature_radius: float = 6.0, gap: float = 0.5) -> Template:
    """42-bead two-layer capsomere: two 21-bead n=5 patches joined by springs."""
    pts, edges, faces, rim, corner = _tri_lattice(5)
    top = _curve(pts, curvature_radius)
    # second layer: offset along each bead's local sphere normal (or -z if flat)
    if curvature_radius and curvature_radius > 0:
        c = pts.mean(axis=0)
        centre = np.array([c[0], c[1], curvature_radius])
        nrm = centre - top
        nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
        bot = top - gap * nrm
    else:
        bot = top - np.array([0.0, 0.0, gap])
    n1 = pts.shape[0]
    allpts = np.vstack([top, bot])
    interior = _interior_edges(faces)
    elist, etype = [], []
    for layer in range(2):
        off = layer * n1
        for a, b in edges:
            elist.append((a + off, b + off))
            etype.append(1 if (a, b) in interior else 0)
    for k in range(n1):                      # vertical inter-layer springs
        elist.append((k, k + n1))
        etype.append(0)
    for a, b in edges:                       # one diagonal per in-layer edge
        elist.append((a, b + n1))
        etype.append(0)
    flist = [tuple(f) for f in faces] + [(f[0] + n1, f[1] + n1, f[2] + n1) for f in faces]
    e = np.array(elist, dtype=np.int64)
    len0 = np.sqrt(((allpts[e[:, 0]] - allpts[e[:, 1]]) ** 2).sum(axis=1))
    rim2 = np.concatenate([rim, rim])
    corner2 = np.concatenate([corner, corner])
    types = np.where(rim2 & ~corner2, 2, 1)
    charge = np.where(rim2, -0.5, 0.5)
    n = allpts.shape[0]
    return Template(allpts, types, charge, np.ones(n), np.ones(n), e,
                    np.array(etype, dtype=np.int64), len0,
                    np.array(flist, dtype=np.int64), [(2, 2)], name="bilayer_n5")


def with_rest_dihedral(t: Template) -> Template:
    """A copy of ``t`` whose bending edges relax to the dihedrals of its own (curved) shape."""
    return dataclasses.replace(t, bend_rest=t.pos.copy(), name=t.name + "_rest")


def template_by_name(name: str, curvature_radius: float = 6.0) -> Template:
    if name == "patch_n3":
        return patch_n3(curvature_radius)
    if name == "bilayer_n5":
        return bilayer_n5(curvature_radius)
    raise ValueError(f"unknown template {name!r}")


def write_infile(t: Template, path: str, sigma_si: float = 1e-9, mass_si: float = 3.9434e-26,
                 bondlength: float = 1.122462048) -> None:
    """Write ``t`` in the token layout parsed by src/initialize.cpp:47-128."""
    r = repr
    lines = [f"ks_vdwr  = {bondlength}", f"mass     = {mass_si}", f"sigma    = {sigma_si}", "",
             f"# Number of Particles = {t.n_beads}", "",
             "index\tx\ty\tz\ttype\tcharge\tdiameter\tmass"]
    for i in range(t.n_beads):
        x, y, z = (float(v) for v in t.pos[i])
        lines.append(f"{i}\t{r(x)}\t{r(y)}\t{r(z)}\t{int(t.types[i])}\t{r(float(t.charge[i]))}"
                     f"\t{r(float(t.diameter[i]))}\t{r(float(t.mass[i]))}")
    lines += ["", f"# Number of Edges = {len(t.edges)}", "", "index\te1\te2\ttype\tlength"]
    for k, (a, b) in enumerate(t.edges):
        lines.append(f"{k}\t{int(a)}\t{int(b)}\t{int(t.edge_type[k])}\t{r(float(t.edge_len0[k]))}")
    lines += ["", f"# Number of Triangles = {len(t.faces)}", "",
              "index\tt1\tt2\tt3\ttype\tnormal"]
    for k, (a, b, c) in enumerate(t.faces):
        lines.append(f"{k}\t{int(a)}\t{int(b)}\t{int(c)}\t0\t1")
    lines += ["", f"# Number of LJ Attractions = {len(t.lj_attract)}", "",
              "index  type1  type2  epsilon sigmahc"]
    for k, (a, b) in enumerate(t.lj_attract):
        lines.append(f"{k}\t{a}\t{b}\t2\t1")
    lines += ["", "# Number of LJ Repulsions = 1", "", "index  type1  type2  epsilon sigmahc",
              "0\t1\t1\t1\t1", ""]
    with open(path, "w") as fh:
        fh.write("\n".join(lines))


def read_infile(path: str) -> Tuple[Template, float, float, float]:
    """Parse an infile the way src/initialize.cpp:47-128 does (token counting).

    Returns (template, bondlength, mass_si, sigma_si).
    """
    with open(path) as fh:
        tok = fh.read().split()
    p = 0

    def take(n=1):
        nonlocal p
        out = tok[p:p + n]
        p += n
        return out

    h = take(9)
    bondlength, mass_si, sigma_si = float(h[2]), float(h[5]), float(h[8])
    npart = int(take(6)[5])
    take(8)
    pos, types, charge, diam, mass = [], [], [], [], []
    for _ in range(npart):
        row = take(8)
        pos.append([float(row[1]), float(row[2]), float(row[3])])
        types.append(int(float(row[4])))
        charge.append(float(row[5]))
        diam.append(float(row[6]))
        mass.append(float(row[7]))
    ne = int(take(6)[5])
    take(5)
    edges, etype, len0 = [], [], []
    for _ in range(ne):
        row = take(5)
        edges.append([int(row[1]), int(row[2])])
        etype.append(int(float(row[3])))
        len0.append(float(row[4]))
    nt = int(take(6)[5])
    take(6)
    faces = []
    for _ in range(nt):
        row = take(6)
        faces.append([int(row[1]), int(row[2]), int(row[3])])
    na = int(take(7)[6])
    take(5)
    lj = []
    for _ in range(na):
        row = take(5)
        lj.append((int(row[1]), int(row[2])))
    t = Template(np.array(pos, dtype=np.float64), np.array(types, dtype=np.int64),
                 np.array(charge), np.array(diam), np.array(mass),
                 np.array(edges, dtype=np.int64).reshape(-1, 2), np.array(etype, dtype=np.int64),
                 np.array(len0), np.array(faces, dtype=np.int64).reshape(-1, 3), lj,
                 name=path.rsplit("/", 1)[-1])
    return t, bondlength, mass_si, sigma_si
