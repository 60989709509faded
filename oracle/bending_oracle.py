"""CPU restatement (FP64) of the rest-dihedral bending option, for tests only (the checker, never
the product).  The reference has no rest angle (src/edge.cpp:51-67: E = kb (1 - n0 . n1) with the
normal flip of src/edge.cpp:78-81); this option is an extension, so its parity is pinned by
finite differences of this file's own energy (tests/test_bending_oracle.py), and the GPU is
checked against it.

Bending quad of an edge (b0, b1) with faces f0, f1 (the edge's faces in face order, the
reference's face <-> edge matching, src/initialize.cpp:370-401) and the beads across them, a0 on
f0 and a1 on f1.  Bend angle: the dihedral phi of (a0, b0, b1, a1), shifted so that a flat quad
(a0 and a1 on opposite sides of the edge) has beta = 0:

    b1 = x_b0 - x_a0, b2 = x_b1 - x_b0, b3 = x_a1 - x_b1, m = b1 x b2, n = b2 x b3
    beta = atan2(-|b2| b1 . n, -m . n)                       (= phi - pi, wrapped)
    E = kb (1 - cos(beta - beta0)), credited kb/4 to each of the four beads

beta0 is beta of the rest shape.  For |beta| < pi/2 and beta0 = 0 this is the reference's
kb (1 - |n0 . n1|).  Gradient of phi (Blondel and Karplus 1996, rewritten for the vectors above;
p = b1.b2/|b2|^2, s = b3.b2/|b2|^2; the four sum to zero):
    d/dx_a0 = -|b2| m / |m|^2,   d/dx_a1 = |b2| n / |n|^2
    d/dx_b0 = -(1 + p) d/dx_a0 + s d/dx_a1
    d/dx_b1 = p d/dx_a0 - (1 + s) d/dx_a1
"""
import numpy as np


def quads(edges, edge_type, faces):
    """(b0, b1, a0, a1) for every bending edge, in edge order."""
    out = []
    for e, (b0, b1) in enumerate(edges):
        if edge_type[e] == 0:
            continue
        fs = [f for f in faces if b0 in f and b1 in f]
        a0 = [b for b in fs[0] if b != b0 and b != b1][0]
        a1 = [b for b in fs[1] if b != b0 and b != b1][0]
        out.append((int(b0), int(b1), int(a0), int(a1)))
    return out


def _parts(x, q):
    b0, b1, a0, a1 = q
    v1 = x[b0] - x[a0]
    v2 = x[b1] - x[b0]
    v3 = x[a1] - x[b1]
    return v1, v2, v3, np.cross(v1, v2), np.cross(v2, v3)


def bend_angle(x, q):
    v1, v2, v3, m, n = _parts(x, q)
    return float(np.arctan2(-np.linalg.norm(v2) * (v1 @ n), -(m @ n)))


def bend_angle_grad(x, q):
    """d beta / d x for (b0, b1, a0, a1)."""
    v1, v2, v3, m, n = _parts(x, q)
    l2 = v2 @ v2
    nv2 = np.sqrt(l2)
    ga0 = -nv2 / (m @ m) * m
    ga1 = nv2 / (n @ n) * n
    p, s = (v1 @ v2) / l2, (v3 @ v2) / l2
    gb0 = -(1 + p) * ga0 + s * ga1
    gb1 = p * ga0 - (1 + s) * ga1
    return gb0, gb1, ga0, ga1


def rest_angles(rest, qs):
    return np.array([bend_angle(rest, q) for q in qs])


def energy(x, qs, beta0, kb):
    return sum(kb * (1 - np.cos(bend_angle(x, q) - b0)) for q, b0 in zip(qs, beta0))


def forces_and_bead_energies(x, qs, beta0, kb):
    """Bending forces (-grad E) and per-bead energies (kb/4 of each edge per quad bead)."""
    f = np.zeros_like(x)
    be = np.zeros(len(x))
    for q, b0 in zip(qs, beta0):
        beta = bend_angle(x, q)
        c = -kb * np.sin(beta - b0)
        for bead, g in zip(q, bend_angle_grad(x, q)):
            f[bead] += c * g
            be[bead] += 0.25 * kb * (1 - np.cos(beta - b0))
    return f, be
