"""Generate the post-run analysis fixtures in this folder from the reference itself.

Writes seeded synthetic outfiles/energy.out and outfiles/ovito.lammpstrj in the reference's
formats (src/md.cpp:339-353,616-623 and 647-678), runs the reference's analyze_output
(src/analysis.cpp:16-297, compiled unmodified by oracle/ref.mk into oracle/_ref/ref_analyze)
on them, and stores inputs and the files it writes as .npz.  The reference works out the
subunit size from the bead count (41, 43 or 78 beads, src/analysis.cpp:81-83), so the synthetic
subunits have 43 beads.  Coordinates are multiples of 1/64 (exact in binary, printed exactly),
and the layout puts subunits in contact inside the box, across box faces and across box corners,
so that every branch of the analysis sees work: mass spectrum, type-0 sub-oligomers and the
type-5 pair correlation.

    python tests/golden/make_golden_analysis.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_ANALYZE = os.path.join(REPO, "oracle", "_ref", "ref_analyze")

NP = 43
Q = 1.0 / 64.0


def template_offsets(rng):
    """43 bead offsets within ~1.6 sigma of the subunit centre, on the 1/64 grid, distinct."""
    pts = set()
    out = []
    while len(out) < NP:
        v = rng.uniform(-1.6, 1.6, 3)
        if np.linalg.norm(v) > 1.6:
            continue
        g = tuple(np.round(v / Q).astype(int))
        if g in pts:
            continue
        pts.add(g)
        out.append(np.array(g, dtype=float) * Q)
    out[0] = np.zeros(3)
    return np.array(out)


def bead_types():
    t = np.ones(NP, dtype=int)
    t[1:7] = 0      # sub-oligomer beads
    t[7:11] = 5     # pair-correlation beads
    t[11:14] = 2
    return t


def layout(L, rng, S):
    """Subunit centres: two clusters inside the box, corner pairs, face-straddling pairs with
    identical transverse coordinates, and the rest spread out."""
    h = L / 2
    c = []
    for base in (np.array([-5.0, -5.0, 0.0]), np.array([6.0, 4.0, -3.0])):   # clusters
        for k in range(4):
            c.append(base + np.array([2.75 * (k % 2), 2.75 * (k // 2), 0.0]))
    for sx in (-1, 1):                                                        # corners
        for sy in (-1, 1):
            for sz in (-1, 1):
                c.append(np.array([sx, sy, sz]) * (h - 0.875))
    for axis, (u, v) in enumerate(((3.0, -7.0), (-9.0, 2.5), (4.5, 8.0))):    # across faces
        for s in (-1, 1):
            p = np.array([u, v, u])
            p[axis] = s * (h - 0.75)
            c.append(p)
    while len(c) < S:
        p = np.round(rng.uniform(-h + 2, h - 2, 3) / Q) * Q
        if all(np.linalg.norm(p - q) > 5.0 for q in c):
            c.append(p)
    return np.array(c[:S])


def wrap(x, L):
    return (x + L / 2) % L - L / 2


def write_trajectory(path, frames, L):
    with open(path, "w") as f:
        for step, pos, types in frames:
            f.write("ITEM: TIMESTEP\n%d\nITEM: NUMBER OF ATOMS\n%d\nITEM: BOX BOUNDS\n" % (step, len(pos)))
            for _ in range(3):
                f.write("%g%15g\n" % (-L / 2, L / 2))
            f.write("ITEM: ATOMS index type x y z b charge\n")
            for i, (p, t) in enumerate(zip(pos, types)):
                f.write("%d%15d%15.6f%15.6f%15.6f%15g%15g\n" % (i + 1, t, p[0], p[1], p[2], 0.0, 0.5))


def write_energy(path, rows, aligned=False):
    """energy.out as the MD writes it: a 12-token header, row 0 with 11 columns, later rows 12.
    aligned: 11 header tokens and 11 columns in every row, the layout the reader expects."""
    with open(path, "w") as f:
        f.write("time" + "".join("%15s" % s for s in ("kinetic", "stretching", "bending", "LJ",
                "electrostatics", "total", "potential", "temperature")) +
                "%20s%15s" % ("thermo_potential", "thermo_kinetic") +
                ("" if aligned else "%15s" % "system_velocity_magnitude") + "\n")
        for k, r in enumerate(rows):
            vals = list(r[:11]) if aligned else (list(r) if k > 0 else list(r[:11]))
            f.write("%d" % int(vals[0]) + "".join("%15g" % v for v in vals[1:]) + "\n")


def energy_rows(rng, n, steps_per_row, eq_frac):
    """Rows with a potential energy that relaxes, then fluctuates (so that the trust factor finds
    an equilibrium part), and kinetic energy fluctuating about 1.5."""
    rows = []
    for k in range(n):
        t = k * steps_per_row
        relax = max(0.0, 1.0 - k / (n * (1 - eq_frac))) if eq_frac < 1 else 0.0
        pe = -3.0 + 2.0 * relax + 0.004 * rng.standard_normal()
        ke = 1.5 + 0.01 * rng.standard_normal()
        total = pe + ke + 0.001 * rng.standard_normal()
        rows.append([t, ke, 0.2, 0.1, -0.5, 0.05, total, pe, 2 * ke / 3, 0.0, 0.0, 1e-9])
    return rows


def make_case(name, seed, S, L, n_frames, frame_every, energy_n, eq_frac, aligned=False):
    rng = np.random.default_rng(seed)
    off = template_offsets(rng)
    types1 = bead_types()
    centres = layout(L, rng, S)
    frames = []
    for f in range(n_frames):
        shift = np.round(rng.uniform(-0.25, 0.25, (S, 3)) / Q) * Q if f > 0 else np.zeros((S, 3))
        pos = (centres + shift)[:, None, :] + off[None, :, :]
        pos = wrap(pos.reshape(-1, 3), L)
        frames.append((f * frame_every, pos, np.tile(types1, S)))
    rows = energy_rows(rng, energy_n, frame_every * n_frames // energy_n + 1, eq_frac)
    with tempfile.TemporaryDirectory() as wd:
        os.makedirs(os.path.join(wd, "outfiles"))
        write_trajectory(os.path.join(wd, "outfiles", "ovito.lammpstrj"), frames, L)
        write_energy(os.path.join(wd, "outfiles", "energy.out"), rows, aligned)
        r = subprocess.run([REF_ANALYZE], cwd=wd, capture_output=True, text=True, check=True)
        out = {}
        for fn in ("analysis.ms", "analysis.gr", "analysis.so", "analysis.rdat", "info.gr"):
            p = os.path.join(wd, "outfiles", fn)
            out[fn] = open(p).read() if os.path.exists(p) else ""
        traj = open(os.path.join(wd, "outfiles", "ovito.lammpstrj")).read()
        energy = open(os.path.join(wd, "outfiles", "energy.out")).read()
    np.savez_compressed(
        os.path.join(HERE, f"analysis_{name}.npz"),
        np_=NP, box=L, n_sub=S, trajectory=np.array(traj), energy=np.array(energy),
        ref_stdout=np.array(r.stdout),
        **{"out_" + k.replace(".", "_"): np.array(v) for k, v in out.items()})
    print(name, "frames", n_frames, "beads", S * NP, "->", {k: len(v) for k, v in out.items()})


if __name__ == "__main__":
    if not os.path.exists(REF_ANALYZE):
        sys.exit("build the reference first: make -f oracle/ref.mk")
    make_case("contacts", 2468, 40, 40.0, 6, 500, 200, 0.6)
    make_case("no_equilibrium", 1357, 30, 36.0, 4, 250, 120, 1.0)
    make_case("aligned_energy", 97531, 32, 38.0, 8, 400, 320, 0.5, aligned=True)
