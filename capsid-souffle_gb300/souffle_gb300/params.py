"""Run parameters with SOUFFLE's command-line letters and its unit derivation.

Option letters and defaults follow the reference option table
(src/md.cpp:53-90).  ``derive`` repeats the reference's conversion from
physical inputs to reduced units (src/md.cpp:135-173, pair-list capacity
src/md.cpp:229-239) in the same double-precision expression order, so the
derived cut-offs are bit-identical to the reference's.
"""
from __future__ import annotations

import dataclasses
import math

AVOGADRO = 6.022e23    # src/md.cpp:45
BOLTZMANN = 1.3806e-23  # src/md.cpp:46
PI_REF = 3.14159        # src/md.cpp:49


@dataclasses.dataclass
class CliOptions:
    """The reference's options (src/md.cpp:53-90), same letters and defaults."""

    D: str = "m"           # dynamics: 'm' = MD with Nose-Hoover chain, 'b' = Brownian
    f: str = "41part_c"    # infile name under infiles/
    C: float = 200.0       # capsomere concentration (uM)
    c: float = 500.0       # salt concentration (mM)
    S: float = 64          # number of subunits
    s: float = 50.0        # stretching constant ks (kT)
    b: float = 20.0        # bending constant kb (kT)
    T: float = 2500        # number of MD steps
    t: float = 0.004       # time step
    r: float = 1.0         # friction (Brownian only)
    d: float = 100.0       # damping (Brownian only)
    q: float = 5           # Nose-Hoover chain length
    Q: float = 10.0        # Nose-Hoover mass
    K: float = 298.0       # temperature (K)
    e: float = 12.0        # electrostatic cut-off in screening lengths (0 = none)
    R: bool = True         # restart from outfiles/restart_* if present
    X: bool = False        # preformed clusters
    V: bool = True         # verbose
    E: float = 2.0         # attractive LJ well depth
    B: int = 20            # pair-list rebuild period (steps)
    L: float = 7.5         # pair-list skin added to the largest cut-off
    M: int = 1000          # movie (ovito.lammpstrj) period
    W: int = 1000          # energy.out period
    w: int = 1000000       # restart file period
    N: int = 4             # unused by the MD path
    p: bool = False        # encapsulation big beads
    a: float = 3.0
    G: float = -78.0
    m: int = 1
    H: float = 3.5


@dataclasses.dataclass
class Derived:
    box: float
    T_reduced: float
    ecut: float
    lb: float
    ni: float
    kappa: float
    ecut_el: float
    nlist_cutoff: float
    nlist_capacity: int
    si_time: float


def derive(opt: CliOptions, sigma_si: float, mass_si: float, n_beads: int) -> Derived:
    """src/md.cpp:135-173 and :229-239, same expression order."""
    si_energy = opt.K * BOLTZMANN
    si_time = math.sqrt(sigma_si * sigma_si * mass_si / si_energy)
    T = opt.K / float(298)
    box_x = math.pow((opt.S * 1000 / (opt.C * math.pow(sigma_si, 3) * AVOGADRO)), 1.0 / 3.0)
    ecut = 2.5 * (sigma_si / 1e-9)
    lb = (0.701e-9) / sigma_si
    qs = 1.0
    ni = opt.c * AVOGADRO * sigma_si * sigma_si * sigma_si
    kappa = math.sqrt(8 * PI_REF * ni * lb * qs * qs)
    screen = 1 / kappa
    ecut_el = screen * opt.e
    if ecut_el > ecut:
        nl = ecut_el + opt.L
    else:
        nl = ecut + opt.L
    cap = math.ceil((nl + 0.5) * (nl + 0.5) * (nl + 0.5))
    if cap > n_beads:
        cap = n_beads
    return Derived(box_x, T, ecut, lb, ni, kappa, ecut_el, nl, int(cap), si_time)
