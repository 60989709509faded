"""CPU restatement of the reference's post-run analysis, for tests only (the checker, never the
product).

Follows analyze_output (src/analysis.cpp:16-297) and compute_MD_trust_factor_R
(src/functions.cpp:119-258) step by step, including the behaviour of the code as shipped:

* energy.out is read as a token stream: 11 header tokens skipped, then groups of 11 tokens
  (src/functions.cpp:133-135), although the MD writes a 12-token header and 12 columns after
  row 0, so the groups drift through the file; a group whose columns 1, 2, 5, 7 or 8 do not
  parse as a number is skipped (src/functions.cpp:136-147; the number test is the stream
  extraction of boost::lexical_cast<double>);
* the section slope divides by xx_sum - n x_m y_m (src/functions.cpp:174), section 10 is always
  flat (:195), and the equilibrium step is time[index] truncated to an integer (:205);
* in the frame loop the beads' half-box vector is never set (BEAD's default, src/bead.h:62-69,
  with only bx assigned at src/analysis.cpp:88-92), so dist() (src/functions.h:42-56) shifts
  every nonzero coordinate difference by a full box length: per axis |d| becomes L - |d|
  (IMAGE_REFERENCE).  IMAGE_MINIMUM is the minimum image for comparison;
* oligomers are the connected components of subunits with any bead pair closer than 2
  (src/analysis.cpp:144-178), sub-oligomers the connected components of type-0 beads closer
  than 2 inside an oligomer (:191-238); the mass spectrum is averaged over the analysed frames
  weighted by size (:268-276);
* output files use C++ stream formatting: 6 significant digits, and a setw(15) that carries
  over to the first value of the next line (:134-137, :240-243, :279-281, functions.cpp:250-252).

Parsing is the reference's; distances are evaluated in double (the reference: long double) from
the same decimal inputs.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import re

import numpy as np

IMAGE_REFERENCE = 0
IMAGE_MINIMUM = 1

_NUM = re.compile(r"[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?$")


def _lexical_double(tok: str):
    """boost::lexical_cast<double> as an istringstream extraction with nothing left over."""
    return float(tok) if _NUM.match(tok) else None


def cpp_g(v) -> str:
    """operator<< of a double with default stream flags: %g with 6 significant digits."""
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    if math.isnan(v):
        return "-nan" if math.copysign(1.0, v) < 0 else "nan"
    if math.isinf(v):
        return "inf" if v > 0 else "-inf"
    return "%g" % v


class CppStream:
    """The piece of std::ostream state the reference's writers rely on: a pending field width
    set by setw and consumed by the next formatted value."""

    def __init__(self):
        self.parts = []
        self.width = 0

    def val(self, v):
        s = cpp_g(v) if not isinstance(v, str) else v
        self.parts.append(s.rjust(self.width) if self.width else s)
        self.width = 0
        return self

    def setw(self, w):
        self.width = w
        return self

    def endl(self):
        self.parts.append("\n")
        return self

    def text(self) -> str:
        return "".join(self.parts)


class RunningStat:
    """Welford mean / sample variance (src/RunningStat.h:9-47)."""

    def __init__(self):
        self.n = 0
        self.m = self.s = 0.0

    def push(self, x):
        self.n += 1
        if self.n == 1:
            self.m, self.s = x, 0.0
        else:
            m = self.m + (x - self.m) / self.n
            self.s = self.s + (x - self.m) * (x - m)
            self.m = m

    def stdev(self):
        return math.sqrt(self.s / (self.n - 1)) if self.n > 1 else 0.0


def trust_factor(energy_text: str) -> dict:
    """compute_MD_trust_factor_R: the equilibrium step, the flat-section count and R."""
    tok = energy_text.split()[11:]
    time, ext, ke, pe = [], [], [], []
    skipped = 0
    for g in range(len(tok) // 11):
        c = tok[11 * g: 11 * g + 11]
        vals = [_lexical_double(c[k]) for k in (0, 1, 6, 7, 4)]
        if any(v is None for v in vals):
            skipped += 1
            continue
        c1, c2, c7, c8, _c5 = vals
        time.append(c1)
        ext.append(c7)
        ke.append(c2)
        pe.append(c8)
    nsec = 10
    ss = len(pe) // nsec
    flat = []
    for i in range(nsec):
        xs = ys = xys = xxs = 0.0
        rs = RunningStat()
        for j in range(ss):
            y = pe[i * ss + j]
            xs += j
            ys += y
            xys += j * y
            xxs += float(j * j)
            rs.push(y)
        if ss > 0:
            xm, ym = xs / float(ss), ys / float(ss)
            den = xxs - float(ss) * xm * ym
            num = xys - float(ss) * xm * ym
            slope = num / den if den != 0 else (math.nan if num == 0 else math.copysign(math.inf, num))
        else:
            slope = math.nan
        sd = rs.stdev()
        flat.append(sd < 0.02 and slope < 1e-4 and slope > -1e-4)
    flat[nsec - 1] = True
    nflat, idx = 0, 0
    for i in range(nsec - 1, -1, -1):
        if flat[i]:
            nflat += 1
            idx = i * ss
        else:
            break
    hiteqm = int(time[idx])

    def mean_sd(v):
        m = 0.0
        for x in v:
            m += x
        m = m / len(v)
        s = 0.0
        for x in v:
            s += (x - m) * (x - m)
        return math.sqrt(s / len(v))

    ext_sd, ke_sd = mean_sd(ext), mean_sd(ke)
    R = ext_sd / ke_sd
    rdat = CppStream()
    rdat.val("Sample size ").val(len(ext)).endl()
    rdat.val("Standard Deviation: total energy, kinetic energy | R").endl()
    rdat.val(ext_sd).setw(15).val(ke_sd).setw(15).val(R).endl()
    return {"hiteqm": hiteqm, "flat_sections": nflat, "section_size": ss, "samples": len(ext),
            "skipped_groups": skipped, "ext_sd": ext_sd, "ke_sd": ke_sd, "R": R, "rdat": rdat.text()}


def read_trajectory(text: str):
    """Frames of ovito.lammpstrj as the reference reads them (src/analysis.cpp:77-113):
    (timestep, half box, types (N,), positions (N, 3))."""
    tok = text.split()
    p, frames = 0, []
    while p < len(tok):
        step = int(tok[p + 2])
        n = int(tok[p + 7])
        half = float(tok[p + 12])
        p += 8 + 5 + 13
        rows = np.array(tok[p: p + 7 * n], dtype=object).reshape(n, 7)
        p += 7 * n
        frames.append((step, half, rows[:, 1].astype(np.int64), rows[:, 2:5].astype(np.float64)))
    return frames


def subunit_size(n_beads: int) -> int:
    """src/analysis.cpp:81-83: the last of 41, 43, 78 that divides the bead count (0 if none)."""
    size = 0
    for k in (41, 43, 78):
        if n_beads % k == 0:
            size = k
    return size


def separation(pa, pb, L, image):
    """dist() magnitude between bead rows pa (..., 3) and pb (..., 3)."""
    d = pa - pb
    if image == IMAGE_REFERENCE:
        d = np.where(d > 0, d - L, np.where(d < 0, d + L, d))
    else:
        d = np.where(d > L / 2, d - L, np.where(d < -L / 2, d + L, d))
    return np.sqrt(d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1] + d[..., 2] * d[..., 2])


def _components(n, edges):
    parent = list(range(n))

    def find(x):
        while parent[x] != x:
            parent[x] = parent[parent[x]]
            x = parent[x]
        return x

    for a, b in edges:
        ra, rb = find(a), find(b)
        if ra != rb:
            parent[max(ra, rb)] = min(ra, rb)
    return [find(x) for x in range(n)]


def frame_analysis(types, pos, L, np_, image=IMAGE_REFERENCE, pcf_type=5, pcf_bins=100,
                   so_type=0, contact=2.0):
    """One analysed frame: pair-correlation counts, oligomer sizes, sub-oligomer sizes."""
    n = len(pos)
    S = n // np_
    dg = L / (2 * pcf_bins)
    half = L / 2
    gr = np.zeros(pcf_bins, dtype=np.int64)
    idx = np.nonzero(types == pcf_type)[0]
    for a in range(len(idx)):
        d = separation(pos[idx[a]][None, :], pos[idx[a + 1:]], L, image)
        d = d[d < half]
        np.add.at(gr, np.floor(d / dg).astype(np.int64), 1)
    # bead contacts closer than `contact` between different subunits
    sub = np.arange(n) // np_
    edges = set()
    for i in range(n):
        d = separation(pos[i][None, :], pos[i + 1:], L, image)
        for j in np.nonzero(d < contact)[0] + i + 1:
            if sub[i] != sub[j]:
                edges.add((sub[i], sub[j]))
    lab = _components(S, edges)
    olig = np.bincount(np.unique(lab, return_inverse=True)[1])
    # sub-oligomers: type-0 beads in contact (an oligomer holds every bead in contact with it)
    t0 = np.nonzero(types == so_type)[0]
    e0 = []
    for a in range(len(t0)):
        d = separation(pos[t0[a]][None, :], pos[t0[a + 1:]], L, image)
        for b in np.nonzero(d < contact)[0] + a + 1:
            e0.append((a, b))
    lab0 = _components(len(t0), e0)
    so = np.bincount(np.unique(lab0, return_inverse=True)[1]) if len(t0) else np.zeros(0, dtype=np.int64)
    return gr, olig, so


def analyze(energy_text: str, trajectory_text: str, np_: int | None = None, image=IMAGE_REFERENCE,
            pcf_type=5, pcf_bins=100, so_type=0) -> dict:
    """analyze_output: the texts of analysis.rdat, .gr, .so, .ms and info.gr."""
    tf = trust_factor(energy_text)
    frames = read_trajectory(trajectory_text)
    n = len(frames[0][2])
    np_ = np_ or subunit_size(n)
    S = n // np_
    L = frames[0][1] * 2
    dg = L / (2 * pcf_bins)
    n_type = int(np.count_nonzero(frames[0][2] == pcf_type))
    rho = n_type / (L * L * L)
    gr_s, so_s = CppStream(), CppStream()
    ms_frames = []
    for step, _half, types, pos in frames:
        if step < tf["hiteqm"]:
            continue
        gr, olig, so = frame_analysis(types, pos, L, np_, image, pcf_type, pcf_bins, so_type)
        for v in gr:
            gr_s.val(int(v)).setw(15)
        gr_s.endl()
        ms = np.zeros(S, dtype=np.int64)
        for size in olig:
            ms[size - 1] += 1
        ms_frames.append(ms)
        sob = np.zeros(2 * S, dtype=np.int64)
        for size in so:
            sob[(size - 1) // 3] += 1
        for v in sob:
            so_s.val(int(v)).setw(15)
        so_s.endl()
    hist = np.zeros(S)
    for ms in ms_frames:
        for j in range(S):
            hist[j] += ms[j] * (j + 1)
    ms_s = CppStream()
    with np.errstate(invalid="ignore", divide="ignore"):
        for j in range(S):
            ms_s.val(float(hist[j] / len(ms_frames)) if ms_frames else math.nan).setw(15)
    ms_s.endl()
    info = CppStream()
    info.val("Number of Subunits: ").val(S).endl()
    info.val("PCF bin size: ").val(dg).endl()
    info.val("PCF bin number: ").val(pcf_bins).endl()
    info.val("Box size: ").val(L).val(" ").val(L).val(" ").val(L).endl()
    info.val("Number density: ").val(rho).endl()
    info.val("Bead Type: ").val(pcf_type).endl()
    return {"analysis.rdat": tf["rdat"], "analysis.gr": gr_s.text(), "analysis.so": so_s.text(),
            "analysis.ms": ms_s.text(), "info.gr": info.text(), "trust": tf,
            "frames_analysed": len(ms_frames)}


_PORT = None


def port_frame(types, pos, L, np_, image=IMAGE_REFERENCE, pcf_type=5, pcf_bins=100, so_type=0,
               contact=2.0):
    """One frame through the C restatement of the reference's loops (oracle/analysis_port.c, long
    double, single thread): (gr (bins,), oligomer size histogram (S,), sub-oligomer bins (2S,))."""
    global _PORT
    if _PORT is None:
        lib = C.CDLL(os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "liboracle.so"))
        lp = C.POINTER(C.c_longlong)
        lib.oracle_analysis_frame.argtypes = [C.c_long, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                              C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                              lp, lp, lp]
        _PORT = lib
    t = np.ascontiguousarray(types, dtype=np.int32)
    p = np.ascontiguousarray(pos, dtype=np.float64)
    n = len(t)
    S = n // np_
    gr = np.zeros(pcf_bins, dtype=np.int64)
    ms = np.zeros(S, dtype=np.int64)
    so = np.zeros(2 * S, dtype=np.int64)
    lp = C.POINTER(C.c_longlong)
    rc = _PORT.oracle_analysis_frame(n, np_, t.ctypes.data_as(C.POINTER(C.c_int)),
                                     p.ctypes.data_as(C.POINTER(C.c_double)), L, image, pcf_type, pcf_bins,
                                     so_type, contact, gr.ctypes.data_as(lp), ms.ctypes.data_as(lp),
                                     so.ctypes.data_as(lp))
    if rc:
        raise ValueError("a sub-oligomer lies past the histogram")
    return gr, ms, so
