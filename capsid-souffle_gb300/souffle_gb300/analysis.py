"""ctypes binding of the trajectory analysis in include/souffle_analysis.h.

The per-frame products of the reference's analyze_output (src/analysis.cpp:117-262) on the GPU:
pair-correlation counts, the oligomer size histogram and the sub-oligomer histogram.  No
fallback: without the library or a GPU every call raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import gpu

IMAGE_REFERENCE = 0
IMAGE_MINIMUM = 1


class AnalysisOptions_(C.Structure):
    _fields_ = [("image", C.c_int32), ("pcf_type", C.c_int32), ("pcf_bins", C.c_int32),
                ("so_type", C.c_int32), ("contact", C.c_double)]


def _load():
    lib = gpu.load()
    if getattr(lib, "_analysis_typed", False):
        return lib
    vp, i64p = C.c_void_p, C.POINTER(C.c_int64)
    dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int32)
    lib.souffle_analysis_default_options.restype = None
    lib.souffle_analysis_default_options.argtypes = [C.POINTER(AnalysisOptions_)]
    lib.souffle_analysis_create.argtypes = [C.c_int64, C.c_int32, C.c_double, C.POINTER(AnalysisOptions_),
                                            C.c_int32, C.POINTER(vp)]
    lib.souffle_analysis_destroy.argtypes = [vp]
    lib.souffle_analysis_frames.argtypes = [vp, C.c_int64, dp, ip, i64p, i64p, i64p, ip]
    lib.souffle_analysis_enqueue.argtypes = [vp, vp, vp, vp, vp, vp, vp]
    lib.souffle_analysis_synchronize.argtypes = [vp]
    lib.souffle_analysis_stream.restype = C.c_void_p
    lib.souffle_analysis_stream.argtypes = [vp]
    lib.souffle_analysis_last_counts.argtypes = [vp, i64p, i64p]
    lib._analysis_typed = True
    return lib


class Analysis:
    """One analysis handle for trajectories of n_beads beads in subunits of beads_per_subunit."""

    def __init__(self, n_beads: int, beads_per_subunit: int, box: float, image: int = IMAGE_REFERENCE,
                 pcf_type: int = 5, pcf_bins: int = 100, so_type: int = 0, contact: float = 2.0,
                 device: int = 0):
        self.lib = _load()
        o = AnalysisOptions_(image, pcf_type, pcf_bins, so_type, contact)
        h = C.c_void_p()
        gpu._check(self.lib.souffle_analysis_create(int(n_beads), int(beads_per_subunit), float(box), C.byref(o),
                                                    int(device), C.byref(h)))
        self.h = h
        self.n_beads = int(n_beads)
        self.n_sub = int(n_beads) // int(beads_per_subunit)
        self.bins = int(pcf_bins)

    def frames(self, pos: np.ndarray, types: np.ndarray | None) -> dict:
        """pos (F, N, 3) float64; types (F, N) or (N,) int, or None to keep the last types."""
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, self.n_beads, 3)
        F = pos.shape[0]
        tp = None
        if types is not None:
            t = np.asarray(types, dtype=np.int32)
            if t.ndim == 1:
                t = np.broadcast_to(t, (F, self.n_beads))
            tp = np.ascontiguousarray(t)
        pcf = np.zeros((F, self.bins), dtype=np.int64)
        olig = np.zeros((F, self.n_sub), dtype=np.int64)
        so = np.zeros((F, 2 * self.n_sub), dtype=np.int64)
        labels = np.zeros((F, self.n_sub), dtype=np.int32)
        i64 = lambda a: a.ctypes.data_as(C.POINTER(C.c_int64))  # noqa: E731
        gpu._check(self.lib.souffle_analysis_frames(
            self.h, F, gpu._dp(pos), gpu._ip(tp) if tp is not None else None, i64(pcf), i64(olig), i64(so),
            gpu._ip(labels)))
        return {"pcf": pcf, "oligomers": olig, "so_bins": so, "labels": labels}

    def enqueue(self, pos_dev: int, types_dev: int, pcf_dev: int, olig_dev: int, so_dev: int,
                labels_dev: int | None = None) -> None:
        """Device pointers (integers); results are valid after synchronize()."""
        gpu._check(self.lib.souffle_analysis_enqueue(self.h, pos_dev, types_dev, pcf_dev, olig_dev, so_dev,
                                                     labels_dev))

    def synchronize(self) -> None:
        gpu._check(self.lib.souffle_analysis_synchronize(self.h))

    def stream(self) -> int:
        return self.lib.souffle_analysis_stream(self.h)

    def last_counts(self) -> tuple[int, int]:
        a, b = C.c_int64(), C.c_int64()
        gpu._check(self.lib.souffle_analysis_last_counts(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def close(self) -> None:
        if self.h:
            self.lib.souffle_analysis_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
