"""Run the compiled reference dump (oracle/_ref/ref_dump) and parse its output.

Test infrastructure: used to generate the golden fixtures in this folder and
by the container-only tests that compare the oracle with the reference live.
"""
from __future__ import annotations

import os
import subprocess

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF_DUMP = os.path.join(REPO, "oracle", "_ref", "ref_dump")
REF_RUN = os.path.join(REPO, "oracle", "_ref", "ref_run")


def _num(s: str) -> float:
    """Parse a C99 hex float (exact) or a decimal."""
    return float.fromhex(s) if "0x" in s.lower() else float(s)


def available() -> bool:
    return os.path.exists(REF_DUMP) and os.path.exists(REF_RUN)


def run_dump(workdir: str, args: list[str]) -> dict:
    out = subprocess.run([REF_DUMP] + args, cwd=workdir, check=True, capture_output=True,
                         text=True).stdout
    P, F, N, E, BB = {}, {}, {}, {}, {}
    ke = None
    big = None
    for line in out.splitlines():
        t = line.split()
        if not t:
            continue
        if t[0] == "P":
            P[t[1]] = _num(t[2])
        elif t[0] == "F":
            F[int(t[1])] = [_num(x) for x in t[2:11]]
        elif t[0] == "N":
            N[int(t[1])] = [int(x) for x in t[3:3 + int(t[2])]]
        elif t[0] == "E":
            E[int(t[1])] = [_num(x) for x in t[2:7]]
        elif t[0] == "K":
            ke = _num(t[1])
        elif t[0] == "BB":
            BB[int(t[1])] = [_num(x) for x in t[2:5]]
        elif t[0] == "G":
            big = (_num(t[1]), _num(t[2]))
    n = len(F)
    f = np.array([F[i] for i in range(n)])
    e = np.array([E[i] for i in range(n)])
    return dict(params=P, tforce=f[:, 0:3], sforce=f[:, 3:6], bforce=f[:, 6:9],
                nlist=[N[i] for i in range(n)], se=e[:, 0], ke=e[:, 1], be=e[:, 2],
                ne=e[:, 3], ce=e[:, 4], ke_total=ke,
                big_pos=np.array([BB[i] for i in range(len(BB))]).reshape(-1, 3), big_energies=big)
