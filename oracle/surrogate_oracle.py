"""CPU restatement of the surrogate's geometry and training targets, for tests only (the checker,
never the product).  The learned part has no reference counterpart; the physics it stands in for
is the pair loop of forceCalculation (src/forces.cpp:67-145) restricted to subunit pairs whose
closest beads are beyond the switch radius, where only the Debye-Hueckel term (src/forces.cpp:
95-108) is left (the LJ/WCA cut-offs are shorter).  States capsid-souffle_gb300/csrc/surrogate.cu:

  body frame   e1 = unit(anchor1 - centre), e3 = unit(e1 x (anchor2 - centre)), e2 = e3 x e1,
               anchors = the bead farthest from the centre in the rest shape and the bead
               farthest from that axis
  far pairs    ordered (A, B), B a candidate of A (centre distance^2 < 2.25 r_list^2,
               src/functions.cpp:80-91), closest bead distance >= switch radius, in ascending B
  targets      g_i = body-frame force on A's bead i from B; F = sum g, tau = sum d_i x g_i,
               w = J^-1 tau with J = sum |d|^2 I - d d^T, residual r_i = g_i - F/np - w x d_i
"""
import numpy as np


def min_image(d, box):
    return d - box * np.round(d / box)


def anchors(rest, center):
    d = rest - rest[center]
    b1 = int(np.argmax(np.linalg.norm(d, axis=1)))
    e1 = d[b1] / np.linalg.norm(d[b1])
    b2 = int(np.argmax(np.linalg.norm(np.cross(e1, d), axis=1)))
    return b1, b2


def frame(pos_sub, center, b1, b2, box):
    """(e1, e2, e3, m, d): frame axes, centre of mass offset from the centre bead, and bead
    offsets from the centre bead (minimum image)."""
    d = min_image(pos_sub - pos_sub[center], box)
    m = d.mean(axis=0)
    e1 = d[b1] / np.linalg.norm(d[b1])
    e3 = np.cross(e1, d[b2])
    e3 /= np.linalg.norm(e3)
    e2 = np.cross(e3, e1)
    return e1, e2, e3, m, d


def far_pairs(pos, n_sub, np_, center, box, r_list, r_switch, reach=np.inf):
    """Candidate subunit pairs (the centre-bead prefilter) whose closest bead pair is at least
    r_switch apart, leaving out pairs whose closest bead pair lies beyond ``reach`` (the largest
    pair cut-off, with the GPU classifier's 1e-4 relative margin on the square): those exert no
    force and are in neither list."""
    p = pos.reshape(n_sub, np_, 3)
    c = p[:, center, :]
    out = []
    for a in range(n_sub):
        dc = min_image(c - c[a], box)
        cand = np.nonzero((dc ** 2).sum(axis=1) < 2.25 * r_list ** 2)[0]
        for b in cand:
            if b == a:
                continue
            dd = min_image(p[a][:, None, :] - p[b][None, :, :], box)
            dmin = float(np.sqrt((dd ** 2).sum(-1).min()))
            if dmin >= r_switch and not dmin * dmin > reach * reach * 1.0001:
                out.append((a, int(b), dmin))
    return out


def dh_weights(charge, sigma, kappa, lb):
    return charge * np.exp(kappa * sigma / 2) / (1 + kappa * sigma / 2) * np.sqrt(lb)


def exact_far_forces(pa, pb, box, w, kappa, ecut_el, r_list):
    """Debye-Hueckel forces on the beads of A from all beads of B (pairs inside the list radius
    and the DH cut-off), lab frame."""
    d = min_image(pa[:, None, :] - pb[None, :, :], box)
    r2 = (d ** 2).sum(-1)
    r = np.sqrt(r2)
    ww = w[:, None] * w[None, :]
    c = np.where((r2 < r_list ** 2) & (r2 < ecut_el ** 2) & (ww != 0),
                 ww * np.exp(-kappa * r) / r2 * (kappa + 1 / r), 0.0)
    return (d * c[..., None]).sum(axis=1)


def targets(f_lab, fr):
    e1, e2, e3, m, d = fr
    R = np.stack([e1, e2, e3])           # rows: body axes
    g = f_lab @ R.T                       # body-frame forces
    db = (d - m) @ R.T                    # body-frame positions about the centre of mass
    F = g.sum(axis=0)
    tau = np.cross(db, g).sum(axis=0)
    J = (db ** 2).sum() * np.eye(3) - db.T @ db
    w = np.linalg.solve(J, tau)
    res = g - F / len(g) - np.cross(w, db)
    return np.concatenate([F, tau, res.ravel()]), g, db, J


def reconstruct(t, db, J):
    """Body-frame per-bead forces from (F, tau, residuals)."""
    n = db.shape[0]
    F, tau, res = t[:3], t[3:6], t[6:6 + 3 * n].reshape(n, 3)
    w = np.linalg.solve(J, tau)
    return F / n + np.cross(w, db) + res
