"""CPU restatement of the surrogate network, for tests only (the checker, never the product).

The network has no counterpart in the reference (SOUFFLE has no learned part), so this oracle
is pinned by finite differences of its own loss (tests/test_mlp_oracle.py) instead of by
reference outputs.  It states the math of capsid-souffle_gb300/csrc/mlp.cu:

    z_l = a_{l-1} W_l^T + b_l,  a_l = SiLU(z_l) for the three hidden layers, y = a_3 W_4^T + b_4
    loss = mean over m x n_out of (y - t)^2

``emulate=True`` also reproduces the GPU's rounding points: BF16 weights, inputs, hidden
activations and back-propagated gradients (round to nearest even), FP32 elsewhere.
Parameters are one flat FP32 array: W1 [width][n_in], b1, W2, b2, W3, b3, W4 [n_out][width], b4.
"""
import numpy as np


def bf16(x):
    """Round float32 values to the nearest bfloat16 (ties to even), returned as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(x.shape)


def shapes(n_in, width, n_out):
    dims = [n_in, width, width, width, n_out]
    return [((dims[l + 1], dims[l]), (dims[l + 1],)) for l in range(4)]


def unpack(p, n_in, width, n_out):
    out, k = [], 0
    for (ws, bs) in shapes(n_in, width, n_out):
        nw = ws[0] * ws[1]
        out.append((p[k:k + nw].reshape(ws), p[k + nw:k + nw + bs[0]]))
        k += nw + bs[0]
    assert k == len(p)
    return out


def pack(layers):
    return np.concatenate([np.concatenate([w.ravel(), b.ravel()]) for w, b in layers])


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def loss_and_grads(p, x, t, n_in, width, n_out, emulate=True):
    """Loss and flat gradient for one batch x [m][n_in], t [m][n_out]."""
    dt = np.float32 if emulate else np.float64
    rnd = bf16 if emulate else (lambda a: a)
    layers = [(rnd(w.astype(dt)), b.astype(dt)) for w, b in unpack(np.asarray(p, dt), n_in, width, n_out)]
    m = x.shape[0]
    a = [rnd(np.asarray(x, dt))]
    zs = []
    for l, (w, b) in enumerate(layers):
        z = (a[-1].astype(np.float64) @ w.T.astype(np.float64)).astype(dt) + b
        if l < 3:
            zs.append(z)
            a.append(rnd((z * _sig(z)).astype(dt)))
        else:
            y = z
    d = y - np.asarray(t, dt)
    loss = float(np.mean(d.astype(np.float64) ** 2))
    dz = rnd((2.0 * d / (m * n_out)).astype(dt))
    grads = [None] * 4
    for l in range(3, -1, -1):
        w, _ = layers[l]
        gw = (dz.T.astype(np.float64) @ a[l].astype(np.float64)).astype(dt)
        gb = dz.astype(np.float64).sum(axis=0).astype(dt)
        grads[l] = (gw, gb)
        if l == 0:
            break
        z = zs[l - 1]
        s = _sig(z)
        da = (dz.astype(np.float64) @ w.astype(np.float64)).astype(dt)
        dz = rnd((da * (s * (1 + z * (1 - s)))).astype(dt))
    return loss, pack(grads)


def forward(p, x, n_in, width, n_out, emulate=True):
    dt = np.float32 if emulate else np.float64
    rnd = bf16 if emulate else (lambda a: a)
    a = rnd(np.asarray(x, dt))
    for l, (w, b) in enumerate(unpack(np.asarray(p, dt), n_in, width, n_out)):
        z = (a.astype(np.float64) @ rnd(w.astype(dt)).T.astype(np.float64)).astype(dt) + b.astype(dt)
        a = rnd((z * _sig(z)).astype(dt)) if l < 3 else z
    return a
