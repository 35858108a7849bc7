"""CPU oracle of the learned warm start (test infrastructure only).

The reference has no learned component, so this is the restatement the GPU
network is checked against: features of a point (from the scene arrays),
the MLP forward pass, its backward pass and Adam, in numpy float64.

``forward``/``backward`` take ``bf16=True`` to round, like the GPU, every
tensor-core operand to BF16 (features, weights, hidden activations, the
output gradient and the hidden-layer gradients), accumulating in float64;
with ``bf16=False`` they are the exact float64 network (the one whose
gradient is checked against finite differences).  Only tests/,
__graft_entry__.smoke() and bench.py's cpu_baseline leg import this module.
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID, N_OUT = 16, 64, 3
OFF_W1 = 0
OFF_W2 = OFF_W1 + N_HID * N_IN
OFF_B2 = OFF_W2 + N_HID * N_HID
OFF_W3 = OFF_B2 + N_HID
OFF_B3 = OFF_W3 + N_OUT * N_HID
N_PARAMS = OFF_B3 + N_OUT

DISTANCE, BENDING = 0x001, 0x010


def bf16(a):
    """round float32 values to BF16 (nearest even), returned as float64"""
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[OFF_W1:OFF_W2].reshape(N_HID, N_IN), p[OFF_W2:OFF_B2].reshape(N_HID, N_HID),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3].reshape(N_OUT, N_HID), p[OFF_B3:N_PARAMS])


def pack(W1, W2, b2, W3, b3):
    return np.concatenate([np.ravel(W1), np.ravel(W2), np.ravel(b2), np.ravel(W3),
                           np.ravel(b3)]).astype(np.float64)


def init_params(seed=0):
    """He-style initialisation (uniform, fan-in scaled); output layer small"""
    rng = np.random.default_rng(seed)
    W1 = rng.uniform(-1, 1, (N_HID, N_IN)) * np.sqrt(3.0 / N_IN)
    W2 = rng.uniform(-1, 1, (N_HID, N_HID)) * np.sqrt(3.0 / N_HID)
    W3 = rng.uniform(-1, 1, (N_OUT, N_HID)) * 0.1 * np.sqrt(3.0 / N_HID)
    return pack(W1, W2, np.zeros(N_HID), W3, np.zeros(N_OUT)).astype(np.float32)


def _sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * _sig(z)


def dsilu(z):
    s = _sig(z)
    return s * (1.0 + z * (1.0 - s))


def _r(a, on):
    return bf16(a) if on else np.asarray(a, np.float64)


def forward(params, X, bf16_ops=True):
    """returns y (n, 3) and the cache for backward"""
    W1, W2, b2, W3, b3 = unpack(params)
    X = np.array(X, np.float64)
    X[:, 15] = 1.0
    Xb = _r(X, bf16_ops)
    W1b, W2b, W3b = _r(W1, bf16_ops), _r(W2, bf16_ops), _r(W3, bf16_ops)
    Z1 = Xb @ W1b.T
    H1 = _r(silu(Z1), bf16_ops)
    Z2 = H1 @ W2b.T + b2
    H2 = _r(silu(Z2), bf16_ops)
    Y = H2 @ W3b.T + b3
    return Y, (Xb, W1b, W2b, W3b, Z1, H1, Z2, H2)


def loss_and_grad(params, X, T, mask=None, bf16_ops=True):
    """L = 1/(2m) sum_{masked rows} |y - t|^2 and dL/dparams"""
    Y, (Xb, W1b, W2b, W3b, Z1, H1, Z2, H2) = forward(params, X, bf16_ops)
    n = len(Y)
    mk = np.ones(n) if mask is None else (np.asarray(mask) != 0).astype(np.float64)
    m = max(mk.sum(), 1.0)
    E = (Y - np.asarray(T, np.float64)) * mk[:, None]
    loss = 0.5 * np.sum(E * E) / m
    dY = E / m
    db3 = dY.sum(0)
    dYb = _r(dY.astype(np.float32), bf16_ops)
    dW3 = dYb.T @ H2
    dH2 = dYb @ W3b
    dZ2 = _r((dH2 * dsilu(Z2)).astype(np.float32), bf16_ops)
    dW2 = dZ2.T @ H1
    db2 = dZ2.sum(0)
    dH1 = dZ2 @ W2b
    dZ1 = _r((dH1 * dsilu(Z1)).astype(np.float32), bf16_ops)
    dW1 = dZ1.T @ Xb
    return loss, pack(dW1, dW2, db2, dW3, db3)


def adam(params, m, v, g, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """one Adam step (Kingma & Ba 2015, bias-corrected), step number t >= 1"""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** t)
    vh = v / (1 - b2 ** t)
    return params - lr * mh / (np.sqrt(vh) + eps), m, v


# ---------------------------------------------------------------------------
# features
# ---------------------------------------------------------------------------
def stencil(scene):
    """first six incident distance constraints (other point, rest length)
    and first four incident bending prims of every point, by prim id;
    lbar = mean incident rest length; wrel = w / (w + mean neighbour w)"""
    n = len(scene["pos"])
    pl, ind, ct = scene["prim_list"], scene["indices"], scene["ctype"]
    rl = scene["rest_length"]
    w = np.asarray(scene["mass"], np.float64)
    nb = -np.ones((n, 6), np.int64)
    rr = np.zeros((n, 6))
    hg = -np.ones((n, 4), np.int64)
    nd = np.zeros(n, np.int64)
    nh = np.zeros(n, np.int64)
    lsum = np.zeros(n)
    wsum = np.zeros(n)
    cnt = np.zeros(n)
    for p in range(len(ct)):
        s = pl[p, 0]
        if ct[p] == DISTANCE:
            a, b = ind[s], ind[s + 1]
            for i, j in ((a, b), (b, a)):
                if nd[i] < 6:
                    nb[i, nd[i]] = j
                    rr[i, nd[i]] = rl[p]
                nd[i] += 1
                lsum[i] += rl[p]
                wsum[i] += w[j]
                cnt[i] += 1
        elif ct[p] == BENDING:
            for i in ind[s:s + 4]:
                if nh[i] < 4:
                    hg[i, nh[i]] = p
                nh[i] += 1
    lbar = np.where(cnt > 0, lsum / np.maximum(cnt, 1), 0.0).astype(np.float32)
    wm = np.where(cnt > 0, wsum / np.maximum(cnt, 1), 0.0)
    wrel = np.where(w + wm > 0, w / np.where(w + wm > 0, w + wm, 1), 0.0)
    return {"nb": nb, "rest": rr.astype(np.float32), "hinge": hg, "lbar": lbar,
            "wrel": wrel.astype(np.float32), "w": w}


def dihedral_dev(scene, pos, prim):
    """wrapped theta - theta0 of bending prim `prim` at positions pos"""
    s = scene["prim_list"][prim, 0]
    i = scene["indices"][s:s + 4]
    q = np.asarray(pos, np.float64)[i]
    E = q[1] - q[0]
    na = np.cross(q[2] - q[0], q[2] - q[1])
    nb = np.cross(q[3] - q[1], q[3] - q[0])
    el = np.linalg.norm(E)
    if el == 0:
        return 0.0
    c = np.arctan2(np.dot(np.cross(na, nb), E) / el, np.dot(na, nb)) - scene["rest_angle"][prim]
    if c > np.pi:
        c -= 2 * np.pi
    if c < -np.pi:
        c += 2 * np.pi
    return c


def features(scene, pos, dprev=None, st=None, scales=None):
    """(n, 16) features of every point at positions pos (float64); scales
    (17) multiply features 0..14 as in the network's input"""
    st = stencil(scene) if st is None else st
    pos = np.asarray(pos, np.float64)
    n = len(pos)
    F = np.zeros((n, 16))
    for k in range(6):
        j = st["nb"][:, k]
        ok = j >= 0
        d = np.linalg.norm(pos[ok] - pos[j[ok]], axis=1)
        F[ok, k] = (d - st["rest"][ok, k]) / st["rest"][ok, k]
    lb = st["lbar"].astype(np.float64)
    inv = np.where(lb > 0, 1.0 / np.where(lb > 0, lb, 1), 0.0)
    if dprev is not None:
        F[:, 6:9] = np.asarray(dprev, np.float64) * inv[:, None]
    F[:, 9] = st["wrel"]
    F[:, 10] = (st["w"] == 0).astype(np.float64)
    cache = {}
    for k in range(4):
        h = st["hinge"][:, k]
        for i in np.nonzero(h >= 0)[0]:
            p = int(h[i])
            if p not in cache:
                cache[p] = dihedral_dev(scene, pos, p)
            F[i, 11 + k] = cache[p]
    if scales is not None:
        F[:, :15] *= np.asarray(scales, np.float64)[:15]
    F[:, 15] = 1.0
    return F
