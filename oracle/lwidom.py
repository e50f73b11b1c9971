"""Oracle for the learned Widom proposal (test infrastructure, not product code).

A numpy restatement of what the device computes for the learned insertion
proposal, so that tests can check the CUDA kernels value for value:

* sub-cell occupancy and the 27-bit neighbourhood pattern of every sub-cell;
* the MLP 27 -> 64 -> 64 -> 1 with the device's rounding points: operands of
  the tensor-core products (inputs, W1, hidden layer 1, W2, and in the
  backward pass dh2, dh1) are rounded to bfloat16, every product accumulates
  in FP32, the output layer runs in FP32;
* binary cross-entropy with logits and its gradient, per-sample weights;
* Adam;
* the mixture proposal and its importance weights, replayed from the same
  Philox draws as the device.

The uniform Widom test itself (compute_mu, src/compute_widom_chem_pot.c:32-182)
is the reference's; only the proposal of insertion points is new, and each
point carries the weight 1 / (V q(x)) so that the estimate of
<exp(-beta dU)> = P(insertion succeeds) stays unbiased.
"""
from __future__ import annotations

import numpy as np

from .philox import draw4

HIDDEN = 64
KIN = 32          # 27 occupancy inputs, the constant 1 (bias of layer 1), 4 zeros
BIAS_COL = 27
TAG_LWIDOM = 6


# ------------------------------------------------------------------ bfloat16
def bf16(x) -> np.ndarray:
    """Round float32 values to bfloat16 (round to nearest, ties to even),
    returned as float32."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    nan = np.isnan(a)
    out = (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32).reshape(a.shape)
    return np.where(nan, a, out)


# ------------------------------------------------------------------ sub-cells
def subgrid(box, target_edge: float = 0.5):
    """Sub-cells per axis: the most that keep the edge >= target_edge."""
    ns = np.array([max(3, int(np.floor(b / target_edge))) for b in box], dtype=np.int64)
    return ns


def subcell_of(x, inv_e, ns):
    c = np.floor(np.asarray(x, dtype=np.float64) * inv_e).astype(np.int64)
    return np.minimum(np.maximum(c, 0), ns - 1)


def occupancy(conf, box, ns):
    """Particles per sub-cell, saturating at 255; index cx + ns0 (cy + ns1 cz)."""
    box = np.asarray(box, dtype=np.float64)
    inv = ns.astype(np.float64) / box
    occ = np.zeros(int(np.prod(ns)), dtype=np.int64)
    idx = [subcell_of(conf[:, 1 + d], inv[d], ns[d]) for d in range(3)]
    flat = idx[0] + ns[0] * (idx[1] + ns[1] * idx[2])
    np.add.at(occ, flat, 1)
    return np.minimum(occ, 255).astype(np.uint8)


def patterns(occ, ns):
    """27-bit pattern of every sub-cell: bit (dx+1) + 3 (dy+1) + 9 (dz+1) set
    when that periodic neighbour holds a particle."""
    g = (occ.reshape(ns[2], ns[1], ns[0]) > 0).astype(np.uint32)
    pat = np.zeros_like(g)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                bit = (dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)
                pat |= np.roll(g, shift=(-dz, -dy, -dx), axis=(0, 1, 2)) << np.uint32(bit)
    return pat.reshape(-1)


def features(pat) -> np.ndarray:
    """Network input rows (float32, exact in bfloat16)."""
    pat = np.asarray(pat, dtype=np.uint32)
    x = ((pat[:, None] >> np.arange(27, dtype=np.uint32)[None, :]) & 1).astype(np.float32)
    out = np.zeros((pat.shape[0], KIN), dtype=np.float32)
    out[:, :27] = x
    out[:, BIAS_COL] = 1.0
    return out


# ------------------------------------------------------------------ network
def init_params(seed: int = 0):
    rng = np.random.default_rng(seed)
    w1 = (rng.standard_normal((HIDDEN, KIN)) * np.sqrt(2.0 / 28)).astype(np.float32)
    w1[:, 28:] = 0.0
    w1[:, BIAS_COL] = 0.0
    w2 = (rng.standard_normal((HIDDEN, HIDDEN)) * np.sqrt(2.0 / HIDDEN)).astype(np.float32)
    b2 = np.zeros(HIDDEN, dtype=np.float32)
    w3 = (rng.standard_normal(HIDDEN) * np.sqrt(1.0 / HIDDEN)).astype(np.float32)
    b3 = np.zeros(1, dtype=np.float32)
    return {"w1": w1, "w2": w2, "b2": b2, "w3": w3, "b3": b3}


def pack(p) -> np.ndarray:
    """Flat float32 parameter vector in the device order w1, w2, b2, w3, b3."""
    return np.concatenate([p["w1"].ravel(), p["w2"].ravel(), p["b2"], p["w3"], p["b3"]]).astype(np.float32)


def unpack(v):
    v = np.asarray(v, dtype=np.float32)
    o = 0
    out = {}
    for name, shape in (("w1", (HIDDEN, KIN)), ("w2", (HIDDEN, HIDDEN)), ("b2", (HIDDEN,)),
                        ("w3", (HIDDEN,)), ("b3", (1,))):
        n = int(np.prod(shape))
        out[name] = v[o:o + n].reshape(shape).copy()
        o += n
    return out


N_PARAMS = HIDDEN * KIN + HIDDEN * HIDDEN + HIDDEN + HIDDEN + 1  # 6273


def forward(p, pat, quant: bool = True):
    """Logits z with the device's rounding points (float32).  quant=False
    drops every rounding and works in float64, for finite-difference checks
    of the backward formulas."""
    r = bf16 if quant else (lambda a: np.asarray(a, dtype=np.float64))
    ft = np.float32 if quant else np.float64
    x = features(pat).astype(np.float64)
    w1 = r(p["w1"]).astype(np.float64)
    w2 = r(p["w2"]).astype(np.float64)
    h1p = (x @ w1.T).astype(ft)
    h1 = r(np.maximum(h1p, 0.0)).astype(np.float64)
    h2p = (h1 @ w2.T).astype(ft) + np.asarray(p["b2"], dtype=ft)
    h2 = np.maximum(h2p, 0.0).astype(np.float64)
    z = (h2 @ np.asarray(p["w3"], dtype=np.float64)).astype(ft) + ft(p["b3"][0])
    return z.astype(ft), (x, h1, h2)


def loss_and_grad(p, pat, y, wt, quant: bool = True):
    """Weighted mean BCE-with-logits over the batch and its gradient.  The
    mean divides by the number of samples (not the weight sum)."""
    r = bf16 if quant else (lambda a: np.asarray(a, dtype=np.float64))
    ft = np.float32 if quant else np.float64
    y = np.asarray(y, dtype=np.float64)
    wt = np.asarray(wt, dtype=np.float64)
    n = y.shape[0]
    z, (x, h1, h2) = forward(p, pat, quant)
    zz = z.astype(np.float64)
    loss = np.sum(wt * (np.maximum(zz, 0) - zz * y + np.log1p(np.exp(-np.abs(zz))))) / n
    sig = 1.0 / (1.0 + np.exp(-zz))
    dz = (wt * (sig - y) / n).astype(ft).astype(np.float64)
    w3 = np.asarray(p["w3"], dtype=np.float64)
    g = {}
    g["w3"] = (h2.T @ dz).astype(ft)
    g["b3"] = np.array([dz.sum()], dtype=ft)
    dh2 = r(np.where(h2 > 0, (dz[:, None] * w3[None, :]).astype(ft), 0.0)).astype(np.float64)
    g["w2"] = (dh2.T @ h1).astype(ft)
    g["b2"] = dh2.sum(axis=0).astype(ft)
    w2 = r(p["w2"]).astype(np.float64)
    dh1p = (dh2 @ w2).astype(ft)
    dh1 = r(np.where(h1 > 0, dh1p, 0.0)).astype(np.float64)
    g["w1"] = (dh1.T @ x).astype(ft)
    g["w1"][:, 28:] = 0.0
    return float(loss), g


def prior_params(seed: int = 0, beta: float = 1.5, z0: float = -5.0):
    """Initial network whose output is z0 - beta * (occupied neighbours) plus a
    small random part: hidden unit 0 of both layers carries 27 - count."""
    p = init_params(seed)
    p["w1"][0, :27] = -1.0
    p["w1"][0, BIAS_COL] = 27.0
    p["w2"][0, :] = 0.0
    p["w2"][0, 0] = 1.0
    p["b2"][0] = 0.0
    p["w3"] *= 0.01
    p["w3"][0] = beta
    p["b3"][0] = z0 - 27.0 * beta
    return p


def adam(pv, gv, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba 2015) on flat float32 vectors, in float32."""
    gv = gv.astype(np.float32)
    m[:] = np.float32(b1) * m + np.float32(1 - b1) * gv
    v[:] = np.float32(b2) * v + np.float32(1 - b2) * gv * gv
    c1 = np.float32(1.0 - b1 ** step)
    c2 = np.float32(1.0 - b2 ** step)
    pv[:] = pv - np.float32(lr) * (m / c1) / (np.sqrt(v / c2) + np.float32(eps))
    return pv


# ------------------------------------------------------------------ proposal
def proposal_weights(z):
    """Sub-cell proposal weights pi = sqrt(sigmoid(z)), in float32 as on the
    device: for a proposal that is uniform inside each sub-cell, the variance
    of the importance-sampling estimate of P(success) is smallest with q_c
    proportional to the square root of the success probability in sub-cell
    c."""
    z = np.asarray(z, dtype=np.float32)
    one = np.float32(1.0)
    return np.sqrt(one / (one + np.exp(-z))).astype(np.float64)


def replay_points(seed, seq, n, alpha, cdf, ns, box):
    """The device's insertion points for call `seq`: per insertion i one
    Philox block (i, 0, seq, TAG); r.x chooses the branch (uniform when
    r.x < alpha 2^32) and, in the learned branch, the sub-cell by inverse CDF;
    r.y..r.w place the point.  Returns points (n, 3), sub-cell indices and a
    flag for the uniform branch."""
    ns = np.asarray(ns, dtype=np.int64)
    box = np.asarray(box, dtype=np.float64)
    i = np.arange(n, dtype=np.uint64)
    r = draw4(seed, (i & 0xFFFFFFFF).astype(np.uint32), (i >> 32).astype(np.uint32), seq, TAG_LWIDOM)
    thr = np.uint64(int(alpha * 4294967296.0))
    rx = r[0].astype(np.uint64)
    uni = rx < thr
    total = cdf[-1]
    span = 4294967296.0 - float(thr)
    inv_span = 1.0 / span if span > 0 else 0.0  # alpha = 1: no learned draws
    t = ((rx.astype(np.float64) - float(thr)) + 0.5) * inv_span * total
    cell = np.searchsorted(cdf, t, side="right")
    cell = np.minimum(cell, cdf.shape[0] - 1)
    e = box / ns
    u = [((2 * r[k].astype(np.uint64) + 1).astype(np.float64)) * 2.0 ** -33 for k in (1, 2, 3)]
    pts = np.empty((n, 3), dtype=np.float64)
    cx = cell % ns[0]
    cy = (cell // ns[0]) % ns[1]
    cz = cell // (ns[0] * ns[1])
    sub = (cx, cy, cz)
    for d in range(3):
        learned = (sub[d].astype(np.float64) + u[d]) * e[d]
        pts[:, d] = np.where(uni, u[d] * box[d], learned)
    return pts, cell, uni
