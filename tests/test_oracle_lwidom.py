"""CPU checks of the learned-Widom oracle: bfloat16 rounding, sub-cell
patterns, the backward formulas (finite differences) and the mixture replay."""
import numpy as np
import pytest

from oracle import lwidom as lw


def test_bf16_rounding_is_round_to_nearest_even():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.standard_normal(20000).astype(np.float32) * 10.0 ** rng.integers(-6, 6, 20000),
                        np.array([1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -1.0 - 2.0 ** -8, 0.0, -0.0], np.float32)])
    x = x.astype(np.float32)
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float32).numpy()
    assert np.array_equal(lw.bf16(x).view(np.uint32), ref.view(np.uint32))
    assert lw.bf16(np.float32(1.0 + 2.0 ** -8)) == 1.0          # tie to even
    assert lw.bf16(np.float32(1.0 + 3 * 2.0 ** -8)) == 1.0 + 2.0 ** -6


def test_patterns_against_brute_force():
    rng = np.random.default_rng(1)
    box = np.array([3.2, 2.9, 3.5])
    ns = lw.subgrid(box, 0.5)
    conf = np.zeros((40, 4))
    conf[:, 0] = np.arange(40)
    conf[:, 1:] = rng.uniform(0, 1, (40, 3)) * box
    occ = lw.occupancy(conf, box, ns)
    pat = lw.patterns(occ, ns)
    inv = ns / box
    cells = np.minimum(np.floor(conf[:, 1:] * inv).astype(int), ns - 1)
    full = set(map(tuple, cells))
    for c in range(int(np.prod(ns))):
        cx, cy, cz = c % ns[0], (c // ns[0]) % ns[1], c // (ns[0] * ns[1])
        want = 0
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    nb = ((cx + dx) % ns[0], (cy + dy) % ns[1], (cz + dz) % ns[2])
                    if nb in full:
                        want |= 1 << ((dx + 1) + 3 * (dy + 1) + 9 * (dz + 1))
        assert pat[c] == want


def test_backward_formulas_match_finite_differences():
    rng = np.random.default_rng(2)
    p = lw.init_params(3)
    p["b2"] = rng.standard_normal(lw.HIDDEN).astype(np.float32) * 0.1
    p["b3"] = np.array([0.3], np.float32)
    p = {k: v.astype(np.float64) for k, v in p.items()}
    pat = rng.integers(0, 1 << 27, 64, dtype=np.uint32)
    y = (rng.uniform(size=64) < 0.3).astype(np.float64)
    wt = np.where(y > 0, 2.5, 1.0)
    _, g = lw.loss_and_grad(p, pat, y, wt, quant=False)
    h = 1e-6
    for name, idx in [("w1", (5, 3)), ("w1", (7, 27)), ("w2", (10, 20)), ("b2", (4,)), ("w3", (11,)), ("b3", (0,))]:
        q = {k: v.copy() for k, v in p.items()}
        q[name][idx] += h
        lp, _ = lw.loss_and_grad(q, pat, y, wt, quant=False)
        q[name][idx] -= 2 * h
        lm, _ = lw.loss_and_grad(q, pat, y, wt, quant=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[name][idx]) <= 1e-6 + 1e-5 * abs(fd), (name, idx, fd, g[name][idx])


def test_prior_counts_occupied_neighbours():
    p = lw.prior_params(0, beta=1.5, z0=-5.0)
    pat = np.array([0, 1, 0b111, (1 << 27) - 1], dtype=np.uint32)
    z, _ = lw.forward(p, pat)
    count = np.array([0, 1, 3, 27])
    # the prior unit is exact in bfloat16; the small random part stays small
    assert np.all(np.abs(z - (-5.0 - 1.5 * count)) < 0.5)
    assert np.all(np.diff(z) < 0)


def test_replay_uniform_branch_matches_widom_points():
    from oracle.philox import draw4

    box = np.array([5.0, 6.0, 7.0])
    ns = lw.subgrid(box)
    cdf = np.cumsum(np.ones(int(np.prod(ns))))
    pts, cell, uni = lw.replay_points(7, 3, 500, 1.0, cdf, ns, box)
    assert uni.all()
    r = draw4(7, np.arange(500, dtype=np.uint32), np.zeros(500, np.uint32), 3, lw.TAG_LWIDOM)
    for d, k in enumerate((1, 2, 3)):
        assert np.array_equal(pts[:, d], ((2 * r[k].astype(np.uint64) + 1).astype(np.float64) * 2.0 ** -33) * box[d])
