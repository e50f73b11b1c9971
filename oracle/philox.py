"""Oracle test infrastructure (not product code).

Philox4x32-10 in numpy (Salmon, Moraes, Dror & Shaw, SC'11), vectorised over
counters, used to check the random stream the GPU kernels draw.  The counter
layout mirrors the device helper ``draw4``: (a, b, seq_lo, tag<<28 | seq_hi)
with the 64-bit seed as the key.
"""
from __future__ import annotations

import numpy as np

M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = np.uint32(0x9E3779B9)
W1 = np.uint32(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)

TAG_MOVE, TAG_SHIFT, TAG_PERM, TAG_WIDOM, TAG_VOLUME = 1, 2, 3, 4, 5


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    c0 = np.asarray(c0, dtype=np.uint32).astype(np.uint64)
    c1 = np.asarray(c1, dtype=np.uint32).astype(np.uint64)
    c2 = np.asarray(c2, dtype=np.uint32).astype(np.uint64)
    c3 = np.asarray(c3, dtype=np.uint32).astype(np.uint64)
    k0 = np.uint64(np.uint32(k0))
    k1 = np.uint64(np.uint32(k1))
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        h0, l0 = p0 >> np.uint64(32), p0 & MASK
        h1, l1 = p1 >> np.uint64(32), p1 & MASK
        c0, c1, c2, c3 = (h1 ^ c1 ^ k0) & MASK, l1, (h0 ^ c3 ^ k1) & MASK, l0
        k0 = (k0 + np.uint64(W0)) & MASK
        k1 = (k1 + np.uint64(W1)) & MASK
    return tuple(x.astype(np.uint32) for x in (c0, c1, c2, c3))


def draw4(seed: int, a, b, seq, tag: int):
    seq = np.asarray(seq, dtype=np.uint64)
    c2 = (seq & MASK).astype(np.uint32)
    c3 = ((np.uint64(tag) << np.uint64(28)) | ((seq >> np.uint64(32)) & np.uint64(0x0FFFFFFF))).astype(np.uint32)
    return philox4x32_10(a, b, c2, c3, seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)
