"""The host-side hop orders of the fixed-point H x v (no GPU).

* The bank schedule of the paired-column single-vector kernel on real spin
  spaces (the 4x4 cluster's half-filled space, a 2x7 space with two hopping
  magnitudes): every row's hops appear exactly once, in its own lane, in the
  rounds of their (class, sign) group; idle lanes read zero units in a bank
  group no real lane of their quarter warp uses that round; the per-warp
  round counts are the largest group counts of the warp's rows; and almost
  every quarter-warp round is free of bank conflicts.
* The parity order of the chains' kernel: each row keeps its hops in each
  sign group, and rows 2i, 2i+1 meet sources of equal parity far less often.
"""
import numpy as np
import pytest

from vca_gb300.solver import hop_parity_order, hop_schedule


def _hops(nx, ny, n, ty=None):
    """Sign-sorted hop words (src | class << 24 | sign << 31) of the spin space
    with n electrons on an open nx x ny lattice; ty: a second magnitude on
    the vertical bonds (class 1)."""
    ns = nx * ny
    bonds = []
    for y in range(ny):
        for x in range(nx):
            i = y * nx + x
            if x + 1 < nx:
                bonds.append((i, i + 1, 0))
            if y + 1 < ny:
                bonds.append((i, i + nx, 0 if ty is None else 1))
    words = [w for w in range(1 << ns) if bin(w).count("1") == n]
    index = {w: r for r, w in enumerate(words)}
    rows = []
    for w in words:
        pos, neg = [], []
        for a, c, cls in bonds:
            if ((w >> a) & 1) != ((w >> c) & 1):
                lo, hi = min(a, c), max(a, c)
                between = bin(w & ((1 << hi) - 1) & ~((1 << (lo + 1)) - 1)).count("1")
                word = index[w ^ (1 << a) ^ (1 << c)] | (cls << 24)
                # amplitude -t times the fermionic sign
                (pos if between % 2 else neg).append(word if between % 2 else word | (1 << 31))
        rows.append(pos + neg)
    dim, width = len(words), 2 * len(bonds)
    hop = np.zeros((width, dim), dtype=np.uint32)
    cnt = np.array([len(r) for r in rows], dtype=np.int32)
    npos = np.array([sum(1 for x in r if not x >> 31) for r in rows], dtype=np.int32)
    for r, lst in enumerate(rows):
        hop[:len(lst), r] = lst
    return dim, cnt, npos, hop


@pytest.mark.parametrize("case,K", [((4, 4, 8, None), 1), ((7, 2, 7, 0.7), 2)])
def test_bank_schedule_places_every_hop_once_without_conflicts(case, K):
    dim, cnt, npos, hop = _hops(*case)
    sched, wround, wgrp, conflicts = hop_schedule(cnt, hop, K)
    nw = (dim + 31) // 32
    assert wround[0] == 0 and wround[-1] == sched.shape[0]
    units = sched // 16
    bad_idle = 0
    for w in range(nw):
        rows = list(range(w * 32, min(dim, w * 32 + 32)))
        got = [[] for _ in range(32)]
        r = wround[w]
        for g in range(2 * K):
            cls, neg = g >> 1, g & 1
            want_max = 0
            for lane, row in enumerate(rows):
                mine = [int(x) for x in hop[:cnt[row], row] if ((x >> 24) & 3) == cls and (x >> 31) == neg]
                want_max = max(want_max, len(mine))
            assert wgrp[w, g] == want_max
            for rd in range(wgrp[w, g]):
                u = units[r + rd]
                for q in range(4):
                    quarter = u[8 * q:8 * q + 8]
                    real = [x for x in quarter if x < dim]
                    used = {x % 8 for x in real}
                    for x in quarter:
                        if x >= dim and x % 8 in used:
                            bad_idle += 1
                for lane in range(32):
                    if u[lane] < dim:
                        got[lane].append(int(u[lane]) | (cls << 24) | (neg << 31))
            r += wgrp[w, g]
        assert r == wround[w + 1]
        for lane, row in enumerate(rows):
            assert sorted(got[lane]) == sorted(int(x) for x in hop[:cnt[row], row]), (w, lane)
        for lane in range(len(rows), 32):
            assert not got[lane]
    assert bad_idle == 0
    assert conflicts <= 0.03 * 4 * sched.shape[0]


def test_parity_order_keeps_each_sign_group_and_pairs_parities():
    dim, cnt, npos, hop = _hops(4, 3, 6)
    before = hop.copy()
    after = hop_parity_order(cnt, npos, hop.copy())

    def same_parity(t):
        n = same = 0
        for r in range(0, dim - 1, 2):
            for a0, a1, b0, b1 in ((0, npos[r], 0, npos[r + 1]), (npos[r], cnt[r], npos[r + 1], cnt[r + 1])):
                for h in range(min(a1 - a0, b1 - b0)):
                    x, y = int(t[a0 + h, r]) & 0xFFFFFF, int(t[b0 + h, r + 1]) & 0xFFFFFF
                    n += 1
                    same += (x & 1) == (y & 1) and x != y
        return same / n

    for r in range(dim):
        for a, b in ((0, npos[r]), (npos[r], cnt[r])):
            assert sorted(after[a:b, r].tolist()) == sorted(before[a:b, r].tolist())
    assert same_parity(before) > 0.25
    assert same_parity(after) < 0.10
