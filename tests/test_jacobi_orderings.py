"""Index invariants of the Jacobi eigensolver's kernels (corr_gb300/csrc/jacobi.cu),
restated in Python and checked on the CPU:

* the round-robin pairing (round_pair) meets every unordered index pair exactly
  once per sweep of n-1 rounds, and each round is a perfect matching;
* next_pair steps from pair k to pair k+1 of the same round;
* the A update (kRowsA row pairs per thread, pairs k <= l, upper triangle
  addressed by (min, max)) writes every stored element exactly once per round,
  each from one thread;
* the V update (kRowsV rows per thread) covers every V element exactly once;
* the FP32 block stage pairs the m = np / 32 blocks with the same ordering,
  every 64 x 64 tile of A and of V belongs to exactly one block_apply CTA.
"""
import itertools

import pytest


def round_pair(n, r, k):
    if k == 0:
        return n - 1, r
    return (r + k) % (n - 1), (r - k + (n - 1)) % (n - 1)


def next_pair(n, r, k, p, q):
    if k == 0:
        return round_pair(n, r, 1)
    p = 0 if p + 1 == n - 1 else p + 1
    q = n - 2 if q == 0 else q - 1
    return p, q


def sym(x, y):
    return (x, y) if x < y else (y, x)


@pytest.mark.parametrize("n", [2, 4, 6, 10, 34, 64, 130])
def test_round_robin_sweep_covers_each_pair_once(n):
    seen = {}
    for r in range(n - 1):
        used = set()
        for k in range(n // 2):
            p, q = round_pair(n, r, k)
            assert p != q and p not in used and q not in used
            used.update((p, q))
            seen[sym(p, q)] = seen.get(sym(p, q), 0) + 1
        assert len(used) == n
        if n > 2:
            for k in range(n // 2 - 1):
                assert next_pair(n, r, k, *round_pair(n, r, k)) == round_pair(n, r, k + 1)
    assert len(seen) == n * (n - 1) // 2 and set(seen.values()) == {1}


@pytest.mark.parametrize("n", [4, 6, 10, 34, 130])
@pytest.mark.parametrize("rows_a,rows_v", [(4, 4)])
def test_apply_partition(n, rows_a, rows_v):
    h = n // 2
    n_a = (h + rows_a - 1) // rows_a * h
    n_v = (n + rows_v - 1) // rows_v * h
    for r in (0, 1, n - 2):
        owner = {}
        vcount = {}
        for tid in range(n_a + n_v):
            if tid < n_a:
                kb, l = divmod(tid, h)
                u, w = round_pair(n, r, l)
                for i in range(rows_a):
                    k = kb * rows_a + i
                    if k >= h or k > l:
                        continue
                    p, q = round_pair(n, r, k)
                    for e in {sym(p, u), sym(p, w), sym(q, u), sym(q, w)}:
                        assert owner.setdefault(e, tid) == tid
            else:
                xb, l = divmod(tid - n_a, h)
                u, w = round_pair(n, r, l)
                for i in range(rows_v):
                    x = xb * rows_v + i
                    if x < n:
                        for c in (u, w):
                            vcount[(x, c)] = vcount.get((x, c), 0) + 1
        assert len(owner) == n * (n + 1) // 2
        assert len(vcount) == n * n and set(vcount.values()) == {1}


@pytest.mark.parametrize("np_", [64, 128, 192, 1536])
def test_block_stage_tiles(np_):
    blk = 32
    m = np_ // blk
    h = m // 2
    for r in range(min(m - 1, 5)):
        rows = lambda t: set(range(round_pair(m, r, t)[0] * blk, round_pair(m, r, t)[0] * blk + blk)) | \
            set(range(round_pair(m, r, t)[1] * blk, round_pair(m, r, t)[1] * blk + blk))
        groups = [rows(t) for t in range(h)]
        # the block pairs of a round partition the indices
        assert sorted(itertools.chain.from_iterable(groups)) == list(range(np_))
        # A tiles (s, t) and V tiles (rb, t) cover every element once
        covered = sum(len(groups[s_]) * len(groups[t]) for s_ in range(h) for t in range(h))
        assert covered == np_ * np_
        assert (np_ // 64) * h * 64 * 64 == np_ * np_
    # inner pair table of a 64-index block pair: a full sweep of 63 rounds
    seen = set()
    for rr in range(63):
        for k in range(32):
            seen.add(sym(*round_pair(64, rr, k)))
    assert len(seen) == 64 * 63 // 2
