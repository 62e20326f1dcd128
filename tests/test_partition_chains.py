"""The shortcuts the device partition takes through the reference's swap chains,
restated in Python and checked against the swap sequence itself on CPU.

The reference partitions a node (RCBForceTree.cxx:647-669) by collecting the
positions idx of the elements below the split in order and swapping the j-th
of them into slot j.  A right element at p < nleft then moves along
p -> idx[p] -> idx[idx[p]] -> ... until it lands at or after nleft.  The CUDA
kernels follow those chains with two shortcuts:

* run jumps (k_part_right, chain_jump): the q-th left element has
  c = idx[q] - q right elements before it, and so has every left element up
  to the c-th right element (position ridx[c]); their ranks run to
  ridx[c] - c, and within that run each step adds c;
* pointer jumping (k_part_node): idx[q] <- idx[idx[q]] in place until every
  entry is the end of its chain, skipping the left elements no swap moves
  (idx[q] == q).

The GPU parity tests compare the kernels with the host build on real trees;
these tests cover the two formulas on adversarial inputs (sorted runs, a few
right elements in front of long left runs) far faster.
"""
import numpy as np
import pytest


def swap_sequence(left):
    """Final source position of every slot after the reference's swaps."""
    a = list(range(len(left)))
    idx = [i for i, l in enumerate(left) if l]
    for j, i in enumerate(idx):
        a[i], a[j] = a[j], a[i]
    return a


def by_run_jumps(left, plain_steps=4):
    n = len(left)
    idx = [i for i in range(n) if left[i]]
    ridx = [i for i in range(n) if not left[i]]
    nleft, nright = len(idx), len(ridx)
    out = [None] * n
    for r, i in enumerate(idx):
        out[r] = i
    for e in range(n):
        if left[e]:
            continue
        if e >= nleft:
            out[e] = e
            continue
        q, steps = e, 0
        while q < nleft:
            c = idx[q] - q
            assert c > 0
            if steps < plain_steps:
                q = idx[q]
            else:
                lim = nleft
                if c < nright:
                    b = ridx[c] - c
                    assert b > q
                    lim = min(lim, b)
                k = 1 if lim <= q + c else (lim - q + c - 1) // c
                q += k * c
            steps += 1
        out[q] = e
    return out


def by_pointer_jumping(left, rng, chain_steps=32):
    n = len(left)
    sidx = [i for i in range(n) if left[i]]
    nleft = len(sidx)
    out = [None] * n
    for r, i in enumerate(sidx):
        out[r] = i
    for e in range(nleft, n):
        if not left[e]:
            out[e] = e
    pending = []
    for e in range(nleft):
        if left[e]:
            continue
        q, steps = e, 0
        while q < nleft and steps < chain_steps:
            q, steps = sidx[q], steps + 1
        if q < nleft:
            pending.append(e)
        else:
            out[q] = e
    if pending:
        for _ in range(42):
            changed = False
            order = rng.permutation(nleft)  # any interleaving of the block's threads
            for q in order:
                j = sidx[q]
                if j != q and j < nleft:
                    sidx[q] = sidx[j]
                    changed = True
            if not changed:
                break
        else:
            raise AssertionError("pointer jumping did not converge")
        for e in range(nleft):
            if not left[e]:
                assert sidx[e] >= nleft
                out[sidx[e]] = e
    return out


def _cases():
    rng = np.random.default_rng(7)
    for t in range(300):
        n = int(rng.integers(0, 1500))
        kind = t % 5
        if kind == 0:
            keys = rng.random(n)
        elif kind == 1:
            keys = np.sort(rng.random(n))
        elif kind == 2:  # a few right elements in front of a sorted run: long chains
            keys = np.sort(rng.random(n))
            keys[:min(n, int(rng.integers(1, 5)))] = 2.0
        elif kind == 3:
            keys = rng.random(n) ** 4
        else:  # descending with a few strays
            keys = np.sort(rng.random(n))[::-1].copy()
            if n > 4:
                keys[rng.integers(0, n, 4)] = rng.random(4)
        split = float(np.quantile(keys, rng.random())) if n else 0.5
        yield t, list(keys < split)


@pytest.mark.parametrize("method", ["runs", "pointers"])
def test_chain_shortcuts_equal_swap_sequence(method):
    rng = np.random.default_rng(11)
    for t, left in _cases():
        want = swap_sequence(left)
        got = by_run_jumps(left) if method == "runs" else by_pointer_jumping(left, rng)
        assert got == want, (method, t, len(left))


def test_one_chain_through_every_left_element():
    """The largest key in front of a sorted node: one chain of nleft steps,
    which the run jump takes in one step after the plain ones."""
    n = 5000
    left = [False] + [True] * (n // 2) + [False] * (n - 1 - n // 2)
    assert by_run_jumps(left) == swap_sequence(left)
    assert by_pointer_jumping(left, np.random.default_rng(0)) == swap_sequence(left)
