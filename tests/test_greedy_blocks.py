"""CPU check of the block-by-block greedy that one warp runs over a sorted
batch in the TOTAL selection (warp_greedy_sorted in mlp_total.cu): members
taken 32 at a time, a member conflicting with a kept member of an earlier
block leaves at once, the rest of its block is settled by rounds in which a
member joins once every earlier conflicting member of its block has left (or
leaves once one has joined).  It must keep exactly the members the sequential
greedy in key order keeps (the reference's testSwapTotal / test2OptTotal /
testOrOptTotal zero every later move that conflicts with an earlier kept one,
mlkernel.cu:183-250).  The procedure below restates the kernel's steps on
bit masks, one Python int per 32-member block."""
import random

import pytest


def sequential_greedy(n, conflict):
    kept = []
    for x in range(n):
        if not any(conflict[x][y] for y in kept):
            kept.append(x)
    return set(kept)


def block_greedy(n, conflict):
    # rows: bit y of row x <=> y < x and the two conflict (words of 32 bits)
    W = (n + 31) // 32
    words = [[0] * W for _ in range(n)]
    for x in range(n):
        for y in range(x):
            if conflict[x][y]:
                words[x][y // 32] |= 1 << (y % 32)
    kept_masks = [0] * W
    state = {}
    for b in range(W):
        lanes = [x for x in range(32 * b, min(n, 32 * b + 32))]
        st = {}
        for x in lanes:
            ext = 0
            for w in range(b):
                ext |= words[x][w] & kept_masks[w]
            st[x] = "out" if ext else "undec"
        und = sum(1 << (x % 32) for x in lanes if st[x] == "undec")
        inb = 0
        rounds = 0
        while und:
            rounds += 1
            assert rounds <= 33, "a round must settle the first undecided member"
            new = dict(st)
            for x in lanes:
                if st[x] != "undec":
                    continue
                diag = words[x][b]
                if diag & inb:
                    new[x] = "out"
                elif not (diag & und):
                    new[x] = "in"
            st = new
            inb = sum(1 << (x % 32) for x in lanes if st[x] == "in")
            und = sum(1 << (x % 32) for x in lanes if st[x] == "undec")
        kept_masks[b] = inb
        state.update(st)
    return {x for x, s in state.items() if s == "in"}


@pytest.mark.parametrize("seed", range(40))
def test_block_greedy_equals_sequential(seed):
    rnd = random.Random(seed)
    n = rnd.choice([1, 2, 31, 32, 33, 63, 64, 65, 100, 200, 256])
    p = rnd.choice([0.0, 0.01, 0.05, 0.2, 0.6, 1.0])
    conflict = [[False] * n for _ in range(n)]
    for x in range(n):
        for y in range(x):
            if rnd.random() < p:
                conflict[x][y] = conflict[y][x] = True
    assert block_greedy(n, conflict) == sequential_greedy(n, conflict)


def test_block_greedy_chains_inside_a_block():
    # A chain 0-1-2-...-31 inside one block (the deepest case for the
    # rounds): the greedy keeps the even members.
    n = 32
    conflict = [[False] * n for _ in range(n)]
    for x in range(1, n):
        conflict[x][x - 1] = conflict[x - 1][x] = True
    assert block_greedy(n, conflict) == set(range(0, n, 2)) == sequential_greedy(n, conflict)
