"""CPU check of the threshold search of the TOTAL selection (k_total_select,
mlp_total.cu, step 1): on the remaining keys of a list, a 2048-bin histogram of
their offsets from the smallest takes the lowest bins that fit a budget of
256 keys, refining into the first bin that did not fit while less than half a
batch is taken.  The keys <= T form the next batch.  Restated here on Python
integers, the batches must each hold between 1 and 256 keys, be the smallest
remaining keys, and cover the list in key order; every round removes at least
the smallest key, so the rounds end."""
import random

import pytest

BINS, BATCH = 2048, 256


def bitlen(v):
    return v.bit_length()


def bin_shift(bl):
    return bl - 11 if bl > 11 else 0


def threshold(keys, lo, hi):
    """T for the remaining keys (all in [lo, hi])."""
    if len(keys) <= BATCH:
        return hi
    rng_ = hi - lo
    sft = bin_shift(bitlen(rng_))
    T, budget, have_t = hi, BATCH, False
    for _ in range(16):
        hist = [0] * BINS
        for k in keys:
            if lo <= k and k - lo <= rng_:
                hist[(k - lo) >> sft] += 1
        cum, gg, cnt = 0, -1, 0
        for g in range(BINS):
            cum += hist[g]
            if cum <= budget:
                gg, cnt = g, cum
            else:
                break
        if gg >= 0:
            T = lo + ((gg + 1) << sft) - 1
            have_t = True
            budget -= cnt
        if gg == BINS - 1 or sft == 0 or budget < BATCH // 2:
            break
        lo = lo + ((gg + 1) << sft)
        rng_ = (1 << sft) - 1
        sft = bin_shift(bitlen(rng_))
    return T if have_t else hi


def batches(keys):
    rest = sorted(keys)
    lo, hi = rest[0], rest[-1]
    out = []
    while rest:
        T = threshold(rest, lo, hi)
        b = [k for k in rest if k <= T]
        out.append(b)
        rest = [k for k in rest if k > T]
        lo = T + 1
    return out


def draw(rnd, m, kind):
    if kind == "uniform":
        return rnd.sample(range(1 << 40), m)
    if kind == "clustered":  # many keys within a few small ranges
        base = [rnd.randrange(1 << 44) for _ in range(3)]
        return list({rnd.choice(base) + rnd.randrange(1 << rnd.choice([4, 12, 20])) for _ in range(m)})
    if kind == "skewed":  # a dense low end (the improving deltas) and a long tail
        s = {rnd.randrange(5000) for _ in range(max(1, m // 2))} | {rnd.randrange(1 << 50) for _ in range(m // 2)}
        return list(s)
    return list(range(m))  # consecutive keys: single-key bins


@pytest.mark.parametrize("seed", range(12))
@pytest.mark.parametrize("kind", ["uniform", "clustered", "skewed", "consecutive"])
def test_threshold_batches(seed, kind):
    rnd = random.Random(seed * 7 + len(kind))
    m = rnd.choice([1, 200, 256, 257, 1000, 5000])
    keys = draw(rnd, m, kind)
    out = batches(keys)
    flat = [k for b in out for k in b]
    assert flat == sorted(keys)
    for b in out:
        assert 1 <= len(b) <= BATCH
