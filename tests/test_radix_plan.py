"""The digit plan of the device radix select (prox.cu, k_radix_select),
restated on the host and checked on many inputs: 11-bit digits of the
magnitude key from the top (FP64: 11,11,11,11,11,8 bits; FP32: 11,11,9), the
bucket holding the k-th largest key picked per digit, and once that bucket
holds at most `cap` keys (with digits left after the next one) the next scan
also lists its keys and the remaining digits run over the list.  The result
must be the k-th largest key t, G = #{key > t} and E = #{key == t}, whatever
the list size; the device code runs the same plan with cap = 32768."""
import numpy as np
import pytest

PLAN = {8: ([52, 41, 30, 19, 8, 0], [11, 11, 11, 11, 11, 8]), 4: ([20, 9, 0], [11, 11, 9])}


def sel_keys(v, pos):
    """Magnitude keys of pos_adj(v): integer tests only, as on the device."""
    bits = v.view(np.uint64 if v.dtype == np.float64 else np.uint32).astype(np.uint64)
    top = 63 if v.dtype == np.float64 else 31
    mag = bits & np.uint64((1 << top) - 1)
    inf = np.uint64(0x7FF0000000000000 if v.dtype == np.float64 else 0x7F800000)
    neg = ((bits >> np.uint64(top)) == 1) & (mag != 0) & (mag <= inf)
    return np.where(pos & neg, np.uint64(0), mag)


def radix_plan(keys, k, size, cap):
    shifts, bits = PLAN[size]
    npass = len(shifts)
    prefix = mask = np.uint64(0)
    krem, G, E = k, 0, 0
    src, listed = keys, None
    for p in range(npass):
        sh, nb = np.uint64(shifts[p]), 1 << bits[p]
        collect = listed is None and p > 0 and p + 1 < npass and E <= cap
        match = src[(src & mask) == prefix]
        if collect:
            listed = match.copy()  # the keys of the current bucket, in any order
        hist = np.bincount(((match >> sh) & np.uint64(nb - 1)).astype(np.int64), minlength=nb)
        cum = 0
        for b in range(nb - 1, -1, -1):  # descending bins
            if cum + hist[b] >= krem:
                G += cum
                krem -= cum
                prefix = prefix | (np.uint64(b) << sh)
                mask = mask | (np.uint64(nb - 1) << sh)
                E = int(hist[b])
                break
            cum += hist[b]
        else:
            raise AssertionError("k beyond the keys")
        if collect:
            src = listed  # later digits scan the list only
    return prefix, G, E, krem


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("cap", [0, 16, 300, 32768])
def test_radix_plan_finds_kth_key(dtype, cap):
    rng = np.random.default_rng(cap + (dtype == np.float32))
    for trial in range(40):
        n = int(rng.integers(1, 4000))
        kind = trial % 4
        if kind == 0:
            v = rng.standard_normal(n)
        elif kind == 1:  # spread over binades
            v = np.ldexp(1 + rng.random(n), -rng.integers(0, 40, n)) * rng.choice([-1, 1], n)
        elif kind == 2:  # heavy ties and zeros
            v = rng.integers(-3, 4, n) / 8.0
        else:  # a few values, with signed zeros and infinities
            v = rng.choice([0.0, -0.0, 1.5, -1.5, np.inf, -np.inf, 2.0 ** -30], n)
        v = v.astype(dtype)
        pos = bool(trial % 3 == 0)
        keys = sel_keys(v, pos)
        k = int(rng.integers(1, n + 1))
        t, G, E, krem = radix_plan(keys, k, v.dtype.itemsize, cap)
        ref = np.sort(keys)[::-1]
        assert t == ref[k - 1], trial
        assert G == int(np.sum(keys > t)) and E == int(np.sum(keys == t)), trial
        assert G + krem == k and 1 <= krem <= E, trial


def test_sel_keys_match_pos_clamp():
    v = np.array([1.5, -1.5, 0.0, -0.0, np.inf, -np.inf, np.nan, -np.nan], np.float64)
    keys = sel_keys(v, True)
    clamped = np.where(v < 0, 0.0, v)  # pre_prox_pos: negatives to 0 (NaN stays)
    assert np.array_equal(keys, np.abs(clamped).view(np.uint64) & np.uint64((1 << 63) - 1))
