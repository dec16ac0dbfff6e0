"""The library's radix sort on chosen key distributions, against numpy's
stable argsort: keys, the original index of every sorted slot (equal keys
keep their input order), and a clear device status word.

Up to 2^17 keys the sort takes one tile pass on the top 7-bit digit, then
sorts each top-digit bucket in shared memory: a bucket of up to 128 pairs is
sorted by one warp's network; a larger one is split wide on its next bits
and its sub-buckets are ranked by threads (up to 16 pairs) or warp networks
(up to 128), a bucket of m pairs shared by min(4, ceil(m / 1024)) CTAs, or,
with a sub-bucket above 128 pairs, finished by LSD passes of one CTA; a
bucket over 8192 pairs sends the whole array through the cooperative tile
passes.  The cases below put buckets and sub-buckets on each side of those
limits."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sf():
    import __graft_entry__
    __graft_entry__.build()
    import starflood_gb300
    return starflood_gb300


def check_sort(sf, keys, bits):
    keys = np.ascontiguousarray(keys, np.uint64)
    out, idx, st = sf.sort_keys(keys, bits)
    want = np.argsort(keys, kind="stable")
    assert st == 0
    np.testing.assert_array_equal(idx, want.astype(np.uint32))
    np.testing.assert_array_equal(out, keys[want])


def compose(top, sub, low, bits):
    """Keys from a top digit, the next digit and the bits below."""
    shift = ((bits + 6) // 7 - 1) * 7
    return (np.uint64(top) << np.uint64(shift)) | (np.uint64(sub) << np.uint64(shift - 7)) | np.uint64(low)


@pytest.mark.parametrize("n", [2, 3, 100, 1000, 65536, 131072, 131073, 300000])
@pytest.mark.parametrize("bits", [49, 14, 37])
def test_sort_random(sf, n, bits):
    rng = np.random.default_rng(n + bits)
    keys = rng.integers(0, 1 << bits, n, dtype=np.uint64)
    check_sort(sf, keys, bits)


@pytest.mark.parametrize("bits", [8, 64])
def test_sort_key_widths(sf, bits):
    rng = np.random.default_rng(bits)
    hi = np.iinfo(np.uint64).max if bits == 64 else (1 << bits) - 1
    keys = rng.integers(0, hi, 20000, dtype=np.uint64, endpoint=True)
    check_sort(sf, keys, bits)


def test_sort_few_distinct(sf):
    """Many equal keys: every bucket and sub-bucket ties throughout."""
    rng = np.random.default_rng(3)
    keys = rng.choice(np.array([5, 1 << 40, (1 << 40) + 1, 7 << 42], np.uint64), 60000)
    check_sort(sf, keys, 49)
    check_sort(sf, np.full(5000, 12345, np.uint64), 49)  # one bucket, one sub-bucket of 5000


@pytest.mark.parametrize("sizes", [(127, 128, 129, 1, 0, 300), (128,), (129,), (8191,), (4000, 4000)])
def test_sort_sub_bucket_limits(sf, sizes):
    """One top-digit bucket built from sub-buckets of the given sizes (and
    the same sizes as whole buckets), interleaved and in random order."""
    rng = np.random.default_rng(sum(sizes))
    parts = []
    for d, m in enumerate(sizes):
        low = rng.integers(0, 1 << 35, m, dtype=np.uint64)
        parts.append(compose(9, 3 + 5 * d, low, 49))          # sub-buckets of bucket 9
        parts.append(compose(20 + d, d, low & np.uint64(7), 49))  # whole buckets, many ties
    keys = np.concatenate(parts)
    keys = keys[rng.permutation(len(keys))]
    check_sort(sf, keys, 49)


@pytest.mark.parametrize("size", [1025, 2048, 3000, 6606, 8000])
def test_sort_shared_buckets(sf, size):
    """Top-digit buckets of over 1024 pairs with small sub-buckets, sorted by
    up to four CTAs that each take a range of the sub-buckets; a quarter of
    the keys repeat others (equal keys keep their order across the CTAs'
    ranges)."""
    rng = np.random.default_rng(size)
    low = rng.integers(0, 1 << 42, size, dtype=np.uint64)
    low[: size // 4] = low[size // 2: size // 2 + size // 4]
    a = compose(33, 0, 0, 49) + low
    b = compose(90, 0, 0, 49) + rng.integers(0, 1 << 42, size // 2 + 1, dtype=np.uint64)
    c = rng.integers(0, 1 << 49, 3000, dtype=np.uint64)
    keys = np.concatenate([a, b, c])
    keys = keys[rng.permutation(len(keys))]
    check_sort(sf, keys, 49)


def test_sort_bucket_overflow(sf):
    """A top-digit bucket of 20,000 pairs (over the 8192 a CTA holds): the
    cooperative tile passes sort everything."""
    rng = np.random.default_rng(11)
    a = compose(64, 0, 0, 49) + rng.integers(0, 1 << 42, 20000, dtype=np.uint64)
    b = rng.integers(0, 1 << 49, 30000, dtype=np.uint64)
    keys = np.concatenate([a, b])[rng.permutation(50000)]
    check_sort(sf, keys, 49)


def test_sort_tree_like_keys(sf):
    """Morton keys of a Plummer sphere (a dense core: large buckets and
    sub-buckets), as the tree build makes them."""
    from starflood_gb300.ics import plummer
    pos, _, _ = plummer(65536, seed=4)
    lo, hi = pos.min(0), pos.max(0)
    q = np.clip(((pos - lo) / (hi - lo).max() * (1 << 16)).astype(np.int64), 0, (1 << 16) - 1).astype(np.uint64)

    def spread(v):
        out = np.zeros_like(v)
        for b in range(16):
            out |= ((v >> np.uint64(b)) & np.uint64(1)) << np.uint64(3 * b)
        return out

    keys = (spread(q[:, 0]) << np.uint64(2)) | (spread(q[:, 1]) << np.uint64(1)) | spread(q[:, 2])
    check_sort(sf, keys, 48)
