"""Properties of Karras radix trees that the build kernels rely on, checked
on the CPU over random sorted codes (with many equal codes, so the index
tie-break of the common-prefix length is exercised):

* every inner node's index is one end of its Morton range;
* the largest node whose range starts at leaf l > 0 is inner node l, and the
  largest whose range ends at leaf r < n - 1 is inner node r -- so the refit
  writes a segment-crossing node's suffix and prefix unions only at the
  leaves whose own inner node crosses (plus the last leaf's prefix);
* "common prefix of i and j longer than c" equals the XOR-threshold test the
  split searches use (x < 2^(W-1-c); x == 0 and i ^ j < 2^(W+31-c); true for
  c = -1).

The tree is built the way build_tree_karras does it (bbvh-cuda/lbvh-kernels.cu
:205-249): direction from the neighbours' prefix lengths, exponential and
binary search for the range end.
"""
import numpy as np
import pytest


def _clz(x: int, width: int) -> int:
    return width - x.bit_length() if x else width


def _cpl(codes, i, j, width):
    # __cpl (lbvh-kernels.cu:84-92): -1 out of range; equal codes fall back to
    # the indices
    if j < 0 or j >= len(codes):
        return -1
    x = int(codes[i]) ^ int(codes[j])
    return _clz(x, width) + _clz(i ^ j, 32) if x == 0 else _clz(x, width)


def _ranges(codes, width):
    n = len(codes)
    out = []
    for i in range(n - 1):
        d = 1 if _cpl(codes, i, i + 1, width) - _cpl(codes, i, i - 1, width) >= 0 else -1
        cmin = _cpl(codes, i, i - d, width)
        lmax = 2
        while _cpl(codes, i, i + lmax * d, width) > cmin:
            lmax *= 2
        length, t = 0, lmax // 2
        while t >= 1:
            if _cpl(codes, i, i + (length + t) * d, width) > cmin:
                length += t
            t //= 2
        j = i + length * d
        out.append((min(i, j), max(i, j)))
    return out


def _codes(rng, n, width):
    span = int(rng.choice([4, 64, 1 << (width - 2)]))
    return np.sort(rng.integers(0, span, n, dtype=np.uint64))


@pytest.mark.parametrize("width", [32, 64])
def test_node_index_is_a_range_end_and_largest_node_per_end(width):
    rng = np.random.default_rng(width)
    for _ in range(12):
        n = int(rng.integers(2, 700))
        codes = _codes(rng, n, width)
        ranges = _ranges(codes, width)
        starts, ends = {}, {}
        for i, (l, r) in enumerate(ranges):
            assert i in (l, r)
            starts.setdefault(l, []).append(r - l)
            ends.setdefault(r, []).append(r - l)
        for l, sizes in starts.items():
            if l > 0:
                # inner node l starts at l and is the largest range starting there
                assert ranges[l][0] == l and ranges[l][1] - l == max(sizes)
        for r, sizes in ends.items():
            if r < n - 1:
                assert ranges[r][1] == r and r - ranges[r][0] == max(sizes)


@pytest.mark.parametrize("seg", [4, 16, 256])
def test_crossing_node_ends_are_written_by_their_own_nodes(seg):
    rng = np.random.default_rng(seg)
    for _ in range(10):
        n = int(rng.integers(2, 900))
        codes = _codes(rng, n, 64)
        ranges = _ranges(codes, 64)
        suf, pre = set(), {n - 1}
        for i, (l, r) in enumerate(ranges):
            if l // seg != r // seg:
                (suf if i == l else pre).add(i)
        for l, r in ranges:
            if l // seg != r // seg:
                assert l in suf and r in pre


@pytest.mark.parametrize("width", [32, 64])
def test_prefix_threshold_equals_common_prefix_compare(width):
    rng = np.random.default_rng(7 + width)

    def threshold(c):
        if c < 0:
            return (1 << width) - 1, 0
        if c < width:
            return 1 << (width - 1 - c), 0
        return 0, 1 << (width + 31 - c)

    for _ in range(40):
        n = int(rng.integers(2, 300))
        codes = _codes(rng, n, width)
        for _ in range(200):
            b = int(rng.integers(0, n))
            j = int(rng.integers(-2, n + 2))
            c = int(rng.integers(-1, width + 32))
            th, tl = threshold(c)
            if 0 <= j < n:
                x = int(codes[b]) ^ int(codes[j])
                fast = x < th or (x == th and (b ^ j) < tl)
            else:
                fast = False
            assert fast == (_cpl(codes, b, j, width) > c)
