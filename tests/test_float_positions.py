"""The float-position form's pop (csrc/cbq_flat.cuh, lane_walk) reads the integer
bits of a child position p from the float32 bit pattern of p + 1.5 * 2^23 and
rebuilds the popped position by masking that pattern and subtracting the bias.
These tests check the arithmetic it relies on with numpy float32 (IEEE
round-to-nearest, the same as the kernel's -fmad=false adds), for every |p| <=
2^21, the range cbq_dag_create admits for the form:

- p + 1.5 * 2^23 is exact and its pattern is 0x4B400000 + p;
- for positions a, b the low 21 bits of pattern(a) ^ pattern(b) are those of
  a ^ b, and a difference at bit 21 or above in one form is one in the other
  (the pop leaves the SubDAG then, its height being at most 21);
- bit m (m < 21) of the pattern is bit m of p, and masking the pattern below
  bit m then subtracting the bias gives p with its low m bits cleared;
- the child size 2^m built from its exponent field is the float of 1 << m.
"""
import numpy as np

BIAS = np.float32(12582912.0)  # 1.5 * 2^23
LIM = 1 << 21


def pattern(p):
    return (np.asarray(p, dtype=np.int64).astype(np.float32) + BIAS).view(np.uint32)


def test_bias_is_exact_with_a_fixed_exponent():
    p = np.arange(-LIM, LIM + 1, dtype=np.int64)
    bits = pattern(p).astype(np.int64)
    assert np.array_equal(bits, 0x4B400000 + p)
    back = (bits.astype(np.uint32).view(np.float32) - BIAS).astype(np.int64)
    assert np.array_equal(back, p)


def test_differing_bits_match_the_integers():
    rng = np.random.default_rng(7)
    a = rng.integers(-LIM, LIM + 1, size=2_000_000)
    # b: a moved by a power of two (an advance), or anywhere in range
    step = 1 << rng.integers(0, 21, size=a.size)
    b = np.where(rng.random(a.size) < 0.5, a + step, rng.integers(-LIM, LIM + 1, size=a.size))
    b = np.clip(b, -LIM, LIM)
    x_int = (a ^ b).astype(np.int64) & 0xFFFFFFFF
    x_bits = (pattern(a) ^ pattern(b)).astype(np.int64)
    low = (1 << 21) - 1
    assert np.array_equal(x_int & low, x_bits & low)
    assert np.array_equal(x_int > low, x_bits > low)  # a difference at bit 21 or above in both or neither
    # the pop's height: msb + 1 equal while below 22, and above every SubDAG's otherwise
    def msb(v):
        out = np.full(v.shape, -1, dtype=np.int64)
        nz = v > 0
        out[nz] = np.floor(np.log2(v[nz].astype(np.float64))).astype(np.int64)
        return out
    m_int, m_bits = msb(x_int), msb(x_bits)
    small = m_int < 21
    assert np.array_equal(m_int[small], m_bits[small])
    assert np.all(m_bits[~small] >= 21)


def test_child_bits_and_masked_positions():
    rng = np.random.default_rng(11)
    p = rng.integers(-LIM, LIM + 1, size=1_000_000)
    m = rng.integers(0, 21, size=p.size)
    bits = pattern(p)
    assert np.array_equal((bits.astype(np.int64) >> m) & 1, (p >> m) & 1)
    keep = (~((np.int64(1) << m) - 1)) & 0xFFFFFFFF
    rebuilt = ((bits.astype(np.int64) & keep).astype(np.uint32).view(np.float32) - BIAS).astype(np.int64)
    assert np.array_equal(rebuilt, p & ~((np.int64(1) << m) - 1))


def test_child_size_from_exponent():
    for m in range(0, 22):
        built = np.array([(127 + m) << 23], dtype=np.uint32).view(np.float32)[0]
        assert built == np.float32(1 << m)
