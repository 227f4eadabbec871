"""The float64 pass rounds its residual to float32 with integer operations
(d2f_rn in flowlab_gb300/csrc/fl_common.cuh) when the result is a normal
float: keep the top 23 mantissa bits under the float exponent, add one when
the 29 bits rounded away exceed half an ulp, or equal it with the kept value
odd. This restates that formula with numpy's integers and checks it against
IEEE double -> float conversion (numpy's astype) on random doubles across
the whole fast-path exponent range and on the halfway, carry and overflow
cases (CPU)."""
import numpy as np


def d2f_formula(bits):
    """bits: uint64 array of doubles in the fast path (float exponent 1..254);
    returns the float32 bit patterns."""
    ex = (bits >> np.uint64(52)) & np.uint64(0x7FF)
    m = bits & np.uint64(0xFFFFFFFFFFFFF)
    rem = m & np.uint64(0x1FFFFFFF)
    f = ((ex - np.uint64(896)) << np.uint64(23)) | (m >> np.uint64(29))
    half = np.uint64(0x10000000)
    up = (rem > half) | ((rem == half) & ((f & np.uint64(1)) == np.uint64(1)))
    f = f + up.astype(np.uint64)
    sign = (bits >> np.uint64(63)) << np.uint64(31)
    return (sign | f).astype(np.uint32)


def check(bits):
    ex = (bits >> np.uint64(52)) & np.uint64(0x7FF)
    assert ((ex >= 897) & (ex <= 1150)).all()
    with np.errstate(over="ignore"):  # the cases that round past the largest float
        want = bits.view(np.float64).astype(np.float32).view(np.uint32)
    got = d2f_formula(bits)
    bad = np.nonzero(want != got)[0]
    assert bad.size == 0, [hex(int(b)) for b in bits[bad[:5]]]


def test_random_doubles_round_like_ieee():
    rng = np.random.default_rng(7)
    n = 2_000_000
    ex = rng.integers(897, 1151, n, dtype=np.uint64)
    m = rng.integers(0, 1 << 52, n, dtype=np.uint64)
    sign = rng.integers(0, 2, n, dtype=np.uint64)
    check((sign << np.uint64(63)) | (ex << np.uint64(52)) | m)


def test_halfway_carry_and_overflow_cases():
    cases = []
    for ex in (897, 898, 1000, 1023, 1149, 1150):
        for hi in (0, 1, 2, 0x3FFFFE, 0x3FFFFF, 0x7FFFFE, 0x7FFFFF):  # kept mantissa (23 bits)
            for lo in (0, 1, 0x0FFFFFFF, 0x10000000, 0x10000001, 0x1FFFFFFF):  # rounded-away bits (29)
                for sign in (0, 1):
                    cases.append((sign << 63) | (ex << 52) | (hi << 29) | lo)
    check(np.array(cases, dtype=np.uint64))
