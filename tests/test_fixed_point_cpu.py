"""CPU: the integer identities the emulated-FP64 kernels rely on, restated in
exact Python integers (f90_dns_gb300/csrc/tc.cuh, step.cu):

* digit pairs (tc_digit_pairs): the 7-bit fields of U + 64 (1 + 128 + ... +
  128^7), minus 64, are U's balanced base-128 digits (tc_digits), and the
  FP16 with bits 0x6400 | v is 1024 + v, so one subtraction of 1088 gives the
  digit exactly;
* class combination (tc_combine8): pairing adjacent weight classes in 32-bit
  integers gives the same T as summing every class term in 64 bits;
* limb products (fx_mac, the fixed-point Poisson solve): four 32 x 32-bit
  limb products of a 58-bit and a 54-bit integer, summed in 64-bit partial
  sums over up to 65 terms, recombine to the exact 128-bit dot product
  without overflow;
* column keys (tc_key, tc_exponent_key): the largest 32-bit key of a column
  gives the same power-of-two scale as its largest |x|.
"""
import random

import numpy as np

BIAS = 0x0081020408102040  # 64 in each of the 8 base-128 digit places


def balanced_digits(u):
    """tc_digits: 8 balanced base-128 digits, most significant first."""
    c = [0] * 8
    for s in range(7, -1, -1):
        r = u & 127
        d = r - 128 if r >= 64 else r
        c[s] = d
        u = (u - d) >> 7
    assert u == 0
    return c


def biased_field_digits(u):
    v = u + BIAS
    assert 0 <= v < 2**56
    return [((v >> (7 * (7 - s))) & 127) - 64 for s in range(8)]


def test_bias_constant():
    assert BIAS == sum(64 * 128**s for s in range(8))


def test_biased_fields_are_the_balanced_digits():
    rng = random.Random(1)
    cases = [0, 1, -1, 2**54, -2**54, 63, 64, -64, -65, 2**53 + 12345]
    cases += [rng.randint(-2**54, 2**54) for _ in range(20000)]
    for u in cases:
        d = biased_field_digits(u)
        assert d == balanced_digits(u), u
        assert all(-64 <= x <= 63 for x in d)
        assert sum(x * 128**(7 - s) for s, x in enumerate(d)) == u


def test_fp16_field_encoding():
    for v in range(128):
        bits = np.array([0x6400 | v], dtype=np.uint16)
        h = bits.view(np.float16)[0]
        assert float(h) == 1024.0 + v
        assert float(np.float16(h) - np.float16(1088.0)) == v - 64  # exact in FP16
    assert np.array([0x6440], dtype=np.uint16).view(np.float16)[0] == np.float16(1088.0)


def class_sum_64(D):
    t = sum(D[c] * 2**(7 * (6 - c)) for c in range(7))
    return t + ((D[7] + 64) >> 7)


def class_sum_paired(D):
    def i32(x):
        assert -2**31 <= x < 2**31
        return x
    pa = i32(D[0] * 128 + D[1])
    pb = i32(D[2] * 128 + D[3])
    pc = i32(D[4] * 128 + D[5])
    tail = i32(D[6] + ((D[7] + 64) >> 7))
    t = pa * 16384 + pb
    t = t * 16384 + pc
    return t * 128 + tail


def test_paired_class_combination():
    rng = random.Random(2)
    lim = 2**22 - 1
    for _ in range(20000):
        D = [rng.randint(-lim, lim) for _ in range(8)]
        assert class_sum_paired(D) == class_sum_64(D)
    for D in ([lim] * 8, [-lim] * 8, [lim, -lim] * 4):
        assert class_sum_paired(D) == class_sum_64(D)


def limb_dot(A, B):
    p = [0, 0, 0, 0]  # weights 2^0, 2^27, 2^29, 2^56
    for a, b in zip(A, B):
        a0, a1 = a & 0x1FFFFFFF, a >> 29
        b0, b1 = b & 0x7FFFFFF, b >> 27
        for x in (a0, a1, b0, b1):
            assert -2**31 <= x < 2**31
        p[0] += a0 * b0
        p[1] += a0 * b1
        p[2] += a1 * b0
        p[3] += a1 * b1
        assert all(-2**63 <= x < 2**63 for x in p)
    return p[0] + p[1] * 2**27 + p[2] * 2**29 + p[3] * 2**56


def test_limb_products_exact_up_to_65_terms():
    rng = random.Random(3)
    for n in (1, 17, 33, 49, 65):
        for _ in range(300):
            A = [rng.randint(-2**58, 2**58) for _ in range(n)]
            B = [rng.randint(-2**54, 2**54) for _ in range(n)]
            assert limb_dot(A, B) == sum(a * b for a, b in zip(A, B))
        # the extreme magnitudes, all of one sign: the partial sums' worst case
        A = [2**58] * n
        B = [-2**54] * n
        assert limb_dot(A, B) == sum(a * b for a, b in zip(A, B))


def _exponent(x_max):
    """tc_exponent: the smallest f with |x| < 2^f for the largest |x| (0 if zero)."""
    if x_max == 0.0:
        return 0
    m, e = np.frexp(x_max)  # x = m 2^e, 0.5 <= m < 1
    return int(e)


def _fixed(x, f, bits):
    """tc_fixed_bits: round(x 2^(bits - f)), ties away from zero, exactly."""
    from fractions import Fraction
    v = Fraction(x) * Fraction(2) ** (bits - f)
    a = abs(v)
    r = int(a + Fraction(1, 2)) if a.denominator != 1 else int(a)
    return r if v >= 0 else -r


def test_fixed_point_solve_error_bound():
    """The fixed-point Poisson solve restated (k_fixed_rows, pressure_solve_body):
    58-bit rows with per-row exponents, a 54-bit column with one exponent over
    its re and im parts (one more for the exact even/odd fold), exact products,
    T = round(S / 2^56).  The error of every output is bounded by the operand
    roundings (half a unit of 2^(f-54) per column entry times |G_kj|, half a
    unit of 2^(e-58) per row entry times |b_j|) and the one final rounding:
    the bound of an FP64 dot product, normwise."""
    from fractions import Fraction
    rng = np.random.default_rng(5)
    for n in (9, 33, 65):
        M = rng.standard_normal((n, n)) + n * np.eye(n)
        G = np.linalg.inv(M @ M.T)  # a symmetric positive inverse, like the Poisson blocks
        b = rng.standard_normal(n) * 10.0 ** rng.uniform(-3, 3)
        f = _exponent(float(np.max(np.abs(b)))) + 1
        B = [_fixed(v, f, 54) for v in b]
        assert all(abs(x) <= 2**54 for x in B)
        for k in range(n):
            row = G[k]
            e = _exponent(float(np.max(np.abs(row))))
            A = [_fixed(v, e, 58) for v in row]
            assert all(abs(x) <= 2**58 for x in A)
            S = sum(a * c for a, c in zip(A, B))
            T = (S + 2**55) >> 56
            x = Fraction(T) * Fraction(2) ** (e + f - 56)
            exact = sum(Fraction(float(g)) * Fraction(float(v)) for g, v in zip(row, b))
            bound = (sum(Fraction(abs(float(g))) for g in row) * Fraction(2) ** (f - 55)
                     + sum(abs(c) for c in B) * Fraction(2) ** (f - 54) * Fraction(2) ** (e - 59)
                     + Fraction(2) ** (e + f - 57))
            assert abs(x - exact) <= bound, (n, k)


def _key(x):
    """tc_key: the high word of |x| with the low word's nonzero-ness in its lowest bit."""
    ab = int(np.array([x], dtype=np.float64).view(np.uint64)[0]) & 0x7FFFFFFFFFFFFFFF
    return (ab >> 32) | (1 if (ab & 0xFFFFFFFF) else 0)


def _exponent_bits(absbits):
    """tc_exponent on the bits of the largest |x|."""
    if absbits == 0:
        return 0
    ex = absbits >> 52
    return (-1022 if ex == 0 else ex - 1023) + 1


def _exponent_key(key):
    """tc_exponent_key."""
    if key == 0:
        return 0
    ex = key >> 20
    return (-1022 if ex == 0 else ex - 1023) + 1


def test_column_keys_give_the_column_exponent():
    """The viscous tensor-core kernel takes a column's power-of-two scale from
    the largest 32-bit key of its values (a warp maximum and a shared atomic)
    instead of the largest 64-bit |x|: the key orders like |x| and keeps the
    exponent field and zero-ness, so the exponent is the same, for zeros,
    subnormals, infinities and NaNs as well."""
    rng = np.random.default_rng(7)
    specials = [0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1.0, -1.0, 1.5, 2.0 ** -1022,
                2.0 ** -1023, np.inf, -np.inf, np.nan, 1.7976931348623157e308, 2.0 ** 52 + 1.0]
    for trial in range(3000):
        n = int(rng.integers(1, 80))
        col = rng.standard_normal(n) * 10.0 ** rng.uniform(-300, 300, n)
        col[rng.random(n) < 0.2] = 0.0
        if trial % 3 == 0:
            col[rng.integers(0, n)] = specials[trial // 3 % len(specials)]
        bits = col.view(np.uint64) & np.uint64(0x7FFFFFFFFFFFFFFF)
        ref = _exponent_bits(int(bits.max()))
        got = _exponent_key(max(_key(float(v)) for v in col))
        assert got == ref, (col, got, ref)
    # one column of values that differ only in their low word
    col = np.array([1.0, np.nextafter(1.0, 2.0), -np.nextafter(2.0, 1.0)])
    assert _exponent_key(max(_key(v) for v in col)) == 1
