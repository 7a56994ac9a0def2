"""The double-float arithmetic of the FP64 degridders (rc_gb300/csrc/gb_plain.cu:
df_split, df_cmac, two_sum_acc), restated operation by operation in numpy
float32 and checked without a GPU: the bit-pattern split holds every double
to 2^-48 of itself, and complex sums of products stay within 1e-12 of the
exact (extended-precision) sum relative to the sum of the magnitudes, over
magnitudes 1e+-150 and dynamic ranges to 1e12.  The GPU kernels themselves are
checked against the oracle in tests/test_gpu_fp64_df.py and the FP64 parity
tests."""
import numpy as np

f32 = np.float32


def _u32_to_f32(u):
    return np.array([u & 0xFFFFFFFF], np.uint32).view(np.float32)[0]


def df_split(x, k):
    """x * 2^-k as (hi, lo) floats from x's bit pattern (gb_plain.cu df_split)."""
    b = int(np.array([x], np.float64).view(np.uint64)[0])
    hi32, lo32 = b >> 32, b & 0xFFFFFFFF
    e = (hi32 >> 20) & 0x7FF
    fe = e - k - 896
    if e == 0 or fe <= 0:
        return f32(0), f32(0)
    sign = hi32 & 0x80000000
    top = ((hi32 & 0xFFFFF) << 3) | (lo32 >> 29)
    up = (lo32 >> 28) & 1
    hi = _u32_to_f32(sign | (((fe << 23) | top) + up))
    lo = f32(0)
    if fe > 52:
        rem = (lo32 & 0x1FFFFFFF) - (up << 29)
        lo = f32(f32(rem) * _u32_to_f32((fe - 52) << 23))
    lo = _u32_to_f32(int(np.array([lo], np.float32).view(np.uint32)[0]) ^ sign)
    return hi, lo


def fma(a, b, c):
    # a*b is exact in float64 for float32 operands; one rounding to float32
    # after the add (a second, float64 rounding of the add is far below it)
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def two_sum_acc(s, c, p):
    t = f32(s + p)
    bp = f32(t - s)
    e = f32(f32(s - f32(t - bp)) + f32(p - bp))
    return t, f32(c + e)


def df_cmac(a, b, acc, conj):
    ax, ay, az, aw = a
    bx, by, bz, bw = b
    if conj:
        bz, bw = -bz, -bw
    p1 = f32(ax * bx); e1 = fma(ax, bx, -p1)
    p2 = f32(az * bz); e2 = fma(az, bz, -p2)
    p3 = f32(ax * bz); e3 = fma(ax, bz, -p3)
    p4 = f32(az * bx); e4 = fma(az, bx, -p4)
    lr = fma(ax, by, fma(ay, bx, f32(e1 - e2)))
    lr = fma(-az, bw, fma(-aw, bz, lr))
    li = fma(ax, bw, fma(ay, bz, f32(e3 + e4)))
    li = fma(az, by, fma(aw, bx, li))
    sx, sy, cz, cw = acc
    cz = f32(cz + lr)
    cw = f32(cw + li)
    sx, cz = two_sum_acc(sx, cz, p1)
    sx, cz = two_sum_acc(sx, cz, -p2)
    sy, cw = two_sum_acc(sy, cw, p3)
    sy, cw = two_sum_acc(sy, cw, p4)
    return sx, sy, cz, cw


def scale_exp(arr):
    e = int(((arr.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)).max())
    return e - 1023 if 0 < e < 0x7FF else 0


def test_split_holds_every_double_to_2_pow_minus_48():
    rng = np.random.default_rng(1)
    xs = list(rng.standard_normal(400) * 10.0 ** rng.uniform(-30, 30, 400))
    xs += [1.0, -2.5, 3.0e-300, 1e300, np.nextafter(1.0, 2.0), 1.0 - 2.0 ** -53]
    for x in xs:
        for k in (0, 50, -50, 995, -1000):
            ref = np.ldexp(np.longdouble(x), -k)
            if abs(ref) >= 2.0 ** 127:
                continue  # the kernel's k always puts the array's largest value in [1, 2)
            hi, lo = df_split(x, k)
            if abs(ref) >= 2.0 ** -74:
                assert abs(np.longdouble(hi) + np.longdouble(lo) - ref) <= abs(ref) * 2.0 ** -48
            elif abs(ref) >= 2.0 ** -126:
                assert abs(np.longdouble(hi) - ref) <= abs(ref) * 2.0 ** -24  # low part dropped
            else:
                assert hi == 0 and lo == 0


def test_complex_sums_of_products():
    rng = np.random.default_rng(2)
    worst = 0.0
    for trial in range(24):
        n = int(rng.integers(1, 200))
        dyn = rng.uniform(0, 12)
        g = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * 10.0 ** (
            rng.uniform(-150, 150) + rng.uniform(-dyn, 0, n))
        c = (rng.standard_normal(n) + 1j * rng.standard_normal(n)) * 10.0 ** (
            rng.uniform(-150, 150) + rng.uniform(-dyn, 0, n))
        conj = bool(trial & 1)
        kg, kc = scale_exp(g.view(np.float64)), scale_exp(c.view(np.float64))
        acc = (f32(0), f32(0), f32(0), f32(0))
        for t in range(n):
            a = df_split(g[t].real, kg) + df_split(g[t].imag, kg)
            b = df_split(c[t].real, kc) + df_split(c[t].imag, kc)
            acc = df_cmac((a[0], a[1], a[2], a[3]), (b[0], b[1], b[2], b[3]), acc, conj)
        got = complex(np.ldexp(np.float64(acc[0]) + np.float64(acc[2]), kg + kc),
                      np.ldexp(np.float64(acc[1]) + np.float64(acc[3]), kg + kc))
        gl, cl = g.astype(np.clongdouble), c.astype(np.clongdouble)
        exact = complex((gl * (np.conj(cl) if conj else cl)).sum())
        mag = float((np.abs(gl) * np.abs(cl)).sum())
        worst = max(worst, abs(got - exact) / mag)
    assert worst < 1e-12
