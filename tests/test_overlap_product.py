"""CPU: the mixed form's overlap product (r1 + r2)^2 - d^2 from fixed-point
integers (units 2^-40), restated in Python integers exactly as the pair
kernel forms it: v = h 2^20 + l with h = v >> 20 (arithmetic) and
l = v & (2^20 - 1); k1 = h_r^2 - sum h^2, k2 = h_r l_r - sum h l; the
product is (k1 + (k2 >> 19)) 2^-40 before its one FP32 rounding. Checked
against the exact product on random overlapping pairs, for negative
differences too: the integer value is within 2^-38 absolute of the exact
one, and the brackets stay inside 64-bit integers while r1 + r2 < 16."""
import numpy as np

FIX = 1 << 40


def split(v):
    return v >> 20, v & 0xFFFFF  # Python's >> floors, as the arithmetic shift does


def kernel_product(ex, ey, ez, rq):
    (hx, lx), (hy, ly), (hz, lz), (hr, lr) = split(ex), split(ey), split(ez), split(rq)
    k1 = hr * hr - (hx * hx + hy * hy + hz * hz)
    k2 = hr * lr - (hx * lx + hy * ly + hz * lz)
    for k in (k1, k2, hr * hr, hx * hx + hy * hy + hz * hz):
        assert -(1 << 63) <= k < (1 << 63)
    return k1 + (k2 >> 19)  # units 2^-40


def test_split_identity():
    rng = np.random.default_rng(3)
    for v in rng.integers(-(1 << 45), 1 << 45, 2000).tolist():
        h, l = split(v)
        assert h * (1 << 20) + l == v and 0 <= l < (1 << 20)


def test_overlap_product_exact_to_2_38():
    rng = np.random.default_rng(4)
    worst = 0.0
    for _ in range(5000):
        r1, r2 = rng.uniform(0.05, 7.9, 2)
        R = r1 + r2
        d = R * rng.uniform(0.0, 1.0)  # overlapping
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        e = [int(round(c * d * FIX)) for c in u]
        rq = int(round(r1 * FIX)) + int(round(r2 * FIX))
        assert rq < (1 << 44)
        exact = rq * rq - sum(c * c for c in e)  # units 2^-80
        got = kernel_product(e[0], e[1], e[2], rq) * FIX  # units 2^-80
        worst = max(worst, abs(got - exact) / 2.0 ** 80)
    assert worst <= 2.0 ** -38, worst
