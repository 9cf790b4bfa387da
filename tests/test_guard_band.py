"""CPU: the FP32 prefilter of the 3D warp-per-cell search pass against exact
arithmetic, emulated bit for bit in numpy (FP32 roundings, the 64-bit fixed
point x 2^40, the two-word int -> float conversion).

The pass decides a candidate pair in FP32 unless e = d^2 - cut^2 lies within
+-tb of zero, tb = 2 cutmax band, band = 4e-6 cw + 2e-6 (cw the cell edge);
there the reference's FP64 test decides. That is exact as long as the FP32
e never differs from the exact one by tb or more. Sampled here on pairs in
neighbouring cells (periodic images included) near the cutoff, in a large
box, the worst error stays below a quarter of tb."""
import numpy as np

FIX = 2.0 ** 40


def f32(x):
    return np.float32(x)


def fma32(a, b, c):
    # float32 product is exact in float64; one rounding to float32 at the end
    return np.float32(np.float64(a) * np.float64(b) + np.float64(c))


def len_from_fix(d):
    """The kernel's fixed-point difference -> FP32 (two 32-bit conversions,
    an FMA, a product by 2^-40)."""
    a = abs(int(d))
    hi = np.float32(a >> 32)
    lo = np.float32(a & 0xFFFFFFFF)
    f = fma32(hi, np.float32(4294967296.0), lo)
    f = np.float32(f * np.float32(9.094947017729282e-13))
    return -f if d < 0 else f


def fix(x):
    return int(np.trunc(x * FIX))  # toward zero, as fix_from_double


def test_cell_relative_band_covers_fp32_error():
    rng = np.random.default_rng(5)
    L = 380.0  # the 10^7-bubble foam's box edge
    skin = 0.3
    rmax = 1.75
    cut_max = 2 * rmax + skin
    cd = int(L // cut_max)
    cw = L / cd
    lq = int(round(L * FIX))
    cwq = lq // cd
    cw_f = np.float32(cwq * 2.0 ** -40)
    band = 4e-6 * float(cw_f) + 2e-6
    tb = np.float32(2.0 * band * (2.0 * (rmax + 1e-3) + skin))
    worst = 0.0
    for _ in range(20000):
        ri, rj = rng.uniform(0.3, rmax, 2)
        cut = ri + rj + skin
        # home bubble anywhere; the partner at a distance within 1e-3 of the
        # cutoff in a random direction, wrapped into the box
        xi = rng.uniform(0.0, L, 3)
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        xj = xi + u * (cut + rng.uniform(-1e-3, 1e-3))
        xj = np.mod(xj, L)
        ki = np.minimum((xi * cd / L).astype(int), cd - 1)
        kj = np.minimum((xj * cd / L).astype(int), cd - 1)
        off = kj - ki
        off = np.where(off > 1, off - cd, np.where(off < -1, off + cd, off))
        if np.any(np.abs(off) > 1):
            continue
        pi = [len_from_fix(fix(xi[a]) - (0 + int(ki[a]) * cwq)) for a in range(3)]
        pj = [len_from_fix(fix(xj[a]) - (0 + int(kj[a]) * cwq)) for a in range(3)]
        pj = [fma32(np.float32(off[a]), cw_f, pj[a]) for a in range(3)]
        dx, dy, dz = (np.float32(pi[a] - pj[a]) for a in range(3))
        d2 = fma32(dz, dz, fma32(dy, dy, np.float32(dx * dx)))
        wj = np.float32(f32(rj) + f32(skin))
        c32 = np.float32(f32(ri) + wj)
        e = fma32(-c32, c32, d2)
        # exact: minimum-image difference of the FP64 positions
        d = xi - xj
        d -= L * np.round(d / L)
        e_exact = float(np.dot(d, d)) - cut * cut
        worst = max(worst, abs(float(e) - e_exact))
    assert worst < 0.25 * float(tb), (worst, float(tb))


def test_box_relative_band_covers_fp32_error():
    """The same for the thread-per-bubble pass (FP32 absolute coordinates and
    the FP32 minimum image, band 2e-6 (max|x| + L) + 1e-5 as a distance)."""
    rng = np.random.default_rng(6)
    L = 380.0
    skin = 0.3
    band = 2e-6 * (L + L) + 1e-5
    L32 = np.float32(L)
    half32 = np.float32(0.5 * L)
    worst = 0.0
    for _ in range(20000):
        ri, rj = rng.uniform(0.3, 1.75, 2)
        cut = ri + rj + skin
        xi = rng.uniform(0.0, L, 3)
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        xj = np.mod(xi + u * (cut + rng.uniform(-1e-3, 1e-3)), L)
        dd = []
        for a in range(3):
            t = np.float32(abs(np.float32(xi[a]) - np.float32(xj[a])))
            if t > half32:
                t = np.float32(L32 - t)
            dd.append(t)
        d2 = fma32(dd[2], dd[2], fma32(dd[1], dd[1], np.float32(dd[0] * dd[0])))
        dist32 = float(np.sqrt(np.float64(d2)))
        d = xi - xj
        d -= L * np.round(d / L)
        dist = float(np.sqrt(np.dot(d, d)))
        worst = max(worst, abs(dist32 - dist))
    assert worst < 0.25 * band, (worst, band)
