// Test harness (CPU): the float-float helpers of the FP64 pair kernel
// (cubble_gb300/csrc/ff.cuh) against long double arithmetic. Prints one line
// "name max_relative_error" per helper. Built and run by tests/test_ff.py with
// -ffp-contract=off (the error-free transformations must not be fused).
#include <algorithm>
#include <cstdio>
#include <random>

#include "../cubble_gb300/csrc/ff.cuh"

using cbg::ff;
typedef long double ld;

static ld val(ff a) { return (ld)a.h + (ld)a.l; }
static ld rel(ld got, ld want) {
    const ld d = got - want;
    const ld m = want < 0 ? -want : want;
    return (d < 0 ? -d : d) / (m > 0 ? m : 1);
}
struct Max {
    const char *name;
    ld v = 0;
    void add(ld e) {
        if (e > v) v = e;
    }
};

int main() {
    std::mt19937_64 rng(12345);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    auto logu = [&](double lo, double hi) { return std::exp2(lo + (hi - lo) * U(rng)); };
    auto sgn = [&]() { return U(rng) < 0.5 ? -1.0 : 1.0; };
    auto rnd_ff = [&](double lo, double hi) { return cbg::ff_of(sgn() * logu(lo, hi)); };

    Max split{"split"}, back{"to_double"}, back_ulp{"to_double_ulps"}, add{"add"},
        addc{"add_cancel_abs"}, mul{"mul"}, sqr{"sqr"}, rcp{"rcp"}, rsq{"rsqrt"},
        sqt{"sqrt"}, pair{"pair_velocity"}, chord{"chord_area_abs"}, rsqd{"rsqrt_d_ulps"},
        rcpd{"rcp_d_ulps"}, sqd{"sqrt_ffd"}, small{"add_small_ulps"},
        subx{"sub_exact_mismatches"};
    const int N = 400000;
    for (int it = 0; it < N; it++) {
        // split: top 24 bits exact, the rest to 2^-47
        const double x = sgn() * logu(-70, 100);
        const ff s = cbg::ff_of(x);
        split.add(rel(val(s), (ld)x));
        // back to double: normalised pairs, including h = 2^k with l of the
        // opposite sign
        float h = (float)(sgn() * logu(-60, 60));
        if (it % 7 == 0) h = std::ldexp(1.0f, (int)(U(rng) * 80) - 40) * (float)sgn();
        const float l = (float)(sgn() * std::fabs((double)h) * logu(-60, -24));
        const ff v = cbg::fast_two_sum(h, l);
        const double d = cbg::ff_to_double(v);
        const ld exact = val(v);
        back.add(rel((ld)d, exact));
        const double ulp = std::ldexp(1.0, std::ilogb(d) - 52);
        const ld du = ((ld)d - exact) / (ld)ulp;
        back_ulp.add(du < 0 ? -du : du);
        // arithmetic
        const ff a = rnd_ff(-20, 20), b = rnd_ff(-20, 20);
        add.add(rel(val(cbg::ff_add(a, cbg::ff_abs(b))) , val(a) + val(cbg::ff_abs(b))) *
                ((val(a) > 0) ? 1 : 0));
        {   // cancellation: absolute error against |a| + |b|
            const ff c = cbg::ff_mul(a, cbg::ff_of(1.0 + 1e-9 * sgn() * U(rng)));
            const ld got = val(cbg::ff_sub(a, c)), want = val(a) - val(c);
            const ld m = (val(a) < 0 ? -val(a) : val(a)) + (val(c) < 0 ? -val(c) : val(c));
            addc.add((got > want ? got - want : want - got) / m);
        }
        mul.add(rel(val(cbg::ff_mul(a, b)), val(a) * val(b)));
        sqr.add(rel(val(cbg::ff_sqr(a)), val(a) * val(a)));
        const ff p = cbg::ff_abs(a);
        rcp.add(rel(val(cbg::ff_rcp(p)), 1.0L / val(p)));
        rsq.add(rel(val(cbg::ff_rsqrt(p)), 1.0L / std::sqrt(val(p))));
        sqt.add(rel(val(cbg::ff_sqrt(p)), std::sqrt(val(p))));
        // FP64 results with few FP64 instructions: 1/sqrt and 1/x to ~1 ulp
        {
            const double q = logu(-90, 90);
            const double rd = cbg::rsqrt_d_core(q), cd = cbg::rcp_d_core(q);
            const ld rq = 1.0L / std::sqrt((ld)q), cq = 1.0L / (ld)q;
            rsqd.add((rd > rq ? rd - rq : rq - rd) / (ld)std::ldexp(1.0, std::ilogb(rd) - 52));
            rcpd.add((cd > cq ? cd - cq : cq - cd) / (ld)std::ldexp(1.0, std::ilogb(cd) - 52));
            sqd.add(rel((ld)cbg::sqrt_ffd(q), std::sqrt((ld)q)));
            // y + c for |c| <= 2^-31 y, near binade edges too
            double y = logu(-60, 60);
            if (it % 5 == 0) y = std::ldexp(1.0, (int)(U(rng) * 100) - 50) * (1.0 + 1e-15 * sgn());
            const float cc = (float)(sgn() * y * logu(-70, -31));
            const double z = cbg::ff_add_small(y, cc);
            const ld zq = (ld)y + (ld)cc;
            small.add((z > zq ? z - zq : zq - z) / (ld)std::ldexp(1.0, std::ilogb(z) - 52));
        }
        // exact subtraction: bit-identical to the FP64 one on nearby values
        // (both signs, across binade edges, equal), far apart, zeros and
        // values of opposite sign
        {
            double p = sgn() * logu(-40, 40);
            if (it % 3 == 0) p = sgn() * std::ldexp(1.0, (int)(U(rng) * 60) - 30);
            double q = p + sgn() * std::fabs(p) * logu(-55, 2);
            if (it % 11 == 0) q = p;
            if (it % 13 == 0) q = -q;
            if (it % 17 == 0) q = 0.0;
            if (it % 19 == 0) p = std::ldexp(p, -1000);
            const double want = p - q, got = cbg::sub_exact(p, q);
            if (std::memcmp(&want, &got, 8) != 0) subx.add(subx.v + 1);
        }
        // the pair velocity factor f0 (1/|d| - 1/(r1 + r2)) and the chord
        // area r2^2 - w^2 / 4, w = (r2^2 - r1^2 + m) / |d|, on overlapping
        // pairs of radii ~ 1 (|d| < r1 + r2)
        const double r1 = 0.3 + 2.0 * U(rng), r2 = 0.3 + 2.0 * U(rng);
        // chord branch only: neither centre inside the other bubble
        const double lo = std::max(r1, r2) / (r1 + r2);
        const double dist = (r1 + r2) * (lo + (0.999 - lo) * U(rng));
        const double ux = sgn() * U(rng), uy = sgn() * U(rng), uz = sgn() * U(rng);
        const double un = std::sqrt(ux * ux + uy * uy + uz * uz) + 1e-300;
        const double dx = dist * ux / un, dy = dist * uy / un, dz = dist * uz / un;
        const ff X = cbg::ff_of(dx), Y = cbg::ff_of(dy), Z = cbg::ff_of(dz);
        const ff m = cbg::ff_add(cbg::ff_add(cbg::ff_sqr(X), cbg::ff_sqr(Y)), cbg::ff_sqr(Z));
        const ff R = cbg::ff_add(cbg::ff_of(r1), cbg::ff_of(r2));
        const ff rs = cbg::ff_rsqrt(m);
        const ff sv = cbg::ff_sub(rs, cbg::ff_rcp(R));
        const ld mL = (ld)dx * dx + (ld)dy * dy + (ld)dz * dz;
        const ld rsL = 1.0L / std::sqrt(mL);
        const ld svL = rsL - 1.0L / ((ld)r1 + (ld)r2);
        // absolute error of the factor against its first term 1/|d|
        pair.add((val(sv) > svL ? val(sv) - svL : svL - val(sv)) / rsL);
        const ff r1sq = cbg::ff_of(r1 * r1), r2sq = cbg::ff_of(r2 * r2);
        const ff w = cbg::ff_mul(cbg::ff_add(cbg::ff_sub(r2sq, r1sq), m), rs);
        const ff oa = cbg::ff_abs(cbg::ff_sub(r2sq, cbg::ff_scale(cbg::ff_sqr(w), 0.25f)));
        const ld wL = ((ld)(r2 * r2) - (ld)(r1 * r1) + mL) * rsL;
        ld oaL = (ld)(r2 * r2) - wL * wL / 4;
        oaL = oaL < 0 ? -oaL : oaL;
        const ld scale = (ld)(r1 * r1) + (ld)(r2 * r2) + mL;
        chord.add((val(oa) > oaL ? val(oa) - oaL : oaL - val(oa)) / scale);
    }
    for (Max *m : {&split, &back, &back_ulp, &add, &addc, &mul, &sqr, &rcp, &rsq, &sqt, &pair,
                   &chord, &rsqd, &rcpd, &sqd, &small, &subx})
        std::printf("%s %.6Le\n", m->name, m->v);
    return 0;
}
