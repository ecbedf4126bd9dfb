// The integer forms of f64 operations (f64_int.cuh) against the host's f64
// arithmetic, on the host: lerp_half_int against a + (b - a) / 2; f64_eq,
// f64_lt and f64_le against ==, < and <=; f64_abs against fabs;
// f64_scale_pow2 against x * 2^k; f64_round_i32 against (int32_t)round(x);
// f64_to_f32 against (float)x; f64_add_int against a + b and a - b;
// f64_div_int against a / b.  Operands: random bit patterns, pairs in the
// same binade, in neighbouring binades, a few ulps apart, of either sign,
// drawing coordinates, exact and nearly exact quotients, the exponent limits
// of each integer form, zeros, subnormals, infinities and NaNs.  Whenever an
// integer form takes an operand, its result must have the f64 result's bits.
// Exit status 0 when no result differs.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>

#include "f64_int.cuh"
using namespace z2dg;

static uint64_t s = 0x243F6A8885A308D3ull;
static uint64_t xs() {
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    return s;
}
static double bits(uint64_t b) { return f64_from(b); }
static uint64_t raw(double d) { return f64_bits(d); }
static uint32_t raw32(float f) {
    uint32_t b;
    memcpy(&b, &f, 4);
    return b;
}

// volatile keeps the reference expressions from being folded or fused
static volatile double two = 2.0;
static double ref_lerp(double a, double b) {
    const double h = (b - a) / two;
    return a + h;
}

struct Count {
    const char *name;
    unsigned long long n = 0, taken = 0, wrong = 0;
    void report() const { printf("%s: cases %llu  integer %llu  wrong %llu\n", name, n, taken, wrong); }
};

int main() {
    Count lerp{"lerp_half"}, eq{"eq"}, lt{"lt"}, scale{"scale_pow2"}, rnd{"round_i32"}, cvt{"to_f32"}, add{"add"}, dv{"div"};
    auto pair = [&](double a, double b) {
        bool done;
        const double r = lerp_half_int(a, b, done);
        lerp.n++;
        if (done) {
            lerp.taken++;
            const double t = ref_lerp(a, b);
            if (raw(r) != raw(t)) {
                if (lerp.wrong < 5) printf("lerp a=%a b=%a int=%a f64=%a\n", a, b, r, t);
                lerp.wrong++;
            }
        }
        for (int neg = 0; neg < 2; neg++) {
            const double bb = neg ? -b : b;
            const double ra = f64_add_int(a, bb, done);
            add.n++;
            if (done) {
                add.taken++;
                volatile double va = a;
                const double t = va + bb;
                if (raw(ra) != raw(t)) {
                    if (add.wrong < 5) printf("add a=%a b=%a int=%a f64=%a\n", a, bb, ra, t);
                    add.wrong++;
                }
            }
        }
        {
            const double rq = f64_div_int(a, b, done);
            dv.n++;
            if (done) {
                dv.taken++;
                volatile double va = a;
                const double t = va / b;
                if (raw(rq) != raw(t)) {
                    if (dv.wrong < 5) printf("div a=%a b=%a int=%a f64=%a\n", a, b, rq, t);
                    dv.wrong++;
                }
            }
        }
        eq.n++;
        eq.taken++;
        if (f64_eq(a, b) != (a == b)) {
            if (eq.wrong < 5) printf("eq a=%a b=%a\n", a, b);
            eq.wrong++;
        }
        lt.n++;
        lt.taken++;
        if (f64_lt(a, b) != (a < b) || f64_le(a, b) != (a <= b) || raw(f64_abs(a)) != raw(fabs(a))) {
            if (lt.wrong < 5) printf("lt/le/abs a=%a b=%a\n", a, b);
            lt.wrong++;
        }
    };
    auto single = [&](double x) {
        bool done;
        static const double pows[] = {1.0, 2.0, 4.0, 16.0, 0.25, 0x1p100, 0x1p-100, 3.0, 0.0, -4.0};
        for (double p : pows) {
            const double r = f64_scale_pow2(x, p, done);
            scale.n++;
            if (done) {
                scale.taken++;
                volatile double vp = p;
                const double t = x * vp;
                if (raw(r) != raw(t)) {
                    if (scale.wrong < 5) printf("scale x=%a p=%a int=%a f64=%a\n", x, p, r, t);
                    scale.wrong++;
                }
            }
        }
        const int32_t ri = f64_round_i32(x, done);
        rnd.n++;
        if (done) {
            rnd.taken++;
            const int32_t t = (int32_t)round(x);
            if (ri != t) {
                if (rnd.wrong < 5) printf("round x=%a int=%d f64=%d\n", x, ri, t);
                rnd.wrong++;
            }
        }
        const float rf = f64_to_f32(x, done);
        cvt.n++;
        if (done) {
            cvt.taken++;
            volatile double vx = x;
            const float t = (float)vx;
            if (raw32(rf) != raw32(t)) {
                if (cvt.wrong < 5) printf("to_f32 x=%a int=%a f64=%a\n", x, (double)rf, (double)t);
                cvt.wrong++;
            }
        }
    };
    for (int i = 0; i < 12000000; i++) {
        const uint64_t A = xs();
        const int kind = (int)(xs() % 8);
        uint64_t B;
        if (kind == 0) B = xs();                                                                  // unrelated
        else if (kind == 1) B = (A & ~kF64Mant) | (xs() & kF64Mant);                             // same binade
        else if (kind == 2) B = A + (xs() % 64) - 32;                                             // a few ulps apart
        else if (kind == 3) B = (A + (1ull << 52)) ^ (xs() & kF64Mant);                           // next binade up
        else if (kind == 4) B = (A - (1ull << 52)) ^ (xs() & kF64Mant);                           // next binade down
        else if (kind == 5) B = A ^ (1ull << 63);                                                 // opposite sign
        else if (kind == 6) B = (A + (1ull << 52)) - (xs() % 4);                                  // near twice a
        else B = (A & (1ull << 63)) | ((uint64_t)(xs() % 6) << 52) | (xs() & kF64Mant);           // tiny
        pair(bits(A), bits(B));
        pair(bits(B), bits(A));
        single(bits(A));
        // coordinates of a drawing: moderate magnitudes, close together,
        // halves and f32 rounding ties
        const double c = ((double)(xs() >> 11) / 9007199254740992.0 - 0.25) * 8192.0;
        const double d = c + ((double)(xs() >> 11) / 9007199254740992.0 - 0.5) * ldexp(1.0, -(int)(xs() % 40));
        pair(c, d);
        single(c);
        single(d);
        single(floor(c) + 0.5);
        single(bits((raw(c) & ~((1ull << 29) - 1)) | (1ull << 28)));  // an exact f32 tie
        single(ldexp(c, (int)(xs() % 300) - 150));
    }
    for (int i = 0; i < 4000000; i++) {
        // exact and near-exact quotients: b times a short integer, nudged by an ulp
        const double b = ldexp(1.0 + (double)(xs() >> 12) / 4503599627370496.0, (int)(xs() % 40) - 20);
        const double q = (double)(xs() % 4096 + 1) / (double)(1u << (xs() % 12));
        const double a = b * q;
        pair(a, b);
        pair(bits(raw(a) + 1), b);
        pair(bits(raw(a) - 1), b);
        pair(a, bits(raw(b) + 1));
    }
    const uint64_t edge_exp[] = {0, 1, 2, 3, 896, 897, 1021, 1022, 1023, 1052, 1053, 1150, 1151, 2044, 2045, 2046, 2047};
    for (uint64_t ea : edge_exp)
        for (uint64_t eb : edge_exp)
            for (int k = 0; k < 20000; k++) {
                const uint64_t sa = (xs() & 1) << 63;
                const double a = bits(sa | (ea << 52) | (xs() & kF64Mant));
                const double b = bits(sa | (eb << 52) | (xs() & kF64Mant));
                pair(a, b);
                single(a);
            }
    const double sp[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, -NAN, 1.0, -1.0, 2.0, 0.5, -0.5, 1.5, -2.5,
                         4.9e-324, 2.2250738585072014e-308, 1073741823.5, -1073741823.5, 3.4028235677973366e38,
                         3.4028234663852886e38, 1.1754943508222875e-38, 1.1754942106924411e-38};
    for (double a : sp) {
        single(a);
        for (double b : sp) pair(a, b);
    }
    const Count *all[] = {&lerp, &eq, &lt, &scale, &rnd, &cvt, &add, &dv};
    bool ok = true;
    for (const Count *c : all) {
        c->report();
        ok &= c->wrong == 0 && c->taken > c->n / 4;
    }
    printf("%s\n", ok ? "wrong 0" : "FAILED");
    return ok ? 0 : 1;
}
