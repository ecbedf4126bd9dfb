// f64_int.cuh -- exact f64 operations on the integer pipes.
//
// GB300 executes f64 instructions at 1/64 of its f32 rate: one warp
// instruction occupies an SM's f64 pipe for 16 cycles, comparisons and
// conversions included.  The flattener and the edge builder must produce
// the reference's f64 results bit for bit, so the operations below give
// exactly the IEEE result (round to nearest even where rounding applies)
// from the operands' bit patterns.  Each one covers the operands that occur
// in drawing coordinates; the others report `done == false` (or are written
// so that they need no f64 instruction at all) and the caller takes the
// f64 instruction.  Everything here is host and device code, so that the
// same functions are checked against the host's f64 arithmetic.
#pragma once
#include <stdint.h>
#include <string.h>

// host and device in CUDA translation units, plain inline functions in the
// host-only C++ ones (the host stroke builder shares the stroke geometry)
#ifdef __CUDACC__
#define Z2D_F64 __host__ __device__ __forceinline__
#else
#define Z2D_F64 inline
#endif

namespace z2dg {

Z2D_F64 uint64_t f64_bits(double d) {
    uint64_t b;
    memcpy(&b, &d, 8);
    return b;
}
Z2D_F64 double f64_from(uint64_t b) {
    double d;
    memcpy(&d, &b, 8);
    return d;
}
Z2D_F64 int clz64(uint64_t v) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)v);
#else
    return __builtin_clzll(v);
#endif
}

constexpr uint64_t kF64Mant = (1ull << 52) - 1;
constexpr uint64_t kF64Abs = ~(1ull << 63);

Z2D_F64 bool f64_nan_bits(uint64_t A) { return (A << 1) > 0xFFE0000000000000ull; }

// a == b: equal bit patterns that are not NaN, or two zeros of any sign.
Z2D_F64 bool f64_eq(double a, double b) {
    const uint64_t A = f64_bits(a), B = f64_bits(b);
    return (A == B && !f64_nan_bits(A)) || ((A | B) << 1) == 0;
}

// a < b: false when either is NaN; -0 and +0 are equal.  Finite and
// infinite values compare through an order-preserving map of their bits.
Z2D_F64 bool f64_lt(double a, double b) {
    uint64_t A = f64_bits(a), B = f64_bits(b);
    if (f64_nan_bits(A) || f64_nan_bits(B)) return false;
    if ((A << 1) == 0) A = 0;
    if ((B << 1) == 0) B = 0;
    const uint64_t ka = A ^ ((uint64_t)((int64_t)A >> 63) | (1ull << 63));
    const uint64_t kb = B ^ ((uint64_t)((int64_t)B >> 63) | (1ull << 63));
    return ka < kb;
}
// a <= b, false when either is NaN
Z2D_F64 bool f64_le(double a, double b) { return f64_lt(a, b) || f64_eq(a, b); }
// |a|, by clearing the sign bit
Z2D_F64 double f64_abs(double a) { return f64_from(f64_bits(a) & kF64Abs); }

// x * s when s is a power of two and both x and the product are normal (or
// x is a zero): the exponent moves, the significand stays.
Z2D_F64 double f64_scale_pow2(double x, double s, bool &done) {
    const uint64_t X = f64_bits(x), S = f64_bits(s);
    const int32_t es = (int32_t)(S >> 52);  // sign bit clear for s > 0
    const int32_t ex = (int32_t)((X >> 52) & 0x7FF);
    done = false;
    if ((S & kF64Mant) != 0 || es < 1 || es > 2046) return 0.0;
    if ((X << 1) == 0) {
        done = true;
        return x;
    }
    const int32_t e = ex + es - 1023;
    if (ex < 1 || ex > 2046 || e < 1 || e > 2046) return 0.0;
    done = true;
    return f64_from(X + ((uint64_t)(int64_t)(es - 1023) << 52));
}

// (int32_t)round(x), half away from zero, for |x| < 2^30.
Z2D_F64 int32_t f64_round_i32(double x, bool &done) {
    const uint64_t X = f64_bits(x);
    const uint32_t e = (uint32_t)((X >> 52) & 0x7FF);
    done = e <= 1052;
    if (!done) return 0;
    if (e < 1022) return 0;  // |x| < 0.5
    const uint32_t sh = 1075 - e;  // 22..53
    const uint64_t m = (X & kF64Mant) | (1ull << 52);
    const int32_t r = (int32_t)((m + (1ull << (sh - 1))) >> sh);
    return (X >> 63) ? -r : r;
}

// (float)x, round to nearest even, when the result is a normal f32 or an
// overflow to infinity from a finite x, or x is a zero.
Z2D_F64 float f64_to_f32(double x, bool &done) {
    const uint64_t X = f64_bits(x);
    const uint32_t e = (uint32_t)((X >> 52) & 0x7FF);
    const uint32_t sign = (uint32_t)(X >> 32) & 0x80000000u;
    float out;
    if ((X << 1) == 0) {
        done = true;
        memcpy(&out, &sign, 4);
        return out;
    }
    done = e >= 897 && e <= 1150;  // f32 exponents 1..254
    if (!done) return 0.0f;
    const uint64_t m = X & kF64Mant;
    uint32_t r = (uint32_t)(m >> 29);
    const uint64_t rem = m & ((1ull << 29) - 1);
    r += (rem > (1ull << 28) || (rem == (1ull << 28) && (r & 1u))) ? 1u : 0u;
    const uint32_t F = sign | (((e - 896u) << 23) + r);  // a carry out of r raises the exponent (to inf at the top)
    memcpy(&out, &F, 4);
    return out;
}

// a + (b - a) / 2 as f64 arithmetic rounds it (lerpHalf, Spline.zig:158-165),
// when a and b have the same sign and the same biased exponent e in
// [2, 2045]: b - a is then exact (Sterbenz), so is its half, and the sum
// rounds once, so the result is (a + b) / 2 rounded to nearest even.  With
// m_a, m_b the 53-bit significands, S = m_a + m_b has 54 bits and the
// result keeps exponent e and significand S / 2 rounded to even: it cannot
// carry into the next binade.  Only this case is taken (and no operands in
// neighbouring binades, which the same argument would allow): the short
// form keeps the subdivision loops small in the instruction cache, which
// measured faster than taking more operand pairs with a longer form.
Z2D_F64 double lerp_half_int(double a, double b, bool &done) {
    const uint64_t A = f64_bits(a), B = f64_bits(b);
    const uint32_t e = (uint32_t)(A >> 52) & 0x7FFu;
    done = ((A ^ B) >> 52) == 0 && e - 2u <= 2043u;
    const uint64_t S = (A & kF64Mant) + (B & kF64Mant) + (1ull << 53);
    const uint64_t r = (S >> 1) + (S & (S >> 1) & 1);
    return f64_from((A & ~kF64Mant) | (r & kF64Mant));
}

// a + b, round to nearest even, for finite a and b (`done` false for an
// infinite or NaN operand).  The larger magnitude's significand and the
// smaller one's, aligned to it with ten extra low bits and a sticky bit,
// are added or subtracted; the sum is normalised (into the subnormal range
// where the exponent runs out) and rounded once.  Ten extra bits keep an
// alignment shift of one exact and give guard, round and sticky bits for
// longer shifts, which is what a single correct rounding needs.
Z2D_F64 double f64_add_int(double a, double b, bool &done) {
    uint64_t A = f64_bits(a), B = f64_bits(b);
    uint64_t aa = A & kF64Abs, ab = B & kF64Abs;
    done = aa < 0x7FF0000000000000ull && ab < 0x7FF0000000000000ull;
    if (!done) return 0.0;
    if (aa < ab) {
        const uint64_t t = A;
        A = B;
        B = t;
        const uint64_t u = aa;
        aa = ab;
        ab = u;
    }
    const uint64_t sign = A & ~kF64Abs;
    const bool sub = ((A ^ B) >> 63) != 0;
    if (ab == 0) {  // b is a zero: a, or for two zeros -0 only when both are
        if (aa == 0) return f64_from(A & B & ~kF64Abs);
        return f64_from(A);
    }
    int32_t ea = (int32_t)(aa >> 52), eb = (int32_t)(ab >> 52);
    uint64_t ma = aa & kF64Mant, mb = ab & kF64Mant;
    if (ea) ma |= 1ull << 52;
    else ea = 1;
    if (eb) mb |= 1ull << 52;
    else eb = 1;
    ma <<= 10;
    mb <<= 10;
    const int32_t d = ea - eb;
    if (d >= 63) mb = 1;  // only a sticky bit remains (mb is not zero)
    else if (d > 0) mb = (mb >> d) | ((mb << (64 - d)) != 0 ? 1u : 0u);
    uint64_t m = sub ? ma - mb : ma + mb;
    if (m == 0) return 0.0;  // exact cancellation: +0
    int32_t e = ea;
    const int lz = clz64(m);
    if (lz == 0) {  // carry out of bit 62
        m = (m >> 1) | (m & 1);
        e++;
    } else if (lz > 1) {  // cancellation: shift left, but not below the subnormal exponent
        int32_t sh = lz - 1;
        if (sh > e - 1) sh = e - 1;
        m <<= sh;
        e -= sh;
    }
    uint64_t r = m >> 10;
    const uint64_t rem = m & 1023u;
    r += (rem > 512u || (rem == 512u && (r & 1))) ? 1 : 0;
    if (r >> 53) {
        r >>= 1;
        e++;
    }
    if (e >= 2047) return f64_from(sign | 0x7FF0000000000000ull);
    const uint64_t field = (r >> 52) ? (uint64_t)e : 0;  // a significand below 2^52 only occurs at e == 1
    return f64_from(sign | (field << 52) | (r & kF64Mant));
}

// a / b, round to nearest even, for normal a and b whose quotient is normal,
// and for a zero a over a normal b (`done` false otherwise: a zero b,
// subnormals, infinities, NaNs, underflow and overflow).  Schoolbook long division of the significands in radix
// 2^11: with X = m_a (or 2 m_a, so that X / m_b lies in [1, 2)) the
// quotient's leading bit is 1 and R = X - m_b; each of five steps shifts
// the remainder by 11 bits (R < m_b < 2^53 keeps it below 2^64), estimates
// the digit floor(T / m_b) from the top bits of T and m_b with a 30-bit
// reciprocal of the divisor's top bits (off by at most one), and corrects
// the digit against the exact remainder.  The 56-bit quotient
// floor(X 2^55 / m_b) and the final remainder give the significand, the
// guard bits and the sticky bit of the single rounding.
Z2D_F64 double f64_div_int(double a, double b, bool &done) {
    const uint64_t A = f64_bits(a), B = f64_bits(b);
    const int32_t ea = (int32_t)((A >> 52) & 0x7FF), eb = (int32_t)((B >> 52) & 0x7FF);
    if ((A << 1) == 0 && eb >= 1 && eb <= 2046) {  // a zero over a normal b: a zero of the quotient's sign
        done = true;
        return f64_from((A ^ B) & ~kF64Abs);
    }
    done = ea >= 1 && ea <= 2046 && eb >= 1 && eb <= 2046;
    if (!done) return 0.0;
    const uint64_t ma = (A & kF64Mant) | (1ull << 52), mb = (B & kF64Mant) | (1ull << 52);
    const bool shift = ma < mb;
    int32_t e = ea - eb + (shift ? 1022 : 1023);
    done = e >= 1 && e <= 2046;
    if (!done) return 0.0;
    const uint64_t X = shift ? ma << 1 : ma;
    const uint32_t mh = (uint32_t)(mb >> 33);  // [2^19, 2^20)
    // 2^50 / mh within a relative 2^-21 (the digit estimate needs far less):
    // on the device the f32 reciprocal approximation of the special-function
    // unit (the correctly rounded reciprocal spends f64-pipe instructions)
#ifdef __CUDA_ARCH__
    float rcp;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rcp) : "f"((float)mh));
#else
    const float rcp = 1.0f / (float)mh;
#endif
    const uint32_t inv = (uint32_t)(rcp * 1125899906842624.0f);  // (2^30, 2^31]
    uint64_t R = X - mb, Q = 1;
#pragma unroll 1
    for (int i = 0; i < 5; i++) {
        const uint64_t T = R << 11;
        uint64_t d = ((uint64_t)(uint32_t)(T >> 33) * inv) >> 50;
        const uint64_t P = d * mb;
        if (P > T) {  // one too many (d >= 1, so P >= mb)
            d--;
            R = T - (P - mb);
        } else {
            R = T - P;
        }
        if (R >= mb) {
            d++;
            R -= mb;
        }
        Q = (Q << 11) | d;
    }
    uint64_t r = Q >> 3;  // 53 bits
    const uint32_t rest = (uint32_t)(Q & 7);
    r += (rest > 4 || (rest == 4 && (R != 0 || (r & 1)))) ? 1 : 0;
    if (r >> 53) {
        r >>= 1;
        e++;
    }
    const uint64_t sign = (A ^ B) & ~kF64Abs;
    if (e >= 2047) return f64_from(sign | 0x7FF0000000000000ull);
    return f64_from(sign | ((uint64_t)e << 52) | (r & kF64Mant));
}

#ifdef __CUDACC__
// The f64 instructions for the operands the integer forms decline, out of
// line: behind a call the compiler cannot evaluate them speculatively on
// every lane (a select between the two results would run the f64 form for
// all lanes and keep the f64 pipe as busy as before).
static __device__ __noinline__ double f64_add_hw(double a, double b) { return a + b; }
static __device__ __noinline__ double f64_mul_hw(double a, double b) { return a * b; }
static __device__ __noinline__ double f64_div_hw(double a, double b) { return a / b; }
static __device__ __noinline__ int32_t f64_round_i32_hw(double x) { return (int32_t)round(x); }
static __device__ __noinline__ float f64_to_f32_hw(double x) { return (float)x; }

// a / b through the integer long division (an f64 division is several f64
// instructions), out of line: one copy serves every call site.
static __device__ __noinline__ double f64_div_dev(double a, double b) {
    bool ok;
    const double r = f64_div_int(a, b, ok);
    if (ok) return r;
    return f64_div_hw(a, b);
}
#endif

}  // namespace z2dg
