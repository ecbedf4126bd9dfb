// The integer forms of f64 operations (f64_int.cuh) as the device compiles
// them, against the device's own f64 instructions: every thread draws
// operand pairs of the kinds the host check uses (random bit patterns, same
// and neighbouring binades, a few ulps apart, opposite signs, drawing
// coordinates, nearly exact quotients) and counts the results that differ
// from a + (b - a) / 2, a / b, ==, <, <=, x * 2^k, (int32_t)round(x) and
// (float)x.  Built with --fmad=false (no contraction of the reference
// expressions).  Exit status 0 when no result differs.
#include <cstdint>
#include <cstdio>

#include "f64_int.cuh"
using namespace z2dg;

__device__ uint64_t xs(uint64_t &s) {
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    return s;
}

__device__ unsigned long long g_count[4];  // [0] wrong, [1] integer results checked, [2] cases, [3] divisions taken

__device__ void check_pair(double a, double b, unsigned long long &wrong, unsigned long long &taken,
                           unsigned long long &divs) {
    bool done;
    const double m = lerp_half_int(a, b, done);
    if (done) {
        taken++;
        const double h = (b - a) * 0.5;
        if (f64_bits(m) != f64_bits(a + h)) wrong++;
    }
    const double q = f64_div_int(a, b, done);
    if (done) {
        taken++;
        divs++;
        if (f64_bits(q) != f64_bits(a / b)) wrong++;
    }
    taken += 3;
    if (f64_eq(a, b) != (a == b) || f64_lt(a, b) != (a < b) || f64_le(a, b) != (a <= b)) wrong++;
}

__device__ void check_single(double x, unsigned long long &wrong, unsigned long long &taken) {
    bool done;
    const double s4 = f64_scale_pow2(x, 4.0, done);
    if (done) {
        taken++;
        if (f64_bits(s4) != f64_bits(x * 4.0)) wrong++;
    }
    const int32_t r = f64_round_i32(x, done);
    if (done) {
        taken++;
        if (r != (int32_t)round(x)) wrong++;
    }
    const float f = f64_to_f32(x, done);
    if (done) {
        taken++;
        if (__float_as_uint(f) != __float_as_uint(__double2float_rn(x))) wrong++;
    }
}

__global__ void k_check(int iters) {
    uint64_t s = 0x9E3779B97F4A7C15ull * (uint64_t)(blockIdx.x * blockDim.x + threadIdx.x + 1);
    unsigned long long wrong = 0, taken = 0, divs = 0, cases = 0;
    for (int i = 0; i < iters; i++) {
        const uint64_t A = xs(s);
        const int kind = (int)(xs(s) % 7);
        uint64_t B;
        if (kind == 0) B = xs(s);
        else if (kind == 1) B = (A & ~kF64Mant) | (xs(s) & kF64Mant);
        else if (kind == 2) B = A + (xs(s) % 64) - 32;
        else if (kind == 3) B = (A + (1ull << 52)) ^ (xs(s) & kF64Mant);
        else if (kind == 4) B = A ^ (1ull << 63);
        else if (kind == 5) B = (A & (1ull << 63)) | ((uint64_t)(xs(s) % 6) << 52) | (xs(s) & kF64Mant);
        else B = (A - (1ull << 52)) ^ (xs(s) & kF64Mant);
        check_pair(f64_from(A), f64_from(B), wrong, taken, divs);
        check_pair(f64_from(B), f64_from(A), wrong, taken, divs);
        check_single(f64_from(A), wrong, taken);
        // drawing coordinates and nearly exact quotients
        const double c = ((double)(xs(s) >> 11) * (1.0 / 9007199254740992.0) - 0.25) * 8192.0;
        const double d = c + ((double)(xs(s) >> 11) * (1.0 / 9007199254740992.0) - 0.5) * ldexp(1.0, -(int)(xs(s) % 40));
        check_pair(c, d, wrong, taken, divs);
        check_single(c, wrong, taken);
        check_single(floor(c) + 0.5, wrong, taken);
        const double qb = ldexp(1.0 + (double)(xs(s) >> 12) * (1.0 / 4503599627370496.0), (int)(xs(s) % 40) - 20);
        const double qa = qb * (double)(xs(s) % 4096 + 1);
        check_pair(qa, qb, wrong, taken, divs);
        check_pair(f64_from(f64_bits(qa) + 1), qb, wrong, taken, divs);
        cases += 7;
    }
    atomicAdd(&g_count[0], wrong);
    atomicAdd(&g_count[1], taken);
    atomicAdd(&g_count[2], cases);
    atomicAdd(&g_count[3], divs);
}

int main() {
    k_check<<<152 * 4, 256>>>(64);
    const cudaError_t e = cudaDeviceSynchronize();
    unsigned long long h[4] = {0, 0, 0, 0};
    cudaMemcpyFromSymbol(h, g_count, sizeof(h));
    printf("status %s  cases %llu  integer results %llu  divisions %llu  wrong %llu\n", cudaGetErrorString(e), h[2],
           h[1], h[3], h[0]);
    return (e == cudaSuccess && h[0] == 0 && h[3] > 0) ? 0 : 1;
}
