// The f32 flatness tests of the curve subdivision (spline.cuh) against the
// f64 comparison errorSq < tol^2 they stand in for, on random knots whose
// control points lie near the tolerance from the chord, at coordinate
// magnitudes up to 2^15: every decision an f32 test takes must be the f64 one.
// Exit status 0 when no decision differs.
#include <cstdio>
#include <cstdint>
#include "spline.cuh"
using namespace z2dg;
__device__ uint64_t xs(uint64_t &s) { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; }
__device__ double ur(uint64_t &s) { return (double)(xs(s) >> 11) * (1.0 / 9007199254740992.0); }
__global__ void k(unsigned long long *out, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t s = 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1);
    unsigned long long bad = 0, dec = 0, bad_old = 0;
    for (int it = 0; it < 64; it++) {
        const double mag = ldexp(1.0, (int)(xs(s) % 16));           // coordinate magnitude up to 2^15
        const double tol = (it & 1) ? 0.1 : ldexp(1.0, -(int)(xs(s) % 6));
        const Tol t = make_tol(tol);
        const double len = ldexp(ur(s) + 0.01, -(int)(xs(s) % 10)) * 64;  // chord length
        const double ax = (ur(s) * 2 - 1) * mag, ay = (ur(s) * 2 - 1) * mag;
        const double ang = ur(s) * 6.283185307179586;
        const double dx = ax + len * cos(ang), dy = ay + len * sin(ang);
        // control points at distance near tol from the chord
        const double nx = -sin(ang), ny = cos(ang);
        const double db = tol * (0.9 + 0.2 * ur(s)) * ((xs(s) & 1) ? 1 : -1);
        const double dc = tol * ur(s) * ((xs(s) & 1) ? 1 : -1);
        const double fb = ur(s) * 1.4 - 0.2, fc = ur(s) * 1.4 - 0.2;
        Knots kn{ax, ay, ax + (dx - ax) * fb + nx * db, ay + (dy - ay) * fb + ny * db,
                 ax + (dx - ax) * fc + nx * dc, ay + (dy - ay) * fc + ny * dc, (it % 7 == 0) ? ax : dx, (it % 7 == 0) ? ay : dy};
        const bool truth = error_sq(kn) < t.d;
        const bool proj = kn.ax != kn.dx || kn.ay != kn.dy;
        if (t.f_ok) {
            const int r = error_sq_lt_f32_pts(kn.ax, kn.ay, kn.bx, kn.by, kn.cx, kn.cy, kn.dx, kn.dy, proj, t.f, t.e);
            if (r >= 0) { dec++; if ((r != 0) != truth) bad++; }
            const int r2 = error_sq_lt_f32(kn.bx - kn.ax, kn.by - kn.ay, kn.cx - kn.ax, kn.cy - kn.ay, proj, kn.dx - kn.ax, kn.dy - kn.ay, t.f, t.e);
            if (r2 >= 0 && (r2 != 0) != truth) bad_old++;
        }
    }
    atomicAdd(&out[0], bad); atomicAdd(&out[1], dec); atomicAdd(&out[2], bad_old);
}
int main() {
    unsigned long long *d, h[3] = {0, 0, 0};
    cudaMalloc(&d, 3 * sizeof(unsigned long long));
    cudaMemset(d, 0, 3 * sizeof(unsigned long long));
    const int n = 1 << 20;
    k<<<n / 256, 256>>>(d, n);
    cudaError_t e = cudaDeviceSynchronize();
    cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    printf("status %s  cases %d  decided %llu  wrong(pts) %llu  wrong(diff) %llu\n", cudaGetErrorString(e), n * 64, h[1], h[0], h[2]);
    return (e == cudaSuccess && h[0] == 0 && h[2] == 0) ? 0 : 1;
}
