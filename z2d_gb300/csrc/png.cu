// png.cu -- the PNG exporter (src/export_png.zig) with the pixel encoding
// on the device.
//
// writeToPNGFile writes the signature, IHDR, an optional gAMA chunk, the
// zlib-compressed scanlines in IDAT chunks and IEND.  The scanlines use no
// filtering: each row is a 0 byte followed by the row's pixels as
// writePNGIDATStream encodes them (export_png.zig:153-311):
//   RGBA / ARGB  R, G, B, A bytes, demultiplied (RGBA16.demultiply)
//   RGB / XRGB   R, G, B bytes
//   alpha8       the alpha byte
//   alpha4/2/1   packed most significant bits first within each byte
// with, for the sRGB profile, the channels taken through the sRGB gamma
// (encodeRGBAVec, export_png.zig:319-372).  k_png_rows writes that stream
// from the surface in HBM (one thread per pixel, or per output byte for the
// packed formats); the host compresses it (zlib at its default level when
// the library is available, stored deflate blocks otherwise) and writes the
// chunks with their CRC-32.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#ifdef Z2D_HAVE_ZLIB
#include <zlib.h>
#endif

#include "raster_px.cuh"
#include "z2d_internal.h"

namespace z2dg {

namespace {

// decodeRGBAVecRaw (x / 255 in f32), applyGammaVec (pow(x, 1 / 2.2) for the
// colour channels), encodeRGBAVecRaw (round(255 x)) (color_vector.zig:210-284)
__device__ __forceinline__ uint32_t srgb_encode(uint32_t c, bool gamma) {
    float v = (float)c / 255.0f;
    if (gamma) v = zpow(v, Z2D_INV_GAMMA);
    return (uint32_t)roundf(255.0f * v);
}

__global__ void k_png_rows(DevSurface s, int srgb, uint8_t *__restrict__ out, long long row_bytes,
                           long long units_per_row, long long n_units) {
    const long long u = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= n_units) return;
    long long y, k;
    if (n_units <= 0xFFFFFFFFll) {  // 32-bit division where it is enough
        const uint32_t uu = (uint32_t)u, up = (uint32_t)units_per_row;
        y = uu / up;
        k = uu - (uint32_t)y * up;
    } else {
        y = u / units_per_row;
        k = u - y * units_per_row;
    }
    uint8_t *row = out + y * row_bytes;
    if (k == 0) row[0] = 0;  // filter type: none
    const int fmt = s.fmt;
    if (fmt <= Z2D_FORMAT_RGBA) {
        const uint32_t w = reinterpret_cast<const uint32_t *>(s.data)[(size_t)y * s.w + k];
        const I16 p = word_to_i16(w, fmt);
        uint32_t r = p.r, g = p.g, b = p.b, a = p.a;
        const bool has_alpha = fmt == Z2D_FORMAT_RGBA || fmt == Z2D_FORMAT_ARGB;
        if (has_alpha) {  // RGBA16.demultiply (pixel_vector.zig:27-60)
            // x / a as umulhi(x, ceil(2^32 / a)): exact for x <= 255 * 255
            // (the error x / 2^32 stays below 1 / a)
            const uint32_t m = a > 1u ? 0xFFFFFFFFu / a + 1u : 0u;
            r = a == 0 ? 0 : (a == 1 ? r * 255u : __umulhi(r * 255u, m));
            g = a == 0 ? 0 : (a == 1 ? g * 255u : __umulhi(g * 255u, m));
            b = a == 0 ? 0 : (a == 1 ? b * 255u : __umulhi(b * 255u, m));
        } else {
            a = 255;
        }
        if (srgb) {
            r = srgb_encode(r, true);
            g = srgb_encode(g, true);
            b = srgb_encode(b, true);
            a = srgb_encode(a, false);
        }
        uint8_t *o = row + 1 + k * (has_alpha ? 4 : 3);
        o[0] = (uint8_t)r;
        o[1] = (uint8_t)g;
        o[2] = (uint8_t)b;
        if (has_alpha) o[3] = (uint8_t)a;
    } else if (fmt == Z2D_FORMAT_ALPHA8) {
        row[1 + k] = s.data[(size_t)y * s.w + k];
    } else {  // one output byte: 8 / bits pixels, the first in the high bits
        const int bits = fmt_bits(fmt), per = 8 / bits;
        uint32_t v = 0;
        for (int i = 0; i < per; i++) {
            const long long x = k * per + i;
            if (x >= s.w) break;
            v |= load_raw(s, (size_t)(y * s.w + x)) << (8 - bits - i * bits);
        }
        row[1 + k] = (uint8_t)v;
    }
}

// CRC-32 of PNG chunks (ISO 3309 / ITU-T V.42 polynomial, reflected)
struct Crc32 {
    uint32_t t[256];
    Crc32() {
        for (uint32_t n = 0; n < 256; n++) {
            uint32_t c = n;
            for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[n] = c;
        }
    }
    uint32_t update(uint32_t crc, const uint8_t *p, size_t n) const {
        uint32_t c = crc ^ 0xFFFFFFFFu;
        for (size_t i = 0; i < n; i++) c = t[(c ^ p[i]) & 0xFF] ^ (c >> 8);
        return c ^ 0xFFFFFFFFu;
    }
};
const Crc32 &crc_table() {
    static const Crc32 t;
    return t;
}

void put32(std::vector<uint8_t> &o, uint32_t v) {
    o.push_back((uint8_t)(v >> 24));
    o.push_back((uint8_t)(v >> 16));
    o.push_back((uint8_t)(v >> 8));
    o.push_back((uint8_t)v);
}

// writePNGWriteChunk (export_png.zig:391-412)
void chunk(std::vector<uint8_t> &o, const char type[4], const uint8_t *data, size_t n) {
    put32(o, (uint32_t)n);
    const size_t at = o.size();
    o.insert(o.end(), type, type + 4);
    if (n) o.insert(o.end(), data, data + n);
    put32(o, crc_table().update(0, o.data() + at, n + 4));
}

// A zlib stream of `raw` (RFC 1950/1951): zlib's default compression level
// when the library was found at build time (pieces compressed on all host
// threads), stored blocks otherwise.
bool zlib_stream(const uint8_t *raw, size_t n, std::vector<uint8_t> &out) {
#ifdef Z2D_HAVE_ZLIB
    // Pieces of the data are deflated in parallel, each a raw deflate stream
    // ending on a byte boundary (a sync flush; the last piece finishes the
    // stream), so that their concatenation is one valid deflate stream.
    const size_t nt = std::max(1u, std::thread::hardware_concurrency());
    const size_t piece = std::max<size_t>((size_t)1 << 20, (n + nt - 1) / nt);
    const size_t n_pieces = std::max<size_t>(1, (n + piece - 1) / piece);
    std::vector<std::vector<uint8_t>> parts(n_pieces);
    std::vector<int> ok(n_pieces, 0);
    std::atomic<size_t> next{0};
    auto work = [&] {
        for (size_t k; (k = next.fetch_add(1)) < n_pieces;) {
            const size_t a = k * piece, m = std::min(piece, n - a);
            z_stream z;
            memset(&z, 0, sizeof(z));
            if (deflateInit2(&z, Z_DEFAULT_COMPRESSION, Z_DEFLATED, -15, 8, Z_DEFAULT_STRATEGY) != Z_OK) continue;
            std::vector<uint8_t> &o = parts[k];
            o.resize(deflateBound(&z, (uLong)m) + 16);
            z.next_in = const_cast<Bytef *>(raw + a);
            z.avail_in = (uInt)m;
            z.next_out = o.data();
            z.avail_out = (uInt)o.size();
            const int r = deflate(&z, k + 1 == n_pieces ? Z_FINISH : Z_SYNC_FLUSH);
            ok[k] = (k + 1 == n_pieces ? r == Z_STREAM_END : r == Z_OK) && z.avail_in == 0;
            o.resize(o.size() - z.avail_out);
            deflateEnd(&z);
        }
    };
    std::vector<std::thread> pool;
    for (size_t t = 1; t < std::min(nt, n_pieces); t++) pool.emplace_back(work);
    work();
    for (auto &t : pool) t.join();
    out.clear();
    out.push_back(0x78);  // zlib header: deflate, 32 KiB window, default level
    out.push_back(0x9C);
    for (size_t k = 0; k < n_pieces; k++) {
        if (!ok[k]) return false;
        out.insert(out.end(), parts[k].begin(), parts[k].end());
    }
    uLong ad = adler32(0L, Z_NULL, 0);
    for (size_t i = 0; i < n; i += (size_t)1 << 30) ad = adler32(ad, raw + i, (uInt)std::min(n - i, (size_t)1 << 30));
    put32(out, (uint32_t)ad);
    return true;
#else
    out.clear();
    out.push_back(0x78);
    out.push_back(0x01);
    size_t i = 0;
    do {
        const size_t m = std::min<size_t>(65535, n - i);
        out.push_back(i + m == n ? 1 : 0);  // BFINAL, BTYPE 00
        out.push_back((uint8_t)m);
        out.push_back((uint8_t)(m >> 8));
        out.push_back((uint8_t)~m);
        out.push_back((uint8_t)(~m >> 8));
        out.insert(out.end(), raw + i, raw + i + m);
        i += m;
    } while (i < n);
    uint32_t a = 1, b = 0;  // Adler-32
    for (size_t k = 0; k < n; k++) {
        a = (a + raw[k]) % 65521u;
        b = (b + a) % 65521u;
    }
    put32(out, (b << 16) | a);
    return true;
#endif
}

}  // namespace

int png_scanlines(Ctx &c, const DevSurface &s, int profile, std::vector<uint8_t> &raw) {
    const int fmt = s.fmt;
    const int bits = fmt <= Z2D_FORMAT_RGBA ? ((fmt == Z2D_FORMAT_RGBA || fmt == Z2D_FORMAT_ARGB) ? 32 : 24)
                                              : fmt_bits(fmt);
    const long long row_bytes = 1 + ((long long)s.w * bits + 7) / 8;
    const long long units = fmt <= Z2D_FORMAT_ALPHA8 ? s.w : row_bytes - 1;
    const size_t total = (size_t)(row_bytes * s.h);
    if (c.surface2.ensure(total + 16)) return Z2D_ERR_OUT_OF_MEMORY;
    uint8_t *d = c.surface2.as<uint8_t>();
    const long long n_units = units * s.h;
    if (n_units > 0) {
        cudaEvent_t te = c.timer_begin(c.t_export);
        k_png_rows<<<(unsigned)((n_units + 255) / 256), 256, 0, c.stream>>>(s, profile == Z2D_PROFILE_SRGB ? 1 : 0, d,
                                                                          row_bytes, units, n_units);
        c.timer_end(c.t_export, te);
        c.launches++;
    }
    raw.resize(total);
    Z2D_CUDA(cudaMemcpyAsync(raw.data(), d, total, cudaMemcpyDeviceToHost, c.stream));
    Z2D_CUDA(cudaStreamSynchronize(c.stream));
    return Z2D_OK;
}

int png_file(Ctx &c, const DevSurface &s, int profile, std::vector<uint8_t> &png) {
    std::vector<uint8_t> raw;
    int rc = png_scanlines(c, s, profile, raw);
    if (rc) return rc;
    png.clear();
    static const uint8_t magic[8] = {0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    png.insert(png.end(), magic, magic + 8);
    // IHDR (export_png.zig:97-131)
    const int fmt = s.fmt;
    const uint8_t depth = fmt <= Z2D_FORMAT_ALPHA8 ? 8 : (uint8_t)fmt_bits(fmt);
    const uint8_t ctype = (fmt == Z2D_FORMAT_RGBA || fmt == Z2D_FORMAT_ARGB) ? 6
                          : (fmt == Z2D_FORMAT_RGB || fmt == Z2D_FORMAT_XRGB) ? 2
                                                                              : 0;
    std::vector<uint8_t> ihdr;
    put32(ihdr, (uint32_t)s.w);
    put32(ihdr, (uint32_t)s.h);
    ihdr.push_back(depth);
    ihdr.push_back(ctype);
    ihdr.push_back(0);  // compression
    ihdr.push_back(0);  // filter
    ihdr.push_back(0);  // interlace
    chunk(png, "IHDR", ihdr.data(), ihdr.size());
    if (profile == Z2D_PROFILE_LINEAR || profile == Z2D_PROFILE_SRGB) {  // gAMA (export_png.zig:133-147)
        const float g = profile == Z2D_PROFILE_SRGB ? 1.0f / 2.2f : 1.0f / 1.0f;
        std::vector<uint8_t> gb;
        put32(gb, (uint32_t)(g * 100000.0f));
        chunk(png, "gAMA", gb.data(), gb.size());
    }
    std::vector<uint8_t> z;
    if (!zlib_stream(raw.data(), raw.size(), z)) return Z2D_ERR_OUT_OF_MEMORY;
    for (size_t i = 0; i < z.size(); i += (size_t)1 << 20)  // IDAT chunks of up to 1 MiB
        chunk(png, "IDAT", z.data() + i, std::min<size_t>((size_t)1 << 20, z.size() - i));
    chunk(png, "IEND", nullptr, 0);
    return Z2D_OK;
}

}  // namespace z2dg
