// Output stage: the image a pass writes (ppm_probabilistic.cc:96-106) from
// the accumulation buffer, optionally tone mapped (Image::tonemap,
// image.cc:498-524), and a PNG encoder for the bytes. The reference keeps
// its buffer in double; the bytes here are formed in double from the FP32
// accumulator.
#include <cmath>
#include <cstring>
#include <vector>

#include "context.h"

namespace pppm {

namespace {

// Image::toByte (image.cc:530-533): std::max(0.0, std::min(d, 1.0)) (NaN
// gives 0), times 255, truncated
__device__ __forceinline__ unsigned char toByte(double d) {
    const double m = (1.0 < d) ? 1.0 : d;
    const double v = (0.0 < m) ? m : 0.0;
    return (unsigned char)__dmul_rn(255.0, v);
}

// Vector3D::dot(c, (0.2126, 0.7152, 0.0722)), rounded step by step
__device__ __forceinline__ double lum(double r, double g, double b) {
    return __dadd_rn(__dadd_rn(__dmul_rn(r, 0.2126), __dmul_rn(g, 0.7152)), __dmul_rn(b, 0.0722));
}

// Reinhard statistics of buffer / t: sum of log(l + 1e-8) and max l, with
// l = 0.2126 r + 0.7152 g + 0.0722 b (in double, per block, then atomics on
// the ordered bits of the max and a double add of the sums).
__global__ void kTonemapStats(const float* __restrict__ acc, int64_t n, double invT, double* sumLog,
                              unsigned long long* maxBits) {
    double s = 0.0, m = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double l = lum(__dmul_rn(acc[3 * i], invT), __dmul_rn(acc[3 * i + 1], invT), __dmul_rn(acc[3 * i + 2], invT));
        s += log(__dadd_rn(l, 1.0e-8));
        m = fmax(m, l);
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(sumLog, s);
        // l >= 0: the bits of a non-negative double order like the value
        atomicMax(maxBits, (unsigned long long)__double_as_longlong(m));
    }
}

// One pixel of the output: result(x, H - 1 - y) = buffer(x, y) / t,
// optionally tone mapped, then gamma(2.2, inverse) and toByte.
__global__ void kImage(const float* __restrict__ acc, int w, int h, double invT, int tonemap, const double* sumLog,
                       const unsigned long long* maxBits, unsigned char* __restrict__ out) {
    const int64_t n = (int64_t)w * h;
    double a = 0.0, lwBar = 1.0, lWhite2 = 1.0;
    if (tonemap) {
        a = 0.18;
        lwBar = exp(__ddiv_rn(*sumLog, (double)n));
        const double lw = __longlong_as_double((long long)*maxBits);
        lWhite2 = __dmul_rn(lw, lw);
    }
    const double gg = 1.0 / 2.2;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t x = i % w, y = i / w;
        // Vector3D / t multiplies by 1 / t
        double c[3] = {__dmul_rn(acc[3 * i], invT), __dmul_rn(acc[3 * i + 1], invT), __dmul_rn(acc[3 * i + 2], invT)};
        if (tonemap) {
            // ret = c * a / lw_bar; ret = ret * (1 + ret / l_white^2) / (1 + ret)
            for (int k = 0; k < 3; k++) {
                const double r = __ddiv_rn(__dmul_rn(c[k], a), lwBar);
                c[k] = __ddiv_rn(__dmul_rn(r, __dadd_rn(1.0, __ddiv_rn(r, lWhite2))), __dadd_rn(1.0, r));
            }
        }
        unsigned char* o = out + 3 * ((h - 1 - y) * (int64_t)w + x);
        for (int k = 0; k < 3; k++) o[k] = toByte(pow(c[k], gg));
    }
}

// CRC-32 of PNG chunks (ISO 3309 polynomial, reflected)
struct CrcTable {
    uint32_t t[256];
    CrcTable() {
        for (uint32_t n = 0; n < 256; n++) {
            uint32_t c = n;
            for (int k = 0; k < 8; k++) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[n] = c;
        }
    }
};

uint32_t crc32(const uint8_t* p, size_t n) {
    static const CrcTable tab;
    uint32_t c = 0xFFFFFFFFu;
    for (size_t i = 0; i < n; i++) c = tab.t[(c ^ p[i]) & 0xFF] ^ (c >> 8);
    return c ^ 0xFFFFFFFFu;
}

}  // namespace

}  // namespace pppm

using namespace pppm;

extern "C" {

// The output bytes of a device accumulator acc (w*h*3 floats) after
// `passes` passes into rgb8 (host or device).
static int imageBytes(pppm_ctx* c, const float* acc, int w, int h, int passes, int32_t tonemap, uint8_t* rgb8) {
    const int64_t n = (int64_t)w * h;
    void* dout;
    int r;
    if ((r = stageOut(c, rgb8, (size_t)n * 3, 0, &dout))) return r;
    const double invT = 1.0 / (double)passes;
    PPPM_CUDA(c, c->stageCount.ensure(16));
    double* sumLog = c->stageCount.as<double>();
    unsigned long long* maxBits = reinterpret_cast<unsigned long long*>(sumLog + 1);
    if (tonemap) {
        PPPM_CUDA(c, cudaMemsetAsync(sumLog, 0, 16, c->stream));
        kTonemapStats<<<152 * 4, 256, 0, c->stream>>>(acc, n, invT, sumLog, maxBits);
    }
    kImage<<<152 * 8, 256, 0, c->stream>>>(acc, w, h, invT, tonemap ? 1 : 0, sumLog, maxBits,
                                           static_cast<unsigned char*>(dout));
    PPPM_CUDA(c, cudaGetLastError());
    if ((r = finishOut(c, rgb8, dout, (size_t)n * 3))) return r;
    PPPM_CUDA(c, cudaStreamSynchronize(c->stream));
    return PPPM_OK;
}

int pppm_render_image(pppm_ctx* c, int32_t tonemap, uint8_t* rgb8) {
    if (!c || !rgb8) return fail(c, PPPM_E_ARG, "render_image: bad arguments");
    const RenderState& rs = c->rs;
    if (!rs.active || rs.passesDone < 1) return fail(c, PPPM_E_STATE, "render_image: no pass rendered");
    cudaSetDevice(c->device);
    return imageBytes(c, rs.accum.as<float>(), rs.cam.width, rs.cam.height, rs.passesDone, tonemap, rgb8);
}

int pppm_image_bytes(pppm_ctx* c, const float* accum, int32_t w, int32_t h, int32_t passes, int32_t tonemap,
                     uint8_t* rgb8) {
    if (!c || !accum || !rgb8 || w < 1 || h < 1 || passes < 1) return fail(c, PPPM_E_ARG, "image_bytes: bad arguments");
    cudaSetDevice(c->device);
    const void* dacc;
    int r;
    // staging slot 1: imageBytes writes through slot 0
    if ((r = stageIn(c, accum, (size_t)w * h * 12, 1, &dacc))) return r;
    return imageBytes(c, static_cast<const float*>(dacc), w, h, passes, tonemap, rgb8);
}

int pppm_png_encode(const uint8_t* rgb8, int32_t w, int32_t h, uint8_t* out, int64_t cap, int64_t* size) {
    if (!rgb8 || w < 1 || h < 1 || !size || (cap > 0 && !out) || (int64_t)w * 3 + 1 > 65535) return PPPM_E_ARG;
    // zlib stream of stored deflate blocks: one block per row (filter 0 + row)
    const int64_t row = (int64_t)w * 3 + 1;
    const int64_t idat = 2 + (int64_t)h * (5 + row) + 4;
    const int64_t total = 8 + (12 + 13) + (12 + idat) + 12;
    *size = total;
    if (!out) return PPPM_OK;
    if (cap < total) return PPPM_E_CAPACITY;
    uint8_t* p = out;
    auto put32 = [&](uint32_t v) {
        p[0] = (uint8_t)(v >> 24); p[1] = (uint8_t)(v >> 16); p[2] = (uint8_t)(v >> 8); p[3] = (uint8_t)v;
        p += 4;
    };
    auto chunk = [&](const char* type, int64_t len, auto&& body) {
        put32((uint32_t)len);
        uint8_t* start = p;
        std::memcpy(p, type, 4);
        p += 4;
        body();
        const uint32_t crc = crc32(start, (size_t)(p - start));
        put32(crc);
    };
    static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    std::memcpy(p, sig, 8);
    p += 8;
    chunk("IHDR", 13, [&]() {
        put32((uint32_t)w);
        put32((uint32_t)h);
        *p++ = 8;  // bit depth
        *p++ = 2;  // RGB
        *p++ = 0;  // deflate
        *p++ = 0;  // filter method
        *p++ = 0;  // no interlace
    });
    chunk("IDAT", idat, [&]() {
        *p++ = 0x78;  // zlib: deflate, 32K window
        *p++ = 0x01;  // no dictionary, fastest; (0x78 << 8 | 0x01) % 31 == 0
        uint32_t a = 1, b = 0;  // Adler-32
        for (int y = 0; y < h; y++) {
            *p++ = (uint8_t)(y == h - 1 ? 1 : 0);  // stored block, final on the last row
            const uint16_t len = (uint16_t)row, nlen = (uint16_t)~len;
            *p++ = (uint8_t)(len & 0xFF); *p++ = (uint8_t)(len >> 8);
            *p++ = (uint8_t)(nlen & 0xFF); *p++ = (uint8_t)(nlen >> 8);
            *p++ = 0;  // filter type None
            std::memcpy(p, rgb8 + (int64_t)y * w * 3, (size_t)w * 3);
            const uint8_t* rp = p - 1;
            for (int64_t i = 0; i < row; i++) {
                a = (a + rp[i]) % 65521u;
                b = (b + a) % 65521u;
            }
            p += (int64_t)w * 3;
        }
        put32((b << 16) | a);
    });
    chunk("IEND", 0, [&]() {});
    return PPPM_OK;
}

}  // extern "C"
