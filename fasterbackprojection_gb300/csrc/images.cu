// Transient images: the output step of the depth-plane reconstruction
// (Laser::reconstructDepthConfocal / Exhaustive, Laser.cu:409-424, 461-476)
// and the capture export NLosData::saveImages (NLosData.cpp:161-180).
//
// The reference downloads the [L][D] activation and, per depth d, builds a
// TransientImage: grey RGBA8 pixels clamp(uint(v * 255), 0, 255) from
// slice[d + idx * D] (TransientImage.cpp:46-57), rows flipped
// (Image.h:160-178), a bilinear resize to the output size (Image.h:45-66,
// 92-138), then a PNG file per plane (SOIL2).  Here one kernel makes every
// plane's final pixels on the device, in the reference's FP32 expression order
// (no contraction), and the host only encodes the PNG files.  Pixel idx of
// plane p is data[p * plane_stride + idx * pixel_stride]: (1, D) for the depth
// planes of an [L][D] activation, (W * H, 1) for contiguous slices.
//
// normalize != 0 divides each plane by its own maximum (at least 0) first.
// The reference's normalizeImage divides the first width x height floats of
// the buffer (TransientImage.cpp:66-78), which is the plane itself only for
// stride 1 and offset 0 (saveImages' case); the depth path passes false.
// A value whose v * 255 is negative or NaN becomes 0 (the reference's
// float-to-unsigned conversion is undefined there).
#include "fbp_internal.cuh"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

namespace fbp {
namespace {

// Per-plane maximum of max(0, v) as the bits of a non-negative float.
__global__ void plane_max_kernel(const float* __restrict__ act, uint32_t npix, uint64_t pixel_stride,
                                 uint64_t plane_stride, unsigned int* __restrict__ maxbits) {
    const uint32_t d = blockIdx.y;
    float m = 0.f;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < npix; i += gridDim.x * blockDim.x)
        m = fmaxf(m, act[d * plane_stride + i * pixel_stride]);
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(maxbits + d, __float_as_uint(m));
}

struct ImageGeom {
    uint32_t w, h;         // source plane (w x h pixels)
    uint64_t pixel_stride, plane_stride;
    uint32_t ow, oh;       // output size
    float xr, yr;          // (w - 1) / (ow - 1), (h - 1) / (oh - 1) when resizing
    int normalize;
};

// TransientImage.cpp:55 for pixel (x, row) of the flipped plane.
__device__ __forceinline__ float grey(const float* __restrict__ act, const ImageGeom& g, uint32_t d, float inv_src,
                                      uint32_t x, uint32_t row) {
    const uint32_t idx = (g.h - 1 - row) * g.w + x;  // Image.h:160-178: row r of the flipped image
    float v = act[d * g.plane_stride + idx * g.pixel_stride];
    if (g.normalize) v = __fdiv_rn(v, inv_src);
    return (float)min(__float2uint_rz(__fmul_rn(v, 255.0f)), 255u);
}

// Image.h:45-66 for one channel value of the four corners.
__device__ __forceinline__ float bilinear(float dx, float dy, float p00, float p01, float p10, float p11) {
    const float ex = __fsub_rn(1.0f, dx), ey = __fsub_rn(1.0f, dy);
    float s = __fmul_rn(__fmul_rn(ex, ey), p00);
    s = __fadd_rn(s, __fmul_rn(__fmul_rn(dx, ey), p01));
    s = __fadd_rn(s, __fmul_rn(__fmul_rn(ex, dy), p10));
    return __fadd_rn(s, __fmul_rn(__fmul_rn(dx, dy), p11));
}

template <bool RESIZE>
__global__ void __launch_bounds__(256) plane_image_kernel(const float* __restrict__ act, ImageGeom g,
                                                          const unsigned int* __restrict__ maxbits,
                                                          uchar4* __restrict__ out) {
    const uint32_t d = blockIdx.y;
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= g.ow * g.oh) return;
    const uint32_t x = p % g.ow, y = p / g.ow;
    const float mx = g.normalize ? __uint_as_float(maxbits[d]) : 1.f;
    uchar4 px;
    if (!RESIZE) {
        const unsigned char c = (unsigned char)grey(act, g, d, mx, x, y);
        px = make_uchar4(c, c, c, 255);
    } else {
        const float xs = __fmul_rn((float)x, g.xr), ys = __fmul_rn((float)y, g.yr);
        const uint32_t x0 = min((uint32_t)__float2int_rz(xs), g.w - 1), y0 = min((uint32_t)__float2int_rz(ys), g.h - 1);
        const uint32_t x1 = min(x0 + 1, g.w - 1), y1 = min(y0 + 1, g.h - 1);
        const float dx = __fsub_rn(xs, (float)x0), dy = __fsub_rn(ys, (float)y0);
        const float c = bilinear(dx, dy, grey(act, g, d, mx, x0, y0), grey(act, g, d, mx, x1, y0),
                                 grey(act, g, d, mx, x0, y1), grey(act, g, d, mx, x1, y1));
        const float a = bilinear(dx, dy, 255.f, 255.f, 255.f, 255.f);
        const unsigned char cu = (unsigned char)min(__float2uint_rz(c), 255u);
        px = make_uchar4(cu, cu, cu, (unsigned char)min(__float2uint_rz(a), 255u));
    }
    out[((uint64_t)d * g.oh + y) * g.ow + x] = px;
}

// ---- PNG encoding (host) ----------------------------------------------------
// zlib stream (RFC 1950) of one DEFLATE block with the fixed Huffman codes
// (RFC 1951 3.2.6), greedy LZ77 over a 32 KiB window with hash chains; PNG
// rows filtered per row with the None / Sub / Up filter whose bytes have the
// smallest sum of magnitudes.

uint32_t crc32_update(uint32_t crc, const uint8_t* p, size_t n) {
    static const std::vector<uint32_t> table = [] {
        std::vector<uint32_t> t(256);
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            t[i] = c;
        }
        return t;
    }();
    crc = ~crc;
    for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xFF] ^ (crc >> 8);
    return ~crc;
}

struct BitOut {
    std::vector<uint8_t>& out;
    uint64_t acc = 0;
    int n = 0;
    void put(uint32_t bits, int count) {  // LSB first, count <= 16
        acc |= (uint64_t)bits << n;
        n += count;
        if (n >= 32) {  // four whole bytes at a time
            const uint8_t four[4] = {(uint8_t)acc, (uint8_t)(acc >> 8), (uint8_t)(acc >> 16), (uint8_t)(acc >> 24)};
            out.insert(out.end(), four, four + 4);
            acc >>= 32;
            n -= 32;
        }
    }
    void flush() {
        for (; n > 0; n -= 8) {
            out.push_back((uint8_t)acc);
            acc >>= 8;
        }
        acc = 0;
        n = 0;
    }
};

// The fixed literal/length code of RFC 1951 3.2.6, bit-reversed once for the
// LSB-first writer: code[sym] | length << 16.
struct FixedCodes {
    uint32_t lit[288];
    uint32_t dist[30];
    static uint32_t reversed(uint32_t code, int len) {
        uint32_t r = 0;
        for (int i = 0; i < len; ++i) r |= ((code >> i) & 1u) << (len - 1 - i);
        return r;
    }
    FixedCodes() {
        for (uint32_t sym = 0; sym < 288; ++sym) {
            uint32_t code, len;
            if (sym < 144) code = 0x30 + sym, len = 8;
            else if (sym < 256) code = 0x190 + (sym - 144), len = 9;
            else if (sym < 280) code = sym - 256, len = 7;
            else code = 0xC0 + (sym - 280), len = 8;
            lit[sym] = reversed(code, (int)len) | len << 16;
        }
        for (uint32_t d = 0; d < 30; ++d) dist[d] = reversed(d, 5) | 5u << 16;
    }
};
const FixedCodes kFixed;

void put_literal(BitOut& b, uint32_t sym) {
    const uint32_t c = kFixed.lit[sym];
    b.put(c & 0xFFFF, (int)(c >> 16));
}

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27,
                               31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129,
                                193, 257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

void put_match(BitOut& b, uint32_t len, uint32_t dist) {
    int lc = 28;
    while (kLenBase[lc] > len) --lc;
    put_literal(b, 257 + lc);
    b.put(len - kLenBase[lc], kLenExtra[lc]);
    int dc = 29;
    while (kDistBase[dc] > dist) --dc;
    b.put(kFixed.dist[dc] & 0xFFFF, 5);
    b.put(dist - kDistBase[dc], kDistExtra[dc]);
}

void zlib_compress(const std::vector<uint8_t>& in, std::vector<uint8_t>& out) {
    out.reserve(out.size() + in.size() + in.size() / 8 + 64);  // fixed codes: at most 9 bits per byte
    out.push_back(0x78);
    out.push_back(0x01);
    BitOut b{out};
    b.put(1, 1);  // BFINAL
    b.put(1, 2);  // BTYPE = fixed Huffman
    constexpr uint32_t kWin = 32768, kHash = 1u << 15, kChain = 24;
    std::vector<int32_t> head(kHash, -1), prev(kWin, -1);
    const size_t n = in.size();
    // Multiplicative (Fibonacci) hash of the three bytes: filtered RGBA rows
    // are full of zero bytes, which a shift-and-xor hash folds into few buckets.
    auto hash3 = [&](size_t i) {
        const uint32_t v = (uint32_t)in[i] | (uint32_t)in[i + 1] << 8 | (uint32_t)in[i + 2] << 16;
        return (v * 2654435761u) >> 17;  // 15 bits
    };
    auto insert = [&](size_t i) {
        if (i + 2 >= n) return;
        const uint32_t h = hash3(i);
        prev[i & (kWin - 1)] = head[h];
        head[h] = (int32_t)i;
    };
    size_t i = 0;
    while (i < n) {
        uint32_t best = 0, best_d = 0;
        if (i + 2 < n) {
            int32_t c = head[hash3(i)];
            const uint32_t maxlen = (uint32_t)std::min<size_t>(258, n - i);
            for (uint32_t k = 0; k < kChain && c >= 0 && i - (size_t)c <= kWin; ++k) {
                // A candidate that differs at the current best length cannot be longer.
                if (best < maxlen && in[c + best] != in[i + best]) {
                    const int32_t nx = prev[c & (kWin - 1)];
                    if (nx >= c) break;
                    c = nx;
                    continue;
                }
                uint32_t l = 0;
                while (l < maxlen && in[c + l] == in[i + l]) ++l;
                if (l > best) {
                    best = l;
                    best_d = (uint32_t)(i - c);
                    if (l == maxlen) break;
                }
                const int32_t nx = prev[c & (kWin - 1)];
                if (nx >= c) break;  // the slot was reused by a newer position
                c = nx;
            }
        }
        if (best >= 3) {
            put_match(b, best, best_d);
            for (uint32_t k = 0; k < best; ++k) insert(i + k);
            i += best;
        } else {
            put_literal(b, in[i]);
            insert(i);
            ++i;
        }
    }
    put_literal(b, 256);
    b.flush();
    // Adler-32 (RFC 1950 8.2), reduced modulo 65521 once per 5552 bytes: the
    // longest run whose sums cannot overflow 32 bits.
    uint32_t s1 = 1, s2 = 0;
    for (size_t at = 0; at < n;) {
        const size_t end = std::min(n, at + 5552);
        for (; at < end; ++at) {
            s1 += in[at];
            s2 += s1;
        }
        s1 %= 65521u;
        s2 %= 65521u;
    }
    const uint32_t adler = (s2 << 16) | s1;
    for (int k = 3; k >= 0; --k) out.push_back((uint8_t)(adler >> (8 * k)));
}

void put_be32(std::vector<uint8_t>& v, uint32_t x) {
    for (int k = 3; k >= 0; --k) v.push_back((uint8_t)(x >> (8 * k)));
}

void put_chunk(std::vector<uint8_t>& file, const char type[4], const std::vector<uint8_t>& data) {
    put_be32(file, (uint32_t)data.size());
    const size_t at = file.size();
    file.insert(file.end(), type, type + 4);
    file.insert(file.end(), data.begin(), data.end());
    put_be32(file, crc32_update(0, file.data() + at, data.size() + 4));
}

std::vector<uint8_t> encode_png(const uint8_t* rgba, uint32_t w, uint32_t h) {
    const size_t row = (size_t)w * 4;
    std::vector<uint8_t> raw;
    raw.reserve((row + 1) * h);
    std::vector<uint8_t> cand[3];
    for (auto& c : cand) c.resize(row);
    for (uint32_t y = 0; y < h; ++y) {
        const uint8_t* cur = rgba + y * row;
        const uint8_t* up = y ? cur - row : nullptr;
        uint64_t cost[3] = {0, 0, 0};
        for (size_t i = 0; i < row; ++i) {
            const uint8_t f[3] = {cur[i], (uint8_t)(cur[i] - (i >= 4 ? cur[i - 4] : 0)),
                                  (uint8_t)(cur[i] - (up ? up[i] : 0))};
            for (int k = 0; k < 3; ++k) {
                cand[k][i] = f[k];
                cost[k] += (uint64_t)std::abs((int)(int8_t)f[k]);
            }
        }
        const int best = (int)(std::min_element(cost, cost + 3) - cost);
        raw.push_back((uint8_t)best);  // filter types 0 None, 1 Sub, 2 Up
        raw.insert(raw.end(), cand[best].begin(), cand[best].end());
    }
    std::vector<uint8_t> file = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
    std::vector<uint8_t> ihdr;
    put_be32(ihdr, w);
    put_be32(ihdr, h);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});  // 8-bit RGBA, deflate, adaptive filters, no interlace
    put_chunk(file, "IHDR", ihdr);
    std::vector<uint8_t> z;
    zlib_compress(raw, z);
    put_chunk(file, "IDAT", z);
    put_chunk(file, "IEND", {});
    return file;
}

bool write_file(const std::string& path, const std::vector<uint8_t>& bytes) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) return false;
    const bool ok = std::fwrite(bytes.data(), 1, bytes.size(), f) == bytes.size();
    return (std::fclose(f) == 0) && ok;
}

fbp_status check_image_args(const char* fn, const float* act, uint32_t w, uint32_t h, uint32_t D, uint64_t pixel_stride,
                            uint64_t plane_stride, uint32_t ow, uint32_t oh) {
    if (!act) return set_error(FBP_ERR_INVALID_ARG, std::string(fn) + ": null data");
    if (w == 0 || h == 0 || D == 0 || ow == 0 || oh == 0 || w > 65535 || h > 65535 || ow > 65535 || oh > 65535)
        return set_error(FBP_ERR_INVALID_ARG, std::string(fn) + ": sizes must be in 1..65535 and D > 0");
    if (pixel_stride == 0 || (D > 1 && plane_stride == 0) || pixel_stride > (1ull << 40) || plane_stride > (1ull << 40))
        return set_error(FBP_ERR_INVALID_ARG, std::string(fn) + ": bad strides");
    if ((ow != w || oh != h) && (ow < 2 || oh < 2))
        return set_error(FBP_ERR_INVALID_ARG, std::string(fn) + ": a resized image needs at least 2 x 2 pixels");
    if (D > 65535) return set_error(FBP_ERR_INVALID_ARG, std::string(fn) + ": at most 65535 planes");
    return FBP_OK;
}

}  // namespace

fbp_status transient_images(fbp_context* ctx, const float* act, uint32_t w, uint32_t h, uint32_t D,
                            uint64_t pixel_stride, uint64_t plane_stride, uint32_t ow, uint32_t oh, int normalize,
                            uint8_t* rgba, cudaStream_t s) {
    unsigned int* maxbits = nullptr;
    if (normalize) {
        void* ws = nullptr;
        FBP_TRY(workspace(ctx, WS_PARTIALS, (size_t)D * sizeof(unsigned int), s, &ws));
        maxbits = static_cast<unsigned int*>(ws);
        FBP_TRY_CUDA(cudaMemsetAsync(maxbits, 0, (size_t)D * sizeof(unsigned int), s));
        const uint32_t npix = w * h;
        plane_max_kernel<<<dim3(std::min(cdiv(npix, 256), 64u), D), 256, 0, s>>>(act, npix, pixel_stride,
                                                                                  plane_stride, maxbits);
        FBP_CHECK_LAUNCH(ctx, "plane_max_kernel");
    }
    ImageGeom g{w, h, pixel_stride, plane_stride, ow, oh, 0.f, 0.f, normalize};
    const bool resize = ow != w || oh != h;
    if (resize) {
        g.xr = (float)(w - 1) / (float)(ow - 1);  // Image.h:97-98
        g.yr = (float)(h - 1) / (float)(oh - 1);
    }
    const dim3 grid(cdiv((uint64_t)ow * oh, 256), D);
    if (resize) plane_image_kernel<true><<<grid, 256, 0, s>>>(act, g, maxbits, reinterpret_cast<uchar4*>(rgba));
    else plane_image_kernel<false><<<grid, 256, 0, s>>>(act, g, maxbits, reinterpret_cast<uchar4*>(rgba));
    FBP_CHECK_LAUNCH(ctx, "plane_image_kernel");
    return FBP_OK;
}

}  // namespace fbp

using namespace fbp;

extern "C" fbp_status fbp_transient_images(fbp_context* ctx, const float* data, uint32_t width, uint32_t height,
                                           uint32_t num_planes, uint64_t pixel_stride, uint64_t plane_stride,
                                           uint32_t out_width, uint32_t out_height, int normalize, uint8_t* rgba,
                                           void* stream) {
    return guarded("fbp_transient_images", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        FBP_TRY(check_image_args("fbp_transient_images", data, width, height, num_planes, pixel_stride, plane_stride,
                                 out_width, out_height));
        if (!rgba) return set_error(FBP_ERR_INVALID_ARG, "fbp_transient_images: null output");
        return transient_images(ctx, data, width, height, num_planes, pixel_stride, plane_stride, out_width, out_height,
                                normalize, rgba, (cudaStream_t)stream);
    });
}

// The encoder indexes the filtered rows with 32-bit positions.
constexpr uint64_t kPngMaxRaw = (uint64_t)1 << 30;

extern "C" fbp_status fbp_write_png(const char* path, const uint8_t* rgba, uint32_t width, uint32_t height) {
    return guarded("fbp_write_png", [&]() -> fbp_status {
        clear_error();
        if (!path || !rgba || width == 0 || height == 0 || width > 65535 || height > 65535)
            return set_error(FBP_ERR_INVALID_ARG, "fbp_write_png: bad arguments");
        if (((uint64_t)width * 4 + 1) * height > kPngMaxRaw)
            return set_error(FBP_ERR_UNSUPPORTED, "fbp_write_png: image larger than 1 GiB of pixels");
        if (!write_file(path, encode_png(rgba, width, height)))
            return set_error(FBP_ERR_IO, std::string("fbp_write_png: cannot write ") + path);
        return FBP_OK;
    });
}

extern "C" fbp_status fbp_save_transient_images(fbp_context* ctx, const float* data, uint32_t width, uint32_t height,
                                                uint32_t num_planes, uint64_t pixel_stride, uint64_t plane_stride,
                                                uint32_t out_width, uint32_t out_height, int normalize,
                                                const char* prefix, void* stream) {
    return guarded("fbp_save_transient_images", [&]() -> fbp_status {
        clear_error();
        FBP_TRY(check_ctx(ctx));
        FBP_TRY(check_image_args("fbp_save_transient_images", data, width, height, num_planes, pixel_stride, plane_stride,
                                 out_width, out_height));
        if (!prefix) return set_error(FBP_ERR_INVALID_ARG, "fbp_save_transient_images: null prefix");
        if (((uint64_t)out_width * 4 + 1) * out_height > kPngMaxRaw)
            return set_error(FBP_ERR_UNSUPPORTED, "fbp_save_transient_images: image larger than 1 GiB of pixels");
        const uint32_t num_depths = num_planes;
        cudaStream_t s = (cudaStream_t)stream;
        const size_t plane = (size_t)out_width * out_height * 4, bytes = plane * num_depths;
        void* dev = nullptr;
        FBP_TRY(workspace(ctx, WS_MISC, bytes, s, &dev));
        FBP_TRY(transient_images(ctx, data, width, height, num_planes, pixel_stride, plane_stride, out_width, out_height,
                                 normalize, static_cast<uint8_t*>(dev), s));
        std::vector<uint8_t> host(bytes);
        FBP_TRY_CUDA(cudaMemcpyAsync(host.data(), dev, bytes, cudaMemcpyDeviceToHost, s));
        FBP_TRY_CUDA(cudaStreamSynchronize(s));
        FBP_TRY(fbp_check_device_status(ctx, stream));
        // Laser.cu:419-423, NLosData.cpp:172-178: "<prefix>transient_<p>.png", one
        // file per plane, in parallel.
        const unsigned nthreads = std::max(1u, std::min(num_depths, std::thread::hardware_concurrency()));
        std::vector<int> failed(num_depths, 0);
        std::vector<std::thread> pool;
        for (unsigned t = 0; t < nthreads; ++t)
            pool.emplace_back([&, t] {
                for (uint32_t d = t; d < num_depths; d += nthreads) {
                    const std::string path = std::string(prefix) + "transient_" + std::to_string(d) + ".png";
                    failed[d] = !write_file(path, encode_png(host.data() + d * plane, out_width, out_height));
                }
            });
        for (auto& th : pool) th.join();
        for (uint32_t d = 0; d < num_depths; ++d)
            if (failed[d])
                return set_error(FBP_ERR_IO, std::string("fbp_save_transient_images: cannot write ") + prefix + "transient_" +
                                                 std::to_string(d) + ".png");
        return FBP_OK;
    });
}
