// Image development on the device and the image writers: the reference's
// host-side tail of a render (main.cpp:505-521), after BDPTRenderer::render.
//
//   k_develop   film sums -> PinholeCamera::stop normalisation (rgb / count,
//               PinholeCamera.cpp:70-78) -> gammaCorrection -> 8-bit rgba, in
//               one pass over the film; each output optional
//   k_tonemap   gammaCorrection (ToneMapping.cpp:24-53) in place: per pixel
//               rgb *= A l^gamma / l for the luminance l when l > FLT_EPSILON,
//               every channel clamped to [0, 1], alpha 1
//   k_median3   SimpleDenoiserMedian<1> (Denoiser.h:24-64): per-channel median
//               of the 3x3 window on pixels one away from every edge (alpha 1
//               there), the border copied; a shared-memory tile per block
//   k_median    the same for windows of 5x5 and 7x7
//   k_rgba8     saveImage's conversion (main.cpp:92): unsigned char(255 f),
//               rows optionally flipped (ImageSaver::flipVerticallyOnWrite)
//
// All are bound by HBM traffic: 16 B read and 16 B written per pixel for the
// float passes, 28 B read for the film.  The luminance and scaling use
// explicitly rounded operations (no contraction) so they round like the
// reference; only powf differs from the host's within its error bound.
//
// save_image writes PFM as ImageSaver::savePfm does with flipping on, and PNG
// (stored deflate blocks), BMP and TGA (uncompressed) with the same pixels as
// the reference's stb_image_write output.
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "scene.h"

namespace omv {
namespace {

// clamp01f (UtilityFunctions.h:452) with the reference's comparison order:
// max(0, min(v, 1)), so NaN maps to 1
__device__ __forceinline__ float clamp01(float v)
{
    const float m = v < 1.0f ? v : 1.0f;
    return 0.0f > m ? 0.0f : m;
}

__device__ __forceinline__ float4 gamma_correct(float4 p, float A, float gamma)
{
    const float l = __fadd_rn(__fadd_rn(__fmul_rn(0.2126f, p.x), __fmul_rn(0.7152f, p.y)), __fmul_rn(0.0722f, p.z));
    const float o = __fmul_rn(A, powf(l, gamma));
    const float f = l > FLT_EPSILON ? __fdiv_rn(o, l) : 1.0f;
    return make_float4(clamp01(__fmul_rn(f, p.x)), clamp01(__fmul_rn(f, p.y)), clamp01(__fmul_rn(f, p.z)), 1.0f);
}

// unsigned char(255 f); the clamp only matters outside [0, 1], where the
// reference's conversion is undefined
__device__ __forceinline__ uint8_t to_u8(float f)
{
    const float v = __fmul_rn(255.0f, f);
    return v >= 255.0f ? (uint8_t)255 : (v > 0.0f ? (uint8_t)__float2uint_rz(v) : (uint8_t)0);
}

__device__ __forceinline__ uchar4 to_u8x4(float4 p)
{
    return make_uchar4(to_u8(p.x), to_u8(p.y), to_u8(p.z), to_u8(p.w));
}

__global__ void k_develop(const double* __restrict__ sum, const uint32_t* __restrict__ count, int w, int h, float A,
                          float gamma, float4* __restrict__ linear, float4* __restrict__ toned,
                          uchar4* __restrict__ rgba8, int flip)
{
    const int64_t n = (int64_t)w * h;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double c = (double)count[i];
        const double s = c < 0.5 ? 1.0 : __drcp_rn(c);  // 1.0 / c, the same correctly rounded bits
        const float4 lin = make_float4((float)(sum[3 * i] * s), (float)(sum[3 * i + 1] * s),
                                       (float)(sum[3 * i + 2] * s), 1.0f);
        if (linear) linear[i] = lin;
        if (!toned && !rgba8) continue;
        const float4 t = gamma_correct(lin, A, gamma);
        if (toned) toned[i] = t;
        if (rgba8) {  // i < 2^31: a 32-bit division for the row
            const int64_t y = (int64_t)((uint32_t)i / (uint32_t)w), x = i - y * w;
            rgba8[flip ? (h - 1 - y) * (int64_t)w + x : i] = to_u8x4(t);
        }
    }
}

__global__ void k_tonemap(float4* __restrict__ img, int64_t n, float A, float gamma)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        img[i] = gamma_correct(img[i], A, gamma);
}

__global__ void k_rgba8(const float4* __restrict__ in, uchar4* __restrict__ out, int w, int h, int flip)
{
    const int64_t n = (int64_t)w * h;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t y = (int64_t)((uint32_t)i / (uint32_t)w), x = i - y * w;  // i < 2^31
        out[flip ? (h - 1 - y) * (int64_t)w + x : i] = to_u8x4(in[i]);
    }
}

constexpr int kTileW = 32, kTileH = 8;

__device__ __forceinline__ void order(float& a, float& b)
{
    const float lo = fminf(a, b), hi = fmaxf(a, b);
    a = lo;
    b = hi;
}

// median of nine by Paeth's 19-exchange network (A. Paeth, "Median finding on
// a 3x3 grid", Graphics Gems, 1990): after the exchanges p[4] holds the value
// that sorting the nine would put in the middle
__device__ __forceinline__ float median9(float p[9])
{
    order(p[1], p[2]); order(p[4], p[5]); order(p[7], p[8]);
    order(p[0], p[1]); order(p[3], p[4]); order(p[6], p[7]);
    order(p[1], p[2]); order(p[4], p[5]); order(p[7], p[8]);
    order(p[0], p[3]); order(p[5], p[8]); order(p[4], p[7]);
    order(p[3], p[6]); order(p[1], p[4]); order(p[2], p[5]);
    order(p[4], p[7]); order(p[4], p[2]); order(p[6], p[4]);
    order(p[4], p[2]);
    return p[4];
}

// one 32x8 block of output pixels from a (32+2)x(8+2) tile in shared memory;
// tile loads are clamped to the image, and only border pixels (which copy
// their input) would see a clamped value
__global__ void __launch_bounds__(kTileW* kTileH) k_median3(const float4* __restrict__ in, float4* __restrict__ out,
                                                            int w, int h)
{
    __shared__ float4 tile[kTileH + 2][kTileW + 2];
    const int x0 = blockIdx.x * kTileW - 1, y0 = blockIdx.y * kTileH - 1;
    const int tid = threadIdx.y * kTileW + threadIdx.x;
    for (int k = tid; k < (kTileW + 2) * (kTileH + 2); k += kTileW * kTileH) {
        const int ty = k / (kTileW + 2), tx = k - ty * (kTileW + 2);
        const int gx = min(max(x0 + tx, 0), w - 1), gy = min(max(y0 + ty, 0), h - 1);
        tile[ty][tx] = in[(size_t)gy * w + gx];
    }
    __syncthreads();
    const int x = blockIdx.x * kTileW + threadIdx.x, y = blockIdx.y * kTileH + threadIdx.y;
    if (x >= w || y >= h) return;
    const int cx = threadIdx.x + 1, cy = threadIdx.y + 1;
    if (x < 1 || y < 1 || x >= w - 1 || y >= h - 1) {
        out[(size_t)y * w + x] = tile[cy][cx];
        return;
    }
    float r[9], g[9], b[9];
#pragma unroll
    for (int dy = 0; dy < 3; ++dy)
#pragma unroll
        for (int dx = 0; dx < 3; ++dx) {
            const float4 p = tile[cy - 1 + dy][cx - 1 + dx];
            r[3 * dy + dx] = p.x;
            g[3 * dy + dx] = p.y;
            b[3 * dy + dx] = p.z;
        }
    out[(size_t)y * w + x] = make_float4(median9(r), median9(g), median9(b), 1.0f);
}

// the value with (n - 1) / 2 window elements before it in sorted order (ties
// broken by position): the element sorting would put in the middle
template <int N>
__device__ float select_median(const float* v)
{
    constexpr int target = (N - 1) / 2;
    for (int a = 0; a < N; ++a) {
        int before = 0;
#pragma unroll
        for (int b = 0; b < N; ++b) before += (v[b] < v[a] || (v[b] == v[a] && b < a)) ? 1 : 0;
        if (before == target) return v[a];
    }
    return v[target];
}

template <int H>
__global__ void k_median(const float4* __restrict__ in, float4* __restrict__ out, int w, int h)
{
    constexpr int S = 2 * H + 1;
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const size_t o = (size_t)y * w + x;
    if (x < H || y < H || x >= w - H || y >= h - H) {
        out[o] = in[o];
        return;
    }
    float r[S * S], g[S * S], b[S * S];
    for (int dy = 0; dy < S; ++dy)
        for (int dx = 0; dx < S; ++dx) {
            const float4 p = in[(size_t)(y - H + dy) * w + (x - H + dx)];
            r[S * dy + dx] = p.x;
            g[S * dy + dx] = p.y;
            b[S * dy + dx] = p.z;
        }
    out[o] = make_float4(select_median<S * S>(r), select_median<S * S>(g), select_median<S * S>(b), 1.0f);
}

int stream_grid(int64_t n, int threads)
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
            sms = 152;
    }
    const int64_t need = (n + threads - 1) / threads;
    return (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)sms * 8));
}

void check_image(int w, int h)
{
    if (w <= 0 || h <= 0) throw ArgError("image width and height must be positive");
    if ((int64_t)w * h > ((int64_t)1 << 31)) throw ArgError("image too large");
}

// ------------------------------------------------------------ writers ---
void put16(std::vector<uint8_t>& v, uint32_t x)
{
    v.push_back(x & 0xFF);
    v.push_back((x >> 8) & 0xFF);
}
void put32(std::vector<uint8_t>& v, uint32_t x)
{
    put16(v, x & 0xFFFF);
    put16(v, x >> 16);
}
void put32be(std::vector<uint8_t>& v, uint32_t x)
{
    v.push_back(x >> 24);
    v.push_back((x >> 16) & 0xFF);
    v.push_back((x >> 8) & 0xFF);
    v.push_back(x & 0xFF);
}

// CRC-32 of ISO 3309 / ITU-T V.42 (the PNG chunk checksum), bitwise
uint32_t crc32(const uint8_t* p, size_t n)
{
    uint32_t c = 0xFFFFFFFFu;
    for (size_t i = 0; i < n; ++i) {
        c ^= p[i];
        for (int k = 0; k < 8; ++k) c = (c >> 1) ^ (0xEDB88320u & (0u - (c & 1u)));
    }
    return ~c;
}

// PNG (RFC 2083): 8-bit RGBA, filter 0 on every row, the zlib stream (RFC 1950)
// made of stored deflate blocks (RFC 1951 section 3.2.4)
std::vector<uint8_t> encode_png(const uint8_t* rgba, int w, int h)
{
    std::vector<uint8_t> raw;
    raw.reserve((size_t)h * (4 * (size_t)w + 1));
    for (int y = 0; y < h; ++y) {
        raw.push_back(0);
        raw.insert(raw.end(), rgba + (size_t)y * 4 * w, rgba + (size_t)(y + 1) * 4 * w);
    }
    std::vector<uint8_t> z{0x78, 0x01};
    z.reserve(raw.size() + raw.size() / 65535 * 5 + 16);
    size_t off = 0;
    do {
        const size_t len = std::min<size_t>(65535, raw.size() - off);
        z.push_back(off + len >= raw.size() ? 1 : 0);
        put16(z, (uint32_t)len);
        put16(z, (uint32_t)(~len & 0xFFFF));
        z.insert(z.end(), raw.begin() + off, raw.begin() + off + len);
        off += len;
    } while (off < raw.size());
    uint32_t a = 1, b = 0;  // Adler-32
    for (uint8_t c : raw) {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    put32be(z, (b << 16) | a);

    std::vector<uint8_t> out{0x89, 'P', 'N', 'G', 0x0D, 0x0A, 0x1A, 0x0A};
    auto chunk = [&out](const char* type, const std::vector<uint8_t>& data) {
        put32be(out, (uint32_t)data.size());
        const size_t start = out.size();
        out.insert(out.end(), type, type + 4);
        out.insert(out.end(), data.begin(), data.end());
        put32be(out, crc32(out.data() + start, out.size() - start));
    };
    std::vector<uint8_t> ihdr;
    put32be(ihdr, (uint32_t)w);
    put32be(ihdr, (uint32_t)h);
    ihdr.insert(ihdr.end(), {8, 6, 0, 0, 0});
    chunk("IHDR", ihdr);
    chunk("IDAT", z);
    chunk("IEND", {});
    return out;
}

// BMP: BITMAPINFOHEADER, 32 bits per pixel BGRA, rows stored bottom-up
std::vector<uint8_t> encode_bmp(const uint8_t* rgba, int w, int h)
{
    const uint32_t data = 4u * (uint32_t)w * (uint32_t)h;
    std::vector<uint8_t> v{'B', 'M'};
    v.reserve(54 + data);
    put32(v, 54 + data);
    put32(v, 0);
    put32(v, 54);
    put32(v, 40);
    put32(v, (uint32_t)w);
    put32(v, (uint32_t)h);
    put16(v, 1);
    put16(v, 32);
    put32(v, 0);
    put32(v, data);
    put32(v, 2835);
    put32(v, 2835);
    put32(v, 0);
    put32(v, 0);
    for (int y = h - 1; y >= 0; --y)
        for (int x = 0; x < w; ++x) {
            const uint8_t* p = rgba + 4 * ((size_t)y * w + x);
            v.insert(v.end(), {p[2], p[1], p[0], p[3]});
        }
    return v;
}

// TGA: uncompressed true colour, 32 bits BGRA, top-left origin
std::vector<uint8_t> encode_tga(const uint8_t* rgba, int w, int h)
{
    std::vector<uint8_t> v{0, 0, 2, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    v.reserve(18 + 4 * (size_t)w * h);
    put16(v, (uint32_t)w);
    put16(v, (uint32_t)h);
    v.push_back(32);
    v.push_back(0x28);
    for (size_t i = 0; i < (size_t)w * h; ++i) {
        const uint8_t* p = rgba + 4 * i;
        v.insert(v.end(), {p[2], p[1], p[0], p[3]});
    }
    return v;
}

}  // namespace

void develop_film(const double* d_sum, const uint32_t* d_count, int w, int h, float A, float gamma, float* d_linear,
                  float* d_toned, uint8_t* d_rgba8, bool flip, cudaStream_t st)
{
    check_image(w, h);
    if (!d_sum || !d_count) throw ArgError("develop: film sums and counts are required");
    const int64_t n = (int64_t)w * h;
    k_develop<<<stream_grid(n, 256), 256, 0, st>>>(d_sum, d_count, w, h, A, gamma, reinterpret_cast<float4*>(d_linear),
                                                  reinterpret_cast<float4*>(d_toned),
                                                  reinterpret_cast<uchar4*>(d_rgba8), flip ? 1 : 0);
    OMV_CUDA(cudaGetLastError());
}

void tonemap(float* d_rgba, int64_t pixels, float A, float gamma, cudaStream_t st)
{
    if (pixels < 0) throw ArgError("tonemap: negative pixel count");
    if (pixels == 0) return;
    if (!d_rgba) throw ArgError("tonemap: image is NULL");
    k_tonemap<<<stream_grid(pixels, 256), 256, 0, st>>>(reinterpret_cast<float4*>(d_rgba), pixels, A, gamma);
    OMV_CUDA(cudaGetLastError());
}

void denoise_median(const float* d_in, float* d_out, int w, int h, int half, cudaStream_t st)
{
    check_image(w, h);
    if (!d_in || !d_out) throw ArgError("median: image is NULL");
    if (d_in == d_out) throw ArgError("median: input and output must be distinct buffers");
    const auto* in = reinterpret_cast<const float4*>(d_in);
    auto* out = reinterpret_cast<float4*>(d_out);
    if (half == 1) {
        const dim3 g((w + kTileW - 1) / kTileW, (h + kTileH - 1) / kTileH);
        k_median3<<<g, dim3(kTileW, kTileH), 0, st>>>(in, out, w, h);
    } else if (half == 2 || half == 3) {
        const dim3 b(16, 8), g((w + 15) / 16, (h + 7) / 8);
        if (half == 2)
            k_median<2><<<g, b, 0, st>>>(in, out, w, h);
        else
            k_median<3><<<g, b, 0, st>>>(in, out, w, h);
    } else {
        throw ArgError("median: half size must be 1, 2 or 3");
    }
    OMV_CUDA(cudaGetLastError());
}

void rgba8(const float* d_in, uint8_t* d_out, int w, int h, bool flip, cudaStream_t st)
{
    check_image(w, h);
    if (!d_in || !d_out) throw ArgError("rgba8: image is NULL");
    const int64_t n = (int64_t)w * h;
    k_rgba8<<<stream_grid(n, 256), 256, 0, st>>>(reinterpret_cast<const float4*>(d_in),
                                                reinterpret_cast<uchar4*>(d_out), w, h, flip ? 1 : 0);
    OMV_CUDA(cudaGetLastError());
}

void save_image(const char* path, const float* rgba, int w, int h)
{
    if (!path || !rgba) throw ArgError("save_image: path and image are required");
    check_image(w, h);
    const std::string p(path);
    const size_t dot = p.find_last_of('.');
    std::string ext = dot == std::string::npos ? "" : p.substr(dot + 1);
    for (char& c : ext) c = (char)((c >= 'A' && c <= 'Z') ? c - 'A' + 'a' : c);
    const size_t n = (size_t)w * h;
    std::vector<uint8_t> bytes;
    if (ext == "pfm") {
        // ImageSaver::savePfm with flipping on: rows in stored order, rgb floats
        const std::string head = "PF\n" + std::to_string(w) + " " + std::to_string(h) + "\n-1.000000\n";
        bytes.assign(head.begin(), head.end());
        bytes.reserve(head.size() + 12 * n);
        for (size_t i = 0; i < n; ++i) {
            const auto* b = reinterpret_cast<const uint8_t*>(rgba + 4 * i);
            bytes.insert(bytes.end(), b, b + 12);
        }
    } else if (ext == "png" || ext == "bmp" || ext == "tga") {
        // saveImage (main.cpp:86-120): 8 bits per channel; flipVerticallyOnWrite(true)
        // puts the last row of the buffer at the top of the picture
        std::vector<uint8_t> q(4 * n);
        for (size_t y = 0; y < (size_t)h; ++y) {
            const float* src = rgba + 4 * (h - 1 - y) * (size_t)w;
            uint8_t* dst = q.data() + 4 * y * (size_t)w;
            for (size_t k = 0; k < 4 * (size_t)w; ++k) {
                const float v = 255.0f * src[k];
                dst[k] = v >= 255.0f ? 255 : (v > 0.0f ? (uint8_t)v : 0);
            }
        }
        bytes = ext == "png" ? encode_png(q.data(), w, h) : ext == "bmp" ? encode_bmp(q.data(), w, h)
                                                                          : encode_tga(q.data(), w, h);
    } else {
        throw ArgError("save_image: the extension must be png, bmp, tga or pfm");
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) throw ArgError(std::string("save_image: cannot open ") + path);
    const size_t wr = std::fwrite(bytes.data(), 1, bytes.size(), f);
    const int rc = std::fclose(f);
    if (wr != bytes.size() || rc != 0) throw ArgError(std::string("save_image: short write to ") + path);
}

}  // namespace omv
