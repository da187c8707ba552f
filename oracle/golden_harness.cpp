/*
 * ORACLE -- test infrastructure only.  Calls the reference renderer's own
 * functions (compiled from its unmodified sources) on inputs read from a file
 * and writes their outputs, to produce the golden vectors under tests/golden/.
 *
 *   golden_harness eval   in out          BSDFModel<GGX>::evaluateDirect (BRDFModel.h:211)
 *       in: 17 floats/case I O N color(4) metallness alpha pad pad; out: 3 floats
 *   golden_harness sample in out          BSDFModel<GGX>::sampleIndirect (BRDFModel.h:265)
 *       in: 24 floats/case I N T color(4) metallness alpha eta transmissive seed(u32) ...;
 *       RandomSampler(seed) supplies the draws; out: 6 floats O brdf
 *   golden_harness om     material in out OpenMaterial::getBrdf (OpenMaterial.cpp:95) at normal (0,0,1)
 *       in: 1 float/case cos; out: 3 floats
 *   golden_harness ior    ior in out      AssetMaterialIor::getIor (AssetMaterialIor.cpp:133)
 *       in: 2 floats/case temperature wavelength; out: 2 floats n k
 *   golden_harness env    hdr in out      HDRBackground::getRadiance (HdrBackground.cpp:55)
 *       in: 10 floats rotation(9) scale, then 3 floats/case direction; out: 3 floats
 *   golden_harness camera props W H seed out   PinholeCamera::getRay (PinholeCamera.cpp:80)
 *       out: halfW halfH focus, then 6 floats/pixel (row-major) from one RandomSampler(seed)
 *   golden_harness mt     seed n out      RandomSampler::rand (RandomSampler.h:59)
 *   golden_harness tonemap W H gamma in out   gammaCorrection(img, W, H, 1, gamma) (ToneMapping.cpp:24)
 *       in/out: W*H*4 floats (rgba, row-major)
 *   golden_harness median  W H in out     SimpleDenoiserMedian<1> (Denoiser.h:24); in/out as tonemap
 *   golden_harness rgba8   W H in out     saveImage's conversion (main.cpp:92): unsigned char(255 f),
 *       out: W*H*4 bytes
 *   golden_harness png     in out        stb_image as tinygltf loads images (4 channels; 16-bit
 *       files through stbi_load_16), out: int32 W H then W*H*4 uint16 samples
 *   golden_harness hdr     in out        stbi_loadf(in, 0 channels) as HDRBackground loads a .hdr
 *       (HdrBackground.cpp:42), out: int32 W H channels then W*H*channels floats
 *   golden_harness texture W H img uv out BitmapTexture::texture(u, v, fvec4) (BitmapTexture.cpp:108-125)
 *       img: W*H*4 bytes; uv: 2 floats/case; out: 4 floats/case
 */
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "BRDFModel.h"
#include "HdrBackground.h"
#include "OpenMaterial.h"
#include "PinholeCamera.h"
#include "RandomSampler.h"
#include "ToneMapping.h"
#include "Denoiser.h"
#include "BitmapTexture.h"
#include "stb_image.h"
#include "materials/AssetMaterial.h"
#include "materials/AssetMaterialIor.h"

static std::vector<float> read_floats(const char* path)
{
    std::vector<float> v;
    FILE* f = std::fopen(path, "rb");
    if (!f) {
        std::perror(path);
        std::exit(2);
    }
    float x;
    while (std::fread(&x, sizeof(float), 1, f) == 1) v.push_back(x);
    std::fclose(f);
    return v;
}

static void write_floats(const char* path, const std::vector<float>& v)
{
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        std::perror(path);
        std::exit(2);
    }
    std::fwrite(v.data(), sizeof(float), v.size(), f);
    std::fclose(f);
}

using BSDF = BSDFModel<ndf::GGX>;

int main(int argc, char** argv)
{
    if (argc < 2) return 1;
    std::string mode = argv[1];
    std::vector<float> out;
    if (mode == "eval" && argc == 4) {
        auto in = read_floats(argv[2]);
        for (size_t i = 0; i + 17 <= in.size(); i += 17) {
            BSDFData d;
            std::memcpy(d.I, &in[i], 3 * sizeof(float));
            std::memcpy(d.O, &in[i + 3], 3 * sizeof(float));
            std::memcpy(d.N, &in[i + 6], 3 * sizeof(float));
            std::memcpy(d.color, &in[i + 9], 4 * sizeof(float));
            d.metallness = in[i + 13];
            d.alpha = in[i + 14];
            fvec3 brdf;
            BSDF::evaluateDirect(d, brdf);
            out.insert(out.end(), brdf, brdf + 3);
        }
        write_floats(argv[3], out);
    } else if (mode == "sample" && argc == 4) {
        auto in = read_floats(argv[2]);
        for (size_t i = 0; i + 24 <= in.size(); i += 24) {
            BSDFData d;
            std::memcpy(d.I, &in[i], 3 * sizeof(float));
            std::memcpy(d.N, &in[i + 3], 3 * sizeof(float));
            std::memcpy(d.T, &in[i + 6], 3 * sizeof(float));
            std::memcpy(d.color, &in[i + 9], 4 * sizeof(float));
            d.metallness = in[i + 13];
            d.alpha = in[i + 14];
            d.eta = in[i + 15];
            d.isTransmissive = in[i + 16] != 0.0f;
            uint32_t seed;
            std::memcpy(&seed, &in[i + 17], 4);
            RandomSampler rs(seed);
            fvec3 brdf;
            BSDF::sampleIndirect(d, &rs, brdf);
            out.insert(out.end(), d.O, d.O + 3);
            out.insert(out.end(), brdf, brdf + 3);
        }
        write_floats(argv[3], out);
    } else if (mode == "om" && argc == 5) {
        AssetMaterial mat{std::string(argv[2])};
        OpenMaterial om;
        om.setMaterial(&mat);
        auto in = read_floats(argv[3]);
        SurfacePoint sp;
        assignVector(sp.m_normal, 0.0f, 0.0f, 1.0f);
        for (float c : in) {
            float s = std::sqrt(std::max(0.0f, 1.0f - c * c));
            fvec3 inV = {s, 0.0f, -c};
            fvec3 outV = {s, 0.0f, c};
            fvec3 brdf;
            om.getBrdf(inV, &sp, outV, brdf);
            out.insert(out.end(), brdf, brdf + 3);
        }
        write_floats(argv[4], out);
    } else if (mode == "ior" && argc == 5) {
        AssetMaterialIor ior{std::string(argv[2])};
        auto in = read_floats(argv[3]);
        for (size_t i = 0; i + 2 <= in.size(); i += 2) {
            float n = 0, k = 0;
            ior.getIor(in[i], in[i + 1], n, k);
            out.push_back(n);
            out.push_back(k);
        }
        write_floats(argv[4], out);
    } else if (mode == "env" && argc == 5) {
        HDRBackground bg(argv[2]);
        auto in = read_floats(argv[3]);
        fmat3 R;
        std::memcpy(R, in.data(), 9 * sizeof(float));
        bg.setRotation(R);
        bg.setRadianceScale(in[9]);
        for (size_t i = 10; i + 3 <= in.size(); i += 3) {
            fvec3 dir = {in[i], in[i + 1], in[i + 2]}, val;
            bg.getRadiance(dir, val);
            out.insert(out.end(), val, val + 3);
        }
        write_floats(argv[4], out);
    } else if (mode == "camera" && argc == 7) {
        int W = std::atoi(argv[3]), H = std::atoi(argv[4]);
        uint32_t seed = (uint32_t)std::strtoul(argv[5], nullptr, 10);
        fvec3 pos = {0.0f, 0.0f, 0.0f}, up = {0.0f, 1.0f, 0.0f}, fwd = {0.0f, 0.0f, -1.0f}, left;
        cross3(fwd, up, left);
        cross3(left, fwd, up);
        PinholeCamera cam({pos, left, up, fwd}, W, H);
        cam.loadProperties(argv[2]);
        auto sz = cam.getRealSizes();
        out.push_back(sz.first);
        out.push_back(sz.second);
        out.push_back(cam.getFocus());
        RandomSampler rs(seed);
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                RenderRay r = cam.getRay(x, y, rs);
                out.insert(out.end(), r.O(), r.O() + 3);
                out.insert(out.end(), r.R(), r.R() + 3);
            }
        write_floats(argv[6], out);
    } else if (mode == "mt" && argc == 5) {
        RandomSampler rs((uint32_t)std::strtoul(argv[2], nullptr, 10));
        long n = std::atol(argv[3]);
        for (long i = 0; i < n; ++i) out.push_back(rs.rand());
        write_floats(argv[4], out);
    } else if (mode == "png" && argc == 4) {
        int w = 0, h = 0, c = 0;
        std::vector<uint16_t> px;
        if (stbi_is_16_bit(argv[2])) {
            stbi_us* d = stbi_load_16(argv[2], &w, &h, &c, 4);
            if (!d) return 2;
            px.assign(d, d + (size_t)w * h * 4);
            stbi_image_free(d);
        } else {
            stbi_uc* d = stbi_load(argv[2], &w, &h, &c, 4);
            if (!d) return 2;
            px.assign(d, d + (size_t)w * h * 4);
            stbi_image_free(d);
        }
        FILE* f = std::fopen(argv[3], "wb");
        if (!f) return 2;
        const int32_t wh[2] = {w, h};
        std::fwrite(wh, sizeof(int32_t), 2, f);
        std::fwrite(px.data(), sizeof(uint16_t), px.size(), f);
        std::fclose(f);
        return 0;
    } else if (mode == "hdr" && argc == 4) {
        int w = 0, h = 0, c = 0;
        float* d = stbi_loadf(argv[2], &w, &h, &c, 0);
        if (!d) return 2;
        FILE* f = std::fopen(argv[3], "wb");
        if (!f) return 2;
        const int32_t whc[3] = {w, h, c};
        std::fwrite(whc, sizeof(int32_t), 3, f);
        std::fwrite(d, sizeof(float), (size_t)w * h * 3, f);
        std::fclose(f);
        stbi_image_free(d);
        return 0;
    } else if (mode == "texture" && argc == 7) {
        const int W = std::atoi(argv[2]), H = std::atoi(argv[3]);
        FILE* f = std::fopen(argv[4], "rb");
        if (!f) return 2;
        std::vector<unsigned char> img((size_t)W * H * 4);
        if (std::fread(img.data(), 1, img.size(), f) != img.size()) return 2;
        std::fclose(f);
        BitmapTexture tex(W, H, reinterpret_cast<ubvec4*>(img.data()));
        auto uv = read_floats(argv[5]);
        for (size_t i = 0; i + 2 <= uv.size(); i += 2) {
            fvec4 t;
            tex.texture(uv[i], uv[i + 1], t);
            out.insert(out.end(), t, t + 4);
        }
        write_floats(argv[6], out);
    } else if ((mode == "tonemap" && argc == 7) || ((mode == "median" || mode == "rgba8") && argc == 6)) {
        const int W = std::atoi(argv[2]), H = std::atoi(argv[3]);
        const bool tm = mode == "tonemap";
        auto img = read_floats(argv[tm ? 5 : 4]);
        if (img.size() != (size_t)4 * W * H) {
            std::fprintf(stderr, "image size mismatch\n");
            return 1;
        }
        const char* dst = argv[tm ? 6 : 5];
        auto px = reinterpret_cast<fvec4*>(img.data());
        if (tm) {
            gammaCorrection(px, W, H, 1.0f, (float)std::atof(argv[4]));
        } else if (mode == "median") {
            SimpleDenoiserMedian<1>(px, W, H);
        } else {
            std::vector<unsigned char> q(img.size());
            std::transform(img.begin(), img.end(), q.begin(), [](float f) { return static_cast<unsigned char>(255.0f * f); });
            FILE* f = std::fopen(dst, "wb");
            if (!f) return 2;
            std::fwrite(q.data(), 1, q.size(), f);
            std::fclose(f);
            return 0;
        }
        write_floats(dst, img);
        return 0;
    } else {
        std::fprintf(stderr, "bad arguments\n");
        return 1;
    }
    return 0;
}
