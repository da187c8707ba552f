/*
 * ORACLE -- test infrastructure only.  C restatement of the reference's image
 * post-processing, the checker for the device kernels of post.cu:
 *   oc_tonemap  gammaCorrection (pathtracer/src/tonemapping/ToneMapping.cpp:24-53)
 *   oc_median   SimpleDenoiserMedian<H> (pathtracer/src/utilities/Denoiser.h:24-64)
 *   oc_rgba8    saveImage's 8-bit conversion (pathtracer/src/main.cpp:92)
 * Built with -ffp-contract=off like the reference objects, so the float
 * results are the reference's bit for bit (pinned by tests/golden/post.npz).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* clamp01f (UtilityFunctions.h:452): max(0, min(v, 1)) with the reference's
 * comparison order, so NaN maps to 1 and -0 stays -0 */
static float clamp01(float v)
{
    const float m = v < 1.0f ? v : 1.0f;
    return 0.0f > m ? 0.0f : m;
}

/* per pixel: luminance l = dot((0.2126, 0.7152, 0.0722), rgb); rgb *= A l^g / l
 * when l > FLT_EPSILON; then every channel clamped to [0, 1], alpha = 1.  The
 * reference's min/max bookkeeping (ToneMapping.cpp:29-48) changes no pixel. */
void oc_tonemap(float* img, int64_t n, float A, float gamma)
{
    for (int64_t i = 0; i < n; ++i) {
        float* p = img + 4 * i;
        const float l = 0.2126f * p[0] + 0.7152f * p[1] + 0.0722f * p[2];
        const float o = A * powf(l, gamma);
        const float f = l > FLT_EPSILON ? o / l : 1.0f;
        for (int c = 0; c < 3; ++c) p[c] = clamp01(f * p[c]);
        p[3] = 1.0f;
    }
}

static int cmp_float(const void* a, const void* b)
{
    const float x = *(const float*)a, y = *(const float*)b;
    return (x > y) - (x < y);
}

/* median of each channel over the (2 half + 1)^2 window, written for pixels
 * at least `half` from every edge (alpha 1 there); the border keeps its input */
void oc_median(float* img, int w, int h, int half)
{
    const int size = 2 * half + 1, size2 = size * size;
    float* out = (float*)malloc(sizeof(float) * 4 * (size_t)w * h);
    float* win = (float*)malloc(sizeof(float) * size2);
    if (!out || !win) {
        free(out);
        free(win);
        return;
    }
    memcpy(out, img, sizeof(float) * 4 * (size_t)w * h);
    for (int y = half; y < h - half; ++y)
        for (int x = half; x < w - half; ++x) {
            float* o = out + 4 * ((size_t)y * w + x);
            for (int c = 0; c < 3; ++c) {
                int k = 0;
                for (int yy = y - half; yy <= y + half; ++yy)
                    for (int xx = x - half; xx <= x + half; ++xx) win[k++] = img[4 * ((size_t)yy * w + xx) + c];
                qsort(win, size2, sizeof(float), cmp_float);
                o[c] = win[(size2 - 1) / 2];
            }
            o[3] = 1.0f;
        }
    memcpy(img, out, sizeof(float) * 4 * (size_t)w * h);
    free(out);
    free(win);
}

/* unsigned char(255 f) for f in [0, 1]; values outside are clamped (the
 * reference's cast is undefined there and never sees them after tone mapping) */
void oc_rgba8(const float* img, int64_t n, uint8_t* out)
{
    for (int64_t i = 0; i < n; ++i) {
        const float v = 255.0f * img[i];
        out[i] = v >= 255.0f ? 255 : (v > 0.0f ? (uint8_t)v : 0);
    }
}
