// CPU restatement of the caustic compute pass (caustics_compute.wgsl:1-126). TEST INFRASTRUCTURE
// (see oracle.h): it checks the CUDA caustics kernel and is never linked into the product.
// float arithmetic, left to right, no contraction; pow in double rounded to float.
#include <cmath>

#include "oracle.h"

namespace {

float sample(const float *h, size_t pitch, int w, int hgt, int x, int y) {
    int sx = x % w;  // sample_thickness: wrap x, clamp y
    if (sx < 0) sx += w;
    const int sy = y < 0 ? 0 : (y > hgt - 1 ? hgt - 1 : y);
    return h[(size_t)sy * pitch + (size_t)sx];
}

}  // namespace

extern "C" void orc_caustics(const sbs_caustic_params *p, const float *h, size_t pitch, float *out) {
    const int w = (int)p->grid_width, hgt = (int)p->grid_height;
    for (int y = 0; y < hgt; ++y)
        for (int x = 0; x < w; ++x) {
            auto s = [&](int dx, int dy) { return sample(h, pitch, w, hgt, x + dx, y + dy); };
            // thickness_gradient, h = 1
            const float gx = (s(1, 0) - s(-1, 0)) / (2.0f * 1.0f);
            const float gy = (s(0, 1) - s(0, -1)) / (2.0f * 1.0f);
            // thickness_laplacian
            const float c = s(0, 0), l = s(-1, 0), r = s(1, 0), u = s(0, -1), d = s(0, 1);
            const float lap = (l + r + u + d - 4.0f * c) / (1.0f * 1.0f);
            // thickness_hessian_det
            const float d2x = (l + r - 2.0f * c) / (1.0f * 1.0f);
            const float d2y = (u + d - 2.0f * c) / (1.0f * 1.0f);
            const float dxy = (s(1, 1) - s(-1, 1) - s(1, -1) + s(-1, -1)) / (4.0f * (1.0f * 1.0f));
            const float det = d2x * d2y - dxy * dxy;
            const float focusing = 1.0f / std::fmax(std::fabs(1.0f - (-lap * p->focal_length)), 0.01f);
            const float branch = det < -p->branch_threshold ? 1.5f : 1.0f;
            const float refraction = 1.0f + std::sqrt(gx * gx + gy * gy) * 0.5f;
            float it = focusing * branch * refraction;
            it = (float)std::pow((double)it, (double)p->caustic_sharpness);
            it *= p->caustic_intensity;
            out[(size_t)y * w + x] = std::fmin(std::fmax(it, 0.0f), 10.0f);
        }
}
