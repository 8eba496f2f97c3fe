// The per-cell arithmetic of the caustic compute pass (caustics_compute.wgsl:29-111), shared by
// the standalone caustic kernel (caustics.cu) and the drainage launch that writes the map of its
// result (drainage_wtb.cu), so both give the same bits. The library is compiled without FMA
// contraction, so the expressions round left to right as written.
#pragma once

#include <cuda_runtime.h>

#include "../../include/sbs.h"

namespace sbs {

// One row of the 3 x 3 neighbourhood: left, centre, right (phi - 1, phi, phi + 1).
struct CausticRow {
    float l, c, r;
};

// pow(x, y) for x > 0 through the special-function unit: 2^(y log2 x) with the hardware base-2
// logarithm and exponential (each ~2^-22 relative), i.e. well below 1e-6 relative for the
// exponents and magnitudes of this pass.
__device__ __forceinline__ float pow_sfu(float x, float y) {
    float l, r;
    asm("lg2.approx.f32 %0, %1;" : "=f"(l) : "f"(x));
    const float e = y * l;
    asm("ex2.approx.f32 %0, %1;" : "=f"(r) : "f"(e));
    return r;
}

__device__ __forceinline__ CausticRow caustic_load_row(const float *__restrict__ h, size_t pitch, int H, int y,
                                                       int xl, int x, int xr) {
    const float *p = h + (size_t)min(max(y, 0), H - 1) * pitch;  // theta clamped
    return CausticRow{__ldg(p + xl), __ldg(p + x), __ldg(p + xr)};
}

// compute_caustic_intensity (caustics_compute.wgsl:87-111) from the 3 x 3 neighbourhood:
// a = row above (y - 1), b = the cell's row, c = row below (y + 1)
__device__ __forceinline__ float caustic_intensity(float focal_length, float intensity, float sharpness,
                                                   float branch_threshold, CausticRow a, CausticRow b, CausticRow c) {
    const float center = b.c, left = b.l, right = b.r, up = a.c, down = c.c;
    const float ul = a.l, ur = a.r, dl = c.l, dr = c.r;
    // thickness_gradient (h = 1)
    const float gx = (right - left) / 2.0f, gy = (down - up) / 2.0f;
    // thickness_laplacian
    const float lap = (left + right + up + down - 4.0f * center) / 1.0f;
    // thickness_hessian_det
    const float d2x = (left + right - 2.0f * center) / 1.0f;
    const float d2y = (up + down - 2.0f * center) / 1.0f;
    const float dxy = (dr - dl - ur + ul) / 4.0f;
    const float hdet = d2x * d2y - dxy * dxy;
    const float curvature = -lap * focal_length;
    const float focusing = 1.0f / fmaxf(fabsf(1.0f - curvature), 0.01f);
    const float branch = hdet < -branch_threshold ? 1.5f : 1.0f;
    const float gmag = sqrtf(gx * gx + gy * gy);
    const float refraction = 1.0f + gmag * 0.5f;
    float it = focusing * branch * refraction;
    it = pow_sfu(it, sharpness);  // it >= 0.01 (the focusing clamp keeps it positive)
    it *= intensity;
    return fminf(fmaxf(it, 0.0f), 10.0f);
}

}  // namespace sbs
