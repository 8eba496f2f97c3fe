// Headless film shading: the bubble fragment shader (bubble.wgsl) as CUDA kernels.
//
// shade_fragments_kernel evaluates fs_main (bubble.wgsl:486-545) for a batch of fragments
// (normal, world position); shade_frame_kernel produces one frame of the headless renderer
// (render/headless.rs): a ray per pixel through the inverse view-projection, the front surface of
// the bubble sphere as the fragment, alpha blending over the background, sRGB encoding.
//
// Arithmetic follows the WGSL expression by expression in FP32, left to right, with no
// contraction (the library is built with -fmad=false): the simplex noise (Gustavson's 3-D
// simplex, bubble.wgsl:104-180) uses only exact operations on integer-valued floats plus adds
// and multiplies, so it is reproducible bit for bit by a CPU restatement; so are the FBM, the
// drainage and swirl terms (the swirl rotation's cos / sin depend only on the frame time and are
// evaluated once on the host), the LUT sampling and the alpha terms. Transcendental calls remain
// in the gravity ripple (sin), the branched-flow lookup (atan2, acos, pow) and the sRGB encoding
// (pow), and there results agree to the rounding of those functions. pow(x, 1.5) of the edge
// smoothing is evaluated as x * sqrt(x).
//
// The film is FP32-arithmetic bound: five simplex evaluations per fragment (~0.7 kFLOP), 16 B
// (linear f32) or 4 B (sRGB bytes) written per pixel.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "sbs_internal.h"

namespace sbs {
namespace {

constexpr float kLutMaxNm = 2000.f;  // LUT_MAX_THICKNESS_NM (bubble.wgsl:63)

struct ShadeConsts {
    sbs_bubble_uniform u;
    float cam[3];
    float swirl_c, swirl_s;  // cos / sin (film_time * 0.5)
    float inv_vp[16];        // column-major inverse of view_proj (frames)
    float radius;            // sphere radius (frames)
    int has_branched;
};

struct V3 {
    float x, y, z;
};
struct V4 {
    float x, y, z, w;
};

__device__ __forceinline__ float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float dot4(V4 a, V4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
// WGSL % on f32 by 289, i.e. fmodf(x, 289): truncated quotient, result with the sign of x. Every
// argument here is an integer-valued float; below 2^24 the quotient x * (1/289) truncates to the
// exact one or one off, the remainder x - 289 q is exact, and one correction step gives fmodf's
// result bit for bit (copysignf keeps the sign of a zero remainder). Larger magnitudes take fmodf.
__device__ __forceinline__ float mod289(float x) {
    if (!(fabsf(x) < 16777216.f)) return fmodf(x, 289.f);
    const float q = truncf(x * (1.f / 289.f));
    float r = x - q * 289.f;
    if (x >= 0.f) {
        if (r >= 289.f) r -= 289.f;
        else if (r < 0.f) r += 289.f;
    } else {
        if (r <= -289.f) r += 289.f;
        else if (r > 0.f) r -= 289.f;
    }
    return copysignf(r, x);
}
// permute (bubble.wgsl:105-107), one component
__device__ __forceinline__ float permute1(float x) { return mod289((x * 34.f + 1.f) * x); }
// step(edge, x) = x >= edge
__device__ __forceinline__ float step1(float edge, float x) { return x >= edge ? 1.f : 0.f; }
__device__ __forceinline__ float tinv(float r) { return 1.79284291400159f - 0.85373472095314f * r; }

// simplex_noise_3d (bubble.wgsl:113-180)
__device__ float simplex3(V3 v) {
    const float Cx = 1.0f / 6.0f, Cy = 1.0f / 3.0f;
    const float s = v.x * Cy + v.y * Cy + v.z * Cy;  // dot(v, vec3(C.y))
    V3 i{floorf(v.x + s), floorf(v.y + s), floorf(v.z + s)};
    const float t = i.x * Cx + i.y * Cx + i.z * Cx;  // dot(i, vec3(C.x))
    const V3 x0{v.x - i.x + t, v.y - i.y + t, v.z - i.z + t};
    // g = step(x0.yzx, x0.xyz), l = 1 - g, i1 = min(g.xyz, l.zxy), i2 = max(g.xyz, l.zxy)
    const float gx = step1(x0.y, x0.x), gy = step1(x0.z, x0.y), gz = step1(x0.x, x0.z);
    const float lx = 1.f - gx, ly = 1.f - gy, lz = 1.f - gz;
    const V3 i1{fminf(gx, lz), fminf(gy, lx), fminf(gz, ly)};
    const V3 i2{fmaxf(gx, lz), fmaxf(gy, lx), fmaxf(gz, ly)};
    const V3 x1{x0.x - i1.x + Cx, x0.y - i1.y + Cx, x0.z - i1.z + Cx};
    const V3 x2{x0.x - i2.x + Cy, x0.y - i2.y + Cy, x0.z - i2.z + Cy};
    const V3 x3{x0.x - 0.5f, x0.y - 0.5f, x0.z - 0.5f};
    i = V3{mod289(i.x), mod289(i.y), mod289(i.z)};
    // p = permute(permute(permute(i.z + (0, i1.z, i2.z, 1)) + i.y + (0, i1.y, i2.y, 1))
    //                                                       + i.x + (0, i1.x, i2.x, 1))
    V4 p{permute1(i.z + 0.f), permute1(i.z + i1.z), permute1(i.z + i2.z), permute1(i.z + 1.f)};
    p = V4{permute1(p.x + i.y + 0.f), permute1(p.y + i.y + i1.y), permute1(p.z + i.y + i2.y),
           permute1(p.w + i.y + 1.f)};
    p = V4{permute1(p.x + i.x + 0.f), permute1(p.y + i.x + i1.x), permute1(p.z + i.x + i2.x),
           permute1(p.w + i.x + 1.f)};
    // ns = n_ * D.wyz - D.xzx with D = (0, 0.5, 1, 2)
    const float n_ = 0.142857142857f;
    const float nsx = n_ * 2.f - 0.f, nsy = n_ * 0.5f - 1.f, nsz = n_ * 1.f - 0.f;
    const float pv[4] = {p.x, p.y, p.z, p.w};
    float xv[4], yv[4], hv[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float j = pv[k] - 49.f * floorf(pv[k] * nsz * nsz);
        const float x_ = floorf(j * nsz);
        const float y_ = floorf(j - 7.f * x_);
        xv[k] = x_ * nsx + nsy;
        yv[k] = y_ * nsx + nsy;
        hv[k] = 1.f - fabsf(xv[k]) - fabsf(yv[k]);
    }
    // b0 = (x.xy, y.xy), b1 = (x.zw, y.zw); s = floor(b) * 2 + 1; sh = -step(h, 0)
    const V4 b0{xv[0], xv[1], yv[0], yv[1]}, b1{xv[2], xv[3], yv[2], yv[3]};
    const V4 s0{floorf(b0.x) * 2.f + 1.f, floorf(b0.y) * 2.f + 1.f, floorf(b0.z) * 2.f + 1.f, floorf(b0.w) * 2.f + 1.f};
    const V4 s1{floorf(b1.x) * 2.f + 1.f, floorf(b1.y) * 2.f + 1.f, floorf(b1.z) * 2.f + 1.f, floorf(b1.w) * 2.f + 1.f};
    const V4 sh{-step1(hv[0], 0.f), -step1(hv[1], 0.f), -step1(hv[2], 0.f), -step1(hv[3], 0.f)};
    // a0 = b0.xzyw + s0.xzyw * sh.xxyy, a1 = b1.xzyw + s1.xzyw * sh.zzww
    const V4 a0{b0.x + s0.x * sh.x, b0.z + s0.z * sh.x, b0.y + s0.y * sh.y, b0.w + s0.w * sh.y};
    const V4 a1{b1.x + s1.x * sh.z, b1.z + s1.z * sh.z, b1.y + s1.y * sh.w, b1.w + s1.w * sh.w};
    V3 p0{a0.x, a0.y, hv[0]}, p1{a0.z, a0.w, hv[1]}, p2{a1.x, a1.y, hv[2]}, p3{a1.z, a1.w, hv[3]};
    const float n0 = tinv(dot3(p0, p0)), n1 = tinv(dot3(p1, p1)), n2 = tinv(dot3(p2, p2)), n3 = tinv(dot3(p3, p3));
    p0 = V3{p0.x * n0, p0.y * n0, p0.z * n0};
    p1 = V3{p1.x * n1, p1.y * n1, p1.z * n1};
    p2 = V3{p2.x * n2, p2.y * n2, p2.z * n2};
    p3 = V3{p3.x * n3, p3.y * n3, p3.z * n3};
    V4 m{fmaxf(0.6f - dot3(x0, x0), 0.f), fmaxf(0.6f - dot3(x1, x1), 0.f), fmaxf(0.6f - dot3(x2, x2), 0.f),
         fmaxf(0.6f - dot3(x3, x3), 0.f)};
    m = V4{m.x * m.x, m.y * m.y, m.z * m.z, m.w * m.w};
    const V4 mm{m.x * m.x, m.y * m.y, m.z * m.z, m.w * m.w};
    return 42.f * dot4(mm, V4{dot3(p0, x0), dot3(p1, x1), dot3(p2, x2), dot3(p3, x3)});
}

// fbm_noise (bubble.wgsl:183-195)
__device__ float fbm4(V3 p) {
    float value = 0.f, amplitude = 0.5f, frequency = 1.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        value += amplitude * simplex3(V3{p.x * frequency, p.y * frequency, p.z * frequency});
        amplitude *= 0.5f;
        frequency *= 2.f;
    }
    return value;
}

// get_film_thickness (bubble.wgsl:203-229)
__device__ float film_thickness(V3 n, const ShadeConsts &c) {
    const sbs_bubble_uniform &u = c.u;
    const float base = u.base_thickness_nm, t = u.film_time, scale = u.pattern_scale, swirl = u.swirl_intensity;
    const float drain_progress = fminf(t * u.drainage_speed * 0.1f, 1.f);
    const float drainage = 0.4f * (1.f - n.y) * 0.5f * (1.f + drain_progress);
    const float nt = t * 0.08f;
    const V3 nc{n.x * scale * 3.f + nt, n.y * scale * 3.f + nt * 0.7f, n.z * scale * 3.f + nt * 0.5f};
    const float organic = fbm4(nc) * swirl * 0.12f;
    const float sx = n.x * c.swirl_c - n.z * c.swirl_s;
    const float sz = n.x * c.swirl_s + n.z * c.swirl_c;
    const float ts = t * 0.2f;
    const float swirl_noise = simplex3(V3{sx * 5.f + ts, n.y * 5.f + ts, sz * 5.f + ts}) * swirl * 0.05f;
    const float wave = 0.02f * swirl * sinf(n.y * scale * 8.f - t * 2.f) * (1.f - fabsf(n.y));
    return base * (1.f - drainage + organic + swirl_noise - wave);
}

// mix(a, b, t) = a (1 - t) + b t
__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.f - t) + b * t; }

// Bilinear sample of the RGBA8 LUT ([64 rows: cos][256 columns: thickness]) at (u, v) in [0, 1]:
// texel centres at (k + 0.5) / size, clamp to edge (pipeline.rs:350-359).
__device__ V3 sample_lut(const uint8_t *__restrict__ lut, float uu, float vv) {
    const float x = uu * (float)SBS_LUT_THICKNESSES - 0.5f, y = vv * (float)SBS_LUT_ANGLES - 0.5f;
    const float fx0 = floorf(x), fy0 = floorf(y);
    const float tx = x - fx0, ty = y - fy0;
    const int x0 = min(max((int)fx0, 0), SBS_LUT_THICKNESSES - 1), x1 = min(max((int)fx0 + 1, 0), SBS_LUT_THICKNESSES - 1);
    const int y0 = min(max((int)fy0, 0), SBS_LUT_ANGLES - 1), y1 = min(max((int)fy0 + 1, 0), SBS_LUT_ANGLES - 1);
    const uchar4 c00 = __ldg(reinterpret_cast<const uchar4 *>(lut) + y0 * SBS_LUT_THICKNESSES + x0);
    const uchar4 c10 = __ldg(reinterpret_cast<const uchar4 *>(lut) + y0 * SBS_LUT_THICKNESSES + x1);
    const uchar4 c01 = __ldg(reinterpret_cast<const uchar4 *>(lut) + y1 * SBS_LUT_THICKNESSES + x0);
    const uchar4 c11 = __ldg(reinterpret_cast<const uchar4 *>(lut) + y1 * SBS_LUT_THICKNESSES + x1);
    const float k = 1.f / 255.f;
    V3 r;
    r.x = mixf(mixf(c00.x * k, c10.x * k, tx), mixf(c01.x * k, c11.x * k, tx), ty);
    r.y = mixf(mixf(c00.y * k, c10.y * k, tx), mixf(c01.y * k, c11.y * k, tx), ty);
    r.z = mixf(mixf(c00.z * k, c10.z * k, tx), mixf(c01.z * k, c11.z * k, tx), ty);
    return r;
}

// compute_branched_flow (bubble.wgsl:329-355) with its texture lookup (:240-279) and patch
// mapping (:282-303)
__device__ float branched_flow(V3 n, const uint32_t *__restrict__ tex, const sbs_bubble_uniform &u) {
    const float PI = 3.14159265f;
    const float phi = atan2f(n.z, n.x);
    const float theta = acosf(fminf(fmaxf(n.y, -1.f), 1.f));
    float su = (phi + PI) / (2.f * PI), sv = theta / PI;
    if (u.patch_enabled != 0u) {
        const float du = fabsf(su - u.patch_center_u), dv = fabsf(sv - u.patch_center_v);
        if (!(du <= u.patch_half_size && dv <= u.patch_half_size)) return 0.f;
        const float min_u = fmaxf(u.patch_center_u - u.patch_half_size, 0.f);
        const float max_u = fminf(u.patch_center_u + u.patch_half_size, 1.f);
        const float min_v = fmaxf(u.patch_center_v - u.patch_half_size, 0.f);
        const float max_v = fminf(u.patch_center_v + u.patch_half_size, 1.f);
        const float lu = (su - min_u) / fmaxf(max_u - min_u, 0.001f);
        const float lv = (sv - min_v) / fmaxf(max_v - min_v, 0.001f);
        su = fminf(fmaxf(lu, 0.f), 1.f);
        sv = fminf(fmaxf(lv, 0.f), 1.f);
    }
    const float fx = su * (float)(SBS_BRANCHED_W - 1), fy = sv * (float)(SBS_BRANCHED_H - 1);
    const int x0 = (int)floorf(fx), y0 = (int)floorf(fy);
    const float tx = fx - (float)x0, ty = fy - (float)y0;
    const int W = SBS_BRANCHED_W, H = SBS_BRANCHED_H;
    const int sx0 = ((x0 % W) + W) % W, sx1 = (((x0 + 1) % W) + W) % W;
    const int sy0 = min(max(y0, 0), H - 1), sy1 = min(max(y0 + 1, 0), H - 1);
    const float c00 = (float)__ldg(tex + sy0 * W + sx0) / 256.f, c10 = (float)__ldg(tex + sy0 * W + sx1) / 256.f;
    const float c01 = (float)__ldg(tex + sy1 * W + sx0) / 256.f, c11 = (float)__ldg(tex + sy1 * W + sx1) / 256.f;
    float it = mixf(mixf(c00, c10, tx), mixf(c01, c11, tx), ty);
    it *= u.branched_flow_intensity;
    it = powf(it, u.branched_flow_sharpness);
    return fminf(fmaxf(it, 0.f), 3.f);
}

// fs_main (bubble.wgsl:486-545): straight-alpha colour of one fragment
__device__ float4 shade(V3 nin, V3 wp, const ShadeConsts &c, const uint8_t *__restrict__ lut,
                        const uint32_t *__restrict__ branched) {
    const sbs_bubble_uniform &u = c.u;
    const float nl = sqrtf(dot3(nin, nin));
    const V3 n{nin.x / nl, nin.y / nl, nin.z / nl};
    const V3 vd0{c.cam[0] - wp.x, c.cam[1] - wp.y, c.cam[2] - wp.z};
    const float vl = sqrtf(dot3(vd0, vd0));
    const V3 vd{vd0.x / vl, vd0.y / vl, vd0.z / vl};
    const float cos_theta = fabsf(dot3(vd, n));
    const float thickness = film_thickness(n, c);
    const float edge = 1.f - cos_theta;
    float smooth_edge;
    if (u.edge_smoothing_mode == 1u)
        smooth_edge = edge * edge * (3.f - 2.f * edge);
    else if (u.edge_smoothing_mode == 2u)
        smooth_edge = edge * sqrtf(edge);
    else
        smooth_edge = edge;
    const float alpha = u.base_alpha + u.edge_alpha * smooth_edge;
    if (thickness < 30.f) return make_float4(0.02f, 0.02f, 0.02f, alpha * 0.5f);
    const V3 lc = sample_lut(lut, fminf(fmaxf(thickness / kLutMaxNm, 0.f), 1.f), fminf(fmaxf(cos_theta, 0.f), 1.f));
    const float ii = u.interference_intensity;
    const V3 ic{fminf(fmaxf(lc.x * ii, 0.f), 1.f), fminf(fmaxf(lc.y * ii, 0.f), 1.f), fminf(fmaxf(lc.z * ii, 0.f), 1.f)};
    V3 fc{0.95f * 0.1f + ic.x, 0.97f * 0.1f + ic.y, 1.0f * 0.1f + ic.z};
    if (u.branched_flow_enabled != 0u && c.has_branched) {
        const float bf = branched_flow(n, branched, u);
        if (bf > 0.f) fc = V3{fc.x + 1.0f * bf, fc.y + 0.95f * bf, fc.z + 0.85f * bf};
    }
    return make_float4(fc.x, fc.y, fc.z, alpha);
}

__global__ void shade_fragments_kernel(ShadeConsts c, const uint8_t *__restrict__ lut,
                                       const uint32_t *__restrict__ branched, size_t n, const float *__restrict__ normal,
                                       const float *__restrict__ wpos, float4 *__restrict__ out) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const V3 nn{normal[3 * k], normal[3 * k + 1], normal[3 * k + 2]};
    const V3 wp{wpos[3 * k], wpos[3 * k + 1], wpos[3 * k + 2]};
    out[k] = shade(nn, wp, c, lut, branched);
}

// linear -> sRGB byte as an Rgba8UnormSrgb target stores it
__device__ __forceinline__ uint8_t srgb8(float x) {
    x = fminf(fmaxf(x, 0.f), 1.f);
    const float e = x <= 0.0031308f ? 12.92f * x : 1.055f * powf(x, 1.f / 2.4f) - 0.055f;
    return (uint8_t)__float2int_rn(e * 255.f);
}

// M (column-major) times (x, y, z, 1)
__device__ __forceinline__ V4 xform(const float *m, float x, float y, float z) {
    return V4{m[0] * x + m[4] * y + m[8] * z + m[12], m[1] * x + m[5] * y + m[9] * z + m[13],
              m[2] * x + m[6] * y + m[10] * z + m[14], m[3] * x + m[7] * y + m[11] * z + m[15]};
}

// One pixel per thread, a 16 x 16 tile per block.
__global__ void __launch_bounds__(256) shade_frame_kernel(ShadeConsts c, const uint8_t *__restrict__ lut,
                                                          const uint32_t *__restrict__ branched, uint32_t width,
                                                          uint32_t height, uchar4 *__restrict__ rgba8,
                                                          float4 *__restrict__ linear) {
    const uint32_t px = blockIdx.x * 16 + (threadIdx.x & 15), py = blockIdx.y * 16 + (threadIdx.x >> 4);
    if (px >= width || py >= height) return;
    const sbs_bubble_uniform &u = c.u;
    // pixel centre in wgpu NDC (y up), unprojected on the far plane
    const float ndx = 2.f * ((float)px + 0.5f) / (float)width - 1.f;
    const float ndy = 1.f - 2.f * ((float)py + 0.5f) / (float)height;
    const V4 f = xform(c.inv_vp, ndx, ndy, 1.f);
    const V3 far{f.x / f.w, f.y / f.w, f.z / f.w};
    const V3 o{c.cam[0], c.cam[1], c.cam[2]};
    V3 d{far.x - o.x, far.y - o.y, far.z - o.z};
    const float dl = sqrtf(dot3(d, d));
    d = V3{d.x / dl, d.y / dl, d.z / dl};
    // nearest intersection with |x - centre| = radius
    const V3 oc{o.x - u.position_x, o.y - u.position_y, o.z - u.position_z};
    const float b = dot3(oc, d), cc = dot3(oc, oc) - c.radius * c.radius;
    const float disc = b * b - cc;
    float4 col = make_float4(u.background_r, u.background_g, u.background_b, 1.f);
    if (disc >= 0.f) {
        const float sq = sqrtf(disc);
        float t = -b - sq;
        if (t <= 0.f) t = -b + sq;
        if (t > 0.f) {
            const V3 hit{o.x + d.x * t, o.y + d.y * t, o.z + d.z * t};
            const V3 nrm{(hit.x - u.position_x) / c.radius, (hit.y - u.position_y) / c.radius,
                         (hit.z - u.position_z) / c.radius};
            const float4 s = shade(nrm, hit, c, lut, branched);
            const float a = fminf(fmaxf(s.w, 0.f), 1.f);
            const float r = fminf(fmaxf(s.x, 0.f), 1.f), g = fminf(fmaxf(s.y, 0.f), 1.f), bb = fminf(fmaxf(s.z, 0.f), 1.f);
            // BlendState::ALPHA_BLENDING: colour src a + dst (1 - a); alpha src + dst (1 - a)
            col = make_float4(r * a + col.x * (1.f - a), g * a + col.y * (1.f - a), bb * a + col.z * (1.f - a),
                              a + 1.f * (1.f - a));
        }
    }
    const size_t idx = (size_t)py * width + px;
    if (linear) linear[idx] = col;
    if (rgba8) rgba8[idx] = make_uchar4(srgb8(col.x), srgb8(col.y), srgb8(col.z), (uint8_t)__float2int_rn(fminf(fmaxf(col.w, 0.f), 1.f) * 255.f));
}

// 4 x 4 inverse in double (column-major), false when singular
bool invert4(const float *m, float *out) {
    double a[16], inv[16];
    for (int k = 0; k < 16; ++k) a[k] = m[k];
    inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    const double det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
    if (!(std::fabs(det) > 0.0) || !std::isfinite(det)) return false;
    for (int k = 0; k < 16; ++k) out[k] = (float)(inv[k] / det);
    return true;
}

ShadeConsts make_consts(const sbs_bubble_uniform *u, const float cam[3], int has_branched) {
    ShadeConsts c;
    std::memset(&c, 0, sizeof(c));
    c.u = *u;
    for (int k = 0; k < 3; ++k) c.cam[k] = cam[k];
    const double ang = (double)(u->film_time * 0.5f);
    c.swirl_c = (float)std::cos(ang);
    c.swirl_s = (float)std::sin(ang);
    c.has_branched = has_branched;
    return c;
}

}  // namespace
}  // namespace sbs

using namespace sbs;

extern "C" {

int sbs_bubble_uniform_default(sbs_bubble_uniform *out) {
    clear_error();
    SBS_CHECK_ARG(out != nullptr, "out is null");
    std::memset(out, 0, sizeof(*out));
    out->refractive_index = 1.33f;
    out->base_thickness_nm = 500.f;
    out->interference_intensity = 4.f;
    out->base_alpha = 0.3f;
    out->edge_alpha = 0.6f;
    out->background_r = 0.1f;
    out->background_g = 0.1f;
    out->background_b = 0.15f;
    out->swirl_intensity = 1.f;
    out->drainage_speed = 0.5f;
    out->pattern_scale = 1.f;
    out->edge_smoothing_mode = 1;
    out->branched_flow_intensity = 1.f;
    out->branched_flow_scale = 5.f;
    out->branched_flow_sharpness = 2.f;
    out->light_dir_x = 0.577f;
    out->light_dir_y = 0.577f;
    out->light_dir_z = 0.577f;
    out->patch_enabled = 1;
    out->patch_center_u = 0.5f;
    out->patch_center_v = 0.5f;
    out->patch_half_size = 0.158f;
    return SBS_OK;
}

int sbs_shade_fragments(const sbs_bubble_uniform *u, const float camera_pos[3], const uint8_t *lut,
                        const uint32_t *branched, size_t n, const float *normal, const float *world_pos, float *rgba,
                        int mem, void *stream) {
    clear_error();
    SBS_CHECK_ARG(u != nullptr && camera_pos != nullptr && lut != nullptr, "null uniform, camera or LUT");
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "bad mem flag %d", mem);
    SBS_CHECK_ARG(u->edge_smoothing_mode <= 2u, "edge_smoothing_mode must be 0, 1 or 2");
    if (n == 0) return SBS_OK;
    SBS_CHECK_ARG(normal && world_pos && rgba, "null pointer");
    int rc = require_device();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const ShadeConsts c = make_consts(u, camera_pos, branched != nullptr);
    const size_t lut_b = (size_t)SBS_LUT_ANGLES * SBS_LUT_THICKNESSES * 4;
    const size_t br_b = branched ? (size_t)SBS_BRANCHED_W * SBS_BRANCHED_H * 4 : 0;
    const uint8_t *dl = lut;
    const uint32_t *db = branched;
    const float *dn = normal, *dw = world_pos;
    float *dout = rgba;
    char *base = nullptr;
    if (mem == SBS_MEM_HOST) {
        const size_t bytes = lut_b + br_b + 6 * n * sizeof(float) + 4 * n * sizeof(float) + 256;
        SBS_CUDA_TRY(scratch_alloc((void **)&base, bytes, s));
        char *q = base;
        cudaError_t e = cudaMemcpyAsync(q, lut, lut_b, cudaMemcpyHostToDevice, s);
        dl = (const uint8_t *)q;
        q += lut_b;
        if (e == cudaSuccess && branched) e = cudaMemcpyAsync(q, branched, br_b, cudaMemcpyHostToDevice, s);
        db = branched ? (const uint32_t *)q : nullptr;
        q += br_b;
        q = (char *)(((uintptr_t)q + 15) & ~(uintptr_t)15);
        if (e == cudaSuccess) e = cudaMemcpyAsync(q, normal, 3 * n * sizeof(float), cudaMemcpyHostToDevice, s);
        dn = (const float *)q;
        q += 3 * n * sizeof(float);
        if (e == cudaSuccess) e = cudaMemcpyAsync(q, world_pos, 3 * n * sizeof(float), cudaMemcpyHostToDevice, s);
        dw = (const float *)q;
        q += 3 * n * sizeof(float);
        q = (char *)(((uintptr_t)q + 15) & ~(uintptr_t)15);
        dout = (float *)q;
        if (e != cudaSuccess) {
            cudaFreeAsync(base, s);
            return set_error(SBS_E_CUDA, "shade: upload failed: %s", cudaGetErrorString(e));
        }
    } else {
        SBS_CHECK_ARG(((uintptr_t)rgba & 15) == 0, "rgba must be 16-byte aligned");
        SBS_CHECK_ARG(((uintptr_t)lut & 3) == 0 && ((uintptr_t)branched & 3) == 0, "textures must be 4-byte aligned");
    }
    shade_fragments_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(c, dl, db, n, dn, dw,
                                                                     reinterpret_cast<float4 *>(dout));
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && mem == SBS_MEM_HOST)
        e = cudaMemcpyAsync(rgba, dout, 4 * n * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (base) cudaFreeAsync(base, s);
    if (e == cudaSuccess && mem == SBS_MEM_HOST) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(SBS_E_CUDA, "shade: %s", cudaGetErrorString(e));
    return SBS_OK;
}

int sbs_shade_frame(const sbs_bubble_uniform *u, const float view_proj[16], const float camera_pos[3], float radius,
                    const uint8_t *lut, const uint32_t *branched, uint32_t width, uint32_t height, uint8_t *rgba8,
                    float *linear, int mem, void *stream) {
    clear_error();
    SBS_CHECK_ARG(u != nullptr && view_proj != nullptr && camera_pos != nullptr && lut != nullptr,
                  "null uniform, matrix, camera or LUT");
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "bad mem flag %d", mem);
    SBS_CHECK_ARG(u->edge_smoothing_mode <= 2u, "edge_smoothing_mode must be 0, 1 or 2");
    SBS_CHECK_ARG(radius > 0.f && std::isfinite(radius), "radius must be positive");
    SBS_CHECK_ARG(width >= 1 && height >= 1 && width <= 32768 && height <= 32768, "frame size out of range");
    if (!rgba8 && !linear) return SBS_OK;
    int rc = require_device();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    ShadeConsts c = make_consts(u, camera_pos, branched != nullptr);
    c.radius = radius;
    SBS_CHECK_ARG(invert4(view_proj, c.inv_vp), "view_proj is singular");
    const size_t px = (size_t)width * height;
    const size_t lut_b = (size_t)SBS_LUT_ANGLES * SBS_LUT_THICKNESSES * 4;
    const size_t br_b = branched ? (size_t)SBS_BRANCHED_W * SBS_BRANCHED_H * 4 : 0;
    const uint8_t *dl = lut;
    const uint32_t *db = branched;
    uchar4 *d8 = reinterpret_cast<uchar4 *>(rgba8);
    float4 *dlin = reinterpret_cast<float4 *>(linear);
    char *base = nullptr;
    if (mem == SBS_MEM_HOST) {
        const size_t bytes = lut_b + br_b + (rgba8 ? 4 * px : 0) + (linear ? 16 * px : 0) + 512;
        SBS_CUDA_TRY(scratch_alloc((void **)&base, bytes, s));
        char *q = base;
        cudaError_t e = cudaMemcpyAsync(q, lut, lut_b, cudaMemcpyHostToDevice, s);
        dl = (const uint8_t *)q;
        q += lut_b;
        if (e == cudaSuccess && branched) e = cudaMemcpyAsync(q, branched, br_b, cudaMemcpyHostToDevice, s);
        db = branched ? (const uint32_t *)q : nullptr;
        q += br_b;
        q = (char *)(((uintptr_t)q + 15) & ~(uintptr_t)15);
        d8 = rgba8 ? (uchar4 *)q : nullptr;
        q += rgba8 ? 4 * px : 0;
        q = (char *)(((uintptr_t)q + 15) & ~(uintptr_t)15);
        dlin = linear ? (float4 *)q : nullptr;
        if (e != cudaSuccess) {
            cudaFreeAsync(base, s);
            return set_error(SBS_E_CUDA, "shade: upload failed: %s", cudaGetErrorString(e));
        }
    } else {
        SBS_CHECK_ARG(((uintptr_t)rgba8 & 3) == 0 && ((uintptr_t)linear & 15) == 0, "output arrays misaligned");
        SBS_CHECK_ARG(((uintptr_t)lut & 3) == 0 && ((uintptr_t)branched & 3) == 0, "textures must be 4-byte aligned");
    }
    const dim3 grid((width + 15) / 16, (height + 15) / 16);
    shade_frame_kernel<<<grid, 256, 0, s>>>(c, dl, db, width, height, d8, dlin);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && mem == SBS_MEM_HOST && rgba8)
        e = cudaMemcpyAsync(rgba8, d8, 4 * px, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && mem == SBS_MEM_HOST && linear)
        e = cudaMemcpyAsync(linear, dlin, 16 * px, cudaMemcpyDeviceToHost, s);
    if (base) cudaFreeAsync(base, s);
    if (e == cudaSuccess && mem == SBS_MEM_HOST) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(SBS_E_CUDA, "shade: %s", cudaGetErrorString(e));
    return SBS_OK;
}

}  // extern "C"
