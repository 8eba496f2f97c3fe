// CPU restatement of the bubble fragment shader (bubble.wgsl) and of one headless frame
// (render/headless.rs). TEST INFRASTRUCTURE (see oracle.h): it checks the CUDA shading kernels and
// is never linked into the product.
//
// Every WGSL expression is evaluated in float, left to right, without contraction (this file is
// built with -ffp-contract=off): simplex_noise_3d bubble.wgsl:113-180, fbm_noise :183-195,
// get_film_thickness :203-229, sample_branched_flow_texture :240-279, is_in_patch /
// uv_to_patch_local :282-303, compute_branched_flow :329-355, thin_film_interference :445-461 with
// the sampler of pipeline.rs:350-359 (bilinear, clamp to edge, texel centres), fs_main :486-545.
// pow(x, 1.5) of the edge smoothing is x * sqrt(x); cos / sin of the swirl angle are taken in
// double once per frame. The frame: a ray per pixel centre through the inverse view-projection,
// the nearest front intersection with the sphere, BlendState::ALPHA_BLENDING over the clear
// colour (alpha 1), sRGB encoding of an Rgba8UnormSrgb store.
#include <cmath>
#include <cstring>

#include "oracle.h"

namespace {

struct V3 {
    float x, y, z;
};

float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
float fmod289(float x) { return std::fmod(x, 289.0f); }
float permute(float x) { return fmod289((x * 34.0f + 1.0f) * x); }
float stepf(float edge, float x) { return x >= edge ? 1.0f : 0.0f; }

float simplex(V3 v) {
    const float cx = 1.0f / 6.0f, cy = 1.0f / 3.0f;
    const float s = v.x * cy + v.y * cy + v.z * cy;
    float ix = std::floor(v.x + s), iy = std::floor(v.y + s), iz = std::floor(v.z + s);
    const float t = ix * cx + iy * cx + iz * cx;
    const V3 x0{v.x - ix + t, v.y - iy + t, v.z - iz + t};
    const float g[3] = {stepf(x0.y, x0.x), stepf(x0.z, x0.y), stepf(x0.x, x0.z)};
    const float l[3] = {1.0f - g[0], 1.0f - g[1], 1.0f - g[2]};
    // l.zxy = (l[2], l[0], l[1])
    const float i1[3] = {std::fmin(g[0], l[2]), std::fmin(g[1], l[0]), std::fmin(g[2], l[1])};
    const float i2[3] = {std::fmax(g[0], l[2]), std::fmax(g[1], l[0]), std::fmax(g[2], l[1])};
    const V3 x1{x0.x - i1[0] + cx, x0.y - i1[1] + cx, x0.z - i1[2] + cx};
    const V3 x2{x0.x - i2[0] + cy, x0.y - i2[1] + cy, x0.z - i2[2] + cy};
    const V3 x3{x0.x - 0.5f, x0.y - 0.5f, x0.z - 0.5f};
    ix = fmod289(ix);
    iy = fmod289(iy);
    iz = fmod289(iz);
    const float oz[4] = {0.0f, i1[2], i2[2], 1.0f}, oy[4] = {0.0f, i1[1], i2[1], 1.0f}, ox[4] = {0.0f, i1[0], i2[0], 1.0f};
    float p[4];
    for (int k = 0; k < 4; ++k) p[k] = permute(iz + oz[k]);
    for (int k = 0; k < 4; ++k) p[k] = permute(p[k] + iy + oy[k]);
    for (int k = 0; k < 4; ++k) p[k] = permute(p[k] + ix + ox[k]);
    const float n_ = 0.142857142857f;
    // ns = n_ * D.wyz - D.xzx, D = (0, 0.5, 1, 2)
    const float nsx = n_ * 2.0f - 0.0f, nsy = n_ * 0.5f - 1.0f, nsz = n_ * 1.0f - 0.0f;
    float x[4], y[4], h[4];
    for (int k = 0; k < 4; ++k) {
        const float j = p[k] - 49.0f * std::floor(p[k] * nsz * nsz);
        const float xx = std::floor(j * nsz);
        const float yy = std::floor(j - 7.0f * xx);
        x[k] = xx * nsx + nsy;
        y[k] = yy * nsx + nsy;
        h[k] = 1.0f - std::fabs(x[k]) - std::fabs(y[k]);
    }
    const float b0[4] = {x[0], x[1], y[0], y[1]}, b1[4] = {x[2], x[3], y[2], y[3]};
    float s0[4], s1[4], sh[4];
    for (int k = 0; k < 4; ++k) {
        s0[k] = std::floor(b0[k]) * 2.0f + 1.0f;
        s1[k] = std::floor(b1[k]) * 2.0f + 1.0f;
        sh[k] = -stepf(h[k], 0.0f);
    }
    // a0 = b0.xzyw + s0.xzyw * sh.xxyy; a1 = b1.xzyw + s1.xzyw * sh.zzww
    const int sw[4] = {0, 2, 1, 3};
    const int s0i[4] = {0, 0, 1, 1}, s1i[4] = {2, 2, 3, 3};
    float a0[4], a1[4];
    for (int k = 0; k < 4; ++k) {
        a0[k] = b0[sw[k]] + s0[sw[k]] * sh[s0i[k]];
        a1[k] = b1[sw[k]] + s1[sw[k]] * sh[s1i[k]];
    }
    V3 g0{a0[0], a0[1], h[0]}, g1{a0[2], a0[3], h[1]}, g2{a1[0], a1[1], h[2]}, g3{a1[2], a1[3], h[3]};
    auto tis = [](float r) { return 1.79284291400159f - 0.85373472095314f * r; };
    const float q0 = tis(dot3(g0, g0)), q1 = tis(dot3(g1, g1)), q2 = tis(dot3(g2, g2)), q3 = tis(dot3(g3, g3));
    g0 = V3{g0.x * q0, g0.y * q0, g0.z * q0};
    g1 = V3{g1.x * q1, g1.y * q1, g1.z * q1};
    g2 = V3{g2.x * q2, g2.y * q2, g2.z * q2};
    g3 = V3{g3.x * q3, g3.y * q3, g3.z * q3};
    float m[4] = {std::fmax(0.6f - dot3(x0, x0), 0.0f), std::fmax(0.6f - dot3(x1, x1), 0.0f),
                  std::fmax(0.6f - dot3(x2, x2), 0.0f), std::fmax(0.6f - dot3(x3, x3), 0.0f)};
    for (int k = 0; k < 4; ++k) m[k] = m[k] * m[k];
    const float mm[4] = {m[0] * m[0], m[1] * m[1], m[2] * m[2], m[3] * m[3]};
    const float d[4] = {dot3(g0, x0), dot3(g1, x1), dot3(g2, x2), dot3(g3, x3)};
    return 42.0f * (mm[0] * d[0] + mm[1] * d[1] + mm[2] * d[2] + mm[3] * d[3]);
}

float fbm(V3 p) {
    float value = 0.0f, amplitude = 0.5f, frequency = 1.0f;
    for (int i = 0; i < 4; ++i) {
        value += amplitude * simplex(V3{p.x * frequency, p.y * frequency, p.z * frequency});
        amplitude *= 0.5f;
        frequency *= 2.0f;
    }
    return value;
}

struct Frame {
    const sbs_bubble_uniform *u;
    float sc, ss;  // cos / sin (film_time * 0.5)
};

Frame frame_of(const sbs_bubble_uniform *u) {
    const double a = (double)(u->film_time * 0.5f);
    return Frame{u, (float)std::cos(a), (float)std::sin(a)};
}

float thickness(V3 n, const Frame &f) {
    const sbs_bubble_uniform &u = *f.u;
    const float base = u.base_thickness_nm, t = u.film_time, scale = u.pattern_scale, swirl = u.swirl_intensity;
    const float drain_progress = std::fmin(t * u.drainage_speed * 0.1f, 1.0f);
    const float drainage = 0.4f * (1.0f - n.y) * 0.5f * (1.0f + drain_progress);
    const float nt = t * 0.08f;
    const V3 nc{n.x * scale * 3.0f + nt, n.y * scale * 3.0f + nt * 0.7f, n.z * scale * 3.0f + nt * 0.5f};
    const float organic = fbm(nc) * swirl * 0.12f;
    const float sx = n.x * f.sc - n.z * f.ss;
    const float sz = n.x * f.ss + n.z * f.sc;
    const float ts = t * 0.2f;
    const float swirl_noise = simplex(V3{sx * 5.0f + ts, n.y * 5.0f + ts, sz * 5.0f + ts}) * swirl * 0.05f;
    const float wave =
        0.02f * swirl * (float)std::sin((double)(n.y * scale * 8.0f - t * 2.0f)) * (1.0f - std::fabs(n.y));
    return base * (1.0f - drainage + organic + swirl_noise - wave);
}

float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }

void sample_lut(const uint8_t *lut, float u, float v, float out[3]) {
    const int W = SBS_LUT_THICKNESSES, H = SBS_LUT_ANGLES;
    const float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    const float fx = std::floor(x), fy = std::floor(y);
    const float tx = x - fx, ty = y - fy;
    auto cl = [](int k, int n) { return k < 0 ? 0 : (k > n - 1 ? n - 1 : k); };
    const int x0 = cl((int)fx, W), x1 = cl((int)fx + 1, W), y0 = cl((int)fy, H), y1 = cl((int)fy + 1, H);
    for (int c = 0; c < 3; ++c) {
        const float c00 = lut[(y0 * W + x0) * 4 + c] * (1.0f / 255.0f), c10 = lut[(y0 * W + x1) * 4 + c] * (1.0f / 255.0f);
        const float c01 = lut[(y1 * W + x0) * 4 + c] * (1.0f / 255.0f), c11 = lut[(y1 * W + x1) * 4 + c] * (1.0f / 255.0f);
        out[c] = mixf(mixf(c00, c10, tx), mixf(c01, c11, tx), ty);
    }
}

float branched(V3 n, const uint32_t *tex, const sbs_bubble_uniform &u) {
    const float pi = 3.14159265f;
    const float phi = (float)std::atan2((double)n.z, (double)n.x);
    const float theta = (float)std::acos((double)std::fmin(std::fmax(n.y, -1.0f), 1.0f));
    float su = (phi + pi) / (2.0f * pi), sv = theta / pi;
    if (u.patch_enabled != 0u) {
        const float du = std::fabs(su - u.patch_center_u), dv = std::fabs(sv - u.patch_center_v);
        if (!(du <= u.patch_half_size && dv <= u.patch_half_size)) return 0.0f;
        const float min_u = std::fmax(u.patch_center_u - u.patch_half_size, 0.0f);
        const float max_u = std::fmin(u.patch_center_u + u.patch_half_size, 1.0f);
        const float min_v = std::fmax(u.patch_center_v - u.patch_half_size, 0.0f);
        const float max_v = std::fmin(u.patch_center_v + u.patch_half_size, 1.0f);
        su = std::fmin(std::fmax((su - min_u) / std::fmax(max_u - min_u, 0.001f), 0.0f), 1.0f);
        sv = std::fmin(std::fmax((sv - min_v) / std::fmax(max_v - min_v, 0.001f), 0.0f), 1.0f);
    }
    const int W = SBS_BRANCHED_W, H = SBS_BRANCHED_H;
    const float fx = su * (float)(W - 1), fy = sv * (float)(H - 1);
    const int x0 = (int)std::floor(fx), y0 = (int)std::floor(fy);
    const float tx = fx - (float)x0, ty = fy - (float)y0;
    const int sx0 = ((x0 % W) + W) % W, sx1 = (((x0 + 1) % W) + W) % W;
    auto cl = [](int k, int n) { return k < 0 ? 0 : (k > n - 1 ? n - 1 : k); };
    const int sy0 = cl(y0, H), sy1 = cl(y0 + 1, H);
    const float c00 = (float)tex[sy0 * W + sx0] / 256.0f, c10 = (float)tex[sy0 * W + sx1] / 256.0f;
    const float c01 = (float)tex[sy1 * W + sx0] / 256.0f, c11 = (float)tex[sy1 * W + sx1] / 256.0f;
    float it = mixf(mixf(c00, c10, tx), mixf(c01, c11, tx), ty);
    it *= u.branched_flow_intensity;
    it = (float)std::pow((double)it, (double)u.branched_flow_sharpness);
    return std::fmin(std::fmax(it, 0.0f), 3.0f);
}

void fragment(V3 nin, V3 wp, const float cam[3], const Frame &f, const uint8_t *lut, const uint32_t *tex,
              float out[4]) {
    const sbs_bubble_uniform &u = *f.u;
    const float nl = std::sqrt(dot3(nin, nin));
    const V3 n{nin.x / nl, nin.y / nl, nin.z / nl};
    const V3 w{cam[0] - wp.x, cam[1] - wp.y, cam[2] - wp.z};
    const float wl = std::sqrt(dot3(w, w));
    const V3 vd{w.x / wl, w.y / wl, w.z / wl};
    const float cos_theta = std::fabs(dot3(vd, n));
    const float th = thickness(n, f);
    const float e = 1.0f - cos_theta;
    const float se = u.edge_smoothing_mode == 1u ? e * e * (3.0f - 2.0f * e)
                                                 : (u.edge_smoothing_mode == 2u ? e * std::sqrt(e) : e);
    const float alpha = u.base_alpha + u.edge_alpha * se;
    if (th < 30.0f) {
        out[0] = out[1] = out[2] = 0.02f;
        out[3] = alpha * 0.5f;
        return;
    }
    float lc[3];
    sample_lut(lut, std::fmin(std::fmax(th / 2000.0f, 0.0f), 1.0f), std::fmin(std::fmax(cos_theta, 0.0f), 1.0f), lc);
    const float base[3] = {0.95f, 0.97f, 1.0f}, hue[3] = {1.0f, 0.95f, 0.85f};
    float bf = 0.0f;
    if (u.branched_flow_enabled != 0u && tex) bf = branched(n, tex, u);
    for (int c = 0; c < 3; ++c) {
        const float ic = std::fmin(std::fmax(lc[c] * u.interference_intensity, 0.0f), 1.0f);
        out[c] = base[c] * 0.1f + ic;
        if (bf > 0.0f) out[c] = out[c] + hue[c] * bf;
    }
    out[3] = alpha;
}

// 4 x 4 inverse of a column-major matrix by Gauss-Jordan elimination with partial pivoting, double
bool inverse4(const float *m, double inv[16]) {
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            a[r][c] = m[c * 4 + r];
            a[r][c + 4] = r == c ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; ++c) {
        int piv = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
        if (!(std::fabs(a[piv][c]) > 0.0)) return false;
        if (piv != c)
            for (int k = 0; k < 8; ++k) std::swap(a[c][k], a[piv][k]);
        const double d = a[c][c];
        for (int k = 0; k < 8; ++k) a[c][k] /= d;
        for (int r = 0; r < 4; ++r)
            if (r != c) {
                const double f = a[r][c];
                for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
            }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) inv[c * 4 + r] = a[r][c + 4];
    return true;
}

uint8_t srgb8(float x) {
    x = std::fmin(std::fmax(x, 0.0f), 1.0f);
    const float e = x <= 0.0031308f ? 12.92f * x : 1.055f * (float)std::pow((double)x, 1.0 / 2.4) - 0.055f;
    return (uint8_t)std::lrint(e * 255.0f);
}

}  // namespace

extern "C" {

float orc_simplex3(float x, float y, float z) { return simplex(V3{x, y, z}); }

float orc_film_thickness(const sbs_bubble_uniform *u, float nx, float ny, float nz) {
    return thickness(V3{nx, ny, nz}, frame_of(u));
}

void orc_shade_fragments(const sbs_bubble_uniform *u, const float cam[3], const uint8_t *lut, const uint32_t *tex,
                         size_t n, const float *normal, const float *wpos, float *rgba) {
    const Frame f = frame_of(u);
    for (size_t k = 0; k < n; ++k)
        fragment(V3{normal[3 * k], normal[3 * k + 1], normal[3 * k + 2]},
                 V3{wpos[3 * k], wpos[3 * k + 1], wpos[3 * k + 2]}, cam, f, lut, tex, rgba + 4 * k);
}

int orc_shade_frame(const sbs_bubble_uniform *u, const float view_proj[16], const float cam[3], float radius,
                    const uint8_t *lut, const uint32_t *tex, uint32_t width, uint32_t height, uint8_t *rgba8,
                    float *linear) {
    double inv[16];
    if (!inverse4(view_proj, inv)) return -1;
    const Frame f = frame_of(u);
#pragma omp parallel for schedule(dynamic, 4)
    for (int64_t py = 0; py < (int64_t)height; ++py)
        for (uint32_t px = 0; px < width; ++px) {
            const float ndx = 2.0f * ((float)px + 0.5f) / (float)width - 1.0f;
            const float ndy = 1.0f - 2.0f * ((float)py + 0.5f) / (float)height;
            double h[4];
            for (int r = 0; r < 4; ++r) h[r] = inv[r] * ndx + inv[4 + r] * ndy + inv[8 + r] * 1.0 + inv[12 + r];
            const V3 far{(float)(h[0] / h[3]), (float)(h[1] / h[3]), (float)(h[2] / h[3])};
            V3 d{far.x - cam[0], far.y - cam[1], far.z - cam[2]};
            const float dl = std::sqrt(dot3(d, d));
            d = V3{d.x / dl, d.y / dl, d.z / dl};
            const V3 oc{cam[0] - u->position_x, cam[1] - u->position_y, cam[2] - u->position_z};
            const float b = dot3(oc, d), c = dot3(oc, oc) - radius * radius, disc = b * b - c;
            float col[4] = {u->background_r, u->background_g, u->background_b, 1.0f};
            if (disc >= 0.0f) {
                const float sq = std::sqrt(disc);
                float t = -b - sq;
                if (t <= 0.0f) t = -b + sq;
                if (t > 0.0f) {
                    const V3 hit{cam[0] + d.x * t, cam[1] + d.y * t, cam[2] + d.z * t};
                    const V3 nrm{(hit.x - u->position_x) / radius, (hit.y - u->position_y) / radius,
                                 (hit.z - u->position_z) / radius};
                    float s[4];
                    fragment(nrm, hit, cam, f, lut, tex, s);
                    const float a = std::fmin(std::fmax(s[3], 0.0f), 1.0f);
                    for (int k = 0; k < 3; ++k) col[k] = std::fmin(std::fmax(s[k], 0.0f), 1.0f) * a + col[k] * (1.0f - a);
                    col[3] = a + 1.0f * (1.0f - a);
                }
            }
            const size_t idx = (size_t)py * width + px;
            if (linear)
                for (int k = 0; k < 4; ++k) linear[4 * idx + k] = col[k];
            if (rgba8) {
                for (int k = 0; k < 3; ++k) rgba8[4 * idx + k] = srgb8(col[k]);
                rgba8[4 * idx + 3] = (uint8_t)std::lrint(std::fmin(std::fmax(col[3], 0.0f), 1.0f) * 255.0f);
            }
        }
    return 0;
}

}  // extern "C"
