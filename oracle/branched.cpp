// CPU restatement of the branched-flow ray tracer (branched_flow_compute.wgsl:100-479) and of the
// scatterer generation (branched_flow.rs:164-240). TEST INFRASTRUCTURE (see oracle.h): it checks
// the CUDA kernels and is never linked into the product.
//
// Literal to the WGSL: every invocation recomputes the entry point, tangent basis and beam;
// total_scatterer_force loops over all scatterers with the 3 x 3 grid-cell early exit; float
// arithmetic left to right without contraction. acos, atan2 and exp are the published
// approximations the library documents (Abramowitz & Stegun 4.4.46 and 4.4.49, Cody-Waite
// reduction + Taylor series to degree 7), restated here from those sources.
#include <cmath>
#include <cstring>
#include <vector>

#include "oracle.h"

namespace {

const float PI = 3.14159265359f;

float acos_ref(float x) {  // A&S 4.4.46 on |x|, reflected for x < 0
    const float a[8] = {1.5707963050f, -0.2145988016f, 0.0889789874f, -0.0501743046f,
                        0.0308918810f, -0.0170881256f, 0.0066700901f, -0.0012624911f};
    const float t = std::fabs(x);
    float p = a[7];
    for (int k = 6; k >= 0; --k) p = p * t + a[k];
    const float r = std::sqrt(1.0f - t) * p;
    return x >= 0.0f ? r : PI - r;
}

float atan_ref(float z) {  // A&S 4.4.49, |z| <= 1: z (1 + a2 z^2 + ... + a16 z^16)
    const float a[9] = {1.0f, -0.3333314528f, 0.1999355085f, -0.1420889944f, 0.1065626393f,
                        -0.0752896400f, 0.0429096138f, -0.0161657367f, 0.0028662257f};
    const float z2 = z * z;
    float p = a[8];
    for (int k = 7; k >= 0; --k) p = p * z2 + a[k];
    return z * p;
}

float atan2_ref(float y, float x) {
    const float ax = std::fabs(x), ay = std::fabs(y);
    if (ax == 0.0f && ay == 0.0f) return 0.0f;
    float a = ay <= ax ? atan_ref(ay / ax) : 1.57079632679f - atan_ref(ax / ay);
    if (x < 0.0f) a = PI - a;
    return std::copysign(a, y);
}

float exp_ref(float x) {  // Cody-Waite: x = n ln2 + f, e^f by Taylor to degree 7, times 2^n
    if (x < -87.0f) return 0.0f;
    if (x > 88.0f) return INFINITY;
    const float n = std::rint(x * 1.44269504f);
    const float f = (x - n * 0.693145751953125f) - n * 1.428606820309417232e-6f;
    const float c[8] = {1.0f, 1.0f, 0.5f, 1.0f / 6.0f, 1.0f / 24.0f, 1.0f / 120.0f, 1.0f / 720.0f, 1.0f / 5040.0f};
    float p = c[7];
    for (int k = 6; k >= 0; --k) p = p * f + c[k];
    return std::ldexp(p, (int)n);
}

float fract_w(float x) { return x - std::floor(x); }  // WGSL fract
float fract_r(float x) { return x - std::trunc(x); }  // Rust f32::fract

float hash21(float x, float y) {
    float p3[3] = {fract_w(x * 0.1031f), fract_w(y * 0.1031f), fract_w(x * 0.1031f)};
    const float d = p3[0] * (p3[1] + 33.33f) + p3[1] * (p3[2] + 33.33f) + p3[2] * (p3[0] + 33.33f);
    for (float &v : p3) v += d;
    return fract_w((p3[0] + p3[1]) * p3[2]);
}

struct V3 {
    float x, y, z;
};
V3 norm3(V3 a) {
    const float l = std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
    return V3{a.x / l, a.y / l, a.z / l};
}
V3 cross(V3 a, V3 b) { return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

unsigned cell_of(float u) { return (unsigned)std::fmin(std::fmax(u / 0.1f, 0.0f), 9.0f); }

struct Ctx {
    const sbs_branched_params *p;
    const float *th;
    unsigned w, h;
    size_t pitch;
    const sbs_scatterer *sc;
    unsigned nsc;
    uint32_t *tex;
};

float sample_uv(const Ctx &c, float u, float v) {
    const unsigned x = (unsigned)(std::fmin(std::fmax(u, 0.0f), 1.0f) * (float)(c.w - 1));
    const unsigned y = (unsigned)(std::fmin(std::fmax(v, 0.0f), 1.0f) * (float)(c.h - 1));
    return c.th[(size_t)y * c.pitch + x];
}

void deposit(const Ctx &c, float u, float v, float intensity) {
    const unsigned tw = c.p->tex_width, th = c.p->tex_height;
    const float fx = std::fmin(std::fmax(u, 0.0f), 1.0f) * (float)(tw - 1), fy = std::fmin(std::fmax(v, 0.0f), 1.0f) * (float)(th - 1);
    const unsigned x0 = (unsigned)std::floor(fx), y0 = (unsigned)std::floor(fy);
    const unsigned x1 = std::min(x0 + 1, tw - 1), y1 = std::min(y0 + 1, th - 1);
    const float sx = fx - std::floor(fx), sy = fy - std::floor(fy);
    const float base = intensity * 256.0f;
    c.tex[y0 * tw + x0] += (uint32_t)(base * ((1.0f - sx) * (1.0f - sy)));
    c.tex[y0 * tw + x1] += (uint32_t)(base * (sx * (1.0f - sy)));
    c.tex[y1 * tw + x0] += (uint32_t)(base * ((1.0f - sx) * sy));
    c.tex[y1 * tw + x1] += (uint32_t)(base * (sx * sy));
}

void trace_ray(const Ctx &c, unsigned ray) {
    const sbs_branched_params &p = *c.p;
    const V3 entry = norm3(V3{p.entry_point[0], p.entry_point[1], p.entry_point[2]});
    const V3 braw{p.beam_dir[0], p.beam_dir[1], p.beam_dir[2]};
    const float be = dot3(braw, entry);
    const V3 beam = norm3(V3{braw.x - entry.x * be, braw.y - entry.y * be, braw.z - entry.z * be});
    V3 up{0.0f, 1.0f, 0.0f};
    if (std::fabs(dot3(entry, up)) > 0.99f) up = V3{1.0f, 0.0f, 0.0f};
    const V3 t1 = norm3(cross(entry, up)), t2 = norm3(cross(entry, t1));
    const float rand1 = hash21((float)ray * 0.1f, 0.0f), rand2 = hash21((float)ray * 0.1f + 100.0f, 1.0f);
    float vx = dot3(beam, t1), vy = dot3(beam, t2);
    const float vl = std::sqrt(vx * vx + vy * vy);
    vx /= vl;
    vy /= vl;
    const float perp_x = -vy, perp_y = vx;
    const float po = (rand1 - 0.5f) * p.spread_angle, ao = (rand2 - 0.5f) * p.spread_angle * 0.1f;
    float px = perp_x * po + vx * ao, py = perp_y * po + vy * ao;
    float intensity = 1.0f;
    const float dt = p.step_size;
    for (unsigned step = 0; step < p.ray_steps; ++step) {
        const V3 q = norm3(V3{entry.x + t1.x * px + t2.x * py, entry.y + t1.y * px + t2.y * py,
                              entry.z + t1.z * px + t2.z * py});
        const float u = (atan2_ref(q.z, q.x) + PI) / (2.0f * PI);
        const float v = acos_ref(std::fmin(std::fmax(q.y, -1.0f), 1.0f)) / PI;
        if (p.patch_enabled != 0u) {
            if (std::fabs(u - p.patch_center_u) <= p.patch_half_size && std::fabs(v - p.patch_center_v) <= p.patch_half_size) {
                const float min_u = std::fmax(p.patch_center_u - p.patch_half_size, 0.0f);
                const float max_u = std::fmin(p.patch_center_u + p.patch_half_size, 1.0f);
                const float min_v = std::fmax(p.patch_center_v - p.patch_half_size, 0.0f);
                const float max_v = std::fmin(p.patch_center_v + p.patch_half_size, 1.0f);
                const float lu = std::fmin(std::fmax((u - min_u) / std::fmax(max_u - min_u, 0.001f), 0.0f), 1.0f);
                const float lv = std::fmin(std::fmax((v - min_v) / std::fmax(max_v - min_v, 0.001f), 0.0f), 1.0f);
                deposit(c, lu, lv, intensity * 0.15f);
            }
        } else {
            deposit(c, u, v, intensity * 0.15f);
        }
        const float eps = 0.01f;
        const float gx = (sample_uv(c, u + eps, v) - sample_uv(c, u - eps, v)) / (2.0f * eps) * (1.0f - p.particle_weight);
        const float gy = (sample_uv(c, u, v + eps) - sample_uv(c, u, v - eps)) / (2.0f * eps) * (1.0f - p.particle_weight);
        // total_scatterer_force: all scatterers, skipping those outside the 3 x 3 cells
        float fx = 0.0f, fy = 0.0f;
        const unsigned rcu = cell_of(u), rcv = cell_of(v);
        const unsigned min_cu = rcu >= 1 ? rcu - 1 : 0, max_cu = std::min(rcu + 1, 9u);
        const unsigned min_cv = rcv >= 1 ? rcv - 1 : 0, max_cv = std::min(rcv + 1, 9u);
        for (unsigned i = 0; i < c.nsc; ++i) {
            const sbs_scatterer &s = c.sc[i];
            const unsigned su = cell_of(s.pos_u), sv = cell_of(s.pos_v);
            if (su < min_cu || su > max_cu || sv < min_cv || sv > max_cv) continue;
            const float dx = u - s.pos_u, dy = v - s.pos_v;
            const float r2 = dx * dx + dy * dy;
            float ex = 0.0f, ey = 0.0f;
            if (!(r2 > 4.5f / s.inv_sigma_sq)) {
                const float e = exp_ref(-r2 * s.inv_sigma_sq);
                ex = dx * s.strength * s.inv_sigma_sq * 2.0f * e;
                ey = dy * s.strength * s.inv_sigma_sq * 2.0f * e;
                fx += ex;
                fy += ey;
            }
        }
        const float tx = gx + fx * p.particle_weight, ty = gy + fy * p.particle_weight;
        vx = vx + tx * p.bend_strength * dt;
        vy = vy + ty * p.bend_strength * dt;
        const float vm = std::sqrt(vx * vx + vy * vy);
        if (vm > 0.001f) {
            vx = vx / vm;
            vy = vy / vm;
        }
        px = px + vx * dt;
        py = py + vy * dt;
        intensity = intensity * (1.0f - p.intensity_falloff);
        if (std::sqrt(px * px + py * py) > 2.5f || intensity < 0.01f) break;
    }
}

float halton(unsigned index, unsigned base) {
    float result = 0.0f, f = 1.0f / (float)base;
    unsigned i = index;
    while (i > 0) {
        result += f * (float)(i % base);
        i /= base;
        f /= (float)base;
    }
    return result;
}

}  // namespace

extern "C" {

float orc_acos_as(float x) { return acos_ref(x); }
float orc_atan2_as(float y, float x) { return atan2_ref(y, x); }
float orc_exp_cw(float x) { return exp_ref(x); }

void orc_branched_scatterers(const sbs_branched_params *p, uint32_t num, float time, sbs_scatterer *out) {
    for (unsigned i = 0; i < num; ++i) {
        const float u = halton(i + 1, 2), v = halton(i + 1, 3);
        const float hs = (float)i * 0.1031f + time * 0.1f;
        const float ju = fract_r(std::sin(hs) * 43758.547f) * 0.02f, jv = fract_r(std::cos(hs) * 43758.547f) * 0.02f;
        float pu, pv;
        if (p->patch_enabled != 0u) {
            const float min_u = std::fmax(p->patch_center_u - p->patch_half_size, 0.0f);
            const float min_v = std::fmax(p->patch_center_v - p->patch_half_size, 0.0f);
            const float max_u = std::fmin(p->patch_center_u + p->patch_half_size, 1.0f);
            const float max_v = std::fmin(p->patch_center_v + p->patch_half_size, 1.0f);
            pu = std::fmin(std::fmax(min_u + u * (max_u - min_u) + ju * p->patch_half_size * 2.0f, 0.0f), 1.0f);
            pv = std::fmin(std::fmax(min_v + v * (max_v - min_v) + jv * p->patch_half_size * 2.0f, 0.0f), 1.0f);
        } else {
            pu = std::fmod(u + ju, 1.0f);
            if (pu < 0.0f) pu += 1.0f;
            pv = std::fmod(v + jv, 1.0f);
            if (pv < 0.0f) pv += 1.0f;
        }
        const float sign = fract_r(std::sin((float)i * 0.7531f + 0.3f) * 43758.547f) > 0.5f ? 1.0f : -1.0f;
        const float svar = 0.8f + 0.4f * fract_r(std::sin((float)i * 0.9371f) * 43758.547f);
        const float rvar = 0.8f + 0.4f * fract_r(std::cos((float)i * 0.5791f) * 43758.547f);
        const float sigma = p->scatterer_radius * rvar;
        out[i] = sbs_scatterer{pu, pv, sign * p->scatterer_strength * svar, 1.0f / (2.0f * sigma * sigma)};
    }
}

void orc_branched_flow(const sbs_branched_params *p, const float *th, uint32_t w, uint32_t h, size_t pitch,
                       const sbs_scatterer *sc, uint32_t *tex, int fade) {
    const size_t n = (size_t)p->tex_width * p->tex_height;
    if (fade)
        for (size_t i = 0; i < n; ++i) tex[i] = (uint32_t)((float)tex[i] * 0.85f);
    const Ctx c{p, th, w, h, pitch, sc, std::min(p->num_scatterers, 2048u), tex};
    for (unsigned r = 0; r < p->num_rays; ++r) trace_ray(c, r);
}

}  // extern "C"
