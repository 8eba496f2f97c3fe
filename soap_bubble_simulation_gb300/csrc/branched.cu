// Branched flow of light through the soap film: the kick-drift ray tracer of
// branched_flow_compute.wgsl:365-468 with its clear / fade pass (:470-479), and the host-side
// scatterer generation of branched_flow.rs:164-240.
//
// One thread per ray (the reference's one invocation per ray), the rays' 400 steps in sequence.
// Per step: the film position and its (u, v) on the sphere, a bilinear deposit of
// 0.15 x intensity x 256 into the u32 texture by four atomic adds, the GRIN kick from the
// thickness gradient and the particle kick from the scatterers, drift, falloff.
//
// Scatterers. The reference loops over all scatterers and skips those whose grid cell (10 x 10
// cells of 0.1 in uv) is outside the ray cell's 3 x 3 neighbourhood. Here each cell has the list
// of exactly those scatterers, in index order, built on the host: the same terms summed in the
// same order, about 9 % of the loop. The lists and the scatterers sit in shared memory.
//
// Reproducibility. Every operation is FP32 in the WGSL's order without contraction; acos, atan2
// and exp are the library's own evaluations of published approximations (acos: Abramowitz &
// Stegun 4.4.46, |error| <= 2e-8; atan: A&S 4.4.49, |error| <= 2e-8, with the usual octant
// reduction; exp: Cody-Waite reduction by ln 2 and the Taylor series of e^f to degree 7), so the
// CPU restatement reproduces each ray bit for bit and, the deposits being integer atomic adds,
// the texture too.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "sbs_internal.h"

namespace sbs {
namespace {

constexpr float kPi = 3.14159265359f;    // PI (branched_flow_compute.wgsl:87)
constexpr float kHalfPi = 1.57079632679f;
constexpr int kGrid = 10;                 // GRID_SIZE_U = GRID_SIZE_V
constexpr float kCellSize = 0.1f;         // GRID_CELL_SIZE
constexpr int kMaxScatterers = 2048;

// ---- the library's acos / atan2 / exp ----------------------------------------------------
__host__ __device__ __forceinline__ float acos_as(float x) {
    const float t = fabsf(x);
    float p = -0.0012624911f;
    p = p * t + 0.0066700901f;
    p = p * t + -0.0170881256f;
    p = p * t + 0.0308918810f;
    p = p * t + -0.0501743046f;
    p = p * t + 0.0889789874f;
    p = p * t + -0.2145988016f;
    p = p * t + 1.5707963050f;
    const float r = sqrtf(1.0f - t) * p;
    return x >= 0.0f ? r : kPi - r;
}

__host__ __device__ __forceinline__ float atan_as(float z) {  // |z| <= 1
    const float z2 = z * z;
    float p = 0.0028662257f;
    p = p * z2 + -0.0161657367f;
    p = p * z2 + 0.0429096138f;
    p = p * z2 + -0.0752896400f;
    p = p * z2 + 0.1065626393f;
    p = p * z2 + -0.1420889944f;
    p = p * z2 + 0.1999355085f;
    p = p * z2 + -0.3333314528f;
    p = p * z2 + 1.0f;
    return z * p;
}

__host__ __device__ __forceinline__ float atan2_as(float y, float x) {
    const float ax = fabsf(x), ay = fabsf(y);
    if (ax == 0.0f && ay == 0.0f) return 0.0f;
    float a = ay <= ax ? atan_as(ay / ax) : kHalfPi - atan_as(ax / ay);
    if (x < 0.0f) a = kPi - a;
    return copysignf(a, y);
}

__device__ __forceinline__ float exp_cw(float x) {
    if (x < -87.0f) return 0.0f;
    if (x > 88.0f) return INFINITY;
    const float n = rintf(x * 1.44269504f);
    const float f = (x - n * 0.693145751953125f) - n * 1.428606820309417232e-6f;
    float p = 1.0f / 5040.0f;
    p = p * f + 1.0f / 720.0f;
    p = p * f + 1.0f / 120.0f;
    p = p * f + 1.0f / 24.0f;
    p = p * f + 1.0f / 6.0f;
    p = p * f + 0.5f;
    p = p * f + 1.0f;
    p = p * f + 1.0f;
    return ldexpf(p, (int)n);
}

__device__ __forceinline__ float fract(float x) { return x - floorf(x); }

// hash21 (branched_flow_compute.wgsl:164-168)
__device__ __forceinline__ float hash21(float px, float py) {
    float a = fract(px * 0.1031f), b = fract(py * 0.1031f), c = fract(px * 0.1031f);
    const float d = a * (b + 33.33f) + b * (c + 33.33f) + c * (a + 33.33f);  // dot(p3, p3.yzx + 33.33)
    a += d;
    b += d;
    c += d;
    return fract((a + b) * c);
}

// uv_to_grid_cell (:110-114), one coordinate
__host__ __device__ __forceinline__ int grid_cell(float u) {
    return (int)fminf(fmaxf(u / kCellSize, 0.0f), (float)(kGrid - 1));
}

struct Setup {  // per-frame values every ray shares (the shader computes them per invocation)
    float ex, ey, ez;        // entry point (normalised)
    float t1x, t1y, t1z;     // tangent basis
    float t2x, t2y, t2z;
    float vx, vy;            // collimated beam direction in the tangent plane
};

struct TraceArgs {
    sbs_branched_params p;
    Setup s;
    const float *thickness;
    size_t pitch;
    int width, height;
    const sbs_scatterer *scat;  // nscat entries
    const uint32_t *list_off;   // kGrid * kGrid + 1 offsets into list
    const uint16_t *list;       // scatterer indices per cell, ascending
    int nscat, nlist;
    uint32_t *tex;
};

__device__ __forceinline__ float sample_uv(const TraceArgs &a, float u, float v) {
    const int x = (int)(fminf(fmaxf(u, 0.0f), 1.0f) * (float)(a.width - 1));
    const int y = (int)(fminf(fmaxf(v, 0.0f), 1.0f) * (float)(a.height - 1));
    return __ldg(a.thickness + (size_t)y * a.pitch + x);
}

__device__ __forceinline__ void deposit(const TraceArgs &a, float u, float v, float intensity) {
    const uint32_t tw = a.p.tex_width, th = a.p.tex_height;
    const float fx = fminf(fmaxf(u, 0.0f), 1.0f) * (float)(tw - 1u);
    const float fy = fminf(fmaxf(v, 0.0f), 1.0f) * (float)(th - 1u);
    const uint32_t x0 = (uint32_t)floorf(fx), y0 = (uint32_t)floorf(fy);
    const uint32_t x1 = min(x0 + 1u, tw - 1u), y1 = min(y0 + 1u, th - 1u);
    const float sx = fx - floorf(fx), sy = fy - floorf(fy);
    const float w00 = (1.0f - sx) * (1.0f - sy), w10 = sx * (1.0f - sy), w01 = (1.0f - sx) * sy, w11 = sx * sy;
    const float base = intensity * 256.0f;
    atomicAdd(a.tex + y0 * tw + x0, (uint32_t)(base * w00));
    atomicAdd(a.tex + y0 * tw + x1, (uint32_t)(base * w10));
    atomicAdd(a.tex + y1 * tw + x0, (uint32_t)(base * w01));
    atomicAdd(a.tex + y1 * tw + x1, (uint32_t)(base * w11));
}

__global__ void __launch_bounds__(128) trace_kernel(TraceArgs a) {
    extern __shared__ __align__(16) uint8_t smem[];
    sbs_scatterer *sc = reinterpret_cast<sbs_scatterer *>(smem);
    float *scut = reinterpret_cast<float *>(sc + a.nscat);  // each scatterer's cutoff 4.5 / inv_sigma_sq
    uint32_t *off = reinterpret_cast<uint32_t *>(scut + a.nscat);
    uint16_t *lst = reinterpret_cast<uint16_t *>(off + kGrid * kGrid + 1);
    for (int k = threadIdx.x; k < a.nscat; k += blockDim.x) {
        sc[k] = a.scat[k];
        scut[k] = 4.5f / a.scat[k].inv_sigma_sq;
    }
    for (int k = threadIdx.x; k <= kGrid * kGrid; k += blockDim.x) off[k] = a.list_off[k];
    for (int k = threadIdx.x; k < a.nlist; k += blockDim.x) lst[k] = a.list[k];
    __syncthreads();
    const uint32_t ray = blockIdx.x * blockDim.x + threadIdx.x;
    const sbs_branched_params &p = a.p;
    if (ray >= p.num_rays) return;
    const Setup &s = a.s;
    const float rand1 = hash21((float)ray * 0.1f, 0.0f);
    const float rand2 = hash21((float)ray * 0.1f + 100.0f, 1.0f);
    const float px_ = -s.vy, py_ = s.vx;  // perpendicular to the beam
    const float pos_off = (rand1 - 0.5f) * p.spread_angle;
    const float along_off = (rand2 - 0.5f) * p.spread_angle * 0.1f;
    float posx = px_ * pos_off + s.vx * along_off, posy = py_ * pos_off + s.vy * along_off;
    float vx = s.vx, vy = s.vy;
    float intensity = 1.0f;
    const float dt = p.step_size;
    const bool patch = p.patch_enabled != 0u;
    const float min_u = fmaxf(p.patch_center_u - p.patch_half_size, 0.0f);
    const float max_u = fminf(p.patch_center_u + p.patch_half_size, 1.0f);
    const float min_v = fmaxf(p.patch_center_v - p.patch_half_size, 0.0f);
    const float max_v = fminf(p.patch_center_v + p.patch_half_size, 1.0f);
    const float gw = 1.0f - p.particle_weight;
    for (uint32_t step = 0; step < p.ray_steps; ++step) {
        // pos_3d = normalize(entry + tangent1 * pos.x + tangent2 * pos.y); uv = normal_to_uv(pos_3d)
        const float qx = s.ex + s.t1x * posx + s.t2x * posy;
        const float qy = s.ey + s.t1y * posx + s.t2y * posy;
        const float qz = s.ez + s.t1z * posx + s.t2z * posy;
        const float ql = sqrtf(qx * qx + qy * qy + qz * qz);
        const float nx = qx / ql, ny = qy / ql, nz = qz / ql;
        const float u = (atan2_as(nz, nx) + kPi) / (2.0f * kPi);
        const float v = acos_as(fminf(fmaxf(ny, -1.0f), 1.0f)) / kPi;
        if (patch) {
            const float du = fabsf(u - p.patch_center_u), dv = fabsf(v - p.patch_center_v);
            if (du <= p.patch_half_size && dv <= p.patch_half_size) {
                const float lu = fminf(fmaxf((u - min_u) / fmaxf(max_u - min_u, 0.001f), 0.0f), 1.0f);
                const float lv = fminf(fmaxf((v - min_v) / fmaxf(max_v - min_v, 0.001f), 0.0f), 1.0f);
                deposit(a, lu, lv, intensity * 0.15f);
            }
        } else {
            deposit(a, u, v, intensity * 0.15f);
        }
        // GRIN kick: thickness_gradient_uv (:197-211)
        const float eps = 0.01f;
        const float hr = sample_uv(a, u + eps, v), hl = sample_uv(a, u - eps, v);
        const float hu = sample_uv(a, u, v + eps), hd = sample_uv(a, u, v - eps);
        const float gx = (hr - hl) / (2.0f * eps) * gw, gy = (hu - hd) / (2.0f * eps) * gw;
        // particle kick: total_scatterer_force (:256-290) over the ray cell's neighbourhood list
        float fx = 0.0f, fy = 0.0f;
        const int cell = grid_cell(v) * kGrid + grid_cell(u);
        const uint32_t k1 = off[cell + 1];
#pragma unroll 2
        for (uint32_t k = off[cell]; k < k1; ++k) {
            const uint32_t idx = lst[k];
            const sbs_scatterer q = sc[idx];
            const float dx = u - q.pos_u, dy = v - q.pos_v;
            const float r2 = dx * dx + dy * dy;
            if (r2 > scut[idx]) continue;  // scatterer_force's cutoff: adds zero
            const float e = exp_cw(-r2 * q.inv_sigma_sq);
            fx += dx * q.strength * q.inv_sigma_sq * 2.0f * e;
            fy += dy * q.strength * q.inv_sigma_sq * 2.0f * e;
        }
        const float tx = gx + fx * p.particle_weight, ty = gy + fy * p.particle_weight;
        vx = vx + tx * p.bend_strength * dt;
        vy = vy + ty * p.bend_strength * dt;
        const float vm = sqrtf(vx * vx + vy * vy);
        if (vm > 0.001f) {
            vx = vx / vm;
            vy = vy / vm;
        }
        posx = posx + vx * dt;
        posy = posy + vy * dt;
        intensity = intensity * (1.0f - p.intensity_falloff);
        if (sqrtf(posx * posx + posy * posy) > 2.5f || intensity < 0.01f) break;
    }
}

__global__ void fade_kernel(uint32_t *tex, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) tex[i] = (uint32_t)((float)tex[i] * 0.85f);
}

float halton(uint32_t index, uint32_t base) {
    float result = 0.0f;
    float f = 1.0f / (float)base;
    uint32_t i = index;
    while (i > 0) {
        result += f * (float)(i % base);
        i /= base;
        f /= (float)base;
    }
    return result;
}

// Rust's f32::fract (x - trunc(x): negative for negative x), as generate_scatterers uses it
float fract_rust(float x) { return x - std::trunc(x); }

// Setup of one frame: entry point, tangent basis and beam direction (:371-403), in FP32.
Setup make_setup(const sbs_branched_params &p) {
    Setup s;
    float ex = p.entry_point[0], ey = p.entry_point[1], ez = p.entry_point[2];
    float l = std::sqrt(ex * ex + ey * ey + ez * ez);
    ex /= l;
    ey /= l;
    ez /= l;
    const float bx0 = p.beam_dir[0], by0 = p.beam_dir[1], bz0 = p.beam_dir[2];
    const float be = bx0 * ex + by0 * ey + bz0 * ez;
    float bx = bx0 - ex * be, by = by0 - ey * be, bz = bz0 - ez * be;
    l = std::sqrt(bx * bx + by * by + bz * bz);
    bx /= l;
    by /= l;
    bz /= l;
    float ux = 0.0f, uy = 1.0f, uz = 0.0f;
    if (std::fabs(ex * ux + ey * uy + ez * uz) > 0.99f) {
        ux = 1.0f;
        uy = 0.0f;
    }
    // tangent1 = normalize(cross(entry, up)); tangent2 = normalize(cross(entry, tangent1))
    float t1x = ey * uz - ez * uy, t1y = ez * ux - ex * uz, t1z = ex * uy - ey * ux;
    l = std::sqrt(t1x * t1x + t1y * t1y + t1z * t1z);
    t1x /= l;
    t1y /= l;
    t1z /= l;
    float t2x = ey * t1z - ez * t1y, t2y = ez * t1x - ex * t1z, t2z = ex * t1y - ey * t1x;
    l = std::sqrt(t2x * t2x + t2y * t2y + t2z * t2z);
    t2x /= l;
    t2y /= l;
    t2z /= l;
    float vx = bx * t1x + by * t1y + bz * t1z, vy = bx * t2x + by * t2y + bz * t2z;
    l = std::sqrt(vx * vx + vy * vy);
    s.ex = ex;
    s.ey = ey;
    s.ez = ez;
    s.t1x = t1x;
    s.t1y = t1y;
    s.t1z = t1z;
    s.t2x = t2x;
    s.t2y = t2y;
    s.t2z = t2z;
    s.vx = vx / l;
    s.vy = vy / l;
    return s;
}

}  // namespace
}  // namespace sbs

using namespace sbs;

extern "C" {

int sbs_branched_params_default(sbs_branched_params *out) {
    clear_error();
    SBS_CHECK_ARG(out != nullptr, "out is null");
    std::memset(out, 0, sizeof(*out));
    out->entry_point[2] = 1.0f;
    out->beam_dir[0] = -0.5f;
    out->beam_dir[1] = -0.866f;
    out->num_rays = 32768;
    out->ray_steps = 400;
    out->step_size = 0.005f;
    out->bend_strength = 5.0f;
    out->spread_angle = 0.4f;
    out->intensity_falloff = 0.001f;
    out->tex_width = 512;
    out->tex_height = 256;
    out->thickness_scale = 1e6f;
    out->base_thickness_nm = 500.0f;
    out->swirl_intensity = 1.0f;
    out->drainage_speed = 1.0f;
    out->pattern_scale = 1.0f;
    out->num_scatterers = 800;
    out->scatterer_strength = 0.5f;
    out->scatterer_radius = 0.03f;
    out->particle_weight = 0.1f;
    out->patch_enabled = 1;
    out->patch_center_u = 0.5f;
    out->patch_center_v = 0.5f;
    out->patch_half_size = 0.158f;
    return SBS_OK;
}

int sbs_branched_scatterers(const sbs_branched_params *p, uint32_t num, float time, sbs_scatterer *out) {
    clear_error();
    SBS_CHECK_ARG(p != nullptr && (out != nullptr || num == 0), "null argument");
    SBS_CHECK_ARG(num <= (uint32_t)kMaxScatterers, "at most %d scatterers", kMaxScatterers);
    const bool patch = p->patch_enabled != 0u;
    for (uint32_t i = 0; i < num; ++i) {
        const float u = halton(i + 1, 2), v = halton(i + 1, 3);
        const float jitter_scale = 0.02f;
        const float hash_seed = (float)i * 0.1031f + time * 0.1f;
        const float jitter_u = fract_rust(std::sin(hash_seed) * 43758.547f) * jitter_scale;
        const float jitter_v = fract_rust(std::cos(hash_seed) * 43758.547f) * jitter_scale;
        float pu, pv;
        if (patch) {
            const float min_u = std::max(p->patch_center_u - p->patch_half_size, 0.0f);
            const float min_v = std::max(p->patch_center_v - p->patch_half_size, 0.0f);
            const float max_u = std::min(p->patch_center_u + p->patch_half_size, 1.0f);
            const float max_v = std::min(p->patch_center_v + p->patch_half_size, 1.0f);
            const float mu = min_u + u * (max_u - min_u), mv = min_v + v * (max_v - min_v);
            pu = std::min(std::max(mu + jitter_u * p->patch_half_size * 2.0f, 0.0f), 1.0f);
            pv = std::min(std::max(mv + jitter_v * p->patch_half_size * 2.0f, 0.0f), 1.0f);
        } else {
            // rem_euclid(1.0)
            pu = std::fmod(u + jitter_u, 1.0f);
            if (pu < 0.0f) pu += 1.0f;
            pv = std::fmod(v + jitter_v, 1.0f);
            if (pv < 0.0f) pv += 1.0f;
        }
        const float sign_hash = fract_rust(std::sin((float)i * 0.7531f + 0.3f) * 43758.547f);
        const float sign = sign_hash > 0.5f ? 1.0f : -1.0f;
        const float strength_var = 0.8f + 0.4f * fract_rust(std::sin((float)i * 0.9371f) * 43758.547f);
        const float radius_var = 0.8f + 0.4f * fract_rust(std::cos((float)i * 0.5791f) * 43758.547f);
        const float sigma = p->scatterer_radius * radius_var;
        out[i] = sbs_scatterer{pu, pv, sign * p->scatterer_strength * strength_var, 1.0f / (2.0f * sigma * sigma)};
    }
    return SBS_OK;
}

int sbs_branched_flow(const sbs_branched_params *p, const float *thickness, uint32_t width, uint32_t height,
                      size_t pitch, const sbs_scatterer *scatterers, uint32_t *texture, int fade, int mem,
                      void *stream) {
    clear_error();
    SBS_CHECK_ARG(p != nullptr && thickness != nullptr && texture != nullptr, "null argument");
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "bad mem flag %d", mem);
    SBS_CHECK_ARG(width >= 1 && height >= 1 && pitch >= width, "bad thickness grid");
    SBS_CHECK_ARG(p->tex_width >= 2 && p->tex_height >= 2 && p->tex_width <= 16384 && p->tex_height <= 16384,
                  "texture size out of range");
    const int nscat = (int)std::min(p->num_scatterers, (uint32_t)kMaxScatterers);
    SBS_CHECK_ARG(nscat == 0 || scatterers != nullptr, "null scatterers");
    int rc = require_device();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    // host copies of the scatterers (for the lists) and the per-cell neighbourhood lists
    std::vector<sbs_scatterer> hs(nscat);
    if (nscat > 0) {
        if (mem == SBS_MEM_HOST) {
            std::memcpy(hs.data(), scatterers, sizeof(sbs_scatterer) * nscat);
        } else {
            SBS_CUDA_TRY(cudaMemcpyAsync(hs.data(), scatterers, sizeof(sbs_scatterer) * nscat,
                                         cudaMemcpyDeviceToHost, s));
            SBS_CUDA_TRY(cudaStreamSynchronize(s));
        }
    }
    std::vector<int> sc_u(nscat), sc_v(nscat);
    for (int i = 0; i < nscat; ++i) {
        sc_u[i] = grid_cell(hs[i].pos_u);
        sc_v[i] = grid_cell(hs[i].pos_v);
    }
    std::vector<uint32_t> off(kGrid * kGrid + 1, 0);
    std::vector<uint16_t> lst;
    lst.reserve((size_t)nscat * 9);
    for (int cv = 0; cv < kGrid; ++cv)
        for (int cu = 0; cu < kGrid; ++cu) {
            const int lo_u = cu >= 1 ? cu - 1 : 0, hi_u = std::min(cu + 1, kGrid - 1);
            const int lo_v = cv >= 1 ? cv - 1 : 0, hi_v = std::min(cv + 1, kGrid - 1);
            off[cv * kGrid + cu] = (uint32_t)lst.size();
            for (int i = 0; i < nscat; ++i)
                if (sc_u[i] >= lo_u && sc_u[i] <= hi_u && sc_v[i] >= lo_v && sc_v[i] <= hi_v)
                    lst.push_back((uint16_t)i);
        }
    off[kGrid * kGrid] = (uint32_t)lst.size();
    const size_t tex_n = (size_t)p->tex_width * p->tex_height;
    const size_t th_b = sizeof(float) * pitch * height;
    const size_t sc_b = sizeof(sbs_scatterer) * nscat, off_b = sizeof(uint32_t) * off.size(),
                 lst_b = sizeof(uint16_t) * std::max<size_t>(lst.size(), 1);
    const size_t bytes = sc_b + off_b + lst_b + 1024 + (mem == SBS_MEM_HOST ? th_b + 4 * tex_n : 0);
    char *base = nullptr;
    SBS_CUDA_TRY(scratch_alloc((void **)&base, bytes, s));
    char *q = base;
    auto carve = [&](size_t b) {
        char *r = q;
        q += (b + 255) / 256 * 256;
        return r;
    };
    sbs_scatterer *d_sc = (sbs_scatterer *)carve(sc_b);
    uint32_t *d_off = (uint32_t *)carve(off_b);
    uint16_t *d_lst = (uint16_t *)carve(lst_b);
    const float *d_th = thickness;
    uint32_t *d_tex = texture;
    cudaError_t e = cudaSuccess;
    if (nscat > 0) e = cudaMemcpyAsync(d_sc, hs.data(), sc_b, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_off, off.data(), off_b, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && !lst.empty()) e = cudaMemcpyAsync(d_lst, lst.data(), sizeof(uint16_t) * lst.size(),
                                                              cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && mem == SBS_MEM_HOST) {
        float *t = (float *)carve(th_b);
        e = cudaMemcpyAsync(t, thickness, th_b, cudaMemcpyHostToDevice, s);
        d_th = t;
        d_tex = (uint32_t *)carve(4 * tex_n);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_tex, texture, 4 * tex_n, cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess && fade) {
        fade_kernel<<<(unsigned)((tex_n + 255) / 256), 256, 0, s>>>(d_tex, tex_n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && p->num_rays > 0) {
        TraceArgs a;
        a.p = *p;
        a.s = make_setup(*p);
        a.thickness = d_th;
        a.pitch = pitch;
        a.width = (int)width;
        a.height = (int)height;
        a.scat = d_sc;
        a.list_off = d_off;
        a.list = d_lst;
        a.nscat = nscat;
        a.nlist = (int)lst.size();
        a.tex = d_tex;
        const size_t smem = sc_b + sizeof(float) * nscat + off_b + sizeof(uint16_t) * lst.size() + 16;
        e = cudaFuncSetAttribute(trace_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e == cudaSuccess) {
            trace_kernel<<<(p->num_rays + 127) / 128, 128, smem, s>>>(a);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess && mem == SBS_MEM_HOST) e = cudaMemcpyAsync(texture, d_tex, 4 * tex_n, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(base, s);
    if (e == cudaSuccess && mem == SBS_MEM_HOST) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(SBS_E_CUDA, "branched flow: %s", cudaGetErrorString(e));
    return SBS_OK;
}

}  // extern "C"
