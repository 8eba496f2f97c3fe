// Thin-film interference kernels: the InterferenceCalculator colour (interference.rs:127-512),
// its 1-D/2-D lookup tables, the RGBA8 spectral LUT (interference_lut.rs:18-163), the Schlick /
// transmitted-Airy evaluation (wall.wgsl:176-207) and LUT lookups (bubble.wgsl:425-439).
//
// Each point is independent, so every kernel is a flat grid of threads, one point (or one LUT
// entry) per thread; the work per point is a handful of sqrt/cos/pow evaluations and the
// kernels are bound by issue latency at the reference's sizes, by HBM at large point counts.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "sbs_internal.h"

namespace sbs {
namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kEpsF64 = 2.220446049250313e-16;  // f64::EPSILON
constexpr float kPiF = 3.14159265358979323846f;

// ---------------------------------------------------------------------------
// f64 InterferenceCalculator
// ---------------------------------------------------------------------------
struct Terms {
    double ct, opd, phase, Rs, Rp, R, I;
};

// calculate_transmission_angle_cos (interference.rs:197-211), n_medium = 1.
__device__ __forceinline__ double cos_t64(double n, double ci) {
    const double c = ci < -1.0 ? -1.0 : (ci > 1.0 ? 1.0 : ci);
    const double si = sqrt(1.0 - c * c);
    const double st = (1.0 / n) * si;
    if (fabs(st) > 1.0) return 0.0;
    return sqrt(1.0 - st * st);
}

// calculate_reflected_intensity with its intermediate terms (interference.rs:312-353).
__device__ Terms terms64(double n, double t, double ci, double wl) {
    Terms o{};
    const double c = ci < -1.0 ? -1.0 : (ci > 1.0 ? 1.0 : ci);
    o.ct = cos_t64(n, ci);
    o.opd = 2.0 * n * t * o.ct + wl / 2.0;
    o.phase = 2.0 * kPi * o.opd / wl;
    const double n1ci = 1.0 * c, n2ct = n * o.ct, n2ci = n * c, n1ct = 1.0 * o.ct;
    const double rs = (n1ci - n2ct) / (n1ci + n2ct);
    const double rp = (n2ci - n1ct) / (n2ci + n1ct);
    o.Rs = rs * rs;
    o.Rp = rp * rp;
    o.R = (o.Rs + o.Rp) / 2.0;
    if (t <= 0.0) {
        o.I = 0.0;
        return o;
    }
    const double cp = cos(o.phase);
    const double num = 2.0 * o.R * (1.0 - cp);
    const double den = 1.0 + o.R * o.R - 2.0 * o.R * cp;
    if (fabs(den) < kEpsF64) {
        o.I = o.R;
        return o;
    }
    const double q = num / den;
    o.I = q < 0.0 ? 0.0 : (q > 1.0 ? 1.0 : q);
    return o;
}

__device__ __forceinline__ double channel64(double n, double t, double ci, double wl, int gamma) {
    if (t <= 0.0) return gamma ? pow(0.0, 1.0 / 2.2) : 0.0;
    double I = terms64(n, t, ci, wl).I;
    if (gamma) I = pow(I, 1.0 / 2.2);
    return I < 0.0 ? 0.0 : (I > 1.0 ? 1.0 : I);  // RgbColor::new (:54-60)
}

struct Wl3 {
    double w[3];
};

__global__ void rgb64_kernel(double n, Wl3 wl, const double *t, const double *ci, size_t count, int gamma,
                             double *rgb) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const double tk = t[k], ck = ci[k];
#pragma unroll
    for (int c = 0; c < 3; ++c) rgb[3 * k + c] = channel64(n, tk, ck, wl.w[c], gamma);
}

__global__ void terms64_kernel(double n, double wl, const double *t, const double *ci, size_t count, double *out) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const Terms o = terms64(n, t[k], ci[k], wl);
    double *p = out + 8 * k;
    p[0] = o.ct;
    p[1] = o.opd;
    p[2] = o.phase;
    p[3] = o.Rs;
    p[4] = o.Rp;
    p[5] = o.R;
    p[6] = o.I;
    p[7] = 0.0;
}

// calculate_optical_path_difference / calculate_phase_difference (interference.rs:226-254).
__global__ void path_kernel(double n, const double *t, const double *ct, const double *wl, const double *opd_in,
                            size_t count, double *out) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    if (opd_in == nullptr)
        out[k] = 2.0 * n * t[k] * ct[k] + wl[k] / 2.0;
    else
        out[k] = 2.0 * kPi * opd_in[k] / wl[k];
}

// generate_2d_color_lookup_table (interference.rs:491-512): entry (i, j) of a T x A table.
__global__ void lut2d_kernel(double n, Wl3 wl, double tmin, double tstep, double astep, int T, int A, double *rgb) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= T * A) return;
    const int i = idx / A, j = idx % A;
    const double t = tmin + (double)i * tstep;
    const double ci = (double)j * astep;
#pragma unroll
    for (int c = 0; c < 3; ++c) rgb[3 * (size_t)idx + c] = channel64(n, t, ci, wl.w[c], 1);
}

// generate_color_lookup_table (interference.rs:461-477).
__global__ void lut1d_kernel(double n, Wl3 wl, double tmin, double tstep, int count, double ci, double *rgb) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const double t = tmin + (double)i * tstep;
#pragma unroll
    for (int c = 0; c < 3; ++c) rgb[3 * (size_t)i + c] = channel64(n, t, ci, wl.w[c], 1);
}

// ---------------------------------------------------------------------------
// f32 InterferenceCalculator variant: 1 - cos(delta) is evaluated as 2 sin^2(delta/2) with
// sinpi of the path difference in wavelengths, so reflectance near destructive interference keeps
// its relative accuracy (the gamma curve magnifies absolute errors near zero).
// ---------------------------------------------------------------------------
struct Wl3f {
    float w[3];
};

__device__ __forceinline__ float channel32(float n, float t, float ci, float wl, int gamma) {
    if (t <= 0.f) return 0.f;
    const float c = ci < -1.f ? -1.f : (ci > 1.f ? 1.f : ci);
    const float si = sqrtf(1.f - c * c);
    const float st = (1.f / n) * si;
    const float ct = fabsf(st) > 1.f ? 0.f : sqrtf(1.f - st * st);
    const float y = (2.f * n * t * ct) / wl + 0.5f;  // optical path difference in wavelengths
    const float s = sinpif(y);
    const float s2 = s * s;
    const float rs = (c - n * ct) / (c + n * ct);
    const float rp = (n * c - ct) / (n * c + ct);
    const float R = (rs * rs + rp * rp) * 0.5f;
    const float omr = 1.f - R;
    const float num = 4.f * R * s2;
    const float den = omr * omr + num;
    float I = den < 2.220446049250313e-16f ? R : num / den;
    I = I < 0.f ? 0.f : (I > 1.f ? 1.f : I);
    if (gamma) I = powf(I, 1.f / 2.2f);
    return I < 0.f ? 0.f : (I > 1.f ? 1.f : I);
}

__global__ void rgb32_kernel(float n, Wl3f wl, const float *t, const float *ci, size_t count, int gamma,
                             float *rgb) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const float tk = t[k], ck = ci[k];
#pragma unroll
    for (int c = 0; c < 3; ++c) rgb[3 * k + c] = channel32(n, tk, ck, wl.w[c], gamma);
}

// ---------------------------------------------------------------------------
// generate_interference_lut (interference_lut.rs:18-163) in the same f32 operation order. The
// seven CIE weights depend only on the wavelength and arrive precomputed; sin is evaluated in f64
// and rounded once, i.e. the correctly rounded f32 sine.
// ---------------------------------------------------------------------------
struct Cie7 {
    float xyz[7][3];
};

__device__ __forceinline__ float fmax_rs(float a, float b) { return a > b ? a : (b == b ? b : a); }
__device__ __forceinline__ float clamp01(float x) { return x < 0.f ? 0.f : (x > 1.f ? 1.f : x); }

__global__ void lut_rgba8_kernel(float n_film, float intensity, Cie7 cie, uchar4 *out) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= SBS_LUT_THICKNESS_SAMPLES * SBS_LUT_ANGLE_SAMPLES) return;
    const int a = idx / SBS_LUT_THICKNESS_SAMPLES, ti = idx % SBS_LUT_THICKNESS_SAMPLES;
    const float t_nm = ((float)ti / (float)(SBS_LUT_THICKNESS_SAMPLES - 1)) * SBS_LUT_MAX_THICKNESS_NM;
    const float cs = (float)a / (float)(SBS_LUT_ANGLE_SAMPLES - 1);
    // snells_law (:96-100)
    const float sin_i = sqrtf(fmax_rs(1.0f - cs * cs, 0.0f));
    const float sin_t = sin_i / n_film;
    const float ct = sqrtf(fmax_rs(1.0f - sin_t * sin_t, 0.0f));
    // fresnel_unpolarized (:103-120), n1 = 1
    const float n1ci = 1.0f * cs, n2ct = n_film * ct;
    const float rs = (n1ci - n2ct) / fmax_rs(n1ci + n2ct, 0.0001f);
    const float n2ci = n_film * cs, n1ct = 1.0f * ct;
    const float rp = (n2ci - n1ct) / fmax_rs(n2ci + n1ct, 0.0001f);
    const float fr = (rs * rs + rp * rp) * 0.5f;
    const float opd = 2.0f * n_film * t_nm * ct;
    // airy_interference constants (:123-133)
    const float omr = fmax_rs(1.0f - fr, 0.001f);
    const float f = 4.0f * fr / (omr * omr);
    const float W[7] = {400.0f, 450.0f, 500.0f, 550.0f, 600.0f, 650.0f, 700.0f};
    float x = 0.f, y = 0.f, z = 0.f;
#pragma unroll
    for (int k = 0; k < 7; ++k) {
        const float phase = 2.0f * kPiF * opd / W[k] + kPiF;
        const float s = (float)sin((double)(phase * 0.5f));
        const float s2 = s * s;
        const float ai = (f * s2) / fmax_rs(1.0f + f * s2, 0.001f);
        x += cie.xyz[k][0] * ai;
        y += cie.xyz[k][1] * ai;
        z += cie.xyz[k][2] * ai;
    }
    x /= 7.0f;
    y /= 7.0f;
    z /= 7.0f;
    // xyz_to_rgb (:158-163)
    const float r = 3.2404542f * x - 1.5371385f * y - 0.4985314f * z;
    const float g = -0.969266f * x + 1.8760108f * y + 0.0415560f * z;
    const float b = 0.0556434f * x - 0.2040259f * y + 1.0572252f * z;
    uchar4 o;
    o.x = (unsigned char)(clamp01(r * intensity) * 255.0f);
    o.y = (unsigned char)(clamp01(g * intensity) * 255.0f);
    o.z = (unsigned char)(clamp01(b * intensity) * 255.0f);
    o.w = 255;
    out[idx] = o;
}

// ---------------------------------------------------------------------------
// wall.wgsl:160-207: Schlick reflectance, transmitted Airy term, three wavelengths.
// ---------------------------------------------------------------------------
__global__ void schlick_kernel(float n_film, float w0, float w1, float w2, const float *t, const float *ci,
                               size_t count, float *out) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const float tk = t[k], c = ci[k];
    const float n_ratio = 1.0f / n_film;
    const float sin_i_sq = 1.0f - c * c;
    const float sin_t_sq = sin_i_sq * n_ratio * n_ratio;
    const float ct = sin_t_sq > 1.0f ? 0.0f : sqrtf(1.0f - sin_t_sq);
    const float opd = 2.0f * n_film * tk * ct;
    const float r0 = ((1.0f - n_film) / (1.0f + n_film)) * ((1.0f - n_film) / (1.0f + n_film));
    const float R = r0 + (1.0f - r0) * powf(1.0f - c, 5.0f);
    const float F = 4.0f * R / ((1.0f - R) * (1.0f - R));
    const float wl[3] = {w0, w1, w2};
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        const float delta = 2.0f * kPiF * opd / wl[ch] + kPiF;
        const float shd = sinf(delta / 2.0f);
        out[3 * k + ch] = 1.0f / (1.0f + F * shd * shd);
    }
}

// ---------------------------------------------------------------------------
// Lookups
// ---------------------------------------------------------------------------
__global__ void lut_rgba8_lookup_kernel(const uchar4 *lut, int W, int H, float max_nm, float intensity,
                                        int addressing, const float *t, const float *ci, size_t count, float *rgb) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const float u = clamp01(t[k] / max_nm);
    const float v = clamp01(ci[k]);
    float x, y;
    if (addressing == SBS_LOOKUP_TEXEL) {
        x = u * (float)W - 0.5f;
        y = v * (float)H - 0.5f;
    } else {
        x = u * (float)(W - 1);
        y = v * (float)(H - 1);
    }
    const float xf = floorf(x), yf = floorf(y);
    const float ax = x - xf, ay = y - yf;
    int x0 = (int)xf, y0 = (int)yf;
    int x1 = x0 + 1, y1 = y0 + 1;
    x0 = min(max(x0, 0), W - 1);
    x1 = min(max(x1, 0), W - 1);
    y0 = min(max(y0, 0), H - 1);
    y1 = min(max(y1, 0), H - 1);
    const uchar4 q00 = lut[(size_t)y0 * W + x0], q10 = lut[(size_t)y0 * W + x1];
    const uchar4 q01 = lut[(size_t)y1 * W + x0], q11 = lut[(size_t)y1 * W + x1];
    const unsigned char a00[3] = {q00.x, q00.y, q00.z}, a10[3] = {q10.x, q10.y, q10.z};
    const unsigned char a01[3] = {q01.x, q01.y, q01.z}, a11[3] = {q11.x, q11.y, q11.z};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float top = (float)a00[c] / 255.0f * (1.0f - ax) + (float)a10[c] / 255.0f * ax;
        const float bot = (float)a01[c] / 255.0f * (1.0f - ax) + (float)a11[c] / 255.0f * ax;
        const float s = top * (1.0f - ay) + bot * ay;
        rgb[3 * k + c] = clamp01(s * intensity);
    }
}

__global__ void lut2d_lookup_kernel(const double *lut, int T, int A, double tmin, double tmax, const double *t,
                                    const double *ci, size_t count, double *rgb) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    double ti = (t[k] - tmin) / (tmax - tmin) * (double)(T - 1);
    ti = ti < 0.0 ? 0.0 : (ti > (double)(T - 1) ? (double)(T - 1) : ti);
    const double cc = ci[k] < 0.0 ? 0.0 : (ci[k] > 1.0 ? 1.0 : ci[k]);
    const double aj = cc * (double)(A - 1);
    int i0 = (int)floor(ti), j0 = (int)floor(aj);
    if (i0 > T - 2) i0 = T - 2;
    if (j0 > A - 2) j0 = A - 2;
    const double fi = ti - (double)i0, fj = aj - (double)j0;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const double v00 = lut[((size_t)i0 * A + j0) * 3 + c], v01 = lut[((size_t)i0 * A + j0 + 1) * 3 + c];
        const double v10 = lut[((size_t)(i0 + 1) * A + j0) * 3 + c];
        const double v11 = lut[((size_t)(i0 + 1) * A + j0 + 1) * 3 + c];
        const double x = v00 * (1.0 - fj) + v01 * fj;
        const double y = v10 * (1.0 - fj) + v11 * fj;
        rgb[3 * k + c] = x * (1.0 - fi) + y * fi;
    }
}

unsigned blocks_for(size_t n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// CIE 1931 Gaussian fits (interference_lut.rs:136-155) at the seven LUT wavelengths, f32 with the
// host libm's expf (the reference evaluates them on the CPU too).
Cie7 cie7() {
    auto g = [](float x, float mean, float sigma) {
        const float t = (x - mean) / sigma;
        return expf(-0.5f * t * t);
    };
    auto mx = [](float a, float b) { return a > b ? a : (b == b ? b : a); };
    const float W[7] = {400.0f, 450.0f, 500.0f, 550.0f, 600.0f, 650.0f, 700.0f};
    Cie7 c{};
    for (int k = 0; k < 7; ++k) {
        const float wl = W[k];
        const float x = 1.056f * g(wl, 599.8f, 37.9f) + 0.362f * g(wl, 442.0f, 16.0f) - 0.065f * g(wl, 501.1f, 20.4f);
        const float y = 0.821f * g(wl, 568.8f, 46.9f) + 0.286f * g(wl, 530.9f, 31.1f);
        const float z = 1.217f * g(wl, 437.0f, 11.8f) + 0.681f * g(wl, 459.0f, 26.0f);
        c.xyz[k][0] = mx(x, 0.0f);
        c.xyz[k][1] = mx(y, 0.0f);
        c.xyz[k][2] = mx(z, 0.0f);
    }
    return c;
}

// Scratch for host-memory calls: device allocation from the stream-ordered pool.
struct Scratch {
    void *p = nullptr;
    cudaStream_t s = nullptr;
    ~Scratch() {
        if (p) cudaFreeAsync(p, s);
    }
};

int check_mem(int mem) {
    if (mem != SBS_MEM_HOST && mem != SBS_MEM_DEVICE) return set_error(SBS_E_INVALID, "bad mem flag %d", mem);
    return SBS_OK;
}

}  // namespace
}  // namespace sbs

using namespace sbs;

extern "C" {

int sbs_interference_color_batch(double n_film, const double wl[3], const void *t_nm, const void *cos_i, size_t n,
                                 int gamma, int prec, void *rgb, int mem, void *stream) {
    clear_error();
    int rc = check_mem(mem);
    if (rc) return rc;
    SBS_CHECK_ARG(wl != nullptr, "wl is null");
    SBS_CHECK_ARG(prec == SBS_PREC_F64 || prec == SBS_PREC_F32, "bad precision %d", prec);
    if (n == 0) return SBS_OK;
    SBS_CHECK_ARG(t_nm && cos_i && rgb, "null pointer");
    rc = require_device();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t es = prec == SBS_PREC_F64 ? sizeof(double) : sizeof(float);
    const void *dt = t_nm, *dc = cos_i;
    void *dout = rgb;
    Scratch scr;
    if (mem == SBS_MEM_HOST) {
        scr.s = s;
        SBS_CUDA_TRY(scratch_alloc((void **)&scr.p, 5 * n * es, s));
        char *base = (char *)scr.p;
        SBS_CUDA_TRY(cudaMemcpyAsync(base, t_nm, n * es, cudaMemcpyHostToDevice, s));
        SBS_CUDA_TRY(cudaMemcpyAsync(base + n * es, cos_i, n * es, cudaMemcpyHostToDevice, s));
        dt = base;
        dc = base + n * es;
        dout = base + 2 * n * es;
    }
    if (prec == SBS_PREC_F64) {
        Wl3 w{{wl[0], wl[1], wl[2]}};
        rgb64_kernel<<<blocks_for(n, 128), 128, 0, s>>>(n_film, w, (const double *)dt, (const double *)dc, n, gamma,
                                                          (double *)dout);
    } else {
        Wl3f w{{(float)wl[0], (float)wl[1], (float)wl[2]}};
        rgb32_kernel<<<blocks_for(n, 128), 128, 0, s>>>((float)n_film, w, (const float *)dt, (const float *)dc, n,
                                                          gamma, (float *)dout);
    }
    SBS_CUDA_TRY(cudaGetLastError());
    if (mem == SBS_MEM_HOST) {
        SBS_CUDA_TRY(cudaMemcpyAsync(rgb, dout, 3 * n * es, cudaMemcpyDeviceToHost, s));
        SBS_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return SBS_OK;
}

int sbs_interference_terms_batch(double n_film, double wl_nm, const double *t_nm, const double *cos_i, size_t n,
                                 double *out, int mem, void *stream) {
    clear_error();
    int rc = check_mem(mem);
    if (rc) return rc;
    if (n == 0) return SBS_OK;
    SBS_CHECK_ARG(t_nm && cos_i && out, "null pointer");
    rc = require_device();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const double *dt = t_nm, *dc = cos_i;
    double *dout = out;
    Scratch scr;
    if (mem == SBS_MEM_HOST) {
        scr.s = s;
        SBS_CUDA_TRY(scratch_alloc((void **)&scr.p, 10 * n * sizeof(double), s));
        double *base = (double *)scr.p;
        SBS_CUDA_TRY(cudaMemcpyAsync(base, t_nm, n * sizeof(double), cudaMemcpyHostToDevice, s));
        SBS_CUDA_TRY(cudaMemcpyAsync(base + n, cos_i, n * sizeof(double), cudaMemcpyHostToDevice, s));
        dt = base;
        dc = base + n;
        dout = base + 2 * n;
    }
    terms64_kernel<<<blocks_for(n, 128), 128, 0, s>>>(n_film, wl_nm, dt, dc, n, dout);
    SBS_CUDA_TRY(cudaGetLastError());
    if (mem == SBS_MEM_HOST) {
        SBS_CUDA_TRY(cudaMemcpyAsync(out, dout, 8 * n * sizeof(double), cudaMemcpyDeviceToHost, s));
        SBS_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return SBS_OK;
}

// Shared host wrapper of path_kernel: inputs a, b, c (c may be null), output out.
static int path_call(double n_film, const double *a, const double *b, const double *c, bool phase, size_t n,
                     double *out, int mem, void *stream) {
    clear_error();
    int rc = check_mem(mem);
    if (rc) return rc;
    if (n == 0) return SBS_OK;
    SBS_CHECK_ARG(a && b && out && (phase || c), "null pointer");
    rc = require_device();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const double *da = a, *db = b, *dc = c;
    double *dout = out;
    Scratch scr;
    if (mem == SBS_MEM_HOST) {
        scr.s = s;
        SBS_CUDA_TRY(scratch_alloc((void **)&scr.p, 4 * n * sizeof(double), s));
        double *base = (double *)scr.p;
        SBS_CUDA_TRY(cudaMemcpyAsync(base, a, n * sizeof(double), cudaMemcpyHostToDevice, s));
        SBS_CUDA_TRY(cudaMemcpyAsync(base + n, b, n * sizeof(double), cudaMemcpyHostToDevice, s));
        da = base;
        db = base + n;
        if (!phase) {
            SBS_CUDA_TRY(cudaMemcpyAsync(base + 2 * n, c, n * sizeof(double), cudaMemcpyHostToDevice, s));
            dc = base + 2 * n;
        }
        dout = base + 3 * n;
    }
    if (phase)
        path_kernel<<<blocks_for(n, 128), 128, 0, s>>>(0.0, nullptr, nullptr, db, da, n, dout);
    else
        path_kernel<<<blocks_for(n, 128), 128, 0, s>>>(n_film, da, db, dc, nullptr, n, dout);
    SBS_CUDA_TRY(cudaGetLastError());
    if (mem == SBS_MEM_HOST) {
        SBS_CUDA_TRY(cudaMemcpyAsync(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost, s));
        SBS_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return SBS_OK;
}

int sbs_optical_path_batch(double n_film, const double *t_nm, const double *cos_t, const double *wl, size_t n,
                           double *opd, int mem, void *stream) {
    return path_call(n_film, t_nm, cos_t, wl, false, n, opd, mem, stream);
}

int sbs_phase_difference_batch(const double *opd_nm, const double *wl, size_t n, double *phase, int mem,
                               void *stream) {
    return path_call(0.0, opd_nm, wl, nullptr, true, n, phase, mem, stream);
}

int sbs_lut1d_build(double n_film, const double wl[3], double tmin, double tmax, uint32_t count, double cos_i,
                    double *rgb, int mem, void *stream) {
    clear_error();
    int rc = check_mem(mem);
    if (rc) return rc;
    SBS_CHECK_ARG(wl != nullptr, "wl is null");
    if (count == 0) return SBS_OK;
    SBS_CHECK_ARG(rgb != nullptr, "rgb is null");
    rc = require_device();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    // thickness_step = (max - min) / (num_samples - 1) as f64 (interference.rs:469)
    const double tstep = (tmax - tmin) / (double)(count - 1);
    double *dout = rgb;
    Scratch scr;
    if (mem == SBS_MEM_HOST) {
        scr.s = s;
        SBS_CUDA_TRY(scratch_alloc((void **)&scr.p, 3 * (size_t)count * sizeof(double), s));
        dout = (double *)scr.p;
    }
    Wl3 w{{wl[0], wl[1], wl[2]}};
    lut1d_kernel<<<blocks_for(count, 128), 128, 0, s>>>(n_film, w, tmin, tstep, (int)count, cos_i, dout);
    SBS_CUDA_TRY(cudaGetLastError());
    if (mem == SBS_MEM_HOST) {
        SBS_CUDA_TRY(cudaMemcpyAsync(rgb, dout, 3 * (size_t)count * sizeof(double), cudaMemcpyDeviceToHost, s));
        SBS_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return SBS_OK;
}

int sbs_lut2d_build(double n_film, const double wl[3], double tmin, double tmax, uint32_t T, uint32_t A, double *rgb,
                    int mem, void *stream) {
    clear_error();
    int rc = check_mem(mem);
    if (rc) return rc;
    SBS_CHECK_ARG(wl != nullptr, "wl is null");
    SBS_CHECK_ARG(T >= 1 && A >= 1, "T and A must be >= 1");
    SBS_CHECK_ARG((uint64_t)T * A <= (1ull << 30), "LUT too large");
    SBS_CHECK_ARG(rgb != nullptr, "rgb is null");
    rc = require_device();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const double tstep = (tmax - tmin) / (double)(T - 1 > 1 ? T - 1 : 1);  // (:498)
    const double astep = 1.0 / (double)(A - 1 > 1 ? A - 1 : 1);            // (:499)
    const size_t n = (size_t)T * A;
    double *dout = rgb;
    Scratch scr;
    if (mem == SBS_MEM_HOST) {
        scr.s = s;
        SBS_CUDA_TRY(scratch_alloc((void **)&scr.p, 3 * n * sizeof(double), s));
        dout = (double *)scr.p;
    }
    Wl3 w{{wl[0], wl[1], wl[2]}};
    lut2d_kernel<<<blocks_for(n, 128), 128, 0, s>>>(n_film, w, tmin, tstep, astep, (int)T, (int)A, dout);
    SBS_CUDA_TRY(cudaGetLastError());
    if (mem == SBS_MEM_HOST) {
        SBS_CUDA_TRY(cudaMemcpyAsync(rgb, dout, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, s));
        SBS_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return SBS_OK;
}

int sbs_interference_lut_rgba8(float n_film, float intensity, uint8_t *out, int mem, void *stream) {
    clear_error();
    int rc = check_mem(mem);
    if (rc) return rc;
    SBS_CHECK_ARG(out != nullptr, "out is null");
    rc = require_device();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)SBS_LUT_THICKNESS_SAMPLES * SBS_LUT_ANGLE_SAMPLES;
    uchar4 *dout = (uchar4 *)out;
    Scratch scr;
    if (mem == SBS_MEM_HOST) {
        scr.s = s;
        SBS_CUDA_TRY(scratch_alloc((void **)&scr.p, 4 * n, s));
        dout = (uchar4 *)scr.p;
    } else {
        SBS_CHECK_ARG(((uintptr_t)out & 3) == 0, "device output must be 4-byte aligned");
    }
    lut_rgba8_kernel<<<blocks_for(n, 128), 128, 0, s>>>(n_film, intensity, cie7(), dout);
    SBS_CUDA_TRY(cudaGetLastError());
    if (mem == SBS_MEM_HOST) {
        SBS_CUDA_TRY(cudaMemcpyAsync(out, dout, 4 * n, cudaMemcpyDeviceToHost, s));
        SBS_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return SBS_OK;
}

int sbs_schlick_rgb_batch(float n_film, const float wl[3], const float *t_nm, const float *cos_i, size_t n,
                          float *out, int mem, void *stream) {
    clear_error();
    int rc = check_mem(mem);
    if (rc) return rc;
    SBS_CHECK_ARG(wl != nullptr, "wl is null");
    if (n == 0) return SBS_OK;
    SBS_CHECK_ARG(t_nm && cos_i && out, "null pointer");
    rc = require_device();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const float *dt = t_nm, *dc = cos_i;
    float *dout = out;
    Scratch scr;
    if (mem == SBS_MEM_HOST) {
        scr.s = s;
        SBS_CUDA_TRY(scratch_alloc((void **)&scr.p, 5 * n * sizeof(float), s));
        float *base = (float *)scr.p;
        SBS_CUDA_TRY(cudaMemcpyAsync(base, t_nm, n * sizeof(float), cudaMemcpyHostToDevice, s));
        SBS_CUDA_TRY(cudaMemcpyAsync(base + n, cos_i, n * sizeof(float), cudaMemcpyHostToDevice, s));
        dt = base;
        dc = base + n;
        dout = base + 2 * n;
    }
    schlick_kernel<<<blocks_for(n, 128), 128, 0, s>>>(n_film, wl[0], wl[1], wl[2], dt, dc, n, dout);
    SBS_CUDA_TRY(cudaGetLastError());
    if (mem == SBS_MEM_HOST) {
        SBS_CUDA_TRY(cudaMemcpyAsync(out, dout, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, s));
        SBS_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return SBS_OK;
}

int sbs_lut_rgba8_lookup_batch(const uint8_t *lut, uint32_t W, uint32_t H, float max_nm, float intensity,
                               int addressing, const float *t_nm, const float *cos_i, size_t n, float *rgb, int mem,
                               void *stream) {
    clear_error();
    int rc = check_mem(mem);
    if (rc) return rc;
    SBS_CHECK_ARG(lut != nullptr, "lut is null");
    SBS_CHECK_ARG(W >= 2 && H >= 2, "LUT must be at least 2 x 2");
    SBS_CHECK_ARG(addressing == SBS_LOOKUP_GRID || addressing == SBS_LOOKUP_TEXEL, "bad addressing %d", addressing);
    SBS_CHECK_ARG(max_nm > 0.f, "max_nm must be > 0");
    if (n == 0) return SBS_OK;
    SBS_CHECK_ARG(t_nm && cos_i && rgb, "null pointer");
    rc = require_device();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t lut_bytes = (size_t)W * H * 4;
    const uchar4 *dl = (const uchar4 *)lut;
    const float *dt = t_nm, *dc = cos_i;
    float *dout = rgb;
    Scratch scr;
    if (mem == SBS_MEM_HOST) {
        scr.s = s;
        SBS_CUDA_TRY(scratch_alloc((void **)&scr.p, 5 * n * sizeof(float) + lut_bytes + 16, s));
        float *base = (float *)scr.p;
        dt = base;
        dc = base + n;
        dout = base + 2 * n;
        uchar4 *l = (uchar4 *)(base + 5 * n);
        SBS_CUDA_TRY(cudaMemcpyAsync(base, t_nm, n * sizeof(float), cudaMemcpyHostToDevice, s));
        SBS_CUDA_TRY(cudaMemcpyAsync(base + n, cos_i, n * sizeof(float), cudaMemcpyHostToDevice, s));
        SBS_CUDA_TRY(cudaMemcpyAsync(l, lut, lut_bytes, cudaMemcpyHostToDevice, s));
        dl = l;
    } else {
        SBS_CHECK_ARG(((uintptr_t)lut & 3) == 0, "device LUT must be 4-byte aligned");
    }
    lut_rgba8_lookup_kernel<<<blocks_for(n, 128), 128, 0, s>>>(dl, (int)W, (int)H, max_nm, intensity, addressing, dt,
                                                               dc, n, dout);
    SBS_CUDA_TRY(cudaGetLastError());
    if (mem == SBS_MEM_HOST) {
        SBS_CUDA_TRY(cudaMemcpyAsync(rgb, dout, 3 * n * sizeof(float), cudaMemcpyDeviceToHost, s));
        SBS_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return SBS_OK;
}

int sbs_lut2d_lookup_batch(const double *lut, uint32_t T, uint32_t A, double tmin, double tmax, const double *t_nm,
                           const double *cos_i, size_t n, double *rgb, int mem, void *stream) {
    clear_error();
    int rc = check_mem(mem);
    if (rc) return rc;
    SBS_CHECK_ARG(lut != nullptr, "lut is null");
    SBS_CHECK_ARG(T >= 2 && A >= 2, "LUT must be at least 2 x 2");
    SBS_CHECK_ARG(tmax > tmin, "tmax must exceed tmin");
    if (n == 0) return SBS_OK;
    SBS_CHECK_ARG(t_nm && cos_i && rgb, "null pointer");
    rc = require_device();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t lut_n = (size_t)T * A * 3;
    const double *dl = lut, *dt = t_nm, *dc = cos_i;
    double *dout = rgb;
    Scratch scr;
    if (mem == SBS_MEM_HOST) {
        scr.s = s;
        SBS_CUDA_TRY(scratch_alloc((void **)&scr.p, (5 * n + lut_n) * sizeof(double), s));
        double *base = (double *)scr.p;
        SBS_CUDA_TRY(cudaMemcpyAsync(base, t_nm, n * sizeof(double), cudaMemcpyHostToDevice, s));
        SBS_CUDA_TRY(cudaMemcpyAsync(base + n, cos_i, n * sizeof(double), cudaMemcpyHostToDevice, s));
        SBS_CUDA_TRY(cudaMemcpyAsync(base + 5 * n, lut, lut_n * sizeof(double), cudaMemcpyHostToDevice, s));
        dt = base;
        dc = base + n;
        dout = base + 2 * n;
        dl = base + 5 * n;
    }
    lut2d_lookup_kernel<<<blocks_for(n, 128), 128, 0, s>>>(dl, (int)T, (int)A, tmin, tmax, dt, dc, n, dout);
    SBS_CUDA_TRY(cudaGetLastError());
    if (mem == SBS_MEM_HOST) {
        SBS_CUDA_TRY(cudaMemcpyAsync(rgb, dout, 3 * n * sizeof(double), cudaMemcpyDeviceToHost, s));
        SBS_CUDA_TRY(cudaStreamSynchronize(s));
    }
    return SBS_OK;
}

}  // extern "C"
