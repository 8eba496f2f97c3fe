// Parity oracle: CPU restatement of the reference's thin-film interference
// arithmetic. Test infrastructure only (see oracle.h).
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace {
const double kPi = 3.14159265358979323846;
const double kAir = 1.0;  // constants::REFRACTIVE_INDEX_AIR (interference.rs:36)

double clamp64(double x, double lo, double hi) { return std::min(std::max(x, lo), hi); }
float maxf(float a, float b) { return a > b ? a : (b == b ? b : a); }  // f32::max
float clampf(float x, float lo, float hi) { return x < lo ? lo : (x > hi ? hi : x); }
}  // namespace

extern "C" {

// calculate_transmission_angle_cos (interference.rs:197-211)
double orc_transmission_angle_cos(double n_film, double cos_i) {
    double c = clamp64(cos_i, -1.0, 1.0);
    double sin_i = std::sqrt(1.0 - c * c);
    double sin_t = (kAir / n_film) * sin_i;
    if (std::fabs(sin_t) > 1.0) return 0.0;
    return std::sqrt(1.0 - sin_t * sin_t);
}

// calculate_optical_path_difference (interference.rs:226-238)
double orc_optical_path_difference(double n_film, double t_nm, double cos_t, double wl_nm) {
    double geometric_path = 2.0 * n_film * t_nm * cos_t;
    return geometric_path + wl_nm / 2.0;
}

// calculate_phase_difference (interference.rs:248-254)
double orc_phase_difference(double opd_nm, double wl_nm) { return 2.0 * kPi * opd_nm / wl_nm; }

// calculate_fresnel_reflection (interference.rs:266-298)
void orc_fresnel(double n_film, double cos_i, double out3[3]) {
    double ci = clamp64(cos_i, -1.0, 1.0);
    double ct = orc_transmission_angle_cos(n_film, ci);
    double n1 = kAir, n2 = n_film;
    double n1_cos_i = n1 * ci, n2_cos_t = n2 * ct, n2_cos_i = n2 * ci, n1_cos_t = n1 * ct;
    double rs = (n1_cos_i - n2_cos_t) / (n1_cos_i + n2_cos_t);
    double Rs = rs * rs;
    double rp = (n2_cos_i - n1_cos_t) / (n2_cos_i + n1_cos_t);
    double Rp = rp * rp;
    out3[0] = Rs;
    out3[1] = Rp;
    out3[2] = (Rs + Rp) / 2.0;
}

// calculate_reflected_intensity (interference.rs:312-353)
double orc_reflected_intensity(double n_film, double t_nm, double cos_i, double wl_nm) {
    if (t_nm <= 0.0) return 0.0;
    double ct = orc_transmission_angle_cos(n_film, cos_i);
    double opd = orc_optical_path_difference(n_film, t_nm, ct, wl_nm);
    double phase = orc_phase_difference(opd, wl_nm);
    double fr[3];
    orc_fresnel(n_film, cos_i, fr);
    double R = fr[2];
    double cp = std::cos(phase);
    double num = 2.0 * R * (1.0 - cp);
    double den = 1.0 + R * R - 2.0 * R * cp;
    if (std::fabs(den) < 2.220446049250313e-16) return R;  // f64::EPSILON
    return clamp64(num / den, 0.0, 1.0);
}

// calculate_interference_color / _linear (interference.rs:380-426), RgbColor::new clamp (:54-60)
void orc_interference_color(double n_film, const double wl[3], double t_nm, double cos_i, int gamma,
                            double rgb[3]) {
    for (int c = 0; c < 3; ++c) {
        double I = orc_reflected_intensity(n_film, t_nm, cos_i, wl[c]);
        if (gamma) I = std::pow(I, 1.0 / 2.2);
        rgb[c] = clamp64(I, 0.0, 1.0);
    }
}

void orc_interference_color_batch(double n_film, const double wl[3], const double *t_nm, const double *cos_i,
                                  size_t n, int gamma, double *rgb) {
    for (size_t k = 0; k < n; ++k) orc_interference_color(n_film, wl, t_nm[k], cos_i[k], gamma, rgb + 3 * k);
}

// generate_color_lookup_table (interference.rs:461-477)
void orc_lut1d(double n_film, const double wl[3], double tmin, double tmax, uint32_t count, double cos_i,
               double *rgb) {
    double step = (tmax - tmin) / (double)(count - 1);
    for (uint32_t i = 0; i < count; ++i)
        orc_interference_color(n_film, wl, tmin + (double)i * step, cos_i, 1, rgb + 3 * (size_t)i);
}

// generate_2d_color_lookup_table (interference.rs:491-512)
void orc_lut2d(double n_film, const double wl[3], double tmin, double tmax, uint32_t T, uint32_t A,
               double *rgb) {
    double tstep = (tmax - tmin) / (double)std::max<uint32_t>(T - 1, 1);
    double astep = 1.0 / (double)std::max<uint32_t>(A - 1, 1);
    for (uint32_t i = 0; i < T; ++i) {
        double t = tmin + (double)i * tstep;
        for (uint32_t j = 0; j < A; ++j)
            orc_interference_color(n_film, wl, t, (double)j * astep, 1, rgb + 3 * ((size_t)i * A + j));
    }
}

// ------------------------------------------------------------------
// interference_lut.rs (f32)
// ------------------------------------------------------------------
float orc_lut_snells_law(float cos_i, float n_film) {  // :96-100
    float sin_i = std::sqrt(maxf(1.0f - cos_i * cos_i, 0.0f));
    float sin_t = sin_i / n_film;
    return std::sqrt(maxf(1.0f - sin_t * sin_t, 0.0f));
}

float orc_lut_fresnel_unpolarized(float ci, float ct, float n1, float n2) {  // :103-120
    float n1ci = n1 * ci, n2ct = n2 * ct;
    float rs = (n1ci - n2ct) / maxf(n1ci + n2ct, 0.0001f);
    float n2ci = n2 * ci, n1ct = n1 * ct;
    float rp = (n2ci - n1ct) / maxf(n2ci + n1ct, 0.0001f);
    return (rs * rs + rp * rp) * 0.5f;
}

static float airy7(float phase, float R) {  // :123-133
    float omr = maxf(1.0f - R, 0.001f);
    float f = 4.0f * R / (omr * omr);
    float s = std::sin(phase * 0.5f);
    float s2 = s * s;
    return (f * s2) / maxf(1.0f + f * s2, 0.001f);
}

static float gauss(float x, float mean, float sigma) {  // :152-155
    float t = (x - mean) / sigma;
    return std::exp(-0.5f * t * t);
}

static void cie(float wl, float out[3]) {  // :136-148
    float x = 1.056f * gauss(wl, 599.8f, 37.9f) + 0.362f * gauss(wl, 442.0f, 16.0f) -
              0.065f * gauss(wl, 501.1f, 20.4f);
    float y = 0.821f * gauss(wl, 568.8f, 46.9f) + 0.286f * gauss(wl, 530.9f, 31.1f);
    float z = 1.217f * gauss(wl, 437.0f, 11.8f) + 0.681f * gauss(wl, 459.0f, 26.0f);
    out[0] = maxf(x, 0.0f);
    out[1] = maxf(y, 0.0f);
    out[2] = maxf(z, 0.0f);
}

// thin_film_interference (interference_lut.rs:45-93)
void orc_thin_film_interference7(float t_nm, float cos_t_in, float n_film, float intensity, float out3[3]) {
    static const float W[7] = {400.0f, 450.0f, 500.0f, 550.0f, 600.0f, 650.0f, 700.0f};
    const float PI = 3.14159265358979323846f;  // std::f32::consts::PI
    float ct = orc_lut_snells_law(cos_t_in, n_film);
    float fr = orc_lut_fresnel_unpolarized(cos_t_in, ct, 1.0f, n_film);
    float opd = 2.0f * n_film * t_nm * ct;
    float xyz[3] = {0.f, 0.f, 0.f};
    for (int k = 0; k < 7; ++k) {
        float phase = 2.0f * PI * opd / W[k] + PI;
        float a = airy7(phase, fr);
        float c[3];
        cie(W[k], c);
        xyz[0] += c[0] * a;
        xyz[1] += c[1] * a;
        xyz[2] += c[2] * a;
    }
    xyz[0] /= 7.0f;
    xyz[1] /= 7.0f;
    xyz[2] /= 7.0f;
    // xyz_to_rgb (:158-163)
    float r = 3.2404542f * xyz[0] - 1.5371385f * xyz[1] - 0.4985314f * xyz[2];
    float g = -0.969266f * xyz[0] + 1.8760108f * xyz[1] + 0.0415560f * xyz[2];
    float b = 0.0556434f * xyz[0] - 0.2040259f * xyz[1] + 1.0572252f * xyz[2];
    out3[0] = r * intensity;
    out3[1] = g * intensity;
    out3[2] = b * intensity;
}

// generate_interference_lut (interference_lut.rs:18-41): [angle 64][thickness 256][RGBA]
void orc_interference_lut_rgba8(float n_film, float intensity, uint8_t *out) {
    const uint32_t TS = 256, AS = 64;
    const float MAXNM = 2000.0f;
    size_t o = 0;
    for (uint32_t a = 0; a < AS; ++a) {
        for (uint32_t t = 0; t < TS; ++t) {
            float t_nm = ((float)t / (float)(TS - 1)) * MAXNM;
            float cs = (float)a / (float)(AS - 1);
            float rgb[3];
            orc_thin_film_interference7(t_nm, cs, n_film, intensity, rgb);
            for (int c = 0; c < 3; ++c) out[o++] = (uint8_t)(clampf(rgb[c], 0.0f, 1.0f) * 255.0f);  // truncation
            out[o++] = 255;
        }
    }
}

// ------------------------------------------------------------------
// wall.wgsl:160-207 Schlick reflectance with transmitted Airy, f32
// ------------------------------------------------------------------
float orc_schlick_interference(float t_nm, float wl, float cos_i, float n_film) {
    const float PI = 3.14159265358979323846f;
    float n_ratio = 1.0f / n_film;
    // snells_law_cos_theta_t
    float sin_i_sq = 1.0f - cos_i * cos_i;
    float sin_t_sq = sin_i_sq * n_ratio * n_ratio;
    float ct = sin_t_sq > 1.0f ? 0.0f : std::sqrt(1.0f - sin_t_sq);
    float opd = 2.0f * n_film * t_nm * ct;
    float delta = 2.0f * PI * opd / wl + PI;
    // fresnel_schlick
    float n_air = 1.0f;
    float r0 = ((n_air - n_film) / (n_air + n_film)) * ((n_air - n_film) / (n_air + n_film));
    float R = r0 + (1.0f - r0) * std::pow(1.0f - cos_i, 5.0f);
    // airy_intensity (transmitted)
    float F = 4.0f * R / ((1.0f - R) * (1.0f - R));
    float shd = std::sin(delta / 2.0f);
    return 1.0f / (1.0f + F * shd * shd);
}

// ------------------------------------------------------------------
// Lookups
// ------------------------------------------------------------------
// bubble.wgsl:425-439 with a ClampToEdge/Linear sampler (pipeline.rs:350-359): texel centres at
// (i+0.5)/W; unorm8 texels decode as v/255.
void orc_lut_rgba8_sample(const uint8_t *lut, uint32_t W, uint32_t H, float t_nm, float cos_i, float max_nm,
                          float intensity, float out3[3]) {
    float u = clampf(t_nm / max_nm, 0.0f, 1.0f);
    float v = clampf(cos_i, 0.0f, 1.0f);
    float x = u * (float)W - 0.5f, y = v * (float)H - 0.5f;
    float xf = std::floor(x), yf = std::floor(y);
    float ax = x - xf, ay = y - yf;
    int x0 = (int)xf, y0 = (int)yf;
    int x1 = x0 + 1, y1 = y0 + 1;
    auto cx = [&](int i) { return std::min(std::max(i, 0), (int)W - 1); };
    auto cy = [&](int i) { return std::min(std::max(i, 0), (int)H - 1); };
    for (int c = 0; c < 3; ++c) {
        auto tex = [&](int xi, int yi) { return (float)lut[((size_t)cy(yi) * W + cx(xi)) * 4 + c] / 255.0f; };
        float top = tex(x0, y0) * (1.0f - ax) + tex(x1, y0) * ax;
        float bot = tex(x0, y1) * (1.0f - ax) + tex(x1, y1) * ax;
        float s = top * (1.0f - ay) + bot * ay;
        out3[c] = clampf(s * intensity, 0.0f, 1.0f);
    }
}

void orc_lut2d_lookup(const double *lut, uint32_t T, uint32_t A, double tmin, double tmax, double t_nm,
                      double cos_i, double out3[3]) {
    double ti = (t_nm - tmin) / (tmax - tmin) * (double)(T - 1);
    ti = clamp64(ti, 0.0, (double)(T - 1));
    double aj = clamp64(cos_i, 0.0, 1.0) * (double)(A - 1);
    uint32_t i0 = std::min((uint32_t)std::floor(ti), T - 2);
    uint32_t j0 = std::min((uint32_t)std::floor(aj), A - 2);
    double fi = ti - (double)i0, fj = aj - (double)j0;
    for (int c = 0; c < 3; ++c) {
        double v00 = lut[((size_t)i0 * A + j0) * 3 + c], v01 = lut[((size_t)i0 * A + j0 + 1) * 3 + c];
        double v10 = lut[((size_t)(i0 + 1) * A + j0) * 3 + c], v11 = lut[((size_t)(i0 + 1) * A + j0 + 1) * 3 + c];
        double a = v00 * (1.0 - fj) + v01 * fj;
        double b = v10 * (1.0 - fj) + v11 * fj;
        out3[c] = a * (1.0 - fi) + b * fi;
    }
}

// get_thickness (drainage.rs:516-552) on a bare field
static double field_query(const double *h, uint32_t nt, uint32_t np, double theta, double phi) {
    double dth = kPi / (double)(nt - 1), dph = 2.0 * kPi / (double)np;
    double theta_clamped = std::min(std::max(theta, 0.0), kPi);
    double two_pi = 2.0 * kPi;
    double r = std::fmod(phi, two_pi);
    double phin = r < 0.0 ? r + two_pi : r;
    double tc = theta_clamped / dth, pc = phin / dph;
    double tfl = std::floor(tc), pfl = std::floor(pc);
    size_t til = tfl <= 0.0 ? 0 : (size_t)tfl;
    til = std::min(til, (size_t)nt - 2);
    size_t pil = (pfl <= 0.0 ? 0 : (size_t)pfl) % np;
    size_t tih = til + 1, pih = (pil + 1) % np;
    double tf = tc - (double)til, pf = pc - (double)pil;
    double v0 = h[til * np + pil] * (1.0 - pf) + h[til * np + pih] * pf;
    double v1 = h[tih * np + pil] * (1.0 - pf) + h[tih * np + pih] * pf;
    return v0 * (1.0 - tf) + v1 * tf;
}

void orc_vertex_colors(const double *field, uint32_t nt, uint32_t np, const double *xyz, size_t nv,
                       const double *lut, uint32_t T, uint32_t A, double tmin, double tmax, double *rgb) {
    for (size_t k = 0; k < nv; ++k) {
        double x = xyz[3 * k], y = xyz[3 * k + 1], z = xyz[3 * k + 2];
        double theta = std::acos(std::min(std::max(y, -1.0), 1.0));
        double phi = std::atan2(z, x);
        if (phi < 0.0) phi += 2.0 * kPi;
        double t_nm = field_query(field, nt, np, theta, phi) * 1e9;
        orc_lut2d_lookup(lut, T, A, tmin, tmax, t_nm, std::fabs(z), rgb + 3 * k);
    }
}

// ------------------------------------------------------------------
// Spectral reflectance contracted against a colour-matching matrix, f64
// ------------------------------------------------------------------
void orc_spectral_rgb(const float *t_nm, const float *cos_i, const float *n_film, size_t n, const double *wl,
                      uint32_t nl, const double *cmf, double *rgb) {
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < (int64_t)n; ++k) {
        double ci = (double)cos_i[k], nf = (double)n_film[k], t = (double)t_nm[k];
        double sin_i = std::sqrt(std::max(1.0 - ci * ci, 0.0));
        double sin_t = sin_i / nf;
        double ct = std::sqrt(std::max(1.0 - sin_t * sin_t, 0.0));
        double rs = (ci - nf * ct) / std::max(ci + nf * ct, 1e-4);
        double rp = (nf * ci - ct) / std::max(nf * ci + ct, 1e-4);
        double R = (rs * rs + rp * rp) * 0.5;
        double omr = std::max(1.0 - R, 0.001);
        double F = 4.0 * R / (omr * omr);
        double opd = 2.0 * nf * t * ct;
        double acc[3] = {0.0, 0.0, 0.0};
        for (uint32_t l = 0; l < nl; ++l) {
            double phase = 2.0 * kPi * opd / wl[l] + kPi;
            double s = std::sin(phase * 0.5);
            double s2 = s * s;
            double I = (F * s2) / std::max(1.0 + F * s2, 0.001);
            acc[0] += I * cmf[3 * l + 0];
            acc[1] += I * cmf[3 * l + 1];
            acc[2] += I * cmf[3 * l + 2];
        }
        rgb[3 * k + 0] = acc[0];
        rgb[3 * k + 1] = acc[1];
        rgb[3 * k + 2] = acc[2];
    }
}

}  // extern "C"
