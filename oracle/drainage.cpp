// Parity oracle: CPU restatement of the reference's drainage arithmetic.
// Test infrastructure only (see oracle.h). Each function names the reference
// lines it restates.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double kPi = 3.14159265358979323846;
const double kHalfPi = kPi / 2.0;

// TfeFront (drainage.rs:23-88)
struct Front {
    double phi_center, extent, width, velocity;
    void advance(double dt) { extent = std::min(extent + velocity * dt, kHalfPi); }  // :47-49
    bool contains(double theta, double phi) const {                                     // :55-71
        double dist_from_equator = std::fabs(theta - kHalfPi);
        if (dist_from_equator > extent) return false;
        double phi_diff = std::fabs(phi - phi_center);
        if (phi_diff > kPi) phi_diff = 2.0 * kPi - phi_diff;
        return phi_diff < width / 2.0;
    }
};

}  // namespace

struct orc_sim {
    uint32_t nt, np;
    int precision;  // 0 f64 faithful, 1 f32 kernel order, 2 f32x2 (compensated) kernel order
    int threads;
    double dth, dph;
    std::vector<double> h, scratch;    // f64 mode
    std::vector<float> hf, scratchf;   // f32 modes (high words)
    std::vector<float> lf, scratchl;   // f32x2 low words
    double density, gravity, viscosity, diffusion, critical, radius;
    double current_time;
    std::vector<Front> fronts;
    double tfe_ratio;
    bool mr_enabled;
    double next_spawn, spawn_interval;
    // f32 kernel-order per-row coefficients
    std::vector<float> rowA, rowE, rowF;
    float cb, cDR2;
};

namespace {

// ThicknessField::new spacing (drainage.rs:121-133)
void init_geometry(orc_sim *s) {
    s->dth = kPi / (double)(s->nt - 1);
    s->dph = 2.0 * kPi / (double)s->np;
}

// Per-row coefficients of the CUDA kernel's f32 arithmetic, computed in f64 and rounded once.
// This is the same closed form the product computes on its host; the kernel-order oracle
// uses it so that GPU and oracle round identically.
void init_rows_f32(orc_sim *s) {
    s->rowA.assign(s->nt, 0.f);
    s->rowE.assign(s->nt, 0.f);
    s->rowF.assign(s->nt, 0.f);
    double coef = s->density * s->gravity / (3.0 * s->viscosity);
    for (uint32_t i = 0; i < s->nt; ++i) {
        double th = (double)i * s->dth;
        double sn = std::sin(th), cs = std::cos(th);
        double ss = std::fabs(sn) < 1e-10 ? std::copysign(1e-10, sn) : sn;  // drainage.rs:320-324
        s->rowA[i] = (float)(-coef * sn);
        s->rowE[i] = (float)((cs / ss) / (2.0 * s->dth));
        s->rowF[i] = (float)((1.0 / (ss * ss)) / (s->dph * s->dph));
    }
    s->cb = (float)(1.0 / (s->dth * s->dth));
    s->cDR2 = (float)(s->diffusion / (s->radius * s->radius));
}

// DrainageSimulator::step stencil loop, f64 (drainage.rs:298-381)
void stencil_f64(orc_sim *s, double dt) {
    const uint32_t nt = s->nt, np = s->np;
    const double dth = s->dth, dph = s->dph;
    const double drainage_coefficient = s->density * s->gravity / (3.0 * s->viscosity);
    const double diffusion_scaled = s->diffusion;
    std::memcpy(s->scratch.data(), s->h.data(), sizeof(double) * nt * np);  // :311
    const double *sc = s->scratch.data();
    double *th = s->h.data();
    const double crit = s->critical, R = s->radius;
#pragma omp parallel for schedule(static) num_threads(s->threads > 0 ? s->threads : omp_get_max_threads())
    for (int64_t ti = 1; ti < (int64_t)nt - 1; ++ti) {
        double theta = (double)ti * dth;
        double sin_theta = std::sin(theta);
        double cos_theta = std::cos(theta);
        double sin_theta_safe = std::fabs(sin_theta) < 1e-10 ? std::copysign(1e-10, sin_theta) : sin_theta;
        for (uint32_t pj = 0; pj < np; ++pj) {
            double hc = sc[ti * np + pj];
            if (hc < crit) continue;  // :331
            double htm = sc[(ti - 1) * np + pj];
            double htp = sc[(ti + 1) * np + pj];
            uint32_t pm = (pj + np - 1) % np, pp = (pj + 1) % np;
            double hpm = sc[ti * np + pm];
            double hpp = sc[ti * np + pp];
            double cubed = hc * hc * hc;
            double drainage_term = -drainage_coefficient * cubed * sin_theta;
            double radius_squared = R * R;
            double d2t = (htp - 2.0 * hc + htm) / (dth * dth);
            double d1t = (htp - htm) / (2.0 * dth);
            double d2p = (hpp - 2.0 * hc + hpm) / (dph * dph);
            double lap = (d2t + cos_theta / sin_theta_safe * d1t + d2p / (sin_theta_safe * sin_theta_safe)) /
                         radius_squared;
            double diffusion_term = diffusion_scaled * lap;
            double dh_dt = drainage_term + diffusion_term;
            double nh = hc + dt * dh_dt;
            th[ti * np + pj] = nh > 0.0 ? nh : 0.0;  // f64::max(x, 0.0)
        }
    }
}

// Same loop in the CUDA kernel's f32 order (row coefficients, explicit fmaf); with x2 the cells
// carry hi + lo words and the update is an error-free TwoSum.
void stencil_f32k(orc_sim *s, double dt) {
    const uint32_t nt = s->nt, np = s->np;
    const bool x2 = s->precision == 2;
    std::memcpy(s->scratchf.data(), s->hf.data(), sizeof(float) * nt * np);
    if (x2) std::memcpy(s->scratchl.data(), s->lf.data(), sizeof(float) * nt * np);
    const float *sc = s->scratchf.data();
    const float *sl = s->scratchl.data();
    float *th = s->hf.data();
    float *tl = s->lf.data();
    const float crit = (float)s->critical;
    const float b = s->cb, DR2 = s->cDR2, dtf = (float)dt;
#pragma omp parallel for schedule(static) num_threads(s->threads > 0 ? s->threads : omp_get_max_threads())
    for (int64_t ti = 1; ti < (int64_t)nt - 1; ++ti) {
        const float A = s->rowA[ti], E = s->rowE[ti], F = s->rowF[ti];
        for (uint32_t pj = 0; pj < np; ++pj) {
            const size_t ic = ti * np + pj, itm = (ti - 1) * np + pj, itp = (ti + 1) * np + pj;
            const size_t ipm = ti * np + (pj + np - 1) % np, ipp = ti * np + (pj + 1) % np;
            float h = sc[ic];
            if (h < crit) continue;
            float tm = sc[itm], tp = sc[itp], pm = sc[ipm], pp = sc[ipp];
            float lt = (tp - h) + (tm - h);
            float d1 = tp - tm;
            float lp = (pp - h) + (pm - h);
            float l = 0.f;
            if (x2) {
                l = sl[ic];
                lt = lt + ((sl[itp] - l) + (sl[itm] - l));
                d1 = d1 + (sl[itp] - sl[itm]);
                lp = lp + ((sl[ipp] - l) + (sl[ipm] - l));
            }
            float L = std::fma(F, lp, std::fma(E, d1, b * lt));
            float h3 = (h * h) * h;
            float inc = std::fma(DR2, L, A * h3);
            if (x2) {
                float t = std::fma(dtf, inc, l);
                float sm = h + t;
                float bb = sm - h;
                float e = (h - (sm - bb)) + (t - bb);
                th[ic] = sm < 0.f ? 0.f : sm;
                tl[ic] = sm < 0.f ? 0.f : e;
            } else {
                float v = std::fma(dtf, inc, h);
                th[ic] = v > 0.f ? v : 0.f;
            }
        }
    }
}

// Kernel order of a ring sum: every f32 word (the thickness, plus the low word in the
// compensated storage) as a two's-complement integer in units of 2^-96 m, truncated toward
// zero, summed exactly in 256 bits (wide enough for any finite f32 word); the total rounded to
// the nearest double (ties to even). An infinite or NaN word makes the sum NaN. Integer addition
// does not depend on the order, so this equals the kernels' per-lane / per-warp / per-block
// groupings bit for bit.
struct Wide {
    unsigned __int128 lo = 0, hi = 0;  // two's complement, 256 bits
};

void wide_add(Wide &a, unsigned __int128 lo, unsigned __int128 hi) {
    const unsigned __int128 s = a.lo + lo;
    a.hi = a.hi + hi + (s < lo ? 1 : 0);
    a.lo = s;
}

bool fix_word(float x, Wide &acc) {
    if (!std::isfinite(x)) return false;
    if (x == 0.0f) return true;
    int e = 0;
    const float fr = std::frexp(x, &e);                        // x = fr 2^e, 0.5 <= |fr| < 1
    const long long m = (long long)std::ldexp((double)fr, 24); // exact: 24 significant bits
    const int sh = e - 24 + 96;                                // x = m 2^(sh - 96)
    const unsigned __int128 mag = (unsigned __int128)(m < 0 ? -m : m);
    unsigned __int128 lo = 0, hi = 0;
    if (sh < 0)
        lo = sh <= -64 ? 0 : mag >> -sh;
    else if (sh < 128) {
        lo = mag << sh;
        hi = sh > 104 ? mag >> (128 - sh) : 0;
    } else {
        hi = mag << (sh - 128);
    }
    if (m < 0) {
        lo = ~lo + 1;
        hi = ~hi + (lo == 0 ? 1 : 0);
    }
    wide_add(acc, lo, hi);
    return true;
}

bool wide_bit(const Wide &v, int i) { return i < 128 ? ((v.lo >> i) & 1) != 0 : ((v.hi >> (i - 128)) & 1) != 0; }

double fix_total_to_double(Wide v) {
    const bool neg = (v.hi >> 127) != 0;
    if (neg) {
        v.lo = ~v.lo + 1;
        v.hi = ~v.hi + (v.lo == 0 ? 1 : 0);
    }
    int nbits = 0;
    for (int i = 255; i >= 0; --i)
        if (wide_bit(v, i)) {
            nbits = i + 1;
            break;
        }
    unsigned long long q = 0;
    int drop = 0;
    if (nbits <= 53) {
        q = (unsigned long long)v.lo;
    } else {
        drop = nbits - 53;
        for (int i = nbits - 1; i >= drop; --i) q = (q << 1) | (wide_bit(v, i) ? 1ull : 0ull);
        const bool round = wide_bit(v, drop - 1);
        bool sticky = false;
        for (int i = drop - 2; i >= 0 && !sticky; --i) sticky = wide_bit(v, i);
        if (round && (sticky || (q & 1))) q += 1;  // round half to even
    }
    const double d = std::ldexp((double)q, drop - 96);
    return neg ? -d : d;
}

double ring_sum(const orc_sim *s, uint32_t row) {
    Wide tot;
    bool ok = true;
    for (uint32_t j = 0; j < s->np; ++j) {
        if (!fix_word(s->hf[(size_t)row * s->np + j], tot)) ok = false;
        if (s->precision == 2 && !fix_word(s->lf[(size_t)row * s->np + j], tot)) ok = false;
    }
    return ok ? fix_total_to_double(tot) : std::nan("");
}

// update_poles (drainage.rs:480-503): ring means in f64, sequential order.
void update_poles(orc_sim *s) {
    const uint32_t np = s->np, last = s->nt - 1;
    if (s->precision == 0) {
        double top = 0.0, bot = 0.0;
        for (uint32_t j = 0; j < np; ++j) top += s->h[1 * np + j];
        double ta = top / (double)np;
        for (uint32_t j = 0; j < np; ++j) s->h[j] = ta;
        for (uint32_t j = 0; j < np; ++j) bot += s->h[(size_t)(last - 1) * np + j];
        double ba = bot / (double)np;
        for (uint32_t j = 0; j < np; ++j) s->h[(size_t)last * np + j] = ba;
    } else {
        // kernel order: exact fixed-point ring sums, mean in f64, stored rounded (f32) or split (f32x2)
        const double mt = ring_sum(s, 1) / (double)np;
        const double mb = ring_sum(s, last - 1) / (double)np;
        const float th = (float)mt, bh = (float)mb;
        for (uint32_t j = 0; j < np; ++j) {
            s->hf[j] = th;
            s->hf[(size_t)last * np + j] = bh;
            if (s->precision == 2) {
                s->lf[j] = (float)(mt - (double)th);
                s->lf[(size_t)last * np + j] = (float)(mb - (double)bh);
            }
        }
    }
}

// spawn_tfe_front (drainage.rs:464-477)
void spawn_front(orc_sim *s) {
    double t = s->current_time;
    double phi = std::fabs(std::sin(t * 7.89 + 1.23)) * 2.0 * kPi;
    double width = 0.3 + std::fabs(std::sin(t * 3.21)) * 0.4;
    double velocity = 0.05 + std::fabs(std::cos(t * 5.67)) * 0.05;
    s->fronts.push_back(Front{phi, 0.0, width, velocity});
    if (s->fronts.size() > 8) s->fronts.erase(s->fronts.begin());
}

// update_marginal_regeneration (drainage.rs:395-461)
void update_mr(orc_sim *s, double dt) {
    s->next_spawn -= dt;
    if (s->next_spawn <= 0.0) {
        spawn_front(s);
        double random_factor = 0.5 + std::fabs(std::sin(s->current_time * 12.345));
        s->next_spawn = s->spawn_interval * random_factor;
    }
    for (auto &f : s->fronts) f.advance(dt);
    s->fronts.erase(std::remove_if(s->fronts.begin(), s->fronts.end(),
                                   [](const Front &f) { return !(f.extent < kHalfPi * 0.95); }),
                    s->fronts.end());
    if (s->fronts.empty()) return;
    const uint32_t nt = s->nt, np = s->np;
    size_t min_idx = nt, max_idx = 0;
    for (const auto &f : s->fronts) {
        double mn = kHalfPi - f.extent, mx = kHalfPi + f.extent;
        double a = std::floor(mn / s->dth), b = std::ceil(mx / s->dth);
        size_t lo = a <= 0.0 ? 0 : (size_t)a;  // `as usize` saturates at 0
        size_t hi = b <= 0.0 ? 0 : (size_t)b;
        hi = std::min(hi, (size_t)nt - 1);
        min_idx = std::min(min_idx, lo);
        max_idx = std::max(max_idx, hi);
    }
    min_idx = std::min(min_idx, (size_t)nt - 1);
    const double rr = (1.0 - s->tfe_ratio) * 0.5;
    const double factor64 = 1.0 - rr * dt;
    const float factor32 = (float)factor64;
    const float factor32_lo = (float)(factor64 - (double)factor32);
    for (size_t ti = min_idx; ti <= max_idx; ++ti) {
        double theta = (double)ti * s->dth;
        for (uint32_t pj = 0; pj < np; ++pj) {
            double phi = (double)pj * s->dph;
            for (const auto &f : s->fronts) {
                if (f.contains(theta, phi)) {
                    if (s->precision == 0) {
                        double cur = s->h[ti * np + pj];
                        s->h[ti * np + pj] = cur * (1.0 - rr * dt);
                    } else if (s->precision == 1) {
                        s->hf[ti * np + pj] = s->hf[ti * np + pj] * factor32;
                    } else {
                        // double-float product (hi + lo) * (factor + factor_lo)
                        const float vh = s->hf[ti * np + pj], vl = s->lf[ti * np + pj];
                        const float p = vh * factor32;
                        const float pe = std::fma(vh, factor32, -p);
                        const float q = std::fma(vh, factor32_lo, std::fma(vl, factor32, pe));
                        const float sm = p + q;
                        s->lf[ti * np + pj] = q - (sm - p);
                        s->hf[ti * np + pj] = sm;
                    }
                    break;
                }
            }
        }
    }
}

// ------------------------------------------------------------------
// Film volume: V = sum_{i,j} h_ij R^2 sin(theta_i) dtheta dphi, summed row by row in f64
// ------------------------------------------------------------------
template <typename T>
double volume_impl(const T *h, uint32_t nt, uint32_t np, double radius) {
    double dth = kPi / (double)(nt - 1), dph = 2.0 * kPi / (double)np;
    double total = 0.0;
    for (uint32_t i = 0; i < nt; ++i) {
        double w = radius * radius * std::sin((double)i * dth) * dth * dph;
        double row = 0.0;
        for (uint32_t j = 0; j < np; ++j) row += (double)h[(size_t)i * np + j];
        total += row * w;
    }
    return total;
}

}  // namespace

extern "C" {

orc_sim *orc_sim_new(const orc_sim_params *p, int precision, int threads) {
    if (!p || p->resolution < 3) return nullptr;
    orc_sim *s = new orc_sim();
    s->nt = p->resolution;
    s->np = p->resolution * 2;
    s->precision = precision;
    s->threads = threads;
    init_geometry(s);
    double h0 = p->film_thickness_nm * 1e-9;
    size_t n = (size_t)s->nt * s->np;
    if (precision == 0) {
        s->h.assign(n, h0);
        s->scratch = s->h;
    } else {
        s->hf.assign(n, (float)h0);
        s->scratchf = s->hf;
        s->lf.assign(n, precision == 2 ? (float)(h0 - (double)(float)h0) : 0.f);
        s->scratchl = s->lf;
    }
    s->density = p->density;
    s->gravity = p->gravity;
    s->viscosity = p->viscosity;
    s->diffusion = p->surfactant_diffusion;
    s->critical = p->critical_thickness_nm * 1e-9;
    s->radius = p->diameter / 2.0;
    s->current_time = 0.0;
    s->tfe_ratio = 0.85;
    s->mr_enabled = true;
    s->next_spawn = 0.5;
    s->spawn_interval = 2.0;
    init_rows_f32(s);
    return s;
}

void orc_sim_free(orc_sim *s) { delete s; }
uint32_t orc_sim_num_theta(const orc_sim *s) { return s->nt; }
uint32_t orc_sim_num_phi(const orc_sim *s) { return s->np; }

void orc_sim_set_field(orc_sim *s, const double *h) {
    size_t n = (size_t)s->nt * s->np;
    if (s->precision == 0) {
        std::memcpy(s->h.data(), h, n * sizeof(double));
    } else {
        for (size_t i = 0; i < n; ++i) {
            s->hf[i] = (float)h[i];
            s->lf[i] = s->precision == 2 ? (float)(h[i] - (double)s->hf[i]) : 0.f;
        }
    }
}

void orc_sim_get_field(const orc_sim *s, double *h) {
    size_t n = (size_t)s->nt * s->np;
    if (s->precision == 0)
        std::memcpy(h, s->h.data(), n * sizeof(double));
    else
        for (size_t i = 0; i < n; ++i) h[i] = (double)s->hf[i] + (double)s->lf[i];
}

// DrainageSimulator::step (drainage.rs:298-392)
void orc_sim_step(orc_sim *s, double dt) {
    if (s->precision == 0)
        stencil_f64(s, dt);
    else
        stencil_f32k(s, dt);
    update_poles(s);
    if (s->mr_enabled) update_mr(s, dt);
    s->current_time += dt;
}

void orc_sim_step_n(orc_sim *s, double dt, uint32_t n) {
    for (uint32_t i = 0; i < n; ++i) orc_sim_step(s, dt);
}

// get_thickness (drainage.rs:516-552)
double orc_sim_get_thickness(const orc_sim *s, double theta, double phi) {
    const uint32_t nt = s->nt, np = s->np;
    double theta_clamped = std::min(std::max(theta, 0.0), kPi);
    double two_pi = 2.0 * kPi;
    double r = std::fmod(phi, two_pi);  // f64::rem_euclid
    double phi_normalized = r < 0.0 ? r + std::fabs(two_pi) : r;
    double tc = theta_clamped / s->dth;
    double pc = phi_normalized / s->dph;
    double tfl = std::floor(tc), pfl = std::floor(pc);
    size_t til = tfl <= 0.0 ? 0 : (size_t)tfl;
    til = std::min(til, (size_t)nt - 2);
    size_t pil = (pfl <= 0.0 ? 0 : (size_t)pfl) % np;
    size_t tih = til + 1;
    size_t pih = (pil + 1) % np;
    double tf = tc - (double)til;
    double pf = pc - (double)pil;
    auto get = [&](size_t i, size_t j) {
        return s->precision == 0 ? s->h[i * np + j] : (double)s->hf[i * np + j] + (double)s->lf[i * np + j];
    };
    double v00 = get(til, pil), v01 = get(til, pih), v10 = get(tih, pil), v11 = get(tih, pih);
    double v0 = v00 * (1.0 - pf) + v01 * pf;
    double v1 = v10 * (1.0 - pf) + v11 * pf;
    return v0 * (1.0 - tf) + v1 * tf;
}

double orc_sim_current_time(const orc_sim *s) { return s->current_time; }

// The kernels' exact ring mean of n f32 words (kernel-order pole means) over a ring of np cells.
double orc_fix_ring_mean(const float *words, size_t n, uint32_t np) {
    Wide tot;
    bool ok = true;
    for (size_t j = 0; j < n; ++j)
        if (!fix_word(words[j], tot)) ok = false;
    return ok ? fix_total_to_double(tot) / (double)np : std::nan("");
}

double orc_sim_min_thickness(const orc_sim *s) {
    double m = INFINITY;
    if (s->precision == 0)
        for (double v : s->h) m = std::fmin(m, v);
    else
        for (size_t i = 0; i < s->hf.size(); ++i) m = std::fmin(m, (double)s->hf[i] + (double)s->lf[i]);
    return m;
}

double orc_sim_max_thickness(const orc_sim *s) {
    double m = -INFINITY;
    if (s->precision == 0)
        for (double v : s->h) m = std::fmax(m, v);
    else
        for (size_t i = 0; i < s->hf.size(); ++i) m = std::fmax(m, (double)s->hf[i] + (double)s->lf[i]);
    return m;
}

int orc_sim_has_critical_region(const orc_sim *s) { return orc_sim_min_thickness(s) < s->critical; }

// reset (drainage.rs:575-583)
void orc_sim_reset(orc_sim *s, double h0) {
    if (s->precision == 0) {
        std::fill(s->h.begin(), s->h.end(), h0);
    } else {
        std::fill(s->hf.begin(), s->hf.end(), (float)h0);
        std::fill(s->lf.begin(), s->lf.end(), s->precision == 2 ? (float)(h0 - (double)(float)h0) : 0.f);
    }
    s->current_time = 0.0;
    s->fronts.clear();
    s->next_spawn = 0.5;
}

void orc_sim_set_marginal_regeneration(orc_sim *s, int enabled) {  // :588-593
    s->mr_enabled = enabled != 0;
    if (!enabled) s->fronts.clear();
}

void orc_sim_set_tfe_thickness_ratio(orc_sim *s, double ratio) {  // :601-603
    s->tfe_ratio = std::min(std::max(ratio, 0.5), 0.95);
}

double orc_sim_tfe_thickness_ratio(const orc_sim *s) { return s->tfe_ratio; }
uint32_t orc_sim_active_tfe_count(const orc_sim *s) { return (uint32_t)s->fronts.size(); }

uint32_t orc_sim_get_fronts(const orc_sim *s, double *out, uint32_t cap) {
    uint32_t n = 0;
    for (const auto &f : s->fronts) {
        if (n >= cap) break;
        out[4 * n + 0] = f.phi_center;
        out[4 * n + 1] = f.extent;
        out[4 * n + 2] = f.width;
        out[4 * n + 3] = f.velocity;
        ++n;
    }
    return n;
}

// ------------------------------------------------------------------
// WGSL drainage_step (drainage.wgsl:72-202)
// ------------------------------------------------------------------
static void wgsl_pass(const orc_wgsl_params *p, int mode, const float *hin, const float *cin, float *hout,
                      float *cout, int threads) {
    const uint32_t W = p->grid_width, H = p->grid_height;
    const float PI = 3.14159265358979323846f;
    // kernel-order row coefficients (computed in f64 from the f32 angle, rounded once)
    std::vector<float> rA(H), rE(H), rF(H), rG(H);
    const float dth32 = PI / (float)(H - 1u);
    const float dph32 = 2.0f * PI / (float)W;
    const double dth = (double)dth32, dph = (double)dph32, R = (double)p->bubble_radius;
    const double coef = (double)p->density * (double)p->gravity / (3.0 * (double)p->viscosity);
    for (uint32_t i = 0; i < H; ++i) {
        float th32 = (float)i * dth32;
        double sn = std::sin((double)th32), cs = std::cos((double)th32);
        double ss = std::fabs(sn) < 1e-4 ? (sn > 0 ? 1e-4 : (sn < 0 ? -1e-4 : 0.0)) : sn;
        rA[i] = (float)(-coef * sn);
        rE[i] = (float)((cs / ss) / (2.0 * dth));
        rF[i] = (float)((1.0 / (ss * ss)) / (dph * dph));
        rG[i] = (float)(1.0 / (2.0 * dph * R * ss));
    }
    const float kb = (float)(1.0 / (dth * dth));
    const float kDR2 = (float)((double)p->diffusion_coeff / (R * R));
    const float kDsR2 = (float)((double)p->surfactant_diffusion / (R * R));
    const float kGt = (float)(1.0 / (2.0 * dth * R));
    const float kM = (float)((double)p->marangoni_coeff * (double)p->gamma_reduction);

#pragma omp parallel for schedule(static) num_threads(threads > 0 ? threads : omp_get_max_threads())
    for (int64_t ti = 0; ti < (int64_t)H; ++ti) {
        for (uint32_t pj = 0; pj < W; ++pj) {
            size_t idx = (size_t)ti * W + pj;
            if (ti == 0 || ti == (int64_t)H - 1) {  // :85-89
                hout[idx] = hin[idx];
                cout[idx] = cin[idx];
                continue;
            }
            float h = hin[idx], conc = cin[idx];
            if (h < p->critical_thickness) {  // :108-112
                hout[idx] = h;
                cout[idx] = conc;
                continue;
            }
            auto at = [&](const float *a, int64_t t, int64_t f) {  // :47-64
                int64_t tt = std::min(std::max(t, (int64_t)0), (int64_t)H - 1);
                int64_t pf = f % (int64_t)W;
                if (pf < 0) pf += W;
                return a[(size_t)tt * W + pf];
            };
            float htm = at(hin, ti - 1, pj), htp = at(hin, ti + 1, pj);
            float hpm = at(hin, ti, (int64_t)pj - 1), hpp = at(hin, ti, (int64_t)pj + 1);
            float ctm = at(cin, ti - 1, pj), ctp = at(cin, ti + 1, pj);
            float cpm = at(cin, ti, (int64_t)pj - 1), cpp = at(cin, ti, (int64_t)pj + 1);
            if (mode == 0) {
                // drainage.wgsl operation order, IEEE f32
                float delta_theta = PI / (float)(H - 1u);
                float delta_phi = 2.0f * PI / (float)W;
                float theta = (float)ti * delta_theta;
                float sin_theta = std::sin(theta);
                float cos_theta = std::cos(theta);
                float sgn = sin_theta > 0.f ? 1.f : (sin_theta < 0.f ? -1.f : 0.f);
                float sts = std::fabs(sin_theta) < 0.0001f ? sgn * 0.0001f : sin_theta;
                float drainage_coeff = p->density * p->gravity / (3.0f * p->viscosity);
                float h_cubed = h * h * h;
                float drainage_term = -drainage_coeff * h_cubed * sin_theta;
                float r2 = p->bubble_radius * p->bubble_radius;
                float d2t = (htp - 2.0f * h + htm) / (delta_theta * delta_theta);
                float d1t = (htp - htm) / (2.0f * delta_theta);
                float d2p = (hpp - 2.0f * h + hpm) / (delta_phi * delta_phi);
                float hlap = (d2t + cos_theta / sts * d1t + d2p / (sts * sts)) / r2;
                float diffusion_term = p->diffusion_coeff * hlap;
                float mterm = 0.0f;
                if (p->marangoni_enabled != 0u) {
                    float dc_dtheta = (ctp - ctm) / (2.0f * delta_theta);
                    float dc_dphi = (cpp - cpm) / (2.0f * delta_phi);
                    float gct = dc_dtheta / p->bubble_radius;
                    float gcp = dc_dphi / (p->bubble_radius * sts);
                    float mag = std::sqrt(gct * gct + gcp * gcp);
                    float stress = p->gamma_reduction * mag;
                    mterm = p->marangoni_coeff * stress * h * h;
                }
                float dh_dt = drainage_term + diffusion_term + mterm;
                float nh = h + p->dt * dh_dt;
                hout[idx] = nh > 0.0f ? nh : 0.0f;
                float d2c = (ctp - 2.0f * conc + ctm) / (delta_theta * delta_theta);
                float d1c = (ctp - ctm) / (2.0f * delta_theta);
                float d2cp = (cpp - 2.0f * conc + cpm) / (delta_phi * delta_phi);
                float clap = (d2c + cos_theta / sts * d1c + d2cp / (sts * sts)) / r2;
                float dc_dt = p->surfactant_diffusion * clap;
                if (p->marangoni_enabled != 0u) {
                    float coupling = 0.001f * (hlap * p->bubble_radius * p->bubble_radius);
                    dc_dt += coupling * conc;
                }
                float nc = conc + p->dt * dc_dt;
                cout[idx] = std::min(std::max(nc, 0.0f), 1.0f);
            } else {
                // CUDA kernel order
                float A = rA[ti], E = rE[ti], F = rF[ti];
                float h3 = (h * h) * h;
                float lt = (htp - h) + (htm - h);
                float d1 = htp - htm;
                float lp = (hpp - h) + (hpm - h);
                float L = std::fma(F, lp, std::fma(E, d1, kb * lt));
                float inc = std::fma(kDR2, L, A * h3);
                if (p->marangoni_enabled != 0u) {
                    float gt = kGt * (ctp - ctm);
                    float gp = rG[ti] * (cpp - cpm);
                    float mag = std::sqrt(std::fma(gt, gt, gp * gp));
                    inc = inc + (kM * mag) * (h * h);
                }
                float v = std::fma(p->dt, inc, h);
                hout[idx] = v > 0.f ? v : 0.f;
                float lc = (ctp - conc) + (ctm - conc);
                float d1c = ctp - ctm;
                float lpc = (cpp - conc) + (cpm - conc);
                float Lc = std::fma(F, lpc, std::fma(E, d1c, kb * lc));
                float dc = kDsR2 * Lc;
                if (p->marangoni_enabled != 0u) dc = std::fma(0.001f * L, conc, dc);
                float c = std::fma(p->dt, dc, conc);
                c = c > 0.f ? c : 0.f;
                cout[idx] = c < 1.f ? c : 1.f;
            }
        }
    }
}

void orc_wgsl_run(const orc_wgsl_params *p, int mode, const float *h_in, const float *c_in, float *h_out,
                  float *c_out, uint32_t passes, int threads) {
    size_t n = (size_t)p->grid_width * p->grid_height;
    std::vector<float> ha(h_in, h_in + n), ca(c_in, c_in + n), hb(n), cb(n);
    for (uint32_t k = 0; k < passes; ++k) {
        wgsl_pass(p, mode, ha.data(), ca.data(), hb.data(), cb.data(), threads);
        ha.swap(hb);
        ca.swap(cb);
    }
    std::memcpy(h_out, ha.data(), n * sizeof(float));
    std::memcpy(c_out, ca.data(), n * sizeof(float));
}

double orc_film_volume_f64(const double *h, uint32_t nt, uint32_t np, double radius) {
    return volume_impl(h, nt, np, radius);
}
double orc_film_volume_f32(const float *h, uint32_t nt, uint32_t np, double radius) {
    return volume_impl(h, nt, np, radius);
}

}  // extern "C"
