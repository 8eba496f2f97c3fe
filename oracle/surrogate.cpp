// CPU restatement of the drainage surrogate (include/sbs_nn.h): features, forward pass, masked
// MSE loss and its gradient. TEST INFRASTRUCTURE (see oracle.h): it checks the CUDA training and
// inference kernels and is never linked into the product.
//
// Arithmetic: every convolution sums in double over operands rounded to BF16 exactly where the
// CUDA path rounds them (features, weights, activations, per-layer output gradients); values the
// CUDA path keeps in FP32 (pre-activations, the layer-4 gradient, input gradients before the
// activation derivative) are rounded to float here too. The remaining difference to the GPU is the order of
// FP32 accumulation inside the tensor-core sums.
//
// The surrogate has no counterpart in the reference; what it approximates is the WGSL drainage
// step (drainage.wgsl:72-202), run SBS_NN_STEPS times.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../include/sbs_nn.h"
#include "oracle.h"

namespace {

float bf16r(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    if ((u & 0x7f800000u) == 0x7f800000u) {
        if (u & 0x007fffffu) u = 0x7fc00000u;  // NaN -> canonical quiet NaN
    } else {
        u += 0x7fffu + ((u >> 16) & 1u);  // round to nearest even
    }
    u &= 0xffff0000u;
    float r;
    std::memcpy(&r, &u, 4);
    return r;
}

// exact mode (orc_nn_set_exact): no BF16 / float rounding anywhere, for finite-difference checks
// of the backward pass against the forward pass.
int g_exact = 0;

inline double rb(double v) { return g_exact ? v : (double)bf16r((float)v); }
inline double rf(double v) { return g_exact ? v : (double)(float)v; }

// activations of include/sbs_nn.h in double (exact mode)
double gelu_d(double x) {
    const double t = std::fmin(std::fmax(x, -3.0), 3.0), u = t * t;
    const double p = (((SBS_NN_Q4 * u + SBS_NN_Q3) * u + SBS_NN_Q2) * u + SBS_NN_Q1) * u + SBS_NN_Q0;
    return x * (0.5 + t * p);
}

double gelu_grad_d(double x) {
    const double t = std::fmin(std::fmax(x, -3.0), 3.0), u = t * t;
    const double p = (((SBS_NN_Q4 * u + SBS_NN_Q3) * u + SBS_NN_Q2) * u + SBS_NN_Q1) * u + SBS_NN_Q0;
    const double dp = ((4.0 * (double)SBS_NN_Q4 * u + 3.0 * (double)SBS_NN_Q3) * u + 2.0 * (double)SBS_NN_Q2) * u +
                      (double)SBS_NN_Q1;
    const double dphi = std::fabs(x) < 3.0 ? p + 2.0 * u * dp : 0.0;
    return (0.5 + t * p) + x * dphi;
}

double hswish_d(double x) {
    const double s = std::fmin(std::fmax(x * (double)SBS_NN_HS_SLOPE + 0.5, 0.0), 1.0);
    return x * s;
}

double hswish_grad_d(double x) {
    const double r = x * (double)SBS_NN_HS_SLOPE + 0.5;
    return r <= 0.0 ? 0.0 : (r >= 1.0 ? 1.0 : r + x * (double)SBS_NN_HS_SLOPE);
}

double act_d(int act, double x) { return act == SBS_NN_ACT_HSWISH ? hswish_d(x) : gelu_d(x); }
double act_grad_d(int act, double x) { return act == SBS_NN_ACT_HSWISH ? hswish_grad_d(x) : gelu_grad_d(x); }

struct Grid {
    std::vector<float> cp, cg, sg;
    std::vector<float> lip;  // log10(1 / (dph^2 se^2))
    std::vector<char> mask;
    float ct = 0.f;
    float lith = 0.f;  // log10(1 / dth^2)
};

Grid make_grid(uint32_t nt, uint32_t np) {
    Grid g;
    const double dth = M_PI / (double)(nt - 1), dph = 2.0 * M_PI / (double)np, S2 = SBS_NN_S2;
    g.ct = (float)(1.0 / (dth * dth * S2));
    g.lith = (float)std::log10(1.0 / (dth * dth));
    g.cp.resize(nt);
    g.cg.resize(nt);
    g.sg.resize(nt);
    g.lip.resize(nt);
    g.mask.resize(nt);
    for (uint32_t i = 0; i < nt; ++i) {
        const double sn = std::sin((double)i * dth), cs = std::cos((double)i * dth);
        const double se = std::max(sn, SBS_NN_SIN_FLOOR);
        g.cp[i] = (float)(1.0 / (dph * dph * se * se * S2));
        g.cg[i] = (float)(cs / (se * 2.0 * dth * S2));
        g.sg[i] = (float)sn;
        g.lip[i] = (float)std::log10(1.0 / (dph * dph * se * se));
        g.mask[i] = (i > 0 && i + 1 < nt && sn >= SBS_NN_MASK_SIN) ? 1 : 0;
    }
    return g;
}

struct FieldConsts {
    float gk, f5, f6, kout, lm;
};

FieldConsts field_consts(const orc_wgsl_params *p) {
    const double R = (double)p->bubble_radius, S2 = SBS_NN_S2;
    const double dr2 = (double)p->diffusion_coeff / (R * R);
    const double coef = (double)p->density * (double)p->gravity / (3.0 * (double)p->viscosity);
    FieldConsts f;
    f.gk = (float)(-coef / (dr2 * S2));
    f.f5 = (float)std::log10((double)p->viscosity / 1e-3);
    f.f6 = (float)(3.0 * std::log10(2.0 * R / 0.035));
    const double mu = (double)SBS_NN_STEPS * (double)p->dt * dr2;
    f.kout = (float)(mu * S2);
    f.lm = (float)std::log10(mu / SBS_NN_MU_REF);
    return f;
}

inline float clampf(float v) { return std::fmin(std::fmax(v, -SBS_NN_FEATURE_CLAMP), SBS_NN_FEATURE_CLAMP); }

inline uint32_t refl(int64_t i, uint32_t nt) {
    if (i < 0) return 1;
    if (i >= (int64_t)nt) return nt - 2;
    return (uint32_t)i;
}

// the activations and their derivatives in the FP32 operation order of include/sbs_nn.h
float gelu_f(float x) {
    const float t = std::fmin(std::fmax(x, -3.f), 3.f);
    const float u = t * t;
    const float p = std::fma(std::fma(std::fma(std::fma(SBS_NN_Q4, u, SBS_NN_Q3), u, SBS_NN_Q2), u, SBS_NN_Q1),
                             u, SBS_NN_Q0);
    const float phi = std::fma(t, p, 0.5f);
    return x * phi;
}

float gelu_grad_f(float x) {
    const float t = std::fmin(std::fmax(x, -3.f), 3.f);
    const float u = t * t;
    const float p = std::fma(std::fma(std::fma(std::fma(SBS_NN_Q4, u, SBS_NN_Q3), u, SBS_NN_Q2), u, SBS_NN_Q1),
                             u, SBS_NN_Q0);
    const float phi = std::fma(t, p, 0.5f);
    const float dp = std::fma(std::fma(std::fma(SBS_NN_Q4X4, u, SBS_NN_Q3X3), u, SBS_NN_Q2X2), u, SBS_NN_Q1);
    const float dphi = std::fabs(x) < 3.f ? std::fma(u + u, dp, p) : 0.f;
    return std::fma(x, dphi, phi);
}

// sat() of include/sbs_nn.h: clamp to [0, 1], NaN -> 0
inline float sat01(float r) { return r > 0.f ? (r < 1.f ? r : 1.f) : 0.f; }

float hswish_f(float x) { return x * sat01(std::fma(x, SBS_NN_HS_SLOPE, 0.5f)); }

float hswish_grad_f(float x) {
    const float r = std::fma(x, SBS_NN_HS_SLOPE, 0.5f), s = sat01(r);
    return (r > 0.f && r < 1.f) ? std::fma(x, SBS_NN_HS_SLOPE, s) : s;
}

float act_f(int act, float x) { return act == SBS_NN_ACT_HSWISH ? hswish_f(x) : gelu_f(x); }
float act_grad_f(int act, float x) { return act == SBS_NN_ACT_HSWISH ? hswish_grad_f(x) : gelu_grad_f(x); }

struct Layer {
    int ci, co;
    std::vector<double> w, b;  // w[tap][co][ci], BF16-rounded
};

std::vector<Layer> layers_from(const float *params) {
    const int off_w[4] = {SBS_NN_W1, SBS_NN_W2, SBS_NN_W3, SBS_NN_W4};
    const int off_b[4] = {SBS_NN_B1, SBS_NN_B2, SBS_NN_B3, SBS_NN_B4};
    const int ci[4] = {SBS_NN_NF, SBS_NN_C, SBS_NN_C, SBS_NN_C};
    const int co[4] = {SBS_NN_C, SBS_NN_C, SBS_NN_C, 1};
    std::vector<Layer> L(4);
    for (int l = 0; l < 4; ++l) {
        L[l].ci = ci[l];
        L[l].co = co[l];
        L[l].w.resize((size_t)9 * co[l] * ci[l]);
        L[l].b.resize(co[l]);
        for (size_t k = 0; k < L[l].w.size(); ++k) L[l].w[k] = rb((double)params[off_w[l] + k]);
        for (int k = 0; k < co[l]; ++k) L[l].b[k] = (double)params[off_b[l] + k];
    }
    return L;
}

// y[cell][co] = b + sum_{tap, ci} w * x[src(cell, tap)][ci], rounded to float.
void conv_fwd(const Layer &L, const double *x, uint32_t nb, uint32_t nt, uint32_t np, std::vector<double> &y) {
    const size_t cells = (size_t)nb * nt * np;
    y.assign(cells * L.co, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < (int64_t)cells; ++c) {
        const uint32_t j = (uint32_t)(c % np), i = (uint32_t)((c / np) % nt), n = (uint32_t)(c / ((size_t)np * nt));
        std::vector<double> acc(L.b.begin(), L.b.end());
        for (int t = 0; t < 9; ++t) {
            const int dy = t / 3 - 1, dx = t % 3 - 1;
            const uint32_t r = refl((int64_t)i + dy, nt), q = (uint32_t)(((int64_t)j + dx + np) % np);
            const double *xs = x + (((size_t)n * nt + r) * np + q) * L.ci;
            const double *w = L.w.data() + (size_t)t * L.co * L.ci;
            for (int o = 0; o < L.co; ++o) {
                double s = 0.0;
                for (int k = 0; k < L.ci; ++k) s += w[(size_t)o * L.ci + k] * xs[k];
                acc[o] += s;
            }
        }
        for (int o = 0; o < L.co; ++o) y[(size_t)c * L.co + o] = rf(acc[o]);
    }
}

struct Fwd {
    std::vector<double> x, y[4], a[3];
};

void forward(const std::vector<Layer> &L, const float *x, uint32_t nb, uint32_t nt, uint32_t np, int act, Fwd &F) {
    F.x.assign(x, x + (size_t)nb * nt * np * SBS_NN_NF);
    const double *in = F.x.data();
    for (int l = 0; l < 4; ++l) {
        conv_fwd(L[l], in, nb, nt, np, F.y[l]);
        if (l < 3) {
            F.a[l].resize(F.y[l].size());
            for (size_t k = 0; k < F.y[l].size(); ++k)
                F.a[l][k] = g_exact ? act_d(act, F.y[l][k]) : (double)bf16r(act_f(act, (float)F.y[l][k]));
            in = F.a[l].data();
        }
    }
}

// Gradients of one layer given g (dL/dy, [cell][co]) and its input x ([cell][ci]):
// dW[tap][co][ci] += sum_cell g[cell][co] * x[src(cell,tap)][ci]; db[co] += sum g;
// dx[src(cell,tap)][ci] += sum_co g[cell][co] * w[tap][co][ci] (if dx != null).
void conv_bwd(const Layer &L, const std::vector<double> &g, const double *x, uint32_t nb, uint32_t nt, uint32_t np,
              std::vector<double> &dW, std::vector<double> &db, std::vector<double> *dx) {
    const size_t cells = (size_t)nb * nt * np;
    dW.assign((size_t)9 * L.co * L.ci, 0.0);
    db.assign(L.co, 0.0);
    for (size_t c = 0; c < cells; ++c)
        for (int o = 0; o < L.co; ++o) db[o] += g[c * L.co + o];
#pragma omp parallel for schedule(static)
    for (int t = 0; t < 9; ++t) {
        const int dy = t / 3 - 1, dx_ = t % 3 - 1;
        for (size_t c = 0; c < cells; ++c) {
            const uint32_t j = (uint32_t)(c % np), i = (uint32_t)((c / np) % nt), n = (uint32_t)(c / ((size_t)np * nt));
            const uint32_t r = refl((int64_t)i + dy, nt), q = (uint32_t)(((int64_t)j + dx_ + np) % np);
            const double *xs = x + (((size_t)n * nt + r) * np + q) * L.ci;
            for (int o = 0; o < L.co; ++o) {
                const double go = g[c * L.co + o];
                if (go == 0.0) continue;
                double *d = dW.data() + ((size_t)t * L.co + o) * L.ci;
                for (int k = 0; k < L.ci; ++k) d[k] += go * xs[k];
            }
        }
    }
    if (!dx) return;
    dx->assign(cells * L.ci, 0.0);
    // scatter in a fixed order (sequential: reflected rows receive from two sources)
    for (size_t c = 0; c < cells; ++c) {
        const uint32_t j = (uint32_t)(c % np), i = (uint32_t)((c / np) % nt), n = (uint32_t)(c / ((size_t)np * nt));
        for (int t = 0; t < 9; ++t) {
            const int dy = t / 3 - 1, dx_ = t % 3 - 1;
            const uint32_t r = refl((int64_t)i + dy, nt), q = (uint32_t)(((int64_t)j + dx_ + np) % np);
            double *d = dx->data() + (((size_t)n * nt + r) * np + q) * L.ci;
            const double *w = L.w.data() + (size_t)t * L.co * L.ci;
            for (int o = 0; o < L.co; ++o) {
                const double go = g[c * L.co + o];
                if (go == 0.0) continue;
                for (int k = 0; k < L.ci; ++k) d[k] += go * w[(size_t)o * L.ci + k];
            }
        }
    }
}

}  // namespace

extern "C" {

void orc_nn_set_exact(int exact) { g_exact = exact ? 1 : 0; }

float orc_nn_gelu(float x) { return gelu_f(x); }
float orc_nn_gelu_grad(float x) { return gelu_grad_f(x); }
float orc_nn_hswish(float x) { return hswish_f(x); }
float orc_nn_hswish_grad(float x) { return hswish_grad_f(x); }

float orc_nn_kout(const orc_wgsl_params *p) { return field_consts(p).kout; }

void orc_nn_features(const float *h, const float *c, const orc_wgsl_params *p, float *x) {
    const uint32_t nt = p->grid_height, np = p->grid_width;
    const Grid g = make_grid(nt, np);
    const FieldConsts f = field_consts(p);
    const float lt = f.lm + g.lith;
    for (uint32_t i = 0; i < nt; ++i) {
        const float *rn = h + (size_t)refl((int64_t)i - 1, nt) * np, *rs = h + (size_t)refl((int64_t)i + 1, nt) * np;
        const float *rc = h + (size_t)i * np;
        const float grav = f.gk * g.sg[i];
        const float lp = f.lm + g.lip[i];
        for (uint32_t j = 0; j < np; ++j) {
            const float hc = rc[j], hn = rn[j], hs = rs[j], hw = rc[(j + np - 1) % np], he = rc[(j + 1) % np];
            float v[SBS_NN_NF] = {};
            v[0] = (hc - SBS_NN_H0) * SBS_NN_INV_HS;
            v[1] = ((hn + hs) - (hc + hc)) * g.ct;
            v[2] = ((hw + he) - (hc + hc)) * g.cp[i];
            v[3] = (hs - hn) * g.cg[i];
            v[4] = (c[(size_t)i * np + j] - 0.5f) * 10.f;
            v[5] = f.f5;
            v[6] = f.f6;
            v[7] = ((hc * hc) * hc) * grav;
            v[8] = lt;
            v[9] = lp;
            v[10] = g.sg[i];
            float *o = x + ((size_t)i * np + j) * SBS_NN_NF;
            for (int k = 0; k < SBS_NN_NF; ++k) o[k] = bf16r(clampf(v[k]));
        }
    }
}

void orc_nn_forward(const float *params, uint32_t nb, uint32_t nt, uint32_t np, const float *x, float *y, int act) {
    const std::vector<Layer> L = layers_from(params);
    Fwd F;
    forward(L, x, nb, nt, np, act, F);
    for (size_t k = 0; k < F.y[3].size(); ++k) y[k] = (float)F.y[3][k];
}

double orc_nn_loss_grad(const float *params, uint32_t nb, uint32_t nt, uint32_t np, const float *x,
                        const float *target, float *grad, int act) {
    const std::vector<Layer> L = layers_from(params);
    Fwd F;
    forward(L, x, nb, nt, np, act, F);
    const Grid g = make_grid(nt, np);
    const size_t cells = (size_t)nb * nt * np;
    size_t nmask = 0;
    for (uint32_t i = 0; i < nt; ++i) nmask += g.mask[i] ? (size_t)np * nb : 0;
    std::vector<double> gy(cells, 0.0);
    double loss = 0.0;
    for (size_t cidx = 0; cidx < cells; ++cidx) {
        const uint32_t i = (uint32_t)((cidx / np) % nt);
        if (!g.mask[i]) continue;
        const double d = (double)F.y[3][cidx] - (double)target[cidx];
        loss += d * d;
        gy[cidx] = rf(2.0 * d / (double)nmask);  // FP32 on the GPU
    }
    loss /= (double)nmask;
    const int off_w[4] = {SBS_NN_W1, SBS_NN_W2, SBS_NN_W3, SBS_NN_W4};
    const int off_b[4] = {SBS_NN_B1, SBS_NN_B2, SBS_NN_B3, SBS_NN_B4};
    std::vector<double> dW, db, dx;
    for (int l = 3; l >= 0; --l) {
        const double *xin = l == 0 ? F.x.data() : F.a[l - 1].data();
        conv_bwd(L[l], gy, xin, nb, nt, np, dW, db, l > 0 ? &dx : nullptr);
        for (size_t k = 0; k < dW.size(); ++k) grad[off_w[l] + k] = (float)dW[k];
        for (size_t k = 0; k < db.size(); ++k) grad[off_b[l] + k] = (float)db[k];
        if (l == 0) break;
        // g of the layer below: bf16( float(dx) * act'(y) )
        const std::vector<double> &yl = F.y[l - 1];
        gy.assign(dx.size(), 0.0);
        for (size_t k = 0; k < dx.size(); ++k)
            gy[k] = g_exact ? dx[k] * act_grad_d(act, yl[k]) : (double)bf16r((float)dx[k] * act_grad_f(act, (float)yl[k]));
    }
    return loss;
}

void orc_nn_apply(const float *h, const float *y, uint32_t nt, uint32_t np, float kout, float *h_out) {
    for (uint32_t i = 0; i < nt; ++i)
        for (uint32_t j = 0; j < np; ++j) {
            const size_t k = (size_t)i * np + j;
            if (i == 0 || i + 1 == nt) {
                h_out[k] = h[k];
            } else {
                const float t = kout * y[k];
                h_out[k] = std::fmax(h[k] + t, 0.f);
            }
        }
}

}  // extern "C"
