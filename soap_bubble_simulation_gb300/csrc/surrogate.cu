// Drainage surrogate (include/sbs_nn.h): handle, training data from the plain WGSL solver,
// Adam training with the layered tensor-core kernels, evaluation, and the surrogate-accelerated
// rollout in which the plain solver checks every K-th interval and takes over on a miss.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <utility>
#include <vector>

#include "nn.cuh"
#include "nn_kernels.h"
#include "sbs_internal.h"

using namespace sbs;
using namespace sbs::nn;

namespace sbs {
namespace nn {
// fused tcgen05 forward pass (nn_fused.cu)
int fused_forward(sbs_surrogate *s, const Fields &fs, int nf, const GridTab &g, float *hout, size_t pitch_out,
                  float *y_out);
int fused_pack(sbs_surrogate *s);
void fused_release(sbs_surrogate *s);
}  // namespace nn
}  // namespace sbs

namespace {

struct FieldC {
    float gk, f5, f6, kout, lm;
};

// include/sbs_nn.h field scalars, computed in double and rounded once.
FieldC field_consts(const sbs_drainage_params &p) {
    const double R = (double)p.bubble_radius, S2 = SBS_NN_S2;
    const double dr2 = (double)p.diffusion_coeff / (R * R);
    const double coef = (double)p.density * (double)p.gravity / (3.0 * (double)p.viscosity);
    FieldC f;
    f.gk = (float)(-coef / (dr2 * S2));
    f.f5 = (float)std::log10((double)p.viscosity / 1e-3);
    f.f6 = (float)(3.0 * std::log10(2.0 * R / 0.035));
    const double mu = (double)SBS_NN_STEPS * (double)p.dt * dr2;
    f.kout = (float)(mu * S2);
    f.lm = (float)std::log10(mu / SBS_NN_MU_REF);
    return f;
}

struct GridDev {
    float4 *rows = nullptr;
    float *lip = nullptr;
    float ct = 0.f, lith = 0.f;
    int nt = 0, np = 0;
    size_t mask_rows = 0;
    GridTab tab() const { return GridTab{rows, lip, ct, lith, nt, np}; }
};

struct Traj {
    float *h = nullptr;  // [pairs + 1][nt * np]
    float *c = nullptr;
    sbs_drainage_params p{};
    FieldC fc{};
    uint32_t pairs = 0;
};

uint64_t splitmix64(uint64_t &x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

double uniform01(uint64_t &x) { return ((splitmix64(x) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

double normal(uint64_t &x) {
    const double u1 = uniform01(x), u2 = uniform01(x);
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
}

}  // namespace

struct sbs_surrogate {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    float *theta = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr;
    Packed pk{};
    void *pk_mem = nullptr;
    int adam_step = 0;
    std::map<std::pair<int, int>, GridDev> grids;
    // workspace (cells = fields x nt x np)
    size_t cap = 0;
    void *ws = nullptr;
    bf16 *x0 = nullptr, *a1 = nullptr, *a2 = nullptr, *a3 = nullptr, *g1 = nullptr, *g2 = nullptr, *g3 = nullptr;
    float *y1 = nullptr, *y2 = nullptr, *y3 = nullptr, *y4 = nullptr, *g4 = nullptr, *tgt = nullptr;
    float *stage = nullptr;  // host inputs staged on the device: h | c | target
    size_t stage_cap = 0;
    float *partial = nullptr;
    int nblocks = 0;
    double *loss_part = nullptr;
    size_t loss_cap = 0;
    unsigned *err2 = nullptr;
    float *scratch = nullptr;  // rollout check output
    size_t scratch_cap = 0;
    // training data
    std::vector<Traj> data;
    int dnt = 0, dnp = 0;
    sbs_drainage *plain = nullptr;
    // fused-kernel state (nn_fused.cu)
    void *fused_w = nullptr;
    int fused_dirty = 1;
};

namespace sbs {
namespace nn {
// accessors for nn_fused.cu
cudaStream_t stream_of(sbs_surrogate *s) { return s->stream; }
const float *theta_of(sbs_surrogate *s) { return s->theta; }
void **fused_slot(sbs_surrogate *s) { return &s->fused_w; }
int *fused_dirty_flag(sbs_surrogate *s) { return &s->fused_dirty; }
int sms_of(sbs_surrogate *s) { return s->sms; }
int act_of(sbs_surrogate *s) { return s->pk.act; }
}  // namespace nn
}  // namespace sbs

namespace {

#define CHECK_S(s) SBS_CHECK_ARG((s) != nullptr, "surrogate handle is null")

int grid_of(sbs_surrogate *s, int nt, int np, const GridDev **out) {
    auto key = std::make_pair(nt, np);
    auto it = s->grids.find(key);
    if (it != s->grids.end()) {
        *out = &it->second;
        return SBS_OK;
    }
    GridDev g;
    g.nt = nt;
    g.np = np;
    const double dth = M_PI / (double)(nt - 1), dph = 2.0 * M_PI / (double)np, S2 = SBS_NN_S2;
    g.ct = (float)(1.0 / (dth * dth * S2));
    g.lith = (float)std::log10(1.0 / (dth * dth));
    std::vector<float4> rows(nt);
    std::vector<float> lip(nt);
    for (int i = 0; i < nt; ++i) {
        const double sn = std::sin((double)i * dth), cs = std::cos((double)i * dth);
        const double se = std::max(sn, SBS_NN_SIN_FLOOR);
        const bool mask = i > 0 && i + 1 < nt && sn >= SBS_NN_MASK_SIN;
        rows[i] = make_float4((float)(1.0 / (dph * dph * se * se * S2)), (float)(cs / (se * 2.0 * dth * S2)), (float)sn,
                              mask ? 1.f : 0.f);
        lip[i] = (float)std::log10(1.0 / (dph * dph * se * se));
        g.mask_rows += mask ? 1 : 0;
    }
    SBS_CUDA_TRY(cudaMalloc(&g.rows, sizeof(float4) * nt + sizeof(float) * nt));
    g.lip = reinterpret_cast<float *>(g.rows + nt);
    SBS_CUDA_TRY(cudaMemcpy(g.rows, rows.data(), sizeof(float4) * nt, cudaMemcpyHostToDevice));
    SBS_CUDA_TRY(cudaMemcpy(g.lip, lip.data(), sizeof(float) * nt, cudaMemcpyHostToDevice));
    auto res = s->grids.emplace(key, g);
    *out = &res.first->second;
    return SBS_OK;
}

int ensure_ws(sbs_surrogate *s, size_t cells) {
    if (cells <= s->cap) return SBS_OK;
    SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    cudaFree(s->ws);
    s->ws = nullptr;
    s->cap = 0;
    // bytes per cell: x0 32, a1..a3 3*64, g1..g3 3*64, y1..y3 3*128, y4 g4 tgt 12
    const size_t per = 32 + 6 * 64 + 3 * 128 + 12;
    char *p = nullptr;
    SBS_CUDA_TRY(cudaMalloc(&p, per * cells + 1024));
    s->ws = p;
    auto take = [&](size_t bytes) {
        char *r = p;
        p += (bytes + 255) / 256 * 256;
        return r;
    };
    s->x0 = (bf16 *)take(32 * cells);
    s->a1 = (bf16 *)take(64 * cells);
    s->a2 = (bf16 *)take(64 * cells);
    s->a3 = (bf16 *)take(64 * cells);
    s->g1 = (bf16 *)take(64 * cells);
    s->g2 = (bf16 *)take(64 * cells);
    s->g3 = (bf16 *)take(64 * cells);
    s->y1 = (float *)take(128 * cells);
    s->y2 = (float *)take(128 * cells);
    s->y3 = (float *)take(128 * cells);
    s->y4 = (float *)take(4 * cells);
    s->g4 = (float *)take(4 * cells);
    s->tgt = (float *)take(4 * cells);
    s->cap = cells;
    // one loss partial per 128-cell row segment of the output layer: rows have at least 3 cells,
    // so there are at most cells / 3 segments
    const size_t lp = cells / 3 + 1;
    if (lp > s->loss_cap) {
        cudaFree(s->loss_part);
        s->loss_part = nullptr;
        SBS_CUDA_TRY(cudaMalloc(&s->loss_part, sizeof(double) * lp));
        s->loss_cap = lp;
    }
    return SBS_OK;
}

int ensure_stage(sbs_surrogate *s, size_t floats) {
    if (floats <= s->stage_cap) return SBS_OK;
    SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    cudaFree(s->stage);
    s->stage = nullptr;
    SBS_CUDA_TRY(cudaMalloc(&s->stage, sizeof(float) * floats));
    s->stage_cap = floats;
    return SBS_OK;
}

// Fields of nf inputs (h, c in device memory, contiguous [nf][nt][np]).
Fields make_fields(const float *h, const float *c, size_t pitch, size_t field_stride, const sbs_drainage_params *p,
                   int nf) {
    Fields fs{};
    for (int b = 0; b < nf; ++b) {
        const FieldC fc = field_consts(p[b]);
        fs.f[b] = Field{h + field_stride * b, c + field_stride * b, pitch, fc.gk, fc.f5, fc.f6, fc.kout, fc.lm};
    }
    return fs;
}

// A timed-out wait of the tensor-core convolutions (herr: the error word, read after the stream
// drained) becomes SBS_E_TIMEOUT; the word is cleared for the next call.
int tc_result(sbs_surrogate *s, unsigned herr) {
    if (!herr) return SBS_OK;
    SBS_CUDA_TRY(cudaMemsetAsync(s->pk.err, 0, sizeof(unsigned), s->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return set_error(SBS_E_TIMEOUT, "surrogate: a tensor-core convolution wait timed out");
}

// Reads the error word after the work queued so far (synchronises the stream).
int tc_status(sbs_surrogate *s) {
    unsigned herr = 0;
    SBS_CUDA_TRY(cudaMemcpyAsync(&herr, s->pk.err, sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return tc_result(s, herr);
}

int layered_forward(sbs_surrogate *s, const Fields &fs, int nf, const GridDev &g) {
    const int nt = g.nt, np = g.np;
    SBS_CUDA_TRY(features(fs, nf, g.tab(), s->x0, s->stream));
    SBS_CUDA_TRY(conv_forward(1, s->x0, s->pk, s->y1, s->a1, nf, nt, np, s->stream));
    SBS_CUDA_TRY(conv_forward(2, s->a1, s->pk, s->y2, s->a2, nf, nt, np, s->stream));
    SBS_CUDA_TRY(conv_forward(3, s->a2, s->pk, s->y3, s->a3, nf, nt, np, s->stream));
    return SBS_OK;
}

// loss (masked MSE against s->tgt) and the full gradient into s->grad
int loss_and_grad(sbs_surrogate *s, const Fields &fs, int nf, const GridDev &g, double *loss) {
    const int nt = g.nt, np = g.np;
    int rc = layered_forward(s, fs, nf, g);
    if (rc) return rc;
    const double nmask = (double)g.mask_rows * np * nf;
    int nlb = 0;
    SBS_CUDA_TRY(output_layer(s->a3, s->pk, s->y4, s->tgt, s->g4, s->loss_part, (float)(2.0 / nmask), g.tab(), nf,
                              s->stream, &nlb));
    SBS_CUDA_TRY(output_backward(s->g4, s->a3, s->y3, s->pk, s->g3, s->partial, s->nblocks, s->grad, g.tab(), nf,
                                 s->stream));
    SBS_CUDA_TRY(conv_backward_weight(3, s->g3, s->a2, s->partial, s->nblocks, s->grad, s->pk.err, nf, nt, np,
                                      s->stream));
    SBS_CUDA_TRY(conv_backward_data(3, s->g3, s->pk, s->y2, s->g2, nf, nt, np, s->stream));
    SBS_CUDA_TRY(conv_backward_weight(2, s->g2, s->a1, s->partial, s->nblocks, s->grad, s->pk.err, nf, nt, np,
                                      s->stream));
    SBS_CUDA_TRY(conv_backward_data(2, s->g2, s->pk, s->y1, s->g1, nf, nt, np, s->stream));
    SBS_CUDA_TRY(conv_backward_weight(1, s->g1, s->x0, s->partial, s->nblocks, s->grad, s->pk.err, nf, nt, np,
                                      s->stream));
    if (loss) {
        std::vector<double> lp(nlb);
        unsigned herr = 0;
        SBS_CUDA_TRY(cudaMemcpyAsync(lp.data(), s->loss_part, sizeof(double) * nlb, cudaMemcpyDeviceToHost, s->stream));
        SBS_CUDA_TRY(cudaMemcpyAsync(&herr, s->pk.err, sizeof(unsigned), cudaMemcpyDeviceToHost, s->stream));
        SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
        if ((rc = tc_result(s, herr))) return rc;
        double sum = 0.0;
        for (double v : lp) sum += v;
        *loss = sum / nmask;
        return SBS_OK;
    }
    return tc_status(s);
}

int check_grid_params(uint32_t nf, const sbs_drainage_params *p) {
    SBS_CHECK_ARG(nf >= 1 && nf <= (uint32_t)kMaxFields, "nf must be 1..%d", kMaxFields);
    SBS_CHECK_ARG(p != nullptr, "params is null");
    for (uint32_t b = 0; b < nf; ++b) {
        SBS_CHECK_ARG(p[b].grid_height == p[0].grid_height && p[b].grid_width == p[0].grid_width,
                      "every field needs the same grid");
        SBS_CHECK_ARG(p[b].bubble_radius > 0.f && p[b].viscosity > 0.f && p[b].diffusion_coeff > 0.f &&
                          std::isfinite(p[b].dt) && p[b].dt > 0.f,
                      "field %u: radius, viscosity, diffusion and dt must be positive", b);
    }
    SBS_CHECK_ARG(p[0].grid_height >= 4 && p[0].grid_width >= 3, "grid needs >= 4 theta rows and >= 3 phi columns");
    return SBS_OK;
}

// h, c (nf fields, mem) -> device pointers (staged copies for host memory)
int stage_inputs(sbs_surrogate *s, uint32_t nf, size_t cells1, const float *h, const float *c, int mem,
                 const float **hd, const float **cd) {
    if (mem == SBS_MEM_DEVICE) {
        *hd = h;
        *cd = c;
        return SBS_OK;
    }
    int rc = ensure_stage(s, 3 * nf * cells1);
    if (rc) return rc;
    SBS_CUDA_TRY(cudaMemcpyAsync(s->stage, h, sizeof(float) * nf * cells1, cudaMemcpyHostToDevice, s->stream));
    SBS_CUDA_TRY(
        cudaMemcpyAsync(s->stage + nf * cells1, c, sizeof(float) * nf * cells1, cudaMemcpyHostToDevice, s->stream));
    *hd = s->stage;
    *cd = s->stage + nf * cells1;
    return SBS_OK;
}

int repack(sbs_surrogate *s) {
    SBS_CUDA_TRY(pack(s->theta, s->pk, s->stream));
    s->fused_dirty = 1;
    return SBS_OK;
}

// One forward pass of nf fields into s->y4 (layered) or straight into h_out (fused, if given).
int forward_any(sbs_surrogate *s, const Fields &fs, int nf, const GridDev &g, int mode, float *h_out,
                size_t pitch_out) {
    if (mode == SBS_NN_FUSED) return fused_forward(s, fs, nf, g.tab(), h_out, pitch_out, h_out ? nullptr : s->y4);
    SBS_CHECK_ARG(mode == SBS_NN_LAYERED, "mode must be SBS_NN_LAYERED or SBS_NN_FUSED");
    int rc = ensure_ws(s, (size_t)nf * g.nt * g.np);
    if (rc) return rc;
    rc = layered_forward(s, fs, nf, g);
    if (rc) return rc;
    SBS_CUDA_TRY(output_layer(s->a3, s->pk, s->y4, nullptr, nullptr, nullptr, 0.f, g.tab(), nf, s->stream, nullptr));
    if (h_out) {
        SBS_CUDA_TRY(apply(fs.f[0].h, fs.f[0].pitch, s->y4, fs.f[0].kout, g.nt, g.np, h_out, pitch_out, s->stream));
    }
    return SBS_OK;
}

}  // namespace

extern "C" {

int sbs_surrogate_create(uint64_t seed, sbs_surrogate **out) {
    clear_error();
    SBS_CHECK_ARG(out != nullptr, "out is null");
    *out = nullptr;
    int rc = require_device();
    if (rc) return rc;
    sbs_surrogate *s = new sbs_surrogate();
    auto fail = [&](int code) {
        sbs_surrogate_destroy(s);
        return code;
    };
    if (cudaGetDevice(&s->device) != cudaSuccess) return fail(set_error(SBS_E_CUDA, "cudaGetDevice failed"));
    cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
    s->nblocks = 2 * std::max(1, s->sms);
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&s->theta, sizeof(float) * SBS_NN_PARAMS * 4) != cudaSuccess)
        return fail(set_error(SBS_E_NOMEM, "surrogate allocation failed"));
    s->m = s->theta + SBS_NN_PARAMS;
    s->v = s->m + SBS_NN_PARAMS;
    s->grad = s->v + SBS_NN_PARAMS;
    // packed weights: wf1 32x144, wf2/wf3/wb2/wb3 32x288 (bf16), w4 288 + b 97 (f32)
    const size_t pkb = (size_t)2 * (32 * 144 + 4 * 32 * 288) + 4 * (288 + 97) + 256;
    const size_t partial_floats = (size_t)s->nblocks * (32 * 9 * 32 + 32);
    char *pm = nullptr;
    if (cudaMalloc(&pm, pkb + sizeof(float) * partial_floats + 64) != cudaSuccess)
        return fail(set_error(SBS_E_NOMEM, "surrogate allocation failed"));
    s->pk_mem = pm;
    s->pk.wf1 = (bf16 *)pm;
    s->pk.wf2 = s->pk.wf1 + 32 * 144;
    s->pk.wf3 = s->pk.wf2 + 32 * 288;
    s->pk.wb2 = s->pk.wf3 + 32 * 288;
    s->pk.wb3 = s->pk.wb2 + 32 * 288;
    s->pk.w4 = (float *)(s->pk.wb3 + 32 * 288);
    s->pk.b = s->pk.w4 + 288;
    s->partial = (float *)(pm + (pkb + 255) / 256 * 256);
    if (cudaMalloc(&s->err2, 16) != cudaSuccess || cudaMemset(s->err2, 0, 16) != cudaSuccess)
        return fail(set_error(SBS_E_NOMEM, "surrogate allocation failed"));
    s->pk.err = s->err2 + 2;  // words 0-1: masked_error's result
    // He-normal weights (fan-in 9 * ci), zero biases; the output layer starts small.
    std::vector<float> th(SBS_NN_PARAMS, 0.f);
    uint64_t st = seed;
    const int offw[4] = {SBS_NN_W1, SBS_NN_W2, SBS_NN_W3, SBS_NN_W4};
    const int ci[4] = {SBS_NN_NF, SBS_NN_C, SBS_NN_C, SBS_NN_C};
    const int co[4] = {SBS_NN_C, SBS_NN_C, SBS_NN_C, 1};
    for (int l = 0; l < 4; ++l) {
        const double sd = (l < 3 ? std::sqrt(2.0 / (9.0 * ci[l])) : 0.1 * std::sqrt(1.0 / (9.0 * ci[l])));
        for (int k = 0; k < 9 * ci[l] * co[l]; ++k) th[offw[l] + k] = (float)(sd * normal(st));
    }
    rc = sbs_surrogate_set_params(s, th.data(), th.size());
    if (rc) return fail(rc);
    *out = s;
    return SBS_OK;
}

int sbs_surrogate_destroy(sbs_surrogate *s) {
    clear_error();
    if (!s) return SBS_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    fused_release(s);
    if (s->plain) sbs_drainage_destroy(s->plain);
    for (auto &t : s->data) {
        cudaFree(t.h);
        cudaFree(t.c);
    }
    for (auto &kv : s->grids) cudaFree(kv.second.rows);
    cudaFree(s->theta);
    cudaFree(s->pk_mem);
    cudaFree(s->ws);
    cudaFree(s->stage);
    cudaFree(s->loss_part);
    cudaFree(s->err2);
    cudaFree(s->scratch);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return SBS_OK;
}

int sbs_surrogate_stream(const sbs_surrogate *s, void **out) {
    clear_error();
    CHECK_S(s);
    SBS_CHECK_ARG(out != nullptr, "out is null");
    *out = (void *)s->stream;
    return SBS_OK;
}

int sbs_surrogate_set_params(sbs_surrogate *s, const float *params, size_t n) {
    clear_error();
    CHECK_S(s);
    SBS_CHECK_ARG(params != nullptr && n == SBS_NN_PARAMS, "params must hold SBS_NN_PARAMS (%d) floats", SBS_NN_PARAMS);
    for (size_t k = 0; k < n; ++k) SBS_CHECK_ARG(std::isfinite(params[k]), "parameter %zu is not finite", k);
    SBS_CUDA_TRY(cudaMemcpyAsync(s->theta, params, sizeof(float) * n, cudaMemcpyHostToDevice, s->stream));
    SBS_CUDA_TRY(cudaMemsetAsync(s->m, 0, sizeof(float) * 2 * SBS_NN_PARAMS, s->stream));
    s->adam_step = 0;
    int rc = repack(s);
    if (rc) return rc;
    SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return SBS_OK;
}

int sbs_surrogate_set_activation(sbs_surrogate *s, int activation) {
    clear_error();
    CHECK_S(s);
    SBS_CHECK_ARG(activation == SBS_NN_ACT_GELU || activation == SBS_NN_ACT_HSWISH, "unknown activation %d",
                  activation);
    s->pk.act = activation;
    return SBS_OK;
}

int sbs_surrogate_get_activation(const sbs_surrogate *s, int *out) {
    clear_error();
    CHECK_S(s);
    SBS_CHECK_ARG(out != nullptr, "out is null");
    *out = s->pk.act;
    return SBS_OK;
}

int sbs_surrogate_get_params(sbs_surrogate *s, float *params, size_t n) {
    clear_error();
    CHECK_S(s);
    SBS_CHECK_ARG(params != nullptr && n == SBS_NN_PARAMS, "params must hold SBS_NN_PARAMS (%d) floats", SBS_NN_PARAMS);
    SBS_CUDA_TRY(cudaMemcpyAsync(params, s->theta, sizeof(float) * n, cudaMemcpyDeviceToHost, s->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return SBS_OK;
}

int sbs_surrogate_features(sbs_surrogate *s, uint32_t nf, const float *h, const float *c,
                           const sbs_drainage_params *p, float *x, int mem) {
    clear_error();
    CHECK_S(s);
    int rc = check_grid_params(nf, p);
    if (rc) return rc;
    SBS_CHECK_ARG(h && c && x, "null buffer");
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "mem must be SBS_MEM_HOST or SBS_MEM_DEVICE");
    const int nt = (int)p[0].grid_height, np = (int)p[0].grid_width;
    const size_t cells1 = (size_t)nt * np;
    const GridDev *g = nullptr;
    if ((rc = grid_of(s, nt, np, &g))) return rc;
    if ((rc = ensure_ws(s, nf * cells1))) return rc;
    const float *hd, *cd;
    if ((rc = stage_inputs(s, nf, cells1, h, c, mem, &hd, &cd))) return rc;
    SBS_CUDA_TRY(features(make_fields(hd, cd, np, cells1, p, nf), nf, g->tab(), s->x0, s->stream));
    // BF16 -> f32 on the host side of the copy
    std::vector<uint16_t> raw(nf * cells1 * SBS_NN_NF);
    SBS_CUDA_TRY(cudaMemcpyAsync(raw.data(), s->x0, raw.size() * 2, cudaMemcpyDeviceToHost, s->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    std::vector<float> xf(raw.size());
    for (size_t k = 0; k < raw.size(); ++k) {
        const uint32_t u = (uint32_t)raw[k] << 16;
        std::memcpy(&xf[k], &u, 4);
    }
    if (mem == SBS_MEM_HOST) {
        std::memcpy(x, xf.data(), xf.size() * 4);
    } else {
        SBS_CUDA_TRY(cudaMemcpy(x, xf.data(), xf.size() * 4, cudaMemcpyHostToDevice));
    }
    return SBS_OK;
}

int sbs_surrogate_forward(sbs_surrogate *s, uint32_t nf, const float *h, const float *c,
                          const sbs_drainage_params *p, float *y, int mode, int mem) {
    clear_error();
    CHECK_S(s);
    int rc = check_grid_params(nf, p);
    if (rc) return rc;
    SBS_CHECK_ARG(h && c && y, "null buffer");
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "mem must be SBS_MEM_HOST or SBS_MEM_DEVICE");
    const int nt = (int)p[0].grid_height, np = (int)p[0].grid_width;
    const size_t cells1 = (size_t)nt * np;
    const GridDev *g = nullptr;
    if ((rc = grid_of(s, nt, np, &g))) return rc;
    if ((rc = ensure_ws(s, nf * cells1))) return rc;
    const float *hd, *cd;
    if ((rc = stage_inputs(s, nf, cells1, h, c, mem, &hd, &cd))) return rc;
    if ((rc = forward_any(s, make_fields(hd, cd, np, cells1, p, nf), (int)nf, *g, mode, nullptr, 0))) return rc;
    SBS_CUDA_TRY(cudaMemcpyAsync(y, s->y4, sizeof(float) * nf * cells1,
                                 mem == SBS_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, s->stream));
    return tc_status(s);
}

int sbs_surrogate_loss_grad(sbs_surrogate *s, uint32_t nf, const float *h, const float *c,
                            const sbs_drainage_params *p, const float *target, double *loss, float *grad) {
    clear_error();
    CHECK_S(s);
    int rc = check_grid_params(nf, p);
    if (rc) return rc;
    SBS_CHECK_ARG(h && c && target && loss && grad, "null buffer");
    const int nt = (int)p[0].grid_height, np = (int)p[0].grid_width;
    const size_t cells1 = (size_t)nt * np;
    const GridDev *g = nullptr;
    if ((rc = grid_of(s, nt, np, &g))) return rc;
    if ((rc = ensure_ws(s, nf * cells1))) return rc;
    const float *hd, *cd;
    if ((rc = stage_inputs(s, nf, cells1, h, c, SBS_MEM_HOST, &hd, &cd))) return rc;
    SBS_CUDA_TRY(cudaMemcpyAsync(s->tgt, target, sizeof(float) * nf * cells1, cudaMemcpyHostToDevice, s->stream));
    if ((rc = loss_and_grad(s, make_fields(hd, cd, np, cells1, p, nf), (int)nf, *g, loss))) return rc;
    SBS_CUDA_TRY(cudaMemcpyAsync(grad, s->grad, sizeof(float) * SBS_NN_PARAMS, cudaMemcpyDeviceToHost, s->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return SBS_OK;
}

int sbs_surrogate_add_trajectory(sbs_surrogate *s, const float *h0, const float *c0, const sbs_drainage_params *p,
                                 uint32_t pairs, uint32_t substeps) {
    clear_error();
    CHECK_S(s);
    int rc = check_grid_params(1, p);
    if (rc) return rc;
    SBS_CHECK_ARG(h0 && c0, "null buffer");
    SBS_CHECK_ARG(pairs >= 1 && pairs <= 64, "pairs must be 1..64");
    SBS_CHECK_ARG(substeps <= 4096, "substeps must be 0 (automatic) .. 4096");
    SBS_CHECK_ARG(p->marangoni_enabled == 0, "the surrogate models marangoni_enabled = 0");
    const int nt = (int)p->grid_height, np = (int)p->grid_width;
    if (s->data.empty()) {
        if (s->plain) {
            sbs_drainage_destroy(s->plain);
            s->plain = nullptr;
        }
        s->dnt = nt;
        s->dnp = np;
    }
    SBS_CHECK_ARG(nt == s->dnt && np == s->dnp, "every trajectory needs the grid of the first (%d x %d)", s->dnt,
                  s->dnp);
    if (!s->plain) {
        if ((rc = sbs_gpu_drainage_create(500e-9f, (uint32_t)np, (uint32_t)nt, &s->plain))) return rc;
    }
    if (substeps == 0) {
        // largest per-pass diffusion number of the grid (theta + phi at the row nearest a pole, with
        // the WGSL kernel's sin floor 1e-4) kept at or below 0.2
        const double dth = M_PI / (double)(nt - 1), dph = 2.0 * M_PI / (double)np;
        const double s1 = std::max(std::sin(dth), 1e-4);
        const double mu = (double)p->dt * (double)p->diffusion_coeff / ((double)p->bubble_radius * p->bubble_radius) *
                          (2.0 / (dth * dth) + 2.0 / (dph * dph * s1 * s1));
        substeps = 1;
        while (mu / substeps > 0.2 && substeps < 4096) substeps *= 2;
    }
    sbs_drainage_params ps = *p;
    ps.dt = (float)((double)p->dt / substeps);
    if ((rc = sbs_gpu_drainage_update_params(s->plain, &ps))) return rc;
    const size_t cells = (size_t)nt * np;
    Traj t;
    t.p = *p;
    t.fc = field_consts(*p);
    t.pairs = pairs;
    SBS_CUDA_TRY(cudaMalloc(&t.h, sizeof(float) * cells * (pairs + 1)));
    if (cudaMalloc(&t.c, sizeof(float) * cells * (pairs + 1)) != cudaSuccess) {
        cudaFree(t.h);
        return set_error(SBS_E_NOMEM, "trajectory allocation failed");
    }
    auto fail = [&](int code) {
        cudaFree(t.h);
        cudaFree(t.c);
        return code;
    };
    if ((rc = sbs_drainage_set_thickness(s->plain, h0, cells, SBS_MEM_HOST))) return fail(rc);
    if ((rc = sbs_drainage_set_concentration(s->plain, c0, cells, SBS_MEM_HOST))) return fail(rc);
    for (uint32_t k = 0; k <= pairs; ++k) {
        if (k > 0 && (rc = sbs_gpu_drainage_run(s->plain, SBS_NN_STEPS * substeps))) return fail(rc);
        if ((rc = sbs_drainage_get_thickness_field(s->plain, t.h + cells * k, cells, SBS_MEM_DEVICE))) return fail(rc);
        if ((rc = sbs_drainage_get_concentration_field(s->plain, t.c + cells * k, cells, SBS_MEM_DEVICE)))
            return fail(rc);
    }
    s->data.push_back(t);
    return SBS_OK;
}

int sbs_surrogate_num_trajectories(const sbs_surrogate *s, uint32_t *out) {
    clear_error();
    CHECK_S(s);
    SBS_CHECK_ARG(out != nullptr, "out is null");
    *out = (uint32_t)s->data.size();
    return SBS_OK;
}

int sbs_surrogate_clear_data(sbs_surrogate *s) {
    clear_error();
    CHECK_S(s);
    SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    for (auto &t : s->data) {
        cudaFree(t.h);
        cudaFree(t.c);
    }
    s->data.clear();
    return SBS_OK;
}

int sbs_surrogate_train(sbs_surrogate *s, uint32_t n_train, uint32_t iters, uint32_t batch, float lr, uint64_t seed,
                        float *losses) {
    clear_error();
    CHECK_S(s);
    SBS_CHECK_ARG(n_train >= 1 && n_train <= s->data.size(), "n_train must be 1..%zu", s->data.size());
    SBS_CHECK_ARG(batch >= 1 && batch <= (uint32_t)kMaxFields, "batch must be 1..%d", kMaxFields);
    SBS_CHECK_ARG(std::isfinite(lr) && lr > 0.f, "lr must be positive");
    const int nt = s->dnt, np = s->dnp;
    const size_t cells1 = (size_t)nt * np;
    const GridDev *g = nullptr;
    int rc = grid_of(s, nt, np, &g);
    if (rc) return rc;
    if ((rc = ensure_ws(s, batch * cells1))) return rc;
    // pair index -> (trajectory, pair)
    std::vector<std::pair<uint32_t, uint32_t>> pool;
    for (uint32_t k = 0; k < n_train; ++k)
        for (uint32_t q = 0; q < s->data[k].pairs; ++q) pool.emplace_back(k, q);
    uint64_t st = seed;
    for (uint32_t it = 0; it < iters; ++it) {
        Fields fs{};
        const float *h0[kMaxFields], *h1[kMaxFields];
        float kout[kMaxFields];
        for (uint32_t b = 0; b < batch; ++b) {
            const auto &pr = pool[splitmix64(st) % pool.size()];
            const Traj &t = s->data[pr.first];
            const float *hp = t.h + cells1 * pr.second, *cp = t.c + cells1 * pr.second;
            fs.f[b] = Field{hp, cp, (size_t)np, t.fc.gk, t.fc.f5, t.fc.f6, t.fc.kout, t.fc.lm};
            h0[b] = hp;
            h1[b] = hp + cells1;
            kout[b] = t.fc.kout;
        }
        SBS_CUDA_TRY(targets(h0, h1, kout, (int)batch, nt, np, s->tgt, s->stream));
        double loss = 0.0;
        if ((rc = loss_and_grad(s, fs, (int)batch, *g, &loss))) return rc;
        if (!std::isfinite(loss)) return set_error(SBS_E_NONFINITE, "training loss became non-finite at step %u", it);
        if (losses) losses[it] = (float)loss;
        const double frac = iters > 1 ? (double)it / (double)(iters - 1) : 0.0;
        const float lr_t = (float)(lr * (0.05 + 0.95 * 0.5 * (1.0 + std::cos(M_PI * frac))));
        ++s->adam_step;
        SBS_CUDA_TRY(adam(s->theta, s->m, s->v, s->grad, lr_t, 0.9f, 0.999f, 1e-8f, s->adam_step, s->stream));
        if ((rc = repack(s))) return rc;
    }
    SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return SBS_OK;
}

int sbs_surrogate_evaluate(sbs_surrogate *s, uint32_t first, uint32_t count, int mode, sbs_surrogate_eval *out) {
    clear_error();
    CHECK_S(s);
    SBS_CHECK_ARG(out != nullptr, "out is null");
    SBS_CHECK_ARG(count >= 1 && (size_t)first + count <= s->data.size(), "trajectory range out of bounds");
    const int nt = s->dnt, np = s->dnp;
    const size_t cells1 = (size_t)nt * np;
    const GridDev *g = nullptr;
    int rc = grid_of(s, nt, np, &g);
    if (rc) return rc;
    if ((rc = ensure_ws(s, cells1))) return rc;
    if (s->scratch_cap < cells1) {
        cudaFree(s->scratch);
        s->scratch = nullptr;
        SBS_CUDA_TRY(cudaMalloc(&s->scratch, sizeof(float) * cells1));
        s->scratch_cap = cells1;
    }
    double sl = 0.0, sl0 = 0.0, r = 0.0, r0 = 0.0;
    size_t n = 0;
    const double nmask = (double)g->mask_rows * np;
    std::vector<double> lp;
    for (uint32_t k = first; k < first + count; ++k) {
        const Traj &t = s->data[k];
        for (uint32_t q = 0; q < t.pairs; ++q) {
            const float *hp = t.h + cells1 * q, *cp = t.c + cells1 * q, *hn = hp + cells1;
            Fields fs{};
            fs.f[0] = Field{hp, cp, (size_t)np, t.fc.gk, t.fc.f5, t.fc.f6, t.fc.kout, t.fc.lm};
            if ((rc = forward_any(s, fs, 1, *g, mode, s->scratch, (size_t)np))) return rc;
            if (mode == SBS_NN_FUSED) {
                // the fused kernel writes h' directly; y = (h' - h) / kout is not needed for rel_linf, the loss
                // is taken from the layered path below
                if ((rc = forward_any(s, fs, 1, *g, SBS_NN_LAYERED, nullptr, 0))) return rc;
            }
            const float *h0a[1] = {hp}, *h1a[1] = {hn};
            const float ko[1] = {t.fc.kout};
            SBS_CUDA_TRY(targets(h0a, h1a, ko, 1, nt, np, s->tgt, s->stream));
            int nlb = 0;
            SBS_CUDA_TRY(output_layer(s->a3, s->pk, s->y4, s->tgt, s->g4, s->loss_part, (float)(2.0 / nmask),
                                      g->tab(), 1, s->stream, &nlb));
            lp.resize(nlb);
            SBS_CUDA_TRY(
                cudaMemcpyAsync(lp.data(), s->loss_part, sizeof(double) * nlb, cudaMemcpyDeviceToHost, s->stream));
            unsigned e2[2], e20[2];
            SBS_CUDA_TRY(masked_error(s->scratch, np, hn, np, g->tab(), s->err2, s->stream));
            SBS_CUDA_TRY(cudaMemcpyAsync(e2, s->err2, 8, cudaMemcpyDeviceToHost, s->stream));
            SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
            SBS_CUDA_TRY(masked_error(hp, np, hn, np, g->tab(), s->err2, s->stream));
            SBS_CUDA_TRY(cudaMemcpyAsync(e20, s->err2, 8, cudaMemcpyDeviceToHost, s->stream));
            // identity loss: mean of target^2 over the mask
            std::vector<float> tg(cells1);
            SBS_CUDA_TRY(cudaMemcpyAsync(tg.data(), s->tgt, sizeof(float) * cells1, cudaMemcpyDeviceToHost, s->stream));
            SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
            double l = 0.0;
            for (double v : lp) l += v;
            sl += l / nmask;
            std::vector<float> rowsw(nt);
            double l0 = 0.0;
            {
                const double dth = M_PI / (double)(nt - 1);
                for (int i = 1; i + 1 < nt; ++i) {
                    if (std::sin(i * dth) < SBS_NN_MASK_SIN) continue;
                    for (int j = 0; j < np; ++j) l0 += (double)tg[(size_t)i * np + j] * tg[(size_t)i * np + j];
                }
            }
            sl0 += l0 / nmask;
            float fd, fm, fd0, fm0;
            std::memcpy(&fd, &e2[0], 4);
            std::memcpy(&fm, &e2[1], 4);
            std::memcpy(&fd0, &e20[0], 4);
            std::memcpy(&fm0, &e20[1], 4);
            r = std::max(r, (double)fd / (double)fm);
            r0 = std::max(r0, (double)fd0 / (double)fm0);
            ++n;
        }
    }
    out->loss = sl / (double)n;
    out->loss_identity = sl0 / (double)n;
    out->rel_linf = r;
    out->rel_linf_identity = r0;
    return tc_status(s);
}

int sbs_surrogate_masked_error(const float *a, const float *b, uint32_t nt, uint32_t np, int mem, double *out) {
    clear_error();
    SBS_CHECK_ARG(a && b && out, "null buffer");
    SBS_CHECK_ARG(nt >= 4 && np >= 3, "grid needs >= 4 theta rows and >= 3 phi columns");
    const double dth = M_PI / (double)(nt - 1);
    auto absdiff = [&](const float *ha, const float *hb) {
        float d = 0.f, m = 0.f;
        for (uint32_t i = 1; i + 1 < nt; ++i) {
            if (std::sin(i * dth) < SBS_NN_MASK_SIN) continue;
            for (uint32_t j = 0; j < np; ++j) {
                float e = std::fabs(ha[(size_t)i * np + j] - hb[(size_t)i * np + j]);
                if (e != e) e = INFINITY;
                d = std::max(d, e);
                m = std::max(m, std::fabs(hb[(size_t)i * np + j]));
            }
        }
        return (double)d / (double)m;
    };
    if (mem == SBS_MEM_HOST) {
        *out = absdiff(a, b);
        return SBS_OK;
    }
    SBS_CHECK_ARG(mem == SBS_MEM_DEVICE, "mem must be SBS_MEM_HOST or SBS_MEM_DEVICE");
    std::vector<float> ha((size_t)nt * np), hb((size_t)nt * np);
    SBS_CUDA_TRY(cudaMemcpy(ha.data(), a, sizeof(float) * ha.size(), cudaMemcpyDeviceToHost));
    SBS_CUDA_TRY(cudaMemcpy(hb.data(), b, sizeof(float) * hb.size(), cudaMemcpyDeviceToHost));
    *out = absdiff(ha.data(), hb.data());
    return SBS_OK;
}

}  // extern "C"

namespace {

// One surrogate interval on handle d: h[cur] -> h[1 - cur] (or into `into` when given), concentration
// copied along, clock advanced.
int advance_into(sbs_surrogate *s, sbs_drainage *d, int mode, float *into) {
    const GridDev *g = nullptr;
    int rc = grid_of(s, d->nt, d->np, &g);
    if (rc) return rc;
    const FieldC fc = field_consts(d->params);
    Fields fs{};
    fs.f[0] = Field{d->h[d->cur], d->c[d->cur], d->pitch, fc.gk, fc.f5, fc.f6, fc.kout, fc.lm};
    // order the handle's queued work before ours
    cudaEvent_t ev;
    SBS_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaEventRecord(ev, d->stream);
    cudaStreamWaitEvent(s->stream, ev, 0);
    float *dst = into ? into : d->h[1 - d->cur];
    const size_t pitch_out = into ? (size_t)d->np : d->pitch;
    if (mode == SBS_NN_LAYERED) {
        if ((rc = ensure_ws(s, (size_t)d->nt * d->np))) {
            cudaEventDestroy(ev);
            return rc;
        }
    }
    rc = forward_any(s, fs, 1, *g, mode, dst, pitch_out);
    if (rc) {
        cudaEventDestroy(ev);
        return rc;
    }
    if (!into) {
        SBS_CUDA_TRY(cudaMemcpy2DAsync(d->c[1 - d->cur], d->pitch * 4, d->c[d->cur], d->pitch * 4, (size_t)d->np * 4,
                                       d->nt, cudaMemcpyDeviceToDevice, s->stream));
    }
    cudaEventRecord(ev, s->stream);
    cudaStreamWaitEvent(d->stream, ev, 0);
    cudaEventDestroy(ev);
    if (!into) {
        d->prev = d->cur;
        d->cur = 1 - d->cur;
        d->current_time += (double)SBS_NN_STEPS * (double)d->params.dt;
    }
    return SBS_OK;
}

}  // namespace

extern "C" {

int sbs_surrogate_advance(sbs_surrogate *s, sbs_drainage *d, int mode) {
    clear_error();
    CHECK_S(s);
    SBS_CHECK_ARG(d != nullptr, "drainage handle is null");
    SBS_CHECK_ARG(d->sem == SBS_WGSL_SEMANTICS, "the surrogate advances WGSL-semantics handles");
    SBS_CHECK_ARG(d->params.marangoni_enabled == 0, "the surrogate models marangoni_enabled = 0");
    SBS_CHECK_ARG(d->nt >= 4, "grid needs >= 4 theta rows");
    int rc = advance_into(s, d, mode, nullptr);
    if (rc) return rc;
    SBS_CUDA_TRY(cudaStreamSynchronize(d->stream));
    return tc_status(s);
}

int sbs_surrogate_rollout(sbs_surrogate *s, sbs_drainage *d, uint32_t passes, uint32_t check_every, double tol,
                          int mode, sbs_surrogate_stats *stats) {
    clear_error();
    CHECK_S(s);
    SBS_CHECK_ARG(d != nullptr, "drainage handle is null");
    SBS_CHECK_ARG(d->sem == SBS_WGSL_SEMANTICS, "the surrogate advances WGSL-semantics handles");
    SBS_CHECK_ARG(d->params.marangoni_enabled == 0, "the surrogate models marangoni_enabled = 0");
    SBS_CHECK_ARG(passes % SBS_NN_STEPS == 0, "passes must be a multiple of %d", SBS_NN_STEPS);
    SBS_CHECK_ARG(std::isfinite(tol) && tol > 0.0, "tol must be positive");
    SBS_CHECK_ARG(d->nt >= 4, "grid needs >= 4 theta rows");
    sbs_surrogate_stats st{};
    const size_t cells1 = (size_t)d->nt * d->np;
    if (check_every && s->scratch_cap < cells1) {
        SBS_CUDA_TRY(cudaStreamSynchronize(s->stream));
        cudaFree(s->scratch);
        s->scratch = nullptr;
        SBS_CUDA_TRY(cudaMalloc(&s->scratch, sizeof(float) * cells1));
        s->scratch_cap = cells1;
    }
    const GridDev *g = nullptr;
    int rc = grid_of(s, d->nt, d->np, &g);
    if (rc) return rc;
    const uint32_t R = passes / SBS_NN_STEPS;
    uint32_t fallback = 0;
    for (uint32_t r = 0; r < R; ++r) {
        if (check_every && r % check_every == 0) {
            if ((rc = advance_into(s, d, mode, s->scratch))) return rc;
            if ((rc = drainage_run_async(d, SBS_NN_STEPS))) return rc;
            SBS_CUDA_TRY(masked_error(s->scratch, d->np, d->h[d->cur], d->pitch, g->tab(), s->err2, d->stream));
            unsigned e2[2];
            SBS_CUDA_TRY(cudaMemcpyAsync(e2, s->err2, 8, cudaMemcpyDeviceToHost, d->stream));
            SBS_CUDA_TRY(cudaStreamSynchronize(d->stream));
            float fd, fm;
            std::memcpy(&fd, &e2[0], 4);
            std::memcpy(&fm, &e2[1], 4);
            const double err = (double)fd / (double)fm;
            st.checks++;
            st.plain++;
            st.last_check_error = err;
            st.max_check_error = std::max(st.max_check_error, std::isfinite(err) ? err : INFINITY);
            if (!(err <= tol)) {
                st.failed_checks++;
                fallback = check_every - 1;
            }
        } else if (fallback > 0) {
            if ((rc = drainage_run_async(d, SBS_NN_STEPS))) return rc;
            st.plain++;
            --fallback;
        } else {
            if ((rc = advance_into(s, d, mode, nullptr))) return rc;
            st.surrogate++;
        }
        st.rollouts++;
    }
    SBS_CUDA_TRY(cudaStreamSynchronize(d->stream));
    if ((rc = tc_status(s))) return rc;
    if (stats) *stats = st;
    return SBS_OK;
}

}  // extern "C"
