// Shared device pieces of the drainage surrogate (include/sbs_nn.h): the FP32 activations (GELU
// polynomial and hard-swish) and their derivatives in the exact operation order of the
// definition, BF16 packing, and the argument structs of the kernels in nn_kernels.cu /
// nn_fused.cu.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sbs_nn.h"

namespace sbs {
namespace nn {

typedef __nv_bfloat16 bf16;

constexpr int kMaxFields = 16;  // fields per batched launch

__device__ __forceinline__ float phi_poly(float t, float u, float *p_out) {
    const float p =
        __fmaf_rn(__fmaf_rn(__fmaf_rn(__fmaf_rn(SBS_NN_Q4, u, SBS_NN_Q3), u, SBS_NN_Q2), u, SBS_NN_Q1), u, SBS_NN_Q0);
    *p_out = p;
    return __fmaf_rn(t, p, 0.5f);
}

__device__ __forceinline__ float gelu(float x) {
    const float t = fminf(fmaxf(x, -3.f), 3.f);
    const float u = __fmul_rn(t, t);
    float p;
    const float phi = phi_poly(t, u, &p);
    return __fmul_rn(x, phi);
}

__device__ __forceinline__ float gelu_grad(float x) {
    const float t = fminf(fmaxf(x, -3.f), 3.f);
    const float u = __fmul_rn(t, t);
    float p;
    const float phi = phi_poly(t, u, &p);
    const float dp = __fmaf_rn(__fmaf_rn(__fmaf_rn(SBS_NN_Q4X4, u, SBS_NN_Q3X3), u, SBS_NN_Q2X2), u, SBS_NN_Q1);
    const float dphi = fabsf(x) < 3.f ? __fmaf_rn(__fadd_rn(u, u), dp, p) : 0.f;
    return __fmaf_rn(x, dphi, phi);
}

// Two GELUs with packed FP32x2 arithmetic: the same IEEE round-to-nearest operations as gelu(),
// so the results are bitwise those of two gelu() calls.
__device__ __forceinline__ float2 gelu2(float2 x) {
    const float2 t = make_float2(fminf(fmaxf(x.x, -3.f), 3.f), fminf(fmaxf(x.y, -3.f), 3.f));
    const float2 u = __fmul2_rn(t, t);
    float2 p = __ffma2_rn(make_float2(SBS_NN_Q4, SBS_NN_Q4), u, make_float2(SBS_NN_Q3, SBS_NN_Q3));
    p = __ffma2_rn(p, u, make_float2(SBS_NN_Q2, SBS_NN_Q2));
    p = __ffma2_rn(p, u, make_float2(SBS_NN_Q1, SBS_NN_Q1));
    p = __ffma2_rn(p, u, make_float2(SBS_NN_Q0, SBS_NN_Q0));
    const float2 phi = __ffma2_rn(t, p, make_float2(0.5f, 0.5f));
    return __fmul2_rn(x, phi);
}

// sat(fma(a, b, c)) in one instruction: round-to-nearest FMA, then clamp to [0, 1] (NaN -> +0).
__device__ __forceinline__ float fma_sat(float a, float b, float c) {
    float r;
    asm("fma.rn.sat.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Hard-swish: x * sat(fma(x, 1/6, 0.5)).
__device__ __forceinline__ float hswish(float x) { return __fmul_rn(x, fma_sat(x, SBS_NN_HS_SLOPE, 0.5f)); }

__device__ __forceinline__ float hswish_grad(float x) {
    const float r = __fmaf_rn(x, SBS_NN_HS_SLOPE, 0.5f);
    const float s = __saturatef(r);
    return (r > 0.f && r < 1.f) ? __fmaf_rn(x, SBS_NN_HS_SLOPE, s) : s;
}

// Two hard-swishes: the saturating FMAs are scalar (there is no saturating FP32x2 FMA), the
// product is one packed FP32x2 multiply; bitwise the results of two hswish() calls.
__device__ __forceinline__ float2 hswish2(float2 x) {
    const float2 s = make_float2(fma_sat(x.x, SBS_NN_HS_SLOPE, 0.5f), fma_sat(x.y, SBS_NN_HS_SLOPE, 0.5f));
    return __fmul2_rn(x, s);
}

// Two GELU derivatives with packed FP32x2 arithmetic: the operations of gelu_grad() (the
// derivative term is formed for both halves and then selected), so bitwise two gelu_grad() calls.
__device__ __forceinline__ float2 gelu_grad2(float2 x) {
    const float2 t = make_float2(fminf(fmaxf(x.x, -3.f), 3.f), fminf(fmaxf(x.y, -3.f), 3.f));
    const float2 u = __fmul2_rn(t, t);
    float2 p = __ffma2_rn(make_float2(SBS_NN_Q4, SBS_NN_Q4), u, make_float2(SBS_NN_Q3, SBS_NN_Q3));
    p = __ffma2_rn(p, u, make_float2(SBS_NN_Q2, SBS_NN_Q2));
    p = __ffma2_rn(p, u, make_float2(SBS_NN_Q1, SBS_NN_Q1));
    p = __ffma2_rn(p, u, make_float2(SBS_NN_Q0, SBS_NN_Q0));
    const float2 phi = __ffma2_rn(t, p, make_float2(0.5f, 0.5f));
    float2 dp = __ffma2_rn(make_float2(SBS_NN_Q4X4, SBS_NN_Q4X4), u, make_float2(SBS_NN_Q3X3, SBS_NN_Q3X3));
    dp = __ffma2_rn(dp, u, make_float2(SBS_NN_Q2X2, SBS_NN_Q2X2));
    dp = __ffma2_rn(dp, u, make_float2(SBS_NN_Q1, SBS_NN_Q1));
    const float2 d = __ffma2_rn(__fadd2_rn(u, u), dp, p);
    const float2 dphi = make_float2(fabsf(x.x) < 3.f ? d.x : 0.f, fabsf(x.y) < 3.f ? d.y : 0.f);
    return __ffma2_rn(x, dphi, phi);
}

// Two hard-swish derivatives: bitwise two hswish_grad() calls.
__device__ __forceinline__ float2 hswish_grad2(float2 x) {
    const float2 r = __ffma2_rn(x, make_float2(SBS_NN_HS_SLOPE, SBS_NN_HS_SLOPE), make_float2(0.5f, 0.5f));
    const float2 s = make_float2(__saturatef(r.x), __saturatef(r.y));
    const float2 g = __ffma2_rn(x, make_float2(SBS_NN_HS_SLOPE, SBS_NN_HS_SLOPE), s);
    return make_float2((r.x > 0.f && r.x < 1.f) ? g.x : s.x, (r.y > 0.f && r.y < 1.f) ? g.y : s.y);
}

// The network's activation (SBS_NN_ACT_*), chosen by a value that is uniform over the launch.
__device__ __forceinline__ float act(int kind, float x) { return kind == SBS_NN_ACT_HSWISH ? hswish(x) : gelu(x); }
__device__ __forceinline__ float act_grad(int kind, float x) {
    return kind == SBS_NN_ACT_HSWISH ? hswish_grad(x) : gelu_grad(x);
}
// The same for two values at once (packed FP32x2), bitwise two scalar calls.
__device__ __forceinline__ float2 act2(int kind, float2 x) {
    return kind == SBS_NN_ACT_HSWISH ? hswish2(x) : gelu2(x);
}
__device__ __forceinline__ float2 act_grad2(int kind, float2 x) {
    return kind == SBS_NN_ACT_HSWISH ? hswish_grad2(x) : gelu_grad2(x);
}

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ float clampf(float v) {
    return fminf(fmaxf(v, -SBS_NN_FEATURE_CLAMP), SBS_NN_FEATURE_CLAMP);
}

// One field of a batched launch: thickness / concentration rows (pitch in elements) and the
// per-field scalars of include/sbs_nn.h.
struct Field {
    const float *h;
    const float *c;
    size_t pitch;
    float gk, f5, f6, kout, lm;
};

struct Fields {
    Field f[kMaxFields];
};

// Per-grid tables: rows[i] = (cp, cg, sin(theta), loss/check mask 1.0 / 0.0), lip[i] =
// log10(1 / (dph^2 se^2)), lith = log10(1 / dth^2).
struct GridTab {
    const float4 *rows;
    const float *lip;
    float ct, lith;
    int nt, np;
};

// Writes the 16 features of one cell (include/sbs_nn.h) as two 16-byte planes.
__device__ __forceinline__ void cell_features(float hc, float hn, float hs, float hw, float he, float cc, float4 row,
                                              float lip, const Field &f, const GridTab &g, uint4 &p0, uint4 &p1) {
    const float h2 = __fadd_rn(hc, hc);
    p0.x = pack2(clampf(__fmul_rn(__fsub_rn(hc, SBS_NN_H0), SBS_NN_INV_HS)),
                 clampf(__fmul_rn(__fsub_rn(__fadd_rn(hn, hs), h2), g.ct)));
    p0.y = pack2(clampf(__fmul_rn(__fsub_rn(__fadd_rn(hw, he), h2), row.x)), clampf(__fmul_rn(__fsub_rn(hs, hn), row.y)));
    p0.z = pack2(clampf(__fmul_rn(__fsub_rn(cc, 0.5f), 10.f)), clampf(f.f5));
    p0.w = pack2(clampf(f.f6), clampf(__fmul_rn(__fmul_rn(__fmul_rn(hc, hc), hc), __fmul_rn(f.gk, row.z))));
    p1.x = pack2(clampf(__fadd_rn(f.lm, g.lith)), clampf(__fadd_rn(f.lm, lip)));
    p1.y = pack2(clampf(row.z), 0.f);
    p1.z = 0u;
    p1.w = 0u;
}

}  // namespace nn
}  // namespace sbs
