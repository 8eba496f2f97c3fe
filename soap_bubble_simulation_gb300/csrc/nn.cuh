// Shared device pieces of the drainage surrogate (include/sbs_nn.h): the FP32 GELU and its
// derivative in the exact operation order of the definition, BF16 packing, and the argument
// structs of the kernels in nn_kernels.cu / nn_fused.cu.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/sbs_nn.h"

namespace sbs {
namespace nn {

typedef __nv_bfloat16 bf16;

constexpr int kTileCols = 128;  // output columns per tile of the layered kernels
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
    float gk, f5, f6, kout;
};

struct Fields {
    Field f[kMaxFields];
};

// Per-grid row table: cp, cg, sin(theta), loss/check mask (1.0 / 0.0).
struct GridTab {
    const float4 *rows;
    float ct;
    int nt, np;
};

}  // namespace nn
}  // namespace sbs
