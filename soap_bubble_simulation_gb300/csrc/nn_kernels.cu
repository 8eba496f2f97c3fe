// Training-side kernels of the drainage surrogate (include/sbs_nn.h) and its layered forward
// pass: features, the one-channel output layer and its gradients on the FP32 pipe, loss,
// deterministic gradient reduction, Adam, and weight packing. The 3x3 convolutions, their input
// gradients and their weight gradients run on tcgen05 (nn_conv_tc.cu).
//
// Layouts (channel-last, cells = fields x nt x np):
//   features x        BF16 [cells][16]
//   pre-activations y FP32 [cells][32]       activations a BF16 [cells][32]
//   output y4 / gradient g4 FP32 [cells]     layer gradients g BF16 [cells][32]
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>

#include "nn.cuh"
#include "nn_kernels.h"
#include "sbs_internal.h"

namespace sbs {
namespace nn {
namespace {

__device__ __forceinline__ int refl_row(int i, int nt) { return i < 0 ? 1 : (i >= nt ? nt - 2 : i); }

// ----------------------------------------------------------------------------------- features
__global__ void features_kernel(Fields fs, GridTab g, uint4 *x) {
    const int b = blockIdx.z, i = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= g.np) return;
    const Field &f = fs.f[b];
    const int nt = g.nt, np = g.np;
    const float *rc = f.h + (size_t)i * f.pitch;
    const float *rn = f.h + (size_t)refl_row(i - 1, nt) * f.pitch;
    const float *rs = f.h + (size_t)refl_row(i + 1, nt) * f.pitch;
    uint4 p0, p1;
    cell_features(rc[j], rn[j], rs[j], rc[j == 0 ? np - 1 : j - 1], rc[j + 1 == np ? 0 : j + 1],
                  f.c[(size_t)i * f.pitch + j], g.rows[i], g.lip[i], f, g, p0, p1);
    uint4 *o = x + (((size_t)b * nt + i) * np + j) * 2;
    o[0] = p0;
    o[1] = p1;
}

// ------------------------------------------------------------ output layer (one channel, FP32)
// y4 = b4 + sum_{tap, ic} W4[tap][ic] a3[src][ic]; with a target, also the masked loss gradient
// g4 = 2 (y4 - target) / n_mask and per-block partial sums of (y4 - target)^2.
struct OutArgs {
    const bf16 *a3;
    const float *w4;  // [9][32], BF16-rounded values
    const float *b4;
    float *y4;
    const float *target;  // null: forward only
    float *g4;
    double *loss_part;
    float inv_nmask2;  // 2 / n_mask
    GridTab g;
    int nf;
};

// The three source rows i - 1, i, i + 1 (theta reflected) of a3 for cells j0 - 1 .. j0 + 128 (phi
// wrapped) into dst[row][cell][0..31], one 16-byte copy per thread and step. For rows of at least
// 128 cells one correction wraps a column (the cells span less than two row lengths).
constexpr int kSegCells = 128;  // cells per row segment of the layer-4 kernels
template <int STRIDE>
__device__ __forceinline__ void stage_rows3(bf16 (*dst)[kSegCells + 2][STRIDE], const bf16 *a3, size_t fb, int i,
                                            int nt, int np, int j0) {
    const int ru = refl_row(i - 1, nt), rd = refl_row(i + 1, nt);
    const bool wide = np >= kSegCells;
    for (int e = threadIdx.x; e < 3 * (kSegCells + 2) * 4; e += blockDim.x) {
        const int d = e / ((kSegCells + 2) * 4), rem = e - d * ((kSegCells + 2) * 4), q = rem >> 2, ch = rem & 3;
        int col = j0 - 1 + q;
        if (wide) {
            col = col < 0 ? col + np : (col >= np ? col - np : col);
        } else {
            col %= np;
            col = col < 0 ? col + np : col;
        }
        const int r = d == 0 ? ru : (d == 1 ? i : rd);
        *reinterpret_cast<uint4 *>(&dst[d][q][ch * 8]) =
            *reinterpret_cast<const uint4 *>(a3 + (fb + (size_t)r * np + col) * 32 + ch * 8);
    }
}

// One block per item (an output row x a 128-cell segment): the three source rows of a3 (130 cells
// each, phi wrapped, theta reflected) are staged in shared memory with 80 bytes per cell (16-byte
// reads of consecutive cells fall in distinct banks), then one thread per cell. The four chunk sums
// of a cell run as two packed FP32x2 pairs (chunks 0, 1 and 2, 3): each half performs its chunk's
// multiply-adds tap by tap and channel by channel, so y is bitwise that of four scalar chains.
constexpr int kOutCells = kSegCells;
constexpr int kOutStride = 40;  // BF16 values per staged cell (32 + 8)

__global__ void __launch_bounds__(kOutCells, 7) out_kernel(OutArgs a) {  // 7 blocks: the shared-memory limit
    __shared__ float2 swp[9][2][8];  // tap, chunk pair: (W4[tap][16 kp + c], W4[tap][16 kp + 8 + c])
    __shared__ __align__(16) bf16 sa[3][kOutCells + 2][kOutStride];
    __shared__ double sred[kOutCells / 32];
    const int nt = a.g.nt, np = a.g.np;
    const int segs = (np + kOutCells - 1) / kOutCells;
    const int row = (int)(blockIdx.x / segs), j0 = (int)(blockIdx.x % segs) * kOutCells;
    const int i = row % nt;
    const size_t fb = (size_t)(row / nt) * nt * np;
    for (int e = threadIdx.x; e < 9 * 16; e += blockDim.x) {
        const int t = e >> 4, kp = (e >> 3) & 1, c = e & 7;
        swp[t][kp][c] = make_float2(a.w4[t * 32 + 16 * kp + c], a.w4[t * 32 + 16 * kp + 8 + c]);
    }
    stage_rows3<kOutStride>(sa, a.a3, fb, i, nt, np, j0);
    __syncthreads();
    const int m = threadIdx.x, j = j0 + m;
    double l = 0.0;
    if (j < np) {
        const size_t c = fb + (size_t)i * np + j;
        // four independent partial sums (one per 8-channel chunk), as the pairs (0, 1) and (2, 3)
        float2 y01 = make_float2(0.f, 0.f), y23 = y01;
#pragma unroll
        for (int t = 0; t < 9; ++t) {
            const int d = t / 3, x = t % 3;  // source row i + d - 1 (reflected when staged), cell j + x - 1
            const uint4 *p = reinterpret_cast<const uint4 *>(&sa[d][m + x][0]);
            const uint4 v0 = p[0], v1 = p[1], v2 = p[2], v3 = p[3];
            const uint32_t u0[4] = {v0.x, v0.y, v0.z, v0.w}, u1[4] = {v1.x, v1.y, v1.z, v1.w};
            const uint32_t u2[4] = {v2.x, v2.y, v2.z, v2.w}, u3[4] = {v3.x, v3.y, v3.z, v3.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const float2 f0 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&u0[e]));
                const float2 f1 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&u1[e]));
                const float2 f2 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&u2[e]));
                const float2 f3 = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&u3[e]));
                y01 = __ffma2_rn(swp[t][0][2 * e], make_float2(f0.x, f1.x), y01);
                y01 = __ffma2_rn(swp[t][0][2 * e + 1], make_float2(f0.y, f1.y), y01);
                y23 = __ffma2_rn(swp[t][1][2 * e], make_float2(f2.x, f3.x), y23);
                y23 = __ffma2_rn(swp[t][1][2 * e + 1], make_float2(f2.y, f3.y), y23);
            }
        }
        const float y = __fadd_rn(*a.b4, __fadd_rn(__fadd_rn(y01.x, y01.y), __fadd_rn(y23.x, y23.y)));
        a.y4[c] = y;
        if (a.target) {
            const float mk = a.g.rows[i].w;
            float gr = 0.f;
            if (mk != 0.f) {
                const float dd = __fsub_rn(y, a.target[c]);
                l = (double)dd * (double)dd;
                gr = __fmul_rn(dd, a.inv_nmask2);
            }
            a.g4[c] = gr;
        }
    }
    if (a.target) {
        for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
        if ((threadIdx.x & 31) == 0) sred[threadIdx.x >> 5] = l;
        __syncthreads();
        if (threadIdx.x == 0) {
            double sum = 0.0;
            for (int k = 0; k < kOutCells / 32; ++k) sum += sred[k];
            a.loss_part[blockIdx.x] = sum;
        }
    }
}

// dW4[tap][ic] = sum g4[cell] a3[src(cell,tap)][ic], db4 = sum g4. Work item: one output row x one
// 128-cell segment; block b takes items b, b + nblocks, ... Per item the block stages the three
// source rows of a3 (130 cells each, phi wrapped, theta reflected) and the row's g4 in shared
// memory; warp w sums the item's cells w, w + 8, ... with lane = ic and nine accumulators per lane
// (one per tap). One partial row [289] per block, warps summed in a fixed order. An item's rows are
// loaded and then used with nothing else in flight, so the grid is sized for six blocks per SM
// (kW4BlocksPerSm): other blocks' loads cover each block's wait.
struct Wgrad4Args {
    const float *g4;
    const bf16 *a3;
    float *partial;
    GridTab g;
    int rows;  // fields x nt
};

constexpr int kW4Warps = 8;
constexpr int kW4Cells = kSegCells;
constexpr int kW4BlocksPerSm = 6;  // 34.7 KB of shared memory and 40 registers a thread each

__global__ void __launch_bounds__(32 * kW4Warps, kW4BlocksPerSm) wgrad4_kernel(Wgrad4Args a) {
    __shared__ __align__(16) bf16 sa[3][kW4Cells + 2][32];
    __shared__ float sg[kW4Cells];
    __shared__ float sp[kW4Warps][289];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nt = a.g.nt, np = a.g.np;
    const int segs = (np + kW4Cells - 1) / kW4Cells, items = a.rows * segs;
    float acc[9];
#pragma unroll
    for (int t = 0; t < 9; ++t) acc[t] = 0.f;
    float gsum = 0.f;
    for (int item = blockIdx.x; item < items; item += gridDim.x) {
        const int row = item / segs, j0 = (item % segs) * kW4Cells;
        const int i = row % nt;
        const size_t fb = (size_t)(row / nt) * nt * np;
        const int n = min(kW4Cells, np - j0);
        __syncthreads();  // the previous item's tiles are read
        for (int e = tid; e < 3 * (kW4Cells + 2) * 4; e += blockDim.x) {
            const int d = e / ((kW4Cells + 2) * 4), q = (e / 4) % (kW4Cells + 2), ch = e % 4;
            int col = (j0 - 1 + q) % np;
            col = col < 0 ? col + np : col;
            const size_t src = (fb + (size_t)refl_row(i + d - 1, nt) * np + col) * 32 + ch * 8;
            *reinterpret_cast<uint4 *>(&sa[d][q][ch * 8]) = *reinterpret_cast<const uint4 *>(a.a3 + src);
        }
        for (int e = tid; e < kW4Cells; e += blockDim.x) sg[e] = e < n ? a.g4[fb + (size_t)i * np + j0 + e] : 0.f;
        __syncthreads();
        for (int m = warp; m < n; m += kW4Warps) {
            const float gv = sg[m];
            if (lane == 0) gsum = __fadd_rn(gsum, gv);
#pragma unroll
            for (int d = 0; d < 3; ++d)
#pragma unroll
                for (int x = 0; x < 3; ++x)
                    acc[3 * d + x] = __fmaf_rn(gv, __bfloat162float(sa[d][m + x][lane]), acc[3 * d + x]);
        }
    }
#pragma unroll
    for (int t = 0; t < 9; ++t) sp[warp][t * 32 + lane] = acc[t];
    if (lane == 0) sp[warp][288] = gsum;
    __syncthreads();
    for (int k = tid; k < 289; k += blockDim.x) {
        float v = 0.f;
        for (int w = 0; w < kW4Warps; ++w) v = __fadd_rn(v, sp[w][k]);
        a.partial[(size_t)blockIdx.x * 289 + k] = v;
    }
}

// g3[cell][ic] = bf16( (sum over the taps that read `cell` of g4[out] W4[tap][ic]) * act'(y3) ):
// one thread per cell with its 32 channels in registers (taps in the order t = 0..8, each tap's
// pole-reflection source right after its own term).
struct Dgrad4Args {
    const float *g4;
    const float *w4;
    const float *y3;
    bf16 *g3;
    GridTab g;
    size_t cells;
    int act;  // SBS_NN_ACT_*
};

__global__ void __launch_bounds__(256) dgrad4_kernel(Dgrad4Args a) {
    __shared__ float sw[288];
    for (int k = threadIdx.x; k < 288; k += blockDim.x) sw[k] = a.w4[k];
    __syncthreads();
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.cells) return;
    const int nt = a.g.nt, np = a.g.np;
    const int j = (int)(c % np), i = (int)((c / np) % nt);
    const size_t fb = (c / ((size_t)np * nt)) * nt * np;
    float s[32];
#pragma unroll
    for (int ic = 0; ic < 32; ++ic) s[ic] = 0.f;
#pragma unroll
    for (int t = 0; t < 9; ++t) {
        const int dy = t / 3 - 1, dx = t % 3 - 1;
        const int r = i - dy;
        int q = j - dx;
        q = q < 0 ? q + np : (q >= np ? q - np : q);
        const float gm = r >= 0 && r < nt ? a.g4[fb + (size_t)r * np + q] : 0.f;
        const bool xt = i == 1 && dy == -1, xb = i == nt - 2 && dy == 1;
        const float ge = xt ? a.g4[fb + q] : xb ? a.g4[fb + (size_t)(nt - 1) * np + q] : 0.f;
        const bool has_m = r >= 0 && r < nt;
#pragma unroll
        for (int ic = 0; ic < 32; ++ic) {
            if (has_m) s[ic] = __fmaf_rn(gm, sw[t * 32 + ic], s[ic]);
            if (xt || xb) s[ic] = __fmaf_rn(ge, sw[t * 32 + ic], s[ic]);
        }
    }
    const float4 *yp = reinterpret_cast<const float4 *>(a.y3 + c * 32);
    uint4 *gp = reinterpret_cast<uint4 *>(a.g3 + c * 32);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float4 y0 = yp[2 * k], y1 = yp[2 * k + 1];
        const float v[8] = {y0.x, y0.y, y0.z, y0.w, y1.x, y1.y, y1.z, y1.w};
        uint32_t w[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const float2 g = __fmul2_rn(make_float2(s[8 * k + 2 * e], s[8 * k + 2 * e + 1]),
                                        act_grad2(a.act, make_float2(v[2 * e], v[2 * e + 1])));
            w[e] = pack2(g.x, g.y);
        }
        gp[k] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// Column sums over the blocks' partial rows, in a fixed order: a block of 32 x ROWS threads takes
// 32 adjacent columns; thread (r, c) sums rows r, r + ROWS, ... of column c (coalesced 128-byte
// rows), then the ROWS partial sums are added in order r = 0, 1, ... Returns the sum in the threads
// with r = 0.
constexpr int kRedCols = 32, kRedRows = 8, kRed4Rows = 32;
template <int ROWS>
__device__ __forceinline__ float column_sum(const float *partial, int nblocks, int ncol, int col) {
    __shared__ float s_part[ROWS][kRedCols];
    const int c = threadIdx.x % kRedCols, r = threadIdx.x / kRedCols;
    float s = 0.f;
    if (col < ncol)
        for (int k = r; k < nblocks; k += ROWS) s = __fadd_rn(s, partial[(size_t)k * ncol + col]);
    s_part[r][c] = s;
    __syncthreads();
    float t = 0.f;
    if (r == 0)
        for (int q = 0; q < ROWS; ++q) t = __fadd_rn(t, s_part[q][c]);
    return t;
}

// sum of partial rows scattered into the canonical parameter layout W[tap][oc][ic] (partial column
// oc * 9 * CIN + tap * CIN + ic) and b[oc].
__global__ void __launch_bounds__(kRedCols *kRedRows) reduce_partials_kernel(const float *partial, int nblocks,
                                                                               int ci, int co, float *grad_w,
                                                                               float *grad_b) {
    const int ncol = co * 9 * ci + co;
    const int e = blockIdx.x * kRedCols + threadIdx.x % kRedCols;
    const float s = column_sum<kRedRows>(partial, nblocks, ncol, e);
    if (threadIdx.x >= kRedCols || e >= ncol) return;
    if (e < co * 9 * ci) {
        const int oc = e / (9 * ci), r = e % (9 * ci), t = r / ci, ic = r % ci;
        grad_w[((size_t)t * co + oc) * ci + ic] = s;
    } else {
        grad_b[e - co * 9 * ci] = s;
    }
}

// layer-4 partial rows are [block][tap*32 + ic] then db4
__global__ void __launch_bounds__(kRedCols *kRed4Rows) reduce4_kernel(const float *partial, int nblocks,
                                                                        float *grad_w4, float *grad_b4) {
    const int e = blockIdx.x * kRedCols + threadIdx.x % kRedCols;
    const float s = column_sum<kRed4Rows>(partial, nblocks, 289, e);
    if (threadIdx.x >= kRedCols || e >= 289) return;
    if (e < 288)
        grad_w4[e] = s;
    else
        *grad_b4 = s;
}

__global__ void adam_kernel(float *theta, float *m, float *v, const float *grad, int n, float lr, float b1,
                            float b2, float eps, float c1, float c2) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    const float g = grad[e];
    const float mm = b1 * m[e] + (1.f - b1) * g;
    const float vv = b2 * v[e] + (1.f - b2) * g * g;
    m[e] = mm;
    v[e] = vv;
    theta[e] -= lr * (mm * c1) / (sqrtf(vv * c2) + eps);
}

// BF16 weight layouts for the layered kernels from the FP32 parameter vector.
__global__ void pack_kernel(const float *theta, Packed p) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    // forward layouts [oc][tap*CIN+ic]
    if (e < 32 * 144) {
        const int oc = e / 144, k = e % 144;
        p.wf1[e] = __float2bfloat16_rn(theta[SBS_NN_W1 + ((k / 16) * 32 + oc) * 16 + (k % 16)]);
    }
    if (e < 32 * 288) {
        const int n = e / 288, k = e % 288, t = k / 32, r = k % 32;
        // forward: n = oc, r = ic;  transpose: n = ic, r = oc
        p.wf2[e] = __float2bfloat16_rn(theta[SBS_NN_W2 + (t * 32 + n) * 32 + r]);
        p.wf3[e] = __float2bfloat16_rn(theta[SBS_NN_W3 + (t * 32 + n) * 32 + r]);
        p.wb2[e] = __float2bfloat16_rn(theta[SBS_NN_W2 + (t * 32 + r) * 32 + n]);
        p.wb3[e] = __float2bfloat16_rn(theta[SBS_NN_W3 + (t * 32 + r) * 32 + n]);
    }
    if (e < 288) p.w4[e] = __bfloat162float(__float2bfloat16_rn(theta[SBS_NN_W4 + e]));
    if (e < 32) {
        p.b[e] = theta[SBS_NN_B1 + e];
        p.b[32 + e] = theta[SBS_NN_B2 + e];
        p.b[64 + e] = theta[SBS_NN_B3 + e];
    }
    if (e == 0) p.b[96] = theta[SBS_NN_B4];
}

// h' = max(h + kout y, 0) on rows 1..nt-2, rows 0 and nt-1 copied (one field).
__global__ void apply_kernel(const float *h, size_t pitch_in, const float *y, float kout, int nt, int np, float *out,
                             size_t pitch_out) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (j >= np) return;
    const float hc = h[(size_t)i * pitch_in + j];
    float r = hc;
    if (i > 0 && i + 1 < nt) r = fmaxf(__fadd_rn(hc, __fmul_rn(kout, y[(size_t)i * np + j])), 0.f);
    out[(size_t)i * pitch_out + j] = r;
}

// target[b][cell] = (h_next - h) / kout for a batch of snapshot pairs
struct TargetArgs {
    const float *h0[kMaxFields];
    const float *h1[kMaxFields];
    float kout[kMaxFields];
};

__global__ void target_kernel(TargetArgs t, int nt, int np, float *target) {
    const int b = blockIdx.z, i = blockIdx.y;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= np) return;
    const size_t k = (size_t)i * np + j;
    target[((size_t)b * nt) * np + k] = __fdiv_rn(__fsub_rn(t.h1[b][k], t.h0[b][k]), t.kout[b]);
}

// max |a - b| and max |b| over the masked rows (rows[i].w != 0) as float bit patterns (both are
// non-negative, so unsigned order is float order); a NaN difference counts as +inf.
__global__ void masked_err_kernel(const float *a, size_t pa, const float *b, size_t pb, const float4 *rows, int nt,
                                  int np, unsigned *out) {
    const int i = blockIdx.y;
    float d = 0.f, m = 0.f;
    if (rows[i].w != 0.f) {
        for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < np; j += gridDim.x * blockDim.x) {
            const float va = a[(size_t)i * pa + j], vb = b[(size_t)i * pb + j];
            float e = fabsf(__fsub_rn(va, vb));
            if (e != e) e = __int_as_float(0x7f800000);
            d = fmaxf(d, e);
            m = fmaxf(m, fabsf(vb));
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        d = fmaxf(d, __shfl_xor_sync(0xffffffffu, d, o));
        m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, __float_as_uint(d));
        atomicMax(out + 1, __float_as_uint(m));
    }
}


}  // namespace

// ------------------------------------------------------------------------------ host wrappers
cudaError_t features(const Fields &fs, int nf, const GridTab &g, bf16 *x, cudaStream_t st) {
    dim3 grid((g.np + 127) / 128, g.nt, nf);
    features_kernel<<<grid, 128, 0, st>>>(fs, g, (uint4 *)x);
    return cudaGetLastError();
}


cudaError_t conv_backward_weight(int layer, const bf16 *g, const bf16 *x, float *partial, int nblocks, float *grad,
                                 unsigned *err, int nf, int nt, int np, cudaStream_t st) {
    const int ci = layer == 1 ? 16 : 32;
    const int ow = layer == 1 ? SBS_NN_W1 : (layer == 2 ? SBS_NN_W2 : SBS_NN_W3);
    const int ob = layer == 1 ? SBS_NN_B1 : (layer == 2 ? SBS_NN_B2 : SBS_NN_B3);
    cudaError_t e = wgrad_tc(ci, g, x, partial, nblocks, err, nf, nt, np, st);
    if (e != cudaSuccess) return e;
    const int ncol = 32 * 9 * ci + 32;
    reduce_partials_kernel<<<(ncol + kRedCols - 1) / kRedCols, kRedCols * kRedRows, 0, st>>>(partial, nblocks, ci, 32,
                                                                                         grad + ow, grad + ob);
    return cudaGetLastError();
}

cudaError_t output_layer(const bf16 *a3, const Packed &p, float *y4, const float *target, float *g4,
                         double *loss_part, float inv_nmask2, const GridTab &g, int nf, cudaStream_t st,
                         int *nblocks_out) {
    OutArgs o{};
    o.a3 = a3;
    o.w4 = p.w4;
    o.y4 = y4;
    o.target = target;
    o.g4 = g4;
    o.loss_part = loss_part;
    o.inv_nmask2 = inv_nmask2;
    o.g = g;
    o.nf = nf;
    o.b4 = p.b + 96;
    const int nb = nf * g.nt * ((g.np + kOutCells - 1) / kOutCells);  // one block per row segment
    out_kernel<<<nb, kOutCells, 0, st>>>(o);
    if (nblocks_out) *nblocks_out = nb;
    return cudaGetLastError();
}

cudaError_t output_backward(const float *g4, const bf16 *a3, const float *y3, const Packed &p, bf16 *g3,
                            float *partial, int nblocks, float *grad, const GridTab &g, int nf, cudaStream_t st) {
    const size_t cells = (size_t)nf * g.nt * g.np;
    Wgrad4Args w{};
    w.g4 = g4;
    w.a3 = a3;
    w.partial = partial;
    w.g = g;
    w.rows = nf * g.nt;
    // nblocks is two per SM (the 3x3 layers' partial rows); six per SM here, whose rows of 289
    // floats fit the same buffer of nblocks x (32 x 9 x 32 + 32) floats
    static_assert(kW4BlocksPerSm * 289 <= 2 * (32 * 9 * 32 + 32), "layer-4 partial rows fit the buffer");
    const int nb4 = nblocks / 2 * kW4BlocksPerSm;
    wgrad4_kernel<<<nb4, 32 * kW4Warps, 0, st>>>(w);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    reduce4_kernel<<<(289 + kRedCols - 1) / kRedCols, kRedCols * kRed4Rows, 0, st>>>(partial, nb4, grad + SBS_NN_W4,
                                                                                  grad + SBS_NN_B4);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    Dgrad4Args d{};
    d.g4 = g4;
    d.w4 = p.w4;
    d.y3 = y3;
    d.g3 = g3;
    d.g = g;
    d.cells = cells;
    d.act = p.act;
    dgrad4_kernel<<<(unsigned)((cells + 255) / 256), 256, 0, st>>>(d);
    return cudaGetLastError();
}

cudaError_t adam(float *theta, float *m, float *v, const float *grad, float lr, float b1, float b2, float eps,
                 int step, cudaStream_t st) {
    const float c1 = (float)(1.0 / (1.0 - std::pow((double)b1, step)));
    const float c2 = (float)(1.0 / (1.0 - std::pow((double)b2, step)));
    adam_kernel<<<(SBS_NN_PARAMS + 255) / 256, 256, 0, st>>>(theta, m, v, grad, SBS_NN_PARAMS, lr, b1, b2, eps, c1,
                                                             c2);
    return cudaGetLastError();
}

cudaError_t pack(const float *theta, const Packed &p, cudaStream_t st) {
    pack_kernel<<<(32 * 288 + 255) / 256, 256, 0, st>>>(theta, p);
    return cudaGetLastError();
}

cudaError_t apply(const float *h, size_t pitch_in, const float *y, float kout, int nt, int np, float *out,
                  size_t pitch_out, cudaStream_t st) {
    dim3 grid((np + 127) / 128, nt);
    apply_kernel<<<grid, 128, 0, st>>>(h, pitch_in, y, kout, nt, np, out, pitch_out);
    return cudaGetLastError();
}

cudaError_t targets(const float *const *h0, const float *const *h1, const float *kout, int nf, int nt, int np,
                    float *target, cudaStream_t st) {
    TargetArgs t{};
    for (int b = 0; b < nf; ++b) {
        t.h0[b] = h0[b];
        t.h1[b] = h1[b];
        t.kout[b] = kout[b];
    }
    dim3 grid((np + 127) / 128, nt, nf);
    target_kernel<<<grid, 128, 0, st>>>(t, nt, np, target);
    return cudaGetLastError();
}

cudaError_t masked_error(const float *a, size_t pa, const float *b, size_t pb, const GridTab &g, unsigned *out2,
                         cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(out2, 0, 2 * sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)std::min(8, (g.np + 255) / 256), g.nt);
    masked_err_kernel<<<grid, 256, 0, st>>>(a, pa, b, pb, g.rows, g.nt, g.np, out2);
    return cudaGetLastError();
}

}  // namespace nn
}  // namespace sbs
