// The surrogate's 3x3 convolutions for training (include/sbs_nn.h) on the tcgen05 tensor cores:
// the forward pass of layers 1-3 (pre-activations and activations kept for the backward pass) and
// the input gradient of layers 2-3 (the transposed convolution times the activation's derivative).
//
// Work item: 16 output rows of one 128-cell column segment of one field; one CTA (8 warps) per
// item walks it top to bottom. Input rows are staged through a ring of five row buffers by
// per-thread cp.async copies, three rows ahead of the row whose MMAs are issued, as planes of 8 channels with 16 bytes per cell (the K-major, no-swizzle layout of
// an MMA's A operand: 8-cell core matrices 128 B apart, planes a plane apart), 130 cells wide (one
// halo cell each side, phi wrapped). The dx = -1 / 0 / +1 taps read the same buffer at start
// addresses 16 bytes apart, so there is no im2col copy. One output row is 9 taps x CIN/16 MMAs of
// M = 128 cells x N = 32 channels x K = 16 into a 32-column TMEM accumulator; two accumulators
// alternate, so the epilogue of row r - 1 (tcgen05.ld, bias and activation, or the activation's
// derivative, and the stores) runs while the MMAs of row r execute. The weights are staged once per
// CTA as the B operand (32 rows of 16-byte K chunks).
//
// theta: the forward pass reflects at the poles (source row -1 is row 1, row nt is row nt-2); the
// transposed pass reads the gradient at row i - dy, skips rows outside the grid, and adds the
// reflected sources (row 1 also receives output row 0's dy = -1 taps, row nt-2 output row nt-1's
// dy = +1 taps). Every source a row needs lies in rows r-1..r+1, which the ring holds.
//
// Every mbarrier wait is bounded (sbs_set_wait_limit); the block votes on the outcome, so a timeout
// ends the work of all its threads together, records the error and still releases the TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "nn.cuh"
#include "nn_kernels.h"
#include "sbs_internal.h"
#include "tc.cuh"

namespace sbs {
namespace nn {
namespace {

constexpr int kTcThreads = 256;                 // 8 warps: two per TMEM lane quarter (16 channels each)
constexpr int kTcCells = 128;                   // output cells per segment (MMA M)
constexpr int kTcStage = kTcCells + 2;          // staged cells per input row
constexpr uint32_t kTcPlane = kTcStage * 16;    // one 8-channel plane: 2080 B
constexpr int kTcRing = 5;                      // input row buffers: rows r-1..r+1 read, r+2, r+3 landing
constexpr int kTcRows = 16;                     // output rows per work item
constexpr uint32_t kTcId = tc::idesc_bf16_m128(32);

constexpr int kTcYS = 36;  // floats per cell in the FP32 tiles (32 + 4: conflict-free 16 B accesses)
constexpr int kTcAS = 40;  // BF16 values per cell in the output tile (32 + 8)

template <int CIN, bool BWD>
struct TcLayout {
    static constexpr int PL = CIN / 8;                   // planes per input row
    static constexpr uint32_t ROWB = PL * kTcPlane;      // bytes per staged row
    static constexpr int KC = CIN / 16;                  // K16 steps per tap
    static constexpr uint32_t BCH = 32 * 16;             // one 8-element K chunk of B (32 rows)
    static constexpr uint32_t BSTEP = 2 * BCH;           // one K16 step
    static constexpr uint32_t YT = kTcCells * kTcYS * 4; // one FP32 row tile
    static constexpr uint32_t OFF_B = kTcRing * ROWB;
    static constexpr uint32_t OFF_A = OFF_B + 9 * KC * BSTEP;       // BF16 output tile
    static constexpr uint32_t OFF_Y = OFF_A + kTcCells * kTcAS * 2; // forward: FP32 pre-activations out;
                                                                    // transposed: two prefetched y rows
    static constexpr uint32_t OFF_BIAS = OFF_Y + (BWD ? 2 : 1) * YT;
    static constexpr uint32_t OFF_BAR = OFF_BIAS + 32 * 4;
    static constexpr uint32_t OFF_MISC = OFF_BAR + 16;   // TMEM base
    static constexpr uint32_t SMEM = OFF_MISC + 16;
};

struct TcConvArgs {
    const bf16 *in;       // [cells][CIN]: activations below (forward) or this layer's gradient
    const bf16 *w;        // packed BF16: forward [oc][tap*CIN + ic], transposed [ic][tap*32 + oc]
    const float *bias;    // forward: 32 biases
    const float *yprev;   // transposed: pre-activations of the layer below [cells][32]
    float *yout;          // forward: pre-activations [cells][32]
    bf16 *aout;           // forward: activations; transposed: gradient of the layer below
    unsigned *err;        // bit 1: a wait timed out
    long long wait_cycles;
    int nt, np, segs, nrb, nitems;
    int act;              // SBS_NN_ACT_*
    int stall;            // timeout test: issue neither MMAs nor commits
};

template <int CIN, bool BWD>
__global__ void __launch_bounds__(kTcThreads) tc_conv_kernel(const TcConvArgs a) {
    using Lay = TcLayout<CIN, BWD>;
    extern __shared__ __align__(128) uint8_t smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t sb = tc::smem_u32(smem);
    const uint32_t bar0 = sb + Lay::OFF_BAR;  // accumulator b completes on bar0 + 8 b
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(smem + Lay::OFF_MISC);
    float *s_bias = reinterpret_cast<float *>(smem + Lay::OFF_BIAS);
    float *s_y = reinterpret_cast<float *>(smem + Lay::OFF_Y);  // [cells][kTcYS] (x2 transposed)
    bf16 *s_a = reinterpret_cast<bf16 *>(smem + Lay::OFF_A);    // [cells][kTcAS]
    const int nt = a.nt, np = a.np;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(tc::smem_u32(s_tmem)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        tc::mbar_init(bar0, 1);
        tc::mbar_init(bar0 + 8, 1);
        tc::fence_mbar_init();
    }
    // B: element (tap t, K step kc, chunk ch, row n, e) = w[n][t * CIN + kc * 16 + ch * 8 + e]
    constexpr int KP = 9 * CIN;
    for (int g = tid; g < 9 * Lay::KC * 2 * 32; g += kTcThreads) {
        const int n = g % 32, ch = (g / 32) % 2, tk = g / 64;
        const int t = tk / Lay::KC, kc = tk % Lay::KC;
        *reinterpret_cast<uint4 *>(smem + Lay::OFF_B + (uint32_t)g * 16) =
            *reinterpret_cast<const uint4 *>(a.w + (size_t)n * KP + t * CIN + kc * 16 + ch * 8);
    }
    if (!BWD && tid < 32) s_bias[tid] = a.bias[tid];
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *s_tmem;
    const int quarter = warp & 3, half = warp >> 2;  // TMEM lanes 32 quarter.., channels 16 half..
    const uint32_t tl = tmem + ((uint32_t)(quarter * 32) << 16) + 16u * half;

    // descriptors: A at the start of the ring (rows, shifts and planes are added in 16-byte units),
    // B per (tap, K step), built once
    const uint64_t a_desc0 = tc::make_desc(sb, kTcPlane, 128);
    uint64_t b_desc[9 * Lay::KC];
#pragma unroll
    for (int i = 0; i < 9 * Lay::KC; ++i) b_desc[i] = tc::make_desc(sb + Lay::OFF_B + (uint32_t)i * Lay::BSTEP, Lay::BCH, 128);
    uint32_t issued[2] = {0u, 0u};  // commits on each barrier so far (block-uniform)
    bool failed = false;

    for (int item = blockIdx.x; item < a.nitems && !failed; item += gridDim.x) {
        const int rb = item % a.nrb, seg = (item / a.nrb) % a.segs, f = item / (a.nrb * a.segs);
        const int r0 = rb * kTcRows, r1 = min(nt, r0 + kTcRows);
        const int j0 = seg * kTcCells;
        const bf16 *base = a.in + (size_t)f * nt * np * CIN;
        const size_t cell0 = (size_t)f * nt * np;

        auto stage = [&](int r) {  // input row r into buffer r mod kTcRing (all threads)
            uint8_t *dst = smem + (r % kTcRing) * Lay::ROWB;
            const bf16 *rowp = base + (size_t)r * np * CIN;
            for (int e = tid; e < kTcStage * Lay::PL; e += kTcThreads) {
                const int q = e / Lay::PL, p = e % Lay::PL;
                int col = (j0 - 1 + q) % np;
                col = col < 0 ? col + np : col;
                tc::cp_async16(dst + p * kTcPlane + q * 16, rowp + (size_t)col * CIN + p * 8);
            }
        };
        auto issue = [&](int r, uint32_t dacc) {  // the MMAs of output row r (one thread)
            // buffers of rows r - 1, r, r + 1 in 16-byte units of the A descriptor's address field
            const int bc = r % kTcRing;
            const uint64_t a_up = a_desc0 + (uint64_t)(((bc + kTcRing - 1) % kTcRing) * (Lay::ROWB >> 4));
            const uint64_t a_mid = a_desc0 + (uint64_t)(bc * (Lay::ROWB >> 4));
            const uint64_t a_dn = a_desc0 + (uint64_t)(((bc + 1) % kTcRing) * (Lay::ROWB >> 4));
            bool acc = false;
            auto tap = [&](uint64_t arow, int shift, int t) {
#pragma unroll
                for (int kc = 0; kc < Lay::KC; ++kc) {
                    tc::mma_bf16(dacc, arow + (uint64_t)(1 + shift + kc * 2 * (kTcPlane >> 4)), b_desc[t * Lay::KC + kc],
                                 kTcId, acc);
                    acc = true;
                }
            };
#pragma unroll
            for (int t = 0; t < 9; ++t) {
                const int dy = t / 3 - 1, dx = t % 3 - 1;
                if (!BWD) {  // source row refl(r + dy)
                    const uint64_t arow = dy == 0 ? a_mid : dy < 0 ? (r == 0 ? a_dn : a_up) : (r == nt - 1 ? a_up : a_dn);
                    tap(arow, dx, t);
                } else {  // source row r - dy when inside the grid, plus the reflected sources
                    if (dy == 0) tap(a_mid, -dx, t);
                    if (dy < 0 && r + 1 < nt) tap(a_dn, -dx, t);
                    if (dy > 0 && r >= 1) tap(a_up, -dx, t);
                    if (r == 1 && dy < 0) tap(a_up, -dx, t);        // row 0
                    if (r == nt - 2 && dy > 0) tap(a_dn, -dx, t);   // row nt - 1
                }
            }
        };
        const int nvalid = min(kTcCells, np - j0);  // cells of the segment inside the grid
        // transposed: pre-activations of output row r into tile (r - r0) & 1, 16 B per copy
        auto prefetch_y = [&](int r) {
            float *dst = s_y + ((r - r0) & 1) * kTcCells * kTcYS;
            const float *src = a.yprev + (cell0 + (size_t)r * np + j0) * 32;
            for (int e = tid; e < nvalid * 8; e += kTcThreads)
                tc::cp_async16(dst + (e >> 3) * kTcYS + (e & 7) * 4, src + (size_t)e * 4);
        };
        // output row r from accumulator columns col..col+31: each thread its cell's 16 channels into
        // the shared tiles, then the block copies the row out in contiguous 16-byte pieces
        auto epilogue = [&](int r, uint32_t col) {
            uint32_t v[16];
            tc::tld16(tl + col, v);
            tc::wait_ld();
#pragma unroll
            for (int k = 0; k < 16; ++k) tc::pin(v[k]);
            const int m = quarter * 32 + lane, c0 = 16 * half;
            uint4 *ap = reinterpret_cast<uint4 *>(s_a + m * kTcAS + c0);
            if (!BWD) {
                float y[16];
#pragma unroll
                for (int n = 0; n < 16; ++n) y[n] = __fadd_rn(__uint_as_float(v[n]), s_bias[c0 + n]);
                float4 *yp = reinterpret_cast<float4 *>(s_y + m * kTcYS + c0);
#pragma unroll
                for (int k = 0; k < 4; ++k) yp[k] = make_float4(y[4 * k], y[4 * k + 1], y[4 * k + 2], y[4 * k + 3]);
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    uint32_t w4[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const float2 g = act2(a.act, make_float2(y[8 * k + 2 * e], y[8 * k + 2 * e + 1]));
                        w4[e] = pack2(g.x, g.y);
                    }
                    ap[k] = make_uint4(w4[0], w4[1], w4[2], w4[3]);
                }
            } else {
                const float4 *yp =
                    reinterpret_cast<const float4 *>(s_y + ((r - r0) & 1) * kTcCells * kTcYS + m * kTcYS + c0);
#pragma unroll
                for (int k = 0; k < 2; ++k) {
                    const float4 u0 = yp[2 * k], u1 = yp[2 * k + 1];
                    const float y[8] = {u0.x, u0.y, u0.z, u0.w, u1.x, u1.y, u1.z, u1.w};
                    uint32_t w4[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int n = 8 * k + 2 * e;
                        const float2 g = __fmul2_rn(make_float2(__uint_as_float(v[n]), __uint_as_float(v[n + 1])),
                                                    act_grad2(a.act, make_float2(y[2 * e], y[2 * e + 1])));
                        w4[e] = pack2(g.x, g.y);
                    }
                    ap[k] = make_uint4(w4[0], w4[1], w4[2], w4[3]);
                }
            }
            __syncthreads();
            const size_t cb = cell0 + (size_t)r * np + j0;
            uint4 *ga = reinterpret_cast<uint4 *>(a.aout + cb * 32);
            for (int e = tid; e < nvalid * 4; e += kTcThreads)
                ga[e] = *reinterpret_cast<const uint4 *>(s_a + (e >> 2) * kTcAS + (e & 3) * 8);
            if (!BWD) {
                float4 *gy = reinterpret_cast<float4 *>(a.yout + cb * 32);
                for (int e = tid; e < nvalid * 8; e += kTcThreads)
                    gy[e] = *reinterpret_cast<const float4 *>(s_y + (e >> 3) * kTcYS + (e & 7) * 4);
            }
        };
        // block-uniform: every thread waits for the same completion; the block agrees on the outcome
        auto wait_acc = [&](int b) -> bool {
            const bool ok = tc::mbar_wait_n(bar0 + 8u * b, issued[b] - 1u, a.wait_cycles);
            return __syncthreads_or(ok ? 0 : 1) == 0;
        };

        const int rlast = min(nt - 1, r1);  // the last input row the item reads
        for (int r = max(0, r0 - 1); r <= min(rlast, r0 + 2); ++r) stage(r);
        if (BWD) prefetch_y(r0);
        tc::cp_async_commit();
        tc::cp_async_wait_all();
        tc::fence_async_smem();
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
        for (int r = r0; r < r1; ++r) {
            const int b = (r - r0) & 1;
            if (warp == 0 && !a.stall) {
                if (tc::elect_one()) {
                    issue(r, tmem + 32u * b);
                    tc::commit(bar0 + 8u * b);
                }
                __syncwarp();
            }
            ++issued[b];
            if (r > r0) {
                if (!wait_acc(b ^ 1)) {
                    failed = true;
                    break;
                }
                tc::fence_after();
            }
            // row r + 3 replaces row r - 2, whose last reader (output row r - 1) has completed; it is
            // needed one iteration later, so only row r + 2 must have landed at this iteration's end
            // (one copy group per iteration, possibly empty)
            if (r + 3 <= rlast) stage(r + 3);
            if (r > r0) epilogue(r - 1, 32u * (b ^ 1));
            // transposed: y of row r + 1 into the tile the epilogue above has finished reading
            if (BWD && r + 1 < r1) prefetch_y(r + 1);
            tc::cp_async_commit();
            asm volatile("cp.async.wait_group 1;\n" ::: "memory");
            tc::fence_async_smem();
            tc::fence_before();
            __syncthreads();
            tc::fence_after();
        }
        if (failed) break;
        if (!wait_acc((r1 - 1 - r0) & 1)) {
            failed = true;
            break;
        }
        tc::fence_after();
        epilogue(r1 - 1, 32u * ((r1 - 1 - r0) & 1));
        tc::fence_before();
        __syncthreads();
        tc::fence_after();
    }
    if (failed) {
        // nothing may still write the accumulators when the columns are released: wait (bounded)
        // for the last commit on each barrier
        if (tid == 0) {
            atomicOr(a.err, 2u);
            if (!a.stall)
                for (int b = 0; b < 2; ++b)
                    if (issued[b]) tc::mbar_wait_n(bar0 + 8u * b, issued[b] - 1u, a.wait_cycles);
        }
    }
    tc::cp_async_wait_all();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem));
}

// ------------------------------------------------------------------------------------------------
// Weight gradients of a 3x3 layer: dW[tap][oc][ic] = sum over cells of g[cell][oc] x[src(cell, tap)][ic]
// (src: theta reflected, phi wrapped) and db[oc] = sum of g[cell][oc], as GEMMs over the cells.
// A chunk is 64 cells of one output row. With the cells as K, an 8-channel plane with 16 B per cell is
// an MN-major operand (8 channels x 8 cells per 128-byte core matrix), so the dx taps are start
// offsets of 16 B. One MMA group per dx: M = 128 rows = (dy, ic) over the 3 x CIN/8 planes of x,
// a plane of ones (its rows of D are db) and padding, N = 32 output channels (g, staged the same
// way), K = 16 cells; D[dx] accumulates over all of the CTA's chunks.
//
// Roles: one thread of warp 0 stages chunks through a ring of four stages with TMA (one box per
// plane and source row: 66 cells of x from j0 - 1, 64 cells of g; cells outside the row arrive as
// zeros, which also zeroes g past a ragged row end); warp 1 writes the two cells of the phi seam
// (x[np - 1] left of cell 0, x[0] right of cell np - 1) over those zeros once a chunk has landed,
// and one of its threads issues the chunk's MMAs and commits them to the stage's empty barrier.
// Every wait is bounded; after a timeout the CTA still waits (bounded) for the copies and MMAs it
// started before it releases the TMEM. The CTA's sums go to one partial row, reduced over the CTAs
// in a fixed order afterwards.
constexpr int kWgCells = 64;                      // cells per chunk
constexpr int kWgStage = kWgCells + 2;            // staged x cells per plane (one halo cell each side)
constexpr uint32_t kWgPlaneA = 1152;              // x plane: 66 x 16 B, padded to 128-byte TMA alignment
constexpr uint32_t kWgPlaneB = kWgCells * 16;     // g plane: 1024 B
constexpr int kWgStages = 4;
constexpr int kWgThreads = 128;                   // 4 warps: one per TMEM lane quarter in the epilogue

template <int CIN>
struct WgLayout {
    static constexpr int PL = CIN / 8;                // planes per x row
    static constexpr int ONES = 3 * PL;               // the plane of ones
    static constexpr uint32_t ABUF = 16 * kWgPlaneA;  // 16 planes = M 128
    static constexpr uint32_t BBUF = 4 * kWgPlaneB;
    static constexpr uint32_t OFF_B = kWgStages * ABUF;
    static constexpr uint32_t OFF_BAR = OFF_B + kWgStages * BBUF;  // full[stages], empty[stages]
    static constexpr uint32_t OFF_MISC = OFF_BAR + 16 * kWgStages;
    static constexpr uint32_t SMEM = OFF_MISC + 16 + 128;           // + slack to align the base to 128 B
    static constexpr uint32_t TX = 3 * PL * kWgStage * 16 + 4 * kWgPlaneB;  // bytes of one chunk's boxes
};

struct TcWgradArgs {
    CUtensorMap tx;  // x as [rows][np][CIN/8][8], box 8 x 1 x 66 x 1
    CUtensorMap tg;  // g as [rows][np][4][8], box 8 x 1 x 64 x 1
    const bf16 *x;   // [cells][CIN]: the layer's input (the seam cells)
    float *partial;  // [gridDim.x][32 * 9 * CIN + 32]
    unsigned *err;
    long long wait_cycles;
    int nt, np, cps, nchunks;  // chunks per row, chunks in all
    int stall;
};

template <int CIN>
__global__ void __launch_bounds__(kWgThreads) tc_wgrad_kernel(const __grid_constant__ TcWgradArgs a) {
    using Lay = WgLayout<CIN>;
    static_assert(3 * Lay::PL + 1 <= 16, "the dy x channel planes and the ones fit one M = 128 group");
    extern __shared__ __align__(128) uint8_t smem_raw[];
    uint8_t *smem = smem_raw + ((128u - (tc::smem_u32(smem_raw) & 127u)) & 127u);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t sb = tc::smem_u32(smem);
    const uint32_t full0 = sb + Lay::OFF_BAR, empty0 = full0 + 8u * kWgStages;  // stage s: + 8 s
    volatile uint32_t *s_misc = reinterpret_cast<volatile uint32_t *>(smem + Lay::OFF_MISC);
    // s_misc: [0] TMEM base, [1] failed, [2] chunks whose copies the MMA warp has seen land
    const int nt = a.nt, np = a.np;
    constexpr uint32_t kId = tc::idesc_bf16_m128(32) | (1u << 15) | (1u << 16);  // A and B MN-major

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(
            tc::smem_u32(const_cast<uint32_t *>(s_misc))));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 32) {
        for (int s = 0; s < kWgStages; ++s) {
            tc::mbar_init(full0 + 8u * s, 1);
            tc::mbar_init(empty0 + 8u * s, 1);
        }
        tc::fence_mbar_init();
        s_misc[1] = 0u;
        s_misc[2] = 0u;
    }
    for (int e = tid; e < kWgStages * (int)(kWgPlaneA / 16); e += kWgThreads) {  // bf16 1.0 pairs
        const int s = e / (int)(kWgPlaneA / 16), q = e % (int)(kWgPlaneA / 16);
        *reinterpret_cast<uint4 *>(smem + s * Lay::ABUF + Lay::ONES * kWgPlaneA + q * 16) =
            make_uint4(0x3F803F80u, 0x3F803F80u, 0x3F803F80u, 0x3F803F80u);
    }
    tc::fence_async_smem();
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = s_misc[0];

    const int nmine = a.nchunks > (int)blockIdx.x ? (a.nchunks - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    // chunk k of this CTA: first row of its field, row i in the field, first cell j0
    auto where = [&](int k, int &fr, int &i, int &j0) {
        const int c = (int)blockIdx.x + k * (int)gridDim.x;
        const int row = c / a.cps;
        i = row % nt;
        fr = row - i;
        j0 = (c % a.cps) * kWgCells;
    };
    auto reflect = [&](int r) { return r < 0 ? 1 : (r >= nt ? nt - 2 : r); };

    int produced = 0;  // producer thread
    if (warp == 0) {
        if (lane == 0) {
            for (int k = 0; k < nmine; ++k) {
                const int s = k % kWgStages;
                if (s_misc[1]) break;
                if (k >= kWgStages && !tc::mbar_wait_n(empty0 + 8u * s, (uint32_t)(k / kWgStages - 1), a.wait_cycles)) {
                    s_misc[1] = 1u;
                    break;
                }
                int fr, i, j0;
                where(k, fr, i, j0);
                const uint32_t bar = full0 + 8u * s;
                tc::mbar_arrive_expect_tx(bar, Lay::TX);
                for (int dyi = 0; dyi < 3; ++dyi) {
                    const int src = fr + reflect(i + dyi - 1);
                    for (int p = 0; p < Lay::PL; ++p)
                        tc::tma_load_4d(sb + s * Lay::ABUF + (dyi * Lay::PL + p) * kWgPlaneA, &a.tx, 0, p, j0 - 1, src,
                                        bar);
                }
                for (int p = 0; p < 4; ++p)
                    tc::tma_load_4d(sb + Lay::OFF_B + s * Lay::BBUF + p * kWgPlaneB, &a.tg, 0, p, j0, fr + i, bar);
                produced = k + 1;
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        const uint64_t a_desc0 = tc::make_desc(sb, 128, kWgPlaneA);
        const uint64_t b_desc0 = tc::make_desc(sb + Lay::OFF_B, 128, kWgPlaneB);
        // seam cells: lane L < 6 PL takes side L / (3 PL) (0: left of cell 0, 1: right of cell np - 1)
        // and plane P = L % (3 PL) = (dy + 1) PL + p
        const int side = lane / (3 * Lay::PL), P = lane % (3 * Lay::PL);
        int issued = 0, seen = 0;
        for (int k = 0; k < nmine; ++k) {
            const int s = k % kWgStages;
            int fr, i, j0;
            where(k, fr, i, j0);
            const int n = min(kWgCells, np - j0);
            bool mine = false;
            uint4 hv = make_uint4(0u, 0u, 0u, 0u);
            uint32_t hoff = 0;
            if (side < 2 && ((side == 0 && j0 == 0) || (side == 1 && j0 + n == np))) {
                const int src = fr + reflect(i + P / Lay::PL - 1);
                hv = __ldg(reinterpret_cast<const uint4 *>(a.x + ((size_t)src * np + (side ? 0 : np - 1)) * CIN +
                                                           (P % Lay::PL) * 8));
                hoff = s * Lay::ABUF + P * kWgPlaneA + (side ? n + 1 : 0) * 16;
                mine = true;
            }
            const bool ok = tc::mbar_wait_n(full0 + 8u * s, (uint32_t)(k / kWgStages), a.wait_cycles);
            if (__any_sync(0xffffffffu, !ok || s_misc[1] != 0u)) {  // one decision for the warp
                if (lane == 0) s_misc[1] = 1u;
                break;
            }
            seen = k + 1;
            if (mine) *reinterpret_cast<uint4 *>(smem + hoff) = hv;
            tc::fence_async_smem();
            __syncwarp();
            if (lane == 0 && !a.stall) {
                tc::fence_after();
                const uint64_t ab = a_desc0 + (uint64_t)((s * Lay::ABUF) >> 4);
                const uint64_t bd = b_desc0 + (uint64_t)((s * Lay::BBUF) >> 4);
#pragma unroll
                for (int kk = 0; kk < kWgCells / 16; ++kk)
#pragma unroll
                    for (int dx = 0; dx < 3; ++dx)  // start cell kk * 16 + dx of the staged plane
                        tc::mma_bf16(tmem + 32u * dx, ab + (uint64_t)(kk * 16 + dx), bd + (uint64_t)(kk * 16), kId,
                                     !(k == 0 && kk == 0));
                tc::commit(empty0 + 8u * s);
            }
            issued = a.stall ? 0 : k + 1;
            __syncwarp();
        }
        // the last commit covers every MMA of this CTA; wait for it even after a failure (the MMAs
        // read this CTA's shared memory and write its TMEM)
        if (lane == 0 && issued > 0 &&
            !tc::mbar_wait_n(empty0 + 8u * ((issued - 1) % kWgStages), (uint32_t)((issued - 1) / kWgStages),
                             a.wait_cycles))
            s_misc[1] = 1u;
        if (lane == 0) s_misc[2] = (uint32_t)seen;
        __syncwarp();
    }
    __syncthreads();
    const bool failed = s_misc[1] != 0u;
    if (failed && warp == 0 && lane == 0)  // copies still in flight land before the CTA leaves
        for (int k = (int)s_misc[2]; k < produced; ++k)
            tc::mbar_wait_n(full0 + 8u * (k % kWgStages), (uint32_t)(k / kWgStages), a.wait_cycles);
    tc::fence_after();

    float *out = a.partial + (size_t)blockIdx.x * (32 * 9 * CIN + 32);
    const bool have = nmine > 0 && !failed;  // block-uniform
    const int m = warp * 32 + lane, P = m / 8;
    for (int dx = 0; dx < 3; ++dx) {
        uint32_t v[32];
        if (have) {
            tc::tld32(tmem + ((uint32_t)(warp * 32) << 16) + 32u * dx, v);
            tc::wait_ld();
#pragma unroll
            for (int c = 0; c < 32; ++c) tc::pin(v[c]);
        }
        if (P < 3 * Lay::PL) {
            const int t = (P / Lay::PL) * 3 + dx, ic = (P % Lay::PL) * 8 + m % 8;
#pragma unroll
            for (int oc = 0; oc < 32; ++oc) out[oc * 9 * CIN + t * CIN + ic] = have ? __uint_as_float(v[oc]) : 0.f;
        } else if (dx == 1 && m == 8 * Lay::ONES) {
#pragma unroll
            for (int oc = 0; oc < 32; ++oc) out[32 * 9 * CIN + oc] = have ? __uint_as_float(v[oc]) : 0.f;
        }
    }
    if (failed && tid == 0) atomicOr(a.err, 4u);
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tmem));
}

template <int CIN, bool BWD>
cudaError_t launch_tc(TcConvArgs a, int nf, cudaStream_t st) {
    using Lay = TcLayout<CIN, BWD>;
    // set on every launch (about a microsecond): the attribute belongs to the current device's context
    cudaError_t e = cudaFuncSetAttribute(tc_conv_kernel<CIN, BWD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)Lay::SMEM);
    if (e != cudaSuccess) return e;
    a.segs = (a.np + kTcCells - 1) / kTcCells;
    a.nrb = (a.nt + kTcRows - 1) / kTcRows;
    a.nitems = nf * a.segs * a.nrb;
    const WaitConfig w = wait_config();
    a.wait_cycles = w.cycles;
    a.stall = (w.stall & SBS_STALL_TENSOR_COMMITS) ? 1 : 0;
    // one CTA per item (the items loop covers grids capped below); at most 3 CTAs share an SM by
    // shared memory (2 with 32 input channels), 192 of its 512 TMEM columns
    const int grid = a.nitems < 65535 * 16 ? a.nitems : 65535 * 16;
    tc_conv_kernel<CIN, BWD><<<grid, kTcThreads, Lay::SMEM, st>>>(a);
    return cudaGetLastError();
}

// cuTensorMapEncodeTiled from the driver (the library links only the runtime)
using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
    static const EncodeTiledFn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return (EncodeTiledFn) nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// a [rows][np][ch/8][8] BF16 tensor (cells of ch channels) in boxes of one 8-channel plane x `cells`
cudaError_t plane_map(CUtensorMap *map, const bf16 *base, int ch, int np, int rows, int cells) {
    const EncodeTiledFn enc = encode_tiled();
    if (!enc) return cudaErrorNotSupported;
    const cuuint64_t dim[4] = {8, (cuuint64_t)(ch / 8), (cuuint64_t)np, (cuuint64_t)rows};
    const cuuint64_t stride[3] = {16, (cuuint64_t)ch * 2, (cuuint64_t)np * ch * 2};
    const cuuint32_t box[4] = {8, 1, (cuuint32_t)cells, 1};
    const cuuint32_t one[4] = {1, 1, 1, 1};
    const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<bf16 *>(base), dim, stride, box, one,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

template <int CIN>
cudaError_t launch_wgrad(const TcWgradArgs &w, int nblocks, cudaStream_t st) {
    // set on every launch, like the convolution's: the attribute belongs to the current device's context
    cudaError_t e = cudaFuncSetAttribute(tc_wgrad_kernel<CIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)WgLayout<CIN>::SMEM);
    if (e != cudaSuccess) return e;
    tc_wgrad_kernel<CIN><<<nblocks, kWgThreads, WgLayout<CIN>::SMEM, st>>>(w);
    return cudaGetLastError();
}

}  // namespace

cudaError_t wgrad_tc(int cin, const bf16 *g, const bf16 *x, float *partial, int nblocks, unsigned *err, int nf, int nt,
                     int np, cudaStream_t st) {
    TcWgradArgs w{};
    const int rows = nf * nt;
    cudaError_t e = plane_map(&w.tx, x, cin, np, rows, kWgStage);
    if (e == cudaSuccess) e = plane_map(&w.tg, g, 32, np, rows, kWgCells);
    if (e != cudaSuccess) return e;
    w.x = x;
    w.partial = partial;
    w.err = err;
    w.nt = nt;
    w.np = np;
    w.cps = (np + kWgCells - 1) / kWgCells;
    w.nchunks = rows * w.cps;
    const WaitConfig wc = wait_config();
    w.wait_cycles = wc.cycles;
    w.stall = (wc.stall & SBS_STALL_TENSOR_COMMITS) ? 1 : 0;
    return cin == 16 ? launch_wgrad<16>(w, nblocks, st) : launch_wgrad<32>(w, nblocks, st);
}

cudaError_t conv_forward(int layer, const bf16 *in, const Packed &p, float *y, bf16 *a, int nf, int nt, int np,
                         cudaStream_t st) {
    TcConvArgs c{};
    c.in = in;
    c.yout = y;
    c.aout = a;
    c.nt = nt;
    c.np = np;
    c.act = p.act;
    c.err = p.err;
    if (layer == 1) {
        c.w = p.wf1;
        c.bias = p.b;
        return launch_tc<16, false>(c, nf, st);
    }
    c.w = layer == 2 ? p.wf2 : p.wf3;
    c.bias = p.b + 32 * (layer - 1);
    return launch_tc<32, false>(c, nf, st);
}

cudaError_t conv_backward_data(int layer, const bf16 *g, const Packed &p, const float *yprev, bf16 *gprev, int nf,
                               int nt, int np, cudaStream_t st) {
    TcConvArgs c{};
    c.in = g;
    c.w = layer == 2 ? p.wb2 : p.wb3;
    c.yprev = yprev;
    c.aout = gprev;
    c.act = p.act;
    c.err = p.err;
    c.nt = nt;
    c.np = np;
    return launch_tc<32, true>(c, nf, st);
}

}  // namespace nn
}  // namespace sbs
