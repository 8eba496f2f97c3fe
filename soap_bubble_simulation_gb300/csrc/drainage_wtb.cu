// Temporally blocked drainage step for the GPUDrainageSimulator semantics (drainage.wgsl).
//
// One launch advances the field by K steps with one read and one write of h and Gamma, instead of
// K reads and writes. The pole rows never change in these semantics, so K steps of the 5-point
// stencil only depend on a cone K cells wide around each output cell, which one warp can hold:
//
//  * phi: a warp loads 128 consecutive cells (32 lanes x float4) but keeps only the middle 120.
//    Each level spoils one more cell at each warp edge (the neighbour beyond the warp is not
//    available), so for K <= 4 only lanes 0 and 31 go bad; warps therefore start 120 cells apart
//    and the loads wrap around the row end (row length a multiple of 4).
//  * theta: a thread sweeps its strip top to bottom as a time-skewed pipeline. After loading row t
//    (level 0) it computes level l of row t - l from a three-row window of level l - 1, for
//    l = 1..K, and stores level K. Each level's windows rotate through three register slots whose
//    index is fixed at compile time (the row loop is unrolled by three), so nothing is copied.
//
// The per-cell arithmetic is wgsl_cell(), the same function the single-step kernel uses, so K
// launches of one and one launch of this give bit-identical fields.
#include <cuda_runtime.h>

#include "cell.cuh"
#include "sbs_internal.h"
#include "wtb.cuh"

namespace sbs {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kWarpsPerBlock = 4;
constexpr int kSegStride = 120;  // output cells per warp

__device__ __forceinline__ double wtb_block_sum(double v, double *smem) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    if (lane == 0) smem[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < nw; ++i) t += smem[i];
    __syncthreads();
    return t;
}

// At least three blocks per SM: caps the K = 4 pipeline at 168 registers (164-168 used, 12 warps
// per SM). Left to itself the compiler allocates 188-198 registers, two blocks per SM fit, and the
// 2048 x 4096 step takes 14.84 us against 13.84 (median of 7 x 2048 steps, measured A/B/A in one
// process each); four blocks (128 registers, spills) 15.49.
constexpr int kMinBlocksPerSm = 3;

// CAU: the launch also writes the caustic map of its result (wtb_iter); K must be kWtbCausticK.
template <int K, bool VOL, bool MAR, bool CAU = false>
__global__ void __launch_bounds__(kWarpsPerBlock * 32, kMinBlocksPerSm) wtb_wgsl_kernel(const StepArgs a) {
    constexpr int E = CAU ? 1 : 0;  // extra final rows on each side of the strip
    __shared__ double s_red[32];
    __shared__ int s_last;
    extern __shared__ float4 s_co[];  // coefficient rows [r0 - K - E, r1 + K + E) of this strip
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int np = a.np;
    const int seg = blockIdx.x * kWarpsPerBlock + warp;
    const int out0 = seg * kSegStride;
    const int c_unwrapped = out0 - 4 + 4 * lane;
    const int col = ((c_unwrapped % np) + np) % np;

    Wtb w;
    w.hin = a.hin + col;
    w.cin = a.cin + col;
    w.hout = a.hout + col;
    w.cout = a.cout + col;
    w.nt = a.nt;
    w.pitch = a.pitch;
    w.r0 = 1 + blockIdx.y * a.rb;
    w.r1 = min(w.r0 + a.rb, a.nt - 1);
    w.store = lane >= 1 && lane <= 30 && c_unwrapped < np;
    w.b = a.b;
    w.DR2 = a.DR2;
    w.DsR2 = a.DsR2;
    w.Gt = a.Gt;
    w.M = a.M;
    w.dt = a.dt;
    w.crit = a.crit;
    w.vol_w = a.vol_w;
    w.cau_out = CAU ? a.cau_out + col : nullptr;
    w.cau_stride = np;
    w.cau_j0 = w.r0 == 1 ? 0 : w.r0;
    w.cau_j1 = w.r1 == a.nt - 1 ? a.nt : w.r1;
    w.cau_focal = a.cau_focal;
    w.cau_scale = a.cau_scale;
    w.cau_sharp = a.cau_sharp;
    w.cau_branch = a.cau_branch;
    w.sco_base = w.r0 - K - E;
    w.sco = s_co;
    for (int i = threadIdx.x; i < a.rb + 2 * (K + E); i += blockDim.x) {
        const int r = w.sco_base + i;
        s_co[i] = (r >= 0 && r < a.nt) ? __ldg(a.rows + r) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();

    float4 wh[K][3], wc[K][3];
#pragma unroll
    for (int l = 0; l < K; ++l)
#pragma unroll
        for (int s = 0; s < 3; ++s) {
            wh[l][s] = make_float4(0.f, 0.f, 0.f, 0.f);
            wc[l][s] = wh[l][s];
        }

    float4 wk[3];  // the last three final rows (CAU)
#pragma unroll
    for (int s = 0; s < 3; ++s) wk[s] = make_float4(0.f, 0.f, 0.f, 0.f);

    double vacc = 0.0;
    const int t0 = w.r0 - K - E, t1 = w.r1 + K + E;  // level-0 rows [t0, t1)
    float4 ph = make_float4(0.f, 0.f, 0.f, 0.f), pc = ph;
    if (SBS_WTB_PREFETCH && t0 >= 0) {
        ph = __ldg(reinterpret_cast<const float4 *>(w.hin + (size_t)t0 * w.pitch));
        pc = __ldg(reinterpret_cast<const float4 *>(w.cin + (size_t)t0 * w.pitch));
    }
    // iterations t in [ts, te) are steady (wtb_iter): every level's row t - l inside [r0 - (K - l),
    // r1 + (K - l)) and in 1..nt-2, the final row t - K in [r0, r1), the prefetched row t + 1 < nt
    const int ts = w.r0 + K, te = min(w.r1 + K, a.nt - 1);
    for (int t = t0; t < t1; t += 3) {
        if (!CAU && t >= ts && t + 2 < te) {
            wtb_iter<K, 0, VOL, MAR, false, false, true>(w, t, wh, wc, ph, pc, vacc, wk);
            wtb_iter<K, 1, VOL, MAR, false, false, true>(w, t + 1, wh, wc, ph, pc, vacc, wk);
            wtb_iter<K, 2, VOL, MAR, false, false, true>(w, t + 2, wh, wc, ph, pc, vacc, wk);
            continue;
        }
        wtb_iter<K, 0, VOL, MAR, false, CAU>(w, t, wh, wc, ph, pc, vacc, wk);
        if (t + 1 < t1) wtb_iter<K, 1, VOL, MAR, false, CAU>(w, t + 1, wh, wc, ph, pc, vacc, wk);
        if (t + 2 < t1) wtb_iter<K, 2, VOL, MAR, false, CAU>(w, t + 2, wh, wc, ph, pc, vacc, wk);
    }

    if (VOL) {
        const double s = wtb_block_sum(vacc, s_red);
        const unsigned nblocks = gridDim.x * gridDim.y;
        const unsigned bid = blockIdx.y * gridDim.x + blockIdx.x;
        if (threadIdx.x == 0) {
            a.vol_partials[bid] = s;
            __threadfence();
            const unsigned tk = atomicAdd(a.vol_counter, 1u);
            s_last = (tk == nblocks - 1);
        }
        __syncthreads();
        if (s_last) {
            __threadfence();
            double tot = 0.0;
            for (unsigned i = threadIdx.x; i < nblocks; i += blockDim.x) tot += __ldcg(a.vol_partials + i);
            double pole = 0.0;  // the frozen pole rows of the input
            for (int j = threadIdx.x; j < np; j += blockDim.x) {
                pole += (double)__ldg(a.hin + j) * __ldg(a.vol_w);
                pole += (double)__ldg(a.hin + (size_t)(a.nt - 1) * a.pitch + j) * __ldg(a.vol_w + a.nt - 1);
            }
            tot = wtb_block_sum(tot, s_red);
            pole = wtb_block_sum(pole, s_red);
            if (threadIdx.x == 0) {
                const unsigned idx = *a.vol_index;
                a.vol_out[idx] = tot + pole;
                *a.vol_index = idx + 1;
                *a.vol_counter = 0u;
                __threadfence();
            }
        }
    }
}

template <int K>
const void *wtb_fn(bool vol, bool mar) {
    if (vol) return mar ? (const void *)wtb_wgsl_kernel<K, true, true> : (const void *)wtb_wgsl_kernel<K, true, false>;
    return mar ? (const void *)wtb_wgsl_kernel<K, false, true> : (const void *)wtb_wgsl_kernel<K, false, false>;
}

const void *wtb_kernel(int K, bool vol, bool mar, bool cau = false) {
    if (cau) {
        if (K != kWtbCausticK || vol) return nullptr;
        return mar ? (const void *)wtb_wgsl_kernel<kWtbCausticK, false, true, true>
                   : (const void *)wtb_wgsl_kernel<kWtbCausticK, false, false, true>;
    }
    switch (K) {
        case 2:
            return wtb_fn<2>(vol, mar);
        case 3:
            return wtb_fn<3>(vol, mar);
        case 4:
            return wtb_fn<4>(vol, mar);
        default:
            return nullptr;
    }
}

}  // namespace

bool wtb_supported(int nt, int np) { return np % 4 == 0 && np >= 8 && nt >= 3; }

StepGeom wtb_geometry(int nt, int np, int K) {
    StepGeom g{};
    const int segs = (np + kSegStride - 1) / kSegStride;
    g.wx = kWarpsPerBlock;
    g.nbx = (segs + kWarpsPerBlock - 1) / kWarpsPerBlock;
    int dev = 0, sms = 148, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, wtb_kernel(K, false, false), kWarpsPerBlock * 32,
                                                  sizeof(float4) * 64);
    if (per_sm < 1) per_sm = 1;
    const int resident = per_sm * sms;
    int strips = resident / g.nbx;
    if (strips < 1) strips = 1;
    int rb = (nt - 2 + strips - 1) / strips;
    if (rb < 4 * K) rb = 4 * K;
    g.rb = rb;
    g.nby = (nt - 2 + rb - 1) / rb;
    return g;
}

cudaError_t launch_wtb(int K, const StepArgs &a, const StepGeom &g, cudaStream_t s) {
    const bool cau = a.cau_out != nullptr;
    const void *fn = wtb_kernel(K, a.vol_w != nullptr, a.marangoni != 0, cau);
    if (fn == nullptr) return cudaErrorInvalidValue;
    dim3 grid(g.nbx, g.nby), block(kWarpsPerBlock * 32);
    void *args[] = {(void *)&a};
    return cudaLaunchKernel(fn, grid, block, args, sizeof(float4) * (g.rb + 2 * (K + (cau ? 1 : 0))), s);
}

}  // namespace sbs
