// Temporally blocked drainage step for the DrainageSimulator semantics (drainage.rs:298-503):
// one launch advances the field by K steps of the stencil, the pole-ring means and the
// marginal-regeneration fronts, reading and writing h (and its low words) once.
//
// The interior works like the WGSL-semantics kernel (drainage_wtb.cu): a warp holds a 128-column
// window of a strip of rows (keeping the middle 120) and runs a time-skewed register pipeline,
// computing step l of row t - l once step l - 1 of rows t - l - 1 .. t - l + 1 exists.
//
// What the WGSL kernel does not have are the poles: after every step, row 0 becomes the mean of
// the whole of ring 1 and row N-1 the mean of ring N-2 (update_poles, drainage.rs:480-503), and
// the next step's ring-1 update reads it. So every row strip is one thread-block cluster whose
// warps together cover the full ring (cluster rank r holds segments r W .. r W + W - 1). When a
// strip's pipeline produces ring 1 or ring N-2 at some step, its warps form compensated (TwoSum)
// partial sums of the ring, publish them in shared memory, meet at a cluster barrier, and every
// warp gathers all partials through distributed shared memory in the same fixed order, so all
// of them hold the same mean. Interior strips never reach a ring row (strips are at least K + 1
// rows, so their dependency cones stop short of rows 1 and N-2) and never synchronise.
//
// Order within one step is the reference's: stencil (rows 1..N-2), the pole means from the
// stencil's ring values, then the fronts thin their cells. In the skewed pipeline the top pole
// of step l is known one iteration after its row was due, so its register slot is filled in
// when ring 1 of step l is reduced (it is first read one iteration later); the bottom pole of
// step l is reduced one iteration before it is due and written ahead into its slot.
//
// The per-cell arithmetic is cpu_cell4() (cell.cuh) and the front factor the double-float
// product of the single-step kernel, so K single steps and one launch of this give the same bits
// (the ring sums are compensated, which makes them independent of the summation order).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "cell.cuh"
#include "sbs_internal.h"

namespace cg = cooperative_groups;

namespace sbs {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kSegStride = 120;  // output columns per warp
constexpr int kMaxWarps = 8;      // warps per block
// Registers per thread. The pipeline is latency-bound at the few warps a wave of ring-wide
// clusters leaves per SM, so more warps beat fewer spills: at 2048 x 4096, compensated K = 2
// measured 32.8 us per step capped at 128 registers and 36-38 us with its own ~138; K = 4,
// which needs ~180, 37.7 us at 128 and 50.3 uncapped; plain f32 K = 4 19.7 us either way.
constexpr int kMaxRegs = 128;
constexpr int kMaxCluster = 16;  // blocks per cluster (above 8 needs the non-portable opt-in)
constexpr int kMaxK = 4;

__device__ __forceinline__ float4 splat4(float v) { return make_float4(v, v, v, v); }

__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e) {
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// (s, c) += (s2, c2): compensated combination; the same bits whichever operand comes first.
__device__ __forceinline__ void comp_merge(double &s, double &c, double s2, double c2) {
    double e;
    two_sum(s, s2, s, e);
    c = c + c2 + e;
}

__device__ __forceinline__ void comp_warp(double &s, double &c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double s2 = __shfl_xor_sync(kFull, s, o), c2 = __shfl_xor_sync(kFull, c, o);
        comp_merge(s, c, s2, c2);
    }
}

struct Ctx {
    const float *hin, *lin;  // column-offset input pointers of this lane
    float *hout, *lout;
    const float4 *sco;       // per-row coefficients of rows [t0, t1) in shared memory
    const unsigned *fsel;    // [K][t1 - t0]: front selection nibbles per step and row
    int t0, span;
    int nt, np, pitch, r0, r1;
    bool keep;               // lane owns kept, valid columns (stores and ring sums)
    float b, DR2, dt, crit;
    const double *vol_w;
    double2 *red;            // [2][K][W] ring partials in shared memory (top, bottom)
    int W, C;
    unsigned colbits[kMaxK]; // per step: 4 bits per front, the lane's columns inside it
    const TfeStep *tfe;      // the K steps' front records in shared memory
    bool fronts;             // some step of the launch has a front
};

// Mean of a ring row over the cluster: compensated sums per lane, per warp, then every warp
// gathers the nparts warp partials (all blocks' slots `mine`, rank-major) in the same order.
// All threads of the cluster call this.
template <bool X2>
__device__ __noinline__ double ring_mean(float4 oh, float4 ol, bool keep, double2 *mine, int W, int nparts, int np) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double s = 0.0, c = 0.0;
    if (keep) {
        double e;
        const float hv[4] = {oh.x, oh.y, oh.z, oh.w}, lv[4] = {ol.x, ol.y, ol.z, ol.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const double x = X2 ? (double)hv[k] + (double)lv[k] : (double)hv[k];
            two_sum(s, x, s, e);
            c += e;
        }
    }
    comp_warp(s, c);
    if (lane == 0) mine[warp] = make_double2(s, c);
    cg::cluster_group cl = cg::this_cluster();
    cl.sync();
    double S = 0.0, Cc = 0.0;
    for (int j = lane; j < nparts; j += 32) {
        const double2 *rp = cl.map_shared_rank(mine, (unsigned)(j / W));
        const double2 v = rp[j % W];
        comp_merge(S, Cc, v.x, v.y);
    }
    comp_warp(S, Cc);
    return (S + Cc) / (double)np;
}

// Thins the cells of one row of step l that lie inside a front of that step (drainage.rs:425-460).
template <bool X2>
__device__ __forceinline__ void apply_fronts(const Ctx &w, int l, int i, float4 &oh, float4 &ol) {
    if (!w.fronts) return;
    unsigned x = w.colbits[l - 1] & w.fsel[(l - 1) * w.span + (i - w.t0)];
    x |= x >> 16;
    x |= x >> 8;
    x |= x >> 4;
    x &= 0xfu;
    if (!x) return;
    const float fh = w.tfe[l - 1].factor, fl = w.tfe[l - 1].factor_lo;
    float hv[4] = {oh.x, oh.y, oh.z, oh.w}, lv[4] = {ol.x, ol.y, ol.z, ol.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (!(x & (1u << k))) continue;
        if (X2) {
            const float vh = hv[k], vl = lv[k];
            const float p = vh * fh;
            const float pe = fmaf(vh, fh, -p);
            const float q = fmaf(vh, fl, fmaf(vl, fh, pe));
            const float s = p + q;
            lv[k] = q - (s - p);
            hv[k] = s;
        } else {
            hv[k] = hv[k] * fh;
        }
    }
    oh = make_float4(hv[0], hv[1], hv[2], hv[3]);
    ol = make_float4(lv[0], lv[1], lv[2], lv[3]);
}

template <bool VOL>
__device__ __forceinline__ void store_row(const Ctx &w, int i, float4 oh, float4 ol, bool x2, double &vacc) {
    *reinterpret_cast<float4 *>(w.hout + (size_t)i * w.pitch) = oh;
    if (x2) *reinterpret_cast<float4 *>(w.lout + (size_t)i * w.pitch) = ol;
    if (VOL) {
        const double wi = __ldg(w.vol_w + i);
        vacc += ((double)oh.x + (double)oh.y + (double)oh.z + (double)oh.w) * wi;
        if (x2) vacc += ((double)ol.x + (double)ol.y + (double)ol.z + (double)ol.w) * wi;
    }
}

// One pipeline iteration: receive level-0 row t (prefetched), request row t + 1, then level l of
// row t - l for l = 1..K. Slot P holds each level's newest row.
// Poles: row 0 of step l is written into its slot (CUR, the previous iteration's) when ring 1 of
// step l is reduced; row N-1 of step l is written into the slot it will occupy in the next
// iteration (UP, free once level l + 1 of this iteration has read it) when ring N-2 is reduced.
// Step K's pole rows are stored at the reduction.
template <int K, int P, bool X2, bool VOL, bool POLAR>
__device__ __forceinline__ void iter(const Ctx &w, int t, float4 (&wh)[K][3], float4 (&wl)[K][3], float4 &ph,
                                     float4 &pl, double &vacc) {
    constexpr int CUR = (P + 2) % 3, UP = (P + 1) % 3;
    const int tl = t + 1;
    float4 nh = splat4(0.f), nl = nh;
    if (tl >= 0 && tl < w.nt && tl < w.t0 + w.span) {
        nh = __ldg(reinterpret_cast<const float4 *>(w.hin + (size_t)tl * w.pitch));
        if (X2) nl = __ldg(reinterpret_cast<const float4 *>(w.lin + (size_t)tl * w.pitch));
    }
    wh[0][P] = ph;
    if (X2) wl[0][P] = pl;
    ph = nh;
    pl = nl;
    double mbot = 0.0;  // ring N-2 mean of the level reduced in this iteration
#pragma unroll
    for (int l = 1; l <= K; ++l) {
        const int i = t - l;
        // cluster-uniform: every thread of the strip walks the same rows
        const bool need = i >= w.r0 - (K - l) && i < w.r1 + (K - l) && i >= 0 && i < w.nt;
        float4 oh = splat4(0.f), ol = oh;
        if (POLAR && need && i == w.nt - 1 && l < K) {  // the bottom pole, written one iteration ago
            oh = wh[l][P];
            if (X2) ol = wl[l][P];
        } else if (need && (!POLAR || (i != 0 && i != w.nt - 1))) {
            const float4 hc = wh[l - 1][CUR], hu = wh[l - 1][UP], hd = wh[l - 1][P];
            float4 lc = splat4(0.f), lu = lc, ld = lc;
            if (X2) {
                lc = wl[l - 1][CUR];
                lu = wl[l - 1][UP];
                ld = wl[l - 1][P];
            }
            const float4 co = w.sco[i - w.t0];
            const float hlft = __shfl_up_sync(kFull, hc.w, 1), hrgt = __shfl_down_sync(kFull, hc.x, 1);
            float llft = 0.f, lrgt = 0.f;
            if (X2) {
                llft = __shfl_up_sync(kFull, lc.w, 1);
                lrgt = __shfl_down_sync(kFull, lc.x, 1);
            }
            const float4 hpm = make_float4(hlft, hc.x, hc.y, hc.z), hpp = make_float4(hc.y, hc.z, hc.w, hrgt);
            const float4 lpm = make_float4(llft, lc.x, lc.y, lc.z), lpp = make_float4(lc.y, lc.z, lc.w, lrgt);
            cpu_cell4<X2>(hc, hu, hd, hpm, hpp, lc, lu, ld, lpm, lpp, co, w.b, w.DR2, w.dt, w.crit, oh, ol);
            if (POLAR && (i == 1 || i == w.nt - 2)) {
                // pole means of this step from the ring's stencil values (before the fronts)
                if (i == 1) {
                    const double m = ring_mean<X2>(oh, ol, w.keep, w.red + (l - 1) * w.W, w.W, w.W * w.C, w.np);
                    const float mh = (float)m;
                    const float4 ph4 = splat4(mh), pl4 = splat4(X2 ? (float)(m - (double)mh) : 0.f);
                    if (l < K) {
                        wh[l][CUR] = ph4;
                        if (X2) wl[l][CUR] = pl4;
                    } else if (w.r0 == 0 && w.keep) {
                        store_row<VOL>(w, 0, ph4, pl4, X2, vacc);
                    }
                }
                if (i == w.nt - 2) {
                    mbot = ring_mean<X2>(oh, ol, w.keep, w.red + (K + l - 1) * w.W, w.W, w.W * w.C, w.np);
                    if (l == K && w.r1 == w.nt && w.keep) {
                        const float mh = (float)mbot;
                        store_row<VOL>(w, w.nt - 1, splat4(mh), splat4(X2 ? (float)(mbot - (double)mh) : 0.f), X2,
                                       vacc);
                    }
                }
            }
            apply_fronts<X2>(w, l, i, oh, ol);
        }
        if (l < K) {
            wh[l][P] = oh;
            if (X2) wl[l][P] = ol;
        } else if (need && (!POLAR || (i != 0 && i != w.nt - 1)) && i >= w.r0 && i < w.r1 && w.keep) {
            store_row<VOL>(w, i, oh, ol, X2, vacc);
        }
        if (POLAR && l >= 2 && t - (l - 1) == w.nt - 2) {  // ring N-2 was reduced at level l - 1 above
            const float mh = (float)mbot;
            wh[l - 1][UP] = splat4(mh);
            if (X2) wl[l - 1][UP] = splat4((float)(mbot - (double)mh));
        }
    }
}

__device__ __forceinline__ double block_sum(double v, double *smem) {
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

template <int K, bool X2, bool VOL>
__global__ void __maxnreg__(kMaxRegs) wtbc_kernel(const StepArgs a) {
    __shared__ double2 s_red[2 * kMaxK * kMaxWarps];
    __shared__ TfeStep s_tfe[kMaxK];
    __shared__ double s_vred[32];
    __shared__ int s_last;
    extern __shared__ float4 s_dyn[];  // coefficients of rows [t0, t1), then the front table

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, W = blockDim.x >> 5;
    const int np = a.np, nt = a.nt;
    const int segs = (np + kSegStride - 1) / kSegStride;
    const int seg = blockIdx.x * W + warp;
    const int c_unwrapped = seg * kSegStride - 4 + 4 * lane;
    const int col = ((c_unwrapped % np) + np) % np;
    const int ns = gridDim.y;
    const int r0 = (int)((long long)blockIdx.y * nt / ns), r1 = (int)((long long)(blockIdx.y + 1) * nt / ns);

    Ctx w;
    w.hin = a.hin + col;
    w.lin = a.lin ? a.lin + col : nullptr;
    w.hout = a.hout + col;
    w.lout = a.lout ? a.lout + col : nullptr;
    w.nt = nt;
    w.np = np;
    w.pitch = a.pitch;
    w.r0 = r0;
    w.r1 = r1;
    w.t0 = r0 - K;
    w.span = (r1 + K) - (r0 - K);
    w.keep = seg < segs && lane >= 1 && lane <= 30 && c_unwrapped < np;
    w.b = a.b;
    w.DR2 = a.DR2;
    w.dt = a.dt;
    w.crit = a.crit;
    w.vol_w = a.vol_w;
    w.red = s_red;
    w.W = W;
    w.C = gridDim.x;
    float4 *sco = s_dyn;
    unsigned *fsel = reinterpret_cast<unsigned *>(s_dyn + w.span);
    w.sco = sco;
    w.fsel = fsel;
    w.tfe = s_tfe;
    w.fronts = false;

    // the K steps' front records (all zero when the fronts are off)
    for (int i = threadIdx.x; i < (int)(K * sizeof(TfeStep) / sizeof(int)); i += blockDim.x)
        reinterpret_cast<int *>(s_tfe)[i] = a.tfe ? reinterpret_cast<const int *>(a.tfe)[i] : 0;
    for (int i = threadIdx.x; i < w.span; i += blockDim.x) {
        const int r = w.t0 + i;
        sco[i] = (r >= 0 && r < nt) ? __ldg(a.rows + r) : splat4(0.f);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < K * w.span; i += blockDim.x) {
        const int l = i / w.span, r = w.t0 + i % w.span;
        unsigned sel = 0;
        for (int f = 0; f < s_tfe[l].nf; ++f)
            if (r >= s_tfe[l].fr[f].x && r <= s_tfe[l].fr[f].y) sel |= 0xfu << (4 * f);
        fsel[i] = sel;
    }
#pragma unroll
    for (int l = 0; l < K; ++l) {
        unsigned bits = 0;
        for (int f = 0; f < s_tfe[l].nf; ++f) {
            const int4 fr = s_tfe[l].fr[f];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                int d = col + k - fr.z;
                if (d < 0) d += np;
                if (d < fr.w) bits |= 1u << (4 * f + k);
            }
        }
        w.colbits[l] = bits;
        w.fronts = w.fronts || s_tfe[l].nf > 0;
    }
    __syncthreads();

    float4 wh[K][3], wl[K][3];
#pragma unroll
    for (int l = 0; l < K; ++l)
#pragma unroll
        for (int s = 0; s < 3; ++s) {
            wh[l][s] = splat4(0.f);
            wl[l][s] = wh[l][s];
        }

    double vacc = 0.0;
    const int t0 = w.t0, t1 = w.t0 + w.span;
    float4 ph = splat4(0.f), pl = ph;
    if (t0 >= 0) {
        ph = __ldg(reinterpret_cast<const float4 *>(w.hin + (size_t)t0 * w.pitch));
        if (X2) pl = __ldg(reinterpret_cast<const float4 *>(w.lin + (size_t)t0 * w.pitch));
    }
    if (r0 == 0 || r1 == nt) {  // a polar strip (cluster-uniform)
        for (int t = t0; t < t1; t += 3) {
            iter<K, 0, X2, VOL, true>(w, t, wh, wl, ph, pl, vacc);
            if (t + 1 < t1) iter<K, 1, X2, VOL, true>(w, t + 1, wh, wl, ph, pl, vacc);
            if (t + 2 < t1) iter<K, 2, X2, VOL, true>(w, t + 2, wh, wl, ph, pl, vacc);
        }
    } else {
        for (int t = t0; t < t1; t += 3) {
            iter<K, 0, X2, VOL, false>(w, t, wh, wl, ph, pl, vacc);
            if (t + 1 < t1) iter<K, 1, X2, VOL, false>(w, t + 1, wh, wl, ph, pl, vacc);
            if (t + 2 < t1) iter<K, 2, X2, VOL, false>(w, t + 2, wh, wl, ph, pl, vacc);
        }
    }
    // no block may leave while a cluster peer can still read its ring partials
    cg::this_cluster().sync();

    if (VOL) {
        const double s = block_sum(vacc, s_vred);
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
            tot = block_sum(tot, s_vred);
            if (threadIdx.x == 0) {
                const unsigned idx = *a.vol_index;
                a.vol_out[idx] = tot;
                *a.vol_index = idx + 1;
                *a.vol_counter = 0u;
                __threadfence();
            }
        }
    }
}

template <int K, bool X2>
const void *pick_vol(bool vol) {
    return vol ? (const void *)wtbc_kernel<K, X2, true> : (const void *)wtbc_kernel<K, X2, false>;
}

const void *wtbc_fn(int K, bool x2, bool vol) {
    switch (K) {
        case 2:
            return x2 ? pick_vol<2, true>(vol) : pick_vol<2, false>(vol);
        case 3:
            return x2 ? pick_vol<3, true>(vol) : pick_vol<3, false>(vol);
        case 4:
            return x2 ? pick_vol<4, true>(vol) : pick_vol<4, false>(vol);
        default:
            return nullptr;
    }
}

size_t dyn_smem(int span, int K) { return sizeof(float4) * (size_t)span + sizeof(unsigned) * (size_t)K * span; }

}  // namespace

// Geometry of the blocked CPU-semantics step: W warps per block and C = ceil(segments / W)
// blocks per cluster cover the ring's 120-column segments (C <= 16). A launch is one wave of
// clusters, one per row strip, so the W that lets the most clusters be resident at once wins
// (the strips are then shortest); ties go to fewer idle warps, then W nearest 4. Strips have at
// least K + 1 rows. nby = 0: unsupported.
StepGeom wtbc_geometry(int nt, int np, int K, int x2) {
    StepGeom g{};
    if (K < 2 || K > kMaxK || np % 4 != 0 || np < 8 || nt < 2 * (K + 1)) return g;
    const int segs = (np + kSegStride - 1) / kSegStride;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int span_guess = (nt + sms - 1) / sms + 2 * K + 64;
    int bestW = 0, bestC = 0, bestN = 0, bestWaste = 1 << 30, bestD = 1 << 30;
    for (int W = 1; W <= kMaxWarps; ++W) {
        const int C = (segs + W - 1) / W;
        if (C > kMaxCluster) continue;
        if (C > 8) {
            bool ok = true;
            for (int v = 0; v < 2; ++v)
                ok = ok && cudaFuncSetAttribute(wtbc_fn(K, x2 != 0, v == 1),
                                                cudaFuncAttributeNonPortableClusterSizeAllowed, 1) == cudaSuccess;
            if (!ok) {
                cudaGetLastError();
                continue;
            }
        }
        cudaLaunchConfig_t cfg{};
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = C;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(C, 1);
        cfg.blockDim = dim3(32 * W);
        cfg.dynamicSmemBytes = dyn_smem(span_guess, K);
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, wtbc_fn(K, x2 != 0, true), &cfg) != cudaSuccess) {
            cudaGetLastError();
            n = 0;
        }
        if (n < 1) continue;
        const int waste = C * W - segs, d = W > 4 ? W - 4 : 4 - W;
        if (n > bestN || (n == bestN && (waste < bestWaste || (waste == bestWaste && d < bestD)))) {
            bestW = W;
            bestC = C;
            bestN = n;
            bestWaste = waste;
            bestD = d;
        }
    }
    if (bestW == 0) return g;
    int ns = bestN < nt / (K + 1) ? bestN : nt / (K + 1);
    if (ns < 1) ns = 1;
    g.wx = bestW;
    g.nbx = bestC;
    g.nby = ns;
    g.rb = (nt + ns - 1) / ns;
    return g;
}

cudaError_t launch_wtbc(int K, int x2, const StepArgs &a, const StepGeom &g, cudaStream_t s) {
    const void *fn = wtbc_fn(K, x2 != 0, a.vol_w != nullptr);
    if (fn == nullptr || g.nby < 1) return cudaErrorInvalidValue;
    const int span = g.rb + 2 * K;
    cudaLaunchConfig_t cfg{};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = g.nbx;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(g.nbx, g.nby);
    cfg.blockDim = dim3(32 * g.wx);
    cfg.dynamicSmemBytes = dyn_smem(span, K);
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    void *args[] = {(void *)&a};
    return cudaLaunchKernelExC(&cfg, fn, args);
}

}  // namespace sbs
