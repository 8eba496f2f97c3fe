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
// the next step's ring-1 update reads it. A row strip is C blocks of W warps that together cover
// the full ring (block b holds segments b W .. b W + W - 1). When a polar strip's pipeline
// produces ring 1 or ring N-2 at some step, its warps form compensated (TwoSum) partial sums of
// the ring, publish them in global memory, meet at a barrier of the strip's C blocks, and every
// warp gathers all partials in the same fixed order, so all of them hold the same mean. The
// launch is cooperative (every block resident at once), so the barrier cannot wait for a block
// that is not running; its wait is bounded all the same. Interior strips never reach a ring row
// (strips are at least K + 1 rows, so their dependency cones stop short of rows 1 and N-2) and
// never synchronise.
//
// An earlier form made every strip one thread-block cluster and gathered the partials through
// distributed shared memory. Clusters of C = 9 blocks are placed whole on one GPC, which at
// 2048 x 4096 left some SMs without a block and the average SM busy 56 % of the launch (33.5 us
// per step); the plain grid keeps every SM at its four blocks. The ring sums are exact integer
// sums (fixsum.cuh): the compensated double sums before them kept the polar strips' warps on
// the FP64 pipe for ~10 us per ring mean.
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
#include <cuda_runtime.h>

#include "cell.cuh"
#include "fixsum.cuh"
#include "sbs_internal.h"

namespace sbs {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kSegStride = 120;  // output columns per warp
// Registers per thread: 128 lets four blocks of four warps share an SM. The pipeline needs more
// warps more than fewer spills (an earlier, cluster-launched form at 2048 x 4096: compensated
// K = 2 32.8 us per step capped at 128 registers against 36-38 us with its own ~138).
constexpr int kMaxRegs = 128;
constexpr int kMaxK = 4;
// Rows in flight per lane. Row t + kDepth is requested while row t is consumed, through a
// per-warp ring of kDepth + 1 row slots (hi and lo words) in shared memory filled by per-thread
// 16-byte cp.async copies: each lane waits only for its own copies (cp.async.wait_group), so no
// handshake between warps is needed and the rows in flight cost no registers. Depths 2 to 6
// measured within 2 % of each other.
constexpr int kDepth = 3;
constexpr int kSlots = kDepth + 1;

__device__ __forceinline__ void cp_async16(float4 *smem, const float *gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__device__ __forceinline__ float4 splat4(float v) { return make_float4(v, v, v, v); }

// Where a polar strip's blocks exchange their ring partials.
struct RingX {
    FixSum *part;            // [2][kMaxK][nparts] warp partials in global memory (top, bottom)
    unsigned *bar;           // [2][kMaxK] barrier words (arrivals, generation), then the status word
    unsigned *status_host;   // host-mapped copy of the status word
    long long limit;         // barrier wait limit, SM cycles
    unsigned narrive;        // arrivals a barrier waits for (C, plus one in the timeout test)
    int nparts;              // warp partials per ring = C W
};

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
    RingX x;                 // the polar strips' ring exchange
    unsigned colbits[kMaxK]; // per step: 4 bits per front, the lane's columns inside it
    const TfeStep *tfe;      // the K steps' front records in shared memory
    bool fronts;             // some step of the launch has a front
    float4 *ring;            // this lane's row slots: ring[(slot * 2 + word) * 32]
};

// Requests row r (hi and lo words) into its ring slot and closes the copy group; rows outside
// [0, nt) and past the strip's span are not fetched (the group is then empty).
template <bool X2>
__device__ __forceinline__ void request_row(const Ctx &w, int r) {
    if (r >= 0 && r < w.nt && r < w.t0 + w.span) {
        float4 *slot = w.ring + ((r - w.t0) % kSlots) * 64;
        cp_async16(slot, w.hin + (size_t)r * w.pitch);
        if (X2) cp_async16(slot + 32, w.lin + (size_t)r * w.pitch);
    }
    cp_async_commit();
}

// Barrier of the C blocks of one polar strip. All threads of the block call it. Bounded: after
// `limit` cycles it records a timeout in the status words and returns; once a timeout is
// recorded, later barriers of the launch do not wait.
__device__ __forceinline__ void strip_barrier(unsigned *b, unsigned *status, unsigned *status_host, long long limit,
                                              unsigned narrive) {
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned gen = atomicAdd(b + 1, 0u);
        __threadfence();
        if (atomicAdd(b, 1u) + 1 == narrive) {
            atomicExch(b, 0u);
            __threadfence();
            atomicAdd(b + 1, 1u);
        } else if (atomicAdd(status, 0u) == 0u) {
            const long long t0 = clock64();
            while (atomicAdd(b + 1, 0u) == gen) {
                if (clock64() - t0 > limit) {
                    atomicOr(status, 1u);
                    *(volatile unsigned *)status_host = 1u;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

// Mean of a ring row over the strip: exact fixed-point sums (fixsum.cuh) per lane and per warp,
// published per warp; every warp then adds all nparts partials, so all of them hold the same
// mean. All threads of the strip's blocks call this; slot = side * kMaxK + level - 1. Scalar
// arguments keep the caller's context in registers.
template <bool X2>
__device__ __noinline__ double ring_mean(float4 oh, float4 ol, bool keep, FixSum *part_all, unsigned *bar,
                                         unsigned *status_host, long long limit, unsigned narrive, int nparts, int np,
                                         int slot) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    FixSum acc = fix_zero();
    if (keep) {
        fix_add_float(acc, oh.x);
        fix_add_float(acc, oh.y);
        fix_add_float(acc, oh.z);
        fix_add_float(acc, oh.w);
        if (X2) {
            fix_add_float(acc, ol.x);
            fix_add_float(acc, ol.y);
            fix_add_float(acc, ol.z);
            fix_add_float(acc, ol.w);
        }
    }
    fix_warp(acc);
    FixSum *part = part_all + (size_t)slot * nparts;
    if (lane == 0) part[blockIdx.x * (blockDim.x >> 5) + warp] = acc;
    strip_barrier(bar + 2 * slot, bar + 4 * kMaxK, status_host, limit, narrive);
    FixSum tot = fix_zero();
    for (int j = lane; j < nparts; j += 32) {
        fix_add(tot, fix_ldcg(part + j));
    }
    fix_warp(tot);
    return fix_to_double(tot) / (double)np;
}

template <bool X2>
__device__ __forceinline__ double ring_mean_of(const Ctx &w, float4 oh, float4 ol, int slot) {
    return ring_mean<X2>(oh, ol, w.keep, w.x.part, w.x.bar, w.x.status_host, w.x.limit, w.x.narrive, w.x.nparts,
                         w.np, slot);
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

// One pipeline iteration: receive level-0 row t from the ring, request row t + kDepth, then level l
// of row t - l for l = 1..K. Slot P holds each level's newest row.
// Poles: row 0 of step l is written into its slot (CUR, the previous iteration's) when ring 1 of
// step l is reduced; row N-1 of step l is written into the slot it will occupy in the next
// iteration (UP, free once level l + 1 of this iteration has read it) when ring N-2 is reduced.
// Step K's pole rows are stored at the reduction.
template <int K, int P, bool X2, bool VOL, bool POLAR>
__device__ __forceinline__ void iter(const Ctx &w, int t, float4 (&wh)[K][3], float4 (&wl)[K][3], double &vacc) {
    constexpr int CUR = (P + 2) % 3, UP = (P + 1) % 3;
    cp_async_wait<kDepth - 1>();  // the groups of rows <= t have landed
    float4 nh = splat4(0.f), nl = nh;
    if (t >= 0 && t < w.nt) {  // t < t0 + span always
        const float4 *slot = w.ring + ((t - w.t0) % kSlots) * 64;
        nh = slot[0];
        if (X2) nl = slot[32];
    }
    wh[0][P] = nh;
    if (X2) wl[0][P] = nl;
    // the slot of row t + kDepth last held row t - 1, read one iteration ago
    request_row<X2>(w, t + kDepth);
    double mbot = 0.0;  // ring N-2 mean of the level reduced in this iteration
#pragma unroll
    for (int l = 1; l <= K; ++l) {
        const int i = t - l;
        // strip-uniform: every thread of the strip walks the same rows
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
                    const double m = ring_mean_of<X2>(w, oh, ol, l - 1);
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
                    mbot = ring_mean_of<X2>(w, oh, ol, kMaxK + l - 1);
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

// Rows [r0, r1) of strip `by` of `ns`: the two polar strips have prow rows each, the interior
// strips share the rest evenly. prow = 0: all strips even.
__host__ __device__ inline void strip_rows(int by, int ns, int nt, int prow, int &r0, int &r1) {
    if (prow <= 0 || ns < 3) {
        r0 = (int)((long long)by * nt / ns);
        r1 = (int)((long long)(by + 1) * nt / ns);
    } else if (by == 0) {
        r0 = 0;
        r1 = prow;
    } else if (by == ns - 1) {
        r0 = nt - prow;
        r1 = nt;
    } else {
        const long long rest = nt - 2 * prow;
        r0 = prow + (int)((by - 1) * rest / (ns - 2));
        r1 = prow + (int)(by * rest / (ns - 2));
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
    __shared__ TfeStep s_tfe[kMaxK];
    __shared__ double s_vred[32];
    __shared__ int s_last;
    extern __shared__ float4 s_dyn[];  // row rings of the warps, coefficients of rows [t0, t1), front table

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, W = blockDim.x >> 5;
    const int np = a.np, nt = a.nt;
    const int segs = (np + kSegStride - 1) / kSegStride;
    const int seg = blockIdx.x * W + warp;
    const int c_unwrapped = seg * kSegStride - 4 + 4 * lane;
    const int col = ((c_unwrapped % np) + np) % np;
    int r0, r1;
    strip_rows(blockIdx.y, gridDim.y, nt, a.prow, r0, r1);

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
    w.x.part = a.ring_part;
    w.x.bar = a.ring_bar;
    w.x.status_host = a.status_host;
    w.x.limit = a.wait_cycles;
    w.x.narrive = gridDim.x + a.extra;
    w.x.nparts = gridDim.x * W;
    w.ring = s_dyn + (size_t)warp * kSlots * 64 + lane;
    float4 *sco = s_dyn + (size_t)W * kSlots * 64;
    unsigned *fsel = reinterpret_cast<unsigned *>(sco + w.span);
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
#pragma unroll
    for (int j = 0; j < kDepth; ++j) request_row<X2>(w, t0 + j);
    if (r0 == 0 || r1 == nt) {  // a polar strip (block-uniform)
        for (int t = t0; t < t1; t += 3) {
            iter<K, 0, X2, VOL, true>(w, t, wh, wl, vacc);
            if (t + 1 < t1) iter<K, 1, X2, VOL, true>(w, t + 1, wh, wl, vacc);
            if (t + 2 < t1) iter<K, 2, X2, VOL, true>(w, t + 2, wh, wl, vacc);
        }
    } else {
        for (int t = t0; t < t1; t += 3) {
            iter<K, 0, X2, VOL, false>(w, t, wh, wl, vacc);
            if (t + 1 < t1) iter<K, 1, X2, VOL, false>(w, t + 1, wh, wl, vacc);
            if (t + 2 < t1) iter<K, 2, X2, VOL, false>(w, t + 2, wh, wl, vacc);
        }
    }
    cp_async_wait<0>();  // every copy was consumed; nothing may still be landing at exit

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

size_t dyn_smem(int W, int span, int K) {
    return sizeof(float4) * ((size_t)W * kSlots * 64 + span) + sizeof(unsigned) * (size_t)K * span;
}

}  // namespace

// Geometry of the blocked CPU-semantics step: blocks of W = 4 warps (fewer on narrow grids), C =
// ceil(segments / W) blocks per strip across the ring's 120-column segments, and as many strips
// as fit one wave (the cooperative launch needs every block resident). The two polar strips get
// K + 1 rows, the fewest the pipeline allows: their blocks also meet at a barrier for every
// ring mean, and with equal strips they finished last (2048 x 4096, compensated K = 2: 28.6 us per
// step with equal strips, 20.2 with polar strips of K + 1 rows). Interior strips have at least
// K + 1 rows. nby = 0: unsupported.
StepGeom wtbc_geometry(int nt, int np, int K, int x2) {
    StepGeom g{};
    if (K < 2 || K > kMaxK || np % 4 != 0 || np < 8 || nt < 2 * (K + 1)) return g;
    const int segs = (np + kSegStride - 1) / kSegStride;
    int dev = 0, sms = 148, coop = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (!coop) return g;
    for (int v = 0; v < 2; ++v)  // the rings alone take up to 32 KB a block
        if (cudaFuncSetAttribute(wtbc_fn(K, x2 != 0, v == 1), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 160 * 1024) != cudaSuccess) {
            cudaGetLastError();
            return g;
        }
    const int W = segs < 4 ? segs : 4, C = (segs + W - 1) / W;
    // strips that fit one wave: shrink until the blocks of the real strip height fit
    int ns = nt / (K + 1);
    for (int it = 0; it < 8 && ns >= 1; ++it) {
        int prow = 0, rmax = 0;
        if (ns >= 3) {
            prow = K + 1;
            if ((nt - 2 * prow) / (ns - 2) < K + 1) prow = 0;
        }
        for (int by = 0; by < ns; ++by) {
            int r0, r1;
            strip_rows(by, ns, nt, prow, r0, r1);
            rmax = r1 - r0 > rmax ? r1 - r0 : rmax;
        }
        int per_sm = 0;
        for (int v = 0; v < 2; ++v) {
            int n = 0;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, wtbc_fn(K, x2 != 0, v == 1), 32 * W,
                                                              dyn_smem(W, rmax + 2 * K, K)) != cudaSuccess) {
                cudaGetLastError();
                n = 0;
            }
            per_sm = v == 0 || n < per_sm ? n : per_sm;
        }
        const int fit = per_sm * sms / C;
        if (fit >= ns) {
            if (dyn_smem(W, rmax + 2 * K, K) > 160 * 1024) return g;
            g.wx = W;
            g.nbx = C;
            g.nby = ns;
            g.rb = rmax;
            g.prow = prow;
            return g;
        }
        ns = fit;
    }
    return g;
}

int wtbc_ring_parts(const StepGeom &g) { return g.nbx * g.wx; }

cudaError_t launch_wtbc(int K, int x2, const StepArgs &a, const StepGeom &g, cudaStream_t s) {
    const void *fn = wtbc_fn(K, x2 != 0, a.vol_w != nullptr);
    if (fn == nullptr || g.nby < 1 || a.ring_part == nullptr || a.ring_bar == nullptr) return cudaErrorInvalidValue;
    const int span = g.rb + 2 * K;
    void *args[] = {(void *)&a};
    return cudaLaunchCooperativeKernel(fn, dim3(g.nbx, g.nby), dim3(32 * g.wx), args, dyn_smem(g.wx, span, K), s);
}

}  // namespace sbs
