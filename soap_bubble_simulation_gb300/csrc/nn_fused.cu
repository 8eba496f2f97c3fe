// Fused forward pass of the drainage surrogate (include/sbs_nn.h) on the tcgen05 tensor cores:
// features, the four 3x3 convolutions, GELUs and the thickness update in one persistent kernel,
// activations kept in shared memory and accumulators in tensor memory.
//
// Tiling. A tile is a strip of 128 consecutive phi columns (lanes; the middle 120 are output, the
// 4 on each side are the halo the four layers consume) times a block of theta rows of one field.
// The block runs eight agents that only talk through mbarriers: four MMA warps (one per layer:
// for each input row, wait for the row and for the accumulator slot it starts, issue, commit) and
// four epilogue warpgroups (warpgroup l-1 reads layer l's finished row from TMEM, zeroes the slot,
// adds the bias, applies GELU and writes the activation row into one of three input buffers of layer
// l+1; warpgroup 3 writes the features and the thickness update). Every ring (activation buffers:
// full / empty; accumulator rows: full / empty, and a per-tile barrier for the last three rows) is
// balanced per tile, so each waiter is at most one phase behind and parity waits are exact.
// The block streams its rows top to bottom through all four layers at once, each layer as far
// behind the one before as its inputs require.
//
// Convolution as MMAs. Activations of one row live in shared memory as planes of 8 channels with
// 16 B per cell (K-major, rows of the A operand = cells, SBO = 128 B), so the dx = -1/0/+1 taps
// are the same tile read at start offsets of 16 B apart: no im2col buffer. The three dy taps are
// stacked along N: one M=128 x N=96 MMA multiplies an input row by [W(dy) for three output rows]
// and accumulates into a ring of three 32-column TMEM slots (output row r lives in slot r mod 3).
// B holds the dy blocks as [W+1; W0; W-1; W+1; W0]; a window of three consecutive blocks, chosen by
// the input row mod 3, matches the ring order, so each input row is one contiguous N=96 operand.
// A slot is read by the epilogue once its row's three input rows are in, then zeroed for reuse.
// theta reflection at the poles adds one N=32 MMA (input row 1 into output row 0 with W-1, input
// row nt-2 into output row nt-1 with W+1).
//
// TMEM columns: layer 1 [0, 96), layer 2 [96, 192), layer 3 [192, 288), layer 4 [288, 304)
// (N = 16, rows of B beyond the dy ring are zero). Every MMA's D column is a multiple of 16: the
// layer-4 pole extras keep D at column 288 and place their single weight row at the target slot
// by the B window offset. One CTA per SM (it allocates all 512 columns).
// Every mbarrier wait is bounded; a timeout sets the error flag and the kernel drains and exits.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "nn.cuh"
#include "nn_kernels.h"
#include "sbs_internal.h"

namespace sbs {
namespace nn {

cudaStream_t stream_of(sbs_surrogate *s);
const float *theta_of(sbs_surrogate *s);
void **fused_slot(sbs_surrogate *s);
int *fused_dirty_flag(sbs_surrogate *s);
int sms_of(sbs_surrogate *s);

namespace {

constexpr int kLanes = 128;                    // TMEM lanes = cells of a strip
constexpr int kGroups = 4;                     // warpgroups: each owns one 8-channel plane
constexpr int kEpi = kLanes * kGroups;         // epilogue threads (16 warps)
constexpr int kThreads = kEpi + 4 * 32;        // + one MMA-issuing warp per layer
constexpr int kOut = 120;                      // output columns per strip
constexpr int kHalo = 4;                       // lanes on each side of the outputs
constexpr int kCells = 136;                    // staged cells per plane (q = lane + 1)
constexpr uint32_t kPlane = kCells * 16;       // 2176 B
constexpr uint32_t kRowX = 4 * kPlane;         // one 32-channel row buffer
constexpr uint32_t kRowX0 = 2 * kPlane;        // one 16-feature row buffer
constexpr uint32_t kBRows = 96;                // dy blocks [W+1; W0; W-1] (3 x 32 rows)
constexpr uint32_t kBChunk = kBRows * 16;      // one 8-channel K chunk
constexpr uint32_t kBStep = 2 * kBChunk;       // one K16 step
constexpr uint32_t kBlk = 32 * 16;             // one 32-row block
constexpr uint32_t kB4Rows = 40, kB4Chunk = kB4Rows * 16, kB4Step = 2 * kB4Chunk;  // W4 at rows 15, 16, 17
constexpr uint32_t kBxRows = 32, kBxChunk = kBxRows * 16, kBxStep = 2 * kBxChunk;  // one W4 block at row 15
// smem image of the packed weights (built once per parameter change by pack_fused_kernel)
constexpr uint32_t kOffB1 = 0;                          // 3 steps (dx)
constexpr uint32_t kOffB2 = kOffB1 + 3 * kBStep;        // 6 steps (dx x 16-channel half)
constexpr uint32_t kOffB3 = kOffB2 + 6 * kBStep;        // 6 steps
constexpr uint32_t kOffB4 = kOffB3 + 6 * kBStep;        // 6 steps, 40 rows
constexpr uint32_t kOffB4t = kOffB4 + 6 * kB4Step;      // W4(dy=-1) alone (top pole extra)
constexpr uint32_t kOffB4b = kOffB4t + 6 * kBxStep;     // W4(dy=+1) alone (bottom pole extra)
constexpr uint32_t kOffBias = kOffB4b + 6 * kBxStep;    // 97 floats (padded to 128)
constexpr uint32_t kImage = kOffBias + 128 * 4;
// accumulator rings: layers 1-3 keep kDepth rows of 32 columns, layer 4 kDepth4 single columns
constexpr int kDepth = 4, kDepth4 = 16;
__host__ __device__ constexpr int depth_of(int l) { return l < 4 ? kDepth : kDepth4; }  // l 1-based
__host__ __device__ constexpr uint32_t acc_col(int l) { return 128u * (uint32_t)l; }    // l 0-based; 3 -> 384
// rest of shared memory
constexpr int kNBuf = 3;                                   // activation rows in flight per layer input
constexpr uint32_t kOffX0 = (kImage + 1023) / 1024 * 1024;  // feature rows
constexpr uint32_t kOffX = kOffX0 + kNBuf * kRowX0;         // 3 layers x kNBuf rows
constexpr uint32_t kOffBar = kOffX + 3 * kNBuf * kRowX;
// barriers of layer l: xfull[kNBuf], xempty[kNBuf], afull[depth], aempty[depth]
__host__ __device__ constexpr int bar_base(int l) { return (l - 1) * (2 * kNBuf + 2 * kDepth); }
constexpr int kNumBars = 3 * (2 * kNBuf + 2 * kDepth) + 2 * kNBuf + 2 * kDepth4;
constexpr uint32_t kSmem = kOffBar + 8 * (kNumBars + 1) + 64;  // + the exit drain barrier
constexpr long long kWaitCycles = 2000000000LL;  // ~1 s at 2 GHz

__host__ __device__ constexpr uint32_t idesc(int n) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(kLanes >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t make_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // tcgen05 descriptor version; base offset 0, no swizzle
    return d;
}

__device__ __forceinline__ void mma(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t id) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, 1, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(id));
}

// One lane of a converged warp (the elected issuer of tensor-core instructions).
__device__ __forceinline__ bool elect_one() {
    uint32_t pred = 0;
    asm volatile("{\n .reg .pred P;\n .reg .b32 L;\n elect.sync L|P, 0xffffffff;\n selp.b32 %0, 1, 0, P;\n}\n"
                 : "=r"(pred));
    return pred != 0;
}

__device__ __forceinline__ void commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > kWaitCycles) return false;
    return true;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ uint32_t tld1(uint32_t taddr) {
    uint32_t v;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=r"(v) : "r"(taddr));
    return v;
}

__device__ __forceinline__ void tzero1(uint32_t taddr) {
    const uint32_t z = 0;
    asm volatile("tcgen05.st.sync.aligned.32x32b.x1.b32 [%0], {%1};" ::"r"(taddr), "r"(z) : "memory");
}

__device__ __forceinline__ void wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// Registers written by tcgen05.ld are valid only after tcgen05.wait::ld: tie them to a point after
// the wait so the compiler cannot schedule their uses earlier.
__device__ __forceinline__ void pin(uint32_t &r) { asm volatile("" : "+r"(r)); }
__device__ __forceinline__ void wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ int refl_row(int i, int nt) { return i < 0 ? 1 : (i >= nt ? nt - 2 : i); }

struct FusedArgs {
    Fields fs;
    GridTab g;
    const uint8_t *image;  // packed weights (kImage bytes)
    float *y_out;          // [nf][nt][np] or null
    float *h_out;          // field 0 only, or null
    size_t pitch_out;
    int nf, nstrips, nrb, rows_per_block, ntiles;
    unsigned *err;
};

// MMAs of layer l (1-based) for input row s into the layer's accumulator ring (or, for the pole
// extras, into one slot): issued by one thread.
// Descriptor of the no-swizzle K-major tile at smem byte address addr (< 256 KB): base | addr >> 4.
__device__ __forceinline__ uint64_t desc_at(uint64_t base, uint32_t addr) { return base | (uint64_t)(addr >> 4); }

// MMAs of layer L (1-based) for one input row, fully unrolled: ad0 / bd0 are the descriptors of
// the row's activation buffer and of the layer's B tile, the per-step offsets are compile-time
// (descriptor address fields count 16-byte units). c = ring slot of output row s-1.
// Operands of one input row of layer L (computed by the whole warp from warp-uniform values, so
// they stay in uniform registers), then the MMAs back to back from one elected lane.
template <int L>
struct RowOps {
    static constexpr int NS = L == 1 ? 3 : 6;
    uint64_t ad[NS], b1[NS], b2[NS];
    uint32_t d1, d2, i1, i2;
    bool two;
    __device__ __forceinline__ RowOps(uint32_t dacc, uint64_t ad0, uint64_t bd0, int c) {
        if constexpr (L < 4) {
            two = c > kDepth - 3;
            d1 = dacc + 32 * c;
            d2 = dacc;
            i1 = c <= kDepth - 3 ? idesc(96) : (c == kDepth - 2 ? idesc(64) : idesc(32));
            i2 = c == kDepth - 2 ? idesc(32) : idesc(64);
            const uint64_t o2 = c == kDepth - 2 ? (2 * kBlk >> 4) : (kBlk >> 4);
#pragma unroll
            for (int st = 0; st < NS; ++st) {
                const int dxi = L == 1 ? st : st >> 1, kk = L == 1 ? 0 : st & 1;
                ad[st] = ad0 + (uint64_t)((2 * kk * kPlane + 16 * dxi) >> 4);
                b1[st] = bd0 + (uint64_t)((st * kBStep) >> 4);
                b2[st] = b1[st] + o2;
            }
        } else {
            // B rows 15..17 hold W4(dy = +1, 0, -1): window start 15 - c puts them at columns c..c+2;
            // the part past the last slot wraps to column 0 through a second window
            two = c >= kDepth4 - 2;
            d1 = d2 = dacc;
            i1 = i2 = idesc(16);
#pragma unroll
            for (int st = 0; st < NS; ++st) {
                const int dxi = st >> 1, kk = st & 1;
                ad[st] = ad0 + (uint64_t)((2 * kk * kPlane + 16 * dxi) >> 4);
                b1[st] = bd0 + (uint64_t)((st * kB4Step) >> 4) + (uint64_t)(15 - c);
                b2[st] = bd0 + (uint64_t)((st * kB4Step) >> 4) + (uint64_t)(31 - c);
            }
        }
    }
    __device__ __forceinline__ void issue() const {
        if (!two) {
#pragma unroll
            for (int st = 0; st < NS; ++st) mma(d1, ad[st], b1[st], i1);
        } else {
#pragma unroll
            for (int st = 0; st < NS; ++st) {
                mma(d1, ad[st], b1[st], i1);
                mma(d2, ad[st], b2[st], i2);
            }
        }
    }
};

// theta-reflection extra MMAs of layer L: input row 1 into output row 0 with W(dy=-1) (top) or input
// row nt-2 into output row nt-1 with W(dy=+1) (bottom), oslot = that output row's ring slot.
template <int L>
__device__ __forceinline__ void issue_pole(uint32_t dacc, uint64_t ad0, uint32_t sbase, bool top, int oslot) {
    constexpr int NS = L == 1 ? 3 : 6;
    const uint32_t boff = sbase + (L == 1 ? kOffB1 : (L == 2 ? kOffB2 : (L == 3 ? kOffB3 : 0u)));
#pragma unroll
    for (int st = 0; st < NS; ++st) {
        const int dxi = L == 1 ? st : st >> 1, kk = L == 1 ? 0 : st & 1;
        const uint64_t ad = ad0 + (uint64_t)((2 * kk * kPlane + 16 * dxi) >> 4);
        if constexpr (L < 4) {
            const uint32_t blk = top ? 2 * kBlk : 0;  // W-1 block / W+1 block
            mma(dacc + 32 * oslot, ad, desc_at(make_desc(0, kBChunk, 128), boff + st * kBStep + blk), idesc(32));
        } else {
            // B tile row 15 holds the weights: window start 15 - slot puts them at D column 384 + slot
            mma(dacc, ad,
                desc_at(make_desc(0, kBxChunk, 128),
                        sbase + (top ? kOffB4t : kOffB4b) + st * kBxStep + (uint32_t)(15 - oslot) * 16u),
                idesc(16));
        }
    }
}

// Inputs of one row's features for one lane, loaded a row ahead of their use.
struct FeatIn {
    float hc, hn, hs, hw, he, cc, lip;
    float4 row;
};

__device__ __forceinline__ void feat_load(FeatIn &p, int i, int nt, const Field &fd, const GridTab &g, int col, int cw,
                                          int ce) {
    const float *rc = fd.h + (size_t)i * fd.pitch;
    p.row = g.rows[i];
    p.lip = g.lip[i];
    p.hc = rc[col];
    p.hn = fd.h[(size_t)refl_row(i - 1, nt) * fd.pitch + col];
    p.hs = fd.h[(size_t)refl_row(i + 1, nt) * fd.pitch + col];
    p.hw = rc[cw];
    p.he = rc[ce];
    p.cc = fd.c[(size_t)i * fd.pitch + col];
}

// The lane's 16 features as two 16-byte planes (include/sbs_nn.h; the same FP32 operations as
// cell_features).
__device__ __forceinline__ void feat_store(const FeatIn &p, const Field &fd, const GridTab &g, uint8_t *x0, int lane) {
    uint4 p0, p1;
    cell_features(p.hc, p.hn, p.hs, p.hw, p.he, p.cc, p.row, p.lip, fd, g, p0, p1);
    *reinterpret_cast<uint4 *>(x0 + (lane + 1) * 16) = p0;
    *reinterpret_cast<uint4 *>(x0 + kPlane + (lane + 1) * 16) = p1;
}

__device__ __forceinline__ void tld32(uint32_t taddr, uint32_t *v) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
          "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
          "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
          "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
}

__device__ __forceinline__ void tzero32(uint32_t taddr) {
    const uint32_t z = 0;
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, "
        "%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1};" ::"r"(taddr),
        "r"(z)
        : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Per-thread phase tracking of one barrier: waits for completion number `count` (0, 1, ...).
struct Waiter {
    volatile int *fail;
    unsigned *err;
    __device__ __forceinline__ void wait(uint32_t bar, uint32_t count) {
        if (*fail) return;
        if (!mbar_wait_bounded(bar, count & 1u)) {
            atomicOr(err, 1u);
            *fail = 1;
        }
    }
};

__device__ __forceinline__ void tile_rows(const FusedArgs &a, int tile, int *lo, int *hi, int &strip, int &f) {
    strip = tile % a.nstrips;
    const int rb = (tile / a.nstrips) % a.nrb;
    f = tile / (a.nstrips * a.nrb);
    const int y0 = rb * a.rows_per_block, y1 = min(a.g.nt, y0 + a.rows_per_block);
    for (int l = 0; l <= 4; ++l) {
        lo[l] = max(0, y0 - 4 + l);
        hi[l] = min(a.g.nt, y1 + 4 - l);
    }
}

__global__ void __launch_bounds__(kThreads, 1) fused_kernel(FusedArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + kOffBar);
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(bar + kNumBars + 1);
    const uint32_t drain = smem_u32(bar + kNumBars);  // every MMA warp's final commit (4 arrivals)
    volatile int *s_fail = reinterpret_cast<volatile int *>(s_tmem + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int grp = tid >> 7, lane = tid & (kLanes - 1);
    const int nt = a.g.nt, np = a.g.np;
    const uint32_t sbase = smem_u32(smem);
    // barriers of layer l (1-based): input-row buffers of layer l (full: written by the producer
    // warpgroup, empty: released by layer l's MMAs) and accumulator ring slots (full: the slot's row
    // has all its contributions, empty: its epilogue has read and zeroed it)
    auto xfull = [&](int l, int b) { return smem_u32(bar + bar_base(l) + b); };
    auto xempty = [&](int l, int b) { return smem_u32(bar + bar_base(l) + kNBuf + b); };
    auto afull = [&](int l, int j) { return smem_u32(bar + bar_base(l) + 2 * kNBuf + j); };
    auto aempty = [&](int l, int j) { return smem_u32(bar + bar_base(l) + 2 * kNBuf + depth_of(l) + j); };
    auto xbuf = [&](int l, int b) {  // input row buffer b of layer l
        return l == 1 ? kOffX0 + (uint32_t)b * kRowX0 : kOffX + ((uint32_t)(l - 2) * kNBuf + b) * kRowX;
    };

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(s_tmem)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int l = 1; l <= 4; ++l) {
            for (int b = 0; b < kNBuf; ++b) {
                asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(xfull(l, b)), "r"(kLanes));
                asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(xempty(l, b)));
            }
            for (int j = 0; j < depth_of(l); ++j) {
                asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(afull(l, j)));
                asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(aempty(l, j)), "r"(kLanes));
            }
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 4;" ::"r"(drain));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *s_fail = 0;
    }
    // weights image and zeroed activation buffers
    for (uint32_t i = tid * 16; i < kImage; i += kThreads * 16)
        *reinterpret_cast<uint4 *>(smem + i) = *reinterpret_cast<const uint4 *>(a.image + i);
    for (uint32_t i = kOffX0 + tid * 16; i < kOffBar; i += kThreads * 16)
        *reinterpret_cast<uint4 *>(smem + i) = make_uint4(0, 0, 0, 0);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *s_tmem;
    const uint32_t tl = tmem + ((uint32_t)((warp & 3) * 32) << 16);  // epilogue thread's lane quarter
    if (tid < kEpi) {
        for (int c = 128 * grp; c < 128 * grp + 128; c += 32) tzero32(tl + c);
        wait_st();
    }
    const float *bias = reinterpret_cast<const float *>(smem + kOffBias);
    Waiter wt{s_fail, a.err};
    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    if (tid >= kEpi) {
        // ================= MMA warp of layer l: for each input row s, wait for the row and for the
        // ring slot it starts (row s+1's, last used by row s+1-depth), issue, then commit to the row
        // buffer's release and to "row s-1 complete"
        const int l = ((tid - kEpi) >> 5) + 1;
        const int D = depth_of(l);
        uint32_t use[kNBuf] = {0, 0, 0}, ce[kDepth4];
        for (int j = 0; j < kDepth4; ++j) ce[j] = 0;
        const uint32_t dacc = tmem + acc_col(l - 1);
        uint64_t adb[kNBuf];
        for (int b = 0; b < kNBuf; ++b) adb[b] = make_desc(sbase + xbuf(l, b), kPlane, 128);
        const uint64_t bd0 = l < 4 ? make_desc(sbase + (l == 1 ? kOffB1 : (l == 2 ? kOffB2 : kOffB3)), kBChunk, 128)
                                   : make_desc(sbase + kOffB4, kB4Chunk, 128);
        for (int tile = blockIdx.x; tile < a.ntiles && !*s_fail; tile += gridDim.x) {
            int lo[5], hi[5], strip, f;
            tile_rows(a, tile, lo, hi, strip, f);
            const int L = lo[l - 1], H = hi[l - 1];
            const bool top_ok = lo[l] == 0, bot_ok = hi[l] == nt;
            for (int s = L; s < H && !*s_fail; ++s) {
                const int b = s % kNBuf;
                wt.wait(xfull(l, b), use[b]++);
                if (s + 1 - D >= L - 1) {
                    const int j = (s + 1) & (D - 1);
                    wt.wait(aempty(l, j), ce[j]++);
                }
                {
                    const int c = (s - 1) & (D - 1);
                    const uint64_t ad0 = b == 0 ? adb[0] : (b == 1 ? adb[1] : adb[2]);
                    const bool top = s == 1 && top_ok, bot = s == nt - 2 && bot_ok;
                    const int oslot = (nt - 1) & (D - 1);
                    const bool go = !*s_fail;
                    switch (l) {
                        case 1: {
                            const RowOps<1> ops(dacc, ad0, bd0, c);
                            if (go && elect_one()) {
                                tc_fence_after();
                                ops.issue();
                                if (top) issue_pole<1>(dacc, ad0, sbase, true, 0);
                                if (bot) issue_pole<1>(dacc, ad0, sbase, false, oslot);
                                commit(xempty(l, b));
                                commit(afull(l, c));
                            }
                            break;
                        }
                        case 2: {
                            const RowOps<2> ops(dacc, ad0, bd0, c);
                            if (go && elect_one()) {
                                tc_fence_after();
                                ops.issue();
                                if (top) issue_pole<2>(dacc, ad0, sbase, true, 0);
                                if (bot) issue_pole<2>(dacc, ad0, sbase, false, oslot);
                                commit(xempty(l, b));
                                commit(afull(l, c));
                            }
                            break;
                        }
                        case 3: {
                            const RowOps<3> ops(dacc, ad0, bd0, c);
                            if (go && elect_one()) {
                                tc_fence_after();
                                ops.issue();
                                if (top) issue_pole<3>(dacc, ad0, sbase, true, 0);
                                if (bot) issue_pole<3>(dacc, ad0, sbase, false, oslot);
                                commit(xempty(l, b));
                                commit(afull(l, c));
                            }
                            break;
                        }
                        default: {
                            const RowOps<4> ops(dacc, ad0, bd0, c);
                            if (go && elect_one()) {
                                tc_fence_after();
                                ops.issue();
                                if (top) issue_pole<4>(dacc, ad0, sbase, true, 0);
                                if (bot) issue_pole<4>(dacc, ad0, sbase, false, oslot);
                                commit(xempty(l, b));
                                commit(afull(l, c));
                            }
                            break;
                        }
                    }
                }
                __syncwarp();
            }
            // rows H-1 and H are complete with the last row's MMAs
            if (!*s_fail && elect_one()) {
                commit(afull(l, (H - 1) & (D - 1)));
                commit(afull(l, H & (D - 1)));
            }
            __syncwarp();
            // the epilogue of the slots the next tile starts on
            for (int r = max(L - 1, H - D + 1); r <= H; ++r) {
                const int j = r & (D - 1);
                wt.wait(aempty(l, j), ce[j]++);
            }
            tc_fence_after();
        }
        // completes when every MMA this warp issued has finished
        if (elect_one()) commit(drain);
        __syncwarp();
    } else if (grp < 3) {
        // ================= epilogue of layer l = grp + 1, producer of layer l+1's input rows
        const int l = grp + 1;
        uint32_t ca[kDepth] = {0, 0, 0, 0}, fills[kNBuf] = {0, 0, 0};
        for (int tile = blockIdx.x; tile < a.ntiles && !*s_fail; tile += gridDim.x) {
            int lo[5], hi[5], strip, f;
            tile_rows(a, tile, lo, hi, strip, f);
            for (int r = lo[l - 1] - 1; r <= hi[l - 1] && !*s_fail; ++r) {
                const int j = r & (kDepth - 1);
                wt.wait(afull(l, j), ca[j]++);
                tc_fence_after();
                const uint32_t ta = tl + acc_col(l - 1) + 32 * j;
                uint32_t v[32];
                tld32(ta, v);
                wait_ld();
#pragma unroll
                for (int k = 0; k < 32; ++k) pin(v[k]);
                tzero32(ta);  // completes while the GELUs run (waited below)
                if (r >= lo[l] && r < hi[l]) {
                    const int bx = r % kNBuf;
                    if (fills[bx] > 0) wt.wait(xempty(l + 1, bx), fills[bx] - 1);  // previous row consumed
                    const float *bl_ = bias + 32 * (l - 1);
                    uint8_t *dst = smem + xbuf(l + 1, bx) + (lane + 1) * 16;
#pragma unroll
                    for (int pl = 0; pl < 4; ++pl) {
                        uint4 o;
                        uint32_t *ow = reinterpret_cast<uint32_t *>(&o);
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int c = pl * 8 + 2 * e;
                            const float2 y = __fadd2_rn(make_float2(__uint_as_float(v[c]), __uint_as_float(v[c + 1])),
                                                        make_float2(bl_[c], bl_[c + 1]));
                            const float2 gy = gelu2(y);
                            ow[e] = pack2(gy.x, gy.y);
                        }
                        *reinterpret_cast<uint4 *>(dst + pl * kPlane) = o;
                    }
                    fills[bx]++;
                    fence_async_smem();
                    mbar_arrive(xfull(l + 1, bx));
                }
                wait_st();
                tc_fence_before();
                mbar_arrive(aempty(l, j));
            }
        }
    } else {
        // ================= warpgroup 3: features (input rows of layer 1), running 8 rows ahead of the
        // layer-4 epilogue (output rows)
        uint32_t ca[kDepth4], fills[kNBuf] = {0, 0, 0};
        for (int j = 0; j < kDepth4; ++j) ca[j] = 0;
        for (int tile = blockIdx.x; tile < a.ntiles && !*s_fail; tile += gridDim.x) {
            int lo[5], hi[5], strip, f;
            tile_rows(a, tile, lo, hi, strip, f);
            const Field &fd = a.fs.f[f];
            const int xcol = strip * kOut - kHalo + lane;  // this lane's column (before wrap)
            const int col = ((xcol % np) + np) % np;
            const bool lane_out = lane >= kHalo && lane < kHalo + kOut && strip * kOut + (lane - kHalo) < np;
            const int cw = col == 0 ? np - 1 : col - 1, ce_ = col + 1 == np ? 0 : col + 1;
            constexpr int kLead = 8;
            const int nfeat = hi[0] - lo[0], nepi = hi[3] - lo[3] + 2;
            FeatIn pre;
            if (nfeat > 0) feat_load(pre, lo[0], nt, fd, a.g, col, cw, ce_);
            float hout = 0.f;
            for (int t = 0; t < max(nfeat, nepi + kLead) && !*s_fail; ++t) {
                if (t < nfeat) {
                    const int srow = lo[0] + t, b = srow % kNBuf;
                    if (fills[b] > 0) wt.wait(xempty(1, b), fills[b] - 1);
                    feat_store(pre, fd, a.g, smem + xbuf(1, b), lane);
                    fills[b]++;
                    fence_async_smem();
                    mbar_arrive(xfull(1, b));
                    if (t + 1 < nfeat) feat_load(pre, srow + 1, nt, fd, a.g, col, cw, ce_);
                }
                const int te = t - kLead;
                if (te >= 0 && te < nepi) {
                    const int r = lo[3] - 1 + te;
                    const bool emit = r >= lo[4] && r < hi[4];
                    if (emit && lane_out) hout = fd.h[(size_t)r * fd.pitch + col];
                    const int j = r & (kDepth4 - 1);
                    wt.wait(afull(4, j), ca[j]++);
                    tc_fence_after();
                    const uint32_t ta = tl + acc_col(3) + j;
                    uint32_t yv = tld1(ta);
                    wait_ld();
                    pin(yv);
                    tzero1(ta);
                    const float y = __fadd_rn(__uint_as_float(yv), bias[96]);
                    if (emit && lane_out) {
                        if (a.y_out) a.y_out[((size_t)f * nt + r) * np + col] = y;
                        if (a.h_out) {
                            float o = hout;
                            if (r > 0 && r + 1 < nt) o = fmaxf(__fadd_rn(hout, __fmul_rn(fd.kout, y)), 0.f);
                            a.h_out[(size_t)r * a.pitch_out + col] = o;
                        }
                    }
                    wait_st();
                    tc_fence_before();
                    mbar_arrive(aempty(4, j));
                }
            }
        }
    }
    __syncthreads();
    // no MMA may still write the accumulators when the columns are released
    if (tid == 0 && !mbar_wait_bounded(drain, 0u)) atomicOr(a.err, 1u);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
}

// Packs the parameter vector into the shared-memory image of fused_kernel.
__global__ void pack_fused_kernel(const float *theta, uint8_t *img) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int dy_of_block[3] = {1, 0, -1};
    bf16 *B = reinterpret_cast<bf16 *>(img);
    // layers 1-3: element (step, chunk, row n, e8); layer 1 step = dx, chunk = 8-feature plane
    const int per1 = 3 * 2 * kBRows * 8, per23 = 6 * 2 * kBRows * 8;
    if (e < per1) {
        const int e8 = e % 8, n = (e / 8) % kBRows, ch = (e / (8 * kBRows)) % 2, st = e / (16 * kBRows);
        const int dy = dy_of_block[n / 32], oc = n % 32, dx = st - 1;
        const float v = theta[SBS_NN_W1 + (((dy + 1) * 3 + (dx + 1)) * 32 + oc) * 16 + ch * 8 + e8];
        B[(kOffB1 + st * kBStep + ch * kBChunk) / 2 + n * 8 + e8] = __float2bfloat16_rn(v);
    }
    if (e < per23) {
        const int e8 = e % 8, n = (e / 8) % kBRows, ch = (e / (8 * kBRows)) % 2, st = e / (16 * kBRows);
        const int dy = dy_of_block[n / 32], oc = n % 32, dx = (st >> 1) - 1, kk = st & 1;
        const int ic = kk * 16 + ch * 8 + e8, t = (dy + 1) * 3 + (dx + 1);
        const size_t o = (size_t)(st * kBStep + ch * kBChunk) / 2 + n * 8 + e8;
        B[kOffB2 / 2 + o] = __float2bfloat16_rn(theta[SBS_NN_W2 + (t * 32 + oc) * 32 + ic]);
        B[kOffB3 / 2 + o] = __float2bfloat16_rn(theta[SBS_NN_W3 + (t * 32 + oc) * 32 + ic]);
    }
    // layer 4: rows 15, 16, 17 = dy +1, 0, -1 (all other rows zero)
    if (e < 6 * 2 * kB4Rows * 8) {
        const int e8 = e % 8, n = (e / 8) % kB4Rows, ch = (e / (8 * kB4Rows)) % 2, st = e / (16 * kB4Rows);
        const int dx = (st >> 1) - 1, kk = st & 1, ic = kk * 16 + ch * 8 + e8;
        float v = 0.f;
        if (n >= 15 && n <= 17) v = theta[SBS_NN_W4 + ((1 - (n - 15) + 1) * 3 + (dx + 1)) * 32 + ic];
        B[(kOffB4 + st * kB4Step + ch * kB4Chunk) / 2 + n * 8 + e8] = __float2bfloat16_rn(v);
    }
    if (e < 6 * 2 * kBxRows * 8) {
        const int e8 = e % 8, n = (e / 8) % kBxRows, ch = (e / (8 * kBxRows)) % 2, st = e / (16 * kBxRows);
        const int dx = (st >> 1) - 1, kk = st & 1, ic = kk * 16 + ch * 8 + e8;
        float vt = 0.f, vb = 0.f;
        if (n == 15) {
            vt = theta[SBS_NN_W4 + (0 * 3 + (dx + 1)) * 32 + ic];  // dy = -1
            vb = theta[SBS_NN_W4 + (2 * 3 + (dx + 1)) * 32 + ic];  // dy = +1
        }
        B[(kOffB4t + st * kBxStep + ch * kBxChunk) / 2 + n * 8 + e8] = __float2bfloat16_rn(vt);
        B[(kOffB4b + st * kBxStep + ch * kBxChunk) / 2 + n * 8 + e8] = __float2bfloat16_rn(vb);
    }
    float *bias = reinterpret_cast<float *>(img + kOffBias);
    if (e < 128) {
        float v = 0.f;
        if (e < 32)
            v = theta[SBS_NN_B1 + e];
        else if (e < 64)
            v = theta[SBS_NN_B2 + e - 32];
        else if (e < 96)
            v = theta[SBS_NN_B3 + e - 64];
        else if (e == 96)
            v = theta[SBS_NN_B4];
        bias[e] = v;
    }
}

struct FusedState {
    uint8_t *image = nullptr;
    unsigned *err = nullptr;
};

}  // namespace

int fused_pack(sbs_surrogate *s) {
    FusedState *fs = reinterpret_cast<FusedState *>(*fused_slot(s));
    if (!fs) {
        fs = new FusedState();
        *fused_slot(s) = fs;
        if (cudaMalloc(&fs->image, kImage) != cudaSuccess || cudaMalloc(&fs->err, sizeof(unsigned)) != cudaSuccess)
            return set_error(SBS_E_NOMEM, "fused weight image allocation failed");
        SBS_CUDA_TRY(cudaFuncSetAttribute(fused_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem));
    }
    const int n = 6 * 2 * kBRows * 8;  // the largest element count of the image's parts
    pack_fused_kernel<<<(n + 255) / 256, 256, 0, stream_of(s)>>>(theta_of(s), fs->image);
    SBS_CUDA_TRY(cudaGetLastError());
    *fused_dirty_flag(s) = 0;
    return SBS_OK;
}

void fused_release(sbs_surrogate *s) {
    FusedState *fs = reinterpret_cast<FusedState *>(*fused_slot(s));
    if (!fs) return;
    cudaFree(fs->image);
    cudaFree(fs->err);
    delete fs;
    *fused_slot(s) = nullptr;
}

int fused_forward(sbs_surrogate *s, const Fields &fields, int nf, const GridTab &g, float *hout, size_t pitch_out,
                  float *y_out) {
    if (*fused_dirty_flag(s) || !*fused_slot(s)) {
        int rc = fused_pack(s);
        if (rc) return rc;
    }
    FusedState *st = reinterpret_cast<FusedState *>(*fused_slot(s));
    SBS_CHECK_ARG(hout == nullptr || nf == 1, "the fused update writes one field");
    FusedArgs a{};
    a.fs = fields;
    a.g = g;
    a.image = st->image;
    a.y_out = y_out;
    a.h_out = hout;
    a.pitch_out = pitch_out;
    a.nf = nf;
    a.nstrips = (g.np + kOut - 1) / kOut;
    a.err = st->err;
    // rows per block: the smallest block count whose tile count fills the grid evenly (>= 16 rows)
    const int sms = std::max(1, sms_of(s));
    const int per_field = a.nstrips;
    int best_nrb = 1;
    double best = 1e30;
    for (int nrb = 1; nrb <= std::max(1, g.nt / 16); ++nrb) {
        const int tiles = per_field * nrb * nf;
        const int waves = (tiles + sms - 1) / sms;
        const double rows = (double)g.nt / nrb + 16.0;  // streamed rows per tile incl. fill and halo
        const double cost = waves * rows;
        if (cost < best - 1e-9) {
            best = cost;
            best_nrb = nrb;
        }
    }
    a.nrb = best_nrb;
    a.rows_per_block = (g.nt + best_nrb - 1) / best_nrb;
    a.nrb = (g.nt + a.rows_per_block - 1) / a.rows_per_block;
    a.ntiles = a.nstrips * a.nrb * nf;
    const int grid = std::min(a.ntiles, sms);
    cudaStream_t stream = stream_of(s);
    SBS_CUDA_TRY(cudaMemsetAsync(st->err, 0, sizeof(unsigned), stream));
    fused_kernel<<<grid, kThreads, kSmem, stream>>>(a);
    SBS_CUDA_TRY(cudaGetLastError());
    unsigned herr = 0;
    SBS_CUDA_TRY(cudaMemcpyAsync(&herr, st->err, sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(stream));
    if (herr) return set_error(SBS_E_TIMEOUT, "fused surrogate kernel: a tensor-core wait timed out");
    return SBS_OK;
}

}  // namespace nn
}  // namespace sbs
