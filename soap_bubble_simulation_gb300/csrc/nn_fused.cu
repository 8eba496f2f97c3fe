// Fused forward pass of the drainage surrogate (include/sbs_nn.h) on the tcgen05 tensor cores:
// features, the four 3x3 convolutions, activations and the thickness update in one persistent kernel,
// activations kept in shared memory and accumulators in tensor memory.
//
// Tiling. A tile is a strip of 128 consecutive phi columns (lanes; the middle 120 are output, the
// 4 on each side are the halo the four layers consume) times a block of theta rows of one field.
// The block runs nine agents that only talk through mbarriers: four MMA warps (one per layer:
// for each input row, wait for the row and for the accumulator slot it starts, issue, commit),
// three epilogue warpgroups (warpgroup l-1 reads layer l's finished row from TMEM, restarts the
// slot from the bias at once, then applies the activation and writes the row into
// one of four input buffers of layer l+1), a feature warpgroup (the input rows of layer 1) and an
// output warpgroup (layer 4's rows: y and the thickness update). Every ring (activation buffers:
// full / empty; accumulator rows: full / empty) is balanced per tile, so each waiter is at most
// one phase behind and parity waits are exact. The block streams its rows top to bottom through
// all four layers at once, each layer as far behind the one before as its inputs require.
// The epilogue and the MMA loop are one code copy each for all layers (the layer is a runtime
// value): separate instantiations of these unrolled bodies cost ~30 % in instruction-cache misses.
//
// Convolution as MMAs. Activations of one row live in shared memory as planes of 8 channels with
// 16 B per cell (K-major, rows of the A operand = cells, SBO = 128 B), so the dx = -1/0/+1 taps
// are the same tile read at start offsets of 16 B apart: no im2col buffer. The three dy taps are
// stacked along N: one M=128 x N=96 MMA multiplies an input row by the three dy blocks of W and
// accumulates into a ring of three 32-column slots (output row r lives in slot r mod 3). B holds
// the blocks as [W+1; W0; W-1; W+1; W0]; the window of three blocks that starts at (1 - s) mod 3
// lines them up with the slots of rows s-1, s, s+1, so every input row is one N=96 MMA per K step
// whatever its position in the ring. A slot is read by the epilogue once its row's three input
// rows are in, then zeroed for reuse; the next row's MMAs wait for that (the ring has no spare
// slot), and the other layers' MMAs keep the tensor pipe busy meanwhile. theta reflection at the poles adds one
// N=32 MMA (input row 1 into output row 0 with W-1, input row nt-2 into output row nt-1 with W+1).
// Operand bandwidth: an N=96 MMA reads 4 KB of A and 3 KB of B from shared memory (~56 cycles at
// 128 B/clk), which is the measured issue-to-issue time of back-to-back MMAs of this shape.
//
// TMEM columns: layer 1 [0, 96), layer 2 [128, 224), layer 3 [256, 352), layer 4 [384, 400)
// (a ring of 16 single columns; the N=16 MMA always writes columns 384..399 and B places the three
// dy weight rows at the right columns by its window offset). Every MMA's D column is a multiple of
// 16. One CTA per SM (it allocates all 512 columns).
// Because every layer-4 MMA also adds exact zeros to the 13 columns it does not own, no column of
// that ring may be zeroed while a layer-4 MMA is in flight (the MMA's read-modify-write could put
// the old value back). The output warpgroup therefore never zeroes a column inside a tile: it
// reads the running sum and subtracts its previous reading of the column (kept in shared memory),
// and it zeroes the whole ring at the end of the tile, when every MMA of the tile has completed
// (the last row's completion barrier is committed after them) and before it releases the last
// slot. Tiles are at most 256 rows, so a column sums at most 17 rows (FP32 error ~1e-6 relative).
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
int act_of(sbs_surrogate *s);

namespace {

constexpr int kLanes = 128;                    // TMEM lanes = cells of a strip
constexpr int kGroups = 4;                     // warpgroups: each owns one 8-channel plane
constexpr int kEpi = kLanes * kGroups;         // epilogue + feature threads (16 warps)
constexpr int kOutT = kEpi + kLanes;           // + the layer-4 epilogue warpgroup
constexpr int kThreads = kOutT + 4 * 32;       // + one MMA-issuing warp per layer
constexpr int kOut = 120;                      // output columns per strip
constexpr int kHalo = 4;                       // lanes on each side of the outputs
constexpr int kCells = 136;                    // staged cells per plane (q = lane + 1)
constexpr uint32_t kPlane = kCells * 16;       // 2176 B
constexpr uint32_t kRowX = 4 * kPlane;         // one 32-channel row buffer
constexpr uint32_t kRowX0 = 2 * kPlane;        // one 16-feature row buffer
constexpr uint32_t kBRows = 160;               // dy blocks [W+1; W0; W-1; W+1; W0] (5 x 32 rows)
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
constexpr int kDepth = 3, kDepth4 = 16;
__host__ __device__ constexpr int depth_of(int l) { return l < 4 ? kDepth : kDepth4; }  // l 1-based
__host__ __device__ constexpr uint32_t acc_col(int l) { return 128u * (uint32_t)l; }    // l 0-based; 3 -> 384
static_assert(acc_col(3) + 16 <= 512, "TMEM columns");
// ring slot of row r >= -D
template <int D>
__device__ __forceinline__ int ring(int r) { return (r + D) % D; }
// rest of shared memory
constexpr int kNBuf = 4;                                   // activation rows in flight per layer input
static_assert((kNBuf & (kNBuf - 1)) == 0, "kNBuf is a power of two");
constexpr uint32_t kOffX0 = (kImage + 1023) / 1024 * 1024;  // feature rows
constexpr uint32_t kOffX = kOffX0 + kNBuf * kRowX0;         // 3 layers x kNBuf rows
constexpr uint32_t kOffBar = kOffX + 3 * kNBuf * kRowX;
// barriers of layer l: xfull[kNBuf], xempty[kNBuf], afull[depth], aempty[depth]
__host__ __device__ constexpr int bar_base(int l) { return (l - 1) * (2 * kNBuf + 2 * kDepth); }
constexpr int kNumBars = 3 * (2 * kNBuf + 2 * kDepth) + 2 * kNBuf + 2 * kDepth4;
// + the exit drain barrier, the TMEM base and the fail flag; then the layer-4 epilogue's previous
// readings [16 columns][128 lanes]
constexpr uint32_t kOffPrev = (kOffBar + 8 * (kNumBars + 1) + 64 + 15) / 16 * 16;
constexpr uint32_t kSmem = kOffPrev + kDepth4 * kLanes * 4;
constexpr int kMaxTileRows = 256;
static_assert(kSmem <= 227 * 1024, "shared memory per CTA");
// try_wait may suspend the thread until the phase completes or this many ns pass (waiting warps
// then take no issue slots from the working ones)
constexpr uint32_t kSuspendNs = 1000000;

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
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity), "r"(kSuspendNs)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase; false after `limit` cycles (sbs_set_wait_limit).
__device__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, long long limit) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > limit) return false;
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

__device__ __forceinline__ void tzero16(uint32_t taddr) {
    const uint32_t z = 0;
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, "
        "%1};" ::"r"(taddr),
        "r"(z)
        : "memory");
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
    int act;  // SBS_NN_ACT_*
    unsigned *err;
    long long wait_cycles;  // bound on every mbarrier wait
    int stall;              // 1 (the timeout test): the MMA warps issue neither MMAs nor commits
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
            // one N=96 MMA over the whole ring: the B window starting at block (3 - c) mod 3 of
            // [W+1; W0; W-1; W+1; W0] puts W+1 at slot c (row s-1), W0 at slot c+1 (row s) and W-1 at
            // slot c+2 (row s+1), mod 3
            static_assert(kDepth == 3, "the rotated B window covers a ring of three slots");
            two = false;
            d1 = d2 = dacc;
            i1 = i2 = idesc(96);
            const uint64_t blk = (uint64_t)(((3 - c) % 3) * (kBlk >> 4));
#pragma unroll
            for (int st = 0; st < NS; ++st) {
                const int dxi = L == 1 ? st : st >> 1, kk = L == 1 ? 0 : st & 1;
                ad[st] = ad0 + (uint64_t)((2 * kk * kPlane + 16 * dxi) >> 4);
                b1[st] = bd0 + (uint64_t)((st * kBStep) >> 4) + blk;
                b2[st] = b1[st];
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

// Writes layer bias b[0..31] into the 32 columns at taddr (every lane of the warp's quarter): the
// accumulator of a row then starts at the bias and the MMAs add onto it.
__device__ __forceinline__ void tset_bias(uint32_t taddr, const float *b) {
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const float4 u = *reinterpret_cast<const float4 *>(b + 4 * k);
        asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1, %2, %3, %4};" ::"r"(taddr + 4 * k), "f"(u.x),
                     "f"(u.y), "f"(u.z), "f"(u.w)
                     : "memory");
    }
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// Per-thread phase tracking of one barrier: waits for completion number `count` (0, 1, ...).
struct Waiter {
    volatile int *fail;
    unsigned *err;
    long long limit;
    __device__ __forceinline__ void wait(uint32_t bar, uint32_t count) {
        if (*fail) return;
        if (!mbar_wait_bounded(bar, count & 1u, limit)) {
            atomicOr(err, 1u);
            *fail = 1;
        }
    }
};

// Rows of one tile: the block's output rows are [y0, y1); layer l (0 = features) needs rows
// [lo(l), hi(l)) of its input. Computed on demand (an array indexed by a runtime layer would live
// in local memory).
struct TileRows {
    int y0, y1, nt, strip, f;
    __device__ __forceinline__ TileRows(const FusedArgs &a, int tile) : nt(a.g.nt) {
        strip = tile % a.nstrips;
        const int rb = (tile / a.nstrips) % a.nrb;
        f = tile / (a.nstrips * a.nrb);
        y0 = rb * a.rows_per_block;
        y1 = min(nt, y0 + a.rows_per_block);
    }
    __device__ __forceinline__ int lo(int l) const { return max(0, y0 - 4 + l); }
    __device__ __forceinline__ int hi(int l) const { return min(nt, y1 + 4 - l); }
};

// Barriers of layer l (1-based): input-row buffers of layer l (full: written by the producer
// warpgroup, empty: released by layer l's MMAs) and accumulator ring slots (full: the slot's row
// has all its contributions, empty: its epilogue has read and zeroed it).
struct Bars {
    uint32_t base;  // shared-memory address of barrier 0
    __device__ __forceinline__ uint32_t xfull(int l, int b) const { return base + 8u * (bar_base(l) + b); }
    __device__ __forceinline__ uint32_t xempty(int l, int b) const { return base + 8u * (bar_base(l) + kNBuf + b); }
    __device__ __forceinline__ uint32_t afull(int l, int j) const { return base + 8u * (bar_base(l) + 2 * kNBuf + j); }
    __device__ __forceinline__ uint32_t aempty(int l, int j) const {
        return base + 8u * (bar_base(l) + 2 * kNBuf + depth_of(l) + j);
    }
};

// Byte offset of input row buffer b of layer l (1-based).
__host__ __device__ constexpr uint32_t xbuf(int l, int b) {
    return l == 1 ? kOffX0 + (uint32_t)b * kRowX0 : kOffX + ((uint32_t)(l - 2) * kNBuf + b) * kRowX;
}

// Phase parity of each barrier of a ring, one bit per barrier: wait on the bit, then flip it.
__device__ __forceinline__ uint32_t take(uint32_t &bits, int i) {
    const uint32_t p = (bits >> i) & 1u;
    bits ^= 1u << i;
    return p;
}

// Layer-specific MMAs of one input row, issued by one elected lane, then the commits that release
// the row buffer (xempty) and mark row s-1 complete (afull).
template <int L>
__device__ __forceinline__ void issue_row(uint32_t dacc, uint64_t ad0, uint64_t bd0, int c, uint32_t sbase, bool top,
                                          bool bot, int oslot, uint32_t xempty, uint32_t afull) {
    const RowOps<L> ops(dacc, ad0, bd0, c);
    if (elect_one()) {
        tc_fence_after();
        ops.issue();
        if (top) issue_pole<L>(dacc, ad0, sbase, true, 0);
        if (bot) issue_pole<L>(dacc, ad0, sbase, false, oslot);
        commit(xempty);
        commit(afull);
    }
}

// MMA warp of layer L: for each input row s, wait for the row and for the ring slot it starts (row
// s+1's, last used by row s+1-D), issue, then commit to the row buffer's release and to "row s-1
// complete". One loop for all four layers; only the issue differs.
__device__ void mma_agent(const int L, const FusedArgs &a, const Bars &bars, uint32_t tmem, uint32_t sbase, Waiter &wt,
                          volatile int *s_fail) {
    const int D = depth_of(L);
    const int nt = a.g.nt;
    const uint32_t row_step = (L == 1 ? kRowX0 : kRowX) >> 4;  // descriptor units between buffers
    const uint32_t dacc = tmem + acc_col(L - 1);
    const uint64_t adb = make_desc(sbase + xbuf(L, 0), kPlane, 128);
    const uint64_t bd0 = L < 4 ? make_desc(sbase + (L == 1 ? kOffB1 : (L == 2 ? kOffB2 : kOffB3)), kBChunk, 128)
                               : make_desc(sbase + kOffB4, kB4Chunk, 128);
    auto slot = [D](int r) { return D == kDepth ? ring<kDepth>(r) : ring<kDepth4>(r); };
    uint32_t xph = 0, eph = 0;
    for (int tile = blockIdx.x; tile < a.ntiles && !*s_fail; tile += gridDim.x) {
        const TileRows tr(a, tile);
        const int R0 = tr.lo(L - 1), H = tr.hi(L - 1);
        const bool top_ok = tr.lo(L) == 0, bot_ok = tr.hi(L) == nt;
        const int oslot = slot(nt - 1);
        for (int s = R0; s < H && !*s_fail; ++s) {
            const int b = s & (kNBuf - 1);
            wt.wait(bars.xfull(L, b), take(xph, b));
            if (s + 1 - D >= R0 - 1) {
                const int j = slot(s + 1);
                wt.wait(bars.aempty(L, j), take(eph, j));
            }
            const int c = slot(s - 1);
            const uint64_t ad0 = adb + (uint64_t)((uint32_t)b * row_step);
            const bool top = s == 1 && top_ok, bot = s == nt - 2 && bot_ok;
            if (!*s_fail && !a.stall) {
                const uint32_t xe = bars.xempty(L, b), af = bars.afull(L, c);
                switch (L) {
                    case 1: issue_row<1>(dacc, ad0, bd0, c, sbase, top, bot, oslot, xe, af); break;
                    case 2: issue_row<2>(dacc, ad0, bd0, c, sbase, top, bot, oslot, xe, af); break;
                    case 3: issue_row<3>(dacc, ad0, bd0, c, sbase, top, bot, oslot, xe, af); break;
                    default: issue_row<4>(dacc, ad0, bd0, c, sbase, top, bot, oslot, xe, af); break;
                }
            }
            __syncwarp();
        }
        // rows H-1 and H are complete with the last row's MMAs
        if (!*s_fail && !a.stall && elect_one()) {
            commit(bars.afull(L, slot(H - 1)));
            commit(bars.afull(L, slot(H)));
        }
        __syncwarp();
        // the epilogue of the slots the next tile starts on
        for (int r = max(R0 - 1, H - D + 1); r <= H; ++r) {
            const int j = slot(r);
            wt.wait(bars.aempty(L, j), take(eph, j));
        }
        tc_fence_after();
    }
}

// A finished row's 32 activations (slot values already include the bias) as four BF16 planes.
template <int ACT>
__device__ __forceinline__ void store_row(const uint32_t *v, uint8_t *dst) {
#pragma unroll
    for (int pl = 0; pl < 4; ++pl) {
        uint4 o;
        uint32_t *ow = reinterpret_cast<uint32_t *>(&o);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int c = pl * 8 + 2 * e;
            const float2 y = make_float2(__uint_as_float(v[c]), __uint_as_float(v[c + 1]));
            const float2 gy = ACT == SBS_NN_ACT_HSWISH ? hswish2(y) : gelu2(y);
            ow[e] = pack2(gy.x, gy.y);
        }
        *reinterpret_cast<uint4 *>(dst + pl * kPlane) = o;
    }
}

// One code copy serves the three warpgroups (L is a runtime value): the epilogue is the largest
// code of the kernel, and three instantiations cost instruction-cache misses.
__device__ void epi_agent(const int L, const FusedArgs &a, const Bars &bars, uint8_t *smem, uint32_t tl, int lane,
                          const float *bias, Waiter &wt, volatile int *s_fail) {
    constexpr int D = kDepth;
    uint32_t aph = 0, pph = 0, used = 0;
    const float *bl_ = bias + 32 * (L - 1);
    for (int tile = blockIdx.x; tile < a.ntiles && !*s_fail; tile += gridDim.x) {
        const TileRows tr(a, tile);
        const int r_end = tr.hi(L - 1), o_lo = tr.lo(L), o_hi = tr.hi(L);
        for (int r = tr.lo(L - 1) - 1; r <= r_end && !*s_fail; ++r) {
            const int j = ring<D>(r);
            wt.wait(bars.afull(L, j), take(aph, j));
            tc_fence_after();
            const uint32_t ta = tl + acc_col(L - 1) + 32 * j;
            uint32_t v[32];
            tld32(ta, v);
            wait_ld();
#pragma unroll
            for (int k = 0; k < 32; ++k) pin(v[k]);
            tset_bias(ta, bl_);  // the slot's next row starts from the bias
            wait_st();
            tc_fence_before();
            mbar_arrive(bars.aempty(L, j));  // the slot is free before the activations run
            if (r >= o_lo && r < o_hi) {
                const int bx = r & (kNBuf - 1);
                if ((used >> bx) & 1u) wt.wait(bars.xempty(L + 1, bx), ((pph >> bx) & 1u) ^ 1u);  // previous row consumed
                used |= 1u << bx;
                pph ^= 1u << bx;
                uint8_t *dst = smem + xbuf(L + 1, bx) + (lane + 1) * 16;
                if (a.act == SBS_NN_ACT_HSWISH)
                    store_row<SBS_NN_ACT_HSWISH>(v, dst);
                else
                    store_row<SBS_NN_ACT_GELU>(v, dst);
                fence_async_smem();
                mbar_arrive(bars.xfull(L + 1, bx));
            }
        }
    }
}

// The lane's column in the field and whether it is one of the strip's output columns.
struct LaneCol {
    int col, cw, ce;
    bool out;
    __device__ __forceinline__ LaneCol(int strip, int lane, int np) {
        const int xcol = strip * kOut - kHalo + lane;  // before wrap
        col = ((xcol % np) + np) % np;
        out = lane >= kHalo && lane < kHalo + kOut && strip * kOut + (lane - kHalo) < np;
        cw = col == 0 ? np - 1 : col - 1;
        ce = col + 1 == np ? 0 : col + 1;
    }
};

// Warpgroup 3: the features of every input row of layer 1, each row's inputs loaded a row ahead.
__device__ void feature_agent(const FusedArgs &a, const Bars &bars, uint8_t *smem, int lane, Waiter &wt,
                              volatile int *s_fail) {
    const int nt = a.g.nt;
    uint32_t pph = 0, used = 0;
    for (int tile = blockIdx.x; tile < a.ntiles && !*s_fail; tile += gridDim.x) {
        const TileRows tr(a, tile);
        const Field &fd = a.fs.f[tr.f];
        const LaneCol lc(tr.strip, lane, a.g.np);
        const int r0 = tr.lo(0), r1 = tr.hi(0);
        FeatIn pre;
        if (r1 > r0) feat_load(pre, r0, nt, fd, a.g, lc.col, lc.cw, lc.ce);
        for (int srow = r0; srow < r1 && !*s_fail; ++srow) {
            const int b = srow & (kNBuf - 1);
            if ((used >> b) & 1u) wt.wait(bars.xempty(1, b), ((pph >> b) & 1u) ^ 1u);
            used |= 1u << b;
            pph ^= 1u << b;
            feat_store(pre, fd, a.g, smem + xbuf(1, b), lane);
            fence_async_smem();
            mbar_arrive(bars.xfull(1, b));
            if (srow + 1 < r1) feat_load(pre, srow + 1, nt, fd, a.g, lc.col, lc.cw, lc.ce);
        }
    }
}

// Warpgroup 4: the layer-4 epilogue (output rows: y and the thickness update).
__device__ void output_agent(const FusedArgs &a, const Bars &bars, uint8_t *smem, uint32_t tl, int lane,
                             const float *bias, Waiter &wt, volatile int *s_fail) {
    const int nt = a.g.nt, np = a.g.np;
    uint32_t aph = 0;
    float *prev = reinterpret_cast<float *>(smem + kOffPrev) + lane;  // [column][lane]
    for (int j = 0; j < kDepth4; ++j) prev[j * kLanes] = 0.f;
    for (int tile = blockIdx.x; tile < a.ntiles && !*s_fail; tile += gridDim.x) {
        const TileRows tr(a, tile);
        const int f = tr.f;
        const Field &fd = a.fs.f[f];
        const LaneCol lc(tr.strip, lane, np);
        const int r_end = tr.hi(3), o_lo = tr.lo(4), o_hi = tr.hi(4);
        for (int r = tr.lo(3) - 1; r <= r_end && !*s_fail; ++r) {
            const bool emit = r >= o_lo && r < o_hi && lc.out;
            float hout = 0.f;
            if (emit && a.h_out) hout = fd.h[(size_t)r * fd.pitch + lc.col];
            const int j = ring<kDepth4>(r);
            wt.wait(bars.afull(4, j), take(aph, j));
            tc_fence_after();
            uint32_t yv = tld1(tl + acc_col(3) + j);
            wait_ld();
            pin(yv);
            const float sum = __uint_as_float(yv), acc = __fsub_rn(sum, prev[j * kLanes]);
            prev[j * kLanes] = sum;
            if (r == r_end) {
                // every MMA of the tile has completed: restart the ring from zero
                tzero16(tl + acc_col(3));
                wait_st();
                for (int k = 0; k < kDepth4; ++k) prev[k * kLanes] = 0.f;
            }
            tc_fence_before();
            mbar_arrive(bars.aempty(4, j));
            const float y = __fadd_rn(acc, bias[96]);
            if (emit) {
                if (a.y_out) a.y_out[((size_t)f * nt + r) * np + lc.col] = y;
                if (a.h_out) {
                    float o = hout;
                    if (r > 0 && r + 1 < nt) o = fmaxf(__fadd_rn(hout, __fmul_rn(fd.kout, y)), 0.f);
                    a.h_out[(size_t)r * a.pitch_out + lc.col] = o;
                }
            }
        }
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
    const uint32_t sbase = smem_u32(smem);
    const Bars bars{smem_u32(bar)};

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(s_tmem)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int l = 1; l <= 4; ++l) {
            for (int b = 0; b < kNBuf; ++b) {
                asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bars.xfull(l, b)), "r"(kLanes));
                asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bars.xempty(l, b)));
            }
            for (int j = 0; j < depth_of(l); ++j) {
                asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bars.afull(l, j)));
                asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bars.aempty(l, j)), "r"(kLanes));
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
    const float *bias = reinterpret_cast<const float *>(smem + kOffBias);
    if (tid < kEpi) {
        // warpgroup g < 3 owns layer g+1's columns [128 g, 128 g + 128): its ring slots start at the
        // bias; everything else (and layer 4's ring, owned by warpgroup 3 here) starts at zero
        for (int c = 0; c < 128; c += 32) {
            if (grp < 3 && c < 32 * kDepth)
                tset_bias(tl + 128 * grp + c, bias + 32 * grp);
            else
                tzero32(tl + 128 * grp + c);
        }
        wait_st();
    }
    Waiter wt{s_fail, a.err, a.wait_cycles};
    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    if (tid >= kOutT) {
        mma_agent(((tid - kOutT) >> 5) + 1, a, bars, tmem, sbase, wt, s_fail);
        // completes when every MMA this warp issued has finished
        if (elect_one()) commit(drain);
        __syncwarp();
    } else if (grp < 3) {
        epi_agent(grp + 1, a, bars, smem, tl, lane, bias, wt, s_fail);
    } else if (grp == 3) {
        feature_agent(a, bars, smem, lane, wt, s_fail);
    } else {
        output_agent(a, bars, smem, tl, lane, bias, wt, s_fail);
    }
    __syncthreads();
    // no MMA may still write the accumulators when the columns are released
    if (tid == 0 && !mbar_wait_bounded(drain, 0u, a.wait_cycles)) atomicOr(a.err, 1u);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
}

// Packs the parameter vector into the shared-memory image of fused_kernel.
__global__ void pack_fused_kernel(const float *theta, uint8_t *img) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int dy_of_block[5] = {1, 0, -1, 1, 0};
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
    a.act = act_of(s);
    a.err = st->err;
    const WaitConfig w = wait_config();
    a.wait_cycles = w.cycles;
    a.stall = (w.stall & SBS_STALL_TENSOR_COMMITS) ? 1 : 0;
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
    best_nrb = std::max(best_nrb, (g.nt + kMaxTileRows - 1) / kMaxTileRows);
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
