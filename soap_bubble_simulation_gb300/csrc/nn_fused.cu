// Fused forward pass of the drainage surrogate (include/sbs_nn.h) on the tcgen05 tensor cores:
// features, the four 3x3 convolutions, GELUs and the thickness update in one persistent kernel,
// activations kept in shared memory and accumulators in tensor memory.
//
// Tiling. A tile is a strip of 128 consecutive phi columns (lanes; the middle 120 are output, the
// 4 on each side are the halo the four layers consume) times a block of theta rows of one field.
// The block streams its rows top to bottom through all four layers at once, layer l two rows
// behind layer l-1 ("row time" tau: layer l consumes its input row tau - 2(l-1) and finishes its
// output row tau - 2l).
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

constexpr int kLanes = 128;
constexpr int kOut = 120;                      // output columns per strip
constexpr int kHalo = 4;                       // lanes on each side of the outputs
constexpr int kCells = 136;                    // staged cells per plane (q = lane + 1)
constexpr uint32_t kPlane = kCells * 16;       // 2176 B
constexpr uint32_t kRowX = 4 * kPlane;         // one 32-channel row buffer
constexpr uint32_t kBRows = 160;               // stacked dy ring rows (5 x 32)
constexpr uint32_t kBChunk = kBRows * 16;      // one 8-channel K chunk
constexpr uint32_t kBStep = 2 * kBChunk;       // one K16 step
constexpr uint32_t kB4Rows = 24, kB4Chunk = kB4Rows * 16, kB4Step = 2 * kB4Chunk;
constexpr uint32_t kBxRows = 24, kBxChunk = kBxRows * 16, kBxStep = 2 * kBxChunk;  // weights at row 2
// smem image of the packed weights (built once per parameter change by pack_fused_kernel)
constexpr uint32_t kOffB1 = 0;                          // 2 steps
constexpr uint32_t kOffB2 = kOffB1 + 2 * kBStep;        // 6 steps
constexpr uint32_t kOffB3 = kOffB2 + 6 * kBStep;        // 6 steps
constexpr uint32_t kOffB4 = kOffB3 + 6 * kBStep;        // 6 steps, 24 rows
constexpr uint32_t kOffB4t = kOffB4 + 6 * kB4Step;      // W4(dy=-1) alone (top pole extra)
constexpr uint32_t kOffB4b = kOffB4t + 6 * kBxStep;     // W4(dy=+1) alone (bottom pole extra)
constexpr uint32_t kOffBias = kOffB4b + 6 * kBxStep;    // 97 floats (padded to 128)
constexpr uint32_t kImage = kOffBias + 128 * 4;
// rest of shared memory
constexpr uint32_t kOffX0 = (kImage + 1023) / 1024 * 1024;  // 2 feature rows
constexpr uint32_t kOffX = kOffX0 + 2 * kPlane;             // 3 layers x 2 rows
constexpr uint32_t kOffBar = kOffX + 6 * kRowX;
constexpr uint32_t kSmem = kOffBar + 64;
__host__ __device__ constexpr uint32_t acc_col(int l) { return 96u * (uint32_t)l; }  // layer l (0-based)
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

__device__ __forceinline__ int mod3(int r) { return ((r % 3) + 3) % 3; }
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

__global__ void __launch_bounds__(kLanes, 1) fused_kernel(FusedArgs a) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t *bar = reinterpret_cast<uint64_t *>(smem + kOffBar);  // 4 layer barriers
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(bar + 4);
    volatile int *s_fail = reinterpret_cast<volatile int *>(s_tmem + 1);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int nt = a.g.nt, np = a.g.np;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(s_tmem)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int l = 0; l < 4; ++l) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar + l)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *s_fail = 0;
    }
    // weights image and zeroed activation buffers
    for (uint32_t i = tid * 16; i < kImage; i += kLanes * 16)
        *reinterpret_cast<uint4 *>(smem + i) = *reinterpret_cast<const uint4 *>(a.image + i);
    for (uint32_t i = kOffX0 + tid * 16; i < kOffBar; i += kLanes * 16)
        *reinterpret_cast<uint4 *>(smem + i) = make_uint4(0, 0, 0, 0);
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *s_tmem;
    const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);  // this warp's lane quarter
    for (int c = 0; c < 512; c += 32) tzero32(tl + c);
    wait_st();
    const float *bias = reinterpret_cast<const float *>(smem + kOffBias);
    const uint32_t sbase = smem_u32(smem);
    uint32_t phase = 0;  // bit l: parity of layer l's next commit completion
    bool ok = true;

    tc_fence_before();
    __syncthreads();
    tc_fence_after();

    for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += gridDim.x) {
        const int strip = tile % a.nstrips;
        const int rb = (tile / a.nstrips) % a.nrb;
        const int f = tile / (a.nstrips * a.nrb);
        const Field &fd = a.fs.f[f];
        const int y0 = rb * a.rows_per_block, y1 = min(nt, y0 + a.rows_per_block);
        int lo[5], hi[5];
        for (int l = 0; l <= 4; ++l) {
            lo[l] = max(0, y0 - 4 + l);
            hi[l] = min(nt, y1 + 4 - l);
        }
        const int xcol = strip * kOut - kHalo + tid;  // this lane's column (before wrap)
        const int col = ((xcol % np) + np) % np;
        const bool lane_out = tid >= kHalo && tid < kHalo + kOut && strip * kOut + (tid - kHalo) < np;
        const int cw = col == 0 ? np - 1 : col - 1, ce = col + 1 == np ? 0 : col + 1;

        for (int tau = lo[0]; tau <= hi[3] + 8 && ok; ++tau) {
            // ---- features of row tau into X0[tau & 1]
            if (tau < hi[0]) {
                const int i = tau;
                const float *rc = fd.h + (size_t)i * fd.pitch;
                const float *rn = fd.h + (size_t)refl_row(i - 1, nt) * fd.pitch;
                const float *rs = fd.h + (size_t)refl_row(i + 1, nt) * fd.pitch;
                const float4 row = a.g.rows[i];
                const float hc = rc[col], hn = rn[col], hs = rs[col], hw = rc[cw], he = rc[ce];
                const float cc = fd.c[(size_t)i * fd.pitch + col];
                const float h2 = __fadd_rn(hc, hc);
                uint4 o;
                o.x = pack2(clampf(__fmul_rn(__fsub_rn(hc, SBS_NN_H0), SBS_NN_INV_HS)),
                            clampf(__fmul_rn(__fsub_rn(__fadd_rn(hn, hs), h2), a.g.ct)));
                o.y = pack2(clampf(__fmul_rn(__fsub_rn(__fadd_rn(hw, he), h2), row.x)),
                            clampf(__fmul_rn(__fsub_rn(hs, hn), row.y)));
                o.z = pack2(clampf(__fmul_rn(__fsub_rn(cc, 0.5f), 10.f)), clampf(fd.f5));
                o.w = pack2(clampf(fd.f6), clampf(__fmul_rn(__fmul_rn(__fmul_rn(hc, hc), hc), __fmul_rn(fd.gk, row.z))));
                *reinterpret_cast<uint4 *>(smem + kOffX0 + (tau & 1) * kPlane + (tid + 1) * 16) = o;
            }
#pragma unroll 1
            for (int l = 1; l <= 4; ++l) {
                const int r = tau - 2 * l;          // epilogue row
                const int s = tau - 2 * l + 2;      // MMA input row
                const uint32_t bl = smem_u32(bar + (l - 1));
                if (tau > lo[0]) {
                    if (!mbar_wait_bounded(bl, (phase >> (l - 1)) & 1u)) {
                        atomicOr(a.err, 1u);
                        *s_fail = 1;
                    }
                    phase ^= 1u << (l - 1);
                    tc_fence_after();
                }
                if (r >= lo[l - 1] - 1 && r <= hi[l - 1]) {
                    const int j = mod3(r);
                    const bool emit = r >= lo[l] && r < hi[l];
                    if (l < 4) {
                        const uint32_t ta = tl + acc_col(l - 1) + 32 * j;
                        uint32_t v[32];
                        tld32(ta, v);
                        wait_ld();
#pragma unroll
                        for (int k = 0; k < 32; ++k) pin(v[k]);
                        if (emit) {
                            const float *bl_ = bias + 32 * (l - 1);
                            uint8_t *dst = smem + kOffX + ((l - 1) * 2 + (r & 1)) * kRowX + (tid + 1) * 16;
#pragma unroll
                            for (int p = 0; p < 4; ++p) {
                                uint4 o;
                                uint32_t *ow = reinterpret_cast<uint32_t *>(&o);
#pragma unroll
                                for (int e = 0; e < 4; ++e) {
                                    const int c = p * 8 + 2 * e;
                                    ow[e] = pack2(gelu(__fadd_rn(__uint_as_float(v[c]), bl_[c])),
                                                  gelu(__fadd_rn(__uint_as_float(v[c + 1]), bl_[c + 1])));
                                }
                                *reinterpret_cast<uint4 *>(dst + p * kPlane) = o;
                            }
                        }
                        tzero32(ta);
                    } else {
                        const uint32_t ta = tl + acc_col(3) + j;
                        uint32_t yv = tld1(ta);
                        wait_ld();
                        pin(yv);
                        const float y = __fadd_rn(__uint_as_float(yv), bias[96]);
                        if (emit && lane_out) {
                            const float hc = fd.h[(size_t)r * fd.pitch + col];
                            if (a.y_out) a.y_out[((size_t)f * nt + r) * np + col] = y;
                            if (a.h_out) {
                                float o = hc;
                                if (r > 0 && r + 1 < nt) o = fmaxf(__fadd_rn(hc, __fmul_rn(fd.kout, y)), 0.f);
                                a.h_out[(size_t)r * a.pitch_out + col] = o;
                            }
                        }
                        tzero1(ta);
                    }
                    wait_st();
                }
                fence_async_smem();
                tc_fence_before();
                __syncthreads();
                if (*s_fail) {
                    ok = false;
                    break;
                }
                if (tid == 0) {
                    tc_fence_after();
                    if (s >= lo[l - 1] && s < hi[l - 1]) {
                        const int w = mod3(1 - mod3(s));
                        const uint32_t dacc = tmem + acc_col(l - 1);
                        if (l == 1) {
                            const uint32_t xa = sbase + kOffX0 + (s & 1) * kPlane;
                            for (int st = 0; st < 2; ++st) {
                                const uint64_t ad = make_desc(xa + 32 * st, 16, 128);
                                const uint64_t bd = make_desc(sbase + kOffB1 + st * kBStep + w * 512, kBChunk, 128);
                                mma(dacc, ad, bd, idesc(96));
                            }
                        } else {
                            const uint32_t xa = sbase + kOffX + ((l - 2) * 2 + (s & 1)) * kRowX;
                            const uint32_t boff = l == 2 ? kOffB2 : (l == 3 ? kOffB3 : kOffB4);
                            for (int st = 0; st < 6; ++st) {
                                const int dxi = st >> 1, kk = st & 1;
                                const uint64_t ad = make_desc(xa + 2 * kk * kPlane + 16 * dxi, kPlane, 128);
                                if (l < 4) {
                                    const uint64_t bd =
                                        make_desc(sbase + boff + st * kBStep + w * 512, kBChunk, 128);
                                    mma(dacc, ad, bd, idesc(96));
                                } else {
                                    const uint64_t bd = make_desc(sbase + boff + st * kB4Step + w * 16, kB4Chunk, 128);
                                    mma(dacc, ad, bd, idesc(16));
                                }
                            }
                        }
                        // theta reflection: row -1 reads row 1, row nt reads row nt-2
                        const bool top = s == 1 && lo[l] == 0;
                        const bool bot = s == nt - 2 && hi[l] == nt;
                        for (int e = 0; e < 2; ++e) {
                            if (!(e == 0 ? top : bot)) continue;
                            const int orow = e == 0 ? 0 : nt - 1;
                            const int blk = e == 0 ? 2 : 0;  // W-1 block / W+1 block of the ring
                            if (l < 4) {
                                const uint32_t dx = tmem + acc_col(l - 1) + 32 * mod3(orow);
                                if (l == 1) {
                                    const uint32_t xa = sbase + kOffX0 + (s & 1) * kPlane;
                                    for (int st = 0; st < 2; ++st)
                                        mma(dx, make_desc(xa + 32 * st, 16, 128),
                                            make_desc(sbase + kOffB1 + st * kBStep + blk * 512, kBChunk, 128),
                                            idesc(32));
                                } else {
                                    const uint32_t xa = sbase + kOffX + ((l - 2) * 2 + (s & 1)) * kRowX;
                                    const uint32_t boff = l == 2 ? kOffB2 : kOffB3;
                                    for (int st = 0; st < 6; ++st) {
                                        const int dxi = st >> 1, kk = st & 1;
                                        mma(dx, make_desc(xa + 2 * kk * kPlane + 16 * dxi, kPlane, 128),
                                            make_desc(sbase + boff + st * kBStep + blk * 512, kBChunk, 128),
                                            idesc(32));
                                    }
                                }
                            } else {
                                // B tile row 2 holds the weights: window start 2 - slot puts them at
                                // D column 288 + slot
                                const uint32_t dx = tmem + acc_col(3);
                                const uint32_t xa = sbase + kOffX + (4 + (s & 1)) * kRowX;
                                const uint32_t boff = e == 0 ? kOffB4t : kOffB4b;
                                const uint32_t wo = (uint32_t)(2 - mod3(orow)) * 16u;
                                for (int st = 0; st < 6; ++st) {
                                    const int dxi = st >> 1, kk = st & 1;
                                    mma(dx, make_desc(xa + 2 * kk * kPlane + 16 * dxi, kPlane, 128),
                                        make_desc(sbase + boff + st * kBxStep + wo, kBxChunk, 128), idesc(16));
                                }
                            }
                        }
                    }
                    commit(bl);
                }
            }
        }
        if (!ok) break;
        // drain: the commits of the tile's last row time
        for (int l = 0; l < 4; ++l) {
            if (!mbar_wait_bounded(smem_u32(bar + l), (phase >> l) & 1u)) {
                atomicOr(a.err, 1u);
                *s_fail = 1;
            }
            phase ^= 1u << l;
        }
        tc_fence_after();
        __syncthreads();
        if (*s_fail) ok = false;
    }
    if (!ok && tid == 0) {
        for (int l = 0; l < 4; ++l) mbar_wait_bounded(smem_u32(bar + l), (phase >> l) & 1u);
    }
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
    // layers 1-3: element (step, chunk, row n, e8)
    const int per1 = 2 * 2 * kBRows * 8, per23 = 6 * 2 * kBRows * 8;
    if (e < per1) {
        const int e8 = e % 8, n = (e / 8) % kBRows, ch = (e / (8 * kBRows)) % 2, st = e / (16 * kBRows);
        const int dy = dy_of_block[n / 32], oc = n % 32;
        // step 0: chunk 0 dx=-1, chunk 1 dx=0; step 1: chunk 0 dx=+1, chunk 1 zero
        const int dx = st == 0 ? (ch == 0 ? -1 : 0) : (ch == 0 ? 1 : 2);
        float v = 0.f;
        if (dx <= 1) v = theta[SBS_NN_W1 + (((dy + 1) * 3 + (dx + 1)) * 32 + oc) * 8 + e8];
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
    if (e < 6 * 2 * kB4Rows * 8) {
        const int e8 = e % 8, n = (e / 8) % kB4Rows, ch = (e / (8 * kB4Rows)) % 2, st = e / (16 * kB4Rows);
        const int dx = (st >> 1) - 1, kk = st & 1, ic = kk * 16 + ch * 8 + e8;
        float v = 0.f;
        if (n < 5) v = theta[SBS_NN_W4 + ((dy_of_block[n] + 1) * 3 + (dx + 1)) * 32 + ic];
        B[(kOffB4 + st * kB4Step + ch * kB4Chunk) / 2 + n * 8 + e8] = __float2bfloat16_rn(v);
    }
    if (e < 6 * 2 * kBxRows * 8) {
        const int e8 = e % 8, n = (e / 8) % kBxRows, ch = (e / (8 * kBxRows)) % 2, st = e / (16 * kBxRows);
        const int dx = (st >> 1) - 1, kk = st & 1, ic = kk * 16 + ch * 8 + e8;
        float vt = 0.f, vb = 0.f;
        if (n == 2) {
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
    const int n = 6 * 2 * kBRows * 8;
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
    fused_kernel<<<grid, kLanes, kSmem, stream>>>(a);
    SBS_CUDA_TRY(cudaGetLastError());
    unsigned herr = 0;
    SBS_CUDA_TRY(cudaMemcpyAsync(&herr, st->err, sizeof(unsigned), cudaMemcpyDeviceToHost, stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(stream));
    if (herr) return set_error(SBS_E_TIMEOUT, "fused surrogate kernel: a tensor-core wait timed out");
    return SBS_OK;
}

}  // namespace nn
}  // namespace sbs
