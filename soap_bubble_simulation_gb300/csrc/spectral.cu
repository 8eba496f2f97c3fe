// Spectral thin-film colour: per point, the Airy reflectance at nl wavelengths (the formulation of
// interference_lut.rs:45-133 with full unpolarised Fresnel and the pi phase shift), contracted
// against an nl x 3 colour-matching matrix.
//
// Tensor-core mode (tcgen05, sm_103a): a CTA of 128 threads takes tiles of 128 points. Each thread
// writes its point's reflectance spectrum, rounded to BF16, as one row of the A tile in shared
// memory (K-major, 8 x 16-byte core matrices, no swizzle); one thread issues K/16
// tcgen05.mma.kind::f16 instructions against the colour-matching B tile (16 x K, channels 3..15
// zero) with the FP32 accumulator D (128 x 16) in tensor memory, and commits them to an mbarrier;
// each warp then reads its 32 rows of D with tcgen05.ld. Every wait is bounded (sbs_set_wait_limit):
// on timeout the CTA records the failure in a device flag, waits (bounded) for contractions still
// in flight, frees its tensor memory and returns.
//
// FP32 mode: the same spectra in FP32 contracted with FP32 FMAs (the precision reference for the
// BF16 contraction).
//
// Spectrum generation: sin(phase/2) with phase = 2 pi opd/lambda + pi equals cos(pi y), y =
// opd/lambda; cos^2 has period 1 in y, so y is reduced exactly to u = y - rint(y) in [-1/2, 1/2]
// and cos(pi u) is the Taylor series of cos up to u^14 (truncation < 1e-8 on that interval; FP32
// mode) or up to u^8 (< 2.6e-5; the BF16 tensor-core mode, whose spectra are rounded to BF16),
// evaluated two wavelengths at a time with packed FP32 instructions.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "cell.cuh"
#include "sbs_internal.h"

namespace sbs {
namespace {

constexpr int kTileM = 128;
constexpr int kNPad = 16;         // MMA N (channels 0..2 used)
constexpr int kMaxLambda = 128;   // K padded to a multiple of 16, at most 128

// The BF16 CMF^T tile (B operand) passed by value in the kernel parameters: no per-call device
// buffer, no upload.
struct BTile {
    uint4 v[kNPad * kMaxLambda * 2 / 16];
};

struct SpecConsts {
    float invl[kMaxLambda];     // 1 / lambda (nm^-1), zero beyond nl
    float cmf[kMaxLambda][3];   // FP32 colour-matching weights (FP32 mode)
    int nl;
};

// cos(pi u) for v = u^2, Taylor coefficients (-1)^k pi^(2k) / (2k)!, k = 0..7
__device__ __forceinline__ float2 cos_pi_u2(float2 v) {
    float2 c = f2(-0.00010463810492484565f);
    c = fma2(c, v, f2(0.001929574309403922f));
    c = fma2(c, v, f2(-0.02580689139001405f));
    c = fma2(c, v, f2(0.23533063035889312f));
    c = fma2(c, v, f2(-1.3352627688545893f));
    c = fma2(c, v, f2(4.058712126416768f));
    c = fma2(c, v, f2(-4.934802200544679f));
    c = fma2(c, v, f2(1.0f));
    return c;
}

// The same series to u^8 (k = 0..4; truncation below 2.6e-5 for |u| <= 1/2): enough for spectra
// that are rounded to BF16 (relative step 3.9e-3) for the tensor-core contraction.
__device__ __forceinline__ float2 cos_pi_u2_short(float2 v) {
    float2 c = f2(0.23533063035889312f);
    c = fma2(c, v, f2(-1.3352627688545893f));
    c = fma2(c, v, f2(4.058712126416768f));
    c = fma2(c, v, f2(-4.934802200544679f));
    c = fma2(c, v, f2(1.0f));
    return c;
}

// Airy reflectance F s^2 / (1 + F s^2) at two wavelengths (interference_lut.rs:123-133); SHORT:
// the u^8 cosine series (BF16 spectra).
template <bool SHORT = false>
__device__ __forceinline__ float2 airy2(float opd, float F, float il0, float il1) {
    const float2 y = mul2(f2(opd), make_float2(il0, il1));
    const float2 u = sub2(y, make_float2(rintf(y.x), rintf(y.y)));
    const float2 c = SHORT ? cos_pi_u2_short(mul2(u, u)) : cos_pi_u2(mul2(u, u));
    const float2 fs = mul2(f2(F), mul2(c, c));
    const float2 den = add2(f2(1.0f), fs);
    return make_float2(__fdividef(fs.x, den.x), __fdividef(fs.y, den.y));
}

// Per-point Snell / Fresnel / optical path (interference_lut.rs:54-61, 96-120 and the finesse F).
__device__ __forceinline__ void point_setup(float t, float ci, float nf, float &F, float &opd) {
    const float sin_i = sqrtf(fmaxf(1.0f - ci * ci, 0.0f));
    const float sin_t = sin_i / nf;
    const float ct = sqrtf(fmaxf(1.0f - sin_t * sin_t, 0.0f));
    const float rs = (ci - nf * ct) / fmaxf(ci + nf * ct, 1e-4f);
    const float rp = (nf * ci - ct) / fmaxf(nf * ci + ct, 1e-4f);
    const float R = (rs * rs + rp * rp) * 0.5f;
    const float omr = fmaxf(1.0f - R, 1e-3f);
    F = 4.0f * R / (omr * omr);
    opd = 2.0f * nf * t * ct;
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t make_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // descriptor version for tcgen05; base offset 0, no swizzle
    return d;
}

// Byte offset of element (row, k) in a K-major, no-swizzle tile of core matrices (8 rows x 16 B):
// core matrices adjacent along K are 128 B apart (LBO), 8-row groups are sbo bytes apart (SBO).
__device__ __host__ __forceinline__ uint32_t tile_off(int row, int k, uint32_t sbo) {
    return (uint32_t)(row / 8) * sbo + (uint32_t)(k / 8) * 128u + (uint32_t)(row % 8) * 16u + (uint32_t)(k % 8) * 2u;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait on an mbarrier phase; returns false after `limit` cycles.
__device__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, long long limit) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > limit) return false;
    return true;
}

// Writes one point's spectrum (row `row` of an A tile) as KPAD BF16 values.
template <int KPAD>
__device__ __forceinline__ void write_spectrum_row(uint8_t *sA, int row, float opd, float F, const SpecConsts &c) {
    constexpr uint32_t SBO = (KPAD / 8) * 128;
#pragma unroll
    for (int k8 = 0; k8 < KPAD; k8 += 8) {
        uint32_t w[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int l = k8 + 2 * j;
            float2 v = make_float2(0.f, 0.f);  // padding beyond nl: zeros, not evaluated
            if (l < c.nl) {
                v = airy2<true>(opd, F, c.invl[l], c.invl[l + 1]);
                if (l + 1 >= c.nl) v.y = 0.f;
            }
            __nv_bfloat162 b2 = __floats2bfloat162_rn(v.x, v.y);
            w[j] = *reinterpret_cast<uint32_t *>(&b2);
        }
        *reinterpret_cast<uint4 *>(sA + tile_off(row, k8, SBO)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// With NBUF = 2 tiles are double-buffered: while the tensor core contracts tile i (A buffer i % 2
// into accumulator columns 16 * (i % 2)), the threads generate tile i + 1 in the other buffer, and
// only then wait for tile i's result. With NBUF = 1 a CTA waits for each contraction, and the other
// CTAs on the SM (twice as many fit) fill the gap.
template <int KPAD, int NBUF>
__global__ void __launch_bounds__(kTileM) spectral_tc_kernel(const float *__restrict__ t_nm,
                                                            const float *__restrict__ cos_i,
                                                            const float *__restrict__ n_film, size_t n,
                                                            const BTile b_tile, const SpecConsts c,
                                                            float *__restrict__ rgb, unsigned *err,
                                                            long long wait_cycles, int stall) {
    constexpr uint32_t SBO = (KPAD / 8) * 128;
    constexpr uint32_t A_BYTES = kTileM * KPAD * 2;
    constexpr uint32_t B_BYTES = kNPad * KPAD * 2;
    // instruction descriptor, kind::f16: D f32 (bits 4-5 = 1), A bf16 (7-9 = 1), B bf16 (10-12 = 1),
    // both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28
    constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kNPad >> 3) << 17) |
                               ((uint32_t)(kTileM >> 4) << 24);
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *sA0 = smem;
    uint8_t *sB = smem + NBUF * A_BYTES;
    uint64_t *bar = reinterpret_cast<uint64_t *>(sB + B_BYTES);  // two mbarriers
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(bar + 2);
    int *s_fail = reinterpret_cast<int *>(s_tmem + 1);

    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(smem_u32(s_tmem)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar + 1)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        *s_fail = 0;
    }
    for (uint32_t i = tid; i < B_BYTES / 16; i += kTileM) reinterpret_cast<uint4 *>(sB)[i] = b_tile.v[i];
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *s_tmem;
    const uint32_t b_base = smem_u32(sB);
    uint32_t phases = 0u;  // bit b: parity of the next completion of barrier b

    // waits for the contraction of `tile` (buffer b) and writes its colours; false on timeout
    auto finish = [&](size_t tile, int b) -> bool {
        if (tid == 0 && !mbar_wait_bounded(smem_u32(bar + b), (phases >> b) & 1u, wait_cycles)) {
            atomicOr(err, 1u);
            *s_fail = 1;
        }
        phases ^= 1u << b;
        __syncthreads();
        if (*s_fail) return false;
        tc_fence_after();
        uint32_t r0, r1, r2, r3;
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(16 * b);
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0, %1, %2, %3}, [%4];"
                     : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                     : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        const size_t p = tile * kTileM + tid;
        if (p < n) {
            rgb[3 * p] = __uint_as_float(r0);
            rgb[3 * p + 1] = __uint_as_float(r1);
            rgb[3 * p + 2] = __uint_as_float(r2);
        }
        tc_fence_before();
        __syncthreads();
        return true;
    };

    const size_t ntiles = (n + kTileM - 1) / kTileM;
    size_t prev = 0;
    int it = 0;
    bool ok = true;
    for (size_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
        const int b = NBUF == 2 ? (it & 1) : 0;
        uint8_t *sA = sA0 + b * A_BYTES;
        const size_t p = tile * kTileM + tid;
        float F = 0.f, opd = 0.f;
        if (p < n) point_setup(t_nm[p], cos_i[p], n_film[p], F, opd);
        write_spectrum_row<KPAD>(sA, tid, opd, F, c);
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0 && !stall) {  // stall (the timeout test): neither MMAs nor their commit
            const uint32_t a_base = smem_u32(sA);
#pragma unroll
            for (int kk = 0; kk < KPAD / 16; ++kk) {
                const uint64_t ad = make_desc(a_base + kk * 256, 128, SBO);
                const uint64_t bd = make_desc(b_base + kk * 256, 128, SBO);
                const uint32_t acc = kk > 0 ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem + 16u * b),
                    "l"(ad), "l"(bd), "r"(IDESC), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(bar + b))
                         : "memory");
        }
        if (NBUF == 1) {
            if (!(ok = finish(tile, 0))) break;
            continue;
        }
        if (it > 0 && !(ok = finish(prev, b ^ 1))) break;
        prev = tile;
    }
    if (NBUF == 2 && ok && it > 0) ok = finish(prev, (it - 1) & 1);
    if (!ok && tid == 0) {
        // contractions may still be in flight: give each barrier one more bounded wait before freeing
        mbar_wait_bounded(smem_u32(bar), phases & 1u, wait_cycles);
        mbar_wait_bounded(smem_u32(bar + 1), (phases >> 1) & 1u, wait_cycles);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(tmem));
}

template <int KPAD>
__global__ void __launch_bounds__(128) spectral_fp32_kernel(const float *__restrict__ t_nm,
                                                           const float *__restrict__ cos_i,
                                                           const float *__restrict__ n_film, size_t n,
                                                           const SpecConsts c, float *__restrict__ rgb) {
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    float F, opd;
    point_setup(t_nm[p], cos_i[p], n_film[p], F, opd);
    float r = 0.f, g = 0.f, b = 0.f;
#pragma unroll
    for (int l = 0; l < KPAD; l += 2) {
        if (l < c.nl) {
            const float2 v = airy2(opd, F, c.invl[l], c.invl[l + 1]);
            r = fmaf(v.x, c.cmf[l][0], r);
            g = fmaf(v.x, c.cmf[l][1], g);
            b = fmaf(v.x, c.cmf[l][2], b);
            if (l + 1 < c.nl) {
                r = fmaf(v.y, c.cmf[l + 1][0], r);
                g = fmaf(v.y, c.cmf[l + 1][1], g);
                b = fmaf(v.y, c.cmf[l + 1][2], b);
            }
        }
    }
    rgb[3 * p] = r;
    rgb[3 * p + 1] = g;
    rgb[3 * p + 2] = b;
}

#ifndef SBS_SPECTRAL_NBUF
#define SBS_SPECTRAL_NBUF 1  // A-tile buffers per CTA (1 or 2)
#endif

template <int KPAD>
cudaError_t launch_tc(const float *t, const float *ci, const float *nf, size_t n, const BTile &btile,
                      const SpecConsts &c, float *rgb, unsigned *err, cudaStream_t s) {
    constexpr int NBUF = SBS_SPECTRAL_NBUF;
    const size_t smem = NBUF * (size_t)kTileM * KPAD * 2 + (size_t)kNPad * KPAD * 2 + 16 + 64;
    cudaError_t e = cudaFuncSetAttribute(spectral_tc_kernel<KPAD, NBUF>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 148, per_sm = 0, smem_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    // CTAs per SM from shared memory (1 KB per CTA reserved by the runtime)
    per_sm = smem_sm > 0 ? (int)(smem_sm / (smem + 1024)) : 1;
    if (per_sm < 1) per_sm = 1;
    if (per_sm > 16) per_sm = 16;  // each CTA holds 32 of the SM's 512 tensor-memory columns
    const size_t ntiles = (n + kTileM - 1) / kTileM;
    size_t grid = (size_t)per_sm * sms;
    if (grid > ntiles) grid = ntiles;
    const WaitConfig w = wait_config();
    spectral_tc_kernel<KPAD, NBUF><<<(unsigned)grid, kTileM, smem, s>>>(
        t, ci, nf, n, btile, c, rgb, err, w.cycles, (w.stall & SBS_STALL_TENSOR_COMMITS) ? 1 : 0);
    return cudaGetLastError();
}

}  // namespace
}  // namespace sbs

using namespace sbs;



extern "C" int sbs_spectral_rgb(const float *t_nm, const float *cos_i, const float *n_film, size_t n,
                                const float *wl_nm, uint32_t nl, const float *cmf, int mode, float *rgb, int mem,
                                void *stream) {
    clear_error();
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "bad mem flag %d", mem);
    SBS_CHECK_ARG(mode == SBS_SPECTRAL_TC_BF16 || mode == SBS_SPECTRAL_FP32, "bad mode %d", mode);
    SBS_CHECK_ARG(wl_nm != nullptr && cmf != nullptr, "null wavelength or CMF table");
    SBS_CHECK_ARG(nl >= 1 && nl <= (uint32_t)kMaxLambda, "nl must be 1..%d (got %u)", kMaxLambda, nl);
    if (n == 0) return SBS_OK;
    SBS_CHECK_ARG(t_nm && cos_i && n_film && rgb, "null pointer");
    int rc = require_device();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;

    SpecConsts c{};
    c.nl = (int)nl;
    for (uint32_t l = 0; l < nl; ++l) {
        SBS_CHECK_ARG(wl_nm[l] > 0.f, "wavelengths must be positive");
        c.invl[l] = 1.0f / wl_nm[l];
        for (int ch = 0; ch < 3; ++ch) c.cmf[l][ch] = cmf[3 * l + ch];
    }
    const int kpad = nl <= 32 ? 32 : (nl <= 64 ? 64 : (nl <= 96 ? 96 : 128));
    // B tile: CMF^T (16 x kpad) in BF16, K-major core matrices, channels 3..15 zero
    BTile bt;
    std::memset(&bt, 0, sizeof(bt));
    uint8_t *btile = reinterpret_cast<uint8_t *>(bt.v);
    const uint32_t sbo = (uint32_t)(kpad / 8) * 128u;
    for (int ch = 0; ch < 3; ++ch)
        for (uint32_t l = 0; l < nl; ++l) {
            const __nv_bfloat16 v = __float2bfloat16_rn(cmf[3 * l + ch]);
            std::memcpy(btile + tile_off(ch, (int)l, sbo), &v, 2);
        }

    // scratch: the timeout flag, plus staging buffers for host inputs
    const size_t in_bytes = 3 * n * sizeof(float), out_bytes = 3 * n * sizeof(float);
    char *base = nullptr;
    SBS_CUDA_TRY(scratch_alloc((void **)&base, 256 + (mem == SBS_MEM_HOST ? in_bytes + out_bytes : 0), s));
    unsigned *d_err = reinterpret_cast<unsigned *>(base);
    const float *dt = t_nm, *dc = cos_i, *dn = n_film;
    float *dout = rgb;
    cudaError_t e = cudaMemsetAsync(d_err, 0, sizeof(unsigned), s);
    if (e == cudaSuccess && mem == SBS_MEM_HOST) {
        float *in = reinterpret_cast<float *>(base + 256);
        e = cudaMemcpyAsync(in, t_nm, n * sizeof(float), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(in + n, cos_i, n * sizeof(float), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(in + 2 * n, n_film, n * sizeof(float), cudaMemcpyHostToDevice, s);
        dt = in;
        dc = in + n;
        dn = in + 2 * n;
        dout = in + 3 * n;
    }
    if (e == cudaSuccess) {
        if (mode == SBS_SPECTRAL_FP32) {
            const unsigned g = (unsigned)((n + 127) / 128);
            if (kpad == 32)
                spectral_fp32_kernel<32><<<g, 128, 0, s>>>(dt, dc, dn, n, c, dout);
            else if (kpad == 64)
                spectral_fp32_kernel<64><<<g, 128, 0, s>>>(dt, dc, dn, n, c, dout);
            else if (kpad == 96)
                spectral_fp32_kernel<96><<<g, 128, 0, s>>>(dt, dc, dn, n, c, dout);
            else
                spectral_fp32_kernel<128><<<g, 128, 0, s>>>(dt, dc, dn, n, c, dout);
            e = cudaGetLastError();
        } else if (kpad == 32) {
            e = launch_tc<32>(dt, dc, dn, n, bt, c, dout, d_err, s);
        } else if (kpad == 64) {
            e = launch_tc<64>(dt, dc, dn, n, bt, c, dout, d_err, s);
        } else if (kpad == 96) {
            e = launch_tc<96>(dt, dc, dn, n, bt, c, dout, d_err, s);
        } else {
            e = launch_tc<128>(dt, dc, dn, n, bt, c, dout, d_err, s);
        }
    }
    unsigned herr = 0;
    if (e == cudaSuccess && mem == SBS_MEM_HOST) e = cudaMemcpyAsync(rgb, dout, out_bytes, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&herr, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(base, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(SBS_E_CUDA, "spectral: %s", cudaGetErrorString(e));
    if (herr) return set_error(SBS_E_TIMEOUT, "spectral: a tensor-core wait timed out");
    return SBS_OK;
}
