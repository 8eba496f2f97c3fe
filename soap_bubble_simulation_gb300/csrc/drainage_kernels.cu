// Drainage step kernels for sm_103a.
//
// One launch advances the whole theta-phi field by one forward-Euler step. The field is row-major
// [theta][phi] f32 with a row pitch that is a multiple of 128 elements, so each lane owns one
// aligned float4 of four consecutive phi cells and a warp covers 128 cells of a row. A block
// walks down a strip of `rb` theta rows keeping the rows above, at and below the current one in
// registers (each row is read once per strip, plus one halo row at each end) and prefetching the
// row after next. Phi neighbours come from the neighbouring lane by shuffle; only lanes 0 and 31
// read the one cell beyond the warp, and the row ends wrap periodically.
//
// Arithmetic: the reference's forward-Euler update written with per-row coefficients (computed
// once in f64 on the host, rounded to f32) and explicit fmaf, so the oracle can repeat it bit for
// bit:
//   lt = (h[i+1]-h) + (h[i-1]-h),  d1 = h[i+1]-h[i-1],  lp = (h[j+1]-h) + (h[j-1]-h)
//   L   = F*lp + E*d1 + b*lt                 (F, E per row; b = 1/dtheta^2)
//   inc = D/R^2 * L + A*h^3 [+ Marangoni]    (A = -rho g/(3 eta) sin(theta))
//   h'  = max(h + dt*inc, 0)
// CPU semantics (drainage.rs:298-392) also averages the pole rings and applies the TFE fronts;
// WGSL semantics (drainage.wgsl:72-202) co-evolves the surfactant field and leaves the pole rows.
//
// Compensated mode (CPU semantics): the reference integrates in f64 and the gravity increment of a
// 500 nm film is ~1/1000 of an f32 ulp, so plain f32 loses it. Each cell then carries a second f32
// word, value = hi + lo; the differences include the lo words and the update h + dt*inc is an
// error-free TwoSum, giving ~48 significant bits with f32 arithmetic at 16 B per cell-step.
#include <cuda_runtime.h>

#include "cell.cuh"
#include "sbs_internal.h"

namespace sbs {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kBlockThreadsMax = 128;

__device__ __forceinline__ float4 ld4(const float *base, int r, int pitch, int c) {
    return __ldg(reinterpret_cast<const float4 *>(base + (size_t)r * pitch + c));
}

__device__ __forceinline__ float4 splat4(float v) { return make_float4(v, v, v, v); }

__device__ __forceinline__ float getk(const float4 &v, int k) {
    return k == 0 ? v.x : (k == 1 ? v.y : (k == 2 ? v.z : v.w));
}

__device__ __forceinline__ void setk(float4 &v, int k, float x) {
    if (k == 0)
        v.x = x;
    else if (k == 1)
        v.y = x;
    else if (k == 2)
        v.z = x;
    else
        v.w = x;
}

// Sum of a double over the block, deterministic order; result valid in thread 0.
__device__ double block_sum(double v, double *smem) {
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

// Exact fixed-point sum over the block (fixsum.cuh); result valid in thread 0.
__device__ void block_fix_sum(FixSum &a, FixSum *smem /*32*/) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    fix_warp(a);
    if (lane == 0) smem[warp] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        FixSum t = fix_zero();
        for (int i = 0; i < nw; ++i) fix_add(t, smem[i]);
        a = t;
    }
    __syncthreads();
}

// Mean of a pole ring from its per-block partial sums.
__device__ __forceinline__ double ring_mean(const FixSum *part, int nbx, int np) {
    FixSum t = fix_zero();
    for (int b = 0; b < nbx; ++b) {
        fix_add(t, fix_ldcg(part + b));
    }
    return fix_to_double(t) / (double)np;
}

// Phi neighbours of the four cells c..c+3 of row `rowp` whose values are v (all lanes call).
__device__ __forceinline__ void phi_neighbors(const float *rowp, const float4 &v, int c, int np, int lane,
                                              bool active, float4 &pm, float4 &pp) {
    float lh = __shfl_up_sync(kFull, v.w, 1);
    float rh = __shfl_down_sync(kFull, v.x, 1);
    if (!active) return;
    if (lane == 0) lh = __ldg(rowp + (c == 0 ? np - 1 : c - 1));
    float w0 = 0.f;
    if (c + 4 >= np) w0 = __ldg(rowp);
    if (lane == 31 && c + 4 < np) rh = __ldg(rowp + c + 4);
    pm = make_float4(lh, v.x, v.y, v.z);
    pp.x = (c + 1 < np) ? v.y : w0;
    pp.y = (c + 2 < np) ? v.z : w0;
    pp.z = (c + 3 < np) ? v.w : w0;
    pp.w = (c + 4 < np) ? rh : w0;
}

template <int SEM, int X2, bool VOL, bool MAR = false>
__global__ void __launch_bounds__(kBlockThreadsMax) drain_step_kernel(const StepArgs a) {
    __shared__ double s_red[64];
    __shared__ FixSum s_fix[32];
    __shared__ TfeStep s_tfe;
    __shared__ int s_last;
    constexpr bool CPU = SEM == SBS_CPU_SEMANTICS;
    constexpr bool WGSL = SEM == SBS_WGSL_SEMANTICS;

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wx = blockDim.x >> 5;
    const int np = a.np, nt = a.nt, pitch = a.pitch;
    const int c = (blockIdx.x * wx + warp) * 128 + lane * 4;
    const bool active = c < np;
    const int r0 = 1 + blockIdx.y * a.rb;
    const int r1 = min(r0 + a.rb, nt - 1);  // exclusive

    int nf = 0;
    if (CPU && a.tfe != nullptr) {
        for (int i = threadIdx.x; i < (int)(sizeof(TfeStep) / sizeof(int)); i += blockDim.x)
            reinterpret_cast<int *>(&s_tfe)[i] = reinterpret_cast<const int *>(a.tfe)[i];
        __syncthreads();
        nf = s_tfe.nf;
    }

    // pole rows of the input, when they are the ring means of the previous step
    float ptop = 0.f, pbot = 0.f, ptop_lo = 0.f, pbot_lo = 0.f;
    const bool virt = CPU && a.poles_virtual;
    if (virt) {
        const int nbx = gridDim.x;
        if (r0 == 1) {
            const double m = ring_mean(a.pin, nbx, np);
            ptop = (float)m;
            ptop_lo = (float)(m - (double)ptop);
        }
        if (r1 == nt - 1) {
            const double m = ring_mean(a.pin + nbx, nbx, np);
            pbot = (float)m;
            pbot_lo = (float)(m - (double)pbot);
        }
    }

    auto load_h = [&](int r) -> float4 {
        if (!active) return splat4(0.f);
        if (virt && r == 0) return splat4(ptop);
        if (virt && r == nt - 1) return splat4(pbot);
        return ld4(a.hin, r, pitch, c);
    };
    auto load_l = [&](int r) -> float4 {
        if (!active) return splat4(0.f);
        if (virt && r == 0) return splat4(ptop_lo);
        if (virt && r == nt - 1) return splat4(pbot_lo);
        return ld4(a.lin, r, pitch, c);
    };
    auto load_c = [&](int r) -> float4 {
        if (!active) return splat4(0.f);
        return ld4(a.cin, r, pitch, c);
    };

    float4 hp = load_h(r0 - 1), hc = load_h(r0), hn = load_h(r0 + 1);
    float4 lp4 = splat4(0.f), lc4 = splat4(0.f), ln4 = splat4(0.f);
    float4 cp = splat4(0.f), cc = splat4(0.f), cn = splat4(0.f);
    if (X2) {
        lp4 = load_l(r0 - 1);
        lc4 = load_l(r0);
        ln4 = load_l(r0 + 1);
    }
    if (WGSL) {
        cp = load_c(r0 - 1);
        cc = load_c(r0);
        cn = load_c(r0 + 1);
    }

    double vacc = 0.0;
    const float b = a.b, DR2 = a.DR2, dt = a.dt, crit = a.crit;

    for (int r = r0; r < r1; ++r) {
        // prefetch the row after next
        float4 hnn = splat4(0.f), lnn = splat4(0.f), cnn = splat4(0.f);
        if (r + 1 < r1) {
            hnn = load_h(r + 2);
            if (X2) lnn = load_l(r + 2);
            if (WGSL) cnn = load_c(r + 2);
        }
        const float4 co = __ldg(a.rows + r);  // A, E, F, G
        float4 hpm, hpp;
        phi_neighbors(a.hin + (size_t)r * pitch, hc, c, np, lane, active, hpm, hpp);
        float4 lpm = splat4(0.f), lpp = splat4(0.f);
        if (X2) phi_neighbors(a.lin + (size_t)r * pitch, lc4, c, np, lane, active, lpm, lpp);
        float4 cpm = splat4(0.f), cpp = splat4(0.f);
        if (WGSL) phi_neighbors(a.cin + (size_t)r * pitch, cc, c, np, lane, active, cpm, cpp);

        unsigned fmask = 0;
        if (CPU)
            for (int f = 0; f < nf; ++f)
                if (r >= s_tfe.fr[f].x && r <= s_tfe.fr[f].y) fmask |= 1u << f;

        float4 outh, outl = splat4(0.f), outc = splat4(0.f);
        FixSum ring = fix_zero();
        float4 wh4, wc4;
        if (WGSL)
            wgsl_cell4<MAR>(hc, hp, hn, hpm, hpp, cc, cp, cn, cpm, cpp, co, b, DR2, a.DsR2, a.Gt, a.M, dt, crit, wh4,
                            wc4);
        else
            cpu_cell4<X2 != 0>(hc, hp, hn, hpm, hpp, lc4, lp4, ln4, lpm, lpp, co, b, DR2, dt, crit, wh4, wc4);
        const bool ring_row = CPU && (r == 1 || r == nt - 2);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const bool valid = active && (c + k < np);
            float vh = getk(wh4, k), vl = 0.f, vc = 0.f;
            if (WGSL) vc = getk(wc4, k);
            if (X2) vl = getk(wc4, k);
            if (CPU) {
                if (ring_row && valid) {
                    fix_add_float(ring, vh);
                    if (X2) fix_add_float(ring, vl);
                }
                if (fmask) {
                    const int col = c + k;
                    for (int f = 0; f < nf; ++f) {
                        if (!(fmask & (1u << f))) continue;
                        int d = col - s_tfe.fr[f].z;
                        if (d < 0) d += np;
                        if (d < s_tfe.fr[f].w) {
                            if (X2) {
                                // (vh + vl) * (factor + factor_lo), double-float product
                                const float fh = s_tfe.factor, fl = s_tfe.factor_lo;
                                const float p = vh * fh;
                                const float pe = fmaf(vh, fh, -p);
                                const float q = fmaf(vh, fl, fmaf(vl, fh, pe));
                                const float s = p + q;
                                vl = q - (s - p);
                                vh = s;
                            } else {
                                vh = vh * s_tfe.factor;
                            }
                            break;
                        }
                    }
                }
            }
            setk(outh, k, vh);
            if (X2) setk(outl, k, vl);
            if (WGSL) setk(outc, k, vc);
            if (VOL && valid) vacc += ((double)vh + (double)vl) * __ldg(a.vol_w + r);
        }
        if (active) {
            *reinterpret_cast<float4 *>(a.hout + (size_t)r * pitch + c) = outh;
            if (X2) *reinterpret_cast<float4 *>(a.lout + (size_t)r * pitch + c) = outl;
            if (WGSL) *reinterpret_cast<float4 *>(a.cout + (size_t)r * pitch + c) = outc;
        }
        if (CPU && (r == 1 || r == nt - 2)) {
            // block-uniform branch: every thread of the block walks the same rows
            block_fix_sum(ring, s_fix);
            if (threadIdx.x == 0) {
                if (r == 1) a.pout[blockIdx.x] = ring;
                if (r == nt - 2) a.pout[gridDim.x + blockIdx.x] = ring;
            }
        }
        hp = hc;
        hc = hn;
        hn = hnn;
        if (X2) {
            lp4 = lc4;
            lc4 = ln4;
            ln4 = lnn;
        }
        if (WGSL) {
            cp = cc;
            cc = cn;
            cn = cnn;
        }
    }

    if (VOL) {
        const double s = block_sum(vacc, s_red);
        const unsigned nblocks = gridDim.x * gridDim.y;
        const unsigned bid = blockIdx.y * gridDim.x + blockIdx.x;
        if (threadIdx.x == 0) {
            a.vol_partials[bid] = s;
            __threadfence();
            const unsigned t = atomicAdd(a.vol_counter, 1u);
            s_last = (t == nblocks - 1);
        }
        __syncthreads();
        if (s_last) {
            __threadfence();
            double t = 0.0;
            for (unsigned i = threadIdx.x; i < nblocks; i += blockDim.x) t += __ldcg(a.vol_partials + i);
            // pole rows: CPU semantics holds this step's ring means; WGSL keeps the input pole rows
            double pole = 0.0;
            if (WGSL) {
                for (int j = threadIdx.x; j < np; j += blockDim.x) {
                    pole += (double)__ldg(a.hin + j) * __ldg(a.vol_w);
                    pole += (double)__ldg(a.hin + (size_t)(nt - 1) * pitch + j) * __ldg(a.vol_w + nt - 1);
                }
            }
            t = block_sum(t, s_red);
            pole = block_sum(pole, s_red);
            if (threadIdx.x == 0) {
                if (CPU) {
                    const double mt = ring_mean(a.pout, gridDim.x, np);
                    const double mb = ring_mean(a.pout + gridDim.x, gridDim.x, np);
                    const float mth = (float)mt, mbh = (float)mb;
                    // the pole rows hold the split (or rounded) means
                    const double vt = X2 ? (double)mth + (double)(float)(mt - (double)mth) : (double)mth;
                    const double vb = X2 ? (double)mbh + (double)(float)(mb - (double)mbh) : (double)mbh;
                    pole = (double)np * vt * a.vol_w[0] + (double)np * vb * a.vol_w[nt - 1];
                }
                const unsigned idx = *a.vol_index;
                a.vol_out[idx] = t + pole;
                *a.vol_index = idx + 1;
                *a.vol_counter = 0u;
                __threadfence();
            }
        }
    }
}

__global__ void finalize_poles_kernel(float *h, float *hl, const FixSum *part, int nbx, int nt, int np, int pitch) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= np) return;
    const double mt = ring_mean(part, nbx, np);
    const double mb = ring_mean(part + nbx, nbx, np);
    const float th = (float)mt, bh = (float)mb;
    h[j] = th;
    h[(size_t)(nt - 1) * pitch + j] = bh;
    if (hl) {
        hl[j] = (float)(mt - (double)th);
        hl[(size_t)(nt - 1) * pitch + j] = (float)(mb - (double)bh);
    }
}

// ---------------------------------------------------------------------------
// Field reduction: min, max and FP64 weighted sum over valid columns.
// ---------------------------------------------------------------------------
constexpr int kReduceThreads = 256;

__global__ void __launch_bounds__(kReduceThreads)
    field_reduce_kernel(const float *h, const float *hl, int nt, int np, size_t pitch, const double *w,
                        double *partials, unsigned *counter, ReduceOut *out) {
    __shared__ double s_min[kReduceThreads / 32], s_max[kReduceThreads / 32], s_sum[32];
    __shared__ int s_last;
    double vmin = INFINITY, vmax = -INFINITY, vsum = 0.0;
    for (int r = blockIdx.x; r < nt; r += gridDim.x) {
        const double wr = w ? w[r] : 0.0;
        double rs = 0.0;
        for (int j = threadIdx.x; j < np; j += blockDim.x) {
            double v = (double)h[(size_t)r * pitch + j];
            if (hl) v += (double)hl[(size_t)r * pitch + j];
            vmin = fmin(vmin, v);
            vmax = fmax(vmax, v);
            rs += v;
        }
        vsum += rs * wr;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        vmin = fmin(vmin, __shfl_xor_sync(kFull, vmin, o));
        vmax = fmax(vmax, __shfl_xor_sync(kFull, vmax, o));
    }
    if (lane == 0) {
        s_min[warp] = vmin;
        s_max[warp] = vmax;
    }
    __syncthreads();
    const double bs = block_sum(vsum, s_sum);
    if (threadIdx.x == 0) {
        double m0 = INFINITY, m1 = -INFINITY;
        for (int i = 0; i < kReduceThreads / 32; ++i) {
            m0 = fmin(m0, s_min[i]);
            m1 = fmax(m1, s_max[i]);
        }
        partials[3 * blockIdx.x + 0] = m0;
        partials[3 * blockIdx.x + 1] = m1;
        partials[3 * blockIdx.x + 2] = bs;
        __threadfence();
        const unsigned t = atomicAdd(counter, 1u);
        s_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        __threadfence();
        double m0 = INFINITY, m1 = -INFINITY, s = 0.0;
        for (unsigned i = 0; i < gridDim.x; ++i) {
            m0 = fmin(m0, __ldcg(partials + 3 * i));
            m1 = fmax(m1, __ldcg(partials + 3 * i + 1));
            s += __ldcg(partials + 3 * i + 2);
        }
        out->vmin = m0;
        out->vmax = m1;
        out->volume = s;
        *counter = 0u;
        __threadfence();
    }
}

// ---------------------------------------------------------------------------
// get_thickness (drainage.rs:516-552), f64 arithmetic on the f32 (or f32x2) field.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double cell(const float *h, const float *hl, size_t idx) {
    double v = (double)h[idx];
    if (hl) v += (double)hl[idx];
    return v;
}

__device__ double query_one(const float *h, const float *hl, int nt, int np, size_t pitch, double theta,
                            double phi) {
    const double PI = 3.14159265358979323846;
    const double dth = PI / (double)(nt - 1), dph = 2.0 * PI / (double)np;
    const double tcl = theta < 0.0 ? 0.0 : (theta > PI ? PI : theta);
    const double two_pi = 2.0 * PI;
    const double rr = fmod(phi, two_pi);
    const double phin = rr < 0.0 ? rr + two_pi : rr;
    const double tc = tcl / dth, pc = phin / dph;
    const double tfl = floor(tc), pfl = floor(pc);
    unsigned long long til = tfl <= 0.0 ? 0ull : (unsigned long long)tfl;
    if (til > (unsigned long long)(nt - 2)) til = nt - 2;
    const unsigned long long pil = (pfl <= 0.0 ? 0ull : (unsigned long long)pfl) % (unsigned long long)np;
    const unsigned long long tih = til + 1, pih = (pil + 1) % (unsigned long long)np;
    const double tf = tc - (double)til, pf = pc - (double)pil;
    const double v00 = cell(h, hl, til * pitch + pil), v01 = cell(h, hl, til * pitch + pih);
    const double v10 = cell(h, hl, tih * pitch + pil), v11 = cell(h, hl, tih * pitch + pih);
    const double v0 = v00 * (1.0 - pf) + v01 * pf;
    const double v1 = v10 * (1.0 - pf) + v11 * pf;
    return v0 * (1.0 - tf) + v1 * tf;
}

__global__ void query_kernel(const float *h, const float *hl, int nt, int np, size_t pitch, const double *theta,
                             const double *phi, double *out, size_t n) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = query_one(h, hl, nt, np, pitch, theta[i], phi[i]);
}

__device__ void lut2d_read(const double *lut, int T, int A, double tmin, double tmax, double t_nm, double cos_i,
                           double *o) {
    double ti = (t_nm - tmin) / (tmax - tmin) * (double)(T - 1);
    ti = ti < 0.0 ? 0.0 : (ti > (double)(T - 1) ? (double)(T - 1) : ti);
    const double cc = cos_i < 0.0 ? 0.0 : (cos_i > 1.0 ? 1.0 : cos_i);
    const double aj = cc * (double)(A - 1);
    int i0 = (int)floor(ti), j0 = (int)floor(aj);
    if (i0 > T - 2) i0 = T - 2;
    if (j0 > A - 2) j0 = A - 2;
    const double fi = ti - (double)i0, fj = aj - (double)j0;
    for (int c = 0; c < 3; ++c) {
        const double v00 = lut[((size_t)i0 * A + j0) * 3 + c], v01 = lut[((size_t)i0 * A + j0 + 1) * 3 + c];
        const double v10 = lut[((size_t)(i0 + 1) * A + j0) * 3 + c];
        const double v11 = lut[((size_t)(i0 + 1) * A + j0 + 1) * 3 + c];
        const double x = v00 * (1.0 - fj) + v01 * fj;
        const double y = v10 * (1.0 - fj) + v11 * fj;
        o[c] = x * (1.0 - fi) + y * fi;
    }
}

__global__ void vertex_colors_kernel(const float *h, const float *hl, int nt, int np, size_t pitch, const double *xyz,
                                     size_t nv, const double *lut, int T, int A, double tmin, double tmax,
                                     double *rgb) {
    const size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nv) return;
    const double PI = 3.14159265358979323846;
    const double x = xyz[3 * k], y = xyz[3 * k + 1], z = xyz[3 * k + 2];
    const double yc = y < -1.0 ? -1.0 : (y > 1.0 ? 1.0 : y);
    const double theta = acos(yc);
    double phi = atan2(z, x);
    if (phi < 0.0) phi += 2.0 * PI;
    const double t_nm = query_one(h, hl, nt, np, pitch, theta, phi) * 1e9;
    double o[3];
    lut2d_read(lut, T, A, tmin, tmax, t_nm, fabs(z), o);
    rgb[3 * k] = o[0];
    rgb[3 * k + 1] = o[1];
    rgb[3 * k + 2] = o[2];
}

__global__ void fill_kernel(float *p, size_t pitch, int nt, int np, float v) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)nt * np) return;
    const size_t r = i / np, c = i % np;
    p[r * pitch + c] = v;
}

__global__ void split_kernel(const double *src, float *hi, float *lo, int nt, int np, size_t pitch) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)nt * np) return;
    const size_t r = i / np, c = i % np;
    const double v = src[i];
    const float h = (float)v;
    hi[r * pitch + c] = h;
    lo[r * pitch + c] = (float)(v - (double)h);
}

__global__ void join_kernel(const float *hi, const float *lo, double *dst, int nt, int np, size_t pitch) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (size_t)nt * np) return;
    const size_t r = i / np, c = i % np;
    double v = (double)hi[r * pitch + c];
    if (lo) v += (double)lo[r * pitch + c];
    dst[i] = v;
}

}  // namespace

cudaError_t launch_fill(float *p, size_t pitch, int nt, int np, float v, cudaStream_t s) {
    const size_t n = (size_t)nt * np;
    fill_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(p, pitch, nt, np, v);
    return cudaGetLastError();
}

cudaError_t launch_split_f64(const double *src, float *hi, float *lo, int nt, int np, size_t pitch, cudaStream_t s) {
    const size_t n = (size_t)nt * np;
    split_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(src, hi, lo, nt, np, pitch);
    return cudaGetLastError();
}

cudaError_t launch_join_f64(const float *hi, const float *lo, double *dst, int nt, int np, size_t pitch,
                            cudaStream_t s) {
    const size_t n = (size_t)nt * np;
    join_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(hi, lo, dst, nt, np, pitch);
    return cudaGetLastError();
}

StepGeom step_geometry(int nt, int np, int semantics, int x2) {
    StepGeom g{};
    const int chunks = (np + 127) / 128;
    g.wx = chunks < 4 ? chunks : 4;
    g.nbx = (chunks + g.wx - 1) / g.wx;
    // strips sized so the grid is about one wave of resident blocks
    int dev = 0, sms = 148, per_sm = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const void *fn = semantics == SBS_CPU_SEMANTICS
                         ? (x2 ? (const void *)drain_step_kernel<SBS_CPU_SEMANTICS, 1, false>
                               : (const void *)drain_step_kernel<SBS_CPU_SEMANTICS, 0, false>)
                         : (const void *)drain_step_kernel<SBS_WGSL_SEMANTICS, 0, false>;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32 * g.wx, 0);
    if (per_sm < 1) per_sm = 1;
    int strips = per_sm * sms / g.nbx;
    if (strips < 1) strips = 1;
    int rb = (nt - 2 + strips - 1) / strips;
    if (rb < 4) rb = 4;
    g.rb = rb;
    g.nby = (nt - 2 + g.rb - 1) / g.rb;
    return g;
}

cudaError_t launch_step(int semantics, int x2, const StepArgs &a, const StepGeom &g, cudaStream_t s) {
    dim3 grid(g.nbx, g.nby), block(32 * g.wx);
    const bool vol = a.vol_w != nullptr;
    if (semantics == SBS_CPU_SEMANTICS) {
        if (x2) {
            if (vol)
                drain_step_kernel<SBS_CPU_SEMANTICS, 1, true><<<grid, block, 0, s>>>(a);
            else
                drain_step_kernel<SBS_CPU_SEMANTICS, 1, false><<<grid, block, 0, s>>>(a);
        } else {
            if (vol)
                drain_step_kernel<SBS_CPU_SEMANTICS, 0, true><<<grid, block, 0, s>>>(a);
            else
                drain_step_kernel<SBS_CPU_SEMANTICS, 0, false><<<grid, block, 0, s>>>(a);
        }
    } else if (a.marangoni) {
        if (vol)
            drain_step_kernel<SBS_WGSL_SEMANTICS, 0, true, true><<<grid, block, 0, s>>>(a);
        else
            drain_step_kernel<SBS_WGSL_SEMANTICS, 0, false, true><<<grid, block, 0, s>>>(a);
    } else {
        if (vol)
            drain_step_kernel<SBS_WGSL_SEMANTICS, 0, true, false><<<grid, block, 0, s>>>(a);
        else
            drain_step_kernel<SBS_WGSL_SEMANTICS, 0, false, false><<<grid, block, 0, s>>>(a);
    }
    return cudaGetLastError();
}

cudaError_t launch_finalize_poles(float *h, float *hl, const FixSum *part, int nbx, int nt, int np, int pitch,
                                  cudaStream_t s) {
    finalize_poles_kernel<<<(np + 255) / 256, 256, 0, s>>>(h, hl, part, nbx, nt, np, pitch);
    return cudaGetLastError();
}

int reduce_partials_count(int nt, int /*np*/) { return nt < 1024 ? nt : 1024; }

cudaError_t launch_field_reduce(const float *h, const float *hl, int nt, int np, size_t pitch, const double *w,
                                double *partials, unsigned *counter, ReduceOut *out, cudaStream_t s) {
    const int nb = reduce_partials_count(nt, np);
    field_reduce_kernel<<<nb, kReduceThreads, 0, s>>>(h, hl, nt, np, pitch, w, partials, counter, out);
    return cudaGetLastError();
}

cudaError_t launch_query(const float *h, const float *hl, int nt, int np, size_t pitch, const double *theta,
                         const double *phi, double *out, size_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    query_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(h, hl, nt, np, pitch, theta, phi, out, n);
    return cudaGetLastError();
}

cudaError_t launch_vertex_colors(const float *h, const float *hl, int nt, int np, size_t pitch, const double *xyz,
                                 size_t nv, const double *lut, int T, int A, double tmin, double tmax, double *rgb,
                                 cudaStream_t s) {
    if (nv == 0) return cudaSuccess;
    vertex_colors_kernel<<<(unsigned)((nv + 127) / 128), 128, 0, s>>>(h, hl, nt, np, pitch, xyz, nv, lut, T, A,
                                                                      tmin, tmax, rgb);
    return cudaGetLastError();
}

}  // namespace sbs
