// One row of the time-skewed register pipeline that advances a warp's 128-column window of the
// WGSL-semantics fields by K steps (used by the single-bubble and the batched foam kernels, so
// both round identically). See drainage_wtb.cu for the scheme.
#pragma once

#include <cuda_runtime.h>

#include "caustics.cuh"
#include "cell.cuh"

namespace sbs {

#ifndef SBS_WTB_PREFETCH
#define SBS_WTB_PREFETCH 1  // request level-0 row t+1 while computing row t (0: load it at row t)
#endif

struct Wtb {
    const float *hin, *cin;  // column-offset input pointers of this lane
    float *hout, *cout;      // column-offset output pointers
    const float4 *sco;       // this strip's per-row coefficients in shared memory, from row sco_base
    int sco_base;
    int nt, pitch, r0, r1;
    bool store;
    float b, DR2, DsR2, Gt, M, dt, crit;
    const double *vol_w;
    // caustic map of the launch's result (CAU launches only)
    float *cau_out;          // column-offset map pointer (rows of cau_stride floats)
    int cau_stride;
    int cau_j0, cau_j1;      // map rows this strip writes
    float cau_focal, cau_scale, cau_sharp, cau_branch;
};

// Caustic map row j (caustics_compute.wgsl:87-111) from the final rows above (a), at (b) and below
// (c) j; phi neighbours by shuffle (all lanes call; kept lanes store).
__device__ __forceinline__ void wtb_caustic_row(const Wtb &w, int j, const float4 &a, const float4 &b,
                                                const float4 &c) {
    const float al = __shfl_up_sync(0xffffffffu, a.w, 1), ar = __shfl_down_sync(0xffffffffu, a.x, 1);
    const float bl = __shfl_up_sync(0xffffffffu, b.w, 1), br = __shfl_down_sync(0xffffffffu, b.x, 1);
    const float cl = __shfl_up_sync(0xffffffffu, c.w, 1), cr = __shfl_down_sync(0xffffffffu, c.x, 1);
    const float av[6] = {al, a.x, a.y, a.z, a.w, ar}, bv[6] = {bl, b.x, b.y, b.z, b.w, br};
    const float cv[6] = {cl, c.x, c.y, c.z, c.w, cr};
    float o[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
        o[k] = caustic_intensity(w.cau_focal, w.cau_scale, w.cau_sharp, w.cau_branch,
                                 CausticRow{av[k], av[k + 1], av[k + 2]}, CausticRow{bv[k], bv[k + 1], bv[k + 2]},
                                 CausticRow{cv[k], cv[k + 1], cv[k + 2]});
    if (w.store) *reinterpret_cast<float4 *>(w.cau_out + (size_t)j * w.cau_stride) = make_float4(o[0], o[1], o[2], o[3]);
}

// One pipeline iteration: load level-0 row t, then compute level l of row t - l for l = 1..K.
// Slot P holds the row most recently written to each level's window.
// With SBS_WTB_PREFETCH the level-0 row t arrives in (ph, pc), loaded one iteration earlier, and
// row t + 1 is requested here; otherwise row t is loaded here.
// CAU: the launch also writes the caustic map of its result. Every level then covers one more row
// on each side (the strip's final rows r0 - 1 and r1 are needed), wk keeps the last three final
// rows, and map row j is written once final row j + 1 exists (theta clamped at the poles).
// STEADY: the caller guarantees that every level's row lies inside the strip's window and the
// grid, none is a pole row, the final row is one of the strip's own rows and the prefetched row
// t + 1 exists; the iteration then skips those tests (same arithmetic, same bits).
template <int K, int P, bool VOL, bool MAR, bool CG = false, bool CAU = false, bool STEADY = false>
__device__ __forceinline__ void wtb_iter(const Wtb &w, int t, float4 (&wh)[K][3], float4 (&wc)[K][3], float4 &ph,
                                         float4 &pc, double &vacc, float4 *wk = nullptr) {
    constexpr int CUR = (P + 2) % 3, UP = (P + 1) % 3;
    constexpr int E = CAU ? 1 : 0;
    const int tl = SBS_WTB_PREFETCH ? t + 1 : t;
    float4 nh = make_float4(0.f, 0.f, 0.f, 0.f), nc = nh;
    if (STEADY || (tl >= 0 && tl < w.nt)) {
        const float4 *ph4 = reinterpret_cast<const float4 *>(w.hin + (size_t)tl * w.pitch);
        const float4 *pc4 = reinterpret_cast<const float4 *>(w.cin + (size_t)tl * w.pitch);
        nh = CG ? __ldcg(ph4) : __ldg(ph4);
        nc = CG ? __ldcg(pc4) : __ldg(pc4);
    }
    if (SBS_WTB_PREFETCH) {
        wh[0][P] = ph;
        wc[0][P] = pc;
        ph = nh;
        pc = nc;
    } else {
        wh[0][P] = nh;
        wc[0][P] = nc;
    }
#pragma unroll
    for (int l = 1; l <= K; ++l) {
        const int i = t - l;
        const bool need =
            STEADY || (i >= w.r0 - (K - l) - E && i < w.r1 + (K - l) + E && i >= 0 && i < w.nt);  // warp-uniform
        float4 oh = make_float4(0.f, 0.f, 0.f, 0.f), oc = oh;
        if (need) {
            const float4 hc = wh[l - 1][CUR], cc = wc[l - 1][CUR];
            if (!STEADY && (i == 0 || i == w.nt - 1)) {  // pole rows are frozen (drainage.wgsl:85-89)
                oh = hc;
                oc = cc;
            } else {
                const float4 hu = wh[l - 1][UP], hd = wh[l - 1][P];
                const float4 cu = wc[l - 1][UP], cd = wc[l - 1][P];
                const float4 co = w.sco[i - w.sco_base];
                const float hl = __shfl_up_sync(0xffffffffu, hc.w, 1), hr = __shfl_down_sync(0xffffffffu, hc.x, 1);
                const float cl = __shfl_up_sync(0xffffffffu, cc.w, 1), cr = __shfl_down_sync(0xffffffffu, cc.x, 1);
                const float4 hpm = make_float4(hl, hc.x, hc.y, hc.z), hpp = make_float4(hc.y, hc.z, hc.w, hr);
                const float4 cpm = make_float4(cl, cc.x, cc.y, cc.z), cpp = make_float4(cc.y, cc.z, cc.w, cr);
                wgsl_cell4<MAR>(hc, hu, hd, hpm, hpp, cc, cu, cd, cpm, cpp, co, w.b, w.DR2, w.DsR2, w.Gt, w.M, w.dt,
                                w.crit, oh, oc);
            }
        }
        if (l < K) {
            wh[l][P] = oh;
            wc[l][P] = oc;
        } else {
            if (STEADY ? w.store : (need && i >= w.r0 && i < w.r1 && w.store)) {
                *reinterpret_cast<float4 *>(w.hout + (size_t)i * w.pitch) = oh;
                *reinterpret_cast<float4 *>(w.cout + (size_t)i * w.pitch) = oc;
                if (VOL) vacc += ((double)oh.x + (double)oh.y + (double)oh.z + (double)oh.w) * __ldg(w.vol_w + i);
            }
            if (CAU) {
                wk[P] = oh;
                const int j = i - 1;  // warp-uniform
                if (j >= w.cau_j0 && j < w.cau_j1) wtb_caustic_row(w, j, j == 0 ? wk[CUR] : wk[UP], wk[CUR], wk[P]);
                if (i == w.nt - 1 && i >= w.cau_j0 && i < w.cau_j1) wtb_caustic_row(w, i, wk[CUR], wk[P], wk[P]);
            }
        }
    }
}


}  // namespace sbs
