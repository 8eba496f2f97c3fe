// Per-cell update of the drainage step, shared by every step kernel so that all of them round
// identically (and the oracle's kernel-order mode can repeat them).
//
// The update runs on pairs of neighbouring cells with Blackwell's packed FP32 instructions
// (__fadd2_rn / __fmul2_rn / __ffma2_rn: two IEEE round-to-nearest f32 operations per
// instruction). Each half rounds exactly like the scalar operation, and a - b is written as
// a + (-b) (negation is exact), so results are bit-identical to the scalar formula while the
// floating-point instruction count halves.
#pragma once

#include <cuda_runtime.h>

namespace sbs {

__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, neg2(b)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

// GPUDrainageSimulator semantics (drainage.wgsl:104-201) for two cells of h and surfactant Gamma.
//   co = per-row (A, E, F, G); neighbours theta-1 (tm), theta+1 (tp), phi-1 (pm), phi+1 (pp).
//   lt = (tp-h)+(tm-h), d1 = tp-tm, lp = (pp-h)+(pm-h), L = F*lp + E*d1 + b*lt
//   h' = max(h + dt*(D/R^2*L + A*h^3 [+ M*|grad Gamma|*h^2]), 0)
//   Gamma' = clamp(Gamma + dt*(Ds/R^2*L_Gamma [+ 0.001*L*Gamma]), 0, 1)
// Branch-free: the update is always evaluated and cells below the critical thickness keep their
// values by selection (drainage.wgsl:108-112), which gives the same bits as skipping them.
template <bool MAR>
__device__ __forceinline__ void wgsl_cell2(float2 h, float2 tm, float2 tp, float2 pm, float2 pp, float2 cv, float2 ctm,
                                           float2 ctp, float2 cpm, float2 cpp, const float4 &co, float b, float DR2,
                                           float DsR2, float Gt, float M, float dt, float crit, float2 &vh,
                                           float2 &vc) {
    const float2 lt = add2(sub2(tp, h), sub2(tm, h));
    const float2 d1 = sub2(tp, tm);
    const float2 lp = add2(sub2(pp, h), sub2(pm, h));
    const float2 L = fma2(f2(co.z), lp, fma2(f2(co.y), d1, mul2(f2(b), lt)));
    const float2 h3 = mul2(mul2(h, h), h);
    float2 inc = fma2(f2(DR2), L, mul2(f2(co.x), h3));
    if (MAR) {
        const float2 gt = mul2(f2(Gt), sub2(ctp, ctm));
        const float2 gp = mul2(f2(co.w), sub2(cpp, cpm));
        const float2 sq = fma2(gt, gt, mul2(gp, gp));
        const float2 mag = make_float2(sqrtf(sq.x), sqrtf(sq.y));
        inc = add2(inc, mul2(mul2(f2(M), mag), mul2(h, h)));
    }
    const float2 lc = add2(sub2(ctp, cv), sub2(ctm, cv));
    const float2 d1c = sub2(ctp, ctm);
    const float2 lpc = add2(sub2(cpp, cv), sub2(cpm, cv));
    const float2 Lc = fma2(f2(co.z), lpc, fma2(f2(co.y), d1c, mul2(f2(b), lc)));
    float2 dc = mul2(f2(DsR2), Lc);
    if (MAR) dc = fma2(mul2(f2(0.001f), L), cv, dc);
    const float2 y = fma2(f2(dt), dc, cv);
    const float2 x = fma2(f2(dt), inc, h);
    float y0 = y.x > 0.f ? y.x : 0.f, y1 = y.y > 0.f ? y.y : 0.f;
    y0 = y0 < 1.f ? y0 : 1.f;
    y1 = y1 < 1.f ? y1 : 1.f;
    const float x0 = x.x > 0.f ? x.x : 0.f, x1 = x.y > 0.f ? x.y : 0.f;
    vh.x = h.x < crit ? h.x : x0;
    vh.y = h.y < crit ? h.y : x1;
    vc.x = h.x < crit ? cv.x : y0;
    vc.y = h.y < crit ? cv.y : y1;
}

// The same update for the four cells of a float4 (two pairs).
template <bool MAR>
__device__ __forceinline__ void wgsl_cell4(const float4 &h, const float4 &tm, const float4 &tp, const float4 &pm,
                                           const float4 &pp, const float4 &cv, const float4 &ctm, const float4 &ctp,
                                           const float4 &cpm, const float4 &cpp, const float4 &co, float b, float DR2,
                                           float DsR2, float Gt, float M, float dt, float crit, float4 &vh,
                                           float4 &vc) {
    float2 a, c, e, g;
    wgsl_cell2<MAR>(make_float2(h.x, h.y), make_float2(tm.x, tm.y), make_float2(tp.x, tp.y), make_float2(pm.x, pm.y),
                    make_float2(pp.x, pp.y), make_float2(cv.x, cv.y), make_float2(ctm.x, ctm.y),
                    make_float2(ctp.x, ctp.y), make_float2(cpm.x, cpm.y), make_float2(cpp.x, cpp.y), co, b, DR2, DsR2,
                    Gt, M, dt, crit, a, c);
    wgsl_cell2<MAR>(make_float2(h.z, h.w), make_float2(tm.z, tm.w), make_float2(tp.z, tp.w), make_float2(pm.z, pm.w),
                    make_float2(pp.z, pp.w), make_float2(cv.z, cv.w), make_float2(ctm.z, ctm.w),
                    make_float2(ctp.z, ctp.w), make_float2(cpm.z, cpm.w), make_float2(cpp.z, cpp.w), co, b, DR2, DsR2,
                    Gt, M, dt, crit, e, g);
    vh = make_float4(a.x, a.y, e.x, e.y);
    vc = make_float4(c.x, c.y, g.x, g.y);
}

}  // namespace sbs

namespace sbs {

// DrainageSimulator semantics (drainage.rs:326-379) for two cells, plain f32 (X2 = false) or
// compensated hi + lo words (X2 = true: differences include the lo words and h + dt*inc is an
// error-free TwoSum). Cells below the critical thickness keep their words (drainage.rs:331).
template <bool X2>
__device__ __forceinline__ void cpu_cell2(float2 h, float2 tm, float2 tp, float2 pm, float2 pp, float2 l, float2 tml,
                                          float2 tpl, float2 pml, float2 ppl, const float4 &co, float b, float DR2,
                                          float dt, float crit, float2 &vh, float2 &vl) {
    float2 lt = add2(sub2(tp, h), sub2(tm, h));
    float2 d1 = sub2(tp, tm);
    float2 lp = add2(sub2(pp, h), sub2(pm, h));
    if (X2) {
        lt = add2(lt, add2(sub2(tpl, l), sub2(tml, l)));
        d1 = add2(d1, sub2(tpl, tml));
        lp = add2(lp, add2(sub2(ppl, l), sub2(pml, l)));
    }
    const float2 L = fma2(f2(co.z), lp, fma2(f2(co.y), d1, mul2(f2(b), lt)));
    const float2 h3 = mul2(mul2(h, h), h);
    const float2 inc = fma2(f2(DR2), L, mul2(f2(co.x), h3));
    if (X2) {
        const float2 t = fma2(f2(dt), inc, l);
        const float2 s = add2(h, t);
        const float2 bb = sub2(s, h);
        const float2 e = add2(sub2(h, sub2(s, bb)), sub2(t, bb));
        vh.x = h.x < crit ? h.x : (s.x < 0.f ? 0.f : s.x);
        vh.y = h.y < crit ? h.y : (s.y < 0.f ? 0.f : s.y);
        vl.x = h.x < crit ? l.x : (s.x < 0.f ? 0.f : e.x);
        vl.y = h.y < crit ? l.y : (s.y < 0.f ? 0.f : e.y);
    } else {
        const float2 x = fma2(f2(dt), inc, h);
        vh.x = h.x < crit ? h.x : (x.x > 0.f ? x.x : 0.f);
        vh.y = h.y < crit ? h.y : (x.y > 0.f ? x.y : 0.f);
        vl = make_float2(0.f, 0.f);
    }
}

template <bool X2>
__device__ __forceinline__ void cpu_cell4(const float4 &h, const float4 &tm, const float4 &tp, const float4 &pm,
                                          const float4 &pp, const float4 &l, const float4 &tml, const float4 &tpl,
                                          const float4 &pml, const float4 &ppl, const float4 &co, float b, float DR2,
                                          float dt, float crit, float4 &vh, float4 &vl) {
    float2 a, c, e, g;
    cpu_cell2<X2>(make_float2(h.x, h.y), make_float2(tm.x, tm.y), make_float2(tp.x, tp.y), make_float2(pm.x, pm.y),
                  make_float2(pp.x, pp.y), make_float2(l.x, l.y), make_float2(tml.x, tml.y), make_float2(tpl.x, tpl.y),
                  make_float2(pml.x, pml.y), make_float2(ppl.x, ppl.y), co, b, DR2, dt, crit, a, c);
    cpu_cell2<X2>(make_float2(h.z, h.w), make_float2(tm.z, tm.w), make_float2(tp.z, tp.w), make_float2(pm.z, pm.w),
                  make_float2(pp.z, pp.w), make_float2(l.z, l.w), make_float2(tml.z, tml.w), make_float2(tpl.z, tpl.w),
                  make_float2(pml.z, pml.w), make_float2(ppl.z, ppl.w), co, b, DR2, dt, crit, e, g);
    vh = make_float4(a.x, a.y, e.x, e.y);
    vl = make_float4(c.x, c.y, g.x, g.y);
}

}  // namespace sbs
