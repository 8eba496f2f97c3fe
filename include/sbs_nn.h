/*
 * Definition of the drainage surrogate: a 4-layer convolutional neural
 * operator that advances a WGSL-semantics film (drainage.wgsl:72-202, the
 * GPUDrainageSimulator path) by SBS_NN_STEPS drainage steps in one pass.
 * Pure constants: the CUDA implementation and any CPU restatement of the
 * network follow this file, and a saved weight vector is only meaningful
 * together with it.
 *
 * Map.  h' = h + kout * y  on rows 1 .. nt-2 (then max(., 0)); rows 0 and nt-1
 * are copied (the WGSL kernel freezes the poles).  y is the network output:
 *
 *   x  = features(h, surfactant, viscosity, diameter)           [nt][np][16]
 *   a1 = act(conv3x3(x,  W1) + b1)    16 -> 32
 *   a2 = act(conv3x3(a1, W2) + b2)    32 -> 32
 *   a3 = act(conv3x3(a2, W3) + b3)    32 -> 32
 *   y  =      conv3x3(a3, W4) + b4    32 -> 1
 *
 * conv3x3 pads periodically in phi (columns) and by reflection in theta
 * (rows): row -1 reads row 1 and row nt reads row nt-2.  x and a1..a3 are
 * BF16, the weights are BF16, every sum accumulates in FP32.
 *
 * Features (FP32, then clamped to +-SBS_NN_FEATURE_CLAMP and rounded to BF16),
 * with n/s = rows i-1/i+1 (reflected), w/e = columns j-1/j+1 (periodic):
 *   f0 = (h - SBS_NN_H0) * SBS_NN_INV_HS                       film thickness
 *   f1 = ((h_n + h_s) - (h + h)) * ct                          theta curvature
 *   f2 = ((h_w + h_e) - (h + h)) * cp[i]                       phi curvature / sin^2
 *   f3 = (h_s - h_n) * cg[i]                                   cot(theta) * slope
 *   f4 = (surfactant - 0.5) * 10                               surfactant
 *   f5 = log10(viscosity / 1e-3)                               log-viscosity
 *   f6 = 3 * log10(diameter / 0.035)                           log-diameter
 *   f7 = (h * h * h) * (gk * sin(theta_i))                     gravity drainage
 *   f8 = lt                                                    log10 theta diffusion number / MU_REF
 *   f9 = lp[i]                                                 log10 phi diffusion number / MU_REF
 *   f10 = sin(theta_i);  f11 .. f15 = 0
 * with dth = pi/(nt-1), dph = 2 pi/np, se_i = max(sin(i dth), SBS_NN_SIN_FLOOR),
 *   ct = 1/(dth^2 S2), cp[i] = 1/(dph^2 se_i^2 S2), cg[i] = cos(i dth)/(se_i 2 dth S2),
 *   gk = -(density gravity / (3 viscosity)) / ((diffusion_coeff / R^2) S2),
 *   mu = SBS_NN_STEPS * dt * diffusion_coeff / R^2,  lm = log10(mu / SBS_NN_MU_REF),
 *   lt = lm + log10(1 / dth^2),  lp[i] = lm + log10(1 / (dph^2 se_i^2))  (each log
 *   computed in double and rounded to float, the sums in float),
 *   kout = mu * S2,  R = bubble_radius,
 * the other constants computed in double and rounded to float.  The geometry-weighted finite
 * differences carry the latitude dependence of the surface Laplacian (a
 * translation-invariant convolution cannot see theta) and keep the curvature
 * of a smooth field, which is below BF16 resolution relative to h itself at
 * fine grids, exact in FP32 before the network sees it.  The diffusion numbers
 * of the SBS_NN_STEPS-pass interval (per cell, in each direction) tell the
 * network how far the interval spreads a perturbation, which sets the response
 * independently of the grid resolution.
 *
 * Parameters: one FP32 vector of SBS_NN_PARAMS values, per layer W[tap][oc][ic]
 * then b[oc], tap = (dy + 1) * 3 + (dx + 1) with dy the row (theta) offset and
 * dx the column (phi) offset of the input cell read for an output cell.
 *
 * Activation (after every layer but the last), chosen per network
 * (sbs_surrogate_set_activation):
 *
 * SBS_NN_ACT_GELU (default): gelu(x) = x * phi(x), phi(x) = 0.5 + t p(t^2),
 * t = clamp(x, -3, 3), p(u) = Q0 + Q1 u + Q2 u^2 + Q3 u^3 + Q4 u^4.  The Qk are a
 * least-squares fit of the normal CDF minus 1/2 on [0, 3] under the constraint
 * phi(3) = 1, so phi is 0 / 1 (to float rounding) beyond -3 / 3 (max
 * |phi - normal CDF| = 1.35e-3, max |gelu - x * normal CDF| = 4.0e-3).  In FP32:
 *   p = fma(fma(fma(fma(Q4, u, Q3), u, Q2), u, Q1), u, Q0); phi = fma(t, p, 0.5)
 * and the derivative
 *   dp = fma(fma(fma(Q4x4, u, Q3x3), u, Q2x2), u, Q1)
 *   dphi = |x| < 3 ? fma(u + u, dp, p) : 0;  gelu'(x) = fma(x, dphi, phi).
 *
 * SBS_NN_ACT_HSWISH: hard-swish, hswish(x) = x * s(x), s(x) = sat(x / 6 + 1/2),
 * sat() clamping to [0, 1]: two FP32 operations (the saturation is a modifier of
 * the fused multiply-add on the GPU) against eleven for the GELU polynomial.  In
 * FP32:
 *   r = fma(x, SBS_NN_HS_SLOPE, 0.5);  s = sat(r) (NaN -> 0);  hswish = x * s
 * and the derivative
 *   hswish'(x) = (0 < r < 1) ? fma(x, SBS_NN_HS_SLOPE, s) : s.
 */
#pragma once

#define SBS_NN_NF 16
#define SBS_NN_C 32
#define SBS_NN_STEPS 64

#define SBS_NN_W1 0
#define SBS_NN_B1 4608
#define SBS_NN_W2 4640
#define SBS_NN_B2 13856
#define SBS_NN_W3 13888
#define SBS_NN_B3 23104
#define SBS_NN_W4 23136
#define SBS_NN_B4 23424
#define SBS_NN_PARAMS 23425

#define SBS_NN_H0 5.5e-7f
#define SBS_NN_INV_HS 6666666.5f /* float(1 / 150 nm) */
#define SBS_NN_S2 1e-5
#define SBS_NN_SIN_FLOOR 0.05
#define SBS_NN_FEATURE_CLAMP 1.0e4f
/* Rows with sin(theta) >= SBS_NN_MASK_SIN form the training loss and the
 * surrogate-versus-plain checks (rows nearer the poles are excluded: at fine
 * grids the explicit scheme is unstable there). */
#define SBS_NN_MASK_SIN 0.2
#define SBS_NN_MU_REF 0.044

#define SBS_NN_ACT_GELU 0
#define SBS_NN_ACT_HSWISH 1

#define SBS_NN_Q0 0.39817786f
#define SBS_NN_Q1 (-0.064430825f)
#define SBS_NN_Q2 0.0083782589f
#define SBS_NN_Q3 (-0.00064844202f)
#define SBS_NN_Q4 2.1710333e-05f
#define SBS_NN_Q2X2 0.016756518f
#define SBS_NN_Q3X3 (-0.0019453261f)
#define SBS_NN_Q4X4 8.6841333e-05f
#define SBS_NN_HS_SLOPE 0.16666667f /* float(1 / 6) */
