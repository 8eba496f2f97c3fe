/*
 * Parity oracle for the soap-film physics path: a plain C++17 restatement of
 * the reference's CPU and WGSL arithmetic, compiled with gcc and
 * -ffp-contract=off so that every product and sum rounds exactly as the
 * reference's Rust (which never contracts to FMA) does.
 *
 * This is TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py load it, and only as the checker or
 * as the timed CPU baseline. The product library (libsbs) never links it.
 *
 * Pinning: the reference ships no numeric golden vectors for this path and
 * cannot be built here (Rust/wgpu, no toolchain). The oracle is pinned by the
 * reference's own known-answer unit tests (drainage.rs:621-719,
 * interference.rs:619-790, interference_lut.rs:170-204, config.rs:431-464),
 * ported as tests/test_oracle_*.py, plus analytic checks (uniform-field ODE,
 * sphere area). The WGSL semantics (drainage.wgsl) has no numeric test in the
 * reference at all: its parity is "unpinned" beyond this restatement.
 *
 * Precision modes of the drainage restatements:
 *   f64 faithful    - drainage.rs:298-503 exactly (f64, libm sin/cos).
 *   f32 kernel-order- the exact f32 arithmetic of the CUDA kernel (per-row
 *                     coefficients computed in f64 then rounded, explicit fmaf),
 *                     used for bitwise GPU parity.
 *   f32 WGSL        - drainage.wgsl:72-202 in its own operation order (IEEE
 *                     f32 division, sinf/cosf of an f32 angle).
 */
#pragma once
#include <stddef.h>
#include <stdint.h>

#include "../include/sbs.h" /* interface types only (sbs_bubble_uniform, texture sizes) */

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------ */
/* CPU-semantics drainage simulator (drainage.rs:212-614)              */
/* ------------------------------------------------------------------ */
typedef struct orc_sim orc_sim;

typedef struct orc_sim_params {
    uint32_t resolution;          /* N_theta = resolution, N_phi = 2*resolution (drainage.rs:264-265) */
    double diameter;              /* m; radius = diameter/2 (config.rs:357) */
    double film_thickness_nm;     /* initial uniform thickness (config.rs:368) */
    double critical_thickness_nm; /* drainage.rs:278 */
    double density;
    double gravity;
    double viscosity;
    double surfactant_diffusion;  /* used as the thickness diffusion coefficient (drainage.rs:277) */
} orc_sim_params;

/* precision: 0 = f64 faithful, 1 = f32 kernel-order, 2 = compensated f32x2 kernel-order
 * (hi + lo words, TwoSum update, compensated ring sums). threads: OpenMP threads for the
 * stencil loop (0 = OpenMP default, 1 = sequential like the reference). */
orc_sim *orc_sim_new(const orc_sim_params *p, int precision, int threads);
void orc_sim_free(orc_sim *s);
uint32_t orc_sim_num_theta(const orc_sim *s);
uint32_t orc_sim_num_phi(const orc_sim *s);
void orc_sim_set_field(orc_sim *s, const double *h);   /* N_theta*N_phi, meters */
void orc_sim_get_field(const orc_sim *s, double *h);
void orc_sim_step(orc_sim *s, double dt);
void orc_sim_step_n(orc_sim *s, double dt, uint32_t n);
double orc_sim_get_thickness(const orc_sim *s, double theta, double phi);
double orc_sim_current_time(const orc_sim *s);
int orc_sim_has_critical_region(const orc_sim *s);
double orc_sim_min_thickness(const orc_sim *s);
double orc_fix_ring_mean(const float *words, size_t n, uint32_t np);
double orc_sim_max_thickness(const orc_sim *s);
void orc_sim_reset(orc_sim *s, double h0);
void orc_sim_set_marginal_regeneration(orc_sim *s, int enabled);
void orc_sim_set_tfe_thickness_ratio(orc_sim *s, double ratio);
double orc_sim_tfe_thickness_ratio(const orc_sim *s);
uint32_t orc_sim_active_tfe_count(const orc_sim *s);
/* fronts as 4 doubles each: phi_center, extent, width, velocity; returns count */
uint32_t orc_sim_get_fronts(const orc_sim *s, double *out, uint32_t cap);

/* ------------------------------------------------------------------ */
/* WGSL-semantics drainage step (drainage.wgsl:72-202)                 */
/* ------------------------------------------------------------------ */
typedef struct orc_wgsl_params { /* mirrors DrainageParams, gpu_drainage.rs:12-44 */
    float dt, gravity, viscosity, density, diffusion_coeff, bubble_radius, critical_thickness;
    uint32_t grid_width, grid_height, marangoni_enabled;
    float gamma_air, gamma_reduction, surfactant_diffusion, marangoni_coeff;
    uint32_t _padding1, _padding2;
} orc_wgsl_params;

/* mode 0 = WGSL operation order (IEEE f32), mode 1 = CUDA kernel order. n passes, ping-pong
 * internally; results land in h_out/c_out. threads as above. */
void orc_wgsl_run(const orc_wgsl_params *p, int mode, const float *h_in, const float *c_in,
                  float *h_out, float *c_out, uint32_t passes, int threads);

/* ------------------------------------------------------------------ */
/* Film volume (no reference counterpart): sum h * R^2 sin(theta) dth dphi */
/* ------------------------------------------------------------------ */
double orc_film_volume_f64(const double *h, uint32_t n_theta, uint32_t n_phi, double radius);
double orc_film_volume_f32(const float *h, uint32_t n_theta, uint32_t n_phi, double radius);

/* ------------------------------------------------------------------ */
/* InterferenceCalculator (interference.rs:127-512), f64               */
/* ------------------------------------------------------------------ */
double orc_transmission_angle_cos(double n_film, double cos_i);
double orc_optical_path_difference(double n_film, double t_nm, double cos_t, double wl_nm);
double orc_phase_difference(double opd_nm, double wl_nm);
void orc_fresnel(double n_film, double cos_i, double out3[3]); /* s, p, average */
double orc_reflected_intensity(double n_film, double t_nm, double cos_i, double wl_nm);
/* gamma: 1 = calculate_interference_color, 0 = _linear */
void orc_interference_color(double n_film, const double wl[3], double t_nm, double cos_i, int gamma,
                            double rgb[3]);
void orc_interference_color_batch(double n_film, const double wl[3], const double *t_nm,
                                  const double *cos_i, size_t n, int gamma, double *rgb);
void orc_lut1d(double n_film, const double wl[3], double tmin, double tmax, uint32_t count,
               double cos_i, double *rgb /*count*3*/);
void orc_lut2d(double n_film, const double wl[3], double tmin, double tmax, uint32_t T, uint32_t A,
               double *rgb /*T*A*3, [thickness][angle][c]*/);

/* ------------------------------------------------------------------ */
/* generate_interference_lut (interference_lut.rs:18-163), f32 -> RGBA8 */
/* ------------------------------------------------------------------ */
void orc_interference_lut_rgba8(float n_film, float intensity, uint8_t *out /*64*256*4*/);
void orc_thin_film_interference7(float t_nm, float cos_t, float n_film, float intensity,
                                 float out3[3]);
float orc_lut_snells_law(float cos_i, float n_film);
float orc_lut_fresnel_unpolarized(float cos_i, float cos_t, float n1, float n2);

/* ------------------------------------------------------------------ */
/* Schlick / transmitted Airy path (wall.wgsl:176-207), f32            */
/* ------------------------------------------------------------------ */
float orc_schlick_interference(float t_nm, float wl_nm, float cos_i, float n_film);

/* ------------------------------------------------------------------ */
/* LUT lookups (bubble.wgsl:425-439 and the grid-aligned 2-D LUT read) */
/* ------------------------------------------------------------------ */
/* texel-centre bilinear lookup of the RGBA8 LUT ([angle][thickness][4], W x H texels), the
 * ClampToEdge/Linear sampler of pipeline.rs:350-359; result * intensity clamped to [0,1]. */
void orc_lut_rgba8_sample(const uint8_t *lut, uint32_t W, uint32_t H, float t_nm, float cos_i,
                          float max_nm, float intensity, float out3[3]);
/* grid-aligned bilinear read of a [T][A][3] f64 LUT over [tmin,tmax] x cos in [0,1]. */
void orc_lut2d_lookup(const double *lut, uint32_t T, uint32_t A, double tmin, double tmax,
                      double t_nm, double cos_i, double out3[3]);

/* C0 vertex colouring: for each unit vertex (x,y,z): theta = acos(y), phi = atan2(z,x) mod 2pi
 * (geometry.rs:40-60), t = get_thickness(theta,phi)*1e9 on an f64 field, cos = |z| (view +z),
 * rgb = grid-aligned lookup into the [T][A][3] LUT. */
void orc_vertex_colors(const double *field, uint32_t n_theta, uint32_t n_phi, const double *xyz,
                       size_t nv, const double *lut, uint32_t T, uint32_t A, double tmin,
                       double tmax, double *rgb);

/* ------------------------------------------------------------------ */
/* Spectral interference (81 wavelengths) against a CMF, f64           */
/* ------------------------------------------------------------------ */
/* per point: R(l) = Airy reflectance (interference_lut.rs:45-93 formulation with full Fresnel,
 * phase + pi) at wavelength l; rgb[c] = sum_l R(l) * cmf[l][c]. */
void orc_spectral_rgb(const float *t_nm, const float *cos_i, const float *n_film, size_t n,
                      const double *wl, uint32_t nl, const double *cmf /*nl*3*/, double *rgb);


/* ------------------------------------------------------------------ */
/* Drainage surrogate (conv neural operator, include/sbs_nn.h)          */
/* ------------------------------------------------------------------ */
/* Restates the network definition of include/sbs_nn.h in double arithmetic on BF16-rounded
 * operands (x, weights, activations, and in the backward pass the per-layer output gradients),
 * rounding the layer pre-activations to float where the CUDA path holds them in FP32.
 * Tensors are channel-last: [nb][nt][np][ch]. */
/* features of one field (nt = grid_height, np = grid_width of p); x: nt*np*16 BF16-valued floats */
void orc_nn_features(const float *h, const float *c, const orc_wgsl_params *p, float *x);
/* kout of one field (include/sbs_nn.h) */
float orc_nn_kout(const orc_wgsl_params *p);
/* forward: y (nb*nt*np) from x (nb*nt*np*16) with the FP32 parameter vector (BF16-rounded inside);
 * act = SBS_NN_ACT_GELU or SBS_NN_ACT_HSWISH */
void orc_nn_forward(const float *params, uint32_t nb, uint32_t nt, uint32_t np, const float *x, float *y, int act);
/* masked mean-square loss of y against target over rows with sin(theta) >= SBS_NN_MASK_SIN and its
 * gradient (SBS_NN_PARAMS floats). Returns the loss. */
double orc_nn_loss_grad(const float *params, uint32_t nb, uint32_t nt, uint32_t np, const float *x,
                        const float *target, float *grad, int act);
/* h_out = surrogate update of h given the network output y (include/sbs_nn.h "Map") */
void orc_nn_apply(const float *h, const float *y, uint32_t nt, uint32_t np, float kout, float *h_out);
/* 1: drop every BF16 / float rounding (all-double network), for finite-difference checks */
void orc_nn_set_exact(int exact);
/* the activations and their derivatives in the FP32 form of include/sbs_nn.h */
float orc_nn_gelu(float x);
float orc_nn_gelu_grad(float x);
float orc_nn_hswish(float x);
float orc_nn_hswish_grad(float x);

/* ------------------------------------------------------------------ */
/* Bubble fragment shader (bubble.wgsl) and headless frame             */
/* ------------------------------------------------------------------ */
/* simplex_noise_3d (bubble.wgsl:113-180) and get_film_thickness (:203-229) */
float orc_simplex3(float x, float y, float z);
float orc_film_thickness(const sbs_bubble_uniform *u, float nx, float ny, float nz);
/* fs_main (:486-545) for n fragments: normal, wpos [n][3] -> rgba [n][4] (straight alpha) */
void orc_shade_fragments(const sbs_bubble_uniform *u, const float cam[3], const uint8_t *lut, const uint32_t *tex,
                         size_t n, const float *normal, const float *wpos, float *rgba);
/* one headless frame (render/headless.rs), as sbs_shade_frame; -1 if view_proj is singular */
int orc_shade_frame(const sbs_bubble_uniform *u, const float view_proj[16], const float cam[3], float radius,
                    const uint8_t *lut, const uint32_t *tex, uint32_t width, uint32_t height, uint8_t *rgba8,
                    float *linear);

/* caustic compute pass (caustics_compute.wgsl:1-126): out [grid_height][grid_width] */
void orc_caustics(const sbs_caustic_params *p, const float *h, size_t pitch, float *out);

/* branched flow (branched_flow_compute.wgsl, branched_flow.rs): the library's acos / atan2 / exp,
 * scatterer generation, and one fade + trace step into tex (accumulated in place) */
float orc_acos_as(float x);
float orc_atan2_as(float y, float x);
float orc_exp_cw(float x);
void orc_branched_scatterers(const sbs_branched_params *p, uint32_t num, float time, sbs_scatterer *out);
void orc_branched_flow(const sbs_branched_params *p, const float *th, uint32_t w, uint32_t h, size_t pitch,
                       const sbs_scatterer *sc, uint32_t *tex, int fade);

/* foam cluster dynamics (foam_dynamics.rs, foam.rs), the reference's O(n^2) loops: forces [n][3]
 * of compute_forces; `steps` FoamSimulator::step calls on arrays in cluster order (updated in place,
 * the new count returned), the final connections() into conn (up to cap, *nconn = count) */
float orc_pow15(float x);
void orc_foam_forces(const sbs_foam_physics *p, uint32_t n, const float *pos, const float *vel, const float *radius,
                     const float *thick, float *out);
void orc_foam_forces_subset(const sbs_foam_physics *p, uint32_t n, const float *pos, const float *vel,
                            const float *radius, const float *thick, const uint32_t *idx, uint32_t m, float *out);
uint32_t orc_foam_step(const sbs_foam_physics *p, float dt, uint32_t steps, uint32_t n, float *pos, float *vel,
                       float *radius, float *thick, uint32_t *ids, uint32_t *next_id, sbs_bubble_connection *conn,
                       uint32_t cap, uint32_t *nconn);

#ifdef __cplusplus
}
#endif
