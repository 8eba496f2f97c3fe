/*
 * sbs.h - C ABI of the GB300 soap-film physics library (libsbs.so).
 *
 * The library replaces, one for one, the data-parallel physics path of the
 * soap-bubble simulation: the film-drainage time step on the bubble's
 * theta-phi thickness grid and the thin-film interference evaluation. Every
 * entry point below names the reference item it replaces (path:line inside
 * the reference project). All compute runs as CUDA kernels on one GPU; there
 * is no CPU fallback, and a missing or unusable GPU makes calls fail with
 * SBS_E_CUDA.
 *
 * Conventions
 *  - Every function returns SBS_OK (0) or a negative SBS_E_* code; the text of
 *    the last error of the calling thread is sbs_last_error().
 *  - A drainage handle owns its device memory and one CUDA stream. It is used
 *    by one thread at a time (the reference takes &mut self). Different
 *    handles are independent.
 *  - Host pointers are borrowed for the duration of the call. Calls that take
 *    or return host data are synchronous.
 *  - Stateless batch calls take `int mem` (SBS_MEM_HOST or SBS_MEM_DEVICE) and
 *    `void *stream` (a cudaStream_t, NULL = the legacy default stream). With
 *    SBS_MEM_HOST the call copies in, computes, copies out and synchronises.
 *    With SBS_MEM_DEVICE all pointers are device pointers and the call only
 *    enqueues work on `stream` (asynchronous).
 *  - Thickness is in metres on the drainage side and in nanometres on the
 *    interference side, as in the reference.
 */
#ifndef SBS_H
#define SBS_H

#include <stddef.h>
#include <stdint.h>

#include "sbs_nn.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SBS_OK 0
#define SBS_E_INVALID (-1)   /* bad argument or size */
#define SBS_E_CUDA (-2)      /* CUDA runtime error, or no usable GPU */
#define SBS_E_TIMEOUT (-3)   /* a bounded device-side wait ran out */
#define SBS_E_NONFINITE (-4) /* a result was NaN or infinite where the caller asked for a check */
#define SBS_E_NOMEM (-5)     /* device or host allocation failed */
#define SBS_E_STATE (-6)     /* call not valid for this handle's semantics or state */

#define SBS_MEM_HOST 0
#define SBS_MEM_DEVICE 1

/* Which reference solver a drainage handle reproduces. */
#define SBS_CPU_SEMANTICS 0  /* DrainageSimulator (drainage.rs:212-614): pole ring means, TFE fronts */
#define SBS_WGSL_SEMANTICS 1 /* GPUDrainageSimulator + drainage.wgsl: surfactant field, frozen poles */

/* Interference arithmetic precision. */
#define SBS_PREC_F64 0 /* same f64 arithmetic as InterferenceCalculator */
#define SBS_PREC_F32 1 /* f32 arithmetic (within 1e-4 of f64 on RGB) */

/* LUT lookup addressing. */
#define SBS_LOOKUP_GRID 0  /* bilinear in index space: entry i sits at tmin + i*(tmax-tmin)/(T-1) */
#define SBS_LOOKUP_TEXEL 1 /* texture addressing: texel centres at (i+0.5)/W, clamp to edge */

const char *sbs_last_error(void);
const char *sbs_version(void);
/* Number of CUDA devices visible, or a negative code. */
int sbs_device_count(int *out);

/* Bounded device-side waits (no reference counterpart). Every wait inside this
 * library's kernels - the foam batch's grid barrier, the pole-ring barrier of the
 * blocked DrainageSimulator step, the mbarrier waits of the tensor-core spectral
 * contraction and of the fused surrogate kernel - gives up
 * after `cycles` SM clock cycles (default 2e9, about one second): the kernel
 * records the timeout, finishes its outstanding tensor-core work, frees its
 * tensor memory and exits, and the call returns SBS_E_TIMEOUT; the context and
 * the handles stay usable. The limit is process-wide and applies to launches
 * made after the call (handles rebuild their captured CUDA graphs). */
int sbs_set_wait_limit(uint64_t cycles);
int sbs_wait_limit(uint64_t *out);

/* Test switch for the timeout path (no reference counterpart): makes the
 * bounded waits of later launches unsatisfiable without faulting anything.
 * SBS_STALL_TENSOR_COMMITS: the tensor-core kernels issue neither their MMAs
 * nor the commits that signal them, so nothing asynchronous is in flight when
 * the waits expire. SBS_STALL_GRID_BARRIER: the foam kernel's grid barrier and
 * the pole-ring barrier of the blocked DrainageSimulator step expect one arrival
 * more than there are blocks. 0 (the default) turns both off.
 * Process-wide; meant for tests, which set a short wait limit first. */
#define SBS_STALL_TENSOR_COMMITS 1
#define SBS_STALL_GRID_BARRIER 2
int sbs_set_stall_injection(int flags);

/* ------------------------------------------------------------------ */
/* Configuration: SimulationConfig (config.rs:283-302) and its         */
/* defaults (config.rs:26-35, 56-66, 93-103, 305-316).                 */
/* ------------------------------------------------------------------ */
typedef struct sbs_config {
    /* BubbleParameters (config.rs:12-24) */
    double diameter;              /* m */
    double film_thickness_nm;     /* initial uniform thickness */
    double critical_thickness_nm; /* cells thinner than this are frozen */
    double refractive_index;
    /* FluidParameters (config.rs:38-54) */
    double viscosity;                /* Pa s */
    double surface_tension;          /* N/m (not used by either drainage solver, as in the reference) */
    double density;                  /* kg/m^3 */
    double surfactant_diffusion;     /* m^2/s; the thickness diffusion coefficient (drainage.rs:277) */
    double surfactant_concentration; /* initial Gamma for the WGSL-semantics solver */
    /* EnvironmentParameters (config.rs:70-88) */
    double gravity;     /* m/s^2 */
    double temperature; /* K */
    double pressure;    /* Pa */
    double dt;          /* s */
    uint32_t resolution; /* N_theta = resolution, N_phi = 2*resolution */
    uint32_t _reserved;
} sbs_config;

/* SimulationConfig::default (config.rs:305-316). */
int sbs_config_default(sbs_config *out);

/* DrainageParams (gpu_drainage.rs:12-44), 64 bytes, same field order. */
typedef struct sbs_drainage_params {
    float dt;
    float gravity;
    float viscosity;
    float density;
    float diffusion_coeff;
    float bubble_radius;
    float critical_thickness;
    uint32_t grid_width;  /* phi points */
    uint32_t grid_height; /* theta points */
    uint32_t marangoni_enabled;
    float gamma_air;
    float gamma_reduction;
    float surfactant_diffusion;
    float marangoni_coeff;
    uint32_t _padding1;
    uint32_t _padding2;
} sbs_drainage_params;

/* DrainageParams::default (gpu_drainage.rs:46-68). */
int sbs_drainage_params_default(sbs_drainage_params *out);

/* ------------------------------------------------------------------ */
/* Drainage handle                                                     */
/* ------------------------------------------------------------------ */
typedef struct sbs_drainage sbs_drainage;

/* DrainageSimulator::new (drainage.rs:263-288): CPU semantics, uniform field
 * film_thickness_nm*1e-9, marginal regeneration on, TFE ratio 0.85, first
 * front at t = 0.5 s, compensated f32x2 storage. resolution >= 3. */
int sbs_drainage_create(const sbs_config *cfg, sbs_drainage **out);

/* Thickness storage of a CPU-semantics handle. */
#define SBS_DRAIN_F32 0   /* one f32 word per cell: 8 B per cell-step */
#define SBS_DRAIN_F32X2 1 /* compensated hi + lo f32 words: ~48 significant bits, 16 B per cell-step */

/* DrainageSimulator::new with an explicit thickness storage. The reference
 * integrates in f64; with SBS_DRAIN_F32 the gravity increment of a 500 nm
 * film (~1e-3 of an f32 ulp per 1 ms step) is lost, with SBS_DRAIN_F32X2 (the
 * default of sbs_drainage_create) it is kept. */
int sbs_drainage_create_ex(const sbs_config *cfg, int precision, sbs_drainage **out);
int sbs_drainage_precision(const sbs_drainage *h, int *out);

/* GPUDrainageSimulator::new (gpu_drainage.rs:118-331): WGSL semantics,
 * grid_width (phi) x grid_height (theta), thickness initial_thickness (m),
 * concentration 0.5, DrainageParams::default otherwise, enabled = false,
 * time_scale 100, steps_per_frame 10. grid_height >= 3, grid_width >= 3. */
int sbs_gpu_drainage_create(float initial_thickness, uint32_t grid_width, uint32_t grid_height,
                            sbs_drainage **out);

int sbs_drainage_destroy(sbs_drainage *h);

/* Semantics (SBS_CPU_SEMANTICS / SBS_WGSL_SEMANTICS), grid size (theta rows, phi columns). */
int sbs_drainage_semantics(const sbs_drainage *h, int *out);
/* GPUDrainageSimulator::grid_size (gpu_drainage.rs:482-484) returns (width, height). */
int sbs_drainage_grid_size(const sbs_drainage *h, uint32_t *num_theta, uint32_t *num_phi);

/* DrainageSimulator::step (drainage.rs:298-392): one forward-Euler step of
 * size dt, pole rings averaged, TFE fronts applied, time advanced by dt.
 * CPU semantics only. */
int sbs_drainage_step(sbs_drainage *h, double dt);

/* n consecutive calls of sbs_drainage_step(h, dt), replayed as CUDA graphs in
 * chunks. CPU semantics only. */
int sbs_drainage_step_n(sbs_drainage *h, double dt, uint32_t n);

/* GPUDrainageSimulator::step (gpu_drainage.rs:338-370): if enabled, runs
 * steps_per_frame passes of drainage_step with params.dt and advances the
 * clock by frame_dt*time_scale/steps_per_frame per pass. WGSL semantics only. */
int sbs_gpu_drainage_step(sbs_drainage *h, float frame_dt);

/* Runs `passes` WGSL-semantics passes (each uses params.dt and advances the
 * clock by params.dt), independent of `enabled`. WGSL semantics only. */
int sbs_gpu_drainage_run(sbs_drainage *h, uint32_t passes);

/* The film-volume conservation run: advances n steps (CPU semantics: of size
 * dt; WGSL semantics: passes with params.dt, dt ignored) and computes the FP64
 * film volume V = sum h R^2 sin(theta) dtheta dphi of the field after every
 * `check_every`-th step, fused into that step's kernel. volumes_out (host)
 * receives n / check_every values. check_every = 0 disables the check. */
int sbs_drainage_run_checked(sbs_drainage *h, double dt, uint32_t n, uint32_t check_every,
                             double *volumes_out);

/* Field I/O. Fields are row-major [theta][phi], num_theta*num_phi f32 values
 * in metres (thickness) or 0..1 (concentration). mem = SBS_MEM_HOST or
 * SBS_MEM_DEVICE. In f32x2 storage the f32 setter clears the low words and
 * the f32 getter returns the high words (the value rounded to f32); the f64
 * calls carry the full value. Replaces ThicknessField::data/data_mut (drainage.rs:195-203)
 * and the buffer getters (gpu_drainage.rs:458-480). */
int sbs_drainage_set_thickness(sbs_drainage *h, const float *src, size_t n, int mem);
int sbs_drainage_get_thickness_field(sbs_drainage *h, float *dst, size_t n, int mem);
int sbs_drainage_set_concentration(sbs_drainage *h, const float *src, size_t n, int mem);
int sbs_drainage_get_concentration_field(sbs_drainage *h, float *dst, size_t n, int mem);
/* f64 host convenience for the reference's f64 ThicknessField. */
int sbs_drainage_set_thickness_f64(sbs_drainage *h, const double *src, size_t n);
int sbs_drainage_get_thickness_field_f64(sbs_drainage *h, double *dst, size_t n);

/* Device view of the current fields: pitch in elements (row stride). The
 * pointers stay valid until the next step/run/set call on the handle.
 * which = 0: the most recent output; which = 1: the buffer the reference's
 * GPUDrainageSimulator::current_buffer() (gpu_drainage.rs:473-479) hands out,
 * which after a step is the previous pass's input (one pass stale). */
int sbs_drainage_thickness_device(sbs_drainage *h, int which, const float **ptr, size_t *pitch);
int sbs_drainage_concentration_device(sbs_drainage *h, int which, const float **ptr, size_t *pitch);
/* The handle's CUDA stream (a cudaStream_t). */
int sbs_drainage_stream(const sbs_drainage *h, void **out);

/* DrainageSimulator::get_thickness (drainage.rs:516-552): bilinear query, theta
 * clamped to [0,pi], phi wrapped with rem_euclid. f64 arithmetic on the GPU. */
int sbs_drainage_get_thickness(sbs_drainage *h, double theta, double phi, double *out);
/* Batched get_thickness. theta/phi/out: n values in `mem`. */
int sbs_drainage_query_batch(sbs_drainage *h, const double *theta, const double *phi, double *out, size_t n,
                             int mem);

/* current_time (drainage.rs:560), has_critical_region (:565),
 * critical_thickness (:570), ThicknessField::min/max_thickness (:180-193). */
int sbs_drainage_current_time(const sbs_drainage *h, double *out);
int sbs_drainage_has_critical_region(sbs_drainage *h, int *out);
int sbs_drainage_critical_thickness(const sbs_drainage *h, double *out);
int sbs_drainage_min_max(sbs_drainage *h, double *min_out, double *max_out);
/* FP64 film volume of the current field. */
int sbs_drainage_film_volume(sbs_drainage *h, double *out);

/* reset (drainage.rs:575-583); for WGSL semantics GPUDrainageSimulator::reset
 * (gpu_drainage.rs:418-433): both buffers, concentration back to 0.5. */
int sbs_drainage_reset(sbs_drainage *h, double initial_thickness);

/* Marginal regeneration control (drainage.rs:588-613). CPU semantics. */
int sbs_drainage_set_marginal_regeneration(sbs_drainage *h, int enabled);
int sbs_drainage_marginal_regeneration_enabled(const sbs_drainage *h, int *out);
int sbs_drainage_set_tfe_thickness_ratio(sbs_drainage *h, double ratio); /* clamped to [0.5, 0.95] */
int sbs_drainage_tfe_thickness_ratio(const sbs_drainage *h, double *out);
int sbs_drainage_active_tfe_count(const sbs_drainage *h, uint32_t *out);

/* GPUDrainageSimulator setters (gpu_drainage.rs:377-456). WGSL semantics. */
int sbs_gpu_drainage_update_params(sbs_drainage *h, const sbs_drainage_params *p);
int sbs_gpu_drainage_params(const sbs_drainage *h, sbs_drainage_params *out);
int sbs_gpu_drainage_set_dt(sbs_drainage *h, float dt);
int sbs_gpu_drainage_set_physics(sbs_drainage *h, float viscosity, float density, float gravity, float diffusion);
int sbs_gpu_drainage_set_bubble_radius(sbs_drainage *h, float radius);
int sbs_gpu_drainage_set_marangoni_enabled(sbs_drainage *h, int enabled);
int sbs_gpu_drainage_set_marangoni_params(sbs_drainage *h, float gamma_air, float gamma_reduction,
                                          float surfactant_diffusion, float marangoni_coeff);
/* Steps advanced per kernel launch (no reference counterpart). 2..4 use the
 * temporally blocked kernel (one read and one write of the fields per K steps;
 * grid_width must be a multiple of 4), 0 or 1 launch one step at a time. The
 * results are bit-identical either way. Default 4 where supported. */
int sbs_gpu_drainage_set_time_blocking(sbs_drainage *h, int steps_per_launch);
int sbs_gpu_drainage_time_blocking(const sbs_drainage *h, int *out);
/* The same for a handle of either semantics (no reference counterpart). For the
 * DrainageSimulator semantics 2..4 steps per launch advance the stencil, the
 * pole-ring means and the marginal-regeneration fronts K steps at a time (row
 * strips of blocks spanning the ring, all resident at once; the two polar
 * strips meet at a bounded barrier per ring mean, see sbs_set_wait_limit); it
 * needs an even resolution and at least 2 (K + 1) theta rows. Results are
 * bit-identical to single steps. Default where supported: 3 for the
 * compensated f32x2 storage, 4 for plain f32 (WGSL semantics: 4). */
int sbs_drainage_set_time_blocking(sbs_drainage *h, int steps_per_launch);
int sbs_drainage_time_blocking(const sbs_drainage *h, int *out);

/* Public fields of GPUDrainageSimulator (gpu_drainage.rs:100-107). */
int sbs_gpu_drainage_set_enabled(sbs_drainage *h, int enabled);
int sbs_gpu_drainage_set_time_scale(sbs_drainage *h, float time_scale);
int sbs_gpu_drainage_set_steps_per_frame(sbs_drainage *h, uint32_t steps);

/* ------------------------------------------------------------------ */
/* Film volume of a bare device field                                  */
/* ------------------------------------------------------------------ */
/* V = sum_{i,j} h[i*pitch+j] R^2 sin(i*pi/(nt-1)) (pi/(nt-1)) (2pi/np), FP64
 * accumulation, deterministic order. h: device pointer. Synchronous. The
 * per-block partial sums live in memory this call allocates. No reference
 * counterpart (the reference has no conservation check). */
int sbs_film_volume_device(const float *h, uint32_t num_theta, uint32_t num_phi, size_t pitch, double radius,
                           double *out, void *stream);

/* The same film volume as sbs_film_volume_device, computed without allocating
 * any memory. It has no counterpart in the reference. It is meant for callers
 * that must not allocate GPU memory while they run: for example an engine that
 * has given the GPU's memory to its own pool and budgets it per frame, or a
 * real-time loop that cannot afford the stall an allocation may cause. Instead
 * of asking CUDA for scratch space, the call works in one fixed array of
 * 155,680 bytes that libsbs places in device memory when it is loaded; every GPU
 * that loads the library keeps that array until the process exits.
 * Rules:
 *  - num_theta <= 16384 (the rows whose weights fit in the array); larger
 *    grids are rejected with SBS_E_INVALID.
 *  - Each call looks up the array's device address in the current device's
 *    context (so a cudaDeviceReset, after which the array lives at a new
 *    address, is followed); the first call on a device also loads the
 *    library's device code there: make that first call before any stream
 *    capture on that device.
 *  - Every call uses the same array, which keeps the previous call's contents
 *    (the call clears its own counter). Calls whose work overlaps on the GPU,
 *    from different streams or threads, race and can return wrong sums:
 *    serialise them.
 *  - Synchronous: returns after the result has been copied to *out. */
int sbs_film_volume_device_noalloc(const float *h, uint32_t num_theta, uint32_t num_phi, size_t pitch,
                                   double radius, double *out, void *stream);

/* ------------------------------------------------------------------ */
/* Interference (interference.rs:127-512)                              */
/* ------------------------------------------------------------------ */
/* calculate_interference_color (gamma=1) / _linear (gamma=0) (interference.rs:380-426)
 * for n points: rgb[3*k+c] for thickness t_nm[k] and cos_i[k]. wl: the three
 * channel wavelengths in nm (650/532/450 by default; with_custom_wavelengths
 * :165-176). prec: SBS_PREC_F64 / SBS_PREC_F32. rgb is f64 when prec = F64
 * and f32 when prec = F32; t_nm/cos_i are f64 for F64 and f32 for F32. */
int sbs_interference_color_batch(double n_film, const double wl[3], const void *t_nm, const void *cos_i, size_t n,
                                 int gamma, int prec, void *rgb, int mem, void *stream);

/* Per-wavelength terms of calculate_reflected_intensity for n points (f64):
 * out[8*k + 0..7] = cos_t (:197), opd (:226), phase (:248), Rs, Rp, R (:266),
 * intensity (:312), and 0 (pad). */
int sbs_interference_terms_batch(double n_film, double wl_nm, const double *t_nm, const double *cos_i, size_t n,
                                 double *out, int mem, void *stream);

/* calculate_optical_path_difference (interference.rs:226-238) for n triples:
 * opd[k] = 2 n t_nm[k] cos_t[k] + wl[k]/2 (f64). */
int sbs_optical_path_batch(double n_film, const double *t_nm, const double *cos_t, const double *wl, size_t n,
                           double *opd, int mem, void *stream);
/* calculate_phase_difference (interference.rs:248-254): phase[k] = 2 pi opd[k] / wl[k] (f64). */
int sbs_phase_difference_batch(const double *opd_nm, const double *wl, size_t n, double *phase, int mem,
                               void *stream);

/* generate_color_lookup_table (interference.rs:461-477): count gamma-corrected
 * colours over [tmin, tmax] at cos_i. rgb: count*3 f64. */
int sbs_lut1d_build(double n_film, const double wl[3], double tmin, double tmax, uint32_t count, double cos_i,
                    double *rgb, int mem, void *stream);

/* generate_2d_color_lookup_table (interference.rs:491-512): [T][A][3] f64,
 * cos_j = j/(A-1). T, A >= 1. */
int sbs_lut2d_build(double n_film, const double wl[3], double tmin, double tmax, uint32_t T, uint32_t A,
                    double *rgb, int mem, void *stream);

/* generate_interference_lut (interference_lut.rs:18-41): RGBA8 [64 angle][256
 * thickness][4], thickness 0..2000 nm, f32 arithmetic, truncating quantiser. */
#define SBS_LUT_THICKNESS_SAMPLES 256
#define SBS_LUT_ANGLE_SAMPLES 64
#define SBS_LUT_MAX_THICKNESS_NM 2000.0f
int sbs_interference_lut_rgba8(float n_film, float intensity, uint8_t *out, int mem, void *stream);

/* Schlick reflectance with transmitted Airy (wall.wgsl:176-207) at three
 * wavelengths: out[3k+c] for t_nm[k], cos_i[k]; f32. */
int sbs_schlick_rgb_batch(float n_film, const float wl[3], const float *t_nm, const float *cos_i, size_t n,
                          float *out, int mem, void *stream);

/* LUT lookups. RGBA8 lookup: thin_film_interference of bubble.wgsl:425-439
 * (u = t/max_nm, v = cos, bilinear, * intensity, clamp) with addressing
 * SBS_LOOKUP_TEXEL (the sampler of pipeline.rs:350-359) or SBS_LOOKUP_GRID.
 * lut: W x H RGBA8 texels [H][W][4]. */
int sbs_lut_rgba8_lookup_batch(const uint8_t *lut, uint32_t W, uint32_t H, float max_nm, float intensity,
                               int addressing, const float *t_nm, const float *cos_i, size_t n, float *rgb,
                               int mem, void *stream);
/* Grid-aligned bilinear read of a [T][A][3] f64 LUT over [tmin,tmax] x cos[0,1]. */
int sbs_lut2d_lookup_batch(const double *lut, uint32_t T, uint32_t A, double tmin, double tmax, const double *t_nm,
                           const double *cos_i, size_t n, double *rgb, int mem, void *stream);

/* Vertex colouring: each unit vertex (x,y,z) gets theta = acos(y), phi =
 * atan2(z,x) mod 2pi (geometry.rs:40-60, 184-186), t = get_thickness(theta,
 * phi) in nm from the handle's current field, cos = |z| (view along +z), and
 * rgb from a grid-aligned read of a [T][A][3] f64 LUT. One fused kernel.
 * xyz: 3*nv f64, rgb: 3*nv f64, lut: T*A*3 f64, all in `mem`. */
int sbs_drainage_vertex_colors(sbs_drainage *h, const double *xyz, size_t nv, const double *lut, uint32_t T,
                               uint32_t A, double tmin, double tmax, double *rgb, int mem);

/* ------------------------------------------------------------------ */
/* Batched foam drainage                                               */
/* ------------------------------------------------------------------ */
/* Many bubbles, each with its own GPUDrainageSimulator-semantics grid
 * (resolution x 2 resolution cells, own radius), advanced together. No
 * reference counterpart: the reference's foam bubbles carry one scalar film
 * thickness each (foam.rs:44). The physics of each bubble is drainage.wgsl's,
 * with the shared DrainageParams (bubble_radius overridden per bubble; grid
 * fields ignored); a bubble advanced here matches a single GPUDrainageSimulator
 * bit for bit. Fields start at 500 nm and surfactant 0.5. */
typedef struct sbs_foam sbs_foam;
int sbs_foam_create(uint32_t nbubbles, const uint32_t *resolution, const float *radius_m,
                    const sbs_drainage_params *params, sbs_foam **out);
int sbs_foam_destroy(sbs_foam *f);
int sbs_foam_total_cells(const sbs_foam *f, uint64_t *out);
/* Per-bubble fields, [resolution][2 resolution] f32, mem = SBS_MEM_HOST or SBS_MEM_DEVICE. */
int sbs_foam_set_thickness(sbs_foam *f, uint32_t bubble, const float *src, size_t n, int mem);
int sbs_foam_get_thickness(sbs_foam *f, uint32_t bubble, float *dst, size_t n, int mem);
int sbs_foam_set_concentration(sbs_foam *f, uint32_t bubble, const float *src, size_t n, int mem);
int sbs_foam_get_concentration(sbs_foam *f, uint32_t bubble, float *dst, size_t n, int mem);
/* Advances every bubble `steps` passes: one persistent kernel (cooperative,
 * grid barriers between phases of steps_per_phase steps; a second launch for a
 * remainder), replayed from a CUDA graph. SBS_E_TIMEOUT if a barrier wait ran out. */
int sbs_foam_run(sbs_foam *f, uint32_t steps);
/* Tile shape: steps per phase (1, 2 or 4) and theta rows per work item (4..256). */
int sbs_foam_set_tiles(sbs_foam *f, uint32_t steps_per_phase, uint32_t strip_rows);
/* Times every candidate tile shape for trial_steps steps on the bubbles (fields
 * are saved and restored), keeps the fastest and reports it. */
int sbs_foam_autotune(sbs_foam *f, uint32_t trial_steps, uint32_t *steps_per_phase, uint32_t *strip_rows);
int sbs_foam_stream(const sbs_foam *f, void **out);

/* ------------------------------------------------------------------ */
/* Spectral interference contracted against colour-matching functions */
/* ------------------------------------------------------------------ */
#define SBS_SPECTRAL_TC_BF16 0 /* BF16 spectra x BF16 CMF on the tensor cores (tcgen05), FP32 accumulation */
#define SBS_SPECTRAL_FP32 1    /* FP32 spectra and FP32 FMA contraction (precision reference) */

/* For n points (thickness t_nm, cos_i, film index n_film; f32), the Airy
 * reflectance F s^2/(1 + F s^2) with s = sin(pi opd/lambda + pi/2), opd =
 * 2 n t cos_t, full unpolarised Fresnel R and F = 4R/(1-R)^2 (the formulation
 * of generate_interference_lut, interference_lut.rs:45-133, with arbitrary
 * wavelengths) at nl <= 128 wavelengths wl_nm, contracted with the nl x 3
 * matrix cmf: rgb[3k+c] = sum_l R_l(k) cmf[3l+c]. The generalisation of the
 * reference's 7-sample CIE sum to a dense spectral contraction. Synchronous
 * in both memory modes (it reads back a device status flag). */
int sbs_spectral_rgb(const float *t_nm, const float *cos_i, const float *n_film, size_t n, const float *wl_nm,
                     uint32_t nl, const float *cmf, int mode, float *rgb, int mem, void *stream);

/* ------------------------------------------------------------------ */
/* Headless film shading: the bubble fragment shader as a CUDA kernel  */
/* ------------------------------------------------------------------ */
/* The renderer's per-bubble uniform, field for field (pipeline.rs:23-67,
 * 128 bytes; the same #[repr(C)] layout the renderer uploads). */
typedef struct sbs_bubble_uniform {
    float refractive_index, base_thickness_nm, time, interference_intensity;
    float base_alpha, edge_alpha, background_r, background_g, background_b;
    float film_time, swirl_intensity, drainage_speed, pattern_scale;
    float position_x, position_y, position_z;
    uint32_t edge_smoothing_mode; /* 0 linear, 1 smoothstep, 2 power 1.5 */
    uint32_t branched_flow_enabled;
    float branched_flow_intensity, branched_flow_scale, branched_flow_sharpness;
    float light_dir_x, light_dir_y, light_dir_z;
    uint32_t patch_enabled;
    float patch_center_u, patch_center_v, patch_half_size;
    uint32_t padding[4];
} sbs_bubble_uniform;

#define SBS_LUT_ANGLES 64       /* generate_interference_lut rows (cos theta 0..1) */
#define SBS_LUT_THICKNESSES 256 /* columns (0..2000 nm) */
#define SBS_BRANCHED_W 512      /* branched-flow texture (bubble.wgsl:59-60), u32 value * 256 */
#define SBS_BRANCHED_H 256

/* BubbleUniform::default() (pipeline.rs:69-111). */
int sbs_bubble_uniform_default(sbs_bubble_uniform *out);

/* Colour and alpha of n fragments (fs_main, bubble.wgsl:486-545): unit-sphere
 * normals and world positions [n][3] in, straight-alpha rgba [n][4] out (the
 * fragment output before blending). The thickness is the procedural film of
 * get_film_thickness (:200-229: drainage term, 4-octave simplex FBM, swirl
 * noise, gravity ripple), the colour the LUT of generate_interference_lut
 * ([64 angle][256 thickness][4] RGBA8) sampled bilinearly at texel centres
 * with clamp-to-edge (pipeline.rs:350-359), black film below 30 nm. branched
 * is the 512 x 256 branched-flow texture or null (then the term is off, as
 * when branched_flow_enabled = 0). mem applies to every array. */
int sbs_shade_fragments(const sbs_bubble_uniform *u, const float camera_pos[3], const uint8_t *lut,
                        const uint32_t *branched, size_t n, const float *normal, const float *world_pos, float *rgba,
                        int mem, void *stream);
/* One headless frame (the reference's headless renderer, render/headless.rs):
 * every pixel of a width x height target casts a ray through view_proj
 * (column-major 4 x 4, wgpu clip space, depth 0..1) from camera_pos; where it
 * meets the sphere of `radius` around the uniform's position the front
 * surface is shaded as in sbs_shade_fragments and alpha-blended over the
 * background (BlendState::ALPHA_BLENDING over a clear of the background colour
 * with alpha 1; the source clamped to 0..1 as for a unorm target). Outputs,
 * either may be null: rgba8 [height][width][4] sRGB-encoded as an
 * Rgba8UnormSrgb target stores it, linear [height][width][4] f32. */
int sbs_shade_frame(const sbs_bubble_uniform *u, const float view_proj[16], const float camera_pos[3], float radius,
                    const uint8_t *lut, const uint32_t *branched, uint32_t width, uint32_t height, uint8_t *rgba8,
                    float *linear, int mem, void *stream);

/* ------------------------------------------------------------------ */
/* Caustic intensity map over the drained thickness                    */
/* ------------------------------------------------------------------ */
/* CausticParams (caustics.rs:17-52, 64 bytes, the same #[repr(C)] layout). */
typedef struct sbs_caustic_params {
    uint32_t grid_width, grid_height;
    float refractive_index, film_thickness_scale;
    float light_dir_x, light_dir_y, light_dir_z, light_intensity;
    float focal_length, caustic_intensity, caustic_sharpness, branch_threshold;
    float ground_y, bubble_radius, time;
    uint32_t padding;
} sbs_caustic_params;

/* CausticParams::default() (caustics.rs:54-76). */
int sbs_caustic_params_default(sbs_caustic_params *out);
/* The caustic compute pass (caustics_compute.wgsl:1-126): caustic_map
 * [grid_height][grid_width] from the thickness field [grid_height][pitch]
 * (pitch >= grid_width elements; phi wrapped, theta clamped). To map a drainage
 * handle's field without a copy, pass sbs_drainage_thickness_device's pointer
 * and pitch with SBS_MEM_DEVICE and the handle's stream
 * (sbs_drainage_stream); which = 1 there is the buffer the reference binds
 * (gpu_drainage.rs:478). */
int sbs_caustics(const sbs_caustic_params *p, const float *thickness, size_t pitch, float *caustic_map, int mem,
                 void *stream);
/* The caustic pass over a WGSL-semantics handle's field (which as in
 * sbs_drainage_thickness_device), on the handle's stream, no copy of the
 * field; p's grid must equal the handle's. caustic_map per mem (host: the call
 * returns when the map is there; device: ordered on the handle's stream). */
int sbs_gpu_drainage_caustics(sbs_drainage *h, const sbs_caustic_params *p, int which, float *caustic_map, int mem);
/* sbs_gpu_drainage_run(h, passes) followed by sbs_gpu_drainage_caustics(h, p, 1,
 * caustic_map, mem) - the map of the field one pass behind the newest, the
 * buffer the renderer binds - with the same results, but the map is written by
 * the run's final blocked launch from the field it holds on chip, so the field
 * is not read again (runs of fewer than 4 passes, or with time blocking off,
 * use the separate pass). The map's device destination and p are part of the
 * captured graph: a caller that reuses them runs without recapture. */
int sbs_gpu_drainage_run_caustics(sbs_drainage *h, uint32_t passes, const sbs_caustic_params *p, float *caustic_map,
                                  int mem);
/* sbs_gpu_drainage_step(h, frame_dt) (steps_per_frame passes, none when
 * disabled; the frame-dt clock) followed by the caustic map as above. */
int sbs_gpu_drainage_step_caustics(sbs_drainage *h, float frame_dt, const sbs_caustic_params *p, float *caustic_map,
                                   int mem);

/* ------------------------------------------------------------------ */
/* Branched flow of light through the film (ray tracing)               */
/* ------------------------------------------------------------------ */
/* BranchedFlowParams (branched_flow.rs:43-94, 112 bytes, same layout). */
typedef struct sbs_branched_params {
    float entry_point[3], beam_dir[3];
    uint32_t num_rays, ray_steps;
    float step_size, bend_strength, spread_angle, intensity_falloff;
    uint32_t tex_width, tex_height;
    float time, thickness_scale, base_thickness_nm, swirl_intensity, drainage_speed, pattern_scale;
    uint32_t num_scatterers;
    float scatterer_strength, scatterer_radius, particle_weight;
    uint32_t patch_enabled;
    float patch_center_u, patch_center_v, patch_half_size;
} sbs_branched_params;

/* ScattererGPU (branched_flow.rs:19-30). */
typedef struct sbs_scatterer {
    float pos_u, pos_v, strength, inv_sigma_sq;
} sbs_scatterer;

/* BranchedFlowParams::default() (branched_flow.rs:96-134). */
int sbs_branched_params_default(sbs_branched_params *out);
/* generate_scatterers (branched_flow.rs:164-226) on the host: num scatterers
 * at Halton positions with time jitter, in the patch of p when
 * p->patch_enabled; out holds num entries (num <= 2048). */
int sbs_branched_scatterers(const sbs_branched_params *p, uint32_t num, float time, sbs_scatterer *out);
/* One step of BranchedFlowSimulator (branched_flow.rs:575-601): the fade pass
 * (texture *= 0.85, truncated) when fade != 0, then the kick-drift trace of
 * p->num_rays rays (branched_flow_compute.wgsl:365-468) depositing into the
 * u32 texture [tex_height][tex_width] (value * 256, atomic adds). thickness is
 * the drainage field [height][pitch] (the shader's 128 x 64 grid generalised
 * to width x height); scatterers holds min(p->num_scatterers, 2048) entries.
 * acos, atan2 and exp are evaluated by the library's own published
 * approximations (Abramowitz & Stegun 4.4.46 and 4.4.49; Cody-Waite
 * reduction + Taylor series), so the texture is reproducible bit for bit. mem
 * applies to thickness, scatterers and texture. */
int sbs_branched_flow(const sbs_branched_params *p, const float *thickness, uint32_t width, uint32_t height,
                      size_t pitch, const sbs_scatterer *scatterers, uint32_t *texture, int fade, int mem,
                      void *stream);

/* ------------------------------------------------------------------ */
/* Foam cluster dynamics (FoamSimulator)                               */
/* ------------------------------------------------------------------ */
/* FoamSimulator's physics fields (foam_dynamics.rs:11-34), 48 bytes. */
typedef struct sbs_foam_physics {
    float surface_tension, viscosity, density;
    float gravity[3];
    float van_der_waals_strength, repulsion_stiffness, damping;
    uint32_t coalescence_enabled;
    float coalescence_threshold;
    uint32_t padding;
} sbs_foam_physics;

/* BubbleConnection (foam.rs:90-105), 40 bytes; bubble_a < bubble_b are bubble ids. */
typedef struct sbs_bubble_connection {
    uint32_t bubble_a, bubble_b;
    float contact_point[3], contact_normal[3];
    float wall_curvature_radius, wall_thickness_nm;
} sbs_bubble_connection;

typedef struct sbs_foam_sim sbs_foam_sim;

/* FoamSimulator::new's defaults (foam_dynamics.rs:38-53). */
int sbs_foam_physics_default(sbs_foam_physics *out);
/* A cluster of n bubbles in the order of BubbleCluster::bubbles() (ids 0..n-1, at rest):
 * position [n][3] and radius [n] in metres, thickness_nm [n] (null: 500 nm, Bubble::new). The
 * state lives on the GPU. */
int sbs_foam_sim_create(uint32_t n, const float *position, const float *radius, const float *thickness_nm,
                        const sbs_foam_physics *p, sbs_foam_sim **out);
int sbs_foam_sim_destroy(sbs_foam_sim *s);
int sbs_foam_sim_set_physics(sbs_foam_sim *s, const sbs_foam_physics *p);
/* `steps` FoamSimulator::step(dt) calls (foam_dynamics.rs:172-211): forces over all pairs in the
 * reference's accumulation order, semi-implicit Euler with damping and the 0.1 m/s speed clamp,
 * update_connections, and with coalescence_enabled the merge of the first connection whose
 * Weber number exceeds the threshold. Pairs farther apart than 3 (r_a + r_b) contribute exact
 * zeros in the reference; they are skipped through a neighbour list sorted by bubble order, so
 * the sums are the reference's f32 sums. Returns when the steps are done. */
int sbs_foam_sim_step(sbs_foam_sim *s, float dt, uint32_t steps);
/* bubble_count() and connection_count() (either pointer may be null). */
int sbs_foam_sim_counts(sbs_foam_sim *s, uint32_t *bubbles, uint32_t *connections);
/* The bubbles in cluster order: position and velocity [n][3], radius, thickness_nm [n], ids [n];
 * any pointer may be null; n = the current bubble count. */
int sbs_foam_sim_get_state(sbs_foam_sim *s, float *position, float *velocity, float *radius, float *thickness_nm,
                           uint32_t *ids, int mem);
/* Overwrites the listed fields of the current bubbles (null = keep), as the reference's public
 * Bubble fields allow; the count stays. */
int sbs_foam_sim_set_state(sbs_foam_sim *s, const float *position, const float *velocity, const float *radius,
                           const float *thickness_nm, int mem);
/* compute_forces (foam_dynamics.rs:62-94) on the current state: forces [n][3]. */
int sbs_foam_sim_forces(sbs_foam_sim *s, float *forces, int mem);
/* The cluster's connections() after the last step (foam.rs:304-307), in its order; writes
 * min(count, capacity) records to out (host memory) and the full count to *count. */
int sbs_foam_sim_connections(sbs_foam_sim *s, sbs_bubble_connection *out, uint32_t capacity, uint32_t *count);
/* Couples the cluster to a batched drainage foam with the same bubble count: bubble i's
 * thickness_nm becomes the area-weighted (sin theta) mean of batch bubble i's current thickness
 * field, in nm. */
int sbs_foam_sim_couple_thickness(sbs_foam_sim *s, sbs_foam *batch);


/* ------------------------------------------------------------------ */
/* Drainage surrogate: conv neural operator over SBS_NN_STEPS passes   */
/* ------------------------------------------------------------------ */
/* The network, its features, parameter layout and activation are defined in
 * sbs_nn.h. The surrogate approximates SBS_NN_STEPS WGSL-semantics passes
 * (drainage.wgsl:72-202 with marangoni_enabled = 0, where the surfactant does
 * not feed back into the thickness) and is trained here, on this GPU, on
 * trajectories that the plain solver generates. */
typedef struct sbs_surrogate sbs_surrogate;

#define SBS_NN_LAYERED 0 /* one kernel per layer (tcgen05 convolutions), activations through HBM */
#define SBS_NN_FUSED 1   /* all four layers in one persistent tcgen05 kernel, activations on chip */

/* New surrogate with He-initialised weights (normal, splitmix64 seed). */
int sbs_surrogate_create(uint64_t seed, sbs_surrogate **out);
int sbs_surrogate_destroy(sbs_surrogate *s);
/* FP32 parameter vector, n = SBS_NN_PARAMS, host memory. */
int sbs_surrogate_set_params(sbs_surrogate *s, const float *params, size_t n);
int sbs_surrogate_get_params(sbs_surrogate *s, float *params, size_t n);
/* Activation of the network: SBS_NN_ACT_GELU (default) or SBS_NN_ACT_HSWISH
 * (sbs_nn.h). Weights trained with one do not fit the other; set it before
 * training. */
int sbs_surrogate_set_activation(sbs_surrogate *s, int activation);
int sbs_surrogate_get_activation(const sbs_surrogate *s, int *out);
/* Features of nf <= 16 fields: h, c [nf][nt][np] (nt = p[k].grid_height, np =
 * p[k].grid_width, the same for every field), x out [nf][nt][np][SBS_NN_NF]
 * (BF16 values as f32). mem applies to h, c and x. */
int sbs_surrogate_features(sbs_surrogate *s, uint32_t nf, const float *h, const float *c,
                           const sbs_drainage_params *p, float *x, int mem);
/* Network output y [nf][nt][np] (mode SBS_NN_LAYERED or SBS_NN_FUSED). */
int sbs_surrogate_forward(sbs_surrogate *s, uint32_t nf, const float *h, const float *c,
                          const sbs_drainage_params *p, float *y, int mode, int mem);
/* Masked mean-square loss of the network output against target [nf][nt][np]
 * (rows with sin(theta) >= SBS_NN_MASK_SIN) and its gradient (SBS_NN_PARAMS
 * floats). Host memory. */
int sbs_surrogate_loss_grad(sbs_surrogate *s, uint32_t nf, const float *h, const float *c,
                            const sbs_drainage_params *p, const float *target, double *loss, float *grad);
/* Training data: runs the plain WGSL-semantics solver (the sbs_gpu_drainage
 * kernels) from (h0, c0, host) with parameters p over pairs intervals of
 * SBS_NN_STEPS * p->dt and keeps the pairs + 1 snapshots on the device. Each
 * interval is integrated as SBS_NN_STEPS * substeps passes of p->dt / substeps;
 * substeps = 0 picks the smallest power of two that keeps every row of the
 * explicit scheme stable (1 wherever p->dt itself is stable), so that small
 * bubbles on a coarse grid - the same per-cell diffusion numbers as large
 * bubbles on a fine grid - give clean targets up to the poles. Every trajectory
 * of one surrogate has the grid of the first. */
int sbs_surrogate_add_trajectory(sbs_surrogate *s, const float *h0, const float *c0, const sbs_drainage_params *p,
                                 uint32_t pairs, uint32_t substeps);
int sbs_surrogate_num_trajectories(const sbs_surrogate *s, uint32_t *out);
int sbs_surrogate_clear_data(sbs_surrogate *s);
/* Adam (0.9, 0.999, 1e-8) with a cosine learning-rate decay from lr to lr/20
 * over iters steps; each step a batch of `batch` (<= 16) snapshot pairs drawn
 * (splitmix64 seed) from trajectories [0, n_train). losses (host, iters) gets
 * each step's loss; may be null. */
int sbs_surrogate_train(sbs_surrogate *s, uint32_t n_train, uint32_t iters, uint32_t batch, float lr, uint64_t seed,
                        float *losses);
typedef struct sbs_surrogate_eval {
    double loss;              /* masked MSE of the network output against (h' - h) / kout */
    double loss_identity;     /* the same for y = 0 (h' = h) */
    double rel_linf;          /* max over pairs of the masked relative L-inf error of the predicted h' */
    double rel_linf_identity; /* the same for h' = h */
} sbs_surrogate_eval;
/* Evaluates every pair of trajectories [first, first + count). */
int sbs_surrogate_evaluate(sbs_surrogate *s, uint32_t first, uint32_t count, int mode, sbs_surrogate_eval *out);
/* One surrogate rollout of a WGSL-semantics handle: h <- h + kout y, the
 * concentration held, the clock advanced by SBS_NN_STEPS * dt. */
int sbs_surrogate_advance(sbs_surrogate *s, sbs_drainage *h, int mode);
typedef struct sbs_surrogate_stats {
    uint32_t rollouts;         /* SBS_NN_STEPS-pass intervals advanced */
    uint32_t surrogate;        /* of which by the surrogate alone */
    uint32_t plain;            /* by the plain solver (checks and fallback) */
    uint32_t checks;
    uint32_t failed_checks;
    uint32_t pad;
    double max_check_error;    /* largest masked relative L-inf error seen in a check */
    double last_check_error;
} sbs_surrogate_stats;
/* Surrogate-accelerated run of `passes` WGSL passes (a multiple of
 * SBS_NN_STEPS) on handle h. Every check_every-th interval (0 = never) both
 * the surrogate and the plain solver advance from the same state; the plain
 * result is kept, and if the masked relative L-inf difference exceeds tol the
 * plain solver also runs the next check_every - 1 intervals. */
int sbs_surrogate_rollout(sbs_surrogate *s, sbs_drainage *h, uint32_t passes, uint32_t check_every, double tol,
                          int mode, sbs_surrogate_stats *stats);
/* Masked relative L-inf difference max|a - b| / max|b| over rows with
 * sin(theta) >= SBS_NN_MASK_SIN of two nt x np fields (device or host). */
int sbs_surrogate_masked_error(const float *a, const float *b, uint32_t nt, uint32_t np, int mem, double *out);
int sbs_surrogate_stream(const sbs_surrogate *s, void **out);

#ifdef __cplusplus
}
#endif

#endif /* SBS_H */
