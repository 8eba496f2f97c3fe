// Internal declarations shared by the libsbs translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <map>
#include <string>
#include <vector>

#include "../../include/sbs.h"
#include "fixsum.cuh"

namespace sbs {

// ---------------------------------------------------------------------------
// Error reporting: thread-local last error text, negative SBS_E_* codes.
// ---------------------------------------------------------------------------
int set_error(int code, const char *fmt, ...);
void clear_error();

#define SBS_CUDA_TRY(expr)                                                                         \
    do {                                                                                           \
        cudaError_t _e = (expr);                                                                   \
        if (_e != cudaSuccess)                                                                     \
            return ::sbs::set_error(SBS_E_CUDA, "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                                    __FILE__, __LINE__);                                           \
    } while (0)

#define SBS_CHECK_ARG(cond, ...)                                                                   \
    do {                                                                                           \
        if (!(cond)) return ::sbs::set_error(SBS_E_INVALID, __VA_ARGS__);                         \
    } while (0)

// Makes sure a CUDA device exists and the runtime is usable; fails with SBS_E_CUDA otherwise.
int require_device();

// Bounded device-side waits: every spin or mbarrier wait of a kernel gives up after `cycles` SM
// clock cycles, records the timeout in a device flag and lets the kernel exit; the host reports
// SBS_E_TIMEOUT. `stall` holds the SBS_STALL_* test switches (sbs_set_stall_injection); `epoch`
// changes with every setting, so handles that captured launches in CUDA graphs rebuild them.
constexpr long long kDefaultWaitCycles = 2000000000LL;  // ~1 s at 2 GHz
struct WaitConfig {
    long long cycles;
    int stall;
    unsigned epoch;
};
WaitConfig wait_config();

// Stream-ordered scratch for one call (release it with cudaFreeAsync on the same stream). Blocks of
// up to 64 MB come from a per-device pool that keeps freed memory for the next call (the default
// pool returns it to the system at every synchronisation, and mapping it again costs ~100 us);
// larger blocks come from the default pool.
cudaError_t scratch_alloc(void **p, size_t bytes, cudaStream_t s);

// WGSL-semantics passes (params.dt each) enqueued on the handle's stream without a final
// synchronisation (sbs_gpu_drainage_run minus the wait).
int drainage_run_async(sbs_drainage *h, uint32_t passes);

// Area-weighted (sin theta) mean of each bubble's current thickness field of a batched foam, in
// nm, into out[cap] (device memory); *nb = the batch's bubble count (out is written only when
// nb <= cap). Returns when the values are there.
int foam_mean_thickness_nm(sbs_foam *f, float *out, uint32_t cap, uint32_t *nb);

// ---------------------------------------------------------------------------
// Drainage kernels
// ---------------------------------------------------------------------------
constexpr int kMaxFronts = 8;

// Marginal-regeneration fronts active during one step, as integer cell ranges: front f covers
// rows [r0, r1] and the circular column interval starting at c0 of length clen. The thinning
// factor 1 - (1 - ratio) * 0.5 * dt (drainage.rs:453-454) is given as the double-float pair
// factor + factor_lo (factor alone in plain f32 mode).
struct TfeStep {
    int nf;
    float factor;
    float factor_lo;
    int pad;
    int4 fr[kMaxFronts];  // x = r0, y = r1, z = c0, w = clen
};

// Arguments of one drainage step launch.
struct StepArgs {
    const float *hin;
    float *hout;
    const float *cin;  // concentration (WGSL semantics)
    float *cout;
    const float *lin;  // low-order thickness words (compensated f32x2 mode)
    float *lout;
    const float4 *rows;    // per theta row: A = -rho g/(3 eta) sin, E = cot/(2 dth), F = 1/(ss^2 dphi^2), G
    const FixSum *pin;     // pole-ring partial sums (ring 1 per block, then ring N-2) of the input field
    FixSum *pout;          // pole-ring partial sums written by this step (CPU semantics)
    const TfeStep *tfe;    // fronts of this step (nullptr = none)
    const double *vol_w;   // per-row volume weights R^2 sin dth dphi (nullptr = no volume check)
    double *vol_partials;  // one per block
    unsigned *vol_counter; // arrival ticket for the last-block reduction
    double *vol_out;       // volume results, appended at *vol_index
    unsigned *vol_index;
    int nt, np, pitch;
    int rb;             // rows per block strip
    int poles_virtual;  // 1: pole rows of hin are the means of pin, not memory
    int marangoni;
    float crit, b, DR2, DsR2, Gt, M, dt;
    // blocked CPU-semantics step only: the polar strips' ring exchange
    FixSum *ring_part;      // [2][4][C W] warp partials of ring 1 / ring N-2 per step of the launch
    unsigned *ring_bar;     // [2][4] barrier words (arrivals, generation), then the status word
    unsigned *status_host;  // host-mapped status word (nonzero: a barrier wait timed out)
    long long wait_cycles;  // barrier wait limit
    unsigned extra;         // arrivals beyond the strip's blocks (1 only in the timeout test)
    int prow;               // rows of each polar strip (0: all strips even)
    // blocked WGSL step only: the caustic map of the launch's result (nullptr: none)
    float *cau_out;         // grid_width x grid_height floats, row stride np
    float cau_focal, cau_scale, cau_sharp, cau_branch;
};

struct StepGeom {
    int wx;   // warps per block along phi
    int nbx;  // column blocks
    int nby;  // row strips
    int rb;   // rows of the tallest strip
    int prow; // blocked CPU-semantics step: rows of each polar strip (0: all strips even)
};

StepGeom step_geometry(int nt, int np, int semantics, int x2);
// Temporally blocked WGSL step (K = 2..4 steps per launch), drainage_wtb.cu.
bool wtb_supported(int nt, int np);
StepGeom wtb_geometry(int nt, int np, int K);
cudaError_t launch_wtb(int K, const StepArgs &a, const StepGeom &g, cudaStream_t s);
// K for a launch that also writes the caustic map of its result (a.cau_out): its final level must
// leave one valid column beyond the kept 120 on each side of a warp's window.
constexpr int kWtbCausticK = 3;
// Temporally blocked CPU-semantics step (K = 2..4 steps per launch, pole means and fronts
// included), drainage_wtb_cpu.cu. Each row strip is nbx blocks of wx warps that span the ring;
// nby strips of at most rb rows, all resident at once (cooperative launch). nby == 0: the grid
// is not supported. The ring exchange needs 2 x 4 x wtbc_ring_parts(g) FixSum partials and
// kWtbcBarWords barrier words (zeroed before first use and after a timeout).
constexpr int kWtbcBarWords = 17;
StepGeom wtbc_geometry(int nt, int np, int K, int x2);
int wtbc_ring_parts(const StepGeom &g);
cudaError_t launch_wtbc(int K, int x2, const StepArgs &a, const StepGeom &g, cudaStream_t s);
// x2: compensated f32x2 thickness (hi + lo words); CPU semantics only.
cudaError_t launch_step(int semantics, int x2, const StepArgs &a, const StepGeom &g, cudaStream_t s);
// Writes the pole rows of `h` (and `hl`, if not null) from the ring partials of the last step.
cudaError_t launch_finalize_poles(float *h, float *hl, const FixSum *part, int nbx, int nt, int np,
                                  int pitch, cudaStream_t s);

// Field reductions: min, max and FP64 volume sum of a pitched field (valid columns only).
struct ReduceOut {
    double vmin, vmax, volume;
};
int reduce_partials_count(int nt, int np);
// hl: optional low-order words (value = h + hl).
cudaError_t launch_field_reduce(const float *h, const float *hl, int nt, int np, size_t pitch,
                                const double *w, double *partials /*3*count*/, unsigned *counter,
                                ReduceOut *out, cudaStream_t s);

cudaError_t launch_query(const float *h, const float *hl, int nt, int np, size_t pitch,
                         const double *theta, const double *phi, double *out, size_t n,
                         cudaStream_t s);
cudaError_t launch_vertex_colors(const float *h, const float *hl, int nt, int np, size_t pitch,
                                 const double *xyz, size_t nv, const double *lut, int T, int A,
                                 double tmin, double tmax, double *rgb, cudaStream_t s);
// Splits f64 values into (hi, lo) f32 words of a pitched field.
cudaError_t launch_split_f64(const double *src, float *hi, float *lo, int nt, int np, size_t pitch,
                             cudaStream_t s);
// Joins (hi, lo) words of a pitched field into dense f64 values.
cudaError_t launch_join_f64(const float *hi, const float *lo, double *dst, int nt, int np, size_t pitch,
                            cudaStream_t s);

// ---------------------------------------------------------------------------
// Host-side marginal-regeneration clock (the bookkeeping of drainage.rs:395-477; the per-cell
// thinning runs in the step kernel).
// ---------------------------------------------------------------------------
struct HostFront {
    double phi_center, extent, width, velocity;
    int c0, clen;
};

struct TfeClock {
    double next_spawn = 0.5;
    double spawn_interval = 2.0;
    double ratio = 0.85;
    bool enabled = true;
    bool error = false;  // a front's columns did not form one interval
    std::vector<HostFront> fronts;
    // Advances the bookkeeping by one step of size dt taken at time t and fills the ranges the
    // kernel applies after the stencil.
    void advance(double t, double dt, int nt, int np, TfeStep *out);
    void reset() {
        fronts.clear();
        next_spawn = 0.5;
    }
};

// f32 constants of the step kernel (derived from the parameters; see drainage.cu).
struct KernelConsts {
    float b = 0, DR2 = 0, DsR2 = 0, Gt = 0, M = 0, crit = 0;
};

cudaError_t launch_fill(float *p, size_t pitch, int nt, int np, float v, cudaStream_t s);

// Per-row coefficients and kernel constants of the WGSL semantics for an H x W grid.
void wgsl_tables(int H, int W, const sbs_drainage_params &p, std::vector<float4> *rows, std::vector<double> *w,
                 float *b, float *DR2, float *DsR2, float *Gt, float *M);

}  // namespace sbs

// ---------------------------------------------------------------------------
// The drainage handle.
// ---------------------------------------------------------------------------
struct sbs_drainage {
    int sem = SBS_CPU_SEMANTICS;
    int nt = 0, np = 0;
    size_t pitch = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    float *h[2] = {nullptr, nullptr};
    float *c[2] = {nullptr, nullptr};
    float *hl[2] = {nullptr, nullptr};  // low-order words in compensated mode
    int x2 = 0;                          // 1: compensated f32x2 thickness
    int cur = 0;   // buffer index holding the newest field
    int prev = 1;  // buffer holding the field one pass older (WGSL quirk accessor)
    sbs::FixSum *part[2] = {nullptr, nullptr};  // per-block pole-ring partials (single-step kernel)
    float4 *rows = nullptr;
    double *vol_w = nullptr;
    double *vol_partials = nullptr;
    unsigned *vol_counter = nullptr;
    double *vol_out = nullptr;
    unsigned *vol_index = nullptr;
    size_t vol_out_cap = 0;
    double *red_partials = nullptr;
    unsigned *red_counter = nullptr;
    sbs::ReduceOut *red_out = nullptr;  // device
    sbs::TfeStep *sched_dev = nullptr;
    sbs::TfeStep *sched_host[2] = {nullptr, nullptr};
    cudaEvent_t sched_ev[2] = {nullptr, nullptr};
    int sched_slot = 0;
    size_t sched_cap = 0;
    double *qbuf = nullptr;
    size_t qcap = 0;
    sbs::StepGeom geom{};
    int wtb_k = 0;  // steps per temporally blocked launch (WGSL semantics; 0 = single steps only)
    sbs::StepGeom wgeom{};
    int cpu_k = 0;  // steps per temporally blocked launch (CPU semantics; 0 = single steps only)
    sbs::StepGeom cgeom{};
    sbs::FixSum *ring_part = nullptr;  // the blocked step's ring exchange (CPU semantics)
    unsigned *ring_bar = nullptr;
    unsigned *ring_status = nullptr;   // host-mapped timeout word
    unsigned *ring_status_dev = nullptr;
    unsigned wait_epoch = 0;           // the wait settings the captured graphs were made with
    // caustic map written by the run in progress (sbs_gpu_drainage_run_caustics)
    bool cau_on = false;
    bool cau_fused = false;            // the final chunk of the last run wrote the map
    float *cau_out = nullptr;          // device destination of the map
    float cau_p[4] = {0.f, 0.f, 0.f, 0.f};  // focal length, intensity, sharpness, branch threshold
    float *cau_buf = nullptr;          // device map for calls with host memory
    sbs::StepGeom cau_geom{};          // geometry of the launch that writes the map

    // CPU semantics parameters (from sbs_config)
    sbs_config cfg{};
    double radius = 0.0, critical = 0.0;
    // WGSL semantics parameters
    sbs_drainage_params params{};
    bool enabled = false;
    float time_scale = 100.0f;
    uint32_t steps_per_frame = 10;

    double current_time = 0.0;
    sbs::TfeClock tfe;
    sbs::KernelConsts k{};

    // Graph cache: chunk graphs keyed by (start buffer, length, volume flag, tfe flag, dt bits).
    std::map<std::string, cudaGraphExec_t> graphs;
};
