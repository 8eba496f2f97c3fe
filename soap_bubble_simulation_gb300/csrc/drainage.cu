// Host side of the drainage handle: geometry, per-row coefficient tables, the marginal
// regeneration clock, buffer management, CUDA-graph replay of step chunks and the C ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "sbs_internal.h"

namespace sbs {

namespace {

const double kPi = 3.14159265358979323846;
const double kHalfPi = kPi / 2.0;
constexpr int kMaxChunk = 256;  // steps per replayed graph / schedule upload
constexpr int kGraphMin = 8;    // shorter chunks launch directly

// TfeFront::contains split into its theta and phi tests (drainage.rs:55-71).
bool theta_inside(const HostFront &f, double theta) { return !(std::fabs(theta - kHalfPi) > f.extent); }

bool phi_inside(const HostFront &f, double phi) {
    double d = std::fabs(phi - f.phi_center);
    if (d > kPi) d = 2.0 * kPi - d;
    return d < f.width / 2.0;
}

// Columns phi_j = j * dphi inside a front form one circular interval; found once at spawn with
// the reference's own f64 predicate. Returns false if the set is not one interval.
bool front_columns(HostFront &f, int np) {
    const double dph = 2.0 * kPi / (double)np;
    std::vector<char> in(np);
    int cnt = 0;
    for (int j = 0; j < np; ++j) {
        in[j] = phi_inside(f, (double)j * dph) ? 1 : 0;
        cnt += in[j];
    }
    if (cnt == 0) {
        f.c0 = 0;
        f.clen = 0;
        return true;
    }
    if (cnt == np) {
        f.c0 = 0;
        f.clen = np;
        return true;
    }
    int start = 0;
    for (int j = 0; j < np; ++j)
        if (in[j] && !in[(j - 1 + np) % np]) {
            start = j;
            break;
        }
    int len = 0;
    while (len < np && in[(start + len) % np]) ++len;
    f.c0 = start;
    f.clen = len;
    return len == cnt;
}

// Rows theta_i = i * dtheta with |theta_i - pi/2| <= extent (contiguous: the distance is V-shaped).
void front_rows(const HostFront &f, int nt, int *r0, int *r1) {
    const double dth = kPi / (double)(nt - 1);
    const long center = (long)std::ceil(kHalfPi / dth);
    long i = (long)std::ceil((kHalfPi - f.extent) / dth);
    i = std::max(0L, std::min(i, (long)nt - 1));
    while (i > 0 && theta_inside(f, (double)(i - 1) * dth)) --i;
    while (i < nt && i <= center + 1 && !theta_inside(f, (double)i * dth)) ++i;
    if (i >= nt || !theta_inside(f, (double)i * dth)) {
        *r0 = 1;
        *r1 = 0;
        return;
    }
    long j = (long)std::floor((kHalfPi + f.extent) / dth);
    j = std::max(i, std::min(j, (long)nt - 1));
    while (j + 1 < nt && theta_inside(f, (double)(j + 1) * dth)) ++j;
    while (j > i && !theta_inside(f, (double)j * dth)) --j;
    *r0 = (int)i;
    *r1 = (int)j;
}

}  // namespace

// update_marginal_regeneration bookkeeping (drainage.rs:395-411) and spawn_tfe_front (:464-477).
void TfeClock::advance(double t, double dt, int nt, int np, TfeStep *out) {
    next_spawn -= dt;
    if (next_spawn <= 0.0) {
        HostFront f{};
        f.phi_center = std::fabs(std::sin(t * 7.89 + 1.23)) * 2.0 * kPi;
        f.width = 0.3 + std::fabs(std::sin(t * 3.21)) * 0.4;
        f.velocity = 0.05 + std::fabs(std::cos(t * 5.67)) * 0.05;
        f.extent = 0.0;
        if (!front_columns(f, np)) error = true;
        fronts.push_back(f);
        if (fronts.size() > (size_t)kMaxFronts) fronts.erase(fronts.begin());
        const double random_factor = 0.5 + std::fabs(std::sin(t * 12.345));
        next_spawn = spawn_interval * random_factor;
    }
    for (auto &f : fronts) f.extent = std::min(f.extent + f.velocity * dt, kHalfPi);
    fronts.erase(std::remove_if(fronts.begin(), fronts.end(),
                                [](const HostFront &f) { return !(f.extent < kHalfPi * 0.95); }),
                 fronts.end());
    std::memset(out, 0, sizeof(*out));
    const double rr = (1.0 - ratio) * 0.5;
    const double factor = 1.0 - rr * dt;
    out->factor = (float)factor;
    out->factor_lo = (float)(factor - (double)out->factor);
    int n = 0;
    for (const auto &f : fronts) {
        int r0, r1;
        front_rows(f, nt, &r0, &r1);
        if (r1 < r0 || f.clen == 0) continue;
        out->fr[n++] = make_int4(r0, r1, f.c0, f.clen);
    }
    out->nf = n;
}

// Per-row coefficients of the WGSL semantics (f32 angle grid, sin floor 1e-4 with sign,
// drainage.wgsl:92-101) and the kernel constants, from the DrainageParams; f64 volume weights.
void wgsl_tables(int H, int W, const sbs_drainage_params &p, std::vector<float4> *rows, std::vector<double> *w,
                 float *b, float *DR2, float *DsR2, float *Gt, float *M) {
    const float PI32 = 3.14159265358979323846f;
    const float dth32 = PI32 / (float)(H - 1), dph32 = 2.0f * PI32 / (float)W;
    const double dth = (double)dth32, dph = (double)dph32, R = (double)p.bubble_radius;
    const double coef = (double)p.density * (double)p.gravity / (3.0 * (double)p.viscosity);
    rows->resize(H);
    if (w) w->resize(H);
    const double vdth = kPi / (double)(H - 1), vdph = 2.0 * kPi / (double)W;
    for (int i = 0; i < H; ++i) {
        const float th32 = (float)i * dth32;
        const double sn = std::sin((double)th32), cs = std::cos((double)th32);
        const double ss = std::fabs(sn) < 1e-4 ? (sn > 0 ? 1e-4 : (sn < 0 ? -1e-4 : 0.0)) : sn;
        (*rows)[i] = make_float4((float)(-coef * sn), (float)((cs / ss) / (2.0 * dth)),
                                 (float)((1.0 / (ss * ss)) / (dph * dph)), (float)(1.0 / (2.0 * dph * R * ss)));
        if (w) (*w)[i] = R * R * std::sin((double)i * vdth) * vdth * vdph;
    }
    *b = (float)(1.0 / (dth * dth));
    *DR2 = (float)((double)p.diffusion_coeff / (R * R));
    *DsR2 = (float)((double)p.surfactant_diffusion / (R * R));
    *Gt = (float)(1.0 / (2.0 * dth * R));
    *M = (float)((double)p.marangoni_coeff * (double)p.gamma_reduction);
}

}  // namespace sbs

using namespace sbs;

namespace {

size_t round_up(size_t x, size_t m) { return (x + m - 1) / m * m; }

void destroy_graphs(sbs_drainage *h) {
    for (auto &kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
}

// Per-row coefficients (CPU semantics: f64 angle grid, sin floor 1e-10, drainage.rs:315-324).
void rows_cpu(sbs_drainage *h, std::vector<float4> &rows, std::vector<double> &w, float *b, float *DR2) {
    const int nt = h->nt, np = h->np;
    const double dth = kPi / (double)(nt - 1), dph = 2.0 * kPi / (double)np;
    const double coef = h->cfg.density * h->cfg.gravity / (3.0 * h->cfg.viscosity);
    const double R = h->radius;
    rows.resize(nt);
    w.resize(nt);
    for (int i = 0; i < nt; ++i) {
        const double th = (double)i * dth;
        const double sn = std::sin(th), cs = std::cos(th);
        const double ss = std::fabs(sn) < 1e-10 ? std::copysign(1e-10, sn) : sn;
        rows[i] = make_float4((float)(-coef * sn), (float)((cs / ss) / (2.0 * dth)),
                              (float)((1.0 / (ss * ss)) / (dph * dph)), 0.f);
        w[i] = R * R * std::sin((double)i * dth) * dth * dph;
    }
    *b = (float)(1.0 / (dth * dth));
    *DR2 = (float)(h->cfg.surfactant_diffusion / (R * R));
}

// Per-row coefficients (WGSL semantics: f32 angle grid, sin floor 1e-4 with sign, drainage.wgsl:92-101).
struct WgslConsts {
    float b, DR2, DsR2, Gt, M;
};

void rows_wgsl(sbs_drainage *h, std::vector<float4> &rows, std::vector<double> &w, WgslConsts *k) {
    wgsl_tables(h->nt, h->np, h->params, &rows, &w, &k->b, &k->DR2, &k->DsR2, &k->Gt, &k->M);
}

using Consts = KernelConsts;

int upload_tables(sbs_drainage *h, Consts *k) {
    std::vector<float4> rows;
    std::vector<double> w;
    if (h->sem == SBS_CPU_SEMANTICS) {
        rows_cpu(h, rows, w, &k->b, &k->DR2);
        k->crit = (float)h->critical;
    } else {
        WgslConsts wc{};
        rows_wgsl(h, rows, w, &wc);
        k->b = wc.b;
        k->DR2 = wc.DR2;
        k->DsR2 = wc.DsR2;
        k->Gt = wc.Gt;
        k->M = wc.M;
        k->crit = h->params.critical_thickness;
    }
    SBS_CUDA_TRY(cudaMemcpyAsync(h->rows, rows.data(), sizeof(float4) * h->nt, cudaMemcpyHostToDevice, h->stream));
    SBS_CUDA_TRY(cudaMemcpyAsync(h->vol_w, w.data(), sizeof(double) * h->nt, cudaMemcpyHostToDevice, h->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return SBS_OK;
}

int refresh(sbs_drainage *h, Consts *k) {
    destroy_graphs(h);
    return upload_tables(h, k);
}

Consts &consts_of(sbs_drainage *h) { return h->k; }

int allocate(sbs_drainage *h) {
    const size_t bytes = h->pitch * (size_t)h->nt * sizeof(float);
    SBS_CUDA_TRY(cudaGetDevice(&h->device));
    SBS_CUDA_TRY(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    for (int i = 0; i < 2; ++i) {
        SBS_CUDA_TRY(cudaMalloc(&h->h[i], bytes));
        SBS_CUDA_TRY(cudaMemset(h->h[i], 0, bytes));
        if (h->sem == SBS_WGSL_SEMANTICS) {
            SBS_CUDA_TRY(cudaMalloc(&h->c[i], bytes));
            SBS_CUDA_TRY(cudaMemset(h->c[i], 0, bytes));
        }
        if (h->x2) {
            SBS_CUDA_TRY(cudaMalloc(&h->hl[i], bytes));
            SBS_CUDA_TRY(cudaMemset(h->hl[i], 0, bytes));
        }
    }
    h->geom = step_geometry(h->nt, h->np, h->sem, h->x2);
    if (h->sem == SBS_WGSL_SEMANTICS && wtb_supported(h->nt, h->np)) {
        h->wtb_k = 4;
        h->wgeom = wtb_geometry(h->nt, h->np, h->wtb_k);
        h->cau_geom = wtb_geometry(h->nt, h->np, kWtbCausticK);
    }
    if (h->sem == SBS_CPU_SEMANTICS) {
        // steps per launch measured fastest at 2048 x 4096: 3 for the compensated storage (19.7 us
        // per step; K = 2 20.2, K = 4 spills), 4 for plain f32 (10.7 us)
        const int k = h->x2 ? 3 : 4;
        h->cgeom = wtbc_geometry(h->nt, h->np, k, h->x2);
        if (h->cgeom.nby > 0) h->cpu_k = k;
    }
    for (int i = 0; i < 2; ++i) {
        SBS_CUDA_TRY(cudaMalloc(&h->part[i], sizeof(FixSum) * 2 * h->geom.nbx));
        SBS_CUDA_TRY(cudaMemset(h->part[i], 0, sizeof(FixSum) * 2 * h->geom.nbx));
    }
    SBS_CUDA_TRY(cudaMalloc(&h->rows, sizeof(float4) * h->nt));
    SBS_CUDA_TRY(cudaMalloc(&h->vol_w, sizeof(double) * h->nt));
    // one volume partial per block of whichever step kernel runs the check
    size_t vol_blocks = (size_t)h->geom.nbx * h->geom.nby;
    if (h->sem == SBS_WGSL_SEMANTICS && wtb_supported(h->nt, h->np))
        for (int k = 2; k <= 4; ++k) {
            const StepGeom g = wtb_geometry(h->nt, h->np, k);
            vol_blocks = std::max(vol_blocks, (size_t)g.nbx * g.nby);
        }
    if (h->sem == SBS_CPU_SEMANTICS) {
        size_t parts = 1;
        for (int k = 2; k <= 4; ++k) {
            const StepGeom g = wtbc_geometry(h->nt, h->np, k, h->x2);
            vol_blocks = std::max(vol_blocks, (size_t)g.nbx * g.nby);
            parts = std::max(parts, (size_t)wtbc_ring_parts(g));
        }
        SBS_CUDA_TRY(cudaMalloc(&h->ring_part, sizeof(FixSum) * 2 * 4 * parts));
        SBS_CUDA_TRY(cudaMalloc(&h->ring_bar, sizeof(unsigned) * kWtbcBarWords));
        SBS_CUDA_TRY(cudaMemset(h->ring_bar, 0, sizeof(unsigned) * kWtbcBarWords));
        SBS_CUDA_TRY(cudaHostAlloc(&h->ring_status, sizeof(unsigned), cudaHostAllocMapped));
        *h->ring_status = 0u;
        SBS_CUDA_TRY(cudaHostGetDevicePointer(&h->ring_status_dev, h->ring_status, 0));
        h->wait_epoch = wait_config().epoch;
    }
    SBS_CUDA_TRY(cudaMalloc(&h->vol_partials, sizeof(double) * vol_blocks));
    SBS_CUDA_TRY(cudaMalloc(&h->vol_counter, sizeof(unsigned) * 2));
    SBS_CUDA_TRY(cudaMemset(h->vol_counter, 0, sizeof(unsigned) * 2));
    h->vol_index = h->vol_counter + 1;
    h->vol_out_cap = 128;
    SBS_CUDA_TRY(cudaMalloc(&h->vol_out, sizeof(double) * h->vol_out_cap));
    SBS_CUDA_TRY(cudaMalloc(&h->red_partials, sizeof(double) * 3 * reduce_partials_count(h->nt, h->np)));
    SBS_CUDA_TRY(cudaMalloc(&h->red_counter, sizeof(unsigned)));
    SBS_CUDA_TRY(cudaMemset(h->red_counter, 0, sizeof(unsigned)));
    SBS_CUDA_TRY(cudaMalloc(&h->red_out, sizeof(ReduceOut)));
    h->sched_cap = kMaxChunk;
    SBS_CUDA_TRY(cudaMalloc(&h->sched_dev, sizeof(TfeStep) * h->sched_cap));
    for (int i = 0; i < 2; ++i) {
        SBS_CUDA_TRY(cudaMallocHost(&h->sched_host[i], sizeof(TfeStep) * h->sched_cap));
        SBS_CUDA_TRY(cudaEventCreateWithFlags(&h->sched_ev[i], cudaEventDisableTiming));
    }
    return SBS_OK;
}

void release(sbs_drainage *h) {
    if (h->stream) cudaStreamSynchronize(h->stream);
    destroy_graphs(h);
    for (int i = 0; i < 2; ++i) {
        cudaFree(h->h[i]);
        cudaFree(h->c[i]);
        cudaFree(h->hl[i]);
        cudaFree(h->part[i]);
        if (h->sched_host[i]) cudaFreeHost(h->sched_host[i]);
        if (h->sched_ev[i]) cudaEventDestroy(h->sched_ev[i]);
    }
    cudaFree(h->rows);
    cudaFree(h->vol_w);
    cudaFree(h->vol_partials);
    cudaFree(h->vol_counter);
    cudaFree(h->vol_out);
    cudaFree(h->red_partials);
    cudaFree(h->red_counter);
    cudaFree(h->red_out);
    cudaFree(h->sched_dev);
    cudaFree(h->qbuf);
    cudaFree(h->ring_part);
    cudaFree(h->ring_bar);
    cudaFree(h->cau_buf);
    if (h->ring_status) cudaFreeHost(h->ring_status);
    if (h->stream) cudaStreamDestroy(h->stream);
}

// Whether a chunk of `count` WGSL passes ends with the launch that also writes the caustic map:
// the final chunk of a run that asked for the map, blocked, with three passes before the final
// single pass (the map is of the field one pass behind the newest, the buffer the renderer binds).
bool cau_plan(const sbs_drainage *h, int count, bool last_single) {
    return h->cau_on && h->sem == SBS_WGSL_SEMANTICS && h->wtb_k > 1 && last_single && h->cau_geom.nby > 0 &&
           count - 1 >= kWtbCausticK;
}

// Enqueues `count` steps starting from buffer `start`; returns the buffer holding the result.
// CPU semantics: step i reads pole rows from memory when i == 0 (the chunk starts from a
// materialised field) and from the ring partials of step i-1 otherwise; the chunk ends by
// materialising the pole rows. WGSL semantics: runs of wtb_k steps go through the temporally
// blocked kernel, a remainder of 2 or 3 through one shorter blocked launch; with last_single the
// final step is a single-step launch, so the other buffer ends one pass behind the newest (what
// the reference's current_buffer() returns). A run that asks for the caustic map ends
// [..., blocked launch of kWtbCausticK passes that writes the map of its result, single pass].
int enqueue_steps(sbs_drainage *h, int start, int count, float dt, bool vol_last, bool use_sched, bool last_single,
                  int *end) {
    const Consts &k = consts_of(h);
    if (h->sem == SBS_CPU_SEMANTICS) {
        // runs of cpu_k steps through the blocked kernel (pole rows materialised in memory
        // before and after each launch), then the remainder as single steps whose pole rows
        // after the first are the ring partials of the previous step
        const int K = h->cpu_k > 1 ? h->cpu_k : 1;
        const int groups = K > 1 ? count / K : 0;
        const int singles = count - groups * K;
        const int total = groups + singles;
        int cur = start, step = 0;
        for (int n = 0; n < total; ++n) {
            const bool blocked = n < groups;
            const int j = n - groups;  // index among the single steps
            StepArgs a{};
            a.hin = h->h[cur];
            a.hout = h->h[cur ^ 1];
            a.lin = h->hl[cur];
            a.lout = h->hl[cur ^ 1];
            a.rows = h->rows;
            a.pin = h->part[(j + 1) & 1];
            a.pout = h->part[j & 1];
            a.tfe = use_sched ? h->sched_dev + step : nullptr;
            a.vol_w = vol_last && n + 1 == total ? h->vol_w : nullptr;
            a.vol_partials = h->vol_partials;
            a.vol_counter = h->vol_counter;
            a.vol_out = h->vol_out;
            a.vol_index = h->vol_index;
            a.nt = h->nt;
            a.np = h->np;
            a.pitch = (int)h->pitch;
            a.rb = blocked ? h->cgeom.rb : h->geom.rb;
            a.poles_virtual = !blocked && j > 0 ? 1 : 0;
            a.crit = k.crit;
            a.b = k.b;
            a.DR2 = k.DR2;
            a.dt = dt;
            a.prow = h->cgeom.prow;
            a.ring_part = h->ring_part;
            a.ring_bar = h->ring_bar;
            a.status_host = h->ring_status_dev;
            {
                const WaitConfig wc = wait_config();
                a.wait_cycles = wc.cycles;
                a.extra = (wc.stall & SBS_STALL_GRID_BARRIER) ? 1u : 0u;
            }
            if (blocked)
                SBS_CUDA_TRY(launch_wtbc(K, h->x2, a, h->cgeom, h->stream));
            else
                SBS_CUDA_TRY(launch_step(h->sem, h->x2, a, h->geom, h->stream));
            step += blocked ? K : 1;
            cur ^= 1;
        }
        if (singles > 0)
            SBS_CUDA_TRY(launch_finalize_poles(h->h[cur], h->hl[cur], h->part[(singles - 1) & 1], h->geom.nbx, h->nt,
                                               h->np, (int)h->pitch, h->stream));
        *end = cur;
        return SBS_OK;
    }
    std::vector<int> plan;  // steps per launch; -kWtbCausticK: the launch that also writes the map
    if (h->sem == SBS_WGSL_SEMANTICS && h->wtb_k > 1) {
        const bool cau = cau_plan(h, count, last_single);
        int rem = count - (last_single && count > 0 ? 1 : 0) - (cau ? kWtbCausticK : 0);
        while (rem >= h->wtb_k) {
            plan.push_back(h->wtb_k);
            rem -= h->wtb_k;
        }
        if (rem >= 2) {  // a remainder of 2 or 3 passes in one shorter blocked launch
            plan.push_back(rem);
            rem = 0;
        }
        for (; rem > 0; --rem) plan.push_back(1);
        if (cau) plan.push_back(-kWtbCausticK);
        if (last_single && count > 0) plan.push_back(1);
    } else {
        plan.assign(count, 1);
    }
    int cur = start;
    for (size_t i = 0; i < plan.size(); ++i) {
        StepArgs a{};
        a.hin = h->h[cur];
        a.hout = h->h[cur ^ 1];
        a.cin = h->c[cur];
        a.cout = h->c[cur ^ 1];
        a.lin = h->hl[cur];
        a.lout = h->hl[cur ^ 1];
        a.rows = h->rows;
        a.pin = h->part[(i + 1) & 1];
        a.pout = h->part[i & 1];
        a.tfe = use_sched ? h->sched_dev + i : nullptr;
        const bool vol = vol_last && i + 1 == plan.size();
        a.vol_w = vol ? h->vol_w : nullptr;
        a.vol_partials = h->vol_partials;
        a.vol_counter = h->vol_counter;
        a.vol_out = h->vol_out;
        a.vol_index = h->vol_index;
        a.nt = h->nt;
        a.np = h->np;
        a.pitch = (int)h->pitch;
        const bool cau_launch = plan[i] < 0;
        const int steps = cau_launch ? -plan[i] : plan[i];
        a.rb = cau_launch ? h->cau_geom.rb : steps > 1 ? h->wgeom.rb : h->geom.rb;
        if (cau_launch) {
            a.cau_out = h->cau_out;
            a.cau_focal = h->cau_p[0];
            a.cau_scale = h->cau_p[1];
            a.cau_sharp = h->cau_p[2];
            a.cau_branch = h->cau_p[3];
        }
        a.poles_virtual = i > 0 ? 1 : 0;
        a.marangoni = h->params.marangoni_enabled ? 1 : 0;
        a.crit = k.crit;
        a.b = k.b;
        a.DR2 = k.DR2;
        a.DsR2 = k.DsR2;
        a.Gt = k.Gt;
        a.M = k.M;
        a.dt = dt;
        if (steps > 1)
            SBS_CUDA_TRY(launch_wtb(steps, a, cau_launch ? h->cau_geom : h->wgeom, h->stream));
        else
            SBS_CUDA_TRY(launch_step(h->sem, h->x2, a, h->geom, h->stream));
        cur ^= 1;
    }
    if (h->sem == SBS_CPU_SEMANTICS && count > 0)
        SBS_CUDA_TRY(launch_finalize_poles(h->h[cur], h->hl[cur], h->part[(count - 1) & 1], h->geom.nbx, h->nt,
                                           h->np, (int)h->pitch, h->stream));
    *end = cur;
    return SBS_OK;
}

// Number of launches enqueue_steps uses for `count` steps (each flips the ping-pong buffers).
int launches_in(const sbs_drainage *h, int count, bool last_single) {
    if (h->sem == SBS_CPU_SEMANTICS) return h->cpu_k > 1 ? count / h->cpu_k + count % h->cpu_k : count;
    if (!(h->sem == SBS_WGSL_SEMANTICS && h->wtb_k > 1)) return count;
    const int tail = last_single && count > 0 ? 1 : 0;
    const int cau = cau_plan(h, count, last_single) ? 1 : 0;
    const int body = count - tail - cau * kWtbCausticK;
    const int rem = body % h->wtb_k;
    return body / h->wtb_k + (rem >= 2 ? 1 : rem) + cau + tail;
}

// Runs one chunk (count <= kMaxChunk) through a cached CUDA graph (or directly when short).
int run_chunk(sbs_drainage *h, int count, double dt, bool vol_last, bool last_single) {
    const bool cpu = h->sem == SBS_CPU_SEMANTICS;
    const bool use_sched = cpu && h->tfe.enabled;
    float dtf;
    if (cpu) {
        dtf = (float)dt;
        if (use_sched) {
            const int slot = h->sched_slot;
            SBS_CUDA_TRY(cudaEventSynchronize(h->sched_ev[slot]));
            TfeStep *hs = h->sched_host[slot];
            for (int i = 0; i < count; ++i) {
                h->tfe.advance(h->current_time, dt, h->nt, h->np, hs + i);
                h->current_time += dt;
            }
            SBS_CUDA_TRY(cudaMemcpyAsync(h->sched_dev, hs, sizeof(TfeStep) * count, cudaMemcpyHostToDevice,
                                         h->stream));
            SBS_CUDA_TRY(cudaEventRecord(h->sched_ev[slot], h->stream));
            h->sched_slot ^= 1;
        } else {
            for (int i = 0; i < count; ++i) h->current_time += dt;
        }
    } else {
        dtf = h->params.dt;
        for (int i = 0; i < count; ++i) h->current_time += (double)h->params.dt;
    }
    int end = h->cur;
    if (count < kGraphMin) {
        int rc = enqueue_steps(h, h->cur, count, dtf, vol_last, use_sched, last_single, &end);
        if (rc) return rc;
    } else {
        uint32_t bits;
        std::memcpy(&bits, &dtf, 4);
        std::string key = std::to_string(h->cur) + ":" + std::to_string(count) + ":" + std::to_string(vol_last) +
                          ":" + std::to_string(use_sched) + ":" + std::to_string(bits) + ":" +
                          std::to_string(last_single) + ":" + std::to_string(h->wtb_k) + ":" +
                          std::to_string(h->cpu_k);
        if (cau_plan(h, count, last_single)) {  // the map's destination and parameters are in the graph
            uint32_t pb[4];
            std::memcpy(pb, h->cau_p, sizeof(pb));
            key += ":cau:" + std::to_string((uintptr_t)h->cau_out);
            for (uint32_t v : pb) key += ":" + std::to_string(v);
        }
        auto it = h->graphs.find(key);
        cudaGraphExec_t exec = nullptr;
        if (it == h->graphs.end()) {
            cudaGraph_t graph = nullptr;
            SBS_CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
            int rc = enqueue_steps(h, h->cur, count, dtf, vol_last, use_sched, last_single, &end);
            cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            SBS_CUDA_TRY(ce);
            cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
            cudaGraphDestroy(graph);
            SBS_CUDA_TRY(ie);
            h->graphs[key] = exec;
        } else {
            exec = it->second;
        }
        end = h->cur ^ (launches_in(h, count, last_single) & 1);
        SBS_CUDA_TRY(cudaGraphLaunch(exec, h->stream));
    }
    if (last_single && h->cau_on) h->cau_fused = cau_plan(h, count, last_single);
    h->cur = end;
    h->prev = end ^ 1;
    return SBS_OK;
}

// After the stream has drained: a timed-out ring barrier of the blocked CPU-semantics step turns
// into SBS_E_TIMEOUT, and the barrier words are cleared for the next call.
int check_ring_status(sbs_drainage *h) {
    if (!h->ring_status || *(volatile unsigned *)h->ring_status == 0u) return SBS_OK;
    *(volatile unsigned *)h->ring_status = 0u;
    SBS_CUDA_TRY(cudaMemsetAsync(h->ring_bar, 0, sizeof(unsigned) * kWtbcBarWords, h->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return set_error(SBS_E_TIMEOUT, "drainage: a pole-ring barrier wait timed out");
}

// Advances n steps in chunks; a volume check follows every check_every-th step (0 = none).
int run_steps(sbs_drainage *h, double dt, uint64_t n, uint32_t check_every) {
    if (h->tfe.error) return set_error(SBS_E_STATE, "TFE front columns are not one interval");
    if (h->ring_bar) {
        const unsigned epoch = wait_config().epoch;
        if (epoch != h->wait_epoch) {  // the launches carry the wait settings: capture them again
            SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
            destroy_graphs(h);
            h->wait_epoch = epoch;
        }
    }
    uint64_t done = 0;
    while (done < n) {
        uint64_t g = std::min<uint64_t>(kMaxChunk, n - done);
        bool vol = false;
        if (check_every > 0) {
            const uint64_t to_check = check_every - (done % check_every);
            if (to_check <= g) {
                g = to_check;
                vol = true;
            }
        }
        int rc = run_chunk(h, (int)g, dt, vol, done + g == n);
        if (rc) return rc;
        done += g;
    }
    if (h->tfe.error) return set_error(SBS_E_STATE, "TFE front columns are not one interval");
    return SBS_OK;
}

// `passes` WGSL passes, then the caustic map of the field one pass behind the newest (the buffer
// the reference's caustic renderer binds) into `map` (device or host memory): the final blocked
// launch writes the map of its result, so the field is not read again; runs too short for that
// launch use the standalone caustic pass.
int run_with_caustics(sbs_drainage *h, uint32_t passes, const sbs_caustic_params *p, float *map, int mem) {
    const size_t bytes = sizeof(float) * (size_t)h->np * (size_t)h->nt;
    float *dst = map;
    if (mem == SBS_MEM_HOST) {
        if (!h->cau_buf) SBS_CUDA_TRY(cudaMalloc(&h->cau_buf, bytes));
        dst = h->cau_buf;
    }
    h->cau_on = true;
    h->cau_fused = false;
    h->cau_out = dst;
    h->cau_p[0] = p->focal_length;
    h->cau_p[1] = p->caustic_intensity;
    h->cau_p[2] = p->caustic_sharpness;
    h->cau_p[3] = p->branch_threshold;
    int rc = run_steps(h, 0.0, passes, 0);
    h->cau_on = false;
    if (rc) return rc;
    if (!h->cau_fused) {
        rc = sbs_caustics(p, h->h[h->prev], h->pitch, dst, SBS_MEM_DEVICE, h->stream);
        if (rc) return rc;
    }
    if (mem == SBS_MEM_HOST) SBS_CUDA_TRY(cudaMemcpyAsync(map, dst, bytes, cudaMemcpyDeviceToHost, h->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return SBS_OK;
}

int field_reduce(sbs_drainage *h, ReduceOut *out) {
    SBS_CUDA_TRY(launch_field_reduce(h->h[h->cur], h->hl[h->cur], h->nt, h->np, h->pitch, h->vol_w,
                                     h->red_partials, h->red_counter, h->red_out, h->stream));
    SBS_CUDA_TRY(cudaMemcpyAsync(out, h->red_out, sizeof(ReduceOut), cudaMemcpyDeviceToHost, h->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return SBS_OK;
}

int ensure_qbuf(sbs_drainage *h, size_t bytes) {
    if (h->qcap >= bytes) return SBS_OK;
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    cudaFree(h->qbuf);
    h->qbuf = nullptr;
    h->qcap = 0;
    size_t cap = std::max<size_t>(bytes, 1 << 16);
    SBS_CUDA_TRY(cudaMalloc(&h->qbuf, cap));
    h->qcap = cap;
    return SBS_OK;
}

int copy_field_in(sbs_drainage *h, float *const *dst_bufs, int nbufs, const float *src, size_t n, int mem) {
    SBS_CHECK_ARG(src != nullptr, "src is null");
    SBS_CHECK_ARG(n == (size_t)h->nt * h->np, "field has %zu values, expected %d x %d", n, h->nt, h->np);
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "bad mem flag %d", mem);
    const cudaMemcpyKind kind = mem == SBS_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    // the first buffer from the source, further ping-pong buffers from the first on the device
    SBS_CUDA_TRY(cudaMemcpy2DAsync(dst_bufs[0], h->pitch * sizeof(float), src, h->np * sizeof(float),
                                   h->np * sizeof(float), h->nt, kind, h->stream));
    for (int i = 1; i < nbufs; ++i)
        SBS_CUDA_TRY(cudaMemcpyAsync(dst_bufs[i], dst_bufs[0], h->pitch * h->nt * sizeof(float),
                                     cudaMemcpyDeviceToDevice, h->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return SBS_OK;
}

int copy_field_out(sbs_drainage *h, const float *buf, float *dst, size_t n, int mem) {
    SBS_CHECK_ARG(dst != nullptr, "dst is null");
    SBS_CHECK_ARG(n == (size_t)h->nt * h->np, "field has %zu values, expected %d x %d", n, h->nt, h->np);
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "bad mem flag %d", mem);
    const cudaMemcpyKind kind = mem == SBS_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    SBS_CUDA_TRY(cudaMemcpy2DAsync(dst, h->np * sizeof(float), buf, h->pitch * sizeof(float), h->np * sizeof(float),
                                   h->nt, kind, h->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return SBS_OK;
}

int create_common(sbs_drainage *h) {
    int rc = require_device();
    if (rc) return rc;
    h->pitch = round_up((size_t)h->np, 128);
    rc = allocate(h);
    if (rc) return rc;
    return upload_tables(h, &consts_of(h));
}

#define CHECK_HANDLE(h) SBS_CHECK_ARG((h) != nullptr, "handle is null")
#define REQUIRE_SEM(h, s)                                                                                    \
    do {                                                                                                     \
        if ((h)->sem != (s))                                                                                 \
            return set_error(SBS_E_STATE, "call needs %s semantics",                                         \
                             (s) == SBS_CPU_SEMANTICS ? "CPU (DrainageSimulator)" : "WGSL (GPUDrainageSimulator)"); \
    } while (0)

}  // namespace

namespace sbs {
int drainage_run_async(sbs_drainage *h, uint32_t passes) { return run_steps(h, 0.0, passes, 0); }
}  // namespace sbs

extern "C" {

int sbs_drainage_create(const sbs_config *cfg, sbs_drainage **out) {
    return sbs_drainage_create_ex(cfg, SBS_DRAIN_F32X2, out);
}

int sbs_drainage_create_ex(const sbs_config *cfg, int precision, sbs_drainage **out) {
    clear_error();
    SBS_CHECK_ARG(cfg != nullptr && out != nullptr, "null argument");
    SBS_CHECK_ARG(precision == SBS_DRAIN_F32 || precision == SBS_DRAIN_F32X2, "bad precision %d", precision);
    SBS_CHECK_ARG(cfg->resolution >= 3, "resolution must be >= 3 (got %u)", cfg->resolution);
    SBS_CHECK_ARG(cfg->resolution <= 32768, "resolution %u too large", cfg->resolution);
    SBS_CHECK_ARG(cfg->diameter > 0 && std::isfinite(cfg->diameter), "diameter must be finite and > 0");
    SBS_CHECK_ARG(cfg->viscosity > 0 && std::isfinite(cfg->viscosity), "viscosity must be finite and > 0");
    SBS_CHECK_ARG(std::isfinite(cfg->density) && std::isfinite(cfg->gravity) &&
                      std::isfinite(cfg->surfactant_diffusion) && std::isfinite(cfg->film_thickness_nm) &&
                      std::isfinite(cfg->critical_thickness_nm),
                  "non-finite config value");
    *out = nullptr;
    sbs_drainage *h = new sbs_drainage();
    h->sem = SBS_CPU_SEMANTICS;
    h->x2 = precision == SBS_DRAIN_F32X2 ? 1 : 0;
    h->cfg = *cfg;
    h->nt = (int)cfg->resolution;
    h->np = 2 * (int)cfg->resolution;
    h->radius = cfg->diameter / 2.0;
    h->critical = cfg->critical_thickness_nm * 1e-9;
    sbs_drainage_params_default(&h->params);
    int rc = create_common(h);
    if (rc == SBS_OK) {
        const double v = cfg->film_thickness_nm * 1e-9;
        const float hi = (float)v;
        cudaError_t e = launch_fill(h->h[0], h->pitch, h->nt, h->np, hi, h->stream);
        if (e == cudaSuccess && h->x2) e = launch_fill(h->hl[0], h->pitch, h->nt, h->np, (float)(v - (double)hi), h->stream);
        if (e != cudaSuccess) rc = set_error(SBS_E_CUDA, "fill failed: %s", cudaGetErrorString(e));
    }
    if (rc == SBS_OK && cudaStreamSynchronize(h->stream) != cudaSuccess) rc = set_error(SBS_E_CUDA, "sync failed");
    if (rc) {
        release(h);
        delete h;
        return rc;
    }
    *out = h;
    return SBS_OK;
}

int sbs_gpu_drainage_create(float initial_thickness, uint32_t grid_width, uint32_t grid_height, sbs_drainage **out) {
    clear_error();
    SBS_CHECK_ARG(out != nullptr, "out is null");
    SBS_CHECK_ARG(grid_width >= 3 && grid_height >= 3, "grid must be at least 3 x 3 (got %u x %u)", grid_width,
                  grid_height);
    SBS_CHECK_ARG(grid_width <= 65536 && grid_height <= 32768, "grid too large");
    SBS_CHECK_ARG(std::isfinite(initial_thickness), "initial thickness not finite");
    *out = nullptr;
    sbs_drainage *h = new sbs_drainage();
    h->sem = SBS_WGSL_SEMANTICS;
    sbs_config_default(&h->cfg);
    sbs_drainage_params_default(&h->params);
    h->params.grid_width = grid_width;
    h->params.grid_height = grid_height;
    h->nt = (int)grid_height;
    h->np = (int)grid_width;
    h->radius = h->params.bubble_radius;
    h->critical = h->params.critical_thickness;
    h->tfe.enabled = false;
    int rc = create_common(h);
    for (int i = 0; rc == SBS_OK && i < 2; ++i) {
        if (launch_fill(h->h[i], h->pitch, h->nt, h->np, initial_thickness, h->stream) != cudaSuccess ||
            launch_fill(h->c[i], h->pitch, h->nt, h->np, 0.5f, h->stream) != cudaSuccess)
            rc = set_error(SBS_E_CUDA, "fill failed");
    }
    if (rc == SBS_OK && cudaStreamSynchronize(h->stream) != cudaSuccess) rc = set_error(SBS_E_CUDA, "sync failed");
    if (rc) {
        release(h);
        delete h;
        return rc;
    }
    *out = h;
    return SBS_OK;
}

int sbs_drainage_destroy(sbs_drainage *h) {
    if (!h) return SBS_OK;
    release(h);
    delete h;
    return SBS_OK;
}

int sbs_drainage_precision(const sbs_drainage *h, int *out) {
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(out, "out is null");
    *out = h->x2 ? SBS_DRAIN_F32X2 : SBS_DRAIN_F32;
    return SBS_OK;
}

int sbs_drainage_semantics(const sbs_drainage *h, int *out) {
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(out, "out is null");
    *out = h->sem;
    return SBS_OK;
}

int sbs_drainage_grid_size(const sbs_drainage *h, uint32_t *num_theta, uint32_t *num_phi) {
    CHECK_HANDLE(h);
    if (num_theta) *num_theta = (uint32_t)h->nt;
    if (num_phi) *num_phi = (uint32_t)h->np;
    return SBS_OK;
}

int sbs_drainage_step(sbs_drainage *h, double dt) { return sbs_drainage_step_n(h, dt, 1); }

int sbs_drainage_step_n(sbs_drainage *h, double dt, uint32_t n) {
    clear_error();
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_CPU_SEMANTICS);
    SBS_CHECK_ARG(std::isfinite(dt), "dt must be finite");
    int rc = run_steps(h, dt, n, 0);
    if (rc) return rc;
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return check_ring_status(h);
}

int sbs_gpu_drainage_step(sbs_drainage *h, float frame_dt) {
    clear_error();
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    if (!h->enabled) return SBS_OK;  // gpu_drainage.rs:339-341
    const float scaled_dt = frame_dt * h->time_scale;
    const float step_dt = scaled_dt / (float)h->steps_per_frame;
    const double t0 = h->current_time;
    int rc = run_steps(h, 0.0, h->steps_per_frame, 0);
    if (rc) return rc;
    h->current_time = t0;
    for (uint32_t i = 0; i < h->steps_per_frame; ++i) h->current_time += (double)step_dt;
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return SBS_OK;
}

int sbs_gpu_drainage_run(sbs_drainage *h, uint32_t passes) {
    clear_error();
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    int rc = run_steps(h, 0.0, passes, 0);
    if (rc) return rc;
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return SBS_OK;
}

int sbs_gpu_drainage_run_caustics(sbs_drainage *h, uint32_t passes, const sbs_caustic_params *p, float *caustic_map,
                                  int mem) {
    clear_error();
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    SBS_CHECK_ARG(p != nullptr && caustic_map != nullptr, "null argument");
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "bad mem flag %d", mem);
    SBS_CHECK_ARG(p->grid_width == (uint32_t)h->np && p->grid_height == (uint32_t)h->nt,
                  "caustic grid %ux%u differs from the handle's %dx%d", p->grid_width, p->grid_height, h->np, h->nt);
    return run_with_caustics(h, passes, p, caustic_map, mem);
}

int sbs_gpu_drainage_step_caustics(sbs_drainage *h, float frame_dt, const sbs_caustic_params *p, float *caustic_map,
                                   int mem) {
    clear_error();
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    SBS_CHECK_ARG(p != nullptr && caustic_map != nullptr, "null argument");
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "bad mem flag %d", mem);
    SBS_CHECK_ARG(p->grid_width == (uint32_t)h->np && p->grid_height == (uint32_t)h->nt,
                  "caustic grid %ux%u differs from the handle's %dx%d", p->grid_width, p->grid_height, h->np, h->nt);
    const uint32_t passes = h->enabled ? h->steps_per_frame : 0u;  // gpu_drainage.rs:339-341
    const float step_dt = frame_dt * h->time_scale / (float)h->steps_per_frame;
    const double t0 = h->current_time;
    int rc = run_with_caustics(h, passes, p, caustic_map, mem);
    if (rc) return rc;
    h->current_time = t0;
    for (uint32_t i = 0; i < passes; ++i) h->current_time += (double)step_dt;
    return SBS_OK;
}

int sbs_drainage_run_checked(sbs_drainage *h, double dt, uint32_t n, uint32_t check_every, double *volumes_out) {
    clear_error();
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(std::isfinite(dt), "dt must be finite");
    const uint32_t nchecks = check_every ? n / check_every : 0;
    SBS_CHECK_ARG(nchecks == 0 || volumes_out != nullptr, "volumes_out is null");
    if (nchecks > h->vol_out_cap) {
        SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
        cudaFree(h->vol_out);
        h->vol_out = nullptr;
        destroy_graphs(h);
        SBS_CUDA_TRY(cudaMalloc(&h->vol_out, sizeof(double) * nchecks));
        h->vol_out_cap = nchecks;
    }
    SBS_CUDA_TRY(cudaMemsetAsync(h->vol_index, 0, sizeof(unsigned), h->stream));
    int rc = run_steps(h, dt, n, check_every);
    if (rc) return rc;
    if (nchecks)
        SBS_CUDA_TRY(cudaMemcpyAsync(volumes_out, h->vol_out, sizeof(double) * nchecks, cudaMemcpyDeviceToHost,
                                     h->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return check_ring_status(h);
}

int sbs_drainage_set_thickness(sbs_drainage *h, const float *src, size_t n, int mem) {
    clear_error();
    CHECK_HANDLE(h);
    if (h->sem == SBS_WGSL_SEMANTICS) {
        float *bufs[2] = {h->h[0], h->h[1]};
        return copy_field_in(h, bufs, 2, src, n, mem);
    }
    float *bufs[1] = {h->h[h->cur]};
    int rc = copy_field_in(h, bufs, 1, src, n, mem);
    if (rc == SBS_OK && h->x2) {
        SBS_CUDA_TRY(launch_fill(h->hl[h->cur], h->pitch, h->nt, h->np, 0.0f, h->stream));
        SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    }
    return rc;
}

int sbs_drainage_get_thickness_field(sbs_drainage *h, float *dst, size_t n, int mem) {
    clear_error();
    CHECK_HANDLE(h);
    return copy_field_out(h, h->h[h->cur], dst, n, mem);
}

int sbs_drainage_set_concentration(sbs_drainage *h, const float *src, size_t n, int mem) {
    clear_error();
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    float *bufs[2] = {h->c[0], h->c[1]};
    return copy_field_in(h, bufs, 2, src, n, mem);
}

int sbs_drainage_get_concentration_field(sbs_drainage *h, float *dst, size_t n, int mem) {
    clear_error();
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    return copy_field_out(h, h->c[h->cur], dst, n, mem);
}

int sbs_drainage_set_thickness_f64(sbs_drainage *h, const double *src, size_t n) {
    clear_error();
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(src != nullptr, "src is null");
    SBS_CHECK_ARG(n == (size_t)h->nt * h->np, "field has %zu values, expected %d x %d", n, h->nt, h->np);
    if (!h->x2) {
        std::vector<float> tmp(n);
        for (size_t i = 0; i < n; ++i) tmp[i] = (float)src[i];
        return sbs_drainage_set_thickness(h, tmp.data(), n, SBS_MEM_HOST);
    }
    int rc = ensure_qbuf(h, n * sizeof(double));
    if (rc) return rc;
    SBS_CUDA_TRY(cudaMemcpyAsync(h->qbuf, src, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    SBS_CUDA_TRY(launch_split_f64(h->qbuf, h->h[h->cur], h->hl[h->cur], h->nt, h->np, h->pitch, h->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return SBS_OK;
}

int sbs_drainage_get_thickness_field_f64(sbs_drainage *h, double *dst, size_t n) {
    clear_error();
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(dst != nullptr, "dst is null");
    SBS_CHECK_ARG(n == (size_t)h->nt * h->np, "field has %zu values, expected %d x %d", n, h->nt, h->np);
    int rc = ensure_qbuf(h, n * sizeof(double));
    if (rc) return rc;
    SBS_CUDA_TRY(launch_join_f64(h->h[h->cur], h->hl[h->cur], h->qbuf, h->nt, h->np, h->pitch, h->stream));
    SBS_CUDA_TRY(cudaMemcpyAsync(dst, h->qbuf, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return SBS_OK;
}

int sbs_drainage_thickness_device(sbs_drainage *h, int which, const float **ptr, size_t *pitch) {
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(ptr != nullptr, "ptr is null");
    SBS_CHECK_ARG(which == 0 || which == 1, "which must be 0 or 1");
    if (which == 1) REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    *ptr = which == 0 ? h->h[h->cur] : h->h[h->prev];
    if (pitch) *pitch = h->pitch;
    return SBS_OK;
}

int sbs_drainage_concentration_device(sbs_drainage *h, int which, const float **ptr, size_t *pitch) {
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    SBS_CHECK_ARG(ptr != nullptr, "ptr is null");
    SBS_CHECK_ARG(which == 0 || which == 1, "which must be 0 or 1");
    *ptr = which == 0 ? h->c[h->cur] : h->c[h->prev];
    if (pitch) *pitch = h->pitch;
    return SBS_OK;
}

int sbs_drainage_stream(const sbs_drainage *h, void **out) {
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(out != nullptr, "out is null");
    *out = (void *)h->stream;
    return SBS_OK;
}

int sbs_drainage_query_batch(sbs_drainage *h, const double *theta, const double *phi, double *out, size_t n,
                             int mem) {
    clear_error();
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "bad mem flag %d", mem);
    if (n == 0) return SBS_OK;
    SBS_CHECK_ARG(theta && phi && out, "null pointer");
    const float *field = h->h[h->cur];
    if (mem == SBS_MEM_DEVICE) {
        SBS_CUDA_TRY(launch_query(field, h->hl[h->cur], h->nt, h->np, h->pitch, theta, phi, out, n, h->stream));
    } else {
        int rc = ensure_qbuf(h, 3 * n * sizeof(double));
        if (rc) return rc;
        double *dt = h->qbuf, *dp = h->qbuf + n, *dout = h->qbuf + 2 * n;
        SBS_CUDA_TRY(cudaMemcpyAsync(dt, theta, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        SBS_CUDA_TRY(cudaMemcpyAsync(dp, phi, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        SBS_CUDA_TRY(launch_query(field, h->hl[h->cur], h->nt, h->np, h->pitch, dt, dp, dout, n, h->stream));
        SBS_CUDA_TRY(cudaMemcpyAsync(out, dout, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    }
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return SBS_OK;
}

int sbs_drainage_get_thickness(sbs_drainage *h, double theta, double phi, double *out) {
    SBS_CHECK_ARG(out != nullptr, "out is null");
    return sbs_drainage_query_batch(h, &theta, &phi, out, 1, SBS_MEM_HOST);
}

int sbs_drainage_current_time(const sbs_drainage *h, double *out) {
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(out != nullptr, "out is null");
    *out = h->current_time;
    return SBS_OK;
}

int sbs_drainage_min_max(sbs_drainage *h, double *min_out, double *max_out) {
    clear_error();
    CHECK_HANDLE(h);
    ReduceOut r{};
    int rc = field_reduce(h, &r);
    if (rc) return rc;
    if (min_out) *min_out = r.vmin;
    if (max_out) *max_out = r.vmax;
    return SBS_OK;
}

int sbs_drainage_has_critical_region(sbs_drainage *h, int *out) {
    SBS_CHECK_ARG(out != nullptr, "out is null");
    double mn = 0.0;
    int rc = sbs_drainage_min_max(h, &mn, nullptr);
    if (rc) return rc;
    const double crit = h->sem == SBS_CPU_SEMANTICS ? h->critical : (double)h->params.critical_thickness;
    *out = mn < crit ? 1 : 0;
    return SBS_OK;
}

int sbs_drainage_critical_thickness(const sbs_drainage *h, double *out) {
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(out != nullptr, "out is null");
    *out = h->sem == SBS_CPU_SEMANTICS ? h->critical : (double)h->params.critical_thickness;
    return SBS_OK;
}

int sbs_drainage_film_volume(sbs_drainage *h, double *out) {
    clear_error();
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(out != nullptr, "out is null");
    ReduceOut r{};
    int rc = field_reduce(h, &r);
    if (rc) return rc;
    *out = r.volume;
    return SBS_OK;
}

int sbs_drainage_reset(sbs_drainage *h, double initial_thickness) {
    clear_error();
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(std::isfinite(initial_thickness), "initial thickness not finite");
    if (h->sem == SBS_CPU_SEMANTICS) {
        if (h->x2) {
            const double v = initial_thickness;
            const float hi = (float)v;
            SBS_CUDA_TRY(launch_fill(h->h[h->cur], h->pitch, h->nt, h->np, hi, h->stream));
            SBS_CUDA_TRY(launch_fill(h->hl[h->cur], h->pitch, h->nt, h->np, (float)(v - (double)hi), h->stream));
        } else {
            SBS_CUDA_TRY(launch_fill(h->h[h->cur], h->pitch, h->nt, h->np, (float)initial_thickness, h->stream));
        }
        h->tfe.reset();
    } else {
        for (int i = 0; i < 2; ++i) {
            SBS_CUDA_TRY(launch_fill(h->h[i], h->pitch, h->nt, h->np, (float)initial_thickness, h->stream));
            SBS_CUDA_TRY(launch_fill(h->c[i], h->pitch, h->nt, h->np, 0.5f, h->stream));
        }
        h->cur = 0;
        h->prev = 1;
    }
    h->current_time = 0.0;
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return SBS_OK;
}

int sbs_drainage_set_marginal_regeneration(sbs_drainage *h, int enabled) {
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_CPU_SEMANTICS);
    h->tfe.enabled = enabled != 0;
    if (!enabled) h->tfe.fronts.clear();
    return SBS_OK;
}

int sbs_drainage_marginal_regeneration_enabled(const sbs_drainage *h, int *out) {
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(out != nullptr, "out is null");
    *out = h->tfe.enabled ? 1 : 0;
    return SBS_OK;
}

int sbs_drainage_set_tfe_thickness_ratio(sbs_drainage *h, double ratio) {
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_CPU_SEMANTICS);
    SBS_CHECK_ARG(!std::isnan(ratio), "ratio is NaN");
    h->tfe.ratio = std::min(std::max(ratio, 0.5), 0.95);
    return SBS_OK;
}

int sbs_drainage_tfe_thickness_ratio(const sbs_drainage *h, double *out) {
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(out != nullptr, "out is null");
    *out = h->tfe.ratio;
    return SBS_OK;
}

int sbs_drainage_active_tfe_count(const sbs_drainage *h, uint32_t *out) {
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(out != nullptr, "out is null");
    *out = (uint32_t)h->tfe.fronts.size();
    return SBS_OK;
}

int sbs_gpu_drainage_update_params(sbs_drainage *h, const sbs_drainage_params *p) {
    clear_error();
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    SBS_CHECK_ARG(p != nullptr, "params is null");
    SBS_CHECK_ARG(p->grid_width == (uint32_t)h->np && p->grid_height == (uint32_t)h->nt,
                  "params grid %ux%u differs from the buffers' %dx%d", p->grid_width, p->grid_height, h->np, h->nt);
    h->params = *p;
    return refresh(h, &consts_of(h));
}

int sbs_gpu_drainage_params(const sbs_drainage *h, sbs_drainage_params *out) {
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(out != nullptr, "out is null");
    *out = h->params;
    return SBS_OK;
}

int sbs_gpu_drainage_set_dt(sbs_drainage *h, float dt) {
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    h->params.dt = dt;
    return refresh(h, &consts_of(h));
}

int sbs_gpu_drainage_set_physics(sbs_drainage *h, float viscosity, float density, float gravity, float diffusion) {
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    h->params.viscosity = viscosity;
    h->params.density = density;
    h->params.gravity = gravity;
    h->params.diffusion_coeff = diffusion;
    return refresh(h, &consts_of(h));
}

int sbs_gpu_drainage_set_bubble_radius(sbs_drainage *h, float radius) {
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    h->params.bubble_radius = radius;
    h->radius = radius;
    return refresh(h, &consts_of(h));
}

int sbs_gpu_drainage_set_marangoni_enabled(sbs_drainage *h, int enabled) {
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    h->params.marangoni_enabled = enabled ? 1u : 0u;
    return refresh(h, &consts_of(h));
}

int sbs_gpu_drainage_set_marangoni_params(sbs_drainage *h, float gamma_air, float gamma_reduction,
                                          float surfactant_diffusion, float marangoni_coeff) {
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    h->params.gamma_air = gamma_air;
    h->params.gamma_reduction = gamma_reduction;
    h->params.surfactant_diffusion = surfactant_diffusion;
    h->params.marangoni_coeff = marangoni_coeff;
    return refresh(h, &consts_of(h));
}

int sbs_gpu_drainage_set_time_blocking(sbs_drainage *h, int steps_per_launch) {
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    SBS_CHECK_ARG(steps_per_launch >= 0 && steps_per_launch <= 4, "steps_per_launch must be 0..4");
    if (steps_per_launch > 1 && !wtb_supported(h->nt, h->np))
        return set_error(SBS_E_INVALID, "time blocking needs grid_width a multiple of 4 (got %d)", h->np);
    destroy_graphs(h);
    h->wtb_k = steps_per_launch > 1 ? steps_per_launch : 0;
    if (h->wtb_k) h->wgeom = wtb_geometry(h->nt, h->np, h->wtb_k);
    return SBS_OK;
}

int sbs_gpu_drainage_time_blocking(const sbs_drainage *h, int *out) {
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(out != nullptr, "out is null");
    *out = h->wtb_k > 1 ? h->wtb_k : 1;
    return SBS_OK;
}

int sbs_drainage_set_time_blocking(sbs_drainage *h, int steps_per_launch) {
    clear_error();
    CHECK_HANDLE(h);
    if (h->sem == SBS_WGSL_SEMANTICS) return sbs_gpu_drainage_set_time_blocking(h, steps_per_launch);
    SBS_CHECK_ARG(steps_per_launch >= 0 && steps_per_launch <= 4, "steps_per_launch must be 0..4");
    StepGeom g{};
    if (steps_per_launch > 1) {
        g = wtbc_geometry(h->nt, h->np, steps_per_launch, h->x2);
        if (g.nby < 1)
            return set_error(SBS_E_INVALID,
                             "time blocking needs an even resolution and at least %d theta rows (grid %d x %d)",
                             2 * (steps_per_launch + 1), h->nt, h->np);
    }
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    destroy_graphs(h);
    h->cpu_k = steps_per_launch > 1 ? steps_per_launch : 0;
    h->cgeom = g;
    return SBS_OK;
}

int sbs_drainage_time_blocking(const sbs_drainage *h, int *out) {
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(out != nullptr, "out is null");
    if (h->sem == SBS_WGSL_SEMANTICS) return sbs_gpu_drainage_time_blocking(h, out);
    *out = h->cpu_k > 1 ? h->cpu_k : 1;
    return SBS_OK;
}

int sbs_gpu_drainage_set_enabled(sbs_drainage *h, int enabled) {
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    h->enabled = enabled != 0;
    return SBS_OK;
}

int sbs_gpu_drainage_set_time_scale(sbs_drainage *h, float time_scale) {
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    h->time_scale = time_scale;
    return SBS_OK;
}

int sbs_gpu_drainage_set_steps_per_frame(sbs_drainage *h, uint32_t steps) {
    CHECK_HANDLE(h);
    REQUIRE_SEM(h, SBS_WGSL_SEMANTICS);
    h->steps_per_frame = steps;
    return SBS_OK;
}

int sbs_drainage_vertex_colors(sbs_drainage *h, const double *xyz, size_t nv, const double *lut, uint32_t T,
                               uint32_t A, double tmin, double tmax, double *rgb, int mem) {
    clear_error();
    CHECK_HANDLE(h);
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "bad mem flag %d", mem);
    SBS_CHECK_ARG(T >= 2 && A >= 2, "LUT must be at least 2 x 2");
    SBS_CHECK_ARG(tmax > tmin, "tmax must exceed tmin");
    if (nv == 0) return SBS_OK;
    SBS_CHECK_ARG(xyz && lut && rgb, "null pointer");
    const float *field = h->h[h->cur];
    if (mem == SBS_MEM_DEVICE) {
        SBS_CUDA_TRY(launch_vertex_colors(field, h->hl[h->cur], h->nt, h->np, h->pitch, xyz, nv, lut, (int)T,
                                          (int)A, tmin, tmax, rgb, h->stream));
    } else {
        const size_t lut_n = (size_t)T * A * 3;
        int rc = ensure_qbuf(h, (6 * nv + lut_n) * sizeof(double));
        if (rc) return rc;
        double *dx = h->qbuf, *drgb = h->qbuf + 3 * nv, *dl = h->qbuf + 6 * nv;
        SBS_CUDA_TRY(cudaMemcpyAsync(dx, xyz, 3 * nv * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        SBS_CUDA_TRY(cudaMemcpyAsync(dl, lut, lut_n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
        SBS_CUDA_TRY(launch_vertex_colors(field, h->hl[h->cur], h->nt, h->np, h->pitch, dx, nv, dl, (int)T, (int)A,
                                          tmin, tmax, drgb, h->stream));
        SBS_CUDA_TRY(cudaMemcpyAsync(rgb, drgb, 3 * nv * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    }
    SBS_CUDA_TRY(cudaStreamSynchronize(h->stream));
    return SBS_OK;
}

}  // extern "C"
