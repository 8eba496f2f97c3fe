// Batched foam drainage: thousands of bubbles with uneven theta-phi grids advanced together.
//
// The reference's foam bubbles carry one scalar film thickness each (foam.rs:44); here every
// bubble has its own WGSL-semantics drainage grid (resolution x 2 resolution cells, its own radius)
// and all of them advance in lockstep. Fields of all bubbles live in one arena; a work list splits
// every bubble into warp-sized items (a strip of theta rows x one 120-column segment), so a
// 32 x 64 bubble costs one warp and a 512 x 1024 bubble hundreds.
//
// One persistent kernel (cooperative launch, so every CTA is resident) runs all phases: in each
// phase every warp pulls items and advances them K steps with the register pipeline of wtb.cuh;
// a grid barrier separates phases (the next phase reads what others wrote, through L2 only). The
// barrier's spin is bounded: on timeout the kernel records it in a status word and returns.
// The launch is captured in a CUDA graph and replayed. Strip height and K come from an autotuner
// that times candidate tilings on the bubbles themselves (fields are saved and restored).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "sbs_internal.h"
#include "wtb.cuh"

namespace sbs {
namespace {

constexpr int kWarps = 4;
constexpr int kSeg = 120;                          // output columns per warp item

struct FoamBubble {
    float *h[2], *c[2];
    const float4 *rows;
    int nt, np, pitch;
    float b, DR2, DsR2, Gt, M;
};

struct FoamItem {
    int bubble, r0, r1, seg;
};

struct FoamArgs {
    const FoamBubble *bubbles;
    const FoamItem *items;
    int nitems, nphases, parity0, rbmax;
    float dt, crit;
    unsigned *bar;  // [0] arrival count, [1] generation, [2] status (bit 1: barrier timeout)
    long long wait_cycles;  // bound on one barrier wait
    unsigned extra;         // arrivals the barrier expects beyond the grid (1: the timeout test)
};

// Grid-wide barrier for a cooperative (all-resident) grid of `nblocks` blocks, completed by
// nblocks + extra arrivals (extra is 0 except in the timeout test, where nothing completes it);
// false if the wait ran past `limit` cycles.
__device__ bool grid_barrier(unsigned *bar, unsigned nblocks, unsigned extra, long long limit, int *s_timeout) {
    __syncthreads();
    if (threadIdx.x == 0) {
        *s_timeout = 0;
        const unsigned gen = atomicAdd(bar + 1, 0u);
        __threadfence();
        if (atomicAdd(bar, 1u) + 1 == nblocks + extra) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            const long long t0 = clock64();
            while (atomicAdd(bar + 1, 0u) == gen) {
                if (clock64() - t0 > limit) {
                    atomicOr(bar + 2, 2u);
                    *s_timeout = 1;
                    break;
                }
                __nanosleep(100);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return *s_timeout == 0;
}

// At least three blocks per SM: the K = 4 pipeline fits 168 registers (64 bytes of spills) instead
// of 202 (two blocks), 12 warps per SM instead of 8. Measured on the 4,096-bubble batch: 5.53e11
// cell-steps/s against 5.35e11; four blocks (128 registers) 4.98e11.
constexpr int kMinBlocksPerSm = 3;

template <int K, bool MAR>
__global__ void __launch_bounds__(kWarps * 32, kMinBlocksPerSm) foam_kernel(const FoamArgs a) {
    extern __shared__ float4 s_co_all[];  // per warp: rbmax + 2K coefficient rows
    __shared__ int s_timeout;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gw = blockIdx.x * kWarps + warp, nw = gridDim.x * kWarps;
    float4 *s_co = s_co_all + warp * (a.rbmax + 2 * K);

    for (int ph = 0; ph < a.nphases; ++ph) {
        const int par = (a.parity0 + ph) & 1;
        for (int it = gw; it < a.nitems; it += nw) {
            const FoamItem item = a.items[it];
            const FoamBubble &B = a.bubbles[item.bubble];
            const int nt = B.nt, np = B.np;
            __syncwarp();
            for (int i = lane; i < item.r1 - item.r0 + 2 * K; i += 32) {
                const int r = item.r0 - K + i;
                s_co[i] = (r >= 0 && r < nt) ? __ldg(B.rows + r) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
            __syncwarp();
            const int out0 = item.seg * kSeg;
            const int cu = out0 - 4 + 4 * lane;
            const int col = ((cu % np) + np) % np;
            Wtb w;
            w.hin = B.h[par] + col;
            w.cin = B.c[par] + col;
            w.hout = B.h[par ^ 1] + col;
            w.cout = B.c[par ^ 1] + col;
            w.sco = s_co;
            w.sco_base = item.r0 - K;
            w.nt = nt;
            w.pitch = B.pitch;
            w.r0 = item.r0;
            w.r1 = item.r1;
            w.store = lane >= 1 && lane <= 30 && cu < np;
            w.b = B.b;
            w.DR2 = B.DR2;
            w.DsR2 = B.DsR2;
            w.Gt = B.Gt;
            w.M = B.M;
            w.dt = a.dt;
            w.crit = a.crit;
            w.vol_w = nullptr;
            float4 wh[K][3], wc[K][3];
#pragma unroll
            for (int l = 0; l < K; ++l)
#pragma unroll
                for (int s = 0; s < 3; ++s) {
                    wh[l][s] = make_float4(0.f, 0.f, 0.f, 0.f);
                    wc[l][s] = wh[l][s];
                }
            double vacc = 0.0;
            const int t0 = w.r0 - K, t1 = w.r1 + K;
            float4 ph4 = make_float4(0.f, 0.f, 0.f, 0.f), pc4 = ph4;
            if (SBS_WTB_PREFETCH && t0 >= 0) {
                ph4 = __ldcg(reinterpret_cast<const float4 *>(w.hin + (size_t)t0 * w.pitch));
                pc4 = __ldcg(reinterpret_cast<const float4 *>(w.cin + (size_t)t0 * w.pitch));
            }
            for (int t = t0; t < t1; t += 3) {
                wtb_iter<K, 0, false, MAR, true>(w, t, wh, wc, ph4, pc4, vacc);
                if (t + 1 < t1) wtb_iter<K, 1, false, MAR, true>(w, t + 1, wh, wc, ph4, pc4, vacc);
                if (t + 2 < t1) wtb_iter<K, 2, false, MAR, true>(w, t + 2, wh, wc, ph4, pc4, vacc);
            }
        }
        if (ph + 1 < a.nphases && !grid_barrier(a.bar, gridDim.x, a.extra, a.wait_cycles, &s_timeout)) return;
    }
}

const void *foam_fn(int K, bool mar) {
    if (K == 1) return mar ? (const void *)foam_kernel<1, true> : (const void *)foam_kernel<1, false>;
    if (K == 2) return mar ? (const void *)foam_kernel<2, true> : (const void *)foam_kernel<2, false>;
    if (K == 4) return mar ? (const void *)foam_kernel<4, true> : (const void *)foam_kernel<4, false>;
    return nullptr;
}

}  // namespace
}  // namespace sbs

using namespace sbs;

struct sbs_foam {
    int nb = 0;
    std::vector<int> nt, np, pitch;
    std::vector<size_t> off, roff;
    std::vector<float> radius;
    size_t field_floats = 0;
    float *arena = nullptr;  // h0 | h1 | c0 | c1
    float4 *rows = nullptr;
    FoamBubble *d_bubbles = nullptr;
    FoamItem *d_items = nullptr;
    size_t items_cap = 0;
    int nitems = 0, rbmax = 0;
    unsigned *bar = nullptr;
    int cur = 0, K = 4, rb = 32;
    cudaStream_t stream = nullptr;
    sbs_drainage_params params{};
    bool graphs_ok = true;
    unsigned wait_epoch = 0;  // the wait settings the captured graphs were made with
    std::map<long long, cudaGraphExec_t> graphs;
};

namespace {

void foam_destroy_graphs(sbs_foam *f) {
    for (auto &kv : f->graphs) cudaGraphExecDestroy(kv.second);
    f->graphs.clear();
}

float *field_ptr(sbs_foam *f, int which /*0 h, 1 c*/, int parity, int bubble) {
    return f->arena + (size_t)(2 * which + parity) * f->field_floats + f->off[bubble];
}

int build_items(sbs_foam *f, int rb) {
    std::vector<FoamItem> items;
    for (int b = 0; b < f->nb; ++b) {
        const int segs = (f->np[b] + kSeg - 1) / kSeg;
        for (int r0 = 1; r0 < f->nt[b] - 1; r0 += rb) {
            const int r1 = std::min(r0 + rb, f->nt[b] - 1);
            for (int g = 0; g < segs; ++g) items.push_back(FoamItem{b, r0, r1, g});
        }
    }
    if (items.size() > f->items_cap) {
        cudaFree(f->d_items);
        f->d_items = nullptr;
        f->items_cap = 0;
        SBS_CUDA_TRY(cudaMalloc(&f->d_items, sizeof(FoamItem) * items.size()));
        f->items_cap = items.size();
    }
    SBS_CUDA_TRY(cudaMemcpyAsync(f->d_items, items.data(), sizeof(FoamItem) * items.size(), cudaMemcpyHostToDevice,
                                 f->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(f->stream));
    f->nitems = (int)items.size();
    f->rb = rb;
    f->rbmax = rb;
    foam_destroy_graphs(f);
    return SBS_OK;
}

// Enqueues `phases` phases of k steps as one cooperative launch.
int launch_phases(sbs_foam *f, int k, int phases) {
    if (phases <= 0) return SBS_OK;
    const bool mar = f->params.marangoni_enabled != 0;
    const void *fn = foam_fn(k, mar);
    const size_t smem = sizeof(float4) * (size_t)kWarps * (f->rbmax + 2 * k);
    int dev = 0, sms = 148, per_sm = 0;
    SBS_CUDA_TRY(cudaGetDevice(&dev));
    SBS_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    SBS_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kWarps * 32, smem));
    if (per_sm < 1) return set_error(SBS_E_CUDA, "foam kernel does not fit on an SM");
    FoamArgs a{};
    a.bubbles = f->d_bubbles;
    a.items = f->d_items;
    a.nitems = f->nitems;
    a.nphases = phases;
    a.parity0 = f->cur;
    a.rbmax = f->rbmax;
    a.dt = f->params.dt;
    a.crit = f->params.critical_thickness;
    a.bar = f->bar;
    const WaitConfig w = wait_config();
    a.wait_cycles = w.cycles;
    a.extra = (w.stall & SBS_STALL_GRID_BARRIER) ? 1u : 0u;
    void *args[] = {(void *)&a};
    const dim3 grid((unsigned)(per_sm * sms)), block(kWarps * 32);
    SBS_CUDA_TRY(cudaLaunchCooperativeKernel(fn, grid, block, args, smem, f->stream));
    f->cur ^= (phases & 1);
    return SBS_OK;
}

int enqueue_run(sbs_foam *f, uint32_t steps) {
    const int main_phases = (int)(steps / (uint32_t)f->K);
    const int rest = (int)(steps % (uint32_t)f->K);
    int rc = launch_phases(f, f->K, main_phases);
    if (rc) return rc;
    return launch_phases(f, 1, rest);
}

int check_status(sbs_foam *f) {
    unsigned st = 0;
    SBS_CUDA_TRY(cudaMemcpyAsync(&st, f->bar + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, f->stream));
    SBS_CUDA_TRY(cudaStreamSynchronize(f->stream));
    if (st) {
        cudaMemsetAsync(f->bar, 0, 3 * sizeof(unsigned), f->stream);
        cudaStreamSynchronize(f->stream);
        return set_error(SBS_E_TIMEOUT, "foam: a grid-barrier wait timed out");
    }
    return SBS_OK;
}

int run_steps(sbs_foam *f, uint32_t steps) {
    if (steps == 0) return SBS_OK;
    const unsigned epoch = wait_config().epoch;
    if (epoch != f->wait_epoch) {  // the launches carry the wait settings: capture them again
        SBS_CUDA_TRY(cudaStreamSynchronize(f->stream));
        foam_destroy_graphs(f);
        f->wait_epoch = epoch;
    }
    const long long key = ((long long)steps << 1) | f->cur;
    auto it = f->graphs.find(key);
    if (it != f->graphs.end()) {
        SBS_CUDA_TRY(cudaGraphLaunch(it->second, f->stream));
        const int main_phases = (int)(steps / (uint32_t)f->K), rest = (int)(steps % (uint32_t)f->K);
        f->cur ^= ((main_phases + rest) & 1);
        return SBS_OK;
    }
    if (f->graphs_ok) {
        const int cur0 = f->cur;
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(f->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            const int rc = enqueue_run(f, steps);
            const cudaError_t ce = cudaStreamEndCapture(f->stream, &g);
            cudaGraphExec_t exec = nullptr;
            if (rc == SBS_OK && ce == cudaSuccess && cudaGraphInstantiate(&exec, g, 0) == cudaSuccess) {
                cudaGraphDestroy(g);
                f->graphs[((long long)steps << 1) | cur0] = exec;
                SBS_CUDA_TRY(cudaGraphLaunch(exec, f->stream));
                return SBS_OK;
            }
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
        }
        // the driver could not capture the cooperative launch: launch directly from now on
        f->graphs_ok = false;
        f->cur = cur0;
        clear_error();
    }
    return enqueue_run(f, steps);
}

}  // namespace

extern "C" {

int sbs_foam_create(uint32_t nbubbles, const uint32_t *resolution, const float *radius_m,
                    const sbs_drainage_params *params, sbs_foam **out) {
    clear_error();
    SBS_CHECK_ARG(out && resolution && radius_m, "null argument");
    SBS_CHECK_ARG(nbubbles >= 1 && nbubbles <= (1u << 20), "nbubbles must be 1..2^20");
    *out = nullptr;
    for (uint32_t b = 0; b < nbubbles; ++b) {
        SBS_CHECK_ARG(resolution[b] >= 3 && resolution[b] <= 16384, "bubble %u: resolution %u out of range", b,
                      resolution[b]);
        SBS_CHECK_ARG(radius_m[b] > 0.f && std::isfinite(radius_m[b]), "bubble %u: radius must be > 0", b);
    }
    int rc = require_device();
    if (rc) return rc;
    sbs_foam *f = new sbs_foam();
    if (params)
        f->params = *params;
    else
        sbs_drainage_params_default(&f->params);
    f->nb = (int)nbubbles;
    size_t off = 0, roff = 0;
    for (uint32_t b = 0; b < nbubbles; ++b) {
        const int nt = (int)resolution[b], np = 2 * nt;
        f->nt.push_back(nt);
        f->np.push_back(np);
        f->pitch.push_back((np + 31) / 32 * 32);
        f->off.push_back(off);
        f->roff.push_back(roff);
        f->radius.push_back(radius_m[b]);
        off += (size_t)nt * f->pitch.back();
        roff += nt;
    }
    f->field_floats = off;
    auto fail = [&](int code) {
        sbs_foam_destroy(f);
        return code;
    };
    if (cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&f->arena, sizeof(float) * 4 * f->field_floats) != cudaSuccess ||
        cudaMalloc(&f->rows, sizeof(float4) * roff) != cudaSuccess ||
        cudaMalloc(&f->d_bubbles, sizeof(FoamBubble) * nbubbles) != cudaSuccess ||
        cudaMalloc(&f->bar, 4 * sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        return fail(set_error(SBS_E_NOMEM, "foam: device allocation of %.2f GB failed",
                              4.0 * sizeof(float) * f->field_floats / 1e9));
    }
    cudaMemsetAsync(f->bar, 0, 4 * sizeof(unsigned), f->stream);
    std::vector<float4> all_rows(roff);
    std::vector<FoamBubble> desc(nbubbles);
    for (uint32_t b = 0; b < nbubbles; ++b) {
        sbs_drainage_params p = f->params;
        p.bubble_radius = radius_m[b];
        p.grid_height = (uint32_t)f->nt[b];
        p.grid_width = (uint32_t)f->np[b];
        std::vector<float4> rows;
        FoamBubble &d = desc[b];
        wgsl_tables(f->nt[b], f->np[b], p, &rows, nullptr, &d.b, &d.DR2, &d.DsR2, &d.Gt, &d.M);
        std::copy(rows.begin(), rows.end(), all_rows.begin() + f->roff[b]);
        for (int par = 0; par < 2; ++par) {
            d.h[par] = field_ptr(f, 0, par, (int)b);
            d.c[par] = field_ptr(f, 1, par, (int)b);
        }
        d.rows = f->rows + f->roff[b];
        d.nt = f->nt[b];
        d.np = f->np[b];
        d.pitch = f->pitch[b];
    }
    cudaError_t e = cudaMemcpyAsync(f->rows, all_rows.data(), sizeof(float4) * roff, cudaMemcpyHostToDevice, f->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(f->d_bubbles, desc.data(), sizeof(FoamBubble) * nbubbles, cudaMemcpyHostToDevice,
                            f->stream);
    for (int fld = 0; fld < 2 && e == cudaSuccess; ++fld)
        for (int par = 0; par < 2 && e == cudaSuccess; ++par)
            for (int b = 0; b < f->nb && e == cudaSuccess; ++b)
                e = launch_fill(field_ptr(f, fld, par, b), f->pitch[b], f->nt[b], f->np[b], fld == 0 ? 500e-9f : 0.5f,
                                f->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(f->stream);
    if (e != cudaSuccess) return fail(set_error(SBS_E_CUDA, "foam setup: %s", cudaGetErrorString(e)));
    rc = build_items(f, 32);
    if (rc) return fail(rc);
    *out = f;
    return SBS_OK;
}

int sbs_foam_destroy(sbs_foam *f) {
    if (!f) return SBS_OK;
    if (f->stream) cudaStreamSynchronize(f->stream);
    foam_destroy_graphs(f);
    cudaFree(f->arena);
    cudaFree(f->rows);
    cudaFree(f->d_bubbles);
    cudaFree(f->d_items);
    cudaFree(f->bar);
    if (f->stream) cudaStreamDestroy(f->stream);
    delete f;
    return SBS_OK;
}

int sbs_foam_total_cells(const sbs_foam *f, uint64_t *out) {
    SBS_CHECK_ARG(f && out, "null argument");
    uint64_t n = 0;
    for (int b = 0; b < f->nb; ++b) n += (uint64_t)f->nt[b] * f->np[b];
    *out = n;
    return SBS_OK;
}

static int foam_field_io(sbs_foam *f, int which, uint32_t bubble, float *buf, size_t n, int mem, bool in) {
    clear_error();
    SBS_CHECK_ARG(f != nullptr, "handle is null");
    SBS_CHECK_ARG(bubble < (uint32_t)f->nb, "bubble %u out of range", bubble);
    SBS_CHECK_ARG(buf != nullptr, "null buffer");
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "bad mem flag %d", mem);
    const int b = (int)bubble;
    SBS_CHECK_ARG(n == (size_t)f->nt[b] * f->np[b], "bubble %u field has %zu values, expected %d x %d", bubble, n,
                  f->nt[b], f->np[b]);
    const size_t row = f->np[b] * sizeof(float), dp = f->pitch[b] * sizeof(float);
    float *dev = field_ptr(f, which, f->cur, b);
    if (in) {
        const cudaMemcpyKind k = mem == SBS_MEM_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
        SBS_CUDA_TRY(cudaMemcpy2DAsync(dev, dp, buf, row, row, f->nt[b], k, f->stream));
        // the other buffer too: pole rows are never rewritten by the steps
        SBS_CUDA_TRY(cudaMemcpyAsync(field_ptr(f, which, f->cur ^ 1, b), dev, dp * f->nt[b],
                                     cudaMemcpyDeviceToDevice, f->stream));
    } else {
        const cudaMemcpyKind k = mem == SBS_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
        SBS_CUDA_TRY(cudaMemcpy2DAsync(buf, row, dev, dp, row, f->nt[b], k, f->stream));
    }
    SBS_CUDA_TRY(cudaStreamSynchronize(f->stream));
    return SBS_OK;
}

int sbs_foam_set_thickness(sbs_foam *f, uint32_t bubble, const float *src, size_t n, int mem) {
    return foam_field_io(f, 0, bubble, const_cast<float *>(src), n, mem, true);
}
int sbs_foam_get_thickness(sbs_foam *f, uint32_t bubble, float *dst, size_t n, int mem) {
    return foam_field_io(f, 0, bubble, dst, n, mem, false);
}
int sbs_foam_set_concentration(sbs_foam *f, uint32_t bubble, const float *src, size_t n, int mem) {
    return foam_field_io(f, 1, bubble, const_cast<float *>(src), n, mem, true);
}
int sbs_foam_get_concentration(sbs_foam *f, uint32_t bubble, float *dst, size_t n, int mem) {
    return foam_field_io(f, 1, bubble, dst, n, mem, false);
}

int sbs_foam_set_tiles(sbs_foam *f, uint32_t steps_per_phase, uint32_t strip_rows) {
    clear_error();
    SBS_CHECK_ARG(f != nullptr, "handle is null");
    SBS_CHECK_ARG(steps_per_phase == 1 || steps_per_phase == 2 || steps_per_phase == 4, "steps_per_phase must be 1, 2 or 4");
    SBS_CHECK_ARG(strip_rows >= 4 && strip_rows <= 256, "strip_rows must be 4..256");
    f->K = (int)steps_per_phase;
    return build_items(f, (int)strip_rows);
}

int sbs_foam_run(sbs_foam *f, uint32_t steps) {
    clear_error();
    SBS_CHECK_ARG(f != nullptr, "handle is null");
    int rc = run_steps(f, steps);
    if (rc) return rc;
    return check_status(f);
}

int sbs_foam_autotune(sbs_foam *f, uint32_t trial_steps, uint32_t *steps_per_phase, uint32_t *strip_rows) {
    clear_error();
    SBS_CHECK_ARG(f != nullptr, "handle is null");
    if (trial_steps < 4) trial_steps = 4;
    // save the fields, time every candidate tiling on the bubbles themselves, restore
    float *save = nullptr;
    SBS_CUDA_TRY(cudaMalloc(&save, sizeof(float) * 4 * f->field_floats));
    SBS_CUDA_TRY(cudaMemcpyAsync(save, f->arena, sizeof(float) * 4 * f->field_floats, cudaMemcpyDeviceToDevice,
                                 f->stream));
    const int cur0 = f->cur;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    int bestK = f->K, bestRb = f->rb;
    const int Ks[] = {2, 4};
    const int Rbs[] = {8, 16, 32, 64};
    int rc = SBS_OK;
    for (int K : Ks) {
        for (int rb : Rbs) {
            f->K = K;
            if ((rc = build_items(f, rb))) break;
            if ((rc = run_steps(f, trial_steps))) break;  // warm-up (and graph capture)
            cudaEventRecord(e0, f->stream);
            if ((rc = run_steps(f, trial_steps))) break;
            cudaEventRecord(e1, f->stream);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) {
                best = ms;
                bestK = K;
                bestRb = rb;
            }
        }
        if (rc) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaMemcpyAsync(f->arena, save, sizeof(float) * 4 * f->field_floats, cudaMemcpyDeviceToDevice, f->stream);
    cudaStreamSynchronize(f->stream);
    cudaFree(save);
    f->cur = cur0;
    if (rc) return rc;
    f->K = bestK;
    rc = build_items(f, bestRb);
    if (rc) return rc;
    if (steps_per_phase) *steps_per_phase = (uint32_t)bestK;
    if (strip_rows) *strip_rows = (uint32_t)bestRb;
    return check_status(f);
}

int sbs_foam_stream(const sbs_foam *f, void **out) {
    SBS_CHECK_ARG(f && out, "null argument");
    *out = (void *)f->stream;
    return SBS_OK;
}

}  // extern "C"

namespace sbs {
namespace {

// One block per bubble: sum of h sin(theta_i) and of sin(theta_i) over the grid (theta_i =
// i pi / (nt - 1)), in double.
__global__ void __launch_bounds__(256) mean_thickness_kernel(const FoamBubble *bub, int parity, float *out) {
    __shared__ double s_h[8], s_w[8];
    const FoamBubble B = bub[blockIdx.x];
    const float *h = B.h[parity];
    double sh = 0.0, sw = 0.0;
    const double dth = 3.14159265358979323846 / (double)(B.nt - 1);
    for (int r = threadIdx.x >> 5; r < B.nt; r += 8) {
        const double w = sin(r * dth);
        double row = 0.0;
        for (int c = threadIdx.x & 31; c < B.np; c += 32) row += (double)h[(size_t)r * B.pitch + c];
        sh += row * w;
        sw += w * ((B.np - (threadIdx.x & 31) + 31) / 32);
    }
    for (int o = 16; o; o >>= 1) {
        sh += __shfl_xor_sync(0xffffffffu, sh, o);
        sw += __shfl_xor_sync(0xffffffffu, sw, o);
    }
    if ((threadIdx.x & 31) == 0) {
        s_h[threadIdx.x >> 5] = sh;
        s_w[threadIdx.x >> 5] = sw;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int k = 0; k < 8; ++k) {
            a += s_h[k];
            b += s_w[k];
        }
        out[blockIdx.x] = b > 0.0 ? (float)(a / b * 1e9) : 0.0f;
    }
}

}  // namespace

int foam_mean_thickness_nm(sbs_foam *f, float *out, uint32_t cap, uint32_t *nb) {
    *nb = (uint32_t)f->nb;
    if ((uint32_t)f->nb > cap) return SBS_OK;
    mean_thickness_kernel<<<f->nb, 256, 0, f->stream>>>(f->d_bubbles, f->cur, out);
    SBS_CUDA_TRY(cudaGetLastError());
    SBS_CUDA_TRY(cudaStreamSynchronize(f->stream));
    return SBS_OK;
}

}  // namespace sbs
