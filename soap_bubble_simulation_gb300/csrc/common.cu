// Error reporting, version, device probe and configuration defaults.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>

#include <atomic>
#include <map>
#include <mutex>

#include "sbs_internal.h"

namespace sbs {

namespace {
thread_local char g_last_error[1024] = "";
}

int set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return code;
}

void clear_error() { g_last_error[0] = '\0'; }

int require_device() {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return set_error(SBS_E_CUDA, "no usable CUDA device: %s", cudaGetErrorString(e));
    }
    if (n <= 0) return set_error(SBS_E_CUDA, "no CUDA device visible");
    return SBS_OK;
}

cudaError_t scratch_alloc(void **p, size_t bytes, cudaStream_t s) {
    constexpr size_t kPooled = (size_t)64 << 20;
    if (bytes > kPooled) return cudaMallocAsync(p, bytes, s);
    static std::mutex mu;
    static std::map<int, cudaMemPool_t> pools;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    cudaMemPool_t pool = nullptr;
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = pools.find(dev);
        if (it != pools.end()) {
            pool = it->second;
        } else {
            cudaMemPoolProps props{};
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            if ((e = cudaMemPoolCreate(&pool, &props)) != cudaSuccess) return e;
            uint64_t keep = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
            pools[dev] = pool;
        }
    }
    return cudaMallocFromPoolAsync(p, bytes, pool, s);
}

namespace {
std::atomic<long long> g_wait_cycles{kDefaultWaitCycles};
std::atomic<int> g_stall{0};
std::atomic<unsigned> g_wait_epoch{0};
}  // namespace

WaitConfig wait_config() {
    WaitConfig w;
    w.cycles = g_wait_cycles.load();
    w.stall = g_stall.load();
    w.epoch = g_wait_epoch.load();
    return w;
}

}  // namespace sbs

extern "C" {

int sbs_set_wait_limit(uint64_t cycles) {
    sbs::clear_error();
    SBS_CHECK_ARG(cycles >= 1000 && cycles <= (uint64_t)1 << 40, "wait limit must be 1e3 .. 2^40 cycles (got %llu)",
                  (unsigned long long)cycles);
    sbs::g_wait_cycles.store((long long)cycles);
    sbs::g_wait_epoch.fetch_add(1);
    return SBS_OK;
}

int sbs_wait_limit(uint64_t *out) {
    SBS_CHECK_ARG(out != nullptr, "out is null");
    *out = (uint64_t)sbs::g_wait_cycles.load();
    return SBS_OK;
}

int sbs_set_stall_injection(int flags) {
    sbs::clear_error();
    SBS_CHECK_ARG((flags & ~(SBS_STALL_TENSOR_COMMITS | SBS_STALL_GRID_BARRIER)) == 0, "unknown stall flags %d",
                  flags);
    sbs::g_stall.store(flags);
    sbs::g_wait_epoch.fetch_add(1);
    return SBS_OK;
}

const char *sbs_last_error(void) { return sbs::g_last_error; }

const char *sbs_version(void) { return "sbs 0.1.0 (sm_103a)"; }

int sbs_device_count(int *out) {
    SBS_CHECK_ARG(out != nullptr, "out is null");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *out = 0;
        return sbs::set_error(SBS_E_CUDA, "cudaGetDeviceCount: %s", cudaGetErrorString(e));
    }
    *out = n;
    return SBS_OK;
}

// SimulationConfig::default (config.rs:305-316) with BubbleParameters (:26-35),
// FluidParameters (:56-66) and EnvironmentParameters (:93-103) defaults.
int sbs_config_default(sbs_config *out) {
    SBS_CHECK_ARG(out != nullptr, "out is null");
    std::memset(out, 0, sizeof(*out));
    out->diameter = 0.05;
    out->film_thickness_nm = 500.0;
    out->critical_thickness_nm = 10.0;
    out->refractive_index = 1.33;
    out->viscosity = 0.001;
    out->surface_tension = 0.025;
    out->density = 1000.0;
    out->surfactant_diffusion = 1e-9;
    out->surfactant_concentration = 0.5;
    out->gravity = 9.81;
    out->temperature = 293.15;
    out->pressure = 101325.0;
    out->dt = 0.001;
    out->resolution = 128;
    return SBS_OK;
}

// DrainageParams::default (gpu_drainage.rs:46-68).
int sbs_drainage_params_default(sbs_drainage_params *out) {
    SBS_CHECK_ARG(out != nullptr, "out is null");
    std::memset(out, 0, sizeof(*out));
    out->dt = 0.001f;
    out->gravity = 9.81f;
    out->viscosity = 0.001f;
    out->density = 1000.0f;
    out->diffusion_coeff = 1e-9f;
    out->bubble_radius = 0.025f;
    out->critical_thickness = 30e-9f;
    out->grid_width = 128;
    out->grid_height = 64;
    out->marangoni_enabled = 0;
    out->gamma_air = 0.072f;
    out->gamma_reduction = 0.045f;
    out->surfactant_diffusion = 1e-9f;
    out->marangoni_coeff = 0.01f;
    return SBS_OK;
}

}  // extern "C"
