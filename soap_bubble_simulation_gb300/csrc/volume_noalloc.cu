// Film volume of a device field without allocating memory.
//
// Same reduction as sbs_film_volume_device (per-row FP64 weights, per-block partial sums, a
// last-block finish), but the scratch it needs lives in one fixed array in device memory that the
// library brings with it, so the call never asks CUDA for memory. This serves callers that must
// not allocate while they run, for example an engine that has handed the GPU's memory to its own
// pool and budgets it per frame, or a real-time loop that cannot take the stall an allocation can
// cause.
#include <cuda_runtime.h>

#include "sbs_internal.h"

namespace sbs {
namespace {

constexpr int kNoAllocMaxTheta = 16384;  // rows whose weights fit in the array
constexpr int kNoAllocMaxBlocks = 1024;  // the reduction launches at most this many blocks
// layout in doubles: weights | 3 partials per block | result (3) | arrival counter
constexpr size_t kOffPartials = kNoAllocMaxTheta;
constexpr size_t kOffResult = kOffPartials + 3 * kNoAllocMaxBlocks;
constexpr size_t kOffCounter = kOffResult + 3;
constexpr size_t kScratchDoubles = kOffCounter + 1;  // 19,460 doubles = 155,680 bytes

// The fixed scratch. In host code this name is only a stand-in for the device array: host code
// must use the address cudaGetSymbolAddress returns for it (see scratch_on_current_device).
static __device__ __align__(256) double g_volume_scratch[kScratchDoubles];

// Device address of the scratch array in the current device's context. It is looked up on every
// call (a lookup allocates nothing and costs ~a microsecond): a cached address would outlive a
// cudaDeviceReset, after which the library's module, and the array with it, is loaded again at a
// new address. The first lookup on a device loads the module.
int scratch_on_current_device(double **out) {
    double *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress((void **)&p, g_volume_scratch);
    if (e != cudaSuccess)
        return set_error(SBS_E_CUDA, "cudaGetSymbolAddress(volume scratch): %s", cudaGetErrorString(e));
    *out = p;
    return SBS_OK;
}

__global__ void noalloc_weights_kernel(double *w, int nt, int np, double radius) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt) return;
    const double PI = 3.14159265358979323846;
    const double dth = PI / (double)(nt - 1), dph = 2.0 * PI / (double)np;
    w[i] = radius * radius * sin((double)i * dth) * dth * dph;
}

}  // namespace
}  // namespace sbs

using namespace sbs;

extern "C" int sbs_film_volume_device_noalloc(const float *h, uint32_t num_theta, uint32_t num_phi, size_t pitch,
                                              double radius, double *out, void *stream) {
    clear_error();
    SBS_CHECK_ARG(h != nullptr && out != nullptr, "null pointer");
    SBS_CHECK_ARG(num_theta >= 2 && num_phi >= 1, "grid must be at least 2 x 1");
    SBS_CHECK_ARG(num_theta <= (uint32_t)kNoAllocMaxTheta,
                  "num_theta %u exceeds the no-allocation limit of %d rows", num_theta, kNoAllocMaxTheta);
    SBS_CHECK_ARG(pitch >= num_phi, "pitch %zu smaller than num_phi %u", pitch, num_phi);
    int rc = require_device();
    if (rc) return rc;
    double *scratch = nullptr;
    rc = scratch_on_current_device(&scratch);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const int nt = (int)num_theta, np = (int)num_phi;
    double *w = scratch;
    double *partials = scratch + kOffPartials;
    ReduceOut *res = reinterpret_cast<ReduceOut *>(scratch + kOffResult);
    unsigned *counter = reinterpret_cast<unsigned *>(scratch + kOffCounter);
    // the array keeps the previous call's contents: the arrival counter must start at zero
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) {
        noalloc_weights_kernel<<<(nt + 127) / 128, 128, 0, s>>>(w, nt, np, radius);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = launch_field_reduce(h, nullptr, nt, np, pitch, w, partials, counter, res, s);
    ReduceOut host{};
    if (e == cudaSuccess) e = cudaMemcpyAsync(&host, res, sizeof(ReduceOut), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(SBS_E_CUDA, "film volume (no allocation): %s", cudaGetErrorString(e));
    *out = host.volume;
    return SBS_OK;
}
