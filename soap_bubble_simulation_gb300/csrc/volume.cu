// Film volume of a bare device field: V = sum_ij h_ij R^2 sin(theta_i) dtheta dphi with FP64
// accumulation. The reference has no conservation check; this is the stateless form of the check
// the drainage handle fuses into its step kernel.
#include <cuda_runtime.h>

#include "sbs_internal.h"

namespace sbs {
namespace {

__global__ void volume_weights_kernel(double *w, int nt, int np, double radius) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt) return;
    const double PI = 3.14159265358979323846;
    const double dth = PI / (double)(nt - 1), dph = 2.0 * PI / (double)np;
    w[i] = radius * radius * sin((double)i * dth) * dth * dph;
}

}  // namespace
}  // namespace sbs

using namespace sbs;

extern "C" int sbs_film_volume_device(const float *h, uint32_t num_theta, uint32_t num_phi, size_t pitch,
                                      double radius, double *out, void *stream) {
    clear_error();
    SBS_CHECK_ARG(h != nullptr && out != nullptr, "null pointer");
    SBS_CHECK_ARG(num_theta >= 2 && num_phi >= 1, "grid must be at least 2 x 1");
    SBS_CHECK_ARG(pitch >= num_phi, "pitch %zu smaller than num_phi %u", pitch, num_phi);
    int rc = require_device();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const int nt = (int)num_theta, np = (int)num_phi;
    const int nb = reduce_partials_count(nt, np);
    // scratch: weights, per-block partials, arrival counter, result
    const size_t bytes = sizeof(double) * (size_t)nt + sizeof(double) * 3 * nb + sizeof(ReduceOut) + 16;
    char *scratch = nullptr;
    SBS_CUDA_TRY(scratch_alloc((void **)&scratch, bytes, s));
    double *w = (double *)scratch;
    double *partials = w + nt;
    ReduceOut *res = (ReduceOut *)(partials + 3 * nb);
    unsigned *counter = (unsigned *)(res + 1);
    cudaError_t e = cudaMemsetAsync(counter, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) {
        volume_weights_kernel<<<(nt + 127) / 128, 128, 0, s>>>(w, nt, np, radius);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = launch_field_reduce(h, nullptr, nt, np, pitch, w, partials, counter, res, s);
    ReduceOut host{};
    if (e == cudaSuccess) e = cudaMemcpyAsync(&host, res, sizeof(ReduceOut), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(scratch, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(SBS_E_CUDA, "film volume: %s", cudaGetErrorString(e));
    *out = host.volume;
    return SBS_OK;
}
