// Caustic intensity map from the film thickness (caustics_compute.wgsl:1-126, the compute pass of
// caustics.rs:441-456): per cell, the central-difference gradient, the 5-point Laplacian and the
// determinant of the 9-point Hessian of the thickness field (phi wrapped, theta clamped), turned
// into a focusing x branching x refraction factor, raised to the caustic sharpness and scaled.
//
// One thread per column walks 16 rows with the three rows of the stencil in registers (one new
// row of three loads per cell, two of them L1 hits), so the field is read from HBM once and the
// map written once: 8 bytes per cell, HBM-bound. The arithmetic follows the WGSL in FP32 left to
// right without contraction. pow(x, y) is evaluated as exp2(y log2 x) on the special-function unit,
// as GPU shader compilers evaluate WGSL pow (x >= 0.01 here); it agrees with a correctly rounded
// pow to ~6e-7 relative.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>

#include "caustics.cuh"
#include "sbs_internal.h"

namespace sbs {
namespace {

constexpr int kCols = 128;  // threads (columns) per block
constexpr int kRows = 16;   // rows a thread walks down

// One thread per column, walking kRows rows with the three-row window in registers.
__global__ void __launch_bounds__(kCols) caustics_kernel(sbs_caustic_params p, const float *__restrict__ h,
                                                         size_t pitch, float *__restrict__ out) {
    const int W = (int)p.grid_width, H = (int)p.grid_height;
    const int x = blockIdx.x * kCols + threadIdx.x;
    if (x >= W) return;
    const int xl = x == 0 ? W - 1 : x - 1, xr = x + 1 == W ? 0 : x + 1;  // phi wrapped
    const int y0 = blockIdx.y * kRows, y1 = min(H, y0 + kRows);
    CausticRow a = caustic_load_row(h, pitch, H, y0 - 1, xl, x, xr);
    CausticRow b = caustic_load_row(h, pitch, H, y0, xl, x, xr);
#pragma unroll 4
    for (int y = y0; y < y1; ++y) {
        const CausticRow c = caustic_load_row(h, pitch, H, y + 1, xl, x, xr);
        out[(size_t)y * W + x] =
            caustic_intensity(p.focal_length, p.caustic_intensity, p.caustic_sharpness, p.branch_threshold, a, b, c);
        a = b;
        b = c;
    }
}

}  // namespace
}  // namespace sbs

using namespace sbs;

extern "C" {

int sbs_caustic_params_default(sbs_caustic_params *out) {
    clear_error();
    SBS_CHECK_ARG(out != nullptr, "out is null");
    std::memset(out, 0, sizeof(*out));
    out->grid_width = 128;
    out->grid_height = 64;
    out->refractive_index = 1.33f;
    out->film_thickness_scale = 1e6f;
    out->light_dir_y = -1.0f;
    out->light_intensity = 1.0f;
    out->focal_length = 0.1f;
    out->caustic_intensity = 2.0f;
    out->caustic_sharpness = 1.5f;
    out->branch_threshold = 0.001f;
    out->ground_y = -0.1f;
    out->bubble_radius = 0.025f;
    return SBS_OK;
}

int sbs_caustics(const sbs_caustic_params *p, const float *thickness, size_t pitch, float *caustic_map, int mem,
                 void *stream) {
    clear_error();
    SBS_CHECK_ARG(p != nullptr, "null parameters");
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "bad mem flag %d", mem);
    SBS_CHECK_ARG(p->grid_width >= 1 && p->grid_height >= 1 && p->grid_width <= (1u << 20) &&
                      p->grid_height <= (1u << 20),
                  "grid out of range");
    SBS_CHECK_ARG(pitch >= p->grid_width, "pitch (%zu) below grid_width (%u)", pitch, p->grid_width);
    SBS_CHECK_ARG(thickness != nullptr && caustic_map != nullptr, "null pointer");
    int rc = require_device();
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t W = p->grid_width, H = p->grid_height;
    const float *din = thickness;
    float *dout = caustic_map;
    char *base = nullptr;
    if (mem == SBS_MEM_HOST) {
        const size_t in_b = sizeof(float) * pitch * H, out_b = sizeof(float) * W * H;
        SBS_CUDA_TRY(scratch_alloc((void **)&base, in_b + out_b + 256, s));
        cudaError_t e = cudaMemcpyAsync(base, thickness, in_b, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) {
            cudaFreeAsync(base, s);
            return set_error(SBS_E_CUDA, "caustics: upload failed: %s", cudaGetErrorString(e));
        }
        din = (const float *)base;
        dout = (float *)(base + ((in_b + 255) / 256) * 256);
    }
    const dim3 grid((unsigned)((W + kCols - 1) / kCols), (unsigned)((H + kRows - 1) / kRows));
    caustics_kernel<<<grid, kCols, 0, s>>>(*p, din, pitch, dout);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && mem == SBS_MEM_HOST)
        e = cudaMemcpyAsync(caustic_map, dout, sizeof(float) * W * H, cudaMemcpyDeviceToHost, s);
    if (base) cudaFreeAsync(base, s);
    if (e == cudaSuccess && mem == SBS_MEM_HOST) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(SBS_E_CUDA, "caustics: %s", cudaGetErrorString(e));
    return SBS_OK;
}

int sbs_gpu_drainage_caustics(sbs_drainage *h, const sbs_caustic_params *p, int which, float *caustic_map, int mem) {
    clear_error();
    SBS_CHECK_ARG(h != nullptr && p != nullptr && caustic_map != nullptr, "null argument");
    SBS_CHECK_ARG(mem == SBS_MEM_HOST || mem == SBS_MEM_DEVICE, "bad mem flag %d", mem);
    const float *field = nullptr;
    size_t pitch = 0;
    int rc = sbs_drainage_thickness_device(h, which, &field, &pitch);
    if (rc) return rc;
    sbs_drainage_params dp{};
    if ((rc = sbs_gpu_drainage_params(h, &dp))) return rc;
    SBS_CHECK_ARG(p->grid_width == dp.grid_width && p->grid_height == dp.grid_height,
                  "caustic grid %ux%u differs from the handle's %ux%u", p->grid_width, p->grid_height, dp.grid_width,
                  dp.grid_height);
    void *stream = nullptr;
    if ((rc = sbs_drainage_stream(h, &stream))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (mem == SBS_MEM_DEVICE) return sbs_caustics(p, field, pitch, caustic_map, SBS_MEM_DEVICE, stream);
    float *dout = nullptr;
    const size_t bytes = sizeof(float) * p->grid_width * p->grid_height;
    SBS_CUDA_TRY(scratch_alloc((void **)&dout, bytes, s));
    rc = sbs_caustics(p, field, pitch, dout, SBS_MEM_DEVICE, stream);
    cudaError_t e = rc ? cudaSuccess : cudaMemcpyAsync(caustic_map, dout, bytes, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(dout, s);
    if (rc) return rc;
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return set_error(SBS_E_CUDA, "caustics: %s", cudaGetErrorString(e));
    return SBS_OK;
}

}  // extern "C"
