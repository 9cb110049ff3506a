// noalloc.cu -- Gaussian kernel smoothing that allocates no device memory.
//
// seiswg_sim_kernel_smooth smooths the sensitivity kernel a simulation
// handle owns, with a scratch field the handle allocated.  Some callers
// cannot allocate: a host that hands all device memory to its own pool
// allocator, or that calls in from code where a cudaMalloc (which may
// synchronise the whole device) is not allowed.  seiswg_smooth_noalloc takes
// the caller's input and output buffers and keeps its scratch -- the
// x-pass field and the weight and normaliser tables -- in the fixed-size
// arrays below, which every GPU that loads this library holds until the
// process exits (16 MiB + 64 KiB).
//
// The arithmetic is that of the allocating path (fd_aux.cu): weights
// exp(-d^2 / (2 sigma^2)) up to 8 sigma and full-range normalisers, computed
// in double and rounded to float, then the same x and z passes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>

#include "../../include/seiswg.h"
#include "fd_kernels.h"

namespace seiswg {

// The thread's seiswg_last_error() message (capi.cpp).
void set_last_error(const std::string& msg);

namespace {

constexpr int kMaxCells = 1 << 22;   // nx * nz limit: 4,194,304 cells (2048 x 2048)
constexpr int kMaxEdge = 6144;       // nx, nz limit
constexpr int kMaxRadius = 4095;     // weights per table
constexpr int kAuxFloats = (kMaxRadius + 1) + 2 * kMaxEdge;

// Scratch shared by every call on a device.  Host code must not use these
// names as addresses: it asks the runtime for the device address instead.
__device__ __align__(256) float g_tmp[kMaxCells];
__device__ __align__(256) float g_aux[kAuxFloats];

struct DeviceScratch {
  float* tmp = nullptr;
  float* aux = nullptr;
};

std::mutex g_mu;
DeviceScratch g_by_device[64];

// Device addresses of the scratch arrays on the current device (looked up
// once per device, with that device current).
cudaError_t scratch_for_current_device(DeviceScratch* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  DeviceScratch& s = g_by_device[dev];
  if (!s.tmp) {
    void* tmp = nullptr;
    void* aux = nullptr;
    e = cudaGetSymbolAddress(&tmp, g_tmp);
    if (e != cudaSuccess) return e;
    e = cudaGetSymbolAddress(&aux, g_aux);
    if (e != cudaSuccess) return e;
    s.tmp = static_cast<float*>(tmp);
    s.aux = static_cast<float*>(aux);
  }
  *out = s;
  return cudaSuccess;
}

// Weights w[0..radius], then the normalisers gx[0..nx) and gz[0..nz):
// the reference's GSUM factors, sum_q exp(-(i-q)^2 / (2 sigma^2)) over the
// whole axis (fd2d.wgsl:592-609), summed in double in the order q = 0, 1, ...
__global__ void tables_kernel(float* aux, int radius, int nx, int nz, double s2) {
  float* w = aux;
  float* gx = aux + radius + 1;
  float* gz = gx + nx;
  const int n = radius + 1 + nx + nz;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    if (t <= radius) {
      w[t] = float(exp(-double(t) * double(t) / s2));
    } else {
      const int a = t - (radius + 1);
      const bool is_x = a < nx;
      const int i = is_x ? a : a - nx, len = is_x ? nx : nz;
      double s = 0.0;
      for (int q = 0; q < len; ++q) s += exp(-double(i - q) * double(i - q) / s2);
      (is_x ? gx : gz)[i] = float(s);
    }
  }
}

int fail(int code, const char* msg) {
  set_last_error(msg);
  return code;
}

}  // namespace
}  // namespace seiswg

extern "C" int seiswg_smooth_noalloc(const float* in, float* out, int32_t nx, int32_t nz, float sigma,
                                     void* stream) {
  using namespace seiswg;
  set_last_error("");
  if (!in || !out) return fail(SEISWG_EINVAL, "seiswg_smooth_noalloc: null buffer");
  if (nx < 1 || nz < 1 || nx > kMaxEdge || nz > kMaxEdge || long(nx) * long(nz) > kMaxCells)
    return fail(SEISWG_EINVAL,
                "seiswg_smooth_noalloc: grid too large for the fixed scratch (at most 4194304 cells and 6144 "
                "per axis)");
  if (!(sigma > 0.0f)) return fail(SEISWG_EINVAL, "seiswg_smooth_noalloc: sigma must be positive");
  const double r8 = std::ceil(8.0 * double(sigma));
  const int radius = int(std::min(double(std::max(nx, nz) - 1), r8));
  if (radius > kMaxRadius) return fail(SEISWG_EINVAL, "seiswg_smooth_noalloc: sigma above 511 cells");
  DeviceScratch sc;
  cudaError_t e = scratch_for_current_device(&sc);
  if (e != cudaSuccess) return fail(SEISWG_ECUDA, cudaGetErrorString(e));
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const double s2 = 2.0 * double(sigma) * double(sigma);
  const int n = radius + 1 + nx + nz;
  tables_kernel<<<(n + 127) / 128, 128, 0, s>>>(sc.aux, radius, nx, nz, s2);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = launch_smooth_x(sc.tmp, in, sc.aux, radius, nx, nz, nz, s);
  if (e == cudaSuccess)
    e = launch_smooth_z(out, sc.tmp, sc.aux, radius, sc.aux + radius + 1, sc.aux + radius + 1 + nx, nx, nz, nz, s);
  if (e != cudaSuccess) return fail(SEISWG_ECUDA, cudaGetErrorString(e));
  return SEISWG_OK;
}
