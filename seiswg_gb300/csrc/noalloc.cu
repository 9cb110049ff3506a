// noalloc.cu -- Gaussian kernel smoothing that allocates no device memory.
//
// seiswg_sim_kernel_smooth smooths the sensitivity kernel a simulation
// handle owns, with a scratch field the handle allocated.  Some callers
// cannot allocate: a host that hands all device memory to its own pool
// allocator, or that calls in from code where a cudaMalloc (which may
// synchronise the whole device) is not allowed.  seiswg_smooth_noalloc takes
// the caller's input and output buffers and keeps its scratch -- the
// x-pass field, the weight and normaliser tables and the prefix sums they
// come from -- in the fixed-size arrays below, which every GPU that loads this
// library holds until the process exits (16 MiB + 112 KiB).
//
// The arithmetic is that of the allocating path (fd_aux.cu): weights
// exp(-d^2 / (2 sigma^2)) up to 8 sigma and full-range normalisers, computed
// in double and rounded to float, then the same x and z passes.  The
// normalisers are summed in another order than the allocating path's (which
// adds the terms of each one in turn on the host): a double prefix sum of the
// weights over the longer axis gives every normaliser with one addition, so a
// call costs max(nx, nz) exponentials instead of nx^2 + nz^2.  The two
// double sums differ by rounding (about 1e-12 relative), below the float the
// result is rounded to.
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
constexpr int kTableThreads = 1024;  // one block builds the tables

// Scratch shared by every call on a device.  Host code must not use these
// names as addresses: it asks the runtime for the device address instead.
__device__ __align__(256) float g_tmp[kMaxCells];
__device__ __align__(256) float g_aux[kAuxFloats];
__device__ __align__(256) double g_prefix[kMaxEdge];

struct DeviceScratch {
  float* tmp = nullptr;
  float* aux = nullptr;
  double* prefix = nullptr;
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
    void* prefix = nullptr;
    e = cudaGetSymbolAddress(&tmp, g_tmp);
    if (e != cudaSuccess) return e;
    e = cudaGetSymbolAddress(&aux, g_aux);
    if (e != cudaSuccess) return e;
    e = cudaGetSymbolAddress(&prefix, g_prefix);
    if (e != cudaSuccess) return e;
    s.tmp = static_cast<float*>(tmp);
    s.aux = static_cast<float*>(aux);
    s.prefix = static_cast<double*>(prefix);
  }
  *out = s;
  return cudaSuccess;
}

// One block of kTableThreads threads.  Weights w[0..radius], then the
// normalisers gx[0..nx) and gz[0..nz): the reference's GSUM factors,
// g(i) = sum_{q < n} exp(-(i-q)^2 / (2 sigma^2)) over the whole axis
// (fd2d.wgsl:592-609), as W(i) + W(n-1-i) - 1 with W(m) = sum_{d <= m}
// exp(-d^2 / (2 sigma^2)) in double: prefix[d] = W(d) for d < m = max(nx, nz).
__global__ void __launch_bounds__(kTableThreads) tables_kernel(float* aux, double* prefix, int radius, int nx,
                                                               int nz, double s2) {
  __shared__ double part[kTableThreads];
  const int m = max(nx, nz);
  const int t = threadIdx.x;
  const int per = (m + kTableThreads - 1) / kTableThreads;  // <= 6 at the largest axis
  const int lo = min(m, t * per), hi = min(m, lo + per);
  // each thread: the terms of its run d in [lo, hi), their running sum
  double acc = 0.0;
  for (int d = lo; d < hi; ++d) {
    acc += exp(-double(d) * double(d) / s2);
    prefix[d] = acc;
  }
  part[t] = acc;
  __syncthreads();
  // inclusive scan of the run totals (Hillis-Steele, in shared memory)
  for (int off = 1; off < kTableThreads; off <<= 1) {
    const double v = t >= off ? part[t - off] : 0.0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  const double before = t > 0 ? part[t - 1] : 0.0;
  for (int d = lo; d < hi; ++d) prefix[d] += before;
  __syncthreads();
  float* w = aux;
  float* gx = aux + radius + 1;
  float* gz = gx + nx;
  for (int q = t; q <= radius; q += kTableThreads) w[q] = float(exp(-double(q) * double(q) / s2));
  for (int i = t; i < nx; i += kTableThreads) gx[i] = float(prefix[i] + prefix[nx - 1 - i] - 1.0);
  for (int j = t; j < nz; j += kTableThreads) gz[j] = float(prefix[j] + prefix[nz - 1 - j] - 1.0);
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
  tables_kernel<<<1, kTableThreads, 0, s>>>(sc.aux, sc.prefix, radius, nx, nz, s2);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = launch_smooth_x(sc.tmp, in, sc.aux, radius, nx, nz, nz, s);
  if (e == cudaSuccess)
    e = launch_smooth_z(out, sc.tmp, sc.aux, radius, sc.aux + radius + 1, sc.aux + radius + 1 + nx, nx, nz, nz, s);
  if (e != cudaSuccess) return fail(SEISWG_ECUDA, cudaGetErrorString(e));
  return SEISWG_OK;
}
