// fd_aux.cu -- the non-step kernels: model set-up, the stability and
// finite-value guards, trace assembly, the reference adjoint's imaging
// condition and Gaussian kernel smoothing.
#include "fd_kernels.h"

namespace seiswg {

namespace {

__global__ void fill_rows_kernel(float* f, int rows_lo, int rows_hi, int ld, float value) {
  long n = long(rows_hi - rows_lo) * ld;
  for (long t = blockIdx.x * long(blockDim.x) + threadIdx.x; t < n; t += long(gridDim.x) * blockDim.x)
    f[long(rows_lo) * ld + t] = value;
}

// fd2d.wgsl:188-201: mu = rho*vs*vs; lambda = rho*(vp*vp - 2*vs*vs) if vp > vs else 0.
__global__ void vps2lm_kernel(float* lam_vp, float* mu_vs, const float* rho, int nx, int nz, int ld) {
  long n = long(nx) * nz;
  for (long t = blockIdx.x * long(blockDim.x) + threadIdx.x; t < n; t += long(gridDim.x) * blockDim.x) {
    long k = (t / nz) * ld + (t % nz);
    float vp = lam_vp[k], vs = mu_vs[k], r = rho[k];
    mu_vs[k] = r * vs * vs;
    lam_vp[k] = (vp > vs) ? r * (vp * vp - 2.0f * vs * vs) : 0.0f;
  }
}

__global__ void add_fields_kernel(float* out, const float* a, const float* b, int nx, int nz, int ld) {
  long n = long(nx) * nz;
  for (long t = blockIdx.x * long(blockDim.x) + threadIdx.x; t < n; t += long(gridDim.x) * blockDim.x) {
    long k = (t / nz) * ld + (t % nz);
    out[k] = a[k] + b[k];
  }
}

__global__ void reciprocal_kernel(float* f, int nx, int nz, int ld) {
  long n = long(nx) * nz;
  for (long t = blockIdx.x * long(blockDim.x) + threadIdx.x; t < n; t += long(gridDim.x) * blockDim.x) {
    long k = (t / nz) * ld + (t % nz);
    f[k] = 1.0f / f[k];
  }
}

// out = in * factor over n consecutive floats (whole padded fields).
__global__ void scale_kernel(float* out, const float* in, long n, float factor) {
  for (long t = blockIdx.x * long(blockDim.x) + threadIdx.x; t < n; t += long(gridDim.x) * blockDim.x)
    out[t] = in[t] * factor;
}

// Largest squared wave speeds over the interior, as the bits of non-negative
// floats (which order like unsigned integers): out[0] P (PSV, (lambda +
// 2 mu) b) or S (SH, mu b), out[1] the spin's rotation rate 4 nu / J,
// out[2] its couple-wave speed (mu_c + nu_c) / J.  A non-finite or negative
// value sets out[3].
__global__ void speed_kernel(const float* lam, const float* mu, const float* b, const float* nu, const float* jinv,
                             const float* mc, int psv, int nx, int nz, int ld, unsigned* out) {
  long n = long(nx) * nz;
  float m0 = 0.0f, m1 = 0.0f, m2 = 0.0f;
  unsigned bad = 0;
  for (long t = blockIdx.x * long(blockDim.x) + threadIdx.x; t < n; t += long(gridDim.x) * blockDim.x) {
    const long k = (t / nz) * ld + (t % nz);
    const float c2 = (psv ? lam[k] + 2.0f * mu[k] : mu[k]) * b[k];
    float w2 = 0.0f, q2 = 0.0f;
    if (jinv) {
      w2 = 4.0f * nu[k] * jinv[k];
      q2 = mc[k] * jinv[k];
    }
    if (!(c2 >= 0.0f && c2 < INFINITY && w2 >= 0.0f && w2 < INFINITY && q2 >= 0.0f && q2 < INFINITY)) bad = 1;
    else {
      m0 = fmaxf(m0, c2);
      m1 = fmaxf(m1, w2);
      m2 = fmaxf(m2, q2);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    m0 = fmaxf(m0, __shfl_xor_sync(0xffffffffu, m0, o));
    m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    m2 = fmaxf(m2, __shfl_xor_sync(0xffffffffu, m2, o));
    bad |= __shfl_xor_sync(0xffffffffu, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&out[0], __float_as_uint(m0));
    atomicMax(&out[1], __float_as_uint(m1));
    atomicMax(&out[2], __float_as_uint(m2));
    if (bad) atomicOr(&out[3], 1u);
  }
}

// Sets `bit` in *err when an element of rows x cols (row pitch ld) is not
// finite.
__global__ void finite_kernel(const float* f, long rows, int cols, long ld, int* err, int bit) {
  const long n = rows * cols;
  unsigned bad = 0;
  for (long t = blockIdx.x * long(blockDim.x) + threadIdx.x; t < n; t += long(gridDim.x) * blockDim.x) {
    const float v = f[(t / cols) * ld + (t % cols)];
    if (!(fabsf(v) < INFINITY)) bad = 1;
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(err, bit);
}

__device__ __forceinline__ float fd4d(float a, float b, float c, float d, float den) {
  return (9.0f * (c - b) - (d - a)) / den;
}

__global__ void assemble_traces_kernel(const TraceSpec t) {
  long n = long(t.nrec) * t.nt;
  const long nobs = n;
  for (long q = blockIdx.x * long(blockDim.x) + threadIdx.x; q < n; q += long(gridDim.x) * blockDim.x) {
    const int r = int(q / t.nt), it = int(q % t.nt);
    auto H = [&](int p) { return p >= 0 ? t.hist[long(p) * t.nt + it] : 0.0f; };
    const int* p = t.idx + 12 * r;
    if (t.sh) t.obs[1 * nobs + q] = H(p[0]);  // save_obs_y_sh
    if (t.psv) {
      t.obs[0 * nobs + q] = H(p[1]);          // save_obs_x
      t.obs[2 * nobs + q] = H(p[2]);          // save_obs_z
      if (t.spin) {                           // compute_du_grad + save_obs_ry
        const int i = t.rec_ij[2 * r], j = t.rec_ij[2 * r + 1];
        const int* c = p + 4;
        float duzdx = (i >= 1 && i < t.nx - 2) ? fd4d(H(c[0]), H(c[1]), H(c[2]), H(c[3]), t.den_x) : 0.0f;
        float duxdz = (j >= 1 && j < t.nz - 2) ? fd4d(H(c[4]), H(c[5]), H(c[6]), H(c[7]), t.den_z) : 0.0f;
        float u = H(p[3]);
        float curl = -(duzdx - duxdz);
        t.obs[1 * nobs + q] = u;
        t.obs[3 * nobs + q] = u - 0.5f * curl;
        t.obs[4 * nobs + q] = curl;
      }
    }
  }
}

__global__ void imaging_muy_kernel(float* kmu, const float* vy, const float* fw, int nx, int nz, int ld,
                                   float den_x, float den_z, float ndt) {
  long n = long(nx) * nz;
  for (long t = blockIdx.x * long(blockDim.x) + threadIdx.x; t < n; t += long(gridDim.x) * blockDim.x) {
    const int i = int(t / nz), j = int(t % nz);
    const long k = long(i) * ld + j;
    const bool xf = (i >= 1 && i < nx - 2), zf = (j >= 1 && j < nz - 2);
    float ax = xf ? fd4d(vy[k - ld], vy[k], vy[k + ld], vy[k + 2 * ld], den_x) : 0.0f;
    float az = zf ? fd4d(vy[k - 1], vy[k], vy[k + 1], vy[k + 2], den_z) : 0.0f;
    float bx = xf ? fd4d(fw[k - ld], fw[k], fw[k + ld], fw[k + 2 * ld], den_x) : 0.0f;
    float bz = zf ? fd4d(fw[k - 1], fw[k], fw[k + 1], fw[k + 2], den_z) : 0.0f;
    kmu[k] = kmu[k] + (ax * bx + az * bz) * ndt;
  }
}

// x pass: each thread owns a column j and a row i; reads are coalesced along j.
__global__ void smooth_x_kernel(float* tmp, const float* f, const float* w, int radius, int nx, int nz, int ld) {
  long n = long(nx) * nz;
  for (long t = blockIdx.x * long(blockDim.x) + threadIdx.x; t < n; t += long(gridDim.x) * blockDim.x) {
    const int i = int(t / nz), j = int(t % nz);
    const int lo = max(0, i - radius), hi = min(nx - 1, i + radius);
    float s = 0.0f;
    for (int q = lo; q <= hi; ++q) s = s + w[abs(i - q)] * f[long(q) * ld + j];
    tmp[long(i) * ld + j] = s;
  }
}

__global__ void smooth_z_kernel(float* f, const float* tmp, const float* w, int radius, const float* gx,
                                const float* gz, int nx, int nz, int ld) {
  long n = long(nx) * nz;
  for (long t = blockIdx.x * long(blockDim.x) + threadIdx.x; t < n; t += long(gridDim.x) * blockDim.x) {
    const int i = int(t / nz), j = int(t % nz);
    const int lo = max(0, j - radius), hi = min(nz - 1, j + radius);
    const float* row = tmp + long(i) * ld;
    float s = 0.0f;
    for (int q = lo; q <= hi; ++q) s = s + w[abs(j - q)] * row[q];
    const float g = gx[i] * gz[j];
    f[long(i) * ld + j] = (g > 1e-30f) ? s / g : 0.0f;
  }
}

inline unsigned grid_for(long n, int threads = 256) {
  long b = (n + threads - 1) / threads;
  return unsigned(b < 1 ? 1 : (b > 152L * 32 ? 152L * 32 : b));
}

}  // namespace

cudaError_t launch_fill_rows(float* f, int rows_lo, int rows_hi, int ld, float value, cudaStream_t s) {
  fill_rows_kernel<<<grid_for(long(rows_hi - rows_lo) * ld), 256, 0, s>>>(f, rows_lo, rows_hi, ld, value);
  return cudaGetLastError();
}

cudaError_t launch_vps2lm(float* lam_vp, float* mu_vs, const float* rho, int nx, int nz, int ld, cudaStream_t s) {
  vps2lm_kernel<<<grid_for(long(nx) * nz), 256, 0, s>>>(lam_vp, mu_vs, rho, nx, nz, ld);
  return cudaGetLastError();
}

cudaError_t launch_add_fields(float* out, const float* a, const float* b, int nx, int nz, int ld,
                              cudaStream_t s) {
  add_fields_kernel<<<grid_for(long(nx) * nz), 256, 0, s>>>(out, a, b, nx, nz, ld);
  return cudaGetLastError();
}

cudaError_t launch_reciprocal(float* f, int nx, int nz, int ld, cudaStream_t s) {
  reciprocal_kernel<<<grid_for(long(nx) * nz), 256, 0, s>>>(f, nx, nz, ld);
  return cudaGetLastError();
}

cudaError_t launch_scale(float* out, const float* in, long n, float factor, cudaStream_t s) {
  scale_kernel<<<grid_for(n), 256, 0, s>>>(out, in, n, factor);
  return cudaGetLastError();
}

cudaError_t launch_max_speeds(const float* lam, const float* mu, const float* b, const float* nu, const float* jinv,
                              const float* mc, bool psv, int nx, int nz, int ld, unsigned* out, cudaStream_t s) {
  speed_kernel<<<grid_for(long(nx) * nz), 256, 0, s>>>(lam, mu, b, nu, jinv, mc, psv ? 1 : 0, nx, nz, ld, out);
  return cudaGetLastError();
}

cudaError_t launch_check_finite(const float* f, long rows, int cols, long ld, int* err, int bit, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return cudaSuccess;
  finite_kernel<<<grid_for(rows * cols), 256, 0, s>>>(f, rows, cols, ld, err, bit);
  return cudaGetLastError();
}

cudaError_t launch_assemble_traces(const TraceSpec& t, cudaStream_t s) {
  if (t.nrec == 0 || t.nt == 0) return cudaSuccess;
  assemble_traces_kernel<<<grid_for(long(t.nrec) * t.nt), 256, 0, s>>>(t);
  return cudaGetLastError();
}

cudaError_t launch_imaging_muy(float* kmu, const float* vy_adj, const float* vy_fw, int nx, int nz, int ld,
                               float den_x, float den_z, float ndt, cudaStream_t s) {
  imaging_muy_kernel<<<grid_for(long(nx) * nz), 256, 0, s>>>(kmu, vy_adj, vy_fw, nx, nz, ld, den_x, den_z, ndt);
  return cudaGetLastError();
}

cudaError_t launch_smooth_x(float* tmp, const float* f, const float* w, int radius, int nx, int nz, int ld,
                            cudaStream_t s) {
  smooth_x_kernel<<<grid_for(long(nx) * nz), 256, 0, s>>>(tmp, f, w, radius, nx, nz, ld);
  return cudaGetLastError();
}

cudaError_t launch_smooth_z(float* f, const float* tmp, const float* w, int radius, const float* gsum_x,
                            const float* gsum_z, int nx, int nz, int ld, cudaStream_t s) {
  smooth_z_kernel<<<grid_for(long(nx) * nz), 256, 0, s>>>(f, tmp, w, radius, gsum_x, gsum_z, nx, nz, ld);
  return cudaGetLastError();
}

}  // namespace seiswg
