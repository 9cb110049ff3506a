// fd_fma.cuh -- pieces of the kernels built with multiply-add contraction
// (fd_step2.cu, fd_spin.cu): fourth-order differences before their 1/(8 h)
// factor, which those kernels scale by dt/(8 h) so that dt is folded into the
// derivative, and source injection on that dt scale.
#pragma once

#include "fd_march.cuh"

namespace seiswg {
namespace {

// The fourth-order difference 9 (c - b) - (d - a) before its factor
// (fd2d.wgsl:156); the caller multiplies it by dt/(8 h), folding the time
// step into the derivative (one multiply fewer per update than dt * (...)).
__device__ __forceinline__ float d4(float a, float b, float c, float d) { return fmaf(9.0f, c - b, a - d); }

// Differences along the rows (four row registers) and along the columns
// (neighbour lanes' elements by shuffles), backward- and forward-staggered.
__device__ __forceinline__ f4 d4_rows(const f4& r0, const f4& r1, const f4& r2, const f4& r3) {
  f4 o;
#pragma unroll
  for (int e = 0; e < 4; ++e) o.v[e] = d4(r0.v[e], r1.v[e], r2.v[e], r3.v[e]);
  return o;
}
__device__ __forceinline__ f4 d4_cols_back(const f4& m) {
  const float pz = __shfl_up_sync(kFull, m.v[2], 1);
  const float pw = __shfl_up_sync(kFull, m.v[3], 1);
  const float nx = __shfl_down_sync(kFull, m.v[0], 1);
  f4 o;
  o.v[0] = d4(pz, pw, m.v[0], m.v[1]);
  o.v[1] = d4(pw, m.v[0], m.v[1], m.v[2]);
  o.v[2] = d4(m.v[0], m.v[1], m.v[2], m.v[3]);
  o.v[3] = d4(m.v[1], m.v[2], m.v[3], nx);
  return o;
}
__device__ __forceinline__ f4 d4_cols_fwd(const f4& m) {
  const float pw = __shfl_up_sync(kFull, m.v[3], 1);
  const float n0 = __shfl_down_sync(kFull, m.v[0], 1);
  const float n1 = __shfl_down_sync(kFull, m.v[1], 1);
  f4 o;
  o.v[0] = d4(pw, m.v[0], m.v[1], m.v[2]);
  o.v[1] = d4(m.v[0], m.v[1], m.v[2], m.v[3]);
  o.v[2] = d4(m.v[1], m.v[2], m.v[3], n0);
  o.v[3] = d4(m.v[2], m.v[3], n0, n1);
  return o;
}

// Sources of row i (stf_dsxz, fd2d.wgsl:350-351) added to dt times the
// divergence: dt * f.
__device__ __forceinline__ void inject_dt(const InjectList& inj, int i, int c0, Cursor& cur, float dt, f4& dsx,
                                          f4& dsz) {
  const f4 z4 = {{0.0f, 0.0f, 0.0f, 0.0f}};
  f4 fx = z4, fz = z4;
  inject_at<true, false, true>(inj, i, c0, cur, fx, fx, fz);
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    dsx.v[e] = fmaf(dt, fx.v[e], dsx.v[e]);
    dsz.v[e] = fmaf(dt, fz.v[e], dsz.v[e]);
  }
}

}  // namespace
}  // namespace seiswg
