// fd_common.cuh -- device-side building blocks shared by the seiswg sm_103a
// stencil kernels (layout and work decomposition: fd_types.h).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "fd_types.h"

namespace seiswg {

// Reference difference formula (fd2d.wgsl:155-156): with the four samples
// a,b,c,d at offsets (-2,-1,0,+1) for the backward form or (-1,0,+1,+2) for
// the forward form, (9*(c-b) - (d-a)) / (8*d).  The division is a multiply by
// the rounded reciprocal r = 1/(8*d) (at most one ulp from the quotient; no
// division slow path for the tiny values ahead of a wavefront).
__device__ __forceinline__ float fd4(float a, float b, float c, float d, float r) {
  return (9.0f * (c - b) - (d - a)) * r;
}

struct f4 {
  float v[4];
};

// Loads of state rows and of values other launches write.  In the batch's
// queue kernel (fd_queue.cu, which defines SEISWG_COHERENT_LOADS) other warps
// of the same launch write them, so they go through L2 (ld.global.cg); the
// step kernels read them through the read-only path (ld.global.nc), which
// is valid only for data no thread of the launch writes.
namespace {
#ifdef SEISWG_COHERENT_LOADS
__device__ __forceinline__ f4 ld4(const float* p) {
  const float4 t = __ldcg(reinterpret_cast<const float4*>(p));
#else
__device__ __forceinline__ f4 ld4(const float* __restrict__ p) {
  const float4 t = __ldg(reinterpret_cast<const float4*>(p));
#endif
  f4 r;
  r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
  return r;
}

__device__ __forceinline__ float ld1(const float* p) {
#ifdef SEISWG_COHERENT_LOADS
  return __ldcg(p);
#else
  return __ldg(p);
#endif
}
}  // namespace

__device__ __forceinline__ void st4(float* p, const f4& a) {
  *reinterpret_cast<float4*>(p) = make_float4(a.v[0], a.v[1], a.v[2], a.v[3]);
}

// Store the owned columns of one lane: the full float4 when all four columns
// are owned, element-wise otherwise.
__device__ __forceinline__ void st4_masked(float* p, const f4& a, int own_mask) {
  if (own_mask == 0xF) {
    st4(p, a);
  } else if (own_mask) {
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (own_mask & (1 << e)) p[e] = a.v[e];
  }
}

// z-backward difference of a lane's float4 (columns c0..c0+3): samples
// c-2..c+1; c0-2, c0-1 come from the previous lane, c0+4 from the next.
__device__ __forceinline__ f4 dz_back(const f4& m, float den, int zmask) {
  float pz = __shfl_up_sync(kFull, m.v[2], 1);
  float pw = __shfl_up_sync(kFull, m.v[3], 1);
  float nx = __shfl_down_sync(kFull, m.v[0], 1);
  f4 r;
  r.v[0] = (zmask & 1) ? fd4(pz, pw, m.v[0], m.v[1], den) : 0.0f;
  r.v[1] = (zmask & 2) ? fd4(pw, m.v[0], m.v[1], m.v[2], den) : 0.0f;
  r.v[2] = (zmask & 4) ? fd4(m.v[0], m.v[1], m.v[2], m.v[3], den) : 0.0f;
  r.v[3] = (zmask & 8) ? fd4(m.v[1], m.v[2], m.v[3], nx, den) : 0.0f;
  return r;
}

// z-forward difference: samples c-1..c+2; c0-1 from the previous lane,
// c0+4, c0+5 from the next.
__device__ __forceinline__ f4 dz_fwd(const f4& m, float den, int zmask) {
  float pw = __shfl_up_sync(kFull, m.v[3], 1);
  float n0 = __shfl_down_sync(kFull, m.v[0], 1);
  float n1 = __shfl_down_sync(kFull, m.v[1], 1);
  f4 r;
  r.v[0] = (zmask & 1) ? fd4(pw, m.v[0], m.v[1], m.v[2], den) : 0.0f;
  r.v[1] = (zmask & 2) ? fd4(m.v[0], m.v[1], m.v[2], m.v[3], den) : 0.0f;
  r.v[2] = (zmask & 4) ? fd4(m.v[1], m.v[2], m.v[3], n0, den) : 0.0f;
  r.v[3] = (zmask & 8) ? fd4(m.v[2], m.v[3], n0, n1, den) : 0.0f;
  return r;
}

// x-difference from four rows of a register ring (oldest first).
__device__ __forceinline__ f4 dx4(const f4& r0, const f4& r1, const f4& r2, const f4& r3, float den,
                                  bool ok) {
  f4 r;
#pragma unroll
  for (int e = 0; e < 4; ++e) r.v[e] = ok ? fd4(r0.v[e], r1.v[e], r2.v[e], r3.v[e], den) : 0.0f;
  return r;
}

// Masked differences with the mask folded into the reciprocal: r = 0 where
// the edge rule zeroes the derivative (fd4 of finite samples times 0 is a
// zero, possibly -0, which no later sum or product tells apart from +0).
__device__ __forceinline__ f4 dx4r(const f4& r0, const f4& r1, const f4& r2, const f4& r3, float r) {
  f4 o;
#pragma unroll
  for (int e = 0; e < 4; ++e) o.v[e] = fd4(r0.v[e], r1.v[e], r2.v[e], r3.v[e], r);
  return o;
}

__device__ __forceinline__ f4 dz_back_r(const f4& m, const f4& r) {
  const float pz = __shfl_up_sync(kFull, m.v[2], 1);
  const float pw = __shfl_up_sync(kFull, m.v[3], 1);
  const float nx = __shfl_down_sync(kFull, m.v[0], 1);
  f4 o;
  o.v[0] = fd4(pz, pw, m.v[0], m.v[1], r.v[0]);
  o.v[1] = fd4(pw, m.v[0], m.v[1], m.v[2], r.v[1]);
  o.v[2] = fd4(m.v[0], m.v[1], m.v[2], m.v[3], r.v[2]);
  o.v[3] = fd4(m.v[1], m.v[2], m.v[3], nx, r.v[3]);
  return o;
}

__device__ __forceinline__ f4 dz_fwd_r(const f4& m, const f4& r) {
  const float pw = __shfl_up_sync(kFull, m.v[3], 1);
  const float n0 = __shfl_down_sync(kFull, m.v[0], 1);
  const float n1 = __shfl_down_sync(kFull, m.v[1], 1);
  f4 o;
  o.v[0] = fd4(pw, m.v[0], m.v[1], m.v[2], r.v[0]);
  o.v[1] = fd4(m.v[0], m.v[1], m.v[2], m.v[3], r.v[1]);
  o.v[2] = fd4(m.v[1], m.v[2], m.v[3], n0, r.v[2]);
  o.v[3] = fd4(m.v[2], m.v[3], n0, n1, r.v[3]);
  return o;
}

// Per-lane column facts, fixed for the whole march.
struct LaneCols {
  int c0;        // first column of the lane
  int zb;        // bit e: z-backward derivative allowed at column c0+e (2 <= c < nz-2)
  int zf;        // bit e: z-forward derivative allowed (1 <= c < nz-2)
  int own;       // bit e: column owned by this lane (inside the strip's outputs, < nz)
  int own_lo, own_hi;  // owned column range of the warp's strip [own_lo, own_hi)
};

__device__ __forceinline__ LaneCols lane_cols(const Geom& g, int strip, int lane) {
  LaneCols L;
  // Strips tile [0, nz) in steps of kStripCols; the last strip is shifted
  // left so that it ends at nz and owns only the columns not owned before.
  // j0 stays a multiple of 4 so that every lane's float4 is 16-byte aligned.
  int own_lo = strip * kStripCols;
  int j0 = own_lo;
  if (j0 + kStripCols > g.nz) j0 = g.nz > kStripCols ? ((g.nz - kStripCols + 3) & ~3) : 0;
  int own_hi = min(g.nz, own_lo + kStripCols);
  L.c0 = j0 - 4 + 4 * lane;
  L.own_lo = own_lo;
  L.own_hi = own_hi;
  L.zb = L.zf = L.own = 0;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    int c = L.c0 + e;
    if (c >= 2 && c < g.nz - 2) L.zb |= 1 << e;
    if (c >= 1 && c < g.nz - 2) L.zf |= 1 << e;
    if (lane >= 1 && lane <= 30 && c >= own_lo && c < own_hi) L.own |= 1 << e;
  }
  return L;
}

// r at the lane's columns whose bit is set in `mask`, 0 elsewhere.
__device__ __forceinline__ f4 masked_recip(float r, int mask) {
  f4 o;
#pragma unroll
  for (int e = 0; e < 4; ++e) o.v[e] = (mask & (1 << e)) ? r : 0.0f;
  return o;
}

// Bounded-size cursor over a (i, j)-sorted list: the first entry with row >= i0.
template <typename T>
__device__ __forceinline__ int lower_row(const T* __restrict__ list, int n, int i0) {
  int lo = 0, hi = n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (__ldg(&list[mid].i) < i0) lo = mid + 1; else hi = mid;
  }
  return lo;
}

}  // namespace seiswg
