// fd_group.cuh -- the march parameters of one operation of a batched job
// (JobDesc; the operation's it, a, b, flags as in GroupOp), shared by the
// grouped launches (fd_step.cu, fd_step2.cu, fd_adjoint.cu) and the batch's
// queue kernel (fd_queue.cu).
#pragma once

#include "fd_kernels.h"

namespace seiswg {
namespace {

// Field f of slot `slot` of a job's pool (or adjoint pair), at element (0, 0).
__device__ __forceinline__ float* job_field(float* base, const JobDesc& J, int slot, int f) {
  return base + slot * J.slot_elems + f * J.field_elems + J.halo;
}

__device__ __forceinline__ ProbeList job_probes(const JobDesc& J, int it, int flags) {
  ProbeList pl = J.probes;
  if (!(flags & 1)) pl.n = 0;
  pl.it = it;
  return pl;
}

// Forward step `it` from state slot a to slot b; flags & 1 records the probes.
__device__ __forceinline__ PsvStep job_psv_step(const JobDesc& J, int it, int a, int b, int flags) {
  PsvStep p{};
  p.g = J.g;
  p.vx0 = job_field(J.pool, J, a, 0); p.vz0 = job_field(J.pool, J, a, 1); p.sxx0 = job_field(J.pool, J, a, 2);
  p.szz0 = job_field(J.pool, J, a, 3); p.sxz0 = job_field(J.pool, J, a, 4);
  p.vx1 = job_field(J.pool, J, b, 0); p.vz1 = job_field(J.pool, J, b, 1); p.sxx1 = job_field(J.pool, J, b, 2);
  p.szz1 = job_field(J.pool, J, b, 3); p.sxz1 = job_field(J.pool, J, b, 4);
  p.rho = J.rho; p.lam = J.lam; p.mu = J.mu;
  p.taper_x = J.taper_x; p.taper_zb = J.taper_zb; p.taper_zt = J.taper_zt;
  p.inj = J.src;
  p.inj.it = it;
  p.probes = job_probes(J, it, flags);
  p.err = J.err;
  return p;
}

__device__ __forceinline__ ShStep job_sh_step(const JobDesc& J, int it, int a, int b, int flags) {
  ShStep p{};
  p.g = J.g;
  p.vy0 = job_field(J.pool, J, a, 0); p.sxy0 = job_field(J.pool, J, a, 1); p.szy0 = job_field(J.pool, J, a, 2);
  p.vy1 = job_field(J.pool, J, b, 0); p.sxy1 = job_field(J.pool, J, b, 1); p.szy1 = job_field(J.pool, J, b, 2);
  p.rho = J.rho; p.mu = J.mu;
  p.taper_x = J.taper_x; p.taper_zb = J.taper_zb; p.taper_zt = J.taper_zt;
  p.inj = J.src;
  p.inj.it = it;
  p.probes = job_probes(J, it, flags);
  p.err = J.err;
  return p;
}

// Steps it and it + 1 with the two-step geometry g2 and the dt-scaled
// material (dt/rho, dt*lambda, dt*mu at the material's field stride);
// flags & kOpMid: the state after step `it` into slot b - 1 as well.
__device__ __forceinline__ PsvStep job_psv_step2(const JobDesc& J, int it, int a, int b, int flags) {
  PsvStep p = job_psv_step(J, it, a, b, flags);
  p.g = J.g2;
  const long long dm = J.lam - J.rho;
  p.rho = J.rho_dt; p.lam = J.rho_dt + dm; p.mu = J.rho_dt + 2 * dm;
  if (flags & kOpMid) {
    p.vxm = job_field(J.pool, J, b - 1, 0); p.vzm = job_field(J.pool, J, b - 1, 1);
    p.sxxm = job_field(J.pool, J, b - 1, 2); p.szzm = job_field(J.pool, J, b - 1, 3);
    p.sxzm = job_field(J.pool, J, b - 1, 4);
  }
  return p;
}

__device__ __forceinline__ ShStep job_sh_step2(const JobDesc& J, int it, int a, int b, int flags) {
  ShStep p = job_sh_step(J, it, a, b, flags);
  p.g = J.g2;
  p.rho = J.rho_dt; p.mu = J.rho_dt + 2 * (J.lam - J.rho);
  if (flags & kOpMid) {
    p.vym = job_field(J.pool, J, b - 1, 0); p.sxym = job_field(J.pool, J, b - 1, 1);
    p.szym = job_field(J.pool, J, b - 1, 2);
  }
  return p;
}

// Reverse step `it`: the forward state in pool slot a, the incoming adjoint
// state in adjoint slot (b & 1), the outgoing in the other.
__device__ __forceinline__ PsvAdjoint job_psv_adjoint(const JobDesc& J, int it, int a, int b) {
  const int in = b & 1, out = 1 - in;
  PsvAdjoint p{};
  p.g = J.g;
  p.vx = job_field(J.pool, J, a, 0); p.vz = job_field(J.pool, J, a, 1); p.sxx = job_field(J.pool, J, a, 2);
  p.szz = job_field(J.pool, J, a, 3); p.sxz = job_field(J.pool, J, a, 4);
  p.wx0 = job_field(J.adj, J, in, 0); p.wz0 = job_field(J.adj, J, in, 1); p.bxx0 = job_field(J.adj, J, in, 2);
  p.bzz0 = job_field(J.adj, J, in, 3); p.bxz0 = job_field(J.adj, J, in, 4);
  p.wx1 = job_field(J.adj, J, out, 0); p.wz1 = job_field(J.adj, J, out, 1); p.bxx1 = job_field(J.adj, J, out, 2);
  p.bzz1 = job_field(J.adj, J, out, 3); p.bxz1 = job_field(J.adj, J, out, 4);
  p.rho = J.rho; p.lam = J.lam; p.mu = J.mu;
  p.taper_x = J.taper_x; p.taper_zb = J.taper_zb; p.taper_zt = J.taper_zt;
  p.g_b = J.g_b; p.g_lam = J.g_lam; p.g_mu = J.g_mu;
  p.src = J.src;
  p.src.it = it;
  p.rec = J.rec;
  p.rec.it = it;
  p.err = J.err;
  return p;
}

__device__ __forceinline__ ShAdjoint job_sh_adjoint(const JobDesc& J, int it, int a, int b) {
  const int in = b & 1, out = 1 - in;
  ShAdjoint p{};
  p.g = J.g;
  p.vy = job_field(J.pool, J, a, 0); p.sxy = job_field(J.pool, J, a, 1); p.szy = job_field(J.pool, J, a, 2);
  p.w0 = job_field(J.adj, J, in, 0); p.bxy0 = job_field(J.adj, J, in, 1); p.bzy0 = job_field(J.adj, J, in, 2);
  p.w1 = job_field(J.adj, J, out, 0); p.bxy1 = job_field(J.adj, J, out, 1); p.bzy1 = job_field(J.adj, J, out, 2);
  p.rho = J.rho; p.mu = J.mu;
  p.taper_x = J.taper_x; p.taper_zb = J.taper_zb; p.taper_zt = J.taper_zt;
  p.g_b = J.g_b; p.g_mu = J.g_mu;
  p.src = J.src;
  p.src.it = it;
  p.rec = J.rec;
  p.rec.it = it;
  p.err = J.err;
  return p;
}

// The job's tensor maps (JobDesc::tm) of a two-step PSV or SH operation
// reading state slot a, and of a PSV reverse step reading slot a and adjoint
// slot (b & 1).
__device__ __forceinline__ Tma2Ptrs job_psv2_maps(const JobDesc& J, int a) {
  const CUtensorMap* t = J.tm + 3 * J.tm_nslot;
  return Tma2Ptrs{J.tm + 3 * a + 2, J.tm + 3 * a + 1, t + 8, t + 9};
}

__device__ __forceinline__ Tma2Ptrs job_sh2_maps(const JobDesc& J, int a) {
  return Tma2Ptrs{J.tm + 3 * a + 1, J.tm + 3 * a + 0, J.tm + 3 * J.tm_nslot + 8, nullptr};
}

__device__ __forceinline__ TmaAdjPtrs job_adj_maps(const JobDesc& J, int a, int b) {
  const CUtensorMap* t = J.tm + 3 * J.tm_nslot;
  const int in = b & 1;
  return TmaAdjPtrs{J.tm + 3 * a + 0, J.tm + 3 * a + 1, t + 2 * in, t + 2 * in + 1, t + 4, t + 5, t + 6, t + 7};
}

}  // namespace
}  // namespace seiswg
