// fd_step.cu -- fused one-step kernels for the SH and PSV systems (PSV +
// spin: fd_spin.cu).
//
// One launch advances the wavefield by one time step: the velocity update
// (divergence of stress, source injection, Gaussian taper, displacement at
// probes) and the stress update (velocity gradients, Hooke's law) of
// shaders/fd2d.wgsl, which the reference runs as 6 (SH), 10 (PSV) or 17
// (spin) dispatches with every intermediate field in memory
// (solver.rs:1000-1030).  Here every intermediate lives in registers; each
// state field is read once and written once per step, each material field
// read once: 32 B (SH), 52 B (PSV), 96 B (spin) per cell-update.
//
// A warp marches down x over its chunk of rows.  Iteration k handles
// velocity row i = ib-1+k (stress rows i-2..i+1 in a register ring) and
// stress row r = i-2 (new velocity rows r-1..r+2 in a register ring).  Row
// data arrive through a loader (fd_pipe.cuh): plain loads, or a shared-memory
// ring fed by the TMA bulk-copy engine a few rows ahead.
//
// State is ping-ponged between two buffers (read step n, write step n+1):
// a warp recomputes the velocity of its halo rows/columns from step-n data
// that its neighbours would otherwise be overwriting in place.
//
// Arithmetic follows the reference's expressions operation for operation
// (built with -fmad=false), except that divisions by 8*dx, rho and J are
// multiplies by precomputed reciprocals; results track the FP32 reference to
// rounding (relative L2 ~1e-7 over thousands of steps).
#include "fd_march.cuh"

namespace seiswg {



// --------------------------------------------------------------------------
// SH: state vy, sxy, szy; material 1/rho, mu.  fd2d.wgsl:242-301.
// --------------------------------------------------------------------------
enum ShSeg { SH_SXY = 0, SH_SZY, SH_VY, SH_RHO, SH_MU, SH_NSEG };

// One warp's march over its (strip, chunk); gw is the warp's index within
// the problem.  Shared by the single-problem and the grouped kernels.
template <class Loader>
__device__ __forceinline__ void sh_march(const ShStep& p, int gw, unsigned char* smem) {
  const Geom& g = p.g;
  const March m = march_of(g, gw);
  if (!m.active) return;
  const LaneCols L = lane_cols(g, m.strip, m.lane);
  const size_t ld = size_t(g.ld);
  const float dt = g.dt;
  const int c0 = L.c0;
  auto at = [&](auto* base, int i) { return base + ptrdiff_t(i) * ptrdiff_t(ld) + c0; };

  typename Loader::SegsT segs;
  segs.base[SH_SXY] = p.sxy0; segs.roff[SH_SXY] = 1;
  segs.base[SH_SZY] = p.szy0; segs.roff[SH_SZY] = 1;
  segs.base[SH_VY] = p.vy0; segs.roff[SH_VY] = 0;
  segs.base[SH_RHO] = p.rho; segs.roff[SH_RHO] = 0;
  segs.base[SH_MU] = p.mu; segs.roff[SH_MU] = -2;
  Loader rows = make_loader<Loader>(segs, g, m, L, smem);
  rows.configure(g);
  rows.start();

  const f4 tb = ld4(p.taper_zb + c0), tt = ld4(p.taper_zt + c0);
  // Rings: sxy, szy rows i-2..i+1 (slot 3 arrives with iteration k); new vy rows i-3..i.
  f4 xy0 = ld4(at(p.sxy0, m.ib - 3)), xy1 = ld4(at(p.sxy0, m.ib - 2)), xy2 = ld4(at(p.sxy0, m.ib - 1)), xy3;
  f4 zy0 = ld4(at(p.szy0, m.ib - 3)), zy1 = ld4(at(p.szy0, m.ib - 2)), zy2 = ld4(at(p.szy0, m.ib - 1)), zy3;
  f4 va, vb, vc, vd;
  Cursor ci = cursor_at(p.inj.list, p.inj.n, m.ib - 1);
  Cursor pi = cursor_at(p.probes.list, p.probes.n, m.ib);
  const int nk = m.ie - m.ib + 3;

  for (int k = 0; k < nk; ++k) {
    const int i = m.ib - 1 + k;
    if (!rows.acquire(k)) {
      flag_timeout(p.err);
      rows.drain(k);
      return;
    }
    xy3 = rows.seg(SH_SXY);
    zy3 = rows.seg(SH_SZY);
    const f4 vo = rows.seg(SH_VY);
    const f4 rho = rows.seg(SH_RHO);
    const f4 mu = rows.seg(SH_MU);
    rows.release();
    const float bxi = __ldg(p.taper_x + i);
    const bool xb = (i >= 2 && i < g.nx - 2);

    // div_sy (fd2d.wgsl:247): DSY = dx-(sxy) + dz-(szy)
    f4 ds = dx4(xy0, xy1, xy2, xy3, g.rdx, xb);
    const f4 dz = dz_back(zy2, g.rdz, L.zb);
#pragma unroll
    for (int e = 0; e < 4; ++e) ds.v[e] = ds.v[e] + dz.v[e];
    inject_at<false, true, false>(p.inj, i, c0, ci, ds, ds, ds);  // stf_dsy / adj_dsy

    // add_vy (fd2d.wgsl:268): vy = b * (vy + dt * DSY / rho), with the
    // buoyancy 1/rho stored in place of rho.
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float b = (bxi * tb.v[e]) * tt.v[e];
      vd.v[e] = b * (vo.v[e] + dt * ds.v[e] * rho.v[e]);
    }
    if (i >= m.ib && i < m.ie) {
      st4_masked(at(p.vy1, i), vd, L.own);
      probe_at(p.probes, i, L, pi, dt, [&](int, int e) { return pick4(vd, e); });
    }

    // Stress of row r = i-2 from new vy rows r-1..r+2 = (va, vb, vc, vd).
    if (i >= m.ib + 2) {
      const int r = i - 2;
      const bool xf = (r >= 1 && r < g.nx - 2);
      const f4 gx = dx4(va, vb, vc, vd, g.rdx, xf);
      const f4 gz = dz_fwd(vb, g.rdz, L.zf);
      f4 sx, sz;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float mu_dt = mu.v[e] * dt;  // add_sy_sh, fd2d.wgsl:288-290
        sx.v[e] = xy0.v[e] + mu_dt * gx.v[e];
        sz.v[e] = zy0.v[e] + mu_dt * gz.v[e];
      }
      st4_masked(at(p.sxy1, r), sx, L.own);
      st4_masked(at(p.szy1, r), sz, L.own);
    }

    va = vb; vb = vc; vc = vd;
    xy0 = xy1; xy1 = xy2; xy2 = xy3;
    zy0 = zy1; zy1 = zy2; zy2 = zy3;
  }
}

// --------------------------------------------------------------------------
// PSV: state vx, vz, sxx, szz, sxz; material 1/rho, lambda, mu.
// fd2d.wgsl:308-399.  (PSV + spin: fd_spin.cu.)
// --------------------------------------------------------------------------
enum PsvSeg { PV_SXX = 0, PV_SXZ, PV_SZZ, PV_VX, PV_VZ, PV_RHO, PV_LAM, PV_MU, PV_NSEG };

template <class Loader>
__device__ __forceinline__ void psv_march(const PsvStep& p, int gw, unsigned char* smem) {
  const Geom& g = p.g;
  const March m = march_of(g, gw);
  if (!m.active) return;
  const LaneCols L = lane_cols(g, m.strip, m.lane);
  const size_t ld = size_t(g.ld);
  const float dt = g.dt;
  const int c0 = L.c0;
  auto at = [&](auto* base, int i) { return base + ptrdiff_t(i) * ptrdiff_t(ld) + c0; };

  typename Loader::SegsT segs;
  segs.base[PV_SXX] = p.sxx0; segs.roff[PV_SXX] = 1;
  segs.base[PV_SXZ] = p.sxz0; segs.roff[PV_SXZ] = 1;
  segs.base[PV_SZZ] = p.szz0; segs.roff[PV_SZZ] = 1;
  segs.base[PV_VX] = p.vx0; segs.roff[PV_VX] = 0;
  segs.base[PV_VZ] = p.vz0; segs.roff[PV_VZ] = 0;
  segs.base[PV_RHO] = p.rho; segs.roff[PV_RHO] = 0;
  segs.base[PV_LAM] = p.lam; segs.roff[PV_LAM] = -2;
  segs.base[PV_MU] = p.mu; segs.roff[PV_MU] = -2;
  Loader rows = make_loader<Loader>(segs, g, m, L, smem);
  rows.configure(g);
  rows.start();

  const f4 tb = ld4(p.taper_zb + c0), tt = ld4(p.taper_zt + c0);
  // Edge rule by selects (dx4 / dz_back / dz_fwd): measured 10 % faster here
  // than masks folded into the reciprocals.
  f4 xx0 = ld4(at(p.sxx0, m.ib - 3)), xx1 = ld4(at(p.sxx0, m.ib - 2)), xx2 = ld4(at(p.sxx0, m.ib - 1)), xx3;
  f4 xz0 = ld4(at(p.sxz0, m.ib - 3)), xz1 = ld4(at(p.sxz0, m.ib - 2)), xz2 = ld4(at(p.sxz0, m.ib - 1)), xz3;
  f4 zz0 = ld4(at(p.szz0, m.ib - 3)), zz1 = ld4(at(p.szz0, m.ib - 2)), zz2 = ld4(at(p.szz0, m.ib - 1)), zz3;
  f4 xa, xb_, xc, xd;   // new vx rows i-3..i
  f4 za, zb_, zc, zd;   // new vz rows i-3..i
  Cursor ci = cursor_at(p.inj.list, p.inj.n, m.ib - 1);
  Cursor pi = cursor_at(p.probes.list, p.probes.n, m.ib);
  const int nk = m.ie - m.ib + 3;

  for (int k = 0; k < nk; ++k) {
    const int i = m.ib - 1 + k;
    if (!rows.acquire(k)) {
      flag_timeout(p.err);
      rows.drain(k);
      return;
    }
    xx3 = rows.seg(PV_SXX);
    xz3 = rows.seg(PV_SXZ);
    zz3 = rows.seg(PV_SZZ);
    const f4 vxo = rows.seg(PV_VX);
    const f4 vzo = rows.seg(PV_VZ);
    const f4 rho = rows.seg(PV_RHO);
    const f4 lam = rows.seg(PV_LAM);
    const f4 mu = rows.seg(PV_MU);
    rows.release();
    const float bxi = __ldg(p.taper_x + i);
    const bool xok = (i >= 2 && i < g.nx - 2);

    // div_sxz (fd2d.wgsl:315-316)
    f4 dsx = dx4(xx0, xx1, xx2, xx3, g.rdx, xok);
    f4 dsz = dx4(xz0, xz1, xz2, xz3, g.rdx, xok);
    {
      const f4 a = dz_back(xz2, g.rdz, L.zb);
      const f4 b = dz_back(zz2, g.rdz, L.zb);
#pragma unroll
      for (int e = 0; e < 4; ++e) { dsx.v[e] = dsx.v[e] + a.v[e]; dsz.v[e] = dsz.v[e] + b.v[e]; }
    }
    inject_at<true, false, true>(p.inj, i, c0, ci, dsx, dsx, dsz);  // stf_dsxz, fd2d.wgsl:350-351

    // add_vxz (fd2d.wgsl:362-363), rho holding 1/rho
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float b = (bxi * tb.v[e]) * tt.v[e];
      xd.v[e] = b * (vxo.v[e] + dt * dsx.v[e] * rho.v[e]);
      zd.v[e] = b * (vzo.v[e] + dt * dsz.v[e] * rho.v[e]);
    }
    if (i >= m.ib && i < m.ie) {
      st4_masked(at(p.vx1, i), xd, L.own);
      st4_masked(at(p.vz1, i), zd, L.own);
      probe_at(p.probes, i, L, pi, dt,
               [&](int comp, int e) { return comp == kProbeVX ? pick4(xd, e) : pick4(zd, e); });
    }

    // Stress of row r = i-2.
    if (i >= m.ib + 2) {
      const int r = i - 2;
      const bool rok = (r >= 1 && r < g.nx - 2);
      // div_vxz (fd2d.wgsl:378-381)
      const f4 dvxdx = dx4(xa, xb_, xc, xd, g.rdx, rok);
      const f4 dvzdx = dx4(za, zb_, zc, zd, g.rdx, rok);
      const f4 dvxdz = dz_fwd(xb_, g.rdz, L.zf);
      const f4 dvzdz = dz_fwd(zb_, g.rdz, L.zf);
      f4 sxx, szz, sxz;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        // add_sxz (fd2d.wgsl:396-398)
        const float l = lam.v[e], mm = mu.v[e];
        sxx.v[e] = xx0.v[e] + dt * ((l + 2.0f * mm) * dvxdx.v[e] + l * dvzdz.v[e]);
        szz.v[e] = zz0.v[e] + dt * ((l + 2.0f * mm) * dvzdz.v[e] + l * dvxdx.v[e]);
        sxz.v[e] = xz0.v[e] + dt * mm * (dvxdz.v[e] + dvzdx.v[e]);
      }
      st4_masked(at(p.sxx1, r), sxx, L.own);
      st4_masked(at(p.szz1, r), szz, L.own);
      st4_masked(at(p.sxz1, r), sxz, L.own);
    }

    xa = xb_; xb_ = xc; xc = xd;
    za = zb_; zb_ = zc; zc = zd;
    xx0 = xx1; xx1 = xx2; xx2 = xx3;
    xz0 = xz1; xz1 = xz2; xz2 = xz3;
    zz0 = zz1; zz1 = zz2; zz2 = zz3;
  }
}

template <class Loader>
__global__ void __launch_bounds__(kStepWarps * 32) sh_step_kernel(const ShStep p) {
  extern __shared__ __align__(128) unsigned char smem[];
  sh_march<Loader>(p, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), smem);
}

template <class Loader>
__global__ void __launch_bounds__(kStepWarps * 32) psv_step_kernel(const PsvStep p) {
  extern __shared__ __align__(128) unsigned char smem[];
  psv_march<Loader>(p, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), smem);
}


// --------------------------------------------------------------------------
// Launchers
// --------------------------------------------------------------------------
namespace {
template <class L>
cudaError_t launch_sh(const ShStep& p, cudaStream_t s) {
  const size_t smem = smem_for<L>();
  static const cudaError_t attr = prepare_kernel(sh_step_kernel<L>, smem);
  if (attr != cudaSuccess) return attr;
  sh_step_kernel<L><<<blocks_for(p.g), kStepWarps * 32, smem, s>>>(p);
  return cudaGetLastError();
}

template <class L>
cudaError_t launch_psv(const PsvStep& p, cudaStream_t s) {
  const size_t smem = smem_for<L>();
  static const cudaError_t attr = prepare_kernel(psv_step_kernel<L>, smem);
  if (attr != cudaSuccess) return attr;
  psv_step_kernel<L><<<blocks_for(p.g), kStepWarps * 32, smem, s>>>(p);
  return cudaGetLastError();
}

}  // namespace

// ---- grouped forward steps ----------------------------------------------------
namespace {

__device__ __forceinline__ float* slot_field(const JobDesc& J, int slot, int f) {
  return J.pool + slot * J.slot_elems + f * J.field_elems + J.halo;
}

}  // namespace

template <bool PSV>
__global__ void __launch_bounds__(kStepWarps * 32) grouped_forward_kernel(const JobDesc* __restrict__ jobs,
                                                                          const GroupOp* __restrict__ ops, int nops) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const GroupOp op = ops[group_op_of(ops, nops, gw)];
  const JobDesc& J = jobs[op.job];
  const int lw = gw - op.warp_begin;
  if (lw >= J.g.nstrips * J.g.nchunks) return;
  ProbeList pl = J.probes;
  if (!(op.flags & 1)) pl.n = 0;
  pl.it = op.it;
  InjectList inj = J.src;
  inj.it = op.it;
  if constexpr (PSV) {
    PsvStep p{};
    p.g = J.g;
    p.vx0 = slot_field(J, op.a, 0); p.vz0 = slot_field(J, op.a, 1); p.sxx0 = slot_field(J, op.a, 2);
    p.szz0 = slot_field(J, op.a, 3); p.sxz0 = slot_field(J, op.a, 4);
    p.vx1 = slot_field(J, op.b, 0); p.vz1 = slot_field(J, op.b, 1); p.sxx1 = slot_field(J, op.b, 2);
    p.szz1 = slot_field(J, op.b, 3); p.sxz1 = slot_field(J, op.b, 4);
    p.rho = J.rho; p.lam = J.lam; p.mu = J.mu;
    p.taper_x = J.taper_x; p.taper_zb = J.taper_zb; p.taper_zt = J.taper_zt;
    p.inj = inj;
    p.probes = pl;
    p.err = J.err;
    psv_march<BulkL<PV_NSEG>>(p, lw, smem);
  } else {
    ShStep p{};
    p.g = J.g;
    p.vy0 = slot_field(J, op.a, 0); p.sxy0 = slot_field(J, op.a, 1); p.szy0 = slot_field(J, op.a, 2);
    p.vy1 = slot_field(J, op.b, 0); p.sxy1 = slot_field(J, op.b, 1); p.szy1 = slot_field(J, op.b, 2);
    p.rho = J.rho; p.mu = J.mu;
    p.taper_x = J.taper_x; p.taper_zb = J.taper_zb; p.taper_zt = J.taper_zt;
    p.inj = inj;
    p.probes = pl;
    p.err = J.err;
    sh_march<BulkL<SH_NSEG>>(p, lw, smem);
  }
}

cudaError_t launch_grouped_forward(const JobDesc* jobs, const GroupOp* ops, int nops, int warps, bool psv,
                                   cudaStream_t s) {
  if (nops <= 0 || warps <= 0) return cudaSuccess;
  const unsigned blocks = unsigned((warps + kStepWarps - 1) / kStepWarps);
  if (psv) {
    const size_t smem = smem_for<BulkL<PV_NSEG>>();
    static const cudaError_t attr = prepare_kernel(grouped_forward_kernel<true>, smem);
    if (attr != cudaSuccess) return attr;
    grouped_forward_kernel<true><<<blocks, kStepWarps * 32, smem, s>>>(jobs, ops, nops);
  } else {
    const size_t smem = smem_for<BulkL<SH_NSEG>>();
    static const cudaError_t attr = prepare_kernel(grouped_forward_kernel<false>, smem);
    if (attr != cudaSuccess) return attr;
    grouped_forward_kernel<false><<<blocks, kStepWarps * 32, smem, s>>>(jobs, ops, nops);
  }
  return cudaGetLastError();
}

size_t step_smem_bytes(bool psv, bool spin, int loader) {
  if (loader != kLoaderBulk) return 0;
  if (!psv) return smem_for<BulkL<SH_NSEG>>();
  return spin ? spin_step_smem_bytes(loader) : smem_for<BulkL<PV_NSEG>>();
}

int step_blocks_per_sm(bool psv, bool spin, int loader) {
  int n = 0;
  const int threads = kStepWarps * 32;
  const size_t smem = step_smem_bytes(psv, spin, loader);
  cudaError_t e;
  if (!psv) {
    e = loader == kLoaderBulk
            ? (prepare_kernel(sh_step_kernel<BulkL<SH_NSEG>>, smem),
               cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sh_step_kernel<BulkL<SH_NSEG>>, threads, smem))
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sh_step_kernel<DirectL<SH_NSEG>>, threads, smem);
  } else if (spin) {
    return spin_step_blocks_per_sm(loader);
  } else {
    e = loader == kLoaderBulk
            ? (prepare_kernel(psv_step_kernel<BulkL<PV_NSEG>>, smem),
               cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, psv_step_kernel<BulkL<PV_NSEG>>, threads, smem))
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, psv_step_kernel<DirectL<PV_NSEG>>, threads, smem);
  }
  return e == cudaSuccess ? n : 0;
}


cudaError_t launch_sh_step(const ShStep& p, cudaStream_t s) {
  if (p.g.loader == kLoaderBulk) return launch_sh<BulkL<SH_NSEG>>(p, s);
  return launch_sh<DirectL<SH_NSEG>>(p, s);
}

cudaError_t launch_psv_step(const PsvStep& p, bool spin, cudaStream_t s) {
  if (spin) return launch_psv_spin_step(p, s);
  if (p.g.loader == kLoaderBulk) return launch_psv<BulkL<PV_NSEG>>(p, s);
  return launch_psv<DirectL<PV_NSEG>>(p, s);
}

}  // namespace seiswg
