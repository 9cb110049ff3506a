// fd_step_march.cuh -- the one-step SH and PSV marches (fd_step.cu has the
// algorithm notes and the kernels): one warp advances its (strip, chunk) by
// one time step.  Included by the single-problem and grouped kernels of
// fd_step.cu and by the batch's queue kernel (fd_queue.cu).
#pragma once

#include "fd_march.cuh"

namespace seiswg {
namespace {
// --------------------------------------------------------------------------
// SH: state vy, sxy, szy; material 1/rho, mu.  fd2d.wgsl:242-301.
// --------------------------------------------------------------------------
enum ShSeg { SH_SXY = 0, SH_SZY, SH_VY, SH_RHO, SH_MU, SH_NSEG };

// One warp's march over its (strip, chunk); gw is the warp's index within
// the problem and smem its slice of shared memory (warp_slice).  Shared by
// the single-problem, grouped and queue kernels.  Every march of the step
// kernels returns false when a bounded wait of its row pipeline expired (the
// error word is then set and the copies in flight drained), true otherwise.
template <class Loader>
__device__ __forceinline__ bool sh_march(const ShStep& p, int gw, unsigned char* smem) {
  const Geom& g = p.g;
  const March m = march_of(g, gw);
  if (!m.active) return true;
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
      return false;
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
  return true;
}

// --------------------------------------------------------------------------
// PSV: state vx, vz, sxx, szz, sxz; material 1/rho, lambda, mu.
// fd2d.wgsl:308-399.  (PSV + spin: fd_spin.cu.)
// --------------------------------------------------------------------------
enum PsvSeg { PV_SXX = 0, PV_SXZ, PV_SZZ, PV_VX, PV_VZ, PV_RHO, PV_LAM, PV_MU, PV_NSEG };

template <class Loader>
__device__ __forceinline__ bool psv_march(const PsvStep& p, int gw, unsigned char* smem) {
  const Geom& g = p.g;
  const March m = march_of(g, gw);
  if (!m.active) return true;
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
      return false;
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
  return true;
}

}  // namespace
}  // namespace seiswg
