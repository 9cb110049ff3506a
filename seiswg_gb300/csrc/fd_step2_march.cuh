// fd_step2_march.cuh -- the two-step PSV and SH marches (fd_step2.cu has the
// notes on their arithmetic and the kernels).  Included by the kernels of
// fd_step2.cu and by the batch's queue kernel (fd_queue.cu); both are built
// with multiply-add contraction.
#pragma once

#include <type_traits>

#include "fd_fma.cuh"
#include "fd_tma.cuh"

namespace seiswg {
namespace {
// --------------------------------------------------------------------------
// PSV, two time steps per pass (temporal blocking).
//
// Level 1 is the one-step march above (velocity of row i, stress of row i-2,
// step `it`); its new rows stay in registers and feed level 2, which runs the
// same update for step it+1 three rows behind (velocity of row i-3, stress of
// row i-5).  Only level-2 rows are written: per two steps each state field is
// read and written once and each material field read twice (once per level,
// the second time from L2), 26 B of HBM traffic per cell-update instead of 52.
//
// The divergence is added to v with the material's dt/rho and the sources
// enter the divergence unscaled (stf_dsxz, fd2d.wgsl:344-352).
//
// Reach: two steps need level-1 values 3 columns and 4 rows beyond the
// level-2 outputs, so a strip owns 112 columns (lanes 2..29) and a chunk of
// rows [ib, ie) marches i over [ib-4, ie+4].  Level-1 values outside the grid
// are forced to zero, as a one-step launch leaves the halo of its output.
// Each arithmetic expression is the one-step kernel's; with multiply-add
// contraction the results differ from two one-step launches by rounding only.
// --------------------------------------------------------------------------
enum Psv2Seg {
  P2_SXX = 0, P2_SZZ, P2_SXZ,  // sigma^n, row i+1 (the order of the state's fields)
  P2_VX, P2_VZ,                // v^n, row i
  P2_RHO, P2_LAM, P2_MU,       // 1/rho row i, lambda/mu row i-2
  P2_NSEG
};

// Six stages per warp: two rows in flight and the stages of the last three
// iterations kept, whose 1/rho (row i-3) and lambda/mu (row i-5) are the
// material of level 2.  Lane q issues the copy of segment q (the issue-bound
// march spends fewer instructions that way than with lane 0 issuing all
// eight: 170 against 154 Gcell-updates/s at 4096^2).
struct Bulk2 : BulkRows<P2_NSEG, 6, true, 3> {
  using SegsT = Segs<P2_NSEG>;
  using BulkRows<P2_NSEG, 6, true, 3>::BulkRows;
};

// PSV: sigma^n (sxx, szz, sxz; row i+1), v^n (vx, vz; row i), 1/rho (row
// i), lambda and mu (row i-2): four copies for the eight segments of Psv2Seg.
struct PsvTmaPlan {
  using Maps = Tma2;
  static constexpr int NSEG = P2_NSEG;
  template <class M>
  __device__ __forceinline__ static void issue(float* sb, const M* tm, int x, int y, uint64_t* b) {
    tma3(sb + P2_SXX * kSegFloats, tmap(tm->sig), x, y + 1, 2, b);
    tma3(sb + P2_VX * kSegFloats, tmap(tm->vel), x, y, 0, b);
    tma3(sb + P2_RHO * kSegFloats, tmap(tm->rho), x, y, 0, b);
    tma3(sb + P2_LAM * kSegFloats, tmap(tm->lm), x, y - 2, 1, b);
  }
};

using TmaRows2 = TmaRows<PsvTmaPlan, 6, 3>;

__device__ __forceinline__ LaneCols lane_cols2(const Geom& g, int strip, int lane, int& valid) {
  LaneCols L;
  const int own_lo = strip * kStripCols2;
  int j0 = own_lo;
  if (j0 + kStripCols2 > g.nz) j0 = g.nz > kStripCols2 ? ((g.nz - kStripCols2 + 3) & ~3) : 0;
  const int own_hi = min(g.nz, own_lo + kStripCols2);
  L.c0 = j0 - 8 + 4 * lane;
  L.own_lo = own_lo;
  L.own_hi = own_hi;
  L.zb = L.zf = L.own = 0;
  valid = 0;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const int c = L.c0 + e;
    if (c >= 2 && c < g.nz - 2) L.zb |= 1 << e;
    if (c >= 1 && c < g.nz - 2) L.zf |= 1 << e;
    if (c >= 0 && c < g.nz) valid |= 1 << e;
    if (lane >= 2 && lane <= 29 && c >= own_lo && c < own_hi) L.own |= 1 << e;
  }
  return L;
}

// Zero outside the grid: the whole row when it is not a grid row, else the
// lane's columns outside [0, nz).
__device__ __forceinline__ f4 in_grid(const f4& a, bool row_ok, int valid) {
  f4 o;
#pragma unroll
  for (int e = 0; e < 4; ++e) o.v[e] = (row_ok && (valid & (1 << e))) ? a.v[e] : 0.0f;
  return o;
}

// Sources of row i (stf_dsxz, fd2d.wgsl:344-352) added to the divergence.
__device__ __forceinline__ void inject_add(const InjectList& inj, int i, int c0, Cursor& cur, f4& dsx, f4& dsz) {
  inject_at<true, false, true>(inj, i, c0, cur, dsx, dsx, dsz);
}

// The stress divergence at a velocity row (div_sxz, fd2d.wgsl:309-317):
// x from the sigma_xx / sigma_xz rows a0..a3 / b0..b3, z from the current
// sigma_xz / sigma_zz rows cz / zz.  rx = 1/(8 dx) or 0, rz = 1/(8 dz) or 0
// (0 where the edge rule zeroes the derivative).
__device__ __forceinline__ void vel_div(const f4& a0, const f4& a1, const f4& a2, const f4& a3, const f4& b0,
                                        const f4& b1, const f4& b2, const f4& b3, const f4& cz, const f4& zz,
                                        float rx, const f4& rz, f4& dsx, f4& dsz) {
  const f4 ax = d4_rows(a0, a1, a2, a3), bx = d4_rows(b0, b1, b2, b3);
  const f4 cb = d4_cols_back(cz), zb = d4_cols_back(zz);
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    dsx.v[e] = fmaf(cb.v[e], rz.v[e], ax.v[e] * rx);
    dsz.v[e] = fmaf(zb.v[e], rz.v[e], bx.v[e] * rx);
  }
}

// Stress update of one row from the velocity rows u0..u3 (vx) and w0..w3 (vz)
// (div_vxz and add_sxz, fd2d.wgsl:378-381, 396-398): sxx += (l+2m) dvx/dx +
// l dvz/dz, szz += (l+2m) dvz/dz + l dvx/dx, sxz += m (dvx/dz + dvz/dx), with
// lam and mu holding dt*lambda and dt*mu.
__device__ __forceinline__ void stress(const f4& u0, const f4& u1, const f4& u2, const f4& u3, const f4& w0,
                                       const f4& w1, const f4& w2, const f4& w3, float rx, const f4& rz,
                                       const f4& lam, const f4& mu, const f4& xx, const f4& zz, const f4& xz,
                                       f4& oxx, f4& ozz, f4& oxz) {
  const f4 ux = d4_rows(u0, u1, u2, u3), wx = d4_rows(w0, w1, w2, w3);
  const f4 uz = d4_cols_fwd(u1), wz = d4_cols_fwd(w1);
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    const float l = lam.v[e], m = mu.v[e];
    const float dvxdx = ux.v[e] * rx, dvzdz = wz.v[e] * rz.v[e];
    const float l2m = fmaf(2.0f, m, l);
    oxx.v[e] = fmaf(l2m, dvxdx, fmaf(l, dvzdz, xx.v[e]));
    ozz.v[e] = fmaf(l2m, dvzdz, fmaf(l, dvxdx, zz.v[e]));
    oxz.v[e] = fmaf(m, fmaf(uz.v[e], rz.v[e], wx.v[e] * rx), xz.v[e]);
  }
}

// EDGE: derivatives masked by index and level-1 values outside the grid
// zeroed.  (A second, test-free instantiation for interior warps executed 17 %
// fewer instructions but ran 8 % slower: two bodies of this size no longer
// fit the instruction cache.)  MID: where p.vxm is set, the level-1 rows
// the warp owns are stored too (p.vxm .. p.sxzm: the state after step `it`,
// which a gradient keeps; a separate kernel, not a second body).
template <class Loader, bool EDGE, class M, bool MID = false>
__device__ __forceinline__ bool psv2_body(const PsvStep& p, const March& m, const LaneCols& L, int valid,
                                          unsigned char* smem, const M* tm) {
  const Geom& g = p.g;
  const size_t ld = size_t(g.ld);
  const float dt = g.dt;
  const int c0 = L.c0;
  const int nx = g.nx;
  auto at = [&](auto* base, int i) { return base + ptrdiff_t(i) * ptrdiff_t(ld) + c0; };

  typename Loader::SegsT segs;
  segs.base[P2_SXX] = p.sxx0; segs.roff[P2_SXX] = 1;
  segs.base[P2_SXZ] = p.sxz0; segs.roff[P2_SXZ] = 1;
  segs.base[P2_SZZ] = p.szz0; segs.roff[P2_SZZ] = 1;
  segs.base[P2_VX] = p.vx0; segs.roff[P2_VX] = 0;
  segs.base[P2_VZ] = p.vz0; segs.roff[P2_VZ] = 0;
  segs.base[P2_RHO] = p.rho; segs.roff[P2_RHO] = 0;
  segs.base[P2_LAM] = p.lam; segs.roff[P2_LAM] = -2;
  segs.base[P2_MU] = p.mu; segs.roff[P2_MU] = -2;
  const int i0 = m.ib - 4;                 // first level-1 row
  const int nk = (m.ie - m.ib) + 9;        // level-1 rows [ib-4, ie+4]
  float* buf = nullptr;
  uint64_t* bar = nullptr;
  if (Loader::kStages > 0) slice_ring<Loader>(smem, buf, bar);
  Loader rows(segs, ld, c0, i0 + 1, m.lane, buf, bar, nk);  // iteration k reads row i0 + k
  if constexpr (std::is_same<Loader, TmaRows<PsvTmaPlan, 6, 3, M>>::value) rows.tm = tm;
  rows.configure(g);
  rows.start();

  // Column taper product; difference factors 1/(8 dx) per row (0 where the
  // row derivative is zeroed) and 1/(8 dz) per column (0 where the column
  // derivative is zeroed).  rho, lam and mu hold dt/rho, dt*lambda, dt*mu.
  f4 tbt;
  {
    const f4 tb = ld4(p.taper_zb + c0), tt = ld4(p.taper_zt + c0);
#pragma unroll
    for (int e = 0; e < 4; ++e) tbt.v[e] = tb.v[e] * tt.v[e];
  }
  const float sxr = g.rdx, szr = g.rdz;
  // sigma^n rings, rows i-2..i+1
  f4 xx0 = ld4(at(p.sxx0, i0 - 2)), xx1 = ld4(at(p.sxx0, i0 - 1)), xx2 = ld4(at(p.sxx0, i0)), xx3;
  f4 xz0 = ld4(at(p.sxz0, i0 - 2)), xz1 = ld4(at(p.sxz0, i0 - 1)), xz2 = ld4(at(p.sxz0, i0)), xz3;
  // sigma_zz^n: row i (zz2, for the z difference); row i-2, which the stress
  // update adds to, is read from the stage kept three iterations back.
  f4 zz2 = ld4(at(p.szz0, i0)), zz3;
  const f4 z4 = {{0.0f, 0.0f, 0.0f, 0.0f}};
  f4 xa = z4, xb_ = z4, xc = z4, xd = z4, za = z4, zb_ = z4, zc = z4, zd = z4;  // level-1 v rows i-3..i
  f4 sx0 = z4, sx1 = z4, sx2 = z4, sx3 = z4;    // level-1 sxx rows i-5..i-2
  f4 sq0 = z4, sq1 = z4, sq2 = z4, sq3 = z4;    // level-1 sxz rows i-5..i-2
  f4 sz0 = z4, sz1 = z4, sz2 = z4, sz3 = z4;    // level-1 szz rows i-5..i-2
  f4 ua = z4, ub = z4, uc = z4, ud = z4, wa = z4, wb = z4, wc = z4, wd = z4;  // level-2 v rows i-6..i-3
  InjectList inj2 = p.inj;
  inj2.it = p.inj.it + 1;
  ProbeList pr2 = p.probes;
  pr2.it = p.probes.it + 1;
  Cursor ci1 = cursor_at(p.inj.list, p.inj.n, i0);
  Cursor ci2 = cursor_at(p.inj.list, p.inj.n, m.ib - 1);
  Cursor pi1 = cursor_at(p.probes.list, p.probes.n, m.ib);
  Cursor pi2 = pi1;
  f4 rzb, rzf;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    rzb.v[e] = (!EDGE || (L.zb & (1 << e))) ? szr : 0.0f;
    rzf.v[e] = (!EDGE || (L.zf & (1 << e))) ? szr : 0.0f;
  }
  // Some lane holds columns outside the grid: level-1 values there are zeroed.
  const bool cols_out = EDGE && !__all_sync(kFull, valid == 0xF);
  // Row taper of the two velocity rows of the next iteration (i + 1 and
  // i - 2), loaded one iteration ahead; rows down to -7 and up to nx + 5 lie
  // in the taper's halo.
  float bx1_next = __ldg(p.taper_x + i0), bx2_next = __ldg(p.taper_x + i0 - 3);

  for (int k = 0; k < nk; ++k) {
    const int i = i0 + k;
    const float bx1 = bx1_next, bx2 = bx2_next;
    bx1_next = __ldg(p.taper_x + i + 1);
    bx2_next = __ldg(p.taper_x + i - 2);
    if (!rows.acquire(k)) {
      flag_timeout(p.err);
      rows.drain(k);
      return false;
    }
    xx3 = rows.seg(P2_SXX);
    xz3 = rows.seg(P2_SXZ);
    zz3 = rows.seg(P2_SZZ);
    const f4 vxo = rows.seg(P2_VX);
    const f4 vzo = rows.seg(P2_VZ);
    const f4 rho = rows.seg(P2_RHO);
    const f4 lam = rows.seg(P2_LAM);
    const f4 mu = rows.seg(P2_MU);
    rows.release();

    // ---- level 1, velocity of row i (step it)
    {
      const float rx = (!EDGE || (i >= 2 && i < nx - 2)) ? sxr : 0.0f;
      f4 dsx, dsz;
      vel_div(xx0, xx1, xx2, xx3, xz0, xz1, xz2, xz3, xz2, zz2, rx, rzb, dsx, dsz);
      if (ci1.row == i) inject_add(p.inj, i, c0, ci1, dsx, dsz);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float bb = bx1 * tbt.v[e];
        xd.v[e] = bb * fmaf(dsx.v[e], rho.v[e], vxo.v[e]);
        zd.v[e] = bb * fmaf(dsz.v[e], rho.v[e], vzo.v[e]);
      }
      const bool row_ok = (i >= 0 && i < nx);
      if (EDGE && (!row_ok || cols_out)) {
        xd = in_grid(xd, row_ok, valid);
        zd = in_grid(zd, row_ok, valid);
      }
      if (i >= m.ib && i < m.ie) {
        if constexpr (MID) {
          if (p.vxm) {
            st4_masked(at(p.vxm, i), xd, L.own);
            st4_masked(at(p.vzm, i), zd, L.own);
          }
        }
        probe_at(p.probes, i, L, pi1, dt,
                 [&](int comp, int e) { return comp == kProbeVX ? pick4(xd, e) : pick4(zd, e); });
      }
    }

    // ---- level 1, stress of row i-2 (step it)
    if (k >= 3) {
      const int r = i - 2;
      const float rx = (!EDGE || (r >= 1 && r < nx - 2)) ? sxr : 0.0f;
      stress(xa, xb_, xc, xd, za, zb_, zc, zd, rx, rzf, lam, mu, xx0, rows.seg_back(P2_SZZ, 3), xz0, sx3, sz3, sq3);
      const bool row_ok = (r >= 0 && r < nx);
      if (EDGE && (!row_ok || cols_out)) {
        sx3 = in_grid(sx3, row_ok, valid);
        sz3 = in_grid(sz3, row_ok, valid);
        sq3 = in_grid(sq3, row_ok, valid);
      }
      if constexpr (MID) {
        if (p.vxm && r >= m.ib && r < m.ie) {
          st4_masked(at(p.sxxm, r), sx3, L.own);
          st4_masked(at(p.szzm, r), sz3, L.own);
          st4_masked(at(p.sxzm, r), sq3, L.own);
        }
      }
    }

    // ---- level 2, velocity of row i-3 (step it+1)
    if (k >= 6) {
      const int r = i - 3;
      const f4 rho2 = rows.seg_back(P2_RHO, 3);
      const float rx = (!EDGE || (r >= 2 && r < nx - 2)) ? sxr : 0.0f;
      f4 dsx, dsz;
      vel_div(sx0, sx1, sx2, sx3, sq0, sq1, sq2, sq3, sq2, sz2, rx, rzb, dsx, dsz);
      if (ci2.row == r) inject_add(inj2, r, c0, ci2, dsx, dsz);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float bb = bx2 * tbt.v[e];
        ud.v[e] = bb * fmaf(dsx.v[e], rho2.v[e], xa.v[e]);
        wd.v[e] = bb * fmaf(dsz.v[e], rho2.v[e], za.v[e]);
      }
      if (r >= m.ib && r < m.ie) {
        st4_masked(at(p.vx1, r), ud, L.own);
        st4_masked(at(p.vz1, r), wd, L.own);
        probe_at(pr2, r, L, pi2, dt,
                 [&](int comp, int e) { return comp == kProbeVX ? pick4(ud, e) : pick4(wd, e); });
      }
    }

    // ---- level 2, stress of row i-5 (step it+1)
    if (k >= 9) {
      const int r = i - 5;
      const f4 lam2 = rows.seg_back(P2_LAM, 3), mu2 = rows.seg_back(P2_MU, 3);
      const float rx = (!EDGE || (r >= 1 && r < nx - 2)) ? sxr : 0.0f;
      f4 sxx, szz, sxz;
      stress(ua, ub, uc, ud, wa, wb, wc, wd, rx, rzf, lam2, mu2, sx0, sz0, sq0, sxx, szz, sxz);
      st4_masked(at(p.sxx1, r), sxx, L.own);
      st4_masked(at(p.szz1, r), szz, L.own);
      st4_masked(at(p.sxz1, r), sxz, L.own);
    }

    ua = ub; ub = uc; uc = ud;
    wa = wb; wb = wc; wc = wd;
    sx0 = sx1; sx1 = sx2; sx2 = sx3;
    sq0 = sq1; sq1 = sq2; sq2 = sq3;
    sz0 = sz1; sz1 = sz2; sz2 = sz3;
    xa = xb_; xb_ = xc; xc = xd;
    za = zb_; zb_ = zc; zc = zd;
    xx0 = xx1; xx1 = xx2; xx2 = xx3;
    xz0 = xz1; xz1 = xz2; xz2 = xz3;
    zz2 = zz3;
  }
  return true;
}

template <class Loader, class M = Tma2, bool MID = false>
__device__ __forceinline__ bool psv2_march(const PsvStep& p, int gw, unsigned char* smem,
                                           const M* tm = nullptr) {
  const March m = march_of(p.g, gw);
  if (!m.active) return true;
  int valid;
  const LaneCols L = lane_cols2(p.g, m.strip, m.lane, valid);
  return psv2_body<Loader, true, M, MID>(p, m, L, valid, smem, tm);
}

// --------------------------------------------------------------------------
// SH, two time steps per pass: the PSV scheme above with the SH update
// (fd2d.wgsl:242-301): level 1 velocity of row i and stress of row i-2,
// level 2 velocity of row i-3 and stress of row i-5; 16 B of HBM traffic per
// cell-update instead of 32.
// --------------------------------------------------------------------------
enum Sh2Seg {
  S2_SXY = 0, S2_SZY,  // sigma^n, row i+1
  S2_VY,               // v^n, row i
  S2_RHO, S2_MU,       // 1/rho row i, mu row i-2
  S2_NSEG
};

// SH: sigma^n (sxy, szy; row i+1; the state's fields vy, sxy, szy), v^n (vy;
// row i), 1/rho (row i) and mu (row i-2) of the material's 1/rho, lambda, mu.
struct ShTmaPlan {
  using Maps = Tma2;
  static constexpr int NSEG = S2_NSEG;
  template <class M>
  __device__ __forceinline__ static void issue(float* sb, const M* tm, int x, int y, uint64_t* b) {
    tma3(sb + S2_SXY * kSegFloats, tmap(tm->sig), x, y + 1, 1, b);
    tma3(sb + S2_VY * kSegFloats, tmap(tm->vel), x, y, 0, b);
    tma3(sb + S2_RHO * kSegFloats, tmap(tm->rho), x, y, 0, b);
    tma3(sb + S2_MU * kSegFloats, tmap(tm->rho), x, y - 2, 2, b);
  }
};

// Six stages: two rows in flight, the last three iterations kept (level 2
// reads 1/rho of row i-3 and mu of row i-5 from them); lane q issues the
// copy of segment q (288 against 265 Gcell-updates/s with lane 0 issuing
// all five).
struct ShBulk2 : BulkRows<S2_NSEG, 6, true, 3> {
  using SegsT = Segs<S2_NSEG>;
  using BulkRows<S2_NSEG, 6, true, 3>::BulkRows;
};

// Sources of row i (stf_dsy, fd2d.wgsl:253-260) added to the divergence.
__device__ __forceinline__ void inject_add_y(const InjectList& inj, int i, int c0, Cursor& cur, f4& ds) {
  inject_at<false, true, false>(inj, i, c0, cur, ds, ds, ds);
}

// MID: where p.vym is set, the level-1 rows the warp owns are stored too
// (p.vym, p.sxym, p.szym).
template <class Loader, class M, bool MID = false>
__device__ __forceinline__ bool sh2_body(const ShStep& p, const March& m, const LaneCols& L, int valid,
                                         unsigned char* smem, const M* tm) {
  const Geom& g = p.g;
  const size_t ld = size_t(g.ld);
  const float dt = g.dt;
  const int c0 = L.c0;
  const int nx = g.nx;
  auto at = [&](auto* base, int i) { return base + ptrdiff_t(i) * ptrdiff_t(ld) + c0; };

  typename Loader::SegsT segs;
  segs.base[S2_SXY] = p.sxy0; segs.roff[S2_SXY] = 1;
  segs.base[S2_SZY] = p.szy0; segs.roff[S2_SZY] = 1;
  segs.base[S2_VY] = p.vy0; segs.roff[S2_VY] = 0;
  segs.base[S2_RHO] = p.rho; segs.roff[S2_RHO] = 0;
  segs.base[S2_MU] = p.mu; segs.roff[S2_MU] = -2;
  const int i0 = m.ib - 4;                 // first level-1 row
  const int nk = (m.ie - m.ib) + 9;        // level-1 rows [ib-4, ie+4]
  float* buf = nullptr;
  uint64_t* bar = nullptr;
  if (Loader::kStages > 0) slice_ring<Loader>(smem, buf, bar);
  Loader rows(segs, ld, c0, i0 + 1, m.lane, buf, bar, nk);  // iteration k reads row i0 + k
  if constexpr (std::is_same<Loader, TmaRows<ShTmaPlan, 6, 3, M>>::value) rows.tm = tm;
  rows.configure(g);
  rows.start();

  f4 tbt;
  {
    const f4 tb = ld4(p.taper_zb + c0), tt = ld4(p.taper_zt + c0);
#pragma unroll
    for (int e = 0; e < 4; ++e) tbt.v[e] = tb.v[e] * tt.v[e];
  }
  const float sxr = g.rdx, szr = g.rdz;
  // sigma^n rings, rows i-2..i+1
  f4 xy0 = ld4(at(p.sxy0, i0 - 2)), xy1 = ld4(at(p.sxy0, i0 - 1)), xy2 = ld4(at(p.sxy0, i0)), xy3;
  // sigma_zy^n: row i (zy2, for the z difference); row i-2, which the stress
  // update adds to, is read from the stage kept three iterations back.
  f4 zy2 = ld4(at(p.szy0, i0)), zy3;
  const f4 z4 = {{0.0f, 0.0f, 0.0f, 0.0f}};
  f4 va = z4, vb = z4, vc = z4, vd = z4;        // level-1 vy rows i-3..i
  f4 sx0 = z4, sx1 = z4, sx2 = z4, sx3 = z4;    // level-1 sxy rows i-5..i-2
  f4 sz0 = z4, sz1 = z4, sz2 = z4, sz3 = z4;    // level-1 szy rows i-5..i-2
  f4 ua = z4, ub = z4, uc = z4, ud = z4;        // level-2 vy rows i-6..i-3
  InjectList inj2 = p.inj;
  inj2.it = p.inj.it + 1;
  ProbeList pr2 = p.probes;
  pr2.it = p.probes.it + 1;
  Cursor ci1 = cursor_at(p.inj.list, p.inj.n, i0);
  Cursor ci2 = cursor_at(p.inj.list, p.inj.n, m.ib - 1);
  Cursor pi1 = cursor_at(p.probes.list, p.probes.n, m.ib);
  Cursor pi2 = pi1;
  f4 rzb, rzf;
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    rzb.v[e] = (L.zb & (1 << e)) ? szr : 0.0f;
    rzf.v[e] = (L.zf & (1 << e)) ? szr : 0.0f;
  }
  const bool cols_out = !__all_sync(kFull, valid == 0xF);
  float bx1_next = __ldg(p.taper_x + i0), bx2_next = __ldg(p.taper_x + i0 - 3);

  for (int k = 0; k < nk; ++k) {
    const int i = i0 + k;
    const float bx1 = bx1_next, bx2 = bx2_next;
    bx1_next = __ldg(p.taper_x + i + 1);
    bx2_next = __ldg(p.taper_x + i - 2);
    if (!rows.acquire(k)) {
      flag_timeout(p.err);
      rows.drain(k);
      return false;
    }
    xy3 = rows.seg(S2_SXY);
    zy3 = rows.seg(S2_SZY);
    const f4 vo = rows.seg(S2_VY);
    const f4 rho = rows.seg(S2_RHO);
    const f4 mu = rows.seg(S2_MU);
    rows.release();

    // ---- level 1, velocity of row i (step it): div_sy, source, add_vy
    {
      const float rx = (i >= 2 && i < nx - 2) ? sxr : 0.0f;
      const f4 ax = d4_rows(xy0, xy1, xy2, xy3), az = d4_cols_back(zy2);
      f4 ds;
#pragma unroll
      for (int e = 0; e < 4; ++e) ds.v[e] = fmaf(az.v[e], rzb.v[e], ax.v[e] * rx);
      if (ci1.row == i) inject_add_y(p.inj, i, c0, ci1, ds);
#pragma unroll
      for (int e = 0; e < 4; ++e) vd.v[e] = (bx1 * tbt.v[e]) * fmaf(ds.v[e], rho.v[e], vo.v[e]);
      const bool row_ok = (i >= 0 && i < nx);
      if (!row_ok || cols_out) vd = in_grid(vd, row_ok, valid);
      if (i >= m.ib && i < m.ie) {
        if constexpr (MID) {
          if (p.vym) st4_masked(at(p.vym, i), vd, L.own);
        }
        probe_at(p.probes, i, L, pi1, dt, [&](int, int e) { return pick4(vd, e); });
      }
    }

    // ---- level 1, stress of row i-2 (step it): div_vy, add_sy_sh
    if (k >= 3) {
      const int r = i - 2;
      const float rx = (r >= 1 && r < nx - 2) ? sxr : 0.0f;
      const f4 gx = d4_rows(va, vb, vc, vd), gz = d4_cols_fwd(vb);
      const f4 zy0 = rows.seg_back(S2_SZY, 3);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        sx3.v[e] = fmaf(mu.v[e], gx.v[e] * rx, xy0.v[e]);
        sz3.v[e] = fmaf(mu.v[e], gz.v[e] * rzf.v[e], zy0.v[e]);
      }
      const bool row_ok = (r >= 0 && r < nx);
      if (!row_ok || cols_out) {
        sx3 = in_grid(sx3, row_ok, valid);
        sz3 = in_grid(sz3, row_ok, valid);
      }
      if constexpr (MID) {
        if (p.vym && r >= m.ib && r < m.ie) {
          st4_masked(at(p.sxym, r), sx3, L.own);
          st4_masked(at(p.szym, r), sz3, L.own);
        }
      }
    }

    // ---- level 2, velocity of row i-3 (step it+1)
    if (k >= 6) {
      const int r = i - 3;
      const f4 rho2 = rows.seg_back(S2_RHO, 3);
      const float rx = (r >= 2 && r < nx - 2) ? sxr : 0.0f;
      const f4 ax = d4_rows(sx0, sx1, sx2, sx3), az = d4_cols_back(sz2);
      f4 ds;
#pragma unroll
      for (int e = 0; e < 4; ++e) ds.v[e] = fmaf(az.v[e], rzb.v[e], ax.v[e] * rx);
      if (ci2.row == r) inject_add_y(inj2, r, c0, ci2, ds);
#pragma unroll
      for (int e = 0; e < 4; ++e) ud.v[e] = (bx2 * tbt.v[e]) * fmaf(ds.v[e], rho2.v[e], va.v[e]);
      if (r >= m.ib && r < m.ie) {
        st4_masked(at(p.vy1, r), ud, L.own);
        probe_at(pr2, r, L, pi2, dt, [&](int, int e) { return pick4(ud, e); });
      }
    }

    // ---- level 2, stress of row i-5 (step it+1)
    if (k >= 9) {
      const int r = i - 5;
      const f4 mu2 = rows.seg_back(S2_MU, 3);
      const float rx = (r >= 1 && r < nx - 2) ? sxr : 0.0f;
      const f4 gx = d4_rows(ua, ub, uc, ud), gz = d4_cols_fwd(ub);
      f4 sxy, szy;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        sxy.v[e] = fmaf(mu2.v[e], gx.v[e] * rx, sx0.v[e]);
        szy.v[e] = fmaf(mu2.v[e], gz.v[e] * rzf.v[e], sz0.v[e]);
      }
      st4_masked(at(p.sxy1, r), sxy, L.own);
      st4_masked(at(p.szy1, r), szy, L.own);
    }

    ua = ub; ub = uc; uc = ud;
    sx0 = sx1; sx1 = sx2; sx2 = sx3;
    sz0 = sz1; sz1 = sz2; sz2 = sz3;
    va = vb; vb = vc; vc = vd;
    xy0 = xy1; xy1 = xy2; xy2 = xy3;
    zy2 = zy3;
  }
  return true;
}

template <class Loader, class M = Tma2, bool MID = false>
__device__ __forceinline__ bool sh2_march(const ShStep& p, int gw, unsigned char* smem, const M* tm = nullptr) {
  const March m = march_of(p.g, gw);
  if (!m.active) return true;
  int valid;
  const LaneCols L = lane_cols2(p.g, m.strip, m.lane, valid);
  return sh2_body<Loader, M, MID>(p, m, L, valid, smem, tm);
}

}  // namespace
}  // namespace seiswg
