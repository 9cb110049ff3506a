// fd_adjoint_march.cuh -- the reverse-step marches of the exact discrete
// adjoint (fd_adjoint.cu has the derivation and the kernels).  Included by
// the kernels of fd_adjoint.cu and by the batch's queue kernel
// (fd_queue.cu); both are built with multiply-add contraction.
#pragma once

#include <type_traits>

#include "fd_march.cuh"
#include "fd_tma.cuh"

namespace seiswg {
namespace {

// -fd4(a, b, c, d): the transposed difference (taps already masked).
__device__ __forceinline__ float nfd4(float a, float b, float c, float d, float r) {
  return -((9.0f * (c - b) - (d - a)) * r);
}

__device__ __forceinline__ f4 masked(const f4& a, int bits) {
  f4 o;
#pragma unroll
  for (int e = 0; e < 4; ++e) o.v[e] = (bits & (1 << e)) ? a.v[e] : 0.0f;
  return o;
}

__device__ __forceinline__ f4 scaled(const f4& a, bool keep) {
  f4 o;
#pragma unroll
  for (int e = 0; e < 4; ++e) o.v[e] = keep ? a.v[e] : 0.0f;
  return o;
}

// Transposed x differences over a ring of masked rows (oldest first).
__device__ __forceinline__ f4 dxT(const f4& r0, const f4& r1, const f4& r2, const f4& r3, float r) {
  f4 o;
#pragma unroll
  for (int e = 0; e < 4; ++e) o.v[e] = nfd4(r0.v[e], r1.v[e], r2.v[e], r3.v[e], r);
  return o;
}

// Transposed z differences of a masked lane float4: back taps (c-2..c+1)
// for (D+)^T, forward taps (c-1..c+2) for (D-)^T.
__device__ __forceinline__ f4 dzT_back(const f4& m, float r) {
  const float pz = __shfl_up_sync(kFull, m.v[2], 1);
  const float pw = __shfl_up_sync(kFull, m.v[3], 1);
  const float nx = __shfl_down_sync(kFull, m.v[0], 1);
  f4 o;
  o.v[0] = nfd4(pz, pw, m.v[0], m.v[1], r);
  o.v[1] = nfd4(pw, m.v[0], m.v[1], m.v[2], r);
  o.v[2] = nfd4(m.v[0], m.v[1], m.v[2], m.v[3], r);
  o.v[3] = nfd4(m.v[1], m.v[2], m.v[3], nx, r);
  return o;
}

__device__ __forceinline__ f4 dzT_fwd(const f4& m, float r) {
  const float pw = __shfl_up_sync(kFull, m.v[3], 1);
  const float n0 = __shfl_down_sync(kFull, m.v[0], 1);
  const float n1 = __shfl_down_sync(kFull, m.v[1], 1);
  f4 o;
  o.v[0] = nfd4(pw, m.v[0], m.v[1], m.v[2], r);
  o.v[1] = nfd4(m.v[0], m.v[1], m.v[2], m.v[3], r);
  o.v[2] = nfd4(m.v[1], m.v[2], m.v[3], n0, r);
  o.v[3] = nfd4(m.v[2], m.v[3], n0, n1, r);
  return o;
}

__device__ __forceinline__ bool mask_back(int i, int n) { return i >= 2 && i < n - 2; }  // D-
__device__ __forceinline__ bool mask_fwd(int i, int n) { return i >= 1 && i < n - 2; }   // D+

struct AMarch {
  int lane, warp, strip, chunk, ib, ie;
  bool active;
};

__device__ __forceinline__ AMarch amarch(const Geom& g, int gw) {
  AMarch m;
  m.lane = threadIdx.x & 31;
  m.warp = threadIdx.x >> 5;
  m.strip = gw % g.nstrips;
  m.chunk = gw / g.nstrips;
  m.active = m.chunk < g.nchunks;
  m.ib = m.chunk * g.lx;
  m.ie = min(g.nx, m.ib + g.lx);
  return m;
}

template <class Loader>
__device__ __forceinline__ Loader make_aloader(const typename Loader::SegsT& segs, const Geom& g, const AMarch& m,
                                               const LaneCols& L, unsigned char* slice) {
  float* buf = nullptr;
  uint64_t* bar = nullptr;
  if (Loader::kStages > 0) slice_ring<Loader>(slice, buf, bar);
  return Loader(segs, size_t(g.ld), L.c0, m.ib, m.lane, buf, bar, m.ie - m.ib + 3);
}

template <int NSEG>
struct ADirect : DirectRows<NSEG> {
  using SegsT = Segs<NSEG>;
  static constexpr uint32_t kStageBytes = 0;
  using DirectRows<NSEG>::DirectRows;
};

// The reverse step reads 12 (SH) or 19 (PSV) segments per row: their copies
// are issued one per lane.
template <int NSEG>
struct ABulk : BulkRows<NSEG, kAdjStages, true> {
  using SegsT = Segs<NSEG>;
  using BulkRows<NSEG, kAdjStages, true>::BulkRows;
};

__device__ __forceinline__ void flag(int* err) {
  if ((threadIdx.x & 31) == 0 && err) atomicOr(err, kErrWaitTimeout);
}


// --------------------------------------------------------------------------
// PSV
// --------------------------------------------------------------------------
enum PsvAdjSeg {
  PA_SXX = 0, PA_SXZ, PA_SZZ, PA_VX, PA_VZ,      // forward state S^n
  PA_BXX, PA_BZZ, PA_BXZ,                         // adjoint stress s^{n+1}, row i+1
  PA_WX, PA_WZ,                                   // adjoint velocity w^{n+1}, row i
  PA_OXX, PA_OZZ, PA_OXZ,                         // adjoint stress s^{n+1}, row i-2
  PA_B, PA_LAM, PA_MU,                            // 1/rho (row i), lambda, mu (row i+1)
  PA_GB, PA_GL, PA_GM,                            // gradients: g_B (row i), g_lambda, g_mu (row i-2)
  PA_NSEG
};

// Tensor copies of a PSV reverse-step row: eleven copies for the nineteen
// segments (the forward sigma_xx, sigma_xz of row i+1 and sigma_zz of row i
// one field each, the forward v, the incoming adjoint stresses of rows i+1
// and i-2 and velocities of row i, the material, the gradients).
struct AdjTmaPlan {
  using Maps = TmaAdj;
  static constexpr int NSEG = PA_NSEG;
  template <class M>
  __device__ __forceinline__ static void issue(float* sb, const M* tm, int x, int y, uint64_t* b) {
    tma3(sb + PA_SXX * kSegFloats, tmap(tm->f1), x, y + 1, 2, b);
    tma3(sb + PA_SXZ * kSegFloats, tmap(tm->f1), x, y + 1, 4, b);
    tma3(sb + PA_SZZ * kSegFloats, tmap(tm->f1), x, y, 3, b);
    tma3(sb + PA_VX * kSegFloats, tmap(tm->f2), x, y, 0, b);
    tma3(sb + PA_BXX * kSegFloats, tmap(tm->a3), x, y + 1, 2, b);
    tma3(sb + PA_WX * kSegFloats, tmap(tm->a2), x, y, 0, b);
    tma3(sb + PA_OXX * kSegFloats, tmap(tm->a3), x, y - 2, 2, b);
    tma3(sb + PA_B * kSegFloats, tmap(tm->m1), x, y, 0, b);
    tma3(sb + PA_LAM * kSegFloats, tmap(tm->m2), x, y + 1, 1, b);
    tma3(sb + PA_GB * kSegFloats, tmap(tm->g1), x, y, 2, b);
    tma3(sb + PA_GL * kSegFloats, tmap(tm->g2), x, y - 2, 0, b);
  }
};
using ATma = TmaRows<AdjTmaPlan, kAdjStages, 0>;

template <class Loader, class M = TmaAdj>
__device__ __forceinline__ bool psv_adjoint_march(const PsvAdjoint& p, int gw, unsigned char* smem,
                                                  const M* tm = nullptr) {
  const Geom& g = p.g;
  const AMarch m = amarch(g, gw);
  if (!m.active) return true;
  const LaneCols L = lane_cols(g, m.strip, m.lane);
  const size_t ld = size_t(g.ld);
  const float dt = g.dt;
  const int c0 = L.c0;
  auto at = [&](auto* base, int i) { return base + ptrdiff_t(i) * ptrdiff_t(ld) + c0; };

  typename Loader::SegsT segs;
  segs.base[PA_SXX] = p.sxx; segs.roff[PA_SXX] = 1;
  segs.base[PA_SXZ] = p.sxz; segs.roff[PA_SXZ] = 1;
  segs.base[PA_SZZ] = p.szz; segs.roff[PA_SZZ] = 0;
  segs.base[PA_VX] = p.vx; segs.roff[PA_VX] = 0;
  segs.base[PA_VZ] = p.vz; segs.roff[PA_VZ] = 0;
  segs.base[PA_BXX] = p.bxx0; segs.roff[PA_BXX] = 1;
  segs.base[PA_BZZ] = p.bzz0; segs.roff[PA_BZZ] = 1;
  segs.base[PA_BXZ] = p.bxz0; segs.roff[PA_BXZ] = 1;
  segs.base[PA_WX] = p.wx0; segs.roff[PA_WX] = 0;
  segs.base[PA_WZ] = p.wz0; segs.roff[PA_WZ] = 0;
  segs.base[PA_OXX] = p.bxx0; segs.roff[PA_OXX] = -2;
  segs.base[PA_OZZ] = p.bzz0; segs.roff[PA_OZZ] = -2;
  segs.base[PA_OXZ] = p.bxz0; segs.roff[PA_OXZ] = -2;
  segs.base[PA_B] = p.rho; segs.roff[PA_B] = 0;
  segs.base[PA_LAM] = p.lam; segs.roff[PA_LAM] = 1;
  segs.base[PA_MU] = p.mu; segs.roff[PA_MU] = 1;
  segs.base[PA_GB] = p.g_b; segs.roff[PA_GB] = 0;
  segs.base[PA_GL] = p.g_lam; segs.roff[PA_GL] = -2;
  segs.base[PA_GM] = p.g_mu; segs.roff[PA_GM] = -2;
  Loader rows = make_aloader<Loader>(segs, g, m, L, smem);
  if constexpr (std::is_same<Loader, TmaRows<AdjTmaPlan, kAdjStages, 0, M>>::value) rows.tm = tm;
  rows.configure(g);
  rows.start();

  const f4 tb = ld4(p.taper_zb + c0), tt = ld4(p.taper_zt + c0);
  const f4 rzb = masked_recip(g.rdz, L.zb), rzf = masked_recip(g.rdz, L.zf);
  // Adjoint strains e = dt C s (unmasked) for rows of the ring.
  auto strain_adj = [&](const f4& bxx, const f4& bzz, const f4& bxz, const f4& lam, const f4& mu, f4& exx,
                        f4& ezz, f4& exz) {
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float l = lam.v[e], mm = mu.v[e];
      exx.v[e] = dt * ((l + 2.0f * mm) * bxx.v[e] + l * bzz.v[e]);
      ezz.v[e] = dt * (l * bxx.v[e] + (l + 2.0f * mm) * bzz.v[e]);
      exz.v[e] = dt * mm * bxz.v[e];
    }
  };

  // Prologue rings: forward sxx, sxz rows ib-3..ib-1; adjoint strains of rows ib-3..ib-1.
  f4 xx0 = ld4(at(p.sxx, m.ib - 3)), xx1 = ld4(at(p.sxx, m.ib - 2)), xx2 = ld4(at(p.sxx, m.ib - 1)), xx3;
  f4 xz0 = ld4(at(p.sxz, m.ib - 3)), xz1 = ld4(at(p.sxz, m.ib - 2)), xz2 = ld4(at(p.sxz, m.ib - 1)), xz3;
  f4 ex0, ex1, ex2, ex3;   // e_xx rows i-2..i+1
  f4 eq0, eq1, eq2, eq3;   // e_xz rows i-2..i+1
  f4 ezc, ezn;             // e_zz rows i, i+1
  {
    f4 dummy;
    strain_adj(ld4(at(p.bxx0, m.ib - 3)), ld4(at(p.bzz0, m.ib - 3)), ld4(at(p.bxz0, m.ib - 3)),
               ld4(at(p.lam, m.ib - 3)), ld4(at(p.mu, m.ib - 3)), ex0, dummy, eq0);
    strain_adj(ld4(at(p.bxx0, m.ib - 2)), ld4(at(p.bzz0, m.ib - 2)), ld4(at(p.bxz0, m.ib - 2)),
               ld4(at(p.lam, m.ib - 2)), ld4(at(p.mu, m.ib - 2)), ex1, dummy, eq1);
    strain_adj(ld4(at(p.bxx0, m.ib - 1)), ld4(at(p.bzz0, m.ib - 1)), ld4(at(p.bxz0, m.ib - 1)),
               ld4(at(p.lam, m.ib - 1)), ld4(at(p.mu, m.ib - 1)), ex2, ezn, eq2);
  }
  f4 na, nb, nc, nd;   // recomputed forward vx^{n+1}, rows i-3..i
  f4 za, zb, zc, zd;   // recomputed forward vz^{n+1}
  f4 qxa, qxb, qxc, qxd;  // q = dt B w (x), rows i-3..i
  f4 qza, qzb, qzc, qzd;  // q (z)
  // Source and receiver list cursors; the row taper one iteration ahead
  // (rows up to ie + 2 lie in the taper's halo).
  Cursor cs = cursor_at(p.src.list, p.src.n, m.ib - 1);
  Cursor cr = cursor_at(p.rec.list, p.rec.n, m.ib - 1);
  const int nk = m.ie - m.ib + 3;
  float bx_next = __ldg(p.taper_x + m.ib - 1);

  for (int k = 0; k < nk; ++k) {
    const int i = m.ib - 1 + k;
    const float bxi = bx_next;
    bx_next = __ldg(p.taper_x + i + 1);
    if (!rows.acquire(k)) {
      flag(p.err);
      rows.drain(k);
      return false;
    }
    xx3 = rows.seg(PA_SXX);
    xz3 = rows.seg(PA_SXZ);
    const f4 szz_i = rows.seg(PA_SZZ);
    const f4 vx_i = rows.seg(PA_VX), vz_i = rows.seg(PA_VZ);
    ezc = ezn;
    {
      f4 e1, e2, e3;
      strain_adj(rows.seg(PA_BXX), rows.seg(PA_BZZ), rows.seg(PA_BXZ), rows.seg(PA_LAM), rows.seg(PA_MU), e1, e2,
                 e3);
      ex3 = e1;
      ezn = e2;
      eq3 = e3;
    }
    f4 wx = rows.seg(PA_WX), wz = rows.seg(PA_WZ);
    const f4 oxx = rows.seg(PA_OXX), ozz = rows.seg(PA_OZZ), oxz = rows.seg(PA_OXZ);
    const f4 buoy = rows.seg(PA_B);
    f4 gb = rows.seg(PA_GB);
    f4 gl = rows.seg(PA_GL), gm = rows.seg(PA_GM);
    rows.release();
    const float rxb = mask_back(i, g.nx) ? g.rdx : 0.0f;

    // Forward recompute: D- sigma^n + f^n and v^{n+1} of row i.
    f4 dsx = dx4r(xx0, xx1, xx2, xx3, rxb);
    f4 dsz = dx4r(xz0, xz1, xz2, xz3, rxb);
    {
      const f4 a = dz_back_r(xz2, rzb);
      const f4 b = dz_back_r(szz_i, rzb);
#pragma unroll
      for (int e = 0; e < 4; ++e) { dsx.v[e] = dsx.v[e] + a.v[e]; dsz.v[e] = dsz.v[e] + b.v[e]; }
    }
    inject_at<true, false, true>(p.src, i, c0, cs, dsx, dsx, dsz);
    f4 bb;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      bb.v[e] = (bxi * tb.v[e]) * tt.v[e];
      nd.v[e] = bb.v[e] * (vx_i.v[e] + dt * dsx.v[e] * buoy.v[e]);
      zd.v[e] = bb.v[e] * (vz_i.v[e] + dt * dsz.v[e] * buoy.v[e]);
    }

    // Adjoint velocity of row i: Vbar = w + dt U (receivers) + (D+)^T e.
    {
      const bool m0 = mask_fwd(i - 2, g.nx), m1 = mask_fwd(i - 1, g.nx), m2 = mask_fwd(i, g.nx),
                 m3 = mask_fwd(i + 1, g.nx);
      f4 tx, tzx;
      if (m0 && m1 && m2 && m3) {  // interior rows (uniform over the warp): no row masks
        tx = dxT(ex0, ex1, ex2, ex3, g.rdx);
        tzx = dxT(eq0, eq1, eq2, eq3, g.rdx);
      } else {
        tx = dxT(scaled(ex0, m0), scaled(ex1, m1), scaled(ex2, m2), scaled(ex3, m3), g.rdx);
        tzx = dxT(scaled(eq0, m0), scaled(eq1, m1), scaled(eq2, m2), scaled(eq3, m3), g.rdx);
      }
      const f4 tq = dzT_back(masked(eq2, L.zf), g.rdz);
      const f4 tz = dzT_back(masked(ezc, L.zf), g.rdz);
      inject_at<true, false, true>(p.rec, i, c0, cr, wx, wx, wz);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        wx.v[e] = bb.v[e] * (wx.v[e] + tx.v[e] + tq.v[e]);
        wz.v[e] = bb.v[e] * (wz.v[e] + tz.v[e] + tzx.v[e]);
        qxd.v[e] = dt * buoy.v[e] * wx.v[e];
        qzd.v[e] = dt * buoy.v[e] * wz.v[e];
      }
    }
    if (i >= m.ib && i < m.ie) {
      st4_masked(at(p.wx1, i), wx, L.own);
      st4_masked(at(p.wz1, i), wz, L.own);
#pragma unroll
      for (int e = 0; e < 4; ++e) gb.v[e] = gb.v[e] + dt * (wx.v[e] * dsx.v[e] + wz.v[e] * dsz.v[e]);
      st4_masked(at(p.g_b, i), gb, L.own);
    }

    // Adjoint stress of row r = i-2 and the lambda/mu gradients there.
    if (i >= m.ib + 2) {
      const int r = i - 2;
      const float rxf = mask_fwd(r, g.nx) ? g.rdx : 0.0f;
      const f4 exx = dx4r(na, nb, nc, nd, rxf);
      const f4 ezx = dx4r(za, zb, zc, zd, rxf);
      const f4 exz = dz_fwd_r(nb, rzf);
      const f4 ezz = dz_fwd_r(zb, rzf);
      const bool m0 = mask_back(r - 1, g.nx), m1 = mask_back(r, g.nx), m2 = mask_back(r + 1, g.nx),
                 m3 = mask_back(r + 2, g.nx);
      f4 ax, az;
      if (m0 && m1 && m2 && m3) {
        ax = dxT(qxa, qxb, qxc, qxd, g.rdx);
        az = dxT(qza, qzb, qzc, qzd, g.rdx);
      } else {
        ax = dxT(scaled(qxa, m0), scaled(qxb, m1), scaled(qxc, m2), scaled(qxd, m3), g.rdx);
        az = dxT(scaled(qza, m0), scaled(qzb, m1), scaled(qzc, m2), scaled(qzd, m3), g.rdx);
      }
      const f4 bx = dzT_fwd(masked(qxb, L.zb), g.rdz);
      const f4 bz = dzT_fwd(masked(qzb, L.zb), g.rdz);
      f4 sxx, szz, sxz;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        sxx.v[e] = oxx.v[e] + ax.v[e];
        szz.v[e] = ozz.v[e] + bz.v[e];
        sxz.v[e] = oxz.v[e] + (bx.v[e] + az.v[e]);
        // Explicitly rounded operations: the march is inlined into several
        // kernels (bulk or tensor-copy rows, plain or grouped), and left to
        // contraction the sums could round differently in each.
        gl.v[e] = fmaf(__fmul_rn(dt, __fadd_rn(oxx.v[e], ozz.v[e])), __fadd_rn(exx.v[e], ezz.v[e]), gl.v[e]);
        const float shear = __fmul_rn(oxz.v[e], __fadd_rn(exz.v[e], ezx.v[e]));
        const float dev = fmaf(2.0f * oxx.v[e], exx.v[e], fmaf(2.0f * ozz.v[e], ezz.v[e], shear));
        gm.v[e] = fmaf(dt, dev, gm.v[e]);
      }
      st4_masked(at(p.bxx1, r), sxx, L.own);
      st4_masked(at(p.bzz1, r), szz, L.own);
      st4_masked(at(p.bxz1, r), sxz, L.own);
      st4_masked(at(p.g_lam, r), gl, L.own);
      st4_masked(at(p.g_mu, r), gm, L.own);
    }

    na = nb; nb = nc; nc = nd;
    za = zb; zb = zc; zc = zd;
    qxa = qxb; qxb = qxc; qxc = qxd;
    qza = qzb; qzb = qzc; qzc = qzd;
    xx0 = xx1; xx1 = xx2; xx2 = xx3;
    xz0 = xz1; xz1 = xz2; xz2 = xz3;
    ex0 = ex1; ex1 = ex2; ex2 = ex3;
    eq0 = eq1; eq1 = eq2; eq2 = eq3;
  }
  return true;
}

// --------------------------------------------------------------------------
// SH
// --------------------------------------------------------------------------
enum ShAdjSeg {
  SA_SXY = 0, SA_SZY, SA_VY,   // forward state S^n: sxy (row i+1), szy (row i), vy (row i)
  SA_BXY, SA_BZY,              // adjoint stress s^{n+1}, row i+1
  SA_W,                        // adjoint velocity w^{n+1}, row i
  SA_OXY, SA_OZY,              // adjoint stress s^{n+1}, row i-2
  SA_B, SA_MU,                 // 1/rho (row i), mu (row i+1)
  SA_GB, SA_GM,                // g_B (row i), g_mu (row i-2)
  SA_NSEG
};

template <class Loader>
__device__ __forceinline__ bool sh_adjoint_march(const ShAdjoint& p, int gw, unsigned char* smem) {
  const Geom& g = p.g;
  const AMarch m = amarch(g, gw);
  if (!m.active) return true;
  const LaneCols L = lane_cols(g, m.strip, m.lane);
  const size_t ld = size_t(g.ld);
  const float dt = g.dt;
  const int c0 = L.c0;
  auto at = [&](auto* base, int i) { return base + ptrdiff_t(i) * ptrdiff_t(ld) + c0; };

  typename Loader::SegsT segs;
  segs.base[SA_SXY] = p.sxy; segs.roff[SA_SXY] = 1;
  segs.base[SA_SZY] = p.szy; segs.roff[SA_SZY] = 0;
  segs.base[SA_VY] = p.vy; segs.roff[SA_VY] = 0;
  segs.base[SA_BXY] = p.bxy0; segs.roff[SA_BXY] = 1;
  segs.base[SA_BZY] = p.bzy0; segs.roff[SA_BZY] = 1;
  segs.base[SA_W] = p.w0; segs.roff[SA_W] = 0;
  segs.base[SA_OXY] = p.bxy0; segs.roff[SA_OXY] = -2;
  segs.base[SA_OZY] = p.bzy0; segs.roff[SA_OZY] = -2;
  segs.base[SA_B] = p.rho; segs.roff[SA_B] = 0;
  segs.base[SA_MU] = p.mu; segs.roff[SA_MU] = 1;
  segs.base[SA_GB] = p.g_b; segs.roff[SA_GB] = 0;
  segs.base[SA_GM] = p.g_mu; segs.roff[SA_GM] = -2;
  Loader rows = make_aloader<Loader>(segs, g, m, L, smem);
  rows.configure(g);
  rows.start();

  const f4 tb = ld4(p.taper_zb + c0), tt = ld4(p.taper_zt + c0);
  const f4 rzb = masked_recip(g.rdz, L.zb), rzf = masked_recip(g.rdz, L.zf);
  auto times = [&](const f4& a, const f4& mu) {
    f4 o;
#pragma unroll
    for (int e = 0; e < 4; ++e) o.v[e] = mu.v[e] * dt * a.v[e];  // (mu*dt) as in add_sy_sh
    return o;
  };
  f4 xy0 = ld4(at(p.sxy, m.ib - 3)), xy1 = ld4(at(p.sxy, m.ib - 2)), xy2 = ld4(at(p.sxy, m.ib - 1)), xy3;
  f4 ex0 = times(ld4(at(p.bxy0, m.ib - 3)), ld4(at(p.mu, m.ib - 3)));
  f4 ex1 = times(ld4(at(p.bxy0, m.ib - 2)), ld4(at(p.mu, m.ib - 2)));
  f4 ex2 = times(ld4(at(p.bxy0, m.ib - 1)), ld4(at(p.mu, m.ib - 1)));
  f4 ex3;
  f4 ezc, ezn = times(ld4(at(p.bzy0, m.ib - 1)), ld4(at(p.mu, m.ib - 1)));
  f4 na, nb, nc, nd;
  f4 qa, qb, qc, qd;
  Cursor cs = cursor_at(p.src.list, p.src.n, m.ib - 1);
  Cursor cr = cursor_at(p.rec.list, p.rec.n, m.ib - 1);
  const int nk = m.ie - m.ib + 3;
  float bx_next = __ldg(p.taper_x + m.ib - 1);

  for (int k = 0; k < nk; ++k) {
    const int i = m.ib - 1 + k;
    const float bxi = bx_next;
    bx_next = __ldg(p.taper_x + i + 1);
    if (!rows.acquire(k)) {
      flag(p.err);
      rows.drain(k);
      return false;
    }
    xy3 = rows.seg(SA_SXY);
    const f4 szy_i = rows.seg(SA_SZY);
    const f4 vy_i = rows.seg(SA_VY);
    const f4 mu1 = rows.seg(SA_MU);
    ex3 = times(rows.seg(SA_BXY), mu1);
    ezc = ezn;
    ezn = times(rows.seg(SA_BZY), mu1);
    f4 w = rows.seg(SA_W);
    const f4 oxy = rows.seg(SA_OXY), ozy = rows.seg(SA_OZY);
    const f4 buoy = rows.seg(SA_B);
    f4 gb = rows.seg(SA_GB), gm = rows.seg(SA_GM);
    rows.release();

    f4 ds = dx4r(xy0, xy1, xy2, xy3, mask_back(i, g.nx) ? g.rdx : 0.0f);
    {
      const f4 a = dz_back_r(szy_i, rzb);
#pragma unroll
      for (int e = 0; e < 4; ++e) ds.v[e] = ds.v[e] + a.v[e];
    }
    inject_at<false, true, false>(p.src, i, c0, cs, ds, ds, ds);
    f4 bb;
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      bb.v[e] = (bxi * tb.v[e]) * tt.v[e];
      nd.v[e] = bb.v[e] * (vy_i.v[e] + dt * ds.v[e] * buoy.v[e]);
    }
    {
      const bool m0 = mask_fwd(i - 2, g.nx), m1 = mask_fwd(i - 1, g.nx), m2 = mask_fwd(i, g.nx),
                 m3 = mask_fwd(i + 1, g.nx);
      const f4 tx = (m0 && m1 && m2 && m3)
                        ? dxT(ex0, ex1, ex2, ex3, g.rdx)
                        : dxT(scaled(ex0, m0), scaled(ex1, m1), scaled(ex2, m2), scaled(ex3, m3), g.rdx);
      const f4 tz = dzT_back(masked(ezc, L.zf), g.rdz);
      inject_at<false, true, false>(p.rec, i, c0, cr, w, w, w);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        w.v[e] = bb.v[e] * (w.v[e] + tx.v[e] + tz.v[e]);
        qd.v[e] = dt * buoy.v[e] * w.v[e];
      }
    }
    if (i >= m.ib && i < m.ie) {
      st4_masked(at(p.w1, i), w, L.own);
#pragma unroll
      for (int e = 0; e < 4; ++e) gb.v[e] = gb.v[e] + dt * w.v[e] * ds.v[e];
      st4_masked(at(p.g_b, i), gb, L.own);
    }
    if (i >= m.ib + 2) {
      const int r = i - 2;
      const f4 ex = dx4r(na, nb, nc, nd, mask_fwd(r, g.nx) ? g.rdx : 0.0f);
      const f4 ez = dz_fwd_r(nb, rzf);
      const bool m0 = mask_back(r - 1, g.nx), m1 = mask_back(r, g.nx), m2 = mask_back(r + 1, g.nx),
                 m3 = mask_back(r + 2, g.nx);
      const f4 ax = (m0 && m1 && m2 && m3)
                        ? dxT(qa, qb, qc, qd, g.rdx)
                        : dxT(scaled(qa, m0), scaled(qb, m1), scaled(qc, m2), scaled(qd, m3), g.rdx);
      const f4 az = dzT_fwd(masked(qb, L.zb), g.rdz);
      f4 sxy, szy;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        sxy.v[e] = oxy.v[e] + ax.v[e];
        szy.v[e] = ozy.v[e] + az.v[e];
        gm.v[e] = gm.v[e] + dt * (oxy.v[e] * ex.v[e] + ozy.v[e] * ez.v[e]);
      }
      st4_masked(at(p.bxy1, r), sxy, L.own);
      st4_masked(at(p.bzy1, r), szy, L.own);
      st4_masked(at(p.g_mu, r), gm, L.own);
    }

    na = nb; nb = nc; nc = nd;
    qa = qb; qb = qc; qc = qd;
    xy0 = xy1; xy1 = xy2; xy2 = xy3;
    ex0 = ex1; ex1 = ex2; ex2 = ex3;
  }
  return true;
}

}  // namespace
}  // namespace seiswg
