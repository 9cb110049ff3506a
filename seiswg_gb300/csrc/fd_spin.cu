// fd_spin.cu -- fused one-step kernel for PSV + micropolar spin.
//
// The march of fd_step.cu (velocity row i, stress row i-2, register rings,
// bulk-copy row pipeline) over 15 row segments: the PSV state and material
// plus the spin state vy_c, syx_c, syy_c, syz_c and 1/J, nu, mu_c+nu_c
// (fd2d.wgsl:308-399, 319-339, 405-445; 96 B per cell-update).
//
// At 238 registers (8 warps per SM) the kernel is bound by latency; it is
// built with multiply-add contraction and dt is folded into the difference
// factors (dt/(8 h)), which cut its instructions by 16 %; results match the
// reference's operation order to rounding (relative L2 ~1e-7), not bitwise.
#include "fd_fma.cuh"

namespace seiswg {

namespace {

enum SpinSeg {
  SP_SXX = 0, SP_SXZ, SP_SZZ,     // sigma^n, row i+1
  SP_VX, SP_VZ, SP_RHO,           // v^n and 1/rho, row i
  SP_LAM, SP_MU,                  // row i-2
  SP_SYX, SP_SYY, SP_SYZ,         // spin stresses, row i+1
  SP_VYC, SP_J,                   // spin velocity and 1/J, row i
  SP_NU, SP_MC,                   // nu and mu_c+nu_c, row i-2
  SP_NSEG
};

template <class Loader>
__device__ __forceinline__ void spin_march(const PsvStep& p, int gw, unsigned char* smem) {
  const Geom& g = p.g;
  const March m = march_of(g, gw);
  if (!m.active) return;
  const LaneCols L = lane_cols(g, m.strip, m.lane);
  const size_t ld = size_t(g.ld);
  const float dt = g.dt;
  const int c0 = L.c0;
  auto at = [&](auto* base, int i) { return base + ptrdiff_t(i) * ptrdiff_t(ld) + c0; };

  typename Loader::SegsT segs;
  segs.base[SP_SXX] = p.sxx0; segs.roff[SP_SXX] = 1;
  segs.base[SP_SXZ] = p.sxz0; segs.roff[SP_SXZ] = 1;
  segs.base[SP_SZZ] = p.szz0; segs.roff[SP_SZZ] = 1;
  segs.base[SP_VX] = p.vx0; segs.roff[SP_VX] = 0;
  segs.base[SP_VZ] = p.vz0; segs.roff[SP_VZ] = 0;
  segs.base[SP_RHO] = p.rho; segs.roff[SP_RHO] = 0;
  segs.base[SP_LAM] = p.lam; segs.roff[SP_LAM] = -2;
  segs.base[SP_MU] = p.mu; segs.roff[SP_MU] = -2;
  segs.base[SP_SYX] = p.syx0; segs.roff[SP_SYX] = 1;
  segs.base[SP_SYY] = p.syy0; segs.roff[SP_SYY] = 1;
  segs.base[SP_SYZ] = p.syz0; segs.roff[SP_SYZ] = 1;
  segs.base[SP_VYC] = p.vyc0; segs.roff[SP_VYC] = 0;
  segs.base[SP_J] = p.jm; segs.roff[SP_J] = 0;
  segs.base[SP_NU] = p.nu; segs.roff[SP_NU] = -2;
  segs.base[SP_MC] = p.mc; segs.roff[SP_MC] = -2;
  Loader rows = make_loader<Loader>(segs, g, m, L, smem);
  rows.configure(g);
  rows.start();

  // Column taper product; dt/(8 dz) where the column derivative is allowed.
  f4 tbt;
  {
    const f4 tb = ld4(p.taper_zb + c0), tt = ld4(p.taper_zt + c0);
#pragma unroll
    for (int e = 0; e < 4; ++e) tbt.v[e] = tb.v[e] * tt.v[e];
  }
  const float sx_dt = dt * g.rdx;
  const f4 rzb = masked_recip(dt * g.rdz, L.zb), rzf = masked_recip(dt * g.rdz, L.zf);
  const float dt2 = 2.0f * dt;

  // sigma^n rings, rows i-2..i+1
  f4 xx0 = ld4(at(p.sxx0, m.ib - 3)), xx1 = ld4(at(p.sxx0, m.ib - 2)), xx2 = ld4(at(p.sxx0, m.ib - 1)), xx3;
  f4 xz0 = ld4(at(p.sxz0, m.ib - 3)), xz1 = ld4(at(p.sxz0, m.ib - 2)), xz2 = ld4(at(p.sxz0, m.ib - 1)), xz3;
  f4 zz0 = ld4(at(p.szz0, m.ib - 3)), zz1 = ld4(at(p.szz0, m.ib - 2)), zz2 = ld4(at(p.szz0, m.ib - 1)), zz3;
  f4 yx0 = ld4(at(p.syx0, m.ib - 3)), yx1 = ld4(at(p.syx0, m.ib - 2)), yx2 = ld4(at(p.syx0, m.ib - 1)), yx3;
  f4 yy0 = ld4(at(p.syy0, m.ib - 3)), yy1 = ld4(at(p.syy0, m.ib - 2)), yy2 = ld4(at(p.syy0, m.ib - 1)), yy3;
  f4 yz0 = ld4(at(p.syz0, m.ib - 3)), yz1 = ld4(at(p.syz0, m.ib - 2)), yz2 = ld4(at(p.syz0, m.ib - 1)), yz3;
  f4 xa, xb_, xc, xd;   // new vx rows i-3..i
  f4 za, zb_, zc, zd;   // new vz rows i-3..i
  f4 ya, yb, yc, yd;    // new vy_c rows i-3..i
  Cursor ci = cursor_at(p.inj.list, p.inj.n, m.ib - 1);
  Cursor pi = cursor_at(p.probes.list, p.probes.n, m.ib);
  const int nk = m.ie - m.ib + 3;
  float bx_next = __ldg(p.taper_x + m.ib - 1);  // row taper, loaded one iteration ahead

  for (int k = 0; k < nk; ++k) {
    const int i = m.ib - 1 + k;
    const float bxi = bx_next;
    bx_next = __ldg(p.taper_x + i + 1);  // rows up to ie + 2 lie in the taper's halo
    if (!rows.acquire(k)) {
      flag_timeout(p.err);
      rows.drain(k);
      return;
    }
    xx3 = rows.seg(SP_SXX);
    xz3 = rows.seg(SP_SXZ);
    zz3 = rows.seg(SP_SZZ);
    yx3 = rows.seg(SP_SYX);
    yy3 = rows.seg(SP_SYY);
    yz3 = rows.seg(SP_SYZ);
    const f4 vxo = rows.seg(SP_VX);
    const f4 vzo = rows.seg(SP_VZ);
    const f4 rho = rows.seg(SP_RHO);
    const f4 lam = rows.seg(SP_LAM);
    const f4 mu = rows.seg(SP_MU);
    const f4 vyo = rows.seg(SP_VYC);
    const f4 jj = rows.seg(SP_J);
    const f4 nu = rows.seg(SP_NU);
    const f4 mc = rows.seg(SP_MC);
    rows.release();
    const float rxb = (i >= 2 && i < g.nx - 2) ? sx_dt : 0.0f;

    // dt times: div_sxz (fd2d.wgsl:315-316), div_sy_c (fd2d.wgsl:338) and
    // div_sxyz_c (fd2d.wgsl:326-329).
    f4 dsx, dsz, dsy;
    {
      const f4 ax = d4_rows(xx0, xx1, xx2, xx3), bx = d4_rows(xz0, xz1, xz2, xz3);
      const f4 cx = d4_rows(yx0, yx1, yx2, yx3), yyx = d4_rows(yy0, yy1, yy2, yy3);
      const f4 az = d4_cols_back(xz2), bz = d4_cols_back(zz2), cz = d4_cols_back(yz2), yyz = d4_cols_back(yy2);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        dsx.v[e] = fmaf(yyz.v[e], rzb.v[e], fmaf(az.v[e], rzb.v[e], ax.v[e] * rxb));
        dsz.v[e] = fmaf(-yyx.v[e], rxb, fmaf(bz.v[e], rzb.v[e], bx.v[e] * rxb));
        dsy.v[e] = fmaf(dt2, yy2.v[e], fmaf(cz.v[e], rzb.v[e], cx.v[e] * rxb));
      }
    }
    if (ci.row == i) inject_dt(p.inj, i, c0, ci, dt, dsx, dsz);  // stf_dsxz, fd2d.wgsl:350-351

    // add_vxz (fd2d.wgsl:362-363), rho holding 1/rho; add_vy_c
    // (fd2d.wgsl:412), jm holding 1/J.
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float b = bxi * tbt.v[e];
      xd.v[e] = b * fmaf(dsx.v[e], rho.v[e], vxo.v[e]);
      zd.v[e] = b * fmaf(dsz.v[e], rho.v[e], vzo.v[e]);
      yd.v[e] = b * fmaf(dsy.v[e], jj.v[e], vyo.v[e]);
    }
    if (i >= m.ib && i < m.ie) {
      st4_masked(at(p.vx1, i), xd, L.own);
      st4_masked(at(p.vz1, i), zd, L.own);
      st4_masked(at(p.vyc1, i), yd, L.own);
      probe_at(p.probes, i, L, pi, dt, [&](int comp, int e) {
        return comp == kProbeVX ? pick4(xd, e) : comp == kProbeVZ ? pick4(zd, e) : pick4(yd, e);
      });
    }

    // Stress of row r = i-2.
    if (i >= m.ib + 2) {
      const int r = i - 2;
      const float rxf = (r >= 1 && r < g.nx - 2) ? sx_dt : 0.0f;
      // dt times div_vxz (fd2d.wgsl:378-381) and div_vy_c (fd2d.wgsl:423-424)
      const f4 ux = d4_rows(xa, xb_, xc, xd), wx = d4_rows(za, zb_, zc, zd), gx = d4_rows(ya, yb, yc, yd);
      const f4 uz = d4_cols_fwd(xb_), wz = d4_cols_fwd(zb_), gz = d4_cols_fwd(yb);
      f4 sxx, szz, sxz, syy, syx, syz;
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        // add_sxz (fd2d.wgsl:396-398)
        const float l = lam.v[e], mm = mu.v[e];
        const float dvxdx = ux.v[e] * rxf, dvzdx = wx.v[e] * rxf;
        const float dvxdz = uz.v[e] * rzf.v[e], dvzdz = wz.v[e] * rzf.v[e];
        const float l2m = fmaf(2.0f, mm, l);
        sxx.v[e] = fmaf(l2m, dvxdx, fmaf(l, dvzdz, xx0.v[e]));
        szz.v[e] = fmaf(l2m, dvzdz, fmaf(l, dvxdx, zz0.v[e]));
        sxz.v[e] = fmaf(mm, dvxdz + dvzdx, xz0.v[e]);
        // add_sy_c (fd2d.wgsl:442-444): syy += 2 dt nu (-vy_c - (dvz/dx - dvx/dz) / 2)
        syy.v[e] = fmaf(2.0f * nu.v[e], fmaf(-0.5f, dvzdx - dvxdz, -dt * yb.v[e]), yy0.v[e]);
        syx.v[e] = fmaf(mc.v[e], gx.v[e] * rxf, yx0.v[e]);
        syz.v[e] = fmaf(mc.v[e], gz.v[e] * rzf.v[e], yz0.v[e]);
      }
      st4_masked(at(p.sxx1, r), sxx, L.own);
      st4_masked(at(p.szz1, r), szz, L.own);
      st4_masked(at(p.sxz1, r), sxz, L.own);
      st4_masked(at(p.syy1, r), syy, L.own);
      st4_masked(at(p.syx1, r), syx, L.own);
      st4_masked(at(p.syz1, r), syz, L.own);
    }

    xa = xb_; xb_ = xc; xc = xd;
    za = zb_; zb_ = zc; zc = zd;
    ya = yb; yb = yc; yc = yd;
    xx0 = xx1; xx1 = xx2; xx2 = xx3;
    xz0 = xz1; xz1 = xz2; xz2 = xz3;
    zz0 = zz1; zz1 = zz2; zz2 = zz3;
    yx0 = yx1; yx1 = yx2; yx2 = yx3;
    yy0 = yy1; yy1 = yy2; yy2 = yy3;
    yz0 = yz1; yz1 = yz2; yz2 = yz3;
  }
}

}  // namespace

template <class Loader>
__global__ void __launch_bounds__(kStepWarps * 32) psv_spin_step_kernel(const PsvStep p) {
  extern __shared__ __align__(128) unsigned char smem[];
  spin_march<Loader>(p, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), warp_slice<Loader>(smem));
}

namespace {

template <class L>
cudaError_t launch_spin(const PsvStep& p, cudaStream_t s) {
  const size_t smem = smem_for<L>();
  static const cudaError_t attr = prepare_kernel(psv_spin_step_kernel<L>, smem);
  if (attr != cudaSuccess) return attr;
  return launch_step(psv_spin_step_kernel<L>, p.g.pdl != 0, blocks_for(p.g), smem, s, p);
}

}  // namespace

size_t spin_step_smem_bytes(int loader) {
  return loader == kLoaderBulk ? smem_for<BulkL<SP_NSEG>>() : 0;
}

int spin_step_blocks_per_sm(int loader) {
  int n = 0;
  const int threads = kStepWarps * 32;
  const size_t smem = spin_step_smem_bytes(loader);
  cudaError_t e;
  if (loader == kLoaderBulk) {
    e = prepare_kernel(psv_spin_step_kernel<BulkL<SP_NSEG>>, smem);
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, psv_spin_step_kernel<BulkL<SP_NSEG>>, threads, smem);
  } else {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, psv_spin_step_kernel<DirectL<SP_NSEG>>, threads, smem);
  }
  return e == cudaSuccess ? n : 0;
}

cudaError_t launch_psv_spin_step(const PsvStep& p, cudaStream_t s) {
  if (p.g.loader == kLoaderBulk) return launch_spin<BulkL<SP_NSEG>>(p, s);
  return launch_spin<DirectL<SP_NSEG>>(p, s);
}

}  // namespace seiswg
