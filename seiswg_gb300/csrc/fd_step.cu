// fd_step.cu -- fused one-step kernels for the SH, PSV and PSV+spin systems.
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
// State is ping-ponged between two buffers (read step n, write step n+1):
// a warp recomputes the velocity of its halo rows/columns from step-n data
// that its neighbours are overwriting in place otherwise.
//
// Arithmetic follows the reference's expressions operation for operation
// (built with -fmad=false), except that divisions by 8*dx, rho and J are
// multiplies by precomputed reciprocals; results track the FP32 reference to
// rounding (relative L2 ~1e-7 over thousands of steps).
#include "fd_common.cuh"
#include "fd_kernels.h"

namespace seiswg {

namespace {

// Row march bounds and per-lane set-up shared by both kernels.
struct March {
  int lane, strip, chunk, ib, ie;
  bool active;
};

__device__ __forceinline__ March march_of(const Geom& g) {
  March m;
  m.lane = threadIdx.x & 31;
  int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  m.strip = gw % g.nstrips;
  m.chunk = gw / g.nstrips;
  m.active = m.chunk < g.nchunks;
  m.ib = m.chunk * g.lx;
  m.ie = min(g.nx, m.ib + g.lx);
  return m;
}

// Adds the injections of row i (sources, or adjoint sources at receivers) to
// the lane's divergence values.  `ci` is the list cursor, advanced past row i.
__device__ __forceinline__ void inject_row(const InjectList& inj, int i, int c0, int& ci, f4* ds_x, f4* ds_y,
                                           f4* ds_z) {
  while (ci < inj.n && __ldg(&inj.list[ci].i) == i) {
    int j = __ldg(&inj.list[ci].j);
    int e = j - c0;
    if (e >= 0 && e < 4) {
      size_t o = size_t(__ldg(&inj.list[ci].row)) * inj.nt + inj.it;
      if (ds_x) ds_x->v[e] += __ldg(&inj.val_x[o]);
      if (ds_y) ds_y->v[e] += __ldg(&inj.val_y[o]);
      if (ds_z) ds_z->v[e] += __ldg(&inj.val_z[o]);
    }
    ++ci;
  }
}

// Integrates the displacement of the owned probes of row i and records it.
template <typename Pick>
__device__ __forceinline__ void probe_row(const ProbeList& pr, int i, const LaneCols& L, int& pi, float dt,
                                          Pick pick) {
  while (pi < pr.n && __ldg(&pr.list[pi].i) == i) {
    int j = __ldg(&pr.list[pi].j);
    int e = j - L.c0;
    if (e >= 0 && e < 4 && (L.own & (1 << e))) {
      int idx = __ldg(&pr.list[pi].idx);
      float v = pick(__ldg(&pr.list[pi].comp), e);
      float u = pr.acc[idx] + v * dt;  // af(F_U*, k, v * dt), fd2d.wgsl:270
      pr.acc[idx] = u;
      pr.hist[size_t(idx) * pr.nt + pr.it] = u;
    }
    ++pi;
  }
}

}  // namespace

// --------------------------------------------------------------------------
// SH: state vy, sxy, szy; material rho, mu.  fd2d.wgsl:242-301.
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(128) sh_step_kernel(const ShStep p) {
  const Geom& g = p.g;
  const March m = march_of(g);
  if (!m.active) return;
  const LaneCols L = lane_cols(g, m.strip, m.lane);
  const size_t ld = size_t(g.ld);
  const float dt = g.dt;
  const int c0 = L.c0;
  auto at = [&](auto* base, int i) { return base + ptrdiff_t(i) * ptrdiff_t(ld) + c0; };

  const f4 tb = ld4(p.taper_zb + c0), tt = ld4(p.taper_zt + c0);

  // Rings: sxy rows i-2..i+1, szy rows i-2..i+1, new vy rows i-3..i.
  f4 xy0 = ld4(at(p.sxy0, m.ib - 3)), xy1 = ld4(at(p.sxy0, m.ib - 2)), xy2 = ld4(at(p.sxy0, m.ib - 1)),
     xy3 = ld4(at(p.sxy0, m.ib));
  f4 zy0 = ld4(at(p.szy0, m.ib - 3)), zy1 = ld4(at(p.szy0, m.ib - 2)), zy2 = ld4(at(p.szy0, m.ib - 1)),
     zy3 = ld4(at(p.szy0, m.ib));
  f4 va, vb, vc, vd;
  int ci = lower_row(p.inj.list, p.inj.n, m.ib - 1);
  int pi = lower_row(p.probes.list, p.probes.n, m.ib);

  for (int i = m.ib - 1; i <= m.ie + 1; ++i) {
    const f4 vo = ld4(at(p.vy0, i));
    const f4 rho = ld4(at(p.rho, i));
    const float bxi = __ldg(p.taper_x + i);
    const bool xb = (i >= 2 && i < g.nx - 2);

    // div_sy (fd2d.wgsl:247): DSY = dx-(sxy) + dz-(szy)
    f4 ds = dx4(xy0, xy1, xy2, xy3, g.rdx, xb);
    const f4 dz = dz_back(zy2, g.rdz, L.zb);
#pragma unroll
    for (int e = 0; e < 4; ++e) ds.v[e] = ds.v[e] + dz.v[e];
    inject_row(p.inj, i, c0, ci, nullptr, &ds, nullptr);  // stf_dsy / adj_dsy

    // add_vy (fd2d.wgsl:268): vy = b * (vy + dt * DSY / rho), with the
    // buoyancy 1/rho stored in place of rho.
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float b = (bxi * tb.v[e]) * tt.v[e];
      vd.v[e] = b * (vo.v[e] + dt * ds.v[e] * rho.v[e]);
    }
    if (i >= m.ib && i < m.ie) {
      st4_masked(at(p.vy1, i), vd, L.own);
      if (p.probes.n) probe_row(p.probes, i, L, pi, dt, [&](int, int e) { return vd.v[e]; });
    }

    // Stress of row r = i-2 from new vy rows r-1..r+2 = (va, vb, vc, vd).
    if (i >= m.ib + 2) {
      const int r = i - 2;
      const bool xf = (r >= 1 && r < g.nx - 2);
      const f4 gx = dx4(va, vb, vc, vd, g.rdx, xf);
      const f4 gz = dz_fwd(vb, g.rdz, L.zf);
      const f4 mu = ld4(at(p.mu, r));
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
    if (i <= m.ie) {
      xy3 = ld4(at(p.sxy0, i + 2));
      zy3 = ld4(at(p.szy0, i + 2));
    }
  }
}

// --------------------------------------------------------------------------
// PSV (+ micropolar spin): state vx, vz, sxx, szz, sxz (+ vy_c, syx_c, syy_c,
// syz_c); material rho, lambda, mu (+ nu, J, mu_c+nu_c).
// fd2d.wgsl:308-399 and 319-339, 405-445.
// --------------------------------------------------------------------------
template <bool SPIN>
__global__ void __launch_bounds__(128) psv_step_kernel(const PsvStep p) {
  const Geom& g = p.g;
  const March m = march_of(g);
  if (!m.active) return;
  const LaneCols L = lane_cols(g, m.strip, m.lane);
  const size_t ld = size_t(g.ld);
  const float dt = g.dt;
  const int c0 = L.c0;
  auto at = [&](auto* base, int i) { return base + ptrdiff_t(i) * ptrdiff_t(ld) + c0; };

  const f4 tb = ld4(p.taper_zb + c0), tt = ld4(p.taper_zt + c0);

  f4 xx0 = ld4(at(p.sxx0, m.ib - 3)), xx1 = ld4(at(p.sxx0, m.ib - 2)), xx2 = ld4(at(p.sxx0, m.ib - 1)),
     xx3 = ld4(at(p.sxx0, m.ib));
  f4 xz0 = ld4(at(p.sxz0, m.ib - 3)), xz1 = ld4(at(p.sxz0, m.ib - 2)), xz2 = ld4(at(p.sxz0, m.ib - 1)),
     xz3 = ld4(at(p.sxz0, m.ib));
  f4 zz0 = ld4(at(p.szz0, m.ib - 3)), zz1 = ld4(at(p.szz0, m.ib - 2)), zz2 = ld4(at(p.szz0, m.ib - 1)),
     zz3 = ld4(at(p.szz0, m.ib));
  f4 yx0, yx1, yx2, yx3, yy0, yy1, yy2, yy3, yz0, yz1, yz2, yz3;
  if (SPIN) {
    yx0 = ld4(at(p.syx0, m.ib - 3)); yx1 = ld4(at(p.syx0, m.ib - 2)); yx2 = ld4(at(p.syx0, m.ib - 1));
    yx3 = ld4(at(p.syx0, m.ib));
    yy0 = ld4(at(p.syy0, m.ib - 3)); yy1 = ld4(at(p.syy0, m.ib - 2)); yy2 = ld4(at(p.syy0, m.ib - 1));
    yy3 = ld4(at(p.syy0, m.ib));
    yz0 = ld4(at(p.syz0, m.ib - 3)); yz1 = ld4(at(p.syz0, m.ib - 2)); yz2 = ld4(at(p.syz0, m.ib - 1));
    yz3 = ld4(at(p.syz0, m.ib));
  }
  f4 xa, xb_, xc, xd;   // new vx rows i-3..i
  f4 za, zb_, zc, zd;   // new vz rows i-3..i
  f4 ya, yb, yc, yd;    // new vy_c rows i-3..i
  int ci = lower_row(p.inj.list, p.inj.n, m.ib - 1);
  int pi = lower_row(p.probes.list, p.probes.n, m.ib);

  for (int i = m.ib - 1; i <= m.ie + 1; ++i) {
    const f4 vxo = ld4(at(p.vx0, i));
    const f4 vzo = ld4(at(p.vz0, i));
    const f4 rho = ld4(at(p.rho, i));
    const float bxi = __ldg(p.taper_x + i);
    const bool xbk = (i >= 2 && i < g.nx - 2);

    // div_sxz (fd2d.wgsl:315-316)
    f4 dsx = dx4(xx0, xx1, xx2, xx3, g.rdx, xbk);
    f4 dsz = dx4(xz0, xz1, xz2, xz3, g.rdx, xbk);
    {
      const f4 a = dz_back(xz2, g.rdz, L.zb);
      const f4 b = dz_back(zz2, g.rdz, L.zb);
#pragma unroll
      for (int e = 0; e < 4; ++e) { dsx.v[e] = dsx.v[e] + a.v[e]; dsz.v[e] = dsz.v[e] + b.v[e]; }
    }
    f4 dsy;
    if (SPIN) {
      // div_sy_c (fd2d.wgsl:338), then div_sxyz_c (fd2d.wgsl:326-329)
      dsy = dx4(yx0, yx1, yx2, yx3, g.rdx, xbk);
      const f4 a = dz_back(yz2, g.rdz, L.zb);
      const f4 zy = dz_back(yy2, g.rdz, L.zb);
      const f4 xy = dx4(yy0, yy1, yy2, yy3, g.rdx, xbk);
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        dsy.v[e] = dsy.v[e] + a.v[e];
        dsx.v[e] += zy.v[e];
        dsz.v[e] += -xy.v[e];
        dsy.v[e] += 2.0f * yy2.v[e];
      }
    }
    inject_row(p.inj, i, c0, ci, &dsx, nullptr, &dsz);  // stf_dsxz, fd2d.wgsl:350-351

    // add_vxz (fd2d.wgsl:362-363)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const float b = (bxi * tb.v[e]) * tt.v[e];
      xd.v[e] = b * (vxo.v[e] + dt * dsx.v[e] * rho.v[e]);  // rho holds 1/rho
      zd.v[e] = b * (vzo.v[e] + dt * dsz.v[e] * rho.v[e]);
    }
    if (SPIN) {
      // add_vy_c (fd2d.wgsl:412)
      const f4 vyo = ld4(at(p.vyc0, i));
      const f4 jj = ld4(at(p.jm, i));
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float b = (bxi * tb.v[e]) * tt.v[e];
        yd.v[e] = b * (vyo.v[e] + dt * dsy.v[e] * jj.v[e]);  // jm holds 1/J
      }
    }
    if (i >= m.ib && i < m.ie) {
      st4_masked(at(p.vx1, i), xd, L.own);
      st4_masked(at(p.vz1, i), zd, L.own);
      if (SPIN) st4_masked(at(p.vyc1, i), yd, L.own);
      if (p.probes.n)
        probe_row(p.probes, i, L, pi, dt, [&](int comp, int e) {
          return comp == kProbeVX ? xd.v[e] : comp == kProbeVZ ? zd.v[e] : (SPIN ? yd.v[e] : 0.0f);
        });
    }

    // Stress of row r = i-2.
    if (i >= m.ib + 2) {
      const int r = i - 2;
      const bool xf = (r >= 1 && r < g.nx - 2);
      // div_vxz (fd2d.wgsl:378-381)
      const f4 dvxdx = dx4(xa, xb_, xc, xd, g.rdx, xf);
      const f4 dvzdx = dx4(za, zb_, zc, zd, g.rdx, xf);
      const f4 dvxdz = dz_fwd(xb_, g.rdz, L.zf);
      const f4 dvzdz = dz_fwd(zb_, g.rdz, L.zf);
      const f4 lam = ld4(at(p.lam, r));
      const f4 mu = ld4(at(p.mu, r));
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
      if (SPIN) {
        // div_vy_c (fd2d.wgsl:423-424), add_sy_c (fd2d.wgsl:442-444)
        const f4 gx = dx4(ya, yb, yc, yd, g.rdx, xf);
        const f4 gz = dz_fwd(yb, g.rdz, L.zf);
        const f4 nu = ld4(at(p.nu, r));
        const f4 mc = ld4(at(p.mc, r));
        f4 syy, syx, syz;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          syy.v[e] = yy0.v[e] + 2.0f * dt * nu.v[e] * (-yb.v[e] - 0.5f * (dvzdx.v[e] - dvxdz.v[e]));
          syx.v[e] = yx0.v[e] + dt * mc.v[e] * gx.v[e];
          syz.v[e] = yz0.v[e] + dt * mc.v[e] * gz.v[e];
        }
        st4_masked(at(p.syy1, r), syy, L.own);
        st4_masked(at(p.syx1, r), syx, L.own);
        st4_masked(at(p.syz1, r), syz, L.own);
      }
    }

    xa = xb_; xb_ = xc; xc = xd;
    za = zb_; zb_ = zc; zc = zd;
    xx0 = xx1; xx1 = xx2; xx2 = xx3;
    xz0 = xz1; xz1 = xz2; xz2 = xz3;
    zz0 = zz1; zz1 = zz2; zz2 = zz3;
    if (SPIN) {
      ya = yb; yb = yc; yc = yd;
      yx0 = yx1; yx1 = yx2; yx2 = yx3;
      yy0 = yy1; yy1 = yy2; yy2 = yy3;
      yz0 = yz1; yz1 = yz2; yz2 = yz3;
    }
    if (i <= m.ie) {
      xx3 = ld4(at(p.sxx0, i + 2));
      xz3 = ld4(at(p.sxz0, i + 2));
      zz3 = ld4(at(p.szz0, i + 2));
      if (SPIN) {
        yx3 = ld4(at(p.syx0, i + 2));
        yy3 = ld4(at(p.syy0, i + 2));
        yz3 = ld4(at(p.syz0, i + 2));
      }
    }
  }
}

// --------------------------------------------------------------------------
// Launchers
// --------------------------------------------------------------------------
static inline unsigned blocks_for(const Geom& g) {
  long warps = long(g.nstrips) * g.nchunks;
  return unsigned((warps + kStepWarps - 1) / kStepWarps);
}

cudaError_t launch_sh_step(const ShStep& p, cudaStream_t s) {
  sh_step_kernel<<<blocks_for(p.g), kStepWarps * 32, 0, s>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_psv_step(const PsvStep& p, bool spin, cudaStream_t s) {
  if (spin)
    psv_step_kernel<true><<<blocks_for(p.g), kStepWarps * 32, 0, s>>>(p);
  else
    psv_step_kernel<false><<<blocks_for(p.g), kStepWarps * 32, 0, s>>>(p);
  return cudaGetLastError();
}

}  // namespace seiswg
