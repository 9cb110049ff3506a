// fd2d_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the checker, never the product).
//
// A CPU restatement of seiswg's 2-D staggered-grid finite-difference path,
// written to be read side by side with the reference:
//
//   shaders/fd2d.wgsl        every @compute kernel used on the hot path
//   src/solver.rs            Ricker STF (350-356), waveform misfit (432-467),
//                            forward step order (1000-1030), snapshot timing
//                            (1035-1038), adjoint workflow (1298-1529),
//                            smoothing order (1249-1274)
//
// The stencil is evaluated exactly as the WGSL does it: one full pass over the
// grid per reference kernel, every intermediate field (DSY, DVYDX, ...)
// materialised, operations in the WGSL's left-to-right order, no FMA
// contraction (the build passes -ffp-contract=off).  It is instantiated twice:
// `float` (reference operation order, used for parity with the WGSL fixtures
// and as the timed CPU baseline) and `double` (used to state the rounding
// error of the FP32 results).
//
// Only tests/, the smoke check and the CPU-baseline leg of the benchmark load
// this library.  Nothing in the product links it.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#include <algorithm>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// Field slots, fd2d.wgsl:53-105 / solver.rs:36-84.  Kept identical because
// the oracle restates the reference's own buffer layout.
enum FieldId {
  F_VY = 0, F_UY, F_SXY, F_SZY, F_DSY, F_DVYDX, F_DVYDZ,
  F_VX, F_VZ, F_UX, F_UZ, F_SXX, F_SZZ, F_SXZ, F_DSX, F_DSZ,
  F_DVXDX, F_DVXDZ, F_DVZDX, F_DVZDZ,
  F_VY_C, F_UY_C, F_SYX_C, F_SYY_C, F_SYZ_C, F_DSY_C, F_DVYDX_C, F_DVYDZ_C,
  F_DUZDX, F_DUXDZ,
  F_LAM, F_MU, F_NU, F_J, F_LAM_C, F_MU_C, F_NU_C, F_RHO, F_BOUND,
  F_K_LAM, F_K_MU, F_K_RHO, F_GSUM, F_GTMP,
  N_FIELDS
};
constexpr int N_DYN_FIELDS = 30;  // solver.rs:31

// Observation components, fd2d.wgsl:110-114.
enum { OBS_X = 0, OBS_Y, OBS_Z, OBS_YI, OBS_YC, N_OBS };
// STF components, fd2d.wgsl:117-119.
enum { STF_X = 0, STF_Y, STF_Z };

}  // namespace

extern "C" {

// Parameters of one oracle run.  Real-valued entries are passed as double;
// the FP32 instance rounds them to float on entry, so callers pass the float
// values the reference itself would hold (e.g. dx = lx / (nx-1) in f32).
struct OracleParams {
  int32_t nx, nz, nt;
  double dx, dz, dt;
  int32_t sh, psv, spin;
  int32_t abs_left, abs_right, abs_bottom, abs_top, abs_width;
  double abs_alpha;
  int32_t nsrc, nrec;
};

}  // extern "C"

namespace {

struct OracleBase {
  virtual ~OracleBase() {}
  virtual void set_field(int fid, const double* d) = 0;
  virtual void get_field(int fid, double* d) const = 0;
  virtual void set_sources(const int32_t* k, const double* stf) = 0;
  virtual void set_receivers(const int32_t* k) = 0;
  virtual void init_model() = 0;
  virtual void clear_dynamic() = 0;
  virtual void clear_obs() = 0;
  virtual void forward_step(int it, int isrc) = 0;
  virtual void adjoint_step(int it) = 0;
  virtual void imaging(const double* fw, double ndt) = 0;
  virtual void smooth(double sigma) = 0;
  virtual void get_obs(int comp, double* out) const = 0;
  virtual void set_obs(int comp, const double* in) = 0;
  virtual int run_forward(int isrc, int snap_every, int nfid, const int32_t* fids, double* snaps) = 0;
  virtual int run_adjoint(int nruns, const int32_t* run_isrc, const double* obs_y, int adj_interval,
                          double sigma, double* misfits) = 0;
  virtual int exact_gradient(int isrc, const double* adj, double* g_lam, double* g_mu, double* g_b) = 0;
};

template <typename R>
struct Oracle final : OracleBase {
  int nx, nz, nt;
  size_t npt;
  R dx, dz, dt, abs_alpha;
  bool sh, psv, spin;
  bool abs_left, abs_right, abs_bottom, abs_top;
  uint32_t abs_width;
  int nsrc, nrec;
  std::vector<R> f;           // N_FIELDS * npt, slot-major like fd2d.wgsl:132
  std::vector<int32_t> src_k, rec_k;
  std::vector<R> stf;         // [3][nsrc][nt], solver.rs:721-733
  std::vector<R> obs;         // [5][nrec][nt], solver.rs:764

  explicit Oracle(const OracleParams& p)
      : nx(p.nx), nz(p.nz), nt(p.nt), npt(size_t(p.nx) * size_t(p.nz)),
        dx(R(p.dx)), dz(R(p.dz)), dt(R(p.dt)), abs_alpha(R(p.abs_alpha)),
        sh(p.sh != 0), psv(p.psv != 0), spin(p.spin != 0),
        abs_left(p.abs_left != 0), abs_right(p.abs_right != 0),
        abs_bottom(p.abs_bottom != 0), abs_top(p.abs_top != 0),
        abs_width(uint32_t(p.abs_width)), nsrc(p.nsrc), nrec(p.nrec),
        f(size_t(N_FIELDS) * npt, R(0)), src_k(p.nsrc, 0), rec_k(p.nrec, 0),
        stf(size_t(3) * p.nsrc * p.nt, R(0)), obs(size_t(N_OBS) * p.nrec * p.nt, R(0)) {}

  R* F(int id) { return f.data() + size_t(id) * npt; }
  const R* F(int id) const { return f.data() + size_t(id) * npt; }

  // ---- 4th-order staggered differences, fd2d.wgsl:151-180 ----------------
  // Backward (diff_x / diff_z): zero for i<2 or i>=n-2.
  inline R diff_x(const R* a, int i, size_t k) const {
    if (i < 2 || i >= nx - 2) return R(0);
    return (R(9) * (a[k] - a[k - nz]) - (a[k + nz] - a[k - 2 * size_t(nz)])) / (R(8) * dx);
  }
  inline R diff_z(const R* a, int j, size_t k) const {
    if (j < 2 || j >= nz - 2) return R(0);
    return (R(9) * (a[k] - a[k - 1]) - (a[k + 1] - a[k - 2])) / (R(8) * dz);
  }
  // Forward (diff_x1 / diff_z1): zero for i<1 or i>=n-2.
  inline R diff_x1(const R* a, int i, size_t k) const {
    if (i < 1 || i >= nx - 2) return R(0);
    return (R(9) * (a[k + nz] - a[k]) - (a[k + 2 * size_t(nz)] - a[k - nz])) / (R(8) * dx);
  }
  inline R diff_z1(const R* a, int j, size_t k) const {
    if (j < 1 || j >= nz - 2) return R(0);
    return (R(9) * (a[k + 1] - a[k]) - (a[k + 2] - a[k - 1])) / (R(8) * dz);
  }

  template <typename Fn>
  void grid_pass(Fn fn) {
    // One reference dispatch over all npt points; rows run in parallel.
#pragma omp for schedule(static)
    for (int i = 0; i < nx; ++i) {
      size_t k = size_t(i) * nz;
      for (int j = 0; j < nz; ++j, ++k) fn(i, j, k);
    }
  }

  template <typename Fn>
  void parallel(Fn fn) {
#pragma omp parallel
    { fn(); }
  }

  // ---- initialisation, fd2d.wgsl:188-235 ----------------------------------
  void init_model() override {
    R* lam = F(F_LAM); R* mu = F(F_MU); const R* rho = F(F_RHO); R* b = F(F_BOUND);
    const bool do_vps2lm = !spin;  // solver.rs:908-910
    const uint32_t w = abs_width, unx = uint32_t(nx), unz = uint32_t(nz);
    parallel([&] {
      if (do_vps2lm) {
        grid_pass([&](int, int, size_t k) {
          R vp = lam[k], vs = mu[k], r = rho[k];
          mu[k] = r * vs * vs;
          lam[k] = (vp > vs) ? r * (vp * vp - R(2) * vs * vs) : R(0);
        });
      }
      grid_pass([&](int ii, int jj, size_t k) {
        uint32_t i = uint32_t(ii), j = uint32_t(jj);
        R bb = R(1);
        if (abs_left && (i + 1u) < w) { R aw = abs_alpha * R(w - i - 1u); bb *= std::exp(-aw * aw); }
        if (abs_right && i > (unx - w)) { R aw = abs_alpha * R(w + i - unx); bb *= std::exp(-aw * aw); }
        if (abs_bottom && j > (unz - w)) { R aw = abs_alpha * R(w + j - unz); bb *= std::exp(-aw * aw); }
        if (abs_top && (j + 1u) < w) { R aw = abs_alpha * R(w - j - 1u); bb *= std::exp(-aw * aw); }
        b[k] = bb;
      });
    });
  }

  void clear_dynamic() override { std::fill(f.begin(), f.begin() + size_t(N_DYN_FIELDS) * npt, R(0)); }
  void clear_obs() override { std::fill(obs.begin(), obs.end(), R(0)); }

  R& obs_at(int comp, int ir, int it) { return obs[(size_t(comp) * nrec + ir) * nt + it]; }

  // ---- one forward step, solver.rs:1000-1030 ------------------------------
  // Must be called from inside a parallel region.
  void sh_step_body(int it, int isrc, bool adjoint) {
    R* vy = F(F_VY); R* uy = F(F_UY); R* sxy = F(F_SXY); R* szy = F(F_SZY);
    R* dsy = F(F_DSY); R* dvydx = F(F_DVYDX); R* dvydz = F(F_DVYDZ);
    const R* rho = F(F_RHO); const R* b = F(F_BOUND); const R* mu = F(F_MU);
    grid_pass([&](int i, int j, size_t k) {  // div_sy, fd2d.wgsl:243-248
      dsy[k] = diff_x(sxy, i, k) + diff_z(szy, j, k);
    });
#pragma omp single
    {
      if (!adjoint) {  // stf_dsy, fd2d.wgsl:253-260 (sources in index order)
        for (int s = 0; s < nsrc; ++s) {
          if (isrc >= 0 && s != isrc) continue;
          dsy[src_k[s]] += stf[(size_t(STF_Y) * nsrc + s) * nt + it];
        }
      } else {         // adj_dsy, fd2d.wgsl:563-568 (receivers in index order)
        for (int r = 0; r < nrec; ++r) dsy[rec_k[r]] += obs_at(OBS_Y, r, it);
      }
    }
    grid_pass([&](int, int, size_t k) {  // add_vy, fd2d.wgsl:264-271
      R v = b[k] * (vy[k] + dt * dsy[k] / rho[k]);
      vy[k] = v;
      uy[k] += v * dt;
    });
    grid_pass([&](int i, int j, size_t k) {  // div_vy, fd2d.wgsl:275-281
      dvydx[k] = diff_x1(vy, i, k);
      dvydz[k] = diff_z1(vy, j, k);
    });
    grid_pass([&](int, int, size_t k) {  // add_sy_sh, fd2d.wgsl:285-291
      R mu_dt = mu[k] * dt;
      sxy[k] += mu_dt * dvydx[k];
      szy[k] += mu_dt * dvydz[k];
    });
    if (!adjoint) {
#pragma omp single
      for (int r = 0; r < nrec; ++r) obs_at(OBS_Y, r, it) = uy[rec_k[r]];  // save_obs_y_sh
    }
  }

  void psv_step_body(int it, int isrc) {
    R* vx = F(F_VX); R* vz = F(F_VZ); R* ux = F(F_UX); R* uz = F(F_UZ);
    R* sxx = F(F_SXX); R* szz = F(F_SZZ); R* sxz = F(F_SXZ);
    R* dsx = F(F_DSX); R* dsz = F(F_DSZ);
    R* dvxdx = F(F_DVXDX); R* dvxdz = F(F_DVXDZ); R* dvzdx = F(F_DVZDX); R* dvzdz = F(F_DVZDZ);
    R* vyc = F(F_VY_C); R* uyc = F(F_UY_C); R* syx = F(F_SYX_C); R* syy = F(F_SYY_C); R* syz = F(F_SYZ_C);
    R* dsyc = F(F_DSY_C); R* dvydxc = F(F_DVYDX_C); R* dvydzc = F(F_DVYDZ_C);
    R* duzdx = F(F_DUZDX); R* duxdz = F(F_DUXDZ);
    const R* lam = F(F_LAM); const R* mu = F(F_MU); const R* nu = F(F_NU); const R* jj = F(F_J);
    const R* muc = F(F_MU_C); const R* nuc = F(F_NU_C); const R* rho = F(F_RHO); const R* b = F(F_BOUND);

    grid_pass([&](int i, int j, size_t k) {  // div_sxz, fd2d.wgsl:309-317
      dsx[k] = diff_x(sxx, i, k) + diff_z(sxz, j, k);
      dsz[k] = diff_x(sxz, i, k) + diff_z(szz, j, k);
    });
    if (spin) {
      grid_pass([&](int i, int j, size_t k) {  // div_sy_c, fd2d.wgsl:334-339
        dsyc[k] = diff_x(syx, i, k) + diff_z(syz, j, k);
      });
      grid_pass([&](int i, int j, size_t k) {  // div_sxyz_c, fd2d.wgsl:322-330
        R s = syy[k];
        dsx[k] += diff_z(syy, j, k);
        dsz[k] += -diff_x(syy, i, k);
        dsyc[k] += R(2) * s;
      });
    }
#pragma omp single
    for (int s = 0; s < nsrc; ++s) {  // stf_dsxz, fd2d.wgsl:344-352
      if (isrc >= 0 && s != isrc) continue;
      dsx[src_k[s]] += stf[(size_t(STF_X) * nsrc + s) * nt + it];
      dsz[src_k[s]] += stf[(size_t(STF_Z) * nsrc + s) * nt + it];
    }
    grid_pass([&](int, int, size_t k) {  // add_vxz, fd2d.wgsl:356-368
      R r = rho[k], bd = b[k];
      R x = bd * (vx[k] + dt * dsx[k] / r);
      R z = bd * (vz[k] + dt * dsz[k] / r);
      vx[k] = x; vz[k] = z;
      ux[k] += x * dt; uz[k] += z * dt;
    });
    grid_pass([&](int i, int j, size_t k) {  // div_vxz, fd2d.wgsl:372-382
      dvxdx[k] = diff_x1(vx, i, k);
      dvxdz[k] = diff_z1(vx, j, k);
      dvzdx[k] = diff_x1(vz, i, k);
      dvzdz[k] = diff_z1(vz, j, k);
    });
    grid_pass([&](int, int, size_t k) {  // add_sxz, fd2d.wgsl:386-399
      R l = lam[k], m = mu[k];
      R a = dvxdx[k], bz = dvxdz[k], c = dvzdx[k], d = dvzdz[k];
      sxx[k] += dt * ((l + R(2) * m) * a + l * d);
      szz[k] += dt * ((l + R(2) * m) * d + l * a);
      sxz[k] += dt * m * (bz + c);
    });
    if (spin) {
      grid_pass([&](int, int, size_t k) {  // add_vy_c, fd2d.wgsl:407-415
        R v = b[k] * (vyc[k] + dt * dsyc[k] / jj[k]);
        vyc[k] = v;
        uyc[k] += v * dt;
      });
      grid_pass([&](int i, int j, size_t k) {  // div_vy_c, fd2d.wgsl:419-425
        dvydxc[k] = diff_x1(vyc, i, k);
        dvydzc[k] = diff_z1(vyc, j, k);
      });
      grid_pass([&](int, int, size_t k) {  // add_sy_c, fd2d.wgsl:429-445
        R n = nu[k], mc = muc[k], nc = nuc[k], v = vyc[k];
        syy[k] += R(2) * dt * n * (-v - R(0.5) * (dvzdx[k] - dvxdz[k]));
        syx[k] += dt * (mc + nc) * dvydxc[k];
        syz[k] += dt * (mc + nc) * dvydzc[k];
      });
    }
#pragma omp single
    for (int r = 0; r < nrec; ++r) {  // save_obs_x / save_obs_z, fd2d.wgsl:464-476
      obs_at(OBS_X, r, it) = ux[rec_k[r]];
      obs_at(OBS_Z, r, it) = uz[rec_k[r]];
    }
    if (spin) {
      grid_pass([&](int i, int j, size_t k) {  // compute_du_grad, fd2d.wgsl:450-456
        duzdx[k] = diff_x1(uz, i, k);
        duxdz[k] = diff_z1(ux, j, k);
      });
#pragma omp single
      for (int r = 0; r < nrec; ++r) {  // save_obs_ry, fd2d.wgsl:481-492
        size_t km = size_t(rec_k[r]);
        R u = uyc[km];
        R curl = -(duzdx[km] - duxdz[km]);
        R iso = u - R(0.5) * curl;
        obs_at(OBS_Y, r, it) = u;
        obs_at(OBS_YI, r, it) = iso;
        obs_at(OBS_YC, r, it) = curl;
      }
    }
  }

  void forward_step(int it, int isrc) override {
    parallel([&] {
      if (sh) sh_step_body(it, isrc, false);
      if (psv) psv_step_body(it, isrc);
    });
  }

  // SH adjoint step, solver.rs:1458-1464 (adj_dsy in place of stf_dsy).
  void adjoint_step(int it) override {
    if (!sh) return;
    parallel([&] { sh_step_body(it, -1, true); });
  }

  // Imaging, solver.rs:1468-1491: forward vy uploaded into the DSY slot, then
  // div_uy, div_fw and interaction_muy with ndt in place of abs_alpha.
  void imaging_body(const R* fw, R ndt) {
    R* dsy = F(F_DSY); R* vy = F(F_VY);
    R* dvydx = F(F_DVYDX); R* dvydz = F(F_DVYDZ);
    R* dvydxc = F(F_DVYDX_C); R* dvydzc = F(F_DVYDZ_C); R* kmu = F(F_K_MU);
    grid_pass([&](int, int, size_t k) { dsy[k] = fw[k]; });
    grid_pass([&](int i, int j, size_t k) {  // div_uy, fd2d.wgsl:572-578
      dvydx[k] = diff_x1(vy, i, k);
      dvydz[k] = diff_z1(vy, j, k);
    });
    grid_pass([&](int i, int j, size_t k) {  // div_fw, fd2d.wgsl:582-588
      dvydxc[k] = diff_x1(dsy, i, k);
      dvydzc[k] = diff_z1(dsy, j, k);
    });
    grid_pass([&](int, int, size_t k) {  // interaction_muy, fd2d.wgsl:502-509
      kmu[k] += (dvydx[k] * dvydxc[k] + dvydz[k] * dvydzc[k]) * ndt;
    });
  }

  void imaging(const double* fw, double ndt) override {
    std::vector<R> tmp(fw, fw + npt);
    parallel([&] { imaging_body(tmp.data(), R(ndt)); });
  }

  // Smoothing, solver.rs:1249-1274: init_gsum -> gaussian_x -> gaussian_z,
  // fd2d.wgsl:517-554 and 592-609.  Full-range sums, one exp per term.
  void smooth(double sigma_d) override {
    const R sigma = R(sigma_d);
    R* kmu = F(F_K_MU); R* gsum = F(F_GSUM); R* gtmp = F(F_GTMP);
    parallel([&] {
      grid_pass([&](int i, int j, size_t k) {
        R sx = R(0);
        for (int n = 0; n < nx; ++n) { R d = R(i - n); sx += std::exp(-d * d / (R(2) * sigma * sigma)); }
        R sz = R(0);
        for (int n = 0; n < nz; ++n) { R d = R(j - n); sz += std::exp(-d * d / (R(2) * sigma * sigma)); }
        gsum[k] = sx * sz;
      });
      grid_pass([&](int i, int j, size_t k) {
        R s = R(0);
        for (int n = 0; n < nx; ++n) {
          R d = R(i - n);
          R w = std::exp(-d * d / (R(2) * sigma * sigma));
          s += w * kmu[size_t(n) * nz + j];
        }
        gtmp[k] = s;
      });
      grid_pass([&](int i, int j, size_t k) {
        R s = R(0);
        for (int n = 0; n < nz; ++n) {
          R d = R(j - n);
          R w = std::exp(-d * d / (R(2) * sigma * sigma));
          s += w * gtmp[size_t(i) * nz + n];
        }
        R g = gsum[k];
        kmu[k] = (g > R(1e-30)) ? s / g : R(0);
      });
    });
  }

  void set_field(int fid, const double* d) override {
    R* p = F(fid);
    for (size_t k = 0; k < npt; ++k) p[k] = R(d[k]);
  }
  void get_field(int fid, double* d) const override {
    const R* p = F(fid);
    for (size_t k = 0; k < npt; ++k) d[k] = double(p[k]);
  }
  void set_sources(const int32_t* k, const double* s) override {
    for (int i = 0; i < nsrc; ++i) src_k[i] = k[i];
    for (size_t i = 0; i < stf.size(); ++i) stf[i] = R(s[i]);
  }
  void set_receivers(const int32_t* k) override {
    for (int i = 0; i < nrec; ++i) rec_k[i] = k[i];
  }
  void get_obs(int comp, double* out) const override {
    const R* p = obs.data() + size_t(comp) * nrec * nt;
    for (size_t i = 0; i < size_t(nrec) * nt; ++i) out[i] = double(p[i]);
  }
  void set_obs(int comp, const double* in) override {
    R* p = obs.data() + size_t(comp) * nrec * nt;
    for (size_t i = 0; i < size_t(nrec) * nt; ++i) p[i] = R(in[i]);
  }

  // Whole forward run, solver.rs:977-1044: clear, nt steps, snapshot after
  // step `it` when it>0 && it%snap==0.  Snapshots of the requested fields are
  // appended to `snaps` as [nsnap][nfid][npt].  Returns the snapshot count.
  int run_forward(int isrc, int snap_every, int nfid, const int32_t* fids, double* snaps) override {
    clear_dynamic();
    clear_obs();
    int ns = 0;
    for (int it = 0; it < nt; ++it) {
      forward_step(it, isrc);
      if (snap_every > 0 && it > 0 && it % snap_every == 0) {
        if (snaps) {
          for (int q = 0; q < nfid; ++q)
            get_field(fids[q], snaps + (size_t(ns) * nfid + q) * npt);
        }
        ++ns;
      }
    }
    return ns;
  }

  // Waveform misfit and time-reversed adjoint source, solver.rs:432-467.
  double misfit(const R* syn, const R* ref, R* adstf) const {
    const R pi = R(3.14159265358979323846);
    double m = 0.0;
    R t_end = R(nt - 1) * dt;
    R tw = t_end / R(10);
    R t_min = tw, t_max = t_end - tw;
    for (int ir = 0; ir < nrec; ++ir) {
      for (int it = 0; it < nt; ++it) {
        size_t kt = size_t(ir) * nt + it;
        size_t akt = size_t(ir) * nt + (nt - 1 - it);
        R t = R(it) * dt;
        R taper;
        if (t <= t_min) taper = R(0.5) + R(0.5) * std::cos(pi * (t_min - t) / tw);
        else if (t >= t_max) taper = R(0.5) + R(0.5) * std::cos(pi * (t_max - t) / tw);
        else taper = R(1);
        R diff = (syn[kt] - ref[kt]) * taper;
        m += double(diff) * double(diff);
        adstf[akt] = diff * taper * R(2);
      }
    }
    return std::sqrt(m);
  }

  // Adjoint workflow, solver.rs:1298-1529 (SH imaging only, as in the
  // reference; PSV leaves K_MU at zero).  `obs_y` holds the observed uy
  // traces of each run as [nruns][nrec][nt].
  int run_adjoint(int nruns, const int32_t* run_isrc, const double* obs_y, int adj_interval,
                  double sigma, double* misfits) override {
    if (adj_interval <= 0) return -1;
    int nsa = nt / adj_interval;
    if (nsa == 0) return -1;
    std::fill(F(F_K_MU), F(F_K_MU) + npt, R(0));
    const R ndt = R(adj_interval) * dt;
    std::vector<R> fwd(size_t(nsa) * npt);
    std::vector<R> ref(size_t(nrec) * nt), syn(size_t(nrec) * nt), adstf(size_t(nrec) * nt);
    for (int run = 0; run < nruns; ++run) {
      int isrc = run_isrc[run];
      for (size_t i = 0; i < ref.size(); ++i) ref[i] = R(obs_y[size_t(run) * nrec * nt + i]);
      clear_dynamic();
      clear_obs();
      for (int it = 0; it < nt; ++it) {
        parallel([&] { if (sh) sh_step_body(it, isrc, false); });
        if ((it + 1) % adj_interval == 0) {
          int isa = nsa - (it + 1) / adj_interval;
          std::copy(F(F_VY), F(F_VY) + npt, fwd.begin() + size_t(isa) * npt);
        }
      }
      double m = 0.0;
      if (sh) {
        std::copy(obs.begin() + size_t(OBS_Y) * nrec * nt, obs.begin() + size_t(OBS_Y + 1) * nrec * nt,
                  syn.begin());
        m = misfit(syn.data(), ref.data(), adstf.data());
      } else {
        std::fill(adstf.begin(), adstf.end(), R(0));
      }
      if (misfits) misfits[run] = m;
      std::copy(adstf.begin(), adstf.end(), obs.begin() + size_t(OBS_Y) * nrec * nt);
      clear_dynamic();
      for (int it = 0; it < nt; ++it) {
        if (sh) parallel([&] { sh_step_body(it, -1, true); });
        if (it % adj_interval == 0) {
          int isae = it / adj_interval;
          if (isae < nsa) {
            const R* fw = fwd.data() + size_t(isae) * npt;
            parallel([&] { imaging_body(fw, ndt); });
          }
        }
      }
    }
    smooth(sigma);
    return 0;
  }

  // ---- exact discrete adjoint ---------------------------------------------
  // The reference has no PSV adjoint and only the imaging-condition SH kernel
  // (fd2d.wgsl:501-509); this is the gradient of
  //   J = sum over traces and samples of (misfit taper * (d - obs))^2
  // with respect to lambda, mu and the buoyancy B = 1/rho, for the forward
  // scheme above, by reverse-mode differentiation of every step.  `adj` holds
  // dJ/dd for each recorded sample: PSV [2][nrec][nt] (ux, uz), SH
  // [1][nrec][nt] (uy).  The transposes of the staggered differences are
  // applied in scatter form (each forward stencil application pushes its
  // coefficients back onto its inputs), independently of any closed form.
  // Not defined for spin.
  void scatter_x(R* out, int i, size_t k, R g, bool fwd) const {
    // fwd: diff_x1 taps (k-nz:+1, k:-9, k+nz:+9, k+2nz:-1); else diff_x taps (k-2nz:+1, k-nz:-9, k:+9, k+nz:-1)
    const R r = g / (R(8) * dx);
    if (fwd) {
      if (i < 1 || i >= nx - 2) return;
      out[k - nz] += r; out[k] -= R(9) * r; out[k + nz] += R(9) * r; out[k + 2 * size_t(nz)] -= r;
    } else {
      if (i < 2 || i >= nx - 2) return;
      out[k - 2 * size_t(nz)] += r; out[k - nz] -= R(9) * r; out[k] += R(9) * r; out[k + nz] -= r;
    }
  }
  void scatter_z(R* out, int j, size_t k, R g, bool fwd) const {
    const R r = g / (R(8) * dz);
    if (fwd) {
      if (j < 1 || j >= nz - 2) return;
      out[k - 1] += r; out[k] -= R(9) * r; out[k + 1] += R(9) * r; out[k + 2] -= r;
    } else {
      if (j < 2 || j >= nz - 2) return;
      out[k - 2] += r; out[k - 1] -= R(9) * r; out[k] += R(9) * r; out[k + 1] -= r;
    }
  }

  int exact_gradient(int isrc, const double* adj, double* g_lam, double* g_mu, double* g_b) override {
    if (spin || (sh && psv)) return -1;
    const bool is_sh = sh;
    const int nf = is_sh ? 3 : 6;
    // forward, keeping the divergence (with sources) and strains of each step
    clear_dynamic();
    clear_obs();
    std::vector<R> store(size_t(nt) * nf * npt);
    const int ids_sh[3] = {F_DSY, F_DVYDX, F_DVYDZ};
    const int ids_psv[6] = {F_DSX, F_DSZ, F_DVXDX, F_DVXDZ, F_DVZDX, F_DVZDZ};
    for (int it = 0; it < nt; ++it) {
      forward_step(it, isrc);
      for (int q = 0; q < nf; ++q) {
        const R* src = F(is_sh ? ids_sh[q] : ids_psv[q]);
        std::copy(src, src + npt, store.begin() + (size_t(it) * nf + q) * npt);
      }
    }
    const R* lam = F(F_LAM);
    const R* mu = F(F_MU);
    const R* rho = F(F_RHO);
    const R* bnd = F(F_BOUND);
    const int ncomp = is_sh ? 1 : 2;
    // U[c][r][n] = sum_{m >= n} adj[c][r][m]: the adjoint of the displacement
    // accumulators (d^n = u after step n, u += dt*v every step).
    std::vector<R> U(size_t(ncomp) * nrec * nt);
    for (int c = 0; c < ncomp; ++c)
      for (int r = 0; r < nrec; ++r) {
        R acc = R(0);
        for (int n = nt - 1; n >= 0; --n) {
          acc += R(adj[(size_t(c) * nrec + r) * nt + n]);
          U[(size_t(c) * nrec + r) * nt + n] = acc;
        }
      }
    std::vector<R> gl(npt, R(0)), gm(npt, R(0)), gb(npt, R(0));
    const int nv = is_sh ? 1 : 2, ns = is_sh ? 2 : 3;
    std::vector<std::vector<R>> vb(nv, std::vector<R>(npt, R(0))), V(nv, std::vector<R>(npt));
    std::vector<std::vector<R>> sb(ns, std::vector<R>(npt, R(0)));
    std::vector<R> q0(npt), q1(npt);
    for (int n = nt - 1; n >= 0; --n) {
      const R* st = store.data() + size_t(n) * nf * npt;
      for (int a = 0; a < nv; ++a) V[a] = vb[a];
      for (int r = 0; r < nrec; ++r)
        for (int c = 0; c < ncomp; ++c) V[c][rec_k[r]] += dt * U[(size_t(c) * nrec + r) * nt + n];
      // sigma^{n+1} = sigma^n + dt C eps(v^{n+1})
      for (int i = 0; i < nx; ++i)
        for (int j = 0; j < nz; ++j) {
          const size_t k = size_t(i) * nz + j;
          if (is_sh) {
            const R ex = st[1 * npt + k], ez = st[2 * npt + k];
            const R mdt = mu[k] * dt;
            gm[k] += dt * (sb[0][k] * ex + sb[1][k] * ez);
            scatter_x(V[0].data(), i, k, mdt * sb[0][k], true);
            scatter_z(V[0].data(), j, k, mdt * sb[1][k], true);
          } else {
            const R exx = st[2 * npt + k], exz = st[3 * npt + k], ezx = st[4 * npt + k], ezz = st[5 * npt + k];
            const R l = lam[k], m = mu[k];
            const R bxx = sb[0][k], bzz = sb[1][k], bxz = sb[2][k];
            gl[k] += dt * (bxx + bzz) * (exx + ezz);
            gm[k] += dt * (R(2) * bxx * exx + R(2) * bzz * ezz + bxz * (exz + ezx));
            scatter_x(V[0].data(), i, k, dt * ((l + R(2) * m) * bxx + l * bzz), true);  // exx
            scatter_z(V[1].data(), j, k, dt * (l * bxx + (l + R(2) * m) * bzz), true);  // ezz
            scatter_z(V[0].data(), j, k, dt * m * bxz, true);                           // exz
            scatter_x(V[1].data(), i, k, dt * m * bxz, true);                           // ezx
          }
        }
      // v^{n+1} = b (v^n + dt B (div sigma^n + f^n))
      for (int a = 0; a < nv; ++a)
        for (size_t k = 0; k < npt; ++k) vb[a][k] = bnd[k] * V[a][k];
      for (size_t k = 0; k < npt; ++k) {
        const R B = R(1) / rho[k];
        if (is_sh) {
          gb[k] += dt * vb[0][k] * st[k];
          q0[k] = dt * B * vb[0][k];
        } else {
          gb[k] += dt * (vb[0][k] * st[k] + vb[1][k] * st[npt + k]);
          q0[k] = dt * B * vb[0][k];
          q1[k] = dt * B * vb[1][k];
        }
      }
      for (int i = 0; i < nx; ++i)
        for (int j = 0; j < nz; ++j) {
          const size_t k = size_t(i) * nz + j;
          if (is_sh) {  // dsy = dx-(sxy) + dz-(szy)
            scatter_x(sb[0].data(), i, k, q0[k], false);
            scatter_z(sb[1].data(), j, k, q0[k], false);
          } else {      // dsx = dx-(sxx) + dz-(sxz); dsz = dx-(sxz) + dz-(szz)
            scatter_x(sb[0].data(), i, k, q0[k], false);
            scatter_z(sb[2].data(), j, k, q0[k], false);
            scatter_x(sb[2].data(), i, k, q1[k], false);
            scatter_z(sb[1].data(), j, k, q1[k], false);
          }
        }
    }
    for (size_t k = 0; k < npt; ++k) {
      if (g_lam) g_lam[k] = double(gl[k]);
      if (g_mu) g_mu[k] = double(gm[k]);
      if (g_b) g_b[k] = double(gb[k]);
    }
    return 0;
  }
};

}  // namespace

extern "C" {

void* oracle_create(const OracleParams* p, int precision) {
  if (!p || p->nx < 5 || p->nz < 5 || p->nt < 0 || p->nsrc < 0 || p->nrec < 0) return nullptr;
  if (precision == 32) return static_cast<OracleBase*>(new Oracle<float>(*p));
  if (precision == 64) return static_cast<OracleBase*>(new Oracle<double>(*p));
  return nullptr;
}
void oracle_destroy(void* h) { delete static_cast<OracleBase*>(h); }
void oracle_set_field(void* h, int fid, const double* d) { static_cast<OracleBase*>(h)->set_field(fid, d); }
void oracle_get_field(void* h, int fid, double* d) { static_cast<OracleBase*>(h)->get_field(fid, d); }
void oracle_set_sources(void* h, const int32_t* k, const double* stf) { static_cast<OracleBase*>(h)->set_sources(k, stf); }
void oracle_set_receivers(void* h, const int32_t* k) { static_cast<OracleBase*>(h)->set_receivers(k); }
void oracle_init_model(void* h) { static_cast<OracleBase*>(h)->init_model(); }
void oracle_clear_dynamic(void* h) { static_cast<OracleBase*>(h)->clear_dynamic(); }
void oracle_clear_obs(void* h) { static_cast<OracleBase*>(h)->clear_obs(); }
void oracle_forward_step(void* h, int it, int isrc) { static_cast<OracleBase*>(h)->forward_step(it, isrc); }
void oracle_adjoint_step(void* h, int it) { static_cast<OracleBase*>(h)->adjoint_step(it); }
void oracle_imaging(void* h, const double* fw, double ndt) { static_cast<OracleBase*>(h)->imaging(fw, ndt); }
void oracle_smooth(void* h, double sigma) { static_cast<OracleBase*>(h)->smooth(sigma); }
void oracle_get_obs(void* h, int comp, double* out) { static_cast<OracleBase*>(h)->get_obs(comp, out); }
void oracle_set_obs(void* h, int comp, const double* in) { static_cast<OracleBase*>(h)->set_obs(comp, in); }
int oracle_run_forward(void* h, int isrc, int snap_every, int nfid, const int32_t* fids, double* snaps) {
  return static_cast<OracleBase*>(h)->run_forward(isrc, snap_every, nfid, fids, snaps);
}
int oracle_run_adjoint(void* h, int nruns, const int32_t* run_isrc, const double* obs_y, int adj_interval,
                       double sigma, double* misfits) {
  return static_cast<OracleBase*>(h)->run_adjoint(nruns, run_isrc, obs_y, adj_interval, sigma, misfits);
}

int oracle_exact_gradient(void* h, int isrc, const double* adj, double* g_lam, double* g_mu, double* g_b) {
  return static_cast<OracleBase*>(h)->exact_gradient(isrc, adj, g_lam, g_mu, g_b);
}

// Ricker source-time function, solver.rs:350-356 and the STF table of
// solver.rs:721-733: out[3][nt] = (x, y, z) components for one source.
void oracle_ricker_f32(int nt, float dt, float f0, float t0, float ang_deg, float amp, float* out) {
  const float pi = 3.14159265358979323846f;
  const float rad_per_deg = pi / 180.0f;
  for (int it = 0; it < nt; ++it) {
    float t = float(it) * dt;
    float a = (pi * f0) * (pi * f0);
    float d = t - t0;
    float stf = -amp * (1.0f - 2.0f * a * d * d) * std::exp(-a * d * d);
    float ang = ang_deg * rad_per_deg;
    out[it] = stf * std::sin(ang);
    out[nt + it] = stf;
    out[2 * nt + it] = -stf * std::cos(ang);
  }
}

void oracle_ricker_f64(int nt, double dt, double f0, double t0, double ang_deg, double amp, double* out) {
  const double pi = 3.14159265358979323846;
  for (int it = 0; it < nt; ++it) {
    double t = double(it) * dt;
    double a = (pi * f0) * (pi * f0);
    double d = t - t0;
    double stf = -amp * (1.0 - 2.0 * a * d * d) * std::exp(-a * d * d);
    double ang = ang_deg * (pi / 180.0);
    out[it] = stf * std::sin(ang);
    out[nt + it] = stf;
    out[2 * nt + it] = -stf * std::cos(ang);
  }
}

// Misfit in the FP32 reference arithmetic (solver.rs:432-467) as a free
// function, for tests of the host-side misfit.
double oracle_misfit_f32(int nrec, int nt, float dt, const float* syn, const float* ref, float* adstf) {
  OracleParams p{};
  p.nx = 5; p.nz = 5; p.nt = nt; p.dt = dt; p.nrec = nrec;
  Oracle<float> o(p);
  return o.misfit(syn, ref, adstf);
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
