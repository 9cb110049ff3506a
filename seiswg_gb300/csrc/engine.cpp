// engine.cpp -- device storage, time loop and reference adjoint of one
// simulation.  See engine.h.
#include "engine.h"

#include "batch_plan.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>

namespace seiswg {

void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    throw CudaError(std::string("CUDA error ") + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ") in " +
                    what);
  }
}

// ---------------------------------------------------------------------------
// Arena
// ---------------------------------------------------------------------------
Arena::~Arena() {
  if (base_) cudaFree(base_);
}

void Arena::commit() {
  if (base_ || plan_ == 0) return;
  SW_CUDA(cudaMalloc(reinterpret_cast<void**>(&base_), plan_));
}

void* Arena::take(size_t bytes) {
  size_t b = (bytes + 255) & ~size_t(255);
  if (!base_ || used_ + b > plan_) throw std::logic_error("arena overflow");
  void* p = base_ + used_;
  used_ += b;
  return p;
}

// ---------------------------------------------------------------------------
// Sim
// ---------------------------------------------------------------------------

Sim::Sim(const SimDesc& d, cudaStream_t stream) : d_(d), stream_(stream) {
  if (d.nx < 5 || d.nz < 5) throw std::invalid_argument("grid must be at least 5 x 5");
  if (d.nt < 0) throw std::invalid_argument("nt must be >= 0");
  if (!(d.dx > 0) || !(d.dz > 0)) throw std::invalid_argument("dx and dz must be positive");
  if (!d.sh && !d.psv) throw std::invalid_argument("neither sh nor psv is enabled");
  if (!stream_) {
    SW_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    own_stream_ = true;
  }
  // A warp strip reads columns [j0-4, j0+124) with j0 <= nz-117 (fd_common.cuh).
  ld_ = field_pitch(d.nz);
  const size_t rows_alloc = size_t(d.nx) + 2 * kHaloRows;
  field_elems_ = rows_alloc * size_t(ld_);
  const size_t fb = field_elems_ * sizeof(float);

  int nstate = (d.sh ? 3 : 0) + (d.psv ? 5 : 0) + (d.psv && d.spin ? 4 : 0);
  // The two-step kernels (PSV alone, SH alone) read a dt-scaled copy of the
  // material: dt/rho, dt*lambda, dt*mu.
  const bool scaled = (d.psv && !d.sh && !d.spin) || (d.sh && !d.psv);
  int nmodel = 3 + (d.psv && d.spin ? 5 : 0) + (scaled ? 3 : 0);
  for (int q = 0; q < 2 * nstate + nmodel; ++q) arena_.reserve(fb);
  arena_.reserve(rows_alloc * sizeof(float));
  arena_.reserve(size_t(ld_) * sizeof(float));
  arena_.reserve(size_t(ld_) * sizeof(float));
  arena_.commit();

  for (int b = 0; b < 2; ++b) {
    State& s = st_[b];
    if (d.sh) { s.vy = alloc_field(); s.sxy = alloc_field(); s.szy = alloc_field(); }
    if (d.psv) {
      s.vx = alloc_field(); s.vz = alloc_field(); s.sxx = alloc_field(); s.szz = alloc_field(); s.sxz = alloc_field();
      if (d.spin) { s.vyc = alloc_field(); s.syx = alloc_field(); s.syy = alloc_field(); s.syz = alloc_field(); }
    }
  }
  rho_ = alloc_field(); lam_ = alloc_field(); mu_ = alloc_field();
  if (scaled) { rdt_ = alloc_field(); ldt_ = alloc_field(); mdt_ = alloc_field(); }
  if (d.psv && d.spin) { nu_ = alloc_field(); jm_ = alloc_field(); muc_ = alloc_field(); nuc_ = alloc_field(); mc_ = alloc_field(); }
  taper_x_ = static_cast<float*>(arena_.take(rows_alloc * sizeof(float))) + kHaloRows;
  taper_zb_ = static_cast<float*>(arena_.take(size_t(ld_) * sizeof(float))) + kHaloCols;
  taper_zt_ = static_cast<float*>(arena_.take(size_t(ld_) * sizeof(float))) + kHaloCols;
  // Zero everything; density and micro-inertia halos hold 1 so that the
  // (never used) halo velocities stay finite.
  zero_state();
  for (float* f : {lam_, mu_, nu_, muc_, nuc_, mc_, rdt_, ldt_, mdt_})
    if (f) SW_CUDA(cudaMemsetAsync(f - size_t(kHaloRows) * ld_ - kHaloCols, 0, fb, stream_));
  for (float* f : {rho_, jm_})
    if (f) SW_CUDA(launch_fill_rows(f - kHaloCols, -kHaloRows, d.nx + kHaloRows, ld_, 1.0f, stream_));

  geom_.nx = d.nx;
  geom_.nz = d.nz;
  geom_.ld = ld_;
  geom_.nstrips = (d.nz + kStripCols - 1) / kStripCols;
  geom_.dt = d.dt;
  geom_.rdx = float(1.0 / double(8.0f * d.dx));  // 1 / (8.0 * dx), fd2d.wgsl:156
  geom_.rdz = float(1.0 / double(8.0f * d.dz));
  den_x_ = 8.0f * d.dx;
  den_z_ = 8.0f * d.dz;
  geom_.loader = kLoaderBulk;
  geom_.pdl = 1;
  set_chunk_rows(model_chunk_rows());
  // PSV alone runs its forward passes two steps per launch by default.
  if ((d.psv && !d.sh && !d.spin) || (d.sh && !d.psv)) set_two_step(true);
  SW_CUDA(cudaMalloc(&err_, sizeof(int)));
  SW_CUDA(cudaMemsetAsync(err_, 0, sizeof(int), stream_));
  SW_CUDA(cudaMalloc(&red_, 4 * sizeof(unsigned)));
  use_graphs_ = (size_t(d.nx) * d.nz <= (size_t(1) << 20));
}

Sim::~Sim() {
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  cudaFree(err_);
  cudaFree(red_);
  cudaFree(stf_);
  cudaFree(adstf_);
  cudaFree(inj_dev_[0]);
  cudaFree(inj_dev_[1]);
  cudaFree(probes_);
  cudaFree(probe_acc_);
  cudaFree(probe_hist_);
  cudaFree(tr_idx_);
  cudaFree(obs_);
  cudaFree(fwd_store_);
  cudaFree(ck_store_);
  cudaFree(seg_store_);
  cudaFree(rv_store_);
  cudaFree(adj_store_);
  cudaFree(snap_store_);
  cudaFree(u_tab_);
  cudaFree(obs_in_);
  cudaFree(j_tr_);
  if (g_lam_) cudaFree(g_lam_ - size_t(kHaloRows) * ld_ - kHaloCols);  // the block of the three gradients
  if (kmu_) cudaFree(kmu_ - size_t(kHaloRows) * ld_ - kHaloCols);
  if (tmp_) cudaFree(tmp_ - size_t(kHaloRows) * ld_ - kHaloCols);
  if (own_stream_) cudaStreamDestroy(stream_);
}

void Sim::set_chunk_rows(int lx) {
  if (lx < 4) lx = 4;
  geom_.lx = lx;
  geom_.nchunks = (d_.nx + lx - 1) / lx;
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
}

int Sim::chunk_rows_for(int per_sm, int strip_cols, int extra_rows) const {
  int dev = 0, nsm = 0;
  SW_CUDA(cudaGetDevice(&dev));
  SW_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  if (per_sm < 1) per_sm = 1;
  const long resident = long(per_sm) * nsm * kStepWarps;
  const int nstrips = (d_.nz + strip_cols - 1) / strip_cols;
  int best = 64;
  double best_cost = 1e300;
  for (int lx = 8; lx <= 256; ++lx) {
    const long warps = long(nstrips) * ((d_.nx + lx - 1) / lx);
    const long waves = (warps + resident - 1) / resident;
    const double cost = double(waves) * double(std::min(lx, d_.nx) + extra_rows);
    if (cost < best_cost - 1e-9) { best_cost = cost; best = lx; }
  }
  return best;
}

void Sim::set_two_step(bool on) {
  if (on && !((d_.psv && !d_.sh && !d_.spin) || (d_.sh && !d_.psv)))
    throw std::invalid_argument("the two-step kernels are for PSV alone or SH alone (no spin, not both)");
  if (on && geom2_.lx == 0) set_two_step_rows(0);
  two_step_ = on;
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
}

void Sim::set_two_step_rows(int lx) {
  geom2_ = geom_;
  geom2_.nstrips = (d_.nz + kStripCols2 - 1) / kStripCols2;
  geom2_.lx = lx > 0 ? std::max(lx, 4)
                     : chunk_rows_for(d_.sh ? sh_step2_blocks_per_sm() : step2_blocks_per_sm(), kStripCols2, 11);
  geom2_.nchunks = (d_.nx + geom2_.lx - 1) / geom2_.lx;
  geom2_.loader = kLoaderBulk;
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
}

int Sim::final_buffer(int every) const {
  int b = 0;
  for (int it = 0; it < d_.nt;) {
    const bool snap_between = every > 0 && it > 0 && it % every == 0;
    const int n = (two_step_ && it + 1 < d_.nt && !snap_between) ? 2 : 1;
    b ^= 1;
    it += n;
  }
  return b;
}

namespace {

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link
// against the driver library).
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_tiled() {
  static const EncodeTiled fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return EncodeTiled(nullptr);
    }
    return reinterpret_cast<EncodeTiled>(f);
  }();
  return fn;
}

}  // namespace

// A 3-D map over nfields padded fields (columns ld, rows nx + 2 kHaloRows)
// whose element (0, 0) pointers are `first` + f * stride floats, with boxes of
// 128 columns x 1 row x box_fields fields.
bool encode_fields(CUtensorMap* m, const float* first, ptrdiff_t stride, int nfields, int ld, int rows_alloc,
                   int box_fields) {
  const EncodeTiled fn = encode_tiled();
  if (!fn || stride <= 0) return false;
  const float* base = first - (size_t(kHaloRows) * size_t(ld) + kHaloCols);
  const cuuint64_t dims[3] = {cuuint64_t(ld), cuuint64_t(rows_alloc), cuuint64_t(nfields)};
  const cuuint64_t strides[2] = {cuuint64_t(ld) * sizeof(float), cuuint64_t(stride) * sizeof(float)};
  const cuuint32_t box[3] = {128, 1, cuuint32_t(box_fields)};  // 32 lanes x 4 columns
  const cuuint32_t es[3] = {1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// The material maps (1/rho, lambda, mu at a uniform stride), encoded once.
bool Sim::tma_ready() {
  if (!use_tma_) return false;
  if (tma_mat_ < 0) {
    const int rows_alloc = d_.nx + 2 * kHaloRows;
    const ptrdiff_t dm = lam_ - rho_;
    bool ok = mu_ - lam_ == dm && encode_fields(&mat1_, rho_, dm, 3, ld_, rows_alloc, 1) &&
              encode_fields(&mat2_, rho_, dm, 3, ld_, rows_alloc, 2);
    if (ok && rdt_)  // the two-step kernels' dt-scaled material
      ok = ldt_ - rdt_ == dm && mdt_ - ldt_ == dm && encode_fields(&tma_.rho, rdt_, dm, 3, ld_, rows_alloc, 1) &&
           encode_fields(&tma_.lm, rdt_, dm, 3, ld_, rows_alloc, 2);
    tma_mat_ = ok ? 1 : 0;
  }
  return tma_mat_ == 1;
}

// The PSV reverse step with its rows fetched by tensor copies, where the
// forward state f, the incoming adjoint state a, the material and the
// gradient block lie at uniform strides; false when they do not (the caller
// launches the bulk-copy kernel).
bool Sim::launch_adjoint_tma(const PsvAdjoint& p, const State& f, const State& a) {
  if (!tma_ready()) return false;
  const int rows_alloc = d_.nx + 2 * kHaloRows;
  auto uniform = [](const State& x) {
    const ptrdiff_t d = x.vz - x.vx;
    return d > 0 && x.sxx - x.vz == d && x.szz - x.sxx == d && x.sxz - x.szz == d;
  };
  const ptrdiff_t dg = g_mu_ - g_lam_;
  if (!uniform(f) || !uniform(a) || dg <= 0 || g_b_ - g_mu_ != dg) return false;
  if (tma_grad_ != g_lam_) {
    if (!encode_fields(&tma_adj_.g1, g_lam_, dg, 3, ld_, rows_alloc, 1) ||
        !encode_fields(&tma_adj_.g2, g_lam_, dg, 3, ld_, rows_alloc, 2))
      return false;
    tma_grad_ = g_lam_;
  }
  tma_adj_.m1 = mat1_;
  tma_adj_.m2 = mat2_;
  if (!encode_fields(&tma_adj_.f1, f.vx, f.vz - f.vx, 5, ld_, rows_alloc, 1) ||
      !encode_fields(&tma_adj_.f2, f.vx, f.vz - f.vx, 5, ld_, rows_alloc, 2) ||
      !encode_fields(&tma_adj_.a3, a.vx, a.vz - a.vx, 5, ld_, rows_alloc, 3) ||
      !encode_fields(&tma_adj_.a2, a.vx, a.vz - a.vx, 5, ld_, rows_alloc, 2))
    return false;
  // A producer kernel whose launch register count differs from its register
  // split's is refused before any launch (pc_kernel_ready): the march then
  // issues its own copies.
  const cudaError_t e = reverse_pc_ ? launch_psv_adjoint_pc(p, tma_adj_, stream_) : cudaErrorInvalidConfiguration;
  if (e == cudaErrorInvalidConfiguration) {
    (void)cudaGetLastError();
    reverse_pc_ = false;
    SW_CUDA(launch_psv_adjoint_tma(p, tma_adj_, stream_));
  } else {
    SW_CUDA(e);
  }
  return true;
}

void Sim::set_use_tma(bool on) {
  use_tma_ = on;
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
}

void Sim::enqueue_step2(int it, const State& a, const State& o, const InjectList& inj_in,
                        const ProbeList& probes_in, const State* mid) {
  if (d_.sh) {
    ShStep p{};
    p.g = geom2_;
    p.vy0 = a.vy; p.sxy0 = a.sxy; p.szy0 = a.szy;
    p.vy1 = o.vy; p.sxy1 = o.sxy; p.szy1 = o.szy;
    if (mid) { p.vym = mid->vy; p.sxym = mid->sxy; p.szym = mid->szy; }
    p.rho = rdt_; p.mu = mdt_;  // dt/rho, dt*mu
    p.taper_x = taper_x_; p.taper_zb = taper_zb_; p.taper_zt = taper_zt_;
    p.inj = inj_in;
    p.inj.it = it;
    p.probes = probes_in;
    p.probes.it = it;
    p.err = err_;
    if (probes_in.n) p.probes.n = probe_split_;
    const ptrdiff_t ds = a.sxy - a.vy;
    if (tma_ready() && a.szy - a.sxy == ds && encode_fields(&tma_.sig, a.vy, ds, 3, ld_, d_.nx + 2 * kHaloRows, 2) &&
        encode_fields(&tma_.vel, a.vy, ds, 3, ld_, d_.nx + 2 * kHaloRows, 1)) {
      SW_CUDA(launch_sh_step2_tma(p, tma_, stream_));
    } else {
      SW_CUDA(launch_sh_step2(p, stream_));
    }
    ++launches_;
    return;
  }
  PsvStep p{};
  p.g = geom2_;
  p.vx0 = a.vx; p.vz0 = a.vz; p.sxx0 = a.sxx; p.szz0 = a.szz; p.sxz0 = a.sxz;
  p.vx1 = o.vx; p.vz1 = o.vz; p.sxx1 = o.sxx; p.szz1 = o.szz; p.sxz1 = o.sxz;
  if (mid) { p.vxm = mid->vx; p.vzm = mid->vz; p.sxxm = mid->sxx; p.szzm = mid->szz; p.sxzm = mid->sxz; }
  p.rho = rdt_; p.lam = ldt_; p.mu = mdt_;  // dt/rho, dt*lambda, dt*mu
  p.taper_x = taper_x_; p.taper_zb = taper_zb_; p.taper_zt = taper_zt_;
  p.inj = inj_in;
  p.inj.it = it;
  p.probes = probes_in;
  p.probes.it = it;
  p.err = err_;
  if (probes_in.n) {
    p.probes.list = probes_ + probe_split_;
    p.probes.n = nprobe_ - probe_split_;
  }
  // Tensor copies where the state's five fields and the material's three
  // lie at uniform strides (state buffers and checkpoint slots do).
  const int rows_alloc = d_.nx + 2 * kHaloRows;
  const ptrdiff_t ds = a.vz - a.vx;
  if (tma_ready() && a.sxx - a.vz == ds && a.szz - a.sxx == ds && a.sxz - a.szz == ds &&
      encode_fields(&tma_.sig, a.vx, ds, 5, ld_, rows_alloc, 3) &&
      encode_fields(&tma_.vel, a.vx, ds, 5, ld_, rows_alloc, 2)) {
    const cudaError_t e = two_step_pc_ ? launch_psv_step2_pc(p, tma_, stream_) : cudaErrorInvalidConfiguration;
    if (e == cudaErrorInvalidConfiguration) {  // refused before any launch, as above
      (void)cudaGetLastError();
      two_step_pc_ = false;
      SW_CUDA(launch_psv_step2_tma(p, tma_, stream_));
    } else {
      SW_CUDA(e);
    }
  } else {
    SW_CUDA(launch_psv_step2(p, stream_));
  }
  ++launches_;
}

int Sim::model_chunk_rows() const {
  return chunk_rows_for(step_blocks_per_sm(d_.psv, d_.psv && d_.spin, geom_.loader), kStripCols, 5);
}

Geom Sim::adjoint_geom() {
  if (adj_lx_[geom_.loader] == 0)
    adj_lx_[geom_.loader] = chunk_rows_for(adjoint_blocks_per_sm(d_.psv, geom_.loader), kStripCols, 5);
  Geom g = geom_;
  g.lx = adj_lx_[geom_.loader];
  g.nchunks = (d_.nx + g.lx - 1) / g.lx;
  return g;
}

double Sim::autotune(int steps) {
  if (steps < 1) steps = 1;
  SW_CUDA(cudaStreamSynchronize(stream_));
  const bool graphs = use_graphs_;
  use_graphs_ = false;
  InjectList inj = source_injections(-1);
  ProbeList none{};
  cudaEvent_t e0, e1;
  SW_CUDA(cudaEventCreate(&e0));
  SW_CUDA(cudaEventCreate(&e1));
  std::vector<int> rows = {1, 2, 4, 8, 16, 32, 64, 128};
  const int model = model_chunk_rows();
  if (std::find(rows.begin(), rows.end(), model) == rows.end()) rows.push_back(model);
  float best = 1e30f;
  int best_loader = geom_.loader, best_lx = geom_.lx;
  for (int loader : {kLoaderDirect, kLoaderBulk}) {
    geom_.loader = loader;
    for (int lx : rows) {
      if (lx > std::max(d_.nx, 1) && lx != rows.front()) continue;
      geom_.lx = lx;
      geom_.nchunks = (d_.nx + lx - 1) / lx;
      for (int it = 0; it < 2; ++it) enqueue_step(it, it & 1, inj, none, false);  // warm-up
      SW_CUDA(cudaEventRecord(e0, stream_));
      for (int it = 0; it < steps; ++it) enqueue_step(it % std::max(d_.nt, 1), it & 1, inj, none, false);
      SW_CUDA(cudaEventRecord(e1, stream_));
      SW_CUDA(cudaEventSynchronize(e1));
      float ms = 0.0f;
      SW_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best) { best = ms; best_loader = loader; best_lx = lx; }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  zero_state();
  use_graphs_ = graphs;
  geom_.loader = best_loader;
  set_chunk_rows(best_lx);
  check_device_error();
  return 1e3 * double(best) / steps;
}

void Sim::set_wait_polls(unsigned polls) {
  geom_.wait_polls = geom2_.wait_polls = polls;
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
}

void Sim::set_pdl(bool on) {
  geom_.pdl = geom2_.pdl = on ? 1u : 0u;
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
}

void Sim::set_arm_extra(unsigned bytes) {
  geom_.arm_extra = geom2_.arm_extra = bytes;
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
}

void Sim::set_loader(int loader) {
  if (loader != kLoaderDirect && loader != kLoaderBulk) throw std::invalid_argument("unknown loader");
  geom_.loader = loader;
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
}

// The device error word is reported once: it is cleared after it has been
// read, so that the simulation stays usable for the next run.
void Sim::check_device_error() const {
  int e = 0;
  SW_CUDA(cudaMemcpyAsync(&e, err_, sizeof(int), cudaMemcpyDeviceToHost, stream_));
  SW_CUDA(cudaStreamSynchronize(stream_));
  if (!e) return;
  SW_CUDA(cudaMemsetAsync(err_, 0, sizeof(int), stream_));
  SW_CUDA(cudaStreamSynchronize(stream_));
  if (e & kErrWaitTimeout)
    throw WaitTimeout("a step kernel gave up waiting for its row pipeline (bounded wait expired); "
                      "results of this run are invalid");
  if (e & kErrNonFiniteTraces)
    throw NumericError("the receiver traces hold NaN or infinite values (an unstable run or a bad model)");
  if (e & kErrNonFiniteGradient)
    throw NumericError("the gradient holds NaN or infinite values (an unstable run or a bad adjoint source)");
}

// Von Neumann limits of the staggered fourth-order scheme (leapfrog in time,
// difference weights 9/8 and 1/24 whose magnitudes add up to 7/6):
//   wave:  dt c (7/6) sqrt(1/dx^2 + 1/dz^2) <= 1, c the P speed sqrt((lambda
//          + 2 mu)/rho) with PSV, the S speed sqrt(mu/rho) with SH alone;
//   spin:  (dt/2) sqrt(w0^2 + cc^2 (7/3)^2 (1/dx^2 + 1/dz^2)) <= 1, w0 =
//          sqrt(4 nu / J) the rotation rate and cc = sqrt((mu_c + nu_c)/J)
//          the couple-wave speed.
// Each is necessary for its own subsystem; the coupling terms are not
// analysed.  A run that exceeds either, or a model with non-finite or
// negative squared speeds, is rejected before it starts.
void Sim::check_stability() {
  unsigned h[4] = {0, 0, 0, 0};
  SW_CUDA(cudaMemsetAsync(red_, 0, 4 * sizeof(unsigned), stream_));
  SW_CUDA(launch_max_speeds(lam_, mu_, rho_, nu_, (d_.psv && d_.spin) ? jm_ : nullptr, mc_, d_.psv, d_.nx, d_.nz,
                            ld_, red_, stream_));
  SW_CUDA(cudaMemcpyAsync(h, red_, 4 * sizeof(unsigned), cudaMemcpyDeviceToHost, stream_));
  SW_CUDA(cudaStreamSynchronize(stream_));
  float c2, w2, q2;
  std::memcpy(&c2, &h[0], 4);
  std::memcpy(&w2, &h[1], 4);
  std::memcpy(&q2, &h[2], 4);
  const double k = std::sqrt(1.0 / (double(d_.dx) * d_.dx) + 1.0 / (double(d_.dz) * d_.dz));
  const double dt = d_.dt;
  cfl_wave_ = dt * std::sqrt(double(c2)) * (7.0 / 6.0) * k;
  cfl_spin_ = (d_.psv && d_.spin) ? 0.5 * dt * std::sqrt(double(w2) + double(q2) * (7.0 / 3.0) * (7.0 / 3.0) * k * k)
                                  : 0.0;
  if (!stability_check_) return;
  if (h[3])
    throw std::invalid_argument("model: non-finite or negative squared wave speeds (check rho, vp/vs or the moduli)");
  if (cfl_wave_ > 1.0) {
    char m[256];
    std::snprintf(m, sizeof m,
                  "dt = %g is unstable: dt c (7/6) sqrt(1/dx^2 + 1/dz^2) = %.4f > 1 with c = %.6g m/s "
                  "(largest dt %.6g)",
                  dt, cfl_wave_, std::sqrt(double(c2)), dt / cfl_wave_);
    throw std::invalid_argument(m);
  }
  if (cfl_spin_ > 1.0) {
    char m[256];
    std::snprintf(m, sizeof m,
                  "dt = %g is unstable for the spin field: (dt/2) sqrt(4 nu/J + (mu_c+nu_c)/J (7/3)^2 "
                  "(1/dx^2 + 1/dz^2)) = %.4f > 1 (largest dt %.6g)",
                  dt, cfl_spin_, dt / cfl_spin_);
    throw std::invalid_argument(m);
  }
}

float* Sim::alloc_field() { return field_ptr(static_cast<float*>(arena_.take(field_elems_ * sizeof(float)))); }

void Sim::zero_state() {
  const size_t fb = field_elems_ * sizeof(float);
  for (int b = 0; b < 2; ++b) {
    const State& s = st_[b];
    for (float* f : {s.vy, s.sxy, s.szy, s.vx, s.vz, s.sxx, s.szz, s.sxz, s.vyc, s.syx, s.syy, s.syz})
      if (f) SW_CUDA(cudaMemsetAsync(f - size_t(kHaloRows) * ld_ - kHaloCols, 0, fb, stream_));
  }
}

void Sim::synchronize() const {
  SW_CUDA(cudaStreamSynchronize(stream_));
  check_device_error();
}

void Sim::upload_model(ModelField f, const float* host) {
  float* dst = nullptr;
  switch (f) {
    case ModelField::VP: dst = lam_; vps_input_ = true; break;
    case ModelField::VS: dst = mu_; vps_input_ = true; break;
    case ModelField::RHO: dst = rho_; break;
    case ModelField::LAMBDA: dst = lam_; break;
    case ModelField::MU: dst = mu_; break;
    case ModelField::NU: dst = nu_; break;
    case ModelField::J: dst = jm_; break;
    case ModelField::MU_C: dst = muc_; break;
    case ModelField::NU_C: dst = nuc_; break;
    case ModelField::LAMBDA_C: return;  // loaded but unused by the stencil (fd2d.wgsl:428-445)
  }
  if (!dst) throw std::invalid_argument("model field not used by this physics");
  prepared_ = false;
  SW_CUDA(cudaMemcpy2DAsync(dst, size_t(ld_) * sizeof(float), host, size_t(d_.nz) * sizeof(float),
                            size_t(d_.nz) * sizeof(float), size_t(d_.nx), cudaMemcpyHostToDevice, stream_));
}

void Sim::prepare_model() {
  if (prepared_) throw std::logic_error("prepare_model called twice without a new model upload");
  if (vps_input_) SW_CUDA(launch_vps2lm(lam_, mu_, rho_, d_.nx, d_.nz, ld_, stream_));
  if (mc_) SW_CUDA(launch_add_fields(mc_, muc_, nuc_, d_.nx, d_.nz, ld_, stream_));
  // The step kernels read the buoyancy 1/rho and 1/J.
  SW_CUDA(launch_reciprocal(rho_, d_.nx, d_.nz, ld_, stream_));
  if (jm_) SW_CUDA(launch_reciprocal(jm_, d_.nx, d_.nz, ld_, stream_));
  // The two-step kernels' material, dt/rho, dt*lambda, dt*mu (halos included).
  if (rdt_) {
    const size_t h = size_t(kHaloRows) * ld_ + kHaloCols;
    const float dt = d_.dt;
    SW_CUDA(launch_scale(rdt_ - h, rho_ - h, long(field_elems_), dt, stream_));
    SW_CUDA(launch_scale(ldt_ - h, lam_ - h, long(field_elems_), dt, stream_));
    SW_CUDA(launch_scale(mdt_ - h, mu_ - h, long(field_elems_), dt, stream_));
  }
  prepared_ = true;
  check_stability();

  // Absorbing taper, set_bound (fd2d.wgsl:205-235): b = ((1*eL)*eR)*eB*eT with
  // e = exp(-(alpha*d)^2); separable into a row factor (left, right) and two
  // column factors (bottom, top) applied in the reference's order.
  const uint32_t w = uint32_t(d_.abs_width), nx = uint32_t(d_.nx), nz = uint32_t(d_.nz);
  const float a = d_.abs_alpha;
  std::vector<float> tx(size_t(d_.nx) + 2 * kHaloRows, 1.0f), tb(size_t(ld_), 1.0f), tt(size_t(ld_), 1.0f);
  for (uint32_t i = 0; i < nx; ++i) {
    float b = 1.0f;
    if (d_.abs_left && (i + 1u) < w) { float aw = a * float(w - i - 1u); b *= std::exp(-aw * aw); }
    if (d_.abs_right && i > (nx - w)) { float aw = a * float(w + i - nx); b *= std::exp(-aw * aw); }
    tx[kHaloRows + i] = b;
  }
  for (uint32_t j = 0; j < nz; ++j) {
    if (d_.abs_bottom && j > (nz - w)) { float aw = a * float(w + j - nz); tb[kHaloCols + j] = std::exp(-aw * aw); }
    if (d_.abs_top && (j + 1u) < w) { float aw = a * float(w - j - 1u); tt[kHaloCols + j] = std::exp(-aw * aw); }
  }
  SW_CUDA(cudaMemcpyAsync(taper_x_ - kHaloRows, tx.data(), tx.size() * sizeof(float), cudaMemcpyHostToDevice, stream_));
  SW_CUDA(cudaMemcpyAsync(taper_zb_ - kHaloCols, tb.data(), tb.size() * sizeof(float), cudaMemcpyHostToDevice, stream_));
  SW_CUDA(cudaMemcpyAsync(taper_zt_ - kHaloCols, tt.data(), tt.size() * sizeof(float), cudaMemcpyHostToDevice, stream_));
  SW_CUDA(cudaStreamSynchronize(stream_));  // the host vectors die here
}

void Sim::set_sources(int n, const int* i, const int* j, const float* stf_xyz) {
  if (n < 0) throw std::invalid_argument("negative source count");
  for (int s = 0; s < n; ++s)
    if (i[s] < 0 || i[s] >= d_.nx || j[s] < 0 || j[s] >= d_.nz)
      throw std::invalid_argument("source " + std::to_string(s) + " lies outside the grid");
  SW_CUDA(cudaStreamSynchronize(stream_));  // queued work may still read the old tables
  nsrc_ = n;
  src_i_.assign(i, i + n);
  src_j_.assign(j, j + n);
  cudaFree(stf_);
  stf_ = nullptr;
  cudaFree(inj_dev_[0]);
  inj_dev_[0] = nullptr;
  inj_cap_[0] = 0;
  size_t bytes = size_t(3) * n * d_.nt * sizeof(float);
  if (bytes) {
    SW_CUDA(cudaMalloc(&stf_, bytes));
    SW_CUDA(cudaMemcpyAsync(stf_, stf_xyz, bytes, cudaMemcpyHostToDevice, stream_));
    SW_CUDA(cudaStreamSynchronize(stream_));
  }
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
}

void Sim::set_receivers(int n, const int* i, const int* j) {
  if (n < 0) throw std::invalid_argument("negative receiver count");
  for (int r = 0; r < n; ++r)
    if (i[r] < 0 || i[r] >= d_.nx || j[r] < 0 || j[r] >= d_.nz)
      throw std::invalid_argument("receiver " + std::to_string(r) + " lies outside the grid");
  SW_CUDA(cudaStreamSynchronize(stream_));
  nrec_ = n;
  rec_i_.assign(i, i + n);
  rec_j_.assign(j, j + n);
  build_probe_tables();
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
}

// Probes: SH uy (vy) at each receiver; PSV ux (vx), uz (vz); spin uy_c (vy_c)
// and the 8 displacement samples of the curl stencil (compute_du_grad,
// fd2d.wgsl:450-456).  One probe per (cell, component); SH probes come first
// in the device list, then the PSV ones (each kernel walks its own segment).
void Sim::build_probe_tables() {
  std::map<std::tuple<int, int, int>, int> index;
  std::vector<Probe> list;
  auto probe = [&](int i, int j, int comp) -> int {
    auto k2 = std::make_tuple(i, j, comp);
    auto it = index.find(k2);
    if (it != index.end()) return it->second;
    int idx = int(list.size());
    index[k2] = idx;
    list.push_back(Probe{i, j, comp, idx});
    return idx;
  };
  std::vector<int> tr(size_t(nrec_) * 12, -1);
  for (int r = 0; r < nrec_; ++r) {
    const int i = rec_i_[r], j = rec_j_[r];
    int* t = &tr[size_t(r) * 12];
    if (d_.sh) t[0] = probe(i, j, kProbeVY);
    if (d_.psv) {
      t[1] = probe(i, j, kProbeVX);
      t[2] = probe(i, j, kProbeVZ);
      if (d_.spin) {
        t[3] = probe(i, j, kProbeVYC);
        if (i >= 1 && i < d_.nx - 2)
          for (int q = 0; q < 4; ++q) t[4 + q] = probe(i - 1 + q, j, kProbeVZ);
        if (j >= 1 && j < d_.nz - 2)
          for (int q = 0; q < 4; ++q) t[8 + q] = probe(i, j - 1 + q, kProbeVX);
      }
    }
  }
  // SH segment first, then PSV; each sorted by (i, j).
  std::stable_sort(list.begin(), list.end(), [](const Probe& a, const Probe& b) {
    int sa = a.comp == kProbeVY ? 0 : 1, sb = b.comp == kProbeVY ? 0 : 1;
    if (sa != sb) return sa < sb;
    if (a.i != b.i) return a.i < b.i;
    return a.j < b.j;
  });
  nprobe_ = int(list.size());
  cudaFree(probes_); probes_ = nullptr;
  cudaFree(probe_acc_); probe_acc_ = nullptr;
  cudaFree(probe_hist_); probe_hist_ = nullptr;
  cudaFree(tr_idx_); tr_idx_ = nullptr;
  cudaFree(obs_); obs_ = nullptr;
  if (nprobe_) {
    SW_CUDA(cudaMalloc(&probes_, list.size() * sizeof(Probe)));
    SW_CUDA(cudaMemcpyAsync(probes_, list.data(), list.size() * sizeof(Probe), cudaMemcpyHostToDevice, stream_));
    SW_CUDA(cudaMalloc(&probe_acc_, size_t(nprobe_) * sizeof(float)));
    SW_CUDA(cudaMalloc(&probe_hist_, std::max<size_t>(1, size_t(nprobe_) * d_.nt) * sizeof(float)));
  }
  if (nrec_) {
    SW_CUDA(cudaMalloc(&tr_idx_, tr.size() * sizeof(int) + size_t(nrec_) * 2 * sizeof(int)));
    std::vector<int> packed(tr);
    for (int r = 0; r < nrec_; ++r) { packed.push_back(rec_i_[r]); packed.push_back(rec_j_[r]); }
    SW_CUDA(cudaMemcpyAsync(tr_idx_, packed.data(), packed.size() * sizeof(int), cudaMemcpyHostToDevice, stream_));
    size_t ob = std::max<size_t>(1, size_t(5) * nrec_ * d_.nt) * sizeof(float);
    SW_CUDA(cudaMalloc(&obs_, ob));
    SW_CUDA(cudaMemsetAsync(obs_, 0, ob, stream_));
  }
  SW_CUDA(cudaStreamSynchronize(stream_));  // the host tables above die here
  // Segment boundary: number of SH probes.
  int nsh = 0;
  for (const Probe& p : list) nsh += (p.comp == kProbeVY);
  probe_split_ = nsh;
}

// Uploads on the engine's stream, so that work already queued that reads the
// previous list finishes first (a legacy-stream copy would not wait for it).
void Sim::upload_inject(const std::vector<Inject>& list, int which) {
  int n = int(list.size());
  if (n > inj_cap_[which]) {
    SW_CUDA(cudaStreamSynchronize(stream_));
    cudaFree(inj_dev_[which]);
    inj_dev_[which] = nullptr;
    SW_CUDA(cudaMalloc(&inj_dev_[which], size_t(n) * sizeof(Inject)));
    inj_cap_[which] = n;
  }
  inj_n_[which] = n;
  if (n)
    SW_CUDA(cudaMemcpyAsync(inj_dev_[which], list.data(), size_t(n) * sizeof(Inject), cudaMemcpyHostToDevice,
                            stream_));
}

float* Sim::state_ptr(StateField f, int b) const {
  const State& s = st_[b];
  switch (f) {
    case StateField::VY: return s.vy;
    case StateField::SXY: return s.sxy;
    case StateField::SZY: return s.szy;
    case StateField::VX: return s.vx;
    case StateField::VZ: return s.vz;
    case StateField::SXX: return s.sxx;
    case StateField::SZZ: return s.szz;
    case StateField::SXZ: return s.sxz;
    case StateField::VYC: return s.vyc;
    case StateField::SYX: return s.syx;
    case StateField::SYY: return s.syy;
    case StateField::SYZ: return s.syz;
  }
  return nullptr;
}

void Sim::enqueue_step(int it, int b, const InjectList& inj_in, const ProbeList& probes_in, bool sh_only) {
  enqueue_step_states(it, st_[b], st_[1 - b], inj_in, probes_in, sh_only);
}

void Sim::enqueue_step_states(int it, const State& a, const State& o, const InjectList& inj_in,
                              const ProbeList& probes_in, bool sh_only) {
  InjectList inj = inj_in;
  inj.it = it;
  if (d_.sh) {
    ShStep p{};
    p.g = geom_;
    p.vy0 = a.vy; p.sxy0 = a.sxy; p.szy0 = a.szy;
    p.vy1 = o.vy; p.sxy1 = o.sxy; p.szy1 = o.szy;
    p.rho = rho_; p.mu = mu_;
    p.taper_x = taper_x_; p.taper_zb = taper_zb_; p.taper_zt = taper_zt_;
    p.inj = inj;
    p.probes = probes_in;
    p.probes.it = it;
    p.err = err_;
    if (probes_in.n) p.probes.n = probe_split_;
    SW_CUDA(launch_sh_step(p, stream_));
    ++launches_;
  }
  if (d_.psv && !sh_only) {
    PsvStep p{};
    p.g = geom_;
    p.vx0 = a.vx; p.vz0 = a.vz; p.sxx0 = a.sxx; p.szz0 = a.szz; p.sxz0 = a.sxz;
    p.vx1 = o.vx; p.vz1 = o.vz; p.sxx1 = o.sxx; p.szz1 = o.szz; p.sxz1 = o.sxz;
    p.vyc0 = a.vyc; p.syx0 = a.syx; p.syy0 = a.syy; p.syz0 = a.syz;
    p.vyc1 = o.vyc; p.syx1 = o.syx; p.syy1 = o.syy; p.syz1 = o.syz;
    p.rho = rho_; p.lam = lam_; p.mu = mu_; p.nu = nu_; p.jm = jm_; p.mc = mc_;
    p.taper_x = taper_x_; p.taper_zb = taper_zb_; p.taper_zt = taper_zt_;
    p.inj = inj;
    p.probes = probes_in;
    p.probes.it = it;
    p.err = err_;
    if (probes_in.n) {
      p.probes.list = probes_ + probe_split_;
      p.probes.n = nprobe_ - probe_split_;
    }
    SW_CUDA(launch_psv_step(p, d_.spin, stream_));
    ++launches_;
  }
}

void Sim::run_loop(const std::string& key, const std::function<void()>& body) {
  if (!use_graphs_) {
    body();
    return;
  }
  auto it = graphs_.find(key);
  if (it == graphs_.end()) {
    uint64_t before = launches_;
    cudaGraph_t g = nullptr;
    SW_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    try {
      body();
    } catch (...) {
      cudaStreamEndCapture(stream_, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    SW_CUDA(cudaStreamEndCapture(stream_, &g));
    cudaGraphExec_t exec = nullptr;
    cudaError_t e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    SW_CUDA(e);
    it = graphs_.emplace(key, exec).first;
    graph_nodes_[key] = launches_ - before;
    launches_ = before;
  }
  SW_CUDA(cudaGraphLaunch(it->second, stream_));
  launches_ += graph_nodes_[key];
}

void Sim::copy_field_to_host(const float* dev, float* host) const {
  SW_CUDA(cudaMemcpy2DAsync(host, size_t(d_.nz) * sizeof(float), dev, size_t(ld_) * sizeof(float),
                            size_t(d_.nz) * sizeof(float), size_t(d_.nx), cudaMemcpyDeviceToHost, stream_));
}

InjectList Sim::source_injections(int isrc) {
  if (isrc >= nsrc_) throw std::invalid_argument("source index out of range");
  std::vector<Inject> list;
  for (int s = 0; s < nsrc_; ++s)
    if (isrc < 0 || s == isrc) list.push_back(Inject{src_i_[s], src_j_[s], s, 0});
  std::stable_sort(list.begin(), list.end(),
                   [](const Inject& a, const Inject& b) { return a.i != b.i ? a.i < b.i : a.j < b.j; });
  upload_inject(list, 0);
  InjectList inj{};
  inj.list = inj_dev_[0];
  inj.n = inj_n_[0];
  inj.nt = d_.nt;
  inj.val_x = stf_;
  inj.val_y = stf_ ? stf_ + size_t(nsrc_) * d_.nt : nullptr;
  inj.val_z = stf_ ? stf_ + size_t(2) * nsrc_ * d_.nt : nullptr;
  return inj;
}

ProbeList Sim::probe_list() const {
  ProbeList pl{};
  pl.list = probes_;
  pl.n = nprobe_;
  pl.nt = d_.nt;
  pl.acc = probe_acc_;
  pl.hist = probe_hist_;
  return pl;
}

void Sim::enqueue_traces() {
  if (!nrec_) return;
  TraceSpec t{};
  t.nrec = nrec_;
  t.nt = d_.nt;
  t.sh = d_.sh;
  t.psv = d_.psv;
  t.spin = d_.psv && d_.spin;
  t.idx = tr_idx_;
  t.rec_ij = tr_idx_ + size_t(nrec_) * 12;
  t.nx = d_.nx;
  t.nz = d_.nz;
  t.den_x = den_x_;
  t.den_z = den_z_;
  t.hist = probe_hist_;
  t.obs = obs_;
  SW_CUDA(launch_assemble_traces(t, stream_));
  // NaN / infinity watchdog: a bit in the error word that the call reading
  // the traces reports.
  SW_CUDA(launch_check_finite(obs_, 5, nrec_ * d_.nt, long(nrec_) * d_.nt, err_, kErrNonFiniteTraces, stream_));
  launches_ += 2;
}

void Sim::run_forward(int isrc, Snapshots* snaps) {
  InjectList inj = source_injections(isrc);
  ProbeList pl = probe_list();
  zero_state();
  if (nprobe_) SW_CUDA(cudaMemsetAsync(probe_acc_, 0, size_t(nprobe_) * sizeof(float), stream_));

  int every = snaps ? snaps->every : 0;
  std::vector<int> snap_steps;
  if (every > 0)
    for (int it = 1; it < d_.nt; ++it)
      if (it % every == 0) snap_steps.push_back(it);
  const size_t nf = snaps ? snaps->fields.size() : 0;
  const size_t need = snap_steps.size() * nf;
  if (need > snap_cap_) {
    cudaFree(snap_store_);
    snap_store_ = nullptr;
    SW_CUDA(cudaMalloc(&snap_store_, need * field_elems_ * sizeof(float)));
    snap_cap_ = need;
    for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
    graphs_.clear();
  }
  std::vector<float*> snap_src;
  for (StateField f : (snaps ? snaps->fields : std::vector<StateField>{}))
    for (int b = 0; b < 2; ++b)
      if (!state_ptr(f, b)) throw std::invalid_argument("snapshot field not present in this physics");

  std::string key = "fwd/" + std::to_string(inj.n) + "/" + std::to_string(every);
  for (StateField f : (snaps ? snaps->fields : std::vector<StateField>{})) key += "/" + std::to_string(int(f));
  const size_t fbytes = field_elems_ * sizeof(float);
  // Small SH grids: the whole run on chip in one thread-block cluster.
  bool only_vy = true;
  for (StateField f : (snaps ? snaps->fields : std::vector<StateField>{})) only_vy = only_vy && f == StateField::VY;
  if (use_cluster_ && d_.sh && !d_.psv && only_vy && inj.n <= kClusterSources && probe_split_ <= kClusterProbes &&
      d_.nt > 0) {
    if (cluster_ctas_ < 0) cluster_ctas_ = sh_cluster_ctas(d_.nx, d_.nz);
    if (cluster_ctas_ > 0) {
      ShCluster p{};
      p.nx = d_.nx; p.nz = d_.nz; p.ld = ld_;
      p.rows = (d_.nx + cluster_ctas_ - 1) / cluster_ctas_;
      p.it0 = 0; p.it1 = d_.nt;
      p.dt = geom_.dt; p.rdx = geom_.rdx; p.rdz = geom_.rdz;
      p.vy0 = p.vy1 = st_[0].vy; p.sxy0 = p.sxy1 = st_[0].sxy; p.szy0 = p.szy1 = st_[0].szy;
      p.rho = rho_; p.mu = mu_;
      p.taper_x = taper_x_; p.taper_zb = taper_zb_; p.taper_zt = taper_zt_;
      p.inj = inj;
      p.probes = pl;
      p.probes.n = probe_split_;
      p.probes.it = 0;
      p.snap = (every > 0 && nf > 0) ? snap_store_ + size_t(kHaloRows) * ld_ + kHaloCols : nullptr;
      p.snap_every = every > 0 ? every : 1;
      p.snap_first = 0;
      p.snap_stride = (long long)field_elems_;
      run_loop(key + "/cluster", [&] {
        SW_CUDA(launch_sh_cluster(p, cluster_ctas_, stream_));
        ++launches_;
        enqueue_traces();
      });
      cur_buf_ = 0;
      if (snaps) {
        snaps->steps = snap_steps;
        snaps->frames.assign(need, std::vector<float>());
        for (size_t q = 0; q < need; ++q) {
          snaps->frames[q].resize(size_t(d_.nx) * d_.nz);
          copy_field_to_host(snap_store_ + q * field_elems_ + size_t(kHaloRows) * ld_ + kHaloCols,
                             snaps->frames[q].data());
        }
        SW_CUDA(cudaStreamSynchronize(stream_));
      }
      return;
    }
  }
  if (two_step_) key += "/2";
  run_loop(key, [&] {
    size_t q = 0;
    int b = 0;  // buffer holding the state before step it
    auto snap = [&](int it) {  // the state after step it, if a snapshot is due
      if (!(every > 0 && it > 0 && it % every == 0)) return;
      for (StateField f : snaps->fields) {
        const float* src = state_ptr(f, b) - size_t(kHaloRows) * ld_ - kHaloCols;
        SW_CUDA(cudaMemcpyAsync(snap_store_ + q * field_elems_, src, fbytes, cudaMemcpyDeviceToDevice, stream_));
        ++q;
      }
    };
    for (int it = 0; it < d_.nt;) {
      const bool snap_between = every > 0 && it > 0 && it % every == 0;
      if (two_step_ && it + 1 < d_.nt && !snap_between) {
        enqueue_step2(it, st_[b], st_[1 - b], inj, pl);
        b ^= 1;
        snap(it + 1);
        it += 2;
      } else {
        enqueue_step(it, b, inj, pl, false);
        b ^= 1;
        snap(it);
        ++it;
      }
    }
    enqueue_traces();
  });
  cur_buf_ = final_buffer(every);
  if (snaps) {
    snaps->steps = snap_steps;
    snaps->frames.assign(need, std::vector<float>());
    for (size_t q = 0; q < need; ++q) {
      snaps->frames[q].resize(size_t(d_.nx) * d_.nz);
      copy_field_to_host(snap_store_ + q * field_elems_ + size_t(kHaloRows) * ld_ + kHaloCols,
                         snaps->frames[q].data());
    }
    SW_CUDA(cudaStreamSynchronize(stream_));
  }
}

void Sim::download_traces(float* host, unsigned comps) const {
  check_device_error();
  if (!nrec_) return;
  const size_t n = size_t(nrec_) * d_.nt;
  if ((comps & 0x1f) == 0x1f) {
    SW_CUDA(cudaMemcpyAsync(host, obs_, 5 * n * sizeof(float), cudaMemcpyDeviceToHost, stream_));
  } else {
    for (int c = 0; c < 5; ++c)
      if (comps & (1u << c))
        SW_CUDA(cudaMemcpyAsync(host + c * n, obs_ + c * n, n * sizeof(float), cudaMemcpyDeviceToHost, stream_));
  }
  SW_CUDA(cudaStreamSynchronize(stream_));
}

void Sim::download_state(StateField f, float* host) const {
  const float* p = state_ptr(f, cur_buf_);
  if (!p) throw std::invalid_argument("field not present in this physics");
  copy_field_to_host(p, host);
  SW_CUDA(cudaStreamSynchronize(stream_));
  check_device_error();
}

// ---------------------------------------------------------------------------
// Reference adjoint
// ---------------------------------------------------------------------------
void Sim::clear_kmu() {
  const size_t fb = field_elems_ * sizeof(float);
  if (!kmu_) {
    float* a = nullptr;
    SW_CUDA(cudaMalloc(&a, fb));
    kmu_ = field_ptr(a);
    SW_CUDA(cudaMalloc(&a, fb));
    tmp_ = field_ptr(a);
    SW_CUDA(cudaMemsetAsync(tmp_ - size_t(kHaloRows) * ld_ - kHaloCols, 0, fb, stream_));
  }
  SW_CUDA(cudaMemsetAsync(kmu_ - size_t(kHaloRows) * ld_ - kHaloCols, 0, fb, stream_));
}

void Sim::adjoint_forward(int isrc, int adj_interval) {
  if (adj_interval <= 0) throw std::invalid_argument("adj_interval must be positive");
  const int nsa = d_.nt / adj_interval;
  if (nsa == 0) throw std::invalid_argument("adj_interval >= nt");
  if (!kmu_) clear_kmu();
  const size_t fb = field_elems_ * sizeof(float);
  if (fwd_nsa_ != nsa) {
    cudaFree(fwd_store_);
    fwd_store_ = nullptr;
    fwd_bytes_ = size_t(nsa) * fb;
    SW_CUDA(cudaMalloc(&fwd_store_, fwd_bytes_));
    fwd_nsa_ = nsa;
    for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
    graphs_.clear();
  }
  InjectList inj = source_injections(isrc);
  ProbeList pl = probe_list();
  zero_state();
  if (nprobe_) SW_CUDA(cudaMemsetAsync(probe_acc_, 0, size_t(nprobe_) * sizeof(float), stream_));
  if (!d_.sh) {  // the reference's adjoint loops dispatch SH kernels only (solver.rs:1400)
    SW_CUDA(cudaMemsetAsync(obs_, 0, size_t(5) * nrec_ * d_.nt * sizeof(float), stream_));
    return;
  }
  std::string key = "adjf/" + std::to_string(inj.n) + "/" + std::to_string(adj_interval);
  run_loop(key, [&] {
    for (int it = 0; it < d_.nt; ++it) {
      enqueue_step(it, it & 1, inj, pl, true);
      if ((it + 1) % adj_interval == 0) {  // solver.rs:1411-1414
        const int isa = nsa - (it + 1) / adj_interval;
        const float* src = st_[(it + 1) & 1].vy - size_t(kHaloRows) * ld_ - kHaloCols;
        SW_CUDA(cudaMemcpyAsync(fwd_store_ + size_t(isa) * field_elems_, src, fb, cudaMemcpyDeviceToDevice,
                                stream_));
      }
    }
    enqueue_traces();
  });
  cur_buf_ = d_.nt & 1;
}

void Sim::adjoint_backward(const float* adstf_host, int adj_interval) {
  const int nsa = d_.nt / adj_interval;
  if (!d_.sh) return;
  if (nsa != fwd_nsa_) throw std::logic_error("adjoint_backward without a matching adjoint_forward");
  if (!adstf_ && nrec_) SW_CUDA(cudaMalloc(&adstf_, size_t(nrec_) * d_.nt * sizeof(float)));
  if (nrec_)
    SW_CUDA(cudaMemcpyAsync(adstf_, adstf_host, size_t(nrec_) * d_.nt * sizeof(float), cudaMemcpyHostToDevice,
                            stream_));
  std::vector<Inject> list;
  for (int r = 0; r < nrec_; ++r) list.push_back(Inject{rec_i_[r], rec_j_[r], r, 0});
  std::stable_sort(list.begin(), list.end(),
                   [](const Inject& a, const Inject& b) { return a.i != b.i ? a.i < b.i : a.j < b.j; });
  upload_inject(list, 1);
  InjectList inj{};
  inj.list = inj_dev_[1];
  inj.n = inj_n_[1];
  inj.nt = d_.nt;
  inj.val_y = adstf_;
  ProbeList none{};
  zero_state();
  const float ndt = float(adj_interval) * d_.dt;  // solver.rs:1368
  std::string key = "adjb/" + std::to_string(inj.n) + "/" + std::to_string(adj_interval);
  run_loop(key, [&] {
    for (int it = 0; it < d_.nt; ++it) {
      enqueue_step(it, it & 1, inj, none, true);
      if (it % adj_interval == 0 && it / adj_interval < nsa) {  // solver.rs:1468-1491
        const float* fw = fwd_store_ + size_t(it / adj_interval) * field_elems_ + size_t(kHaloRows) * ld_ + kHaloCols;
        SW_CUDA(launch_imaging_muy(kmu_, st_[(it + 1) & 1].vy, fw, d_.nx, d_.nz, ld_, den_x_, den_z_,
                                   ndt, stream_));
        ++launches_;
      }
    }
  });
  cur_buf_ = d_.nt & 1;
}

// Gaussian smoothing of kmu (solver.rs:1249-1274; fd2d.wgsl:515-554, 590-609).
// The reference sums exp(-d^2 / (2 sigma^2)) over the full grid; terms beyond
// 8 sigma are below 1.3e-14 of the peak and are dropped.  The normaliser
// gsum(i, j) = sx(i) * sz(j) keeps the reference's full-range sums.
void Sim::smooth_kmu(float sigma) {
  if (!kmu_) clear_kmu();
  if (!(sigma > 0.0f)) return;
  const int radius = std::min(std::max(d_.nx, d_.nz) - 1, int(std::ceil(8.0 * double(sigma))));
  std::vector<float> w(size_t(radius) + 1);
  const double s2 = 2.0 * double(sigma) * double(sigma);
  for (int q = 0; q <= radius; ++q) w[q] = float(std::exp(-double(q) * double(q) / s2));
  auto sums = [&](int n) {
    std::vector<float> out(static_cast<size_t>(n));
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int q = 0; q < n; ++q) s += std::exp(-double(i - q) * double(i - q) / s2);
      out[i] = float(s);
    }
    return out;
  };
  std::vector<float> gx = sums(d_.nx), gz = sums(d_.nz);
  float *dw = nullptr, *dgx = nullptr, *dgz = nullptr;
  SW_CUDA(cudaMalloc(&dw, (w.size() + gx.size() + gz.size()) * sizeof(float)));
  dgx = dw + w.size();
  dgz = dgx + gx.size();
  SW_CUDA(cudaMemcpyAsync(dw, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice, stream_));
  SW_CUDA(cudaMemcpyAsync(dgx, gx.data(), gx.size() * sizeof(float), cudaMemcpyHostToDevice, stream_));
  SW_CUDA(cudaMemcpyAsync(dgz, gz.data(), gz.size() * sizeof(float), cudaMemcpyHostToDevice, stream_));
  SW_CUDA(launch_smooth_x(tmp_, kmu_, dw, radius, d_.nx, d_.nz, ld_, stream_));
  SW_CUDA(launch_smooth_z(kmu_, tmp_, dw, radius, dgx, dgz, d_.nx, d_.nz, ld_, stream_));
  launches_ += 2;
  SW_CUDA(cudaStreamSynchronize(stream_));
  cudaFree(dw);
}

void Sim::smooth_field(float* host, float sigma) {
  clear_kmu();
  SW_CUDA(cudaMemcpy2DAsync(kmu_, size_t(ld_) * sizeof(float), host, size_t(d_.nz) * sizeof(float),
                            size_t(d_.nz) * sizeof(float), size_t(d_.nx), cudaMemcpyHostToDevice, stream_));
  smooth_kmu(sigma);
  download_kmu(host);
}

void Sim::download_kmu(float* host) const {
  if (!kmu_) {
    std::fill(host, host + size_t(d_.nx) * d_.nz, 0.0f);
    return;
  }
  copy_field_to_host(kmu_, host);
  SW_CUDA(cudaStreamSynchronize(stream_));
}

}  // namespace seiswg

namespace seiswg {

// ---------------------------------------------------------------------------
// Exact discrete adjoint
// ---------------------------------------------------------------------------
Sim::State Sim::slot_state(float* slot) const {
  State s;
  float* p = slot;
  auto next = [&]() {
    float* f = field_ptr(p);
    p += field_elems_;
    return f;
  };
  if (d_.sh) { s.vy = next(); s.sxy = next(); s.szy = next(); }
  if (d_.psv) { s.vx = next(); s.vz = next(); s.sxx = next(); s.szz = next(); s.sxz = next(); }
  return s;
}

void Sim::copy_state(const State& dst, const State& src) {
  const size_t fb = field_elems_ * sizeof(float);
  const size_t off = size_t(kHaloRows) * ld_ + kHaloCols;
  auto cp = [&](float* d, const float* s) {
    if (d && s) SW_CUDA(cudaMemcpyAsync(d - off, s - off, fb, cudaMemcpyDeviceToDevice, stream_));
  };
  cp(dst.vy, src.vy); cp(dst.sxy, src.sxy); cp(dst.szy, src.szy);
  cp(dst.vx, src.vx); cp(dst.vz, src.vz); cp(dst.sxx, src.sxx); cp(dst.szz, src.szz); cp(dst.sxz, src.sxz);
}

void Sim::gradient_clear() {
  const size_t fb = field_elems_ * sizeof(float);
  if (!g_mu_) {
    // One block, fields lambda, mu, buoyancy at a uniform stride (the
    // reverse step fetches rows of two of them with one tensor copy).
    float* a = nullptr;
    SW_CUDA(cudaMalloc(&a, 3 * fb));
    g_lam_ = field_ptr(a);
    g_mu_ = field_ptr(a + field_elems_);
    g_b_ = field_ptr(a + 2 * field_elems_);
  }
  SW_CUDA(cudaMemsetAsync(g_lam_ - size_t(kHaloRows) * ld_ - kHaloCols, 0, 3 * fb, stream_));
}

// The checkpoint scheme of a forward_op with ckpt_every = 0: every state
// kept where the budget holds them (no recomputation: the reverse sweep only
// runs reverse steps; with two steps per launch the forward launches store
// the state between their two steps as well), else uniform checkpoints every
// second step (half a forward pass recomputed per gradient), else every
// ceil(sqrt(nt)) steps (one forward pass), else binomial checkpointing with
// as many slots as the budget holds.  Budget: the "checkpoint_budget_mb"
// option, or the free device memory less a reserve of a tenth of the
// device's memory (at least 2 GiB), plus what the current checkpoints hold.
// Returns k > 0 (uniform interval) or -S (binomial, S slots).
int Sim::default_checkpoint_interval(double cap) const {
  const int nt = std::max(d_.nt, 1);
  const int k_sqrt = std::max(1, int(std::ceil(std::sqrt(double(nt)))));
  const double state_b = double(nstate()) * double(field_elems_) * sizeof(float);
  double budget = double(ck_budget_);
  if (ck_budget_ == 0) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return k_sqrt;
    const double reserve = std::max(0.1 * double(total_b), double(size_t(2) << 30));
    budget = std::max(0.0, double(free_b) - reserve) + double(ck_bytes_);
  }
  if (cap >= 0.0) budget = std::min(budget, cap);
  if ((double(nt) + 1.0) * state_b <= budget) return 1;
  const int k2 = std::min(2, nt);
  if ((double((nt + k2 - 1) / k2) + k2) * state_b <= budget) return k2;
  if ((double((nt + k_sqrt - 1) / k_sqrt) + k_sqrt) * state_b <= budget) return k_sqrt;
  return -std::max(1, std::min(nt, int(budget / state_b)));
}

void Sim::free_checkpoints() {
  for (float** p : {&ck_store_, &seg_store_, &rv_store_}) {
    cudaFree(*p);
    *p = nullptr;
  }
  ck_k_ = ck_n_ = rv_slots_ = 0;
  ck_bytes_ = 0;
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
}

// Binomial checkpointing (job_ops_revolve, batch_plan.h): slots 0..S-1 of
// rv_store_ (slot 0 the zero state), slots S and S+1 the two state buffers.
Sim::State Sim::rv_slot(int q) const {
  const size_t state_elems = size_t(nstate()) * field_elems_;
  return q < rv_slots_ ? slot_state(rv_store_ + size_t(q) * state_elems) : st_[q - rv_slots_];
}

void Sim::forward_op_binomial(int isrc, int S) {
  const int nt = d_.nt;
  S = std::max(1, std::min(S, std::max(nt, 1)));
  const size_t state_elems = size_t(nstate()) * field_elems_;
  if (S != rv_slots_ || !rv_store_) {
    free_checkpoints();
    SW_CUDA(cudaMalloc(&rv_store_, size_t(S) * state_elems * sizeof(float)));
    // Halos stay zero; so does slot 0 (the zero initial state), which no
    // operation writes.
    SW_CUDA(cudaMemsetAsync(rv_store_, 0, size_t(S) * state_elems * sizeof(float), stream_));
    rv_slots_ = S;
    ck_bytes_ = size_t(S) * state_elems * sizeof(float);
  }
  rv_ops_ = job_ops_revolve(nt, S, d_.psv, two_step_);
  recompute_steps_ = 0;
  for (const HostOp& o : rv_ops_)
    if (!(o.flags & 1) && o.kind != kMisfit && o.kind != kAdjPsv && o.kind != kAdjSh)
      recompute_steps_ += (o.kind == kFwd2Psv || o.kind == kFwd2Sh) ? 2 : 1;
  if (!g_mu_) gradient_clear();
  InjectList inj = source_injections(isrc);
  ProbeList pl = probe_list();
  zero_state();
  if (nprobe_) SW_CUDA(cudaMemsetAsync(probe_acc_, 0, size_t(nprobe_) * sizeof(float), stream_));
  int last = -1;
  const std::string key = "fop/rv/" + std::to_string(inj.n) + "/" + std::to_string(S) + (two_step_ ? "/2" : "");
  run_loop(key, [&] {
    for (const HostOp& o : rv_ops_) {
      if (o.kind == kMisfit) break;
      if (o.kind == kFwd2Psv || o.kind == kFwd2Sh) enqueue_step2(o.it, rv_slot(o.a), rv_slot(o.b), inj, pl);
      else enqueue_step_states(o.it, rv_slot(o.a), rv_slot(o.b), inj, pl, false);
    }
    enqueue_traces();
  });
  for (const HostOp& o : rv_ops_) {
    if (o.kind == kMisfit) break;
    last = o.b;
  }
  cur_buf_ = last >= S ? last - S : 0;  // the step that ends at nt writes a state buffer
  ck_isrc_ = isrc;
}

void Sim::forward_op(int isrc, int ckpt_every) {
  u_ready_ = false;
  if (d_.spin) throw std::invalid_argument("the exact adjoint is defined for SH or PSV without spin");
  if (d_.sh && d_.psv) throw std::invalid_argument("the exact adjoint runs one of SH or PSV at a time");
  const int nt = d_.nt;
  const size_t state_elems = size_t(nstate()) * field_elems_;
  // The scheme the budget allows; should its allocation fail (memory taken
  // meanwhile, or too fragmented for one block), the next scheme that needs
  // less.  An explicit interval or slot count fails instead.
  const bool chosen = ckpt_every <= 0 && rv_force_ <= 0;
  double cap = -1.0;
  int k = 0, ncp = 0;
  for (;;) {
    k = ckpt_every > 0 ? ckpt_every : rv_force_ > 0 ? -rv_force_ : default_checkpoint_interval(cap);
    if (k < 0) break;
    k = std::max(1, std::min(k, std::max(nt, 1)));
    ncp = (nt + k - 1) / k;
    if (k == ck_k_ && ncp == ck_n_ && !rv_slots_) break;
    free_checkpoints();
    const size_t a = size_t(std::max(1, ncp)) * state_elems * sizeof(float);
    const size_t b = size_t(k) * state_elems * sizeof(float);
    const cudaError_t ea = cudaMalloc(&ck_store_, a);
    const cudaError_t eb = ea == cudaSuccess ? cudaMalloc(&seg_store_, b) : ea;
    if (eb == cudaSuccess) {
      // Halos of every stored state stay zero; so does checkpoint 0 (the
      // zero initial state), which no step writes.
      SW_CUDA(cudaMemsetAsync(ck_store_, 0, a, stream_));
      SW_CUDA(cudaMemsetAsync(seg_store_, 0, b, stream_));
      ck_k_ = k;
      ck_n_ = ncp;
      ck_bytes_ = a + b;
      break;
    }
    (void)cudaGetLastError();  // the failed allocation's error, not sticky
    free_checkpoints();
    if (!chosen || eb != cudaErrorMemoryAllocation || k >= nt) SW_CUDA(eb);
    cap = double(a + b) - 1.0;
  }
  if (k < 0) {
    forward_op_binomial(isrc, -k);
    return;
  }
  recompute_steps_ = nt - ncp;  // every interval but its checkpoint, once
  if (!g_mu_) gradient_clear();
  InjectList inj = source_injections(isrc);
  ProbeList pl = probe_list();
  zero_state();
  if (nprobe_) SW_CUDA(cudaMemsetAsync(probe_acc_, 0, size_t(nprobe_) * sizeof(float), stream_));
  // The launches of record_plan (batch_plan.h): steps write straight into
  // the checkpoint they end on, the others alternate between the two state
  // buffers; with every state kept, two-step launches store the state
  // between their steps as well.
  const std::vector<RecordLaunch> plan = record_plan(nt, k, two_step_);
  auto slot = [&](int q) { return q >= 0 ? slot_state(ck_store_ + size_t(q) * state_elems) : st_[-1 - q]; };
  const std::string key = "fop/" + std::to_string(inj.n) + "/" + std::to_string(k) + (two_step_ ? "/2" : "");
  run_loop(key, [&] {
    for (const RecordLaunch& o : plan) {
      if (o.n == 2) {
        const State mid = o.mid >= 0 ? slot(o.mid) : State{};
        enqueue_step2(o.it, slot(o.a), slot(o.b), inj, pl, o.mid >= 0 ? &mid : nullptr);
      } else {
        enqueue_step_states(o.it, slot(o.a), slot(o.b), inj, pl, false);
      }
    }
    enqueue_traces();
  });
  // the buffer of the final state (graph replays skip the body)
  int last = -1;
  for (const RecordLaunch& o : plan)
    if (o.b < 0) last = -1 - o.b;
  cur_buf_ = last < 0 ? 0 : last;
  ck_isrc_ = isrc;
}

void Sim::backward_op(const float* adj_host) {
  if (ck_isrc_ == -2) throw std::logic_error("backward_op without a preceding forward_op");
  const int nt = d_.nt;
  const int ncomp = d_.psv ? 2 : 1;
  const size_t nrt = size_t(nrec_) * nt;
  // dt * U, U^n = sum_{m >= n} dJ/dd^m, summed in double.
  std::vector<float> u(size_t(ncomp) * nrt);
  for (int c = 0; c < ncomp; ++c)
    for (int r = 0; r < nrec_; ++r) {
      double acc = 0.0;
      for (int n = nt - 1; n >= 0; --n) {
        acc += double(adj_host[size_t(c) * nrt + size_t(r) * nt + n]);
        u[size_t(c) * nrt + size_t(r) * nt + n] = float(double(d_.dt) * acc);
      }
    }
  ensure_u_tab();
  if (!u.empty())
    SW_CUDA(cudaMemcpyAsync(u_tab_, u.data(), u.size() * sizeof(float), cudaMemcpyHostToDevice, stream_));
  run_backward();
}

void Sim::ensure_u_tab() {
  const size_t n = size_t(d_.psv ? 2 : 1) * nrec_ * d_.nt;
  if (!u_tab_ && n) SW_CUDA(cudaMalloc(&u_tab_, n * sizeof(float)));
}

void Sim::set_observed(const float* obs_host) {
  const size_t n = size_t(d_.psv ? 2 : 1) * nrec_ * d_.nt;
  if (!n) throw std::invalid_argument("set_observed needs receivers");
  SW_CUDA(cudaStreamSynchronize(stream_));
  cudaFree(obs_in_);
  obs_in_ = nullptr;
  SW_CUDA(cudaMalloc(&obs_in_, n * sizeof(float)));
  SW_CUDA(cudaMemcpyAsync(obs_in_, obs_host, n * sizeof(float), cudaMemcpyHostToDevice, stream_));
  SW_CUDA(cudaStreamSynchronize(stream_));
}

double Sim::misfit_op() {
  if (ck_isrc_ == -2) throw std::logic_error("misfit_op without a preceding forward_op");
  if (!obs_in_) throw std::logic_error("misfit_op without observed traces (set_observed)");
  const int ntr = (d_.psv ? 2 : 1) * nrec_;
  ensure_u_tab();
  if (!j_tr_) SW_CUDA(cudaMalloc(&j_tr_, size_t(ntr) * sizeof(double)));
  SW_CUDA(launch_sim_misfit(obs_, obs_in_, u_tab_, j_tr_, nrec_, d_.nt, d_.psv, d_.dt, stream_));
  ++launches_;
  std::vector<double> jt(ntr);
  SW_CUDA(cudaMemcpyAsync(jt.data(), j_tr_, size_t(ntr) * sizeof(double), cudaMemcpyDeviceToHost, stream_));
  SW_CUDA(cudaStreamSynchronize(stream_));
  double J = 0.0;
  for (double v : jt) J += v;
  u_ready_ = true;
  return J;
}

void Sim::backward_op_device() {
  if (ck_isrc_ == -2) throw std::logic_error("backward_op without a preceding forward_op");
  if (!u_ready_) throw std::logic_error("backward_op_device without a misfit_op after the forward_op");
  run_backward();
}

// One reverse step n: forward state f = S^n, incoming adjoint state a,
// outgoing o.
void Sim::enqueue_reverse(int n, const State& f, const State& a, const State& o, const InjectList& src,
                          const InjectList& rec, const Geom& ga) {
  InjectList s2 = src, r2 = rec;
  s2.it = n;
  r2.it = n;
  if (d_.psv) {
    PsvAdjoint p{};
    p.g = ga;
    p.vx = f.vx; p.vz = f.vz; p.sxx = f.sxx; p.szz = f.szz; p.sxz = f.sxz;
    p.wx0 = a.vx; p.wz0 = a.vz; p.bxx0 = a.sxx; p.bzz0 = a.szz; p.bxz0 = a.sxz;
    p.wx1 = o.vx; p.wz1 = o.vz; p.bxx1 = o.sxx; p.bzz1 = o.szz; p.bxz1 = o.sxz;
    p.rho = rho_; p.lam = lam_; p.mu = mu_;
    p.taper_x = taper_x_; p.taper_zb = taper_zb_; p.taper_zt = taper_zt_;
    p.g_b = g_b_; p.g_lam = g_lam_; p.g_mu = g_mu_;
    p.src = s2;
    p.rec = r2;
    p.err = err_;
    if (!launch_adjoint_tma(p, f, a)) SW_CUDA(launch_psv_adjoint(p, stream_));
  } else {
    ShAdjoint p{};
    p.g = ga;
    p.vy = f.vy; p.sxy = f.sxy; p.szy = f.szy;
    p.w0 = a.vy; p.bxy0 = a.sxy; p.bzy0 = a.szy;
    p.w1 = o.vy; p.bxy1 = o.sxy; p.bzy1 = o.szy;
    p.rho = rho_; p.mu = mu_;
    p.taper_x = taper_x_; p.taper_zb = taper_zb_; p.taper_zt = taper_zt_;
    p.g_b = g_b_; p.g_mu = g_mu_;
    p.src = s2;
    p.rec = r2;
    p.err = err_;
    SW_CUDA(launch_sh_adjoint(p, stream_));
  }
  ++launches_;
}

void Sim::run_backward() {
  const int nt = d_.nt;
  const size_t nrt = size_t(nrec_) * nt;
  std::vector<Inject> list;
  for (int r = 0; r < nrec_; ++r) list.push_back(Inject{rec_i_[r], rec_j_[r], r, 0});
  std::stable_sort(list.begin(), list.end(),
                   [](const Inject& a, const Inject& b) { return a.i != b.i ? a.i < b.i : a.j < b.j; });
  upload_inject(list, 1);
  InjectList rec{};
  rec.list = inj_dev_[1];
  rec.n = inj_n_[1];
  rec.nt = nt;
  if (d_.psv) { rec.val_x = u_tab_; rec.val_z = u_tab_ + nrt; }
  else rec.val_y = u_tab_;
  InjectList src = source_injections(ck_isrc_);
  ProbeList none{};

  const size_t state_elems = size_t(nstate()) * field_elems_;
  if (!adj_store_) SW_CUDA(cudaMalloc(&adj_store_, 2 * state_elems * sizeof(float)));
  SW_CUDA(cudaMemsetAsync(adj_store_, 0, 2 * state_elems * sizeof(float), stream_));
  const State adj[2] = {slot_state(adj_store_), slot_state(adj_store_ + state_elems)};
  const int k = ck_k_;
  const Geom ga = adjoint_geom();
  SW_CUDA(cudaStreamSynchronize(stream_));  // host tables above are released after this call

  if (rv_slots_ > 0) {  // binomial checkpointing: the operation list after the misfit
    const std::string key = "bop/rv/" + std::to_string(src.n) + "/" + std::to_string(rec.n) + "/" +
                            std::to_string(rv_slots_) + (two_step_ ? "/2" : "");
    run_loop(key, [&] {
      bool after = false;
      for (const HostOp& o : rv_ops_) {
        if (o.kind == kMisfit) { after = true; continue; }
        if (!after) continue;
        if (o.kind == kFwdPsv || o.kind == kFwdSh) enqueue_step_states(o.it, rv_slot(o.a), rv_slot(o.b), src, none, false);
        else if (o.kind == kFwd2Psv || o.kind == kFwd2Sh) enqueue_step2(o.it, rv_slot(o.a), rv_slot(o.b), src, none);
        else enqueue_reverse(o.it, rv_slot(o.a), adj[o.b], adj[1 - o.b], src, rec, ga);
      }
      SW_CUDA(launch_check_finite(g_lam_ - size_t(kHaloRows) * ld_ - kHaloCols, 3 * (d_.nx + 2 * kHaloRows), ld_,
                                  ld_, err_, kErrNonFiniteGradient, stream_));
      ++launches_;
    });
    return;
  }

  const std::string key = "bop/" + std::to_string(src.n) + "/" + std::to_string(rec.n) + "/" + std::to_string(k) +
                          (two_step_ ? "/2" : "");
  run_loop(key, [&] {
    int cur = 0;
    for (int seg = ck_n_ - 1; seg >= 0; --seg) {
      const int n0 = seg * k, n1 = std::min(nt, n0 + k);
      // S^n0 is the checkpoint itself; S^(n0+1..n1-1) are recomputed into
      // the interval buffer.
      auto fstate = [&](int n) {
        return n == n0 ? slot_state(ck_store_ + size_t(seg) * state_elems)
                       : slot_state(seg_store_ + size_t(n - n0) * state_elems);
      };
      // Two steps per launch where the forward pass runs them, each launch
      // storing both states.
      for (int n = n0; n < n1 - 1;) {
        if (two_step_ && n + 2 <= n1 - 1) {
          const State mid = fstate(n + 1);
          enqueue_step2(n, fstate(n), fstate(n + 2), src, none, &mid);
          n += 2;
        } else {
          enqueue_step_states(n, fstate(n), fstate(n + 1), src, none, false);
          ++n;
        }
      }
      for (int n = n1 - 1; n >= n0; --n) {
        enqueue_reverse(n, fstate(n), adj[cur], adj[1 - cur], src, rec, ga);
        cur ^= 1;
      }
    }
    // NaN / infinity watchdog over the gradient block (lambda, mu, buoyancy).
    SW_CUDA(launch_check_finite(g_lam_ - size_t(kHaloRows) * ld_ - kHaloCols, 3 * (d_.nx + 2 * kHaloRows), ld_, ld_,
                                err_, kErrNonFiniteGradient, stream_));
    ++launches_;
  });
}

void Sim::release_workspace() {
  SW_CUDA(cudaStreamSynchronize(stream_));
  for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
  graphs_.clear();
  for (float** p : {&ck_store_, &seg_store_, &rv_store_, &adj_store_, &fwd_store_, &snap_store_}) {
    cudaFree(*p);
    *p = nullptr;
  }
  ck_k_ = ck_n_ = rv_slots_ = 0;
  ck_isrc_ = -2;
  ck_bytes_ = 0;
  fwd_nsa_ = 0;
  fwd_bytes_ = 0;
  snap_cap_ = 0;
}

void Sim::download_gradient(int which, float* host) const {
  const float* g = which == 0 ? g_lam_ : which == 1 ? g_mu_ : g_b_;
  if (!g) {
    std::fill(host, host + size_t(d_.nx) * d_.nz, 0.0f);
    return;
  }
  copy_field_to_host(g, host);
  SW_CUDA(cudaStreamSynchronize(stream_));
  check_device_error();
}

}  // namespace seiswg

namespace seiswg {

Sim::View Sim::view() const {
  View v;
  v.geom = geom_;
  v.geom2 = geom2_;
  if (!two_step_) v.geom2.lx = 0;
  v.ld = ld_;
  v.field_elems = field_elems_;
  v.rho = rho_; v.lam = lam_; v.mu = mu_;
  v.rho_dt = rdt_;
  v.taper_x = taper_x_; v.taper_zb = taper_zb_; v.taper_zt = taper_zt_;
  v.stf = stf_;
  v.probes = probes_;
  v.nprobe = nprobe_;
  v.probe_split = probe_split_;
  v.tr_idx = tr_idx_;
  v.src_i = src_i_.data(); v.src_j = src_j_.data();
  v.rec_i = rec_i_.data(); v.rec_j = rec_j_.data();
  return v;
}

}  // namespace seiswg
