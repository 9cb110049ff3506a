// batch.cpp -- see batch.h.
#include "batch.h"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "batch_plan.h"

namespace seiswg {

Batch::Batch(const std::vector<BatchProblem>& problems, int ckpt_every, cudaStream_t stream)
    : problems_(problems), stream_(stream), ckpt_every_(ckpt_every) {
  if (!stream_) {
    SW_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
    own_stream_ = true;
  }
  const int nstreams = kKinds * kMaxStreamGroups;
  aux_.assign(nstreams - 1, nullptr);
  join_.assign(nstreams - 1, nullptr);
  for (int k = 0; k < nstreams - 1; ++k) {
    SW_CUDA(cudaStreamCreateWithFlags(&aux_[k], cudaStreamNonBlocking));
    SW_CUDA(cudaEventCreateWithFlags(&join_[k], cudaEventDisableTiming));
  }
  SW_CUDA(cudaEventCreateWithFlags(&fork_, cudaEventDisableTiming));
  static_assert(kMaxStreamGroups == kPlanGroupsMax, "stream groups of the batch and of its launch plan");
  kst_.assign(kPlanStreams, nullptr);
  kev_.assign(kPlanEvents, nullptr);
  for (int k = 0; k < kPlanStreams; ++k) SW_CUDA(cudaStreamCreateWithFlags(&kst_[k], cudaStreamNonBlocking));
  for (int k = 0; k < kPlanEvents; ++k) SW_CUDA(cudaEventCreateWithFlags(&kev_[k], cudaEventDisableTiming));
  SW_CUDA(cudaMalloc(&err_, sizeof(int)));
  SW_CUDA(cudaMemsetAsync(err_, 0, sizeof(int), stream_));
  for (size_t p = 0; p < problems_.size(); ++p) {
    Sim* sim = problems_[p].sim;
    const SimDesc& d = sim->desc();
    if (d.spin || d.sh == d.psv) throw std::invalid_argument("batched gradients need SH or PSV (no spin)");
    const Sim::View v = sim->view();
    const int nt = d.nt, nrec = sim->nrec(), ncomp = d.psv ? 2 : 1;
    const size_t fe = v.field_elems;
    const size_t halo = size_t(kHaloRows) * v.ld + kHaloCols;
    if (problems_[p].obs.size() != size_t(sim->nsrc()) * ncomp * nrec * nt)
      throw std::invalid_argument("observed traces of problem " + std::to_string(p) + " have the wrong size");
    float* sum = nullptr;
    SW_CUDA(cudaMalloc(&sum, 3 * fe * sizeof(float)));
    SW_CUDA(cudaMemsetAsync(sum, 0, 3 * fe * sizeof(float), stream_));
    sums_.push_back(sum);
    bytes_ += 3 * fe * sizeof(float);
    std::vector<Inject> rec;
    for (int r = 0; r < nrec; ++r) rec.push_back(Inject{v.rec_i[r], v.rec_j[r], r, 0});
    std::stable_sort(rec.begin(), rec.end(),
                     [](const Inject& a, const Inject& b) { return a.i != b.i ? a.i < b.i : a.j < b.j; });
    for (int s = 0; s < sim->nsrc(); ++s) {
      Job j;
      j.problem = int(p);
      j.shot = s;
      j.nt = nt;
      j.psv = d.psv;
      j.nstate = d.psv ? 5 : 3;
      j.ncomp = ncomp;
      j.nrec = nrec;
      j.k = ckpt_every > 0 ? std::min(ckpt_every, std::max(nt, 1))
                           : int(std::ceil(std::sqrt(double(std::max(nt, 1)))));
      j.ncp = (nt + j.k - 1) / j.k;
      j.nslot = j.ncp + j.k + 1;
      const size_t slot = size_t(j.nstate) * fe;
      const size_t ntr = size_t(ncomp) * nrec;
      SW_CUDA(cudaMalloc(&j.adj, 2 * slot * sizeof(float)));
      SW_CUDA(cudaMemsetAsync(j.adj, 0, 2 * slot * sizeof(float), stream_));
      SW_CUDA(cudaMalloc(&j.grads, 3 * fe * sizeof(float)));
      SW_CUDA(cudaMemsetAsync(j.grads, 0, 3 * fe * sizeof(float), stream_));
      SW_CUDA(cudaMalloc(&j.acc, std::max(1, v.nprobe) * sizeof(float)));
      SW_CUDA(cudaMalloc(&j.hist, std::max<size_t>(1, size_t(v.nprobe) * nt) * sizeof(float)));
      SW_CUDA(cudaMalloc(&j.obs, std::max<size_t>(1, ntr * nt) * sizeof(float)));
      SW_CUDA(cudaMalloc(&j.u_tab, std::max<size_t>(1, ntr * nt) * sizeof(float)));
      SW_CUDA(cudaMalloc(&j.J, std::max<size_t>(1, ntr) * sizeof(double)));
      SW_CUDA(cudaMalloc(&j.src, sizeof(Inject)));
      SW_CUDA(cudaMalloc(&j.rec, std::max(1, nrec) * sizeof(Inject)));
      bytes_ += 2 * slot * sizeof(float) + 3 * fe * sizeof(float) +
                (size_t(v.nprobe) * (nt + 1) + 2 * ntr * nt) * sizeof(float);
      const Inject src{v.src_i[s], v.src_j[s], s, 0};
      SW_CUDA(cudaMemcpyAsync(j.src, &src, sizeof(Inject), cudaMemcpyHostToDevice, stream_));
      if (nrec) SW_CUDA(cudaMemcpyAsync(j.rec, rec.data(), nrec * sizeof(Inject), cudaMemcpyHostToDevice, stream_));
      if (ntr)
        SW_CUDA(cudaMemcpyAsync(j.obs, problems_[p].obs.data() + size_t(s) * ntr * nt, ntr * nt * sizeof(float),
                                cudaMemcpyHostToDevice, stream_));
      SW_CUDA(cudaStreamSynchronize(stream_));  // `src` and `rec` are host temporaries

      JobDesc jd{};
      jd.g = v.geom;
      jd.g2 = v.geom2;  // lx 0 unless the problem runs two steps per launch
      jd.psv = d.psv;
      jd.nstate = j.nstate;
      jd.field_elems = (long long)fe;
      jd.slot_elems = (long long)slot;
      jd.halo = (long long)halo;
      jd.pool = j.pool;
      jd.adj = j.adj;
      jd.rho = v.rho; jd.lam = v.lam; jd.mu = v.mu;
      jd.rho_dt = v.rho_dt;
      jd.taper_x = v.taper_x; jd.taper_zb = v.taper_zb; jd.taper_zt = v.taper_zt;
      jd.g_lam = j.grads + halo;
      jd.g_mu = j.grads + fe + halo;
      jd.g_b = j.grads + 2 * fe + halo;
      const size_t nst = size_t(sim->nsrc()) * nt;
      jd.src = InjectList{j.src, 1, nt, 0, v.stf, v.stf + nst, v.stf + 2 * nst};
      jd.probes.list = v.probes + (d.psv ? v.probe_split : 0);
      jd.probes.n = d.psv ? v.nprobe - v.probe_split : v.probe_split;
      jd.probes.nt = nt;
      jd.probes.acc = j.acc;
      jd.probes.hist = j.hist;
      jd.rec = InjectList{j.rec, nrec, nt, 0, nullptr, nullptr, nullptr};
      if (d.psv) { jd.rec.val_x = j.u_tab; jd.rec.val_z = j.u_tab + size_t(nrec) * nt; }
      else jd.rec.val_y = j.u_tab;
      jd.tr_idx = v.tr_idx;
      jd.obs = j.obs;
      jd.u_tab = j.u_tab;
      jd.J = j.J;
      jd.nrec = nrec;
      jd.nt = nt;
      jd.dt = d.dt;
      jd.err = err_;
      descs_.push_back(jd);
      model_geom_.push_back(jd.g);
      model_geom2_.push_back(jd.g2);
      jobs_.push_back(j);
      alloc_pool(jobs_.size() - 1);
    }
  }
  SW_CUDA(cudaMalloc(&d_jobs_, std::max<size_t>(1, descs_.size()) * sizeof(JobDesc)));
  SW_CUDA(cudaMemcpyAsync(d_jobs_, descs_.data(), descs_.size() * sizeof(JobDesc), cudaMemcpyHostToDevice, stream_));
  SW_CUDA(cudaStreamSynchronize(stream_));
  set_chunk_rows(0);  // each problem's own chunk model; builds the schedule
}

// The job's pool of state slots (uniform checkpoints: ncp + k + 1; binomial
// checkpointing: S + 2) and its table of tensor maps (JobDesc): state slots
// with boxes of 1, 2 and 3 fields, the adjoint slots (3, 2), the material
// (1, 2), the gradients (1, 2), the dt-scaled material (1, 2).
void Batch::alloc_pool(size_t q) {
  Job& j = jobs_[q];
  JobDesc& jd = descs_[q];
  const Sim::View v = problems_[j.problem].sim->view();
  const SimDesc& d = problems_[j.problem].sim->desc();
  const size_t fe = v.field_elems;
  const size_t halo = size_t(kHaloRows) * v.ld + kHaloCols;
  const size_t slot = size_t(j.nstate) * fe;
  if (j.pool) {
    bytes_ -= size_t(j.pool_slots) * slot * sizeof(float);
    cudaFree(j.pool);
    j.pool = nullptr;
  }
  if (j.tm) {
    bytes_ -= (size_t(3) * j.pool_slots + kJobTmaTail) * sizeof(CUtensorMap);
    cudaFree(j.tm);
    j.tm = nullptr;
  }
  SW_CUDA(cudaMalloc(&j.pool, size_t(j.nslot) * slot * sizeof(float)));
  SW_CUDA(cudaMemsetAsync(j.pool, 0, size_t(j.nslot) * slot * sizeof(float), stream_));
  j.pool_slots = j.nslot;
  bytes_ += size_t(j.nslot) * slot * sizeof(float);
  jd.pool = j.pool;
  {
    const int rows_alloc = d.nx + 2 * kHaloRows;
    const int nf = j.nstate;
    std::vector<CUtensorMap> maps(size_t(3) * j.nslot + kJobTmaTail);
    bool ok = v.lam - v.rho == v.mu - v.lam && v.lam > v.rho;
    for (int sl = 0; ok && sl < j.nslot; ++sl)
      for (int b = 0; ok && b < 3; ++b)
        ok = encode_fields(&maps[3 * sl + b], j.pool + sl * slot + halo, ptrdiff_t(fe), nf, v.ld, rows_alloc,
                           std::min(b + 1, nf));
    CUtensorMap* t = maps.data() + 3 * j.nslot;
    for (int a = 0; ok && a < 2; ++a)
      ok = encode_fields(&t[2 * a], j.adj + a * slot + halo, ptrdiff_t(fe), nf, v.ld, rows_alloc, std::min(3, nf)) &&
           encode_fields(&t[2 * a + 1], j.adj + a * slot + halo, ptrdiff_t(fe), nf, v.ld, rows_alloc, 2);
    ok = ok && encode_fields(&t[4], v.rho, v.lam - v.rho, 3, v.ld, rows_alloc, 1) &&
         encode_fields(&t[5], v.rho, v.lam - v.rho, 3, v.ld, rows_alloc, 2) &&
         encode_fields(&t[6], j.grads + halo, ptrdiff_t(fe), 3, v.ld, rows_alloc, 1) &&
         encode_fields(&t[7], j.grads + halo, ptrdiff_t(fe), 3, v.ld, rows_alloc, 2) && v.rho_dt &&
         encode_fields(&t[8], v.rho_dt, v.lam - v.rho, 3, v.ld, rows_alloc, 1) &&
         encode_fields(&t[9], v.rho_dt, v.lam - v.rho, 3, v.ld, rows_alloc, 2);
    if (ok) {
      SW_CUDA(cudaMalloc(&j.tm, maps.size() * sizeof(CUtensorMap)));
      SW_CUDA(cudaMemcpy(j.tm, maps.data(), maps.size() * sizeof(CUtensorMap), cudaMemcpyHostToDevice));
      bytes_ += maps.size() * sizeof(CUtensorMap);
    }
    jd.tm = tma_ ? j.tm : nullptr;
    jd.tm_nslot = j.nslot;
  }
}

void Batch::set_checkpoint_slots(int S) {
  if (S < 0) throw std::invalid_argument("checkpoint_slots must be >= 0");
  SW_CUDA(cudaStreamSynchronize(stream_));
  for (size_t q = 0; q < jobs_.size(); ++q) {
    Job& j = jobs_[q];
    j.S = S > 0 ? std::min(S, std::max(j.nt, 1)) : 0;
    j.nslot = j.S > 0 ? j.S + 2 : j.ncp + j.k + 1;
    alloc_pool(q);
  }
  SW_CUDA(cudaMemcpyAsync(d_jobs_, descs_.data(), descs_.size() * sizeof(JobDesc), cudaMemcpyHostToDevice, stream_));
  SW_CUDA(cudaStreamSynchronize(stream_));
  checkpoint_slots_ = S;
  set_chunk_rows(chunk_rows_);  // rebuilds the schedule, drops the graph
}

long long Batch::recompute_steps() const {
  long long n = 0;
  for (size_t q = 0; q < jobs_.size(); ++q) {
    const Job& j = jobs_[q];
    const std::vector<HostOp> L = j.S > 0 ? job_ops_revolve(j.nt, j.S, j.psv, false) : job_ops(j.nt, j.k, j.psv, false);
    bool after = false;
    for (const HostOp& o : L) {
      if (o.kind == kMisfit) after = true;
      else if (after && (o.kind == kFwdPsv || o.kind == kFwdSh)) ++n;
    }
  }
  return n;
}

void Batch::set_chunk_rows(int lx) {
  if (lx != 0 && lx < 4) throw std::invalid_argument("chunk_rows must be 0 or >= 4");
  SW_CUDA(cudaStreamSynchronize(stream_));
  // The same rows for the one- and the two-step marches: in a batch many
  // jobs share each launch, and its duration is the longest march.
  for (size_t q = 0; q < descs_.size(); ++q) {
    Geom g = model_geom_[q], g2 = model_geom2_[q];
    if (lx > 0) {
      g.lx = lx;
      g.nchunks = (g.nx + lx - 1) / lx;
      if (g2.lx > 0) {
        g2.lx = lx;
        g2.nchunks = (g2.nx + lx - 1) / lx;
      }
    }
    if (concurrent_ == 3 && g2.lx > 0 && g2.lx != g.lx) {  // the queue counts finished units per chunk
      const int l = std::max(g.lx, g2.lx);
      g.lx = g2.lx = l;
      g.nchunks = g2.nchunks = (g.nx + l - 1) / l;
    }
    descs_[q].g = g;
    descs_[q].g2 = g2;
  }
  SW_CUDA(cudaMemcpyAsync(d_jobs_, descs_.data(), descs_.size() * sizeof(JobDesc), cudaMemcpyHostToDevice, stream_));
  SW_CUDA(cudaStreamSynchronize(stream_));
  if (graph_) cudaGraphExecDestroy(graph_);
  graph_ = nullptr;
  cudaFree(d_ops_);
  d_ops_ = nullptr;
  chunk_rows_ = lx;
  build_schedule();
}

void Batch::set_two_step(bool on) {
  two_step_ = on;
  set_chunk_rows(chunk_rows_);  // rebuilds the schedule
}

void Batch::set_two_step_recompute(bool on) {
  pair_ = on;
  set_chunk_rows(chunk_rows_);  // rebuilds the schedule
}

double Batch::autotune(int slots) {
  if (slots < 1) slots = 1;
  // The device queue counts units per chunk: short chunks multiply its units
  // (and their claims and waits), so it starts at 32 rows.
  std::vector<int> cand = concurrent_ == 3 ? std::vector<int>{0, 32, 48, 64, 96, 128}
                                           : std::vector<int>{0, 16, 32, 48, 64, 96, 128};
  cudaEvent_t e0, e1;
  SW_CUDA(cudaEventCreate(&e0));
  SW_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int best_lx = chunk_rows_;
  bool best_two = two_step_;
  for (int c = 0; c < 2 * int(cand.size()); ++c) {
    const int lx = cand[c % cand.size()];
    two_step_ = c < int(cand.size());
    set_chunk_rows(lx);
    // A window at the start of the recording pass and one in the middle of
    // the reverse sweep, each scaled to its phase's slot count: two-step
    // recording does twice the steps per slot in half the slots.
    const int rec = std::max(1, rec_slots_), rest = std::max(1, nslots_ - rec_slots_);
    const int w = std::min(slots, rec), rw = std::min(slots, rest);
    const int mid = rec_slots_ + (rest - rw) / 2;
    enqueue_slots(0, std::min(2, nslots_));  // warm-up
    float ms_rec = 0.0f, ms_rev = 0.0f;
    SW_CUDA(cudaEventRecord(e0, stream_));
    enqueue_slots(0, w);
    SW_CUDA(cudaEventRecord(e1, stream_));
    SW_CUDA(cudaEventSynchronize(e1));
    SW_CUDA(cudaEventElapsedTime(&ms_rec, e0, e1));
    SW_CUDA(cudaEventRecord(e0, stream_));
    enqueue_slots(mid, mid + rw);
    SW_CUDA(cudaEventRecord(e1, stream_));
    SW_CUDA(cudaEventSynchronize(e1));
    SW_CUDA(cudaEventElapsedTime(&ms_rev, e0, e1));
    const float ms = ms_rec / float(w) * float(rec) + ms_rev / float(rw) * float(rest);
    if (ms < best) { best = ms; best_lx = lx; best_two = two_step_; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // The windows compute on whatever the slots before them left, so only a
  // wait that ran out is an error here.
  int e = 0;
  SW_CUDA(cudaMemcpy(&e, err_, sizeof(int), cudaMemcpyDeviceToHost));
  SW_CUDA(cudaMemset(err_, 0, sizeof(int)));
  if (e & kErrWaitTimeout) throw WaitTimeout("a batched kernel gave up waiting during the autotuner's windows");
  two_step_ = best_two;
  set_chunk_rows(best_lx);
  return double(best);
}

Batch::~Batch() {
  if (graph_) cudaGraphExecDestroy(graph_);
  free_queue();
  for (Job& j : jobs_) {
    for (void* p : {(void*)j.pool, (void*)j.adj, (void*)j.grads, (void*)j.acc, (void*)j.hist, (void*)j.obs,
                    (void*)j.u_tab, (void*)j.J, (void*)j.src, (void*)j.rec, (void*)j.tm})
      cudaFree(p);
  }
  for (float* s : sums_) cudaFree(s);
  for (cudaStream_t a : aux_) if (a) cudaStreamDestroy(a);
  for (cudaEvent_t e : join_) if (e) cudaEventDestroy(e);
  for (cudaStream_t a : kst_) if (a) cudaStreamDestroy(a);
  for (cudaEvent_t e : kev_) if (e) cudaEventDestroy(e);
  if (fork_) cudaEventDestroy(fork_);
  cudaFree(d_jobs_);
  cudaFree(d_ops_);
  cudaFree(err_);
  if (own_stream_) cudaStreamDestroy(stream_);
}

// Operation list of each job (batch.h), then one launch per (slot, kind).
void Batch::build_schedule() {
  std::vector<std::vector<HostOp>> lists(jobs_.size());
  for (size_t q = 0; q < jobs_.size(); ++q) {
    const Job& j = jobs_[q];
    const bool two = two_step_ && descs_[q].g2.lx > 0;
    // Grouped launches recompute two steps per operation as well (the queue
    // kernel's marches store no middle state).
    lists[q] = j.S > 0 ? job_ops_revolve(j.nt, j.S, j.psv, two)
                       : job_ops(j.nt, j.k, j.psv, two, /*pair=*/pair_ && concurrent_ != 3);
  }
  size_t T = 0;
  rec_slots_ = 0;
  for (auto& L : lists) {
    T = std::max(T, L.size());
    for (size_t t = 0; t < L.size(); ++t)
      if (L[t].kind == kMisfit) rec_slots_ = std::max(rec_slots_, int(t));
  }
  nslots_ = int(T);
  std::vector<GroupOp> all;
  const std::vector<std::vector<PlanLaunch>> launches = plan_launches(lists, groups_);
  plan_.assign(T, {});
  for (size_t t = 0; t < T; ++t) {
    for (const PlanLaunch& pl : launches[t]) {
      Launch l{pl.kind, int(all.size()), 0, 0, pl.deps, pl.group};
      for (int q : pl.jobs) {
        const HostOp& h = lists[q][t];
        const Geom& g = (pl.kind == kFwd2Psv || pl.kind == kFwd2Sh) ? descs_[q].g2 : descs_[q].g;
        all.push_back(GroupOp{q, h.it, h.a, h.b, h.flags, l.warps});
        l.warps += (pl.kind == kMisfit) ? 1 : g.nstrips * g.nchunks;
        ++l.count;
      }
      plan_[t].push_back(l);
    }
  }
  SW_CUDA(cudaMalloc(&d_ops_, std::max<size_t>(1, all.size()) * sizeof(GroupOp)));
  SW_CUDA(cudaMemcpyAsync(d_ops_, all.data(), all.size() * sizeof(GroupOp), cudaMemcpyHostToDevice, stream_));
  SW_CUDA(cudaStreamSynchronize(stream_));
  bytes_ += all.size() * sizeof(GroupOp) - ops_bytes_;
  ops_bytes_ = all.size() * sizeof(GroupOp);
  if (concurrent_ == 3) build_queue(lists);
  else free_queue();
}

// Launch order 3: the queue of every job's units (plan_queue), the jobs'
// operations with their dependency counts, one counter per job and chunk,
// and the claim counter; each job's descriptor points at its part.
void Batch::build_queue(const std::vector<std::vector<HostOp>>& lists) {
  free_queue();
  std::vector<QueueShape> shapes;
  for (const JobDesc& d : descs_) {
    if (d.g2.lx > 0 && (d.g2.lx != d.g.lx || d.g2.nchunks != d.g.nchunks))
      throw std::logic_error("the device queue needs the same chunks for a job's one- and two-step geometries");
    shapes.push_back(QueueShape{d.g.nchunks, d.g.lx, d.g.nstrips, d.g2.lx > 0 ? d.g2.nstrips : d.g.nstrips});
  }
  QueuePlan Q = plan_queue(lists, shapes, queue_band_);
  std::vector<QueueOp> ops;
  std::vector<size_t> op_off;
  need_at_.assign(jobs_.size(), {});
  cnt_off_.assign(jobs_.size(), 0);
  ncnt_ = 0;
  for (size_t q = 0; q < jobs_.size(); ++q) {
    op_off.push_back(ops.size());
    ops.insert(ops.end(), Q.ops[q].begin(), Q.ops[q].end());
    int total = 0;
    for (const QueueOp& o : Q.ops[q]) need_at_[q].push_back(o.need);
    if (!Q.ops[q].empty()) total = Q.ops[q].back().need + queue_units_per_chunk(Q.ops[q].back().kind, shapes[q]);
    need_at_[q].push_back(total);
    cnt_off_[q] = ncnt_;
    ncnt_ += shapes[q].nchunks;
  }
  nunits_ = (long long)Q.units.size();
  slot_begin_ = Q.slot_begin;
  SW_CUDA(cudaMalloc(&d_units_, std::max<size_t>(1, Q.units.size()) * sizeof(QueueUnit)));
  SW_CUDA(cudaMemcpy(d_units_, Q.units.data(), Q.units.size() * sizeof(QueueUnit), cudaMemcpyHostToDevice));
  SW_CUDA(cudaMalloc(&d_qops_, std::max<size_t>(1, ops.size()) * sizeof(QueueOp)));
  SW_CUDA(cudaMemcpy(d_qops_, ops.data(), ops.size() * sizeof(QueueOp), cudaMemcpyHostToDevice));
  SW_CUDA(cudaMalloc(&d_qcnt_, std::max(1, ncnt_) * sizeof(int)));
  SW_CUDA(cudaMalloc(&d_next_, sizeof(unsigned long long)));
  queue_bytes_ = Q.units.size() * sizeof(QueueUnit) + ops.size() * sizeof(QueueOp) + size_t(ncnt_) * sizeof(int) +
                 sizeof(unsigned long long);
  bytes_ += queue_bytes_;
  bool all_maps = true;
  for (size_t q = 0; q < jobs_.size(); ++q) {
    descs_[q].qops = d_qops_ + op_off[q];
    descs_[q].qcnt = d_qcnt_ + cnt_off_[q];
    descs_[q].qreach = queue_reach(descs_[q].g.lx);
    all_maps = all_maps && jobs_[q].tm != nullptr;
  }
  queue_tma_ = tma_ && all_maps;
  int dev = 0, sms = 0;
  SW_CUDA(cudaGetDevice(&dev));
  SW_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  queue_blocks_ = batch_queue_blocks_per_sm(queue_tma_) * sms;
  if (queue_blocks_ <= 0) throw CudaError("the batch's queue kernel cannot be resident on this GPU");
  SW_CUDA(cudaMemcpyAsync(d_jobs_, descs_.data(), descs_.size() * sizeof(JobDesc), cudaMemcpyHostToDevice, stream_));
  SW_CUDA(cudaStreamSynchronize(stream_));
}

void Batch::free_queue() {
  for (void* p : {(void*)d_units_, (void*)d_qops_, (void*)d_qcnt_, (void*)d_next_}) cudaFree(p);
  for (JobDesc& d : descs_) {  // the device copy keeps its stale pointers until the next upload; unused
    d.qops = nullptr;
    d.qcnt = nullptr;
  }
  d_units_ = nullptr;
  d_qops_ = nullptr;
  d_qcnt_ = nullptr;
  d_next_ = nullptr;
  bytes_ -= queue_bytes_;
  queue_bytes_ = 0;
  nunits_ = 0;
  slot_begin_.clear();
  need_at_.clear();
  cnt_off_.clear();
  ncnt_ = 0;
  queue_blocks_ = 0;
}

// The units of slots [t0, t1), widened to whole bands, as one launch.  Every
// job's counters start at the count its first operation at or after slot t0
// waits for, as if the slots before t0 had run (the autotuner's windows; a
// whole run starts at 0).
void Batch::enqueue_queue(int t0, int t1) {
  t0 = std::max(0, t0);
  t1 = std::min(t1, nslots_);
  if (t0 >= t1 || !d_units_) return;
  if (queue_band_ > 0) {
    t0 -= t0 % queue_band_;
    t1 = std::min(nslots_, (t1 + queue_band_ - 1) / queue_band_ * queue_band_);
  }
  if (t0 == 0) {
    SW_CUDA(cudaMemsetAsync(d_qcnt_, 0, std::max(1, ncnt_) * sizeof(int), stream_));
    SW_CUDA(cudaMemsetAsync(d_next_, 0, sizeof(unsigned long long), stream_));
  } else {
    // Copied in stream order from buffers that outlive the copies.
    window_cnt_.assign(size_t(std::max(1, ncnt_)), 0);
    for (size_t q = 0; q < jobs_.size(); ++q) {
      const std::vector<int>& n = need_at_[q];
      const int v = n[std::min(size_t(t0), n.size() - 1)];
      std::fill(window_cnt_.begin() + cnt_off_[q], window_cnt_.begin() + cnt_off_[q] + descs_[q].g.nchunks, v);
    }
    window_next_ = (unsigned long long)slot_begin_[size_t(t0)];
    SW_CUDA(cudaMemcpyAsync(d_qcnt_, window_cnt_.data(), window_cnt_.size() * sizeof(int), cudaMemcpyHostToDevice,
                            stream_));
    SW_CUDA(cudaMemcpyAsync(d_next_, &window_next_, sizeof(window_next_), cudaMemcpyHostToDevice, stream_));
    SW_CUDA(cudaStreamSynchronize(stream_));  // the host buffers are reused by the next window
  }
  SW_CUDA(launch_batch_queue(d_jobs_, d_units_, slot_begin_[size_t(t1)], d_next_, err_, queue_tma_, queue_wait_ns_,
                             queue_need_extra_, queue_blocks_, stream_));
  ++launches_per_run_;
}

void Batch::set_queue_wait_ns(unsigned long long ns) {
  SW_CUDA(cudaStreamSynchronize(stream_));
  queue_wait_ns_ = ns;
  if (graph_) cudaGraphExecDestroy(graph_);
  graph_ = nullptr;
}

void Batch::set_pdl(bool on) {
  SW_CUDA(cudaStreamSynchronize(stream_));
  pdl_ = on;
  if (graph_) cudaGraphExecDestroy(graph_);
  graph_ = nullptr;
}

void Batch::set_queue_band(int slots) {
  if (slots < 0) throw std::invalid_argument("queue_band must be >= 0");
  queue_band_ = slots;
  set_chunk_rows(chunk_rows_);  // rebuilds the schedule, drops the graph
}

void Batch::set_queue_need_extra(int n) {
  if (n < 0) throw std::invalid_argument("queue need_extra must be >= 0");
  SW_CUDA(cudaStreamSynchronize(stream_));
  queue_need_extra_ = n;
  if (graph_) cudaGraphExecDestroy(graph_);
  graph_ = nullptr;
}

void Batch::enqueue_run() {
  launches_per_run_ = 0;
  for (const Job& j : jobs_) {
    const size_t fe = problems_[j.problem].sim->view().field_elems;
    const size_t slot = size_t(j.nstate) * fe;
    SW_CUDA(cudaMemsetAsync(j.adj, 0, 2 * slot * sizeof(float), stream_));
    SW_CUDA(cudaMemsetAsync(j.grads, 0, 3 * fe * sizeof(float), stream_));
    const Sim::View v = problems_[j.problem].sim->view();
    SW_CUDA(cudaMemsetAsync(j.acc, 0, std::max(1, v.nprobe) * sizeof(float), stream_));
  }
  enqueue_slots(0, nslots_);
  // Sum the shots of each problem.
  for (size_t p = 0; p < problems_.size(); ++p) {
    const Sim::View v = problems_[p].sim->view();
    const size_t fe = v.field_elems, halo = size_t(kHaloRows) * v.ld + kHaloCols;
    const SimDesc& d = problems_[p].sim->desc();
    SW_CUDA(cudaMemsetAsync(sums_[p], 0, 3 * fe * sizeof(float), stream_));
    for (const Job& j : jobs_) {
      if (j.problem != int(p)) continue;
      for (int f = 0; f < 3; ++f) {
        float* s = sums_[p] + f * fe + halo;
        SW_CUDA(launch_add_fields(s, s, j.grads + f * fe + halo, d.nx, d.nz, v.ld, stream_));
        ++launches_per_run_;
      }
    }
  }
}

void Batch::enqueue_slots(int t0, int t1) {
  if (concurrent_ == 3) {
    enqueue_queue(t0, t1);
    return;
  }
  if (concurrent_ == 2) {
    // One stream per (kind, group), forked from and joined back into the
    // batch's stream; a job that changes kind between slots makes its new
    // kind's stream wait for its old kind's launch of the previous slot
    // (events per slot parity, batch_plan.h).  Jobs stay in their group, so
    // the waits are within a group.
    SW_CUDA(cudaEventRecord(fork_, stream_));
    for (int k = 0; k < kKinds; ++k)
      for (int g = 0; g < groups_; ++g) SW_CUDA(cudaStreamWaitEvent(kst_[plan_stream(k, g)], fork_, 0));
    const int ta = std::max(0, t0);
    for (int t = ta; t < std::min(t1, nslots_); ++t) {
      for (const Launch& l : plan_[t]) {
        cudaStream_t s = kst_[plan_stream(l.kind, l.group)];
        // A window that starts at ta > 0 (the autotuner's) has no slot ta-1
        // launches to wait for: the fork above orders it after them.
        if (t > ta)
          for (int a = 0; a < kKinds; ++a)
            if (l.deps & (1 << a)) SW_CUDA(cudaStreamWaitEvent(s, kev_[plan_event(a, l.group, t - 1)], 0));
        launch_kind(l, s);
        SW_CUDA(cudaEventRecord(kev_[plan_event(l.kind, l.group, t)], s));
      }
    }
    for (int k = 0; k < kKinds; ++k)
      for (int g = 0; g < groups_; ++g) {
        SW_CUDA(cudaEventRecord(kev_[plan_event(k, g, 0)], kst_[plan_stream(k, g)]));
        SW_CUDA(cudaStreamWaitEvent(stream_, kev_[plan_event(k, g, 0)], 0));
      }
    return;
  }
  for (int t = std::max(0, t0); t < std::min(t1, nslots_); ++t) {
    // Kinds of one slot touch different jobs: the first runs on the batch's
    // stream, the others on forked streams that join before the next slot.
    const bool fork = concurrent_ == 1 && plan_[t].size() > 1;
    if (fork) SW_CUDA(cudaEventRecord(fork_, stream_));
    int n = 0;
    for (const Launch& l : plan_[t]) {
      cudaStream_t s = stream_;
      if (fork && n > 0) {
        s = aux_[n - 1];
        SW_CUDA(cudaStreamWaitEvent(s, fork_, 0));
      }
      launch_kind(l, s);
      if (fork && n > 0) SW_CUDA(cudaEventRecord(join_[n - 1], s));
      ++n;
    }
    for (int q = 1; fork && q < n; ++q) SW_CUDA(cudaStreamWaitEvent(stream_, join_[q - 1], 0));
  }
}

void Batch::launch_kind(const Launch& l, cudaStream_t s) {
  const GroupOp* ops = d_ops_ + l.offset;
  switch (l.kind) {
    case kFwdSh: SW_CUDA(launch_grouped_forward(d_jobs_, ops, l.count, l.warps, false, pdl_, s)); break;
    case kFwdPsv: SW_CUDA(launch_grouped_forward(d_jobs_, ops, l.count, l.warps, true, pdl_, s)); break;
    case kFwd2Sh: SW_CUDA(launch_grouped_forward2(d_jobs_, ops, l.count, l.warps, false, pdl_, s)); break;
    case kFwd2Psv: SW_CUDA(launch_grouped_forward2(d_jobs_, ops, l.count, l.warps, true, pdl_, s)); break;
    case kAdjSh: SW_CUDA(launch_grouped_adjoint(d_jobs_, ops, l.count, l.warps, false, pdl_, s)); break;
    case kAdjPsv:
      if (reverse_pc_ && tma_jobs() == int(descs_.size()))
        SW_CUDA(launch_grouped_adjoint_pc(d_jobs_, ops, l.count, l.warps, pdl_, s));
      else
        SW_CUDA(launch_grouped_adjoint(d_jobs_, ops, l.count, l.warps, true, pdl_, s));
      break;
    case kMisfit: SW_CUDA(launch_grouped_misfit(d_jobs_, ops, l.count, s)); break;
  }
  ++launches_per_run_;
}

void Batch::set_stream_groups(int groups) {
  if (groups < 1 || groups > kMaxStreamGroups)
    throw std::invalid_argument("stream_groups must be 1.." + std::to_string(kMaxStreamGroups));
  groups_ = groups;
  set_chunk_rows(chunk_rows_);  // rebuilds the schedule, drops the graph
}

void Batch::set_tma(bool on) {
  SW_CUDA(cudaStreamSynchronize(stream_));
  tma_ = on;
  bool all_maps = true;
  for (size_t q = 0; q < descs_.size(); ++q) {
    descs_[q].tm = on ? jobs_[q].tm : nullptr;
    all_maps = all_maps && jobs_[q].tm != nullptr;
  }
  if (d_units_) {
    queue_tma_ = on && all_maps;
    int dev = 0, sms = 0;
    SW_CUDA(cudaGetDevice(&dev));
    SW_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    queue_blocks_ = batch_queue_blocks_per_sm(queue_tma_) * sms;
  }
  SW_CUDA(cudaMemcpyAsync(d_jobs_, descs_.data(), descs_.size() * sizeof(JobDesc), cudaMemcpyHostToDevice, stream_));
  SW_CUDA(cudaStreamSynchronize(stream_));
  if (graph_) cudaGraphExecDestroy(graph_);
  graph_ = nullptr;
}

void Batch::set_concurrent(int mode) {
  if (mode < 0 || mode > 3) throw std::invalid_argument("concurrent must be 0, 1, 2 or 3");
  SW_CUDA(cudaStreamSynchronize(stream_));
  const bool rebuild = (mode == 3) != (concurrent_ == 3);
  concurrent_ = mode;
  if (graph_) cudaGraphExecDestroy(graph_);
  graph_ = nullptr;
  if (rebuild) set_chunk_rows(chunk_rows_);
}

void Batch::run() {
  if (!graph_) {
    cudaGraph_t g = nullptr;
    SW_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
    try {
      enqueue_run();
    } catch (...) {
      cudaStreamEndCapture(stream_, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    SW_CUDA(cudaStreamEndCapture(stream_, &g));
    cudaError_t e = cudaGraphInstantiate(&graph_, g, 0);
    cudaGraphDestroy(g);
    SW_CUDA(e);
  }
  SW_CUDA(cudaGraphLaunch(graph_, stream_));
  // NaN / infinity watchdog over every problem's gradient block.
  for (size_t p = 0; p < problems_.size(); ++p) {
    const Sim::View v = problems_[p].sim->view();
    const long rows = 3L * (problems_[p].sim->desc().nx + 2 * kHaloRows);
    SW_CUDA(launch_check_finite(sums_[p], rows, v.ld, v.ld, err_, kErrNonFiniteGradient, stream_));
  }
  // Per-trace misfits, summed per problem in a fixed order.
  host_J_.assign(problems_.size(), 0.0);
  std::vector<double> buf;
  for (const Job& j : jobs_) {
    buf.resize(size_t(j.ncomp) * j.nrec);
    if (!buf.empty())
      SW_CUDA(cudaMemcpyAsync(buf.data(), j.J, buf.size() * sizeof(double), cudaMemcpyDeviceToHost, stream_));
    SW_CUDA(cudaStreamSynchronize(stream_));
    for (double x : buf) host_J_[j.problem] += x;
  }
  int e = 0;
  SW_CUDA(cudaMemcpy(&e, err_, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) SW_CUDA(cudaMemset(err_, 0, sizeof(int)));  // reported once
  if (e & kErrWaitTimeout)
    throw WaitTimeout(
        "a batched kernel gave up waiting for its row pipeline or, in the device queue, for a unit's dependencies "
        "(bounded wait expired)");
  if (e & kErrNonFiniteGradient) throw NumericError("a batched gradient holds NaN or infinite values");
}

void Batch::download_gradient(int problem, int which, float* host) const {
  if (problem < 0 || problem >= int(problems_.size())) throw std::invalid_argument("problem index out of range");
  if (which < 0 || which > 2) throw std::invalid_argument("gradient index out of range");
  const Sim::View v = problems_[problem].sim->view();
  const SimDesc& d = problems_[problem].sim->desc();
  const size_t halo = size_t(kHaloRows) * v.ld + kHaloCols;
  SW_CUDA(cudaMemcpy2DAsync(host, size_t(d.nz) * sizeof(float), sums_[problem] + which * v.field_elems + halo,
                            size_t(v.ld) * sizeof(float), size_t(d.nz) * sizeof(float), size_t(d.nx),
                            cudaMemcpyDeviceToHost, stream_));
  SW_CUDA(cudaStreamSynchronize(stream_));
}

double Batch::misfit(int problem) const {
  if (problem < 0 || problem >= int(host_J_.size())) return 0.0;
  return host_J_[problem];
}

}  // namespace seiswg
