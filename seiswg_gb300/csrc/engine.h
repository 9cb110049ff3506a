// engine.h -- the device-side solver: wavefield and model storage in HBM,
// the time loop (optionally captured as one CUDA graph), receivers,
// snapshots and the reference adjoint.  Host code only; kernels are launched
// through fd_kernels.h.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "batch_plan.h"
#include "fd_kernels.h"

namespace seiswg {

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// A run whose results hold NaN or infinite values.
struct NumericError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// A kernel gave up a bounded wait; the run's results are invalid.
struct WaitTimeout : CudaError {
  using CudaError::CudaError;
};

void cuda_check(cudaError_t e, const char* what);
#define SW_CUDA(call) ::seiswg::cuda_check((call), #call)

// Grid and physics of one simulation (the numeric part of the reference's
// Params uniform, fd2d.wgsl:18-49).
struct SimDesc {
  int nx = 0, nz = 0, nt = 0;
  float dx = 0, dz = 0, dt = 0;
  bool sh = false, psv = true, spin = false;
  bool abs_left = false, abs_right = false, abs_bottom = false, abs_top = false;
  int abs_width = 20;
  float abs_alpha = 0.015f;
};

// Model slots the caller can upload (host arrays indexed k = i*nz + j).
enum class ModelField { VP, VS, RHO, LAMBDA, MU, NU, J, LAMBDA_C, MU_C, NU_C };

// Wavefield components a snapshot can read.
enum class StateField { VY, SXY, SZY, VX, VZ, SXX, SZZ, SXZ, VYC, SYX, SYY, SYZ };

// Device arena: one cudaMalloc carved into 256-byte aligned pieces.
class Arena {
 public:
  Arena() = default;
  ~Arena();
  Arena(const Arena&) = delete;
  Arena& operator=(const Arena&) = delete;
  void reserve(size_t bytes) { plan_ += (bytes + 255) & ~size_t(255); }
  void commit();
  void* take(size_t bytes);
  size_t bytes() const { return plan_; }

 private:
  char* base_ = nullptr;
  size_t plan_ = 0, used_ = 0;
};

// A 3-D tensor map over nfields padded fields (columns ld, rows rows_alloc)
// whose element (0, 0) pointers are `first` + f * stride floats, with boxes of
// 128 columns x 1 row x box_fields fields; false when the driver cannot
// encode it.
bool encode_fields(CUtensorMap* m, const float* first, ptrdiff_t stride, int nfields, int ld, int rows_alloc,
                   int box_fields);

class Sim {
 public:
  Sim(const SimDesc& d, cudaStream_t stream = nullptr);
  ~Sim();
  Sim(const Sim&) = delete;
  Sim& operator=(const Sim&) = delete;

  const SimDesc& desc() const { return d_; }
  int ld() const { return ld_; }
  cudaStream_t stream() const { return stream_; }

  // ---- set-up ----
  void upload_model(ModelField f, const float* host);
  // vps2lm when the model came as vp/vs (fd2d.wgsl:188-201), mu_c + nu_c,
  // the absorbing taper factors (fd2d.wgsl:203-235).
  void prepare_model();
  // Sources at cells (i, j) with STF table [3][n][nt] (x, y, z components).
  void set_sources(int n, const int* i, const int* j, const float* stf_xyz);
  // Receivers at cells (i, j).
  void set_receivers(int n, const int* i, const int* j);
  int nsrc() const { return nsrc_; }
  int nrec() const { return nrec_; }

  // ---- forward ----
  // One shot (isrc >= 0) or all sources together (isrc = -1), nt steps from
  // rest.  Snapshots of `snap_fields` after every step it > 0 with
  // it % snap_every == 0 are copied to host memory.
  struct Snapshots {
    int every = 0;
    std::vector<StateField> fields;
    std::vector<std::vector<float>> frames;  // [nsnap * fields.size()][npt], k = i*nz + j
    std::vector<int> steps;
  };
  void run_forward(int isrc, Snapshots* snaps = nullptr);
  // Traces of the last forward run, [5][nrec][nt] (x, y, z, yi, yc); only
  // the components whose bit is set in `comps` are copied (the others of
  // `host` are left as they are).
  void download_traces(float* host, unsigned comps = 0x1f) const;
  // A wavefield component of the current state.
  void download_state(StateField f, float* host) const;

  // ---- reference adjoint (solver.rs:1298-1529), SH imaging ----
  // Adds one shot's contribution to kmu: forward with vy saved every
  // `adj_interval` steps, adjoint with the time-reversed adjoint source
  // `adstf` [nrec][nt] injected at the receivers, imaging every interval.
  // The caller computes the adjoint source from the forward traces.
  void adjoint_forward(int isrc, int adj_interval);
  void adjoint_backward(const float* adstf_host, int adj_interval);
  void clear_kmu();
  void smooth_kmu(float sigma);
  // The same Gaussian smoothing of a host field (nx*nz values, in place),
  // through the kmu buffer (whose contents it replaces).
  void smooth_field(float* host, float sigma);
  void download_kmu(float* host) const;

  // ---- exact discrete adjoint with checkpointing --------------------------
  // forward_op: one forward run of source isrc (-1: all) that also stores the
  // full wavefield state every `ckpt_every` steps (0: the scheme the budget
  // allows -- every state, every second one, every ceil(sqrt(nt)), else
  // binomial checkpointing; default_checkpoint_interval).
  // backward_op: the reverse sweep for the adjoint source adj = dJ/dd of the
  // recorded traces, [ncomp][nrec][nt] (SH: uy; PSV: ux, uz), rebuilding the
  // forward states of each checkpoint interval by recomputation; gradients
  // with respect to lambda, mu and the buoyancy 1/rho accumulate across calls.
  void gradient_clear();
  void forward_op(int isrc, int ckpt_every);
  void backward_op(const float* adj_host);
  // On-device misfit: the host pair (l2 misfit of downloaded traces, upload of
  // the adjoint source) without the round trip.  set_observed uploads the
  // observed traces [ncomp][nrec][nt] (same components as backward_op);
  // misfit_op, after a forward_op, returns J and leaves dt * U on the device;
  // backward_op_device then runs the reverse sweep with it.
  void set_observed(const float* obs_host);
  double misfit_op();
  void backward_op_device();
  // which: 0 lambda, 1 mu, 2 buoyancy
  void download_gradient(int which, float* host) const;
  int checkpoint_interval() const { return ck_k_; }
  // Binomial checkpointing slots of the last forward_op (0: uniform
  // checkpoints every checkpoint_interval() steps), the forward steps its
  // reverse sweep recomputes, and the bytes its checkpoints hold.
  int checkpoint_slots() const { return rv_slots_; }
  long long recompute_steps() const { return recompute_steps_; }
  // Options of the checkpoint scheme: binomial checkpointing with S slots
  // (0: the default choice), and the memory the default choice may use for
  // checkpoints (0: the free HBM less a reserve of a tenth of the device).
  void set_checkpoint_slots(int S) { rv_force_ = S > 0 ? S : 0; }
  void set_checkpoint_budget(size_t bytes) { ck_budget_ = bytes; }
  // Frees the checkpoint, interval, adjoint and snapshot buffers (they are
  // allocated again on the next use); gradients are kept.
  void release_workspace();
  size_t checkpoint_bytes() const { return ck_bytes_; }

  // Device-side pieces of this simulation that a Batch shares between the
  // jobs of one problem (read-only after set-up).
  struct View {
    Geom geom;
    Geom geom2;             // two-step decomposition (lx 0 when the two-step kernel is off)
    int ld;
    size_t field_elems;
    const float *rho, *lam, *mu, *taper_x, *taper_zb, *taper_zt;
    const float* rho_dt;    // dt/rho, then dt*lambda and dt*mu at the material's stride (null: no two-step kernel)
    const float* stf;       // [3][nsrc][nt]
    const Probe* probes;    // SH segment, then PSV segment
    int nprobe, probe_split;
    const int* tr_idx;      // [nrec][12]
    const int *src_i, *src_j, *rec_i, *rec_j;  // host arrays
  };
  View view() const;

  // Graph capture of whole time loops (replayed on repeated runs).
  void set_use_graphs(bool on) { use_graphs_ = on; }
  void set_chunk_rows(int lx);
  // Rows per warp chunk from a wave-quantisation model: resident warps come
  // from the occupancy of the step kernel; the cost of a choice is
  // ceil(warps / resident) waves x (lx + 5) rows per warp.
  int model_chunk_rows() const;
  // The same model for the reverse-step kernel, whose occupancy differs.
  Geom adjoint_geom();
  // Empirical tuning: times `steps` forward steps for each candidate
  // (row loader x rows per chunk) on this problem and keeps the fastest.
  // Runs on the current state buffers, which every run resets, so it must
  // not be called between a forward_op and its backward_op.  Returns the
  // best time per step in microseconds.
  double autotune(int steps);
  void set_loader(int loader);  // kLoaderDirect or kLoaderBulk
  // Forward runs advance two steps per launch (PSV without SH or spin, the
  // default there; steps before a snapshot and an odd last step run the
  // one-step kernel).  Rows per chunk of that kernel: 0 = its own
  // wave-quantisation model.
  void set_two_step(bool on);
  void set_two_step_rows(int lx);
  bool two_step() const { return two_step_; }
  // Two-step PSV launches with tensor copies take their rows from producer
  // warps (launch_psv_step2_pc; default on) or issue the copies in every
  // march (launch_psv_step2_tma); the same bits.
  void set_two_step_producer(bool on) {
    two_step_pc_ = on;
    for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
    graphs_.clear();
  }
  // PSV reverse steps with tensor copies take their rows from producer warps
  // (launch_psv_adjoint_pc; default on) or issue the copies in every march;
  // the same bits.
  void set_reverse_producer(bool on) {
    reverse_pc_ = on;
    for (auto& kv : graphs_) cudaGraphExecDestroy(kv.second);
    graphs_.clear();
  }
  // Small SH grids run whole forward passes in one thread-block cluster when
  // state and material fit its shared memory (default on).
  void set_use_cluster(bool on) { use_cluster_ = on; }
  // Two-step PSV launches fetch their rows with 3-D tensor copies where the
  // state's fields lie at a uniform stride (default on).
  void set_use_tma(bool on);
  int loader() const { return geom_.loader; }
  // Throws if a kernel recorded an error (a bounded wait ran out, or the
  // traces or gradients of the last run hold NaN or infinite values); the
  // error word is cleared once read.
  void check_device_error() const;
  // Stability numbers of the model and dt (computed by prepare_model; the
  // run is rejected above 1 while the check is on): the wave number dt c
  // (7/6) sqrt(1/dx^2 + 1/dz^2) and, with spin, (dt/2) sqrt(4 nu/J +
  // (mu_c+nu_c)/J (7/3)^2 (1/dx^2 + 1/dz^2)) (0 without spin).
  double stability_wave() const { return cfl_wave_; }
  double stability_spin() const { return cfl_spin_; }
  // prepare_model rejects an unstable dt (default on).
  void set_stability_check(bool on) { stability_check_ = on; }
  // Polls of a bounded row-pipeline wait before a kernel gives up (0: the
  // built-in limit).  arm_extra is a test hook: that many bytes are armed on
  // the first stage of every warp's ring beyond its copies, so that every
  // launch's first wait runs out (0 for normal runs).
  void set_wait_polls(unsigned polls);
  void set_arm_extra(unsigned bytes);
  // Step and reverse launches may start while the previous one finishes
  // (programmatic dependent launch; default on).  Drops the captured graphs.
  void set_pdl(bool on);
  int chunk_rows() const { return geom_.lx; }
  uint64_t kernel_launches() const { return launches_; }
  void synchronize() const;

  size_t device_bytes() const { return arena_.bytes() + (fwd_store_ ? fwd_bytes_ : 0); }

 private:
  struct State {
    float *vy = nullptr, *sxy = nullptr, *szy = nullptr;
    float *vx = nullptr, *vz = nullptr, *sxx = nullptr, *szz = nullptr, *sxz = nullptr;
    float *vyc = nullptr, *syx = nullptr, *syy = nullptr, *syz = nullptr;
  };
  float* field_ptr(float* alloc) const { return alloc + size_t(kHaloRows) * ld_ + kHaloCols; }
  float* alloc_field();
  void zero_state();
  void enqueue_step(int it, int src_buf, const InjectList& inj, const ProbeList& probes, bool sh_only);
  void enqueue_step_states(int it, const struct State& a, const struct State& o, const InjectList& inj,
                           const ProbeList& probes, bool sh_only);
  State slot_state(float* slot) const;  // nstate consecutive fields starting at `slot`
  int nstate() const { return (d_.sh ? 3 : 0) + (d_.psv ? 5 : 0); }
  void copy_state(const State& dst, const State& src);
  InjectList source_injections(int isrc);
  ProbeList probe_list() const;
  void enqueue_traces();
  float* state_ptr(StateField f, int buf) const;
  void build_probe_tables();
  void upload_inject(const std::vector<Inject>& list, int which);
  void run_loop(const std::string& key, const std::function<void()>& body);
  void copy_field_to_host(const float* dev, float* host) const;
  int chunk_rows_for(int blocks_per_sm, int strip_cols, int extra_rows) const;
  // mid: where not null, the state after step `it` is stored there too.
  void enqueue_step2(int it, const State& a, const State& o, const InjectList& inj, const ProbeList& probes,
                     const State* mid = nullptr);
  // cap >= 0: a scheme needing at most `cap` bytes (after an allocation of a
  // larger one failed).
  int default_checkpoint_interval(double cap = -1.0) const;
  int final_buffer(int snap_every) const;  // buffer holding the state after run_forward

  SimDesc d_;
  cudaStream_t stream_;
  bool own_stream_ = false;
  int ld_ = 0;
  size_t field_elems_ = 0;  // rows_alloc * ld
  Geom geom_{};
  Geom geom2_{};            // decomposition of the two-step kernel (lx 0: not yet modelled)
  bool two_step_ = false;
  bool two_step_pc_ = true;
  bool reverse_pc_ = true;
  bool use_cluster_ = true;
  bool use_tma_ = true;
  int tma_mat_ = -1;   // material tensor maps: -1 not yet encoded, 0 unavailable, 1 in tma_
  Tma2 tma_{};         // rho and lm (the dt-scaled material) set once; sig and vel per launch
  CUtensorMap mat1_{}, mat2_{};  // the material (1/rho, lambda, mu) with boxes of 1 and 2 fields
  TmaAdj tma_adj_{};   // reverse step: g1, g2 for the gradient block at tma_grad_, the rest per launch
  const float* tma_grad_ = nullptr;
  bool tma_ready();
  bool launch_adjoint_tma(const PsvAdjoint& p, const State& f, const State& a);
  int cluster_ctas_ = -1;   // CTAs of the cluster path (0: grid too large; -1: not yet queried)
  int adj_lx_[2] = {0, 0};  // reverse-step rows per chunk, per loader (0: not yet modelled)
  Arena arena_;
  State st_[2];
  unsigned* red_ = nullptr;      // device scratch of the stability reduction
  double cfl_wave_ = 0, cfl_spin_ = 0;
  bool stability_check_ = true;
  void check_stability();
  float *rho_ = nullptr, *lam_ = nullptr, *mu_ = nullptr;
  float *rdt_ = nullptr, *ldt_ = nullptr, *mdt_ = nullptr;  // dt/rho, dt*lambda, dt*mu (two-step kernels)
  float *nu_ = nullptr, *jm_ = nullptr, *muc_ = nullptr, *nuc_ = nullptr, *mc_ = nullptr;
  float *taper_x_ = nullptr, *taper_zb_ = nullptr, *taper_zt_ = nullptr;
  float *kmu_ = nullptr, *tmp_ = nullptr;
  bool vps_input_ = false;
  bool prepared_ = false;
  float den_x_ = 0, den_z_ = 0;   // 8*dx, 8*dz (reference denominators)

  // sources and receivers
  int nsrc_ = 0, nrec_ = 0;
  std::vector<int> src_i_, src_j_, rec_i_, rec_j_;
  float* stf_ = nullptr;          // [3][nsrc][nt]
  float* adstf_ = nullptr;        // [nrec][nt]
  Inject* inj_dev_[2] = {nullptr, nullptr};  // 0: sources, 1: receivers (adjoint)
  int inj_n_[2] = {0, 0}, inj_cap_[2] = {0, 0};
  Probe* probes_ = nullptr;
  int nprobe_ = 0;
  int probe_split_ = 0;           // SH probes first, then PSV probes
  float *probe_acc_ = nullptr, *probe_hist_ = nullptr;
  int *tr_idx_ = nullptr;         // per receiver probe indices (device)
  float* obs_ = nullptr;          // [5][nrec][nt]
  int cur_buf_ = 0;               // buffer holding the current state
  float* snap_store_ = nullptr;   // device snapshot frames
  size_t snap_cap_ = 0;

  // reference adjoint forward-wavefield store
  float* fwd_store_ = nullptr;
  size_t fwd_bytes_ = 0;
  int fwd_nsa_ = 0;

  int* err_ = nullptr;            // device error word
  // exact adjoint storage
  int ck_k_ = 0, ck_n_ = 0, ck_isrc_ = -2;
  size_t ck_bytes_ = 0;
  float* ck_store_ = nullptr;   // ck_n_ states
  float* seg_store_ = nullptr;  // ck_k_ states of one interval
  float* adj_store_ = nullptr;  // 2 adjoint states
  float *g_lam_ = nullptr, *g_mu_ = nullptr, *g_b_ = nullptr;
  float* u_tab_ = nullptr;      // dt * U, [ncomp][nrec][nt]
  float* obs_in_ = nullptr;     // observed traces for misfit_op, [ncomp][nrec][nt]
  double* j_tr_ = nullptr;      // misfit per trace
  bool u_ready_ = false;        // u_tab_ holds the adjoint source of the last forward_op
  void run_backward();
  void ensure_u_tab();
  void enqueue_reverse(int n, const State& f, const State& a, const State& o, const InjectList& src,
                       const InjectList& rec, const Geom& ga);
  // binomial checkpointing (batch_plan.h job_ops_revolve)
  int rv_slots_ = 0, rv_force_ = 0;
  size_t ck_budget_ = 0;
  long long recompute_steps_ = 0;
  float* rv_store_ = nullptr;              // rv_slots_ states
  std::vector<HostOp> rv_ops_;
  State rv_slot(int q) const;
  void forward_op_binomial(int isrc, int S);
  void free_checkpoints();

  bool use_graphs_ = true;
  std::map<std::string, cudaGraphExec_t> graphs_;
  std::map<std::string, uint64_t> graph_nodes_;
  uint64_t launches_ = 0;
};

}  // namespace seiswg
