// batch.h -- gradients of many independent problems (uneven grids, SH or
// PSV, several shots each) advanced together.
//
// Every (problem, shot) is a job with its own wavefield storage.  The host
// builds each job's operation list -- a recording forward pass writing a
// checkpoint every k steps, the on-device misfit, then for each checkpoint
// interval from the last one a forward recomputation followed by the reverse
// steps (batch_plan.h) -- and lays all lists side by side: global slot t
// holds operation t of every job that has one.  Each slot is one grouped
// launch per kind (forward SH or PSV, one or two steps; reverse SH or PSV;
// misfit) whose warps cover all jobs doing that kind of work, so that small
// problems share the GPU.  The whole schedule is captured once as a CUDA
// graph and replayed.
#pragma once

#include <memory>
#include <vector>

#include "batch_plan.h"
#include "engine.h"

namespace seiswg {

struct BatchProblem {
  Sim* sim;                  // model, sources and receivers set up; not owned
  std::vector<float> obs;    // observed traces [nshot][ncomp][nrec][nt]
};

class Batch {
 public:
  // ckpt_every: checkpoint interval of every job (0: ceil(sqrt(nt)) per job).
  // stream: nullptr for a stream of the batch's own.
  Batch(const std::vector<BatchProblem>& problems, int ckpt_every, cudaStream_t stream);
  ~Batch();
  Batch(const Batch&) = delete;
  Batch& operator=(const Batch&) = delete;

  // All gradients: every shot of every problem, summed per problem.
  void run();
  // Rows per warp chunk of every job (0: each problem's own chunk model).
  // Rebuilds the schedule; the captured graph is dropped.
  void set_chunk_rows(int lx);
  // Empirical tuning of the chunk rows and of one- or two-step recording:
  // times a window of `slots` slots at the start of the recording pass and
  // one in the middle of the reverse sweep for each candidate, scales each to
  // its phase's slot count and keeps the candidate with the shortest total.
  // Returns that projected time in milliseconds.  The timed launches leave
  // results that the next run() overwrites.
  double autotune(int slots);
  int chunk_rows() const { return chunk_rows_; }
  // Jobs (PSV alone, SH alone) record two steps per launch between
  // checkpoints (default on); rebuilds the schedule.  The autotuner also
  // tries both.
  void set_two_step(bool on);
  bool two_step() const { return two_step_; }
  // With two-step recording, grouped launches also recompute two steps per
  // operation, storing both states (default on; launch order 3 always
  // recomputes one step per operation); rebuilds the schedule.
  void set_two_step_recompute(bool on);
  // Grouped PSV reverse launches take their rows from producer warps when
  // every job fetches by tensor copies (default off: a producer CTA takes a
  // whole SM, which packs worse beside the other kinds' launches); drops the
  // graph.
  void set_reverse_producer(bool on) {
    reverse_pc_ = on;
    if (graph_) cudaGraphExecDestroy(graph_);
    graph_ = nullptr;
  }
  // How the schedule runs.  0: one grouped launch per (slot, kind), one
  // after another on the batch's stream.  1: the launches of one slot run
  // concurrently on forked streams that join before the next slot.  2: one
  // stream per kind; a launch waits only for the previous slot's launches of
  // the kinds its jobs come from, so the kinds pipeline (default).  3: one
  // persistent launch over a device work queue of every job's units
  // (fd_queue.cu, plan_queue in batch_plan.h); the one- and two-step
  // geometries of a job then share their rows per chunk (the larger of the
  // two).  Entering or leaving mode 3 rebuilds the schedule; every change
  // drops the captured graph.
  void set_concurrent(int mode);
  int concurrent() const { return concurrent_; }
  // Jobs split round-robin into this many groups (1..kMaxStreamGroups), each
  // with its own launches per slot and kind, and, in mode 2, its own streams:
  // smaller launches that overlap more.  Rebuilds the schedule.
  static constexpr int kMaxStreamGroups = 4;  // = kPlanGroupsMax (batch_plan.h)
  void set_stream_groups(int groups);
  int stream_groups() const { return groups_; }
  // Grouped launches fetch rows with 3-D tensor copies (default on) or one
  // bulk copy per field; the same results.  Drops the captured graph.
  void set_tma(bool on);
  bool tma() const { return tma_; }
  // Grouped forward and reverse launches may start while the previous launch
  // in their stream finishes (programmatic dependent launch; default on).
  // Drops the captured graph.
  void set_pdl(bool on);
  bool pdl() const { return pdl_; }
  // Jobs whose grouped launches fetch rows by tensor copies: all with a map
  // table while the option is on (a job whose fields do not lie at uniform
  // strides has none), 0 while it is off.
  int tma_jobs() const {
    int n = 0;
    for (const JobDesc& d : descs_) n += d.tm != nullptr;
    return n;
  }
  // Binomial checkpointing (job_ops_revolve, batch_plan.h) with S state
  // slots per job (plus the two working slots); 0 returns to uniform
  // checkpoints.  Reallocates every job's pool and rebuilds the schedule.
  void set_checkpoint_slots(int S);
  int checkpoint_slots() const { return checkpoint_slots_; }
  // Forward steps the reverse sweeps of all jobs recompute per run.
  long long recompute_steps() const;
  // Launch order 3: the bound of a dependency wait in the queue kernel
  // (nanoseconds), and a test hook added to every dependency after a job's
  // first operation so that those waits run out (0 normally).
  void set_queue_wait_ns(unsigned long long ns);
  void set_queue_need_extra(int n);
  // Launch order 3: slots per band of the queue's order (plan_queue; 0:
  // slot-major).  Rebuilds the schedule.
  void set_queue_band(int slots);
  int queue_band() const { return queue_band_; }
  // Units in the device queue (0 outside launch order 3) and its CTAs.
  long long queue_units() const { return nunits_; }
  int queue_blocks() const { return queue_blocks_; }
  // which: 0 lambda, 1 mu, 2 buoyancy (zero for lambda of SH problems).
  void download_gradient(int problem, int which, float* host) const;
  double misfit(int problem) const;  // sum over the problem's shots and traces of the last run
  int jobs() const { return int(jobs_.size()); }
  int slots() const { return nslots_; }
  size_t device_bytes() const { return bytes_; }
  uint64_t launches_per_run() const { return launches_per_run_; }
  cudaStream_t stream() const { return stream_; }

 private:
  struct Job {
    int problem, shot, k, ncp, nslot, nt, nstate, ncomp, nrec;
    int S = 0;           // binomial checkpointing slots (0: uniform checkpoints every k steps)
    int pool_slots = 0;  // slots of the allocated pool
    bool psv;
    CUtensorMap* tm = nullptr;  // the job's tensor-map table in device memory (see JobDesc)
    float *pool = nullptr, *adj = nullptr, *grads = nullptr, *acc = nullptr, *hist = nullptr, *obs = nullptr,
          *u_tab = nullptr;
    double* J = nullptr;
    Inject* src = nullptr;
    Inject* rec = nullptr;
  };
  void build_schedule();
  void alloc_pool(size_t q);
  int checkpoint_slots_ = 0;
  void enqueue_run();
  void enqueue_slots(int t0, int t1);
  std::vector<JobDesc> descs_;   // host copy of d_jobs_
  std::vector<Geom> model_geom_; // each job's geometry from its problem's chunk model
  std::vector<Geom> model_geom2_;  // ... of its two-step kernel (lx 0: none)
  int chunk_rows_ = 0;
  bool two_step_ = true;
  bool pair_ = true;  // two-step recomputation (set_two_step_recompute)
  bool reverse_pc_ = false;
  size_t ops_bytes_ = 0;

  std::vector<BatchProblem> problems_;
  std::vector<Job> jobs_;
  cudaStream_t stream_;
  bool own_stream_ = false;
  int concurrent_ = 2;
  bool tma_ = true;   // grouped launches fetch rows by tensor copies where the job has a map table
  bool pdl_ = true;   // grouped launches with programmatic dependent launch
  int groups_ = 1;
  std::vector<cudaStream_t> aux_;   // mode 1: forked streams for a slot's other kinds
  cudaEvent_t fork_ = nullptr;
  std::vector<cudaEvent_t> join_;
  std::vector<cudaStream_t> kst_;   // mode 2: one stream per (kind, group)
  std::vector<cudaEvent_t> kev_;    // ... one event per (kind, group, slot parity) (plan_event)
  int ckpt_every_;
  JobDesc* d_jobs_ = nullptr;
  GroupOp* d_ops_ = nullptr;
  int* err_ = nullptr;
  // per slot and kind: [offset, count, warps] into d_ops_
  struct Launch {
    int kind, offset, count, warps;
    int deps;  // kinds of the previous slot that some of this launch's jobs come from (bit mask)
    int group;
  };
  std::vector<std::vector<Launch>> plan_;
  void launch_kind(const Launch& l, cudaStream_t s);
  int nslots_ = 0;
  int rec_slots_ = 0;  // slots of the longest recording pass (before the misfit)
  std::vector<float*> sums_;   // per problem: 3 gradient fields
  std::vector<double> host_J_;
  size_t bytes_ = 0;
  cudaGraphExec_t graph_ = nullptr;
  uint64_t launches_per_run_ = 0;

  // Launch order 3: the device queue (plan_queue).
  void build_queue(const std::vector<std::vector<HostOp>>& lists);
  void free_queue();
  void enqueue_queue(int t0, int t1);  // the units of slots [t0, t1)
  QueueUnit* d_units_ = nullptr;
  QueueOp* d_qops_ = nullptr;
  int* d_qcnt_ = nullptr;
  unsigned long long* d_next_ = nullptr;
  long long nunits_ = 0;
  size_t queue_bytes_ = 0;
  std::vector<long long> slot_begin_;       // first unit of each slot
  std::vector<std::vector<int>> need_at_;   // per job: need of each operation, then the total
  std::vector<int> cnt_off_;                // per job: its first counter
  std::vector<int> window_cnt_;             // the counters a window of slots starts from (enqueue_queue)
  unsigned long long window_next_ = 0;
  int ncnt_ = 0;
  int queue_blocks_ = 0;
  bool queue_tma_ = false;
  unsigned long long queue_wait_ns_ = 2000000000ull;
  int queue_need_extra_ = 0;
  int queue_band_ = 0;
};

}  // namespace seiswg
