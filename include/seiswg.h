/*
 * seiswg.h -- C ABI of the GB300 (sm_103a) implementation of seiswg's 2-D
 * staggered-grid finite-difference path.
 *
 * The reference exposes this path through its Rust host API and, one level
 * down, through the WGSL kernel interface.  Both levels are mirrored here
 * with plain pointers and sizes:
 *
 *   reference                                     this header
 *   config::load            (src/config.rs:118)   seiswg_config_load
 *   config::load_from_str   (src/config.rs:132)   seiswg_config_load_str
 *   Vfs = HashMap<String, Vec<u8>> (src/solver.rs:15)   seiswg_vfs_*
 *   Solver::new             (src/solver.rs:578)   seiswg_solver_new
 *   Solver::run_forward     (src/solver.rs:941)   seiswg_solver_run_forward
 *   Solver::run_adjoint     (src/solver.rs:1298)  seiswg_solver_run_adjoint
 *   mode = inversion        (src/main.rs:93-94, planned)  seiswg_solver_run_inversion
 *   fields/idata/obs/stf bindings and the per-step kernel chain
 *     (shaders/fd2d.wgsl:123-127, src/solver.rs:984-1044)   seiswg_sim_*
 *   ricker                  (src/solver.rs:350)   seiswg_ricker
 *   compute_waveform_misfit (src/solver.rs:432)   seiswg_waveform_misfit
 *   make_npy_bytes          (src/solver.rs:270)   seiswg_npy_encode
 *   grid inference          (src/solver.rs:646-656) seiswg_infer_grid
 *
 * Conventions
 *   - Every function returns SEISWG_OK (0) or an error code; the message of
 *     the last failure on the calling thread is seiswg_last_error().  The
 *     reference's anyhow::Result context strings map to these messages.
 *   - Inputs are caller-owned and copied in; outputs are written to
 *     caller-provided buffers or to a seiswg_vfs the caller frees.
 *   - Grids are indexed k = i*nz + j (z contiguous), as in the reference.
 *   - One handle is used by one host thread at a time.  Device work runs on
 *     the handle's CUDA stream (its own, or the one passed at creation).
 */
#ifndef SEISWG_H
#define SEISWG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SEISWG_OK 0
#define SEISWG_EINVAL 1    /* invalid argument or input data */
#define SEISWG_EIO 2       /* a file or VFS entry is missing or unreadable */
#define SEISWG_ECUDA 3     /* CUDA runtime failure (no device, out of memory, launch error) */
#define SEISWG_EINTERNAL 4
#define SEISWG_ENUMERIC 5  /* the run's traces or gradients hold NaN or infinite values */
#define SEISWG_ETIMEOUT 6  /* a kernel's bounded wait expired; the run's results are invalid */

/* Message of the last failed call on this thread ("" after a success). */
const char* seiswg_last_error(void);
const char* seiswg_version(void);

/* ---- virtual file system (src/solver.rs:15, lookups :236-267) ------------ */
typedef struct seiswg_vfs seiswg_vfs;
seiswg_vfs* seiswg_vfs_new(void);
void seiswg_vfs_free(seiswg_vfs* vfs);
/* Inserts (or replaces) `key` with a copy of `len` bytes. */
int seiswg_vfs_insert(seiswg_vfs* vfs, const char* key, const void* data, size_t len);
/* Borrowed view of an entry; valid until the entry is replaced or freed. */
int seiswg_vfs_get(const seiswg_vfs* vfs, const char* key, const void** data, size_t* len);
size_t seiswg_vfs_size(const seiswg_vfs* vfs);
/* Key of the index-th entry in sorted order, or NULL past the end. */
const char* seiswg_vfs_key(const seiswg_vfs* vfs, size_t index);

/* ---- configuration (src/config.rs) ---------------------------------------- */
typedef struct seiswg_config seiswg_config;
/* config::load: reads an INI file; paths resolve relative to its directory. */
int seiswg_config_load(const char* path, seiswg_config** out);
/* config::load_from_str: INI text with paths resolved against base_dir. */
int seiswg_config_load_str(const char* ini_text, const char* base_dir, seiswg_config** out);
void seiswg_config_free(seiswg_config* cfg);
/* Reads one parsed value as text: "workflow", "solver.<key>", "path.<key>"
 * (e.g. "solver.nt", "path.output").  Fails when the key is unset. */
int seiswg_config_get(const seiswg_config* cfg, const char* key, char* buf, size_t buflen);

/* ---- solver (src/solver.rs:194-1530) -------------------------------------- */
typedef struct seiswg_solver seiswg_solver;
/* Solver::new: loads the model, sources and stations (VFS first, then disk),
 * infers the grid, builds the Ricker STF table and uploads everything. */
int seiswg_solver_new(const seiswg_config* cfg, const seiswg_vfs* vfs, seiswg_solver** out);
/* Native builds of the reference write outputs to disk as well as returning
 * them (the default here too); 0 returns them only. */
int seiswg_solver_set_write_files(seiswg_solver* s, int on);
/* Solver::run_forward: traces (uy/ux/uz/ry/yi .npy, raw vy/vx/vz) and
 * snapshots (proc<it>_<field>.bin, "snapshot/..." entries) into `out`. */
int seiswg_solver_run_forward(seiswg_solver* s, seiswg_vfs* out);
/* Solver::run_adjoint: observed uy traces from `vfs` (or disk); writes
 * proc000000_kmu.bin and gradient_kmu.bin into `out`. */
int seiswg_solver_run_adjoint(seiswg_solver* s, const seiswg_vfs* vfs, seiswg_vfs* out);
/* `[workflow] mode = inversion`, which the reference lists as planned
 * (README.md:61) and rejects (src/main.rs:93-94): steepest descent from the
 * initial model ([path] model_init) toward the observed traces ([path]
 * traces: uy_NNNNNN.npy for SH, ux_ and uz_NNNNNN.npy for PSV, one per shot),
 * each gradient the exact discrete adjoint summed over the shots and smoothed,
 * with a backtracking line search.  New keys, which the reference ignores,
 * under [inversion]: iterations (5), parameters ("vp,vs"; of vp, vs, rho),
 * step (0.02, the first relative model change), max_step (0.1),
 * line_search_trials (6), smooth (gradient smoothing sigma in cells; default
 * [solver] smooth).  Writes proc000000_{vp,vs,rho,x,z}.bin and
 * inversion_misfit.txt to [path] output.  SH or PSV alone. */
int seiswg_solver_run_inversion(seiswg_solver* s, const seiswg_vfs* vfs, seiswg_vfs* out);
int seiswg_solver_info(const seiswg_solver* s, int32_t* nx, int32_t* nz, float* dx, float* dz, int32_t* nsrc,
                       int32_t* nrec);
/* Total waveform misfit of the last run_adjoint (solver.rs:1503). */
double seiswg_solver_total_misfit(const seiswg_solver* s);
/* The simulation handle the solver drives (borrowed; owned by the solver). */
struct seiswg_sim* seiswg_solver_sim(seiswg_solver* s);
void seiswg_solver_free(seiswg_solver* s);

/* ---- simulation operator (the kernel-level interface) -------------------- */
typedef struct seiswg_sim seiswg_sim;
typedef struct {
  int32_t nx, nz, nt;
  float dx, dz, dt;
  int32_t sh, psv, spin;
  int32_t abs_left, abs_right, abs_bottom, abs_top;
  int32_t abs_width;
  float abs_alpha;
} seiswg_sim_desc;

/* stream: a cudaStream_t to run on, or NULL for a stream of the handle's own. */
int seiswg_sim_create(const seiswg_sim_desc* desc, void* stream, seiswg_sim** out);
void seiswg_sim_free(seiswg_sim* sim);
/* Model fields, n = nx*nz values: "vp", "vs", "rho" (converted to Lame
 * parameters by seiswg_sim_prepare, fd2d.wgsl:188-201) or "lambda", "mu",
 * "nu", "j", "lambda_c", "mu_c", "nu_c", "rho" for spin models. */
int seiswg_sim_upload_model(seiswg_sim* sim, const char* name, const float* host, size_t n);
/* vps2lm, mu_c+nu_c and the absorbing taper (fd2d.wgsl:188-235).  Also
 * checks stability before any run (the reference has no such check): fails
 * with SEISWG_EINVAL when dt c (7/6) sqrt(1/dx^2 + 1/dz^2) > 1 (c the
 * largest P speed with PSV, S speed with SH alone), when with spin (dt/2)
 * sqrt(4 nu/J + (mu_c+nu_c)/J (7/3)^2 (1/dx^2 + 1/dz^2)) > 1, or when a
 * squared wave speed is negative or not finite.  Option "stability_check" 0
 * (set before this call) turns the rejection off. */
int seiswg_sim_prepare(seiswg_sim* sim);
/* The two stability numbers of the last seiswg_sim_prepare (spin: 0 without
 * spin); a run is rejected above 1. */
int seiswg_sim_stability(const seiswg_sim* sim, double* wave, double* spin);
/* Sources at cells (i[s], j[s]); stf_xyz is [3][n][nt] (x, y, z components). */
int seiswg_sim_set_sources(seiswg_sim* sim, int32_t n, const int32_t* i, const int32_t* j, const float* stf_xyz);
int seiswg_sim_set_receivers(seiswg_sim* sim, int32_t n, const int32_t* i, const int32_t* j);
/* One forward run from rest: all nt steps of source isrc (-1: all sources).
 * Snapshots of `nfields` fields ("vy", "vx", "vz", "vyc", "sxy", ...) after
 * every step it > 0 with it % snap_every == 0 go to snaps_out
 * [nsnap][nfields][nx*nz] (snap_every = 0: none).  sync = 0 returns once
 * the run is queued on the stream (only without snapshots). */
int seiswg_sim_forward(seiswg_sim* sim, int32_t isrc, int32_t snap_every, int32_t nfields,
                       const char* const* fields, float* snaps_out, int32_t sync);
/* Receiver traces of the last run, [5][nrec][nt]: x, y, z, yi, yc
 * (the reference's obs buffer, fd2d.wgsl:110-114).  Fails with
 * SEISWG_ENUMERIC when they hold NaN or infinite values, and with
 * SEISWG_ETIMEOUT when a kernel of the run gave up a bounded wait. */
int seiswg_sim_traces(seiswg_sim* sim, float* host);
/* Current wavefield component, nx*nz values. */
int seiswg_sim_state(seiswg_sim* sim, const char* field, float* host);
/* Reference adjoint, one shot at a time (solver.rs:1380-1498). */
int seiswg_sim_kernel_clear(seiswg_sim* sim);
int seiswg_sim_adjoint_forward(seiswg_sim* sim, int32_t isrc, int32_t adj_interval);
int seiswg_sim_adjoint_backward(seiswg_sim* sim, const float* adstf, int32_t adj_interval);
int seiswg_sim_kernel_smooth(seiswg_sim* sim, float sigma);
int seiswg_sim_kernel(seiswg_sim* sim, float* host);
/* Exact discrete adjoint (no counterpart in the reference, which has only the
 * SH imaging condition above, solver.rs:1386-1498).  The pair
 * behaves like an autograd function: forward_op runs source isrc (-1: all)
 * and stores the wavefield every ckpt_every steps (0: the scheme of the
 * "checkpoint_slots" option below); the
 * traces are then available through seiswg_sim_traces.  backward_op takes
 * dJ/dd of the recorded displacement traces, [ncomp][nrec][nt] with ncomp 1
 * (SH: uy) or 2 (PSV: ux, uz), and accumulates the gradients of J with
 * respect to lambda, mu and the buoyancy 1/rho, recomputing the forward
 * states of each checkpoint interval.  SH or PSV, not spin. */
int seiswg_sim_gradient_clear(seiswg_sim* sim);
int seiswg_sim_forward_op(seiswg_sim* sim, int32_t isrc, int32_t ckpt_every);
int seiswg_sim_backward_op(seiswg_sim* sim, const float* adj);
/* The checkpoint interval of the last forward_op (0 before the first, and
 * under binomial checkpointing). */
int32_t seiswg_sim_checkpoint_interval(const seiswg_sim* sim);
/* The checkpoint plan of the last forward_op: binomial checkpointing slots
 * (0: uniform checkpoints every `interval` steps), the forward steps the
 * reverse sweep recomputes, and the device bytes the checkpoints hold.
 * Binomial checkpointing (Griewank and Walther's revolve schedule; the
 * reference has no checkpointing: it keeps the forward wavefield every
 * adj_interval steps in host memory, solver.rs:1384, 1411-1414) stores S
 * states and recomputes the fewest steps any schedule with S states can:
 * F(nt, S-1) - (nt - 1) with F(n, s) = r n - C(s+1+r, r-1), r the least
 * integer with C(s+1+r, r) >= n. */
int seiswg_sim_checkpoint_plan(const seiswg_sim* sim, int32_t* slots, int32_t* interval, int64_t* recomputed,
                               size_t* bytes);
/* The misfit and adjoint source on the device (the host misfit of
 * solver.rs:432-467 without the trace download and the adjoint-source
 * upload).  set_observed copies the observed traces, [ncomp][nrec][nt] in the
 * components of backward_op; misfit_op, after forward_op, returns the L2
 * waveform misfit J (seiswg_l2_misfit's taper and formula) and keeps its
 * adjoint source on the device; backward_op_device runs the reverse sweep
 * with it. */
int seiswg_sim_set_observed(seiswg_sim* sim, const float* obs);
int seiswg_sim_misfit_op(seiswg_sim* sim, double* J);
int seiswg_sim_backward_op_device(seiswg_sim* sim);
/* param: "lambda", "mu" or "buoyancy"; nx*nz values.  Fails with
 * SEISWG_ENUMERIC when the gradients hold NaN or infinite values. */
int seiswg_sim_gradient(seiswg_sim* sim, const char* param, float* host);
/* Frees the checkpoint, adjoint and snapshot buffers until their next use
 * (gradients are kept). */
int seiswg_sim_release_workspace(seiswg_sim* sim);
/* Options: "graphs" (0/1), "chunk_rows" (rows per warp march; 0: the
 * occupancy model), "loader" (0: plain loads, 1: TMA bulk-copy row pipeline,
 * the default), "autotune" (value = steps timed per candidate: picks the
 * fastest loader and chunk rows for this problem), "two_step" (0/1: forward
 * runs advance two time steps per launch; PSV alone (no SH, no spin) or SH
 * alone, and on by default there; multiply-add contraction, so results
 * match the one-step kernel to rounding), "two_step_rows" (rows per march of
 * the two-step kernel; 0: its occupancy model), "two_step_producer" (0/1,
 * default 1: PSV two-step launches with tensor copies take their rows from
 * producer warps, one per march, instead of each march issuing its own
 * copies; the same results), "reverse_producer" (0/1, default 1: the same
 * for the PSV reverse step), "cluster" (0/1: SH grids
 * whose state and material fit one thread-block cluster's shared memory run
 * each forward pass in one launch with the wavefield on chip; default on;
 * results are the one-step kernel's bits), "tma" (0/1: the two-step and the
 * PSV reverse kernels fetch their rows with 3-D tensor copies where the
 * fields lie at uniform strides, default on; 0: one bulk copy per field;
 * the same results either way), "checkpoint_slots" (forward_op with
 * ckpt_every = 0 uses binomial checkpointing with this many stored states,
 * 1 or more; 0, the default: every state kept where the budget below holds
 * nt + 1 states (no recomputation; two-step launches store the state between
 * their steps), else uniform checkpoints every second step, else every
 * ceil(sqrt(nt)) steps, else binomial checkpointing with as many states as
 * fit), "checkpoint_budget_mb" (the memory that default choice may give to
 * checkpoints; 0: the free HBM less a tenth of the device's memory, at
 * least 2 GiB, kept in reserve), "stability_check" (0/1, default 1: see
 * seiswg_sim_prepare), "pdl" (0/1, default 1: step and reverse launches may
 * start while the previous launch in the stream finishes -- programmatic
 * dependent launch; the same results), "wait_polls" (polls of a kernel's bounded wait for
 * its row pipeline before it gives up and the run fails with
 * SEISWG_ETIMEOUT; 0: the built-in 2^20), "test_arm_extra" (a test hook for
 * that failure path: bytes armed on the first stage of every warp's row
 * pipeline beyond its copies, so that every launch's first wait runs out
 * while all copies still land; 0, the default, for real runs). */
int seiswg_sim_set_option(seiswg_sim* sim, const char* key, int64_t value);
int seiswg_sim_synchronize(seiswg_sim* sim);
/* Number of kernels this handle has launched (graph nodes count per replay). */
uint64_t seiswg_sim_launches(const seiswg_sim* sim);
void* seiswg_sim_stream(const seiswg_sim* sim);
size_t seiswg_sim_device_bytes(const seiswg_sim* sim);

/* ---- batched gradients of many problems ------------------------------------
 * No counterpart in the reference (its shots run one after another,
 * solver.rs:1372).  Each problem is a prepared seiswg_sim (SH or PSV, sources
 * = its shots, receivers set) with observed traces obs[p] laid out
 * [nshot][ncomp][nrec][nt].  seiswg_batch_run computes, for every shot of
 * every problem at once, the recording forward pass with checkpoints every
 * ckpt_every steps (0: ceil(sqrt(nt)) per shot), the L2 misfit and adjoint
 * source on the device (as seiswg_l2_misfit), the reverse sweep, and the
 * gradients summed per problem.  Problems must outlive the batch and must not
 * run other work meanwhile.  The first run captures the schedule as a CUDA
 * graph; later runs replay it. */
typedef struct seiswg_batch seiswg_batch;
int seiswg_batch_create(seiswg_sim* const* sims, const float* const* obs, int32_t nproblems, int32_t ckpt_every,
                        void* stream, seiswg_batch** out);
int seiswg_batch_run(seiswg_batch* batch);
/* key "chunk_rows": rows per warp chunk of every job (0: each problem's own
 * chunk model); "two_step" (0/1): jobs whose problem runs two steps per
 * launch (PSV alone, SH alone) record their forward pass that way (default
 * 1); "reverse_producer" (0/1, default 0): grouped PSV reverse launches
 * take their rows from producer warps (every job by tensor copies; the same
 * results); "two_step_recompute" (0/1, default 1): such jobs also recompute the
 * states of each checkpoint interval two steps per grouped launch, each
 * launch storing both states (launch order 3 recomputes one step per
 * operation); "autotune": tries
 * chunk rows 0, 16 (not in order 3), 32, 48, 64, 96 and 128 with and without two-step
 * recording, timing `value` slots of the recording pass and of the reverse
 * sweep each, and keeps the one whose times, scaled to the slot counts of
 * the two phases, are the shortest (in order 3, the queue's units of those
 * slots); "concurrent": how the schedule runs -- as grouped launches (one
 * per schedule slot and kind of work: SH/PSV forward, reverse, misfit), 0
 * one after another, 1 a slot's launches on forked streams that join before
 * the next slot, 2 (default) one stream per kind, a launch waiting only for
 * the previous slot's launches of the kinds its jobs come from; or 3 as one
 * persistent launch whose warps work through a device queue of every
 * job's units (one warp's march over one strip and chunk of one operation),
 * each unit waiting only for the chunks its rows reach of its job's previous
 * operation; "queue_wait_us" (order 3, default 2 s): the bound of one such
 * wait, after which the run fails with SEISWG_ETIMEOUT; "queue_band" (order
 * 3, default 0): the queue's units slot after slot (0), or in bands of that
 * many slots within which each job's units run diagonally across its
 * operations and chunks, so that an operation reads the rows the previous
 * one wrote while they are still in L2;
 * "test_queue_need_extra" (a test hook, default 0): added to every such
 * dependency after a job's first operation, so that those waits run out;
 * "stream_groups" (1..4, default 1): jobs split round-robin into
 * groups with their own launches (and streams in order 2); "tma" (0/1,
 * default 1): the grouped two-step forward and PSV reverse launches fetch
 * rows with 3-D tensor copies through each job's table of tensor maps, or
 * with one bulk copy per field (the same bits); "pdl" (0/1, default 1): the
 * grouped forward and reverse launches may start while the previous launch
 * of their stream finishes (programmatic dependent launch: a launch's CTAs
 * set up their row pipelines on the SMs the previous launch leaves and wait
 * for it before their first read; the same bits); "checkpoint_slots" (S >= 1:
 * every job keeps S + 2 states and follows the binomial checkpointing
 * schedule of seiswg_sim_checkpoint_plan; 0: back to the uniform checkpoints
 * of seiswg_batch_create), which reallocates the jobs' state pools.  Each
 * drops the captured graph. */
int seiswg_batch_set_option(seiswg_batch* batch, const char* key, int64_t value);
/* The binomial checkpointing slots per job (0: uniform checkpoints) and the
 * forward steps the reverse sweeps of all jobs recompute in one run. */
int seiswg_batch_checkpoint_plan(const seiswg_batch* batch, int32_t* slots, int64_t* recomputed);
/* The chunk rows in use (0: each problem's own chunk model), and whether
 * jobs record two steps per launch. */
int32_t seiswg_batch_chunk_rows(const seiswg_batch* batch);
int32_t seiswg_batch_two_step(const seiswg_batch* batch);
/* The launch order in use ("concurrent": 0 to 3) and the job groups. */
int32_t seiswg_batch_concurrent(const seiswg_batch* batch);
int32_t seiswg_batch_stream_groups(const seiswg_batch* batch);
/* Launch order 3: the units in the device queue and the CTAs of the
 * persistent launch (0 and 0 in the other orders), and the "queue_band"
 * option. */
int seiswg_batch_queue(const seiswg_batch* batch, int64_t* units, int32_t* blocks, int32_t* band);
/* Jobs whose grouped launches fetch rows by tensor copies (0 with "tma" 0). */
int32_t seiswg_batch_tma_jobs(const seiswg_batch* batch);
/* param: "lambda", "mu" or "buoyancy"; nx*nz values of the problem. */
int seiswg_batch_gradient(seiswg_batch* batch, int32_t problem, const char* param, float* host);
double seiswg_batch_misfit(const seiswg_batch* batch, int32_t problem);
int seiswg_batch_info(const seiswg_batch* batch, int32_t* jobs, int32_t* slots, uint64_t* launches_per_run,
                      size_t* device_bytes);
void* seiswg_batch_stream(const seiswg_batch* batch);
void seiswg_batch_free(seiswg_batch* batch);

/* ---- smoothing without device allocation ----------------------------------
 * No counterpart in the reference.  Smooths an nx*nz float field
 * (k = i*nz + j) from `in` into `out` -- device buffers the caller owns,
 * which must not overlap -- with the Gaussian of seiswg_sim_kernel_smooth
 * (sigma in cells), on `stream` (NULL: the default stream).  It is for
 * callers that cannot call cudaMalloc: hosts whose device memory all belongs
 * to their own pool allocator, or code where an allocation (which may
 * synchronise the device) is not allowed.  It allocates nothing; its scratch
 * is a fixed array in the library's device image (16 MiB + 112 KiB, held on
 * every GPU that loads the library until the process exits), which limits the
 * grid to 4,194,304 cells and 6144 per axis, and sigma to 511; larger
 * requests fail with SEISWG_EINVAL.  The first call on a device looks up the
 * scratch address for that device; make that first call before any stream
 * capture.  All calls on a device share the scratch, so calls that may
 * overlap on the GPU (other streams, other threads) race and must be
 * serialised by the caller.  Every scratch value a call reads is written
 * earlier in the same call, so nothing carries over from the previous one.
 * Returns once the work is queued. */
int seiswg_smooth_noalloc(const float* in, float* out, int32_t nx, int32_t nz, float sigma, void* stream);

/* ---- host-side numerics of the reference ---------------------------------- */
/* [3][nt] Ricker STF of one source (solver.rs:350-356, 721-733). */
int seiswg_ricker(int32_t nt, float dt, float f0, float t0, float ang_deg, float amp, float* out);
/* Misfit and time-reversed adjoint source (solver.rs:432-467). */
int seiswg_waveform_misfit(const float* syn, const float* obs, int32_t nrec, int32_t nt, float dt, float* adstf,
                           double* misfit);
/* .npy v1 bytes of a [nrows][ncols] f32 array (solver.rs:270-285).  With
 * out == NULL only *len is set. */
int seiswg_npy_encode(const float* data, size_t nrows, size_t ncols, void* out, size_t* len);
/* J = sum (taper * (syn - obs))^2 over ntr traces of nt samples, with the
 * misfit taper of solver.rs:442-459, and adj = dJ/dsyn (not time-reversed;
 * the reference's adjoint source is adj reversed in time). */
int seiswg_l2_misfit(const float* syn, const float* obs, int32_t ntr, int32_t nt, float dt, float* adj, double* J);
/* Chain rule from (lambda, mu, buoyancy) gradients to (vp, vs, rho) for
 * lambda = rho (vp^2 - 2 vs^2) (0 where vp <= vs), mu = rho vs^2. */
int seiswg_velocity_gradients(const float* g_lam, const float* g_mu, const float* g_b, const float* vp,
                              const float* vs, const float* rho, size_t n, float* g_vp, float* g_vs, float* g_rho);
/* nx, nz, dx, dz from coordinate arrays: the reference's aspect-ratio rule
 * (solver.rs:646-656) where it yields a grid consistent with the coordinate
 * layout (square cells); otherwise, for rectangular cells (dx != dz), the grid
 * read from the layout k = i*nz + j (nz = the first run of equal x). */
int seiswg_infer_grid(const float* x, const float* z, size_t npt, int32_t* nx, int32_t* nz, float* dx, float* dz);

#ifdef __cplusplus
}
#endif

#endif /* SEISWG_H */
