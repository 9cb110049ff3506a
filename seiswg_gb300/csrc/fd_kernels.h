// fd_kernels.h -- launch interface of the seiswg sm_103a kernels (device
// pointers only; the engine owns the memory).
#pragma once

#include <cstddef>
#include <cuda.h>
#include <cuda_runtime.h>

#include "fd_types.h"

namespace seiswg {

constexpr int kStepWarps = 4;  // warps per CTA of the step kernels

struct InjectList {
  const Inject* list;  // sorted by (i, j), stable
  int n;
  int nt, it;
  const float* val_x;  // [rows][nt] value tables (may be null when unused)
  const float* val_y;
  const float* val_z;
};

struct ProbeList {
  const Probe* list;  // sorted by (i, j)
  int n;
  int nt, it;
  float* acc;   // [n] running displacement
  float* hist;  // [n][nt] displacement after each step
};

struct ShStep {
  Geom g;
  const float *vy0, *sxy0, *szy0;
  float *vy1, *sxy1, *szy1;
  float *vym, *sxym, *szym;  // two-step kernels: the state after the first step (null: not stored)
  const float *rho, *mu;
  const float *taper_x, *taper_zb, *taper_zt;
  InjectList inj;
  ProbeList probes;
  int* err;  // device error word (kErr* bits)
};

struct PsvStep {
  Geom g;
  const float *vx0, *vz0, *sxx0, *szz0, *sxz0;
  float *vx1, *vz1, *sxx1, *szz1, *sxz1;
  float *vxm, *vzm, *sxxm, *szzm, *sxzm;  // two-step kernels: the state after the first step (null: not stored)
  const float *vyc0, *syx0, *syy0, *syz0;
  float *vyc1, *syx1, *syy1, *syz1;
  const float *rho, *lam, *mu;
  const float *nu, *jm, *mc;  // spin: nu, J, mu_c + nu_c
  const float *taper_x, *taper_zb, *taper_zt;
  InjectList inj;
  ProbeList probes;
  int* err;
};

// Dynamic shared memory of one step CTA for a loader (0 for direct loads).
size_t step_smem_bytes(bool psv, bool spin, int loader);
// Resident CTAs per SM of the step kernel for a loader (occupancy query).
int step_blocks_per_sm(bool psv, bool spin, int loader);
cudaError_t launch_sh_step(const ShStep& p, cudaStream_t s);
cudaError_t launch_psv_step(const PsvStep& p, bool spin, cudaStream_t s);
// PSV + spin one-step kernel (fd_spin.cu), reached through the three above.
size_t spin_step_smem_bytes(int loader);
int spin_step_blocks_per_sm(int loader);
cudaError_t launch_psv_spin_step(const PsvStep& p, cudaStream_t s);
// Whole forward runs of small SH grids in one thread-block cluster
// (fd_cluster.cu).  State *0 is read at the start and *1 written at the end
// (they may alias); vy snapshots go to snap + q * snap_stride (padded fields)
// for q = snap_first, ... at every step it > 0 with it % snap_every == 0.
constexpr int kClusterThreads = 1024;
constexpr int kClusterSources = 64;    // injections per run the cluster kernel takes
constexpr int kClusterProbes = 4096;   // probes per run the cluster kernel takes
struct ShCluster {
  int nx, nz, ld, rows;  // rows per CTA
  int it0, it1;          // steps [it0, it1)
  float dt, rdx, rdz;
  const float *vy0, *sxy0, *szy0;
  float *vy1, *sxy1, *szy1;
  const float *rho, *mu, *taper_x, *taper_zb, *taper_zt;
  InjectList inj;
  ProbeList probes;
  float* snap;
  int snap_every, snap_first;
  long long snap_stride;
};
// CTAs of the cluster that holds an nx x nz SH grid (8 or 16), 0 when none fits.
int sh_cluster_ctas(int nx, int nz);
size_t sh_cluster_smem_bytes(int nx, int nz, int ctas);
cudaError_t launch_sh_cluster(const ShCluster& p, int ctas, cudaStream_t s);

// Two PSV steps (inj.it and inj.it + 1; no spin) from the *0 state to the *1
// state, and, where p.vxm is not null, the state after step inj.it to the *m
// fields (all five).  p.g describes the two-step decomposition: nstrips over
// kStripCols2-column strips, lx / nchunks its own chunk rows.  The same for
// the SH launchers below with p.vym.
cudaError_t launch_psv_step2(const PsvStep& p, cudaStream_t s);
size_t step2_smem_bytes();
int step2_blocks_per_sm();
// Tensor maps (3-D: columns, rows, fields; 128 x 1 x n boxes) that let the
// two-step PSV kernel fetch a row of several fields in one TMA copy: sigma^n
// (sxx, szz, sxz of a state whose fields vx, vz, sxx, szz, sxz lie at a
// uniform stride), v^n (vx, vz), dt/rho, and dt*lambda, dt*mu (the dt-scaled
// material fields, at a uniform stride).  Encoded on the host.
//
// The two-step kernels (plain and grouped) read the material scaled by dt:
// PsvStep/ShStep rho, lam, mu hold dt/rho, dt*lambda, dt*mu for them.
struct Tma2 {
  CUtensorMap sig, vel, rho, lm;
};
cudaError_t launch_psv_step2_tma(const PsvStep& p, const Tma2& t, cudaStream_t s);
// The same launch with every row copy issued by a producer warpgroup
// (fd_step2pc.cu): eight marches of p.g per CTA; bitwise the results of
// launch_psv_step2_tma.
cudaError_t launch_psv_step2_pc(const PsvStep& p, const Tma2& t, cudaStream_t s);
// Tensor maps of the PSV reverse step: the forward state (vx, vz, sxx, szz,
// sxz) with boxes of 1 and 2 fields, the incoming adjoint state (same field
// order) with boxes of 3 and 2, the material (1/rho, lambda, mu) with boxes of
// 1 and 2, and the gradients (lambda, mu, buoyancy) with boxes of 1 and 2.
struct TmaAdj {
  CUtensorMap f1, f2, a3, a2, m1, m2, g1, g2;
};
// The same maps as pointers into a table in device memory (grouped launches).
struct Tma2Ptrs {
  const CUtensorMap *sig, *vel, *rho, *lm;
};
struct TmaAdjPtrs {
  const CUtensorMap *f1, *f2, *a3, *a2, *m1, *m2, *g1, *g2;
};
// SH: sig = state fields vy, sxy, szy with boxes of 2 (sxy, szy), vel = the
// same with boxes of 1 (vy), rho = material fields with boxes of 1 (1/rho,
// and mu at field 2); lm unused.
cudaError_t launch_sh_step2_tma(const ShStep& p, const Tma2& t, cudaStream_t s);
// Two SH time steps per launch (fd_step2.cu), same decomposition as the PSV one.
cudaError_t launch_sh_step2(const ShStep& p, cudaStream_t s);
int sh_step2_blocks_per_sm();

// ---- exact discrete adjoint (fd_adjoint.cu) --------------------------------
struct PsvAdjoint {
  Geom g;
  const float *vx, *vz, *sxx, *szz, *sxz;       // forward state S^n
  const float *wx0, *wz0, *bxx0, *bzz0, *bxz0;  // adjoint state after step n
  float *wx1, *wz1, *bxx1, *bzz1, *bxz1;        // adjoint state before step n
  const float *rho, *lam, *mu;                  // 1/rho, lambda, mu
  const float *taper_x, *taper_zb, *taper_zt;
  float *g_b, *g_lam, *g_mu;                    // gradient accumulators (buoyancy, lambda, mu)
  InjectList src;                               // forward sources of step n (val_x, val_z)
  InjectList rec;                               // dt * U at the receivers (val_x, val_z)
  int* err;
};

struct ShAdjoint {
  Geom g;
  const float *vy, *sxy, *szy;
  const float *w0, *bxy0, *bzy0;
  float *w1, *bxy1, *bzy1;
  const float *rho, *mu;
  const float *taper_x, *taper_zb, *taper_zt;
  float *g_b, *g_mu;
  InjectList src;  // val_y
  InjectList rec;  // val_y
  int* err;
};

// Resident CTAs per SM of the reverse-step kernel for a loader (occupancy query).
int adjoint_blocks_per_sm(bool psv, int loader);
cudaError_t launch_psv_adjoint(const PsvAdjoint& p, cudaStream_t s);
cudaError_t launch_psv_adjoint_tma(const PsvAdjoint& p, const TmaAdj& t, cudaStream_t s);
// The same reverse step with every row copy issued by producer warps
// (fd_adjointpc.cu): eight marches of p.g per CTA; bitwise the results of
// launch_psv_adjoint_tma.
cudaError_t launch_psv_adjoint_pc(const PsvAdjoint& p, const TmaAdj& t, cudaStream_t s);
cudaError_t launch_sh_adjoint(const ShAdjoint& p, cudaStream_t s);

// ---- grouped launches over many independent jobs (fd_step.cu, fd_adjoint.cu,
// fd_batch.cu) ---------------------------------------------------------------
// A job is one shot of one problem, with its own wavefield storage: a pool of
// state slots (checkpoints, interval buffer, forward ping-pong), two adjoint
// slots, gradient accumulators, probe histories and adjoint-source tables.
// Field f of slot s starts at pool + s*slot_elems + f*field_elems + halo;
// fields in a slot: SH vy, sxy, szy; PSV vx, vz, sxx, szz, sxz.
struct JobDesc {
  Geom g;
  Geom g2;                 // two-step decomposition (PSV; lx 0: one step per launch)
  int psv;                 // 1 PSV, 0 SH
  int nstate;
  long long field_elems, slot_elems, halo;
  float* pool;
  float* adj;              // 2 adjoint slots
  const float *rho, *lam, *mu;
  const float *rho_dt;     // dt/rho, dt*lambda, dt*mu at the material's stride (two-step kernels)
  const float *taper_x, *taper_zb, *taper_zt;
  float *g_b, *g_lam, *g_mu;
  InjectList src;          // the shot's source
  ProbeList probes;        // receiver probes of this physics, with the job's acc/hist
  InjectList rec;          // receivers, val = u_tab components
  const int* tr_idx;       // [nrec][12] probe indices per receiver
  const float* obs;        // observed traces [ncomp][nrec][nt]
  float* u_tab;            // dt * U, [ncomp][nrec][nt]
  double* J;               // per-trace misfit [ncomp][nrec]
  int nrec, nt;
  float dt;
  int* err;
  // Tensor maps of the job (nullptr: bulk copies): for pool slot s, maps of
  // its state fields with boxes of 1, 2 and 3 fields at tm[3 s + 0..2]; then,
  // from tm[3 tm_nslot]: adjoint slot 0 (boxes of 3 and 2), adjoint slot 1
  // (3, 2), the material (1, 2), the gradient block (1, 2) and the dt-scaled
  // material (1, 2).
  const CUtensorMap* tm;
  int tm_nslot;
  // The device work queue (launch order 3 of the batch): the job's
  // operations, its counters of finished units (one per chunk) and how many
  // chunks to each side a unit's rows reach.
  const QueueOp* qops;
  int* qcnt;
  int qreach;
};
constexpr int kJobTmaTail = 10;  // maps after the slots' in a job's table

// One operation of one job in a grouped launch.  Forward: step `it` from slot
// a to slot b (flags & 1: record the probes).  Adjoint: reverse step `it` with
// the forward state in slot a and the adjoint state in slot (b & 1), writing
// slot 1 - (b & 1).  Misfit: traces -> adjoint-source tables and J.  Warps
// [warp_begin, warp_begin + nstrips*nchunks) of the launch belong to the op.
struct GroupOp {
  int job, it, a, b, flags, warp_begin;
};

#ifdef __CUDACC__
// The op of warp gw in a grouped launch: the last op with warp_begin <= gw
// (ops sorted by warp_begin, ops[0].warp_begin == 0).  The warp reads the
// begins of 32 ops per step, up to four steps' loads in flight together, and
// votes, instead of a binary search's chain of dependent loads.  gw is
// uniform over the warp and all lanes are active.
__device__ __forceinline__ int group_op_of(const GroupOp* __restrict__ ops, int nops, int gw) {
  const int lane = threadIdx.x & 31;
  int found = 0;
  for (int base = 0; base < nops; base += 128) {
    bool le[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int q = base + 32 * u + lane;
      le[u] = q < nops && __ldg(&ops[q].warp_begin) <= gw;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const unsigned m = __ballot_sync(0xffffffffu, le[u]);
      if (m == 0u) return found;
      found = base + 32 * u + 31 - __clz(int(m));
    }
  }
  return found;
}
#endif

cudaError_t launch_grouped_forward(const JobDesc* jobs, const GroupOp* ops, int nops, int warps, bool psv,
                                   bool pdl, cudaStream_t s);
cudaError_t launch_grouped_adjoint(const JobDesc* jobs, const GroupOp* ops, int nops, int warps, bool psv,
                                   bool pdl, cudaStream_t s);
// The grouped PSV reverse launch with every row copy issued by producer
// warps (fd_adjointpc.cu); every job of the launch needs its map table.
cudaError_t launch_grouped_adjoint_pc(const JobDesc* jobs, const GroupOp* ops, int nops, int warps, bool pdl,
                                      cudaStream_t s);
// Two PSV (psv) or SH steps (op.it, op.it + 1) of every op's job, with the
// jobs' g2.
cudaError_t launch_grouped_forward2(const JobDesc* jobs, const GroupOp* ops, int nops, int warps, bool psv,
                                    bool pdl, cudaStream_t s);
// Misfit of one problem's assembled traces against obs [ncomp][nrec][nt];
// writes J per trace and the adjoint-source table dt * U.
cudaError_t launch_sim_misfit(const float* syn, const float* obs, float* u_tab, double* J, int nrec, int nt,
                              bool psv, float dt, cudaStream_t s);
cudaError_t launch_grouped_misfit(const JobDesc* jobs, const GroupOp* ops, int nops, cudaStream_t s);

// The batch's persistent queue kernel (fd_queue.cu): `blocks` CTAs whose
// warps claim units units[*next], units[*next + 1], ... below `end` in order
// (*next and the jobs' counters are set by the caller), wait for each unit's
// dependencies -- bounded by wait_ns nanoseconds, after which the error word
// gets kErrWaitTimeout and the warp leaves -- and run its march.  `tma`:
// two-step and PSV reverse units fetch rows by tensor copies (every job has
// a map table), else by bulk copies.  need_extra (a test hook, 0 normally)
// is added to every dependency after a job's first operation, so that those
// waits run out.
cudaError_t launch_batch_queue(const JobDesc* jobs, const QueueUnit* units, long long end, unsigned long long* next,
                               int* err, bool tma, unsigned long long wait_ns, int need_extra, int blocks,
                               cudaStream_t s);
// CTAs of the queue kernel resident per SM (its grid is that times the SMs).
int batch_queue_blocks_per_sm(bool tma);

// ---- auxiliary kernels (fd_aux.cu) ----------------------------------------

// Pitched field helpers.  `f` points at element (0, 0).
cudaError_t launch_fill_rows(float* f, int rows_lo, int rows_hi, int ld, float value, cudaStream_t s);
// vps2lm (fd2d.wgsl:188-201), in place on the vp / vs slots.
cudaError_t launch_vps2lm(float* lam_vp, float* mu_vs, const float* rho, int nx, int nz, int ld, cudaStream_t s);
// out = a + b elementwise over the nx x nz interior.
cudaError_t launch_add_fields(float* out, const float* a, const float* b, int nx, int nz, int ld,
                              cudaStream_t s);
// f = 1/f over the nx x nz interior (buoyancy from density, 1/J).
cudaError_t launch_reciprocal(float* f, int nx, int nz, int ld, cudaStream_t s);
// out = in * factor over n consecutive floats.
cudaError_t launch_scale(float* out, const float* in, long n, float factor, cudaStream_t s);
// Largest squared speeds over the interior (bits of non-negative floats, max
// taken into out[0..2], which the caller zeroes): out[0] (lambda + 2 mu) b
// (psv) or mu b (SH), out[1] 4 nu / J and out[2] (mu_c + nu_c) / J when
// jinv is given (spin; b and jinv hold 1/rho and 1/J); out[3] |= 1 when a
// value is not finite or negative.
cudaError_t launch_max_speeds(const float* lam, const float* mu, const float* b, const float* nu, const float* jinv,
                              const float* mc, bool psv, int nx, int nz, int ld, unsigned* out, cudaStream_t s);
// *err |= bit when an element of rows x cols (row pitch ld floats) is NaN or
// infinite.
cudaError_t launch_check_finite(const float* f, long rows, int cols, long ld, int* err, int bit, cudaStream_t s);

// Receiver traces from probe histories (save_obs_* of fd2d.wgsl:295-301,
// 463-492).  For each receiver r: obs[comp][r][it].
struct TraceSpec {
  int nrec, nt;
  int sh, psv, spin;
  // Probe indices per receiver, [r][12] (-1 when not recorded):
  //   0 uy (SH), 1 ux, 2 uz (PSV), 3 uy_c (spin),
  //   4..7 uz at rows i-1..i+2, 8..11 ux at columns j-1..j+2 (spin curl)
  const int* idx;
  const int* rec_ij; // [r][2]
  int nx, nz;
  float den_x, den_z;
  const float* hist;
  float* obs;        // [5][nrec][nt]
};
cudaError_t launch_assemble_traces(const TraceSpec& t, cudaStream_t s);

// Imaging condition of the reference adjoint (interaction_muy with div_uy and
// div_fw, fd2d.wgsl:501-509, 571-588):
//   kmu += (dx+ vy_adj * dx+ vy_fw + dz+ vy_adj * dz+ vy_fw) * ndt
cudaError_t launch_imaging_muy(float* kmu, const float* vy_adj, const float* vy_fw, int nx, int nz, int ld,
                               float den_x, float den_z, float ndt, cudaStream_t s);

// Separable Gaussian smoothing normalised by gsum (fd2d.wgsl:515-554):
//   tmp = sum_n w[|i-n|] f[n, j];  f = sum_n w[|j-n|] tmp[i, n] / gsum
cudaError_t launch_smooth_x(float* tmp, const float* f, const float* w, int radius, int nx, int nz, int ld,
                            cudaStream_t s);
cudaError_t launch_smooth_z(float* f, const float* tmp, const float* w, int radius, const float* gsum_x,
                            const float* gsum_z, int nx, int nz, int ld, cudaStream_t s);

}  // namespace seiswg
