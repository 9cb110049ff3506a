// fd_queue.cu -- the batch's whole schedule as one persistent launch over a
// device work queue.
//
// The queue (batch_plan.h, plan_queue) lists every unit of work of every
// job: one warp's march over one (strip, chunk) of one operation -- a one-
// or two-step forward step or a reverse step, SH or PSV -- or a job's misfit.
// A grid of resident CTAs (kStepWarps warps each) works through it: each
// warp claims the next unit with an atomic counter, waits until the job's
// earlier operations have finished on the chunks the unit's rows reach (one
// counter of finished units per job and chunk), runs the unit's march and
// counts it finished.  Small and large jobs, and the recording, recomputing
// and reverse phases of different jobs, so share the GPU without a launch
// per operation; a job's operation t+1 starts on one end of its grid while
// operation t finishes on the other.
//
// Memory ordering.  A unit's march writes its rows with ordinary stores;
// then every lane fences at GPU scope, the warp synchronises and its lanes
// add to the chunk counters with release semantics.  A unit's wait reads the
// counters with acquire loads; after it every lane issues a proxy fence, so
// that the tensor and bulk copies (async proxy) the march issues see what the
// other warps wrote.  Data that other warps of this launch write -- state
// rows read outside the copies, probe accumulators and histories, adjoint
// sources -- are read through L2 (SEISWG_COHERENT_LOADS, fd_common.cuh),
// never through the read-only path.
//
// Shared memory.  Each warp owns one slice of the largest ring any kind of
// march uses (warp_slice, fd_pipe.cuh), whatever kind it runs; after a march
// its lane 0 invalidates the ring's barriers, since the next unit may place
// stage data where they were.
//
// Waits are bounded: a dependency wait gives up after wait_ns nanoseconds
// (globaltimer) or as soon as another warp has set the error word, and a
// march's row-pipeline waits are bounded as in the step kernels.  A warp that
// gives up sets kErrWaitTimeout and leaves; the host reports it.
//
// Built with multiply-add contraction, as the two-step and reverse kernels
// are; the one-step forward march, which the single-problem path builds
// without contraction, therefore rounds differently here (recomputed
// forward states differ from the recorded ones in the last bits).
#define SEISWG_COHERENT_LOADS 1

#include "fd_adjoint_march.cuh"
#include "fd_group.cuh"
#include "fd_misfit.cuh"
#include "fd_step2_march.cuh"
#include "fd_step_march.cuh"

namespace seiswg {
namespace {

using QPsv1 = BulkL<PV_NSEG>;
using QSh1 = BulkL<SH_NSEG>;
using QPsv2T = TmaRows<PsvTmaPlan, 6, 3, Tma2Ptrs>;
using QSh2T = TmaRows<ShTmaPlan, 6, 3, Tma2Ptrs>;
using QAdjT = TmaRows<AdjTmaPlan, kAdjStages, 0, TmaAdjPtrs>;
using QAdjB = ABulk<PA_NSEG>;
using QAdjSh = ABulk<SA_NSEG>;

constexpr size_t cmax(size_t a, size_t b) { return a > b ? a : b; }
constexpr size_t kQueueSlice =
    cmax(cmax(cmax(QPsv1::smem_bytes_per_warp(), QSh1::smem_bytes_per_warp()),
              cmax(Bulk2::smem_bytes_per_warp(), ShBulk2::smem_bytes_per_warp())),
         cmax(cmax(QPsv2T::smem_bytes_per_warp(), QSh2T::smem_bytes_per_warp()),
              cmax(cmax(QAdjT::smem_bytes_per_warp(), QAdjB::smem_bytes_per_warp()), QAdjSh::smem_bytes_per_warp())));
constexpr size_t kQueueSmem = size_t(kStepWarps) * kQueueSlice;

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_add(int* p, int v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Orders this thread's earlier generic-proxy accesses (global and shared)
// before its later async-proxy ones (tensor and bulk copies).
__device__ __forceinline__ void fence_proxy_async_all() { asm volatile("fence.proxy.async;" ::: "memory"); }

__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Invalidates the barriers of a finished march's ring (all its copies have
// landed: every stage was waited for).
template <class L>
__device__ __forceinline__ void inval_ring(unsigned char* slice) {
  __syncwarp();
  if ((threadIdx.x & 31) == 0) {
    float* buf;
    uint64_t* bar;
    slice_ring<L>(slice, buf, bar);
    for (int st = 0; st < L::kStages; ++st) mbar_inval(&bar[st]);
  }
  __syncwarp();
}

// Waits until counters [c0, c1) all show at least `need`: lane l watches
// counters c0 + l, c0 + l + 32, ...  False when wait_ns nanoseconds passed
// without that or the error word is set.
__device__ bool wait_counters(const int* cnt, int c0, int c1, int need, unsigned long long wait_ns,
                              const int* err) {
  const int lane = threadIdx.x & 31;
  unsigned long long t0 = 0;
  unsigned sleep_ns = 32;
  for (int base = c0; base < c1; base += 32) {
    const int c = base + lane;
    for (;;) {
      const bool ok = c >= c1 || ld_acquire(cnt + c) >= need;
      if (__all_sync(kFull, ok)) break;
      const unsigned long long now = global_ns();
      if (t0 == 0) t0 = now;
      const bool give_up = now - t0 > wait_ns || (lane == 0 && ld_relaxed(err) != 0);
      if (__any_sync(kFull, give_up)) return false;
      __nanosleep(sleep_ns);
      if (sleep_ns < 1024) sleep_ns *= 2;
    }
  }
  return true;
}

// The job's misfit by one warp: lane l reduces traces l, l + 32, ...
__device__ void queue_misfit(const JobDesc& J) {
  const int ntr = (J.psv ? 2 : 1) * J.nrec;
  for (int tr = threadIdx.x & 31; tr < ntr; tr += 32) {
    const int c = tr / J.nrec, r = tr - c * J.nrec;
    const int p = J.tr_idx[12 * r + (J.psv ? 1 + c : 0)];
    J.J[tr] = misfit_trace(J.probes.hist + size_t(p) * J.nt, J.obs + size_t(tr) * J.nt, J.u_tab + size_t(tr) * J.nt,
                           J.nt, double(J.dt));
  }
}

// The units of each kind.  The job table is passed as a restrict pointer
// (read-only for the whole launch), so that the march's parameters can be
// reloaded from it instead of being spilled.  Built inline: as calls of
// functions of their own they spilled more (each kind's march runs in a
// kernel that holds every kind, at 255 registers).  False when a bounded
// wait expired.
__device__ __forceinline__ bool unit_psv1(const JobDesc* __restrict__ jobs, int job, const QueueOp op, int unit,
                                          unsigned char* slice) {
  const JobDesc& J = jobs[job];
  if (!psv_march<QPsv1>(job_psv_step(J, op.it, op.a, op.b, op.flags), unit, slice)) return false;
  inval_ring<QPsv1>(slice);
  return true;
}

__device__ __forceinline__ bool unit_sh1(const JobDesc* __restrict__ jobs, int job, const QueueOp op, int unit,
                                         unsigned char* slice) {
  const JobDesc& J = jobs[job];
  if (!sh_march<QSh1>(job_sh_step(J, op.it, op.a, op.b, op.flags), unit, slice)) return false;
  inval_ring<QSh1>(slice);
  return true;
}

template <bool TMA>
__device__ __forceinline__ bool unit_psv2(const JobDesc* __restrict__ jobs, int job, const QueueOp op, int unit,
                                          unsigned char* slice) {
  const JobDesc& J = jobs[job];
  const PsvStep p = job_psv_step2(J, op.it, op.a, op.b, op.flags);
  if constexpr (TMA) {
    const Tma2Ptrs mp = job_psv2_maps(J, op.a);
    if (!psv2_march<QPsv2T, Tma2Ptrs>(p, unit, slice, &mp)) return false;
    inval_ring<QPsv2T>(slice);
  } else {
    if (!psv2_march<Bulk2>(p, unit, slice)) return false;
    inval_ring<Bulk2>(slice);
  }
  return true;
}

template <bool TMA>
__device__ __forceinline__ bool unit_sh2(const JobDesc* __restrict__ jobs, int job, const QueueOp op, int unit,
                                         unsigned char* slice) {
  const JobDesc& J = jobs[job];
  const ShStep p = job_sh_step2(J, op.it, op.a, op.b, op.flags);
  if constexpr (TMA) {
    const Tma2Ptrs mp = job_sh2_maps(J, op.a);
    if (!sh2_march<QSh2T, Tma2Ptrs>(p, unit, slice, &mp)) return false;
    inval_ring<QSh2T>(slice);
  } else {
    if (!sh2_march<ShBulk2>(p, unit, slice)) return false;
    inval_ring<ShBulk2>(slice);
  }
  return true;
}

template <bool TMA>
__device__ __forceinline__ bool unit_adj_psv(const JobDesc* __restrict__ jobs, int job, const QueueOp op, int unit,
                                             unsigned char* slice) {
  const JobDesc& J = jobs[job];
  const PsvAdjoint p = job_psv_adjoint(J, op.it, op.a, op.b);
  if constexpr (TMA) {
    const TmaAdjPtrs mp = job_adj_maps(J, op.a, op.b);
    if (!psv_adjoint_march<QAdjT, TmaAdjPtrs>(p, unit, slice, &mp)) return false;
    inval_ring<QAdjT>(slice);
  } else {
    if (!psv_adjoint_march<QAdjB>(p, unit, slice)) return false;
    inval_ring<QAdjB>(slice);
  }
  return true;
}

__device__ __forceinline__ bool unit_adj_sh(const JobDesc* __restrict__ jobs, int job, const QueueOp op, int unit,
                                            unsigned char* slice) {
  const JobDesc& J = jobs[job];
  if (!sh_adjoint_march<QAdjSh>(job_sh_adjoint(J, op.it, op.a, op.b), unit, slice)) return false;
  inval_ring<QAdjSh>(slice);
  return true;
}

__device__ __forceinline__ bool unit_misfit(const JobDesc* __restrict__ jobs, int job) {
  queue_misfit(jobs[job]);
  return true;
}

template <bool TMA>
__device__ __forceinline__ bool run_unit(const JobDesc* __restrict__ jobs, int job, const QueueOp& op, int unit,
                                         unsigned char* slice) {
  switch (op.kind) {
    case kFwdPsv: return unit_psv1(jobs, job, op, unit, slice);
    case kFwdSh: return unit_sh1(jobs, job, op, unit, slice);
    case kFwd2Psv: return unit_psv2<TMA>(jobs, job, op, unit, slice);
    case kFwd2Sh: return unit_sh2<TMA>(jobs, job, op, unit, slice);
    case kAdjPsv: return unit_adj_psv<TMA>(jobs, job, op, unit, slice);
    case kAdjSh: return unit_adj_sh(jobs, job, op, unit, slice);
    default: return unit_misfit(jobs, job);
  }
}

template <bool TMA>
__global__ void __launch_bounds__(kStepWarps * 32, 2)
    batch_queue_kernel(const JobDesc* __restrict__ jobs, const QueueUnit* __restrict__ units, long long end,
                       unsigned long long* next, int* err, unsigned long long wait_ns, int need_extra) {
  extern __shared__ __align__(128) unsigned char smem[];
  // The warp's current unit, kept in shared memory while its march runs so
  // that the march has the registers to itself.
  __shared__ unsigned long long cur[kStepWarps];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned long long q = 0;
  if (lane == 0) q = atomicAdd(next, 1ull);
  q = __shfl_sync(kFull, q, 0);
  for (;;) {
    if (lane == 0) cur[warp] = q;
    __syncwarp();
    const unsigned long long p = q;
    if (p >= (unsigned long long)end) return;
    // Claim the next unit now: the atomic's latency overlaps this unit.
    // Units are run in the order they are claimed.
    if (lane == 0) q = atomicAdd(next, 1ull);
    {
      const QueueUnit U = units[p];
      const JobDesc& J = jobs[U.job];
      const QueueOp op = J.qops[U.op];
      const int nstrips = (op.kind == kFwd2Psv || op.kind == kFwd2Sh) ? J.g2.nstrips : J.g.nstrips;
      const int chunk = op.kind == kMisfit ? 0 : int(U.unit) / nstrips;
      const int c0 = op.kind == kMisfit ? 0 : max(0, chunk - J.qreach);
      const int c1 = op.kind == kMisfit ? J.g.nchunks : min(J.g.nchunks, chunk + J.qreach + 1);
      if (op.need > 0 && !wait_counters(J.qcnt, c0, c1, op.need + need_extra, wait_ns, err)) {
        if (lane == 0) atomicOr(err, kErrWaitTimeout);
        return;
      }
      __syncwarp();
      fence_proxy_async_all();
      if (!run_unit<TMA>(jobs, U.job, op, U.unit, smem + size_t(warp) * kQueueSlice)) return;
    }
    // Finished: publish the unit's writes, then count it on its chunk (on
    // every chunk, for the misfit).
    __threadfence();
    __syncwarp();
    {
      const QueueUnit U = units[*(volatile unsigned long long*)&cur[warp]];
      const JobDesc& J = jobs[U.job];
      const QueueOp op = J.qops[U.op];
      if (op.kind == kMisfit) {
        for (int c = lane; c < J.g.nchunks; c += 32) red_release_add(J.qcnt + c, 1);
      } else if (lane == 0) {
        const int nstrips = (op.kind == kFwd2Psv || op.kind == kFwd2Sh) ? J.g2.nstrips : J.g.nstrips;
        red_release_add(J.qcnt + int(U.unit) / nstrips, 1);
      }
    }
    q = __shfl_sync(kFull, q, 0);
  }
}

template <bool TMA>
cudaError_t prepare_queue() {
  return cudaFuncSetAttribute(batch_queue_kernel<TMA>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kQueueSmem));
}

}  // namespace

cudaError_t launch_batch_queue(const JobDesc* jobs, const QueueUnit* units, long long end, unsigned long long* next,
                               int* err, bool tma, unsigned long long wait_ns, int need_extra, int blocks,
                               cudaStream_t s) {
  if (end <= 0 || blocks <= 0) return cudaSuccess;
  if (tma) {
    static const cudaError_t attr = prepare_queue<true>();
    if (attr != cudaSuccess) return attr;
    batch_queue_kernel<true><<<blocks, kStepWarps * 32, kQueueSmem, s>>>(jobs, units, end, next, err, wait_ns,
                                                                        need_extra);
  } else {
    static const cudaError_t attr = prepare_queue<false>();
    if (attr != cudaSuccess) return attr;
    batch_queue_kernel<false><<<blocks, kStepWarps * 32, kQueueSmem, s>>>(jobs, units, end, next, err, wait_ns,
                                                                         need_extra);
  }
  return cudaGetLastError();
}

int batch_queue_blocks_per_sm(bool tma) {
  int n = 0;
  cudaError_t e;
  if (tma) {
    e = prepare_queue<true>();
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_queue_kernel<true>, kStepWarps * 32, kQueueSmem);
  } else {
    e = prepare_queue<false>();
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_queue_kernel<false>, kStepWarps * 32, kQueueSmem);
  }
  return e == cudaSuccess ? n : 0;
}

}  // namespace seiswg
