// fd_adjointpc.cu -- the PSV reverse step with its rows fetched by producer
// warps (fd_producer.cuh): eight marches per CTA, the march
// psv_adjoint_march unchanged, so the results are psv_adjoint_tma_kernel's
// bits.  The ring keeps the self-issuing kernel's shape: kAdjStages stages of
// the nineteen segments of AdjTmaPlan (eleven tensor copies per row), one row
// in flight.  Also the batch's grouped PSV reverse launch.
#include "fd_adjoint_march.cuh"
#include "fd_group.cuh"
#include "fd_producer.cuh"

namespace seiswg {
namespace {

using PcARows = PcRows<PA_NSEG, kAdjStages, 0>;
constexpr size_t kPcASmem = size_t(kPcConsumers) * PcARows::smem_bytes_per_warp();

__global__ void __launch_bounds__(kPcThreads, 1) psv_adjoint_pc_kernel(const __grid_constant__ PsvAdjoint p,
                                                                       const __grid_constant__ TmaAdj t) {
  extern __shared__ __align__(128) unsigned char smem[];
  pc_init<PcARows>(smem);
  const int c = (threadIdx.x >> 5) % kPcConsumers;  // the march this warp runs or feeds
  const int gw = blockIdx.x * kPcConsumers + c;
  unsigned char* slice = smem + size_t(c) * PcARows::smem_bytes_per_warp();
  if (pc_split()) {
    psv_adjoint_march<PcARows, TmaAdj>(p, gw, slice);
  } else if ((threadIdx.x & 31) == 0) {
    const AMarch m = amarch(p.g, gw);
    if (!m.active) return;
    const LaneCols L0 = lane_cols(p.g, m.strip, 0);  // lane 0's columns: the copies' x
    // the march's rows: ib - 1 .. ie + 1 (iteration k reads row ib - 1 + k)
    pc_produce<PcARows, AdjTmaPlan>(&t, slice, L0.c0 + kHaloCols, m.ib - 1 + kHaloRows, m.ie - m.ib + 3, p.g,
                                    p.err);
  }
}

// Grouped reverse steps of a batch (every job's rows by tensor copies, its
// maps in its table): the warp's job and op as in grouped_adjoint_kernel, the
// producer warp decoding the same op for the march it feeds.
__global__ void __launch_bounds__(kPcThreads, 1) grouped_adjoint_pc_kernel(const JobDesc* __restrict__ jobs,
                                                                           const GroupOp* __restrict__ ops,
                                                                           int nops) {
  extern __shared__ __align__(128) unsigned char smem[];
  pc_init<PcARows>(smem);
  const int c = (threadIdx.x >> 5) % kPcConsumers;
  const int gw = blockIdx.x * kPcConsumers + c;
  unsigned char* slice = smem + size_t(c) * PcARows::smem_bytes_per_warp();
  // The split first (every warp of a warpgroup, before any return); each
  // side then decodes its op within its own register budget.
  if (pc_split()) {
    const GroupOp op = ops[group_op_of(ops, nops, gw)];
    const JobDesc& J = jobs[op.job];
    const int lw = gw - op.warp_begin;
    if (lw >= J.g.nstrips * J.g.nchunks) return;
    psv_adjoint_march<PcARows, TmaAdjPtrs>(job_psv_adjoint(J, op.it, op.a, op.b), lw, slice);
  } else {
    // The op search votes over the warp (group_op_of): the whole producer
    // warp runs it, then lane 0 alone issues.
    const GroupOp op = ops[group_op_of(ops, nops, gw)];
    if ((threadIdx.x & 31) != 0) return;
    const JobDesc& J = jobs[op.job];
    const int lw = gw - op.warp_begin;
    if (lw >= J.g.nstrips * J.g.nchunks) return;
    const AMarch m = amarch(J.g, lw);
    if (!m.active) return;
    const LaneCols L0 = lane_cols(J.g, m.strip, 0);
    const TmaAdjPtrs mp = job_adj_maps(J, op.a, op.b);
    pc_produce<PcARows, AdjTmaPlan>(&mp, slice, L0.c0 + kHaloCols, m.ib - 1 + kHaloRows, m.ie - m.ib + 3, J.g,
                                    J.err);
  }
}

}  // namespace

cudaError_t launch_grouped_adjoint_pc(const JobDesc* jobs, const GroupOp* ops, int nops, int warps, bool pdl,
                                      cudaStream_t s) {
  if (nops <= 0 || warps <= 0) return cudaSuccess;
  static const cudaError_t ready = pc_kernel_ready(grouped_adjoint_pc_kernel, kPcASmem);
  if (ready != cudaSuccess) return ready;
  return pc_launch(grouped_adjoint_pc_kernel, pdl, long(warps), kPcASmem, s, jobs, ops, nops);
}

cudaError_t launch_psv_adjoint_pc(const PsvAdjoint& p, const TmaAdj& t, cudaStream_t s) {
  static const cudaError_t ready = pc_kernel_ready(psv_adjoint_pc_kernel, kPcASmem);
  if (ready != cudaSuccess) return ready;
  return pc_launch(psv_adjoint_pc_kernel, p.g.pdl != 0, long(p.g.nstrips) * p.g.nchunks, kPcASmem, s, p, t);
}

}  // namespace seiswg
