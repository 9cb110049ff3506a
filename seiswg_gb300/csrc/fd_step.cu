// fd_step.cu -- fused one-step kernels for the SH and PSV systems (PSV +
// spin: fd_spin.cu).
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
// A warp marches down x over its chunk of rows.  Iteration k handles
// velocity row i = ib-1+k (stress rows i-2..i+1 in a register ring) and
// stress row r = i-2 (new velocity rows r-1..r+2 in a register ring).  Row
// data arrive through a loader (fd_pipe.cuh): plain loads, or a shared-memory
// ring fed by the TMA bulk-copy engine a few rows ahead.
//
// State is ping-ponged between two buffers (read step n, write step n+1):
// a warp recomputes the velocity of its halo rows/columns from step-n data
// that its neighbours would otherwise be overwriting in place.
//
// Arithmetic follows the reference's expressions operation for operation
// (built with -fmad=false), except that divisions by 8*dx, rho and J are
// multiplies by precomputed reciprocals; results track the FP32 reference to
// rounding (relative L2 ~1e-7 over thousands of steps).
#include "fd_group.cuh"
#include "fd_step_march.cuh"

namespace seiswg {

template <class Loader>
__global__ void __launch_bounds__(kStepWarps * 32) sh_step_kernel(const ShStep p) {
  extern __shared__ __align__(128) unsigned char smem[];
  sh_march<Loader>(p, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), warp_slice<Loader>(smem));
}

template <class Loader>
__global__ void __launch_bounds__(kStepWarps * 32) psv_step_kernel(const PsvStep p) {
  extern __shared__ __align__(128) unsigned char smem[];
  psv_march<Loader>(p, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), warp_slice<Loader>(smem));
}


// --------------------------------------------------------------------------
// Launchers
// --------------------------------------------------------------------------
namespace {
template <class L>
cudaError_t launch_sh(const ShStep& p, cudaStream_t s) {
  const size_t smem = smem_for<L>();
  static const cudaError_t attr = prepare_kernel(sh_step_kernel<L>, smem);
  if (attr != cudaSuccess) return attr;
  return launch_step(sh_step_kernel<L>, p.g.pdl != 0, blocks_for(p.g), smem, s, p);
}

template <class L>
cudaError_t launch_psv(const PsvStep& p, cudaStream_t s) {
  const size_t smem = smem_for<L>();
  static const cudaError_t attr = prepare_kernel(psv_step_kernel<L>, smem);
  if (attr != cudaSuccess) return attr;
  return launch_step(psv_step_kernel<L>, p.g.pdl != 0, blocks_for(p.g), smem, s, p);
}

}  // namespace

// ---- grouped forward steps ----------------------------------------------------

template <bool PSV>
__global__ void __launch_bounds__(kStepWarps * 32) grouped_forward_kernel(const JobDesc* __restrict__ jobs,
                                                                          const GroupOp* __restrict__ ops, int nops) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const GroupOp op = ops[group_op_of(ops, nops, gw)];
  const JobDesc& J = jobs[op.job];
  const int lw = gw - op.warp_begin;
  if (lw >= J.g.nstrips * J.g.nchunks) return;
  if constexpr (PSV) {
    psv_march<BulkL<PV_NSEG>>(job_psv_step(J, op.it, op.a, op.b, op.flags), lw, warp_slice<BulkL<PV_NSEG>>(smem));
  } else {
    sh_march<BulkL<SH_NSEG>>(job_sh_step(J, op.it, op.a, op.b, op.flags), lw, warp_slice<BulkL<SH_NSEG>>(smem));
  }
}

cudaError_t launch_grouped_forward(const JobDesc* jobs, const GroupOp* ops, int nops, int warps, bool psv,
                                   bool pdl, cudaStream_t s) {
  if (nops <= 0 || warps <= 0) return cudaSuccess;
  const unsigned blocks = unsigned((warps + kStepWarps - 1) / kStepWarps);
  if (psv) {
    const size_t smem = smem_for<BulkL<PV_NSEG>>();
    static const cudaError_t attr = prepare_kernel(grouped_forward_kernel<true>, smem);
    if (attr != cudaSuccess) return attr;
    return launch_step(grouped_forward_kernel<true>, pdl, blocks, smem, s, jobs, ops, nops);
  } else {
    const size_t smem = smem_for<BulkL<SH_NSEG>>();
    static const cudaError_t attr = prepare_kernel(grouped_forward_kernel<false>, smem);
    if (attr != cudaSuccess) return attr;
    return launch_step(grouped_forward_kernel<false>, pdl, blocks, smem, s, jobs, ops, nops);
  }
  return cudaGetLastError();
}

size_t step_smem_bytes(bool psv, bool spin, int loader) {
  if (loader != kLoaderBulk) return 0;
  if (!psv) return smem_for<BulkL<SH_NSEG>>();
  return spin ? spin_step_smem_bytes(loader) : smem_for<BulkL<PV_NSEG>>();
}

int step_blocks_per_sm(bool psv, bool spin, int loader) {
  int n = 0;
  const int threads = kStepWarps * 32;
  const size_t smem = step_smem_bytes(psv, spin, loader);
  cudaError_t e;
  if (!psv) {
    e = loader == kLoaderBulk
            ? (prepare_kernel(sh_step_kernel<BulkL<SH_NSEG>>, smem),
               cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sh_step_kernel<BulkL<SH_NSEG>>, threads, smem))
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sh_step_kernel<DirectL<SH_NSEG>>, threads, smem);
  } else if (spin) {
    return spin_step_blocks_per_sm(loader);
  } else {
    e = loader == kLoaderBulk
            ? (prepare_kernel(psv_step_kernel<BulkL<PV_NSEG>>, smem),
               cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, psv_step_kernel<BulkL<PV_NSEG>>, threads, smem))
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, psv_step_kernel<DirectL<PV_NSEG>>, threads, smem);
  }
  return e == cudaSuccess ? n : 0;
}


cudaError_t launch_sh_step(const ShStep& p, cudaStream_t s) {
  if (p.g.loader == kLoaderBulk) return launch_sh<BulkL<SH_NSEG>>(p, s);
  return launch_sh<DirectL<SH_NSEG>>(p, s);
}

cudaError_t launch_psv_step(const PsvStep& p, bool spin, cudaStream_t s) {
  if (spin) return launch_psv_spin_step(p, s);
  if (p.g.loader == kLoaderBulk) return launch_psv<BulkL<PV_NSEG>>(p, s);
  return launch_psv<DirectL<PV_NSEG>>(p, s);
}

}  // namespace seiswg
