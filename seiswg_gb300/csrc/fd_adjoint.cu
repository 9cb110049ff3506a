// fd_adjoint.cu -- fused reverse step of the exact discrete adjoint.
//
// For the forward step n (fd_step.cu)
//   v^{n+1} = b (v^n + dt B (D- sigma^n + f^n)),    B = 1/rho
//   sigma^{n+1} = sigma^n + dt C(lambda, mu) D+ v^{n+1}
//   u_r^{n+1} = u_r^n + dt v^{n+1}(r)               (receiver displacement, d^n = u^{n+1})
// and J(d), reverse-mode differentiation gives, for n = nt-1 .. 0, with the
// carried adjoint velocity w^{n+1} and adjoint stress s^{n+1}:
//   Vbar = w^{n+1} + dt U^n (at receivers) + (D+)^T (dt C s^{n+1})
//   w^n  = b Vbar
//   s^n  = s^{n+1} + (D-)^T (dt B w^n)
//   g_B += dt w^n . (D- sigma^n + f^n)
//   g_lambda, g_mu += dt s^{n+1} . dC/d(lambda, mu) D+ v^{n+1}
// where U^n = sum_{m >= n} dJ/dd^m.  The transposes of the masked staggered
// differences are differences with the other tap pattern applied to the
// masked input: (D-)^T g = -D+taps(M- g), (D+)^T g = -D-taps(M+ g), so the
// reverse step has the same row and column reach as the forward step and
// uses the same warp march: iteration k handles Vbar/w of row i = ib-1+k and
// the adjoint stress of row i-2.  The forward v^{n+1} and D- sigma^n are
// recomputed from the forward state S^n inside the same pass.
//
// Algorithmic bytes per cell-update (PSV): forward state 5 + adjoint state
// 5 r+w + model 3 + gradients 3 r+w = 96 B (SH: 3 + 3 r+w + 2 + 2 r+w = 60 B).
#include "fd_adjoint_march.cuh"
#include "fd_group.cuh"

namespace seiswg {

template <class Loader>
__global__ void __launch_bounds__(kStepWarps * 32, 2) psv_adjoint_kernel(const PsvAdjoint p) {
  extern __shared__ __align__(128) unsigned char smem[];
  psv_adjoint_march<Loader>(p, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5),
                            warp_slice<Loader>(smem));
}

__global__ void __launch_bounds__(kStepWarps * 32, 2) psv_adjoint_tma_kernel(const __grid_constant__ PsvAdjoint p,
                                                                             const __grid_constant__ TmaAdj t) {
  extern __shared__ __align__(128) unsigned char smem[];
  psv_adjoint_march<ATma>(p, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), warp_slice<ATma>(smem),
                          &t);
}

template <class Loader>
__global__ void __launch_bounds__(kStepWarps * 32, 2) sh_adjoint_kernel(const ShAdjoint p) {
  extern __shared__ __align__(128) unsigned char smem[];
  sh_adjoint_march<Loader>(p, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5),
                           warp_slice<Loader>(smem));
}

// --------------------------------------------------------------------------
// Launchers
// --------------------------------------------------------------------------
namespace {

unsigned ablocks(const Geom& g) {
  const long warps = long(g.nstrips) * g.nchunks;
  return unsigned((warps + kStepWarps - 1) / kStepWarps);
}

template <class L>
size_t asmem() {
  return L::kStages ? size_t(kStepWarps) * L::smem_bytes_per_warp() : 0;
}

template <typename K>
cudaError_t aprep(K kernel, size_t smem) {
  if (smem > 48 * 1024)
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  return cudaSuccess;
}

template <class L>
cudaError_t launch_psv_adj(const PsvAdjoint& p, cudaStream_t s) {
  const size_t smem = asmem<L>();
  static const cudaError_t attr = aprep(psv_adjoint_kernel<L>, smem);
  if (attr != cudaSuccess) return attr;
  return launch_step(psv_adjoint_kernel<L>, p.g.pdl != 0, ablocks(p.g), smem, s, p);
}

template <class L>
cudaError_t launch_sh_adj(const ShAdjoint& p, cudaStream_t s) {
  const size_t smem = asmem<L>();
  static const cudaError_t attr = aprep(sh_adjoint_kernel<L>, smem);
  if (attr != cudaSuccess) return attr;
  return launch_step(sh_adjoint_kernel<L>, p.g.pdl != 0, ablocks(p.g), smem, s, p);
}

}  // namespace

// ---- grouped reverse steps ------------------------------------------------------

template <bool PSV>
__global__ void __launch_bounds__(kStepWarps * 32, 2) grouped_adjoint_kernel(const JobDesc* __restrict__ jobs,
                                                                             const GroupOp* __restrict__ ops,
                                                                             int nops) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const GroupOp op = ops[group_op_of(ops, nops, gw)];
  const JobDesc& J = jobs[op.job];
  const int lw = gw - op.warp_begin;
  if (lw >= J.g.nstrips * J.g.nchunks) return;
  if constexpr (PSV) {
    const PsvAdjoint p = job_psv_adjoint(J, op.it, op.a, op.b);
    if (J.tm) {
      const TmaAdjPtrs mp = job_adj_maps(J, op.a, op.b);
      using L = TmaRows<AdjTmaPlan, kAdjStages, 0, TmaAdjPtrs>;
      psv_adjoint_march<L, TmaAdjPtrs>(p, lw, warp_slice<L>(smem), &mp);
    } else {
      psv_adjoint_march<ABulk<PA_NSEG>>(p, lw, warp_slice<ABulk<PA_NSEG>>(smem));
    }
  } else {
    sh_adjoint_march<ABulk<SA_NSEG>>(job_sh_adjoint(J, op.it, op.a, op.b), lw, warp_slice<ABulk<SA_NSEG>>(smem));
  }
}

cudaError_t launch_grouped_adjoint(const JobDesc* jobs, const GroupOp* ops, int nops, int warps, bool psv,
                                   bool pdl, cudaStream_t s) {
  if (nops <= 0 || warps <= 0) return cudaSuccess;
  const unsigned blocks = unsigned((warps + kStepWarps - 1) / kStepWarps);
  if (psv) {
    const size_t smem = asmem<ABulk<PA_NSEG>>();
    static const cudaError_t attr = aprep(grouped_adjoint_kernel<true>, smem);
    if (attr != cudaSuccess) return attr;
    return launch_step(grouped_adjoint_kernel<true>, pdl, blocks, smem, s, jobs, ops, nops);
  } else {
    const size_t smem = asmem<ABulk<SA_NSEG>>();
    static const cudaError_t attr = aprep(grouped_adjoint_kernel<false>, smem);
    if (attr != cudaSuccess) return attr;
    return launch_step(grouped_adjoint_kernel<false>, pdl, blocks, smem, s, jobs, ops, nops);
  }
  return cudaGetLastError();
}

int adjoint_blocks_per_sm(bool psv, int loader) {
  int n = 0;
  const int threads = kStepWarps * 32;
  cudaError_t e;
  if (psv) {
    if (loader == kLoaderBulk) {
      const size_t smem = asmem<ABulk<PA_NSEG>>();
      e = aprep(psv_adjoint_kernel<ABulk<PA_NSEG>>, smem);
      if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, psv_adjoint_kernel<ABulk<PA_NSEG>>, threads, smem);
    } else {
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, psv_adjoint_kernel<ADirect<PA_NSEG>>, threads, 0);
    }
  } else {
    if (loader == kLoaderBulk) {
      const size_t smem = asmem<ABulk<SA_NSEG>>();
      e = aprep(sh_adjoint_kernel<ABulk<SA_NSEG>>, smem);
      if (e == cudaSuccess)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sh_adjoint_kernel<ABulk<SA_NSEG>>, threads, smem);
    } else {
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sh_adjoint_kernel<ADirect<SA_NSEG>>, threads, 0);
    }
  }
  return e == cudaSuccess ? n : 0;
}

cudaError_t launch_psv_adjoint(const PsvAdjoint& p, cudaStream_t s) {
  if (p.g.loader == kLoaderBulk) return launch_psv_adj<ABulk<PA_NSEG>>(p, s);
  return launch_psv_adj<ADirect<PA_NSEG>>(p, s);
}

cudaError_t launch_psv_adjoint_tma(const PsvAdjoint& p, const TmaAdj& t, cudaStream_t s) {
  const size_t smem = asmem<ATma>();
  static const cudaError_t attr = aprep(psv_adjoint_tma_kernel, smem);
  if (attr != cudaSuccess) return attr;
  return launch_step(psv_adjoint_tma_kernel, p.g.pdl != 0, ablocks(p.g), smem, s, p, t);
}

cudaError_t launch_sh_adjoint(const ShAdjoint& p, cudaStream_t s) {
  if (p.g.loader == kLoaderBulk) return launch_sh_adj<ABulk<SA_NSEG>>(p, s);
  return launch_sh_adj<ADirect<SA_NSEG>>(p, s);
}

}  // namespace seiswg
