// fd_step2.cu -- two PSV or SH time steps per launch (temporal blocking).
//
// Built with multiply-add contraction (the one-step kernels keep the
// reference's separate multiply and add): the two-step march is bound by
// instruction issue, not by HBM.
//
// The material these kernels read is scaled by dt on the host side of the
// launch (dt/rho, dt*lambda, dt*mu; Sim::prepare_model), so that dt costs no
// instruction per update and every intermediate keeps the magnitude of the
// reference's own (fd2d.wgsl:362-363, 396-398: dt multiplies the divergence
// after the division by 8 h).  Folding dt into the difference factors instead
// (dt/(8 h) ~ 1e-5 times a raw difference) made the intermediates so small
// that the leading edge of a wavefield underflowed into subnormals sooner
// than in the reference, which moved trace samples ahead of the first arrival
// by 1e-5 relative.
#include "fd_group.cuh"
#include "fd_step2_march.cuh"

namespace seiswg {


// MID (here and below): the kernel also stores the state after the first of
// its two steps (p.vxm .., p.vym ..), for a gradient's forward pass that
// keeps every state.
template <class Loader, bool MID = false>
__global__ void __launch_bounds__(kStepWarps * 32, 2) psv_step2_kernel(const PsvStep p) {
  extern __shared__ __align__(128) unsigned char smem[];
  psv2_march<Loader, Tma2, MID>(p, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), warp_slice<Loader>(smem));
}

// Grouped two-step launch (batched gradients): the warp's job and op as in
// grouped_forward_kernel (fd_step.cu), then the two-step march, which also
// stores the middle state of operations flagged kOpMid (recomputation).
__global__ void __launch_bounds__(kStepWarps * 32, 2) grouped_forward2_kernel(const JobDesc* __restrict__ jobs,
                                                                              const GroupOp* __restrict__ ops,
                                                                              int nops) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const GroupOp op = ops[group_op_of(ops, nops, gw)];
  const JobDesc& J = jobs[op.job];
  const int lw = gw - op.warp_begin;
  if (lw >= J.g2.nstrips * J.g2.nchunks) return;
  const PsvStep p = job_psv_step2(J, op.it, op.a, op.b, op.flags);
  if (J.tm) {
    const Tma2Ptrs mp = job_psv2_maps(J, op.a);
    using L = TmaRows<PsvTmaPlan, 6, 3, Tma2Ptrs>;
    psv2_march<L, Tma2Ptrs, true>(p, lw, warp_slice<L>(smem), &mp);
  } else {
    psv2_march<Bulk2, Tma2, true>(p, lw, warp_slice<Bulk2>(smem));
  }
}

// The same for SH jobs (state slots vy, sxy, szy).
__global__ void __launch_bounds__(kStepWarps * 32, 3) grouped_forward2_sh_kernel(const JobDesc* __restrict__ jobs,
                                                                                 const GroupOp* __restrict__ ops,
                                                                                 int nops) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const GroupOp op = ops[group_op_of(ops, nops, gw)];
  const JobDesc& J = jobs[op.job];
  const int lw = gw - op.warp_begin;
  if (lw >= J.g2.nstrips * J.g2.nchunks) return;
  const ShStep p = job_sh_step2(J, op.it, op.a, op.b, op.flags);
  if (J.tm) {
    const Tma2Ptrs mp = job_sh2_maps(J, op.a);
    using L = TmaRows<ShTmaPlan, 6, 3, Tma2Ptrs>;
    sh2_march<L, Tma2Ptrs, true>(p, lw, warp_slice<L>(smem), &mp);
  } else {
    sh2_march<ShBulk2, Tma2, true>(p, lw, warp_slice<ShBulk2>(smem));
  }
}

cudaError_t launch_grouped_forward2(const JobDesc* jobs, const GroupOp* ops, int nops, int warps, bool psv,
                                    bool pdl, cudaStream_t s) {
  if (nops <= 0 || warps <= 0) return cudaSuccess;
  const unsigned blocks = unsigned((warps + kStepWarps - 1) / kStepWarps);
  if (psv) {
    const size_t smem = smem_for<Bulk2>();
    static const cudaError_t attr = prepare_kernel(grouped_forward2_kernel, smem);
    if (attr != cudaSuccess) return attr;
    return launch_step(grouped_forward2_kernel, pdl, blocks, smem, s, jobs, ops, nops);
  } else {
    const size_t smem = smem_for<ShBulk2>();
    static const cudaError_t attr = prepare_kernel(grouped_forward2_sh_kernel, smem);
    if (attr != cudaSuccess) return attr;
    return launch_step(grouped_forward2_sh_kernel, pdl, blocks, smem, s, jobs, ops, nops);
  }
  return cudaGetLastError();
}

// The two-step PSV kernel with its rows fetched by tensor copies.
template <bool MID>
__global__ void __launch_bounds__(kStepWarps * 32, 2) psv_step2_tma_kernel(const __grid_constant__ PsvStep p,
                                                                           const __grid_constant__ Tma2 t) {
  extern __shared__ __align__(128) unsigned char smem[];
  psv2_march<TmaRows2, Tma2, MID>(p, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5),
                                  warp_slice<TmaRows2>(smem), &t);
}

template <bool MID>
cudaError_t launch_psv2_tma(const PsvStep& p, const Tma2& t, cudaStream_t s) {
  const size_t smem = smem_for<TmaRows2>();
  static const cudaError_t attr = prepare_kernel(psv_step2_tma_kernel<MID>, smem);
  if (attr != cudaSuccess) return attr;
  return launch_step(psv_step2_tma_kernel<MID>, p.g.pdl != 0, blocks_for(p.g), smem, s, p, t);
}

cudaError_t launch_psv_step2_tma(const PsvStep& p, const Tma2& t, cudaStream_t s) {
  return p.vxm ? launch_psv2_tma<true>(p, t, s) : launch_psv2_tma<false>(p, t, s);
}

// SH two-step kernel: fewer registers than the PSV one (three CTAs per SM).
template <bool MID>
__global__ void __launch_bounds__(kStepWarps * 32, 3) sh_step2_kernel(const ShStep p) {
  extern __shared__ __align__(128) unsigned char smem[];
  sh2_march<ShBulk2, Tma2, MID>(p, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), warp_slice<ShBulk2>(smem));
}

template <bool MID>
__global__ void __launch_bounds__(kStepWarps * 32, 3) sh_step2_tma_kernel(const __grid_constant__ ShStep p,
                                                                          const __grid_constant__ Tma2 t) {
  extern __shared__ __align__(128) unsigned char smem[];
  using L = TmaRows<ShTmaPlan, 6, 3>;
  sh2_march<L, Tma2, MID>(p, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), warp_slice<L>(smem), &t);
}

template <bool MID>
cudaError_t launch_sh2_tma(const ShStep& p, const Tma2& t, cudaStream_t s) {
  const size_t smem = smem_for<TmaRows<ShTmaPlan, 6, 3>>();
  static const cudaError_t attr = prepare_kernel(sh_step2_tma_kernel<MID>, smem);
  if (attr != cudaSuccess) return attr;
  return launch_step(sh_step2_tma_kernel<MID>, p.g.pdl != 0, blocks_for(p.g), smem, s, p, t);
}

cudaError_t launch_sh_step2_tma(const ShStep& p, const Tma2& t, cudaStream_t s) {
  return p.vym ? launch_sh2_tma<true>(p, t, s) : launch_sh2_tma<false>(p, t, s);
}

int sh_step2_blocks_per_sm() {
  int n = 0;
  const size_t smem = smem_for<ShBulk2>();
  cudaError_t e = prepare_kernel(sh_step2_kernel<false>, smem);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, sh_step2_kernel<false>, kStepWarps * 32, smem);
  return e == cudaSuccess ? n : 0;
}

template <bool MID>
cudaError_t launch_sh2(const ShStep& p, cudaStream_t s) {
  const size_t smem = smem_for<ShBulk2>();
  static const cudaError_t attr = prepare_kernel(sh_step2_kernel<MID>, smem);
  if (attr != cudaSuccess) return attr;
  return launch_step(sh_step2_kernel<MID>, p.g.pdl != 0, blocks_for(p.g), smem, s, p);
}

cudaError_t launch_sh_step2(const ShStep& p, cudaStream_t s) {
  return p.vym ? launch_sh2<true>(p, s) : launch_sh2<false>(p, s);
}

size_t step2_smem_bytes() { return smem_for<Bulk2>(); }

int step2_blocks_per_sm() {
  int n = 0;
  const size_t smem = smem_for<Bulk2>();
  cudaError_t e = prepare_kernel(psv_step2_kernel<Bulk2>, smem);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, psv_step2_kernel<Bulk2>, kStepWarps * 32, smem);
  return e == cudaSuccess ? n : 0;
}

template <bool MID>
cudaError_t launch_psv2(const PsvStep& p, cudaStream_t s) {
  const size_t smem = smem_for<Bulk2>();
  static const cudaError_t attr = prepare_kernel(psv_step2_kernel<Bulk2, MID>, smem);
  if (attr != cudaSuccess) return attr;
  return launch_step(psv_step2_kernel<Bulk2, MID>, p.g.pdl != 0, blocks_for(p.g), smem, s, p);
}

cudaError_t launch_psv_step2(const PsvStep& p, cudaStream_t s) {
  return p.vxm ? launch_psv2<true>(p, s) : launch_psv2<false>(p, s);
}

}  // namespace seiswg
