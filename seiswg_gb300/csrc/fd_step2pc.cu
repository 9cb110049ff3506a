// fd_step2pc.cu -- the two-step PSV march with its rows fetched by producer
// warps (fd_producer.cuh): eight marches per CTA, the march psv2_body
// unchanged, so the results are psv_step2_tma_kernel's bits.  Its ring keeps
// the self-issuing kernel's shape: six stages of the eight segments of
// PsvTmaPlan, three kept for level 2's material and sigma_zz, two rows in
// flight.
#include "fd_producer.cuh"
#include "fd_step2_march.cuh"

namespace seiswg {
namespace {

using Pc2Rows = PcRows<P2_NSEG, 6, 3>;
constexpr size_t kPc2Smem = size_t(kPcConsumers) * Pc2Rows::smem_bytes_per_warp();

template <bool MID>
__global__ void __launch_bounds__(kPcThreads, 1) psv_step2_pc_kernel(const __grid_constant__ PsvStep p,
                                                                     const __grid_constant__ Tma2 t) {
  extern __shared__ __align__(128) unsigned char smem[];
  pc_init<Pc2Rows>(smem);
  const int c = (threadIdx.x >> 5) % kPcConsumers;  // the march this warp runs or feeds
  const int gw = blockIdx.x * kPcConsumers + c;
  unsigned char* slice = smem + size_t(c) * Pc2Rows::smem_bytes_per_warp();
  if (pc_split()) {
    psv2_march<Pc2Rows, Tma2, MID>(p, gw, slice);
  } else if ((threadIdx.x & 31) == 0) {
    const March m = march_of(p.g, gw);
    if (!m.active) return;
    int valid;
    const LaneCols L0 = lane_cols2(p.g, m.strip, 0, valid);  // lane 0's columns: the copies' x
    // psv2_body's rows: i0 = ib - 4 .. ie + 4 (iteration k reads row i0 + k)
    pc_produce<Pc2Rows, PsvTmaPlan>(&t, slice, L0.c0 + kHaloCols, m.ib - 4 + kHaloRows, (m.ie - m.ib) + 9, p.g,
                                    p.err);
  }
}

template <bool MID>
cudaError_t launch_pc2(const PsvStep& p, const Tma2& t, cudaStream_t s) {
  static const cudaError_t ready = pc_kernel_ready(psv_step2_pc_kernel<MID>, kPc2Smem);
  if (ready != cudaSuccess) return ready;
  return pc_launch(psv_step2_pc_kernel<MID>, p.g.pdl != 0, long(p.g.nstrips) * p.g.nchunks, kPc2Smem, s, p, t);
}

}  // namespace

cudaError_t launch_psv_step2_pc(const PsvStep& p, const Tma2& t, cudaStream_t s) {
  return p.vxm ? launch_pc2<true>(p, t, s) : launch_pc2<false>(p, t, s);
}

}  // namespace seiswg
