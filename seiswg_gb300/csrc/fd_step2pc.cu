// fd_step2pc.cu -- the two-step PSV march with its rows fetched by a
// producer warpgroup (warp specialisation of the copies, not of the
// arithmetic).
//
// In psv_step2_tma_kernel every march issues its own row copies: each
// iteration lane 0 arms the stage's barrier and issues the four tensor
// copies while the other 31 lanes wait for it at the branch's end.  The
// march is bound by instruction issue, so that divergent stretch sits on its
// critical path.  Here a CTA holds four warpgroups: warpgroups 0 and 1
// produce, warpgroups 2 and 3 are eight marches (the consumers).  Lane 0 of
// producer warp w feeds consumer warp w: it waits until a stage is free (the
// consumer's `empty` barrier), arms its `full` barrier and issues its
// copies, two rows ahead of the march as before; a producer warp that waits
// holds up no other march.  A consumer waits on `full`
// and, once it is past a stage's last read (the kept rows three iterations
// back), arrives on `empty`.  The march itself is psv2_body unchanged, so the
// results are psv_step2_tma_kernel's bits.
//
// Registers: the CTA is launched with 128 per thread (512 threads, one CTA
// per SM, the whole register file); the producer warpgroups give back all
// but 24 and the consumer warpgroups take 232 (setmaxnreg; 8 x 32 x 24 +
// 8 x 32 x 232 = 512 x 128), so the marches keep the registers they have in
// the one-warp kernel.  The host checks the launch's register count before
// the first launch.
//
// Every wait is bounded (Geom::wait_polls).  A consumer that gives up stops
// releasing stages, so its producer's next wait runs out too; before it
// leaves, the producer waits (bounded) for every copy it issued, so no copy
// lands in shared memory after the CTA has gone.
#include "fd_step2_march.cuh"

namespace seiswg {
namespace {

constexpr int kPcConsumers = 8;                          // marches per CTA (two warpgroups)
constexpr int kPcThreads = 32 * (2 * kPcConsumers);      // and one producer warp each
constexpr int kPcLaunchRegs = 128;
constexpr int kPcProducerRegs = 24, kPcConsumerRegs = 232;
static_assert(kPcConsumers * 32 * (kPcProducerRegs + kPcConsumerRegs) <= kPcThreads * kPcLaunchRegs,
              "the register split must fit the registers the CTA is launched with");

__device__ __forceinline__ void mbar_arrive_pc(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// The consumer's side of a ring that the producer fills: S stages of one row
// of the eight segments of PsvTmaPlan, then S `full` and S `empty` barriers.
struct PcRows {
  static constexpr int S = 6, KEEP = 3, NSEG = P2_NSEG;
  static constexpr int kStages = S;
  static constexpr uint32_t kStageBytes = NSEG * kSegFloats * sizeof(float);
  using SegsT = Segs<NSEG>;
  int lane, cur, nxt;
  uint32_t par;
  float* buf;
  uint64_t* full;
  uint64_t* empty;
  unsigned lim = kWaitLimit;
  __device__ PcRows(const SegsT&, size_t, int, int, int lane_, float* buf_, uint64_t* bar_, int)
      : lane(lane_), cur(0), nxt(0), par(0), buf(buf_), full(bar_), empty(bar_ + S) {}
  __device__ __forceinline__ void configure(const Geom& g) { lim = g.wait_polls ? g.wait_polls : kWaitLimit; }
  __device__ __forceinline__ void start() {
    pdl_trigger();
    pdl_wait();  // the state rows the march loads itself come from the previous launch
    __syncwarp();
  }
  __device__ __forceinline__ bool acquire(int k) {
    __syncwarp();  // the previous iteration's reads are done
    cur = nxt;
    const uint32_t ph = par;
    if (++nxt == S) {
      nxt = 0;
      par ^= 1u;
    }
    // Row k - 1 - KEEP was last read (a kept row) in iteration k - 1.
    if (lane == 0 && k > KEEP) {
      const int rel = cur - 1 - KEEP;
      mbar_arrive_pc(&empty[rel < 0 ? rel + S : rel]);
    }
    return __all_sync(kFull, mbar_wait(&full[cur], ph, lim));
  }
  __device__ __forceinline__ f4 seg_back(int q, int d) const {
    const int st = cur >= d ? cur - d : cur + S - d;
    const float4 t = *reinterpret_cast<const float4*>(buf + (st * NSEG + q) * kSegFloats + 4 * lane);
    f4 r;
    r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
    return r;
  }
  __device__ __forceinline__ f4 seg(int q) const { return seg_back(q, 0); }
  __device__ __forceinline__ void release() { __syncwarp(); }
  __device__ __forceinline__ void drain(int) { __syncwarp(); }  // the producer drains the copies
  __host__ __device__ static constexpr size_t smem_bytes_per_warp() {
    return (size_t(S) * kStageBytes + 2 * size_t(S) * 8 + 127) / 128 * 128;
  }
};

constexpr size_t kPcSlice = PcRows::smem_bytes_per_warp();
constexpr size_t kPcSmem = size_t(kPcConsumers) * kPcSlice;

// One producer lane: every row copy of consumer warp c's march.
__device__ __forceinline__ void pc_produce(const PsvStep& p, const Tma2* tm, unsigned char* smem, int c) {
  const March m = march_of(p.g, blockIdx.x * kPcConsumers + c);
  if (!m.active) return;
  int valid;
  const LaneCols L0 = lane_cols2(p.g, m.strip, 0, valid);  // lane 0's columns: the copies' x
  const int x0 = L0.c0 + kHaloCols;
  const int i0 = m.ib - 4, nk = (m.ie - m.ib) + 9;  // the march's rows, as psv2_body
  constexpr int S = PcRows::S;
  unsigned char* slice = smem + size_t(c) * kPcSlice;
  float* buf = reinterpret_cast<float*>(slice);
  uint64_t* full = reinterpret_cast<uint64_t*>(slice + size_t(S) * PcRows::kStageBytes);
  uint64_t* empty = full + S;
  const unsigned lim = p.g.wait_polls ? p.g.wait_polls : kWaitLimit;
  const uint32_t extra = p.g.arm_extra;  // test hook: bytes armed on row 0 beyond its copies
  pdl_trigger();
  pdl_wait();
  int k = 0;
  for (; k < nk; ++k) {
    const int s = k % S;
    if (k >= S && !mbar_wait(&empty[s], uint32_t(k / S - 1) & 1u, lim)) {
      flag_timeout(p.err);
      break;
    }
    fence_proxy_async();  // the consumer's reads of the stage before the copies that refill it
    mbar_expect_tx(&full[s], PcRows::kStageBytes + (k == 0 ? extra : 0u));
    PsvTmaPlan::issue(buf + size_t(s) * P2_NSEG * kSegFloats, tm, x0, i0 + k + kHaloRows, &full[s]);
  }
  // Row 0 never completes with the test hook's extra bytes (its consumer and
  // then this loop give up): count them, then wait for every issued copy.
  if (extra && k > 0) mbar_complete_tx(&full[0], extra);
  for (int r = k > S ? k - S : 0; r < k; ++r) (void)mbar_wait(&full[r % S], uint32_t(r / S) & 1u, lim);
}

template <bool MID>
__global__ void __launch_bounds__(kPcThreads, 1) psv_step2_pc_kernel(const __grid_constant__ PsvStep p,
                                                                     const __grid_constant__ Tma2 t) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int c = 0; c < kPcConsumers; ++c) {
      uint64_t* bar = reinterpret_cast<uint64_t*>(smem + size_t(c) * kPcSlice + size_t(PcRows::S) * PcRows::kStageBytes);
      for (int s = 0; s < PcRows::S; ++s) {
        mbar_init(&bar[s], 1);                // full: the producer's arming arrival + the copies' bytes
        mbar_init(&bar[PcRows::S + s], 1);    // empty: the consumer's lane 0
      }
    }
    fence_mbar_init();
  }
  __syncthreads();
  if (w < kPcConsumers) {
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(kPcProducerRegs));
    if (lane == 0) pc_produce(p, &t, smem, w);
  } else {
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(kPcConsumerRegs));
    const int c = w - kPcConsumers;
    psv2_march<PcRows, Tma2, MID>(p, blockIdx.x * kPcConsumers + c, smem + size_t(c) * kPcSlice);
  }
}

template <bool MID>
cudaError_t launch_pc(const PsvStep& p, const Tma2& t, cudaStream_t s) {
  static const cudaError_t ready = [] {
    cudaFuncAttributes a{};
    cudaError_t e = cudaFuncGetAttributes(&a, psv_step2_pc_kernel<MID>);
    if (e != cudaSuccess) return e;
    // setmaxnreg.inc waits for registers the CTA does not have if it was
    // launched with fewer than the split assumes: refuse to launch then.
    if (a.numRegs < kPcLaunchRegs) return cudaErrorInvalidConfiguration;
    return cudaFuncSetAttribute(psv_step2_pc_kernel<MID>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                int(kPcSmem));
  }();
  if (ready != cudaSuccess) return ready;
  const long marches = long(p.g.nstrips) * p.g.nchunks;
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(unsigned((marches + kPcConsumers - 1) / kPcConsumers));
  cfg.blockDim = dim3(kPcThreads);
  cfg.dynamicSmemBytes = kPcSmem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = p.g.pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, psv_step2_pc_kernel<MID>, p, t);
}

}  // namespace

cudaError_t launch_psv_step2_pc(const PsvStep& p, const Tma2& t, cudaStream_t s) {
  return p.vxm ? launch_pc<true>(p, t, s) : launch_pc<false>(p, t, s);
}

}  // namespace seiswg
