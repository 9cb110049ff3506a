// fd_producer.cuh -- row rings filled by producer warps (warp specialisation
// of the copies, not of the arithmetic), shared by the two-step kernel
// (fd_step2pc.cu) and the PSV reverse steps (fd_adjointpc.cu).
//
// In the self-issuing kernels every march issues its own row copies: each
// iteration lane 0 arms the stage's barrier and issues the row's tensor
// copies while the other 31 lanes wait for it at the branch's end, on the
// critical path of a loop bound by instruction issue or latency.  Here a CTA
// holds four warpgroups: warpgroups 0 and 1 produce, warpgroups 2 and 3 are
// eight marches (the consumers).  Lane 0 of producer warp w feeds consumer
// warp w: it waits until a stage is free (the consumer's `empty` barrier),
// arms its `full` barrier and issues its copies (Plan::issue), S - 1 - KEEP
// rows ahead of the march, as the self-issuing ring; a producer that waits
// holds up no other march.  The consumer waits on `full` and, once past a
// stage's last read (KEEP rows kept for reads further back), its 32 lanes
// arrive on `empty`.  The marches are the self-issuing kernels' own code,
// reading the same rows, so the results are their bits.
//
// Registers: such a CTA is launched with 128 per thread (512 threads, one
// CTA per SM, the whole register file); the producer warpgroups give back all
// but 24 and the consumer warpgroups take 232 (setmaxnreg; 8 x 32 x (24 +
// 232) = 512 x 128), so the marches keep the registers of their one-kind
// kernels.  The host checks the launch's register count before the first
// launch (pc_kernel_ready).
//
// Every wait is bounded (Geom::wait_polls).  A consumer that gives up stops
// releasing stages, so its producer's next wait runs out too; before it
// leaves, the producer waits (bounded) for every copy it issued, so no copy
// lands in shared memory after the CTA has gone.
#pragma once

#include "fd_march.cuh"
#include "fd_tma.cuh"

namespace seiswg {
namespace {

constexpr int kPcConsumers = 8;                      // marches per CTA (two warpgroups)
constexpr int kPcThreads = 32 * (2 * kPcConsumers);  // and one producer warp each
constexpr int kPcLaunchRegs = 128;
constexpr int kPcProducerRegs = 24, kPcConsumerRegs = 232;
static_assert(kPcConsumers * 32 * (kPcProducerRegs + kPcConsumerRegs) <= kPcThreads * kPcLaunchRegs,
              "the register split must fit the registers the CTA is launched with");

__device__ __forceinline__ void mbar_arrive_pc(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// The consumer's side of a ring that a producer warp fills: S stages of one
// row of NSEG segments, then S `full` and S `empty` barriers.  The loader
// interface of the self-issuing rings (fd_pipe.cuh, fd_tma.cuh).
template <int NSEG_, int S_, int KEEP_>
struct PcRows {
  static constexpr int S = S_, KEEP = KEEP_, NSEG = NSEG_;
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
    pdl_wait();  // the rows a march loads itself come from the previous launch
    __syncwarp();
  }
  // Each lane releases a stage after its own last read of it (its arrival
  // orders its reads before the producer's refill), so no warp barrier is
  // needed per row.
  __device__ __forceinline__ bool acquire(int k) {
    cur = nxt;
    const uint32_t ph = par;
    if (++nxt == S) {
      nxt = 0;
      par ^= 1u;
    }
    // Row k - 1 - KEEP was last read (directly or as a kept row) in
    // iteration k - 1; every lane arrives (no divergent branch per row).
    if (k > KEEP) {
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
  __device__ __forceinline__ void release() {}
  __device__ __forceinline__ void drain(int) { __syncwarp(); }  // the producer drains the copies
  __host__ __device__ static constexpr size_t smem_bytes_per_warp() {
    return (size_t(S) * kStageBytes + 2 * size_t(S) * 8 + 127) / 128 * 128;
  }
};

// Initialises the barriers of the CTA's eight rings (thread 0), then the
// CTA's barrier.
template <class Rows>
__device__ __forceinline__ void pc_init(unsigned char* smem) {
  if (threadIdx.x == 0) {
    for (int c = 0; c < kPcConsumers; ++c) {
      uint64_t* bar = reinterpret_cast<uint64_t*>(smem + size_t(c) * Rows::smem_bytes_per_warp() +
                                                  size_t(Rows::S) * Rows::kStageBytes);
      for (int s = 0; s < Rows::S; ++s) {
        mbar_init(&bar[s], 1);            // full: the producer's arming arrival and the copies' bytes
        mbar_init(&bar[Rows::S + s], 32);  // empty: the consumer's 32 lanes
      }
    }
    fence_mbar_init();
  }
  __syncthreads();
}

// One producer lane: the copies of rows 0 .. nk-1 of a march into ring
// `slice`, issue(stage buffer, k, barrier) issuing row k's (after the barrier
// is armed with the stage's bytes).
template <class Rows, class Issue>
__device__ __forceinline__ void pc_produce_with(unsigned char* slice, int nk, const Geom& g, int* err,
                                                const Issue& issue) {
  constexpr int S = Rows::S;
  float* buf = reinterpret_cast<float*>(slice);
  uint64_t* full = reinterpret_cast<uint64_t*>(slice + size_t(S) * Rows::kStageBytes);
  uint64_t* empty = full + S;
  const unsigned lim = g.wait_polls ? g.wait_polls : kWaitLimit;
  const uint32_t extra = g.arm_extra;  // test hook: bytes armed on row 0 beyond its copies
  pdl_trigger();
  pdl_wait();
  int k = 0;
  for (; k < nk; ++k) {
    const int s = k % S;
    if (k >= S && !mbar_wait(&empty[s], uint32_t(k / S - 1) & 1u, lim)) {
      if (err) atomicOr(err, kErrWaitTimeout);
      break;
    }
    fence_proxy_async();  // the consumer's reads of the stage before the copies that refill it
    mbar_expect_tx(&full[s], Rows::kStageBytes + (k == 0 ? extra : 0u));
    issue(buf + size_t(s) * Rows::NSEG * kSegFloats, k, &full[s]);
  }
  // Row 0 never completes with the test hook's extra bytes (its consumer and
  // then this loop give up): count them, then wait for every issued copy.
  if (extra && k > 0) mbar_complete_tx(&full[0], extra);
  for (int r = k > S ? k - S : 0; r < k; ++r) (void)mbar_wait(&full[r % S], uint32_t(r / S) & 1u, lim);
}

// The same with a tensor-copy plan: row k at padded row y0 + k and padded
// column x0 (Plan::issue).
template <class Rows, class Plan, class M>
__device__ __forceinline__ void pc_produce(const M* tm, unsigned char* slice, int x0, int y0, int nk, const Geom& g,
                                           int* err) {
  pc_produce_with<Rows>(slice, nk, g, err,
                        [&](float* sb, int k, uint64_t* bar) { Plan::issue(sb, tm, x0, y0 + k, bar); });
}

// The register split of the CTA's warpgroups: true in a consumer warp.
__device__ __forceinline__ bool pc_split() {
  if ((threadIdx.x >> 5) < kPcConsumers) {
    asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(kPcProducerRegs));
    return false;
  }
  asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(kPcConsumerRegs));
  return true;
}

// Before a producer kernel's first launch: its launch register count (the
// register split assumes kPcLaunchRegs; setmaxnreg.inc would wait for
// registers the CTA does not have with fewer), and its shared memory.
template <class K>
cudaError_t pc_kernel_ready(K kernel, size_t smem) {
  cudaFuncAttributes a{};
  cudaError_t e = cudaFuncGetAttributes(&a, kernel);
  if (e != cudaSuccess) return e;
  if (a.numRegs != kPcLaunchRegs) return cudaErrorInvalidConfiguration;
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
}

// Launches a producer kernel over `marches` marches (kPcConsumers per CTA).
template <class K, class... Args>
cudaError_t pc_launch(K kernel, bool pdl, long marches, size_t smem, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(unsigned((marches + kPcConsumers - 1) / kPcConsumers));
  cfg.blockDim = dim3(kPcThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

}  // namespace
}  // namespace seiswg
