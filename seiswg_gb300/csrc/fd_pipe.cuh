// fd_pipe.cuh -- per-warp row pipeline of the step kernels.
//
// Each iteration of a warp's march consumes one "stage": NSEG row segments of
// 128 floats (512 B, the warp's 32 float4 lanes), one per field, each from a
// fixed row offset relative to the iteration's row.  Two loaders provide them:
//
//   DirectRows  plain 16-byte __ldg loads issued at the top of the iteration.
//   BulkRows    a ring of S stages in shared memory filled by the TMA engine's
//               bulk copy (cp.async.bulk ... mbarrier::complete_tx::bytes),
//               issued S-1 iterations ahead by lane 0 or, for many
//               segments, lane q copying segment q; completion is tracked by
//               one mbarrier per stage.  Waits are bounded: after a number
//               of polls (Geom::wait_polls, kWaitLimit when 0) the warp
//               records an error in *err, drains the copies it issued (again
//               bounded) and leaves its march.
#pragma once

#include "fd_common.cuh"

namespace seiswg {

constexpr int kSegFloats = 128;  // 32 lanes x float4
constexpr unsigned kWaitLimit = 1u << 20;  // polls of a bounded wait unless Geom::wait_polls says otherwise

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// Counts `bytes` as arrived on the barrier's transaction count, as a copy
// completing would.  Used only to take back the bytes the wait-expiry test
// hook armed beyond the copies, so that the barrier's phase then completes
// exactly when the copies really issued have landed.
__device__ __forceinline__ void mbar_complete_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.complete_tx.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait for the completion of phase `parity`: at most `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned limit) {
  for (unsigned n = 0; n < limit; ++n)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 16-byte aligned global -> shared bulk copy completing on `bar`.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Programmatic dependent launch.  A step kernel launched with the
// programmatic-serialization attribute may start while the launch before it
// in the stream finishes: its CTAs take the SMs that launch's CTAs leave, set
// up their row pipelines, and wait (pdl_wait) for that launch to complete,
// and for its writes to be visible, before their first read of state.  Every
// CTA first signals (pdl_trigger) that the next such launch may start.  In a
// kernel launched without the attribute both are no-ops.  The loaders' start()
// does both, before their first copy: everything a march does before start()
// touches only data no launch of the stream writes.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// A warp's slice of the CTA's dynamic shared memory: the S stages of its row
// ring, then S mbarriers, rounded up to 128 bytes so that the stages of every
// warp stay 128-byte aligned, as tensor copies require.  Warp w's slice
// starts at w times the kernel's per-warp stride: its loader's own size in
// the step kernels, the largest loader's in the batch's queue kernel.
__host__ __device__ constexpr size_t warp_ring_bytes(int stages, uint32_t stage_bytes) {
  return (size_t(stages) * stage_bytes + size_t(stages) * 8 + 127) / 128 * 128;
}

template <class Loader>
__device__ __forceinline__ unsigned char* warp_slice(unsigned char* smem) {
  return smem + size_t(threadIdx.x >> 5) * Loader::smem_bytes_per_warp();
}

// The ring of a slice: stages first, barriers after them.
template <class Loader>
__device__ __forceinline__ void slice_ring(unsigned char* slice, float*& buf, uint64_t*& bar) {
  buf = reinterpret_cast<float*>(slice);
  bar = reinterpret_cast<uint64_t*>(slice + size_t(Loader::kStages) * Loader::kStageBytes);
}

// Segment table: base pointer (element (0,0)) and row offset of each field.
template <int NSEG>
struct Segs {
  const float* base[NSEG];
  int roff[NSEG];
};

template <int NSEG>
struct DirectRows {
  static constexpr int kStages = 0;
  __host__ __device__ static constexpr size_t smem_bytes_per_warp() { return 0; }
  Segs<NSEG> s;
  size_t ld;
  int c0, ib;
  f4 v[NSEG];
  __device__ DirectRows(const Segs<NSEG>& segs, size_t ld_, int c0_, int ib_, int, float*, uint64_t*, int)
      : s(segs), ld(ld_), c0(c0_), ib(ib_) {}
  __device__ __forceinline__ void configure(const Geom&) {}
  __device__ __forceinline__ void start() {
    pdl_trigger();
    pdl_wait();
  }
  // Loads the stage of iteration k (row i = ib - 1 + k).
  __device__ __forceinline__ bool acquire(int k) {
    const int i = ib - 1 + k;
#pragma unroll
    for (int q = 0; q < NSEG; ++q) v[q] = ld4(s.base[q] + ptrdiff_t(i + s.roff[q]) * ptrdiff_t(ld) + c0);
    return true;
  }
  __device__ __forceinline__ const f4& seg(int q) const { return v[q]; }
  __device__ __forceinline__ void release() {}
  __device__ __forceinline__ void drain(int) {}
};

// KEEP: the stages of the last KEEP iterations stay readable (seg_back), so a
// stage is refilled KEEP iterations later and S-1-KEEP iterations are in
// flight.
template <int NSEG, int S, bool kLaneIssue = false, int KEEP = 0>
struct BulkRows {
  static_assert(!kLaneIssue || NSEG <= 32, "one lane issues each segment's copy");
  static_assert(S - 1 - KEEP >= 1, "at least one stage in flight");
  static constexpr int kAhead = S - 1 - KEEP;
  static constexpr int kStages = S;
  static constexpr uint32_t kStageBytes = NSEG * kSegFloats * sizeof(float);
  __host__ __device__ static constexpr size_t smem_bytes_per_warp() {
    return warp_ring_bytes(S, kStageBytes);
  }
  Segs<NSEG> s;      // serial issue: every segment's field
  const float* src;  // lane issue, lane q < NSEG: segment q's field at row 0, the warp's first column
  int roff;          // lane issue, lane q < NSEG: segment q's row offset
  size_t ld;
  int col0, ib, lane, nk;
  int cur;         // stage of the acquired iteration
  int nxt;         // stage of the next iteration to acquire
  uint32_t par;    // barrier phase parity of the next iteration to acquire
  float* buf;      // [S][NSEG][128]
  uint64_t* bar;   // [S]
  unsigned lim = kWaitLimit;  // polls of a bounded wait
  uint32_t extra = 0;         // test hook: bytes armed on stage 0 beyond its copies
  __device__ BulkRows(const Segs<NSEG>& segs, size_t ld_, int c0_, int ib_, int lane_, float* buf_,
                      uint64_t* bar_, int nk_)
      : s(segs), src(nullptr), roff(0), ld(ld_), col0(c0_ - 4 * lane_), ib(ib_), lane(lane_), nk(nk_), cur(0),
        nxt(0), par(0), buf(buf_), bar(bar_) {
    if constexpr (kLaneIssue) {
#pragma unroll
      for (int q = 0; q < NSEG; ++q)
        if (lane_ == q) {
          src = segs.base[q] + col0;
          roff = segs.roff[q];
        }
    }
  }

  // Arms the stage's barrier with the stage's bytes and copies its NSEG
  // 512-byte segments: all by lane 0 (serial issue), or segment q by lane q
  // (lane issue; a copy completing before lane 0's arrive only takes the
  // transaction count below zero transiently, which the barrier allows).
  // Called by the issuing lanes only.
  __device__ __forceinline__ void issue(int k) { issue_at(k, k % S); }
  // As issue(k), with the stage st = k % S supplied by the caller; `add`
  // bytes are armed beyond the stage's own (the wait-expiry test hook).
  __device__ __forceinline__ void issue_at(int k, int st, uint32_t add = 0) {
    const int i = ib - 1 + k;
    if constexpr (kLaneIssue) {
      if (lane == 0) mbar_expect_tx(&bar[st], kStageBytes + add);
      bulk_g2s(buf + (st * NSEG + lane) * kSegFloats, src + ptrdiff_t(i + roff) * ptrdiff_t(ld),
               kSegFloats * sizeof(float), &bar[st]);
    } else {
      mbar_expect_tx(&bar[st], kStageBytes + add);
#pragma unroll
      for (int q = 0; q < NSEG; ++q)
        bulk_g2s(buf + (st * NSEG + q) * kSegFloats, s.base[q] + ptrdiff_t(i + s.roff[q]) * ptrdiff_t(ld) + col0,
                 kSegFloats * sizeof(float), &bar[st]);
    }
  }
  __device__ __forceinline__ bool issuer() const { return kLaneIssue ? lane < NSEG : lane == 0; }

  // The launch's wait limit and test hook (Geom::wait_polls, arm_extra).
  __device__ __forceinline__ void configure(const Geom& g) {
    lim = g.wait_polls ? g.wait_polls : kWaitLimit;
    extra = g.arm_extra;
  }

  // Barrier set-up and the first stages.  With the test hook on, stage 0 is
  // armed for `extra` bytes more than its copies bring, so that the wait of
  // iteration 0 runs out although every copy lands.
  __device__ __forceinline__ void start() {
    pdl_trigger();
    pdl_wait();
    if (lane == 0) {
      for (int st = 0; st < S; ++st) mbar_init(&bar[st], 1);
      fence_mbar_init();
    }
    __syncwarp();
    if (issuer())
      for (int k = 0; k < kAhead && k < nk; ++k) issue_at(k, k % S, k == 0 ? extra : 0u);
    __syncwarp();
  }

  // Refills the stage consumed in iteration k-1-KEEP with iteration
  // k+kAhead, then waits for iteration k and reads the lane's float4 of every
  // segment.
  __device__ __forceinline__ bool acquire(int k) {
    if (KEEP > 0) __syncwarp();  // the previous iteration's seg_back reads are done
    // Stages advance by one per iteration: cur = k % S, par = (k / S) & 1,
    // and iteration k + kAhead fills stage (k + kAhead) % S.
    cur = nxt;
    const uint32_t ph = par;
    if (++nxt == S) {
      nxt = 0;
      par ^= 1u;
    }
    if (k + kAhead < nk && issuer()) {
      fence_proxy_async();  // order the warp's reads of the old stage before the copy
      issue_at(k + kAhead, cur + kAhead < S ? cur + kAhead : cur + kAhead - S);
    }
    return __all_sync(kFull, mbar_wait(&bar[cur], ph, lim));
  }
  // Segment q of the stage of iteration (current - d), 1 <= d <= KEEP.
  __device__ __forceinline__ f4 seg_back(int q, int d) const {
    const int st = cur >= d ? cur - d : cur + S - d;
    const float4 t = *reinterpret_cast<const float4*>(buf + (st * NSEG + q) * kSegFloats + 4 * lane);
    f4 r;
    r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
    return r;
  }
  // The lane's float4 of segment q of the acquired stage.
  __device__ __forceinline__ f4 seg(int q) const {
    const float4 t = *reinterpret_cast<const float4*>(buf + (cur * NSEG + q) * kSegFloats + 4 * lane);
    f4 r;
    r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
    return r;
  }
  // All lanes have read the stage; it may be refilled.
  __device__ __forceinline__ void release() { __syncwarp(); }
  // After a failed wait at iteration k: wait (bounded) for the copies still
  // in flight so that none lands after the warp has left.  With the test
  // hook on, the wait of iteration 0 is the one that failed; its extra bytes
  // are taken back first, so that stage 0 completes when its copies land.
  __device__ __forceinline__ void drain(int k) {
    if (extra && k == 0 && lane == 0) mbar_complete_tx(&bar[0], extra);
    __syncwarp();
    for (int kk = k; kk <= k + kAhead && kk < nk; ++kk) (void)mbar_wait(&bar[kk % S], uint32_t(kk / S) & 1u, lim);
    __syncwarp();
  }
};

}  // namespace seiswg
