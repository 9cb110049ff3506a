// fd_tma.cuh -- the per-warp row ring of fd_pipe.cuh filled by 3-D tensor
// copies (cp.async.bulk.tensor.3d) instead of one bulk copy per segment.
//
// A tensor map describes several padded fields (columns ld, rows nx + 2
// kHaloRows, fields at a uniform stride) with boxes of 128 columns x 1 row x
// n fields, so that one copy fetches the row of n fields that lie next to
// each other in memory.  Lane 0 issues a stage's copies (Plan::issue); the
// barrier, the bounded waits and the stage bookkeeping are those of
// BulkRows.
#pragma once

#include "fd_kernels.h"
#include "fd_pipe.cuh"

namespace seiswg {
namespace {

// The same ring filled by 3-D tensor copies, issued by lane 0: one copy per
// group of fields that lie next to each other in memory and share a row
// offset (`Plan::issue`).  Coordinates are of the padded fields (halo columns
// and rows included), so every x is the warp's first column plus kHaloCols:
// a multiple of 4 floats, as the tensor copy requires.
__device__ __forceinline__ void tma3(float* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* b) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(b))
      : "memory");
}

// A map given as a kernel parameter (its address) or as a pointer to a map in
// global memory (the batch keeps one table per job there).
__device__ __forceinline__ const CUtensorMap* tmap(const CUtensorMap& m) { return &m; }
__device__ __forceinline__ const CUtensorMap* tmap(const CUtensorMap* m) { return m; }

// Maps: a struct with the plan's named maps, as CUtensorMap members (kernel
// parameter) or as pointers to maps in global memory.
template <class Plan, int S_, int KEEP_, class Maps = typename Plan::Maps>
struct TmaRows {
  static constexpr int S = S_, KEEP = KEEP_, kAhead = S - 1 - KEEP, NSEG = Plan::NSEG;
  static constexpr int kStages = S;
  static constexpr uint32_t kStageBytes = NSEG * kSegFloats * sizeof(float);
  using SegsT = Segs<NSEG>;
  const Maps* tm = nullptr;
  int x0, ib, lane, nk, cur, nxt;
  uint32_t par;
  float* buf;
  uint64_t* bar;
  unsigned lim = kWaitLimit;  // polls of a bounded wait
  uint32_t extra = 0;         // test hook: bytes armed on stage 0 beyond its copies
  __device__ TmaRows(const SegsT&, size_t, int c0_, int ib_, int lane_, float* buf_, uint64_t* bar_, int nk_)
      : x0(c0_ - 4 * lane_ + kHaloCols), ib(ib_), lane(lane_), nk(nk_), cur(0), nxt(0), par(0), buf(buf_),
        bar(bar_) {}
  __device__ __forceinline__ void issue_at(int k, int st, uint32_t add = 0) {
    mbar_expect_tx(&bar[st], kStageBytes + add);
    Plan::issue(buf + st * NSEG * kSegFloats, tm, x0, ib - 1 + k + kHaloRows, &bar[st]);
  }
  __device__ __forceinline__ void configure(const Geom& g) {
    lim = g.wait_polls ? g.wait_polls : kWaitLimit;
    extra = g.arm_extra;
  }
  __device__ __forceinline__ void start() {
    pdl_trigger();
    pdl_wait();
    if (lane == 0) {
      for (int st = 0; st < S; ++st) mbar_init(&bar[st], 1);
      fence_mbar_init();
      for (int k = 0; k < kAhead && k < nk; ++k) issue_at(k, k % S, k == 0 ? extra : 0u);
    }
    __syncwarp();
  }
  __device__ __forceinline__ bool acquire(int k) {
    __syncwarp();  // the previous iteration's seg_back reads are done
    cur = nxt;
    const uint32_t ph = par;
    if (++nxt == S) {
      nxt = 0;
      par ^= 1u;
    }
    if (k + kAhead < nk && lane == 0) {
      fence_proxy_async();
      issue_at(k + kAhead, cur + kAhead < S ? cur + kAhead : cur + kAhead - S);
    }
    return __all_sync(kFull, mbar_wait(&bar[cur], ph, lim));
  }
  __device__ __forceinline__ f4 seg_back(int q, int d) const {
    const int st = cur >= d ? cur - d : cur + S - d;
    const float4 t = *reinterpret_cast<const float4*>(buf + (st * NSEG + q) * kSegFloats + 4 * lane);
    f4 r;
    r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
    return r;
  }
  __device__ __forceinline__ f4 seg(int q) const {
    const float4 t = *reinterpret_cast<const float4*>(buf + (cur * NSEG + q) * kSegFloats + 4 * lane);
    f4 r;
    r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
    return r;
  }
  __device__ __forceinline__ void release() { __syncwarp(); }
  // As BulkRows::drain: the test hook's extra bytes are taken back first.
  __device__ __forceinline__ void drain(int k) {
    if (extra && k == 0 && lane == 0) mbar_complete_tx(&bar[0], extra);
    __syncwarp();
    for (int kk = k; kk <= k + kAhead && kk < nk; ++kk) (void)mbar_wait(&bar[kk % S], uint32_t(kk / S) & 1u, lim);
    __syncwarp();
  }
  __host__ __device__ static constexpr size_t smem_bytes_per_warp() {
    return warp_ring_bytes(S, kStageBytes);
  }
};
}  // namespace
}  // namespace seiswg
