// fd_march.cuh -- pieces shared by the forward step kernels (fd_step.cu,
// fd_step2.cu): the warp's march over its (strip, chunk), source injection
// and receiver probes along a row, the row loaders, and launch helpers.
#pragma once

#include "fd_kernels.h"
#include "fd_pipe.cuh"

namespace seiswg {
namespace {

struct March {
  int lane, warp, strip, chunk, ib, ie;
  bool active;
};

__device__ __forceinline__ March march_of(const Geom& g, int gw) {
  March m;
  m.lane = threadIdx.x & 31;
  m.warp = threadIdx.x >> 5;
  m.strip = gw % g.nstrips;
  m.chunk = gw / g.nstrips;
  m.active = m.chunk < g.nchunks;
  m.ib = m.chunk * g.lx;
  m.ie = min(g.nx, m.ib + g.lx);
  return m;
}

// Adds the injections of row i (sources, or adjoint sources at receivers) to
// the lane's divergence values.  `ci` is the list cursor, advanced past row i.
// Element e of an f4 is selected with unrolled compares: a runtime index
// into a register array would move the whole array to local memory.
template <bool X, bool Y, bool Z>
__device__ __forceinline__ void inject_row(const InjectList& inj, int i, int c0, int& ci, f4& ds_x, f4& ds_y,
                                           f4& ds_z) {
  while (ci < inj.n && __ldg(&inj.list[ci].i) == i) {
    const int e = __ldg(&inj.list[ci].j) - c0;
    if (e >= 0 && e < 4) {
      const size_t o = size_t(__ldg(&inj.list[ci].row)) * inj.nt + inj.it;
      const float ax = X ? ld1(&inj.val_x[o]) : 0.0f;
      const float ay = Y ? ld1(&inj.val_y[o]) : 0.0f;
      const float az = Z ? ld1(&inj.val_z[o]) : 0.0f;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (q == e) {
          if (X) ds_x.v[q] += ax;
          if (Y) ds_y.v[q] += ay;
          if (Z) ds_z.v[q] += az;
        }
      }
    }
    ++ci;
  }
}

// A list cursor that also holds the row of its next entry, so that a row
// without entries costs one compare instead of a load.
struct Cursor {
  int c, row;
};

template <typename T>
__device__ __forceinline__ Cursor cursor_at(const T* __restrict__ list, int n, int i0) {
  Cursor k;
  k.c = lower_row(list, n, i0);
  k.row = k.c < n ? __ldg(&list[k.c].i) : 0x7fffffff;
  return k;
}

template <bool X, bool Y, bool Z>
__device__ __forceinline__ void inject_at(const InjectList& inj, int i, int c0, Cursor& cur, f4& ds_x, f4& ds_y,
                                          f4& ds_z) {
  if (cur.row != i) return;
  inject_row<X, Y, Z>(inj, i, c0, cur.c, ds_x, ds_y, ds_z);
  cur.row = cur.c < inj.n ? __ldg(&inj.list[cur.c].i) : 0x7fffffff;
}

__device__ __forceinline__ float pick4(const f4& a, int e) {
  float r = a.v[0];
#pragma unroll
  for (int q = 1; q < 4; ++q) r = (q == e) ? a.v[q] : r;
  return r;
}

// Integrates the displacement of the owned probes of row i and records it.
template <typename Pick>
__device__ __forceinline__ void probe_row(const ProbeList& pr, int i, const LaneCols& L, int& pi, float dt,
                                          Pick pick) {
  while (pi < pr.n && __ldg(&pr.list[pi].i) == i) {
    int j = __ldg(&pr.list[pi].j);
    int e = j - L.c0;
    if (e >= 0 && e < 4 && (L.own & (1 << e))) {
      int idx = __ldg(&pr.list[pi].idx);
      float v = pick(__ldg(&pr.list[pi].comp), e);
#ifdef SEISWG_COHERENT_LOADS
      float u = __ldcg(&pr.acc[idx]) + v * dt;  // af(F_U*, k, v * dt), fd2d.wgsl:270
#else
      float u = pr.acc[idx] + v * dt;  // af(F_U*, k, v * dt), fd2d.wgsl:270
#endif
      pr.acc[idx] = u;
      pr.hist[size_t(idx) * pr.nt + pr.it] = u;
    }
    ++pi;
  }
}

template <typename Pick>
__device__ __forceinline__ void probe_at(const ProbeList& pr, int i, const LaneCols& L, Cursor& cur, float dt,
                                         Pick pick) {
  if (cur.row != i) return;
  probe_row(pr, i, L, cur.c, dt, pick);
  cur.row = cur.c < pr.n ? __ldg(&pr.list[cur.c].i) : 0x7fffffff;
}

__device__ __forceinline__ void flag_timeout(int* err) {
  if ((threadIdx.x & 31) == 0 && err) atomicOr(err, kErrWaitTimeout);
}

template <int NSEG>
struct DirectL : DirectRows<NSEG> {
  using SegsT = Segs<NSEG>;
  static constexpr uint32_t kStageBytes = 0;
  using DirectRows<NSEG>::DirectRows;
};

template <int NSEG>
struct BulkL : BulkRows<NSEG, kPipeStages> {
  using SegsT = Segs<NSEG>;
  using BulkRows<NSEG, kPipeStages>::BulkRows;
};

// The warp's loader over its slice of shared memory (warp_slice).
template <class Loader>
__device__ __forceinline__ Loader make_loader(const typename Loader::SegsT& segs, const Geom& g, const March& m,
                                              const LaneCols& L, unsigned char* slice) {
  float* buf = nullptr;
  uint64_t* bar = nullptr;
  if (Loader::kStages > 0) slice_ring<Loader>(slice, buf, bar);
  return Loader(segs, size_t(g.ld), L.c0, m.ib, m.lane, buf, bar, m.ie - m.ib + 3);
}


unsigned blocks_for(const Geom& g) {
  long warps = long(g.nstrips) * g.nchunks;
  return unsigned((warps + kStepWarps - 1) / kStepWarps);
}

template <class L>
size_t smem_for() {
  return L::kStages ? size_t(kStepWarps) * L::smem_bytes_per_warp() : 0;
}

// Launches a step or reverse kernel of kStepWarps warps per CTA; with pdl
// it is allowed to start while the previous launch in the stream finishes
// (its loaders wait for that launch, pdl_wait).
template <typename... P, typename... A>
cudaError_t launch_step(void (*kernel)(P...), bool pdl, unsigned blocks, size_t smem, cudaStream_t s,
                        A&&... args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(kStepWarps * 32);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<A&&>(args)...);
}

template <typename K>
cudaError_t prepare_kernel(K kernel, size_t smem) {
  // Opt in to more than 48 KB of dynamic shared memory.
  if (smem > 48 * 1024)
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  return cudaSuccess;
}

}  // namespace
}  // namespace seiswg
