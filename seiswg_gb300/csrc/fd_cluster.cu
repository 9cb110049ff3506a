// fd_cluster.cu -- whole forward runs of small SH grids inside one thread
// block cluster.
//
// When the state and the material of a grid fit in the shared memory of one
// cluster (up to 16 CTAs x 227 KB; the 200 x 200 SH example needs 1.5 MB), the
// cluster keeps the wavefield on chip for the whole run: CTA c owns a block of
// rows, a time step is a velocity phase and a stress phase over the CTA's
// cells (a thread handles four consecutive columns).  The velocity phase also
// recomputes the rows next to the block (the same expression on the same
// inputs as the neighbour that owns them); the stresses those rows need come
// from the neighbouring CTAs, which store their boundary rows into this CTA's
// shared memory (distributed shared memory) as they compute them.  One
// cluster barrier per step; one launch per run instead of one per step, and
// no HBM traffic between steps.
//
// The update of every cell is the one-step kernel's expression for expression
// (fd_step.cu, sh_march; built with -fmad=false), and sources and probes are
// applied in the same order, so the results are the one-step kernel's bits.
#include <cooperative_groups.h>

#include "fd_kernels.h"

namespace cg = cooperative_groups;

namespace seiswg {

namespace {

// fd2d.wgsl:155-156, the division by 8*d as a multiply by its reciprocal (as
// fd_common.cuh's fd4).
__device__ __forceinline__ float fd4c(float a, float b, float c, float d, float r) {
  return (9.0f * (c - b) - (d - a)) * r;
}

__device__ __forceinline__ float v4(const float4& a, int e) {
  return e == 0 ? a.x : e == 1 ? a.y : e == 2 ? a.z : a.w;
}

}  // namespace

// Row pitch in shared memory: 4 zero columns on each side of the row (the
// z stencils of the edge columns read them, masked), a multiple of 4 floats.
__host__ __device__ __forceinline__ int cluster_pitch(int nz) { return (nz + 3) / 4 * 4 + 8; }

// Shared-memory layout of a CTA that owns R rows, in floats (planes of
// pitch P; row li of a plane at base + li * P, columns from +4):
//   vy              rows [-1, R+2)  own rows and the rows next to them,
//                                   recomputed here (redundant with the
//                                   neighbours, bit for bit the same)
//   sxy[2], szy[2]  rows [-3, R+3) and [-1, R+2), one plane per step parity:
//                                   own rows written by this CTA, the other
//                                   rows stored by the neighbours
//   1/rho           rows [-1, R+2),  mu * dt rows [0, R)
//   taper product   rows [-1, R+2)  (row factor x column factors, per cell)
//   taper of rows [-1, R+2), then the two column tapers (set-up only);
//   the CTA's injections (row, column) and their values of this step and the
//   next, and its probes' displacement accumulators.
struct ClusterLayout {
  int P, R, vrows, srows, off_vy, off_sx, off_sz, off_bu, off_mu, off_bt, off_tx, off_tb, off_src, off_val, off_acc;
  int floats;
  __host__ __device__ ClusterLayout(int nz, int rows) {
    P = cluster_pitch(nz);
    R = rows;
    vrows = R + 3;
    srows = R + 6;
    off_vy = 0;
    off_sx = off_vy + vrows * P;
    off_sz = off_sx + 2 * srows * P;
    off_bu = off_sz + 2 * vrows * P;
    off_mu = off_bu + vrows * P;
    off_bt = off_mu + R * P;
    off_tx = off_bt + vrows * P;
    off_tb = off_tx + (R + 3 + 3) / 4 * 4;
    off_src = off_tb + 2 * P;
    off_val = off_src + 2 * kClusterSources;
    off_acc = off_val + 2 * kClusterSources;
    floats = off_acc + kClusterProbes;
  }
};

// One time step per iteration with ONE cluster barrier: the velocity phase
// covers the CTA's rows and the three rows next to them (-1, R, R+1), from
// stresses of rows -3 .. R+2; the stress phase covers the CTA's rows and
// stores its first three / last three rows of sxy (first two / last of szy)
// into the neighbours' planes of the next parity.  A neighbour reads that
// parity only after the barrier that ends the step, and the planes it stores
// into this step are read in the step after that, so the barrier orders
// every store before the loads that read it and after the loads of the data
// it replaces.
__global__ void __launch_bounds__(kClusterThreads, 1) sh_cluster_kernel(const ShCluster p) {
  extern __shared__ __align__(16) float sm[];
  cg::cluster_group cl = cg::this_cluster();
  const int rank = int(cl.block_rank());
  const int nblk = int(cl.num_blocks());
  const int R = p.rows, nz = p.nz, nx = p.nx;
  const ClusterLayout Ly(nz, R);
  const int P = Ly.P, nz4 = (nz + 3) / 4;
  const int r0 = rank * R, r1 = min(nx, r0 + R);
  const int nrow = max(0, r1 - r0);
  const int items = nrow * nz4;           // float4 items of the CTA's rows
  const int vitems = Ly.vrows * nz4;      // ... of rows [-1, R+2)
  float* vy = sm + Ly.off_vy + P + 4;
  float* const sx0 = sm + Ly.off_sx + 3 * P + 4;  // sxy planes of parity 0 and 1
  float* const sx1 = sx0 + Ly.srows * P;
  float* const sz0 = sm + Ly.off_sz + P + 4;      // szy planes
  float* const sz1 = sz0 + Ly.vrows * P;
  float* bu = sm + Ly.off_bu + P + 4;     // 1/rho
  float* mu = sm + Ly.off_mu + 4;         // mu, then mu * dt
  float* bt = sm + Ly.off_bt + P + 4;     // taper product of each cell
  float* tx = sm + Ly.off_tx + 1;         // taper factor of rows -1 .. R+1
  float* tb = sm + Ly.off_tb;             // column factors (16-byte aligned)
  float* tt = tb + P;
  int* src_at = reinterpret_cast<int*>(sm + Ly.off_src);  // (local row, column) of injection s
  float* src_val = sm + Ly.off_val;                       // [2][kClusterSources], by step parity
  float* acc = sm + Ly.off_acc;                           // displacement of local probe k
  const int tid = threadIdx.x, nth = blockDim.x;
  const ptrdiff_t ld = p.ld;
  const float rn4 = 1.0f / float(nz4);
  // Item q -> (row, first column): q / nz4 by a float reciprocal and one
  // correction step (q < 2^16 here).
  auto split = [&](int q, int& li, int& j) {
    li = __float2int_rz(__int2float_rn(q) * rn4);
    int c = q - li * nz4;
    if (c < 0) { --li; c += nz4; } else if (c >= nz4) { ++li; c -= nz4; }
    j = 4 * c;
  };
  const bool up = rank > 0, down = rank + 1 < nblk && r1 < nx;
  // The neighbours' planes (same offsets in their shared memory).
  float* const sx0_up = up ? cl.map_shared_rank(sx0, rank - 1) : nullptr;
  float* const sx1_up = up ? cl.map_shared_rank(sx1, rank - 1) : nullptr;
  float* const sz0_up = up ? cl.map_shared_rank(sz0, rank - 1) : nullptr;
  float* const sz1_up = up ? cl.map_shared_rank(sz1, rank - 1) : nullptr;
  float* const sx0_dn = down ? cl.map_shared_rank(sx0, rank + 1) : nullptr;
  float* const sx1_dn = down ? cl.map_shared_rank(sx1, rank + 1) : nullptr;
  float* const sz0_dn = down ? cl.map_shared_rank(sz0, rank + 1) : nullptr;
  float* const sz1_dn = down ? cl.map_shared_rank(sz1, rank + 1) : nullptr;
  auto at4 = [&](float* f, int lr, int j) { return reinterpret_cast<float4*>(f + lr * P + j); };
  auto in4 = [&](const float* f, int lr, int j) { return *reinterpret_cast<const float4*>(f + lr * P + j); };

  for (int q = tid; q < Ly.floats; q += nth) sm[q] = 0.0f;
  __syncthreads();
  // Rows [-3, R+3) of sxy, [-1, R+2) of vy, szy and 1/rho, the own rows of
  // mu: whatever of them lies in the grid.
  auto load_rows = [&](float* dst, const float* src, int lo, int hi) {
    const int n = (hi - lo) * nz4;
    for (int q = tid; q < n; q += nth) {
      int li, j;
      split(q, li, j);
      li += lo;
      const int i = r0 + li;
      if (i < 0 || i >= nx) continue;
      const ptrdiff_t g = ptrdiff_t(i) * ld + j;
      for (int e = 0; e < 4 && j + e < nz; ++e) dst[li * P + j + e] = src[g + e];
    }
  };
  load_rows(sx0, p.sxy0, -3, R + 3);
  load_rows(vy, p.vy0, -1, R + 2);
  load_rows(sz0, p.szy0, -1, R + 2);
  load_rows(bu, p.rho, -1, R + 2);
  load_rows(mu, p.mu, 0, nrow);
  for (int q = tid; q < R + 3; q += nth) {
    const int i = r0 + q - 1;
    tx[q - 1] = (i >= 0 && i < nx) ? p.taper_x[i] : 1.0f;
  }
  for (int q = tid; q < nz; q += nth) {
    tb[q] = p.taper_zb[q];
    tt[q] = p.taper_zt[q];
  }
  __syncthreads();
  // Per-cell factors of the step, formed once with the step kernel's
  // operations: (row taper x bottom taper) x top taper, and mu * dt.
  const float dt = p.dt;
  for (int q = tid; q < Ly.vrows * nz; q += nth) {
    const int li = q / nz - 1, c = q - (li + 1) * nz;
    bt[li * P + c] = (tx[li] * tb[c]) * tt[c];
  }
  for (int q = tid; q < nrow * nz; q += nth) {
    const int li = q / nz, c = q - li * nz;
    mu[li * P + c] = mu[li * P + c] * dt;
  }
  // The injections of rows [r0-1, r0+R+2) and the probes of the own rows
  // (lists sorted by row).
  int s_lo = 0, s_hi = 0, p_lo = 0, p_hi = 0;
  while (s_lo < p.inj.n && p.inj.list[s_lo].i < r0 - 1) ++s_lo;
  s_hi = s_lo;
  while (s_hi < p.inj.n && p.inj.list[s_hi].i < r0 + R + 2) ++s_hi;
  while (p_lo < p.probes.n && p.probes.list[p_lo].i < r0) ++p_lo;
  p_hi = p_lo;
  while (p_hi < p.probes.n && p.probes.list[p_hi].i < r1) ++p_hi;
  const int ns = s_hi - s_lo, np = p_hi - p_lo;
  // Injection values and probe accumulators live in shared memory, so that
  // no global load sits between two barriers: thread s < ns loads the value
  // of injection s for the next step during the stress phase.
  size_t src_off = 0;
  if (tid < ns) {
    const Inject& in = p.inj.list[s_lo + tid];
    src_at[2 * tid] = in.i - r0;
    src_at[2 * tid + 1] = in.j;
    src_off = size_t(in.row) * p.inj.nt;
    src_val[tid] = p.inj.val_y[src_off + p.it0];
  }
  for (int k = tid; k < np; k += nth) acc[k] = p.probes.acc[p.probes.list[p_lo + k].idx];
  // Every CTA's memory is zero and loaded before any neighbour stores into it.
  cl.sync();

  const float rdx = p.rdx, rdz = p.rdz;
  int snap_q = p.snap_first;
  int par = 0;  // plane of sxy and szy holding the stresses before the step

  // An item is packed as ((row + 1) << 16) | first column with flags: bit 0
  // the row is a grid row, bit 1 its x derivative is taken, bits 2..5 the z
  // derivative of each of its four columns.  A thread's first item of each
  // phase is decoded once, before the time loop; further items (grids with
  // more items than threads) are decoded where they are used.
  auto vdecode = [&](int q, int& pk, int& fl) {
    int li, j;
    split(q, li, j);
    li -= 1;
    const int i = r0 + li;
    fl = (i >= 0 && i < nx) ? 1 : 0;
    if (i >= 2 && i < nx - 2) fl |= 2;
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (j + e >= 2 && j + e < nz - 2) fl |= 4 << e;
    pk = ((li + 1) << 16) | j;
  };
  auto sdecode = [&](int q, int& pk, int& fl) {
    int li, j;
    split(q, li, j);
    const int i = r0 + li;
    fl = 1;
    if (i >= 1 && i < nx - 2) fl |= 2;
#pragma unroll
    for (int e = 0; e < 4; ++e)
      if (j + e >= 1 && j + e < nz - 2) fl |= 4 << e;
    pk = ((li + 1) << 16) | j;
  };
  int vpk = 0, vfl = 0, spk = 0, sfl = 0;
  if (tid < vitems) vdecode(tid, vpk, vfl);
  if (tid < items) sdecode(tid, spk, sfl);

  for (int it = p.it0; it < p.it1; ++it) {
    const float* val = src_val + par * kClusterSources;  // injection values of step it
    const float* sxy = par ? sx1 : sx0;
    const float* szy = par ? sz1 : sz0;
    float* const sxn_p = par ? sx0 : sx1;  // the stresses after the step
    float* const szn_p = par ? sz0 : sz1;
    float* const sxn_up = par ? sx0_up : sx1_up;
    float* const szn_up = par ? sz0_up : sz1_up;
    float* const sxn_dn = par ? sx0_dn : sx1_dn;
    float* const szn_dn = par ? sz0_dn : sz1_dn;
    // Velocity of rows -1 .. R+1: div_sy, source, add_vy (fd2d.wgsl:247-270).
    auto velocity = [&](int pk, int fl) {
      const int li = (pk >> 16) - 1, j = pk & 0xffff;
      const int o = li * P + j;
      const float4 x0 = in4(sxy + o, -2, 0), x1 = in4(sxy + o, -1, 0), x2 = in4(sxy + o, 0, 0),
                   x3 = in4(sxy + o, 1, 0);
      const float* zr = szy + o;
      const float4 z = *reinterpret_cast<const float4*>(zr);
      const float2 zl = *reinterpret_cast<const float2*>(zr - 2);
      const float zs[7] = {zl.x, zl.y, z.x, z.y, z.z, z.w, zr[4]};  // columns j-2 .. j+4
      const float4 b4 = in4(bt + o, 0, 0);
      const float4 bu4 = in4(bu + o, 0, 0);
      const float4 vo = in4(vy + o, 0, 0);
      float out[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        float ds = (fl & 2) ? fd4c(v4(x0, e), v4(x1, e), v4(x2, e), v4(x3, e), rdx) : 0.0f;
        const float dz = (fl & (4 << e)) ? fd4c(zs[e], zs[e + 1], zs[e + 2], zs[e + 3], rdz) : 0.0f;
        ds = ds + dz;
        for (int s = 0; s < ns; ++s)  // in list order, as the step kernel
          if (src_at[2 * s] == li && src_at[2 * s + 1] == j + e) ds += val[s];
        out[e] = v4(b4, e) * (v4(vo, e) + dt * ds * v4(bu4, e));
      }
      *reinterpret_cast<float4*>(vy + o) = make_float4(out[0], out[1], out[2], out[3]);
    };
    if (vfl & 1) velocity(vpk, vfl);
    for (int q = tid + nth; q < vitems; q += nth) {
      int pk, fl;
      vdecode(q, pk, fl);
      if (fl & 1) velocity(pk, fl);
    }
    __syncthreads();
    // Probes (fd2d.wgsl:270), then the stress of the own rows: div_vy,
    // add_sy_sh (fd2d.wgsl:276-290), into the other parity's planes.
    const float next_val = (tid < ns && it + 1 < p.it1) ? p.inj.val_y[src_off + it + 1] : 0.0f;
    for (int k = tid; k < np; k += nth) {
      const Probe pr = p.probes.list[p_lo + k];
      const float u = acc[k] + vy[(pr.i - r0) * P + pr.j] * dt;
      acc[k] = u;
      p.probes.hist[size_t(pr.idx) * p.probes.nt + it] = u;
    }
    const bool snap = p.snap && it > 0 && it % p.snap_every == 0;
    auto stress = [&](int pk, int fl) {
      const int li = (pk >> 16) - 1, j = pk & 0xffff;
      const int o = li * P + j;
      const float* vr = vy + o;
      const float4 a0 = in4(vr, -1, 0), a1 = in4(vr, 0, 0), a2 = in4(vr, 1, 0), a3 = in4(vr, 2, 0);
      const float2 vn = *reinterpret_cast<const float2*>(vr + 4);
      const float vs[7] = {vr[-1], a1.x, a1.y, a1.z, a1.w, vn.x, vn.y};  // columns j-1 .. j+5
      const float4 md = in4(mu + o, 0, 0);  // mu * dt
      const float4 sx = in4(sxy + o, 0, 0), sz = in4(szy + o, 0, 0);
      float ox[4], oz[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const float gx = (fl & 2) ? fd4c(v4(a0, e), v4(a1, e), v4(a2, e), v4(a3, e), rdx) : 0.0f;
        const float gz = (fl & (4 << e)) ? fd4c(vs[e], vs[e + 1], vs[e + 2], vs[e + 3], rdz) : 0.0f;
        ox[e] = v4(sx, e) + v4(md, e) * gx;
        oz[e] = v4(sz, e) + v4(md, e) * gz;
      }
      const float4 sxn = make_float4(ox[0], ox[1], ox[2], ox[3]);
      const float4 szn = make_float4(oz[0], oz[1], oz[2], oz[3]);
      *reinterpret_cast<float4*>(sxn_p + o) = sxn;
      *reinterpret_cast<float4*>(szn_p + o) = szn;
      // Rows 0..2 (sxy) and 0..1 (szy) are the upper neighbour's rows R..;
      // rows R-3.. (sxy) and R-1 (szy) the lower neighbour's rows -3.. .
      if (up && li < 3) *at4(sxn_up + o, R, 0) = sxn;
      if (up && li < 2) *at4(szn_up + o, R, 0) = szn;
      if (down && li >= R - 3) *at4(sxn_dn + o, -R, 0) = sxn;
      if (down && li == R - 1) *at4(szn_dn + o, -R, 0) = szn;
      if (snap)
        for (int e = 0; e < 4 && j + e < nz; ++e)
          p.snap[size_t(snap_q) * p.snap_stride + ptrdiff_t(r0 + li) * ld + j + e] = v4(a1, e);
    };
    if (sfl & 1) stress(spk, sfl);
    for (int q = tid + nth; q < items; q += nth) {
      int pk, fl;
      sdecode(q, pk, fl);
      stress(pk, fl);
    }
    if (snap) ++snap_q;
    if (tid < ns) src_val[(1 - par) * kClusterSources + tid] = next_val;
    par = 1 - par;
    cl.sync();
  }

  for (int k = tid; k < np; k += nth) p.probes.acc[p.probes.list[p_lo + k].idx] = acc[k];
  for (int q = tid; q < items; q += nth) {
    int li, j;
    split(q, li, j);
    const ptrdiff_t g = ptrdiff_t(r0 + li) * ld + j;
    for (int e = 0; e < 4 && j + e < nz; ++e) {
      p.vy1[g + e] = vy[li * P + j + e];
      p.sxy1[g + e] = (par ? sx1 : sx0)[li * P + j + e];
      p.szy1[g + e] = (par ? sz1 : sz0)[li * P + j + e];
    }
  }
}

size_t sh_cluster_smem_bytes(int nx, int nz, int ctas) {
  const int rows = (nx + ctas - 1) / ctas;
  return size_t(ClusterLayout(nz, rows).floats) * sizeof(float);
}

namespace {

// The kernel may use up to the opt-in shared memory per CTA and 16-CTA
// clusters; set once, so that Sims of different sizes never lower it.
int cluster_smem_optin() {
  static const int optin = [] {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
    if (cudaFuncSetAttribute(sh_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, v) != cudaSuccess)
      return 0;
    if (cudaFuncSetAttribute(sh_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess)
      cudaGetLastError();
    return v;
  }();
  return optin;
}

cudaLaunchConfig_t cluster_config(int ctas, size_t smem, cudaStream_t s, cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = dim3(kClusterThreads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  attr->id = cudaLaunchAttributeClusterDimension;
  attr->val.clusterDim.x = ctas;
  attr->val.clusterDim.y = 1;
  attr->val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}

}  // namespace

int sh_cluster_ctas(int nx, int nz) {
  const int optin = cluster_smem_optin();
  if (optin <= 0) {
    cudaGetLastError();
    return 0;
  }
  // More SMs per step where the hardware allows a 16-CTA cluster; every CTA
  // block but the last needs three rows (it stores its first and last three
  // rows into the neighbours' planes).
  for (int ctas : {16, 8, 4, 2}) {
    if ((nx + ctas - 1) / ctas < 3) continue;
    const size_t smem = sh_cluster_smem_bytes(nx, nz, ctas);
    if (smem > size_t(optin)) continue;
    cudaLaunchAttribute attr{};
    cudaLaunchConfig_t cfg = cluster_config(ctas, smem, nullptr, &attr);
    int clusters = 0;
    if (cudaOccupancyMaxActiveClusters(&clusters, sh_cluster_kernel, &cfg) == cudaSuccess && clusters >= 1)
      return ctas;
  }
  cudaGetLastError();
  return 0;
}

cudaError_t launch_sh_cluster(const ShCluster& p, int ctas, cudaStream_t s) {
  if (cluster_smem_optin() <= 0) return cudaErrorInvalidConfiguration;
  cudaLaunchAttribute attr{};
  cudaLaunchConfig_t cfg = cluster_config(ctas, sh_cluster_smem_bytes(p.nx, p.nz, ctas), s, &attr);
  return cudaLaunchKernelEx(&cfg, sh_cluster_kernel, p);
}

}  // namespace seiswg
