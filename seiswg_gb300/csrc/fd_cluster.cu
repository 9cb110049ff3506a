// fd_cluster.cu -- whole forward runs of small SH grids inside one thread
// block cluster.
//
// When the state and the material of a grid fit in the shared memory of one
// cluster (up to 16 CTAs x 227 KB; the 200 x 200 SH example needs 0.8 MB), the
// cluster keeps the wavefield on chip for the whole run: CTA c owns a block of
// rows, a time step is a velocity phase and a stress phase over the CTA's
// cells (a thread handles four consecutive columns), and the two rows next to
// a block come from the neighbouring CTAs, which store their boundary rows
// into this CTA's shared memory (distributed shared memory) as they compute
// them.  A cluster barrier separates the phases; there is one launch per run
// instead of one per step, and no HBM traffic between steps.
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

__global__ void __launch_bounds__(kClusterThreads, 1) sh_cluster_kernel(const ShCluster p) {
  extern __shared__ __align__(16) float sm[];
  cg::cluster_group cl = cg::this_cluster();
  const int rank = int(cl.block_rank());
  const int nblk = int(cl.num_blocks());
  const int R = p.rows, nz = p.nz, nx = p.nx;
  const int P = cluster_pitch(nz), nz4 = (nz + 3) / 4;
  const int r0 = rank * R, r1 = min(nx, r0 + R);
  const int nrow = max(0, r1 - r0);
  const int items = nrow * nz4;  // float4 items of the CTA's rows
  // Planes of (R + 4) rows: vy and sxy use two halo rows above and below,
  // filled by the neighbouring CTAs; szy, 1/rho and mu the CTA's rows only.
  // Column j of local row lr is at plane[(lr + 2) * P + 4 + j].
  const int plane = (R + 4) * P;
  float* vy = sm + 2 * P + 4;
  float* sxy = sm + plane + 2 * P + 4;
  float* szy = sm + 2 * plane + 2 * P + 4;
  float* bu = sm + 3 * plane + 2 * P + 4;   // 1/rho
  float* mu = sm + 4 * plane + 2 * P + 4;
  float* tx = sm + 5 * plane;               // taper factor of each own row
  float* tb = tx + (R + 3) / 4 * 4;         // column factors (16-byte aligned)
  float* tt = tb + P;
  const int smem_floats = 5 * plane + (R + 3) / 4 * 4 + 2 * P;
  const int tid = threadIdx.x, nth = blockDim.x;
  const ptrdiff_t ld = p.ld;
  const float rn4 = 1.0f / float(nz4);
  // Item q -> (local row, first column): q / nz4 by a float reciprocal and
  // one correction step (q < 2^16 here).
  auto split = [&](int q, int& li, int& j) {
    li = __float2int_rz(__int2float_rn(q) * rn4);
    int c = q - li * nz4;
    if (c < 0) { --li; c += nz4; } else if (c >= nz4) { ++li; c -= nz4; }
    j = 4 * c;
  };
  const bool up = rank > 0, down = rank + 1 < nblk && r1 < nx;
  float* vy_up = up ? cl.map_shared_rank(vy, rank - 1) : nullptr;
  float* vy_dn = down ? cl.map_shared_rank(vy, rank + 1) : nullptr;
  float* sx_up = up ? cl.map_shared_rank(sxy, rank - 1) : nullptr;
  float* sx_dn = down ? cl.map_shared_rank(sxy, rank + 1) : nullptr;
  auto at4 = [&](float* f, int lr, int j) { return reinterpret_cast<float4*>(f + lr * P + j); };
  // Boundary rows into the neighbours' halos: vy rows 0, 1 up (as R, R + 1)
  // and R - 1 down (as -1); sxy row 0 up (as R) and R - 2, R - 1 down (as
  // -2, -1).
  auto push_vy = [&](int li, int j, float4 v) {
    if (up && li < 2) *at4(vy_up, R + li, j) = v;
    if (down && li == R - 1) *at4(vy_dn, -1, j) = v;
  };
  auto push_sx = [&](int li, int j, float4 v) {
    if (up && li == 0) *at4(sx_up, R, j) = v;
    if (down && li >= R - 2) *at4(sx_dn, li - R, j) = v;
  };

  for (int q = tid; q < smem_floats; q += nth) sm[q] = 0.0f;
  cl.sync();  // every CTA's memory is zero before any neighbour writes into it
  for (int q = tid; q < items; q += nth) {
    int li, j;
    split(q, li, j);
    const ptrdiff_t g = ptrdiff_t(r0 + li) * ld + j;
    for (int e = 0; e < 4 && j + e < nz; ++e) {
      vy[li * P + j + e] = p.vy0[g + e];
      sxy[li * P + j + e] = p.sxy0[g + e];
      szy[li * P + j + e] = p.szy0[g + e];
      bu[li * P + j + e] = p.rho[g + e];
      mu[li * P + j + e] = p.mu[g + e];
    }
    push_vy(li, j, *at4(vy, li, j));
    push_sx(li, j, *at4(sxy, li, j));
  }
  for (int q = tid; q < R; q += nth) tx[q] = (r0 + q < nx) ? p.taper_x[r0 + q] : 1.0f;
  for (int q = tid; q < nz; q += nth) {
    tb[q] = p.taper_zb[q];
    tt[q] = p.taper_zt[q];
  }
  // The injections and probes of the CTA's rows (lists sorted by row).
  int s_lo = 0, s_hi = 0, p_lo = 0, p_hi = 0;
  while (s_lo < p.inj.n && p.inj.list[s_lo].i < r0) ++s_lo;
  s_hi = s_lo;
  while (s_hi < p.inj.n && p.inj.list[s_hi].i < r1) ++s_hi;
  while (p_lo < p.probes.n && p.probes.list[p_lo].i < r0) ++p_lo;
  p_hi = p_lo;
  while (p_hi < p.probes.n && p.probes.list[p_hi].i < r1) ++p_hi;
  cl.sync();

  const float dt = p.dt, rdx = p.rdx, rdz = p.rdz;
  int snap_q = p.snap_first;

  for (int it = p.it0; it < p.it1; ++it) {
    // Velocity: div_sy, source, add_vy (fd2d.wgsl:247-270).
    for (int q = tid; q < items; q += nth) {
      int li, j;
      split(q, li, j);
      const int i = r0 + li;
      const bool xb = i >= 2 && i < nx - 2;
      const float4 x0 = *at4(sxy, li - 2, j), x1 = *at4(sxy, li - 1, j), x2 = *at4(sxy, li, j),
                   x3 = *at4(sxy, li + 1, j);
      const float* zr = szy + li * P + j;
      const float4 z = *reinterpret_cast<const float4*>(zr);
      const float2 zl = *reinterpret_cast<const float2*>(zr - 2);
      const float zs[7] = {zl.x, zl.y, z.x, z.y, z.z, z.w, zr[4]};  // columns j-2 .. j+4
      const float4 b4 = *reinterpret_cast<const float4*>(tb + j), t4 = *reinterpret_cast<const float4*>(tt + j);
      const float4 bu4 = *at4(bu, li, j);
      const float4 vo = *at4(vy, li, j);
      const float txi = tx[li];
      float out[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int c = j + e;
        float ds = xb ? fd4c(v4(x0, e), v4(x1, e), v4(x2, e), v4(x3, e), rdx) : 0.0f;
        const float dz = (c >= 2 && c < nz - 2) ? fd4c(zs[e], zs[e + 1], zs[e + 2], zs[e + 3], rdz) : 0.0f;
        ds = ds + dz;
        if (s_hi > s_lo)  // only CTAs with sources in their rows look them up
          for (int s = s_lo; s < s_hi; ++s)
            if (p.inj.list[s].i == i && p.inj.list[s].j == c)
              ds += p.inj.val_y[size_t(p.inj.list[s].row) * p.inj.nt + it];
        const float b = (txi * v4(b4, e)) * v4(t4, e);
        out[e] = b * (v4(vo, e) + dt * ds * v4(bu4, e));
      }
      const float4 vn = make_float4(out[0], out[1], out[2], out[3]);
      *at4(vy, li, j) = vn;
      push_vy(li, j, vn);
    }
    cl.sync();
    // Probes (fd2d.wgsl:270), then the stress: div_vy, add_sy_sh (fd2d.wgsl:276-290).
    for (int k = p_lo + tid; k < p_hi; k += nth) {
      const Probe pr = p.probes.list[k];
      const float u = p.probes.acc[pr.idx] + vy[(pr.i - r0) * P + pr.j] * dt;
      p.probes.acc[pr.idx] = u;
      p.probes.hist[size_t(pr.idx) * p.probes.nt + it] = u;
    }
    const bool snap = p.snap && it > 0 && it % p.snap_every == 0;
    for (int q = tid; q < items; q += nth) {
      int li, j;
      split(q, li, j);
      const int i = r0 + li;
      const bool xf = i >= 1 && i < nx - 2;
      const float4 a0 = *at4(vy, li - 1, j), a1 = *at4(vy, li, j), a2 = *at4(vy, li + 1, j),
                   a3 = *at4(vy, li + 2, j);
      const float* vr = vy + li * P + j;
      const float2 vn = *reinterpret_cast<const float2*>(vr + 4);
      const float vs[7] = {vr[-1], a1.x, a1.y, a1.z, a1.w, vn.x, vn.y};  // columns j-1 .. j+5
      const float4 mu4 = *at4(mu, li, j);
      const float4 sx = *at4(sxy, li, j), sz = *at4(szy, li, j);
      float ox[4], oz[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const int c = j + e;
        const float gx = xf ? fd4c(v4(a0, e), v4(a1, e), v4(a2, e), v4(a3, e), rdx) : 0.0f;
        const float gz = (c >= 1 && c < nz - 2) ? fd4c(vs[e], vs[e + 1], vs[e + 2], vs[e + 3], rdz) : 0.0f;
        const float mu_dt = v4(mu4, e) * dt;
        ox[e] = v4(sx, e) + mu_dt * gx;
        oz[e] = v4(sz, e) + mu_dt * gz;
      }
      const float4 sxn = make_float4(ox[0], ox[1], ox[2], ox[3]);
      *at4(sxy, li, j) = sxn;
      *at4(szy, li, j) = make_float4(oz[0], oz[1], oz[2], oz[3]);
      push_sx(li, j, sxn);
      if (snap)
        for (int e = 0; e < 4 && j + e < nz; ++e)
          p.snap[size_t(snap_q) * p.snap_stride + ptrdiff_t(i) * ld + j + e] = v4(a1, e);
    }
    if (snap) ++snap_q;
    cl.sync();
  }

  for (int q = tid; q < items; q += nth) {
    int li, j;
    split(q, li, j);
    const ptrdiff_t g = ptrdiff_t(r0 + li) * ld + j;
    for (int e = 0; e < 4 && j + e < nz; ++e) {
      p.vy1[g + e] = vy[li * P + j + e];
      p.sxy1[g + e] = sxy[li * P + j + e];
      p.szy1[g + e] = szy[li * P + j + e];
    }
  }
}

size_t sh_cluster_smem_bytes(int nx, int nz, int ctas) {
  const int rows = (nx + ctas - 1) / ctas;
  const int P = cluster_pitch(nz);
  return (size_t(5) * (rows + 4) * P + (rows + 3) / 4 * 4 + 2 * size_t(P)) * sizeof(float);
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
  // block but the last needs two rows (the neighbours supply two halo rows).
  for (int ctas : {16, 8, 4, 2}) {
    if ((nx + ctas - 1) / ctas < 2) continue;
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
