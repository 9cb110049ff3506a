// fd_batch.cu -- on-device misfit and adjoint source of grouped jobs.
//
// After a job's recording forward pass, each of its traces (component,
// receiver) is reduced by one thread: d^n from the probe history, J_trace =
// sum_n (tau_n (d^n - o^n))^2 with the cosine taper of solver.rs:442-459, and
// the reverse cumulative adjoint source dt * U^n, U^n = sum_{m >= n}
// 2 tau_m^2 (d^m - o^m), which the reverse sweep injects at the receiver.
// Sums run in double; the arithmetic matches seiswg_l2_misfit on the host.
#include <cmath>

#include "fd_kernels.h"

namespace seiswg {

namespace {

__global__ void grouped_misfit_kernel(const JobDesc* __restrict__ jobs, const GroupOp* __restrict__ ops) {
  const GroupOp op = ops[blockIdx.x];
  const JobDesc& J = jobs[op.job];
  const int ncomp = J.psv ? 2 : 1;
  const int ntr = ncomp * J.nrec;
  const int nt = J.nt;
  const double dt = double(J.dt);
  const double t_end = double(nt - 1) * dt, tw = t_end / 10.0, pi = 3.14159265358979323846;
  for (int tr = threadIdx.x; tr < ntr; tr += blockDim.x) {
    const int c = tr / J.nrec, r = tr - c * J.nrec;
    const int p = J.tr_idx[12 * r + (J.psv ? 1 + c : 0)];
    const float* d = J.probes.hist + size_t(p) * nt;
    const float* o = J.obs + size_t(tr) * nt;
    float* u = J.u_tab + size_t(tr) * nt;
    double sum = 0.0, acc = 0.0;
    for (int it = nt - 1; it >= 0; --it) {
      const double t = double(it) * dt;
      double tau = 1.0;
      if (t <= tw) tau = 0.5 + 0.5 * cos(pi * (tw - t) / tw);
      else if (t >= t_end - tw) tau = 0.5 + 0.5 * cos(pi * ((t_end - tw) - t) / tw);
      const double e = (double(d[it]) - double(o[it])) * tau;
      sum += e * e;
      acc += double(float(2.0 * e * tau));
      u[it] = float(dt * acc);
    }
    J.J[tr] = sum;
  }
}

}  // namespace

cudaError_t launch_grouped_misfit(const JobDesc* jobs, const GroupOp* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return cudaSuccess;
  grouped_misfit_kernel<<<nops, 128, 0, s>>>(jobs, ops);
  return cudaGetLastError();
}

}  // namespace seiswg
