// fd_batch.cu -- on-device misfit and adjoint source, of grouped jobs and of
// one problem.
//
// After a job's recording forward pass, each of its traces (component,
// receiver) is reduced by one thread: d^n from the probe history, J_trace =
// sum_n (tau_n (d^n - o^n))^2 with the cosine taper of solver.rs:442-459, and
// the reverse cumulative adjoint source dt * U^n, U^n = sum_{m >= n}
// 2 tau_m^2 (d^m - o^m), which the reverse sweep injects at the receiver
// (misfit_trace, fd_misfit.cuh).

#include "fd_misfit.cuh"

namespace seiswg {

namespace {

__global__ void grouped_misfit_kernel(const JobDesc* __restrict__ jobs, const GroupOp* __restrict__ ops) {
  const GroupOp op = ops[blockIdx.x];
  const JobDesc& J = jobs[op.job];
  const int ncomp = J.psv ? 2 : 1;
  const int ntr = ncomp * J.nrec;
  for (int tr = threadIdx.x; tr < ntr; tr += blockDim.x) {
    const int c = tr / J.nrec, r = tr - c * J.nrec;
    const int p = J.tr_idx[12 * r + (J.psv ? 1 + c : 0)];
    J.J[tr] = misfit_trace(J.probes.hist + size_t(p) * J.nt, J.obs + size_t(tr) * J.nt, J.u_tab + size_t(tr) * J.nt,
                           J.nt, double(J.dt));
  }
}

// One problem: traces already assembled as [5][nrec][nt] (components x, y,
// z, yi, yc); trace tr = c * nrec + r of the inverted components.
__global__ void sim_misfit_kernel(const float* __restrict__ syn, const float* __restrict__ obs,
                                  float* __restrict__ u_tab, double* __restrict__ J, int nrec, int nt, int psv,
                                  float dt) {
  const int ntr = (psv ? 2 : 1) * nrec;
  const int tr = blockIdx.x * blockDim.x + threadIdx.x;
  if (tr >= ntr) return;
  const int c = tr / nrec, r = tr - c * nrec;
  const int comp = psv ? (c == 0 ? 0 : 2) : 1;
  J[tr] = misfit_trace(syn + (size_t(comp) * nrec + r) * nt, obs + size_t(tr) * nt, u_tab + size_t(tr) * nt, nt,
                       double(dt));
}

}  // namespace

cudaError_t launch_grouped_misfit(const JobDesc* jobs, const GroupOp* ops, int nops, cudaStream_t s) {
  if (nops <= 0) return cudaSuccess;
  grouped_misfit_kernel<<<nops, 128, 0, s>>>(jobs, ops);
  return cudaGetLastError();
}

cudaError_t launch_sim_misfit(const float* syn, const float* obs, float* u_tab, double* J, int nrec, int nt,
                              bool psv, float dt, cudaStream_t s) {
  const int ntr = (psv ? 2 : 1) * nrec;
  if (ntr <= 0 || nt <= 0) return cudaSuccess;
  sim_misfit_kernel<<<(ntr + 63) / 64, 64, 0, s>>>(syn, obs, u_tab, J, nrec, nt, psv ? 1 : 0, dt);
  return cudaGetLastError();
}

}  // namespace seiswg
