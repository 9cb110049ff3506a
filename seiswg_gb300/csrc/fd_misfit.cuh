// fd_misfit.cuh -- the L2 waveform misfit of one trace and its adjoint
// source, on the device (grouped and single-problem kernels of fd_batch.cu,
// the batch's queue kernel in fd_queue.cu).
//
// J_trace = sum_n (tau_n (d^n - o^n))^2 with the cosine taper tau of
// solver.rs:442-459, and u^n = dt * U^n, U^n = sum_{m >= n}
// float(2 tau_m^2 (d^m - o^m)), the reverse cumulative adjoint source the
// reverse sweep injects at the receiver.  Sums run in double from the last
// sample down, the order of seiswg_l2_misfit's host loop; every product and
// sum is an explicitly rounded operation, so that the result is the same in
// files built with and without multiply-add contraction.
#pragma once

#include <cmath>

#include "fd_common.cuh"
#include "fd_kernels.h"

namespace seiswg {
namespace {

// d: the synthetic trace (a probe history, read with ld1: the queue kernel
// reads histories its own warps wrote), o: the observed trace, u: the
// adjoint-source table of the trace.
__device__ double misfit_trace(const float* d, const float* __restrict__ o, float* __restrict__ u, int nt,
                               double dt) {
  const double t_end = __dmul_rn(double(nt - 1), dt), tw = t_end / 10.0, pi = 3.14159265358979323846;
  const double t_hi = __dsub_rn(t_end, tw);
  double sum = 0.0, acc = 0.0;
  for (int it = nt - 1; it >= 0; --it) {
    const double t = __dmul_rn(double(it), dt);
    double tau = 1.0;
    if (t <= tw) tau = __dadd_rn(0.5, __dmul_rn(0.5, cos(__dmul_rn(pi, __dsub_rn(tw, t)) / tw)));
    else if (t >= t_hi) tau = __dadd_rn(0.5, __dmul_rn(0.5, cos(__dmul_rn(pi, __dsub_rn(t_hi, t)) / tw)));
    const double e = __dmul_rn(__dsub_rn(double(ld1(d + it)), double(__ldg(o + it))), tau);
    sum = __dadd_rn(sum, __dmul_rn(e, e));
    acc = __dadd_rn(acc, double(float(__dmul_rn(__dmul_rn(2.0, e), tau))));
    u[it] = float(__dmul_rn(dt, acc));
  }
  return sum;
}

}  // namespace
}  // namespace seiswg
