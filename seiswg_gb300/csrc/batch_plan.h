// batch_plan.h -- the operation list of one batched gradient job (host only,
// no CUDA): what Batch lays side by side into schedule slots.
//
// A job's pool has nslot = ncp + k + 1 state slots: checkpoint c (0 <= c <
// ncp) holds the state at step c*k (slot 0 the initial, zero state), the
// interval slots ncp + m - 1 (1 <= m < k) the recomputed state at step
// n0 + m of the interval being reversed, and the two ping-pong slots ncp + k
// - 1 and ncp + k the recording pass's states between checkpoints.
#pragma once

#include <utility>
#include <vector>

namespace seiswg {

// Kinds of work; one grouped launch per (schedule slot, kind).
enum BatchKind { kFwdSh = 0, kFwdPsv, kFwd2Sh, kFwd2Psv, kAdjSh, kAdjPsv, kMisfit, kKinds };

// Forward: step `it` (two steps for kFwd2*) from slot a to slot b, flags & 1
// records the probes.  Reverse: reverse step `it` with the forward state of
// step `it` in slot a, the incoming adjoint state in adjoint slot b.
struct HostOp {
  int kind, it, a, b, flags;
};

// The operations of a job with nt steps and checkpoints every k steps
// (ncp = ceil(nt / k)): the recording pass (two steps per operation where
// `two` and no checkpoint falls between them), the misfit, then for each
// interval from the last a recomputation of its states followed by its
// reverse steps, newest first.
inline std::vector<HostOp> job_ops(int nt, int k, bool psv, bool two) {
  std::vector<HostOp> L;
  const int ncp = (nt + k - 1) / k;
  auto seg = [&](int m) { return ncp + m - 1; };  // interval slot, m >= 1
  auto pp = [&](int t) { return ncp + k - 1 + (t & 1); };
  const int fwd = psv ? kFwdPsv : kFwdSh, adj = psv ? kAdjPsv : kAdjSh, fwd2 = psv ? kFwd2Psv : kFwd2Sh;
  // Recording pass: a step that ends on a checkpoint writes the checkpoint's
  // slot, the others alternate between the two ping-pong slots.
  int cur = 0, ppi = 0;
  for (int t = 0; t < nt;) {
    const int n = (two && t + 1 < nt && (t + 1) % k != 0) ? 2 : 1;
    const int e = t + n;
    int dst;
    if (e % k == 0 && e < nt) {
      dst = e / k;
    } else {
      dst = pp(ppi);
      ppi ^= 1;
    }
    L.push_back(HostOp{n == 2 ? fwd2 : fwd, t, cur, dst, 1});
    cur = dst;
    t = e;
  }
  L.push_back(HostOp{kMisfit, 0, 0, 0, 0});
  int parity = 0;
  for (int c = ncp - 1; c >= 0; --c) {
    const int n0 = c * k, n1 = nt < n0 + k ? nt : n0 + k;
    for (int m = 1; m <= n1 - n0 - 1; ++m) L.push_back(HostOp{fwd, n0 + m - 1, m == 1 ? c : seg(m - 1), seg(m), 0});
    for (int n = n1 - 1; n >= n0; --n) {
      L.push_back(HostOp{adj, n, n == n0 ? c : seg(n - n0), parity, 0});
      parity ^= 1;
    }
  }
  return L;
}

// One grouped launch of a schedule slot: the jobs (in the order of their
// operations in the launch) whose operation at that slot is of this kind and
// which belong to this group (job q is in group q % groups), and the kinds of
// the previous slot that some of them come from (bit mask).
struct PlanLaunch {
  int kind, group, deps;
  std::vector<int> jobs;
};

// The launches of every slot, kinds in ascending order and groups within a
// kind: slot t holds operation t of every job that has one.
inline std::vector<std::vector<PlanLaunch>> plan_launches(const std::vector<std::vector<HostOp>>& lists,
                                                          int groups) {
  size_t T = 0;
  for (const auto& L : lists) T = L.size() > T ? L.size() : T;
  std::vector<std::vector<PlanLaunch>> plan(T);
  const size_t nj = lists.size();
  for (size_t t = 0; t < T; ++t)
    for (int kind = 0; kind < kKinds; ++kind)
      for (int grp = 0; grp < groups; ++grp) {
        PlanLaunch l{kind, grp, 0, {}};
        for (size_t q = size_t(grp); q < nj; q += size_t(groups)) {
          if (t >= lists[q].size() || lists[q][t].kind != kind) continue;
          if (t > 0 && lists[q][t - 1].kind != kind) l.deps |= 1 << lists[q][t - 1].kind;
          l.jobs.push_back(int(q));
        }
        if (!l.jobs.empty()) plan[t].push_back(std::move(l));
      }
  return plan;
}

}  // namespace seiswg
