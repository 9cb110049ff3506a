// batch_plan.h -- the operation list of one batched gradient job (host only,
// no CUDA): what Batch lays side by side into schedule slots.
//
// A job's pool has nslot = ncp + k + 1 state slots: checkpoint c (0 <= c <
// ncp) holds the state at step c*k (slot 0 the initial, zero state), the
// interval slots ncp + m - 1 (1 <= m < k) the recomputed state at step
// n0 + m of the interval being reversed, and the two ping-pong slots ncp + k
// - 1 and ncp + k the recording pass's states between checkpoints.
#pragma once

#include <algorithm>
#include <stdexcept>
#include <utility>
#include <vector>

#include "fd_types.h"

namespace seiswg {


// Forward: step `it` (two steps for kFwd2*) from slot a to slot b, flags & 1
// records the probes, flags & kOpMid (two-step operations) stores the state
// after step `it` in slot b - 1 as well.  Reverse: reverse step `it` with the
// forward state of step `it` in slot a, the incoming adjoint state in
// adjoint slot b.
struct HostOp {
  int kind, it, a, b, flags;
};

// The operations of a job with nt steps and checkpoints every k steps
// (ncp = ceil(nt / k)): the recording pass (two steps per operation where
// `two` and no checkpoint falls between them), the misfit, then for each
// interval from the last a recomputation of its states followed by its
// reverse steps, newest first.  With `pair` (and `two`) the recomputation
// runs two steps per operation, each storing both states (kOpMid: the
// interval slots of consecutive steps are consecutive), and an odd last
// step alone.
inline std::vector<HostOp> job_ops(int nt, int k, bool psv, bool two, bool pair = false) {
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
    for (int m = 1; m <= n1 - n0 - 1;) {
      const int a = m == 1 ? c : seg(m - 1);
      if (two && pair && m + 1 <= n1 - n0 - 1) {
        L.push_back(HostOp{fwd2, n0 + m - 1, a, seg(m + 1), kOpMid});
        m += 2;
      } else {
        L.push_back(HostOp{fwd, n0 + m - 1, a, seg(m), 0});
        ++m;
      }
    }
    for (int n = n1 - 1; n >= n0; --n) {
      L.push_back(HostOp{adj, n, n == n0 ? c : seg(n - n0), parity, 0});
      parity ^= 1;
    }
  }
  return L;
}

// One launch of a single problem's recording pass (Sim::forward_op, uniform
// checkpoints every k steps): steps [it, it + n) from slot a to slot b, and
// where mid >= 0 the state after step `it` stored in slot mid as well.
// Slots: c >= 0 checkpoint c (checkpoint 0 the zero initial state), -1 and
// -2 the two state buffers.
struct RecordLaunch {
  int it, n, a, b, mid;
};

// A step that ends on a checkpoint writes the checkpoint's slot, the others
// alternate between the two state buffers; two steps per launch (`two`)
// wherever no checkpoint falls between them, and with every state kept
// (k = 1) two steps per launch throughout, each launch storing the state
// between its steps into that step's checkpoint.  An odd last step runs
// alone.
inline std::vector<RecordLaunch> record_plan(int nt, int k, bool two) {
  std::vector<RecordLaunch> L;
  const bool keep_mid = two && k == 1;
  int cur = 0, pp = 0;
  for (int it = 0; it < nt;) {
    const int n = (two && it + 1 < nt && ((it + 1) % k != 0 || keep_mid)) ? 2 : 1;
    const int e = it + n;
    int dst;
    if (e % k == 0 && e < nt) {
      dst = e / k;
    } else {
      dst = -1 - pp;
      pp ^= 1;
    }
    L.push_back(RecordLaunch{it, n, cur, dst, keep_mid && n == 2 ? it + 1 : -1});
    cur = dst;
    it = e;
  }
  return L;
}

// ---------------------------------------------------------------------------
// Binomial checkpointing (Griewank and Walther, "Algorithm 799: revolve",
// ACM TOMS 26(1), 2000), restated for a job with S state slots.
//
// F(n, s): the fewest forward steps that give the reverse sweep of n steps
// [a, a+n) every state it reads, starting from S^a (held) with s more free
// slots.  With r the least number of repetitions such that
// beta(s+1, r) = C(s+1+r, r) >= n, F(n, s) = r n - beta(s+2, r-1) (n >= 2,
// s >= 1), F(1, s) = 0 and F(n, 0) = n (n-1) / 2.  The optimum obeys
// F(n, s) = min over 1 <= m < n of m + F(n-m, s-1) + F(m, s): advance m steps,
// store S^(a+m), reverse [a+m, a+n) with one slot fewer, then [a, a+m).
// The recording pass of a gradient runs every step anyway, so the advances
// along the right spine of that recursion cost nothing: the reverse phase
// recomputes F(nt, S-1) - (nt - 1) steps.
// ---------------------------------------------------------------------------
inline unsigned long long revolve_beta_capped(long long s, long long r, unsigned long long cap) {
  // C(s + r, r), or cap + 1 once it exceeds cap
  unsigned long long b = 1;
  for (long long q = 1; q <= r; ++q) {
    b = b * (unsigned long long)(s + q) / (unsigned long long)q;  // exact: C(s+q, q) = C(s+q-1, q-1) (s+q) / q
    if (b > cap) return cap + 1;
  }
  return b;
}

inline long long revolve_cost(long long n, long long s) {
  if (n <= 1) return 0;
  if (s <= 0) return n * (n - 1) / 2;
  long long r = 0;
  while (revolve_beta_capped(s + 1, r, (unsigned long long)n) < (unsigned long long)n) ++r;
  return r * n - (long long)revolve_beta_capped(s + 2, r - 1, ~0ull >> 1);
}

// A split m (1 <= m < n) at which m + F(n-m, s-1) + F(m, s) = F(n, s); the
// largest such m, which stores the next checkpoint as far ahead as the
// optimum allows.
inline int revolve_split(int n, int s) {
  const long long best = revolve_cost(n, s);
  for (int m = n - 1; m >= 1; --m)
    if (m + revolve_cost(n - m, s - 1) + revolve_cost(m, s) == best) return m;
  return 1;
}

// The operation list of a job under binomial checkpointing with S >= 1
// checkpoint slots: slots 0..S-1 (slot 0 holds S^0, the zero state that no
// step writes), then the working pair S and S+1.  The recording pass stores
// the states of the recursion's right spine; the reverse phase then walks the
// recursion, recomputing with one-step operations (two-step ones with `two`,
// where two steps lead to the next state needed: no state between them is
// read).  When the free slots run
// out before the spine reaches step nt-1, the recording pass ends with a
// one-step operation so that S^(nt-1) stays in a working slot for the first
// reverse step.  The HostOp vocabulary and slot conventions are those of
// job_ops; the reverse phase recomputes exactly F(nt, S-1) - (nt - 1) steps.
inline std::vector<HostOp> job_ops_revolve(int nt, int S, bool psv, bool two) {
  std::vector<HostOp> L;
  if (nt <= 0 || S < 1) return L;
  const int fwd = psv ? kFwdPsv : kFwdSh, adj = psv ? kAdjPsv : kAdjSh, fwd2 = psv ? kFwd2Psv : kFwd2Sh;
  auto pp = [&](int q) { return S + (q & 1); };
  // Right spine: node q reverses [a, a+n) from S^a in `slot`, with free
  // checkpoint slots [lo, S); S^a of node q+1 goes to slot lo of node q.
  struct Node { int a, n, slot, lo; };
  std::vector<Node> spine{{0, nt, 0, 1}};
  while (spine.back().n > 1 && spine.back().lo < S) {
    const Node t = spine.back();
    const int m = revolve_split(t.n, S - t.lo);
    spine.push_back(Node{t.a + m, t.n - m, t.lo, t.lo + 1});
  }
  const Node deep = spine.back();
  const bool keep_last = deep.n > 1;  // no free slot left: keep S^(nt-1) from the recording
  // Recording pass: steps 0..nt, a step ending on a spine position writes its
  // slot (two steps per operation where none falls between them).
  std::vector<int> slot_at(size_t(nt) + 1, -1);
  for (size_t q = 1; q < spine.size(); ++q) slot_at[size_t(spine[q].a)] = spine[q].slot;
  int cur = 0, ppi = 0, last_slot = -1;
  for (int t = 0; t < nt;) {
    const bool pair = two && t + 1 < nt && slot_at[size_t(t) + 1] < 0 && !(keep_last && t + 2 == nt);
    const int n = pair ? 2 : 1;
    const int e = t + n;
    int dst;
    if (e < nt && slot_at[size_t(e)] >= 0) {
      dst = slot_at[size_t(e)];
    } else {
      dst = pp(ppi);
      ppi ^= 1;
    }
    if (e == nt - 1) last_slot = dst;
    L.push_back(HostOp{pair ? fwd2 : fwd, t, cur, dst, 1});
    cur = dst;
    t = e;
  }
  L.push_back(HostOp{kMisfit, 0, 0, 0, 0});
  int parity = 0;
  auto rev = [&](int n, int slot) {
    L.push_back(HostOp{adj, n, slot, parity, 0});
    parity ^= 1;
  };
  // S^b from S^a in slot src, one step per operation (two with `two`, the
  // last one alone when b - a is odd), into slot dst (or, when dst is a
  // working slot, into whichever working slot the alternation ends in);
  // returns the slot holding S^b.
  auto advance = [&](int src, int a, int b, int dst) {
    int from = src, w = 0;
    for (int it = a; it < b;) {
      const int n = (two && it + 2 <= b) ? 2 : 1;
      int to = (it + n == b && dst < S) ? dst : pp(w++);
      if (to == from) to = pp(w++);
      L.push_back(HostOp{n == 2 ? fwd2 : fwd, it, from, to, 0});
      from = to;
      it += n;
    }
    return from;
  };
  // Reverse [a, a+n) from S^a in slot sa with free slots [lo, S).
  struct Frame { int a, n, sa, lo, stage, m; };
  auto reverse = [&](int a0, int n0, int sa0, int lo0) {
    std::vector<Frame> fs{{a0, n0, sa0, lo0, 0, 0}};
    while (!fs.empty()) {
      const Frame f = fs.back();
      fs.pop_back();
      if (f.n == 1) {
        rev(f.a, f.sa);
      } else if (f.lo >= S) {  // no free slot: every state from S^a again
        for (int j = f.a + f.n - 1; j >= f.a; --j) rev(j, j == f.a ? f.sa : advance(f.sa, f.a, j, S));
      } else if (f.stage == 0) {
        const int m = revolve_split(f.n, S - f.lo);
        advance(f.sa, f.a, f.a + m, f.lo);
        fs.push_back(Frame{f.a, f.n, f.sa, f.lo, 1, m});              // then [a, a+m)
        fs.push_back(Frame{f.a + m, f.n - m, f.lo, f.lo + 1, 0, 0});  // first [a+m, a+n)
      } else {
        fs.push_back(Frame{f.a, f.m, f.sa, f.lo, 0, 0});  // the right part's slot is free again
      }
    }
  };
  // Deepest spine node first (the recording passed its whole segment), then
  // each node's left part, whose right part is the next node's segment.
  if (keep_last) {
    rev(nt - 1, last_slot);
    if (deep.n > 1) reverse(deep.a, deep.n - 1, deep.slot, deep.lo);
  } else {
    reverse(deep.a, deep.n, deep.slot, deep.lo);
  }
  for (size_t q = spine.size() - 1; q-- > 0;) reverse(spine[q].a, spine[q + 1].a - spine[q].a, spine[q].slot, spine[q].lo);
  return L;
}

// Launch order 2 (Batch): one stream per (kind, group) and one event per
// (kind, group, slot parity).  A launch of slot t records the event of its
// slot's parity; a launch whose jobs come from kind a waits on kind a's event
// of the other parity, i.e. on slot t-1's launch of kind a, and never on a
// launch of its own slot (which the kind order may have enqueued before it).
constexpr int kPlanGroupsMax = 4;
inline int plan_stream(int kind, int group) { return kind * kPlanGroupsMax + group; }
inline int plan_event(int kind, int group, int slot) {
  return (slot & 1) * kKinds * kPlanGroupsMax + plan_stream(kind, group);
}
constexpr int kPlanStreams = kKinds * kPlanGroupsMax;
constexpr int kPlanEvents = 2 * kPlanStreams;

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

// ---------------------------------------------------------------------------
// Launch order 3 (Batch): the whole schedule as one persistent launch over a
// device work queue (fd_queue.cu).
//
// Every operation of a job is split into units: one per (strip, chunk) of
// the operation's geometry, unit = strip + nstrips * chunk, or one unit for
// the misfit.  The one- and two-step geometries of a job share their chunks
// (the same rows per chunk), so a chunk names the same rows for every kind.
// Units are laid out slot-major -- slot t holds operation t of every job,
// kinds in BatchKind order, jobs in index order, units in index order -- or
// in bands of `band` slots, within which each job's units follow a diagonal
// across its operations and chunks (plan_queue), so that operation t+1 of a
// chunk comes soon after operation t of the chunks below it and finds their
// rows still in L2.  Either way every unit a unit depends on comes earlier in
// the queue.  A job keeps
// one counter of finished units per chunk; the units of its operation t wait
// until the counter of every chunk within `reach` chunks of theirs (of every
// chunk, for the misfit) shows need[t], the units per chunk of operations
// 0..t-1.  A counter can reach need[t] only once operation t-1 has finished
// on that chunk (operation t-1's own units waited for t-2 there, and so on),
// so a unit starts only after every earlier operation of its job has
// finished on the chunks its rows reach: what it reads is written, and what
// it overwrites (a chunk of its own rows) has been read.  Warps claim units
// in queue order and run them in that order, so the first unfinished unit
// always has its dependencies finished and is held by a running warp: the
// queue cannot deadlock, whether or not all CTAs are resident.
// ---------------------------------------------------------------------------

// Chunks and rows per chunk of a job's one- and two-step geometries, and
// their strips.
struct QueueShape {
  int nchunks, lx, nstrips1, nstrips2;
};

// Rows a unit reads beyond its chunk: the two-step marches read from 9 rows
// above to 5 below their chunk, the one-step and reverse marches from 3
// above to 2 below.
constexpr int kQueueReachRows = 9;
inline int queue_reach(int lx) { return (kQueueReachRows + lx - 1) / lx; }

inline int queue_units_per_chunk(int kind, const QueueShape& s) {
  if (kind == kMisfit) return 1;
  return (kind == kFwd2Psv || kind == kFwd2Sh) ? s.nstrips2 : s.nstrips1;
}
inline int queue_units(int kind, const QueueShape& s) {
  return kind == kMisfit ? 1 : queue_units_per_chunk(kind, s) * s.nchunks;
}

struct QueuePlan {
  std::vector<std::vector<QueueOp>> ops;  // per job, its operations with their `need`
  std::vector<QueueUnit> units;           // the queue
  // First unit of each slot's band (of each slot, slot-major), then
  // units.size(): the units of slots [t0, t1) are [slot_begin[t0],
  // slot_begin[t1]) when t0 and t1 start bands.
  std::vector<long long> slot_begin;
};

// band 0: slot-major.  band K > 0: slots [bK, (b+1)K) form band b; a job's
// unit of operation t and chunk c in the band gets the key
//   c + (R + 1) (t - bK) + N m,
// R its reach in chunks, N its chunks and m the misfits of the job in the
// band before t (a misfit gets N - 1 + (R + 1) (t - bK) + N m), and the
// band's units are ordered by key, then job, operation and unit.  A unit's
// dependencies (operation t-1 within R chunks, or every chunk before a
// misfit) have smaller keys or lie in an earlier band.
inline QueuePlan plan_queue(const std::vector<std::vector<HostOp>>& lists, const std::vector<QueueShape>& shapes,
                            int band = 0) {
  QueuePlan Q;
  const size_t nj = lists.size();
  if (nj > 65536) throw std::invalid_argument("the device queue holds at most 65536 jobs");
  size_t T = 0, total = 0;
  Q.ops.resize(nj);
  for (size_t q = 0; q < nj; ++q) {
    T = lists[q].size() > T ? lists[q].size() : T;
    if (size_t(shapes[q].nstrips1) * shapes[q].nchunks > 65536 ||
        size_t(shapes[q].nstrips2) * shapes[q].nchunks > 65536)
      throw std::invalid_argument("a job has more than 65536 warp units per operation (chunk_rows too small)");
    int need = 0;
    for (const HostOp& h : lists[q]) {
      Q.ops[q].push_back(QueueOp{h.kind, h.it, h.a, h.b, h.flags, need});
      need += queue_units_per_chunk(h.kind, shapes[q]);
      total += size_t(queue_units(h.kind, shapes[q]));
    }
  }
  Q.units.reserve(total);
  Q.slot_begin.reserve(T + 1);
  if (band > 0) {
    std::vector<std::pair<long long, QueueUnit>> v;
    for (size_t t0 = 0; t0 < T; t0 += size_t(band)) {
      const size_t t1 = std::min(T, t0 + size_t(band));
      v.clear();
      for (size_t q = 0; q < nj; ++q) {
        const QueueShape& sh = shapes[q];
        const long long R1 = queue_reach(sh.lx) + 1, N = sh.nchunks;
        long long shift = 0;
        for (size_t t = t0; t < std::min(t1, lists[q].size()); ++t) {
          const int kind = lists[q][t].kind;
          const long long tau = (long long)(t - t0);
          if (kind == kMisfit) {
            v.push_back({N - 1 + R1 * tau + shift, QueueUnit{(unsigned short)q, 0, unsigned(t)}});
            shift += N;
            continue;
          }
          const int ns = queue_units_per_chunk(kind, sh), n = queue_units(kind, sh);
          for (int u = 0; u < n; ++u)
            v.push_back({u / ns + R1 * tau + shift, QueueUnit{(unsigned short)q, (unsigned short)u, unsigned(t)}});
        }
      }
      std::stable_sort(v.begin(), v.end(), [](const std::pair<long long, QueueUnit>& a,
                                               const std::pair<long long, QueueUnit>& b) { return a.first < b.first; });
      for (size_t t = t0; t < t1; ++t) Q.slot_begin.push_back((long long)Q.units.size());
      for (const auto& e : v) Q.units.push_back(e.second);
    }
    Q.slot_begin.push_back((long long)Q.units.size());
    return Q;
  }
  for (size_t t = 0; t < T; ++t) {
    Q.slot_begin.push_back((long long)Q.units.size());
    for (int kind = 0; kind < kKinds; ++kind)
      for (size_t q = 0; q < nj; ++q) {
        if (t >= lists[q].size() || lists[q][t].kind != kind) continue;
        const int n = queue_units(kind, shapes[q]);
        for (int u = 0; u < n; ++u) Q.units.push_back(QueueUnit{(unsigned short)q, (unsigned short)u, unsigned(t)});
      }
  }
  Q.slot_begin.push_back((long long)Q.units.size());
  return Q;
}

}  // namespace seiswg
