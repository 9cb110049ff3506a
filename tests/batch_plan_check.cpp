// Replays the operation list of batched gradient jobs (batch_plan.h) on a
// model of the job's slots, for many step counts, checkpoint intervals and
// both recording modes, and checks that every operation finds the state it
// needs:
//   - the recording pass advances the state from step 0 to step nt once, in
//     order, each operation reading the state of its own step and recording
//     its probes;
//   - checkpoint c still holds the state of step c*k whenever it is read;
//   - each reverse step n (nt-1 down to 0, one per operation) reads the
//     forward state of step n, and the adjoint slot alternates 0, 1, 0, ...;
//   - every slot index lies in [0, ncp + k + 1).
// The replay is first shown to catch planted mistakes (two reverse steps
// swapped, a recomputation reading the wrong slot, the misfit dropped).
//
// Then the launch plan of random mixes of jobs (plan_launches) is replayed
// under launch order 2 of Batch: one stream per (kind, group), each launch
// waiting for the previous slot's events of the kinds in its dependency mask
// (plan_event, one event per kind, group and slot parity), each launch
// recording its own event of its slot's parity.  Vector clocks over the
// streams give the happens-before order; every job's operation at slot t must
// come after its operation at slot t-1, and every wait must find an event
// recorded by a launch of slot t-1 (not of slot t, which would serialise
// launches of the same slot).  A dependency mask with a bit removed must be
// reported.
// Binomial checkpointing (job_ops_revolve): the closed-form cost F(n, s) is
// checked against a brute-force minimisation of its recursion for n <= 60,
// s <= 6; the operation lists for many step counts and slot counts are
// replayed on S + 2 slots (every reverse step finds its state, recomputation
// reads the state of its step, slot 0 keeps the zero state), and the steps
// recomputed must equal F(nt, S-1) - (nt - 1) exactly.
// Launch order 3, the device queue (plan_queue): random mixes of jobs (uniform
// and binomial checkpointing, SH and PSV, one- and two-step recording,
// uneven grids and chunk rows) are run by a discrete-event model of the
// queue kernel -- W warps claim units in queue order, each claiming its next
// unit as it starts one; a unit starts once the job's counters of the chunks
// within `reach` of its chunk (all chunks, for the misfit) show its `need`,
// runs for a random time and then counts itself on its chunk -- and every
// unit's accesses are checked against the job's sequential program at the
// rows the marches really touch (two-step: 9 rows above to 5 below the chunk;
// one-step and reverse: 3 above, 2 below): a state or adjoint slot, the
// probe histories, the adjoint sources and the gradients, per chunk.  Every
// read must start after the last earlier write of its cell has ended, every
// write after every earlier access of its cell has ended; the run must end
// with every unit done (no deadlock).  Planted: a queue whose dependencies
// cover only the unit's own chunk must be reported, and so must a queue with
// a unit moved ahead of one it depends on, which deadlocks one warp.  The
// queues are laid out slot-major or in diagonal bands of 1 to 64 slots.
// With two-step recomputation (job_ops with `pair`) the same replay, the
// middle state of each two-step recomputation landing in slot b - 1, and
// ceil(m / 2) operations per interval of m recomputed steps (planted: a
// dropped middle store).
// A single problem's recording pass (record_plan, Sim::forward_op): every nt
// up to 160 and every interval, one- and two-step launches, replayed on the
// checkpoints and the two state buffers; with every state kept the two-step
// launches must store the state between their steps (planted: a dropped
// middle store, a two-step launch across a checkpoint).
// Prints "ok <cases> <mixes> <revolve cases> <queue mixes>" and exits 0, or
// prints the first violation and exits 1.
#include <algorithm>
#include <array>
#include <cstdint>
#include <cstdio>
#include <map>
#include <queue>
#include <utility>
#include <vector>

#include "batch_plan.h"

using namespace seiswg;

static bool quiet = false;

static int fail(int nt, int k, bool two, size_t op, const char* what) {
  if (!quiet) std::printf("nt=%d k=%d two=%d op=%zu: %s\n", nt, k, int(two), op, what);
  return 1;
}

static int replay(int nt, int k, bool psv, bool two, const std::vector<HostOp>& L, bool pair = false) {
  const int ncp = (nt + k - 1) / k, nslot = ncp + k + 1;
  std::vector<int> slot(nslot, -1);
  slot[0] = 0;  // the initial (zero) state
  const int fwd = psv ? kFwdPsv : kFwdSh, fwd2 = psv ? kFwd2Psv : kFwd2Sh, adj = psv ? kAdjPsv : kAdjSh;
  int rec = 0;           // next step of the recording pass
  bool misfit = false;
  int rev = nt - 1;      // next reverse step
  int parity = 0;
  for (size_t q = 0; q < L.size(); ++q) {
    const HostOp& o = L[q];
    if (o.a < 0 || o.a >= nslot) return fail(nt, k, two, q, "source slot out of range");
    if (o.kind == fwd || o.kind == fwd2) {
      const int n = o.kind == fwd2 ? 2 : 1;
      if (o.b < 0 || o.b >= nslot) return fail(nt, k, two, q, "destination slot out of range");
      if (o.a == o.b) return fail(nt, k, two, q, "a step reads and writes the same slot");
      if (slot[o.a] != o.it) return fail(nt, k, two, q, "forward step does not find the state of its step");
      if (o.it + n > nt) return fail(nt, k, two, q, "forward step beyond nt");
      if (!misfit) {
        if (o.it != rec || !(o.flags & 1)) return fail(nt, k, two, q, "recording pass out of order");
        rec += n;
      } else {
        if (o.kind != fwd && !(pair && o.kind == fwd2 && (o.flags & kOpMid)))
          return fail(nt, k, two, q, "recomputation in two-step launches that do not keep both states");
        if (o.flags & 1) return fail(nt, k, two, q, "recomputation records probes");
      }
      if (o.flags & kOpMid) {
        if (o.kind != fwd2 || !misfit) return fail(nt, k, two, q, "a middle state outside a two-step recomputation");
        if (o.b - 1 < ncp || o.b - 1 == o.a) return fail(nt, k, two, q, "the middle state overwrites a checkpoint");
        slot[o.b - 1] = o.it + 1;
      }
      if (o.b < ncp && o.it + n != o.b * k) return fail(nt, k, two, q, "checkpoint slot gets another step");
      slot[o.b] = o.it + n;
    } else if (o.kind == kMisfit) {
      if (misfit || rec != nt) return fail(nt, k, two, q, "misfit before the end of the recording pass");
      misfit = true;
    } else if (o.kind == adj) {
      if (!misfit) return fail(nt, k, two, q, "reverse step before the misfit");
      if (o.it != rev) return fail(nt, k, two, q, "reverse steps out of order");
      if (slot[o.a] != o.it) return fail(nt, k, two, q, "reverse step does not find its forward state");
      if (o.b != parity) return fail(nt, k, two, q, "adjoint slots do not alternate");
      parity ^= 1;
      --rev;
    } else {
      return fail(nt, k, two, q, "unexpected kind");
    }
  }
  if (!misfit || rev != -1) return fail(nt, k, two, L.size(), "reverse sweep incomplete");
  for (int c = 0; c < ncp; ++c)
    if (slot[c] != c * k) return fail(nt, k, two, L.size(), "a checkpoint was overwritten");
  return 0;
}

static int check(int nt, int k, bool psv, bool two) {
  if (replay(nt, k, psv, two, job_ops(nt, k, psv, two))) return 1;
  if (!two) return 0;
  // Two-step recomputation: the same steps, half the operations.
  const std::vector<HostOp> P = job_ops(nt, k, psv, true, true);
  if (replay(nt, k, psv, two, P, true)) return 1;
  size_t fwd_ops = 0, fwd_ops1 = 0;
  bool after = false;
  for (const HostOp& o : P) {
    if (o.kind == kMisfit) after = true;
    else if (after && o.kind != kAdjPsv && o.kind != kAdjSh) ++fwd_ops;
  }
  after = false;
  for (const HostOp& o : job_ops(nt, k, psv, true)) {
    if (o.kind == kMisfit) after = true;
    else if (after && o.kind != kAdjPsv && o.kind != kAdjSh) ++fwd_ops1;
  }
  const int ncp = (nt + k - 1) / k;
  size_t want = 0;  // per interval of m recomputed steps, ceil(m / 2) operations
  for (int c = 0; c < ncp; ++c) {
    const int n0 = c * k, n1 = nt < n0 + k ? nt : n0 + k;
    want += size_t(n1 - n0 - 1 + 1) / 2;
  }
  if (fwd_ops != want || fwd_ops1 < fwd_ops) return fail(nt, k, two, P.size(), "two-step recomputation op count");
  return 0;
}

// Each planted mistake must be reported.
// Replays a binomial schedule on S + 2 slots; *recomputed = forward steps of
// the reverse phase.
static int replay_revolve(int nt, int S, bool psv, bool two, const std::vector<HostOp>& L, long long* recomputed) {
  const int nslot = S + 2;
  std::vector<int> slot(nslot, -1);
  slot[0] = 0;
  const int fwd = psv ? kFwdPsv : kFwdSh, fwd2 = psv ? kFwd2Psv : kFwd2Sh, adj = psv ? kAdjPsv : kAdjSh;
  int rec = 0, rev = nt - 1, parity = 0;
  bool misfit = false;
  *recomputed = 0;
  for (size_t q = 0; q < L.size(); ++q) {
    const HostOp& o = L[q];
    if (o.a < 0 || o.a >= nslot) return fail(nt, S, two, q, "revolve: source slot out of range");
    if (o.kind == fwd || o.kind == fwd2) {
      const int n = o.kind == fwd2 ? 2 : 1;
      if (o.b < 1 || o.b >= nslot) return fail(nt, S, two, q, "revolve: destination out of range (or slot 0)");
      if (o.a == o.b) return fail(nt, S, two, q, "revolve: a step reads and writes the same slot");
      if (slot[o.a] != o.it) return fail(nt, S, two, q, "revolve: forward step does not find its state");
      if (!misfit) {
        if (o.it != rec || !(o.flags & 1)) return fail(nt, S, two, q, "revolve: recording out of order");
        rec += n;
      } else {
        if ((o.kind != fwd && !(two && o.kind == fwd2)) || (o.flags & 1))
          return fail(nt, S, two, q, "revolve: recomputation not a plain step (or two with two-step launches)");
        *recomputed += n;
      }
      slot[o.b] = o.it + n;
    } else if (o.kind == kMisfit) {
      if (misfit || rec != nt) return fail(nt, S, two, q, "revolve: misfit before the end of the recording");
      misfit = true;
    } else if (o.kind == adj) {
      if (!misfit || o.it != rev) return fail(nt, S, two, q, "revolve: reverse steps out of order");
      if (slot[o.a] != o.it) return fail(nt, S, two, q, "revolve: reverse step does not find its state");
      if (o.b != parity) return fail(nt, S, two, q, "revolve: adjoint slots do not alternate");
      parity ^= 1;
      --rev;
    } else {
      return fail(nt, S, two, q, "revolve: unexpected kind");
    }
  }
  if (!misfit || rev != -1) return fail(nt, S, two, L.size(), "revolve: reverse sweep incomplete");
  return 0;
}

static long long brute_cost(int n, int s, std::vector<std::vector<long long>>& memo) {
  if (n <= 1) return 0;
  if (s == 0) return (long long)n * (n - 1) / 2;
  long long& m = memo[size_t(n)][size_t(s)];
  if (m >= 0) return m;
  long long best = -1;
  for (int k = 1; k < n; ++k) {
    const long long c = k + brute_cost(n - k, s - 1, memo) + brute_cost(k, s, memo);
    if (best < 0 || c < best) best = c;
  }
  return m = best;
}

static int check_revolve(int& cases) {
  std::vector<std::vector<long long>> memo(61, std::vector<long long>(7, -1));
  for (int n = 1; n <= 60; ++n)
    for (int sl = 0; sl <= 6; ++sl)
      if (brute_cost(n, sl, memo) != revolve_cost(n, sl)) {
        std::printf("revolve_cost(%d, %d) = %lld, the recursion gives %lld\n", n, sl, revolve_cost(n, sl),
                    brute_cost(n, sl, memo));
        return 1;
      }
  auto one = [&](int nt, int S, bool two) {
    long long rc = 0;
    if (replay_revolve(nt, S, true, two, job_ops_revolve(nt, S, true, two), &rc)) return 1;
    const long long want = revolve_cost(nt, S - 1) - (nt - 1);
    if (rc != want) {
      std::printf("revolve nt=%d S=%d two=%d: %lld steps recomputed, the optimum is %lld\n", nt, S, int(two), rc,
                  want);
      return 1;
    }
    ++cases;
    return 0;
  };
  for (int nt = 1; nt <= 120; ++nt)
    for (int S = 1; S <= 12; ++S)
      for (int two = 0; two < 2; ++two)
        if (one(nt, S, two != 0)) return 1;
  for (int nt : {1000, 3000, 4000})
    for (int S : {2, 3, 10, 40, 56, 110, 1502})
      for (int two = 0; two < 2; ++two)
        if (one(nt, S, two != 0)) return 1;
  return 0;
}

// A single problem's recording pass (record_plan): replayed on its slots
// (checkpoints and the two state buffers), every launch must read the state
// of its first step and write the state after its last, a middle state only
// from a two-step launch and into that step's checkpoint; at the end every
// checkpoint c holds the state of step c*k, the last launch's buffer holds
// step nt, and with every state kept and two-step launches all but an odd
// last step run two per launch.
static int replay_record(int nt, int k, bool two, const std::vector<RecordLaunch>& L) {
  const int ncp = (nt + k - 1) / k;
  std::vector<int> ck(size_t(std::max(ncp, 1)), -1), buf(2, -1);
  ck[0] = 0;
  auto at = [&](int s) -> int& { return s >= 0 ? ck[size_t(s)] : buf[size_t(-1 - s)]; };
  int next = 0, twos = 0;
  for (size_t q = 0; q < L.size(); ++q) {
    const RecordLaunch& o = L[q];
    if (o.it != next || (o.n != 1 && o.n != 2) || o.it + o.n > nt) return fail(nt, k, two, q, "steps out of order");
    if (o.a >= ncp || o.b >= ncp || o.a < -2 || o.b < -2 || o.a == o.b) return fail(nt, k, two, q, "bad slot");
    if (at(o.a) != o.it) return fail(nt, k, two, q, "reads a state of another step");
    if (o.n == 2 && !two) return fail(nt, k, two, q, "two steps without two-step launches");
    if (o.b >= 0 && o.b * k != o.it + o.n) return fail(nt, k, two, q, "writes a checkpoint of another step");
    if (o.mid >= 0 && (o.n != 2 || o.mid != o.it + 1 || o.mid * k != o.it + 1 || o.mid >= ncp))
      return fail(nt, k, two, q, "bad middle state");
    if (o.n == 2 && (o.it + 1) % k == 0 && o.mid < 0) return fail(nt, k, two, q, "skips a checkpoint");
    at(o.b) = o.it + o.n;
    if (o.mid >= 0) at(o.mid) = o.it + 1;
    twos += o.n == 2;
    next = o.it + o.n;
  }
  if (next != nt) return fail(nt, k, two, L.size(), "the pass does not end at nt");
  for (int c = 0; c < ncp; ++c)
    if (ck[size_t(c)] != c * k) return fail(nt, k, two, L.size(), "a checkpoint is missing");
  if (nt > 0 && (L.back().b >= 0 || at(L.back().b) != nt)) return fail(nt, k, two, L.size(), "final state");
  if (two && k == 1 && twos != nt / 2) return fail(nt, k, two, L.size(), "one-step launches with every state kept");
  return 0;
}

static int check_record(int nt, int k, bool two) { return replay_record(nt, k, two, record_plan(nt, k, two)); }


static bool catches_planted_mistakes() {
  const int nt = 23, k = 5;
  quiet = true;
  bool ok = true;
  for (int two = 0; two < 2; ++two) {
    std::vector<HostOp> L = job_ops(nt, k, true, two != 0);
    size_t last = L.size() - 1;  // the last two ops are reverse steps 1 and 0
    std::vector<HostOp> swapped = L;
    std::swap(swapped[last], swapped[last - 1]);
    ok = ok && replay(nt, k, true, two != 0, swapped) == 1;
    std::vector<HostOp> wrong = L;
    for (HostOp& o : wrong)
      if (o.kind == kFwdPsv && !(o.flags & 1) && o.a >= (nt + k - 1) / k) {
        o.a += 1;  // a recomputation reading the next interval slot
        break;
      }
    ok = ok && replay(nt, k, true, two != 0, wrong) == 1;
    std::vector<HostOp> nomisfit;
    for (const HostOp& o : L)
      if (o.kind != kMisfit) nomisfit.push_back(o);
    ok = ok && replay(nt, k, true, two != 0, nomisfit) == 1;
  }
  // A two-step recomputation whose middle-state store is dropped.
  {
    std::vector<HostOp> P = job_ops(nt, k, true, true, true);
    for (HostOp& o : P)
      if (o.flags & kOpMid) {
        o.flags &= ~kOpMid;
        break;
      }
    ok = ok && replay(nt, k, true, true, P, true) == 1;
  }
  // A recording pass with every state kept whose middle-state store is
  // dropped, and one whose two-step launch skips a checkpoint.
  std::vector<RecordLaunch> R = record_plan(12, 1, true);
  R[2].mid = -1;
  ok = ok && replay_record(12, 1, true, R) == 1;
  R = record_plan(12, 3, true);
  for (RecordLaunch& o : R)
    if (o.n == 1 && o.it + 1 < 12) {
      o.n = 2;  // two steps across the checkpoint at it + 1, written nowhere
      break;
    }
  ok = ok && replay_record(12, 3, true, R) == 1;
  quiet = false;
  return ok;
}

// Launch order 2 (Batch::enqueue_slots): true when every job's operations
// are ordered from slot to slot.  `drop`: clear this dependency bit of the
// first launch that has it (a planted mistake), -1 for none.
static bool order2_holds(const std::vector<std::vector<HostOp>>& lists, int groups, int drop) {
  constexpr int kStreams = kPlanStreams;
  using Clock = std::array<int, kStreams>;
  auto plan = plan_launches(lists, groups);
  if (drop >= 0) {
    bool done = false;
    for (auto& slot : plan)
      for (auto& l : slot)
        if (!done && (l.deps >> drop) & 1) {
          l.deps &= ~(1 << drop);
          done = true;
        }
    if (!done) return true;  // nothing to plant: the self-check fails
  }
  Clock zero{};
  std::vector<Clock> stream(kStreams, zero), event(kPlanEvents, zero);
  std::vector<int> event_slot(kPlanEvents, -1);  // slot of the launch that last recorded the event
  std::array<int, kStreams> seq{};
  // where[q] = (stream, seq) of the launch holding job q's previous operation
  std::vector<std::pair<int, int>> where(lists.size(), {-1, 0});
  for (size_t t = 0; t < plan.size(); ++t) {
    std::vector<std::pair<int, int>> now(lists.size(), {-1, 0});
    for (const PlanLaunch& l : plan[t]) {
      const int s = plan_stream(l.kind, l.group);
      Clock c = stream[s];
      for (int a = 0; a < kKinds; ++a)
        if ((l.deps >> a) & 1) {
          const int ev = plan_event(a, l.group, int(t) - 1);
          if (event_slot[ev] != int(t) - 1) {
            if (!quiet) std::printf("slot %zu: a launch waits on an event not recorded at slot %zu\n", t, t - 1);
            return false;
          }
          const Clock& e = event[ev];
          for (int x = 0; x < kStreams; ++x) c[x] = c[x] > e[x] ? c[x] : e[x];
        }
      c[s] = ++seq[s];
      for (int q : l.jobs) {
        const auto [ps, pn] = where[q];
        if (t > 0 && ps >= 0 && c[ps] < pn) return false;
        now[q] = {s, c[s]};
      }
      stream[s] = c;
      event[plan_event(l.kind, l.group, int(t))] = c;
      event_slot[plan_event(l.kind, l.group, int(t))] = int(t);
    }
    for (size_t q = 0; q < lists.size(); ++q)
      if (now[q].first >= 0) where[q] = now[q];
  }
  return true;
}

static uint32_t rng_state = 12345u;
static int rnd(int n) {  // 0 .. n-1
  rng_state = rng_state * 1664525u + 1013904223u;
  return int((rng_state >> 8) % uint32_t(n));
}

static int check_orders(int& mixes) {
  for (int m = 0; m < 3000; ++m) {
    const int nj = 1 + rnd(12), groups = 1 + rnd(4);
    std::vector<std::vector<HostOp>> lists;
    for (int q = 0; q < nj; ++q) {
      const int nt = 1 + rnd(40), k = 1 + rnd(nt);
      lists.push_back(job_ops(nt, k, rnd(2) != 0, rnd(2) != 0));
    }
    if (!order2_holds(lists, groups, -1)) {
      std::printf("launch order 2 misses a dependency (mix %d)\n", m);
      return 1;
    }
    ++mixes;
  }
  // Planted: removing one needed dependency bit must break the order for a
  // mix where a job changes kind (recomputation to reverse steps).
  std::vector<std::vector<HostOp>> lists = {job_ops(30, 6, true, true), job_ops(17, 4, false, false)};
  quiet = true;
  for (int a : {kFwdPsv, kFwdSh, kFwd2Psv, kAdjPsv, kMisfit})
    if (order2_holds(lists, 1, a)) {
      std::printf("the order check misses a dropped dependency on kind %d\n", a);
      return 1;
    }
  quiet = false;
  return 0;
}

// ---- launch order 3: the device queue ---------------------------------------

struct QJob {
  int nx, lx, nchunks, nstrips1, nstrips2;
  std::vector<HostOp> ops;
};

// Buffers of a job: pool slots 0..63, adjoint slots 64, 65, the probe
// histories 66, the adjoint sources 67 (one cell), the gradients 68.
enum { kBufAdj = 64, kBufProbe = 66, kBufU = 67, kBufGrad = 68 };

struct Access {
  int buf, c0, c1;  // chunks [c0, c1)
  bool write;
};

// The cells a unit of operation o at chunk c touches (chunks of the rows the
// march reads or writes).
static std::vector<Access> unit_accesses(const QJob& J, const HostOp& o, int c) {
  std::vector<Access> A;
  const int ib = c * J.lx, ie = std::min(J.nx, ib + J.lx);
  auto span = [&](int above, int below) {
    const int lo = std::max(0, ib - above), hi = std::min(J.nx - 1, ie - 1 + below);
    return std::make_pair(lo / J.lx, hi / J.lx + 1);
  };
  if (o.kind == kMisfit) {
    A.push_back({kBufProbe, 0, J.nchunks, false});
    A.push_back({kBufU, 0, 1, true});
  } else if (o.kind == kAdjSh || o.kind == kAdjPsv) {
    const auto r = span(3, 2);
    A.push_back({o.a, r.first, r.second, false});
    A.push_back({kBufAdj + (o.b & 1), r.first, r.second, false});
    A.push_back({kBufU, 0, 1, false});
    A.push_back({kBufGrad, c, c + 1, true});  // read, modified and written by the unit alone
    A.push_back({kBufAdj + 1 - (o.b & 1), c, c + 1, true});
  } else {
    const bool two = o.kind == kFwd2Sh || o.kind == kFwd2Psv;
    const auto r = two ? span(9, 5) : span(3, 2);
    A.push_back({o.a, r.first, r.second, false});
    A.push_back({o.b, c, c + 1, true});
    if (o.flags & 1) A.push_back({kBufProbe, c, c + 1, true});  // accumulators: the unit's own rows
  }
  return A;
}

// Runs the queue with W warps and random unit times (seeded), then checks
// the access order.  reach_override >= 0 replaces every job's reach (the
// planted mistake).  Returns 0, 1 (hazard) or 2 (deadlock).
static int replay_queue(const std::vector<QJob>& jobs, const QueuePlan& Q, int W, int reach_override) {
  const size_t nu = Q.units.size();
  std::vector<std::vector<int>> cnt(jobs.size());
  for (size_t q = 0; q < jobs.size(); ++q) cnt[q].assign(size_t(jobs[q].nchunks), 0);
  std::vector<double> t_start(nu, -1.0), t_end(nu, -1.0);
  auto chunk_of = [&](const QueueUnit& u) {
    const QJob& J = jobs[u.job];
    const HostOp& o = J.ops[u.op];
    if (o.kind == kMisfit) return 0;
    return int(u.unit) / ((o.kind == kFwd2Sh || o.kind == kFwd2Psv) ? J.nstrips2 : J.nstrips1);
  };
  auto ready = [&](size_t p) {
    const QueueUnit& u = Q.units[p];
    const QJob& J = jobs[u.job];
    const QueueOp& op = Q.ops[u.job][u.op];
    const int reach = reach_override >= 0 ? reach_override : queue_reach(J.lx);
    int c0 = 0, c1 = J.nchunks;
    if (op.kind != kMisfit) {
      const int c = chunk_of(u);
      c0 = std::max(0, c - reach);
      c1 = std::min(J.nchunks, c + reach + 1);
    }
    for (int c = c0; c < c1; ++c)
      if (cnt[u.job][size_t(c)] < op.need) return false;
    return true;
  };
  // Warps: the unit held (claimed, not started or running) and the next.
  struct W8 { long long cur = -1, next = -1; bool running = false; };
  std::vector<W8> warps(static_cast<size_t>(W));
  long long claim = 0;
  auto take = [&]() -> long long { return claim < (long long)nu ? claim++ : -1; };
  for (W8& w : warps) w.cur = take();
  using Ev = std::pair<double, int>;  // (end time, warp)
  std::priority_queue<Ev, std::vector<Ev>, std::greater<Ev>> evq;
  double now = 0.0;
  size_t done = 0;
  for (;;) {
    // Start every waiting warp whose unit is ready (in warp order).
    bool progress = true;
    while (progress) {
      progress = false;
      for (int w = 0; w < W; ++w) {
        W8& s = warps[size_t(w)];
        if (s.running || s.cur < 0 || !ready(size_t(s.cur))) continue;
        s.running = true;
        s.next = take();  // claimed as the unit starts, as the kernel does
        t_start[size_t(s.cur)] = now;
        evq.push({now + 1.0 + rnd(1000) / 100.0, w});
        progress = true;
      }
    }
    if (evq.empty()) break;
    const Ev e = evq.top();
    evq.pop();
    now = e.first;
    W8& s = warps[size_t(e.second)];
    const size_t p = size_t(s.cur);
    t_end[p] = now;
    ++done;
    const QueueUnit& u = Q.units[p];
    if (jobs[u.job].ops[u.op].kind == kMisfit) {
      for (int& c : cnt[u.job]) ++c;
    } else {
      ++cnt[u.job][size_t(chunk_of(u))];
    }
    s.running = false;
    s.cur = s.next;
    s.next = -1;
  }
  if (done != nu) return 2;
  // Per job and cell, the accesses in program order: every access must start
  // after the conflicting accesses of earlier operations have ended.
  for (size_t q = 0; q < jobs.size(); ++q) {
    const QJob& J = jobs[q];
    // cell -> per operation: (min start, max end) of its reading and of its writing units
    struct OpAcc { double rs = 1e300, re = -1.0, ws = 1e300, we = -1.0; };
    std::map<std::pair<int, int>, std::map<int, OpAcc>> cells;
    for (size_t p = 0; p < nu; ++p) {
      const QueueUnit& u = Q.units[p];
      if (u.job != q) continue;
      for (const Access& a : unit_accesses(J, J.ops[u.op], chunk_of(u)))
        for (int c = a.c0; c < a.c1; ++c) {
          OpAcc& x = cells[{a.buf, c}][int(u.op)];
          if (a.write) { x.ws = std::min(x.ws, t_start[p]); x.we = std::max(x.we, t_end[p]); }
          else { x.rs = std::min(x.rs, t_start[p]); x.re = std::max(x.re, t_end[p]); }
        }
    }
    for (const auto& cell : cells) {
      double last_write_end = -1.0, reads_end = -1.0;
      for (const auto& oa : cell.second) {
        const OpAcc& x = oa.second;
        if (x.re >= 0.0 && x.rs < last_write_end) {
          if (!quiet)
            std::printf("job %zu buffer %d chunk %d: op %d reads before the last write ended\n", q, cell.first.first,
                        cell.first.second, oa.first);
          return 1;
        }
        if (x.we >= 0.0) {
          if (x.ws < last_write_end || x.ws < reads_end) {
            if (!quiet)
              std::printf("job %zu buffer %d chunk %d: op %d writes before earlier accesses ended\n", q,
                          cell.first.first, cell.first.second, oa.first);
            return 1;
          }
          last_write_end = x.we;
          reads_end = -1.0;
        }
        if (x.re >= 0.0) reads_end = std::max(reads_end, x.re);
      }
    }
  }
  return 0;
}

static QJob random_qjob() {
  QJob J;
  J.nx = 12 + rnd(120);
  const int lxs[] = {4, 5, 8, 9, 12, 16, 32};
  J.lx = lxs[rnd(7)];
  J.nchunks = (J.nx + J.lx - 1) / J.lx;
  J.nstrips1 = 1 + rnd(3);
  J.nstrips2 = 1 + rnd(3);
  const int nt = 1 + rnd(24);
  const bool psv = rnd(2) != 0, two = rnd(2) != 0;
  if (rnd(3) == 0) J.ops = job_ops_revolve(nt, 1 + rnd(5), psv, two);
  else J.ops = job_ops(nt, 1 + rnd(nt), psv, two);
  return J;
}

static QueuePlan plan_of(const std::vector<QJob>& jobs, int band = 0) {
  std::vector<std::vector<HostOp>> lists;
  std::vector<QueueShape> shapes;
  for (const QJob& J : jobs) {
    lists.push_back(J.ops);
    shapes.push_back(QueueShape{J.nchunks, J.lx, J.nstrips1, J.nstrips2});
  }
  return plan_queue(lists, shapes, band);
}

static int check_queue(int& mixes) {
  for (int m = 0; m < 1500; ++m) {
    std::vector<QJob> jobs;
    const int nj = 1 + rnd(6);
    for (int q = 0; q < nj; ++q) jobs.push_back(random_qjob());
    const int bands[] = {0, 0, 1, 2, 3, 5, 8, 64};
    const int band = bands[rnd(8)];
    const QueuePlan Q = plan_of(jobs, band);
    // slot-major: every unit's operation index equals its slot; bands: every
    // unit between two band starts holds an operation of that band
    const size_t T = Q.slot_begin.size() - 1, B = band > 0 ? size_t(band) : 1;
    for (size_t t = 0; t < T; t += B)
      for (long long p = Q.slot_begin[t]; p < Q.slot_begin[std::min(T, t + B)]; ++p)
        if (Q.units[size_t(p)].op < t || Q.units[size_t(p)].op >= t + B) {
          std::printf("queue mix %d: unit %lld of slot %zu holds operation %u\n", m, p, t, Q.units[size_t(p)].op);
          return 1;
        }
    if (Q.units.size() != size_t(Q.slot_begin[T])) {
      std::printf("queue mix %d: %zu units, the plan counts %lld\n", m, Q.units.size(), Q.slot_begin[T]);
      return 1;
    }
    const int W = 1 + rnd(48);
    const int r = replay_queue(jobs, Q, W, -1);
    if (r) {
      std::printf("queue mix %d (%d warps, band %d): %s\n", m, W, band, r == 2 ? "deadlock" : "access out of order");
      return 1;
    }
    ++mixes;
  }
  // Planted: dependencies on the unit's own chunk only (reach 0) must give a
  // hazard in a multi-chunk two-step job run by many warps.
  quiet = true;
  {
    QJob J;
    J.nx = 96; J.lx = 8; J.nchunks = 12; J.nstrips1 = 2; J.nstrips2 = 2;
    J.ops = job_ops(20, 4, true, true);
    const std::vector<QJob> jobs{J};
    const QueuePlan Q = plan_of(jobs);
    bool caught = false;
    for (int trial = 0; trial < 20 && !caught; ++trial) caught = replay_queue(jobs, Q, 32, 0) == 1;
    if (!caught) {
      std::printf("the queue replay misses a dependency that does not cover the rows read\n");
      return 1;
    }
    // A unit of operation 1 moved to the front: with one warp it waits for
    // operation 0, which no warp can reach.
    QueuePlan bad = Q;
    const long long p1 = bad.slot_begin[1];
    std::rotate(bad.units.begin(), bad.units.begin() + p1, bad.units.begin() + p1 + 1);
    if (replay_queue(jobs, bad, 1, -1) != 2) {
      std::printf("the queue replay misses a deadlock\n");
      return 1;
    }
  }
  quiet = false;
  return 0;
}

int main() {
  if (!catches_planted_mistakes()) {
    std::printf("the replay misses a planted mistake\n");
    return 1;
  }
  int cases = 0;
  for (int nt = 1; nt <= 160; ++nt)
    for (int k = 1; k <= nt + 2; ++k)
      for (int two = 0; two < 2; ++two)
        for (int psv = 0; psv < 2; ++psv) {
          const int kk = k < nt ? k : (nt > 0 ? nt : 1);  // Batch clamps k to nt
          if (check(nt, kk, psv != 0, two != 0)) return 1;
          ++cases;
        }
  // The configurations' sizes: nt 1000..4000 with k = ceil(sqrt(nt)) and every second step.
  for (int nt : {1000, 1001, 2500, 3000, 4000})
    for (int k : {2, 3, 31, 32, 55, 63, 64})
      for (int two = 0; two < 2; ++two) {
        if (check(nt, k, true, two != 0)) return 1;
        ++cases;
      }
  // Single-problem recording passes, every interval including every state.
  for (int nt = 1; nt <= 160; ++nt)
    for (int k = 1; k <= nt; ++k)
      for (int two = 0; two < 2; ++two) {
        if (check_record(nt, k, two != 0)) return 1;
        ++cases;
      }
  for (int nt : {1000, 1001, 3000, 4000})
    for (int k : {1, 2, 55, 64})
      for (int two = 0; two < 2; ++two) {
        if (check_record(nt, k, two != 0)) return 1;
        ++cases;
      }
  int mixes = 0;
  if (check_orders(mixes)) return 1;
  int rcases = 0;
  if (check_revolve(rcases)) return 1;
  int qmixes = 0;
  if (check_queue(qmixes)) return 1;
  std::printf("ok %d %d %d %d\n", cases, mixes, rcases, qmixes);
  return 0;
}
