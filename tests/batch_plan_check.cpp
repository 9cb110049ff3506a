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
// Prints "ok <cases> <mixes> <revolve cases>" and exits 0, or prints the
// first violation and exits 1.
#include <array>
#include <cstdint>
#include <cstdio>
#include <utility>
#include <vector>

#include "batch_plan.h"

using namespace seiswg;

static bool quiet = false;

static int fail(int nt, int k, bool two, size_t op, const char* what) {
  if (!quiet) std::printf("nt=%d k=%d two=%d op=%zu: %s\n", nt, k, int(two), op, what);
  return 1;
}

static int replay(int nt, int k, bool psv, bool two, const std::vector<HostOp>& L) {
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
        if (o.kind != fwd) return fail(nt, k, two, q, "recomputation in two-step launches");
        if (o.flags & 1) return fail(nt, k, two, q, "recomputation records probes");
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

static int check(int nt, int k, bool psv, bool two) { return replay(nt, k, psv, two, job_ops(nt, k, psv, two)); }

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
        if (o.kind != fwd || (o.flags & 1)) return fail(nt, S, two, q, "revolve: recomputation not one plain step");
        *recomputed += 1;
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
  int mixes = 0;
  if (check_orders(mixes)) return 1;
  int rcases = 0;
  if (check_revolve(rcases)) return 1;
  std::printf("ok %d %d %d\n", cases, mixes, rcases);
  return 0;
}
