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
// Prints "ok <cases>" and exits 0, or prints the first violation and exits 1.
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
  std::printf("ok %d\n", cases);
  return 0;
}
