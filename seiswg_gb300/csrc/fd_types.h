// fd_types.h -- plain data shared by the host engine and the sm_103a stencil
// kernels.
//
// Grid layout in HBM (one allocation per field):
//   rows i in [-kHaloRows, nx + kHaloRows), row pitch `ld` floats (a multiple
//   of 32, so every row starts on a 128-byte boundary; field_pitch below);
//   column j of row i is at base[i * ld + j] and the element (0, 0) sits
//   kHaloCols floats into a row, i.e. 32-byte aligned.  z (j) is the contiguous direction, as in the
//   reference (fd2d.wgsl:140-145, k = i*nz + j).  Halo rows and columns are
//   zero and never written; the reference's edge rules (derivatives forced to
//   zero near the edges, fd2d.wgsl:151-180) are applied by index, so halo
//   values never reach a result.
//
// Work decomposition of the streaming kernels: one warp owns a z-strip of
// kStripCols output columns and marches down x over a chunk of rows.  Lane L
// holds the float4 of columns [j0 - 4 + 4L, j0 + 4L); lanes 0 and 31 are the
// strip's halo, lanes 1..30 own the 120 output columns.  z-derivatives take
// their neighbours from adjacent lanes with warp shuffles; x-derivatives read
// register rings of the previous rows.  The two-step kernel advances two time
// steps per pass: its strips own kStripCols2 columns (lanes 2..29; the two
// steps reach 6 columns to each side) and its marches read rows from 9 above
// to 5 below their chunk, hence the halo sizes.
#pragma once

#include <cstdint>

namespace seiswg {

constexpr int kHaloRows = 12;
constexpr int kHaloCols = 8;
constexpr int kStripCols = 120;
constexpr int kStripCols2 = 112;

// Row pitch of every field: room for the strips' reach past nz on the right
// (up to 11 columns) and for kHaloCols on the left, rounded to 128 bytes.
constexpr int field_pitch(int nz) { return ((nz > 128 ? nz : 128) + 24 + 31) / 32 * 32; }
constexpr unsigned kFull = 0xffffffffu;

// An injection (source or adjoint source) at cell (i, j).  `row` indexes the
// value tables [row][nt].  Lists are sorted by (i, j), stable in row, so that
// several injections into one cell add in index order.
struct Inject {
  int i, j, row, pad;
};

// A probe: a cell whose displacement u += v*dt is integrated every step and
// recorded as a history [idx][nt].  comp: 0 vx, 1 vz, 2 vy, 3 vy_c.
struct Probe {
  int i, j, comp, idx;
};

enum ProbeComp { kProbeVX = 0, kProbeVZ = 1, kProbeVY = 2, kProbeVYC = 3 };

struct Geom {
  int nx, nz, ld;
  int lx;        // rows per warp chunk
  int nstrips;   // warps across z
  int nchunks;   // warps along x
  float dt;
  float rdx;     // 1/(8*dx): reciprocal of the reference's denominator (fd2d.wgsl:156)
  float rdz;     // 1/(8*dz)
  int loader;    // kLoaderDirect or kLoaderBulk
  unsigned wait_polls;  // polls of a bounded row-pipeline wait (0: kWaitLimit)
  unsigned arm_extra;   // test hook: bytes armed on the first stage of every warp's
                        // ring beyond its copies, so that its wait runs out (0 normally)
  unsigned pdl;         // single-problem launches may start while the stream's previous
                        // launch finishes (programmatic dependent launch, fd_pipe.cuh)
};

// Row loaders of the step kernels (fd_pipe.cuh).
enum { kLoaderDirect = 0, kLoaderBulk = 1 };
constexpr int kPipeStages = 3;  // shared-memory stages per warp of the step kernels (2 rows in flight)
constexpr int kAdjStages = 2;   // stages of the adjoint kernels (19 row segments per stage)

// Bits of the device error word.
enum { kErrWaitTimeout = 1, kErrNonFiniteTraces = 2, kErrNonFiniteGradient = 4 };

// Kinds of work of a batched job (batch_plan.h): one grouped launch per
// (schedule slot, kind), or the kind of a queue operation.
enum BatchKind { kFwdSh = 0, kFwdPsv, kFwd2Sh, kFwd2Psv, kAdjSh, kAdjPsv, kMisfit, kKinds };
// Flag of a two-step operation: the state after its first step is stored in
// slot b - 1 as well (flags & 1: the probes are recorded).
constexpr int kOpMid = 2;

// The batch's device work queue (batch_plan.h, fd_queue.cu).  QueueOp: one
// operation of a job -- its kind (BatchKind), step, slots and flags as in
// GroupOp (fd_kernels.h) -- and `need`, the count of finished units that the
// counter of every chunk its rows reach must show before one of its units
// may start.  QueueUnit: unit `unit` (warp index strip + nstrips * chunk of
// the operation's geometry; 0 for the misfit) of operation `op` of job `job`.
struct QueueOp {
  int kind, it, a, b, flags, need;
};
struct QueueUnit {
  unsigned short job, unit;
  unsigned op;
};

}  // namespace seiswg
