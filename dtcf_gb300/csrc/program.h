// Persistent iteration program: the kernels of one coupled-cluster iteration
// as a few persistent launches driven by a device-side work queue.
//
// While a recorder is active on the calling thread, the library's kernel
// launchers (tile moves, fused sums, direct contractions, operand splits,
// CUDA-core FP64 GEMMs, the amplitude and energy kernels, zero fills) do not
// launch: each appends a record -- its kernel body, its arguments, its grid
// of virtual blocks and the device buffers it reads and writes -- and the
// split GEMM launches append their tensor-core launches.  The recorded
// iteration is then cut into levels:
//
//   * memory records (the bodies of bodies.cuh) run inside one persistent
//     kernel per level, 256 threads, a few CTAs per SM; a CTA takes the next
//     (record, virtual block) item from an atomic ticket, in record order,
//     waits until the records it depends on have finished all their blocks
//     (bounded: past the limit it sets the program's error word and skips
//     the item), runs the body and counts the block done (release);
//   * the tensor-core GEMM launches of a level are merged by kernel (one
//     k-stationary launch, one per thin-K block width, ...) over all the
//     problems of every contraction at that level;
//   * anything else (the FP64 tensor-pipe GEMM kernels) is launched as it
//     would be, in record order.
//
// A record depends on the record before it in the same step (the steps of
// one contraction stay in order) and on every earlier record that touches a
// registered buffer (a tensor of the iteration) in a conflicting way: it
// reads what an earlier record writes, or writes what an earlier record
// reads or writes.  Memory records of the same level with such a dependency
// wait on each other inside the launch; everything else is ordered by the
// launches.  Tickets follow record order and dependencies point backwards,
// so the lowest unfinished ticket can always run and the queue cannot
// deadlock (no co-residency of the CTAs is assumed).  Every record computes
// exactly what its standalone launch computes, element by element, so the
// results are bit-identical to the kernel-by-kernel iteration.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <memory>
#include <vector>

#include "cc.h"
#include "common.h"
#include "split_dev.h"

namespace gbx {

struct SplitPlan;

enum ProgKind : int32_t {
  PK_NOP = 0,
  PK_ZERO,
  PK_MOVE,
  PK_MOVE4,
  PK_FUSED,
  PK_DIRECT,
  PK_ROWEXP,
  PK_DIGITS,
  PK_SHORTROWS,
  PK_SPLITROWS,
  PK_SPLITRED,
  PK_GEMV,
  PK_SMALLOUT,
  PK_SMALLK,
  PK_SPLITKRED,
  PK_AMP,
  PK_MUL,
  PK_DOTPART,
  PK_ENERGYFIN,
};

struct PaZero { void* p; uint64_t bytes; };
struct PaMove {
  const MoveDesc* descs;
  const uint32_t* first;
  int ndesc;
  uint32_t nchunks;
  const double* src;
  double* dst;
  double alpha;
};
struct PaMove4 {
  const MoveDesc4* descs;
  const uint32_t* chunk_desc;
  uint32_t nchunks;
  int pairs;
  const double* src;
  double* dst;
  double alpha;
};
struct PaFused {
  const FsItem* items;
  const FsTerm* terms;
  const double* scale;
  double* out;
  int nitems;
  FsSrc src;
};
struct PaDirect {
  const DirItem* items;
  const DirPair* pairs;
  const double* A;
  const double* B;
  double* C;
  double alpha;
  int nitems;
  int overwrite;
};
struct PaSplitSets {  // row exponents, digits, short rows
  const SplitRowSet* sets;
  int64_t total;
  int nsets, S;
};
struct PaSplitRed {
  const DevProblem* probs;
  const int* red_prob;
  const int64_t* red_first;
  int64_t total;
  int nred;
};
struct PaGemm {  // matrix-vector, small output, small K
  const GemmProblem* probs;
  const int* first;
  int nprob, total;
};
struct PaKRed {
  const GemmProblem* probs;
  const int* red_prob;
  const uint32_t* red_first;
  int nred;
  uint32_t nchunks;
};
struct PaAmp {
  const CCAmpTile* tiles;
  const CCAmpItem* items;
  const double* t1;
  const double* t2;
  double* tau;
  double* taut;
  double* Q;
  int nitems;
};
struct PaMul { const double* a; const double* b; double* out; int64_t n; };
struct PaDot { const double* x; const double* y; double* partial; int64_t n; };
struct PaEnergyFin { const double* partial; double* hist; int* count; double scale; int np, cap; };

union ProgArgs {
  PaZero zero;
  PaMove move;
  PaMove4 move4;
  PaFused fused;
  PaDirect direct;
  PaSplitSets sets;
  PaSplitRed splitred;
  PaGemm gemm;
  PaKRed kred;
  PaAmp amp;
  PaMul mul;
  PaDot dot;
  PaEnergyFin efin;
};

// One record of a persistent memory launch (device layout).
struct ProgRec {
  int32_t kind;
  uint32_t grid;   // virtual blocks
  uint32_t first;  // first ticket of the record within its launch
  uint32_t dep0;   // its dependencies: deps[dep0 .. dep0 + ndep) (record numbers of the launch)
  uint32_t ndep;
  uint32_t pad[3];
  ProgArgs a;
};

struct ProgTouch {
  const void* p;
  bool write;
};

class ProgRecorder;
// The recorder active on the calling thread, or nullptr (launch as usual).
ProgRecorder* prog_recording();
int prog_mem(ProgRecorder* r, int kind, uint32_t grid, const ProgArgs& a, const std::vector<ProgTouch>& touches);
int prog_ext(ProgRecorder* r, std::function<int(cudaStream_t)> launch, const std::vector<ProgTouch>& touches);
int prog_split(ProgRecorder* r, SplitPlan* sp, int launch);
// cudaMemsetAsync(p, 0, bytes, st), or a zero-fill record while recording.
int zero_async(void* p, size_t bytes, cudaStream_t st);

struct ProgBuffer {
  const void* p;
  size_t bytes;
};
struct Program;
struct ProgramDeleter {
  void operator()(Program* p) const;
};
using ProgramPtr = std::unique_ptr<Program, ProgramDeleter>;

// Starts recording on this thread; conflicts on the registered buffers order
// records of different steps.
int prog_begin(const std::vector<ProgBuffer>& buffers, ProgRecorder** out);
// Records that follow belong to step `step` (and run after the step's
// earlier records).
void prog_step(ProgRecorder* r, int step);
// The stream to hand the recorded steps: it is being captured, so a launch
// that bypasses the recorder is caught (prog_finish then fails).
cudaStream_t prog_stream(ProgRecorder* r);
// Stops recording and builds the program (device tables uploaded); the
// recorder is released in any case.
int prog_finish(ProgRecorder* r, ProgramPtr& out);
// Enqueues one run of the program on st.
int prog_run(const Program& p, cudaStream_t st);
// Bound on every dependency wait of the program's memory launches (clock
// cycles; default about one second).
void prog_set_wait_limit(Program& p, long long cycles);
// Error word of the program's memory launches (0 = ok); syncs.
int prog_error(const Program& p);
struct ProgStats {
  int records, levels, launches, mem_launches, split_launches, ext_launches;
};
void prog_stats(const Program& p, ProgStats* s);
// Runs a two-record launch whose one dependency wait can never be met, with
// the given bound; *err_word receives the launch's error word (syncs st).
int prog_wait_selftest(long long limit_cycles, cudaStream_t st, int* err_word);

}  // namespace gbx
