// Persistent iteration program (program.h): the recorder, the level
// scheduler, and the persistent kernel that runs the memory records of one
// level off a device-side work queue.
#include <algorithm>
#include <cstring>
#include <memory>

#include "bodies.cuh"
#include "program.h"
#include "split.h"

namespace gbx {

namespace {

constexpr int kProgThreads = dev::kBodyThreads;
constexpr int kProgCtasPerSm = 3;
constexpr int kProgMovePer = 8;  // elements per thread and batch of the tile moves
constexpr int kProgBatch = 1;    // consecutive tickets a CTA takes at once
constexpr uint32_t kProgMaxGrid = 912;  // virtual blocks of a record: two per CTA of a launch
constexpr int kSeenWords = 128;  // records of a launch whose completion a CTA remembers: 4096
constexpr long long kProgWaitCycles = 2000000000ll;  // ~1 s at 2 GHz
constexpr int kProgErrWait = 31;  // error word: a dependency wait ran out

struct ProgLaunch {
  const ProgRec* recs;
  const uint32_t* deps;
  uint32_t* ticket;
  uint32_t* done;  // finished blocks per record
  int* err;
  long long limit;
  int nrec;
  uint32_t total;  // tickets (virtual blocks of all records)
};

union ProgSmem {
  dev::FsSmem fs;
  dev::DirSmem dir;
  dev::SmallOutSmem so;
  double red[kProgThreads];
  uint32_t red8[8];
};

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Waits until every dependency of record r has finished all its blocks.
// false (and the error word set) when a wait ran out.
__device__ __forceinline__ bool wait_deps(const ProgLaunch& L, int r, uint32_t* seen) {
  const uint32_t d0 = __ldg(&L.recs[r].dep0), nd = __ldg(&L.recs[r].ndep);
  for (uint32_t i = 0; i < nd; ++i) {
    const uint32_t d = __ldg(L.deps + d0 + i);
    const bool cacheable = d < 32u * kSeenWords;
    if (cacheable && ((seen[d >> 5] >> (d & 31)) & 1u)) continue;
    const uint32_t need = __ldg(&L.recs[d].grid);
    if (ld_acquire(L.done + d) < need) {
      const long long t0 = clock64();
      unsigned ns = 32;
      while (ld_acquire(L.done + d) < need) {
        // once one wait has run out, every later wait gives up at once
        if (clock64() - t0 > L.limit || *(volatile int*)L.err != 0) {
          atomicCAS(L.err, 0, kProgErrWait);
          return false;
        }
        __nanosleep(ns);
        if (ns < 1024) ns *= 2;
      }
    }
    if (cacheable) seen[d >> 5] |= 1u << (d & 31);
  }
  return true;
}

__device__ __forceinline__ void run_record(const ProgRec& r, uint32_t vb, ProgSmem& sm) {
  const ProgArgs& a = r.a;
  const uint32_t g = r.grid;
  switch (r.kind) {
    case PK_ZERO:
      dev::zero_body(a.zero.p, a.zero.bytes, vb, g);
      break;
    case PK_MOVE:
      dev::move_body<true>(a.move.descs, a.move.first, a.move.ndesc, a.move.nchunks, a.move.src, a.move.dst,
                           a.move.alpha, vb, g);
      break;
    case PK_MOVE4:
      dev::move4_body<true, kProgMovePer>(a.move4.descs, a.move4.chunk_desc, a.move4.nchunks, a.move4.src,
                                          a.move4.dst, a.move4.alpha, a.move4.pairs, vb, g);
      break;
    case PK_FUSED:
      dev::fused_sum_body<true>(a.fused.items, a.fused.nitems, a.fused.terms, a.fused.src, a.fused.scale, a.fused.out,
                                vb, g, sm.fs);
      break;
    case PK_DIRECT:
      if (a.direct.overwrite)
        dev::direct_body<kProgThreads, true, true>(a.direct.items, a.direct.nitems, a.direct.pairs, a.direct.A,
                                                   a.direct.B, a.direct.C, a.direct.alpha, vb, g, sm.dir);
      else
        dev::direct_body<kProgThreads, true, false>(a.direct.items, a.direct.nitems, a.direct.pairs, a.direct.A,
                                                    a.direct.B, a.direct.C, a.direct.alpha, vb, g, sm.dir);
      break;
    case PK_ROWEXP:
      dev::row_exponent_body<true>(a.sets.sets, a.sets.nsets, a.sets.total, vb, g, sm.red8);
      break;
    case PK_DIGITS:
      dev::digits_body<true>(a.sets.sets, a.sets.nsets, a.sets.total, a.sets.S, vb, g);
      break;
    case PK_SHORTROWS:
      dev::short_rows_body<true>(a.sets.sets, a.sets.nsets, a.sets.total, a.sets.S, vb, g);
      break;
    case PK_SPLITROWS:
      dev::split_rows_body<true>(a.sets.sets, a.sets.nsets, a.sets.total, a.sets.S, vb, g, sm.red8);
      break;
    case PK_SPLITRED:
      dev::split_reduce_body<true>(a.splitred.probs, a.splitred.red_prob, a.splitred.red_first, a.splitred.nred,
                                   a.splitred.total, vb, g);
      break;
    case PK_GEMV:
      dev::gemv_body<true>(a.gemm.probs, a.gemm.nprob, a.gemm.first, a.gemm.total, vb, g);
      break;
    case PK_SMALLOUT:
      dev::small_out_body<true>(a.gemm.probs, a.gemm.nprob, a.gemm.first, a.gemm.total, vb, g, sm.so);
      break;
    case PK_SMALLK:
      dev::small_k_body<true>(a.gemm.probs, a.gemm.nprob, a.gemm.first, a.gemm.total, vb, g);
      break;
    case PK_SPLITKRED:
      dev::splitk_reduce_body<true>(a.kred.probs, a.kred.red_prob, a.kred.red_first, a.kred.nred, a.kred.nchunks, vb,
                                    g);
      break;
    case PK_AMP:
      dev::cc_amp_body<true>(a.amp.tiles, a.amp.items, a.amp.nitems, a.amp.t1, a.amp.t2, a.amp.tau, a.amp.taut,
                             a.amp.Q, vb, g);
      break;
    case PK_MUL:
      dev::mul_body<true>(a.mul.a, a.mul.b, a.mul.out, a.mul.n, vb, g);
      break;
    case PK_DOTPART:
      dev::dot_partial_body<true>(a.dot.x, a.dot.y, a.dot.n, a.dot.partial, vb, g, sm.red);
      break;
    case PK_ENERGYFIN:
      dev::energy_final_body<true>(a.efin.partial, a.efin.np, a.efin.scale, a.efin.hist, a.efin.count, a.efin.cap,
                                   vb, sm.red);
      break;
    default:
      break;
  }
}

__device__ __forceinline__ void release_add(uint32_t* p, uint32_t n) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(n) : "memory");
}

// One CTA: take a ticket, find its record, wait for the record's
// dependencies, run the record's body for that virtual block.  The next
// ticket is taken while the current one runs.  Finished blocks are counted
// per record and released (one release-add) when the CTA moves on to
// another record or ends: a record's count completes when the last CTA
// working on it leaves it, which is when its last block is done, so nothing
// waits longer, and the CTA pays one release per record instead of one per
// block.  The CTA releases what it holds before it waits on anything.
__global__ void __launch_bounds__(kProgThreads, kProgCtasPerSm) prog_mem_kernel(const ProgLaunch L) {
  __shared__ ProgSmem sm;
  __shared__ ProgRec srec;
  __shared__ uint32_t seen[kSeenWords];
  __shared__ uint32_t s_t, s_next;
  __shared__ int s_r, s_ok;
  const int tid = threadIdx.x;
  for (int i = tid; i < kSeenWords; i += kProgThreads) seen[i] = 0u;
  if (tid == 0) s_t = atomicAdd(L.ticket, (uint32_t)kProgBatch);
  __syncthreads();
  uint32_t t = s_t;
  uint32_t nxt = 0;
  uint32_t batch_end = t + kProgBatch;  // this CTA's tickets run to batch_end (thread 0)
  int prev = -1;       // the record of this CTA's previous block: its dependencies are met, srec holds it
  uint32_t lo_t = 0, hi_t = 0;  // tickets of record prev (thread 0)
  uint32_t pend = 0;   // finished blocks of record prev not yet released (thread 0)
  int ok = 1;
  while (t < L.total) {
    if (tid == 0) {
      // the next batch is taken while the first block of this one runs
      if (t + kProgBatch == batch_end) nxt = atomicAdd(L.ticket, (uint32_t)kProgBatch);
      int r = prev;
      if (!(t >= lo_t && t < hi_t)) {
        int lo = 0, hi = L.nrec - 1;
        while (lo < hi) {
          const int mid = (lo + hi + 1) >> 1;
          if (__ldg(&L.recs[mid].first) <= t) lo = mid; else hi = mid - 1;
        }
        r = lo;
        if (pend) release_add(L.done + prev, pend);
        pend = 0;
        lo_t = __ldg(&L.recs[r].first);
        hi_t = lo_t + __ldg(&L.recs[r].grid);
        s_ok = wait_deps(L, r, seen) ? 1 : 0;
      }
      s_r = r;
    }
    __syncthreads();
    const int r = s_r;
    if (r != prev) {
      ok = s_ok;
      const uint32_t* src = reinterpret_cast<const uint32_t*>(L.recs + r);
      uint32_t* dst = reinterpret_cast<uint32_t*>(&srec);
      for (int i = tid; i < (int)(sizeof(ProgRec) / 4); i += kProgThreads) dst[i] = __ldg(src + i);
      __syncthreads();
      prev = r;
    }
    if (ok) run_record(srec, t - srec.first, sm);
    if (tid == 0) {
      if (t + 1 < batch_end) {
        s_next = t + 1;
      } else {
        s_next = nxt;
        batch_end = nxt + kProgBatch;
      }
      ++pend;
    }
    __syncthreads();
    t = s_next;
  }
  if (tid == 0 && pend) release_add(L.done + prev, pend);
}

static_assert(sizeof(ProgRec) % 4 == 0, "record copy");

struct RecEntry {
  int cls = 0;  // 0 memory record, 1 split GEMM launch, 2 external launch
  int kind = 0;
  uint32_t grid = 0;
  ProgArgs a;
  SplitPlan* sp = nullptr;
  int launch = -1, split_cls = -1;
  std::function<int(cudaStream_t)> ext;
  int step = -1;
  std::vector<int> deps;  // earlier records, any class
  int level = 0;
};

thread_local ProgRecorder* g_rec = nullptr;

}  // namespace

class ProgRecorder {
 public:
  std::vector<ProgBuffer> bufs;  // sorted by address
  std::vector<int> last_writer;
  std::vector<std::vector<int>> readers;
  std::vector<RecEntry> recs;
  // per step: its last record that is not a split GEMM launch, and the split
  // GEMM launches recorded after it (independent of one another)
  std::vector<int> step_last;
  std::vector<std::vector<int>> step_splits;
  int step = -1;
  cudaStream_t cap = nullptr;  // captures (and so detects) any launch that was not recorded

  int find(const void* p) const {
    if (!p) return -1;
    const uintptr_t a = (uintptr_t)p;
    int lo = 0, hi = (int)bufs.size() - 1, best = -1;
    while (lo <= hi) {
      const int mid = (lo + hi) / 2;
      if ((uintptr_t)bufs[mid].p <= a) {
        best = mid;
        lo = mid + 1;
      } else {
        hi = mid - 1;
      }
    }
    if (best < 0 || a >= (uintptr_t)bufs[best].p + bufs[best].bytes) return -1;
    return best;
  }

  int add(RecEntry&& e, const std::vector<ProgTouch>& touches) {
    const int idx = (int)recs.size();
    e.step = step;
    if (step >= 0) {
      if ((int)step_last.size() <= step) {
        step_last.resize(step + 1, -1);
        step_splits.resize(step + 1);
      }
      // the GEMM launches of one contraction (one per kernel) all follow
      // its operand preparation and all precede what reads their outputs
      if (step_last[step] >= 0) e.deps.push_back(step_last[step]);
      if (e.cls == 1) {
        step_splits[step].push_back(idx);
      } else {
        for (int q : step_splits[step]) e.deps.push_back(q);
        step_splits[step].clear();
        step_last[step] = idx;
      }
    }
    // buffers written (a buffer both read and written counts as written)
    std::vector<int> wr, rd;
    for (const ProgTouch& t : touches) {
      const int b = find(t.p);
      if (b < 0) continue;
      (t.write ? wr : rd).push_back(b);
    }
    std::sort(wr.begin(), wr.end());
    wr.erase(std::unique(wr.begin(), wr.end()), wr.end());
    std::sort(rd.begin(), rd.end());
    rd.erase(std::unique(rd.begin(), rd.end()), rd.end());
    for (int b : wr) {
      if (last_writer[b] >= 0) e.deps.push_back(last_writer[b]);
      for (int r : readers[b]) e.deps.push_back(r);
    }
    for (int b : rd) {
      if (std::binary_search(wr.begin(), wr.end(), b)) continue;
      if (last_writer[b] >= 0) e.deps.push_back(last_writer[b]);
    }
    for (int b : wr) {
      last_writer[b] = idx;
      readers[b].clear();
    }
    for (int b : rd)
      if (!std::binary_search(wr.begin(), wr.end(), b)) readers[b].push_back(idx);
    std::sort(e.deps.begin(), e.deps.end());
    e.deps.erase(std::unique(e.deps.begin(), e.deps.end()), e.deps.end());
    recs.push_back(std::move(e));
    return GBX_OK;
  }
};

ProgRecorder* prog_recording() { return g_rec; }

int prog_mem(ProgRecorder* r, int kind, uint32_t grid, const ProgArgs& a, const std::vector<ProgTouch>& touches) {
  if (grid == 0) return GBX_OK;
  // larger work items (every body but the dot product's computes each
  // element the same way whatever its block count)
  if (kind != PK_DOTPART) grid = std::min<uint32_t>(grid, kProgMaxGrid);
  RecEntry e;
  e.cls = 0;
  e.kind = kind;
  e.grid = grid;
  e.a = a;
  return r->add(std::move(e), touches);
}

int prog_ext(ProgRecorder* r, std::function<int(cudaStream_t)> launch, const std::vector<ProgTouch>& touches) {
  RecEntry e;
  e.cls = 2;
  e.ext = std::move(launch);
  return r->add(std::move(e), touches);
}

int prog_split(ProgRecorder* r, SplitPlan* sp, int launch) {
  RecEntry e;
  e.cls = 1;
  e.sp = sp;
  e.launch = launch;
  e.split_cls = split_launch_class(sp, launch);
  if (e.split_cls < 0) return fail(GBX_EINVAL, "program: bad split launch");
  return r->add(std::move(e), {});
}

int zero_async(void* p, size_t bytes, cudaStream_t st) {
  if (bytes == 0) return GBX_OK;
  if (ProgRecorder* r = g_rec) {
    if ((((uintptr_t)p | bytes) & 3) == 0) {
      ProgArgs a;
      a.zero = {p, (uint64_t)bytes};
      const uint64_t words = bytes / 16 + 1;
      const uint32_t grid = (uint32_t)std::min<uint64_t>((words + kProgThreads - 1) / kProgThreads, 152 * 8);
      return prog_mem(r, PK_ZERO, grid, a, {{p, true}});
    }
    return prog_ext(r, [p, bytes](cudaStream_t s2) {
      GBX_CUDA(cudaMemsetAsync(p, 0, bytes, s2));
      return GBX_OK;
    }, {{p, true}});
  }
  GBX_CUDA(cudaMemsetAsync(p, 0, bytes, st));
  return GBX_OK;
}

struct Program {
  struct Op {
    int type;  // 0 memory launch, 1 merged split launch, 2 external
    int idx;
  };
  struct MemLaunch {
    ProgRec* d_recs = nullptr;
    uint32_t* d_deps = nullptr;
    int nrec = 0;
    uint32_t total = 0;
    size_t ticket_off = 0, done_off = 0;  // in counter words
    int grid = 0;
  };
  std::vector<Op> ops;
  std::vector<MemLaunch> mem;
  std::vector<SplitMerged*> merged;
  std::vector<std::function<int(cudaStream_t)>> ext;
  uint32_t* d_counters = nullptr;
  size_t counter_words = 0;
  int* d_err = nullptr;
  long long limit = kProgWaitCycles;
  ProgStats stats{};
  ~Program() {
    for (auto& m : mem) {
      dev_free(m.d_recs);
      dev_free(m.d_deps);
    }
    for (SplitMerged* m : merged) split_merged_destroy(m);
    dev_free(d_counters);
    dev_free(d_err);
  }
};

void ProgramDeleter::operator()(Program* p) const { delete p; }

int prog_begin(const std::vector<ProgBuffer>& buffers, ProgRecorder** out) {
  if (g_rec) return fail(GBX_EINVAL, "program: already recording on this thread");
  auto r = std::make_unique<ProgRecorder>();
  for (const ProgBuffer& b : buffers)
    if (b.p && b.bytes) r->bufs.push_back(b);
  std::sort(r->bufs.begin(), r->bufs.end(), [](const ProgBuffer& x, const ProgBuffer& y) { return x.p < y.p; });
  for (size_t i = 1; i < r->bufs.size(); ++i)
    if ((uintptr_t)r->bufs[i - 1].p + r->bufs[i - 1].bytes > (uintptr_t)r->bufs[i].p)
      return fail(GBX_EINVAL, "program: registered buffers overlap");
  r->last_writer.assign(r->bufs.size(), -1);
  r->readers.assign(r->bufs.size(), {});
  GBX_CUDA(cudaStreamCreateWithFlags(&r->cap, cudaStreamNonBlocking));
  cudaError_t e = cudaStreamBeginCapture(r->cap, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    cudaStreamDestroy(r->cap);
    return cuda_fail(e, "cudaStreamBeginCapture", __FILE__, __LINE__);
  }
  *out = r.release();
  g_rec = *out;
  return GBX_OK;
}

void prog_step(ProgRecorder* r, int step) { r->step = step; }

cudaStream_t prog_stream(ProgRecorder* r) { return r->cap; }

namespace {

// Builds the program from the recorded entries.
int build_program(ProgRecorder& R, Program& P) {
  std::vector<RecEntry>& E = R.recs;
  const int n = (int)E.size();
  // levels
  int nlev = 0;
  for (int i = 0; i < n; ++i) {
    RecEntry& e = E[i];
    int lv = 0;
    for (int d : e.deps) {
      const RecEntry& q = E[d];
      int need;
      if (e.cls == 2) need = q.level;                   // external: stream order after anything of its level
      else need = q.cls == 0 ? q.level : q.level + 1;   // memory and split: after the launches of q's level
      lv = std::max(lv, need);
    }
    e.level = lv;
    nlev = std::max(nlev, lv + 1);
  }
  GBX_TRY(dev_alloc((void**)&P.d_err, sizeof(int)));
  GBX_CUDA(cudaMemset(P.d_err, 0, sizeof(int)));
  int dev = 0, nsm = 152, occ = 0;
  GBX_CUDA(cudaGetDevice(&dev));
  GBX_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  GBX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, prog_mem_kernel, kProgThreads, 0));
  if (occ < 1) return fail(GBX_ECUDA, "program: memory kernel does not fit an SM");
  std::vector<int> local(n, -1);
  size_t words = 0;
  std::vector<size_t> ticket_off(nlev), done_off(nlev);
  int records = 0;
  for (int lv = 0; lv < nlev; ++lv) {
    // memory launch of the level
    std::vector<int> ids;
    for (int i = 0; i < n; ++i)
      if (E[i].level == lv && E[i].cls == 0) ids.push_back(i);
    if (!ids.empty()) {
      // tickets in order of dependency depth inside the launch (program
      // order within a depth): the records of one depth are independent,
      // so CTAs move on to them instead of waiting on a chain
      {
        std::vector<int> depth(n, 0);
        for (int i : ids)
          for (int d : E[i].deps)
            if (E[d].cls == 0 && E[d].level == lv) depth[i] = std::max(depth[i], depth[d] + 1);
        std::stable_sort(ids.begin(), ids.end(), [&](int x, int y) { return depth[x] < depth[y]; });
      }
      for (size_t k = 0; k < ids.size(); ++k) local[ids[k]] = (int)k;
      const int m = (int)ids.size();
      // dependencies inside the launch, transitively reduced
      std::vector<std::vector<int>> dl(m);
      const int words64 = (m + 63) / 64;
      std::vector<std::vector<uint64_t>> reach(m, std::vector<uint64_t>(words64, 0));
      for (int k = 0; k < m; ++k) {
        for (int d : E[ids[k]].deps)
          if (E[d].cls == 0 && E[d].level == lv) dl[k].push_back(local[d]);
        std::sort(dl[k].begin(), dl[k].end());
        for (int d : dl[k]) {
          for (int w = 0; w < words64; ++w) reach[k][w] |= reach[d][w];
          reach[k][d >> 6] |= 1ull << (d & 63);
        }
      }
      std::vector<ProgRec> hr(m);
      std::vector<uint32_t> hd;
      uint32_t tickets = 0;
      for (int k = 0; k < m; ++k) {
        const RecEntry& e = E[ids[k]];
        ProgRec& r = hr[k];
        std::memset(&r, 0, sizeof(r));
        r.kind = e.kind;
        r.grid = e.grid;
        r.first = tickets;
        r.a = e.a;
        r.dep0 = (uint32_t)hd.size();
        for (int d : dl[k]) {
          bool implied = false;
          for (int o : dl[k])
            if (o != d && ((reach[o][d >> 6] >> (d & 63)) & 1ull)) {
              implied = true;
              break;
            }
          if (!implied) hd.push_back((uint32_t)d);
        }
        r.ndep = (uint32_t)hd.size() - r.dep0;
        if ((uint64_t)tickets + e.grid >= (1ull << 31)) return fail(GBX_EUNSUPPORTED, "program: too many work items");
        tickets += e.grid;
      }
      Program::MemLaunch ml;
      ml.nrec = m;
      ml.total = tickets;
      ml.grid = (int)std::min<uint32_t>(tickets, (uint32_t)(nsm * occ));
      ml.ticket_off = words;
      words += 32;  // one counter per 128-byte line
      ml.done_off = words;
      words += ((size_t)m + 31) / 32 * 32;
      GBX_TRY(dev_alloc((void**)&ml.d_recs, sizeof(ProgRec) * m));
      GBX_CUDA(cudaMemcpy(ml.d_recs, hr.data(), sizeof(ProgRec) * m, cudaMemcpyHostToDevice));
      if (!hd.empty()) {
        GBX_TRY(dev_alloc((void**)&ml.d_deps, sizeof(uint32_t) * hd.size()));
        GBX_CUDA(cudaMemcpy(ml.d_deps, hd.data(), sizeof(uint32_t) * hd.size(), cudaMemcpyHostToDevice));
      }
      P.ops.push_back({0, (int)P.mem.size()});
      P.mem.push_back(ml);
      records += m;
    }
    // merged split GEMM launches of the level, one per class, in order of
    // first appearance
    std::vector<int> classes;
    for (int i = 0; i < n; ++i)
      if (E[i].level == lv && E[i].cls == 1 &&
          std::find(classes.begin(), classes.end(), E[i].split_cls) == classes.end())
        classes.push_back(E[i].split_cls);
    for (int c : classes) {
      std::vector<std::pair<SplitPlan*, int>> parts;
      for (int i = 0; i < n; ++i)
        if (E[i].level == lv && E[i].cls == 1 && E[i].split_cls == c) parts.push_back({E[i].sp, E[i].launch});
      SplitMerged* sm = nullptr;
      GBX_TRY(split_merge(parts, P.d_err, &sm));
      P.ops.push_back({1, (int)P.merged.size()});
      P.merged.push_back(sm);
      records += (int)parts.size();
    }
    for (int i = 0; i < n; ++i)
      if (E[i].level == lv && E[i].cls == 2) {
        P.ops.push_back({2, (int)P.ext.size()});
        P.ext.push_back(E[i].ext);
        ++records;
      }
  }
  P.counter_words = std::max<size_t>(words, 32);
  GBX_TRY(dev_alloc((void**)&P.d_counters, sizeof(uint32_t) * P.counter_words));
  GBX_CUDA(cudaMemset(P.d_counters, 0, sizeof(uint32_t) * P.counter_words));
  P.stats.records = records;
  P.stats.levels = nlev;
  P.stats.mem_launches = (int)P.mem.size();
  P.stats.split_launches = (int)P.merged.size();
  P.stats.ext_launches = (int)P.ext.size();
  P.stats.launches = (int)P.ops.size();
  return GBX_OK;
}

}  // namespace

int prog_finish(ProgRecorder* r, ProgramPtr& out) {
  std::unique_ptr<ProgRecorder> R(r);
  if (g_rec == r) g_rec = nullptr;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(R->cap, &g);
  cudaStreamDestroy(R->cap);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
  size_t nodes = 0;
  if (g) {
    cudaGraphGetNodes(g, nullptr, &nodes);
    cudaGraphDestroy(g);
  }
  if (nodes) return fail(GBX_EUNSUPPORTED, "program: %zu operations of the iteration were launched, not recorded", nodes);
  ProgramPtr P(new Program());
  GBX_TRY(build_program(*R, *P));
  out = std::move(P);
  return GBX_OK;
}

int prog_run(const Program& P, cudaStream_t st) {
  GBX_CUDA(cudaMemsetAsync(P.d_counters, 0, sizeof(uint32_t) * P.counter_words, st));
  for (const Program::Op& op : P.ops) {
    if (op.type == 0) {
      const Program::MemLaunch& m = P.mem[op.idx];
      ProgLaunch L;
      L.recs = m.d_recs;
      L.deps = m.d_deps;
      L.ticket = P.d_counters + m.ticket_off;
      L.done = P.d_counters + m.done_off;
      L.err = P.d_err;
      L.limit = P.limit;
      L.nrec = m.nrec;
      L.total = m.total;
      prog_mem_kernel<<<m.grid, kProgThreads, 0, st>>>(L);
      GBX_CUDA(cudaGetLastError());
    } else if (op.type == 1) {
      GBX_TRY(split_merged_run(P.merged[op.idx], st));
    } else {
      GBX_TRY(P.ext[op.idx](st));
    }
  }
  return GBX_OK;
}

void prog_set_wait_limit(Program& p, long long cycles) { p.limit = cycles > 0 ? cycles : kProgWaitCycles; }

int prog_error(const Program& p) {
  int e = 0;
  if (cudaMemcpy(&e, p.d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
  return e;
}

void prog_stats(const Program& p, ProgStats* s) { *s = p.stats; }

// Self-test of the bounded dependency wait: a launch of two records in which
// the second waits for two blocks of the first, of which only one is ever
// issued (the first record's second block has no ticket).  The wait runs
// out after limit_cycles, the error word is set and both CTAs return.
int prog_wait_selftest(long long limit_cycles, cudaStream_t st, int* err_word) {
  ProgRec h[2];
  std::memset(h, 0, sizeof(h));
  h[0].kind = PK_NOP;
  h[0].grid = 2;  // the dependency's target: two finished blocks
  h[0].first = 0;
  h[1].kind = PK_NOP;
  h[1].grid = 1;
  h[1].first = 1;
  h[1].dep0 = 0;
  h[1].ndep = 1;
  uint32_t dep = 0;
  ProgRec* d_recs = nullptr;
  uint32_t *d_deps = nullptr, *d_cnt = nullptr;
  int* d_err = nullptr;
  int rc = dev_alloc((void**)&d_recs, sizeof(h));
  if (rc == GBX_OK) rc = dev_alloc((void**)&d_deps, sizeof(uint32_t));
  if (rc == GBX_OK) rc = dev_alloc((void**)&d_cnt, 64 * sizeof(uint32_t));
  if (rc == GBX_OK) rc = dev_alloc((void**)&d_err, sizeof(int));
  cudaError_t e = cudaSuccess;
  if (rc == GBX_OK) {
    e = cudaMemcpyAsync(d_recs, h, sizeof(h), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_deps, &dep, sizeof(dep), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_cnt, 0, 64 * sizeof(uint32_t), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_err, 0, sizeof(int), st);
    if (e == cudaSuccess) {
      ProgLaunch L;
      L.recs = d_recs;
      L.deps = d_deps;
      L.ticket = d_cnt;
      L.done = d_cnt + 32;
      L.err = d_err;
      L.limit = limit_cycles;
      L.nrec = 2;
      L.total = 2;  // tickets 0 (record 0, block 0) and 1 (record 1)
      prog_mem_kernel<<<2, kProgThreads, 0, st>>>(L);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(err_word, d_err, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  dev_free(d_recs);
  dev_free(d_deps);
  dev_free(d_cnt);
  dev_free(d_err);
  if (rc != GBX_OK) return rc;
  if (e != cudaSuccess) return cuda_fail(e, "program wait self-test", __FILE__, __LINE__);
  return GBX_OK;
}

}  // namespace gbx
