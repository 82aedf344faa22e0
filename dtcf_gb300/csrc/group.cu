// Grouped block triples: every (A-block, B-block -> C-block) product of one
// launch set, C_t (+)= alpha_t A_t B_t^T, planned once and run as one
// persistent launch per kernel kind (FP64 tile shapes on the FP64 pipe, or
// split-precision slices on tcgen05), with an autotuner that picks the
// engine, orientation and tile shape per class of triple shapes by timing.
//
// This is the leaf GEMM work of DTCF's transpose_and_dgemm
// (contraction.cc:1779-1976) and of DLTC's task_mul (DLTC/task.cc:83-137)
// issued as one batch instead of one dgemm call per block pair.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <tuple>
#include <vector>

#include "../../include/gbx.h"
#include "common.h"
#include "plan.h"
#include "split.h"

namespace gbx {
namespace {

// Split-engine outputs that cannot be written in place (accumulate, alpha,
// swapped orientation or strided C) land in a workspace and are applied here.
struct ApplyDesc {
  double* C;
  int64_t c_rs;
  int64_t off;  // workspace offset of the m x n (or n x m when trans) result
  int m, n;
  double alpha;
  int accumulate, trans;
};

__global__ void __launch_bounds__(256) apply_kernel(const ApplyDesc* __restrict__ d, int nd,
                                                    const int64_t* __restrict__ first, int64_t total,
                                                    const double* __restrict__ W) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = nd - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (first[mid] <= e) lo = mid; else hi = mid - 1;
    }
    const ApplyDesc& a = d[lo];
    const int64_t l = e - first[lo];
    int64_t i, j;
    if (a.trans) {  // workspace holds C^T (n x m): walk it in its own order
      j = l / a.m;
      i = l - j * a.m;
    } else {
      i = l / a.n;
      j = l - i * a.n;
    }
    const double v = __dmul_rn(a.alpha, W[a.off + l]);
    double* c = a.C + i * a.c_rs + j;
    *c = a.accumulate ? __dadd_rn(*c, v) : v;
  }
}

// Per-triple choice.  engine 0: FP64 with tile variant `variant` (-1 = the
// model's); engine 1: split with output tile width `width` (0 = model) in
// the given orientation.
struct Choice {
  int engine = 0, variant = -1, width = 0;
  bool swap = false;
  bool operator<(const Choice& o) const {
    return std::tie(engine, variant, width, swap) < std::tie(o.engine, o.variant, o.width, o.swap);
  }
};

bool split_capable(const gbx_triple& t) { return t.a_cs == 1 && t.b_cs == 1; }

Choice model_choice(const gbx_triple& t, int mode, int slices) {
  Choice c;
  if (mode == GBX_MODE_FP64 || !split_capable(t)) return c;
  GroupBlock g;
  g.h = 0;
  g.M = t.m;
  g.N = t.n;
  g.K = t.k;
  choose_engine(g, true, mode == GBX_MODE_SPLIT, slices);
  c.engine = g.engine;
  c.swap = g.swap;
  return c;
}

}  // namespace

// The planned state of one set of triples.
struct GroupPlan {
  std::vector<gbx_triple> tri;
  std::vector<Choice> choice;
  int slices = 6;
  F64Gemm f64;
  SplitPlan* split = nullptr;
  double* d_w = nullptr;
  ApplyDesc* d_apply = nullptr;
  int64_t* d_apply_first = nullptr;
  int napply = 0;
  int64_t apply_total = 0;
  int n_f64 = 0, n_split = 0;
  double flops = 0.0;

  void release() {
    f64.release();
    destroy_split_plan(split);
    split = nullptr;
    dev_free(d_w);
    dev_free(d_apply);
    dev_free(d_apply_first);
    d_w = nullptr;
    d_apply = nullptr;
    d_apply_first = nullptr;
    napply = 0;
    apply_total = 0;
  }
  ~GroupPlan() { release(); }

  int build() {
    release();
    std::vector<GemmProblem> probs;
    std::vector<int> variants;
    std::vector<SplitProblem> sp;
    std::vector<ApplyDesc> ap;
    std::vector<int64_t> ap_first;
    std::vector<int64_t> w_off;  // per split problem: workspace offset of its output, -1 = written in place
    int64_t w_elems = 0;
    flops = 0.0;
    for (size_t i = 0; i < tri.size(); ++i) {
      const gbx_triple& t = tri[i];
      const Choice& c = choice[i];
      flops += 2.0 * t.m * (double)t.n * t.k;
      if (t.m <= 0 || t.n <= 0) continue;
      if (c.engine == 0 || t.k <= 0) {
        GemmProblem q;
        std::memset(&q, 0, sizeof(q));
        q.A = t.A;
        q.B = t.B;
        q.C = t.C;
        q.a_rs = t.a_rs;
        q.a_cs = t.a_cs;
        q.b_rs = t.b_rs;
        q.b_cs = t.b_cs;
        q.c_rs = t.c_rs;
        q.m = t.m;
        q.n = t.n;
        q.k = t.k;
        q.alpha = t.alpha;
        q.accumulate = t.accumulate;
        probs.push_back(q);
        variants.push_back(c.variant);
        continue;
      }
      if (!split_capable(t)) return fail(GBX_EUNSUPPORTED, "triple %zu: the split engine needs unit column strides", i);
      SplitProblem q;
      q.K = t.k;
      q.width = c.width;
      if (c.swap) {  // C^T = B A^T
        q.A = t.B;
        q.B = t.A;
        q.M = t.n;
        q.N = t.m;
        q.lda = t.b_rs;
        q.ldb = t.a_rs;
      } else {
        q.A = t.A;
        q.B = t.B;
        q.M = t.m;
        q.N = t.n;
        q.lda = t.a_rs;
        q.ldb = t.b_rs;
      }
      const bool direct = !c.swap && !t.accumulate && t.alpha == 1.0;
      if (direct) {
        q.C = t.C;
        q.ldc = t.c_rs;
        w_off.push_back(-1);
      } else {
        ApplyDesc a;
        a.C = t.C;
        a.c_rs = t.c_rs;
        a.off = w_elems;
        a.m = t.m;
        a.n = t.n;
        a.alpha = t.alpha;
        a.accumulate = t.accumulate;
        a.trans = c.swap;
        q.C = nullptr;  // set once the workspace exists
        q.ldc = 0;
        w_off.push_back(w_elems);
        ap.push_back(a);
        ap_first.push_back(apply_total);
        apply_total += (int64_t)t.m * t.n;
        w_elems += (int64_t)t.m * t.n;
      }
      sp.push_back(q);
    }
    n_f64 = (int)probs.size();
    n_split = (int)sp.size();
    GBX_TRY(f64.build(probs, false, nullptr, &variants));
    if (w_elems) {
      GBX_TRY(dev_alloc((void**)&d_w, sizeof(double) * w_elems));
      for (size_t i = 0; i < sp.size(); ++i)
        if (w_off[i] >= 0) sp[i].C = d_w + w_off[i];
    }
    if (!sp.empty()) GBX_TRY(create_split_plan(sp, slices, &split));
    if (!ap.empty()) {
      napply = (int)ap.size();
      GBX_TRY(dev_alloc((void**)&d_apply, sizeof(ApplyDesc) * ap.size()));
      GBX_TRY(dev_alloc((void**)&d_apply_first, sizeof(int64_t) * ap.size()));
      GBX_CUDA(cudaMemcpy(d_apply, ap.data(), sizeof(ApplyDesc) * ap.size(), cudaMemcpyHostToDevice));
      GBX_CUDA(cudaMemcpy(d_apply_first, ap_first.data(), sizeof(int64_t) * ap.size(), cudaMemcpyHostToDevice));
    }
    return GBX_OK;
  }

  int run(bool per_triple, cudaStream_t st) {
    if (per_triple) GBX_TRY(f64.run_each(st));
    else GBX_TRY(f64.run(st));
    if (split) GBX_TRY(run_split_plan(split, true, true, st));
    if (napply) {
      const int grid = (int)std::min<int64_t>((apply_total + 255) / 256, 152 * 8);
      apply_kernel<<<grid, 256, 0, st>>>(d_apply, napply, d_apply_first, apply_total, d_w);
      GBX_CUDA(cudaGetLastError());
    }
    return GBX_OK;
  }
};

namespace {

// Shape class of a triple for the autotuner: log4 bins of m, n and k.
int shape_bin(int x) {
  int b = 0;
  while (x >= 16 && b < 7) {
    x >>= 2;
    ++b;
  }
  return b;
}
int bucket_of(const gbx_triple& t) { return (shape_bin(t.m) * 8 + shape_bin(t.n)) * 8 + shape_bin(t.k); }

// Time one candidate over a set of triples written to scratch outputs:
// the marginal cost of the set, (T(4 copies) - T(1 copy)) / 3, so that the
// fixed launch overheads shared by a whole group do not bias the choice.
int time_candidate(const std::vector<gbx_triple>& set, const Choice& c, int slices, double* scratch, int reps,
                   cudaStream_t st, double* out_ms) {
  float t[2] = {0.f, 0.f};
  const int copies[2] = {1, 4};
  cudaEvent_t e0, e1;
  GBX_CUDA(cudaEventCreate(&e0));
  GBX_CUDA(cudaEventCreate(&e1));
  for (int r = 0; r < 2; ++r) {
    GroupPlan g;
    g.slices = slices;
    int64_t off = 0;
    for (int cp = 0; cp < copies[r]; ++cp)
      for (const gbx_triple& x : set) {
        gbx_triple y = x;
        y.C = scratch + off;
        y.c_rs = x.n;
        y.alpha = 1.0;
        y.accumulate = 0;
        off += (int64_t)x.m * x.n;
        g.tri.push_back(y);
        g.choice.push_back(c);
      }
    int rc = g.build();
    if (rc != GBX_OK) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return rc;
    }
    GBX_TRY(g.run(false, st));  // warm
    float best = 1e30f;
    for (int k = 0; k < reps; ++k) {
      GBX_CUDA(cudaEventRecord(e0, st));
      GBX_TRY(g.run(false, st));
      GBX_CUDA(cudaEventRecord(e1, st));
      GBX_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      GBX_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      best = std::min(best, ms);
    }
    t[r] = best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *out_ms = (t[1] - t[0]) / 3.0;
  return GBX_OK;
}

}  // namespace
}  // namespace gbx

struct gbx_group {
  gbx::GroupPlan plan;
  int mode = 0;
};

extern "C" {

int gbx_group_create(const gbx_triple* triples, int num_triples, int mode, int slices, gbx_group** out) {
  using namespace gbx;
  if (!out) return fail(GBX_EINVAL, "null output");
  *out = nullptr;
  if (num_triples < 0 || (num_triples > 0 && !triples)) return fail(GBX_EINVAL, "bad triple array");
  if (mode != GBX_MODE_FP64 && mode != GBX_MODE_SPLIT && mode != GBX_MODE_AUTO)
    return fail(GBX_EINVAL, "unknown mode %d", mode);
  if (slices != 0 && (slices < 2 || slices > 7)) return fail(GBX_EINVAL, "split slices must be 0 or in [2, 7]");
  auto g = std::make_unique<gbx_group>();
  g->mode = mode;
  g->plan.slices = slices ? slices : 6;
  for (int i = 0; i < num_triples; ++i) {
    const gbx_triple& t = triples[i];
    if (t.m < 0 || t.n < 0 || t.k < 0) return fail(GBX_EINVAL, "triple %d: negative extent", i);
    if ((t.m > 0 && t.n > 0) && (!t.C || (t.k > 0 && (!t.A || !t.B))))
      return fail(GBX_EINVAL, "triple %d: null operand", i);
    if (mode == GBX_MODE_SPLIT && t.k > 0 && t.m > 0 && t.n > 0 && !split_capable(t))
      return fail(GBX_EUNSUPPORTED, "triple %d: the split engine needs unit column strides (a_cs = b_cs = 1)", i);
    g->plan.tri.push_back(t);
    g->plan.choice.push_back(model_choice(t, mode, g->plan.slices));
  }
  GBX_TRY(g->plan.build());
  *out = g.release();
  return GBX_OK;
}

int gbx_group_execute(gbx_group* g, int per_triple, void* stream) {
  using namespace gbx;
  if (!g) return fail(GBX_EINVAL, "null group");
  GBX_TRY(g->plan.run(per_triple != 0, (cudaStream_t)stream));
  return GBX_OK;
}

int gbx_group_autotune(gbx_group* g, int reps, void* stream) {
  using namespace gbx;
  if (!g) return fail(GBX_EINVAL, "null group");
  if (reps < 1) reps = 3;
  cudaStream_t st = (cudaStream_t)stream;
  GroupPlan& P = g->plan;
  std::map<int, std::vector<int>> buckets;
  for (size_t i = 0; i < P.tri.size(); ++i) {
    const gbx_triple& t = P.tri[i];
    if (t.m > 0 && t.n > 0 && t.k > 0) buckets[bucket_of(t)].push_back((int)i);
  }
  int64_t scratch_elems = 1;
  for (auto& b : buckets) {
    int64_t e = 0;
    for (int i : b.second) e += (int64_t)P.tri[i].m * P.tri[i].n;
    scratch_elems = std::max(scratch_elems, 4 * e);
  }
  double* scratch = nullptr;
  GBX_TRY(dev_alloc((void**)&scratch, sizeof(double) * scratch_elems));
  int rc = GBX_OK;
  for (auto& b : buckets) {
    std::vector<gbx_triple> set;
    bool splittable = g->mode != GBX_MODE_FP64;
    int maxm = 0, maxn = 0, maxk = 0;
    for (int i : b.second) {
      set.push_back(P.tri[i]);
      splittable = splittable && split_capable(P.tri[i]);
      maxm = std::max(maxm, P.tri[i].m);
      maxn = std::max(maxn, P.tri[i].n);
      maxk = std::max(maxk, P.tri[i].k);
    }
    std::vector<Choice> cand;
    if (g->mode != GBX_MODE_SPLIT)
      for (int v = 0; v < 4; ++v) {
        Choice c;
        c.variant = v;
        cand.push_back(c);
      }
    if (splittable)
      for (int sw = 0; sw < 2; ++sw)
        for (int w : {32, 64, 128, 256}) {
          const int cols = sw ? maxm : maxn;
          if (w > 32 && w / 2 >= cols) continue;  // wider than twice the output: only padding
          Choice c;
          c.engine = 1;
          c.width = w;
          c.swap = sw != 0;
          cand.push_back(c);
        }
    Choice best;
    double best_ms = 1e300;
    for (const Choice& c : cand) {
      double ms = 0.0;
      rc = time_candidate(set, c, P.slices, scratch, reps, st, &ms);
      if (rc != GBX_OK) break;
      if (ms < best_ms) {
        best_ms = ms;
        best = c;
      }
    }
    if (rc != GBX_OK) break;
    for (int i : b.second) P.choice[i] = best;
  }
  dev_free(scratch);
  GBX_TRY(rc);
  GBX_TRY(P.build());
  return GBX_OK;
}

int gbx_group_info(const gbx_group* g, int* engines, int* params, double* flops) {
  using namespace gbx;
  if (!g) return fail(GBX_EINVAL, "null group");
  const GroupPlan& P = g->plan;
  for (size_t i = 0; i < P.tri.size(); ++i) {
    const Choice& c = P.choice[i];
    if (engines) engines[i] = c.engine;
    if (params) params[i] = c.engine ? (c.width * 2 + (c.swap ? 1 : 0)) : c.variant;
  }
  if (flops) *flops = P.flops;
  return GBX_OK;
}

int gbx_group_destroy(gbx_group* g) {
  delete g;
  return GBX_OK;
}

}  // extern "C"
