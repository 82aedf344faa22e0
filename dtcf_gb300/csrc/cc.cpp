// Coupled-cluster iteration driver (see cc.h): builds the synthetic system on
// the device, plans every contraction of one CCD / CCSD iteration once, and
// replays the iteration (optionally as one CUDA graph).
#include "cc.h"
#include "program.h"
#include "split.h"

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <set>

namespace gbx {

uint64_t cc_mix64(uint64_t z) {
  z ^= z >> 30;
  z *= 0xBF58476D1CE4E5B9ull;
  z ^= z >> 27;
  z *= 0x94D049BB133111EBull;
  z ^= z >> 31;
  return z;
}

CCStream::CCStream(uint64_t seed, int k) : state(cc_mix64(seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(k + 1)))) {}

uint64_t CCStream::next() {
  state += 0x9E3779B97F4A7C15ull;
  return cc_mix64(state);
}

double CCStream::uniform() { return (double)(next() >> 11) * 0x1.0p-53; }

namespace {

// irrep occupation counts of one space
std::vector<int> draw_counts(int n, int nirrep, int min_block, uint64_t seed, int stream) {
  CCStream rng(seed, stream);
  int need = std::min(min_block, nirrep > 0 ? n / nirrep : 0);
  for (;;) {
    std::vector<int> c(nirrep, 0);
    for (int i = 0; i < n; ++i) {
      int h = (int)(rng.uniform() * nirrep);
      if (h >= nirrep) h = nirrep - 1;
      ++c[h];
    }
    if (nirrep == 1 || *std::min_element(c.begin(), c.end()) >= need) return c;
  }
}

void blocks_of(const std::vector<int>& counts, int max_block, std::vector<int>& ext, std::vector<int>& irr) {
  for (size_t h = 0; h < counts.size(); ++h) {
    int c = counts[h];
    if (c == 0) continue;
    int nb = (c + max_block - 1) / max_block;
    for (int k = 0; k < nb; ++k) {
      ext.push_back(c / nb + (k < c % nb ? 1 : 0));
      irr.push_back((int)h);
    }
  }
}

}  // namespace

struct CCTensor {
  std::string spaces;
  TensorLayout L;
  double* d = nullptr;
  ~CCTensor() { dev_free(d); }
};

}  // namespace gbx

using namespace gbx;

struct gbx_cc_job {
  gbx_cc_config cfg;
  int o = 0, v = 0, n = 0;
  std::shared_ptr<BlockDim> occ, vir;
  std::vector<int> irrep;
  std::vector<double> eps;
  int* d_irrep = nullptr;
  double* d_eps = nullptr;
  double* d_mag = nullptr;
  CCDeviceTables tab;
  std::map<std::string, std::unique_ptr<CCTensor>> T;
  std::vector<std::unique_ptr<ContractionPlan>> cplans;
  std::vector<std::unique_ptr<FusedSumPlan>> fplans;
  std::vector<std::unique_ptr<MoveSet>> expansions;  // canonical tiles -> the others (fused with groups)
  // tau / taut / Q from t2 and t1 (CCSD): per-tile t1 offsets and work items
  std::vector<CCAmpTile> amp_tiles;
  std::vector<CCAmpItem> amp_items;
  CCAmpSet amp;
  std::vector<std::function<int(cudaStream_t)>> steps;       // one iteration
  std::vector<std::function<int(cudaStream_t)>> init_steps;  // once, after the MP2 guess
  std::set<std::string> dynamic_use;  // tensors read or written outside constant plan operands
  std::vector<std::pair<CCTensor*, CCTensor*>> plan_operands;  // A, B of each contraction plan
  std::vector<CCTensor*> plan_outputs;                         // C of each contraction plan
  std::vector<std::array<std::string, 3>> plan_labels;          // la, lb, lc of each contraction plan
  unsigned char* d_arena = nullptr;  // packed operands and split slices, shared by every plan
  size_t arena_bytes = 0;
  std::atomic<int64_t> account{0};  // device bytes the job's allocations hold
  struct StepInfo {
    std::string name;
    int kind;  // 0 contraction, 1 sum, 2 zero, 3 denominator, 4 energy
    double flops, bytes;
    int plan = -1;  // index into cplans for contractions
  };
  std::vector<StepInfo> info;
  std::vector<std::unique_ptr<CCTileSet>> tilesets;
  CCTileSet *den1 = nullptr, *den2 = nullptr;
  double* d_partial = nullptr;
  double* d_hist = nullptr;
  int* d_count = nullptr;
  int hist_cap = 4096;
  int nenergies = 0;  // host view of the history length
  int npartial = 608;
  double flops = 0.0, gemm_flops = 0.0;
  int launches = 0;
  int iter_plan_begin = 0;  // plans before this index serve only the initial guess
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // use_graph 2: the iteration as a persistent program (a few persistent
  // launches off a device-side work queue), itself captured as the graph
  ProgramPtr prog;

  bool persistent() const { return cfg.use_graph == 2; }
  int record_program();

  ~gbx_cc_job() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    prog.reset();
    cplans.clear();
    fplans.clear();
    expansions.clear();
    amp.release();
    T.clear();
    tilesets.clear();
    dev_free(d_arena);
    dev_free(d_irrep);
    dev_free(d_eps);
    dev_free(d_mag);
    dev_free(d_partial);
    dev_free(d_hist);
    dev_free(d_count);
  }

  std::shared_ptr<BlockDim> dim_of(char s) { return s == 'o' ? occ : vir; }
  int gstart(char s, int b) { return s == 'o' ? (int)occ->start[b] : o + (int)vir->start[b]; }

  // Declares a tensor (layout only; device memory comes with materialize()).
  // groups: antisymmetric index groups (-1 = none) of a tensor that stores
  // only its canonical tiles, as RRR stores unique blocks (tensor.cc:617-640);
  // readers recover the other tiles by permutation and sign.
  int tensor(const std::string& name, const std::string& spaces, const std::vector<int>& groups = {}) {
    auto t = std::make_unique<CCTensor>();
    t->spaces = spaces;
    std::vector<std::shared_ptr<BlockDim>> dims;
    for (char c : spaces) dims.push_back(dim_of(c));
    t->L = TensorLayout::full(dims, groups, groups.empty() ? 1 : -1, !groups.empty());
    T[name] = std::move(t);
    return GBX_OK;
  }

  CCTensor* get(const std::string& name) { return T.at(name).get(); }

  static std::vector<std::string> labels(const char* s) {
    std::vector<std::string> out;
    for (const char* p = s; *p; ++p) out.push_back(std::string(1, *p));
    return out;
  }

  int check_labels(const CCTensor* t, const char* lab, const char* name) {
    if (std::strlen(lab) != t->spaces.size()) return fail(GBX_EINVAL, "%s: label %s vs spaces %s", name, lab, t->spaces.c_str());
    for (size_t i = 0; i < t->spaces.size(); ++i) {
      char want = std::strchr("ijklmn", lab[i]) ? 'o' : 'v';
      if (want != t->spaces[i]) return fail(GBX_EINVAL, "%s: label %s does not fit spaces %s", name, lab, t->spaces.c_str());
    }
    return GBX_OK;
  }

  // C[lc] += alpha * A[la] * B[lb]
  static bool is_integral(const char* name) {
    size_t n = std::strlen(name);
    if (n != 2 && n != 4) return false;
    for (size_t i = 0; i < n; ++i)
      if (name[i] != 'O' && name[i] != 'V') return false;
    return true;
  }

  // pair: two contracted labels in which A and B are both antisymmetric
  // (the packed GEMMs then run over block pairs x >= y, the off-diagonal ones
  // weighted 2 in the pack of the constant operand, or of the smaller one).
  // from_zero: C starts from zero -- the contraction stores alpha A B when it
  // writes every element of C, else C is zero-filled first.
  int contract(const char* c, const char* lc, const char* a, const char* la, const char* b, const char* lb,
               double alpha, const char* pair = nullptr, bool from_zero = false) {
    CCTensor *C = get(c), *A = get(a), *B = get(b);
    GBX_TRY(check_labels(C, lc, c));
    GBX_TRY(check_labels(A, la, a));
    GBX_TRY(check_labels(B, lb, b));
    std::unique_ptr<ContractionPlan> p;
    Engine e = cfg.engine == GBX_MODE_SPLIT ? Engine::Split : Engine::F64;
    ContractionPair cp;
    if (pair) {
      cp.x = std::string(1, pair[0]);
      cp.y = std::string(1, pair[1]);
      const bool a_int = is_integral(a), b_int = is_integral(b);
      cp.scale_b = b_int != a_int ? b_int : B->L.nelem <= A->L.nelem;
    }
    GBX_TRY(plan_contraction(A->L, B->L, C->L, labels(la), labels(lb), labels(lc), e, cfg.slices, p,
                             cfg.split_all != 0, /*defer=*/true, pair ? &cp : nullptr));
    // integrals never change: packed and split once, when the job is built
    // (a direct plan reads them where they are stored, so they stay resident)
    p->a_static = is_integral(a) && !p->direct;
    p->b_static = is_integral(b) && !p->direct;
    if (!p->a_static) dynamic_use.insert(a);
    if (!p->b_static) dynamic_use.insert(b);
    dynamic_use.insert(c);
    const bool stores = from_zero && p->set_overwrite(alpha, C->L.nelem);
    if (from_zero && !stores) GBX_TRY(zero(c));
    flops += p->flops;
    gemm_flops += p->gemm_flops;
    ContractionPlan* pp = p.get();
    steps.push_back([=](cudaStream_t st) { return pp->execute(A->d, B->d, C->d, alpha, st); });
    info.push_back({std::string(c) + "[" + lc + "]" + (stores ? "=" : "+=") + a + "[" + la + "]*" + b + "[" + lb + "]", 0,
                    pp->flops, 8.0 * (double)(A->L.nelem + B->L.nelem + (stores ? 1 : 2) * C->L.nelem),
                    (int)cplans.size()});
    launches += pp->direct ? 1 : 4;
    cplans.push_back(std::move(p));
    plan_operands.push_back({A, B});
    plan_outputs.push_back(C);
    plan_labels.push_back({la, lb, lc});
    return GBX_OK;
  }

  // out[lc] = (sum of coef * A[la] over the terms, in order) [* scale]: one
  // pass that replaces zeroing out and running the terms as separate sums
  struct Term {
    const char* a;
    const char* la;
    double coef;
  };
  // groups (optional): antisymmetric index groups of the result.  The terms
  // are then formed on the canonical tiles only (block coordinates
  // non-increasing within each group: about a quarter of an o^2 v^2 tensor
  // with two groups) and every other tile is filled from its canonical
  // partner by a permuted copy with the sign of the permutation -- the
  // result is stored whole and is exactly antisymmetric.
  int fused(const char* out, const char* lc, const std::vector<Term>& terms, const char* scale = nullptr,
            const std::vector<int>& groups = {}) {
    CCTensor* C = get(out);
    GBX_TRY(check_labels(C, lc, out));
    TensorLayout view;
    std::unique_ptr<MoveSet> expand;
    if (!groups.empty()) GBX_TRY(canonical_view(C->L, groups, view, expand));
    std::vector<FusedTermSpec> specs;
    std::vector<CCTensor*> src;
    std::string name = std::string(out) + "[" + lc + "]=";
    double bytes = 8.0 * (double)C->L.nelem;
    for (const Term& t : terms) {
      CCTensor* A = get(t.a);
      GBX_TRY(check_labels(A, t.la, t.a));
      int slot = -1;
      for (size_t i = 0; i < src.size(); ++i)
        if (src[i] == A) slot = (int)i;
      if (slot < 0) {
        slot = (int)src.size();
        src.push_back(A);
        bytes += 8.0 * (double)A->L.nelem;
      }
      if (slot >= kFsMaxSlots) return fail(GBX_EUNSUPPORTED, "fused sum: too many sources");
      specs.push_back({&A->L, labels(t.la), t.coef, slot});
      dynamic_use.insert(t.a);
      char buf[64];
      std::snprintf(buf, sizeof buf, "%s%s%s[%s]", &t == &terms[0] ? "" : (t.coef < 0 ? "-" : "+"),
                    (t.coef == 1.0 || t.coef == -1.0) ? "" : (std::to_string(std::fabs(t.coef)).substr(0, 4) + "*").c_str(),
                    t.a, t.la);
      name += buf;
    }
    CCTensor* S = scale ? get(scale) : nullptr;
    if (S) {
      if (S->L.nelem != C->L.nelem) return fail(GBX_EINVAL, "fused sum: scale layout differs");
      name += std::string(" *") + scale;
      bytes += 8.0 * (double)S->L.nelem;
      dynamic_use.insert(scale);
    }
    dynamic_use.insert(out);
    std::unique_ptr<FusedSumPlan> p;
    GBX_TRY(plan_fused_sum(groups.empty() ? C->L : view, labels(lc), specs, p));
    FusedSumPlan* pp = p.get();
    MoveSet* ex = expand.get();
    if (expand) {
      name += " (canonical tiles, expanded)";
      expansions.push_back(std::move(expand));
    }
    steps.push_back([=](cudaStream_t st) {
      const double* ptr[kFsMaxSlots] = {};
      for (size_t i = 0; i < src.size(); ++i) ptr[i] = src[i]->d;
      GBX_TRY(pp->execute(ptr, S ? S->d : nullptr, C->d, st));
      return ex ? run_moves(*ex, C->d, C->d, st) : GBX_OK;
    });
    info.push_back({name, 1, 0.0, bytes});
    launches += 1;
    fplans.push_back(std::move(p));
    return GBX_OK;
  }

  // The canonical tiles of L for the antisymmetric groups (a layout view
  // that keeps L's offsets) and the moves that fill L's other tiles from
  // them: tile t gets sign * (its canonical partner, permuted).
  static int canonical_view(const TensorLayout& L, const std::vector<int>& groups, TensorLayout& view,
                            std::unique_ptr<MoveSet>& expand) {
    const TensorLayout G = TensorLayout::full(L.dims, groups, -1, true);
    view = TensorLayout();
    view.rank = L.rank;
    view.dims = L.dims;
    view.nelem = L.nelem;
    expand = std::make_unique<MoveSet>();
    for (size_t t = 0; t < L.tiles.size(); ++t) {
      const Coords& c = L.tiles[t];
      if (G.find(c.data()) >= 0) {
        view.index[coord_key(c.data(), L.rank)] = (int)view.tiles.size();
        view.tiles.push_back(c);
        view.off.push_back(L.off[t]);
        continue;
      }
      int src_dim[kMaxDims];
      double f;
      const int id = G.resolve(c.data(), src_dim, &f);
      if (id < 0) continue;  // a zero tile of the group structure
      const int ct = L.find(G.tiles[id].data());
      if (ct < 0) return fail(GBX_EINVAL, "canonical partner of a tile is not stored");
      const Coords& sc = L.tiles[ct];
      int64_t sst[kMaxDims], ext[kMaxDims], sstr[kMaxDims], dstr[kMaxDims];
      sst[L.rank - 1] = 1;
      dstr[L.rank - 1] = 1;
      for (int d = L.rank - 2; d >= 0; --d) {
        sst[d] = sst[d + 1] * L.dims[d + 1]->ext[sc[d + 1]];
        dstr[d] = dstr[d + 1] * L.dims[d + 1]->ext[c[d + 1]];
      }
      for (int d = 0; d < L.rank; ++d) {
        ext[d] = L.dims[d]->ext[c[d]];
        sstr[d] = sst[src_dim[d]];
      }
      expand->host.push_back(make_move(L.rank, ext, sstr, dstr, L.off[ct], L.off[t], 0, f));
    }
    GBX_TRY(check_moves(*expand, L.nelem, L.nelem, "canonical expansion"));
    if (expand->host.empty()) expand.reset();
    return GBX_OK;
  }

  // tau, taut and Q from t2 and t1 (CCSD), one pass over t2's tiles
  int amp_step() {
    CCTensor *t2 = get("t2"), *t1 = get("t1"), *tau = get("tau"), *taut = get("taut"), *Q = get("Q");
    for (CCTensor* x : {tau, taut, Q})
      if (x->L.tiles != t2->L.tiles) return fail(GBX_EINVAL, "tau family: layout differs from t2");
    if (amp_tiles.empty()) {
      const TensorLayout& L = t2->L;
      for (size_t t = 0; t < L.tiles.size(); ++t) {
        const Coords& c = L.tiles[t];
        CCAmpTile at;
        std::memset(&at, 0, sizeof(at));
        at.off = L.off[t];
        const int pairs[4][2] = {{c[0], c[2]}, {c[1], c[3]}, {c[0], c[3]}, {c[1], c[2]}};
        for (int k = 0; k < 4; ++k) {
          const int cc2[2] = {pairs[k][0], pairs[k][1]};
          const int id = t1->L.find(cc2);
          at.t1[k] = id < 0 ? -1 : t1->L.off[id];
        }
        const int64_t ei = L.dims[0]->ext[c[0]], ej = L.dims[1]->ext[c[1]], ea = L.dims[2]->ext[c[2]],
                      eb = L.dims[3]->ext[c[3]];
        at.fj = FastDiv::make((uint32_t)ej);
        at.fa = FastDiv::make((uint32_t)ea);
        at.fb = FastDiv::make((uint32_t)eb);
        const int64_t n = ei * ej * ea * eb;
        if (n >= ((int64_t)1 << 31)) return fail(GBX_EUNSUPPORTED, "amplitude tile too large");
        for (int64_t f0 = 0; f0 < n; f0 += 2048)
          amp_items.push_back({(uint32_t)t, (uint32_t)f0, (uint32_t)std::min<int64_t>(2048, n - f0), 0u});
        amp_tiles.push_back(at);
      }
    }
    for (const char* nm : {"t2", "t1", "tau", "taut", "Q"}) dynamic_use.insert(nm);
    steps.push_back([=](cudaStream_t st) { return run_cc_amp(amp, t1->d, t2->d, tau->d, taut->d, Q->d, st); });
    info.push_back({"tau,taut,Q[ijab]=t2+t1*t1", 1, 0.0, 32.0 * (double)t2->L.nelem});
    launches += 1;
    return GBX_OK;
  }

  int zero(const char* c) {
    CCTensor* C = get(c);
    size_t bytes = sizeof(double) * C->L.nelem;
    dynamic_use.insert(c);
    steps.push_back([=](cudaStream_t st) { return zero_async(C->d, bytes, st); });
    info.push_back({std::string("zero ") + c, 2, 0.0, (double)bytes});
    launches += 1;
    return GBX_OK;
  }

  CCTileSet* tileset(const CCTensor* t) {
    std::vector<CCTile> h;
    for (size_t i = 0; i < t->L.tiles.size(); ++i) {
      CCTile ct;
      std::memset(&ct, 0, sizeof(ct));
      ct.off = t->L.off[i];
      ct.rank = t->L.rank;
      int64_t nn = 1;
      for (int d = 0; d < t->L.rank; ++d) {
        int b = t->L.tiles[i][d];
        ct.ext[d] = (uint32_t)t->L.dims[d]->ext[b];
        ct.gstart[d] = gstart(t->spaces[d], b);
        nn *= ct.ext[d];
      }
      ct.n = (uint32_t)nn;
      h.push_back(ct);
    }
    auto ts = std::make_unique<CCTileSet>();
    if (ts->upload(h) != GBX_OK) return nullptr;
    tilesets.push_back(std::move(ts));
    return tilesets.back().get();
  }

  // out = in * (1/D), the inverse orbital-energy denominators computed once
  // when the job is built (out, in and the inverse share one tile layout)
  int denom(const char* out, const char* in, const char* dinv) {
    CCTensor *O = get(out), *I = get(in), *Dv = get(dinv);
    dynamic_use.insert(out);
    dynamic_use.insert(in);
    const int64_t n = O->L.nelem;
    steps.push_back([=](cudaStream_t st) { return run_mul(I->d, Dv->d, O->d, n, st); });
    info.push_back({std::string(out) + "=" + in + "/D", 3, 0.0, 24.0 * (double)O->L.nelem});
    launches += 1;
    return GBX_OK;
  }

  int energy_step() {
    CCTensor *V = get("OOVV"), *tau = get(cfg.method == GBX_CC_CCSD ? "tau" : "t2");
    dynamic_use.insert("OOVV");
    int64_t n = V->L.nelem;
    steps.push_back([=](cudaStream_t st) {
      return gbx::run_energy(V->d, tau->d, n, d_partial, npartial, d_hist, d_count, hist_cap, st);
    });
    info.push_back({"energy", 4, 2.0 * (double)n, 16.0 * (double)n});
    launches += 2;
    return GBX_OK;
  }

  int plan_all();
  int materialize(cudaStream_t st);
  int footprint(double* resident, double* peak) const;
  int tau_steps();
};

// tau = t2 + t1 t1 - t1 t1 (i<->j), taut = t2 + (t1 t1 - t1 t1) / 2 and
// Q = t2 / 2 + t1 t1, all from the current t1 and t2 (CCSD)
int gbx_cc_job::tau_steps() { return amp_step(); }

int gbx_cc_job::plan_all() {
  const bool sd = cfg.method == GBX_CC_CCSD;
  // amplitudes, residuals, intermediates
  GBX_TRY(tensor("t2", "oovv"));
  GBX_TRY(tensor("Dinv2", "oovv"));  // 1 / (e_i + e_j - e_a - e_b)
  GBX_TRY(tensor("Xa", "oovv"));
  // every term of X_b (t2 F', Z' t1, t1 <mb||ij>) is antisymmetric in ij,
  // every term of X_j (t2 F', t1 <ab||ej>) in ab: both are formed on
  // canonical tiles only (half the work), read back with sign factors
  GBX_TRY(tensor("Xb", "oovv", {0, 0, -1, -1}));
  GBX_TRY(tensor("Xj", "oovv", {-1, -1, 0, 0}));
  GBX_TRY(tensor("Fae", "vv"));
  GBX_TRY(tensor("Fmi", "oo"));
  // W_mnij is antisymmetric in mn and in ij: canonical tiles only
  GBX_TRY(tensor("Wmnij", "oooo", {0, 0, 1, 1}));
  // both ladder-type terms of R2 (tau W_mnij and tau <ab||ef>) are
  // antisymmetric in ij and in ab: they are formed on canonical tiles (a
  // quarter of the work) and expanded into R2 once
  GBX_TRY(tensor("Lad", "oovv", {0, 0, 1, 1}));
  GBX_TRY(tensor("Wmbej", "ovvo"));
  GBX_TRY(tensor("Q", "oovv"));
  for (const char* nm : {"OOOO", "OOVV", "OVVO", "VVVV"}) {
    std::string sp;
    for (const char* c = nm; *c; ++c) sp += (char)(*c == 'O' ? 'o' : 'v');
    GBX_TRY(tensor(nm, sp));
  }
  if (sd) {
    GBX_TRY(tensor("t1", "ov"));
    GBX_TRY(tensor("Dinv1", "ov"));
    GBX_TRY(tensor("R1", "ov"));
    GBX_TRY(tensor("tau", "oovv"));
    GBX_TRY(tensor("taut", "oovv"));
    GBX_TRY(tensor("Fme", "ov"));
    GBX_TRY(tensor("Fbe", "vv"));
    GBX_TRY(tensor("Fmj", "oo"));
    GBX_TRY(tensor("Xoooo", "oooo"));
    GBX_TRY(tensor("Zp", "ooov", {0, 0, -1, -1}));  // antisymmetric in ij
    GBX_TRY(tensor("V3", "oovo"));
    for (const char* nm : {"OOOV", "OVVV", "OOVO", "OVOV", "VVVO", "OVOO"}) {
      std::string sp;
      for (const char* c = nm; *c; ++c) sp += (char)(*c == 'O' ? 'o' : 'v');
      GBX_TRY(tensor(nm, sp));
    }
  }
  const char* TAU = sd ? "tau" : "t2";
  const char* TAUT = sd ? "taut" : "t2";
  if (sd) {
    // initial tau / taut from the guess, run once when the job is built
    size_t first = steps.size();
    GBX_TRY(tau_steps());
    init_steps.assign(steps.begin() + first, steps.end());
    steps.resize(first);
    info.resize(first);
  }
  launches = 0;
  flops = 0.0;
  gemm_flops = 0.0;
  iter_plan_begin = (int)cplans.size();

  // ---- one iteration --------------------------------------------------------
  // (tau, taut and Q of the current amplitudes exist: formed at the end of
  // the previous iteration, by the initial guess or by set_amplitudes)
  // F_ae, F_mi, F_me
  // (the first contraction into each intermediate starts it from zero)
  if (sd) GBX_TRY(contract("Fae", "ae", "t1", "mf", "OVVV", "mafe", 1.0, nullptr, true));
  // (taut, tau and t2 are antisymmetric in i <-> j and in a <-> b, like <pq||rs>)
  GBX_TRY(contract("Fae", "ae", TAUT, "mnaf", "OOVV", "mnef", -0.5, "mn", !sd));
  if (sd) GBX_TRY(contract("Fmi", "mi", "t1", "ne", "OOOV", "mnie", 1.0, nullptr, true));
  GBX_TRY(contract("Fmi", "mi", TAUT, "inef", "OOVV", "mnef", 0.5, "ef", !sd));
  if (sd) GBX_TRY(contract("Fme", "me", "t1", "nf", "OOVV", "mnef", 1.0, nullptr, true));
  // W_mnij (with the ladder's 1/8 tau <mn||ef> tau term folded in: 1/2 instead of 1/4)
  if (sd) {
    GBX_TRY(contract("Xoooo", "mnij", "t1", "je", "OOOV", "mnie", 1.0, nullptr, true));
    GBX_TRY(fused("Wmnij", "mnij", {{"OOOO", "mnij", 1.0}, {"Xoooo", "mnij", 1.0}, {"Xoooo", "mnji", -1.0}}));
  } else {
    GBX_TRY(fused("Wmnij", "mnij", {{"OOOO", "mnij", 1.0}}));
  }
  GBX_TRY(contract("Wmnij", "mnij", TAU, "ijef", "OOVV", "mnef", 0.5, "ef"));
  // W_mbej
  GBX_TRY(fused("Wmbej", "mbej", {{"OVVO", "mbej", 1.0}}));
  if (sd) {
    GBX_TRY(contract("Wmbej", "mbej", "t1", "jf", "OVVV", "mbef", 1.0));
    GBX_TRY(contract("Wmbej", "mbej", "t1", "nb", "OOVO", "mnej", -1.0));
  }
  // Q = t2 / 2 (+ t1 t1, formed with tau at the end of the previous iteration for CCSD)
  if (!sd) GBX_TRY(fused("Q", "jnfb", {{"t2", "jnfb", 0.5}}));
  GBX_TRY(contract("Wmbej", "mbej", "Q", "jnfb", "OOVV", "mnef", -1.0));
  // T1 residual
  if (sd) {
    GBX_TRY(contract("R1", "ia", "t1", "ie", "Fae", "ae", 1.0, nullptr, true));
    GBX_TRY(contract("R1", "ia", "t1", "ma", "Fmi", "mi", -1.0));
    GBX_TRY(contract("R1", "ia", "t2", "imae", "Fme", "me", 1.0));
    GBX_TRY(contract("R1", "ia", "t1", "nf", "OVOV", "naif", -1.0));
    GBX_TRY(contract("R1", "ia", "t2", "imef", "OVVV", "maef", -0.5, "ef"));
    GBX_TRY(contract("R1", "ia", "t2", "mnae", "OOVO", "nmei", -0.5, "mn"));
  }
  // T2 residual
  const char* FBE = "Fae";
  const char* FMJ = "Fmi";
  if (sd) {
    GBX_TRY(fused("Fbe", "be", {{"Fae", "be", 1.0}}));
    GBX_TRY(contract("Fbe", "be", "t1", "mb", "Fme", "me", -0.5));
    GBX_TRY(fused("Fmj", "mj", {{"Fmi", "mj", 1.0}}));
    GBX_TRY(contract("Fmj", "mj", "t1", "je", "Fme", "me", 0.5));
    FBE = "Fbe";
    FMJ = "Fmj";
  }
  // Terms under the same antisymmetriser share one intermediate, expanded
  // into R2 once: Xb under P(ab), Xj under P(ij), Xa under P(ij)P(ab).
  // P(ab) t_ij^ae F'_be
  GBX_TRY(contract("Xb", "ijab", "t2", "ijae", FBE, "be", 1.0, nullptr, true));
  // -P(ij) t_im^ab F'_mj
  GBX_TRY(contract("Xj", "ijab", "t2", "imab", FMJ, "mj", -1.0, nullptr, true));
  // 1/2 tau_mn^ab W_mnij + 1/2 tau_ij^ef <ab||ef> (the ladder, integrals as
  // the static A operand), on canonical tiles, then into R2
  GBX_TRY(contract("Lad", "ijab", TAU, "mnab", "Wmnij", "mnij", 0.5, "mn", true));
  GBX_TRY(contract("Lad", "ijab", "VVVV", "abef", TAU, "ijef", 0.5, "ef"));
  if (sd) {
    // -1/2 P(ab) t_m^b sum_ef tau_ij^ef <am||ef> = +1/2 P(ab) sum_m t_m^b Z'_ijma
    GBX_TRY(contract("Zp", "ijma", TAU, "ijef", "OVVV", "maef", 1.0, "ef", true));
    GBX_TRY(contract("Xb", "ijab", "Zp", "ijma", "t1", "mb", 0.5));
  }
  // P(ij)P(ab) (t_im^ae W_mbej - t_i^e t_m^a <mb||ej>)
  GBX_TRY(contract("Xa", "ijab", "t2", "imae", "Wmbej", "mbej", 1.0, nullptr, true));
  if (sd) {
    GBX_TRY(contract("V3", "imbj", "t1", "ie", "OVVO", "mbej", 1.0, nullptr, true));
    GBX_TRY(contract("Xa", "ijab", "t1", "ma", "V3", "imbj", -1.0));
    // P(ij) t_i^e <ab||ej>
    GBX_TRY(contract("Xj", "ijab", "t1", "ie", "VVVO", "abej", 1.0));
    // -P(ab) t_m^a <mb||ij>
    GBX_TRY(contract("Xb", "ijab", "t1", "ma", "OVOO", "mbij", -1.0));
  }
  // Jacobi update of T2: the residual R2 = <ij||ab> + ladder + the three
  // antisymmetrised intermediates, times 1 / D, in one pass (R2 itself is
  // never stored); then T1, the tau family and the energy
  GBX_TRY(fused("t2", "ijab",
                {{"OOVV", "ijab", 1.0}, {"Lad", "ijab", 1.0}, {"Xb", "ijab", 1.0}, {"Xb", "ijba", -1.0},
                 {"Xj", "ijab", 1.0}, {"Xj", "jiab", -1.0}, {"Xa", "ijab", 1.0}, {"Xa", "jiab", -1.0},
                 {"Xa", "ijba", -1.0}, {"Xa", "jiba", 1.0}},
                "Dinv2", {0, 0, 1, 1}));
  if (sd) {
    GBX_TRY(denom("t1", "R1", "Dinv1"));
    GBX_TRY(tau_steps());
  }
  GBX_TRY(energy_step());
  return GBX_OK;
}

namespace {
double up256d(double x) { return std::ceil(x / 256.0) * 256.0; }
}  // namespace

// An integral tensor read only as constant plan operands: released once those
// operands are packed and split.
bool gbx_cc_job_static_only(const gbx_cc_job& j, const std::string& name) {
  return gbx_cc_job::is_integral(name.c_str()) && !j.dynamic_use.count(name);
}

// Device bytes of the built job: what stays resident, and the peak while it
// is being built (integral tiles and constant-operand scratch included).
int gbx_cc_job::footprint(double* resident, double* peak) const {
  double keep = 0.0, transient = 0.0, ws = 0.0, scratch = 0.0;
  for (auto& kv : T) {
    const double b = up256d(8.0 * (double)std::max<int64_t>(1, kv.second->L.nelem));
    if (gbx_cc_job_static_only(*this, kv.first)) transient += b; else keep += b;
  }
  for (auto& p : cplans) {
    size_t k = 0, w = 0, sc = 0;
    GBX_TRY(p->sizes(&k, &w, &sc));
    keep += (double)k + p->f64_workspace_estimate();
    // a persistent program runs contractions side by side: each plan keeps
    // its own region of the arena
    ws = persistent() ? ws + up256d((double)w) : std::max(ws, (double)w);
    scratch = std::max(scratch, (double)sc);
  }
  for (auto& p : fplans) keep += up256d((double)(p->items.size() * sizeof(FsItem))) + up256d((double)(p->terms.size() * sizeof(FsTerm)));
  for (auto& m : expansions) keep += up256d((double)m->device_bytes());
  keep += up256d((double)(amp_tiles.size() * sizeof(CCAmpTile))) + up256d((double)(amp_items.size() * sizeof(CCAmpItem)));
  auto tiles_bytes = [](const TensorLayout& L) {
    return up256d((double)L.tiles.size() * sizeof(CCTile)) + up256d(4.0 * (double)(L.tiles.size() + 1));
  };
  transient += tiles_bytes(T.at("t2")->L);
  if (T.count("t1")) transient += tiles_bytes(T.at("t1")->L);
  for (auto& kv : T)
    if (is_integral(kv.first.c_str())) transient += tiles_bytes(kv.second->L);
  keep += up256d(4.0 * n) + up256d(8.0 * n) + up256d(8.0 * (2 * n + 1)) + up256d(8.0 * npartial) +
          up256d(8.0 * hist_cap) + 256.0;
  keep += ws;
  if (resident) *resident = keep;
  if (peak) *peak = keep + transient + scratch;
  return GBX_OK;
}

// Allocates and fills the job: orbital tables, tensors, integrals, the plan
// arena, constant operands (packed and split once), the MP2 guess and the
// initial energy.  Runs on the legacy default stream `st` and waits for it.
int gbx_cc_job::materialize(cudaStream_t st) {
  const bool sd = cfg.method == GBX_CC_CCSD;
  std::vector<double> mag(2 * n + 1);
  for (size_t d = 0; d < mag.size(); ++d) mag[d] = cfg.v_scale * std::exp(-(double)d / cfg.v_decay);
  GBX_TRY(dev_alloc((void**)&d_irrep, sizeof(int) * n));
  GBX_TRY(dev_alloc((void**)&d_eps, sizeof(double) * n));
  GBX_TRY(dev_alloc((void**)&d_mag, sizeof(double) * mag.size()));
  GBX_CUDA(cudaMemcpy(d_irrep, irrep.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
  GBX_CUDA(cudaMemcpy(d_eps, eps.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
  GBX_CUDA(cudaMemcpy(d_mag, mag.data(), sizeof(double) * mag.size(), cudaMemcpyHostToDevice));
  tab.irrep = d_irrep;
  tab.eps = d_eps;
  tab.mag = d_mag;
  tab.norb = n;
  tab.nocc = o;
  GBX_TRY(dev_alloc((void**)&d_partial, sizeof(double) * npartial));
  GBX_TRY(dev_alloc((void**)&d_hist, sizeof(double) * hist_cap));
  GBX_TRY(dev_alloc((void**)&d_count, sizeof(int)));
  GBX_CUDA(cudaMemsetAsync(d_count, 0, sizeof(int), st));
  for (auto& kv : T) {
    CCTensor* t = kv.second.get();
    const size_t bytes = sizeof(double) * std::max<int64_t>(1, t->L.nelem);
    GBX_TRY(dev_alloc((void**)&t->d, bytes));
    GBX_CUDA(cudaMemsetAsync(t->d, 0, bytes, st));
  }
  // integrals on the device (their tile sets are dropped afterwards)
  std::vector<std::unique_ptr<CCTileSet>> once;
  for (auto& kv : T) {
    if (!is_integral(kv.first.c_str())) continue;
    CCTileSet* ts = tileset(kv.second.get());
    if (!ts) return fail(GBX_ENOMEM, "tile set upload failed");
    once.push_back(std::move(tilesets.back()));
    tilesets.pop_back();
    GBX_TRY(run_cc_tiles(*ts, CC_OP_INTEGRAL, tab, nullptr, kv.second->d, st));
  }
  den2 = tileset(get("t2"));
  if (sd) den1 = tileset(get("t1"));
  if (!den2 || (sd && !den1)) return fail(GBX_ENOMEM, "tile set upload failed");
  // one arena for every plan's per-run buffers (the steps run in order on one
  // stream); constant operands are packed into scratch, split, and the
  // scratch is released
  arena_bytes = 0;
  size_t scratch_bytes = 0;
  std::vector<size_t> arena_off(cplans.size(), 0);
  for (size_t i = 0; i < cplans.size(); ++i) {
    size_t k = 0, w = 0, sc = 0;
    GBX_TRY(cplans[i]->sizes(&k, &w, &sc));
    if (persistent()) {  // a region per plan (they run side by side)
      arena_off[i] = arena_bytes;
      arena_bytes += (w + 255) / 256 * 256;
    } else {
      arena_bytes = std::max(arena_bytes, w);
    }
    scratch_bytes = std::max(scratch_bytes, sc);
  }
  if (arena_bytes) {
    GBX_TRY(dev_alloc((void**)&d_arena, arena_bytes));
    GBX_CUDA(cudaMemsetAsync(d_arena, 0, arena_bytes, st));
  }
  unsigned char* d_scratch = nullptr;
  if (scratch_bytes) GBX_TRY(dev_alloc((void**)&d_scratch, scratch_bytes));
  for (auto& p : fplans) GBX_TRY(p->upload());
  for (auto& m : expansions) GBX_TRY(m->upload());
  if (!amp_items.empty()) GBX_TRY(amp.upload(amp_tiles, amp_items));
  for (size_t i = 0; i < cplans.size(); ++i) {
    ContractionPlan* p = cplans[i].get();
    int rc = p->build(d_arena ? d_arena + arena_off[i] : nullptr, d_scratch);
    if (rc == GBX_OK && (p->a_static || p->b_static))
      rc = p->prepare_static(plan_operands[i].first->d, plan_operands[i].second->d, st);
    if (rc == GBX_OK && cfg.autotune) rc = p->tune_split(st);
    if (rc != GBX_OK) {
      cudaStreamSynchronize(st);
      dev_free(d_scratch);
      return rc;
    }
  }
  // MP2 guess t2 = <ij||ab> / D, t1 = 0; tau / taut; energy
  GBX_TRY(run_cc_tiles(*den2, CC_OP_INVDENOM, tab, nullptr, get("Dinv2")->d, st));
  if (sd) GBX_TRY(run_cc_tiles(*den1, CC_OP_INVDENOM, tab, nullptr, get("Dinv1")->d, st));
  GBX_TRY(run_mul(get("OOVV")->d, get("Dinv2")->d, get("t2")->d, get("t2")->L.nelem, st));
  for (auto& f : init_steps) GBX_TRY(f(st));
  GBX_TRY(gbx::run_energy(get("OOVV")->d, get(sd ? "tau" : "t2")->d, get("OOVV")->L.nelem, d_partial, npartial,
                          d_hist, d_count, hist_cap, st));
  GBX_CUDA(cudaStreamSynchronize(st));
  dev_free(d_scratch);
  once.clear();
  // the tile sets only served the build
  tilesets.clear();
  den1 = den2 = nullptr;
  for (auto& kv : T)
    if (gbx_cc_job_static_only(*this, kv.first)) {
      dev_free(kv.second->d);
      kv.second->d = nullptr;
    }
  return GBX_OK;
}

extern "C" {

void gbx_cc_default_config(gbx_cc_config* c) {
  std::memset(c, 0, sizeof(*c));
  c->nocc = 8;
  c->nvir = 24;
  c->nirrep = 1;
  c->max_block = 16;
  c->min_block = 1;
  c->method = GBX_CC_CCSD;
  c->engine = GBX_MODE_FP64;
  c->slices = 0;
  c->use_graph = 1;
  c->seed = 1;
  c->eps_occ_lo = -2.0;
  c->eps_occ_hi = -0.5;
  c->eps_vir_lo = 0.2;
  c->eps_vir_hi = 3.0;
  c->v_scale = 1e-2;
  c->v_decay = 8.0;
}

// Host part of a job: orbitals, blocking and every plan (no device work).
static int cc_setup(const gbx_cc_config* cfg, std::unique_ptr<gbx_cc_job>& job) {
  if (!cfg) return fail(GBX_EINVAL, "null argument");
  if (cfg->nocc < 1 || cfg->nvir < 1 || cfg->max_block < 1 ||
      !(cfg->nirrep == 1 || cfg->nirrep == 2 || cfg->nirrep == 4 || cfg->nirrep == 8) ||
      (cfg->method != GBX_CC_CCD && cfg->method != GBX_CC_CCSD) ||
      (cfg->engine != GBX_MODE_FP64 && cfg->engine != GBX_MODE_SPLIT) || cfg->v_decay <= 0)
    return fail(GBX_EINVAL, "bad CC configuration");
  job = std::make_unique<gbx_cc_job>();
  job->cfg = *cfg;
  job->o = cfg->nocc;
  job->v = cfg->nvir;
  job->n = cfg->nocc + cfg->nvir;
  // orbitals
  std::vector<int> ext_o, irr_o, ext_v, irr_v;
  blocks_of(draw_counts(job->o, cfg->nirrep, cfg->min_block, cfg->seed, 1), cfg->max_block, ext_o, irr_o);
  blocks_of(draw_counts(job->v, cfg->nirrep, cfg->min_block, cfg->seed, 2), cfg->max_block, ext_v, irr_v);
  job->occ = BlockDim::make(ext_o, irr_o);
  job->vir = BlockDim::make(ext_v, irr_v);
  for (size_t b = 0; b < ext_o.size(); ++b)
    for (int k = 0; k < ext_o[b]; ++k) job->irrep.push_back(irr_o[b]);
  for (size_t b = 0; b < ext_v.size(); ++b)
    for (int k = 0; k < ext_v[b]; ++k) job->irrep.push_back(irr_v[b]);
  CCStream eo(cfg->seed, 3), ev(cfg->seed, 4), ei(cfg->seed, 5);
  for (int i = 0; i < job->o; ++i) job->eps.push_back(cfg->eps_occ_lo + (cfg->eps_occ_hi - cfg->eps_occ_lo) * eo.uniform());
  for (int a = 0; a < job->v; ++a) job->eps.push_back(cfg->eps_vir_lo + (cfg->eps_vir_hi - cfg->eps_vir_lo) * ev.uniform());
  job->tab.seed_int = ei.next();
  return job->plan_all();
}

int gbx_cc_footprint(const gbx_cc_config* cfg, double* resident_bytes, double* peak_bytes, double* flops_per_iter) {
  std::unique_ptr<gbx_cc_job> job;
  GBX_TRY(cc_setup(cfg, job));
  if (flops_per_iter) *flops_per_iter = job->flops;
  return job->footprint(resident_bytes, peak_bytes);
}

int gbx_cc_create(const gbx_cc_config* cfg, void* stream, gbx_cc_job** out) {
  if (!out) return fail(GBX_EINVAL, "null argument");
  *out = nullptr;
  std::unique_ptr<gbx_cc_job> job;
  GBX_TRY(cc_setup(cfg, job));
  {
    AllocAccount acct(&job->account);
    GBX_TRY(job->materialize(0));
  }
  job->nenergies = 1;
  (void)stream;
  *out = job.release();
  return GBX_OK;
}

// Records the iteration's steps into the persistent program: the job's
// tensors are the buffers whose conflicts order the records of different
// steps (every other buffer a step touches belongs to that step's plan).
int gbx_cc_job::record_program() {
  std::vector<ProgBuffer> bufs;
  for (auto& kv : T)
    if (kv.second->d) bufs.push_back({kv.second->d, sizeof(double) * (size_t)std::max<int64_t>(1, kv.second->L.nelem)});
  ProgRecorder* rec = nullptr;
  GBX_TRY(prog_begin(bufs, &rec));
  int rc = GBX_OK;
  for (size_t i = 0; i < steps.size() && rc == GBX_OK; ++i) {
    prog_step(rec, (int)i);
    rc = steps[i](prog_stream(rec));
  }
  ProgramPtr p;
  const int frc = prog_finish(rec, p);
  if (rc != GBX_OK) return rc;
  GBX_TRY(frc);
  prog = std::move(p);
  return GBX_OK;
}

int gbx_cc_capture(gbx_cc_job* job) {
  if (!job) return fail(GBX_EINVAL, "null job");
  if (!job->cfg.use_graph || job->exec) return GBX_OK;
  if (job->persistent() && !job->prog) GBX_TRY(job->record_program());
  cudaStream_t cap;
  GBX_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
  GBX_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
  int rc = GBX_OK;
  if (job->prog) {
    rc = prog_run(*job->prog, cap);
  } else {
    for (auto& s : job->steps) {
      rc = s(cap);
      if (rc != GBX_OK) break;
    }
  }
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(cap, &g);
  cudaStreamDestroy(cap);
  if (rc != GBX_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
  job->graph = g;
  GBX_CUDA(cudaGraphInstantiate(&job->exec, g, 0));
  return GBX_OK;
}

int gbx_cc_enqueue(gbx_cc_job* job, int niter, void* stream) {
  if (!job || niter < 0) return fail(GBX_EINVAL, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  if (niter > 0) GBX_TRY(gbx_cc_capture(job));
  for (int it = 0; it < niter; ++it) {
    if (job->exec) {
      GBX_CUDA(cudaGraphLaunch(job->exec, st));
    } else {
      for (auto& s : job->steps) GBX_TRY(s(st));
    }
  }
  job->nenergies += niter;
  return GBX_OK;
}

int gbx_cc_check(gbx_cc_job* job) {
  if (!job) return fail(GBX_EINVAL, "null job");
  for (auto& p : job->cplans) {
    int err = split_plan_error(p->split);
    if (err != 0) return fail(GBX_ETIMEOUT, "split GEMM: a bounded device wait ran out (stage %d)", err);
  }
  if (job->prog) {
    const int err = prog_error(*job->prog);
    if (err != 0) return fail(GBX_ETIMEOUT, "persistent iteration: a bounded device wait ran out (code %d)", err);
  }
  return GBX_OK;
}

int gbx_cc_program_info(gbx_cc_job* job, int* records, int* levels, int* launches) {
  if (!job) return fail(GBX_EINVAL, "null job");
  if (job->persistent() && !job->exec) GBX_TRY(gbx_cc_capture(job));
  ProgStats s{};
  if (job->prog) prog_stats(*job->prog, &s);
  if (records) *records = s.records;
  if (levels) *levels = s.levels;
  if (launches) *launches = s.launches;
  return GBX_OK;
}

int gbx_cc_program_selftest(long long limit_cycles, void* stream) {
  if (limit_cycles <= 0) return fail(GBX_EINVAL, "bad wait limit");
  int err = 0;
  GBX_TRY(prog_wait_selftest(limit_cycles, (cudaStream_t)stream, &err));
  if (err != 0) return fail(GBX_ETIMEOUT, "persistent iteration: a bounded device wait ran out (code %d)", err);
  return GBX_OK;
}

int gbx_cc_iterate(gbx_cc_job* job, int niter, double* energies, void* stream) {
  GBX_TRY(gbx_cc_enqueue(job, niter, stream));
  GBX_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  GBX_TRY(gbx_cc_check(job));
  if (energies && niter > 0) {
    int first = job->nenergies - niter;
    if (first + niter > job->hist_cap) return fail(GBX_EUNSUPPORTED, "energy history full");
    GBX_CUDA(cudaMemcpy(energies, job->d_hist + first, sizeof(double) * niter, cudaMemcpyDeviceToHost));
  }
  return GBX_OK;
}

int gbx_cc_energies(gbx_cc_job* job, double* energies, int* count) {
  if (!job || !count) return fail(GBX_EINVAL, "bad arguments");
  int n = std::min(std::min(*count, job->nenergies), job->hist_cap);
  GBX_CUDA(cudaDeviceSynchronize());
  if (n > 0) GBX_CUDA(cudaMemcpy(energies, job->d_hist, sizeof(double) * n, cudaMemcpyDeviceToHost));
  *count = n;
  return GBX_OK;
}

int gbx_cc_stats_get(const gbx_cc_job* job, gbx_cc_stats* s) {
  if (!job || !s) return fail(GBX_EINVAL, "bad arguments");
  std::memset(s, 0, sizeof(*s));
  s->flops_per_iter = job->flops;
  s->gemm_flops_per_iter = job->gemm_flops;
  s->resident_bytes = (double)job->account.load();
  s->ncontractions = (int)job->cplans.size() - job->iter_plan_begin;
  s->nsums = (int)job->fplans.size();
  s->nblocks_occ = (int)job->occ->ext.size();
  s->nblocks_vir = (int)job->vir->ext.size();
  // once the iteration is captured, its kernel nodes; before, the planned count
  s->launches_per_iter = job->launches;
  if (job->graph) {
    size_t n = 0;
    if (cudaGraphGetNodes(job->graph, nullptr, &n) == cudaSuccess && n > 0) {
      std::vector<cudaGraphNode_t> nodes(n);
      if (cudaGraphGetNodes(job->graph, nodes.data(), &n) == cudaSuccess) {
        int kernels = 0;
        for (size_t i = 0; i < n; ++i) {
          cudaGraphNodeType t;
          if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++kernels;
        }
        s->launches_per_iter = kernels;
      }
    }
  }
  return GBX_OK;
}

int gbx_cc_get_orbitals(const gbx_cc_job* job, int* irrep, double* eps) {
  if (!job) return fail(GBX_EINVAL, "null job");
  if (irrep) std::memcpy(irrep, job->irrep.data(), sizeof(int) * job->n);
  if (eps) std::memcpy(eps, job->eps.data(), sizeof(double) * job->n);
  return GBX_OK;
}

int gbx_cc_get_amplitudes(gbx_cc_job* job, double* t1, double* t2, void* stream) {
  if (!job) return fail(GBX_EINVAL, "null job");
  GBX_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
  const int o = job->o, v = job->v;
  auto dump = [&](const char* name, double* out, int rank) -> int {
    CCTensor* t = job->get(name);
    std::vector<double> h(t->L.nelem);
    GBX_CUDA(cudaMemcpy(h.data(), t->d, sizeof(double) * t->L.nelem, cudaMemcpyDeviceToHost));
    int full[4] = {o, o, v, v};
    if (rank == 2) {
      full[0] = o;
      full[1] = v;
    }
    int64_t total = 1;
    for (int d = 0; d < rank; ++d) total *= full[d];
    std::fill(out, out + total, 0.0);
    for (size_t ti = 0; ti < t->L.tiles.size(); ++ti) {
      const Coords& c = t->L.tiles[ti];
      int ext[4], st[4];
      for (int d = 0; d < rank; ++d) {
        ext[d] = t->L.dims[d]->ext[c[d]];
        st[d] = (int)t->L.dims[d]->start[c[d]];
      }
      int64_t e = 0;
      int idx[4] = {0, 0, 0, 0};
      for (;;) {
        int64_t off = 0;
        for (int d = 0; d < rank; ++d) off = off * full[d] + st[d] + idx[d];
        out[off] = h[t->L.off[ti] + e];
        ++e;
        int d = rank - 1;
        for (; d >= 0; --d) {
          if (++idx[d] < ext[d]) break;
          idx[d] = 0;
        }
        if (d < 0) break;
      }
    }
    return GBX_OK;
  };
  if (t2) GBX_TRY(dump("t2", t2, 4));
  if (t1) {
    if (job->cfg.method == GBX_CC_CCSD) GBX_TRY(dump("t1", t1, 2));
    else std::fill(t1, t1 + (int64_t)o * v, 0.0);
  }
  return GBX_OK;
}

int gbx_cc_gemm_shapes(const gbx_cc_job* job, int64_t* mnk, int* count) {
  if (!job || !count) return fail(GBX_EINVAL, "bad arguments");
  int n = 0;
  for (size_t pi = job->iter_plan_begin; pi < job->cplans.size(); ++pi)
    for (auto& g : job->cplans[pi]->groups) {
      if (g.M == 0 || g.N == 0 || g.K == 0) continue;
      if (mnk && n < *count) {
        mnk[3 * n] = g.M;
        mnk[3 * n + 1] = g.N;
        mnk[3 * n + 2] = g.K;
      }
      ++n;
    }
  *count = n;
  return GBX_OK;
}

int gbx_cc_amplitude_elems(const gbx_cc_job* job, int64_t* n1, int64_t* n2) {
  if (!job) return fail(GBX_EINVAL, "null job");
  auto& T = const_cast<gbx_cc_job*>(job)->T;
  if (n1) *n1 = T.count("t1") ? T.at("t1")->L.nelem : 0;
  if (n2) *n2 = T.at("t2")->L.nelem;
  return GBX_OK;
}

int gbx_cc_set_amplitudes(gbx_cc_job* job, const double* t1, const double* t2, void* stream) {
  if (!job) return fail(GBX_EINVAL, "null job");
  cudaStream_t st = (cudaStream_t)stream;
  if (t2) GBX_CUDA(cudaMemcpyAsync(job->get("t2")->d, t2, sizeof(double) * job->get("t2")->L.nelem,
                                   cudaMemcpyHostToDevice, st));
  if (t1 && job->T.count("t1"))
    GBX_CUDA(cudaMemcpyAsync(job->get("t1")->d, t1, sizeof(double) * job->get("t1")->L.nelem, cudaMemcpyHostToDevice,
                             st));
  // the iteration reads tau, taut and Q of these amplitudes
  if (job->T.count("t1"))
    GBX_TRY(run_cc_amp(job->amp, job->get("t1")->d, job->get("t2")->d, job->get("tau")->d, job->get("taut")->d,
                       job->get("Q")->d, st));
  return GBX_OK;
}

int gbx_cc_save_amplitudes(gbx_cc_job* job, double* t1, double* t2, void* stream) {
  if (!job) return fail(GBX_EINVAL, "null job");
  cudaStream_t st = (cudaStream_t)stream;
  if (t2) GBX_CUDA(cudaMemcpyAsync(t2, job->get("t2")->d, sizeof(double) * job->get("t2")->L.nelem,
                                   cudaMemcpyDeviceToHost, st));
  if (t1 && job->T.count("t1"))
    GBX_CUDA(cudaMemcpyAsync(t1, job->get("t1")->d, sizeof(double) * job->get("t1")->L.nelem, cudaMemcpyDeviceToHost,
                             st));
  return GBX_OK;
}

int gbx_cc_read_energy(gbx_cc_job* job, double* energy, void* stream) {
  if (!job || !energy) return fail(GBX_EINVAL, "bad arguments");
  int k = job->nenergies - 1;
  if (k < 0 || k >= job->hist_cap) return fail(GBX_EUNSUPPORTED, "energy history full");
  GBX_CUDA(cudaMemcpyAsync(energy, job->d_hist + k, sizeof(double), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  return GBX_OK;
}

int gbx_cc_profile(gbx_cc_job* job, int cap, float* ms, double* flops, double* bytes, int* kind, int* plan,
                   char* names, int name_len, int* count, void* stream) {
  if (!job || !count) return fail(GBX_EINVAL, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  int n = (int)job->steps.size();
  std::vector<cudaEvent_t> ev(n + 1);
  for (auto& e : ev) GBX_CUDA(cudaEventCreate(&e));
  GBX_CUDA(cudaEventRecord(ev[0], st));
  for (int i = 0; i < n; ++i) {
    // each step inside an NVTX range of its name, so that a profiler's
    // launch list maps every kernel to its step
    nvtxRangePushA(job->info[i].name.c_str());
    const int rc = job->steps[i](st);
    nvtxRangePop();
    GBX_TRY(rc);
    GBX_CUDA(cudaEventRecord(ev[i + 1], st));
  }
  GBX_CUDA(cudaEventSynchronize(ev[n]));
  job->nenergies += 1;
  for (int i = 0; i < n && i < cap; ++i) {
    float t = 0.f;
    GBX_CUDA(cudaEventElapsedTime(&t, ev[i], ev[i + 1]));
    if (ms) ms[i] = t;
    if (flops) flops[i] = job->info[i].flops;
    if (bytes) bytes[i] = job->info[i].bytes;
    if (kind) kind[i] = job->info[i].kind;
    if (plan) plan[i] = job->info[i].plan;
    if (names && name_len > 0) {
      std::strncpy(names + (size_t)i * name_len, job->info[i].name.c_str(), name_len - 1);
      names[(size_t)i * name_len + name_len - 1] = 0;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  *count = n;
  return GBX_OK;
}

int gbx_cc_plan_info(const gbx_cc_job* job, int contraction, int* split_width, int* n_split, int* n_f64,
                     int* slices) {
  if (!job || contraction < 0 || contraction >= (int)job->cplans.size()) return fail(GBX_EINVAL, "bad arguments");
  const ContractionPlan* p = job->cplans[contraction].get();
  if (split_width) *split_width = p->split_width;
  if (n_split) *n_split = p->n_split_groups;
  if (n_f64) *n_f64 = p->n_f64_groups;
  if (slices) *slices = p->slices > 0 ? p->slices : 6;
  return GBX_OK;
}

int gbx_cc_time_gemm(gbx_cc_job* job, int contraction, int reps, float* ms, double* fp64_flops,
                     double* tensor_flops, int* engine, void* stream) {
  if (!job || contraction < 0 || contraction >= (int)job->cplans.size() || reps < 1)
    return fail(GBX_EINVAL, "bad arguments");
  ContractionPlan* p = job->cplans[contraction].get();
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t e0, e1;
  GBX_CUDA(cudaEventCreate(&e0));
  GBX_CUDA(cudaEventCreate(&e1));
  // the arena is shared by every plan: pack and split this plan's operands
  // again, then time only the GEMM launches (a direct plan: its one launch
  // accumulating with alpha = 0, which leaves C as it is)
  const double* dA = job->plan_operands[contraction].first->d;
  const double* dB = job->plan_operands[contraction].second->d;
  double* dC = job->plan_outputs[contraction]->d;
  GBX_TRY(p->stage(dA, dB, st));
  const bool stores = p->dir_overwrite;
  p->dir_overwrite = false;
  GBX_CUDA(cudaEventRecord(e0, st));
  int rc = GBX_OK;
  for (int r = 0; r < reps && rc == GBX_OK; ++r) {
    if (p->direct) {
      rc = p->execute(dA, dB, dC, 0.0, st);
      continue;
    }
    if (p->split) rc = run_split_plan(p->split, false, false, st);
    if (rc == GBX_OK) rc = p->f64.run(st);
  }
  p->dir_overwrite = stores;
  GBX_TRY(rc);
  GBX_CUDA(cudaEventRecord(e1, st));
  GBX_CUDA(cudaEventSynchronize(e1));
  float t = 0.f;
  GBX_CUDA(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ms) *ms = t / reps;
  if (fp64_flops) *fp64_flops = p->direct ? p->flops : p->gemm_flops;
  if (tensor_flops) *tensor_flops = split_plan_tensor_flops(p->split);
  if (engine) *engine = p->direct ? 3 : p->split ? (p->f64.nprob ? 2 : 1) : 0;
  return GBX_OK;
}

int gbx_cc_contraction_error(gbx_cc_job* job, int contraction, double* rel_frob_err, double* max_abs_err,
                             void* stream) {
  if (!job || contraction < 0 || contraction >= (int)job->cplans.size()) return fail(GBX_EINVAL, "bad arguments");
  cudaStream_t st = (cudaStream_t)stream;
  ContractionPlan* p = job->cplans[contraction].get();
  const CCTensor* A = job->plan_operands[contraction].first;
  const CCTensor* B = job->plan_operands[contraction].second;
  const CCTensor* C = job->plan_outputs[contraction];
  const auto& lab = job->plan_labels[contraction];
  // a plain FP64 plan of the same contraction (its own workspace; constant
  // operands packed like the changing ones)
  std::unique_ptr<ContractionPlan> ref;
  GBX_TRY(plan_contraction(A->L, B->L, C->L, gbx_cc_job::labels(lab[0].c_str()), gbx_cc_job::labels(lab[1].c_str()),
                           gbx_cc_job::labels(lab[2].c_str()), Engine::F64, 0, ref, false, false));
  const int64_t n = C->L.nelem;
  double *c_job = nullptr, *c_ref = nullptr;
  // Integral operands that only served as constant plan operands were
  // released when the job was built (the job's plan keeps them packed and
  // split); the FP64 plan packs them, so they are generated again into
  // scratch from the same device tables.
  std::vector<double*> regen;
  const size_t ntiles0 = job->tilesets.size();
  auto release = [&]() {
    cudaStreamSynchronize(st);
    for (double* d : regen) dev_free(d);
    job->tilesets.resize(ntiles0);
  };
  auto operand = [&](const CCTensor* t, const double** out) -> int {
    *out = t->d;
    if (t->d) return GBX_OK;
    std::string name;
    for (auto& kv : job->T)
      if (kv.second.get() == t) name = kv.first;
    if (!gbx_cc_job::is_integral(name.c_str()))
      return fail(GBX_EINVAL, "operand %s of contraction %d has no device memory", name.c_str(), contraction);
    double* d = nullptr;
    GBX_TRY(dev_alloc((void**)&d, sizeof(double) * std::max<int64_t>(1, t->L.nelem)));
    regen.push_back(d);
    CCTileSet* ts = job->tileset(t);
    if (!ts) return fail(GBX_ENOMEM, "tile set upload failed");
    GBX_TRY(run_cc_tiles(*ts, CC_OP_INTEGRAL, job->tab, nullptr, d, st));
    *out = d;
    return GBX_OK;
  };
  const double *rA = nullptr, *rB = nullptr;
  int rc = operand(A, &rA);
  if (rc == GBX_OK) rc = operand(B, &rB);
  if (rc == GBX_OK) rc = dev_alloc((void**)&c_job, sizeof(double) * std::max<int64_t>(n, 1));
  if (rc == GBX_OK) rc = dev_alloc((void**)&c_ref, sizeof(double) * std::max<int64_t>(n, 1));
  std::vector<double> h_job(n), h_ref(n);
  if (rc == GBX_OK) {
    cudaMemsetAsync(c_job, 0, sizeof(double) * n, st);
    cudaMemsetAsync(c_ref, 0, sizeof(double) * n, st);
    // the job's plan on the current operands (constant ones are already
    // packed and split and are not read again); a plan that stores its
    // result does so with its own factor, which the FP64 plan then takes
    rc = p->execute(A->d, B->d, c_job, 1.0, st);
    if (rc == GBX_OK) rc = ref->execute(rA, rB, c_ref, p->store_scale != 0.0 ? p->store_scale : 1.0, st);
    if (rc == GBX_OK) {
      cudaError_t e = cudaMemcpyAsync(h_job.data(), c_job, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaMemcpyAsync(h_ref.data(), c_ref, sizeof(double) * n, cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) rc = cuda_fail(e, "contraction error readback", __FILE__, __LINE__);
    }
    if (rc == GBX_OK && p->split) {
      const int err = split_plan_error(p->split);
      if (err != 0) rc = fail(GBX_ETIMEOUT, "split GEMM: a bounded device wait ran out (stage %d)", err);
    }
  }
  release();
  dev_free(c_job);
  dev_free(c_ref);
  GBX_TRY(rc);
  double num = 0.0, den = 0.0, mx = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    const double d = h_job[i] - h_ref[i];
    num += d * d;
    den += h_ref[i] * h_ref[i];
    mx = std::max(mx, std::fabs(d));
  }
  if (rel_frob_err) *rel_frob_err = den > 0.0 ? std::sqrt(num / den) : std::sqrt(num);
  if (max_abs_err) *max_abs_err = mx;
  return GBX_OK;
}

int gbx_cc_destroy(gbx_cc_job* job) {
  delete job;
  return GBX_OK;
}

}  // extern "C"
