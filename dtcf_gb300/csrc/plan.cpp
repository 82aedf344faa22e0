// Contraction planning over block-sparse tensor layouts (see plan.h).
#include "plan.h"

#include <algorithm>
#include <cstring>
#include <map>
#include <set>
#include <tuple>

#include "program.h"
#include "split.h"

namespace gbx {

std::shared_ptr<BlockDim> BlockDim::uniform(int nblocks, int extent) {
  return make(std::vector<int>(nblocks, extent), std::vector<int>(nblocks, 0));
}

std::shared_ptr<BlockDim> BlockDim::make(const std::vector<int>& ext, const std::vector<int>& irrep) {
  auto b = std::make_shared<BlockDim>();
  b->ext = ext;
  b->irrep = irrep;
  b->start.resize(ext.size());
  int64_t s = 0;
  for (size_t i = 0; i < ext.size(); ++i) {
    b->start[i] = s;
    s += ext[i];
  }
  b->total = s;
  return b;
}

void TensorLayout::add_tile(const Coords& c) {
  index[coord_key(c.data(), rank)] = (int)tiles.size();
  tiles.push_back(c);
  off.push_back(nelem);
  nelem += tile_size(c.data());
}

int TensorLayout::resolve(const int* v, int* src_dim, double* factor) const {
  *factor = 1.0;
  for (int d = 0; d < rank; ++d) src_dim[d] = d;
  int id = find(v);
  if (id >= 0) return id;
  // canonicalise: within each group sort block coords non-increasing (stable),
  // counting transpositions
  int order[kMaxDims];
  for (int d = 0; d < rank; ++d) order[d] = d;
  int swaps = 0;
  std::vector<int> gids;
  for (int d = 0; d < rank; ++d)
    if (group[d] >= 0 && std::find(gids.begin(), gids.end(), group[d]) == gids.end()) gids.push_back(group[d]);
  int canon[kMaxDims];
  for (int d = 0; d < rank; ++d) canon[d] = v[d];
  for (int g : gids) {
    std::vector<int> pos;
    for (int d = 0; d < rank; ++d)
      if (group[d] == g) pos.push_back(d);
    // bubble sort positions by coordinate (descending), counting swaps
    std::vector<int> who(pos.size());  // virtual dim sitting at pos[i]
    for (size_t i = 0; i < pos.size(); ++i) who[i] = pos[i];
    for (size_t i = 0; i < pos.size(); ++i)
      for (size_t j = 0; j + 1 < pos.size() - i; ++j)
        if (v[who[j]] < v[who[j + 1]]) {
          std::swap(who[j], who[j + 1]);
          ++swaps;
        }
    for (size_t i = 0; i < pos.size(); ++i) {
      canon[pos[i]] = v[who[i]];
      order[pos[i]] = who[i];  // stored dim pos[i] holds virtual dim who[i]
    }
  }
  id = find(canon);
  if (id < 0) return -1;
  for (int s = 0; s < rank; ++s) src_dim[order[s]] = s;
  *factor = (swaps & 1) ? (double)sign : 1.0;
  return id;
}

TensorLayout TensorLayout::full(const std::vector<std::shared_ptr<BlockDim>>& dims, const std::vector<int>& group,
                                int sign, bool canonical_only) {
  TensorLayout t;
  t.rank = (int)dims.size();
  t.dims = dims;
  t.group = group.empty() ? std::vector<int>(t.rank, -1) : group;
  t.sign = sign;
  std::vector<int> c(t.rank, 0);
  if (t.rank == 0) return t;
  for (;;) {
    bool ok = t.irrep_of(c.data()) == 0;
    if (ok && canonical_only)
      for (int i = 0; i < t.rank && ok; ++i)
        for (int j = i + 1; j < t.rank; ++j)
          if (t.group[i] >= 0 && t.group[i] == t.group[j] && c[i] < c[j]) {
            ok = false;
            break;
          }
    if (ok) t.add_tile(c);
    int d = t.rank - 1;
    for (; d >= 0; --d) {
      if (++c[d] < (int)dims[d]->ext.size()) break;
      c[d] = 0;
    }
    if (d < 0) break;
  }
  return t;
}

std::vector<std::string> split_labels(const char* s) {
  std::vector<std::string> out;
  if (!s) return out;
  std::string str(s);
  if (str.find(',') == std::string::npos) {  // one character per index
    for (char ch : str)
      if (ch != ' ') out.push_back(std::string(1, ch));
    return out;
  }
  std::string cur;
  for (char ch : str) {
    if (ch == ',') {
      out.push_back(cur);
      cur.clear();
    } else if (ch != ' ') {
      cur += ch;
    }
  }
  out.push_back(cur);
  return out;
}

int parse_contraction(const std::vector<std::string>& la, const std::vector<std::string>& lb,
                      const std::vector<std::string>& lc, ContractionSpec& out) {
  auto find = [](const std::vector<std::string>& v, const std::string& x) {
    for (size_t i = 0; i < v.size(); ++i)
      if (v[i] == x) return (int)i;
    return -1;
  };
  out = ContractionSpec();
  std::set<std::string> seen;
  for (auto* v : {&la, &lb, &lc})
    for (size_t i = 0; i < v->size(); ++i)
      for (size_t j = i + 1; j < v->size(); ++j)
        if ((*v)[i] == (*v)[j]) return fail(GBX_EINVAL, "index %s repeated in one tensor", (*v)[i].c_str());
  for (size_t i = 0; i < la.size(); ++i) {
    int ib = find(lb, la[i]), ic = find(lc, la[i]);
    if (ib >= 0 && ic >= 0) return fail(GBX_EUNSUPPORTED, "index %s in A, B and C", la[i].c_str());
    if (ib < 0 && ic < 0) return fail(GBX_EUNSUPPORTED, "index %s of A is neither contracted nor kept", la[i].c_str());
    if (ib >= 0) {
      out.contrA.push_back((int)i);
      out.contrB.push_back(ib);
    } else {
      out.extA.push_back((int)i);
    }
  }
  for (size_t i = 0; i < lb.size(); ++i) {
    int ia = find(la, lb[i]), ic = find(lc, lb[i]);
    if (ia < 0 && ic < 0) return fail(GBX_EUNSUPPORTED, "index %s of B is neither contracted nor kept", lb[i].c_str());
    if (ia < 0) out.extB.push_back((int)i);
  }
  out.c_from.assign(lc.size(), 0);
  for (size_t i = 0; i < lc.size(); ++i) {
    int ia = find(la, lc[i]), ib = find(lb, lc[i]);
    if (ia >= 0) {
      int k = (int)(std::find(out.extA.begin(), out.extA.end(), ia) - out.extA.begin());
      out.c_from[i] = k;
    } else if (ib >= 0) {
      int k = (int)(std::find(out.extB.begin(), out.extB.end(), ib) - out.extB.begin());
      out.c_from[i] = -(1 + k);
    } else {
      return fail(GBX_EINVAL, "index %s of C appears in neither A nor B", lc[i].c_str());
    }
  }
  if (out.extA.size() + out.extB.size() != lc.size()) return fail(GBX_EINVAL, "C indices do not match A and B");
  return GBX_OK;
}

// Host-side bounds check of a move set against its buffers (done once per
// plan, so a bad descriptor can never reach the device).
int check_moves(const MoveSet& ms, int64_t src_elems, int64_t dst_elems, const char* what) {
  for (const MoveDesc& m : ms.host) {
    if (m.n == 0) continue;
    int64_t smax = m.src, dmax = m.dst;
    for (int d = 0; d < m.rank; ++d) {
      if (m.sstr[d] < 0 || m.dstr[d] < 0) return fail(GBX_EINVAL, "%s: negative stride", what);
      smax += (int64_t)(m.ext[d] - 1) * m.sstr[d];
      dmax += (int64_t)(m.ext[d] - 1) * m.dstr[d];
    }
    if (m.src < 0 || m.dst < 0 || smax >= src_elems || dmax >= dst_elems)
      return fail(GBX_EINVAL, "%s: move outside its buffers (src %lld/%lld, dst %lld/%lld)", what, (long long)smax,
                  (long long)src_elems, (long long)dmax, (long long)dst_elems);
  }
  return GBX_OK;
}

namespace {

// Enumerates all block tuples over the given dims (odometer order = lexicographic).
template <class F>
void for_tuples(const std::vector<const BlockDim*>& dims, F&& f) {
  std::vector<int> c(dims.size(), 0);
  for (const BlockDim* d : dims)
    if (d->ext.empty()) return;
  for (;;) {
    f(c);
    int d = (int)dims.size() - 1;
    for (; d >= 0; --d) {
      if (++c[d] < (int)dims[d]->ext.size()) break;
      c[d] = 0;
    }
    if (d < 0) break;
  }
}

struct TupleIndex {  // ordered tuples of one irrep with element offsets
  std::map<std::vector<int>, int64_t> off;
  int64_t total = 0;
};

int tuple_irrep(const std::vector<const BlockDim*>& dims, const std::vector<int>& t) {
  int h = 0;
  for (size_t i = 0; i < t.size(); ++i) h ^= dims[i]->irrep[t[i]];
  return h;
}

int64_t tuple_size(const std::vector<const BlockDim*>& dims, const std::vector<int>& t) {
  int64_t n = 1;
  for (size_t i = 0; i < t.size(); ++i) n *= dims[i]->ext[t[i]];
  return n;
}

// strides inside a packed sub-block for a list of dims with given extents:
// dim j of the list gets base * prod(ext of later dims)
void sub_strides(const std::vector<int64_t>& ext, int64_t base, std::vector<int64_t>& str) {
  str.assign(ext.size(), 0);
  int64_t s = base;
  for (int j = (int)ext.size() - 1; j >= 0; --j) {
    str[j] = s;
    s *= ext[j];
  }
}

}  // namespace

void choose_engine(GroupBlock& g, bool split_engine, bool split_all, int slices) {
  g.engine = 0;
  g.swap = false;
  if (!split_engine || g.M == 0 || g.N == 0 || g.K == 0) return;
  auto up = [](int64_t x, int64_t m) { return (double)((x + m - 1) / m * m); };
  const int S = slices > 0 ? slices : 6;
  const double pairs = S * (S + 1) / 2.0;
  const double kp = up(g.K, 64);
  // slice products at ~1 PFLOP/s, or the wide operand's slices streamed once
  // per slice pair (2 bytes per element per pair), whichever binds; a thin-K
  // problem (K <= 64, at most 32 columns) streams each slice once
  auto split_cost = [&](int64_t rows, int64_t cols) {
    const double mp = up(rows, 128);
    if (g.K <= 64 && cols <= 32)
      return std::max(2.0 * pairs * mp * 32.0 * 64.0 / 1.0e15, S * 2.0 * mp * 64.0 / 6e12);
    return std::max(2.0 * pairs * mp * up(cols, 64) * kp / 1.0e15, pairs * 2.0 * mp * kp / 6e12);
  };
  const double t_split = split_cost(g.M, g.N);
  const double t_split_sw = split_cost(g.N, g.M);
  const int mi = (int)std::min<int64_t>(g.M, 1 << 30), ni = (int)std::min<int64_t>(g.N, 1 << 30);
  const int v = f64_variant_planned(mi, ni, (int)std::min<int64_t>(g.K, 1 << 30));
  // thin FP64: exact flops, or streaming the wide operand once, whichever binds
  const double wide = (double)std::max(g.M, g.N) * (double)g.K * 8.0;
  const double outs = (double)g.M * (double)g.N * 8.0;
  const double t_f64 =
      v == 7 ? std::max(2.0 * (double)g.M * (double)g.N * (double)g.K / 0.9e12,
                        (double)(g.M + g.N) * (double)g.K * 8.0 / 5e12) + 4e-6
      : v == 6 ? std::max(2.0 * (double)g.M * (double)g.N * (double)g.K / 0.9e12, outs / 5e12) + 2e-6
      : v >= 4 ? std::max(2.0 * (double)g.M * (double)g.N * (double)g.K / 0.9e12, wide / 5e12) + 2e-6
               : 2.0 * up(g.M, f64_tile_m(v)) * up(g.N, f64_tile_n(v)) * up(g.K, 16) / 0.95e12;
  const double best_split = std::min(t_split, t_split_sw) + 4e-6;  // + split and launch overhead
  if (split_all || best_split < t_f64) {
    g.engine = 1;
    g.swap = t_split_sw < t_split;
  }
}

ContractionPlan::~ContractionPlan() {
  destroy_split_plan(split);
  dev_free(d_dir_items);
  dev_free(d_dir_pairs);
  dev_free(d_keepA);
  dev_free(d_keepB);
  dev_free(d_own_arena);
}

int plan_contraction(const TensorLayout& A, const TensorLayout& B, const TensorLayout& C,
                     const std::vector<std::string>& la, const std::vector<std::string>& lb,
                     const std::vector<std::string>& lc, Engine e, int nslices,
                     std::unique_ptr<ContractionPlan>& out, bool split_all, bool defer,
                     const ContractionPair* pair) {
  if ((int)la.size() != A.rank || (int)lb.size() != B.rank || (int)lc.size() != C.rank)
    return fail(GBX_EINVAL, "index strings do not match tensor ranks (%d/%d, %d/%d, %d/%d)", (int)la.size(), A.rank,
                (int)lb.size(), B.rank, (int)lc.size(), C.rank);
  auto p = std::make_unique<ContractionPlan>();
  p->A = A;
  p->B = B;
  p->C = C;
  GBX_TRY(parse_contraction(la, lb, lc, p->spec));
  const ContractionSpec& s = p->spec;
  // dimension compatibility
  for (size_t i = 0; i < s.contrA.size(); ++i)
    if (!A.dims[s.contrA[i]]->same_as(*B.dims[s.contrB[i]]))
      return fail(GBX_EINVAL, "contracted index %s has different blocking in A and B", la[s.contrA[i]].c_str());
  std::vector<const BlockDim*> dA, dB, dK;
  for (int d : s.extA) dA.push_back(A.dims[d].get());
  for (int d : s.extB) dB.push_back(B.dims[d].get());
  for (int d : s.contrA) dK.push_back(A.dims[d].get());
  for (int i = 0; i < C.rank; ++i) {
    const BlockDim* cd = C.dims[i].get();
    const BlockDim* src = s.c_from[i] >= 0 ? dA[s.c_from[i]] : dB[-1 - s.c_from[i]];
    if (!cd->same_as(*src)) return fail(GBX_EINVAL, "index %s has different blocking in C", lc[i].c_str());
  }
  // rows / columns needed by C's stored tiles, per irrep
  std::map<int, TupleIndex> rows, cols, ks;
  std::vector<std::vector<int>> c_row(C.tiles.size()), c_col(C.tiles.size());
  for (size_t t = 0; t < C.tiles.size(); ++t) {
    const Coords& cc = C.tiles[t];
    std::vector<int> r(s.extA.size()), c(s.extB.size());
    for (int i = 0; i < C.rank; ++i) {
      if (s.c_from[i] >= 0) r[s.c_from[i]] = cc[i]; else c[-1 - s.c_from[i]] = cc[i];
    }
    c_row[t] = r;
    c_col[t] = c;
    rows[tuple_irrep(dA, r)].off[r] = 0;
    cols[tuple_irrep(dB, c)].off[c] = 0;
  }
  // ks_full: every contracted block tuple (the algorithmic flops, the direct
  // engine); ks: the tuples the packed GEMMs run over -- with a symmetric
  // contracted pair, block pairs X >= Y only
  int px = -1, py = -1;
  if (pair) {
    for (size_t t = 0; t < s.contrA.size(); ++t) {
      if (la[s.contrA[t]] == pair->x) px = (int)t;
      if (la[s.contrA[t]] == pair->y) py = (int)t;
    }
    if (px < 0 || py < 0 || px == py)
      return fail(GBX_EINVAL, "pair %s%s is not two contracted indices", pair->x.c_str(), pair->y.c_str());
    if (!dK[px]->same_as(*dK[py])) return fail(GBX_EINVAL, "pair %s%s: blocking differs", pair->x.c_str(), pair->y.c_str());
  }
  std::map<int, TupleIndex> ks_full;
  for_tuples(dK, [&](const std::vector<int>& k) {
    ks_full[tuple_irrep(dK, k)].off[k] = 0;
    if (px < 0 || k[px] >= k[py]) ks[tuple_irrep(dK, k)].off[k] = 0;
  });
  if (dK.empty()) {
    ks[0].off[std::vector<int>()] = 0;
    ks_full[0].off[std::vector<int>()] = 0;
  }
  auto assign = [](TupleIndex& ti, const std::vector<const BlockDim*>& dims) {
    ti.total = 0;
    for (auto& kv : ti.off) {
      kv.second = ti.total;
      ti.total += tuple_size(dims, kv.first);
    }
  };
  for (auto& kv : rows) assign(kv.second, dA);
  for (auto& kv : cols) assign(kv.second, dB);
  for (auto& kv : ks) assign(kv.second, dK);
  for (auto& kv : ks_full) assign(kv.second, dK);
  // irrep groups present in rows, cols and K
  int64_t ao = 0, bo = 0, co = 0;
  std::map<int, int> gidx;
  for (auto& kv : rows) {
    int h = kv.first;
    if (!cols.count(h)) continue;
    GroupBlock g;
    g.h = h;
    g.M = kv.second.total;
    g.N = cols[h].total;
    g.K = ks.count(h) ? ks[h].total : 0;
    g.a_off = ao;
    g.b_off = bo;
    g.c_off = co;
    ao += g.M * g.K;
    bo += g.N * g.K;
    co += g.M * g.N;
    gidx[h] = (int)p->groups.size();
    p->groups.push_back(g);
  }
  p->a_elems = ao;
  p->b_elems = bo;
  p->c_elems = co;
  for (auto& g : p->groups) choose_engine(g, e == Engine::Split, split_all, nslices);

  // pack moves: A (rows = extA tuples of irrep h, cols = K tuples of irrep h)
  auto pack = [&](const TensorLayout& T, const std::vector<int>& ext_dims, const std::vector<int>& contr_dims,
                  std::map<int, TupleIndex>& rowsets, bool isA, MoveSet& ms, bool& needs_zero,
                  bool pair_scaled) -> int {
    std::vector<const BlockDim*> dR;
    for (int d : ext_dims) dR.push_back(T.dims[d].get());
    for (auto& kv : rowsets) {
      int h = kv.first;
      auto gi = gidx.find(h);
      if (gi == gidx.end()) continue;
      const GroupBlock& g = p->groups[gi->second];
      if (g.K == 0) continue;
      TupleIndex& kt = ks[h];
      for (auto& rv : kv.second.off) {
        for (auto& kvv : kt.off) {
          int v[kMaxDims];
          for (size_t i = 0; i < ext_dims.size(); ++i) v[ext_dims[i]] = rv.first[i];
          for (size_t i = 0; i < contr_dims.size(); ++i) v[contr_dims[i]] = kvv.first[i];
          int src_dim[kMaxDims];
          double factor;
          int id = T.resolve(v, src_dim, &factor);
          if (id < 0) {
            needs_zero = true;
            continue;
          }
          // stored tile strides
          const Coords& sc = T.tiles[id];
          int64_t sstr_st[kMaxDims];
          sstr_st[T.rank - 1] = 1;
          for (int d = T.rank - 2; d >= 0; --d) sstr_st[d] = sstr_st[d + 1] * T.dims[d + 1]->ext[sc[d + 1]];
          // destination strides inside the packed block
          std::vector<int64_t> eR, eK, sR, sK;
          for (size_t i = 0; i < ext_dims.size(); ++i) eR.push_back(T.dims[ext_dims[i]]->ext[v[ext_dims[i]]]);
          for (size_t i = 0; i < contr_dims.size(); ++i) eK.push_back(T.dims[contr_dims[i]]->ext[v[contr_dims[i]]]);
          sub_strides(eR, g.K, sR);
          sub_strides(eK, 1, sK);
          int64_t ext[kMaxDims], sstr[kMaxDims], dstr[kMaxDims];
          for (int d = 0; d < T.rank; ++d) {
            ext[d] = T.dims[d]->ext[v[d]];
            sstr[d] = sstr_st[src_dim[d]];
          }
          for (size_t i = 0; i < ext_dims.size(); ++i) dstr[ext_dims[i]] = sR[i];
          for (size_t i = 0; i < contr_dims.size(); ++i) dstr[contr_dims[i]] = sK[i];
          int64_t dst = (isA ? g.a_off : g.b_off) + rv.second * g.K + kvv.second;
          // off-diagonal block pairs of a symmetric contracted pair count twice
          if (pair_scaled && px >= 0 && kvv.first[px] > kvv.first[py]) factor *= 2.0;
          ms.host.push_back(make_move(T.rank, ext, sstr, dstr, T.off[id], dst, 0, factor));
        }
      }
    }
    return GBX_OK;
  };
  std::vector<int> contrB_in_A_order = s.contrB;
  GBX_TRY(pack(A, s.extA, s.contrA, rows, true, p->packA, p->a_needs_zero, pair && !pair->scale_b));
  GBX_TRY(pack(B, s.extB, contrB_in_A_order, cols, false, p->packB, p->b_needs_zero, pair && pair->scale_b));

  // unpack C tiles
  for (size_t t = 0; t < C.tiles.size(); ++t) {
    int hr = tuple_irrep(dA, c_row[t]);
    auto gi = gidx.find(hr);
    if (gi == gidx.end()) continue;
    const GroupBlock& g = p->groups[gi->second];
    if (g.K == 0) continue;
    const Coords& cc = C.tiles[t];
    int64_t roff = rows[hr].off[c_row[t]], coff = cols[hr].off[c_col[t]];
    std::vector<int64_t> eR, eC, sR, sC;
    for (size_t i = 0; i < s.extA.size(); ++i) eR.push_back(dA[i]->ext[c_row[t][i]]);
    for (size_t i = 0; i < s.extB.size(); ++i) eC.push_back(dB[i]->ext[c_col[t][i]]);
    // C block of the group: row-major M x N, or N x M when the GEMM is swapped
    sub_strides(eR, g.swap ? 1 : g.N, sR);
    sub_strides(eC, g.swap ? g.M : 1, sC);
    const int64_t blk_off = g.swap ? coff * g.M + roff : roff * g.N + coff;
    int64_t ext[kMaxDims], sstr[kMaxDims], dstr[kMaxDims];
    dstr[C.rank - 1] = 1;
    for (int d = C.rank - 2; d >= 0; --d) dstr[d] = dstr[d + 1] * C.dims[d + 1]->ext[cc[d + 1]];
    for (int d = 0; d < C.rank; ++d) {
      ext[d] = C.dims[d]->ext[cc[d]];
      sstr[d] = s.c_from[d] >= 0 ? sR[s.c_from[d]] : sC[-1 - s.c_from[d]];
    }
    p->unpackC.host.push_back(make_move(C.rank, ext, sstr, dstr, g.c_off + blk_off, C.off[t], 1, 1.0));
  }

  // algorithmic flops over nonzero (A-block, B-block -> C-block) triples
  double fl = 0.0, gf = 0.0;
  for (auto& g : p->groups) gf += 2.0 * (double)g.M * (double)g.N * (double)g.K;
  for (size_t t = 0; t < C.tiles.size(); ++t) {
    int hr = tuple_irrep(dA, c_row[t]);
    if (!ks_full.count(hr)) continue;
    double mn = (double)tuple_size(dA, c_row[t]) * (double)tuple_size(dB, c_col[t]);
    for (auto& kv : ks_full[hr].off) {
      int v[kMaxDims], sd[kMaxDims];
      double f;
      for (size_t i = 0; i < s.extA.size(); ++i) v[s.extA[i]] = c_row[t][i];
      for (size_t i = 0; i < s.contrA.size(); ++i) v[s.contrA[i]] = kv.first[i];
      if (A.resolve(v, sd, &f) < 0) continue;
      int w[kMaxDims];
      for (size_t i = 0; i < s.extB.size(); ++i) w[s.extB[i]] = c_col[t][i];
      for (size_t i = 0; i < s.contrB.size(); ++i) w[s.contrB[i]] = kv.first[i];
      if (B.resolve(w, sd, &f) < 0) continue;
      fl += 2.0 * mn * (double)tuple_size(dK, kv.first);
    }
  }
  p->flops = fl;
  p->gemm_flops = gf;
  // direct engine: few products per output element, at most two contracted
  // dims, at most kDirMaxPairs operand tile pairs per output tile
  // (tiny contractions too, whose four packed launches cost more than the work)
  const bool few = fl <= 2.0 * kDirectMaxK * (double)C.nelem || (fl <= 4e6 && fl <= 2.0 * 64.0 * (double)C.nelem);
  if (!split_all && fl > 0.0 && few && s.contrA.size() <= 2 && C.rank <= 4 && C.rank >= 1) {
    bool ok = true;
    std::vector<DirItem> items;
    std::vector<DirPair> pairs;
    const int pad = 4 - C.rank;
    for (size_t t = 0; t < C.tiles.size() && ok; ++t) {
      const Coords& cc = C.tiles[t];
      int64_t e4[4] = {1, 1, 1, 1};
      for (int i = 0; i < C.rank; ++i) e4[pad + i] = C.dims[i]->ext[cc[i]];
      const int64_t ntile = e4[0] * e4[1] * e4[2] * e4[3];
      if (ntile >= ((int64_t)1 << 31)) ok = false;
      const int hr = tuple_irrep(dA, c_row[t]);
      const uint32_t pair0 = (uint32_t)pairs.size();
      if (ok && ks_full.count(hr)) {
        for (auto& kv : ks_full[hr].off) {
          int v[kMaxDims], w[kMaxDims], sdA[kMaxDims], sdB[kMaxDims];
          double fA, fB;
          for (size_t i = 0; i < s.extA.size(); ++i) v[s.extA[i]] = c_row[t][i];
          for (size_t i = 0; i < s.contrA.size(); ++i) v[s.contrA[i]] = kv.first[i];
          for (size_t i = 0; i < s.extB.size(); ++i) w[s.extB[i]] = c_col[t][i];
          for (size_t i = 0; i < s.contrB.size(); ++i) w[s.contrB[i]] = kv.first[i];
          const int idA = A.resolve(v, sdA, &fA);
          if (idA < 0) continue;
          const int idB = B.resolve(w, sdB, &fB);
          if (idB < 0) continue;
          // strides of the operands' virtual dims inside their stored tiles
          auto vstrides = [](const TensorLayout& T, int id, const int* sd, int64_t* out) {
            const Coords& sc = T.tiles[id];
            int64_t st[kMaxDims];
            st[T.rank - 1] = 1;
            for (int d = T.rank - 2; d >= 0; --d) st[d] = st[d + 1] * T.dims[d + 1]->ext[sc[d + 1]];
            for (int d = 0; d < T.rank; ++d) out[d] = st[sd[d]];
          };
          int64_t vsA[kMaxDims], vsB[kMaxDims];
          vstrides(A, idA, sdA, vsA);
          vstrides(B, idB, sdB, vsB);
          DirPair pr;
          std::memset(&pr, 0, sizeof(pr));
          pr.offA = A.off[idA];
          pr.offB = B.off[idB];
          for (int i = 0; i < C.rank; ++i) {
            if (s.c_from[i] >= 0) pr.sA[pad + i] = vsA[s.extA[s.c_from[i]]];
            else pr.sB[pad + i] = vsB[s.extB[-1 - s.c_from[i]]];
          }
          pr.ek[0] = pr.ek[1] = 1;
          for (size_t j = 0; j < s.contrA.size(); ++j) {
            pr.sAk[j] = vsA[s.contrA[j]];
            pr.sBk[j] = vsB[s.contrB[j]];
            pr.ek[j] = (uint32_t)A.dims[s.contrA[j]]->ext[kv.first[j]];
          }
          pr.neg = fA * fB < 0.0 ? 1 : 0;
          // every read stays inside the stored tiles
          int64_t ma = 0, mb = 0;
          for (int d = 0; d < 4; ++d) {
            ma += (e4[d] - 1) * pr.sA[d];
            mb += (e4[d] - 1) * pr.sB[d];
          }
          const int64_t ta = A.tile_size(A.tiles[idA].data()), tb = B.tile_size(B.tiles[idB].data());
          if (ta >= ((int64_t)1 << 31) || tb >= ((int64_t)1 << 31)) {  // tile-local offsets are 32-bit
            ok = false;
            break;
          }
          if (ma >= ta || mb >= tb) return fail(GBX_EINVAL, "direct plan: operand read outside its tile");
          for (int j = 0; j < 2; ++j) {
            ma += (int64_t)(pr.ek[j] - 1) * pr.sAk[j];
            mb += (int64_t)(pr.ek[j] - 1) * pr.sBk[j];
          }
          if (ma >= ta || mb >= tb) return fail(GBX_EINVAL, "direct plan: operand read outside its tile");
          pairs.push_back(pr);
        }
      }
      const uint32_t npair = (uint32_t)pairs.size() - pair0;
      if (npair > (uint32_t)kDirMaxPairs) ok = false;
      if (!ok || npair == 0) continue;  // C += alpha * 0: nothing to do for this tile
      for (int64_t f0 = 0; f0 < ntile; f0 += kDirItemElems) {
        DirItem it;
        std::memset(&it, 0, sizeof(it));
        it.coff = C.off[t] + f0;
        it.f1 = FastDiv::make((uint32_t)e4[1]);
        it.f2 = FastDiv::make((uint32_t)e4[2]);
        it.f3 = FastDiv::make((uint32_t)e4[3]);
        it.f0 = (uint32_t)f0;
        it.n = (uint32_t)std::min<int64_t>(kDirItemElems, ntile - f0);
        it.pair0 = pair0;
        it.npair = npair;
        items.push_back(it);
      }
    }
    if (ok && items.size() < ((size_t)1 << 31)) {
      p->direct = true;
      p->dir_items = std::move(items);
      p->dir_pairs = std::move(pairs);
      p->packA.host.clear();
      p->packB.host.clear();
      p->unpackC.host.clear();
      p->a_needs_zero = p->b_needs_zero = false;
    }
  }
  GBX_TRY(check_moves(p->packA, A.nelem, p->a_elems, "pack A"));
  GBX_TRY(check_moves(p->packB, B.nelem, p->b_elems, "pack B"));
  GBX_TRY(check_moves(p->unpackC, p->c_elems, C.nelem, "unpack C"));
  p->split_all = split_all;
  p->engine = e;
  p->slices = nslices;
  for (auto& g : p->groups) {
    if (g.M == 0 || g.N == 0 || g.K == 0 || p->direct) continue;
    if (g.M >= (1ll << 31) || g.N >= (1ll << 31) || g.K >= (1ll << 31))
      return fail(GBX_EUNSUPPORTED, "packed block too large");
    if (g.engine == 1) ++p->n_split_groups; else ++p->n_f64_groups;
  }
  if (!defer) GBX_TRY(p->build());
  out = std::move(p);
  return GBX_OK;
}

namespace {
size_t up256(size_t x) { return (x + 255) / 256 * 256; }
size_t move_bytes(const MoveSet& m) { return m.device_bytes(); }
}  // namespace

// The split engine's problems over the packed buffers (sizes() only needs
// their shapes).
void ContractionPlan::split_problems(std::vector<SplitProblem>& sp) const {
  sp.clear();
  for (auto& g : groups) {
    if (g.M == 0 || g.N == 0 || g.K == 0 || g.engine != 1) continue;
    SplitProblem q;
    if (g.swap) {  // C^T = B A^T: rows from B, C block stored N x M
      q.A = d_Bbig + g.b_off;
      q.B = d_Abig + g.a_off;
      q.M = g.N;
      q.N = g.M;
      q.a_is_plan_b = true;
    } else {
      q.A = d_Abig + g.a_off;
      q.B = d_Bbig + g.b_off;
      q.M = g.M;
      q.N = g.N;
      q.a_is_plan_b = false;
    }
    q.C = d_Cbig + g.c_off;
    q.K = g.K;
    q.width = split_width;
    sp.push_back(q);
  }
}

int ContractionPlan::sizes(size_t* persist, size_t* arena, size_t* static_scratch) const {
  size_t keep = 0, ws = 0, scratch = 0;
  if (direct) {
    if (persist) *persist = up256(dir_items.size() * sizeof(DirItem)) + up256(dir_pairs.size() * sizeof(DirPair));
    if (arena) *arena = 0;
    if (static_scratch) *static_scratch = 0;
    return GBX_OK;
  }
  const size_t ab = up256(sizeof(double) * a_elems), bb = up256(sizeof(double) * b_elems);
  if (keeps_a()) keep += ab; else if (a_static) scratch += ab; else ws += ab;
  if (keeps_b()) keep += bb; else if (b_static) scratch += bb; else ws += bb;
  ws += up256(sizeof(double) * c_elems);
  keep += move_bytes(packA) + move_bytes(packB) + move_bytes(unpackC);
  if (n_split_groups) {
    std::vector<SplitProblem> sp;
    split_problems(sp);
    size_t sp_keep = 0, sp_ws = 0;
    GBX_TRY(split_plan_sizes(sp, slices, a_static, b_static, &sp_keep, &sp_ws));
    // the width autotuner tries every output width in the plan's region:
    // room for the largest of them (split-K partial sums differ by width)
    if (split_width == 0)
      for (int w : {64, 128, 256}) {
        for (auto& q : sp) q.width = w;
        size_t k2 = 0, w2 = 0;
        if (split_plan_sizes(sp, slices, a_static, b_static, &k2, &w2) == GBX_OK) sp_ws = std::max(sp_ws, w2);
      }
    keep += sp_keep;
    ws += sp_ws;
  }
  if (persist) *persist = keep;
  if (arena) *arena = ws;
  if (static_scratch) *static_scratch = scratch;
  return GBX_OK;
}

double ContractionPlan::f64_workspace_estimate() const {
  if (direct) return 0.0;
  std::vector<GemmProblem> fp;
  for (auto& g : groups) {
    if (g.M == 0 || g.N == 0 || g.K == 0 || g.engine == 1) continue;
    GemmProblem q;
    std::memset(&q, 0, sizeof(q));
    q.m = (int)g.M;
    q.n = (int)g.N;
    q.k = (int)g.K;
    fp.push_back(q);
  }
  return 8.0 * (double)f64_partial_elems(fp);
}

int ContractionPlan::build(unsigned char* arena, unsigned char* static_scratch) {
  if (direct) {
    if (!dir_items.empty()) {
      GBX_TRY(dev_alloc((void**)&d_dir_items, sizeof(DirItem) * dir_items.size()));
      GBX_TRY(dev_alloc((void**)&d_dir_pairs, sizeof(DirPair) * dir_pairs.size()));
      GBX_CUDA(cudaMemcpy(d_dir_items, dir_items.data(), sizeof(DirItem) * dir_items.size(), cudaMemcpyHostToDevice));
      GBX_CUDA(cudaMemcpy(d_dir_pairs, dir_pairs.data(), sizeof(DirPair) * dir_pairs.size(), cudaMemcpyHostToDevice));
    }
    return GBX_OK;
  }
  size_t keep = 0, ws = 0, scratch = 0;
  GBX_TRY(sizes(&keep, &ws, &scratch));
  if (!arena && (ws || (scratch && !static_scratch))) {
    GBX_TRY(dev_alloc((void**)&d_own_arena, ws + scratch));
    arena = d_own_arena;
  }
  GBX_TRY(packA.upload());
  GBX_TRY(packB.upload());
  GBX_TRY(unpackC.upload());
  size_t off = 0, soff = 0;
  auto carve = [&](size_t bytes) {
    unsigned char* q = arena + off;
    off += up256(bytes);
    return q;
  };
  unsigned char* sbase = static_scratch ? static_scratch : (arena ? arena + ws : nullptr);
  auto carve_static = [&](size_t bytes) {
    unsigned char* q = sbase + soff;
    soff += up256(bytes);
    return q;
  };
  if (keeps_a()) {
    GBX_TRY(dev_alloc((void**)&d_keepA, std::max<size_t>(8, sizeof(double) * a_elems)));
    d_Abig = d_keepA;
  } else {
    d_Abig = (double*)(a_static ? carve_static(sizeof(double) * a_elems) : carve(sizeof(double) * a_elems));
  }
  if (keeps_b()) {
    GBX_TRY(dev_alloc((void**)&d_keepB, std::max<size_t>(8, sizeof(double) * b_elems)));
    d_Bbig = d_keepB;
  } else {
    d_Bbig = (double*)(b_static ? carve_static(sizeof(double) * b_elems) : carve(sizeof(double) * b_elems));
  }
  d_Cbig = (double*)carve(sizeof(double) * c_elems);
  std::vector<GemmProblem> probs;
  for (auto& g : groups) {
    if (g.M == 0 || g.N == 0 || g.K == 0 || g.engine == 1) continue;
    GemmProblem q;
    std::memset(&q, 0, sizeof(q));
    q.A = d_Abig + g.a_off;
    q.B = d_Bbig + g.b_off;
    q.C = d_Cbig + g.c_off;
    q.a_rs = g.K;
    q.a_cs = 1;
    q.b_rs = g.K;
    q.b_cs = 1;
    q.c_rs = g.N;
    q.m = (int)g.M;
    q.n = (int)g.N;
    q.k = (int)g.K;
    q.alpha = 1.0;
    q.accumulate = 0;
    probs.push_back(q);
  }
  GBX_TRY(f64.build(probs));
  if (n_split_groups) {
    std::vector<SplitProblem> sp;
    split_problems(sp);
    SplitMem mem;
    mem.static_a = a_static;
    mem.static_b = b_static;
    mem.arena = ws > off ? arena + off : nullptr;
    split_arena = mem.arena;
    split_arena_cap = ws > off ? ws - off : 0;
    GBX_TRY(create_split_plan(sp, slices, &split, &mem));
  }
  // uploads and zero fills above ran on the legacy default stream: finish
  // them before any other stream touches the plan's buffers
  GBX_CUDA(cudaStreamSynchronize(cudaStreamLegacy));
  return GBX_OK;
}

int ContractionPlan::tune_split(cudaStream_t st, int reps) {
  if (!split) return GBX_OK;
  cudaEvent_t e0, e1;
  GBX_CUDA(cudaEventCreate(&e0));
  GBX_CUDA(cudaEventCreate(&e1));
  auto time_of = [&](SplitPlan* sp, float* best) -> int {
    GBX_TRY(run_split_plan(sp, !a_static, !b_static, st));  // warm
    *best = 1e30f;
    for (int r = 0; r < reps; ++r) {
      GBX_CUDA(cudaEventRecord(e0, st));
      GBX_TRY(run_split_plan(sp, !a_static, !b_static, st));
      GBX_CUDA(cudaEventRecord(e1, st));
      GBX_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      GBX_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      *best = std::min(*best, ms);
    }
    return GBX_OK;
  };
  float best = 0.f;
  int rc = time_of(split, &best);
  const int keep_w = split_width;
  int best_w = keep_w;
  for (int w : {64, 128, 256}) {
    if (rc != GBX_OK) break;
    if (w == keep_w) continue;
    split_width = w;
    std::vector<SplitProblem> sp;
    split_problems(sp);
    size_t k = 0, ws = 0;
    rc = split_plan_sizes(sp, slices, a_static, b_static, &k, &ws);
    if (rc != GBX_OK) break;
    if (ws > split_arena_cap) continue;  // a candidate must fit the arena the plan was given
    SplitMem mem;
    mem.static_a = a_static;
    mem.static_b = b_static;
    mem.arena = split_arena;
    SplitPlan* alt = nullptr;
    rc = create_split_plan(sp, slices, &alt, &mem);
    if (rc == GBX_OK && cudaStreamSynchronize(cudaStreamLegacy) != cudaSuccess) rc = fail(GBX_ECUDA, "sync failed");
    // constant operands: split again from the packed scratch
    if (rc == GBX_OK && (a_static || b_static)) rc = split_operands(alt, a_static, b_static, st);
    float ms = 0.f;
    if (rc == GBX_OK) rc = time_of(alt, &ms);
    cudaStreamSynchronize(st);
    if (rc == GBX_OK && ms < 0.97f * best) {
      destroy_split_plan(split);
      split = alt;
      best = ms;
      best_w = w;
    } else {
      destroy_split_plan(alt);
    }
  }
  split_width = best_w;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

int ContractionPlan::prepare_static(const double* dA, const double* dB, cudaStream_t st) {
  if (direct) return GBX_OK;  // reads its operands where they are stored
  if (a_static) {
    if (a_needs_zero) GBX_TRY(zero_async(d_Abig, sizeof(double) * a_elems, st));
    GBX_TRY(run_moves(packA, dA, d_Abig, st));
  }
  if (b_static) {
    if (b_needs_zero) GBX_TRY(zero_async(d_Bbig, sizeof(double) * b_elems, st));
    GBX_TRY(run_moves(packB, dB, d_Bbig, st));
  }
  if (split) GBX_TRY(split_operands(split, a_static, b_static, st));
  static_ready = a_static || b_static;
  return GBX_OK;
}

int ContractionPlan::stage(const double* dA, const double* dB, cudaStream_t st) {
  if (direct) return GBX_OK;
  const bool skipA = a_static && static_ready, skipB = b_static && static_ready;
  if ((!skipA && !dA) || (!skipB && !dB)) return fail(GBX_EINVAL, "contraction operand without device memory");
  if (!skipA) {
    if (a_needs_zero) GBX_TRY(zero_async(d_Abig, sizeof(double) * a_elems, st));
    GBX_TRY(run_moves(packA, dA, d_Abig, st));
  }
  if (!skipB) {
    if (b_needs_zero) GBX_TRY(zero_async(d_Bbig, sizeof(double) * b_elems, st));
    GBX_TRY(run_moves(packB, dB, d_Bbig, st));
  }
  if (split) GBX_TRY(split_operands(split, !skipA, !skipB, st));
  return GBX_OK;
}

int ContractionPlan::execute(const double* dA, const double* dB, double* dC, double alpha, cudaStream_t st) {
  if (direct) {
    if (!dA || !dB || !dC) return fail(GBX_EINVAL, "contraction operand without device memory");
    return run_direct(d_dir_items, (int)dir_items.size(), d_dir_pairs, dA, dB, dC, alpha, dir_overwrite, st);
  }
  if (f64.nprob == 0 && !split) return GBX_OK;
  const bool skipA = a_static && static_ready, skipB = b_static && static_ready;
  if ((!skipA && !dA) || (!skipB && !dB)) return fail(GBX_EINVAL, "contraction operand without device memory");
  if (!skipA) {
    if (a_needs_zero) GBX_TRY(zero_async(d_Abig, sizeof(double) * a_elems, st));
    GBX_TRY(run_moves(packA, dA, d_Abig, st));
  }
  if (!skipB) {
    if (b_needs_zero) GBX_TRY(zero_async(d_Bbig, sizeof(double) * b_elems, st));
    GBX_TRY(run_moves(packB, dB, d_Bbig, st));
  }
  GBX_TRY(f64.run(st));
  if (split) GBX_TRY(run_split_plan(split, !skipA, !skipB, st));
  return run_moves_scaled(unpackC, d_Cbig, dC, alpha, st);
}

bool ContractionPlan::set_overwrite(double alpha, int64_t c_elems) {
  int64_t covered = 0;
  if (direct) {
    for (const DirItem& it : dir_items) covered += it.n;
  } else {
    for (const MoveDesc& m : unpackC.host) {
      if (m.op != 1 || m.scale != 1.0) return false;
      covered += m.n;
    }
  }
  if (covered != c_elems) return false;
  if (direct) {
    dir_overwrite = true;
  } else {
    // stores of alpha * the product (a store move ignores the run-time factor)
    for (MoveDesc& m : unpackC.host) {
      m.op = 0;
      m.scale = alpha;
    }
    store_scale = alpha;
  }
  return true;
}

int SumPlan::execute(const double* dA, double* dC, double alpha, cudaStream_t st) {
  return run_moves_scaled(moves, dA, dC, alpha, st);
}

int plan_sum(const TensorLayout& A, const TensorLayout& C, const std::vector<std::string>& la,
             const std::vector<std::string>& lc, double coef, std::unique_ptr<SumPlan>& out, bool defer) {
  if ((int)la.size() != A.rank || (int)lc.size() != C.rank || A.rank != C.rank)
    return fail(GBX_EINVAL, "sum: index strings do not match ranks");
  std::vector<int> a_of_c(C.rank);
  for (int i = 0; i < C.rank; ++i) {
    a_of_c[i] = -1;
    for (int j = 0; j < A.rank; ++j)
      if (la[j] == lc[i]) a_of_c[i] = j;
    if (a_of_c[i] < 0) return fail(GBX_EINVAL, "sum: index %s of C missing in A", lc[i].c_str());
    if (!C.dims[i]->same_as(*A.dims[a_of_c[i]])) return fail(GBX_EINVAL, "sum: blocking differs for %s", lc[i].c_str());
  }
  auto p = std::make_unique<SumPlan>();
  p->A = A;
  p->C = C;
  for (size_t t = 0; t < C.tiles.size(); ++t) {
    const Coords& cc = C.tiles[t];
    int v[kMaxDims];
    for (int i = 0; i < C.rank; ++i) v[a_of_c[i]] = cc[i];  // A's virtual coords
    int src_dim[kMaxDims];
    double f;
    int id = A.resolve(v, src_dim, &f);
    if (id < 0) continue;  // zero tile
    const Coords& sc = A.tiles[id];
    int64_t sst[kMaxDims];
    sst[A.rank - 1] = 1;
    for (int d = A.rank - 2; d >= 0; --d) sst[d] = sst[d + 1] * A.dims[d + 1]->ext[sc[d + 1]];
    int64_t ext[kMaxDims], sstr[kMaxDims], dstr[kMaxDims];
    dstr[C.rank - 1] = 1;
    for (int d = C.rank - 2; d >= 0; --d) dstr[d] = dstr[d + 1] * C.dims[d + 1]->ext[cc[d + 1]];
    for (int i = 0; i < C.rank; ++i) {
      ext[i] = C.dims[i]->ext[cc[i]];
      sstr[i] = sst[src_dim[a_of_c[i]]];
    }
    p->moves.host.push_back(make_move(C.rank, ext, sstr, dstr, A.off[id], C.off[t], 1, coef * f));
  }
  GBX_TRY(check_moves(p->moves, A.nelem, C.nelem, "sum"));
  if (!defer) GBX_TRY(p->moves.upload());
  out = std::move(p);
  return GBX_OK;
}


int FusedSumPlan::upload() {
  release();
  if (items.empty()) return GBX_OK;
  GBX_TRY(dev_alloc((void**)&d_items, sizeof(FsItem) * items.size()));
  GBX_CUDA(cudaMemcpy(d_items, items.data(), sizeof(FsItem) * items.size(), cudaMemcpyHostToDevice));
  if (!terms.empty()) {
    GBX_TRY(dev_alloc((void**)&d_terms, sizeof(FsTerm) * terms.size()));
    GBX_CUDA(cudaMemcpy(d_terms, terms.data(), sizeof(FsTerm) * terms.size(), cudaMemcpyHostToDevice));
  }
  return GBX_OK;
}

void FusedSumPlan::release() {
  dev_free(d_items);
  dev_free(d_terms);
  d_items = nullptr;
  d_terms = nullptr;
}

int FusedSumPlan::execute(const double* const* src, const double* scale, double* out, cudaStream_t st) const {
  if (items.empty()) return GBX_OK;
  if (!d_items) return fail(GBX_EINVAL, "fused sum: plan not uploaded");
  FsSrc s;
  for (int i = 0; i < kFsMaxSlots; ++i) s.p[i] = i < nslots ? src[i] : nullptr;
  for (int i = 0; i < nslots; ++i)
    if (!s.p[i]) return fail(GBX_EINVAL, "fused sum: source %d missing", i);
  return run_fused_sum(d_items, (int)items.size(), d_terms, s, scale, out, st);
}

int plan_fused_sum(const TensorLayout& C, const std::vector<std::string>& lc, const std::vector<FusedTermSpec>& specs,
                   std::unique_ptr<FusedSumPlan>& out) {
  const int r = C.rank;
  if (r < 2 || r > 4 || (int)lc.size() != r) return fail(GBX_EUNSUPPORTED, "fused sum: destination rank %d", r);
  if (C.nelem >= (int64_t)1 << 40) return fail(GBX_EUNSUPPORTED, "fused sum: destination too large");
  const int nt = (int)specs.size();
  if (nt > kFsMaxTerms) return fail(GBX_EUNSUPPORTED, "fused sum: %d terms (at most %d)", nt, kFsMaxTerms);
  std::vector<std::vector<int>> a_of_c(nt, std::vector<int>(r, -1));
  int nslots = 0;
  for (int t = 0; t < nt; ++t) {
    const FusedTermSpec& sp = specs[t];
    if (!sp.A || sp.A->rank != r || (int)sp.la.size() != r)
      return fail(GBX_EINVAL, "fused sum: term %d rank differs from the destination", t);
    if (sp.slot < 0 || sp.slot >= kFsMaxSlots) return fail(GBX_EINVAL, "fused sum: term %d slot %d", t, sp.slot);
    nslots = std::max(nslots, sp.slot + 1);
    for (int i = 0; i < r; ++i) {
      for (int j = 0; j < r; ++j)
        if (sp.la[j] == lc[i]) a_of_c[t][i] = j;
      if (a_of_c[t][i] < 0) return fail(GBX_EINVAL, "fused sum: index %s missing in term %d", lc[i].c_str(), t);
      if (!C.dims[i]->same_as(*sp.A->dims[a_of_c[t][i]]))
        return fail(GBX_EINVAL, "fused sum: blocking differs for %s in term %d", lc[i].c_str(), t);
    }
  }
  auto p = std::make_unique<FusedSumPlan>();
  p->C = C;
  p->nslots = nslots;
  std::vector<int> order(C.tiles.size());
  for (size_t t = 0; t < order.size(); ++t) order[t] = (int)t;
  if (r == 4) {
    auto key = [&](int t) {
      const Coords& c = C.tiles[t];
      return std::make_tuple(std::min(c[0], c[1]), std::max(c[0], c[1]), std::min(c[2], c[3]), std::max(c[2], c[3]));
    };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return key(x) < key(y); });
  }
  for (int t : order) {
    const Coords& cc = C.tiles[t];
    int64_t ext[4];
    for (int i = 0; i < r; ++i) ext[i] = C.dims[i]->ext[cc[i]];
    const int64_t ea = ext[r - 2], eb = ext[r - 1], E = ea * eb;
    const int64_t O0 = r == 4 ? ext[0] : 1, O1 = r >= 3 ? ext[r - 3] : 1;
    if (E == 0 || O0 == 0 || O1 == 0) continue;
    if (O0 * O1 * E >= ((int64_t)1 << 31) || O0 >= 65536 || O1 >= 65536)
      return fail(GBX_EUNSUPPORTED, "fused sum: tile too large");
    const uint32_t term0 = (uint32_t)p->terms.size();
    for (int k = 0; k < nt; ++k) {
      const TensorLayout& A = *specs[k].A;
      int v[kMaxDims];
      for (int i = 0; i < r; ++i) v[a_of_c[k][i]] = cc[i];
      int src_dim[kMaxDims];
      double f;
      const int id = A.resolve(v, src_dim, &f);
      if (id < 0) continue;  // zero tile: the term adds nothing here
      const Coords& sc = A.tiles[id];
      int64_t sst[kMaxDims];
      sst[r - 1] = 1;
      for (int d = r - 2; d >= 0; --d) sst[d] = sst[d + 1] * A.dims[d + 1]->ext[sc[d + 1]];
      int64_t sstr[4];
      for (int i = 0; i < r; ++i) sstr[i] = sst[src_dim[a_of_c[k][i]]];
      FsTerm tm;
      std::memset(&tm, 0, sizeof(tm));
      tm.off = A.off[id];
      tm.so0 = r == 4 ? sstr[0] : 0;
      tm.so1 = r >= 3 ? sstr[r - 3] : 0;
      tm.sa = sstr[r - 2];
      tm.sb = sstr[r - 1];
      tm.coef = specs[k].coef * f;
      tm.slot = specs[k].slot;
      tm.mode = (tm.sb == 1 && tm.sa == eb) ? 0 : (tm.sa == 1 && tm.sb == ea) ? 1 : 2;
      const int64_t span = (O0 - 1) * tm.so0 + (O1 - 1) * tm.so1 + (ea - 1) * tm.sa + (eb - 1) * tm.sb;
      if (tm.off < 0 || tm.off + span >= A.nelem) return fail(GBX_EINVAL, "fused sum: term %d reads outside its source", k);
      if (span >= ((int64_t)1 << 31)) return fail(GBX_EUNSUPPORTED, "fused sum: source tile too large");
      p->terms.push_back(tm);
    }
    const uint32_t nterm = (uint32_t)p->terms.size() - term0;
    // items: runs of whole slabs (across rows) up to kFsItemElems
    // elements, else pieces of one slab
    const int64_t tile_n = O0 * O1 * E;
    const int64_t step = E <= kFsItemElems ? (kFsItemElems / E) * E : kFsItemElems;
    for (int64_t f0 = 0; f0 < tile_n; f0 += step) {
      FsItem it;
      std::memset(&it, 0, sizeof(it));
      const int64_t n = std::min(step, tile_n - f0);
      it.dst = C.off[t] + f0;
      it.fE = FastDiv::make((uint32_t)E);
      it.fea = FastDiv::make((uint32_t)ea);
      it.feb = FastDiv::make((uint32_t)eb);
      it.fo1 = FastDiv::make((uint32_t)O1);
      it.f0 = (uint32_t)f0;
      it.n = (uint32_t)n;
      it.term0 = term0;
      it.nterm = nterm;
      it.whole = (f0 % E == 0 && n % E == 0) ? 1u : 0u;
      if (it.dst < 0 || it.dst + n > C.nelem) return fail(GBX_EINVAL, "fused sum: item outside the destination");
      p->items.push_back(it);
    }
  }
  if (p->items.size() >= ((size_t)1 << 31)) return fail(GBX_EUNSUPPORTED, "fused sum: too many items");
  out = std::move(p);
  return GBX_OK;
}

}  // namespace gbx
