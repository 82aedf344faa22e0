// Coupled-cluster (CCD / CCSD, spin-orbital) iteration driver over the
// block-sparse contraction engine.
//
// Synthetic system (the same definition is restated by the oracle):
//  * splitmix64 streams: stream k of seed s starts from
//    mix64(s ^ (0x9E3779B97F4A7C15 * (k + 1))) and advances by
//    0x9E3779B97F4A7C15; u = (next >> 11) * 2^-53.
//  * orbital irreps (XOR product rule over nirrep = 1, 2, 4 or 8 irreps):
//    each of the n orbitals of a space draws floor(u * nirrep) from stream 1
//    (occupied) or 2 (virtual); the draw repeats until every irrep holds at
//    least min(min_block, n / nirrep) orbitals.  Orbitals are ordered by
//    irrep; an irrep's run is cut into ceil(count / max_block) blocks of
//    near-equal size (larger first).
//  * orbital energies: occupied lo + (hi - lo) * u from stream 3, virtual
//    from stream 4, in orbital order.
//  * <pq||rs> (global orbital indices, occupied first): zero when p == q,
//    r == s or the irrep XOR is non-zero; otherwise order p < q and r < s
//    (one sign flip per swap), P = p*n + q, R = r*n + s, swap so P <= R,
//    value = +-v_scale * exp(-((q - p) + (s - r)) / v_decay) with the sign
//    bit 63 of mix64(seed_int ^ (P * 0x9E3779B97F4A7C15 + R *
//    0xC2B2AE3D27D4EB4F)), seed_int = first draw of stream 5.
//    Antisymmetric in p<->q and r<->s and symmetric under pq<->rs.
//
// Equations: spin-orbital CCSD of Stanton, Gauss, Watts and Bartlett,
// J. Chem. Phys. 94, 4334 (1991), with canonical (diagonal) Fock operator,
// the W_abef ladder factorised into the bare <ab||ef> contraction plus two
// lower-order terms; CCD drops every T1 term.  Jacobi update T = R / D from
// the MP2 guess, energy E = 1/4 sum <ij||ab> tau_ij^ab.
#pragma once
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "../../include/gbx_cc.h"
#include "plan.h"

namespace gbx {

struct CCTile {
  int64_t off;
  uint32_t n;
  int32_t rank;
  uint32_t ext[4];
  int32_t gstart[4];
};

struct CCDeviceTables {
  const int* irrep;   // per global orbital
  const double* eps;  // per global orbital
  const double* mag;  // v_scale * exp(-d / v_decay), d = 0 .. 2 * norb
  int norb, nocc;
  uint64_t seed_int;
};

enum { CC_OP_INTEGRAL = 0, CC_OP_DENOM = 1, CC_OP_INVDENOM = 2 };

struct CCTileSet {
  CCTile* d_tiles = nullptr;
  uint32_t* d_first = nullptr;
  int ntiles = 0;
  uint32_t nchunks = 0;
  int upload(const std::vector<CCTile>& h);
  void release();
  ~CCTileSet() { release(); }
};

int run_cc_tiles(const CCTileSet& ts, int op, const CCDeviceTables& tab, const double* in, double* out,
                 cudaStream_t st);

// The amplitude combinations of one CCSD iteration that need no contraction,
// formed in one pass over t2 (each from the t2 and t1 of the same iteration):
//   tau  = t2 + t1_ia t1_jb - t1_ib t1_ja
//   taut = t2 + (t1_ia t1_jb - t1_ib t1_ja) / 2
//   Q    = t2 / 2 + t1_ia t1_jb            (Q_jn^fb of W_mbej)
// element by element as 0 + t2, then each present product added with its
// coefficient, products and sums separately rounded.  A product is present
// when both t1 tiles are stored (irrep of i equals that of a, and so on).
struct CCAmpTile {
  int64_t off;    // tile offset in t2, tau, taut and Q (one layout)
  int64_t t1[4];  // t1 tiles (i,a), (j,b), (i,b), (j,a); -1 when not stored
  FastDiv fj, fa, fb;
};
struct CCAmpItem {
  uint32_t tile, f0, n, pad;  // elements [f0, f0 + n) of one tile
};
struct CCAmpSet {
  CCAmpTile* d_tiles = nullptr;
  CCAmpItem* d_items = nullptr;
  int nitems = 0;
  size_t bytes = 0;
  int upload(const std::vector<CCAmpTile>& tiles, const std::vector<CCAmpItem>& items);
  void release();
  ~CCAmpSet() { release(); }
};
int run_cc_amp(const CCAmpSet& s, const double* t1, const double* t2, double* tau, double* taut, double* Q,
               cudaStream_t st);
int run_dot(const double* x, const double* y, int64_t n, double scale, double* partial, int npartial, double* out,
            cudaStream_t st);

// E = 1/4 sum V * tau appended to the device history hist[*count++] (fixed
// summation order, so repeated runs give identical energies).
// out[i] = a[i] * b[i] over n elements.
int run_mul(const double* a, const double* b, double* out, int64_t n, cudaStream_t st);
int run_energy(const double* V, const double* tau, int64_t n, double* partial, int npartial, double* hist, int* count,
               int cap, cudaStream_t st);

// Host restatement of the synthetic system's generator (shared with tests via
// gbx_cc_get_orbitals).
uint64_t cc_mix64(uint64_t z);
struct CCStream {
  uint64_t state;
  CCStream(uint64_t seed, int k);
  uint64_t next();
  double uniform();
};

}  // namespace gbx
