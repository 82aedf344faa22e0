/*
 * gbx.h -- C ABI of the GB300-native node-local contraction path for DTCF.
 *
 * Every entry point takes plain pointers and sizes.  Device pointers are
 * prefixed d_; streams are cudaStream_t passed as void*.  Each call returns an
 * int status (GBX_OK or a negative GBX_E* code, with a message from
 * gbx_last_error()); none aborts and no C++ exception crosses the ABI.
 * Plans are immutable after creation; distinct plans may be used from
 * different host threads.
 *
 * Reference interfaces replaced (paths relative to the DTCF source tree) are
 * cited beside each declaration.
 */
#ifndef GBX_H
#define GBX_H
#include <stdint.h>

#if defined(__GNUC__)
#define GBX_API __attribute__((visibility("default")))
#else
#define GBX_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define GBX_OK 0
#define GBX_EINVAL (-1)       /* bad argument or descriptor */
#define GBX_ENOMEM (-2)       /* device or host allocation failed / over budget */
#define GBX_ECUDA (-3)        /* a CUDA call failed */
#define GBX_ETIMEOUT (-4)     /* a bounded device wait ran out; the context stays usable */
#define GBX_EUNSUPPORTED (-5) /* shape or mode not supported by this build */

/* Message of the last failed call on this host thread ("" if none). */
GBX_API const char* gbx_last_error(void);
/* Library version string. */
GBX_API const char* gbx_version(void);

/* ---- leaf entry points ------------------------------------------------- */

/* Permute one dense row-major block: source dimension i lands at output
 * position perm[i]; widths[] are the source extents.  Bit-exact (pure moves).
 * Replaces: void transpose(double*&, double*&, int*, int, int*)
 *           helper.h:105 (helper.cc:275-522).  dims in [1, 8]. */
GBX_API int gbx_transpose(const double* d_in, double* d_out, const int* perm, int dims, const int* widths,
                  void* stream);

/* Permute num_blocks dense blocks of identical extents, block b read from
 * d_in + b*block_size and written to d_out + b*block_size, each with its own
 * permutation perms[b*dims .. b*dims+dims-1] (host array).  The per-block loop
 * of Contraction::transpose_and_dgemm (contraction.cc:1824-1914) and the C
 * pre/post permute of contract() (contraction.cc:2693-2716, 2818-2830). */
GBX_API int gbx_transpose_blocks(const double* d_in, double* d_out, int num_blocks, const int* perms, int dims,
                         const int* widths, void* stream);

/* DLTC transpose: reorder block x (index names ids_x, extents wb_x) into the
 * index order ids_y.  Identity permutations copy.
 * Replaces: void DLTC::transpose(double*, const vector<IndexName>&, double*,
 *           const vector<IndexName>&)  DLTC/transp.h:19 (DLTC/transp.cc:3-59)
 *           and transpose_xxxx  DLTC/transp-kernel.h:4-29. */
GBX_API int gbx_dltc_transpose(const double* d_x, const int* ids_x, double* d_y, const int* ids_y, int dim,
                       const int* wb_x, void* stream);

/* C[n_a x n_b] += alpha * op(A) * op(B), row-major, beta = 1.
 * at = 0: A is n_a x n_k, at = 1: A is n_k x n_a; bt = 0: B is n_k x n_b,
 * bt = 1: B is n_b x n_k.  FP64 arithmetic on the FP64 tensor pipe.
 * Replaces: void local_contraction(int,int,int,double*,double*,double*,int,int,double)
 *           localcontract.h:13 (localcontract.cc:3-20), with the leading
 *           dimension of a transposed operand corrected (the reference passes
 *           n_b, right only when n_b == n_k). */
GBX_API int gbx_local_contraction(int n_a, int n_b, int n_k, const double* d_A, const double* d_B, double* d_C,
                          int at, int bt, double alpha, void* stream);

/* The same product as gbx_local_contraction, for callers that cannot let a
 * library allocate device memory: a framework that has handed nearly all of
 * the GPU's memory to its own caching pool, or a latency-bound loop whose
 * other streams must not be stalled by the device synchronisation of
 * cudaFree.  This entry point calls no cudaMalloc, cudaMallocAsync, cudaFree
 * or allocating library routine.  Its descriptor and split-K partial sums
 * live in one fixed device array of 32 MiB + 4 KiB that the library defines
 * and every GPU that loads the library holds until the process exits.
 * Outputs larger than 4,194,304 elements (n_a * n_b) are rejected with
 * GBX_EINVAL.  The first call on a device looks up that array's device
 * address (cudaGetSymbolAddress); make it before any stream capture.  All
 * calls share the array: calls whose work overlaps on the GPU (different
 * streams, or different host threads without ordering) race and give wrong
 * results.
 * No counterpart in the reference. */
GBX_API int gbx_local_contraction_noalloc(int n_a, int n_b, int n_k, const double* d_A, const double* d_B,
                                          double* d_C, int at, int bt, double alpha, void* stream);

/* DLTC tile product c[m x n] += a[m x k] * b[k x n], row-major.
 * Replaces: void DLTC::compute(double*, double*, double*, Multiplication&)
 *           DLTC/compute.h:28 (DLTC/compute.cc:3-36). */
GBX_API int gbx_dltc_compute(double* d_c, const double* d_a, const double* d_b, int m, int n, int k, void* stream);

/* Place num_tiles permuted tiles (row_per_block x col_per_block each, tile t
 * at d_tiles + t*row_per_block*col_per_block) into one row-major matrix,
 * rows ordered by the tiles' leading num_row_dim permuted block coordinates
 * and columns by the rest, as std::map orders them.  permuted_address (host,
 * dims ints per tile), vgrid and p_map describe the block grid.  *nrows /
 * *ncols receive the block counts.  Returns GBX_EINVAL when the tile pattern
 * is not rectangular (the reference asserts).
 * Replaces: create_big_matrix(Tensor*&, double*&, int*&, int*&, int, int, int,
 *           int, map<int,map<int,int>>*&, double*&)  transpose_helper.h:30
 *           (transpose_helper.cc:20-171); d_big is caller-owned instead of new[]. */
GBX_API int gbx_create_big_matrix(int dims, const int* vgrid, const int* p_map, int num_tiles, const double* d_tiles,
                          const int* permuted_address, int row_per_block, int col_per_block, int num_row_dim,
                          double* d_big, int* nrows, int* ncols, void* stream);

/* The same placement with the tile data looked up by address: entry t of
 * permuted_address takes its data from tile slot address_to_location[rank]
 * of d_tiles (which holds num_slots tiles), rank = the block rank of the
 * entry's permuted address in the permuted grid (grid[p_map[d]] = vgrid[d]).
 * The map is passed as num_locations (loc_ranks[i] -> loc_slots[i]) pairs;
 * a placed tile without a location, or a slot outside [0, num_slots), is
 * GBX_EINVAL (the reference asserts).
 * Replaces: create_big_matrix_nl(Tensor*&, double*&, int*&, int*&, int, int,
 *           int, int, map<int,map<int,int>>*&, double*&, map<int,int>*&)
 *           transpose_helper.h:35 (transpose_helper.cc:184-328), as called by
 *           Contraction::contract, contraction.cc:2399-2410. */
GBX_API int gbx_create_big_matrix_nl(int dims, const int* vgrid, const int* p_map, int num_tiles,
                                     const double* d_tiles, int num_slots, const int* permuted_address,
                                     int row_per_block, int col_per_block, int num_row_dim, const int* loc_ranks,
                                     const int* loc_slots, int num_locations, double* d_big, int* nrows, int* ncols,
                                     void* stream);

/* The inverse placement.
 * Replaces: revert_big_matrix(...)  transpose_helper.h:43 (transpose_helper.cc:331-409). */
GBX_API int gbx_revert_big_matrix(int dims, const int* vgrid, const int* p_map, int num_tiles,
                          const int* permuted_address, int row_per_block, int col_per_block, int num_row_dim,
                          const double* d_big, double* d_tiles, void* stream);

/* ---- contraction plans -------------------------------------------------- */

/* One RRR tensor as it is stored on one process: num_tiles tiles, each a
 * dense row-major block of block_range[] extents, tile t at element offset
 * t*prod(block_range) of the device buffer, with its block address in
 * tile_address[t*dims .. t*dims+dims-1] (host).  sym[] is the RRR symmetry
 * string (tensor.cc:95-170): 'a'/'A' group 0, 'b'/'B' group 1, 'c','C','d','D'
 * none.  Mirrors RRR::Tensor (tensor.h:40-120). */
typedef struct {
    int dims;
    const char* sym;
    const int* block_range;
    const int* vgrid;
    int num_tiles;
    const int* tile_address;
} gbx_tensor_desc;

/* RRR tensor initialization on one process, on the device.
 *
 * The unique tiles of a tensor with this symmetry string ('a'/'A' and
 * 'b'/'B' mark the two symmetry groups, any other letter a free index) and
 * block grid, in the order RRR generates them: lexicographic, kept when the
 * coordinates do not increase inside a group.  d_tile_address (device, dims
 * ints per tile, room for capacity tiles) receives them; *num_tiles their
 * count (the call waits for the stream).  capacity 0 counts only;
 * GBX_EINVAL when more tiles exist than capacity.
 * Replaces: the addresses of Tensor::initialize (tensor.cc:315-335) --
 *           generate_data / isValid / get_bound, tensor.cc:617-694. */
GBX_API int gbx_rrr_unique_tiles(int dims, const char* sym, const int* vgrid, int* d_tile_address, int capacity,
                                 int* num_tiles, void* stream);
/* Every element of tile t (block_size elements at d_tiles + t * block_size)
 * set to the reference's value of its address, sum over d from dims - 1 down
 * to 0 of sin(address_d), bit for bit.  d_tile_address on the device.
 * Replaces: the values of Tensor::initialize / generate_data
 *           (tensor.cc:674-681) and Tensor::get_value (tensor.cc:744-758). */
GBX_API int gbx_rrr_initialize(int dims, const int* vgrid, const int* d_tile_address, int num_tiles,
                               int64_t block_size, double* d_tiles, void* stream);

typedef struct gbx_plan gbx_plan;

#define GBX_MODE_FP64 0  /* FP64 GEMM on the FP64 tensor pipe */
#define GBX_MODE_SPLIT 1 /* FP64 split into exact integer bf16 slices on tcgen05 */

/* Plan C[idxC] += alpha * sum A[idxA] * B[idxB] over the contracted index
 * names (those in both idxA and idxB), index strings as in
 * Contraction::contract("a,b,k,l","m,n,k,l","a,b,m,n") (contraction.h:262).
 * Tiles missing from A or B because only unique blocks are stored are
 * recovered from the stored block with the symmetric permutation
 * (get_symm_permutation, contraction.cc:132-160) times sign^(number of swaps);
 * sign = +1 reproduces the reference, -1 makes the groups antisymmetric.
 * Only C's stored tiles are updated. */
GBX_API int gbx_plan_create(const gbx_tensor_desc* A, const gbx_tensor_desc* B, const gbx_tensor_desc* C,
                    const char* idxA, const char* idxB, const char* idxC, int mode, int sign, int slices,
                    gbx_plan** plan);
/* Execute: d_A, d_B, d_C hold the tiles in descriptor order.
 * Replaces the leaf work of Contraction::contract for one process:
 * transpose_and_dgemm (contraction.cc:1779-1976) + kevin_dgemm (1980-2002)
 * + the C permutes and packs (2693-2716, 2768, 2808, 2818-2830). */
GBX_API int gbx_execute(gbx_plan* plan, const double* d_A, const double* d_B, double* d_C, double alpha, void* stream);
/* Algorithmic FP64 flops of one execute: 2 * sum over (A-block, B-block ->
 * C-block) triples of m*n*k. */
GBX_API double gbx_plan_flops(const gbx_plan* plan);
GBX_API int gbx_plan_destroy(gbx_plan* plan);

/* C[M x N] = A[M x K] * B[N x K]^T, row-major FP64, computed with the
 * split-precision engine: each operand row is split into `slices` exact
 * integer bf16 slices (0 = default 6; 2..7), the slice products run on the
 * tcgen05 tensor cores with exact FP32 accumulation chunks and are recombined
 * in FP64.  Relative error about 2^(-8*slices+1) of the row/column scale.
 * Allocates its workspace and waits for the stream (a one-shot call; plans
 * keep the workspace).  The FP64-emulating counterpart of local_contraction
 * (localcontract.cc:3-20) with at=0, bt=1, alpha=1, beta=0. */
GBX_API int gbx_split_gemm(const double* d_A, const double* d_B, double* d_C, int64_t M, int64_t N, int64_t K,
                           int slices, void* stream);

/* Self-test of the bounded device waits of the split engine's kernels: one
 * CTA waits, through the same bounded mbarrier wait as the split GEMM
 * pipelines, on a barrier that nothing arrives on, gives up after
 * limit_cycles SM clocks (0 .. about one second's worth), records the wait's
 * stage (31) in its error word and returns.  The call waits for the stream and
 * returns GBX_ETIMEOUT with the same message as a split GEMM whose wait ran
 * out; the CUDA context stays usable.  No counterpart in the reference (its
 * waits are blocking MPI calls). */
GBX_API int gbx_wait_selftest(long long limit_cycles, void* stream);

/* Tuning knob of the split engine: output tile width (32, 64, 128 or 256
 * columns) for plans created after the call; 0 restores the built-in
 * throughput model.  Process-wide; used by the autotuner. */
GBX_API int gbx_split_set_width(int width);

/* ---- grouped block GEMM ------------------------------------------------- */

/* One block triple: C[m x n] (+)= alpha * A[m x k] * B[n x k]^T with element
 * strides: A(i,l) at A[i*a_rs + l*a_cs], B(j,l) at B[j*b_rs + l*b_cs],
 * C(i,j) at C[i*c_rs + j]. */
typedef struct {
    const double* A;
    const double* B;
    double* C;
    int64_t a_rs, a_cs, b_rs, b_cs, c_rs;
    int m, n, k;
    double alpha;
    int accumulate; /* 1: C += ..., 0: C = ... */
} gbx_triple;

/* Run all triples in one persistent launch driven by a device-side work
 * queue of 64x64 output tiles.  triples is a host array; it is uploaded with
 * stream-ordered temporaries.  Triples whose C overlap must not share a call. */
GBX_API int gbx_grouped_gemm_f64(const gbx_triple* triples, int num_triples, void* stream);

/* ---- planned triple groups (engine choice and autotuning) --------------- */

#define GBX_MODE_AUTO 2 /* per triple: FP64 or split, by the throughput model */

typedef struct gbx_group gbx_group;

/* Plan a set of triples once (the per-block-pair dgemm calls of
 * transpose_and_dgemm, contraction.cc:1779-1976, and of DLTC task_mul,
 * DLTC/task.cc:83-137, as one batch).  mode GBX_MODE_FP64 runs every triple
 * on the FP64 pipe (DMMA tile shapes 64x64 / 64x16 / 16x64 / 16x16, thin and
 * small-K kernels), GBX_MODE_SPLIT on the split engine (needs a_cs = b_cs =
 * 1; GBX_EUNSUPPORTED otherwise), GBX_MODE_AUTO picks per triple.  slices:
 * split slices (0 = 6).  The triple array is copied; operand memory must
 * stay valid while the group exists.  Triples whose C overlap must not share
 * a group. */
GBX_API int gbx_group_create(const gbx_triple* triples, int num_triples, int mode, int slices, gbx_group** out);
/* Run every triple: one persistent launch per kernel kind (per_triple = 0;
 * capturable in a CUDA graph, allocates nothing), or one launch per FP64
 * triple (per_triple = 1, the per-dgemm-call baseline; split triples still
 * run batched). */
GBX_API int gbx_group_execute(gbx_group* g, int per_triple, void* stream);
/* Autotuner: triples are classed by shape (log4 bins of m, n, k); for each
 * class every candidate (the four FP64 tile shapes; split output widths 32 to
 * 256 in both orientations, as the mode allows) is timed with CUDA events on
 * scratch outputs (marginal cost of 4 copies over 1, best of reps) and the
 * fastest is kept; the group is then re-planned.  Synchronises the stream;
 * writes no triple's C. */
GBX_API int gbx_group_autotune(gbx_group* g, int reps, void* stream);
/* Per triple: engine (0 FP64, 1 split) and parameter (FP64 tile variant, -1
 * = model; split: 2 * width + swapped); flops = 2 * sum m*n*k.  Any pointer
 * may be NULL. */
GBX_API int gbx_group_info(const gbx_group* g, int* engines, int* params, double* flops);
GBX_API int gbx_group_destroy(gbx_group* g);

#ifdef __cplusplus
}
#endif
#endif /* GBX_H */
