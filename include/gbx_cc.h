/*
 * gbx_cc.h -- C ABI of the coupled-cluster iteration driver and the
 * continuous-batching request loop built on the gbx contraction path.
 *
 * The reference has no CC iteration of its own: its DLTC residual tables
 * (DLTC/ccd-t2.cc:45-95, DLTC/ccsd-t1.cc:40-109, DLTC/ccsd-t2.cc:55-216) are
 * the workload definitions this driver executes, completed with the
 * permutation operators, coefficients and the Jacobi update a converging
 * spin-orbital CCSD needs.  Conventions as in gbx.h: int status, messages via
 * gbx_last_error(), streams as void*.
 */
#ifndef GBX_CC_H
#define GBX_CC_H
#include <stdint.h>

#include "gbx.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GBX_CC_CCD 0
#define GBX_CC_CCSD 1

typedef struct {
    int nocc, nvir;      /* spin orbitals */
    int nirrep;          /* 1, 2, 4 or 8 (XOR product rule) */
    int max_block;       /* an irrep's orbitals are cut into blocks of at most this size */
    int min_block;       /* irrep occupation draws repeat until each irrep has this many */
    int method;          /* GBX_CC_CCD or GBX_CC_CCSD */
    int engine;          /* GBX_MODE_FP64 or GBX_MODE_SPLIT */
    int slices;          /* split engine: bf16 slices per operand (0 = default) */
    int use_graph;       /* 0: launch kernel by kernel; 1: capture one iteration as a CUDA graph of its
                            kernels; 2: run the iteration as a persistent program -- a few persistent
                            launches driven by a device-side work queue (one per dependency level of
                            the memory-bound work, one per GEMM kernel and level) -- captured as the
                            graph; each contraction then keeps its own workspace */
    int split_all;       /* split engine on every GEMM, however small (default: large ones only) */
    uint64_t seed;
    double eps_occ_lo, eps_occ_hi, eps_vir_lo, eps_vir_hi;
    double v_scale, v_decay; /* |<pq||rs>| = v_scale * exp(-(|p-q| + |r-s|) / v_decay) */
    int autotune;        /* time each split contraction's output tile widths when the job is built */
} gbx_cc_config;

typedef struct {
    double flops_per_iter;       /* algorithmic FP64 flops of one iteration (nonzero block triples) */
    double gemm_flops_per_iter;  /* flops the packed GEMMs execute */
    double resident_bytes;       /* device bytes held by the job (tensors + plans) */
    int ncontractions;           /* contraction plans of one iteration */
    int nsums;                   /* fused summation steps of one iteration */
    int nblocks_occ, nblocks_vir;
    int launches_per_iter;       /* kernels of one iteration: the captured graph's kernel nodes once it
                                    exists, the planned count before */
} gbx_cc_stats;

typedef struct gbx_cc_job gbx_cc_job;

/* Fill cfg with the defaults of the synthetic system (seed 1, eps ranges
 * [-2,-0.5] / [0.2,3.0], v_scale 1e-2, v_decay 8, block 16, CCSD, FP64). */
GBX_API void gbx_cc_default_config(gbx_cc_config* cfg);
/* Device bytes a job of this configuration will hold once built
 * (resident_bytes) and at most while it is being built (peak_bytes), and the
 * algorithmic flops of one iteration, from host planning alone: no device
 * memory is touched.  The serving loop admits jobs by resident_bytes.  Any
 * output pointer may be NULL. */
GBX_API int gbx_cc_footprint(const gbx_cc_config* cfg, double* resident_bytes, double* peak_bytes,
                             double* flops_per_iter);
/* Build the job: orbitals, integrals (on the device), plans, MP2 guess. */
GBX_API int gbx_cc_create(const gbx_cc_config* cfg, void* stream, gbx_cc_job** job);
/* Captures one iteration as a CUDA graph now (otherwise the first enqueue
 * does it); a no-op when use_graph is 0 or the graph exists. */
GBX_API int gbx_cc_capture(gbx_cc_job* job);
/* GBX_ETIMEOUT if a bounded device wait of the split engine ran out in any
 * iteration so far (reads the error words; call after the work finished). */
GBX_API int gbx_cc_check(gbx_cc_job* job);
/* Enqueue niter Jacobi iterations on stream without waiting; the energy of
 * each lands in the job's device history. */
GBX_API int gbx_cc_enqueue(gbx_cc_job* job, int niter, void* stream);
/* Run niter iterations and return their correlation energies (host array of
 * niter); waits for the stream. */
GBX_API int gbx_cc_iterate(gbx_cc_job* job, int niter, double* energies, void* stream);
/* Energy history: all energies so far (index 0 = MP2 guess); *count in/out. */
GBX_API int gbx_cc_energies(gbx_cc_job* job, double* energies, int* count);
GBX_API int gbx_cc_stats_get(const gbx_cc_job* job, gbx_cc_stats* out);
/* Orbital irreps and energies in orbital order (nocc + nvir entries each). */
GBX_API int gbx_cc_get_orbitals(const gbx_cc_job* job, int* irrep, double* eps);
/* Dense amplitudes (t1: nocc x nvir, t2: nocc^2 x nvir^2, row-major);
 * either may be NULL.  Waits for the stream. */
GBX_API int gbx_cc_get_amplitudes(gbx_cc_job* job, double* t1, double* t2, void* stream);
/* Shapes (M, N, K triples) of every packed GEMM of one iteration; *count in
 * = capacity of mnk (3 int64 per GEMM), out = number of GEMMs. */
GBX_API int gbx_cc_gemm_shapes(const gbx_cc_job* job, int64_t* mnk, int* count);
/* Element counts of the amplitude tensors in their tile storage. */
GBX_API int gbx_cc_amplitude_elems(const gbx_cc_job* job, int64_t* n1, int64_t* n2);
/* Enqueue host -> device copies of the amplitudes (tile storage order) on
 * stream, and the tau / taut / Q combinations of them; the next iteration
 * starts from them.  Pinned host memory keeps the copies asynchronous. */
GBX_API int gbx_cc_set_amplitudes(gbx_cc_job* job, const double* t1, const double* t2, void* stream);
/* Enqueue device -> host copies of the amplitudes in tile storage order (the
 * layout gbx_cc_set_amplitudes takes back) on stream; either pointer may be
 * NULL.  With set_amplitudes, a job's state can leave the device and come
 * back: the iterations after a restore repeat those of the job that saved. */
GBX_API int gbx_cc_save_amplitudes(gbx_cc_job* job, double* t1, double* t2, void* stream);
/* Enqueue a device -> host copy of the latest energy on stream. */
GBX_API int gbx_cc_read_energy(gbx_cc_job* job, double* energy, void* stream);
/* Run one iteration step by step with CUDA events between the steps and
 * report per step: time (ms), algorithmic flops, bytes, kind (0 contraction,
 * 1 permuted sum, 2 zero, 3 denominator, 4 energy), the contraction index
 * (or -1) and a name of name_len chars.  Counts as one iteration. */
GBX_API int gbx_cc_profile(gbx_cc_job* job, int cap, float* ms, double* flops, double* bytes, int* kind, int* plan,
                           char* names, int name_len, int* count, void* stream);
/* Kernel choice of one contraction's packed GEMMs: the split output tile
 * width (64 with at most 4 slices: the k-stationary kernel; 0: the width
 * model's choice per GEMM), the number of split and FP64 GEMMs (both 0 for a
 * contraction on the direct engine), the slices. */
GBX_API int gbx_cc_plan_info(const gbx_cc_job* job, int contraction, int* split_width, int* n_split, int* n_f64,
                             int* slices);
/* Time only the GEMM launches of one contraction (its operands packed and
 * split again first), reps times, with CUDA events on stream.  Reports
 * ms per run, the FP64 flops of the packed GEMMs, the bf16 tensor flops the
 * split engine issues, and the engine (0 FP64, 1 split, 2 both, 3 direct:
 * the unpacked FP64 kernel of contractions with few products per output
 * element, timed with alpha = 0 so that C keeps its values). */
GBX_API int gbx_cc_time_gemm(gbx_cc_job* job, int contraction, int reps, float* ms, double* fp64_flops,
                             double* tensor_flops, int* engine, void* stream);
/* Error of one contraction of the job's iteration against the plain FP64
 * path: the contraction runs on its current operands (call after at least
 * one iteration, so that the intermediates exist) twice into scratch
 * outputs -- with the job's own plan (e.g. the split engine) and with a
 * plain FP64 plan of the same contraction built for the call -- and
 * rel_frob_err = ||C_job - C_fp64||_F / ||C_fp64||_F, max_abs_err = the
 * largest element difference.  The job's tensors are not changed; the call
 * allocates its scratch and waits for the stream. */
GBX_API int gbx_cc_contraction_error(gbx_cc_job* job, int contraction, double* rel_frob_err, double* max_abs_err,
                                     void* stream);
/* The persistent program of a use_graph 2 job (recorded on first use):
 * records (memory work items, GEMM launches, other launches), dependency
 * levels and launches per iteration.  Zeros for other jobs.
 * Replaces: the exec / Barrier structure of ccd_t2 / ccsd_t1 / ccsd_t2
 * (DLTC/ccd-t2.cc:97-134) -- a task pool per dependency layer, barriers
 * between layers -- with a device-side work queue. */
GBX_API int gbx_cc_program_info(gbx_cc_job* job, int* records, int* levels, int* launches);
/* Self-test of the persistent program's bounded dependency wait: runs a
 * two-record launch whose one wait can never be met, bounded by
 * limit_cycles; returns GBX_ETIMEOUT when the wait ran out as it must (the
 * context stays usable), GBX_OK if it did not. */
GBX_API int gbx_cc_program_selftest(long long limit_cycles, void* stream);
GBX_API int gbx_cc_destroy(gbx_cc_job* job);

#ifdef __cplusplus
}
#endif
#endif /* GBX_CC_H */
