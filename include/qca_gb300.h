/*
 * qca_gb300 — C ABI of the GB300 (sm_103a) time-evolution library for the
 * quantum game of life of BenjaminDecker/quantum-cellular-automaton.
 *
 * Every entry point returns an int status (QCA_OK = 0); the message of the last
 * failure on the calling host thread is returned by qca_last_error().  No entry
 * point traps on the device; numerical failures come back as status codes.
 * Host arrays are plain C arrays; complex numbers are interleaved (re, im)
 * doubles, i.e. the memory layout of numpy complex128 in C order.  `stream` is a
 * cudaStream_t passed as void* (NULL = the legacy default stream).  A handle may
 * be used by one host thread at a time; calls on it are stream ordered.
 *
 * The reference interfaces each entry point replaces are cited as
 * file:line of the reference project.
 */
#ifndef QCA_GB300_H
#define QCA_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------- */
#define QCA_OK 0
#define QCA_ERR_INVALID 1        /* bad argument (reference: assert / ValueError)      */
#define QCA_ERR_CUDA 2           /* CUDA runtime error                                  */
#define QCA_ERR_OOM 3            /* device allocation failed                            */
#define QCA_ERR_BREAKDOWN 4      /* Krylov breakdown that could not be absorbed         */
#define QCA_ERR_NOT_CONVERGED 5  /* Lanczos / Jacobi iteration limit reached            */
#define QCA_ERR_NAN 6            /* non-finite norm detected                            */
#define QCA_ERR_ADMISSION 7      /* device-memory budget would be exceeded              */
#define QCA_ERR_NO_DEVICE 8      /* no CUDA device / sm_103a image not loadable         */

/* ---- precision ------------------------------------------------------------- */
#define QCA_PREC_FP64 0  /* complex128 storage and arithmetic ("plain")                 */
#define QCA_PREC_MIXED 1 /* complex64 storage, fp32 products, fp64 Krylov scalars, SVD
                            singular values, truncation weights and normalisation       */

/* ---- algorithms (parameters/parser.py:75-82) -------------------------------- */
#define QCA_ALGO_1TDVP 1
#define QCA_ALGO_2TDVP 2
#define QCA_ALGO_A1TDVP 3 /* 1TDVP whose target bond dimensions are recomputed before every
                             step from 2-site splits (tdvp.py:212-267) */

const char* qca_last_error(void);
int qca_version(void);
/* Number of CUDA devices the library can run on (0 when none). */
int qca_device_count(int* count);

/* =============================================================================
 * Exact state-vector evolution.
 * Replaces algorithms/exact.py:9-28 (Exact.__init__, Exact.do_time_step,
 * the psi property) and the dense propagator lautils/lautils.py:44-54.
 * The Hamiltonian H = sum_i X_i Pi_i of parameters/rules.py is applied matrix
 * free: cell i flips iff the number of alive cells j != i with |i-j| <= distance
 * lies in [interval_lo, interval_hi) (upper bound excluded, as the Python range
 * of parameters/parser.py:182).  Cell 0 is the most significant bit of the
 * amplitude index (tensor_networks/mps.py:194-208).  One step applies
 * exp(-i pi/2 step_size H) by Lanczos with `krylov_dim` vectors resident on the
 * device, split into sub-steps when step_size * ||H|| is large.
 * ============================================================================= */
typedef struct qca_exact qca_exact;

/* Exact.__init__ (exact.py:15-17).  precision: QCA_PREC_FP64 or QCA_PREC_MIXED. */
int qca_exact_create(int n_cells, int distance, int interval_lo, int interval_hi, int precision,
                     int krylov_dim, qca_exact** out);
int qca_exact_destroy(qca_exact* h);
/* psi setter (exact.py:23-25): 2^n complex128 amplitudes from HOST memory. */
int qca_exact_set_state(qca_exact* h, const double* psi, void* stream);
/* psi setter from DEVICE memory (complex128 for FP64, complex64 for MIXED). */
int qca_exact_set_state_device(qca_exact* h, const void* psi_dev, void* stream);
/* psi getter (exact.py:19-21): 2^n complex128 amplitudes into HOST memory. */
int qca_exact_get_state(qca_exact* h, double* psi, void* stream);
/* Device pointer of the resident state (complex128 or complex64 by precision). */
int qca_exact_state_device(qca_exact* h, void** psi_dev);
/* do_time_step (exact.py:27-28) repeated nsteps times with step size dt. */
int qca_exact_step(qca_exact* h, double step_size, int nsteps, void* stream);
/* <n_i> and the 2x2 single-site density matrices rho_i (4 complex128 per cell,
 * row major) of the current state; either output may be NULL.  The reference
 * measures through MPS.from_vector (mps.py:54-73) and MPS.measure (mps.py:100-140). */
int qca_exact_measure(qca_exact* h, double* population, double* rho, void* stream);
/* Bytes of device memory the handle holds. */
int qca_exact_footprint(int n_cells, int precision, int krylov_dim, size_t* bytes);

/* Allocation-free exact step.  No counterpart in the reference: it exists for
 * callers that may not allocate device memory (applications whose device memory
 * is owned by their own pool or budget manager, and latency-critical loops that
 * cannot take the implicit synchronisation of cudaMalloc / cudaFree).
 * Evolves the caller's 2^n_cells complex128 amplitudes (DEVICE memory, psi_in and
 * psi_out may be the same buffer) by nsteps steps of exp(-i pi/2 step_size H) with
 * the kernels of qca_exact_step, in FP64.  Its scratch (Krylov basis, H v buffer,
 * Lanczos scalars) is one file-scope device array of 16 MiB that every GPU loading
 * the library holds until the process exits; it allocates nothing and calls no
 * allocating routine.  Limit: (krylov_dim + 1) * 2^n_cells * 16 bytes plus a few
 * KB must fit in 16 MiB (e.g. n_cells <= 15 at krylov_dim 30, <= 14 at 60); larger
 * requests return QCA_ERR_INVALID.  The first call on a device resolves the
 * array's device address on that device (make it before any stream capture).
 * Every call shares the array: calls that overlap on the GPU (other streams,
 * other host threads) race and must be serialised by the caller. */
int qca_exact_step_noalloc(int n_cells, int distance, int interval_lo, int interval_hi, int krylov_dim,
                           double step_size, int nsteps, const void* psi_in, void* psi_out, void* stream);

/* =============================================================================
 * TDVP engine: many MPS chains evolved side by side on one device.
 * Replaces algorithms/tdvp.py:10-365 (TDVP.__init__, do_time_step, the 1-site
 * and 2-site sweeps, _evolve_split_and_truncate, _evolve_site, _evolve_bond,
 * the environment updates) with the local exponential of lautils.py:57-81
 * computed by Lanczos, and MPS.measure (mps.py:100-140).
 * ============================================================================= */
typedef struct qca_engine qca_engine;

typedef struct qca_chain_desc {
  int n_sites;             /* N >= 2                                                   */
  const int* mpo_bonds;    /* N+1 MPO bond dimensions w_0..w_N (w_0 = w_N = 1)           */
  const double* mpo;       /* W[0..N-1] concatenated; W[i] is (2,2,w_i,w_{i+1}) complex128
                              in C order (tensor_networks/mpo.py:158-200)               */
  const int* mps_bonds;    /* N+1 MPS bond dimensions D_0..D_N (D_0 = D_N = 1)           */
  const double* mps;       /* A[0..N-1] concatenated; A[i] is (2,D_i,D_{i+1}) complex128
                              (tensor_networks/mps.py:14-25)                            */
  int algorithm;           /* QCA_ALGO_1TDVP, QCA_ALGO_2TDVP or QCA_ALGO_A1TDVP (tdvp.py:55-63) */
  int max_bond_dim;        /* --max-bond-dim (parameters/parser.py:106-113)             */
  double svd_epsilon;      /* --svd-epsilon (parameters/parser.py:114-122)              */
  double step_size;        /* dt; the local propagator is exp(-i pi/2 dt/2 H_eff)        */
} qca_chain_desc;

/* Create an engine on the current device.  hbm_budget_bytes bounds the device memory
 * all its chains may hold (0 = 90% of the free memory at creation). */
int qca_engine_create(int precision, size_t hbm_budget_bytes, qca_engine** out);
int qca_engine_destroy(qca_engine* e);
/* Device bytes a chain of this description would hold (admission estimate). */
int qca_chain_footprint(const qca_chain_desc* d, int precision, size_t* bytes);
/* TDVP.__init__ (tdvp.py:12-40): upload now; canonicalisation and the right
 * environments run at the next step/measure/get_mps call, grouped over every chain
 * added before it (one launch per sweep position for all of them).
 * Returns QCA_ERR_ADMISSION when the budget would be exceeded. */
int qca_chain_add(qca_engine* e, const qca_chain_desc* d, void* stream, int* chain_id);
int qca_chain_remove(qca_engine* e, int chain_id);
/* TDVP.do_time_step (tdvp.py:50-63) nsteps times for every chain of the engine.
 * A chain that fails numerically does not stop the others: they complete their
 * steps and the call returns the failure (QCA_ERR_NAN before
 * QCA_ERR_NOT_CONVERGED) naming the first failed chain. */
int qca_engine_step(qca_engine* e, int nsteps, void* stream);
/* do_time_step nsteps times for the listed chains only (the others keep their state). */
int qca_engine_step_chains(qca_engine* e, const int* chain_ids, int count, int nsteps, void* stream);
/* Continuous batching (no counterpart in the reference, which evolves one state at
 * a time): qca_chain_schedule adds nsteps time steps to a chain's budget, and
 * qca_engine_advance runs at most max_ticks lock-step ticks over the listed chains
 * (all chains when count = 0), one local update of every chain inside a time step
 * per tick; a chain that completes a step begins its next scheduled one at the
 * following tick, so chains of different length and bond dimension progress
 * independently and new chains join at any tick.  A call may stop inside a time
 * step; measurements and qca_chain_get_mps need the chain at a step boundary.
 * Chains that fail (QCA_ERR_NAN / QCA_ERR_NOT_CONVERGED, named in the message) are
 * skipped by later calls and stay failed until removed.  qca_chain_progress
 * writes 4 values: [0] time steps completed since the chain was added, [1] steps
 * scheduled and not completed, [2] 1 while inside a step, [3] failure status. */
int qca_chain_schedule(qca_engine* e, int chain_id, int nsteps);
int qca_engine_advance(qca_engine* e, const int* chain_ids, int count, int max_ticks, void* stream);
int qca_chain_progress(qca_engine* e, int chain_id, long long* progress);
/* Algorithm.measure (algorithm.py:58-63 -> mps.py:100-140).  1TDVP chains: mutates
 * the gauge of the stored MPS exactly like the reference.  2TDVP chains whose
 * orthogonality centre is at site 0 (the state after every step): the same left QR
 * sweep runs on scratch copies, which gives the same values without touching the
 * tensors (the result does not depend on the gauge).  Outputs: population[N],
 * d_population[N], single_site_entropy[N], bond_dims[N+1] (any may be NULL). */
int qca_chain_measure(qca_engine* e, int chain_id, double* population, double* d_population,
                      double* single_site_entropy, double* bond_dims, void* stream);
/* Algorithm.measure for `count` chains at once (their QR sweeps run in lock step);
 * the outputs are concatenated over the chains in the given order: N_c values per
 * chain (N_c + 1 for bond_dims).  Gauges as in qca_chain_measure. */
int qca_engine_measure(qca_engine* e, const int* chain_ids, int count, double* population, double* d_population,
                       double* single_site_entropy, double* bond_dims, void* stream);
/* Current MPS bond dimensions D_0..D_N. */
int qca_chain_bonds(qca_engine* e, int chain_id, int* bonds);
/* psi getter (tdvp.py:42-44): the MPS tensors into host memory, concatenated like
 * qca_chain_desc.mps; `capacity` is the number of doubles available. */
int qca_chain_get_mps(qca_engine* e, int chain_id, double* mps, size_t capacity, void* stream);
/* Statistics of the last step of a chain: [0] largest Lanczos dimension used,
 * [1] summed discarded weight (sum of squared truncated singular values). */
int qca_chain_stats(qca_engine* e, int chain_id, double* stats);
/* The first `count` (at most 5) statistics of a chain: [0] and [1] as
 * qca_chain_stats, [2] the most Jacobi sweeps one two-site split of the last step
 * needed, [3] the chain's failure status (0, or the QCA_ERR_* code of the step in
 * which it failed), [4] the device bytes the chain holds.  No counterpart in the
 * reference (whose LAPACK calls report nothing of the kind). */
int qca_chain_stats_ex(qca_engine* e, int chain_id, double* stats, int count);

/* Profiling hook (no counterpart in the reference, which has no tracing): when
 * enabled, every grouped launch is bracketed by CUDA events on its stream.
 * qca_engine_kernel_stats writes 7 kernel classes x 4 values
 * (kernels launched, milliseconds, algorithmic real flops, algorithmic bytes); classes:
 * 0 GEMM contractions, 1 sparse MPO application, 2 Lanczos vector kernels,
 * 3 Lanczos tridiagonal exponential, 4 SVD, 5 QR, 6 other. */
int qca_engine_profile(qca_engine* e, int enable);
int qca_engine_kernel_stats(qca_engine* e, double* out, int reset);

/* Test hook (no counterpart in the reference): C = A B for row-major complex64
 * DEVICE matrices (M x K, K x N, M x N) through the contraction kernels of the
 * mixed path; tensor_cores = 2 selects the 3xTF32 tcgen05 kernel, 1 the 3xTF32
 * mma.sync kernel, 0 the CUDA-core kernel.  Synchronises the stream. */
int qca_test_gemm_c64(int M, int N, int K, const void* A, const void* B, void* C, int tensor_cores, void* stream);
/* Test hook (no counterpart in the reference): the two-site split of 2TDVP alone
 * (tdvp.py:286-296) on DEVICE arrays of the precision's complex type: theta (4, Dl,
 * Dr) -> Al (2, Dl, k) = U and Ar (2, k, Dr) = s Vh / ||s|| with the truncation rule
 * (eps, chi), sv (FP64, min(2 Dl, 2 Dr) values, descending), *k_out = k.  The
 * output arrays need room for k = min(2 Dl, 2 Dr).  Synchronises the stream. */
int qca_test_svd(int precision, int Dl, int Dr, const void* theta, int chi, double eps, void* Al, void* Ar,
                 double* sv, int* k_out, void* stream);
/* Test hook (no counterpart in the reference): qca_test_svd with the Jacobi sweep
 * limit lowered to max_sweeps (0 = the default of 24), so that the
 * QCA_ERR_NOT_CONVERGED path can be exercised on a well-posed problem.  Returns
 * QCA_ERR_NOT_CONVERGED when the sweeps ran out and QCA_ERR_NAN for non-finite
 * input; the outputs are written in either case. */
int qca_test_svd_sweeps(int precision, int Dl, int Dr, const void* theta, int chi, double eps, int max_sweeps,
                        void* Al, void* Ar, double* sv, int* k_out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* QCA_GB300_H */
