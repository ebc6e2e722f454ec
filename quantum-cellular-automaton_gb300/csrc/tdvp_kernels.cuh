// Descriptors and launchers of the TDVP kernels.  Every kernel is "grouped": one
// launch serves a list of independent problems (one per chain in a tick), each
// with its own shapes, so that many chains of different length, bond dimension
// and rule share every launch.
#pragma once

#include "common.cuh"

namespace qca {

// ----------------------------------------------------------------------------------
// complex GEMM:  C[b1,b2](m,n) (+)= sum_g sum_k op(A)[b1,b2,g](m,k) op(B)[b1,b2,g](k,n)
// with arbitrary element strides (transposes are strides) and optional conjugation.
// ----------------------------------------------------------------------------------
template <typename T>
struct GemmDesc {
  const cplx<T>* A;
  const cplx<T>* B;
  cplx<T>* C;
  int M, N, K, G;
  int nb1, nb2;
  long long sAm, sAk, sAg, sAb1, sAb2;
  long long sBk, sBn, sBg, sBb1, sBb2;
  long long sCm, sCn, sCb1, sCb2;
  int conjA, conjB, accumulate;
  int tiles_m, tiles_n;
  int tile_begin;   // first linear tile of this problem in the launch
  const int* skip;  // when non-null and *skip != 0 the problem is skipped
};

template <typename T>
int launch_gemm(const GemmDesc<T>* d_desc, const GemmDesc<T>* h_desc, int ndesc, int tile_cfg, cudaStream_t st);

// 3xTF32 tensor-core variant (complex64 operands, 64 x 64 tiles).
int launch_gemm_tc(const GemmDesc<float>* d_desc, const GemmDesc<float>* h_desc, int ndesc, cudaStream_t st);

// 3xTF32 on the fifth-generation tensor cores (tcgen05.mma, TMEM accumulators),
// complex64 operands, 128 x 64 tiles; for problems with M >= kUmmaMinM and N, K >=
// kUmmaMinNK.  Its cost is set by the operand staging, not the MMAs, so it beats
// the mma.sync kernel even on half-empty tiles (measured on the batched workload:
// thresholds 48 / 32 give +9% over 96 / 64); the smallest problems stay on mma.sync,
// whose per-k8 FP32 accumulation 1TDVP's rank-deficient QRs prefer.
constexpr int kUmmaBM = 128, kUmmaBN = 64, kUmmaMinM = 48, kUmmaMinNK = 32;
int launch_gemm_umma(const GemmDesc<float>* d_desc, const GemmDesc<float>* h_desc, int ndesc, cudaStream_t st);
// number of tensor-core GEMM mbarrier waits that ran out since the last reset (read
// in order on stream st)
int gemm_umma_timeouts(int reset, int* count, cudaStream_t st);

// Tile configuration for a set of problems (0: 16x16, 1: 32x32, 2: 64x64).
int gemm_tile_cfg(int maxM, int maxN);
int gemm_tile_dim(int cfg);

// ----------------------------------------------------------------------------------
// sparse MPO application: out[ob] = sum_{entries e with out block ob} w_e in[ib_e]
// where blocks are contiguous runs of `blk` elements.
// ----------------------------------------------------------------------------------
struct WEntry {
  int in_block;
  int out_block;
  double re, im;
};

template <typename T>
struct WapplyDesc {
  const WEntry* ent;     // sorted by out_block
  const int* out_begin;  // nout + 1 offsets into ent
  int nout;
  long long blk;
  const cplx<T>* in;
  cplx<T>* out;
  int chunks;      // ceil(blk / chunk)
  int tile_begin;  // first CTA of this problem
  const int* skip;
};

template <typename T>
int launch_wapply(const WapplyDesc<T>* d_desc, const WapplyDesc<T>* h_desc, int ndesc, cudaStream_t st);

// ----------------------------------------------------------------------------------
// Lanczos for v <- exp(-i tau H_eff) v with full (twice) reorthogonalisation.
// The basis lives in `V` (slot stride `ld`), scalars in `S` (see lanczos.cu).
// ----------------------------------------------------------------------------------
template <typename T>
struct LanczosDesc {
  cplx<T>* V;        // basis: slot k at V + k * ld
  long long n;       // vector length
  long long ld;      // slot stride (elements)
  double* S;         // scalar block of this problem
  double tau;        // pi/2 * step
  int chunks;        // vector chunks (CTAs) of this problem
  int tile_begin;    // first CTA
  cplx<T>* out;      // destination of the evolved vector (may alias `in`)
  const cplx<T>* in; // source vector (copied + normalised into slot 0)
  double* P;         // partial sums: 2 buffers x chunks x (2 kLzMax + 2)
  int* done_out;     // copy of the done flag for the host
  int* status;       // sticky failure bits of the owning chain (kLzStatus*), may be null
};

// failure bits a Lanczos exponential ORs into LanczosDesc::status
constexpr int kLzStatusNonFinite = 1;  // non-finite norm or Krylov matrix
constexpr int kLzStatusLimit = 2;      // iteration limit reached before the tolerance

constexpr int kLzMax = 48;        // largest Krylov dimension
constexpr int kLzChunk = 2048;    // elements per CTA in the vector kernels

// scalar block layout
enum : int {
  LZ_DONE = 0,     // 1 when converged / exhausted
  LZ_M = 1,        // current number of basis vectors
  LZ_NORM0 = 2,    // ||input||
  LZ_INVB = 3,     // 1 / ||w|| of the last orthogonalisation
  LZ_MEFF = 4,     // final dimension
  LZ_FLAG = 5,     // status bits (1: non-finite)
  LZ_TOL = 6,      // absolute tolerance on the error estimate
  LZ_ALPHA = 16,               // alpha_k
  LZ_BETA = 16 + kLzMax,       // beta_k = ||w_k||
  LZ_H = 16 + 2 * kLzMax,      // projections of the current w (2 * kLzMax)
  LZ_COEF = 16 + 4 * kLzMax,   // combination coefficients (2 * kLzMax)
  LZ_PART = 16 + 6 * kLzMax    // per-chunk partial norms of the input
};
constexpr int kLzPartStride = 2 * kLzMax + 2;
inline long long lz_scal_size(int max_chunks) { return LZ_PART + max_chunks + 8; }
inline long long lz_part_size(int max_chunks) { return 2LL * max_chunks * kLzPartStride; }

template <typename T>
int launch_lz_init(const LanczosDesc<T>* d, const LanczosDesc<T>* h, int nd, int mmax, double tol, cudaStream_t st);
template <typename T>
int launch_lz_orth_pass(const LanczosDesc<T>* d, const LanczosDesc<T>* h, int nd, int j, int pass, cudaStream_t st);
template <typename T>
int launch_lz_finalize_j(const LanczosDesc<T>* d, int nd, int j, int mmax, int check, cudaStream_t st);
template <typename T>
int launch_lz_normalize(const LanczosDesc<T>* d, const LanczosDesc<T>* h, int nd, int j, cudaStream_t st);
template <typename T>
int launch_lz_combine(const LanczosDesc<T>* d, const LanczosDesc<T>* h, int nd, cudaStream_t st);

// ----------------------------------------------------------------------------------
// SVD of the two-site matrix by one-sided Jacobi + truncation (tdvp.py:286-296)
// ----------------------------------------------------------------------------------
// The split is preconditioned by a Householder QR (launch_qr, run first): the
// matrix W = Theta^H (right sweep) or Theta (left sweep), p x q with
// Theta[(s1,a),(s2,c)] = theta[s1*2+s2][a][c], is factored W = Q R (Q p x K, K =
// min(p, q)), and one-sided Jacobi runs on X = R^H (q x K), whose columns are
// graded and nearly orthogonal, so the sweeps converge in a few rounds instead of
// the dozens the raw, strongly graded two-site matrix needs.  With X (rotated)
// orthogonal: W^H = U Sigma (Q V)^H with U = X / Sigma, so the factor the sweep
// needs isometric (A_l on a right sweep, A_r on a left one) is U, whose
// orthogonality the Jacobi tolerance enforces directly, and the other factor is
// W U: Q and the rotations V are never formed.
template <typename T>
struct SvdDesc {
  const cplx<T>* theta;  // theta[s][a][c], s = s1*2+s2, dims (4, Dl, Dr)
  int Dl, Dr;
  int chi;               // bond cap (max_bond_dim)
  int kmax;              // capacity of the output bond (never exceeded by the rule)
  double eps;            // svd_epsilon
  int right_sweep;       // 1: A_l = U, A_r = s Vh ; 0: A_l = U s, A_r = Vh
  cplx<T>* Al;           // out (2, Dl, k)
  cplx<T>* Ar;           // out (2, k, Dr)
  const cplx<T>* rmat;   // R of W = Q R, row major K x q (q = 2 Dl right, 2 Dr left)
  double* sv;            // singular values (n_x), FP64
  int* k_out;            // new bond dimension
  double* discarded;     // discarded weight accumulator (+= sum of dropped s^2 / sum s^2)
  int* status;           // [0]: 0 ok / QCA_ERR_NOT_CONVERGED / QCA_ERR_NAN, [1]: Jacobi sweeps used
  int max_sweeps;        // Jacobi sweep limit (0: the default, 24)
};

template <typename T>
int launch_svd(const SvdDesc<T>* d, const SvdDesc<T>* h, int nd, cudaStream_t st);
// thread-block cluster size the SVD of one (2 Dl) x (2 Dr) problem needs (0: too large)
template <typename T>
int svd_cluster_size(int Dl, int Dr, int right_sweep);

// ----------------------------------------------------------------------------------
// Householder QR with LAPACK's reflector convention (zgeqrf + zungqr):
// beta = -sign(Re alpha) ||x||, tau = (beta - alpha) / beta, v = x / (alpha - beta).
// The input matrix element (r, c) is at in[r * sIr + c * sIc].
// ----------------------------------------------------------------------------------
template <typename T>
struct QrDesc {
  // row r of the input / of Q splits as r = r1 * rsplit + r0; column c of the input
  // as c = c1 * csplit + c0 (csplit 0: no split), element at
  // in[r1 sIr1 + r0 sIr0 + c1 sIc1 + c0 sIc], conjugated when conj_in
  const cplx<T>* in;
  int rsplit;
  long long sIr0, sIr1, sIc;
  int csplit;
  long long sIc1;
  int conj_in;
  int m, n;
  int complete;          // 1: Q is m x m, R is m x n; 0: Q is m x K, R is K x n (K = min(m,n))
  cplx<T>* work;         // m*n (factored matrix) + m*m (Q)
  cplx<T>* tau;          // K reflector scalars
  // outputs written through strides: Q(r, c) -> q[r*sQr + c*sQc] for c < qcols,
  // zero padded to qcols_out columns; R(r, c) -> rr[r*sRr + c*sRc] for r < rrows_out,
  // c < rcols_out, zero padded.
  cplx<T>* q;
  int qsplit;
  long long sQr0, sQr1, sQc;
  int qrows_out, qcols_out;
  cplx<T>* rr;
  long long sRr, sRc;
  int rrows_out, rcols_out;
};

template <typename T>
// gauge != 0: a gauge move of the mixed path (FP32 sums); 0: FP64 sums
int launch_qr(const QrDesc<T>* d, int nd, int gauge, cudaStream_t st);

// The QR that preconditions a two-site split (see SvdDesc): W = Theta^H (right
// sweep, p = 2 Dr, q = 2 Dl) or Theta (left sweep, p = 2 Dl, q = 2 Dr) read
// straight from theta[s1*2+s2][a][c]; R into r_out (row major K x q); Q is not
// formed.  work needs p q + p K elements, tau K.
template <typename T>
QrDesc<T> split_qr_desc(const cplx<T>* theta, int Dl, int Dr, int right_sweep, cplx<T>* work, cplx<T>* tau,
                        cplx<T>* r_out) {
  QrDesc<T> d;
  memset(&d, 0, sizeof(d));
  const long long blk = (long long)Dl * Dr;
  const int p = right_sweep ? 2 * Dr : 2 * Dl, q = right_sweep ? 2 * Dl : 2 * Dr, K = p < q ? p : q;
  d.in = theta;
  if (!right_sweep) {  // W = Theta: rows (s1, a), columns (s2, c)
    d.rsplit = Dl;
    d.sIr1 = 2 * blk;
    d.sIr0 = Dr;
    d.csplit = Dr;
    d.sIc1 = blk;
    d.sIc = 1;
  } else {  // W = Theta^H: rows (s2, c), columns (s1, a), conjugated
    d.rsplit = Dr;
    d.sIr1 = blk;
    d.sIr0 = 1;
    d.csplit = Dl;
    d.sIc1 = 2 * blk;
    d.sIc = Dr;
    d.conj_in = 1;
  }
  d.m = p;
  d.n = q;
  d.complete = 0;
  d.work = work;
  d.tau = tau;
  d.q = nullptr;
  d.rr = r_out;
  d.sRr = q;
  d.sRc = 1;
  d.rrows_out = K;
  d.rcols_out = q;
  return d;
}

// ----------------------------------------------------------------------------------
// elementwise helpers
// ----------------------------------------------------------------------------------
template <typename T>
struct CopyDesc {  // dst(i0,i1,i2) = scale * src(i0,i1,i2) with zero padding
  const cplx<T>* src;
  cplx<T>* dst;
  int n0, n1, n2;           // destination extents
  int m0, m1, m2;           // source extents (elements outside read as 0)
  long long s0, s1, s2;     // source strides
  long long d0, d1, d2;     // destination strides
  int tile_begin, tiles;
};

template <typename T>
int launch_copy(const CopyDesc<T>* d, const CopyDesc<T>* h, int nd, cudaStream_t st);

// single-site reduced density matrices rho[s,s'] = sum_{a,c} A[s][a][c] conj(A[s'][a][c]),
// one CTA per problem; out = {rho00, rho11, Re rho01, Im rho01}
template <typename T>
struct RhoDesc {
  const cplx<T>* A;
  int Dl, Dr;
  double* out;
};

template <typename T>
int launch_rho(const RhoDesc<T>* d, int nd, cudaStream_t st);

}  // namespace qca
