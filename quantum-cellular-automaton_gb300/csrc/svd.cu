// Two-site split of 2TDVP (tdvp.py:286-296): SVD of theta viewed as the
// (2 Dl) x (2 Dr) matrix Theta[(s1,a),(s2,c)], truncation to
//   k = min{ i : ||s[i:]||_2 < eps }  capped at min(chi, len s)
// and s renormalised (lautils.normalize, lautils.py:4-5).
//
// QR-preconditioned one-sided (Hestenes) Jacobi.  The matrix W = Theta^H on a
// right sweep (the left factor must come out an isometry) or W = Theta on a left
// sweep (the right factor must) is first factored W = Q R by Householder
// reflections (qr.cu, launched before these kernels), and the Jacobi rotations
// run on X = R^H (q x K).  The two-site matrices of TDVP have exponentially
// graded spectra; on them Jacobi applied to the matrix directly converges
// linearly and needs dozens of sweeps, while on R^H, whose columns are already
// nearly orthogonal and graded, far fewer suffice.  At convergence (X = R^H V, V
// the product of the rotations) W^H = U Sigma (Q V)^H with U = X / Sigma, so the
// site tensors are written from
//   the isometric factor U = X / Sigma (its orthogonality is what the rotation
//   tolerance enforces, so it holds in FP32 too),
//   the other factor W U = (Q V) Sigma, one product with the two-site matrix per
//   kept column, so that neither Q nor V is ever formed and the rotations only
//   touch X,
// with the renormalised singular values in the non-isometric factor (tdvp.py:
// 121-122 and 141-142).  The singular values are the FP64 norms of X's columns.
//
// Two kernels over a thread-block cluster (1..16 CTAs, distributed shared memory):
//  * svd_block_kernel (column length <= 256): the columns form 2P blocks of at most
//    16; CTA k holds two of them in its own shared memory and rotates every pair
//    between and (once per sweep) inside them with block-local barriers, one column
//    pair per warp.  After each block round the blocks move one position along the
//    Brent-Luk ring (position 0 fixed), so 2P - 1 block rounds meet every block pair
//    once per sweep; only these moves use distributed shared memory and the cluster
//    barrier.
//  * svd_cluster_kernel (longer columns): the columns stay where they were loaded,
//    every round of a round-robin tournament rotates one disjoint column pair per
//    warp through distributed shared memory, and the cluster barrier separates the
//    rounds.
// Every rotation evaluates the pair's squared norms and inner product afresh from
// the columns (one pass, one shuffle tree), so the rotation angles never rest on
// drifted norms and the sweeps keep their quadratic convergence.
#include <cooperative_groups.h>

#include <algorithm>
#include <cstring>

#include "tdvp_kernels.cuh"

namespace cg = cooperative_groups;

namespace qca {

namespace {

constexpr int kSvdThreads = 512;
constexpr int kSvdMaxN = 1024;
constexpr int kSvdMaxSweeps = 24;
constexpr int kSvdBlk = 16;              // columns per block of svd_block_kernel
constexpr size_t kSvdSmem = 200 * 1024;  // dynamic shared memory per CTA

// Rotation tolerance on |u^H v| / (||u|| ||v||).  It must sit clearly above the
// rounding noise of the inner product, or pairs whose true inner product is below
// the noise keep rotating and the sweeps never terminate: FP64 sums over mx
// elements carry up to ~mx eps of noise, hence mx eps (at least 8 eps); the FP32
// inner products (at most 16 elements per lane, then a 5-level tree) carry a few
// eps32, hence 16 eps32.
template <typename T>
__device__ __forceinline__ double jacobi_tol(int mx) {
  return sizeof(T) == 4 ? 16.0 * 1.2e-7 : 2.2e-16 * fmax(8.0, (double)mx);
}

// Jacobi sweep limit of a problem (the descriptor may lower the default)
template <typename T>
__device__ __forceinline__ int svd_max_sweeps(const SvdDesc<T>& D) {
  return D.max_sweeps > 0 && D.max_sweeps < kSvdMaxSweeps ? D.max_sweeps : kSvdMaxSweeps;
}

template <typename T>
struct Prec;
template <>
struct Prec<double> {
  static constexpr double eps = 2.2e-16;
};
template <>
struct Prec<float> {
  static constexpr double eps = 1.2e-7;
};

// Compensated FP32 sums (each product split exactly with an FMA, partial sums
// carried as hi + lo pairs, also through the warp reduction) for the column norms
// that decide the singular values and the rounding floor.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
struct DF {
  float hi = 0.f, lo = 0.f;
  __device__ __forceinline__ void add(float x) {
    float s, e;
    two_sum(hi, x, s, e);
    hi = s;
    lo += e;
  }
  __device__ __forceinline__ void add_prod(float a, float b) {
    const float p = a * b;
    const float pe = fmaf(a, b, -p);  // exact product error
    add(p);
    lo += pe;
  }
  __device__ __forceinline__ void add_df(float h, float l) {
    float s, e;
    two_sum(hi, h, s, e);
    hi = s;
    lo += e + l;
  }
  __device__ __forceinline__ float value() const { return hi + lo; }
};

// Squared norm of one column held in the registers of a warp (compensated in FP32).
template <typename T, int RPL>
__device__ __forceinline__ T col_norm2(const cplx<T> (&ru)[RPL]) {
  T a;
  if constexpr (sizeof(T) == 4) {
    DF d;
#pragma unroll
    for (int k = 0; k < RPL; ++k) {
      d.add_prod(ru[k].re, ru[k].re);
      d.add_prod(ru[k].im, ru[k].im);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d.add_df(__shfl_xor_sync(0xffffffffu, d.hi, o), __shfl_xor_sync(0xffffffffu, d.lo, o));
    a = d.value();
  } else {
    a = 0;
#pragma unroll
    for (int k = 0; k < RPL; ++k) a = fma(ru[k].re, ru[k].re, fma(ru[k].im, ru[k].im, a));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  }
  return __shfl_sync(0xffffffffu, a, 0);
}

template <typename T, int RPL>
__device__ __forceinline__ void col_load(const cplx<T>* p, int len, cplx<T> (&r)[RPL]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < RPL; ++k) {
    const int i = lane + 32 * k;
    r[k] = i < len ? p[i] : mk<T>(0, 0);
  }
}

template <typename T, int RPL>
__device__ __forceinline__ void col_store(cplx<T>* p, int len, const cplx<T> (&r)[RPL]) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < RPL; ++k) {
    const int i = lane + 32 * k;
    if (i < len) p[i] = r[k];
  }
}

// Gram entries of a column pair from the registers of a warp: ||u||^2, ||v||^2 and
// u^H v, each lane summing its RPL <= 16 elements in the working precision, then
// one 5-level shuffle tree for the four sums (error a few eps |u||v|, below the
// rotation tolerance).  Every lane returns lane 0's values, so that all lanes of a
// warp take the same branch and apply the same rotation.
template <typename T, int RPL>
__device__ __forceinline__ void pair_gram(const cplx<T> (&ru)[RPL], const cplx<T> (&rv)[RPL], T& au, T& bv, T& gr,
                                          T& gi) {
  T a = 0, b = 0, r = 0, i = 0;
#pragma unroll
  for (int k = 0; k < RPL; ++k) {
    const cplx<T> u = ru[k], v = rv[k];
    a = fma(u.re, u.re, fma(u.im, u.im, a));
    b = fma(v.re, v.re, fma(v.im, v.im, b));
    r = fma(u.re, v.re, fma(u.im, v.im, r));  // conj(u) v
    i = fma(u.re, v.im, fma(-u.im, v.re, i));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    r += __shfl_xor_sync(0xffffffffu, r, o);
    i += __shfl_xor_sync(0xffffffffu, i, o);
  }
  au = __shfl_sync(0xffffffffu, a, 0);
  bv = __shfl_sync(0xffffffffu, b, 0);
  gr = __shfl_sync(0xffffffffu, r, 0);
  gi = __shfl_sync(0xffffffffu, i, 0);
}

// One Jacobi rotation of the column pair (xu, xv) of X, held in registers.  The squared column norms and the inner product are
// evaluated afresh from the registers for every pair: norms carried from earlier
// rotations in closed form drift (by the rounding of every update, and badly after
// cancellation), and a rotation angle computed from drifted norms leaves an inner
// product of the size of the drift, which turns the quadratic convergence of the
// sweeps into a linear one.  al, be return the new squared norms (closed form).
// Returns false (nothing changed) when the pair is already orthogonal to the
// tolerance or one column is at the rounding floor of the matrix.
//   x_p' = c x_p - s e^{-i phi} x_q ;  x_q' = s e^{i phi} x_p + c x_q   (unitary)
template <typename T, int RPL>
__device__ __forceinline__ bool jacobi_rotate(cplx<T> (&xu)[RPL], cplx<T> (&xv)[RPL], T& al, T& be, double tol,
                                              T floor2) {
  T gr, gi;
  pair_gram<T, RPL>(xu, xv, al, be, gr, gi);
  const T g = sqrt(gr * gr + gi * gi);
  if (!(g > (T)tol * sqrt(al * be)) || al <= floor2 || be <= floor2) return false;
  const T zeta = (be - al) / (2 * g);
  const T t = (zeta >= 0 ? (T)1 : (T)-1) / (fabs(zeta) + sqrt(1 + zeta * zeta));
  const T c = 1 / sqrt(1 + t * t);
  const T s = c * t;
  const T er = gr / g, ei = gi / g;  // e^{i phi}
  const cplx<T> smq = mk<T>(-s * er, s * ei);
  const cplx<T> spq = mk<T>(s * er, s * ei);
#pragma unroll
  for (int r = 0; r < RPL; ++r) {
    const cplx<T> a = xu[r], b = xv[r];
    xu[r] = c * a + smq * b;
    xv[r] = spq * a + c * b;
  }
  al = fmax(al - t * g, (T)0);
  be = fmax(be + t * g, (T)0);
  return true;
}

// X column col (mx rows) into dst, by the whole CTA
template <typename T>
__device__ __forceinline__ void load_x_column(const SvdDesc<T>& D, int mx, int nx, int col, cplx<T>* dst) {
  // column col of X = R^H: X[i][col] = conj(R[col][i]), R row major K x q (q = mx)
  for (int row = threadIdx.x; row < mx; row += blockDim.x) {
    cplx<T> v = mk<T>(0, 0);
    if (col < nx) {
      v = D.rmat[(long long)col * mx + row];
      v.im = -v.im;
    }
    dst[row] = v;
  }
}

// Shape of the preconditioned problem: W (p x q) is Theta^H on a right sweep and
// Theta on a left sweep; Jacobi runs on X = R^H, mx = q rows and nx = K columns.
template <typename T>
__device__ __forceinline__ void split_shape(const SvdDesc<T>& D, int& p, int& mx, int& nx) {
  p = D.right_sweep ? 2 * D.Dr : 2 * D.Dl;
  mx = D.right_sweep ? 2 * D.Dl : 2 * D.Dr;
  nx = p < mx ? p : mx;
}

// After convergence: FP64 norms of the columns (singular values), rank sort in CTA 0,
// the truncation rule, and the site tensors from the kept columns.  L.own(j) says
// whether this CTA holds global column j, L.x(j) / L.v(j) give its X (mx) and V (nx)
// columns.  Ends with a cluster barrier: CTA 0's shared memory is read through
// distributed shared memory until then.
template <typename T, typename Loc>
__device__ void svd_finish(const SvdDesc<T>& D, cg::cluster_group& cluster, int rank, const Loc& L, int p, int mx,
                           int nx, int sweep, T floor2, double* snorm, int* perm, int* s_k, double* s_keep) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int Dr = D.Dr;
  double* snorm0 = cluster.map_shared_rank(snorm, 0);
  for (int j = wid; j < nx; j += nw) {
    if (!L.own(j)) continue;
    const cplx<T>* x = L.x(j);
    double s = 0.0;
    for (int i = lane; i < mx; i += 32) s += (double)x[i].re * x[i].re + (double)x[i].im * x[i].im;
    s = warp_sum(s);
    // a non-finite column is marked (-1) and ranked as zero, so that the rank
    // permutation below stays a permutation; the problem reports QCA_ERR_NAN
    if (lane == 0) snorm0[j] = isfinite(s) ? sqrt(s) : -1.0;
  }
  cluster.sync();
  if (rank == 0) {
    if (threadIdx.x == 0) *s_k = 0;
    __syncthreads();
    for (int j = threadIdx.x; j < nx; j += blockDim.x)
      if (!(snorm[j] >= 0.0)) {
        snorm[j] = 0.0;
        *s_k = 1;
      }
    __syncthreads();
    const bool non_finite = *s_k != 0;
    __syncthreads();
    for (int j = threadIdx.x; j < nx; j += blockDim.x) {
      const double sj = snorm[j];
      int r = 0;
      for (int i = 0; i < nx; ++i) {
        const double si = snorm[i];
        r += (si > sj) || (si == sj && i < j);
      }
      perm[r] = j;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      // tail norms ||s[i:]|| in FP64 (tdvp.py:290-292)
      double acc = 0.0, total = 0.0;
      int first = nx;
      for (int i = nx - 1; i >= 0; --i) {
        const double sv = snorm[perm[i]];
        acc += sv * sv;
        if (sqrt(acc) < D.eps) first = i;
      }
      total = acc;
      int k = first;
      const int cap = D.chi < nx ? D.chi : nx;
      if (k > cap) k = cap;
      if (k > D.kmax) k = D.kmax;
      // never keep a direction at the rounding floor of the working precision: its
      // column was not rotated to orthogonality and would break the isometry of
      // the site tensors (only exact zeros are affected in FP64)
      const double noise = 4.0 * sqrt((double)floor2);
      while (k > 1 && snorm[perm[k - 1]] <= noise) --k;
      if (k < 1) k = 1;
      double keep = 0.0;
      for (int i = 0; i < k; ++i) keep += snorm[perm[i]] * snorm[perm[i]];
      *s_k = k;
      *s_keep = sqrt(keep);
      *D.k_out = k;
      if (D.discarded) *D.discarded += total > 0 ? (total - keep) / total : 0.0;
      for (int i = 0; i < nx; ++i) D.sv[i] = snorm[perm[i]];
      if (D.status) {
        D.status[0] = non_finite ? QCA_ERR_NAN : (sweep >= svd_max_sweeps(D)) ? QCA_ERR_NOT_CONVERGED : 0;
        D.status[1] = sweep + 1;  // sweeps used
      }
    }
  }
  cluster.sync();
  const int k = *cluster.map_shared_rank(s_k, 0);
  const double keep = *cluster.map_shared_rank(s_keep, 0);
  const int* perm0 = cluster.map_shared_rank(perm, 0);
  const double* sn0 = cluster.map_shared_rank(snorm, 0);
  // Kept column i (global column j = perm[i], singular value sigma_j): the
  // isometric factor u_j = x_j / sigma_j (mx = q rows) and the other factor
  // W u_j / ||s_kept|| (p rows): with X orthogonal, W^H = U Sigma (Q V)^H gives
  // W u_j = (Q V)_j sigma_j, so neither Q nor the accumulated rotations are needed.
  //   right sweep (W = Theta^H): A_l[(s1,a)][i] = u_j[(s1,a)],
  //                              A_r[s2][i][c] = conj((W u_j)[(s2,c)]) / keep
  //   left sweep  (W = Theta):   A_l[(s1,a)][i] = (W u_j)[(s1,a)] / keep,
  //                              A_r[s2][i][c] = conj(u_j[(s2,c)])
  const int Dl = D.Dl;
  const long long blk = (long long)Dl * Dr;
  for (int i = 0; i < k; ++i) {
    const int j = perm0[i];
    if (!L.own(j)) continue;
    const cplx<T>* x = L.x(j);
    const double sig = sn0[j];
    const double inv = sig > 0 ? 1.0 / sig : 0.0;
    const double f = keep > 0 ? inv / keep : 0.0;
    for (int row = threadIdx.x; row < p; row += blockDim.x) {
      cplx<T> acc = mk<T>(0, 0);
      if (D.right_sweep) {
        // (Theta^H x)[(s2,c)] = sum_{s1,a} conj(theta[s1*2+s2][a][c]) x[(s1,a)]
        const int s2 = row / Dr, cc = row - s2 * Dr;
        for (int s1 = 0; s1 < 2; ++s1) {
          const cplx<T>* th = D.theta + (long long)(s1 * 2 + s2) * blk + cc;
          const cplx<T>* xs = x + s1 * Dl;
          for (int a = 0; a < Dl; ++a) cfma_conj(acc, th[(long long)a * Dr], xs[a]);
        }
        const cplx<T> w = mk<T>((T)(acc.re * f), (T)(acc.im * f));
        D.Ar[((long long)s2 * k + i) * Dr + cc] = conj(w);
      } else {
        // (Theta x)[(s1,a)] = sum_{s2,c} theta[s1*2+s2][a][c] x[(s2,c)]
        const int s1 = row / Dl, a = row - s1 * Dl;
        for (int s2 = 0; s2 < 2; ++s2) {
          const cplx<T>* th = D.theta + (long long)(s1 * 2 + s2) * blk + (long long)a * Dr;
          const cplx<T>* xs = x + s2 * Dr;
          for (int c = 0; c < Dr; ++c) cfma(acc, th[c], xs[c]);
        }
        D.Al[(long long)row * k + i] = mk<T>((T)(acc.re * f), (T)(acc.im * f));
      }
    }
    for (int row = threadIdx.x; row < mx; row += blockDim.x) {
      const cplx<T> u = x[row];
      const cplx<T> w = mk<T>((T)(u.re * inv), (T)(u.im * inv));
      if (D.right_sweep) {
        D.Al[(long long)row * k + i] = w;
      } else {
        const int s2 = row / Dr, cc = row - s2 * Dr;
        D.Ar[((long long)s2 * k + i) * Dr + cc] = conj(w);
      }
    }
  }
  cluster.sync();
}

// columns rank*cpc .. rank*cpc + cpc - 1 of svd_cluster_kernel
template <typename T>
struct SlabLoc {
  const cplx<T>* X;
  int cpc, mx, nx, rank;
  __device__ bool own(int j) const { return j / cpc == rank; }
  __device__ const cplx<T>* x(int j) const { return X + (long long)(j % cpc) * mx; }
};

// blocks of svd_block_kernel at their sweep-start positions: block be sits in the
// top slot of CTA be (be < P) or the bottom slot of CTA 2P - 1 - be
template <typename T>
struct BlockLoc {
  const cplx<T>* X;   // [slot][b][mx]
  int P, b, mx, nx, rank;
  __device__ int blk(int j) const { return j / b; }
  __device__ int slot(int j) const { return blk(j) < P ? 0 : 1; }
  __device__ bool own(int j) const { return (blk(j) < P ? blk(j) : 2 * P - 1 - blk(j)) == rank; }
  __device__ const cplx<T>* x(int j) const { return X + ((long long)slot(j) * b + j % b) * mx; }
};

template <typename T, int RPL>
__global__ void __launch_bounds__(kSvdThreads) svd_cluster_kernel(const SvdDesc<T>* __restrict__ descs, int cs,
                                                                  int cpc) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const SvdDesc<T>& D = descs[blockIdx.x / cs];
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* Xloc = reinterpret_cast<cplx<T>*>(smem_raw);  // cpc columns of mx elements
  __shared__ double snorm[kSvdMaxN];                     // used in CTA 0
  __shared__ int perm[kSvdMaxN];                         // used in CTA 0
  __shared__ int s_flag[2];                              // rotation flags (CTA 0), by sweep parity
  __shared__ int s_k;
  __shared__ double s_keep;
  __shared__ double s_fro;  // ||Theta||_F^2 (CTA 0)
  __shared__ double red[33];
  int p, mx, nx;
  split_shape(D, p, mx, nx);
  for (int lc = 0; lc < cpc; ++lc) {
    const int col = rank * cpc + lc;
    if (col >= nx) break;
    load_x_column(D, mx, nx, col, Xloc + (long long)lc * mx);
  }
  if (threadIdx.x < 2) s_flag[threadIdx.x] = 0;
  if (threadIdx.x == 0) s_fro = 0.0;
  cluster.sync();
  {
    // Frobenius norm: columns whose norm is at the rounding floor of the matrix
    // carry no information; rotating them against large columns only re-injects
    // rounding noise and would keep the sweeps from terminating.
    double f = 0.0;
    for (int lc = 0; lc < cpc; ++lc) {
      if (rank * cpc + lc >= nx) break;
      for (int row = threadIdx.x; row < mx; row += blockDim.x) f += (double)norm2(Xloc[(long long)lc * mx + row]);
    }
    f = block_sum(f, red);
    if (threadIdx.x == 0) atomicAdd(cluster.map_shared_rank(&s_fro, 0), f);
  }
  cluster.sync();
  const double fro = *cluster.map_shared_rank(&s_fro, 0);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int P = nx + (nx & 1);
  const double tol = jacobi_tol<T>(mx);
  const T floor2 = (T)(16.0 * Prec<T>::eps * Prec<T>::eps * fro);
  int* flag0 = cluster.map_shared_rank(s_flag, 0);
  int sweep = 0;
  const int max_sweeps = svd_max_sweeps(D);
  for (; sweep < max_sweeps; ++sweep) {
    const int par = sweep & 1;
    int rotated = 0;
    for (int round = 0; round < P - 1; ++round) {
      for (int pk = rank + cs * wid; pk < P / 2; pk += cs * nw) {
        int p, q;
        if (pk == 0) {
          p = P - 1;
          q = round;
        } else {
          p = (round + pk) % (P - 1);
          q = (round - pk + P - 1) % (P - 1);
        }
        if (p >= nx || q >= nx) continue;
        if (p > q) {
          const int t = p;
          p = q;
          q = t;
        }
        cplx<T>* xp = cluster.map_shared_rank(Xloc, p / cpc) + (long long)(p % cpc) * mx;
        cplx<T>* xq = cluster.map_shared_rank(Xloc, q / cpc) + (long long)(q % cpc) * mx;
        // both columns staged in registers in one round of (possibly remote) loads;
        // the rotation in the working precision T (the singular values are
        // re-evaluated in FP64 after convergence)
        cplx<T> ru[RPL], rv[RPL];
        col_load<T, RPL>(xp, mx, ru);
        col_load<T, RPL>(xq, mx, rv);
        T al, be;
        if (!jacobi_rotate<T, RPL>(ru, rv, al, be, tol, floor2)) continue;
        rotated = 1;
        col_store<T, RPL>(xp, mx, ru);
        col_store<T, RPL>(xq, mx, rv);
      }
      cluster.sync();
    }
    if (rotated && lane == 0) atomicOr(flag0 + par, 1);
    cluster.sync();
    const int any = *(volatile int*)(flag0 + par);
    cluster.sync();  // everyone has read the flag before it is reset below
    if (rank == 0 && threadIdx.x == 0) s_flag[par] = 0;
    if (!any) break;
  }
  const SlabLoc<T> L{Xloc, cpc, mx, nx, rank};
  svd_finish<T>(D, cluster, rank, L, p, mx, nx, sweep, floor2, snorm, perm, &s_k, &s_keep);
}

template <typename T, int RPL>
__global__ void __launch_bounds__(kSvdThreads) svd_block_kernel(const SvdDesc<T>* __restrict__ descs, int P) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const SvdDesc<T>& D = descs[blockIdx.x / P];
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double snorm[kSvdMaxN];  // used in CTA 0
  __shared__ int perm[kSvdMaxN];      // used in CTA 0
  __shared__ int s_flag[2];           // rotation flags (CTA 0), by sweep parity
  __shared__ int s_k;
  __shared__ double s_keep;
  __shared__ double s_fro;  // ||Theta||_F^2 (CTA 0)
  __shared__ double red[33];
  int p, mx, nx;
  split_shape(D, p, mx, nx);
  const int n2 = 2 * P;                // blocks (tournament players)
  const int b = (nx + n2 - 1) / n2;    // columns per block (<= kSvdBlk)
  // slots [generation][top/bottom][b columns] of mx elements
  cplx<T>* Xs = reinterpret_cast<cplx<T>*>(smem_raw);
  auto xs = [&](int g, int s, int j) { return Xs + ((long long)(g * 2 + s) * b + j) * mx; };
  // block at ring position pos in block round r (circle method, position 0 fixed)
  auto player = [&](int pos, int r) { return pos == 0 ? 0 : 1 + (pos - 1 + r) % (n2 - 1); };
  for (int s = 0; s < 2; ++s) {
    const int be = s == 0 ? rank : n2 - 1 - rank;
    for (int j = 0; j < b; ++j) {
      const int col = be * b + j;
      load_x_column(D, mx, nx, col, xs(0, s, j));
    }
  }
  if (threadIdx.x < 2) s_flag[threadIdx.x] = 0;
  if (threadIdx.x == 0) s_fro = 0.0;
  cluster.sync();
  {
    // Frobenius norm (padding columns are zero)
    double f = 0.0;
    for (int c = 0; c < 2 * b; ++c) {
      const cplx<T>* x = xs(0, c / b, c % b);
      for (int row = threadIdx.x; row < mx; row += blockDim.x) f += (double)norm2(x[row]);
    }
    f = block_sum(f, red);
    if (threadIdx.x == 0) atomicAdd(cluster.map_shared_rank(&s_fro, 0), f);
  }
  cluster.sync();
  const double fro = *cluster.map_shared_rank(&s_fro, 0);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const double tol = jacobi_tol<T>(mx);
  const T floor2 = (T)(16.0 * Prec<T>::eps * Prec<T>::eps * fro);
  int* flag0 = cluster.map_shared_rank(s_flag, 0);
  int gen = 0, sweep = 0;
  const int max_sweeps = svd_max_sweeps(D);
  for (; sweep < max_sweeps; ++sweep) {
    const int par = sweep & 1;
    int rotated = 0;
    for (int r = 0; r < n2 - 1; ++r) {
      const int bt = player(rank, r), bb = player(n2 - 1 - rank, r);
      if (r == 0) {
        // pairs inside each resident block, both blocks at once (round robin over b)
        const int Bp = b + (b & 1), half = Bp / 2;
        for (int ir = 0; ir + 1 < Bp; ++ir) {
          for (int t = wid; t < 2 * half; t += nw) {
            const int s = t / half, pk = t - s * half;
            int p, q;
            if (pk == 0) {
              p = Bp - 1;
              q = ir;
            } else {
              p = (ir + pk) % (Bp - 1);
              q = (ir - pk + Bp - 1) % (Bp - 1);
            }
            if (p >= b || q >= b) continue;
            const int bl = s == 0 ? bt : bb;
            const int gp = bl * b + p, gq = bl * b + q;
            if (gp >= nx || gq >= nx) continue;
            cplx<T> xu[RPL], xv[RPL];
            col_load<T, RPL>(xs(gen, s, p), mx, xu);
            col_load<T, RPL>(xs(gen, s, q), mx, xv);
            T al, be;
            if (!jacobi_rotate<T, RPL>(xu, xv, al, be, tol, floor2)) continue;
            rotated = 1;
            col_store<T, RPL>(xs(gen, s, p), mx, xu);
            col_store<T, RPL>(xs(gen, s, q), mx, xv);
          }
          __syncthreads();
        }
      }
      {
        // pairs across the two blocks: warp w keeps top column w in registers and
        // meets bottom column (w + i) mod b in inner round i
        const int ga = bt * b + wid;
        const bool act = wid < b && ga < nx;
        cplx<T> xu[RPL];
        T al = 0;
        if (act) col_load<T, RPL>(xs(gen, 0, wid), mx, xu);
        bool dirty = false;
        for (int i = 0; i < b; ++i) {
          if (act) {
            const int j = (wid + i) % b;
            const int gb = bb * b + j;
            if (gb < nx) {
              cplx<T> xv[RPL];
              col_load<T, RPL>(xs(gen, 1, j), mx, xv);
              T be;
              if (jacobi_rotate<T, RPL>(xu, xv, al, be, tol, floor2)) {
                rotated = 1;
                dirty = true;
                col_store<T, RPL>(xs(gen, 1, j), mx, xv);
              }
            }
          }
          __syncthreads();
        }
        if (dirty) col_store<T, RPL>(xs(gen, 0, wid), mx, xu);
      }
      // move the blocks one position along the ring: position p takes the block of
      // position p + 1, position 2P - 1 the block of position 1, position 0 keeps its
      // block.  Reads the other CTAs' current generation, writes the own next one.
      cluster.sync();
      if (P > 1) {
        const int ng = gen ^ 1;
        const int tr = rank == 0 ? 0 : (rank + 1 < P ? rank + 1 : rank);
        const int ts = rank == 0 ? 0 : (rank + 1 < P ? 0 : 1);
        const int br = rank >= 1 ? rank - 1 : 1;
        const int bs = rank >= 1 ? 1 : 0;
        for (int s = 0; s < 2; ++s) {
          const int sr = s == 0 ? tr : br, ss = s == 0 ? ts : bs;
          const cplx<T>* src = cluster.map_shared_rank(xs(gen, ss, 0), sr);
          cplx<T>* dst = xs(ng, s, 0);
          for (int e = threadIdx.x; e < b * mx; e += blockDim.x) dst[e] = src[e];
        }
        __syncthreads();
        gen = ng;
      }
    }
    if (rotated && lane == 0) atomicOr(flag0 + par, 1);
    cluster.sync();
    const int any = *(volatile int*)(flag0 + par);
    cluster.sync();  // everyone has read the flag before it is reset below
    if (rank == 0 && threadIdx.x == 0) s_flag[par] = 0;
    if (!any) break;
  }
  // after a whole sweep (2P - 1 moves) every block is back at its starting position
  const BlockLoc<T> L{xs(gen, 0, 0), P, b, mx, nx, rank};
  svd_finish<T>(D, cluster, rank, L, p, mx, nx, sweep, floor2, snorm, perm, &s_k, &s_keep);
}

// block kernel geometry: P CTAs (power of two, P * 32 >= nx where possible), blocks of
// b <= 16 columns, X (and V when it fits) double-buffered in shared memory
template <typename T>
bool svd_block_plan(int mx, int nx, int* P_out, int* b_out, size_t* smem) {
  if (mx > 256) return false;
  int P = 1;
  while (P * 32 < nx && P < 16) P *= 2;
  const int b = (nx + 2 * P - 1) / (2 * P);
  if (b > kSvdBlk) return false;
  const size_t xb = 4ull * b * mx * sizeof(cplx<T>);  // two generations x two slots
  if (xb > kSvdSmem) return false;
  *P_out = P;
  *b_out = b;
  *smem = xb;
  return true;
}

template <typename T>
int svd_cluster_plan(int mx, int nx, int* cs, int* cpc, size_t* smem) {
  const size_t limit = 200 * 1024;
  const int pairs = (nx + 1) / 2, warps = kSvdThreads / 32;
  for (int c = 1; c <= 16; c *= 2) {
    const int per = (nx + c - 1) / c;
    const size_t bytes = (size_t)per * mx * sizeof(cplx<T>);
    // enough warps in the cluster for one column pair each per round
    if (bytes <= limit && (c * warps >= pairs || c == 16)) {
      *cs = c;
      *cpc = per;
      *smem = bytes;
      return QCA_OK;
    }
  }
  return QCA_ERR_INVALID;
}

}  // namespace

// cluster size one problem needs (0 if it does not fit); used to group problems
template <typename T>
int svd_cluster_size(int Dl, int Dr, int right_sweep) {
  const int p = right_sweep ? 2 * Dr : 2 * Dl, mx = right_sweep ? 2 * Dl : 2 * Dr, nx = p < mx ? p : mx;
  int cs, cpc;
  size_t sm;
  if (svd_block_plan<T>(mx, nx, &cs, &cpc, &sm)) return cs;
  if (svd_cluster_plan<T>(mx, nx, &cs, &cpc, &sm) != QCA_OK) return 0;
  return cs;
}

template <typename... Args>
static int launch_clustered(void (*kern)(Args...), int ctas, int cs, size_t smem, cudaStream_t st, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ctas, 1, 1);
  cfg.blockDim = dim3(kSvdThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = cs;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  QCA_CUDA(cudaLaunchKernelEx(&cfg, kern, args...));
  count_launches(1);
  return QCA_OK;
}

template <typename T>
int launch_svd(const SvdDesc<T>* d, const SvdDesc<T>* h, int nd, cudaStream_t st) {
  if (nd <= 0) return QCA_OK;
  int mxmax = 1, nxmax = 1;
  for (int i = 0; i < nd; ++i) {
    // Jacobi runs on X = R^H: q rows (2 Dl right, 2 Dr left), K = min(p, q) columns
    const int p = h[i].right_sweep ? 2 * h[i].Dr : 2 * h[i].Dl, q = h[i].right_sweep ? 2 * h[i].Dl : 2 * h[i].Dr;
    mxmax = std::max(mxmax, q);
    nxmax = std::max(nxmax, std::min(p, q));
  }
  const int rows = (mxmax + 31) / 32;
  if (rows > 16) {
    set_error("SVD column length %d exceeds 512", mxmax);
    return QCA_ERR_INVALID;
  }
  const int rpl = rows <= 2 ? 2 : rows <= 4 ? 4 : rows <= 8 ? 8 : 16;
  const int ti = sizeof(T) == 8 ? 0 : 1, ri = rpl == 2 ? 0 : rpl == 4 ? 1 : rpl == 8 ? 2 : 3;
  const int dv = device_slot();
  int P = 1, b = 1;
  size_t smem = 0;
  if (svd_block_plan<T>(mxmax, nxmax, &P, &b, &smem)) {
    // column length <= 256: RPL <= 8
    static bool configured[kMaxDevices][2][3] = {};
    void (*kern)(const SvdDesc<T>*, int) =
        rpl == 2 ? svd_block_kernel<T, 2> : rpl == 4 ? svd_block_kernel<T, 4> : svd_block_kernel<T, 8>;
    if (dv < 0 || !configured[dv][ti][ri]) {
      QCA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSvdSmem));
      QCA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
      if (dv >= 0) configured[dv][ti][ri] = true;
    }
    return launch_clustered(kern, nd * P, P, smem, st, d, P);
  }
  int cs = 1, cpc = 1;
  if (svd_cluster_plan<T>(mxmax, nxmax, &cs, &cpc, &smem) != QCA_OK) {
    set_error("SVD of %d x %d exceeds the distributed shared memory of a 16-CTA cluster", mxmax, nxmax);
    return QCA_ERR_INVALID;
  }
  static bool configured[kMaxDevices][2][4] = {};
  void (*kern)(const SvdDesc<T>*, int, int) =
      rpl == 2 ? svd_cluster_kernel<T, 2>
               : rpl == 4 ? svd_cluster_kernel<T, 4> : rpl == 8 ? svd_cluster_kernel<T, 8> : svd_cluster_kernel<T, 16>;
  if (dv < 0 || !configured[dv][ti][ri]) {
    QCA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSvdSmem));
    QCA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    if (dv >= 0) configured[dv][ti][ri] = true;
  }
  return launch_clustered(kern, nd * cs, cs, smem, st, d, cs, cpc);
}

template int launch_svd<double>(const SvdDesc<double>*, const SvdDesc<double>*, int, cudaStream_t);
template int launch_svd<float>(const SvdDesc<float>*, const SvdDesc<float>*, int, cudaStream_t);
template int svd_cluster_size<double>(int, int, int);
template int svd_cluster_size<float>(int, int, int);

}  // namespace qca

// Test hook: the two-site split on its own.  theta (4, Dl, Dr), Al (2, Dl, k) and
// Ar (2, k, Dr) are DEVICE arrays of the precision's complex type with room for
// k = min(2 Dl, 2 Dr); sv (device, FP64) receives the min(2 Dl, 2 Dr) singular
// values in descending order; *k_out the truncated bond (right-sweep form: A_l = U,
// A_r = s Vh / ||s||).  Synchronises the stream.
template <typename T>
static int test_svd(int Dl, int Dr, const void* theta, int chi, double eps, int max_sweeps, void* Al, void* Ar,
                    double* sv, int* k_out, cudaStream_t st) {
  using namespace qca;
  const int p = 2 * Dr, q = 2 * Dl, K = std::min(p, q);  // right sweep: W = Theta^H
  const size_t es = sizeof(cplx<T>);
  // scratch: QR work (p q + p K), tau (K), R (K q), flags, descriptors
  const size_t n_work = (size_t)p * q + (size_t)p * K, n_tau = K, n_r = (size_t)K * q;
  const size_t elems = n_work + n_tau + n_r;
  const size_t fbytes = 64, dbytes = 2 * ((sizeof(SvdDesc<T>) + 63) / 64) * 64 + 2 * ((sizeof(QrDesc<T>) + 63) / 64) * 64;
  void* scratch = nullptr;
  QCA_CUDA(cudaMalloc(&scratch, elems * es + fbytes + dbytes));
  cplx<T>* base = (cplx<T>*)scratch;
  cplx<T>* work = base;
  cplx<T>* tau = work + n_work;
  cplx<T>* R = tau + n_tau;
  char* flags = (char*)(base + elems);
  SvdDesc<T>* dd = (SvdDesc<T>*)(flags + fbytes);
  QrDesc<T>* dq = (QrDesc<T>*)((char*)dd + ((sizeof(SvdDesc<T>) + 63) / 64) * 64);
  const QrDesc<T> qd = split_qr_desc<T>((const cplx<T>*)theta, Dl, Dr, 1, work, tau, R);
  SvdDesc<T> d;
  memset(&d, 0, sizeof(d));
  d.theta = (const cplx<T>*)theta;
  d.Dl = Dl;
  d.Dr = Dr;
  d.chi = chi;
  d.kmax = K;
  d.eps = eps;
  d.right_sweep = 1;
  d.max_sweeps = max_sweeps;
  d.Al = (cplx<T>*)Al;
  d.Ar = (cplx<T>*)Ar;
  d.rmat = R;
  d.sv = sv;
  d.k_out = (int*)flags;
  d.status = (int*)(flags + 16);
  d.discarded = (double*)(flags + 32);
  int s = QCA_OK;
  int h[3] = {0, 0, 0};
  if (cudaMemsetAsync(flags, 0, fbytes, st) != cudaSuccess ||
      cudaMemcpyAsync(dd, &d, sizeof(d), cudaMemcpyHostToDevice, st) != cudaSuccess ||
      cudaMemcpyAsync(dq, &qd, sizeof(qd), cudaMemcpyHostToDevice, st) != cudaSuccess) {
    set_error("qca_test_svd: %s", cudaGetErrorString(cudaGetLastError()));
    s = QCA_ERR_CUDA;
  }
  if (s == QCA_OK) s = launch_qr<T>(dq, 1, sizeof(T) == 4 ? 1 : 0, st);
  if (s == QCA_OK) s = launch_svd<T>(dd, &d, 1, st);
  if (s == QCA_OK && (cudaMemcpyAsync(h, flags, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                      cudaMemcpyAsync(h + 1, flags + 16, 2 * sizeof(int), cudaMemcpyDeviceToHost, st) !=
                          cudaSuccess ||
                      cudaStreamSynchronize(st) != cudaSuccess)) {
    set_error("qca_test_svd: %s", cudaGetErrorString(cudaGetLastError()));
    s = QCA_ERR_CUDA;
  }
  cudaFree(scratch);
  if (s != QCA_OK) return s;
  *k_out = h[0];
  if (h[1] == QCA_ERR_NAN) {
    set_error("qca_test_svd: non-finite singular values");
    return QCA_ERR_NAN;
  }
  if (h[1] != 0) {
    set_error("qca_test_svd: Jacobi sweeps did not converge (%d sweeps)", h[2]);
    return QCA_ERR_NOT_CONVERGED;
  }
  return QCA_OK;
}

static int test_svd_any(int precision, int Dl, int Dr, const void* theta, int chi, double eps, int max_sweeps, void* Al,
                        void* Ar, double* sv, int* k_out, void* stream) {
  using namespace qca;
  if (Dl < 1 || Dr < 1 || 2 * std::min(Dl, Dr) > 1024 || 2 * std::max(Dl, Dr) > 512 || !theta || !Al || !Ar ||
      !sv || !k_out || chi < 1 || !(eps >= 0) || max_sweeps < 0) {
    set_error("qca_test_svd: invalid arguments");
    return QCA_ERR_INVALID;
  }
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == QCA_PREC_FP64)
    return test_svd<double>(Dl, Dr, theta, chi, eps, max_sweeps, Al, Ar, sv, k_out, st);
  if (precision == QCA_PREC_MIXED)
    return test_svd<float>(Dl, Dr, theta, chi, eps, max_sweeps, Al, Ar, sv, k_out, st);
  set_error("qca_test_svd: unknown precision %d", precision);
  return QCA_ERR_INVALID;
}

extern "C" int qca_test_svd(int precision, int Dl, int Dr, const void* theta, int chi, double eps, void* Al, void* Ar,
                            double* sv, int* k_out, void* stream) {
  return test_svd_any(precision, Dl, Dr, theta, chi, eps, 0, Al, Ar, sv, k_out, stream);
}

extern "C" int qca_test_svd_sweeps(int precision, int Dl, int Dr, const void* theta, int chi, double eps,
                                   int max_sweeps, void* Al, void* Ar, double* sv, int* k_out, void* stream) {
  return test_svd_any(precision, Dl, Dr, theta, chi, eps, max_sweeps, Al, Ar, sv, k_out, stream);
}
