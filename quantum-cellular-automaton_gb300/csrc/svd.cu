// Two-site split of 2TDVP (tdvp.py:286-296): SVD of theta viewed as the
// (2 Dl) x (2 Dr) matrix Theta[(s1,a),(s2,c)], truncation to
//   k = min{ i : ||s[i:]||_2 < eps }  capped at min(chi, len s)
// and s renormalised (lautils.normalize, lautils.py:4-5).
//
// One-sided (Hestenes) Jacobi on the narrower orientation W (mx >= nx):
// W = Theta when 2 Dr <= 2 Dl, else W = Theta^H.  Its columns are distributed
// over the shared memory of a thread-block cluster (1..16 CTAs, distributed
// shared memory); in every round of a round-robin tournament each warp rotates
// one disjoint column pair, reading and writing both columns through DSMEM, and
// the cluster barrier separates the rounds.  The same rotations accumulate V
// (nx x nx), kept beside X in distributed shared memory when the cluster has
// room and in global memory otherwise.  At convergence X = W V has orthogonal
// columns whose FP64 norms are the singular values; the site tensors are written
// directly from X and V:
//   W = Theta:    U = X / sigma,  Vh = V^H
//   W = Theta^H:  U = V,          Vh = (X / sigma)^H
// with the renormalised singular values multiplied into A_r (right sweep) or
// A_l (left sweep), tdvp.py:121-122 and 141-142.
#include <cooperative_groups.h>

#include "tdvp_kernels.cuh"

namespace cg = cooperative_groups;

namespace qca {

namespace {

constexpr int kSvdThreads = 512;
constexpr int kSvdMaxN = 1024;
constexpr int kSvdMaxSweeps = 24;

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

// Gram entries of a column pair: ||u||^2, ||v||^2 and u^H v.  In FP32 the sums are
// compensated (each product split exactly with an FMA, partial sums carried as
// hi + lo pairs, also through the warp reduction), so that small inner products of
// nearly orthogonal columns are resolved beyond the sqrt(m) eps32 noise of a plain
// FP32 sum and the rotations can drive the columns to FP32-level orthogonality.
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

template <typename T, int RPL>
__device__ __forceinline__ void pair_gram(const cplx<T> (&ru)[RPL], const cplx<T> (&rv)[RPL], T& al, T& be, T& gr,
                                          T& gi) {
  if constexpr (sizeof(T) == 4) {
    DF a, b, r, i;
#pragma unroll
    for (int k = 0; k < RPL; ++k) {
      const cplx<T> u = ru[k], v = rv[k];
      a.add_prod(u.re, u.re);
      a.add_prod(u.im, u.im);
      b.add_prod(v.re, v.re);
      b.add_prod(v.im, v.im);
      r.add_prod(u.re, v.re);  // conj(u) v
      r.add_prod(u.im, v.im);
      i.add_prod(u.re, v.im);
      i.add_prod(-u.im, v.re);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a.add_df(__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o));
      b.add_df(__shfl_xor_sync(0xffffffffu, b.hi, o), __shfl_xor_sync(0xffffffffu, b.lo, o));
      r.add_df(__shfl_xor_sync(0xffffffffu, r.hi, o), __shfl_xor_sync(0xffffffffu, r.lo, o));
      i.add_df(__shfl_xor_sync(0xffffffffu, i.hi, o), __shfl_xor_sync(0xffffffffu, i.lo, o));
    }
    al = a.value();
    be = b.value();
    gr = r.value();
    gi = i.value();
  } else {
    T a = 0, b = 0, r = 0, i = 0;
#pragma unroll
    for (int k = 0; k < RPL; ++k) {
      const cplx<T> u = ru[k], v = rv[k];
      a = fma(u.re, u.re, fma(u.im, u.im, a));
      b = fma(v.re, v.re, fma(v.im, v.im, b));
      r = fma(u.re, v.re, fma(u.im, v.im, r));
      i = fma(u.re, v.im, fma(-u.im, v.re, i));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
      r += __shfl_xor_sync(0xffffffffu, r, o);
      i += __shfl_xor_sync(0xffffffffu, i, o);
    }
    al = a;
    be = b;
    gr = r;
    gi = i;
  }
}

template <typename T, int RPL>
__global__ void __launch_bounds__(kSvdThreads) svd_cluster_kernel(const SvdDesc<T>* __restrict__ descs, int cs,
                                                                  int cpc, int v_smem) {
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
  const int Dl = D.Dl, Dr = D.Dr;
  const int m = 2 * Dl, n = 2 * Dr;
  const bool trans = n > m;
  const int mx = trans ? n : m;
  const int nx = trans ? m : n;
  const long long blk = (long long)Dl * Dr;
  // V columns: after X in shared memory, or slot-major in the global workspace
  cplx<T>* Vloc = v_smem ? Xloc + (long long)cpc * mx : D.work + (long long)rank * cpc * nx;
  for (int lc = 0; lc < cpc; ++lc) {
    const int col = rank * cpc + lc;
    if (col >= nx) break;
    for (int row = threadIdx.x; row < nx; row += blockDim.x)
      Vloc[(long long)lc * nx + row] = mk<T>(row == col ? (T)1 : (T)0, (T)0);
  }
  // load my columns of W
  for (int lc = 0; lc < cpc; ++lc) {
    const int col = rank * cpc + lc;
    if (col >= nx) break;
    for (int row = threadIdx.x; row < mx; row += blockDim.x) {
      const int r = trans ? col : row;
      const int c = trans ? row : col;
      const int s1 = r / Dl, a = r - s1 * Dl, s2 = c / Dr, cc = c - s2 * Dr;
      cplx<T> v = D.theta[(long long)(s1 * 2 + s2) * blk + (long long)a * Dr + cc];
      if (trans) v.im = -v.im;
      Xloc[(long long)lc * mx + row] = v;
    }
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
  const double tol = Prec<T>::eps * (sizeof(T) == 4 ? 8.0 : fmax(8.0, 2.0 * sqrt((double)mx)));
  const T floor2 = (T)(16.0 * Prec<T>::eps * Prec<T>::eps * fro);
  int* flag0 = cluster.map_shared_rank(s_flag, 0);
  int sweep = 0;
  for (; sweep < kSvdMaxSweeps; ++sweep) {
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
        cplx<T>* vp = (v_smem ? cluster.map_shared_rank(Xloc, p / cpc) + (long long)cpc * mx
                              : D.work + (long long)(p / cpc) * cpc * nx) + (long long)(p % cpc) * nx;
        cplx<T>* vq = (v_smem ? cluster.map_shared_rank(Xloc, q / cpc) + (long long)cpc * mx
                              : D.work + (long long)(q / cpc) * cpc * nx) + (long long)(q % cpc) * nx;
        // both columns of X and of V staged in registers in one round of (possibly
        // remote) loads; the Gram entries and the rotation in the working precision T
        // (the singular values are re-evaluated in FP64 after convergence)
        cplx<T> ru[RPL], rv[RPL], wu[RPL], wv[RPL];
#pragma unroll
        for (int r = 0; r < RPL; ++r) {
          const int i = lane + 32 * r;
          ru[r] = i < mx ? xp[i] : mk<T>(0, 0);
          rv[r] = i < mx ? xq[i] : mk<T>(0, 0);
          wu[r] = i < nx ? vp[i] : mk<T>(0, 0);
          wv[r] = i < nx ? vq[i] : mk<T>(0, 0);
        }
        T al, be, gr, gi;
        pair_gram<T, RPL>(ru, rv, al, be, gr, gi);
        const T g = sqrt(gr * gr + gi * gi);
        if (!(g > (T)tol * sqrt(al * be)) || al <= floor2 || be <= floor2) continue;
        rotated = 1;
        const T zeta = (be - al) / (2 * g);
        const T t = (zeta >= 0 ? (T)1 : (T)-1) / (fabs(zeta) + sqrt(1 + zeta * zeta));
        const T c = 1 / sqrt(1 + t * t);
        const T s = c * t;
        const T er = gr / g, ei = gi / g;  // e^{i phi}
        // x_p' = c x_p - s e^{-i phi} x_q ; x_q' = s e^{i phi} x_p + c x_q  (unitary)
        const T cc = c;
        const cplx<T> smq = mk<T>(-s * er, s * ei);
        const cplx<T> spq = mk<T>(s * er, s * ei);
#pragma unroll
        for (int r = 0; r < RPL; ++r) {
          const int i = lane + 32 * r;
          if (i < mx) {
            xp[i] = cc * ru[r] + smq * rv[r];
            xq[i] = spq * ru[r] + cc * rv[r];
          }
          if (i < nx) {
            vp[i] = cc * wu[r] + smq * wv[r];
            vq[i] = spq * wu[r] + cc * wv[r];
          }
        }
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
  // column norms (FP64) gathered in CTA 0
  double* snorm0 = cluster.map_shared_rank(snorm, 0);
  for (int lc = wid; lc < cpc; lc += nw) {
    const int col = rank * cpc + lc;
    if (col >= nx) break;
    const cplx<T>* x = Xloc + (long long)lc * mx;
    double s = 0.0;
    for (int i = lane; i < mx; i += 32) s += (double)x[i].re * x[i].re + (double)x[i].im * x[i].im;
    s = warp_sum(s);
    if (lane == 0) snorm0[col] = sqrt(s);
  }
  cluster.sync();
  if (rank == 0) {
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
      s_k = k;
      s_keep = sqrt(keep);
      *D.k_out = k;
      if (D.discarded) *D.discarded += total > 0 ? (total - keep) / total : 0.0;
      for (int i = 0; i < nx; ++i) D.sv[i] = snorm[perm[i]];
      if (D.status) {
        D.status[0] = (sweep >= kSvdMaxSweeps) ? QCA_ERR_NOT_CONVERGED : 0;
        D.status[1] = sweep + 1;  // sweeps used
      }
    }
  }
  cluster.sync();
  const int k = *cluster.map_shared_rank(&s_k, 0);
  const double keep = *cluster.map_shared_rank(&s_keep, 0);
  const int* perm0 = cluster.map_shared_rank(perm, 0);
  const double* sn0 = cluster.map_shared_rank(snorm, 0);
  // kept columns that live in this CTA
  for (int i = 0; i < k; ++i) {
    const int j = perm0[i];
    if (j / cpc != rank) continue;
    const cplx<T>* x = Xloc + (long long)(j % cpc) * mx;
    const cplx<T>* v = Vloc + (long long)(j % cpc) * nx;
    const double sig = sn0[j];
    const double inv = sig > 0 ? 1.0 / sig : 0.0;
    const double sn = keep > 0 ? sig / keep : 0.0;  // renormalised singular value
    const double fl = D.right_sweep ? 1.0 : sn;     // scale of A_l
    const double fr = D.right_sweep ? sn : 1.0;     // scale of A_r
    if (!trans) {
      // U[:, i] = x / sigma over the m = mx rows (row = s1 * Dl + a); Vh[i, c] = conj(v[c])
      for (int row = threadIdx.x; row < mx; row += blockDim.x) {
        const cplx<T> u = x[row];
        const double f = inv * fl;
        D.Al[(long long)row * k + i] = mk<T>((T)(u.re * f), (T)(u.im * f));
      }
      for (int c = threadIdx.x; c < nx; c += blockDim.x) {
        const cplx<T> u = v[c];
        const int s2 = c / Dr, cc = c - s2 * Dr;
        D.Ar[((long long)s2 * k + i) * Dr + cc] = mk<T>((T)(u.re * fr), (T)(-u.im * fr));
      }
    } else {
      // U[:, i] = v over the m = nx rows; Vh[i, c] = conj(x[c]) / sigma over the n = mx columns
      for (int row = threadIdx.x; row < nx; row += blockDim.x) {
        const cplx<T> u = v[row];
        D.Al[(long long)row * k + i] = mk<T>((T)(u.re * fl), (T)(u.im * fl));
      }
      for (int c = threadIdx.x; c < mx; c += blockDim.x) {
        const cplx<T> u = x[c];
        const double f = inv * fr;
        const int s2 = c / Dr, cc = c - s2 * Dr;
        D.Ar[((long long)s2 * k + i) * Dr + cc] = mk<T>((T)(u.re * f), (T)(-u.im * f));
      }
    }
  }
  // CTA 0's shared memory (perm, norms, k) is read through DSMEM above: no CTA may
  // exit before every CTA of the cluster is done with it.
  cluster.sync();
}

template <typename T>
int svd_cluster_plan(int mx, int nx, int* cs, int* cpc, size_t* smem, int* v_smem) {
  const size_t es = sizeof(cplx<T>);
  const size_t limit = 200 * 1024;
  const int pairs = (nx + 1) / 2, warps = kSvdThreads / 32;
  for (int vs = 1; vs >= 0; --vs) {
    for (int c = 1; c <= 16; c *= 2) {
      const int per = (nx + c - 1) / c;
      const size_t bytes = (size_t)per * (mx + (vs ? nx : 0)) * es;
      // enough warps in the cluster for one column pair each per round
      if (bytes <= limit && (c * warps >= pairs || c == 16)) {
        *cs = c;
        *cpc = per;
        *smem = bytes;
        *v_smem = vs;
        return QCA_OK;
      }
    }
  }
  return QCA_ERR_INVALID;
}

}  // namespace

// cluster size one problem needs (0 if it does not fit); used to group problems
template <typename T>
int svd_cluster_size(int Dl, int Dr) {
  const int m = 2 * Dl, n = 2 * Dr;
  int cs, cpc, vs;
  size_t sm;
  if (svd_cluster_plan<T>(m > n ? m : n, m > n ? n : m, &cs, &cpc, &sm, &vs) != QCA_OK) return 0;
  return cs;
}

// shared-memory footprint check used by the host before choosing this path
template <typename T>
bool svd_fits(int Dl, int Dr) {
  const int m = 2 * Dl, n = 2 * Dr;
  int cs, cpc, vs;
  size_t sm;
  return svd_cluster_plan<T>(m > n ? m : n, m > n ? n : m, &cs, &cpc, &sm, &vs) == QCA_OK;
}

template <typename T>
int launch_svd(const SvdDesc<T>* d, const SvdDesc<T>* h, int nd, cudaStream_t st) {
  if (nd <= 0) return QCA_OK;
  int mxmax = 1, nxmax = 1;
  for (int i = 0; i < nd; ++i) {
    const int m = 2 * h[i].Dl, n = 2 * h[i].Dr;
    mxmax = std::max(mxmax, std::max(m, n));
    nxmax = std::max(nxmax, std::min(m, n));
  }
  int cs = 1, cpc = 1, vs = 1;
  size_t smem = 0;
  if (svd_cluster_plan<T>(mxmax, nxmax, &cs, &cpc, &smem, &vs) != QCA_OK) {
    set_error("SVD of %d x %d exceeds the distributed shared memory of a 16-CTA cluster", mxmax, nxmax);
    return QCA_ERR_INVALID;
  }
  const int rows = (mxmax + 31) / 32;
  const int rpl = rows <= 2 ? 2 : rows <= 4 ? 4 : rows <= 8 ? 8 : 16;
  if (rows > 16) {
    set_error("SVD column length %d exceeds 512", mxmax);
    return QCA_ERR_INVALID;
  }
  void (*kern)(const SvdDesc<T>*, int, int, int) =
      rpl == 2 ? svd_cluster_kernel<T, 2>
               : rpl == 4 ? svd_cluster_kernel<T, 4> : rpl == 8 ? svd_cluster_kernel<T, 8> : svd_cluster_kernel<T, 16>;
  static bool configured[2][5] = {};
  const int ti = sizeof(T) == 8 ? 0 : 1, ri = rpl == 2 ? 0 : rpl == 4 ? 1 : rpl == 8 ? 2 : 3;
  if (!configured[ti][ri]) {
    QCA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    QCA_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    configured[ti][ri] = true;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(nd * cs, 1, 1);
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
  QCA_CUDA(cudaLaunchKernelEx(&cfg, kern, d, cs, cpc, vs));
  return QCA_OK;
}

template int launch_svd<double>(const SvdDesc<double>*, const SvdDesc<double>*, int, cudaStream_t);
template int launch_svd<float>(const SvdDesc<float>*, const SvdDesc<float>*, int, cudaStream_t);
template bool svd_fits<double>(int, int);
template bool svd_fits<float>(int, int);
template int svd_cluster_size<double>(int, int);
template int svd_cluster_size<float>(int, int);

}  // namespace qca
