// Two-site split of 2TDVP (tdvp.py:286-296): SVD of theta viewed as the
// (2 Dl) x (2 Dr) matrix Theta[(s1,a),(s2,c)], truncation to
//   k = min{ i : ||s[i:]||_2 < eps }  capped at min(chi, len s)
// and the new site tensors (right sweep: A_l = U, A_r = diag(s) Vh;
// left sweep: A_l = U diag(s), A_r = Vh) with s renormalised (lautils.normalize).
//
// One CTA per problem runs a one-sided (Hestenes) Jacobi SVD on the narrower
// orientation X (mx >= nx columns): column pairs are rotated in parallel in a
// round-robin tournament until every pair is orthogonal to working precision.
// Singular values are the FP64 norms of the final columns; the tail sums of the
// truncation rule are accumulated in FP64.
#include "tdvp_kernels.cuh"

namespace qca {

namespace {

constexpr int kSvdThreads = 1024;
constexpr int kSvdMaxN = 1024;

template <typename T>
struct Eps;
template <>
struct Eps<double> {
  static constexpr double v = 1e-15;
};
template <>
struct Eps<float> {
  static constexpr double v = 1e-7;
};

template <typename T>
__global__ void __launch_bounds__(kSvdThreads) svd_kernel(const SvdDesc<T>* __restrict__ descs) {
  const SvdDesc<T>& D = descs[blockIdx.x];
  __shared__ double snorm[kSvdMaxN];
  __shared__ int perm[kSvdMaxN];
  __shared__ int s_rot;
  __shared__ int s_k;
  __shared__ double s_keep;
  const int Dl = D.Dl, Dr = D.Dr;
  const int m = 2 * Dl, n = 2 * Dr;
  const bool trans = n > m;
  const int mx = trans ? n : m;
  const int nx = trans ? m : n;
  cplx<T>* X = D.work;                   // column-major mx x nx
  cplx<T>* V = D.work + (long long)mx * nx;  // column-major nx x nx
  const long long blk = (long long)Dl * Dr;
  // load X and V = I
  for (long long e = threadIdx.x; e < (long long)mx * nx; e += blockDim.x) {
    const int col = (int)(e / mx), row = (int)(e - (long long)col * mx);
    // Theta(r, c): r = (s1, a), c = (s2, cc)
    const int r = trans ? col : row;
    const int c = trans ? row : col;
    const int s1 = r / Dl, a = r - s1 * Dl, s2 = c / Dr, cc = c - s2 * Dr;
    cplx<T> v = D.theta[(long long)(s1 * 2 + s2) * blk + (long long)a * Dr + cc];
    if (trans) v.im = -v.im;
    X[e] = v;
  }
  for (long long e = threadIdx.x; e < (long long)nx * nx; e += blockDim.x) {
    const int col = (int)(e / nx), row = (int)(e - (long long)col * nx);
    V[e] = mk<T>(row == col ? (T)1 : (T)0, (T)0);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int P = nx + (nx & 1);
  const double tol = Eps<T>::v * 4.0;
  int sweep = 0;
  for (; sweep < 40; ++sweep) {
    if (threadIdx.x == 0) s_rot = 0;
    __syncthreads();
    int rotated = 0;
    for (int round = 0; round < P - 1; ++round) {
      for (int pk = wid; pk < P / 2; pk += nw) {
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
        cplx<T>* xp = X + (long long)p * mx;
        cplx<T>* xq = X + (long long)q * mx;
        double al = 0.0, be = 0.0, gr = 0.0, gi = 0.0;
        for (int i = lane; i < mx; i += 32) {
          const cplx<T> u = xp[i], v = xq[i];
          al += (double)u.re * u.re + (double)u.im * u.im;
          be += (double)v.re * v.re + (double)v.im * v.im;
          gr += (double)u.re * v.re + (double)u.im * v.im;  // conj(u) v
          gi += (double)u.re * v.im - (double)u.im * v.re;
        }
        al = warp_sum(al);
        be = warp_sum(be);
        gr = warp_sum(gr);
        gi = warp_sum(gi);
        const double g = sqrt(gr * gr + gi * gi);
        if (!(g > tol * sqrt(al * be)) || g == 0.0) continue;
        rotated = 1;
        const double zeta = (be - al) / (2.0 * g);
        const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / sqrt(1.0 + t * t);
        const double s = c * t;
        const double er = gr / g, ei = gi / g;  // e^{i phi}
        // x_p' = c x_p - s e^{-i phi} x_q ; x_q' = s e^{i phi} x_p + c x_q
        const T cc = (T)c;
        const cplx<T> smq = mk<T>((T)(-s * er), (T)(s * ei));   // -s e^{-i phi}
        const cplx<T> spq = mk<T>((T)(s * er), (T)(s * ei));    // s e^{i phi}
        for (int i = lane; i < mx; i += 32) {
          const cplx<T> u = xp[i], v = xq[i];
          xp[i] = cc * u + smq * v;
          xq[i] = spq * u + cc * v;
        }
        cplx<T>* vp = V + (long long)p * nx;
        cplx<T>* vq = V + (long long)q * nx;
        for (int i = lane; i < nx; i += 32) {
          const cplx<T> u = vp[i], v = vq[i];
          vp[i] = cc * u + smq * v;
          vq[i] = spq * u + cc * v;
        }
      }
      __syncthreads();
    }
    if (rotated) s_rot = 1;
    __syncthreads();
    if (!s_rot) break;
    __syncthreads();
  }
  // singular values (FP64 column norms) and descending order
  for (int j = wid; j < nx; j += nw) {
    const cplx<T>* xj = X + (long long)j * mx;
    double s = 0.0;
    for (int i = lane; i < mx; i += 32) s += (double)xj[i].re * xj[i].re + (double)xj[i].im * xj[i].im;
    s = warp_sum(s);
    if (lane == 0) snorm[j] = sqrt(s);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < nx; j += blockDim.x) {
    const double sj = snorm[j];
    int rank = 0;
    for (int i = 0; i < nx; ++i) {
      const double si = snorm[i];
      rank += (si > sj) || (si == sj && i < j);
    }
    perm[rank] = j;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // tail norms ||s[i:]|| in FP64; first i below eps (tdvp.py:290-292)
    const int len = nx;
    int k = len;
    double tail = 0.0, total = 0.0;
    for (int i = len - 1; i >= 0; --i) total += snorm[perm[i]] * snorm[perm[i]];
    double acc = 0.0;
    int first = len;
    for (int i = len - 1; i >= 0; --i) {
      acc += snorm[perm[i]] * snorm[perm[i]];
      if (sqrt(acc) < D.eps) first = i;
    }
    k = first;
    const int cap = D.chi < len ? D.chi : len;
    if (k > cap) k = cap;
    if (k > D.kmax) k = D.kmax;
    if (k < 1) k = 1;
    double keep = 0.0;
    for (int i = 0; i < k; ++i) keep += snorm[perm[i]] * snorm[perm[i]];
    tail = total - keep;
    s_k = k;
    s_keep = sqrt(keep);
    *D.k_out = k;
    if (D.discarded) *D.discarded += total > 0 ? tail / total : 0.0;
    for (int i = 0; i < len; ++i) D.sv[i] = snorm[perm[i]];
    if (D.status) *D.status = (sweep >= 40) ? QCA_ERR_NOT_CONVERGED : 0;
  }
  __syncthreads();
  const int k = s_k;
  const double keep = s_keep;
  // U (m x k) and Vh (k x n) of Theta
  //  not trans: U[:, i] = X[:, perm i] / sigma, Vh[i, c] = conj(V[c, perm i])
  //  trans:     U[:, i] = V[:, perm i],          Vh[i, c] = conj(X[c, perm i]) / sigma
  for (long long e = threadIdx.x; e < (long long)m * k; e += blockDim.x) {
    const int i = (int)(e % k);
    const int r = (int)(e / k);
    const int j = perm[i];
    const double sig = snorm[j];
    cplx<T> u;
    if (!trans) {
      const cplx<T> x = X[(long long)j * mx + r];
      const double f = sig > 0 ? 1.0 / sig : 0.0;
      u = mk<T>((T)(x.re * f), (T)(x.im * f));
    } else {
      u = V[(long long)j * nx + r];
    }
    if (!D.right_sweep) {
      const double sn = keep > 0 ? sig / keep : 0.0;
      u = mk<T>((T)(u.re * sn), (T)(u.im * sn));
    }
    // A_l[s1][a][i], r = s1 * Dl + a
    D.Al[(long long)r * k + i] = u;
  }
  for (long long e = threadIdx.x; e < (long long)n * k; e += blockDim.x) {
    const int c = (int)(e % n);
    const int i = (int)(e / n);
    const int j = perm[i];
    const double sig = snorm[j];
    cplx<T> v;
    if (!trans) {
      v = conj(V[(long long)j * nx + c]);
    } else {
      const cplx<T> x = X[(long long)j * mx + c];
      const double f = sig > 0 ? 1.0 / sig : 0.0;
      v = mk<T>((T)(x.re * f), (T)(-x.im * f));
    }
    if (D.right_sweep) {
      const double sn = keep > 0 ? sig / keep : 0.0;
      v = mk<T>((T)(v.re * sn), (T)(v.im * sn));
    }
    // A_r[s2][i][cc], c = s2 * Dr + cc
    const int s2 = c / Dr, cc = c - s2 * Dr;
    D.Ar[((long long)s2 * k + i) * Dr + cc] = v;
  }
}

}  // namespace

template <typename T>
int launch_svd(const SvdDesc<T>* d, int nd, cudaStream_t st) {
  if (nd <= 0) return QCA_OK;
  svd_kernel<T><<<nd, kSvdThreads, 0, st>>>(d);
  QCA_LAUNCH_CHECK();
  return QCA_OK;
}

template int launch_svd<double>(const SvdDesc<double>*, int, cudaStream_t);
template int launch_svd<float>(const SvdDesc<float>*, int, cudaStream_t);

}  // namespace qca
