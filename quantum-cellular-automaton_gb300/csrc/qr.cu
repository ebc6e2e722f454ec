// Householder QR with LAPACK's conventions (numpy.linalg.qr -> zgeqrf / zungqr),
// used by the MPS gauge moves (mps.py:83-98, 146-192) and by 1TDVP's complete
// QR (tdvp.py:74, 95).  Reproducing the reflector convention matters: 1TDVP
// grows bonds with the complement columns of the complete Q, so another QR
// convention would evolve a different state.
//
// For column k, with alpha = A[k,k] and x = A[k+1:, k] (zlarfg):
//   if ||x|| == 0 and Im(alpha) == 0:   tau = 0 (H = I)
//   else beta = -sign(Re alpha) * |(alpha, ||x||)|,  tau = (beta - alpha) / beta,
//        v = [1, x / (alpha - beta)],  A[k,k] = beta
// and H^H = I - conj(tau) v v^H is applied to the trailing columns (zgeqr2).
// Q = H_0 H_1 ... H_{K-1} is formed explicitly by backward accumulation
// (zung2r), m x m for the complete factorisation.  One CTA per problem.  Sums in
// FP64, except for the mixed path's gauge moves (Acc = float): there the
// reflector is scaled by the reciprocal of alpha - beta (as zlarfg does) and the
// dot products of the reflector applications accumulate in FP32, the precision of
// the stored tensors (FP64 runs at 1/64 of the FP32 rate on this GPU).
#include "tdvp_kernels.cuh"

namespace qca {

namespace {

constexpr int kQrThreads = 512;

template <typename T>
__device__ __forceinline__ cplx<T> cdiv(cplx<double> a, cplx<double> b) {
  // a / b in FP64 (Smith's algorithm is unnecessary at these magnitudes)
  const double d = b.re * b.re + b.im * b.im;
  return mk<T>((T)((a.re * b.re + a.im * b.im) / d), (T)((a.im * b.re - a.re * b.im) / d));
}

template <typename T, typename Acc>
__global__ void __launch_bounds__(kQrThreads) qr_kernel(const QrDesc<T>* __restrict__ descs) {
  const QrDesc<T>& D = descs[blockIdx.x];
  __shared__ double red[33];
  __shared__ double s_tr, s_ti;
  const int m = D.m, n = D.n;
  const int K = m < n ? m : n;
  cplx<T>* A = D.work;                       // column-major m x n
  cplx<T>* Q = D.work + (long long)m * n;    // column-major m x qc
  const int qc = D.complete ? m : K;
  const int csplit = D.csplit > 0 ? D.csplit : n;
  for (long long e = threadIdx.x; e < (long long)m * n; e += blockDim.x) {
    const int c = (int)(e / m), r = (int)(e - (long long)c * m);
    cplx<T> v = D.in[(r / D.rsplit) * D.sIr1 + (r % D.rsplit) * D.sIr0 + (c / csplit) * D.sIc1 + (c % csplit) * D.sIc];
    if (D.conj_in) v.im = -v.im;
    A[e] = v;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k = 0; k < K; ++k) {
    cplx<T>* col = A + (long long)k * m;
    // squares in FP64: an FP32 square underflows below |x| ~ 1e-22, and the residue
    // columns of rank-deficient matrices (1TDVP's complete QRs) reach that range;
    // an underflowed norm makes beta come from alpha alone, v = x / (alpha - beta)
    // huge and the reflector far from unitary
    double xs = 0.0;
    for (int i = k + 1 + threadIdx.x; i < m; i += blockDim.x) {
      const cplx<T> x = col[i];
      xs += (double)x.re * (double)x.re + (double)x.im * (double)x.im;
    }
    xs = block_sum(xs, red);
    const cplx<T> al = col[k];
    const double ar = al.re, ai = al.im;
    double tr = 0.0, ti = 0.0;
    if (!(xs == 0.0 && ai == 0.0)) {
      const double bnorm = sqrt(ar * ar + ai * ai + xs);
      const double beta = ar >= 0 ? -bnorm : bnorm;
      tr = (beta - ar) / beta;
      ti = -ai / beta;
      const cplx<double> den = mk<double>(ar - beta, ai);
      // |x_i / (alpha - beta)| <= 1 always, but the reciprocal of alpha - beta
      // leaves the FP32 range for columns below ~1e-38 (denormal rounding residue):
      // those divide element by element in FP64 instead of turning into inf * 0.
      if (sizeof(Acc) == 8 || bnorm < 1e-30) {
        for (int i = k + 1 + threadIdx.x; i < m; i += blockDim.x) {
          const cplx<T> x = col[i];
          col[i] = cdiv<T>(mk<double>((double)x.re, (double)x.im), den);
        }
      } else {
        const double dd = den.re * den.re + den.im * den.im;
        const cplx<T> inv = mk<T>((T)(den.re / dd), (T)(-den.im / dd));
        for (int i = k + 1 + threadIdx.x; i < m; i += blockDim.x) col[i] = col[i] * inv;
      }
      __syncthreads();
      if (threadIdx.x == 0) col[k] = mk<T>((T)beta, (T)0);
    }
    if (threadIdx.x == 0) {
      s_tr = tr;
      s_ti = ti;
      D.tau[k] = mk<T>((T)tr, (T)ti);
    }
    __syncthreads();
    if (tr != 0.0 || ti != 0.0) {
      // trailing columns j > k: a_j -= conj(tau) v (v^H a_j)
      for (int j = k + 1 + wid; j < n; j += nw) {
        cplx<T>* aj = A + (long long)j * m;
        Acc wr = 0, wi = 0;
        for (int i = k + lane; i < m; i += 32) {
          const cplx<T> v = i == k ? mk<T>(1, 0) : col[i];
          const cplx<T> a = aj[i];
          wr += (Acc)v.re * a.re + (Acc)v.im * a.im;
          wi += (Acc)v.re * a.im - (Acc)v.im * a.re;
        }
        wr = warp_sum(wr);
        wi = warp_sum(wi);
        // f = conj(tau) * w
        const Acc fr = (Acc)tr * wr + (Acc)ti * wi;
        const Acc fi = (Acc)tr * wi - (Acc)ti * wr;
        for (int i = k + lane; i < m; i += 32) {
          const cplx<T> v = i == k ? mk<T>(1, 0) : col[i];
          cplx<T> a = aj[i];
          a.re -= (T)(fr * v.re - fi * v.im);
          a.im -= (T)(fr * v.im + fi * v.re);
          aj[i] = a;
        }
      }
    }
    __syncthreads();
  }
  // Q = H_0 ... H_{K-1} [I]_{:, :qc}, only when it is asked for
  for (long long e = threadIdx.x; D.q && e < (long long)m * qc; e += blockDim.x) {
    const int c = (int)(e / m), r = (int)(e - (long long)c * m);
    Q[e] = mk<T>(r == c ? (T)1 : (T)0, (T)0);
  }
  __syncthreads();
  for (int k = D.q ? K - 1 : -1; k >= 0; --k) {
    const cplx<T> t = D.tau[k];
    const double tr = t.re, ti = t.im;
    if (tr == 0.0 && ti == 0.0) continue;
    const cplx<T>* col = A + (long long)k * m;
    for (int j = k + wid; j < qc; j += nw) {
      cplx<T>* qj = Q + (long long)j * m;
      Acc wr = 0, wi = 0;
      for (int i = k + lane; i < m; i += 32) {
        const cplx<T> v = i == k ? mk<T>(1, 0) : col[i];
        const cplx<T> a = qj[i];
        wr += (Acc)v.re * a.re + (Acc)v.im * a.im;
        wi += (Acc)v.re * a.im - (Acc)v.im * a.re;
      }
      wr = warp_sum(wr);
      wi = warp_sum(wi);
      // H_k q = q - tau v (v^H q)
      const Acc fr = (Acc)tr * wr - (Acc)ti * wi;
      const Acc fi = (Acc)tr * wi + (Acc)ti * wr;
      for (int i = k + lane; i < m; i += 32) {
        const cplx<T> v = i == k ? mk<T>(1, 0) : col[i];
        cplx<T> a = qj[i];
        a.re -= (T)(fr * v.re - fi * v.im);
        a.im -= (T)(fr * v.im + fi * v.re);
        qj[i] = a;
      }
    }
    __syncthreads();
  }
  // outputs through strides, zero padded / truncated
  if (D.q) {
    for (long long e = threadIdx.x; e < (long long)D.qrows_out * D.qcols_out; e += blockDim.x) {
      const int c = (int)(e % D.qcols_out), r = (int)(e / D.qcols_out);
      cplx<T> v = mk<T>(0, 0);
      if (r < m && c < qc) v = Q[(long long)c * m + r];
      D.q[(r / D.qsplit) * D.sQr1 + (r % D.qsplit) * D.sQr0 + c * D.sQc] = v;
    }
  }
  if (D.rr) {
    const int rrows = D.complete ? m : K;
    for (long long e = threadIdx.x; e < (long long)D.rrows_out * D.rcols_out; e += blockDim.x) {
      const int c = (int)(e % D.rcols_out), r = (int)(e / D.rcols_out);
      cplx<T> v = mk<T>(0, 0);
      if (r < rrows && c < n && r <= c) v = A[(long long)c * m + r];
      D.rr[r * D.sRr + c * D.sRc] = v;
    }
  }
}

}  // namespace

template <typename T>
int launch_qr(const QrDesc<T>* d, int nd, int gauge, cudaStream_t st) {
  if (nd <= 0) return QCA_OK;
  if (gauge && sizeof(T) == 4)
    qr_kernel<T, float><<<nd, kQrThreads, 0, st>>>(d);
  else
    qr_kernel<T, double><<<nd, kQrThreads, 0, st>>>(d);
  QCA_LAUNCH_CHECK();
  count_launches(1);
  return QCA_OK;
}

template int launch_qr<double>(const QrDesc<double>*, int, int, cudaStream_t);
template int launch_qr<float>(const QrDesc<float>*, int, int, cudaStream_t);

}  // namespace qca
