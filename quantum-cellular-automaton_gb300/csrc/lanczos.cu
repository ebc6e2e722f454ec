// Lanczos exponential, sparse MPO application and elementwise helpers of the
// TDVP engine.
//
// The reference evolves every local tensor with a dense eigendecomposition of
// the assembled effective Hamiltonian (lautils.py:44-81, tdvp.py:349-365,
// tdvp.py:164-188).  Here v <- exp(-i tau H_eff) v is computed by Lanczos with
// the basis resident on the device and classical Gram-Schmidt applied twice
// (projections accumulated in FP64).  At the convergence check points (every
// third iteration, at the iteration limit and when the Krylov space is exhausted:
// m = n, or beta_j at the rounding level of ||H v_j||) one warp per problem
// evaluates exp(-i tau T) e_1 of the tridiagonal T by a sub-stepped Taylor series
// (FP64) and stops when beta_j |(exp(-i tau T) e_1)_j| < tol; in between it only
// records beta_j.  A finished problem's later launches return at once (done flag).
#include "tdvp_kernels.cuh"

namespace qca {

namespace {

constexpr int kLzThreads = 256;
constexpr int kLzPer = kLzChunk / kLzThreads;  // elements per thread
constexpr int kPartStride = kLzPartStride;

// rounding level of the Lanczos recurrence relative to ||H v_j|| (vectors stored in
// T, matrix-vector products accumulated over long sums): a beta_j below it is
// indistinguishable from zero
template <typename T>
__device__ __forceinline__ double lz_noise() {
  return sizeof(T) == 4 ? 64.0 * 1.2e-7 : 64.0 * 2.2e-16;
}

template <typename D>
__device__ __forceinline__ int find_tile(const D* d, int nd, int tile) {
  int lo = 0, hi = nd - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (d[mid].tile_begin <= tile)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// ----------------------------------------------------------------------------------
// W application
// ----------------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) wapply_kernel(const WapplyDesc<T>* __restrict__ descs, int nd) {
  const int di = find_tile(descs, nd, blockIdx.x);
  const WapplyDesc<T>& D = descs[di];
  if (D.skip && *D.skip) return;
  const int t = blockIdx.x - D.tile_begin;
  const int ob = t / D.chunks;
  const int ch = t - ob * D.chunks;
  if (ob >= D.nout) return;
  const int e0 = D.out_begin[ob], e1 = D.out_begin[ob + 1];
  const long long base = (long long)ch * 1024;
  cplx<T>* out = D.out + (long long)ob * D.blk;
  for (int r = 0; r < 4; ++r) {
    const long long idx = base + r * 256 + threadIdx.x;
    if (idx >= D.blk) break;
    cplx<T> acc = mk<T>(0, 0);
    for (int e = e0; e < e1; ++e) {
      const WEntry w = D.ent[e];
      const cplx<T> v = D.in[(long long)w.in_block * D.blk + idx];
      cfma(acc, mk<T>((T)w.re, (T)w.im), v);
    }
    out[idx] = acc;
  }
}

// ----------------------------------------------------------------------------------
// Lanczos vector kernels
// ----------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void load_chunk(const cplx<T>* v, long long n, long long base, cplx<T> (&r)[kLzPer]) {
#pragma unroll
  for (int q = 0; q < kLzPer; ++q) {
    const long long i = base + q * kLzThreads + threadIdx.x;
    r[q] = i < n ? v[i] : mk<T>(0, 0);
  }
}

// partial ||in||^2 per chunk
template <typename T>
__global__ void __launch_bounds__(kLzThreads) lz_norm_kernel(const LanczosDesc<T>* __restrict__ descs, int nd) {
  __shared__ double red[33];
  const int di = find_tile(descs, nd, blockIdx.x);
  const LanczosDesc<T>& D = descs[di];
  const int ch = blockIdx.x - D.tile_begin;
  const long long base = (long long)ch * kLzChunk;
  cplx<T> r[kLzPer];
  load_chunk(D.in, D.n, base, r);
  double s = 0.0;
#pragma unroll
  for (int q = 0; q < kLzPer; ++q) s += (double)r[q].re * r[q].re + (double)r[q].im * r[q].im;
  s = block_sum(s, red);
  if (threadIdx.x == 0) D.S[LZ_PART + ch] = s;
}

// slot0 = in / ||in||; resets the scalar block
template <typename T>
__global__ void __launch_bounds__(kLzThreads) lz_init_kernel(const LanczosDesc<T>* __restrict__ descs, int nd,
                                                             double tol) {
  __shared__ double red[33];
  const int di = find_tile(descs, nd, blockIdx.x);
  const LanczosDesc<T>& D = descs[di];
  const int ch = blockIdx.x - D.tile_begin;
  double s = 0.0;
  for (int i = threadIdx.x; i < D.chunks; i += blockDim.x) s += D.S[LZ_PART + i];
  s = block_sum(s, red);
  const double nrm = sqrt(s);
  const double inv = nrm > 0.0 ? 1.0 / nrm : 0.0;
  const long long base = (long long)ch * kLzChunk;
  cplx<T> r[kLzPer];
  load_chunk(D.in, D.n, base, r);
#pragma unroll
  for (int q = 0; q < kLzPer; ++q) {
    const long long i = base + q * kLzThreads + threadIdx.x;
    if (i < D.n) D.V[i] = mk<T>((T)(r[q].re * inv), (T)(r[q].im * inv));
  }
  // scalar reset: done by CTA 0 after all CTAs of this problem read the partials.
  // Partials are not touched again until lz_orth, launched later on the stream.
  if (ch == 0 && threadIdx.x == 0) {
    D.S[LZ_NORM0] = nrm;
    D.S[LZ_M] = 1.0;
    D.S[LZ_MEFF] = 1.0;
    D.S[LZ_INVB] = 0.0;
    D.S[LZ_FLAG] = isfinite(nrm) ? 0.0 : 1.0;
    if (!isfinite(nrm) && D.status) atomicOr(D.status, kLzStatusNonFinite);
    D.S[LZ_TOL] = tol;
    D.S[LZ_COEF] = nrm;  // exp of an empty Krylov space: v itself
    D.S[LZ_COEF + 1] = 0.0;
    reinterpret_cast<int*>(D.S + LZ_DONE)[0] = (nrm > 0.0 && isfinite(nrm)) ? 0 : 1;
  }
}

// Classical Gram-Schmidt pass on w = slot j+1 against slots 0..j.
// pass 0: h = V^H w (partials), pass 1: reduce h, w -= V h, h' = V^H w (partials),
// pass 2: reduce h', w -= V h', ||w||^2 (partials), alpha_j = Re(h_j + h'_j).
template <typename T>
__global__ void __launch_bounds__(kLzThreads) lz_orth_kernel(const LanczosDesc<T>* __restrict__ descs, int nd, int j,
                                                             int pass) {
  __shared__ double hs[2 * kLzMax];
  __shared__ double wsum[kLzThreads / 32][2 * kLzMax + 2];
  const int di = find_tile(descs, nd, blockIdx.x);
  const LanczosDesc<T>& D = descs[di];
  if (reinterpret_cast<const int*>(D.S + LZ_DONE)[0]) return;
  const int ch = blockIdx.x - D.tile_begin;
  double* P = D.P;  // [2 buffers][chunks][kPartStride]
  const long long base = (long long)ch * kLzChunk;
  cplx<T>* w = D.V + (long long)(j + 1) * D.ld;
  cplx<T> r[kLzPer];
  load_chunk(w, D.n, base, r);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (pass >= 1) {
    // reduce the previous pass's projections
    const double* Pin = P + (long long)((pass - 1) & 1) * D.chunks * kPartStride;
    for (int i = threadIdx.x; i < 2 * (j + 1); i += blockDim.x) {
      double s = 0.0;
      for (int c = 0; c < D.chunks; ++c) s += Pin[(long long)c * kPartStride + i];
      hs[i] = s;
    }
    __syncthreads();
    if (ch == 0 && threadIdx.x == 0) {
      if (pass == 1) {
        D.S[LZ_H + 2 * j] = hs[2 * j];
      } else {
        D.S[LZ_ALPHA + j] = D.S[LZ_H + 2 * j] + hs[2 * j];
      }
    }
    for (int i = 0; i <= j; ++i) {
      const cplx<T> h = mk<T>((T)hs[2 * i], (T)hs[2 * i + 1]);
      const cplx<T>* v = D.V + (long long)i * D.ld;
#pragma unroll
      for (int q = 0; q < kLzPer; ++q) {
        const long long idx = base + q * kLzThreads + threadIdx.x;
        if (idx < D.n) {
          const cplx<T> vv = v[idx];
          r[q] = r[q] - h * vv;
        }
      }
    }
#pragma unroll
    for (int q = 0; q < kLzPer; ++q) {
      const long long idx = base + q * kLzThreads + threadIdx.x;
      if (idx < D.n) w[idx] = r[q];
    }
  }
  double* Pout = P + (long long)(pass & 1) * D.chunks * kPartStride + (long long)ch * kPartStride;
  if (pass < 2) {
    // projections h_i = <v_i, w>: products and the per-thread partial sum in the
    // element precision T, the sums across threads and chunks in FP64
    for (int i = 0; i <= j; ++i) {
      const cplx<T>* v = D.V + (long long)i * D.ld;
      T tr = 0, ti = 0;
#pragma unroll
      for (int q = 0; q < kLzPer; ++q) {
        const long long idx = base + q * kLzThreads + threadIdx.x;
        if (idx < D.n) {
          const cplx<T> vv = v[idx];
          tr = fma(vv.re, r[q].re, tr);
          tr = fma(vv.im, r[q].im, tr);
          ti = fma(vv.re, r[q].im, ti);
          ti = fma(-vv.im, r[q].re, ti);
        }
      }
      double sr = warp_sum((double)tr);
      double si = warp_sum((double)ti);
      if (lane == 0) {
        wsum[wid][2 * i] = sr;
        wsum[wid][2 * i + 1] = si;
      }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * (j + 1); i += blockDim.x) {
      double s = 0.0;
#pragma unroll
      for (int q = 0; q < kLzThreads / 32; ++q) s += wsum[q][i];
      Pout[i] = s;
    }
  } else {
    T t = 0;
#pragma unroll
    for (int q = 0; q < kLzPer; ++q) t = fma(r[q].re, r[q].re, fma(r[q].im, r[q].im, t));
    const double s = warp_sum((double)t);
    if (lane == 0) wsum[wid][0] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int q = 0; q < kLzThreads / 32; ++q) t += wsum[q][0];
      Pout[0] = t;
    }
  }
}

// One warp per problem: beta_j, exp(-i tau T) e_1, convergence.
template <typename T>
__global__ void lz_finalize_kernel(const LanczosDesc<T>* __restrict__ descs, int nd, int j, int mmax, int check) {
  __shared__ double yr[64], yi[64], tr[64], ti[64], nr[64], ni[64];
  const int di = blockIdx.x;
  const LanczosDesc<T>& D = descs[di];
  double* S = D.S;
  int* done = reinterpret_cast<int*>(S + LZ_DONE);
  if (*done) {
    if (threadIdx.x == 0 && D.done_out) *D.done_out = 1;
    return;
  }
  const int lane = threadIdx.x;
  const double* Pin = D.P;  // pass 2 wrote buffer 0
  double bsq = 0.0;
  for (int c = lane; c < D.chunks; c += 32) bsq += Pin[(long long)c * kPartStride];
  bsq = warp_sum(bsq);
  const double beta = sqrt(bsq);
  const int m = j + 1;  // T is m x m: alpha_0..alpha_j, beta_0..beta_{j-1}
  // The Krylov space is exhausted when it spans the whole problem (m = n) or when
  // beta_j falls to the rounding level of the recurrence w = H v_j - alpha_j v_j -
  // beta_{j-1} v_{j-1}, whose terms are of size ||H v_j|| (this includes the energy
  // of the rest of the chain carried by the environments, large on long chains):
  // a vector normalised from that residue is rounding noise, not orthogonal to the
  // basis, and continuing from it corrupts T.  T is then exact to working
  // precision and the exponential is taken from it.
  const double ja = S[LZ_ALPHA + j], jb = j > 0 ? S[LZ_BETA + j - 1] : 0.0;
  const bool exhausted = (long long)m >= D.n || beta <= lz_noise<T>() * sqrt(ja * ja + jb * jb);
  if (!check && !exhausted && isfinite(beta) && beta >= S[LZ_TOL] * 1e-3 && m + 1 <= mmax && m + 1 <= kLzMax) {
    // not a convergence check point: record beta_j and continue without the
    // tridiagonal exponential (evaluated at check points, breakdown and the end)
    if (lane == 0) {
      S[LZ_BETA + j] = beta;
      S[LZ_MEFF] = (double)m;
      S[LZ_INVB] = 1.0 / beta;
      S[LZ_M] = (double)(m + 1);
      if (D.done_out) *D.done_out = 0;
    }
    return;
  }
  const double* alpha = S + LZ_ALPHA;
  const double* bet = S + LZ_BETA;
  double rho = 0.0;
  for (int k = 0; k < m; ++k) {
    double r = fabs(alpha[k]);
    if (k > 0) r += bet[k - 1];
    if (k + 1 < m) r += bet[k];
    rho = fmax(rho, r);
  }
  const double tau = D.tau;
  if (!isfinite(rho) || fabs(tau) * rho > 1e4) {
    // a non-finite or absurd Krylov matrix: report instead of sub-stepping forever
    if (lane == 0) {
      S[LZ_FLAG] = 1.0;
      S[LZ_MEFF] = (double)m;
      *done = 1;
      if (D.done_out) *D.done_out = 1;
      if (D.status) atomicOr(D.status, kLzStatusNonFinite);
    }
    return;
  }
  const int q = max(1, (int)ceil(fabs(tau) * rho));
  const double h = tau / q;
  for (int k = lane; k < 64; k += 32) {
    yr[k] = k == 0 ? 1.0 : 0.0;
    yi[k] = 0.0;
  }
  __syncwarp();
  for (int sub = 0; sub < q; ++sub) {
    for (int k = lane; k < 64; k += 32) {
      tr[k] = yr[k];
      ti[k] = yi[k];
      nr[k] = yr[k];
      ni[k] = yi[k];
    }
    __syncwarp();
    for (int p = 1; p <= 40; ++p) {
      double ur[2], ui[2], loc = 0.0;
      for (int s = 0; s < 2; ++s) {
        const int k = lane + 32 * s;
        double ar = 0.0, ai = 0.0;
        if (k < m) {
          ar = alpha[k] * tr[k];
          ai = alpha[k] * ti[k];
          if (k > 0) {
            ar += bet[k - 1] * tr[k - 1];
            ai += bet[k - 1] * ti[k - 1];
          }
          if (k + 1 < m) {
            ar += bet[k] * tr[k + 1];
            ai += bet[k] * ti[k + 1];
          }
        }
        const double c = h / p;
        ur[s] = c * ai;
        ui[s] = -c * ar;
        loc = fmax(loc, fabs(ur[s]) + fabs(ui[s]));
      }
      __syncwarp();
      for (int s = 0; s < 2; ++s) {
        const int k = lane + 32 * s;
        tr[k] = ur[s];
        ti[k] = ui[s];
        nr[k] += ur[s];
        ni[k] += ui[s];
      }
      __syncwarp();
      for (int o = 16; o > 0; o >>= 1) loc = fmax(loc, __shfl_xor_sync(0xffffffffu, loc, o));
      if (loc < 1e-18) break;
    }
    for (int k = lane; k < 64; k += 32) {
      yr[k] = nr[k];
      yi[k] = ni[k];
    }
    __syncwarp();
  }
  const double norm0 = S[LZ_NORM0];
  for (int k = lane; k < kLzMax; k += 32) {
    S[LZ_COEF + 2 * k] = k < m ? yr[k] * norm0 : 0.0;
    S[LZ_COEF + 2 * k + 1] = k < m ? yi[k] * norm0 : 0.0;
  }
  __syncwarp();
  if (lane == 0) {
    const double err = beta * sqrt(yr[m - 1] * yr[m - 1] + yi[m - 1] * yi[m - 1]);
    const double tol = S[LZ_TOL];
    const bool finite = isfinite(beta) && isfinite(err);
    S[LZ_BETA + j] = beta;
    S[LZ_MEFF] = (double)m;
    if (!finite) {
      S[LZ_FLAG] = 1.0;
      *done = 1;
      if (D.status) atomicOr(D.status, kLzStatusNonFinite);
    } else if (err < tol || beta < 1e-300 || exhausted || m + 1 > mmax || m + 1 > kLzMax) {
      if (!(err < tol) && !(beta < 1e-300) && !exhausted) {
        S[LZ_FLAG] = 2.0;  // iteration limit reached
        if (D.status) atomicOr(D.status, kLzStatusLimit);
      }
      *done = 1;
    } else if (beta < tol * 1e-3) {
      *done = 1;  // invariant subspace: T is exact
    } else {
      S[LZ_INVB] = 1.0 / beta;
      S[LZ_M] = (double)(m + 1);
    }
    if (D.done_out) *D.done_out = *done;
  }
}

template <typename T>
__global__ void __launch_bounds__(kLzThreads) lz_normalize_kernel(const LanczosDesc<T>* __restrict__ descs, int nd,
                                                                  int j) {
  const int di = find_tile(descs, nd, blockIdx.x);
  const LanczosDesc<T>& D = descs[di];
  if (reinterpret_cast<const int*>(D.S + LZ_DONE)[0]) return;
  const T s = (T)D.S[LZ_INVB];
  const int ch = blockIdx.x - D.tile_begin;
  const long long base = (long long)ch * kLzChunk;
  cplx<T>* w = D.V + (long long)(j + 1) * D.ld;
#pragma unroll
  for (int q = 0; q < kLzPer; ++q) {
    const long long idx = base + q * kLzThreads + threadIdx.x;
    if (idx < D.n) {
      cplx<T> v = w[idx];
      w[idx] = mk<T>(v.re * s, v.im * s);
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kLzThreads) lz_combine_kernel(const LanczosDesc<T>* __restrict__ descs, int nd) {
  __shared__ double cs[2 * kLzMax];
  const int di = find_tile(descs, nd, blockIdx.x);
  const LanczosDesc<T>& D = descs[di];
  const int meff = (int)D.S[LZ_MEFF];
  for (int i = threadIdx.x; i < 2 * kLzMax; i += blockDim.x) cs[i] = D.S[LZ_COEF + i];
  __syncthreads();
  const int ch = blockIdx.x - D.tile_begin;
  const long long base = (long long)ch * kLzChunk;
#pragma unroll
  for (int q = 0; q < kLzPer; ++q) {
    const long long idx = base + q * kLzThreads + threadIdx.x;
    if (idx >= D.n) continue;
    double ar = 0.0, ai = 0.0;
    for (int k = 0; k < meff; ++k) {
      const cplx<T> v = D.V[(long long)k * D.ld + idx];
      ar += cs[2 * k] * (double)v.re - cs[2 * k + 1] * (double)v.im;
      ai += cs[2 * k] * (double)v.im + cs[2 * k + 1] * (double)v.re;
    }
    D.out[idx] = mk<T>((T)ar, (T)ai);
  }
}

// ----------------------------------------------------------------------------------
// strided copy with zero padding and scale
// ----------------------------------------------------------------------------------
template <typename T>
__global__ void copy_kernel(const CopyDesc<T>* __restrict__ descs, int nd) {
  const int di = find_tile(descs, nd, blockIdx.x);
  const CopyDesc<T>& D = descs[di];
  const long long total = (long long)D.n0 * D.n1 * D.n2;
  const long long start = (long long)(blockIdx.x - D.tile_begin) * blockDim.x * 4;
  for (int r = 0; r < 4; ++r) {
    const long long e = start + r * blockDim.x + threadIdx.x;
    if (e >= total) return;
    const int i2 = (int)(e % D.n2);
    const long long e1 = e / D.n2;
    const int i1 = (int)(e1 % D.n1);
    const int i0 = (int)(e1 / D.n1);
    cplx<T> v = mk<T>(0, 0);
    if (i0 < D.m0 && i1 < D.m1 && i2 < D.m2) v = D.src[i0 * D.s0 + i1 * D.s1 + i2 * D.s2];
    D.dst[i0 * D.d0 + i1 * D.d1 + i2 * D.d2] = v;
  }
}

template <typename T>
__global__ void rho_kernel(const RhoDesc<T>* __restrict__ descs) {
  __shared__ double red[33];
  const RhoDesc<T>& D = descs[blockIdx.x];
  const cplx<T>* A = D.A;
  double* out = D.out;
  const long long blk = (long long)D.Dl * D.Dr;
  double r00 = 0, r11 = 0, r01r = 0, r01i = 0;
  for (long long e = threadIdx.x; e < blk; e += blockDim.x) {
    const cplx<T> a = A[e], b = A[blk + e];
    r00 += (double)norm2(a);
    r11 += (double)norm2(b);
    // rho[0,1] = sum A[0] conj(A[1])
    r01r += (double)a.re * b.re + (double)a.im * b.im;
    r01i += (double)a.im * b.re - (double)a.re * b.im;
  }
  r00 = block_sum(r00, red);
  r11 = block_sum(r11, red);
  r01r = block_sum(r01r, red);
  r01i = block_sum(r01i, red);
  if (threadIdx.x == 0) {
    out[0] = r00;
    out[1] = r11;
    out[2] = r01r;
    out[3] = r01i;
  }
}

}  // namespace

template <typename T>
int launch_wapply(const WapplyDesc<T>* d_desc, const WapplyDesc<T>* h_desc, int nd, cudaStream_t st) {
  if (nd <= 0) return QCA_OK;
  const WapplyDesc<T>& last = h_desc[nd - 1];
  const int tiles = last.tile_begin + last.nout * last.chunks;
  if (tiles <= 0) return QCA_OK;
  wapply_kernel<T><<<tiles, 256, 0, st>>>(d_desc, nd);
  QCA_LAUNCH_CHECK();
  count_launches(1);
  return QCA_OK;
}

template <typename T>
int launch_lz_init(const LanczosDesc<T>* d, const LanczosDesc<T>* h, int nd, int mmax, double tol, cudaStream_t st) {
  (void)mmax;
  if (nd <= 0) return QCA_OK;
  const int tiles = h[nd - 1].tile_begin + h[nd - 1].chunks;
  lz_norm_kernel<T><<<tiles, kLzThreads, 0, st>>>(d, nd);
  lz_init_kernel<T><<<tiles, kLzThreads, 0, st>>>(d, nd, tol);
  QCA_LAUNCH_CHECK();
  count_launches(1);
  count_launches(1);  // lz_norm_kernel
  return QCA_OK;
}

template <typename T>
int launch_lz_orth_pass(const LanczosDesc<T>* d, const LanczosDesc<T>* h, int nd, int j, int pass, cudaStream_t st) {
  const int tiles = h[nd - 1].tile_begin + h[nd - 1].chunks;
  lz_orth_kernel<T><<<tiles, kLzThreads, 0, st>>>(d, nd, j, pass);
  QCA_LAUNCH_CHECK();
  count_launches(1);
  return QCA_OK;
}

template <typename T>
int launch_lz_finalize_j(const LanczosDesc<T>* d, int nd, int j, int mmax, int check, cudaStream_t st) {
  lz_finalize_kernel<T><<<nd, 32, 0, st>>>(d, nd, j, mmax, check);
  QCA_LAUNCH_CHECK();
  count_launches(1);
  return QCA_OK;
}

template <typename T>
int launch_lz_normalize(const LanczosDesc<T>* d, const LanczosDesc<T>* h, int nd, int j, cudaStream_t st) {
  const int tiles = h[nd - 1].tile_begin + h[nd - 1].chunks;
  lz_normalize_kernel<T><<<tiles, kLzThreads, 0, st>>>(d, nd, j);
  QCA_LAUNCH_CHECK();
  count_launches(1);
  return QCA_OK;
}

template <typename T>
int launch_lz_combine(const LanczosDesc<T>* d, const LanczosDesc<T>* h, int nd, cudaStream_t st) {
  if (nd <= 0) return QCA_OK;
  const int tiles = h[nd - 1].tile_begin + h[nd - 1].chunks;
  lz_combine_kernel<T><<<tiles, kLzThreads, 0, st>>>(d, nd);
  QCA_LAUNCH_CHECK();
  count_launches(1);
  return QCA_OK;
}

template <typename T>
int launch_copy(const CopyDesc<T>* d, const CopyDesc<T>* h, int nd, cudaStream_t st) {
  if (nd <= 0) return QCA_OK;
  const int tiles = h[nd - 1].tile_begin + h[nd - 1].tiles;
  if (tiles <= 0) return QCA_OK;
  copy_kernel<T><<<tiles, 256, 0, st>>>(d, nd);
  QCA_LAUNCH_CHECK();
  count_launches(1);
  return QCA_OK;
}

template <typename T>
int launch_rho(const RhoDesc<T>* d, int nd, cudaStream_t st) {
  if (nd <= 0) return QCA_OK;
  rho_kernel<T><<<nd, 256, 0, st>>>(d);
  QCA_LAUNCH_CHECK();
  count_launches(1);
  return QCA_OK;
}

#define QCA_INST(T)                                                                                               \
  template int launch_wapply<T>(const WapplyDesc<T>*, const WapplyDesc<T>*, int, cudaStream_t);                   \
  template int launch_lz_init<T>(const LanczosDesc<T>*, const LanczosDesc<T>*, int, int, double, cudaStream_t);   \
  template int launch_lz_orth_pass<T>(const LanczosDesc<T>*, const LanczosDesc<T>*, int, int, int, cudaStream_t);  \
  template int launch_lz_finalize_j<T>(const LanczosDesc<T>*, int, int, int, int, cudaStream_t);                  \
  template int launch_lz_normalize<T>(const LanczosDesc<T>*, const LanczosDesc<T>*, int, int, cudaStream_t);      \
  template int launch_lz_combine<T>(const LanczosDesc<T>*, const LanczosDesc<T>*, int, cudaStream_t);             \
  template int launch_copy<T>(const CopyDesc<T>*, const CopyDesc<T>*, int, cudaStream_t);                         \
  template int launch_rho<T>(const RhoDesc<T>*, int, cudaStream_t);

QCA_INST(double)
QCA_INST(float)

}  // namespace qca
