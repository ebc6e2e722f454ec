// Grouped complex GEMM for the TDVP contractions (environment updates and the
// three stages of the effective-Hamiltonian application, tdvp.py:298-347).
//
// One launch covers many problems: CTA b finds its problem by binary search over
// the problems' first tiles.  Operands are addressed through arbitrary element
// strides, so transposed / reshaped views of the MPS, MPO and environment tensors
// need no copies.  Each CTA computes a BM x BN tile with 256 threads (a 16 x 16
// grid of TM x TN micro-tiles), staging BK-deep slabs of A and B in shared
// memory; complex products are four real FMAs in the element precision.
#include "tdvp_kernels.cuh"

namespace qca {

namespace {

constexpr int kGemmThreads = 256;
constexpr int kBK = 8;

template <typename T>
__device__ __forceinline__ int find_desc(const GemmDesc<T>* d, int nd, int tile) {
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

template <typename T, int BM, int BN>
__global__ void __launch_bounds__(kGemmThreads) gemm_grouped(const GemmDesc<T>* __restrict__ descs, int nd) {
  constexpr int TM = BM / 16, TN = BN / 16;
  __shared__ cplx<T> As[kBK][BM + 1];
  __shared__ cplx<T> Bs[kBK][BN + 1];
  const int di = find_desc(descs, nd, blockIdx.x);
  const GemmDesc<T>& D = descs[di];
  if (D.skip && *D.skip) return;
  int t = blockIdx.x - D.tile_begin;
  const int per_batch = D.tiles_m * D.tiles_n;
  const int b = t / per_batch;
  t -= b * per_batch;
  const int b1 = b / D.nb2, b2 = b - b1 * D.nb2;
  if (b1 >= D.nb1) return;
  const int tm = t / D.tiles_n, tn = t - tm * D.tiles_n;
  const int m0 = tm * BM, n0 = tn * BN;
  const cplx<T>* A = D.A + b1 * D.sAb1 + b2 * D.sAb2;
  const cplx<T>* B = D.B + b1 * D.sBb1 + b2 * D.sBb2;
  cplx<T>* C = D.C + b1 * D.sCb1 + b2 * D.sCb2;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  cplx<T> acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = mk<T>(0, 0);
  const bool a_kfast = D.sAk == 1;
  const bool b_nfast = D.sBn == 1;
  for (int g = 0; g < D.G; ++g) {
    const cplx<T>* Ag = A + g * D.sAg;
    const cplx<T>* Bg = B + g * D.sBg;
    for (int k0 = 0; k0 < D.K; k0 += kBK) {
      // stage A (BM x BK) and B (BK x BN)
      for (int e = threadIdx.x; e < BM * kBK; e += kGemmThreads) {
        int mm, kk;
        if (a_kfast) {
          mm = e / kBK;
          kk = e - mm * kBK;
        } else {
          kk = e / BM;
          mm = e - kk * BM;
        }
        const int m = m0 + mm, k = k0 + kk;
        cplx<T> v = mk<T>(0, 0);
        if (m < D.M && k < D.K) v = Ag[m * D.sAm + k * D.sAk];
        if (D.conjA) v.im = -v.im;
        As[kk][mm] = v;
      }
      for (int e = threadIdx.x; e < BN * kBK; e += kGemmThreads) {
        int nn, kk;
        if (b_nfast) {
          kk = e / BN;
          nn = e - kk * BN;
        } else {
          nn = e / kBK;
          kk = e - nn * kBK;
        }
        const int n = n0 + nn, k = k0 + kk;
        cplx<T> v = mk<T>(0, 0);
        if (n < D.N && k < D.K) v = Bg[k * D.sBk + n * D.sBn];
        if (D.conjB) v.im = -v.im;
        Bs[kk][nn] = v;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < kBK; ++kk) {
        cplx<T> a[TM], bb[TN];
#pragma unroll
        for (int i = 0; i < TM; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
        for (int j = 0; j < TN; ++j) bb[j] = Bs[kk][tx + 16 * j];
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) cfma(acc[i][j], a[i], bb[j]);
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int m = m0 + ty + 16 * i;
    if (m >= D.M) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int n = n0 + tx + 16 * j;
      if (n >= D.N) continue;
      cplx<T>* c = C + m * D.sCm + n * D.sCn;
      if (D.accumulate) {
        *c = *c + acc[i][j];
      } else {
        *c = acc[i][j];
      }
    }
  }
}

}  // namespace

int gemm_tile_cfg(int maxM, int maxN) {
  const int mx = maxM > maxN ? maxM : maxN;
  if (mx <= 16) return 0;
  if (mx <= 32) return 1;
  return 2;
}

int gemm_tile_dim(int cfg) { return cfg == 0 ? 16 : (cfg == 1 ? 32 : 64); }

template <typename T>
int launch_gemm(const GemmDesc<T>* d_desc, const GemmDesc<T>* h_desc, int ndesc, int cfg, cudaStream_t st) {
  if (ndesc <= 0) return QCA_OK;
  const GemmDesc<T>& last = h_desc[ndesc - 1];
  const int tiles = last.tile_begin + last.nb1 * last.nb2 * last.tiles_m * last.tiles_n;
  if (tiles <= 0) return QCA_OK;
  switch (cfg) {
    case 0:
      gemm_grouped<T, 16, 16><<<tiles, kGemmThreads, 0, st>>>(d_desc, ndesc);
      break;
    case 1:
      gemm_grouped<T, 32, 32><<<tiles, kGemmThreads, 0, st>>>(d_desc, ndesc);
      break;
    default:
      gemm_grouped<T, 64, 64><<<tiles, kGemmThreads, 0, st>>>(d_desc, ndesc);
      break;
  }
  QCA_LAUNCH_CHECK();
  return QCA_OK;
}

template int launch_gemm<double>(const GemmDesc<double>*, const GemmDesc<double>*, int, int, cudaStream_t);
template int launch_gemm<float>(const GemmDesc<float>*, const GemmDesc<float>*, int, int, cudaStream_t);

}  // namespace qca
