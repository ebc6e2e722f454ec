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
  count_launches(1);
  return QCA_OK;
}

template int launch_gemm<double>(const GemmDesc<double>*, const GemmDesc<double>*, int, int, cudaStream_t);
template int launch_gemm<float>(const GemmDesc<float>*, const GemmDesc<float>*, int, int, cudaStream_t);

}  // namespace qca

// ==================================================================================
// Tensor-core variant for the mixed path (complex64 operands, FP32 accumulation).
//
// Every complex product is four real products and every real product x*y is
// evaluated from TF32 parts xh = tf32(x), xl = tf32(x - xh) as
// xh*yh + xh*yl + xl*yh (split precision, "3xTF32"); with every k8 step summed
// into zeroed registers and added to the running sums in FP32, the products keep
// FP32 accuracy on the TF32 tensor cores.  The split is done once per element while
// staging the BM x BK / BK x BN slabs into shared memory (planes re_hi, re_lo,
// im_hi, im_lo); each warp then issues mma.sync m16n8k8 TF32 on a 32 x 16 warp
// tile (2 x 2 MMA tiles, 12 MMAs per tile and k8 step).
// ==================================================================================
namespace qca {

namespace {

constexpr int kTcBM = 64, kTcBN = 64, kTcBK = 16, kTcPad = 8;

__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void mma_tf32(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

struct TcSmem {
  // [plane][k][m or n]; planes: 0 re_hi, 1 re_lo, 2 im_hi, 3 im_lo
  uint32_t A[4][kTcBK][kTcBM + kTcPad];
  uint32_t B[4][kTcBK][kTcBN + kTcPad];
};

__device__ __forceinline__ void tc_split_store(uint32_t (&pl)[4][kTcBK][kTcBM + kTcPad], int kk, int mm,
                                               cplx<float> v) {
  const uint32_t rh = to_tf32(v.re), ih = to_tf32(v.im);
  pl[0][kk][mm] = rh;
  pl[1][kk][mm] = to_tf32(v.re - __uint_as_float(rh));
  pl[2][kk][mm] = ih;
  pl[3][kk][mm] = to_tf32(v.im - __uint_as_float(ih));
}

// Double-buffered: while the warps multiply the slab in shared memory, every thread
// already holds its elements of the next slab in registers (4 of A, 4 of B).
__global__ void __launch_bounds__(256, 2) gemm_tc_grouped(const GemmDesc<float>* __restrict__ descs, int nd) {
  extern __shared__ __align__(16) unsigned char tc_smem_raw[];
  TcSmem* sm = reinterpret_cast<TcSmem*>(tc_smem_raw);  // two stages
  const int di = find_desc(descs, nd, blockIdx.x);
  const GemmDesc<float>& D = descs[di];
  if (D.skip && *D.skip) return;
  int t = blockIdx.x - D.tile_begin;
  const int per_batch = D.tiles_m * D.tiles_n;
  const int b = t / per_batch;
  t -= b * per_batch;
  const int b1 = b / D.nb2, b2 = b - b1 * D.nb2;
  if (b1 >= D.nb1) return;
  const int tm = t / D.tiles_n, tn = t - tm * D.tiles_n;
  const int m0 = tm * kTcBM, n0 = tn * kTcBN;
  const cplx<float>* A = D.A + b1 * D.sAb1 + b2 * D.sAb2;
  const cplx<float>* B = D.B + b1 * D.sBb1 + b2 * D.sBb2;
  cplx<float>* C = D.C + b1 * D.sCb1 + b2 * D.sCb2;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int wm = (warp >> 2) * 32;  // warp tile origin in M (2 warps)
  const int wn = (warp & 3) * 16;   // warp tile origin in N (4 warps)
  const int g = lane >> 2, tq = lane & 3;
  float accr[2][2][4], acci[2][2][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) accr[i][j][r] = acci[i][j][r] = 0.f;
  const bool a_kfast = D.sAk == 1;
  const bool b_nfast = D.sBn == 1;
  // this thread's 4 A and 4 B element positions within a slab
  int amm[4], akk[4], bnn[4], bkk[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int e = threadIdx.x + 256 * q;
    if (a_kfast) {
      amm[q] = e / kTcBK;
      akk[q] = e - amm[q] * kTcBK;
    } else {
      akk[q] = e / kTcBM;
      amm[q] = e - akk[q] * kTcBM;
    }
    if (b_nfast) {
      bkk[q] = e / kTcBN;
      bnn[q] = e - bkk[q] * kTcBN;
    } else {
      bnn[q] = e / kTcBK;
      bkk[q] = e - bnn[q] * kTcBK;
    }
  }
  const int ksl = (D.K + kTcBK - 1) / kTcBK;  // slabs per K group
  const int nsl = ksl * D.G;
  cplx<float> ra[4], rb[4];
  auto fetch = [&](int sl) {
    const int gg = sl / ksl, k0 = (sl - gg * ksl) * kTcBK;
    const cplx<float>* Ag = A + gg * D.sAg;
    const cplx<float>* Bg = B + gg * D.sBg;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int m = m0 + amm[q], k = k0 + akk[q];
      ra[q] = (m < D.M && k < D.K) ? Ag[m * D.sAm + k * D.sAk] : mk<float>(0.f, 0.f);
      const int n = n0 + bnn[q], kb = k0 + bkk[q];
      rb[q] = (n < D.N && kb < D.K) ? Bg[kb * D.sBk + n * D.sBn] : mk<float>(0.f, 0.f);
    }
  };
  auto stash = [&](int buf) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      cplx<float> va = ra[q], vb = rb[q];
      if (D.conjA) va.im = -va.im;
      if (D.conjB) vb.im = -vb.im;
      tc_split_store(sm[buf].A, akk[q], amm[q], va);
      tc_split_store(sm[buf].B, bkk[q], bnn[q], vb);
    }
  };
  fetch(0);
  stash(0);
  __syncthreads();
  for (int sl = 0; sl < nsl; ++sl) {
    const int cur = sl & 1;
    if (sl + 1 < nsl) fetch(sl + 1);  // global loads in flight during the MMAs
    const TcSmem& S = sm[cur];
#pragma unroll
    for (int ks = 0; ks < kTcBK; ks += 8) {
      uint32_t af[2][4][4];  // [mtile][plane][reg]
      uint32_t bf[2][4][2];  // [ntile][plane][reg]
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int r0 = wm + 16 * i + g;
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          af[i][p][0] = S.A[p][ks + tq][r0];
          af[i][p][1] = S.A[p][ks + tq][r0 + 8];
          af[i][p][2] = S.A[p][ks + tq + 4][r0];
          af[i][p][3] = S.A[p][ks + tq + 4][r0 + 8];
        }
      }
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        const int c0 = wn + 8 * j + g;
#pragma unroll
        for (int p = 0; p < 4; ++p) {
          bf[j][p][0] = S.B[p][ks + tq][c0];
          bf[j][p][1] = S.B[p][ks + tq + 4][c0];
        }
      }
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        uint32_t nih[4], nil[4];  // -Ai (hi, lo): sign flip is exact
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          nih[r] = af[i][2][r] ^ 0x80000000u;
          nil[r] = af[i][3][r] ^ 0x80000000u;
        }
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          // The tensor core's internal accumulation does not round to nearest, so
          // a k8 step accumulates into zeroed registers and is then added to the
          // running sums with FP32 adds; small terms first.
          float tr[4] = {0.f, 0.f, 0.f, 0.f}, ti[4] = {0.f, 0.f, 0.f, 0.f};
          mma_tf32(tr, af[i][1], bf[j][0]);  // Arl Brh
          mma_tf32(tr, af[i][0], bf[j][1]);  // Arh Brl
          mma_tf32(tr, nil, bf[j][2]);       // -Ail Bih
          mma_tf32(tr, nih, bf[j][3]);       // -Aih Bil
          mma_tf32(tr, af[i][0], bf[j][0]);  // Arh Brh
          mma_tf32(tr, nih, bf[j][2]);       // -Aih Bih
          mma_tf32(ti, af[i][1], bf[j][2]);  // Arl Bih
          mma_tf32(ti, af[i][0], bf[j][3]);  // Arh Bil
          mma_tf32(ti, af[i][3], bf[j][0]);  // Ail Brh
          mma_tf32(ti, af[i][2], bf[j][1]);  // Aih Brl
          mma_tf32(ti, af[i][0], bf[j][2]);  // Arh Bih
          mma_tf32(ti, af[i][2], bf[j][0]);  // Aih Brh
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            accr[i][j][r] += tr[r];
            acci[i][j][r] += ti[r];
          }
        }
      }
    }
    if (sl + 1 < nsl) stash(cur ^ 1);  // the other buffer was last read before the previous barrier
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int m = m0 + wm + 16 * i + g + (r >= 2 ? 8 : 0);
        const int n = n0 + wn + 8 * j + 2 * tq + (r & 1);
        if (m < D.M && n < D.N) {
          cplx<float>* c = C + m * D.sCm + n * D.sCn;
          const cplx<float> v = mk<float>(accr[i][j][r], acci[i][j][r]);
          *c = D.accumulate ? *c + v : v;
        }
      }
}

}  // namespace

int launch_gemm_tc(const GemmDesc<float>* d_desc, const GemmDesc<float>* h_desc, int ndesc, cudaStream_t st) {
  if (ndesc <= 0) return QCA_OK;
  const GemmDesc<float>& last = h_desc[ndesc - 1];
  const int tiles = last.tile_begin + last.nb1 * last.nb2 * last.tiles_m * last.tiles_n;
  if (tiles <= 0) return QCA_OK;
  static bool configured[kMaxDevices] = {};
  const int dv = device_slot();
  if (dv < 0 || !configured[dv]) {
    QCA_CUDA(cudaFuncSetAttribute(gemm_tc_grouped, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * sizeof(TcSmem)));
    if (dv >= 0) configured[dv] = true;
  }
  gemm_tc_grouped<<<tiles, 256, 2 * sizeof(TcSmem), st>>>(d_desc, ndesc);
  QCA_LAUNCH_CHECK();
  count_launches(1);
  return QCA_OK;
}

}  // namespace qca

// Test hook: C = A B for row-major complex64 device matrices through the grouped
// kernels (tensor_cores: 2 = 3xTF32 tcgen05 kernel, 1 = 3xTF32 mma.sync kernel,
// 0 = CUDA-core kernel).
// The single descriptor is passed through a file-scope device slot.
static __device__ qca::GemmDesc<float> g_test_gemm_slot;

extern "C" int qca_test_gemm_c64(int M, int N, int K, const void* A, const void* B, void* C, int tensor_cores,
                                 void* stream) {
  using namespace qca;
  if (M < 1 || N < 1 || K < 1 || !A || !B || !C) {
    set_error("qca_test_gemm_c64: invalid arguments");
    return QCA_ERR_INVALID;
  }
  GemmDesc<float> d;
  memset(&d, 0, sizeof(d));
  d.A = (const c64*)A;
  d.B = (const c64*)B;
  d.C = (c64*)C;
  d.M = M;
  d.N = N;
  d.K = K;
  d.G = 1;
  d.nb1 = 1;
  d.nb2 = 1;
  d.sAm = K;
  d.sAk = 1;
  d.sBk = N;
  d.sBn = 1;
  d.sCm = N;
  d.sCn = 1;
  const bool um = tensor_cores == 2;
  d.tiles_m = ceil_div(M, um ? kUmmaBM : 64);
  d.tiles_n = ceil_div(N, um ? kUmmaBN : 64);
  d.tile_begin = 0;
  GemmDesc<float>* dd = nullptr;
  cudaStream_t st = (cudaStream_t)stream;
  void* addr = nullptr;
  QCA_CUDA(cudaGetSymbolAddress(&addr, g_test_gemm_slot));
  dd = (GemmDesc<float>*)addr;
  QCA_CUDA(cudaMemcpyAsync(dd, &d, sizeof(d), cudaMemcpyHostToDevice, st));
  int s = um ? launch_gemm_umma(dd, &d, 1, st)
             : tensor_cores ? launch_gemm_tc(dd, &d, 1, st) : launch_gemm<float>(dd, &d, 1, 2, st);
  if (s != QCA_OK) return s;
  QCA_CUDA(cudaStreamSynchronize(st));
  if (um) {
    int timeouts = 0;
    QCA_TRY(gemm_umma_timeouts(1, &timeouts, st));
    if (timeouts) {
      set_error("qca_test_gemm_c64: %d tensor-core mbarrier waits ran out", timeouts);
      return QCA_ERR_CUDA;
    }
  }
  return QCA_OK;
}
