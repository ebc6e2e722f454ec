// Grouped complex64 GEMM on the fifth-generation tensor cores: tcgen05.mma
// kind::tf32 with the accumulators in tensor memory (TMEM), 3xTF32 split precision.
// Used by the mixed-precision path for the TDVP contractions with M >= 48 and
// N, K >= 32 (environment updates and the effective-Hamiltonian stages,
// tdvp.py:298-347).
//
// The complex product is one real GEMM over an embedding that doubles K and N
// (per K stage of BK complex elements and per 64-column tile):
//   A'[m][k] = Re A[m][k],  A'[m][BK + k] = Im A[m][k]
//   B'[k][n] = Re B[k][n],  B'[BK + k][n] = -Im B[k][n]
//   B'[k][64 + n] = Im B[k][n],  B'[BK + k][64 + n] = Re B[k][n]
//   C'[m][n] = Re C[m][n],  C'[m][64 + n] = Im C[m][n]
// and each real product x y is evaluated as xh yh + xh yl + xl yh from the TF32
// parts xh = tf32(x), xl = tf32(x - xh).
//
// A CTA (256 threads) computes 128 x 64 complex tiles (128 x 128 real accumulators);
// the kernel is persistent, one CTA per SM walking the tiles b, b + grid, ..., and
// its stage pipeline runs on across tile boundaries.  Per K stage of 16 complex elements all threads convert the
// stage's operands and store them in shared memory in the canonical K-major layout
// without swizzle (core matrices of 8 rows x 16 bytes): a thread owns one row and
// four consecutive K elements and writes whole 16-byte core-matrix rows, lanes on
// consecutive rows (no bank conflicts); one thread issues the 12
// MMAs of the stage (4 k8 steps x 3 products, M = 128, N = 128) into one of two TMEM
// accumulators and commits them to an mbarrier.  The next stage's global loads and
// the previous stage's read-out (tcgen05.ld, added into FP32 registers) overlap
// with the MMAs.  Reading every stage out of TMEM bounds the tensor core's internal
// accumulation to 96 products, so the result keeps FP32-level accuracy.
#include "tdvp_kernels.cuh"

namespace qca {

namespace {

constexpr int kUmBM = 128, kUmBN = 64, kUmBK = 16;   // complex tile and K stage
constexpr int kUmThreads = 256;
constexpr uint32_t kUmPlane = 128u * 2 * kUmBK * 4;  // one operand plane: 128 rows x 32 tf32
constexpr uint32_t kUmStage = 4 * kUmPlane;          // A hi, A lo, B hi, B lo
constexpr size_t kUmSmem = 2 * kUmStage + 1024;      // two stages + alignment slack
constexpr int kUmWaitLimit = 1 << 20;

// instruction descriptor, kind::tf32: D f32 (bits 4-5 = 1), A and B tf32 (bits 7-9,
// 10-12 = 2), both K-major, N >> 3 at bit 17, M >> 4 at bit 24
constexpr uint32_t kUmIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);

__device__ int g_umma_timeouts;  // mbarrier waits that ran out (never expected)

__device__ __forceinline__ int um_find_desc(const GemmDesc<float>* d, int nd, int tile) {
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

__device__ __forceinline__ uint32_t um_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint32_t um_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// byte offset of (row, k') in a 128 x 32 K-major plane: row groups of 8 at 1024 B,
// core matrices along K at 128 B, rows of a core matrix at 16 B
__device__ __forceinline__ uint32_t um_off(int row, int kp) {
  return (uint32_t)((row >> 3) * 1024 + (kp >> 2) * 128 + (row & 7) * 16 + (kp & 3) * 4);
}

__device__ __forceinline__ void um_st4(uint32_t addr, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d));
}

// TF32 hi / lo parts of four values; neg flips the sign (exact)
struct Split4 {
  uint32_t h[4], l[4];
};
__device__ __forceinline__ Split4 um_split(const float (&x)[4], bool neg) {
  Split4 r;
  const uint32_t sg = neg ? 0x80000000u : 0u;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const uint32_t h = um_tf32(x[i]);
    r.h[i] = h ^ sg;
    r.l[i] = um_tf32(x[i] - __uint_as_float(h)) ^ sg;
  }
  return r;
}

// shared-memory matrix descriptor: start >> 4, leading (K) byte offset 128, stride
// (8-row group) byte offset 1024, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t um_desc(uint32_t saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46);
}

__device__ __forceinline__ void um_mma(uint32_t dt, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.u32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dt),
      "l"(a), "l"(b), "r"(kUmIdesc), "r"(accumulate));
}

__device__ __forceinline__ bool um_wait(uint32_t mbar, uint32_t parity) {
  uint32_t done = 0;
  for (int it = 0; it < kUmWaitLimit && !done; ++it) {
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
  }
  return done != 0;
}

__device__ __forceinline__ void um_ld32(uint32_t taddr, float (&r)[32]) {
  uint32_t u[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(u[0]), "=r"(u[1]), "=r"(u[2]), "=r"(u[3]), "=r"(u[4]), "=r"(u[5]), "=r"(u[6]), "=r"(u[7]), "=r"(u[8]),
        "=r"(u[9]), "=r"(u[10]), "=r"(u[11]), "=r"(u[12]), "=r"(u[13]), "=r"(u[14]), "=r"(u[15]), "=r"(u[16]),
        "=r"(u[17]), "=r"(u[18]), "=r"(u[19]), "=r"(u[20]), "=r"(u[21]), "=r"(u[22]), "=r"(u[23]), "=r"(u[24]),
        "=r"(u[25]), "=r"(u[26]), "=r"(u[27]), "=r"(u[28]), "=r"(u[29]), "=r"(u[30]), "=r"(u[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) r[j] = __uint_as_float(u[j]);
}

// one output tile of a problem: operand bases (batch offsets applied) and K stages
struct UmTile {
  const GemmDesc<float>* D;
  const cplx<float>* A;
  const cplx<float>* B;
  cplx<float>* C;
  int m0, n0, ksl, nst;
};

// pipeline cursor: stage s of tile `tile` (s < 0: past the CTA's last tile)
struct UmCur {
  UmTile T;
  int tile, s;
};

// first tiles of the problems, staged in shared memory for the tile lookups of a
// persistent CTA (a binary search over global memory is a chain of dependent loads)
constexpr int kUmMaxDesc = 2048;

__device__ __forceinline__ int um_find_tile(const int* tb, const GemmDesc<float>* d, int nd, int tile) {
  if (nd > kUmMaxDesc) return um_find_desc(d, nd, tile);
  int lo = 0, hi = nd - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tb[mid] <= tile)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ bool um_tile(const int* tb, const GemmDesc<float>* descs, int nd, int tile, UmTile& T) {
  const GemmDesc<float>* D = descs + um_find_tile(tb, descs, nd, tile);
  if (D->skip && *D->skip) return false;
  int t = tile - D->tile_begin;
  const int per_batch = D->tiles_m * D->tiles_n;
  const int bb = t / per_batch;
  t -= bb * per_batch;
  const int b1 = bb / D->nb2, b2 = bb - b1 * D->nb2;
  if (b1 >= D->nb1) return false;
  const int tm = t / D->tiles_n, tn = t - tm * D->tiles_n;
  T.D = D;
  T.m0 = tm * kUmBM;
  T.n0 = tn * kUmBN;
  T.A = D->A + b1 * D->sAb1 + b2 * D->sAb2;
  T.B = D->B + b1 * D->sBb1 + b2 * D->sBb2;
  T.C = D->C + b1 * D->sCb1 + b2 * D->sCb2;
  T.ksl = (D->K + kUmBK - 1) / kUmBK;
  T.nst = T.ksl * D->G;
  return true;
}

// first valid tile at or after `from` in this CTA's stride
__device__ __forceinline__ void um_seek(const int* tb, const GemmDesc<float>* descs, int nd, int total, int from,
                                        UmCur& c) {
  for (int t = from; t < total; t += gridDim.x)
    if (um_tile(tb, descs, nd, t, c.T)) {
      c.tile = t;
      c.s = 0;
      return;
    }
  c.tile = total;
  c.s = -1;
}

__device__ __forceinline__ void um_advance(const int* tb, const GemmDesc<float>* descs, int nd, int total, UmCur& c) {
  if (c.s < 0) return;
  if (c.s + 1 < c.T.nst) {
    ++c.s;
    return;
  }
  um_seek(tb, descs, nd, total, c.tile + gridDim.x, c);
}

// Persistent: CTA b takes tiles b, b + gridDim.x, ...; the stage pipeline runs on
// across tile boundaries, so the MMAs of a tile's first stages overlap with the
// read-out and stores of the previous tile.
__global__ void __launch_bounds__(kUmThreads, 1) gemm_umma_grouped(const GemmDesc<float>* __restrict__ descs, int nd,
                                                                     int total) {
  extern __shared__ __align__(16) unsigned char um_raw[];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tslot;
  __shared__ int s_tb[kUmMaxDesc];
  if (nd <= kUmMaxDesc)
    for (int i = threadIdx.x; i < nd; i += blockDim.x) s_tb[i] = descs[i].tile_begin;
  __syncthreads();
  UmCur F;  // next stage to fetch from global memory
  um_seek(s_tb, descs, nd, total, blockIdx.x, F);
  if (F.s < 0) return;  // no work for this CTA (uniform)
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // operand planes of buffer b: sbase + b * kUmStage + p * kUmPlane (p: A hi, A lo, B hi, B lo)
  const uint32_t sbase = (um_smem(um_raw) + 1023u) & ~1023u;
  const uint32_t mb0 = um_smem(&mbar[0]), mb1 = um_smem(&mbar[1]);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb0));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(um_smem(&tslot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tbase = tslot;

  // staging tasks: A rows m (2 per thread) and B columns n (1 per thread), each with
  // the four consecutive K elements 4 kg .. 4 kg + 3 of the stage; lanes run over
  // consecutive rows, so every 16-byte shared store of a warp hits distinct banks
  const int am = tid & (kUmBM - 1), akg = tid >> 7;  // task q: kg = akg + 2 q
  const int bn = tid & (kUmBN - 1), bkg = tid >> 6;
  cplx<float> ra[2][4], rb[4];
  bool conj_a = false, conj_b = false;  // of the fetched stage
  auto fetch = [&](const UmCur& c) {
    const GemmDesc<float>& D = *c.T.D;
    const int gg = c.s / c.T.ksl, k0 = (c.s - gg * c.T.ksl) * kUmBK;
    const cplx<float>* Ag = c.T.A + gg * D.sAg;
    const cplx<float>* Bg = c.T.B + gg * D.sBg;
    const int M = D.M, N = D.N, K = D.K;
    const long long sAm = D.sAm, sAk = D.sAk, sBk = D.sBk, sBn = D.sBn;
    const int m = c.T.m0 + am;
#pragma unroll
    for (int q = 0; q < 2; ++q)
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int k = k0 + 4 * (akg + 2 * q) + i;
        ra[q][i] = (m < M && k < K) ? Ag[m * sAm + k * sAk] : mk<float>(0.f, 0.f);
      }
    const int n = c.T.n0 + bn;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int k = k0 + 4 * bkg + i;
      rb[i] = (n < N && k < K) ? Bg[k * sBk + n * sBn] : mk<float>(0.f, 0.f);
    }
    conj_a = D.conjA != 0;
    conj_b = D.conjB != 0;
  };
  auto stash = [&](int buf) {
    const uint32_t st0 = sbase + buf * kUmStage;
    const uint32_t ah = st0, al = st0 + kUmPlane, bh = st0 + 2 * kUmPlane, bl = st0 + 3 * kUmPlane;
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const int kg = akg + 2 * q;
      float re[4], im[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        re[i] = ra[q][i].re;
        im[i] = ra[q][i].im;
      }
      const Split4 r = um_split(re, false), c = um_split(im, conj_a);
      const uint32_t o1 = um_off(am, 4 * kg), o2 = um_off(am, kUmBK + 4 * kg);
      um_st4(ah + o1, r.h[0], r.h[1], r.h[2], r.h[3]);
      um_st4(al + o1, r.l[0], r.l[1], r.l[2], r.l[3]);
      um_st4(ah + o2, c.h[0], c.h[1], c.h[2], c.h[3]);
      um_st4(al + o2, c.l[0], c.l[1], c.l[2], c.l[3]);
    }
    {
      float re[4], im[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        re[i] = rb[i].re;
        im[i] = rb[i].im;
      }
      const Split4 r = um_split(re, false), c = um_split(im, conj_b), nc = um_split(im, !conj_b);
      // row n: (Re, -Im) over (k, BK + k); row 64 + n: (Im, Re)
      const uint32_t o1 = um_off(bn, 4 * bkg), o2 = um_off(bn, kUmBK + 4 * bkg);
      const uint32_t o3 = um_off(kUmBN + bn, 4 * bkg), o4 = um_off(kUmBN + bn, kUmBK + 4 * bkg);
      um_st4(bh + o1, r.h[0], r.h[1], r.h[2], r.h[3]);
      um_st4(bl + o1, r.l[0], r.l[1], r.l[2], r.l[3]);
      um_st4(bh + o2, nc.h[0], nc.h[1], nc.h[2], nc.h[3]);
      um_st4(bl + o2, nc.l[0], nc.l[1], nc.l[2], nc.l[3]);
      um_st4(bh + o3, c.h[0], c.h[1], c.h[2], c.h[3]);
      um_st4(bl + o3, c.l[0], c.l[1], c.l[2], c.l[3]);
      um_st4(bh + o4, r.h[0], r.h[1], r.h[2], r.h[3]);
      um_st4(bl + o4, r.l[0], r.l[1], r.l[2], r.l[3]);
    }
  };

  // read-out: warp w holds TMEM lanes 32 (w % 4) .. + 31 (rows) and the complex
  // columns 32 (w / 4) .. + 31: real parts at TMEM columns n, imaginary at 64 + n
  const int q4 = warp & 3, half = warp >> 2;
  float acc[64];  // [0, 32): real parts, [32, 64): imaginary parts
#pragma unroll
  for (int j = 0; j < 64; ++j) acc[j] = 0.f;
  bool ok = true;
  auto readout = [&](int g) {
    const int b = g & 1;
    // warp-uniform outcome: tcgen05.ld below is a warp-collective instruction
    if (!__all_sync(0xffffffffu, um_wait(b ? mb1 : mb0, (uint32_t)((g >> 1) & 1)) ? 1 : 0)) {
      ok = false;
      return;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t ta = tbase + ((uint32_t)(32 * q4) << 16) + (uint32_t)(b * 128 + half * 32);
    float r[32];
    um_ld32(ta, r);
#pragma unroll
    for (int j = 0; j < 32; ++j) acc[j] += r[j];
    um_ld32(ta + kUmBN, r);
#pragma unroll
    for (int j = 0; j < 32; ++j) acc[32 + j] += r[j];
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  };
  // row m, complex columns n0 + 32 half + j of a finished tile
  auto epilogue = [&](const UmTile& T) {
    const GemmDesc<float>& D = *T.D;
    const int m = T.m0 + 32 * q4 + lane;
    if (ok && m < D.M) {
      const int nb = T.n0 + 32 * half;
      const bool accum = D.accumulate != 0;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int n = nb + j;
        if (n < D.N) {
          cplx<float>* c = T.C + m * D.sCm + n * D.sCn;
          const cplx<float> v = mk<float>(acc[j], acc[32 + j]);
          *c = accum ? *c + v : v;
        }
      }
    }
#pragma unroll
    for (int j = 0; j < 64; ++j) acc[j] = 0.f;
  };

  UmCur S = F;  // stage to stash and multiply
  fetch(F);
  um_advance(s_tb, descs, nd, total, F);
  UmCur R;  // stage to read out (previous iteration's)
  R.s = -1;
  int g = 0;
  for (; S.s >= 0; ++g) {
    const int buf = g & 1;
    // buffer buf was last read by the MMAs of stage g - 2, whose completion every
    // thread observed in the read-out of stage g - 2
    stash(buf);
    if (F.s >= 0) fetch(F);  // global loads in flight during the MMAs
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (tid == 0 && ok) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t st0 = sbase + buf * kUmStage;
      const uint32_t dt = tbase + (uint32_t)(buf * 128);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const uint64_t ah = um_desc(st0 + 256 * j), al = um_desc(st0 + kUmPlane + 256 * j);
        const uint64_t bh = um_desc(st0 + 2 * kUmPlane + 256 * j), bl = um_desc(st0 + 3 * kUmPlane + 256 * j);
        um_mma(dt, ah, bl, j > 0 ? 1u : 0u);  // small terms first
        um_mma(dt, al, bh, 1u);
        um_mma(dt, ah, bh, 1u);
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(buf ? mb1
                                                                                                           : mb0)
                   : "memory");
    }
    if (R.s >= 0) {
      if (ok) readout(g - 1);
      if (R.s == R.T.nst - 1) epilogue(R.T);
    }
    R = S;
    S = F;
    um_advance(s_tb, descs, nd, total, F);
  }
  // the last stage issued (R, global index g - 1) ends the CTA's last tile
  if (ok) readout(g - 1);
  epilogue(R.T);
  if (!ok && lane == 0) atomicAdd(&g_umma_timeouts, 1);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tbase));
  }
}

}  // namespace

int launch_gemm_umma(const GemmDesc<float>* d_desc, const GemmDesc<float>* h_desc, int ndesc, cudaStream_t st) {
  if (ndesc <= 0) return QCA_OK;
  const GemmDesc<float>& last = h_desc[ndesc - 1];
  const int tiles = last.tile_begin + last.nb1 * last.nb2 * last.tiles_m * last.tiles_n;
  if (tiles <= 0) return QCA_OK;
  static int sm_count[kMaxDevices] = {};
  const int dv = device_slot();
  int sms = dv >= 0 ? sm_count[dv] : 0;
  if (!sms) {
    QCA_CUDA(cudaFuncSetAttribute(gemm_umma_grouped, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kUmSmem));
    int dev = 0;
    QCA_CUDA(cudaGetDevice(&dev));
    QCA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    if (dv >= 0) sm_count[dv] = sms;
  }
  // persistent: one CTA per SM (shared memory and registers admit one)
  const int grid = tiles < sms ? tiles : sms;
  gemm_umma_grouped<<<grid, kUmThreads, kUmSmem, st>>>(d_desc, ndesc, tiles);
  QCA_LAUNCH_CHECK();
  count_launches(1);
  return QCA_OK;
}

int gemm_umma_timeouts(int reset, int* count, cudaStream_t st) {
  QCA_CUDA(cudaMemcpyFromSymbolAsync(count, g_umma_timeouts, sizeof(int), 0, cudaMemcpyDeviceToHost, st));
  QCA_CUDA(cudaStreamSynchronize(st));
  if (reset && *count) {
    const int z = 0;
    QCA_CUDA(cudaMemcpyToSymbolAsync(g_umma_timeouts, &z, sizeof(int), 0, cudaMemcpyHostToDevice, st));
    QCA_CUDA(cudaStreamSynchronize(st));
  }
  return QCA_OK;
}

}  // namespace qca
