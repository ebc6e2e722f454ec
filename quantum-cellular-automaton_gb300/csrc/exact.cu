// Exact state-vector evolution of the quantum game of life on sm_103a.
//
// Replaces algorithms/exact.py:9-28 (dense U = exp(-i pi/2 dt H) from
// MPO.as_matrix, mpo.py:219-228, and psi <- U psi) with a matrix-free Lanczos
// step: the basis (krylov_dim vectors of 2^N amplitudes) stays resident in HBM
// and H is never stored.
//
// H = sum_i X_i Pi_i: (H v)[x] = sum_b c_b(x) v[x ^ (1 << b)], where bit b is
// cell N-1-b and c_b(x) = [popc(x & nmask_b) in [lo, hi)] (the flip condition of
// tensor_networks/mpo.py:54-200, evaluated from the index alone; for distances up
// to 3 for all bits at once by a bit-sliced neighbour count, flip_mask).
//
// One H application is split by bit groups so that every partner of an amplitude
// lies in the same shared-memory tile:
//   phase 0: tile = 2^g0 contiguous amplitudes, flips of bits [0, g0);
//   phase p: tile = 2^g high bits x 2^kL contiguous low bits (64-byte runs),
//            flips of bits [lo_p, lo_p + g).
// The Lanczos recurrence is fused into the first and last phase:
//   phase 0 (iteration j):  u_j = w_j - alpha_{j-1} v_{j-1}   (written back)
//                           y   = H_0 u_j,  partial ||u_j||^2
//   last phase:             Hv  = (y + H_last u_j) / ||u_j||
//                           w_{j+1} = Hv - beta_{j-1} v_{j-1}, partial alpha_j
// so the basis holds the unnormalised u_j with v_j = u_j / ||u_j||.  All sums
// are reduced per block into partials and then by a single-block kernel, so a
// step is bitwise reproducible.
#include <cmath>
#include <mutex>
#include <vector>

#include "common.cuh"

namespace qca {

namespace {

constexpr int kMaxCells = 30;
constexpr int kExactThreads = 512;

struct PhaseGeom {
  int lo;  // first bit of the group
  int g;   // bits in the group
  int kl;  // contiguous low bits carried in the tile (0 for phase 0)
};

struct ExactParams {
  int n;                       // cells
  int rule_lo, rule_hi;        // flip iff count in [rule_lo, rule_hi)
  uint32_t nmask[kMaxCells];   // neighbour mask of the cell at bit b
  long long dim;               // 2^n
  int dist;                    // rule distance (flip_mask covers distance <= 3)
};

// Bits of x whose cell may flip, for all cells at once: the alive-neighbour count
// of every bit position is accumulated bit-sliced (three planes c0, c1, c2) from
// the index shifted by 1..dist in both directions (bits shifted past either end of
// the chain are dead cells), and the interval test [lo, hi) becomes a few logic
// operations on the planes.  Equivalent to popc(x & nmask_b) in [lo, hi) for
// every b; replaces a popcount and two comparisons per bit and amplitude.
__device__ __forceinline__ uint32_t flip_mask(uint32_t x, const ExactParams& P) {
  const uint32_t full = P.n >= 32 ? 0xffffffffu : ((1u << P.n) - 1u);
  uint32_t c0 = 0, c1 = 0, c2 = 0;
  for (int o = 1; o <= P.dist; ++o) {
#pragma unroll
    for (int side = 0; side < 2; ++side) {
      const uint32_t v = side == 0 ? (x << o) & full : x >> o;
      const uint32_t k0 = c0 & v;
      c0 ^= v;
      const uint32_t k1 = c1 & k0;
      c1 ^= k0;
      c2 |= k1;  // at most 6 alive neighbours: no carry out of c2
    }
  }
  uint32_t m = 0;
  for (int v = P.rule_lo; v < P.rule_hi && v < 8; ++v)
    m |= ((v & 1) ? c0 : ~c0) & ((v & 2) ? c1 : ~c1) & ((v & 4) ? c2 : ~c2);
  return m & full;
}

// flip condition of bit b for the amplitude x (fm = flip_mask(x) when dist <= 3)
__device__ __forceinline__ bool may_flip(uint32_t x, uint32_t fm, int b, const ExactParams& P) {
  if (P.dist <= 3) return (fm >> b) & 1u;
  const int c = __popc(x & P.nmask[b]);
  return c >= P.rule_lo && c < P.rule_hi;
}

// Scalar slots in the device scalar array.
enum : int {
  S_NORM0 = 0,       // ||psi|| of the current sub-step
  S_MEFF = 1,        // effective Krylov dimension (breakdown lowers it)
  S_TAU = 2,         // pi/2 * dt of the sub-step
  S_NORM = 8,        // S_NORM + j : ||u_j||
  S_ALPHA = 8 + 64,  // S_ALPHA + j: alpha_j
  S_COEF = 8 + 128,  // S_COEF + 2k: complex coefficient of slot k in the combination
  S_INV = 8 + 256,   // S_INV + j : 1 / ||u_j||
  S_AOV = 8 + 320,   // S_AOV + j : alpha_j / ||u_j||
  S_TOTAL = 8 + 384
};

__device__ __forceinline__ long long tile_index(const PhaseGeom& G, int n, long long t, int l) {
  const int tb = G.g + G.kl;
  const long long low = l & ((1 << G.kl) - 1);
  const long long hb = l >> G.kl;
  const int midbits = G.lo - G.kl;
  const long long tmid = t & ((1LL << midbits) - 1);
  const long long thi = t >> midbits;
  (void)tb;
  return (thi << (G.lo + G.g)) | (hb << G.lo) | (tmid << G.kl) | low;
}

template <typename T>
__device__ __forceinline__ cplx<T> ld(const cplx<T>* p) { return *p; }

// ---------------------------------------------------------------------------------
// phase 0: Lanczos prologue + H over the low bit group
// ---------------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kExactThreads) ex_phase0(ExactParams P, PhaseGeom G, cplx<T>* basis, cplx<T>* y,
                                                           double* scal, double* partial, int j) {
  if (j >= (int)scal[S_MEFF]) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tile = reinterpret_cast<cplx<T>*>(smem_raw);
  __shared__ double red[33];
  const int tsize = 1 << (G.g + G.kl);
  const long long t = blockIdx.x;
  cplx<T>* w = basis + (long long)j * P.dim;
  const cplx<T>* vp = basis + (long long)(j - 1) * P.dim;
  // u_j = w_j - alpha_{j-1} * v_{j-1}, v_{j-1} = u_{j-1} / ||u_{j-1}||
  const T a = j > 0 ? (T)scal[S_AOV + j - 1] : (T)0;
  T nrm_t = 0;  // per-thread partial in the element precision, summed in FP64 below
  for (int l = threadIdx.x; l < tsize; l += blockDim.x) {
    const long long x = tile_index(G, P.n, t, l);
    cplx<T> u = w[x];
    if (j > 0) {
      const cplx<T> p = vp[x];
      u.re = fma(-a, p.re, u.re);
      u.im = fma(-a, p.im, u.im);
      w[x] = u;
    }
    tile[l] = u;
    nrm_t = fma(u.re, u.re, fma(u.im, u.im, nrm_t));
  }
  double nrm = (double)nrm_t;
  __syncthreads();
  for (int l = threadIdx.x; l < tsize; l += blockDim.x) {
    const long long x = tile_index(G, P.n, t, l);
    const uint32_t fm = P.dist <= 3 ? flip_mask((uint32_t)x, P) : 0u;
    cplx<T> acc = mk<T>(0, 0);
#pragma unroll 4
    for (int b = G.lo; b < G.lo + G.g; ++b) {
      if (may_flip((uint32_t)x, fm, b, P)) {
        const cplx<T> v = tile[l ^ (1 << (G.kl + b - G.lo))];
        acc.re += v.re;
        acc.im += v.im;
      }
    }
    y[x] = acc;
  }
  nrm = block_sum(nrm, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = nrm;
}

// Lanczos epilogue for one amplitude: Hv, w_{j+1}, alpha partial.
template <typename T>
__device__ __forceinline__ T ex_epilogue_one(cplx<T> hu, cplx<T> u, long long x, cplx<T>* basis, long long dim,
                                             int j, bool write_next, T s, T beta_prev, T s_prev) {
  cplx<T> hv = mk<T>(hu.re * s, hu.im * s);
  const cplx<T> v = mk<T>(u.re * s, u.im * s);
  if (j > 0) {
    const cplx<T> p = basis[(long long)(j - 1) * dim + x];
    const T f = beta_prev * s_prev;
    hv.re = fma(-f, p.re, hv.re);
    hv.im = fma(-f, p.im, hv.im);
  }
  if (write_next) basis[(long long)(j + 1) * dim + x] = hv;
  return v.re * hv.re + v.im * hv.im;
}

// ---------------------------------------------------------------------------------
// high phases: y += H_p u_j over a high bit group; the last one runs the epilogue
// ---------------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kExactThreads) ex_phaseH(ExactParams P, PhaseGeom G, cplx<T>* basis, cplx<T>* y,
                                                           double* scal, double* partial, int j, int last, int m) {
  if (j >= (int)scal[S_MEFF]) return;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tile = reinterpret_cast<cplx<T>*>(smem_raw);
  __shared__ double red[33];
  const int tsize = 1 << (G.g + G.kl);
  const long long t = blockIdx.x;
  const cplx<T>* u_j = basis + (long long)j * P.dim;
  for (int l = threadIdx.x; l < tsize; l += blockDim.x) tile[l] = u_j[tile_index(G, P.n, t, l)];
  __syncthreads();
  const T s = (T)scal[S_INV + j];
  const T beta_prev = j > 0 ? (T)scal[S_NORM + j] : (T)0;
  const T s_prev = j > 0 ? (T)scal[S_INV + j - 1] : (T)0;
  const bool write_next = (j + 1) < m;
  T alpha_t = 0;
  for (int l = threadIdx.x; l < tsize; l += blockDim.x) {
    const long long x = tile_index(G, P.n, t, l);
    const uint32_t fm = P.dist <= 3 ? flip_mask((uint32_t)x, P) : 0u;
    cplx<T> acc = y[x];
#pragma unroll 4
    for (int b = G.lo; b < G.lo + G.g; ++b) {
      if (may_flip((uint32_t)x, fm, b, P)) {
        const cplx<T> v = tile[l ^ (1 << (G.kl + b - G.lo))];
        acc.re += v.re;
        acc.im += v.im;
      }
    }
    if (!last) {
      y[x] = acc;
    } else {
      alpha_t += ex_epilogue_one(acc, tile[l], x, basis, P.dim, j, write_next, s, beta_prev, s_prev);
    }
  }
  if (last) {
    const double alpha = block_sum((double)alpha_t, red);
    if (threadIdx.x == 0) partial[blockIdx.x] = alpha;
  }
}

// Elementwise epilogue when phase 0 already covered every bit (n <= tile bits).
template <typename T>
__global__ void ex_epilogue(ExactParams P, cplx<T>* basis, const cplx<T>* y, double* scal, double* partial, int j,
                            int m) {
  if (j >= (int)scal[S_MEFF]) return;
  __shared__ double red[33];
  const T s = (T)scal[S_INV + j];
  const T beta_prev = j > 0 ? (T)scal[S_NORM + j] : (T)0;
  const T s_prev = j > 0 ? (T)scal[S_INV + j - 1] : (T)0;
  const bool write_next = (j + 1) < m;
  T alpha_t = 0;
  const cplx<T>* u_j = basis + (long long)j * P.dim;
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < P.dim; x += (long long)gridDim.x * blockDim.x)
    alpha_t += ex_epilogue_one(y[x], u_j[x], x, basis, P.dim, j, write_next, s, beta_prev, s_prev);
  const double alpha = block_sum((double)alpha_t, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = alpha;
}

// Reduce partials into a scalar.  kind 0: ||u_j|| (with breakdown detection),
// kind 1: alpha_j.
__global__ void ex_reduce(double* scal, const double* partial, int count, int kind, int j, double tol) {
  if (j >= (int)scal[S_MEFF]) return;
  __shared__ double red[33];
  double v = 0.0;
  for (int i = threadIdx.x; i < count; i += blockDim.x) v += partial[i];
  v = block_sum(v, red);
  if (threadIdx.x != 0) return;
  if (kind == 0) {
    const double nrm = sqrt(v);
    if (j == 0) scal[S_NORM0] = nrm;
    if (j > 0 && !(nrm > tol * scal[S_NORM0])) {
      // Krylov space exhausted: H v_{j-1} lies in span(v_0..v_{j-1}).
      scal[S_MEFF] = (double)j;
      return;
    }
    scal[S_NORM + j] = nrm;
    scal[S_INV + j] = 1.0 / nrm;
  } else {
    scal[S_ALPHA + j] = v;
    scal[S_AOV + j] = v / scal[S_NORM + j];
  }
}

// c = exp(-i tau T) e_1 for the real symmetric tridiagonal T (alpha, beta) by a
// Taylor series applied in sub-steps of norm <= 1/2; one warp, FP64.  Writes the
// combination coefficients norm0 * c_k / ||u_k||.
__global__ void ex_finalize(double* scal) {
  __shared__ double yr[64], yi[64], tr[64], ti[64], nr[64], ni[64];
  const int m = (int)scal[S_MEFF];
  const double tau = scal[S_TAU];
  const int lane = threadIdx.x;
  double* alpha = scal + S_ALPHA;
  double* nrm = scal + S_NORM;  // beta_{k} = ||u_{k+1}||
  double rho = 0.0;
  for (int k = 0; k < m; ++k) {
    double r = fabs(alpha[k]);
    if (k > 0) r += nrm[k];
    if (k + 1 < m) r += nrm[k + 1];
    rho = fmax(rho, r);
  }
  if (!isfinite(rho) || fabs(tau) * rho > 1e4) rho = 0.0;  // cannot happen for ||H|| <= n; never loop unbounded
  const int q = max(1, (int)ceil(fabs(tau) * rho / 0.5));
  const double h = tau / q;
  for (int k = lane; k < 64; k += 32) {
    yr[k] = (k == 0) ? 1.0 : 0.0;
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
      // term <- (-i h / p) T term
      double loc = 0.0;
      double ur[2], ui[2];
      for (int s = 0; s < 2; ++s) {
        const int k = lane + 32 * s;
        double ar = 0.0, ai = 0.0;
        if (k < m) {
          ar = alpha[k] * tr[k];
          ai = alpha[k] * ti[k];
          if (k > 0) {
            ar += nrm[k] * tr[k - 1];
            ai += nrm[k] * ti[k - 1];
          }
          if (k + 1 < m) {
            ar += nrm[k + 1] * tr[k + 1];
            ai += nrm[k + 1] * ti[k + 1];
          }
        }
        // multiply by -i h / p: (ar + i ai)(-i c) = c ai - i c ar
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
  for (int k = lane; k < 64; k += 32) {
    double cr = 0.0, ci = 0.0;
    if (k < m) {
      const double f = scal[S_NORM0] / nrm[k];
      cr = yr[k] * f;
      ci = yi[k] * f;
    }
    scal[S_COEF + 2 * k] = cr;
    scal[S_COEF + 2 * k + 1] = ci;
  }
}

// psi (slot 0) <- sum_k coef_k u_k  (in place: each amplitude reads its slots first)
template <typename T>
__global__ void ex_combine(cplx<T>* basis, long long dim, const double* scal, int m) {
  __shared__ T cr[64], ci[64];
  const int meff = (int)scal[S_MEFF];
  if (threadIdx.x < 64) {
    cr[threadIdx.x] = (T)scal[S_COEF + 2 * threadIdx.x];
    ci[threadIdx.x] = (T)scal[S_COEF + 2 * threadIdx.x + 1];
  }
  __syncthreads();
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < dim; x += (long long)gridDim.x * blockDim.x) {
    cplx<T> acc = mk<T>(0, 0);
    for (int k = 0; k < meff; ++k) {
      const cplx<T> u = basis[(long long)k * dim + x];
      acc.re = fma(cr[k], u.re, acc.re);
      acc.re = fma(-ci[k], u.im, acc.re);
      acc.im = fma(cr[k], u.im, acc.im);
      acc.im = fma(ci[k], u.re, acc.im);
    }
    basis[x] = acc;
  }
}

__global__ void ex_begin(double* scal, int m, double tau) {
  if (threadIdx.x == 0) {
    scal[S_MEFF] = (double)m;
    scal[S_TAU] = tau;
  }
}

// ---------------------------------------------------------------------------------
// measurement: per bit b, sums of |psi|^2 over bit b = 1 and of psi[x] conj(psi[x|b])
// over bit b = 0, within tiles of the same bit groups as the H phases.
// ---------------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kExactThreads) ex_measure(ExactParams P, PhaseGeom G, const cplx<T>* psi,
                                                            double* partial) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cplx<T>* tile = reinterpret_cast<cplx<T>*>(smem_raw);
  __shared__ double red[33];
  const int tsize = 1 << (G.g + G.kl);
  const long long t = blockIdx.x;
  for (int l = threadIdx.x; l < tsize; l += blockDim.x) tile[l] = psi[tile_index(G, P.n, t, l)];
  __syncthreads();
  for (int b = G.lo; b < G.lo + G.g; ++b) {
    const int bit = 1 << (G.kl + b - G.lo);
    double p0 = 0.0, p1 = 0.0, orr = 0.0, oi = 0.0;
    for (int l = threadIdx.x; l < tsize; l += blockDim.x) {
      if (l & bit) continue;
      const cplx<T> a = tile[l];
      const cplx<T> c = tile[l | bit];
      p0 += (double)norm2(a);
      p1 += (double)norm2(c);
      // rho[0,1] = sum psi[x with bit 0] * conj(psi[x with bit 1])
      orr += (double)(a.re * c.re + a.im * c.im);
      oi += (double)(a.im * c.re - a.re * c.im);
    }
    p0 = block_sum(p0, red);
    p1 = block_sum(p1, red);
    orr = block_sum(orr, red);
    oi = block_sum(oi, red);
    if (threadIdx.x == 0) {
      double* o = partial + ((long long)blockIdx.x * P.n + (b - G.lo)) * 4;
      o[0] = p0;
      o[1] = p1;
      o[2] = orr;
      o[3] = oi;
    }
  }
}

// reduce measure partials of one phase: out[b*4 + c] = sum over blocks
__global__ void ex_measure_reduce(const double* partial, int blocks, int n, int g, int lo, double* out) {
  __shared__ double red[33];
  for (int k = 0; k < g * 4; ++k) {
    double v = 0.0;
    for (int i = threadIdx.x; i < blocks; i += blockDim.x) v += partial[((long long)i * n + k / 4) * 4 + k % 4];
    v = block_sum(v, red);
    if (threadIdx.x == 0) out[(lo + k / 4) * 4 + k % 4] = v;
  }
}

template <typename T>
__global__ void ex_to_c128(const cplx<T>* src, c128* dst, long long dim) {
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < dim; x += (long long)gridDim.x * blockDim.x)
    dst[x] = mk<double>((double)src[x].re, (double)src[x].im);
}
template <typename T>
__global__ void ex_from_c128(const c128* src, cplx<T>* dst, long long dim) {
  for (long long x = blockIdx.x * (long long)blockDim.x + threadIdx.x; x < dim; x += (long long)gridDim.x * blockDim.x)
    dst[x] = mk<T>((T)src[x].re, (T)src[x].im);
}

}  // namespace

// ===================================================================================
// host side
// ===================================================================================
struct ExactImpl {
  int n, distance, lo, hi, precision, m;
  long long dim;
  size_t esize;  // bytes per amplitude
  void* basis = nullptr;
  void* y = nullptr;
  void* staging = nullptr;  // complex128 staging for MIXED host transfers
  double* scal = nullptr;
  double* partial = nullptr;
  double* meas = nullptr;
  std::vector<PhaseGeom> phases;
  ExactParams P;
  int tile_bits;
  size_t partial_count;
};

}  // namespace qca

struct qca_exact {
  qca::ExactImpl impl;
};

using namespace qca;

namespace {

int plan_phases(ExactImpl& E) {
  // tile capacity: 128 KB of shared memory
  E.tile_bits = 13;  // 128 KB (complex128) / 64 KB (complex64) tiles
  E.phases.clear();
  const int g0 = std::min(E.n, E.tile_bits);
  E.phases.push_back(PhaseGeom{0, g0, 0});
  int lo = g0;
  while (lo < E.n) {
    const int kl_min = 2;  // runs of 4 amplitudes: 64 B (complex128) / 32 B, one sector (complex64)
    int g = std::min(E.n - lo, E.tile_bits - kl_min);
    int kl = std::min(E.tile_bits - g, lo);
    E.phases.push_back(PhaseGeom{lo, g, kl});
    lo += g;
  }
  return QCA_OK;
}

template <typename T>
int exact_step_impl(ExactImpl& E, double step_size, int nsteps, cudaStream_t st) {
  const int m = E.m;
  // sub-steps so that tau * ||H|| <= 4 (||H|| <= n)
  const double tau_total = M_PI / 2 * step_size;
  const int sub = std::max(1, (int)std::ceil(std::fabs(tau_total) * E.n / 4.0));
  const double tau = tau_total / sub;
  cplx<T>* basis = (cplx<T>*)E.basis;
  cplx<T>* y = (cplx<T>*)E.y;
  const int ntile0 = (int)(E.dim >> (E.phases[0].g + E.phases[0].kl));
  const double tol = std::is_same<T, double>::value ? 1e-13 : 1e-6;
  for (int s = 0; s < nsteps * sub; ++s) {
    ex_begin<<<1, 32, 0, st>>>(E.scal, m, tau);
    for (int j = 0; j < m; ++j) {
      const PhaseGeom& g0 = E.phases[0];
      const size_t sm0 = sizeof(cplx<T>) << (g0.g + g0.kl);
      ex_phase0<T><<<ntile0, kExactThreads, sm0, st>>>(E.P, g0, basis, y, E.scal, E.partial, j);
      ex_reduce<<<1, 1024, 0, st>>>(E.scal, E.partial, ntile0, 0, j, tol);
      int count = 0;
      if (E.phases.size() == 1) {
        const int blocks = std::min<long long>(4 * 152, (E.dim + 255) / 256);
        ex_epilogue<T><<<blocks, 256, 0, st>>>(E.P, basis, y, E.scal, E.partial, j, m);
        count = blocks;
      } else {
        for (size_t p = 1; p < E.phases.size(); ++p) {
          const PhaseGeom& g = E.phases[p];
          const int nt = (int)(E.dim >> (g.g + g.kl));
          const size_t smb = sizeof(cplx<T>) << (g.g + g.kl);
          ex_phaseH<T><<<nt, kExactThreads, smb, st>>>(E.P, g, basis, y, E.scal, E.partial, j,
                                                       p + 1 == E.phases.size() ? 1 : 0, m);
          count = nt;
        }
      }
      ex_reduce<<<1, 1024, 0, st>>>(E.scal, E.partial, count, 1, j, tol);
    }
    ex_finalize<<<1, 32, 0, st>>>(E.scal);
    const int blocks = std::min<long long>(8 * 152, (E.dim + 255) / 256);
    ex_combine<T><<<blocks, 256, 0, st>>>(basis, E.dim, E.scal, m);
  }
  QCA_LAUNCH_CHECK();
  return QCA_OK;
}

template <typename T>
int set_smem_attrs() {
  QCA_CUDA(cudaFuncSetAttribute(ex_phase0<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 128 * 1024));
  QCA_CUDA(cudaFuncSetAttribute(ex_phaseH<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 128 * 1024));
  QCA_CUDA(cudaFuncSetAttribute(ex_measure<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 128 * 1024));
  return QCA_OK;
}

template <typename T>
int exact_measure_impl(ExactImpl& E, double* population, double* rho, cudaStream_t st) {
  const cplx<T>* psi = (const cplx<T>*)E.basis;
  for (const PhaseGeom& g : E.phases) {
    const int nt = (int)(E.dim >> (g.g + g.kl));
    const size_t smb = sizeof(cplx<T>) << (g.g + g.kl);
    ex_measure<T><<<nt, kExactThreads, smb, st>>>(E.P, g, psi, E.partial);
    ex_measure_reduce<<<1, 1024, 0, st>>>(E.partial, nt, E.n, g.g, g.lo, E.meas);
  }
  QCA_LAUNCH_CHECK();
  std::vector<double> h(4 * E.n);
  QCA_CUDA(cudaMemcpyAsync(h.data(), E.meas, sizeof(double) * 4 * E.n, cudaMemcpyDeviceToHost, st));
  QCA_CUDA(cudaStreamSynchronize(st));
  for (int i = 0; i < E.n; ++i) {
    const double* v = h.data() + 4 * (E.n - 1 - i);  // cell i lives at bit n-1-i
    if (population) population[i] = v[1];
    if (rho) {
      // rho[s, s'] = sum_rest psi[.., s, ..] conj(psi[.., s', ..])  (mps.py:122-126)
      double* r = rho + 8 * i;
      r[0] = v[0];
      r[1] = 0.0;
      r[2] = v[2];
      r[3] = v[3];
      r[4] = v[2];
      r[5] = -v[3];
      r[6] = v[1];
      r[7] = 0.0;
    }
  }
  return QCA_OK;
}

}  // namespace

extern "C" {

int qca_exact_footprint(int n_cells, int precision, int krylov_dim, size_t* bytes) {
  if (!bytes || n_cells < 1 || n_cells > kMaxCells || krylov_dim < 1 || krylov_dim > 60) {
    set_error("qca_exact_footprint: invalid arguments");
    return QCA_ERR_INVALID;
  }
  const size_t es = precision == QCA_PREC_FP64 ? 16 : 8;
  const size_t dim = (size_t)1 << n_cells;
  *bytes = es * dim * (krylov_dim + 1) + (precision == QCA_PREC_FP64 ? 0 : 16 * dim) + (1 << 20);
  return QCA_OK;
}

int qca_exact_create(int n_cells, int distance, int interval_lo, int interval_hi, int precision, int krylov_dim,
                     qca_exact** out) {
  if (!out) {
    set_error("qca_exact_create: out is NULL");
    return QCA_ERR_INVALID;
  }
  *out = nullptr;
  if (n_cells < 2 || n_cells > kMaxCells || distance < 1 || interval_lo < 0 || interval_hi <= interval_lo ||
      (precision != QCA_PREC_FP64 && precision != QCA_PREC_MIXED) || krylov_dim < 1 || krylov_dim > 60) {
    set_error("qca_exact_create: invalid arguments (n=%d distance=%d interval=[%d,%d) precision=%d krylov=%d)", n_cells,
              distance, interval_lo, interval_hi, precision, krylov_dim);
    return QCA_ERR_INVALID;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("qca_exact_create: no CUDA device");
    return QCA_ERR_NO_DEVICE;
  }
  qca_exact* h = new qca_exact();
  ExactImpl& E = h->impl;
  E.n = n_cells;
  E.distance = distance;
  E.lo = interval_lo;
  E.hi = interval_hi;
  E.precision = precision;
  E.m = krylov_dim;
  E.dim = 1LL << n_cells;
  E.esize = precision == QCA_PREC_FP64 ? 16 : 8;
  E.P.n = n_cells;
  E.P.rule_lo = interval_lo;
  E.P.rule_hi = interval_hi;
  E.P.dim = E.dim;
  E.P.dist = distance;
  for (int b = 0; b < kMaxCells; ++b) E.P.nmask[b] = 0;
  for (int b = 0; b < n_cells; ++b) {
    const int i = n_cells - 1 - b;
    uint32_t mask = 0;
    for (int jc = std::max(0, i - distance); jc <= std::min(n_cells - 1, i + distance); ++jc)
      if (jc != i) mask |= 1u << (n_cells - 1 - jc);
    E.P.nmask[b] = mask;
  }
  plan_phases(E);
  size_t maxtiles = 1;
  for (auto& g : E.phases) maxtiles = std::max(maxtiles, (size_t)(E.dim >> (g.g + g.kl)));
  E.partial_count = std::max<size_t>(maxtiles * n_cells * 4, 8 * 152 + 1024);
  auto fail = [&](int code) {
    qca_exact_destroy(h);
    return code;
  };
  if (cudaMalloc(&E.basis, E.esize * E.dim * E.m) != cudaSuccess ||
      cudaMalloc(&E.y, E.esize * E.dim) != cudaSuccess || cudaMalloc(&E.scal, sizeof(double) * S_TOTAL) != cudaSuccess ||
      cudaMalloc(&E.partial, sizeof(double) * E.partial_count) != cudaSuccess ||
      cudaMalloc(&E.meas, sizeof(double) * 4 * kMaxCells) != cudaSuccess) {
    cudaGetLastError();
    set_error("qca_exact_create: device allocation of %zu bytes failed", E.esize * E.dim * (E.m + 1));
    return fail(QCA_ERR_OOM);
  }
  if (precision == QCA_PREC_MIXED) {
    if (cudaMalloc(&E.staging, 16 * E.dim) != cudaSuccess) {
      cudaGetLastError();
      set_error("qca_exact_create: staging allocation failed");
      return fail(QCA_ERR_OOM);
    }
  }
  int s = precision == QCA_PREC_FP64 ? set_smem_attrs<double>() : set_smem_attrs<float>();
  if (s != QCA_OK) return fail(s);
  if (cudaMemset(E.basis, 0, E.esize * E.dim) != cudaSuccess) return fail(QCA_ERR_CUDA);
  *out = h;
  return QCA_OK;
}

int qca_exact_destroy(qca_exact* h) {
  if (!h) return QCA_OK;
  ExactImpl& E = h->impl;
  cudaFree(E.basis);
  cudaFree(E.y);
  cudaFree(E.staging);
  cudaFree(E.scal);
  cudaFree(E.partial);
  cudaFree(E.meas);
  delete h;
  return QCA_OK;
}

int qca_exact_set_state(qca_exact* h, const double* psi, void* stream) {
  if (!h || !psi) {
    set_error("qca_exact_set_state: NULL argument");
    return QCA_ERR_INVALID;
  }
  ExactImpl& E = h->impl;
  cudaStream_t st = (cudaStream_t)stream;
  if (E.precision == QCA_PREC_FP64) {
    QCA_CUDA(cudaMemcpyAsync(E.basis, psi, 16 * E.dim, cudaMemcpyHostToDevice, st));
  } else {
    QCA_CUDA(cudaMemcpyAsync(E.staging, psi, 16 * E.dim, cudaMemcpyHostToDevice, st));
    ex_from_c128<float><<<8 * 152, 256, 0, st>>>((const c128*)E.staging, (c64*)E.basis, E.dim);
    QCA_LAUNCH_CHECK();
  }
  return QCA_OK;
}

int qca_exact_set_state_device(qca_exact* h, const void* psi_dev, void* stream) {
  if (!h || !psi_dev) {
    set_error("qca_exact_set_state_device: NULL argument");
    return QCA_ERR_INVALID;
  }
  ExactImpl& E = h->impl;
  QCA_CUDA(cudaMemcpyAsync(E.basis, psi_dev, E.esize * E.dim, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  return QCA_OK;
}

int qca_exact_get_state(qca_exact* h, double* psi, void* stream) {
  if (!h || !psi) {
    set_error("qca_exact_get_state: NULL argument");
    return QCA_ERR_INVALID;
  }
  ExactImpl& E = h->impl;
  cudaStream_t st = (cudaStream_t)stream;
  if (E.precision == QCA_PREC_FP64) {
    QCA_CUDA(cudaMemcpyAsync(psi, E.basis, 16 * E.dim, cudaMemcpyDeviceToHost, st));
  } else {
    ex_to_c128<float><<<8 * 152, 256, 0, st>>>((const c64*)E.basis, (c128*)E.staging, E.dim);
    QCA_LAUNCH_CHECK();
    QCA_CUDA(cudaMemcpyAsync(psi, E.staging, 16 * E.dim, cudaMemcpyDeviceToHost, st));
  }
  QCA_CUDA(cudaStreamSynchronize(st));
  return QCA_OK;
}

int qca_exact_state_device(qca_exact* h, void** psi_dev) {
  if (!h || !psi_dev) {
    set_error("qca_exact_state_device: NULL argument");
    return QCA_ERR_INVALID;
  }
  *psi_dev = h->impl.basis;
  return QCA_OK;
}

int qca_exact_step(qca_exact* h, double step_size, int nsteps, void* stream) {
  if (!h || nsteps < 0 || !std::isfinite(step_size)) {
    set_error("qca_exact_step: invalid arguments");
    return QCA_ERR_INVALID;
  }
  ExactImpl& E = h->impl;
  if (nsteps == 0) return QCA_OK;
  cudaStream_t st = (cudaStream_t)stream;
  return E.precision == QCA_PREC_FP64 ? exact_step_impl<double>(E, step_size, nsteps, st)
                                      : exact_step_impl<float>(E, step_size, nsteps, st);
}

int qca_exact_measure(qca_exact* h, double* population, double* rho, void* stream) {
  if (!h) {
    set_error("qca_exact_measure: NULL handle");
    return QCA_ERR_INVALID;
  }
  ExactImpl& E = h->impl;
  cudaStream_t st = (cudaStream_t)stream;
  return E.precision == QCA_PREC_FP64 ? exact_measure_impl<double>(E, population, rho, st)
                                      : exact_measure_impl<float>(E, population, rho, st);
}

}  // extern "C"

// ===================================================================================
// Allocation-free exact step.
//
// Some callers of this library may not allocate device memory at all: host
// applications whose device memory is owned by their own pool or budget manager,
// and latency-critical loops that cannot afford the implicit device
// synchronisation of cudaMalloc / cudaFree.  qca_exact_step_noalloc serves them:
// it evolves a caller-owned complex128 state (device pointers in and out) with the
// same kernels as qca_exact_step, but its scratch (the Krylov basis, the H v
// buffer, the Lanczos scalars and partial sums) lives in the file-scope array
// below, which every GPU that loads the library holds until the process exits.
// ===================================================================================
namespace {

constexpr size_t kNoAllocScratchBytes = 16u << 20;  // 16 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_addr[64] = {};  // per device: device address of g_noalloc_scratch

// Per device, with that device current: resolve the array's device address (the
// host-side symbol is only a stand-in) and set the kernels' shared-memory limit.
int noalloc_setup(void** addr) {
  int dev = 0;
  QCA_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) {
    set_error("qca_exact_step_noalloc: device ordinal %d out of range", dev);
    return QCA_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();  // clear it, so that no later launch check reports it
      set_error("qca_exact_step_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return QCA_ERR_CUDA;
    }
    QCA_TRY(set_smem_attrs<double>());
    g_noalloc_addr[dev] = p;
  }
  *addr = g_noalloc_addr[dev];
  return QCA_OK;
}

}  // namespace

extern "C" int qca_exact_step_noalloc(int n_cells, int distance, int interval_lo, int interval_hi, int krylov_dim,
                                      double step_size, int nsteps, const void* psi_in, void* psi_out,
                                      void* stream) {
  if (!psi_in || !psi_out || n_cells < 2 || n_cells > kMaxCells || distance < 1 || interval_lo < 0 ||
      interval_hi <= interval_lo || krylov_dim < 1 || krylov_dim > 60 || nsteps < 0 || !std::isfinite(step_size)) {
    set_error("qca_exact_step_noalloc: invalid arguments");
    return QCA_ERR_INVALID;
  }
  ExactImpl E;
  E.n = n_cells;
  E.distance = distance;
  E.lo = interval_lo;
  E.hi = interval_hi;
  E.precision = QCA_PREC_FP64;
  E.m = krylov_dim;
  E.dim = 1LL << n_cells;
  E.esize = 16;
  E.P.n = n_cells;
  E.P.rule_lo = interval_lo;
  E.P.rule_hi = interval_hi;
  E.P.dim = E.dim;
  E.P.dist = distance;
  for (int b = 0; b < kMaxCells; ++b) E.P.nmask[b] = 0;
  for (int b = 0; b < n_cells; ++b) {
    const int i = n_cells - 1 - b;
    uint32_t mask = 0;
    for (int jc = std::max(0, i - distance); jc <= std::min(n_cells - 1, i + distance); ++jc)
      if (jc != i) mask |= 1u << (n_cells - 1 - jc);
    E.P.nmask[b] = mask;
  }
  plan_phases(E);
  size_t maxtiles = 1;
  for (auto& g : E.phases) maxtiles = std::max(maxtiles, (size_t)(E.dim >> (g.g + g.kl)));
  E.partial_count = std::max<size_t>(maxtiles * n_cells * 4, 8 * 152 + 1024);
  // scratch carve-up: basis (m slots), y, scalars, partials; 256-byte aligned
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t b_basis = up(E.esize * E.dim * E.m), b_y = up(E.esize * E.dim);
  const size_t b_scal = up(sizeof(double) * S_TOTAL), b_part = up(sizeof(double) * E.partial_count);
  const size_t need = b_basis + b_y + b_scal + b_part;
  if (need > kNoAllocScratchBytes) {
    set_error("qca_exact_step_noalloc: %d cells with Krylov dimension %d need %zu bytes of scratch; the static "
              "scratch holds %zu bytes (use qca_exact_create for larger states)",
              n_cells, krylov_dim, need, kNoAllocScratchBytes);
    return QCA_ERR_INVALID;
  }
  void* base = nullptr;
  QCA_TRY(noalloc_setup(&base));
  char* p = (char*)base;
  E.basis = p;
  E.y = p + b_basis;
  E.scal = (double*)(p + b_basis + b_y);
  E.partial = (double*)(p + b_basis + b_y + b_scal);
  cudaStream_t st = (cudaStream_t)stream;
  // the array keeps the previous call's contents: start from zeroed scalars
  QCA_CUDA(cudaMemsetAsync(E.scal, 0, b_scal, st));
  QCA_CUDA(cudaMemcpyAsync(E.basis, psi_in, E.esize * E.dim, cudaMemcpyDeviceToDevice, st));
  if (nsteps > 0) QCA_TRY(exact_step_impl<double>(E, step_size, nsteps, st));
  QCA_CUDA(cudaMemcpyAsync(psi_out, E.basis, E.esize * E.dim, cudaMemcpyDeviceToDevice, st));
  E.basis = nullptr;  // not owned
  E.y = nullptr;
  E.scal = nullptr;
  E.partial = nullptr;
  return QCA_OK;
}
