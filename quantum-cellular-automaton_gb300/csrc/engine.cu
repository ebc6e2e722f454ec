// TDVP engine: many MPS chains evolved side by side on one GPU.
//
// Replaces algorithms/tdvp.py:10-365.  Each chain owns its site tensors
// A[i] (2, D_i, D_{i+1}) (double buffered), its environments (layout
// E[w][ket][bra]) and a workspace; all live in one device allocation.  Chains
// advance in lock-step "ticks": in a tick every active chain performs its next
// local update (a 2TDVP bond update or a 1TDVP site update) and every stage of
// that update is one grouped launch over all chains (tdvp_kernels.cuh).  The
// host mirrors the bond dimensions; it synchronises once per tick to learn the
// truncated bond dimensions of the 2-site splits, and every few Lanczos
// iterations to stop when every local exponential has converged.  Chains added
// since the last operation are initialised (TDVP.__init__) together, one grouped
// launch per sweep position, before the next step or measurement.
//
// Gauge handling (what "parity" means for TDVP):
//  * 2TDVP is evolved in the gauge-consistent form: the environments always
//    match the tensors, so the result does not depend on the SVD phase
//    convention.
//  * 1TDVP follows the reference's QR sequence (LAPACK reflector convention),
//    including the canonicalisation after a measurement, because its bond
//    growth uses the complement columns of the complete QR (tdvp.py:74, 95).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <limits>
#include <map>
#include <memory>
#include <vector>

#include "tdvp_kernels.cuh"

namespace qca {

namespace {

size_t align_up(size_t x, size_t a = 256) { return (x + a - 1) / a * a; }

struct HostW {  // W[s, s', a, b] complex128, (2, 2, wl, wr) C order
  int wl = 0, wr = 0;
  std::vector<c128> v;
  c128 at(int s, int sp, int a, int b) const { return v[(((size_t)s * 2 + sp) * wl + a) * wr + b]; }
};

struct EntryListHost {
  std::vector<WEntry> ent;
  std::vector<int> begin;
  int nout = 0;
};

// entries (in_block, out_block, value) sorted by out_block
EntryListHost make_list(int nout, std::vector<WEntry> ent) {
  std::stable_sort(ent.begin(), ent.end(), [](const WEntry& a, const WEntry& b) { return a.out_block < b.out_block; });
  EntryListHost L;
  L.nout = nout;
  L.begin.assign(nout + 1, 0);
  for (const WEntry& e : ent) L.begin[e.out_block + 1]++;
  for (int i = 0; i < nout; ++i) L.begin[i + 1] += L.begin[i];
  L.ent = std::move(ent);
  return L;
}

bool nz(c128 z) { return z.re != 0.0 || z.im != 0.0; }

// 1-site effective Hamiltonian: in T1[wr][s], out T2[s'][wl]
EntryListHost list_mv1(const HostW& W) {
  std::vector<WEntry> e;
  for (int s = 0; s < 2; ++s)
    for (int sp = 0; sp < 2; ++sp)
      for (int a = 0; a < W.wl; ++a)
        for (int b = 0; b < W.wr; ++b) {
          const c128 z = W.at(s, sp, a, b);
          if (nz(z)) e.push_back(WEntry{b * 2 + s, sp * W.wl + a, z.re, z.im});
        }
  return make_list(2 * W.wl, e);
}

// 2-site merged W (tdvp.py:281-284): s = s1*2+s2, in T1[wr][s], out T2[s'][wl]
EntryListHost list_mv2(const HostW& W1, const HostW& W2) {
  std::vector<WEntry> e;
  const int wl = W1.wl, wm = W1.wr, wr = W2.wr;
  for (int s1 = 0; s1 < 2; ++s1)
    for (int s2 = 0; s2 < 2; ++s2)
      for (int p1 = 0; p1 < 2; ++p1)
        for (int p2 = 0; p2 < 2; ++p2)
          for (int a = 0; a < wl; ++a)
            for (int b = 0; b < wr; ++b) {
              c128 acc = mk<double>(0, 0);
              for (int m = 0; m < wm; ++m) acc = acc + W1.at(s1, p1, a, m) * W2.at(s2, p2, m, b);
              if (nz(acc)) e.push_back(WEntry{b * 4 + (s1 * 2 + s2), (p1 * 2 + p2) * wl + a, acc.re, acc.im});
            }
  return make_list(4 * wl, e);
}

// left environment: in X[wl][s'], out Y[wr][s]
EntryListHost list_envl(const HostW& W) {
  std::vector<WEntry> e;
  for (int s = 0; s < 2; ++s)
    for (int sp = 0; sp < 2; ++sp)
      for (int a = 0; a < W.wl; ++a)
        for (int b = 0; b < W.wr; ++b) {
          const c128 z = W.at(s, sp, a, b);
          if (nz(z)) e.push_back(WEntry{a * 2 + sp, b * 2 + s, z.re, z.im});
        }
  return make_list(2 * W.wr, e);
}

// right environment: in X[wr][s'], out Y[wl][s]
EntryListHost list_envr(const HostW& W) {
  std::vector<WEntry> e;
  for (int s = 0; s < 2; ++s)
    for (int sp = 0; sp < 2; ++sp)
      for (int a = 0; a < W.wl; ++a)
        for (int b = 0; b < W.wr; ++b) {
          const c128 z = W.at(s, sp, a, b);
          if (nz(z)) e.push_back(WEntry{b * 2 + sp, a * 2 + s, z.re, z.im});
        }
  return make_list(2 * W.wl, e);
}

struct EL {
  const WEntry* ent = nullptr;
  const int* begin = nullptr;
  int nout = 0;
};

}  // namespace

// ==================================================================================
template <typename T>
struct Chain {
  int id = -1;
  int N = 0, algo = 0, chi = 0;
  double eps = 0, dt = 0;
  std::vector<int> w, D, cap, target;
  std::vector<int> maxb;  // min(2^i, 2^(N-i), chi) (tdvp.py:31-35); target is recomputed by a1tdvp
  int* a1flags = nullptr; // a1tdvp pass: [b] new target of bond b, [N + 1 + 2 b] SVD status, [+1] sweeps
  std::vector<cplx<T>*> A[2];
  std::vector<int> par;
  std::vector<cplx<T>*> Lenv, Renv;  // Lenv[i+1]: after site i (Lenv[0] = boundary); Renv[i]: before site i
  std::vector<EL> mv1, mv2, envl, envr;
  cplx<T>* theta = nullptr;
  cplx<T>* basis = nullptr;
  long long nmax = 0;
  cplx<T>* t1 = nullptr;
  cplx<T>* t2 = nullptr;
  cplx<T>* svdw = nullptr;
  cplx<T>* qrw = nullptr;
  cplx<T>* qrtau = nullptr;
  cplx<T>* cbuf = nullptr;
  double* lzS = nullptr;
  double* lzP = nullptr;
  double* sv = nullptr;
  double* dscal = nullptr;  // [0] discarded weight of the current step, [1..4] rho
  int* iflags = nullptr;    // [0] k_out, [1] svd status, [2] svd sweeps, [3] Lanczos failure bits
  void* mem = nullptr;
  size_t bytes = 0;
  int max_chunks = 1;
  int cmax = 1;  // largest bond capacity
  // sweep state
  int dir = 0;  // 0 right, 1 left
  int pos = 0;
  long long todo = 0;  // time steps scheduled and not yet completed (the current one included)
  bool in_step = false;  // a time step has begun and its sweeps are not finished
  long long steps_done = 0;  // time steps completed since the chain was added
  int center = 0;     // orthogonality centre (0 after a full step)
  int lz_used = 0;    // largest Krylov dimension in the current step
  int svd_sweeps = 0; // most Jacobi sweeps of a two-site split in the current step
  double disc_host = 0.0;
  int status = 0;             // QCA_ERR_NAN / QCA_ERR_NOT_CONVERGED once the chain has failed
  int fail_site = -1;         // bond or site of the local update that failed
  const char* fail_what = "";
  bool pending_init = false;  // uploaded, TDVP.__init__ not yet run
  cplx<T>* cur(int i) { return A[par[i]][i]; }
  cplx<T>* alt(int i) { return A[par[i] ^ 1][i]; }
};


// ---------------------------------------------------------------------------------
// Host-side address validation: every operand range a descriptor can touch must lie
// inside the owning chain's device allocation (or the engine's staging).  A failure
// is returned as QCA_ERR_INVALID before anything is launched.
// ---------------------------------------------------------------------------------
// kernel classes reported by qca_engine_kernel_stats
enum : int { KC_GEMM = 0, KC_WAPPLY, KC_LZVEC, KC_LZFIN, KC_SVD, KC_QR, KC_MISC, KC_N };

struct Span {
  const char* lo;
  const char* hi;
};

template <typename T>
bool in_spans(const std::vector<Span>& spans, const void* p, long long max_off) {
  if (!p) return false;
  const char* a = (const char*)p;
  const char* b = a + (max_off + 1) * (long long)sizeof(cplx<T>);
  for (const Span& s : spans)
    if (a >= s.lo && b <= s.hi) return true;
  return false;
}

inline long long ext(long long n, long long s) { return n > 0 ? (n - 1) * (s < 0 ? -s : s) : 0; }

struct EngineBase {
  virtual ~EngineBase() = default;
  virtual int add(const qca_chain_desc* d, cudaStream_t st, int* id) = 0;
  virtual int remove(int id) = 0;
  virtual int step(const int* ids, int count, int nsteps, cudaStream_t st) = 0;
  virtual int schedule(int id, int nsteps) = 0;
  virtual int advance(const int* ids, int count, int max_ticks, cudaStream_t st) = 0;
  virtual int progress(int id, long long* out) = 0;
  virtual int measure(int id, double* pop, double* dpop, double* sse, double* bonds, cudaStream_t st) = 0;
  virtual int measure_many(const int* ids, int count, double* pop, double* dpop, double* sse, double* bonds,
                           cudaStream_t st) = 0;
  virtual int bonds(int id, int* out) = 0;
  virtual int get_mps(int id, double* out, size_t cap, cudaStream_t st) = 0;
  virtual int stats(int id, double* out) = 0;
  virtual int stats_ex(int id, double* out, int count) = 0;
  virtual std::vector<int> ids() const = 0;
  virtual int kernel_stats(double* out, int reset) = 0;
  virtual int set_profile(int on) = 0;
  size_t budget = 0, used = 0;
};

size_t chain_bytes_estimate(const qca_chain_desc* d, size_t esize, int mmax, std::vector<int>* cap_out);

template <typename T>
struct Engine final : EngineBase {
  std::map<int, std::unique_ptr<Chain<T>>> chains;
  int next_id = 0;
  int mmax = 40;
  bool use_tc = true;    // tensor-core GEMMs in the mixed path
  bool use_umma = true;  // ... with the tcgen05 kernel for M >= kUmmaMinM
  // Krylov truncation tolerance of every local exponential (error estimate
  // beta_j |(exp(-i tau T) e_1)_j|).  The mixed path's accuracy is set by its FP32
  // storage (about 1e-7 relative per local update); 1e-7 keeps the Krylov
  // truncation at that level (tighter values add iterations without changing
  // the measured population error).
  double lz_tol = std::is_same<T, double>::value ? 1e-12 : 1e-7;
  // descriptor staging (pinned host + device), bump allocated, reset after a sync
  char* h_stage = nullptr;
  char* d_stage = nullptr;
  size_t stage_cap = 0, stage_off = 0;
  int* h_done = nullptr;
  int* d_done = nullptr;
  int* h_k = nullptr;
  int done_cap = 0;
  cudaStream_t cur_st = nullptr;

  // optional per-kernel-class timing with CUDA events (qca_engine_profile)
  bool prof = false;
  struct Pend {
    int cls;
    cudaEvent_t a, b;
    double flops, bytes, kernels;
  };
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<Pend> pend;
  double acc[KC_N][4] = {};

  cudaEvent_t next_event() {
    if (ev_used == ev_pool.size()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      ev_pool.push_back(e);
    }
    return ev_pool[ev_used++];
  }
  template <typename F>
  int timed(int cls, double flops, double bytes, cudaStream_t st, F&& f) {
    if (!prof) return f();
    cudaEvent_t a = next_event(), b = next_event();
    const long long k0 = launches_so_far();
    cudaEventRecord(a, st);
    const int s = f();
    cudaEventRecord(b, st);
    pend.push_back(Pend{cls, a, b, flops, bytes, (double)(launches_so_far() - k0)});
    return s;
  }
  void resolve() {
    for (auto& p : pend) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, p.a, p.b);
      acc[p.cls][0] += p.kernels;
      acc[p.cls][1] += ms;
      acc[p.cls][2] += p.flops;
      acc[p.cls][3] += p.bytes;
    }
    pend.clear();
    ev_used = 0;
  }
  int kernel_stats(double* out, int reset) override {
    for (int c = 0; c < KC_N; ++c)
      for (int k = 0; k < 4; ++k) out[4 * c + k] = acc[c][k];
    if (reset) memset(acc, 0, sizeof(acc));
    return QCA_OK;
  }
  int set_profile(int on) override {
    prof = on != 0;
    return QCA_OK;
  }

  ~Engine() override {
    for (auto e : ev_pool) cudaEventDestroy(e);
    for (int i = 0; i < 4; ++i) {
      if (aux[i]) cudaStreamDestroy(aux[i]);
      if (join_ev[i]) cudaEventDestroy(join_ev[i]);
    }
    if (fork_ev) cudaEventDestroy(fork_ev);
    for (auto& kv : chains) cudaFree(kv.second->mem);
    cudaFreeHost(h_stage);
    cudaFree(d_stage);
    cudaFreeHost(h_done);
    cudaFree(d_done);
    cudaFreeHost(h_k);
  }

  int init(size_t budget_bytes) {
    stage_cap = 16u << 20;
    QCA_CUDA(cudaMallocHost(&h_stage, stage_cap));
    QCA_CUDA(cudaMalloc(&d_stage, stage_cap));
    done_cap = 4096;
    QCA_CUDA(cudaMallocHost(&h_done, sizeof(int) * done_cap));
    QCA_CUDA(cudaMalloc(&d_done, sizeof(int) * done_cap));
    QCA_CUDA(cudaMallocHost(&h_k, sizeof(int) * 4 * done_cap));
    size_t fr = 0, tot = 0;
    QCA_CUDA(cudaMemGetInfo(&fr, &tot));
    budget = budget_bytes ? budget_bytes : (size_t)(0.9 * fr);
    return QCA_OK;
  }

  int sync(cudaStream_t st) {
    QCA_CUDA(cudaStreamSynchronize(st));
    stage_off = 0;
    if (!pend.empty()) resolve();
    return QCA_OK;
  }

  template <typename Dsc>
  int upload(const std::vector<Dsc>& v, cudaStream_t st, const Dsc** out) {
    const size_t bytes = align_up(sizeof(Dsc) * v.size());
    if (bytes > stage_cap) {
      set_error("descriptor staging overflow (%zu bytes)", bytes);
      return QCA_ERR_INVALID;
    }
    if (stage_off + bytes > stage_cap) QCA_TRY(sync(st));
    memcpy(h_stage + stage_off, v.data(), sizeof(Dsc) * v.size());
    QCA_CUDA(cudaMemcpyAsync(d_stage + stage_off, h_stage + stage_off, sizeof(Dsc) * v.size(), cudaMemcpyHostToDevice,
                             st));
    *out = reinterpret_cast<const Dsc*>(d_stage + stage_off);
    stage_off += bytes;
    return QCA_OK;
  }

  std::vector<Span> spans() const {
    std::vector<Span> s;
    for (auto& kv : chains) s.push_back(Span{(const char*)kv.second->mem, (const char*)kv.second->mem + kv.second->bytes});
    return s;
  }
  static int bad(const char* what) {
    set_error("descriptor validation failed: %s operand outside its chain allocation", what);
    return QCA_ERR_INVALID;
  }

  // ---------------------------------------------------------------- grouped launches
  int run_gemm(std::vector<GemmDesc<T>>& v, cudaStream_t st) {
    if (v.empty()) return QCA_OK;
    const std::vector<Span> sp = spans();
    for (auto& d : v) {
      const long long ea = ext(d.M, d.sAm) + ext(d.K, d.sAk) + ext(d.G, d.sAg) + ext(d.nb1, d.sAb1) + ext(d.nb2, d.sAb2);
      const long long eb = ext(d.K, d.sBk) + ext(d.N, d.sBn) + ext(d.G, d.sBg) + ext(d.nb1, d.sBb1) + ext(d.nb2, d.sBb2);
      const long long ec = ext(d.M, d.sCm) + ext(d.N, d.sCn) + ext(d.nb1, d.sCb1) + ext(d.nb2, d.sCb2);
      if (d.M <= 0 || d.N <= 0 || d.K <= 0 || d.G <= 0 || d.nb1 <= 0 || d.nb2 <= 0) return bad("gemm shape");
      if (!in_spans<T>(sp, d.A, ea)) return bad("gemm A");
      if (!in_spans<T>(sp, d.B, eb)) return bad("gemm B");
      if (!in_spans<T>(sp, d.C, ec)) return bad("gemm C");
    }
    int mx = 1, nxx = 1;
    for (auto& d : v) {
      mx = std::max(mx, d.M);
      nxx = std::max(nxx, d.N);
    }
    const int cfg = gemm_tile_cfg(mx, nxx);
    double fl = 0.0, by = 0.0;
    for (auto& d : v) {
      const double nb = (double)d.nb1 * d.nb2 * d.G;
      fl += 8.0 * d.M * d.N * (double)d.K * nb;
      by += sizeof(cplx<T>) * ((double)d.M * d.K * nb + (double)d.K * d.N * nb + (double)d.M * d.N * d.nb1 * d.nb2);
    }
    auto tile = [](std::vector<GemmDesc<T>>& w, int bm, int bn) {
      int t = 0;
      for (auto& d : w) {
        d.tiles_m = ceil_div(d.M, bm);
        d.tiles_n = ceil_div(d.N, bn);
        d.tile_begin = t;
        t += d.nb1 * d.nb2 * d.tiles_m * d.tiles_n;
      }
    };
    if (!std::is_same<T, float>::value || !use_tc) {
      const int td = gemm_tile_dim(cfg);
      tile(v, td, td);
      const GemmDesc<T>* dd;
      QCA_TRY(upload(v, st, &dd));
      return timed(KC_GEMM, fl, by, st, [&] { return launch_gemm<T>(dd, v.data(), (int)v.size(), cfg, st); });
    }
    // mixed path: 3xTF32 on the tensor cores.  Problems with M >= kUmmaMinM and N,
    // K >= kUmmaMinNK go to the tcgen05 kernel (128 x 64 tiles, 16-deep K stages),
    // the others to the mma.sync kernel (64 x 64); the choice depends on the
    // problem's own shape only, so a chain's arithmetic does not depend on which
    // other chains share the launch.
    std::vector<GemmDesc<T>> big, small;
    for (auto& d : v)
      (use_umma && d.M >= kUmmaMinM && d.N >= kUmmaMinNK && (long long)d.K * d.G >= kUmmaMinNK ? big : small)
          .push_back(d);
    // the persistent tcgen05 kernel strides over the tiles: longest K first balances
    // its CTAs (the order of independent problems changes no arithmetic)
    std::stable_sort(big.begin(), big.end(), [](const GemmDesc<T>& a, const GemmDesc<T>& b) {
      return (long long)a.K * a.G > (long long)b.K * b.G;
    });
    tile(big, kUmmaBM, kUmmaBN);
    tile(small, 64, 64);
    if (!big.empty()) {
      // QCA_UMMA_LOG=<file>: one line per tcgen05 launch (its ordinal among this
      // process's tcgen05 launches, useful flops, algorithmic operand bytes,
      // problems), so that a profiler's per-launch DRAM bytes can be set against
      // the work of that launch
      static long long umma_launches = 0;
      static FILE* umma_log = [] {
        const char* p = getenv("QCA_UMMA_LOG");
        return p && *p ? fopen(p, "w") : (FILE*)nullptr;
      }();
      if (umma_log) {
        double f = 0.0, b = 0.0;
        for (auto& d : big) {
          const double nb = (double)d.nb1 * d.nb2 * d.G;
          f += 8.0 * d.M * d.N * (double)d.K * nb;
          b += sizeof(cplx<T>) *
               ((double)d.M * d.K * nb + (double)d.K * d.N * nb + (double)d.M * d.N * d.nb1 * d.nb2);
        }
        fprintf(umma_log, "%lld %.0f %.0f %zu\n", umma_launches, f, b, big.size());
        fflush(umma_log);
      }
      ++umma_launches;
    }
    const GemmDesc<T>* db = nullptr;
    const GemmDesc<T>* ds = nullptr;
    if (!big.empty()) QCA_TRY(upload(big, st, &db));
    if (!small.empty()) QCA_TRY(upload(small, st, &ds));
    const bool both = !big.empty() && !small.empty();
    if (both) QCA_TRY(ensure_aux());
    return timed(KC_GEMM, fl, by, st, [&] {
      int s = QCA_OK;
      // both kernels at once: the small problems on an auxiliary stream beside the
      // persistent launch, joined before anything reads their results
      cudaStream_t s2 = st;
      if (both) {
        QCA_CUDA(cudaEventRecord(fork_ev, st));
        QCA_CUDA(cudaStreamWaitEvent(aux[0], fork_ev, 0));
        s2 = aux[0];
      }
      if (!small.empty())
        s = launch_gemm_tc(reinterpret_cast<const GemmDesc<float>*>(ds),
                           reinterpret_cast<const GemmDesc<float>*>(small.data()), (int)small.size(), s2);
      if (s == QCA_OK && !big.empty())
        s = launch_gemm_umma(reinterpret_cast<const GemmDesc<float>*>(db),
                             reinterpret_cast<const GemmDesc<float>*>(big.data()), (int)big.size(), st);
      if (both) {
        QCA_CUDA(cudaEventRecord(join_ev[0], aux[0]));
        QCA_CUDA(cudaStreamWaitEvent(st, join_ev[0], 0));
      }
      return s;
    });
  }

  int run_wapply(std::vector<WapplyDesc<T>>& v, cudaStream_t st) {
    if (v.empty()) return QCA_OK;
    const std::vector<Span> sp = spans();
    for (auto& d : v) {
      if (!in_spans<T>(sp, d.out, (long long)d.nout * d.blk - 1)) return bad("wapply out");
    }
    int t = 0;
    for (auto& d : v) {
      d.chunks = ceil_div(d.blk, 1024);
      d.tile_begin = t;
      t += d.nout * d.chunks;
    }
    const WapplyDesc<T>* dd;
    QCA_TRY(upload(v, st, &dd));
    double by = 0.0;
    for (auto& d : v) by += 2.0 * sizeof(cplx<T>) * d.nout * (double)d.blk;
    return timed(KC_WAPPLY, 0.0, by, st, [&] { return launch_wapply<T>(dd, v.data(), (int)v.size(), st); });
  }

  int run_copy(std::vector<CopyDesc<T>>& v, cudaStream_t st) {
    if (v.empty()) return QCA_OK;
    const std::vector<Span> sp = spans();
    for (auto& d : v) {
      if (!in_spans<T>(sp, d.src, ext(d.m0, d.s0) + ext(d.m1, d.s1) + ext(d.m2, d.s2))) return bad("copy src");
      if (!in_spans<T>(sp, d.dst, ext(d.n0, d.d0) + ext(d.n1, d.d1) + ext(d.n2, d.d2))) return bad("copy dst");
    }
    int t = 0;
    for (auto& d : v) {
      d.tiles = ceil_div((long long)d.n0 * d.n1 * d.n2, 1024);
      d.tile_begin = t;
      t += d.tiles;
    }
    const CopyDesc<T>* dd;
    QCA_TRY(upload(v, st, &dd));
    return timed(KC_MISC, 0.0, 0.0, st, [&] { return launch_copy<T>(dd, v.data(), (int)v.size(), st); });
  }

  static GemmDesc<T> gemm0() {
    GemmDesc<T> g;
    memset(&g, 0, sizeof(g));
    g.G = 1;
    g.nb1 = 1;
    g.nb2 = 1;
    return g;
  }

  int check_qr(const std::vector<QrDesc<T>>& q) const {
    const std::vector<Span> sp = spans();
    for (auto& d : q) {
      const int K = std::min(d.m, d.n), qc = d.complete ? d.m : K;
      const long long ein = ext(d.rsplit, d.sIr0) + ext((d.m + d.rsplit - 1) / d.rsplit, d.sIr1) +
                            (d.csplit > 0 ? ext(d.csplit, d.sIc) + ext((d.n + d.csplit - 1) / d.csplit, d.sIc1)
                                          : ext(d.n, d.sIc));
      if (!in_spans<T>(sp, d.in, ein)) return bad("qr in");
      if (!in_spans<T>(sp, d.work, (long long)d.m * d.n + (long long)d.m * qc - 1)) return bad("qr work");
      if (!in_spans<T>(sp, d.tau, K - 1)) return bad("qr tau");
      const long long eq = ext(std::min(d.qsplit, d.qrows_out), d.sQr0) +
                           ext((d.qrows_out + d.qsplit - 1) / d.qsplit, d.sQr1) + ext(d.qcols_out, d.sQc);
      if (d.q && !in_spans<T>(sp, d.q, eq)) return bad("qr q");
      if (d.rr && !in_spans<T>(sp, d.rr, ext(d.rrows_out, d.sRr) + ext(d.rcols_out, d.sRc))) return bad("qr r");
    }
    return QCA_OK;
  }

  int check_svd(const std::vector<SvdDesc<T>>& v) const {
    const std::vector<Span> sp = spans();
    for (auto& d : v) {
      const long long p = d.right_sweep ? 2LL * d.Dr : 2LL * d.Dl, q = d.right_sweep ? 2LL * d.Dl : 2LL * d.Dr;
      const long long K = std::min(p, q);
      if (!in_spans<T>(sp, d.theta, 4LL * d.Dl * d.Dr - 1)) return bad("svd theta");
      if (!in_spans<T>(sp, d.rmat, K * q - 1)) return bad("svd R");
      if (!in_spans<T>(sp, d.Al, 2LL * d.Dl * d.kmax - 1)) return bad("svd Al");
      if (!in_spans<T>(sp, d.Ar, 2LL * d.kmax * d.Dr - 1)) return bad("svd Ar");
      if (K > 1024) return bad("svd size");
    }
    return QCA_OK;
  }

  // SVD problems grouped by the thread-block cluster size they need; the groups run
  // concurrently on auxiliary streams (fork/join with events), so small problems
  // are not launched with the cluster size of the largest one.  The order of the
  // problems does not change any arithmetic.
  cudaStream_t aux[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaEvent_t fork_ev = nullptr, join_ev[4] = {nullptr, nullptr, nullptr, nullptr};

  int ensure_aux() {
    if (aux[0]) return QCA_OK;
    for (int i = 0; i < 4; ++i) {
      QCA_CUDA(cudaStreamCreateWithFlags(&aux[i], cudaStreamNonBlocking));
      QCA_CUDA(cudaEventCreateWithFlags(&join_ev[i], cudaEventDisableTiming));
    }
    QCA_CUDA(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
    return QCA_OK;
  }

  int svd_grouped(std::vector<SvdDesc<T>>& sv, cudaStream_t st) {
    std::vector<SvdDesc<T>> grp[5];
    for (auto& d : sv) {
      const int cs = svd_cluster_size<T>(d.Dl, d.Dr, d.right_sweep);
      const int gi = cs <= 1 ? 0 : cs == 2 ? 1 : cs == 4 ? 2 : cs == 8 ? 3 : 4;
      grp[gi].push_back(d);
    }
    int used_groups = 0;
    for (auto& g : grp) used_groups += !g.empty();
    if (used_groups <= 1) {
      const SvdDesc<T>* ds;
      QCA_TRY(upload(sv, st, &ds));
      return launch_svd<T>(ds, sv.data(), (int)sv.size(), st);
    }
    QCA_TRY(ensure_aux());
    // descriptors first (stream-ordered copies on st), then fork
    std::vector<const SvdDesc<T>*> dptr(5, nullptr);
    for (int g = 0; g < 5; ++g)
      if (!grp[g].empty()) QCA_TRY(upload(grp[g], st, &dptr[g]));
    QCA_CUDA(cudaEventRecord(fork_ev, st));
    int k = 0;
    std::vector<int> joined;
    for (int g = 4; g >= 0; --g) {  // largest first
      if (grp[g].empty()) continue;
      cudaStream_t s2 = st;
      if (k < 4) {
        s2 = aux[k];
        QCA_CUDA(cudaStreamWaitEvent(s2, fork_ev, 0));
      }
      QCA_TRY(launch_svd<T>(dptr[g], grp[g].data(), (int)grp[g].size(), s2));
      if (s2 != st) {
        QCA_CUDA(cudaEventRecord(join_ev[k], s2));
        joined.push_back(k);
      }
      ++k;
    }
    for (int j : joined) QCA_CUDA(cudaStreamWaitEvent(st, join_ev[j], 0));
    return QCA_OK;
  }

  // ------------------------------------------------------------------ local problems
  struct LzProb {
    Chain<T>* c;
    int d;            // physical super-dimension: 4 (2-site), 2 (1-site), 1 (bond)
    int Dl, Dr, wL, wR;
    const cplx<T>* L;
    const cplx<T>* R;
    EL went;          // unused for d == 1
    const cplx<T>* in;
    cplx<T>* out;
    double tau;
  };

  // y = H_eff x for every problem (x in slot j, y in slot j+1)
  int matvec(std::vector<LzProb>& P, int j, cudaStream_t st) {
    std::vector<GemmDesc<T>> g1, g3;
    std::vector<WapplyDesc<T>> wa;
    for (auto& p : P) {
      Chain<T>* c = p.c;
      const long long n = (long long)p.d * p.Dl * p.Dr;
      const cplx<T>* x = c->basis + (long long)j * c->nmax;
      cplx<T>* y = c->basis + (long long)(j + 1) * c->nmax;
      const int* skip = reinterpret_cast<const int*>(c->lzS + LZ_DONE);
      (void)n;
      // T1[wr][s][a][e] = sum_c x[s][a][c] R[wr][c][e]
      GemmDesc<T> a = gemm0();
      a.A = x;
      a.B = p.R;
      a.C = c->t1;
      a.M = p.d * p.Dl;
      a.N = p.Dr;
      a.K = p.Dr;
      a.nb1 = p.wR;
      a.sAm = p.Dr;
      a.sAk = 1;
      a.sBk = p.Dr;
      a.sBn = 1;
      a.sBb1 = (long long)p.Dr * p.Dr;
      a.sCm = p.Dr;
      a.sCn = 1;
      a.sCb1 = (long long)p.d * p.Dl * p.Dr;
      a.skip = skip;
      g1.push_back(a);
      const cplx<T>* t2 = c->t1;
      if (p.d > 1) {
        WapplyDesc<T> w;
        memset(&w, 0, sizeof(w));
        w.ent = p.went.ent;
        w.out_begin = p.went.begin;
        w.nout = p.went.nout;
        w.blk = (long long)p.Dl * p.Dr;
        w.in = c->t1;
        w.out = c->t2;
        w.skip = skip;
        wa.push_back(w);
        t2 = c->t2;
      }
      // y[s'][b][e] = sum_{wl,a} L[wl][a][b] T2[s'][wl][a][e]
      GemmDesc<T> b = gemm0();
      b.A = p.L;
      b.B = t2;
      b.C = y;
      b.M = p.Dl;
      b.N = p.Dr;
      b.K = p.wL * p.Dl;
      b.nb1 = p.d;
      b.sAm = 1;
      b.sAk = p.Dl;
      b.sBk = p.Dr;
      b.sBn = 1;
      b.sBb1 = (long long)p.wL * p.Dl * p.Dr;
      b.sCm = p.Dr;
      b.sCn = 1;
      b.sCb1 = (long long)p.Dl * p.Dr;
      b.skip = skip;
      g3.push_back(b);
    }
    QCA_TRY(run_gemm(g1, st));
    QCA_TRY(run_wapply(wa, st));
    QCA_TRY(run_gemm(g3, st));
    return QCA_OK;
  }

  int lanczos(std::vector<LzProb>& P, cudaStream_t st) {
    if (P.empty()) return QCA_OK;
    const int nd = (int)P.size();
    if (nd > done_cap) {
      set_error("too many simultaneous problems (%d)", nd);
      return QCA_ERR_INVALID;
    }
    std::vector<LanczosDesc<T>> L(nd);
    int t = 0;
    for (int i = 0; i < nd; ++i) {
      LzProb& p = P[i];
      LanczosDesc<T>& d = L[i];
      memset(&d, 0, sizeof(d));
      d.V = p.c->basis;
      d.n = (long long)p.d * p.Dl * p.Dr;
      d.ld = p.c->nmax;
      d.S = p.c->lzS;
      d.tau = p.tau;
      d.chunks = ceil_div(d.n, kLzChunk);
      d.tile_begin = t;
      t += d.chunks;
      d.out = p.out;
      d.in = p.in;
      d.P = p.c->lzP;
      d.done_out = d_done + i;
      d.status = p.c->iflags + 3;
    }
    {
      const std::vector<Span> sp = spans();
      for (int i = 0; i < nd; ++i) {
        const LanczosDesc<T>& d = L[i];
        if (d.n > P[i].c->nmax || d.chunks > P[i].c->max_chunks) return bad("lanczos size");
        if (!in_spans<T>(sp, d.V, (long long)(mmax + 1) * d.ld - 1)) return bad("lanczos basis");
        if (!in_spans<T>(sp, d.in, d.n - 1) || !in_spans<T>(sp, d.out, d.n - 1)) return bad("lanczos in/out");
      }
    }
    const LanczosDesc<T>* dd;
    QCA_TRY(upload(L, st, &dd));
    QCA_TRY(timed(KC_LZVEC, 0, 0, st, [&] { return launch_lz_init<T>(dd, L.data(), nd, mmax, lz_tol, st); }));
    int j = 0;
    for (; j < mmax; ++j) {
      QCA_TRY(matvec(P, j, st));
      // the descriptor copy may have been recycled by a staging reset
      QCA_TRY(upload(L, st, &dd));
      QCA_TRY(timed(KC_LZVEC, 0, 0, st, [&] {
        int s = launch_lz_orth_pass<T>(dd, L.data(), nd, j, 0, st);
        if (s == QCA_OK) s = launch_lz_orth_pass<T>(dd, L.data(), nd, j, 1, st);
        if (s == QCA_OK) s = launch_lz_orth_pass<T>(dd, L.data(), nd, j, 2, st);
        return s;
      }));
      const bool check = (j >= 3 && (j % 3 == 0)) || j + 1 == mmax;
      QCA_TRY(timed(KC_LZFIN, 0, 0, st, [&] { return launch_lz_finalize_j<T>(dd, nd, j, mmax, check ? 1 : 0, st); }));
      QCA_TRY(timed(KC_LZVEC, 0, 0, st, [&] { return launch_lz_normalize<T>(dd, L.data(), nd, j, st); }));
      if (check) {
        QCA_CUDA(cudaMemcpyAsync(h_done, d_done, sizeof(int) * nd, cudaMemcpyDeviceToHost, st));
        QCA_TRY(sync(st));
        bool all = true;
        for (int i = 0; i < nd; ++i) all = all && h_done[i];
        if (all) break;
      }
    }
    QCA_TRY(upload(L, st, &dd));
    QCA_TRY(timed(KC_LZVEC, 0, 0, st, [&] { return launch_lz_combine<T>(dd, L.data(), nd, st); }));
    for (auto& p : P) p.c->lz_used = std::max(p.c->lz_used, std::min(j + 2, mmax));
    return QCA_OK;
  }

  // ------------------------------------------------------------------ environments
  struct EnvJob {
    Chain<T>* c;
    int site;
    bool left;  // true: Lenv[site+1] from Lenv[site]; false: Renv[site] from Renv[site+1]
  };

  int env_update(std::vector<EnvJob>& J, cudaStream_t st) {
    if (J.empty()) return QCA_OK;
    std::vector<GemmDesc<T>> g1, g3;
    std::vector<WapplyDesc<T>> wa;
    for (auto& jb : J) {
      Chain<T>* c = jb.c;
      const int i = jb.site;
      const int Di = c->D[i], Dj = c->D[i + 1];
      const cplx<T>* A = c->cur(i);
      GemmDesc<T> a = gemm0(), b = gemm0();
      WapplyDesc<T> w;
      memset(&w, 0, sizeof(w));
      if (jb.left) {
        const int wl = c->w[i], wr = c->w[i + 1];
        // X[wl][s'][a][e] = sum_b Lold[wl][a][b] conj(A[s'][b][e])
        a.A = c->Lenv[i];
        a.B = A;
        a.C = c->t1;
        a.M = Di;
        a.K = Di;
        a.N = Dj;
        a.nb1 = wl;
        a.nb2 = 2;
        a.sAm = Di;
        a.sAk = 1;
        a.sAb1 = (long long)Di * Di;
        a.sBk = Dj;
        a.sBn = 1;
        a.sBb2 = (long long)Di * Dj;
        a.conjB = 1;
        a.sCm = Dj;
        a.sCn = 1;
        a.sCb1 = 2LL * Di * Dj;
        a.sCb2 = (long long)Di * Dj;
        w.ent = c->envl[i].ent;
        w.out_begin = c->envl[i].begin;
        w.nout = c->envl[i].nout;
        w.blk = (long long)Di * Dj;
        // Lnew[wr][c][e] = sum_{s,a} A[s][a][c] Y[wr][s][a][e]
        b.A = A;
        b.B = c->t2;
        b.C = c->Lenv[i + 1];
        b.M = Dj;
        b.K = 2 * Di;
        b.N = Dj;
        b.nb1 = wr;
        b.sAm = 1;
        b.sAk = Dj;
        b.sBk = Dj;
        b.sBn = 1;
        b.sBb1 = 2LL * Di * Dj;
        b.sCm = Dj;
        b.sCn = 1;
        b.sCb1 = (long long)Dj * Dj;
      } else {
        const int wl = c->w[i], wr = c->w[i + 1];
        // X[wr][s'][c][b] = sum_e Rold[wr][c][e] conj(A[s'][b][e])
        a.A = c->Renv[i + 1];
        a.B = A;
        a.C = c->t1;
        a.M = Dj;
        a.K = Dj;
        a.N = Di;
        a.nb1 = wr;
        a.nb2 = 2;
        a.sAm = Dj;
        a.sAk = 1;
        a.sAb1 = (long long)Dj * Dj;
        a.sBk = 1;
        a.sBn = Dj;
        a.sBb2 = (long long)Di * Dj;
        a.conjB = 1;
        a.sCm = Di;
        a.sCn = 1;
        a.sCb1 = 2LL * Di * Dj;
        a.sCb2 = (long long)Di * Dj;
        w.ent = c->envr[i].ent;
        w.out_begin = c->envr[i].begin;
        w.nout = c->envr[i].nout;
        w.blk = (long long)Di * Dj;
        // Rnew[wl][a][b] = sum_{s,c} A[s][a][c] Y[wl][s][c][b]
        b.A = A;
        b.B = c->t2;
        b.C = c->Renv[i];
        b.M = Di;
        b.N = Di;
        b.K = Dj;
        b.G = 2;
        b.nb1 = wl;
        b.sAm = Dj;
        b.sAk = 1;
        b.sAg = (long long)Di * Dj;
        b.sBk = Di;
        b.sBn = 1;
        b.sBg = (long long)Di * Dj;
        b.sBb1 = 2LL * Di * Dj;
        b.sCm = Di;
        b.sCn = 1;
        b.sCb1 = (long long)Di * Di;
      }
      w.in = c->t1;
      w.out = c->t2;
      g1.push_back(a);
      wa.push_back(w);
      g3.push_back(b);
    }
    QCA_TRY(run_gemm(g1, st));
    QCA_TRY(run_wapply(wa, st));
    QCA_TRY(run_gemm(g3, st));
    return QCA_OK;
  }

  // ------------------------------------------------------------------ gauge moves
  // orthonormalize_left_qr (mps.py:146-164) / orthonormalize_right_qr (mps.py:166-181)
  struct MoveJob {
    Chain<T>* c;
    int site;
    bool left;
  };

  int qr_moves(std::vector<MoveJob>& J, cudaStream_t st) {
    if (J.empty()) return QCA_OK;
    std::vector<QrDesc<T>> q;
    std::vector<GemmDesc<T>> g;
    for (auto& jb : J) {
      Chain<T>* c = jb.c;
      const int i = jb.site;
      QrDesc<T> d;
      memset(&d, 0, sizeof(d));
      d.work = c->qrw;
      d.tau = c->qrtau;
      d.complete = 0;
      GemmDesc<T> a = gemm0();
      if (jb.left) {
        const int Di = c->D[i], Dj = c->D[i + 1], Dk = c->D[i + 2];
        d.in = c->cur(i);
        d.rsplit = Di;
        d.sIr0 = Dj;
        d.sIr1 = (long long)Di * Dj;
        d.sIc = 1;
        d.m = 2 * Di;
        d.n = Dj;
        d.q = c->alt(i);
        d.qsplit = Di;
        d.sQr0 = Dj;
        d.sQr1 = (long long)Di * Dj;
        d.sQc = 1;
        d.qrows_out = 2 * Di;
        d.qcols_out = Dj;
        d.rr = c->cbuf;
        d.sRr = Dj;
        d.sRc = 1;
        d.rrows_out = Dj;
        d.rcols_out = Dj;
        // A[i+1] <- R A[i+1]
        a.A = c->cbuf;
        a.B = c->cur(i + 1);
        a.C = c->alt(i + 1);
        a.M = Dj;
        a.K = Dj;
        a.N = Dk;
        a.nb1 = 2;
        a.sAm = Dj;
        a.sAk = 1;
        a.sBk = Dk;
        a.sBn = 1;
        a.sBb1 = (long long)Dj * Dk;
        a.sCm = Dk;
        a.sCn = 1;
        a.sCb1 = (long long)Dj * Dk;
      } else {
        const int Dh = c->D[i - 1], Di = c->D[i], Dj = c->D[i + 1];
        // M[(s,c), a] = A[s][a][c]
        d.in = c->cur(i);
        d.rsplit = Dj;
        d.sIr0 = 1;
        d.sIr1 = (long long)Di * Dj;
        d.sIc = Dj;
        d.m = 2 * Dj;
        d.n = Di;
        d.q = c->alt(i);
        d.qsplit = Dj;
        d.sQr0 = 1;
        d.sQr1 = (long long)Di * Dj;
        d.sQc = Dj;
        d.qrows_out = 2 * Dj;
        d.qcols_out = Di;
        d.rr = c->cbuf;  // R^T padded to (Di x Di)
        d.sRr = 1;
        d.sRc = Di;
        d.rrows_out = Di;
        d.rcols_out = Di;
        // A[i-1] <- A[i-1] R^T
        a.A = c->cur(i - 1);
        a.B = c->cbuf;
        a.C = c->alt(i - 1);
        a.M = Dh;
        a.K = Di;
        a.N = Di;
        a.nb1 = 2;
        a.sAm = Di;
        a.sAk = 1;
        a.sAb1 = (long long)Dh * Di;
        a.sBk = Di;
        a.sBn = 1;
        a.sCm = Di;
        a.sCn = 1;
        a.sCb1 = (long long)Dh * Di;
      }
      q.push_back(d);
      g.push_back(a);
    }
    QCA_TRY(check_qr(q));
    const QrDesc<T>* dq;
    QCA_TRY(upload(q, st, &dq));
    QCA_TRY(timed(KC_QR, 0, 0, st, [&] { return launch_qr<T>(dq, (int)q.size(), 1, st); }));
    QCA_TRY(run_gemm(g, st));
    for (auto& jb : J) {
      Chain<T>* c = jb.c;
      if (jb.left) {
        c->par[jb.site] ^= 1;
        c->par[jb.site + 1] ^= 1;
        c->center = jb.site + 1;
      } else {
        c->par[jb.site] ^= 1;
        c->par[jb.site - 1] ^= 1;
        c->center = jb.site - 1;
      }
    }
    return QCA_OK;
  }

  // Right QR sweep to site 0 and rebuild of every right environment, in lock step
  // over the chains (make_site_canonical(0), mps.py:184-192, plus tdvp.py:37-39).
  int canonicalize_right(std::vector<Chain<T>*>& C, bool rebuild_env, cudaStream_t st) {
    int maxN = 0;
    for (auto* c : C) maxN = std::max(maxN, c->N);
    // QR moves from the centre down to site 1
    for (int k = maxN - 1; k >= 1; --k) {
      std::vector<MoveJob> J;
      for (auto* c : C)
        if (k < c->N && k <= c->center) J.push_back(MoveJob{c, k, false});
      QCA_TRY(qr_moves(J, st));
    }
    // right environments N-1 .. 1
    for (int k = maxN - 1; rebuild_env && k >= 1; --k) {
      std::vector<EnvJob> J;
      for (auto* c : C)
        if (k < c->N) J.push_back(EnvJob{c, k, false});
      QCA_TRY(env_update(J, st));
    }
    for (auto* c : C) c->center = 0;
    return QCA_OK;
  }

  // TDVP.__init__ (tdvp.py:12-40) with the redundant re-QRs of already
  // orthonormal tensors left out (LAPACK's QR returns R = I for them):
  //   left sweep to N-1, right sweep to 0, left sweep to N-2,
  //   R env at N-1, then for site N-2..1: right QR at site, R env at site.
  // Run for every chain added since the last operation, in lock step: sweep
  // position t of every chain shares one grouped launch (right sweeps aligned at
  // each chain's last site).  Each chain sees the same operations in the same
  // order as when initialised alone.
  int init_many(std::vector<Chain<T>*>& C, cudaStream_t st) {
    int maxN = 0;
    for (auto* c : C) maxN = std::max(maxN, c->N);
    for (int s = 0; s + 1 < maxN; ++s) {
      std::vector<MoveJob> J;
      for (auto* c : C)
        if (s < c->N - 1) J.push_back(MoveJob{c, s, true});
      QCA_TRY(qr_moves(J, st));
    }
    for (int t = 0; t + 1 < maxN; ++t) {  // site N-1-t
      std::vector<MoveJob> J;
      for (auto* c : C)
        if (c->N - 1 - t >= 1) J.push_back(MoveJob{c, c->N - 1 - t, false});
      QCA_TRY(qr_moves(J, st));
    }
    for (int s = 0; s + 2 < maxN; ++s) {
      std::vector<MoveJob> J;
      for (auto* c : C)
        if (s < c->N - 2) J.push_back(MoveJob{c, s, true});
      QCA_TRY(qr_moves(J, st));
    }
    {
      std::vector<EnvJob> J;
      for (auto* c : C) J.push_back(EnvJob{c, c->N - 1, false});
      QCA_TRY(env_update(J, st));
    }
    for (int t = 0; t + 2 < maxN; ++t) {  // site N-2-t
      std::vector<MoveJob> J;
      std::vector<EnvJob> E;
      for (auto* c : C) {
        const int s = c->N - 2 - t;
        if (s < 1) continue;
        J.push_back(MoveJob{c, s, false});
        E.push_back(EnvJob{c, s, false});
      }
      QCA_TRY(qr_moves(J, st));
      QCA_TRY(env_update(E, st));
    }
    for (auto* c : C) {
      c->center = 0;
      c->pending_init = false;
    }
    return QCA_OK;
  }

  // initialise every chain still waiting for it (all of them, so that chains
  // added one at a time share the grouped launches)
  int ensure_init(cudaStream_t st) {
    std::vector<Chain<T>*> C;
    for (auto& kv : chains)
      if (kv.second->pending_init) C.push_back(kv.second.get());
    if (C.empty()) return QCA_OK;
    return init_many(C, st);
  }

  // ------------------------------------------------------------------ one tick
  int tick(std::vector<Chain<T>*>& C, cudaStream_t st) {
    const double hp = M_PI / 2;
    // stage 1: forward local evolution
    std::vector<GemmDesc<T>> form;
    std::vector<LzProb> P;
    for (auto* c : C) {
      if (c->algo == QCA_ALGO_2TDVP) {
        const int l = c->dir == 0 ? c->pos : c->pos - 1, r = l + 1;
        const int Dl = c->D[l], Dm = c->D[l + 1], Dr = c->D[r + 1];
        GemmDesc<T> g = gemm0();
        g.A = c->cur(l);
        g.B = c->cur(r);
        g.C = c->theta;
        g.M = Dl;
        g.K = Dm;
        g.N = Dr;
        g.nb1 = 2;
        g.nb2 = 2;
        g.sAm = Dm;
        g.sAk = 1;
        g.sAb1 = (long long)Dl * Dm;
        g.sBk = Dr;
        g.sBn = 1;
        g.sBb2 = (long long)Dm * Dr;
        g.sCm = Dr;
        g.sCn = 1;
        g.sCb1 = 2LL * Dl * Dr;
        g.sCb2 = (long long)Dl * Dr;
        form.push_back(g);
        P.push_back(LzProb{c, 4, Dl, Dr, c->w[l], c->w[r + 1], c->Lenv[l], c->Renv[r + 1], c->mv2[l], c->theta,
                           c->theta, hp * c->dt / 2});
      } else {
        const int s = c->pos;
        const bool end = c->dir == 0 ? s == c->N - 1 : s == 0;
        P.push_back(LzProb{c, 2, c->D[s], c->D[s + 1], c->w[s], c->w[s + 1], c->Lenv[s], c->Renv[s + 1], c->mv1[s],
                           c->cur(s), end ? c->cur(s) : c->theta, hp * c->dt / 2});
      }
    }
    QCA_TRY(run_gemm(form, st));
    QCA_TRY(lanczos(P, st));
    // stage 2: split (SVD) / complete QR
    std::vector<SvdDesc<T>> sv;
    std::vector<QrDesc<T>> qr, spre;
    std::vector<Chain<T>*> svc;
    for (auto* c : C) {
      if (c->algo == QCA_ALGO_2TDVP) {
        const int l = c->dir == 0 ? c->pos : c->pos - 1, r = l + 1;
        SvdDesc<T> d;
        memset(&d, 0, sizeof(d));
        d.theta = c->theta;
        d.Dl = c->D[l];
        d.Dr = c->D[r + 1];
        d.chi = c->chi;
        d.kmax = c->cap[l + 1];
        d.eps = c->eps;
        d.right_sweep = c->dir == 0;
        d.Al = c->alt(l);
        d.Ar = c->alt(r);
        // R of the preconditioning QR (K q <= 4 cmax^2) in svdw; the QR's own work in qrw
        d.rmat = c->svdw;
        spre.push_back(split_qr_desc<T>(c->theta, d.Dl, d.Dr, d.right_sweep, c->qrw, c->qrtau, c->svdw));
        d.sv = c->sv;
        d.k_out = c->iflags;
        d.discarded = c->dscal;
        d.status = c->iflags + 1;
        sv.push_back(d);
        svc.push_back(c);
      } else {
        const int s = c->pos;
        if (c->dir == 0 && s < c->N - 1) {
          const int Ds = c->D[s], Dt = c->D[s + 1], tg = c->target[s + 1];
          QrDesc<T> d;
          memset(&d, 0, sizeof(d));
          d.in = c->theta;
          d.rsplit = Ds;
          d.sIr0 = Dt;
          d.sIr1 = (long long)Ds * Dt;
          d.sIc = 1;
          d.m = 2 * Ds;
          d.n = Dt;
          d.complete = 1;
          d.work = c->qrw;
          d.tau = c->qrtau;
          d.q = c->alt(s);
          d.qsplit = Ds;
          d.sQr0 = tg;
          d.sQr1 = (long long)Ds * tg;
          d.sQc = 1;
          d.qrows_out = 2 * Ds;
          d.qcols_out = tg;
          d.rr = c->cbuf;
          d.sRr = Dt;
          d.sRc = 1;
          d.rrows_out = tg;
          d.rcols_out = Dt;
          qr.push_back(d);
        } else if (c->dir == 1 && s > 0) {
          const int Ds = c->D[s], Dt = c->D[s + 1], tg = c->target[s];
          QrDesc<T> d;
          memset(&d, 0, sizeof(d));
          d.in = c->theta;
          d.rsplit = Dt;
          d.sIr0 = 1;
          d.sIr1 = (long long)Ds * Dt;
          d.sIc = Dt;
          d.m = 2 * Dt;
          d.n = Ds;
          d.complete = 1;
          d.work = c->qrw;
          d.tau = c->qrtau;
          d.q = c->alt(s);
          d.qsplit = Dt;
          d.sQr0 = 1;
          d.sQr1 = (long long)tg * Dt;
          d.sQc = Dt;
          d.qrows_out = 2 * Dt;
          d.qcols_out = tg;
          d.rr = c->cbuf;  // C[a][j] = R[j][a], (Ds x tg)
          d.sRr = 1;
          d.sRc = tg;
          d.rrows_out = tg;
          d.rcols_out = Ds;
          qr.push_back(d);
        }
      }
    }
    if (!sv.empty()) {
      QCA_TRY(check_svd(sv));
      QCA_TRY(check_qr(spre));
      {  // the preconditioning QRs of the splits (FP32 sums on the mixed path)
        const QrDesc<T>* dq;
        QCA_TRY(upload(spre, st, &dq));
        QCA_TRY(timed(KC_SVD, 0, 0, st, [&] { return launch_qr<T>(dq, (int)spre.size(), 1, st); }));
      }
      double fl = 0.0;
      for (auto& d : sv) {  // Golub-Van Loan thin-SVD count, x4 for complex
        const double m = 2.0 * std::max(d.Dl, d.Dr), n = 2.0 * std::min(d.Dl, d.Dr);
        fl += 4.0 * (4.0 * m * m * n + 8.0 * m * n * n + 9.0 * n * n * n);
      }
      QCA_TRY(timed(KC_SVD, fl, 0, st, [&] { return svd_grouped(sv, st); }));
    }
    if (!qr.empty()) {
      QCA_TRY(check_qr(qr));
      const QrDesc<T>* dq;
      QCA_TRY(upload(qr, st, &dq));
      QCA_TRY(timed(KC_QR, 0, 0, st, [&] { return launch_qr<T>(dq, (int)qr.size(), 0, st); }));
    }
    if (!svc.empty()) {
      if (svc.size() > (size_t)done_cap) {
        set_error("too many simultaneous two-site splits (%zu)", svc.size());
        return QCA_ERR_INVALID;
      }
      for (size_t i = 0; i < svc.size(); ++i)
        QCA_CUDA(cudaMemcpyAsync(h_k + 4 * i, svc[i]->iflags, 4 * sizeof(int), cudaMemcpyDeviceToHost, st));
      QCA_TRY(sync(st));
      for (size_t i = 0; i < svc.size(); ++i) {
        Chain<T>* c = svc[i];
        const int l = c->dir == 0 ? c->pos : c->pos - 1;
        const int k = h_k[4 * i];
        if (k < 1 || k > c->cap[l + 1]) {
          set_error("SVD returned bond dimension %d (capacity %d)", k, c->cap[l + 1]);
          return QCA_ERR_INVALID;
        }
        note_failure(c, h_k[4 * i + 1], h_k[4 * i + 3], l);
        c->svd_sweeps = std::max(c->svd_sweeps, h_k[4 * i + 2]);
        c->D[l + 1] = k;
      }
      for (size_t i = 0; i < svc.size(); ++i) {
        Chain<T>* c = svc[i];
        const int l = c->dir == 0 ? c->pos : c->pos - 1;
        c->par[l] ^= 1;
        c->par[l + 1] ^= 1;
      }
    }
    // 1TDVP bookkeeping after the QR
    std::vector<int> dold(C.size(), 0);
    for (size_t ci = 0; ci < C.size(); ++ci) {
      Chain<T>* c = C[ci];
      if (c->algo == QCA_ALGO_2TDVP) continue;
      const int s = c->pos;
      if (c->dir == 0 && s < c->N - 1) {
        dold[ci] = c->D[s + 1];
        c->D[s + 1] = c->target[s + 1];
        c->par[s] ^= 1;
      } else if (c->dir == 1 && s > 0) {
        dold[ci] = c->D[s];
        c->D[s] = c->target[s];
        c->par[s] ^= 1;
      }
    }
    // stage 3: environment updates
    std::vector<EnvJob> E;
    for (auto* c : C) {
      if (c->algo == QCA_ALGO_2TDVP) {
        if (c->dir == 0 && c->pos < c->N - 2) E.push_back(EnvJob{c, c->pos, true});
        if (c->dir == 1 && c->pos > 1) E.push_back(EnvJob{c, c->pos, false});
      } else {
        if (c->dir == 0 && c->pos < c->N - 1) E.push_back(EnvJob{c, c->pos, true});
        if (c->dir == 1 && c->pos > 0) E.push_back(EnvJob{c, c->pos, false});
      }
    }
    QCA_TRY(env_update(E, st));
    // stage 4: backward evolution
    std::vector<LzProb> B;
    for (size_t ci = 0; ci < C.size(); ++ci) {
      Chain<T>* c = C[ci];
      if (c->algo == QCA_ALGO_2TDVP) {
        if (c->dir == 0 && c->pos < c->N - 2) {
          const int s = c->pos + 1;
          B.push_back(LzProb{c, 2, c->D[s], c->D[s + 1], c->w[s], c->w[s + 1], c->Lenv[s], c->Renv[s + 1],
                             c->mv1[s], c->cur(s), c->cur(s), -hp * c->dt / 2});
        } else if (c->dir == 1 && c->pos > 1) {
          const int s = c->pos - 1;
          B.push_back(LzProb{c, 2, c->D[s], c->D[s + 1], c->w[s], c->w[s + 1], c->Lenv[s], c->Renv[s + 1],
                             c->mv1[s], c->cur(s), c->cur(s), -hp * c->dt / 2});
        }
      } else {
        const int s = c->pos;
        if (c->dir == 0 && s < c->N - 1) {
          // C (target x Dold) with L = Lenv[s+1], R = Renv[s+1]
          B.push_back(LzProb{c, 1, c->D[s + 1], dold[ci], c->w[s + 1], c->w[s + 1], c->Lenv[s + 1], c->Renv[s + 1],
                             EL{}, c->cbuf, c->cbuf, -hp * c->dt / 2});
        } else if (c->dir == 1 && s > 0) {
          // C (Dold x target) with L = Lenv[s], R = Renv[s]
          B.push_back(LzProb{c, 1, dold[ci], c->D[s], c->w[s], c->w[s], c->Lenv[s], c->Renv[s], EL{}, c->cbuf,
                             c->cbuf, -hp * c->dt / 2});
        }
      }
    }
    QCA_TRY(lanczos(B, st));
    // stage 5 (1TDVP): absorb the bond matrix into the next site
    std::vector<GemmDesc<T>> ab;
    std::vector<std::pair<Chain<T>*, int>> flips;
    for (size_t ci = 0; ci < C.size(); ++ci) {
      Chain<T>* c = C[ci];
      if (c->algo == QCA_ALGO_2TDVP) continue;
      const int s = c->pos;
      if (c->dir == 0 && s < c->N - 1) {
        const int tg = c->D[s + 1], Do = dold[ci], Dk = c->D[s + 2];
        GemmDesc<T> g = gemm0();
        g.A = c->cbuf;
        g.B = c->cur(s + 1);
        g.C = c->alt(s + 1);
        g.M = tg;
        g.K = Do;
        g.N = Dk;
        g.nb1 = 2;
        g.sAm = Do;
        g.sAk = 1;
        g.sBk = Dk;
        g.sBn = 1;
        g.sBb1 = (long long)Do * Dk;
        g.sCm = Dk;
        g.sCn = 1;
        g.sCb1 = (long long)tg * Dk;
        ab.push_back(g);
        flips.push_back({c, s + 1});
      } else if (c->dir == 1 && s > 0) {
        const int Dh = c->D[s - 1], Do = dold[ci], tg = c->D[s];
        GemmDesc<T> g = gemm0();
        g.A = c->cur(s - 1);
        g.B = c->cbuf;
        g.C = c->alt(s - 1);
        g.M = Dh;
        g.K = Do;
        g.N = tg;
        g.nb1 = 2;
        g.sAm = Do;
        g.sAk = 1;
        g.sAb1 = (long long)Dh * Do;
        g.sBk = tg;
        g.sBn = 1;
        g.sCm = tg;
        g.sCn = 1;
        g.sCb1 = (long long)Dh * tg;
        ab.push_back(g);
        flips.push_back({c, s - 1});
      }
    }
    QCA_TRY(run_gemm(ab, st));
    for (auto& f : flips) f.first->par[f.second] ^= 1;
    // advance
    for (auto* c : C) {
      if (c->algo == QCA_ALGO_2TDVP) {
        if (c->dir == 0) {
          if (c->pos < c->N - 2) {
            c->pos++;
          } else {
            c->dir = 1;
            c->pos = c->N - 1;
          }
        } else {
          if (c->pos > 1) {
            c->pos--;
          } else {
            c->dir = 0;
            c->pos = 0;
            c->todo--;
            c->center = 0;
            c->in_step = false;
            c->steps_done++;
          }
        }
      } else {
        if (c->dir == 0) {
          if (c->pos < c->N - 1) {
            c->pos++;
          } else {
            c->dir = 1;
            c->pos = c->N - 1;
          }
        } else {
          if (c->pos > 0) {
            c->pos--;
          } else {
            c->dir = 0;
            c->pos = 0;
            c->todo--;
            c->center = 0;
            c->in_step = false;
            c->steps_done++;
          }
        }
      }
    }
    return QCA_OK;
  }

  // ------------------------------------------------------------------ failures
  // Record the first numerical failure of a chain from its device status words:
  // the SVD status (0, QCA_ERR_NAN, QCA_ERR_NOT_CONVERGED) and the sticky Lanczos
  // bits (kLzStatus*).  A failed chain takes no further part in the step.
  static void note_failure(Chain<T>* c, int svd_status, int lz_bits, int site) {
    int code = QCA_OK;
    const char* what = "";
    if ((lz_bits & kLzStatusNonFinite) || svd_status == QCA_ERR_NAN) {
      code = QCA_ERR_NAN;
      what = "non-finite values in a local update";
    } else if (svd_status == QCA_ERR_NOT_CONVERGED) {
      code = QCA_ERR_NOT_CONVERGED;
      what = "Jacobi sweeps of the two-site split ran out";
    } else if (lz_bits & kLzStatusLimit) {
      code = QCA_ERR_NOT_CONVERGED;
      what = "a Lanczos exponential reached its iteration limit";
    }
    if (code != QCA_OK && c->status == QCA_OK) {
      c->status = code;
      c->fail_site = site;
      c->fail_what = what;
    }
  }

  // The status of a set of chains: QCA_ERR_NAN before QCA_ERR_NOT_CONVERGED, with
  // the first failed chain named in the error message.
  static int report_failures(const std::vector<Chain<T>*>& C) {
    Chain<T>* worst = nullptr;
    int nfail = 0;
    for (auto* c : C) {
      if (c->status == QCA_OK) continue;
      ++nfail;
      if (!worst || (c->status == QCA_ERR_NAN && worst->status != QCA_ERR_NAN)) worst = c;
    }
    if (!worst) return QCA_OK;
    set_error("chain %d: %s (at position %d); %d chain(s) failed, the others completed the step", worst->id,
              worst->fail_what, worst->fail_site, nfail);
    return worst->status;
  }

  // ------------------------------------------------------------------ public ops
  int add(const qca_chain_desc* d, cudaStream_t st, int* id_out) override;
  int remove(int id) override {
    auto it = chains.find(id);
    if (it == chains.end()) {
      set_error("unknown chain %d", id);
      return QCA_ERR_INVALID;
    }
    cudaFree(it->second->mem);
    used -= it->second->bytes;
    chains.erase(it);
    return QCA_OK;
  }

  std::vector<Chain<T>*> select(const int* ids, int count, int* status) {
    std::vector<Chain<T>*> C;
    *status = QCA_OK;
    if (ids) {
      for (int i = 0; i < count; ++i) {
        auto it = chains.find(ids[i]);
        if (it == chains.end()) {
          set_error("unknown chain %d", ids[i]);
          *status = QCA_ERR_INVALID;
          return {};
        }
        C.push_back(it->second.get());
      }
    } else {
      for (auto& kv : chains) C.push_back(kv.second.get());
    }
    return C;
  }

  // Begin the next time step of every listed chain that has one scheduled: the
  // gauge-consistent start of tdvp.py:50-54 (chains whose gauge a measurement
  // moved are re-canonicalised and get their right environments rebuilt, grouped)
  // and the per-step statistics reset.
  int begin_steps(const std::vector<Chain<T>*>& C, cudaStream_t st) {
    std::vector<Chain<T>*> starting, dirty;
    for (auto* c : C)
      if (c->todo > 0 && !c->in_step && c->status == QCA_OK) starting.push_back(c);
    if (starting.empty()) return QCA_OK;
    for (auto* c : starting) {
      c->dir = 0;
      c->pos = 0;
      c->lz_used = 0;
      c->svd_sweeps = 0;
      c->disc_host = 0.0;
      c->in_step = true;
      if (c->center != 0) dirty.push_back(c);
      QCA_CUDA(cudaMemsetAsync(c->dscal, 0, sizeof(double), st));
      QCA_CUDA(cudaMemsetAsync(c->iflags + 3, 0, sizeof(int), st));
    }
    // the gauge-consistent start of 2TDVP and 1TDVP rebuilds the right environments
    // after the re-canonicalisation; a1tdvp keeps those of the previous sweep, as
    // the reference does (tdvp.py:54 and 212-267 read them as they are)
    std::vector<Chain<T>*> dirty_env, dirty_keep;
    for (auto* c : dirty) (c->algo == QCA_ALGO_A1TDVP ? dirty_keep : dirty_env).push_back(c);
    if (!dirty_env.empty()) QCA_TRY(canonicalize_right(dirty_env, true, st));
    if (!dirty_keep.empty()) QCA_TRY(canonicalize_right(dirty_keep, false, st));
    std::vector<Chain<T>*> a1;
    for (auto* c : starting)
      if (c->algo == QCA_ALGO_A1TDVP) a1.push_back(c);
    if (!a1.empty()) QCA_TRY(a1_targets(a1, st));
    return QCA_OK;
  }

  // a1tdvp (tdvp.py:212-267): the target bond dimensions of the coming 1TDVP step,
  // for every listed chain in lock step.  A left-canonical sweep with left
  // environments (make_site_canonical(site + 1) and the left layer, tdvp.py:
  // 214-216), then bond by bond from the right end: the two-site tensor evolved by
  // dt/2 with the current environments (the right ones as the previous step left
  // them, as in the reference), its split's truncation rule (first i with
  // ||s[i:]|| < eps, else the maximal bond; clamped to [1, maximal]) as the bond's
  // target, the evolved tensor discarded, and a right gauge move
  // (make_site_canonical(bond - 1)).  The SVDs write their truncated dimension to
  // a per-chain device array read once at the end.
  int a1_targets(std::vector<Chain<T>*>& C, cudaStream_t st) {
    const double hp = M_PI / 2;
    int maxN = 0;
    for (auto* c : C) {
      maxN = std::max(maxN, c->N);
      QCA_CUDA(cudaMemsetAsync(c->a1flags, 0, sizeof(int) * 3 * (c->N + 1), st));
    }
    for (int site = 0; site + 1 < maxN; ++site) {
      std::vector<MoveJob> J;
      std::vector<EnvJob> E;
      for (auto* c : C)
        if (site < c->N - 1) {
          J.push_back(MoveJob{c, site, true});
          E.push_back(EnvJob{c, site, true});
        }
      QCA_TRY(qr_moves(J, st));
      QCA_TRY(env_update(E, st));
    }
    for (int t = 0; t + 1 < maxN; ++t) {  // bond N-1-t of every chain
      std::vector<GemmDesc<T>> form;
      std::vector<LzProb> P;
      std::vector<SvdDesc<T>> sv;
      std::vector<QrDesc<T>> spre;
      std::vector<MoveJob> J;
      for (auto* c : C) {
        const int bond = c->N - 1 - t;
        if (bond < 1) continue;
        const int l = bond - 1, r = bond;
        const int Dl = c->D[l], Dm = c->D[l + 1], Dr = c->D[r + 1];
        GemmDesc<T> g = gemm0();
        g.A = c->cur(l);
        g.B = c->cur(r);
        g.C = c->theta;
        g.M = Dl;
        g.K = Dm;
        g.N = Dr;
        g.nb1 = 2;
        g.nb2 = 2;
        g.sAm = Dm;
        g.sAk = 1;
        g.sAb1 = (long long)Dl * Dm;
        g.sBk = Dr;
        g.sBn = 1;
        g.sBb2 = (long long)Dm * Dr;
        g.sCm = Dr;
        g.sCn = 1;
        g.sCb1 = 2LL * Dl * Dr;
        g.sCb2 = (long long)Dl * Dr;
        form.push_back(g);
        P.push_back(LzProb{c, 4, Dl, Dr, c->w[l], c->w[r + 1], c->Lenv[l], c->Renv[r + 1], c->mv2[l], c->theta,
                           c->theta, hp * c->dt / 2});
        SvdDesc<T> d;
        memset(&d, 0, sizeof(d));
        d.theta = c->theta;
        d.Dl = Dl;
        d.Dr = Dr;
        d.chi = c->maxb[bond];
        d.kmax = c->cap[bond];
        d.eps = c->eps;
        d.right_sweep = 1;
        d.Al = c->t1;  // the split itself is discarded
        d.Ar = c->t2;
        d.rmat = c->svdw;
        d.sv = c->sv;
        d.k_out = c->a1flags + bond;
        d.discarded = c->dscal + 1;
        d.status = c->a1flags + c->N + 1 + 2 * bond;
        sv.push_back(d);
        spre.push_back(split_qr_desc<T>(c->theta, Dl, Dr, 1, c->qrw, c->qrtau, c->svdw));
        J.push_back(MoveJob{c, bond, false});
      }
      QCA_TRY(run_gemm(form, st));
      QCA_TRY(lanczos(P, st));
      QCA_TRY(check_svd(sv));
      QCA_TRY(check_qr(spre));
      const QrDesc<T>* dq;
      QCA_TRY(upload(spre, st, &dq));
      QCA_TRY(timed(KC_SVD, 0, 0, st, [&] { return launch_qr<T>(dq, (int)spre.size(), 1, st); }));
      QCA_TRY(timed(KC_SVD, 0, 0, st, [&] { return svd_grouped(sv, st); }));
      QCA_TRY(qr_moves(J, st));
    }
    for (auto* c : C) {
      std::vector<int> h(3 * (c->N + 1));
      QCA_CUDA(cudaMemcpyAsync(h.data(), c->a1flags, sizeof(int) * h.size(), cudaMemcpyDeviceToHost, st));
      QCA_TRY(sync(st));
      for (int b = 1; b < c->N; ++b) {
        const int k = h[b];
        if (k < 1 || k > c->cap[b]) {
          set_error("a1tdvp: split returned bond dimension %d (capacity %d)", k, c->cap[b]);
          return QCA_ERR_INVALID;
        }
        c->target[b] = k;
        note_failure(c, h[c->N + 1 + 2 * b], 0, b);
      }
      c->center = 0;
    }
    return QCA_OK;
  }

  // Up to max_ticks lock-step ticks (one local update of every chain in a step),
  // starting scheduled steps as chains become free, so that a chain that finishes
  // a time step begins its next one at the following tick (continuous batching).
  // Then the failure bits of the local updates since the last per-tick check are
  // read (1TDVP chains, the backward evolutions after a chain's last split).
  int run_ticks(const std::vector<Chain<T>*>& C, long long max_ticks, cudaStream_t st) {
    QCA_TRY(ensure_init(st));
    for (long long t = 0; t < max_ticks; ++t) {
      QCA_TRY(begin_steps(C, st));
      std::vector<Chain<T>*> act;
      for (auto* c : C)
        if (c->in_step && c->status == QCA_OK) act.push_back(c);
      if (act.empty()) break;
      QCA_TRY(tick(act, st));
    }
    for (size_t b = 0; b < C.size(); b += (size_t)done_cap) {
      const size_t e = std::min(C.size(), b + (size_t)done_cap);
      for (size_t i = b; i < e; ++i)
        QCA_CUDA(cudaMemcpyAsync(h_k + 4 * (i - b), C[i]->iflags, 4 * sizeof(int), cudaMemcpyDeviceToHost, st));
      QCA_TRY(sync(st));
      for (size_t i = b; i < e; ++i) note_failure(C[i], QCA_OK, h_k[4 * (i - b) + 3], -1);
    }
    QCA_TRY(sync(st));
    if (std::is_same<T, float>::value && use_tc && use_umma) {
      int timeouts = 0;
      QCA_TRY(gemm_umma_timeouts(1, &timeouts, st));
      if (timeouts) {
        set_error("tensor-core GEMM: %d mbarrier waits ran out", timeouts);
        return QCA_ERR_CUDA;
      }
    }
    return QCA_OK;
  }

  int step(const int* ids, int count, int nsteps, cudaStream_t st) override {
    int s = QCA_OK;
    std::vector<Chain<T>*> C = select(ids, count, &s);
    if (s != QCA_OK) return s;
    if (C.empty() || nsteps <= 0) return QCA_OK;
    for (auto* c : C) {
      if (c->status != QCA_OK) {
        set_error("chain %d failed in an earlier step (%s at position %d); remove it", c->id, c->fail_what,
                  c->fail_site);
        return c->status;
      }
      if (c->in_step || c->todo > 0) {
        set_error("chain %d has time steps scheduled by qca_engine_advance; finish them first", c->id);
        return QCA_ERR_INVALID;
      }
    }
    for (auto* c : C) c->todo = nsteps;
    QCA_TRY(run_ticks(C, std::numeric_limits<long long>::max(), st));
    return report_failures(C);
  }

  int schedule(int id, int nsteps) override {
    auto it = chains.find(id);
    if (it == chains.end()) {
      set_error("unknown chain %d", id);
      return QCA_ERR_INVALID;
    }
    if (nsteps < 0) {
      set_error("qca_chain_schedule: negative step count");
      return QCA_ERR_INVALID;
    }
    it->second->todo += nsteps;
    return QCA_OK;
  }

  int advance(const int* ids, int count, int max_ticks, cudaStream_t st) override {
    int s = QCA_OK;
    std::vector<Chain<T>*> C = select(ids, count, &s);
    if (s != QCA_OK) return s;
    std::vector<Chain<T>*> live;
    for (auto* c : C)
      if (c->status == QCA_OK) live.push_back(c);
    if (live.empty() || max_ticks <= 0) return QCA_OK;
    QCA_TRY(run_ticks(live, max_ticks, st));
    return report_failures(live);
  }

  int progress(int id, long long* out) override {
    auto it = chains.find(id);
    if (it == chains.end()) {
      set_error("unknown chain %d", id);
      return QCA_ERR_INVALID;
    }
    const Chain<T>* c = it->second.get();
    out[0] = c->steps_done;
    out[1] = c->todo;
    out[2] = c->in_step ? 1 : 0;
    out[3] = c->status;
    return QCA_OK;
  }

  int check_boundary(const Chain<T>* c, const char* what) const {
    if (c->in_step) {
      set_error("%s: chain %d is inside a time step (qca_engine_advance stopped mid-sweep)", what, c->id);
      return QCA_ERR_INVALID;
    }
    return QCA_OK;
  }

  // Algorithm.measure for several chains in lock step (mps.py:100-140): bond dims,
  // make_site_canonical(0), then a left QR sweep with the 2x2 density matrix of
  // every site; mutates the gauge like the reference.  Outputs are concatenated
  // over the chains in the given order (N_c values per chain, N_c + 1 for bonds).
  int measure_many(const int* ids, int count, double* pop, double* dpop, double* sse, double* bonds_out,
                   cudaStream_t st) override {
    std::vector<Chain<T>*> C;
    for (int i = 0; i < count; ++i) {
      auto it = chains.find(ids[i]);
      if (it == chains.end()) {
        set_error("unknown chain %d", ids[i]);
        return QCA_ERR_INVALID;
      }
      C.push_back(it->second.get());
      QCA_TRY(check_boundary(C.back(), "qca_engine_measure"));
    }
    QCA_TRY(ensure_init(st));
    size_t ob = 0;
    for (auto* c : C) {
      if (bonds_out)
        for (int i = 0; i <= c->N; ++i) bonds_out[ob + i] = c->D[i];
      ob += c->N + 1;
    }
    int maxN = 0;
    for (auto* c : C) maxN = std::max(maxN, c->N);
    // 2TDVP chains whose centre is at site 0 are measured without touching their
    // tensors: their result does not depend on the gauge, and the left sweep runs
    // on scratch copies (centre_{s+1} = R_s A[s+1]).  1TDVP chains follow the
    // reference, whose measurement re-gauges the stored MPS (mps.py:110-117).
    std::vector<char> keep(C.size(), 0);
    for (size_t i = 0; i < C.size(); ++i) keep[i] = C[i]->algo == QCA_ALGO_2TDVP && C[i]->center == 0;
    std::vector<const cplx<T>*> cen(C.size(), nullptr);
    for (size_t i = 0; i < C.size(); ++i) cen[i] = C[i]->cur(0);
    const std::vector<Span> sp = spans();
    for (int k = maxN - 1; k >= 1; --k) {
      std::vector<MoveJob> J;
      for (size_t i = 0; i < C.size(); ++i)
        if (!keep[i] && k < C[i]->N && k <= C[i]->center) J.push_back(MoveJob{C[i], k, false});
      QCA_TRY(qr_moves(J, st));
    }
    for (int s = 0; s < maxN; ++s) {
      if (s > 0) {
        std::vector<MoveJob> J;
        for (size_t i = 0; i < C.size(); ++i)
          if (!keep[i] && s < C[i]->N) J.push_back(MoveJob{C[i], s - 1, true});
        QCA_TRY(qr_moves(J, st));
        // scratch sweep: R of the previous centre times the next site tensor
        std::vector<QrDesc<T>> q;
        std::vector<GemmDesc<T>> g;
        std::vector<size_t> who;
        for (size_t i = 0; i < C.size(); ++i) {
          Chain<T>* c = C[i];
          if (!keep[i] || s >= c->N) continue;
          const int Dp = c->D[s - 1], Dq = c->D[s], Dn = c->D[s + 1];
          QrDesc<T> d;
          memset(&d, 0, sizeof(d));
          d.in = cen[i];
          d.rsplit = Dp;
          d.sIr0 = Dq;
          d.sIr1 = (long long)Dp * Dq;
          d.sIc = 1;
          d.m = 2 * Dp;
          d.n = Dq;
          d.work = c->qrw;
          d.tau = c->qrtau;
          d.rr = c->cbuf;
          d.sRr = Dq;
          d.sRc = 1;
          d.rrows_out = Dq;
          d.rcols_out = Dq;
          q.push_back(d);
          GemmDesc<T> a = gemm0();
          a.A = c->cbuf;
          a.B = c->cur(s);
          a.C = (s & 1) ? c->theta : c->t1;
          a.M = Dq;
          a.K = Dq;
          a.N = Dn;
          a.nb1 = 2;
          a.sAm = Dq;
          a.sAk = 1;
          a.sBk = Dn;
          a.sBn = 1;
          a.sBb1 = (long long)Dq * Dn;
          a.sCm = Dn;
          a.sCn = 1;
          a.sCb1 = (long long)Dq * Dn;
          g.push_back(a);
          who.push_back(i);
        }
        if (!q.empty()) {
          QCA_TRY(check_qr(q));
          const QrDesc<T>* dq;
          QCA_TRY(upload(q, st, &dq));
          QCA_TRY(timed(KC_QR, 0, 0, st, [&] { return launch_qr<T>(dq, (int)q.size(), 1, st); }));
          QCA_TRY(run_gemm(g, st));
          for (size_t k = 0; k < who.size(); ++k) cen[who[k]] = g[k].C;
        }
      }
      std::vector<RhoDesc<T>> rd;
      for (size_t i = 0; i < C.size(); ++i) {
        Chain<T>* c = C[i];
        if (s >= c->N) continue;
        const cplx<T>* a = keep[i] ? cen[i] : c->cur(s);
        if (!in_spans<T>(sp, a, 2LL * c->D[s] * c->D[s + 1] - 1)) return bad("rho");
        rd.push_back(RhoDesc<T>{a, c->D[s], c->D[s + 1], c->dscal + 8 + 4 * s});
      }
      if (!rd.empty()) {
        const RhoDesc<T>* dr;
        QCA_TRY(upload(rd, st, &dr));
        QCA_TRY(timed(KC_MISC, 0, 0, st, [&] { return launch_rho<T>(dr, (int)rd.size(), st); }));
      }
    }
    std::vector<std::vector<double>> rho(C.size());
    for (size_t i = 0; i < C.size(); ++i) {
      rho[i].resize(4 * C[i]->N);
      QCA_CUDA(cudaMemcpyAsync(rho[i].data(), C[i]->dscal + 8, sizeof(double) * 4 * C[i]->N, cudaMemcpyDeviceToHost, st));
    }
    QCA_TRY(sync(st));
    size_t o = 0;
    for (size_t i = 0; i < C.size(); ++i) {
      Chain<T>* c = C[i];
      if (!keep[i]) c->center = c->N - 1;
      for (int s = 0; s < c->N; ++s) {
        const double* r = rho[i].data() + 4 * s;
        const double r00 = r[0], r11 = r[1], rr = r[2], ri = r[3];
        if (pop) pop[o + s] = r11;
        if (dpop) dpop[o + s] = std::nearbyint(r11);
        if (sse) {
          // eigenvalues of [[r00, r01], [conj r01, r11]]; -sum l log2 l with 0 log 0 = 0
          const double tr = r00 + r11, det = r00 * r11 - (rr * rr + ri * ri);
          const double disc = std::sqrt(std::max(0.0, tr * tr / 4 - det));
          const double l1 = tr / 2 + disc, l2 = tr / 2 - disc;
          double h = 0.0;
          if (l1 > 0) h -= l1 * std::log2(l1);
          if (l2 > 0) h -= l2 * std::log2(l2);
          sse[o + s] = h;
        }
      }
      o += c->N;
    }
    return QCA_OK;
  }

  int measure(int id, double* pop, double* dpop, double* sse, double* bonds_out, cudaStream_t st) override {
    return measure_many(&id, 1, pop, dpop, sse, bonds_out, st);
  }

  int bonds(int id, int* out) override {
    auto it = chains.find(id);
    if (it == chains.end()) {
      set_error("unknown chain %d", id);
      return QCA_ERR_INVALID;
    }
    for (int i = 0; i <= it->second->N; ++i) out[i] = it->second->D[i];
    return QCA_OK;
  }

  int get_mps(int id, double* out, size_t capd, cudaStream_t st) override {
    auto it = chains.find(id);
    if (it == chains.end()) {
      set_error("unknown chain %d", id);
      return QCA_ERR_INVALID;
    }
    Chain<T>* c = it->second.get();
    QCA_TRY(check_boundary(c, "qca_chain_get_mps"));
    QCA_TRY(ensure_init(st));
    size_t need = 0;
    for (int i = 0; i < c->N; ++i) need += 4ull * c->D[i] * c->D[i + 1];
    if (capd < need) {
      set_error("qca_chain_get_mps: capacity %zu doubles < %zu", capd, need);
      return QCA_ERR_INVALID;
    }
    size_t off = 0;
    std::vector<cplx<T>> tmp;
    for (int i = 0; i < c->N; ++i) {
      const size_t cnt = 2ull * c->D[i] * c->D[i + 1];
      tmp.resize(cnt);
      QCA_CUDA(cudaMemcpyAsync(tmp.data(), c->cur(i), sizeof(cplx<T>) * cnt, cudaMemcpyDeviceToHost, st));
      QCA_CUDA(cudaStreamSynchronize(st));
      for (size_t e = 0; e < cnt; ++e) {
        out[off + 2 * e] = (double)tmp[e].re;
        out[off + 2 * e + 1] = (double)tmp[e].im;
      }
      off += 2 * cnt;
    }
    return QCA_OK;
  }

  int stats(int id, double* out) override {
    auto it = chains.find(id);
    if (it == chains.end()) {
      set_error("unknown chain %d", id);
      return QCA_ERR_INVALID;
    }
    Chain<T>* c = it->second.get();
    double disc = 0.0;
    QCA_CUDA(cudaMemcpy(&disc, c->dscal, sizeof(double), cudaMemcpyDeviceToHost));
    out[0] = c->lz_used;
    out[1] = disc;
    return QCA_OK;
  }

  int stats_ex(int id, double* out, int count) override {
    double base[2];
    QCA_TRY(stats(id, base));
    const Chain<T>* c = chains.find(id)->second.get();
    const double all[5] = {base[0], base[1], (double)c->svd_sweeps, (double)c->status, (double)c->bytes};
    for (int i = 0; i < count && i < 5; ++i) out[i] = all[i];
    return QCA_OK;
  }

  std::vector<int> ids() const override {
    std::vector<int> v;
    for (auto& kv : chains) v.push_back(kv.first);
    return v;
  }
};

// capacities: cap_i = max(min(2^i, 2^(N-i), chi), D_i of the initial state)
static std::vector<int> capacities(const qca_chain_desc* d) {
  const int N = d->n_sites;
  std::vector<int> cap(N + 1);
  for (int i = 0; i <= N; ++i) {
    long long c = d->max_bond_dim;
    if (i < 40) c = std::min<long long>(c, 1LL << i);
    if (N - i < 40) c = std::min<long long>(c, 1LL << (N - i));
    cap[i] = (int)std::max<long long>(c, d->mps_bonds[i]);
  }
  return cap;
}

struct Layout {
  size_t total = 0;
  size_t take(size_t bytes) {
    const size_t off = total;
    total += align_up(bytes);
    return off;
  }
};

template <typename T>
static void plan_chain(const qca_chain_desc* d, int mmax, Layout& Lo, std::vector<size_t>* offs, long long* nmax_out,
                       long long* tmax_out, int* cmax_out, int* chunks_out) {
  const int N = d->n_sites;
  const std::vector<int> cap = capacities(d);
  const int* w = d->mpo_bonds;
  const size_t es = sizeof(cplx<T>);
  int cmax = 1, wmax = 1;
  for (int i = 0; i <= N; ++i) {
    cmax = std::max(cmax, cap[i]);
    wmax = std::max(wmax, w[i]);
  }
  long long nmax = 1, tmax = 1;
  for (int i = 0; i < N; ++i) {
    nmax = std::max(nmax, 2LL * cap[i] * cap[i + 1]);
    nmax = std::max(nmax, (long long)cap[i] * cap[i]);
    tmax = std::max(tmax, 2LL * cap[i] * w[i + 1] * cap[i + 1]);
    tmax = std::max(tmax, 2LL * cap[i] * w[i] * cap[i + 1]);
    tmax = std::max(tmax, (long long)cap[i] * w[i] * cap[i]);
    if (i + 2 <= N) {
      nmax = std::max(nmax, 4LL * cap[i] * cap[i + 2]);
      tmax = std::max(tmax, 4LL * cap[i] * w[i + 2] * cap[i + 2]);
      tmax = std::max(tmax, 4LL * cap[i] * w[i] * cap[i + 2]);
    }
  }
  const int chunks = ceil_div(nmax, kLzChunk);
  auto put = [&](size_t b) {
    if (offs) offs->push_back(Lo.take(b));
    else Lo.take(b);
  };
  for (int i = 0; i < N; ++i) {  // A double buffers
    put(es * 2 * cap[i] * cap[i + 1]);
    put(es * 2 * cap[i] * cap[i + 1]);
  }
  put(es);  // Lenv[0]
  for (int i = 0; i < N; ++i) put(es * (size_t)w[i + 1] * cap[i + 1] * cap[i + 1]);  // Lenv[i+1]
  for (int i = 0; i < N; ++i) put(es * (size_t)w[i] * cap[i] * cap[i]);  // Renv[i]
  put(es);  // Renv[N]
  put(es * nmax);                           // theta
  put(es * nmax * (mmax + 1));              // basis
  put(es * tmax);                           // t1
  put(es * tmax);                           // t2
  put(es * 4ull * cmax * cmax);             // svd work: R (K q), q, K <= 2 cmax
  put(es * (8ull * cmax * cmax + 2 * cmax));  // qr work (m*n + m*m), m <= 2 cmax, n <= 2 cmax
  put(es * 2 * cmax);                       // qr tau
  put(es * (size_t)cmax * cmax * 2);        // cbuf
  put(sizeof(double) * lz_scal_size(chunks));
  put(sizeof(double) * lz_part_size(chunks));
  put(sizeof(double) * 4 * cmax);           // singular values
  put(sizeof(double) * (8 + 4 * N));        // discarded weight + rho
  put(sizeof(int) * 8);                     // flags
  put(sizeof(int) * 3 * (N + 1));           // a1tdvp targets and SVD statuses
  if (nmax_out) *nmax_out = nmax;
  if (tmax_out) *tmax_out = tmax;
  if (cmax_out) *cmax_out = cmax;
  if (chunks_out) *chunks_out = chunks;
}

template <typename T>
int Engine<T>::add(const qca_chain_desc* d, cudaStream_t st, int* id_out) {
  const int N = d->n_sites;
  if (N < 2 || !d->mpo_bonds || !d->mpo || !d->mps_bonds || !d->mps || d->max_bond_dim < 1 ||
      (d->algorithm != QCA_ALGO_1TDVP && d->algorithm != QCA_ALGO_2TDVP && d->algorithm != QCA_ALGO_A1TDVP) ||
      !(d->svd_epsilon >= 0) ||
      !std::isfinite(d->step_size)) {
    set_error("qca_chain_add: invalid chain description");
    return QCA_ERR_INVALID;
  }
  if (d->mps_bonds[0] != 1 || d->mps_bonds[N] != 1 || d->mpo_bonds[0] != 1 || d->mpo_bonds[N] != 1) {
    set_error("qca_chain_add: boundary bond dimensions must be 1");
    return QCA_ERR_INVALID;
  }
  for (int i = 0; i <= N; ++i) {
    if (d->mps_bonds[i] < 1 || d->mpo_bonds[i] < 1 || d->mps_bonds[i] > 4096) {
      set_error("qca_chain_add: invalid bond dimension at %d", i);
      return QCA_ERR_INVALID;
    }
  }
  std::vector<int> cap = capacities(d);
  int cmax = 1;
  for (int x : cap) cmax = std::max(cmax, x);
  if (cmax > 512) {
    set_error("qca_chain_add: bond capacity %d exceeds 512", cmax);
    return QCA_ERR_INVALID;
  }
  Layout Lo;
  std::vector<size_t> offs;
  long long nmax, tmax;
  int chunks;
  plan_chain<T>(d, mmax, Lo, &offs, &nmax, &tmax, &cmax, &chunks);
  // W entry lists
  std::vector<HostW> W(N);
  size_t woff = 0;
  for (int i = 0; i < N; ++i) {
    W[i].wl = d->mpo_bonds[i];
    W[i].wr = d->mpo_bonds[i + 1];
    const size_t cnt = 4ull * W[i].wl * W[i].wr;
    W[i].v.resize(cnt);
    for (size_t e = 0; e < cnt; ++e) W[i].v[e] = mk<double>(d->mpo[2 * (woff + e)], d->mpo[2 * (woff + e) + 1]);
    woff += cnt;
  }
  std::vector<EntryListHost> lists;
  for (int i = 0; i < N; ++i) lists.push_back(list_mv1(W[i]));
  for (int i = 0; i + 1 < N; ++i) lists.push_back(list_mv2(W[i], W[i + 1]));
  for (int i = 0; i < N; ++i) lists.push_back(list_envl(W[i]));
  for (int i = 0; i < N; ++i) lists.push_back(list_envr(W[i]));
  std::vector<size_t> loffs;
  for (auto& l : lists) {
    loffs.push_back(Lo.take(sizeof(WEntry) * std::max<size_t>(1, l.ent.size())));
    loffs.push_back(Lo.take(sizeof(int) * (l.nout + 1)));
  }
  if (used + Lo.total > budget) {
    set_error("qca_chain_add: chain needs %zu bytes, %zu of %zu in use", Lo.total, used, budget);
    return QCA_ERR_ADMISSION;
  }
  auto c = std::make_unique<Chain<T>>();
  if (cudaMalloc(&c->mem, Lo.total) != cudaSuccess) {
    cudaGetLastError();
    set_error("qca_chain_add: device allocation of %zu bytes failed", Lo.total);
    return QCA_ERR_OOM;
  }
  c->bytes = Lo.total;
  char* base = (char*)c->mem;
  // A fresh chain starts from zeros, not from whatever a removed chain left in the
  // recycled memory: zero padding then multiplies as zero (a stale NaN would not),
  // and a chain's arithmetic cannot depend on the chains that came before it.
  QCA_CUDA(cudaMemsetAsync(base, 0, Lo.total, st));
  c->N = N;
  c->algo = d->algorithm;
  c->chi = d->max_bond_dim;
  c->eps = d->svd_epsilon;
  c->dt = d->step_size;
  c->w.assign(d->mpo_bonds, d->mpo_bonds + N + 1);
  c->D.assign(d->mps_bonds, d->mps_bonds + N + 1);
  c->cap = cap;
  c->target.resize(N + 1);
  for (int i = 0; i <= N; ++i) {
    long long t = d->max_bond_dim;
    if (i < 40) t = std::min<long long>(t, 1LL << i);
    if (N - i < 40) t = std::min<long long>(t, 1LL << (N - i));
    c->target[i] = (int)t;
    c->maxb.push_back((int)t);
  }
  c->nmax = nmax;
  c->max_chunks = chunks;
  c->cmax = cmax;
  size_t k = 0;
  c->A[0].resize(N);
  c->A[1].resize(N);
  c->par.assign(N, 0);
  for (int i = 0; i < N; ++i) {
    c->A[0][i] = (cplx<T>*)(base + offs[k++]);
    c->A[1][i] = (cplx<T>*)(base + offs[k++]);
  }
  c->Lenv.resize(N + 1);
  c->Renv.resize(N + 1);
  for (int i = 0; i <= N; ++i) c->Lenv[i] = (cplx<T>*)(base + offs[k++]);
  for (int i = 0; i <= N; ++i) c->Renv[i] = (cplx<T>*)(base + offs[k++]);
  c->theta = (cplx<T>*)(base + offs[k++]);
  c->basis = (cplx<T>*)(base + offs[k++]);
  c->t1 = (cplx<T>*)(base + offs[k++]);
  c->t2 = (cplx<T>*)(base + offs[k++]);
  c->svdw = (cplx<T>*)(base + offs[k++]);
  c->qrw = (cplx<T>*)(base + offs[k++]);
  c->qrtau = (cplx<T>*)(base + offs[k++]);
  c->cbuf = (cplx<T>*)(base + offs[k++]);
  c->lzS = (double*)(base + offs[k++]);
  c->lzP = (double*)(base + offs[k++]);
  c->sv = (double*)(base + offs[k++]);
  c->dscal = (double*)(base + offs[k++]);
  c->iflags = (int*)(base + offs[k++]);
  c->a1flags = (int*)(base + offs[k++]);
  // entry lists: laid out back to back at the end of the allocation, uploaded as
  // one host image
  std::vector<EL> els;
  const size_t lbase = loffs.empty() ? Lo.total : loffs[0];
  std::vector<char> limg(Lo.total - lbase, 0);
  for (size_t li = 0; li < lists.size(); ++li) {
    EL e;
    e.ent = (const WEntry*)(base + loffs[2 * li]);
    e.begin = (const int*)(base + loffs[2 * li + 1]);
    e.nout = lists[li].nout;
    if (!lists[li].ent.empty())
      memcpy(limg.data() + (loffs[2 * li] - lbase), lists[li].ent.data(), sizeof(WEntry) * lists[li].ent.size());
    memcpy(limg.data() + (loffs[2 * li + 1] - lbase), lists[li].begin.data(), sizeof(int) * (lists[li].nout + 1));
    els.push_back(e);
  }
  if (!limg.empty())
    QCA_CUDA(cudaMemcpyAsync(base + lbase, limg.data(), limg.size(), cudaMemcpyHostToDevice, st));
  size_t li = 0;
  for (int i = 0; i < N; ++i) c->mv1.push_back(els[li++]);
  for (int i = 0; i + 1 < N; ++i) c->mv2.push_back(els[li++]);
  for (int i = 0; i < N; ++i) c->envl.push_back(els[li++]);
  for (int i = 0; i < N; ++i) c->envr.push_back(els[li++]);
  // upload the MPS and the boundary environments
  size_t total = 0;
  for (int i = 0; i < N; ++i) total += 2ull * c->D[i] * c->D[i + 1];
  std::vector<cplx<T>> tmp(total);
  for (size_t e = 0; e < total; ++e) tmp[e] = mk<T>((T)d->mps[2 * e], (T)d->mps[2 * e + 1]);
  size_t aoff = 0;
  for (int i = 0; i < N; ++i) {
    const size_t cnt = 2ull * c->D[i] * c->D[i + 1];
    QCA_CUDA(cudaMemcpyAsync(c->A[0][i], tmp.data() + aoff, sizeof(cplx<T>) * cnt, cudaMemcpyHostToDevice, st));
    aoff += cnt;
  }
  const cplx<T> one = mk<T>(1, 0);
  QCA_CUDA(cudaMemcpyAsync(c->Lenv[0], &one, sizeof(one), cudaMemcpyHostToDevice, st));
  QCA_CUDA(cudaMemcpyAsync(c->Renv[N], &one, sizeof(one), cudaMemcpyHostToDevice, st));
  QCA_CUDA(cudaMemsetAsync(c->dscal, 0, sizeof(double) * 8, st));
  QCA_CUDA(cudaMemsetAsync(c->iflags, 0, sizeof(int) * 8, st));
  QCA_CUDA(cudaStreamSynchronize(st));
  Chain<T>* raw = c.get();
  raw->id = next_id++;
  chains[raw->id] = std::move(c);
  used += raw->bytes;
  // TDVP.__init__ runs at the next operation, grouped with every chain added
  // before it
  raw->pending_init = true;
  *id_out = raw->id;
  return QCA_OK;
}

size_t chain_bytes(const qca_chain_desc* d, int precision) {
  Layout Lo;
  if (precision == QCA_PREC_FP64)
    plan_chain<double>(d, 40, Lo, nullptr, nullptr, nullptr, nullptr, nullptr);
  else
    plan_chain<float>(d, 40, Lo, nullptr, nullptr, nullptr, nullptr, nullptr);
  return Lo.total + (size_t)d->n_sites * 64 * 1024;
}

}  // namespace qca

struct qca_engine {
  std::unique_ptr<qca::EngineBase> impl;
  int precision = 0;
};

using namespace qca;

extern "C" {

int qca_engine_create(int precision, size_t hbm_budget_bytes, qca_engine** out) {
  if (!out || (precision != QCA_PREC_FP64 && precision != QCA_PREC_MIXED)) {
    set_error("qca_engine_create: invalid arguments");
    return QCA_ERR_INVALID;
  }
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    set_error("qca_engine_create: no CUDA device");
    return QCA_ERR_NO_DEVICE;
  }
  auto e = new qca_engine();
  e->precision = precision;
  int s;
  if (precision == QCA_PREC_FP64) {
    auto* p = new Engine<double>();
    e->impl.reset(p);
    s = p->init(hbm_budget_bytes);
  } else {
    auto* p = new Engine<float>();
    e->impl.reset(p);
    s = p->init(hbm_budget_bytes);
  }
  if (s != QCA_OK) {
    delete e;
    return s;
  }
  *out = e;
  return QCA_OK;
}

int qca_engine_destroy(qca_engine* e) {
  delete e;
  return QCA_OK;
}

int qca_chain_footprint(const qca_chain_desc* d, int precision, size_t* bytes) {
  if (!d || !bytes || d->n_sites < 2 || !d->mpo_bonds || !d->mps_bonds || d->max_bond_dim < 1) {
    set_error("qca_chain_footprint: invalid arguments");
    return QCA_ERR_INVALID;
  }
  *bytes = chain_bytes(d, precision);
  return QCA_OK;
}

int qca_chain_add(qca_engine* e, const qca_chain_desc* d, void* stream, int* chain_id) {
  if (!e || !d || !chain_id) {
    set_error("qca_chain_add: NULL argument");
    return QCA_ERR_INVALID;
  }
  return e->impl->add(d, (cudaStream_t)stream, chain_id);
}

int qca_chain_remove(qca_engine* e, int chain_id) {
  if (!e) {
    set_error("qca_chain_remove: NULL engine");
    return QCA_ERR_INVALID;
  }
  return e->impl->remove(chain_id);
}

int qca_engine_step(qca_engine* e, int nsteps, void* stream) {
  if (!e || nsteps < 0) {
    set_error("qca_engine_step: invalid arguments");
    return QCA_ERR_INVALID;
  }
  return e->impl->step(nullptr, 0, nsteps, (cudaStream_t)stream);
}

int qca_engine_step_chains(qca_engine* e, const int* chain_ids, int count, int nsteps, void* stream) {
  if (!e || !chain_ids || count < 0 || nsteps < 0) {
    set_error("qca_engine_step_chains: invalid arguments");
    return QCA_ERR_INVALID;
  }
  return e->impl->step(chain_ids, count, nsteps, (cudaStream_t)stream);
}

int qca_chain_schedule(qca_engine* e, int chain_id, int nsteps) {
  if (!e) {
    set_error("qca_chain_schedule: NULL engine");
    return QCA_ERR_INVALID;
  }
  return e->impl->schedule(chain_id, nsteps);
}

int qca_engine_advance(qca_engine* e, const int* chain_ids, int count, int max_ticks, void* stream) {
  if (!e || count < 0 || (count > 0 && !chain_ids)) {
    set_error("qca_engine_advance: invalid arguments");
    return QCA_ERR_INVALID;
  }
  return e->impl->advance(count > 0 ? chain_ids : nullptr, count, max_ticks, (cudaStream_t)stream);
}

int qca_chain_progress(qca_engine* e, int chain_id, long long* progress) {
  if (!e || !progress) {
    set_error("qca_chain_progress: NULL argument");
    return QCA_ERR_INVALID;
  }
  return e->impl->progress(chain_id, progress);
}

int qca_chain_measure(qca_engine* e, int chain_id, double* population, double* d_population,
                      double* single_site_entropy, double* bond_dims, void* stream) {
  if (!e) {
    set_error("qca_chain_measure: NULL engine");
    return QCA_ERR_INVALID;
  }
  return e->impl->measure(chain_id, population, d_population, single_site_entropy, bond_dims, (cudaStream_t)stream);
}

int qca_engine_measure(qca_engine* e, const int* chain_ids, int count, double* population, double* d_population,
                       double* single_site_entropy, double* bond_dims, void* stream) {
  if (!e || !chain_ids || count < 0) {
    set_error("qca_engine_measure: invalid arguments");
    return QCA_ERR_INVALID;
  }
  return e->impl->measure_many(chain_ids, count, population, d_population, single_site_entropy, bond_dims,
                               (cudaStream_t)stream);
}

int qca_chain_bonds(qca_engine* e, int chain_id, int* bonds) {
  if (!e || !bonds) {
    set_error("qca_chain_bonds: NULL argument");
    return QCA_ERR_INVALID;
  }
  return e->impl->bonds(chain_id, bonds);
}

int qca_chain_get_mps(qca_engine* e, int chain_id, double* mps, size_t capacity, void* stream) {
  if (!e || !mps) {
    set_error("qca_chain_get_mps: NULL argument");
    return QCA_ERR_INVALID;
  }
  return e->impl->get_mps(chain_id, mps, capacity, (cudaStream_t)stream);
}

int qca_engine_profile(qca_engine* e, int enable) {
  if (!e) {
    set_error("qca_engine_profile: NULL engine");
    return QCA_ERR_INVALID;
  }
  return e->impl->set_profile(enable);
}

int qca_engine_kernel_stats(qca_engine* e, double* out, int reset) {
  if (!e || !out) {
    set_error("qca_engine_kernel_stats: NULL argument");
    return QCA_ERR_INVALID;
  }
  return e->impl->kernel_stats(out, reset);
}

int qca_chain_stats(qca_engine* e, int chain_id, double* stats) {
  if (!e || !stats) {
    set_error("qca_chain_stats: NULL argument");
    return QCA_ERR_INVALID;
  }
  return e->impl->stats(chain_id, stats);
}

int qca_chain_stats_ex(qca_engine* e, int chain_id, double* stats, int count) {
  if (!e || !stats || count < 0) {
    set_error("qca_chain_stats_ex: invalid arguments");
    return QCA_ERR_INVALID;
  }
  return e->impl->stats_ex(chain_id, stats, count);
}

}  // extern "C"
