// fe_krylov.cuh -- batched Jacobi-preconditioned BiCGStab (van der Vorst
// 1992) on the diagonal blocks of a stacked CSR matrix: the device Newton
// linear solve that replaces the host SuperLU solve of the reference's
// Newton step (pyoomph/solvers/scipy.py, src/pybind/solver.cpp:105).
//
// Included at the end of fe_gb300.cu (one translation unit): it uses that
// file's error helpers and CSR kernels.
//
// Layout: every vector is [S blocks][n rows] in FP64; the matrix values stay
// in the caller's buffer (FP64 or FP32).  Every vector kernel runs on a
// (chunk, block) grid with KR_CHUNK entries per CTA and writes one partial
// sum per (quantity, block, chunk); every consumer reduces a block's
// partials in one fixed order (thread-strided, then a fixed shuffle tree),
// so a block's scalars -- and its iterates -- depend on its own rows only,
// never on which slot it occupies or what the other blocks hold.  Consumers
// that need a scalar (alpha, omega) reduce the partials themselves instead
// of waiting for a separate scalar kernel; one small kernel per iteration
// advances the per-block state word:
//
//   RUNNING -> CONVERGED (||r||_inf <= target) -> IDLE (true residual ok)
//           -> BROKE (non-finite update: iterate restored from the last check)
//           -> RESTART (rho or omega exactly 0: restart from the iterate)
//
// Blocks that are not RUNNING are skipped by every kernel (the SpMV included).
namespace {

constexpr int KR_T = 256;       // threads per CTA
constexpr int KR_CHUNK = 2048;  // vector entries per CTA
enum { KR_RUNNING = 0, KR_CONVERGED = 1, KR_BROKE = 2, KR_IDLE = 3, KR_RESTART = 4 };
enum { KP_RV = 0, KP_TS, KP_TT, KP_RR, KP_MAX, KP_BAD, KP_N };  // partial quantities
enum { KE_ZERO_DIAG = 1, KE_NONFINITE_B = 2, KE_NONFINITE_RESTART = 4 };

struct KrView {
  long long n;  // rows per block
  int S, nchunk;
  double *b, *x, *xg, *r, *rhat, *p, *v, *s, *t, *phat, *shat, *minv;
  double *rho, *rho_old, *alpha, *omega, *target;
  int *status, *err;
  double *part;  // [KP_N][S][nchunk]
  __device__ double *pp(int q, int blk) const { return part + ((long long)q * S + blk) * nchunk; }
};

// GB300 issues FP64 at ~1/64 of the FP32 rate and the solver is bound by
// it (the SpMV spends one FMA per stored entry): everything that need not be
// FP64 arithmetic runs on the integer pipe -- finiteness tests and counts on
// the exponent bits, and maxima of non-negative doubles as maxima of their
// bit patterns (the orders agree).
__device__ __forceinline__ bool kr_finite(double v) {
  return ((unsigned long long)__double_as_longlong(v) >> 52 & 0x7ffULL) != 0x7ffULL;
}
__device__ __forceinline__ unsigned long long kr_absbits(double v) {
  return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffULL;
}

__device__ __forceinline__ double kr_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ unsigned long long kr_warp_max(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long u = __shfl_xor_sync(0xffffffffu, v, o);
    v = u > v ? u : v;
  }
  return v;
}
__device__ __forceinline__ int kr_warp_count(int v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// CTA-wide reductions; every thread gets the same bits (the xor butterfly
// adds the same pairs on every lane).  `sh` holds KR_T / 32 doubles.
__device__ double kr_cta_sum(double v, double *sh) {
  v = kr_warp_sum(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  return kr_warp_sum(l < KR_T / 32 ? sh[l] : 0.0);
}
// max of non-negative doubles given as bit patterns; returns the double
__device__ double kr_cta_max(unsigned long long v, double *sh) {
  v = kr_warp_max(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  unsigned long long *shu = (unsigned long long *)sh;
  __syncthreads();
  if (l == 0) shu[w] = v;
  __syncthreads();
  return __longlong_as_double((long long)kr_warp_max(l < KR_T / 32 ? shu[l] : 0ULL));
}
__device__ double kr_cta_count(int v, double *sh) {
  v = kr_warp_count(v);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  int *shi = (int *)sh;
  __syncthreads();
  if (l == 0) shi[w] = v;
  __syncthreads();
  return (double)kr_warp_count(l < KR_T / 32 ? shi[l] : 0);
}

// reduce one block's partials of quantity q (all CTAs get the same bits)
template <bool MAX>
__device__ double kr_parts(const KrView &k, int q, int blk, double *sh) {
  const double *pp = k.pp(q, blk);
  if (MAX) {
    unsigned long long a = 0;
    for (int c = threadIdx.x; c < k.nchunk; c += KR_T) {
      const unsigned long long u = (unsigned long long)__double_as_longlong(pp[c]);
      a = u > a ? u : a;
    }
    return kr_cta_max(a, sh);
  }
  double a = 0.0;
  for (int c = threadIdx.x; c < k.nchunk; c += KR_T) a += pp[c];
  return kr_cta_sum(a, sh);
}

// the chunk of this CTA: [i0, i1) of block blk, vector offset base
#define KR_CHUNK_RANGE                                              \
  const int blk = blockIdx.y;                                       \
  const long long i0 = (long long)blockIdx.x * KR_CHUNK;            \
  const long long i1 = min(i0 + (long long)KR_CHUNK, k.n);          \
  const long long base = (long long)blk * k.n;

__device__ __forceinline__ double kr_alpha(const KrView &k, int blk, double *sh) {
  return k.rho[blk] / kr_parts<false>(k, KP_RV, blk, sh);
}
__device__ __forceinline__ double kr_omega(const KrView &k, int blk, double *sh) {
  const double ts = kr_parts<false>(k, KP_TS, blk, sh);
  const double tt = kr_parts<false>(k, KP_TT, blk, sh);
  return tt > 0.0 ? ts / tt : 0.0;
}

// -- set-up: minv from the diagonal (in t), x = x_good = 0, |b| and checks
__global__ void __launch_bounds__(KR_T) k_kr_init(KrView k) {
  __shared__ double sh[KR_T / 32];
  KR_CHUNK_RANGE
  int zero = 0, bad = 0;
  unsigned long long bmax = 0;
  for (long long i = i0 + threadIdx.x; i < i1; i += KR_T) {
    const long long j = base + i;
    const double d = k.t[j], bj = k.b[j];
    k.minv[j] = d != 0.0 ? 1.0 / d : 0.0;
    zero += d == 0.0;
    const unsigned long long ab = kr_absbits(bj);
    bmax = ab > bmax ? ab : bmax;
    bad += !kr_finite(bj);
    k.x[j] = 0.0;
    k.xg[j] = 0.0;
  }
  const double zs = kr_cta_count(zero, sh);
  const double bm = kr_cta_max(bmax, sh);
  const double bs = kr_cta_count(bad, sh);
  if (threadIdx.x == 0) {
    k.pp(KP_RR, blk)[blockIdx.x] = zs;
    k.pp(KP_MAX, blk)[blockIdx.x] = bm;
    k.pp(KP_BAD, blk)[blockIdx.x] = bs;
  }
}

// status RESTART (active) or IDLE on entry
__global__ void __launch_bounds__(KR_T) k_kr_init_sc(KrView k, double tol, double atol) {
  __shared__ double sh[KR_T / 32];
  const int blk = blockIdx.x;
  if (k.status[blk] != KR_RESTART) return;
  const double zero = kr_parts<false>(k, KP_RR, blk, sh);
  const double bmax = kr_parts<true>(k, KP_MAX, blk, sh);
  const double bad = kr_parts<false>(k, KP_BAD, blk, sh);
  if (threadIdx.x == 0) {
    int e = 0;
    if (zero > 0.0) e |= KE_ZERO_DIAG;
    if (bad > 0.0) e |= KE_NONFINITE_B;
    k.err[blk] = e;
    const double t = fmax(tol * bmax, atol);
    k.target[blk] = t;
    if (e || bmax == 0.0 || bmax <= t) k.status[blk] = KR_IDLE;  // x_s = 0 already meets the target
  }
}

// -- restart of RESTART blocks from their iterate: r = rhat = b - A x (in t)
__global__ void __launch_bounds__(KR_T) k_kr_restart(KrView k) {
  __shared__ double sh[KR_T / 32];
  KR_CHUNK_RANGE
  if (k.status[blk] != KR_RESTART) return;
  double rr = 0.0;
  int bad = 0;
  for (long long i = i0 + threadIdx.x; i < i1; i += KR_T) {
    const long long j = base + i;
    const double rj = k.b[j] - k.t[j];
    k.r[j] = rj;
    k.rhat[j] = rj;
    k.p[j] = 0.0;
    k.v[j] = 0.0;
    rr = fma(rj, rj, rr);
    bad += !kr_finite(rj);
  }
  const double rs = kr_cta_sum(rr, sh);
  const double bs = kr_cta_count(bad, sh);
  if (threadIdx.x == 0) {
    k.pp(KP_RR, blk)[blockIdx.x] = rs;
    k.pp(KP_BAD, blk)[blockIdx.x] = bs;
  }
}

__global__ void __launch_bounds__(KR_T) k_kr_restart_sc(KrView k) {
  __shared__ double sh[KR_T / 32];
  const int blk = blockIdx.x;
  if (k.status[blk] != KR_RESTART) return;
  const double rr = kr_parts<false>(k, KP_RR, blk, sh);
  const double bad = kr_parts<false>(k, KP_BAD, blk, sh);
  if (threadIdx.x == 0) {
    if (bad > 0.0 || !kr_finite(rr)) {
      k.err[blk] |= KE_NONFINITE_RESTART;
      k.status[blk] = KR_IDLE;
      return;
    }
    k.rho[blk] = rr;
    k.rho_old[blk] = 1.0;
    k.alpha[blk] = 1.0;
    k.omega[blk] = 1.0;
    k.status[blk] = rr == 0.0 ? KR_CONVERGED : KR_RUNNING;
  }
}

// -- one iteration ----------------------------------------------------------
// p = r + beta (p - omega v); phat = M^-1 p
__global__ void __launch_bounds__(KR_T) k_kr_p(KrView k) {
  KR_CHUNK_RANGE
  if (k.status[blk] != KR_RUNNING) return;
  const double om = k.omega[blk];
  const double beta = (k.rho[blk] / k.rho_old[blk]) * (k.alpha[blk] / om);
  for (long long i = i0 + threadIdx.x; i < i1; i += KR_T) {
    const long long j = base + i;
    const double pj = fma(beta, fma(-om, k.v[j], k.p[j]), k.r[j]);
    k.p[j] = pj;
    k.phat[j] = k.minv[j] * pj;
  }
}

// partials of rhat . v
__global__ void __launch_bounds__(KR_T) k_kr_dot1(KrView k) {
  __shared__ double sh[KR_T / 32];
  KR_CHUNK_RANGE
  if (k.status[blk] != KR_RUNNING) return;
  double a = 0.0;
  for (long long i = i0 + threadIdx.x; i < i1; i += KR_T) a = fma(k.rhat[base + i], k.v[base + i], a);
  a = kr_cta_sum(a, sh);
  if (threadIdx.x == 0) k.pp(KP_RV, blk)[blockIdx.x] = a;
}

// alpha = rho / (rhat . v); s = r - alpha v; shat = M^-1 s
__global__ void __launch_bounds__(KR_T) k_kr_s(KrView k) {
  __shared__ double sh[KR_T / 32];
  KR_CHUNK_RANGE
  if (k.status[blk] != KR_RUNNING) return;
  const double al = kr_alpha(k, blk, sh);
  for (long long i = i0 + threadIdx.x; i < i1; i += KR_T) {
    const long long j = base + i;
    const double sj = fma(-al, k.v[j], k.r[j]);
    k.s[j] = sj;
    k.shat[j] = k.minv[j] * sj;
  }
}

// partials of t . s and t . t
__global__ void __launch_bounds__(KR_T) k_kr_dot2(KrView k) {
  __shared__ double sh[KR_T / 32];
  KR_CHUNK_RANGE
  if (k.status[blk] != KR_RUNNING) return;
  double ts = 0.0, tt = 0.0;
  for (long long i = i0 + threadIdx.x; i < i1; i += KR_T) {
    const double tj = k.t[base + i];
    ts = fma(tj, k.s[base + i], ts);
    tt = fma(tj, tj, tt);
  }
  ts = kr_cta_sum(ts, sh);
  tt = kr_cta_sum(tt, sh);
  if (threadIdx.x == 0) {
    k.pp(KP_TS, blk)[blockIdx.x] = ts;
    k.pp(KP_TT, blk)[blockIdx.x] = tt;
  }
}

// omega = (t.s)/(t.t); x += alpha phat + omega shat; r = s - omega t;
// partials of rhat . r, max |r| and non-finite entries
__global__ void __launch_bounds__(KR_T) k_kr_x(KrView k) {
  __shared__ double sh[KR_T / 32];
  KR_CHUNK_RANGE
  if (k.status[blk] != KR_RUNNING) return;
  const double al = kr_alpha(k, blk, sh);
  const double om = kr_omega(k, blk, sh);
  double rr = 0.0;
  unsigned long long mx = 0;
  int bad = 0;
  for (long long i = i0 + threadIdx.x; i < i1; i += KR_T) {
    const long long j = base + i;
    const double xn = fma(om, k.shat[j], fma(al, k.phat[j], k.x[j]));
    const double rn = fma(-om, k.t[j], k.s[j]);
    k.x[j] = xn;
    k.r[j] = rn;
    rr = fma(k.rhat[j], rn, rr);
    const unsigned long long ab = kr_absbits(rn);
    mx = ab > mx ? ab : mx;
    bad += !(kr_finite(xn) && kr_finite(rn));
  }
  const double rs = kr_cta_sum(rr, sh);
  const double ms = kr_cta_max(mx, sh);
  const double bs = kr_cta_count(bad, sh);
  if (threadIdx.x == 0) {
    k.pp(KP_RR, blk)[blockIdx.x] = rs;
    k.pp(KP_MAX, blk)[blockIdx.x] = ms;
    k.pp(KP_BAD, blk)[blockIdx.x] = bs;
  }
}

// per block: the iteration's scalars and the state word
__global__ void __launch_bounds__(KR_T) k_kr_sc(KrView k) {
  __shared__ double sh[KR_T / 32];
  const int blk = blockIdx.x;
  if (k.status[blk] != KR_RUNNING) return;
  const double al = kr_alpha(k, blk, sh);
  const double om = kr_omega(k, blk, sh);
  const double rho_new = kr_parts<false>(k, KP_RR, blk, sh);
  const double mx = kr_parts<true>(k, KP_MAX, blk, sh);
  const double bad = kr_parts<false>(k, KP_BAD, blk, sh);
  if (threadIdx.x == 0) {
    if (bad > 0.0 || !kr_finite(al) || !kr_finite(rho_new))
      k.status[blk] = KR_BROKE;
    else if (mx <= k.target[blk])
      k.status[blk] = KR_CONVERGED;
    else if (om == 0.0 || rho_new == 0.0)
      k.status[blk] = KR_RESTART;  // next beta undefined: new shadow vector
    k.rho_old[blk] = k.rho[blk];
    k.rho[blk] = rho_new;
    k.alpha[blk] = al;
    k.omega[blk] = om;
  }
}

// -- between blocks of iterations -------------------------------------------
// x_good = x for RUNNING blocks; x = x_good for BROKE blocks
__global__ void __launch_bounds__(KR_T) k_kr_copy(KrView k, int want, int to_good) {
  KR_CHUNK_RANGE
  if (k.status[blk] != want) return;
  double *dst = to_good ? k.xg : k.x;
  const double *src = to_good ? k.x : k.xg;
  for (long long i = i0 + threadIdx.x; i < i1; i += KR_T) dst[base + i] = src[base + i];
}

__global__ void k_kr_trans(KrView k, int from, int to) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < k.S; b += gridDim.x * blockDim.x)
    if (k.status[b] == from) k.status[b] = to;
}

// true residual of CONVERGED blocks (A x in t): partials of max |b - A x|
__global__ void __launch_bounds__(KR_T) k_kr_true(KrView k) {
  __shared__ double sh[KR_T / 32];
  KR_CHUNK_RANGE
  if (k.status[blk] != KR_CONVERGED) return;
  unsigned long long mx = 0;
  int bad = 0;
  for (long long i = i0 + threadIdx.x; i < i1; i += KR_T) {
    const double d = k.b[base + i] - k.t[base + i];
    const unsigned long long ab = kr_absbits(d);
    mx = ab > mx ? ab : mx;
    bad += !kr_finite(d);
  }
  const double ms = kr_cta_max(mx, sh);
  const double bs = kr_cta_count(bad, sh);
  if (threadIdx.x == 0) {
    k.pp(KP_MAX, blk)[blockIdx.x] = ms;
    k.pp(KP_BAD, blk)[blockIdx.x] = bs;
  }
}

__global__ void __launch_bounds__(KR_T) k_kr_true_sc(KrView k) {
  __shared__ double sh[KR_T / 32];
  const int blk = blockIdx.x;
  if (k.status[blk] != KR_CONVERGED) return;
  const double mx = kr_parts<true>(k, KP_MAX, blk, sh);
  const double bad = kr_parts<false>(k, KP_BAD, blk, sh);
  if (threadIdx.x == 0) k.status[blk] = (bad == 0.0 && mx <= 10.0 * k.target[blk]) ? KR_IDLE : KR_RESTART;
}

#undef KR_CHUNK_RANGE

} // namespace

struct fe_krylov {
  const int *rowptr = nullptr, *colidx = nullptr;
  const void *vals = nullptr;
  int prec = FE_JAC_F64;
  long long n_total = 0, nnz = 0;
  int check_every = 8;
  bool use_graph = true;
  KrView k{};
  DevBuf vec, sca, stat, part;
  int *h_status = nullptr;  // pinned [2 * S]: state words, error words
  cudaStream_t st = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long blocks_run = 0;
  int64_t launches = 0, graph_replays = 0, restarts = 0;

  dim3 vgrid() const { return dim3((unsigned)k.nchunk, (unsigned)k.S); }
  void spmv_on(const double *x, double *y, const int *bstate, int want, cudaStream_t s) {
    launch_csr_spmv(rowptr, colidx, vals, prec, x, y, n_total, nnz, bstate, want, k.n, s);
    launches++;
  }
  void spmv(const double *x, double *y, int want) { spmv_on(x, y, k.status, want, st); }
  void iteration() {
    k_kr_p<<<vgrid(), KR_T, 0, st>>>(k);
    spmv(k.phat, k.v, KR_RUNNING);
    k_kr_dot1<<<vgrid(), KR_T, 0, st>>>(k);
    k_kr_s<<<vgrid(), KR_T, 0, st>>>(k);
    spmv(k.shat, k.t, KR_RUNNING);
    k_kr_dot2<<<vgrid(), KR_T, 0, st>>>(k);
    k_kr_x<<<vgrid(), KR_T, 0, st>>>(k);
    k_kr_sc<<<k.S, KR_T, 0, st>>>(k);
    launches += 6;
  }
  void restart_sequence() {
    spmv(k.x, k.t, KR_RESTART);
    k_kr_restart<<<vgrid(), KR_T, 0, st>>>(k);
    k_kr_restart_sc<<<k.S, KR_T, 0, st>>>(k);
    launches += 2;
  }
  int read_status() {
    CUDA_TRY(cudaMemcpyAsync(h_status, k.status, sizeof(int) * k.S, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaMemcpyAsync(h_status + k.S, k.err, sizeof(int) * k.S, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return FE_OK;
  }
  // check_every iterations: eagerly the first time (kernels load), then
  // captured once as a graph and replayed
  int run_block() {
    if (!use_graph || blocks_run == 0) {
      for (int i = 0; i < check_every; i++) iteration();
      CUDA_TRY(cudaGetLastError());
    } else {
      if (!exec) {
        cudaGraph_t g = nullptr;
        CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const int64_t l0 = launches;
        for (int i = 0; i < check_every; i++) iteration();
        cudaError_t e = cudaStreamEndCapture(st, &g);
        launches = l0;
        if (e != cudaSuccess || !g) {
          cudaGetLastError();
          use_graph = false;  // capture refused: eager from now on
          return run_block();
        }
        e = cudaGraphInstantiate(&exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
          cudaGetLastError();
          exec = nullptr;
          use_graph = false;
          return run_block();
        }
      }
      CUDA_TRY(cudaGraphLaunch(exec, st));
      graph_replays++;
      launches += 8LL * check_every;
    }
    blocks_run++;
    return FE_OK;
  }
  ~fe_krylov() {
    if (exec) cudaGraphExecDestroy(exec);
    if (h_status) cudaFreeHost(h_status);
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
    if (st) cudaStreamDestroy(st);
  }
};

extern "C" {

int fe_krylov_create(const int32_t *rowptr, const int32_t *colidx, const void *vals, int val_precision, int64_t n,
                     int64_t nnz, int32_t blocks, int32_t check_every, int32_t use_graph, fe_krylov_t **out) {
  if (!out) return fail(FE_ERR_ARG, "fe_krylov_create: null out");
  *out = nullptr;
  if (!rowptr || !colidx || !vals || n <= 0 || nnz <= 0) return fail(FE_ERR_ARG, "fe_krylov_create: empty matrix");
  if (blocks < 1 || blocks > 65535 || n % blocks) return fail(FE_ERR_ARG, "fe_krylov_create: %lld rows do not split "
                                                              "into %d equal blocks", (long long)n, blocks);
  if (val_precision != FE_JAC_F64 && val_precision != FE_JAC_F32) return fail(FE_ERR_ARG, "bad precision");
  if (check_every < 1 || check_every > 1024) return fail(FE_ERR_ARG, "check_every out of range");
  int rc = ensure_context();
  if (rc) return rc;
  std::unique_ptr<fe_krylov> K(new fe_krylov());
  K->rowptr = rowptr;
  K->colidx = colidx;
  K->vals = vals;
  K->prec = val_precision;
  K->n_total = n;
  K->nnz = nnz;
  K->check_every = check_every;
  K->use_graph = use_graph != 0;
  KrView &k = K->k;
  k.S = blocks;
  k.n = n / blocks;
  k.nchunk = (int)((k.n + KR_CHUNK - 1) / KR_CHUNK);
  if ((rc = K->vec.alloc(sizeof(double) * 12 * (size_t)n))) return rc;
  if ((rc = K->sca.alloc(sizeof(double) * 5 * (size_t)blocks))) return rc;
  if ((rc = K->stat.alloc(sizeof(int) * 2 * (size_t)blocks))) return rc;
  if ((rc = K->part.alloc(sizeof(double) * KP_N * (size_t)blocks * k.nchunk))) return rc;
  double *v = (double *)K->vec.p;
  double **vecs[12] = {&k.b, &k.x, &k.xg, &k.r, &k.rhat, &k.p, &k.v, &k.s, &k.t, &k.phat, &k.shat, &k.minv};
  for (int i = 0; i < 12; i++) *vecs[i] = v + (size_t)i * n;
  double *sc = (double *)K->sca.p;
  double **scas[5] = {&k.rho, &k.rho_old, &k.alpha, &k.omega, &k.target};
  for (int i = 0; i < 5; i++) *scas[i] = sc + (size_t)i * blocks;
  k.status = (int *)K->stat.p;
  k.err = k.status + blocks;
  k.part = (double *)K->part.p;
  CUDA_TRY(cudaMemset(K->vec.p, 0, K->vec.bytes));
  CUDA_TRY(cudaMemset(K->sca.p, 0, K->sca.bytes));
  CUDA_TRY(cudaMemset(K->part.p, 0, K->part.bytes));
  CUDA_TRY(cudaMallocHost((void **)&K->h_status, sizeof(int) * 2 * blocks));
  CUDA_TRY(cudaStreamCreateWithFlags(&K->st, cudaStreamNonBlocking));
  CUDA_TRY(cudaEventCreateWithFlags(&K->ev_in, cudaEventDisableTiming));
  CUDA_TRY(cudaEventCreateWithFlags(&K->ev_out, cudaEventDisableTiming));
  *out = K.release();
  return FE_OK;
}

void fe_krylov_destroy(fe_krylov_t *k) {
  if (!k) return;
  if (k->st) cudaStreamSynchronize(k->st);
  delete k;
}

int fe_krylov_matvec(fe_krylov_t *k, const double *x, double *y, void *stream) {
  if (!k || !x || !y) return fail(FE_ERR_ARG, "fe_krylov_matvec: null argument");
  k->spmv_on(x, y, nullptr, 0, (cudaStream_t)stream);
  CUDA_TRY(cudaGetLastError());
  return FE_OK;
}

int fe_krylov_info(const fe_krylov_t *k, int64_t *launches, int64_t *graph_replays, int64_t *restarts) {
  if (!k) return fail(FE_ERR_ARG, "fe_krylov_info: null handle");
  if (launches) *launches = k->launches;
  if (graph_replays) *graph_replays = k->graph_replays;
  if (restarts) *restarts = k->restarts;
  return FE_OK;
}

namespace {
int krylov_solve(fe_krylov_t *K, const double *b, const uint8_t *active, double tol, double atol, int64_t maxiter,
                 int32_t max_restarts, double *x, int64_t *iterations) {
  KrView &k = K->k;
  const int S = k.S;
  cudaStream_t st = K->st;
  std::vector<int64_t> its(S, 0), rst(S, 0);
  for (int s = 0; s < S; s++) K->h_status[s] = (!active || active[s]) ? KR_RESTART : KR_IDLE;
  CUDA_TRY(cudaMemcpyAsync(k.status, K->h_status, sizeof(int) * S, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemsetAsync(k.err, 0, sizeof(int) * S, st));
  CUDA_TRY(cudaMemcpyAsync(k.b, b, sizeof(double) * K->n_total, cudaMemcpyDeviceToDevice, st));
  const int gd = grid_for(K->n_total, 256, sm_count_cached());
  if (K->prec == FE_JAC_F64)
    k_csr_diagonal<double><<<gd, 256, 0, st>>>(K->rowptr, K->colidx, (const double *)K->vals, k.t, K->n_total);
  else
    k_csr_diagonal<float><<<gd, 256, 0, st>>>(K->rowptr, K->colidx, (const float *)K->vals, k.t, K->n_total);
  k_kr_init<<<K->vgrid(), KR_T, 0, st>>>(k);
  k_kr_init_sc<<<S, KR_T, 0, st>>>(k, tol, atol);
  K->launches += 3;
  K->restart_sequence();
  CUDA_TRY(cudaGetLastError());
  int64_t total = 0;
  for (;;) {
    int rc = K->read_status();
    if (rc) return rc;
    const int *hs = K->h_status, *he = K->h_status + S;
    bool conv = false, broke = false, restart = false, running = false;
    for (int s = 0; s < S; s++) {
      if (he[s] & KE_ZERO_DIAG)
        return fail(FE_ERR_SOLVER, "zero diagonal entry in block %d: Jacobi-preconditioned BiCGStab does not "
                                   "apply (saddle-point system); use the host solver", s);
      if (he[s] & KE_NONFINITE_B) return fail(FE_ERR_SOLVER, "non-finite right-hand side in block %d", s);
      if (he[s] & KE_NONFINITE_RESTART) return fail(FE_ERR_SOLVER, "non-finite residual at a restart of block %d", s);
      conv |= hs[s] == KR_CONVERGED;
      broke |= hs[s] == KR_BROKE;
      restart |= hs[s] == KR_RESTART;
      running |= hs[s] == KR_RUNNING;
      if (hs[s] == KR_BROKE || hs[s] == KR_RESTART) {
        K->restarts++;
        if (++rst[s] > max_restarts)
          return fail(FE_ERR_SOLVER, "BiCGStab broke down repeatedly in block %d (%lld iterations)", s,
                      (long long)its[s]);
      }
    }
    if (conv || broke || restart) {
      if (conv) {
        K->spmv(k.x, k.t, KR_CONVERGED);
        k_kr_true<<<K->vgrid(), KR_T, 0, st>>>(k);
        k_kr_true_sc<<<S, KR_T, 0, st>>>(k);
        K->launches += 2;
      }
      if (broke) {
        k_kr_copy<<<K->vgrid(), KR_T, 0, st>>>(k, KR_BROKE, 0);
        k_kr_trans<<<1, 256, 0, st>>>(k, KR_BROKE, KR_RESTART);
        K->launches += 2;
      }
      K->restart_sequence();
      CUDA_TRY(cudaGetLastError());
      continue;
    }
    if (!running) break;
    if (total >= maxiter) return fail(FE_ERR_SOLVER, "BiCGStab did not reach %g in %lld iterations", tol,
                                      (long long)maxiter);
    k_kr_copy<<<K->vgrid(), KR_T, 0, st>>>(k, KR_RUNNING, 1);
    K->launches++;
    if ((rc = K->run_block())) return rc;
    for (int s = 0; s < S; s++)
      if (hs[s] == KR_RUNNING) its[s] += K->check_every;
    total += K->check_every;
  }
  CUDA_TRY(cudaMemcpyAsync(x, k.x, sizeof(double) * K->n_total, cudaMemcpyDeviceToDevice, st));
  if (iterations)
    for (int s = 0; s < S; s++) iterations[s] = its[s];
  return FE_OK;
}
} // namespace

int fe_krylov_solve(fe_krylov_t *K, const double *b, const uint8_t *active, double tol, double atol,
                    int64_t maxiter, int32_t max_restarts, double *x, int64_t *iterations, void *stream) {
  if (!K || !b || !x) return fail(FE_ERR_ARG, "fe_krylov_solve: null argument");
  if (!(tol >= 0.0) || !(atol >= 0.0)) return fail(FE_ERR_ARG, "fe_krylov_solve: tolerances must be >= 0");
  cudaStream_t ust = (cudaStream_t)stream;
  CUDA_TRY(cudaEventRecord(K->ev_in, ust));
  CUDA_TRY(cudaStreamWaitEvent(K->st, K->ev_in, 0));
  int rc = krylov_solve(K, b, active, tol, atol, maxiter, max_restarts, x, iterations);
  if (rc) {
    cudaStreamSynchronize(K->st);  // nothing of a failed solve stays in flight
    return rc;
  }
  CUDA_TRY(cudaEventRecord(K->ev_out, K->st));
  CUDA_TRY(cudaStreamWaitEvent(ust, K->ev_out, 0));
  return FE_OK;
}

} // extern "C"
