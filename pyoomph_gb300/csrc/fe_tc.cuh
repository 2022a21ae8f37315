// fe_tc.cuh -- element Jacobians contracted on the tensor cores (tcgen05).
//
// The reference emits the element matrix as a loop over integration points
// and test/trial functions (write_generic_RJM_jacobian_contribution,
// src/codegen.cpp:1883-2258).  In reference coordinates that matrix is
//
//   J_e[i][j] = sum_q sum_p Phi[q][a_p][i] Dhat_e[q][p] Phi[q][b_p][j]
//
// with Phi the element type's reference basis (value and d/ds components at
// the knots, the same for every element) and Dhat_e the pulled-back pointwise
// derivatives over the pairs p = (a_p, b_p) of components the weak form
// couples.  With A_e[(q,a)][j] = sum_{p: a_p = a} Dhat_e[q][p] Phi[q][b_p][j]
// it is one small GEMM per element, J_e = Phi^T A_e, whose B operand Phi^T
// is shared by all elements.  Here (one CTA per SM, persistent over tiles):
//
//   * rows m of a 128-row tile are (element, trial function j): 4 elements
//     of up to 32 local functions; columns are the test functions i (N = 32);
//     K = (knot, active test component), zero-padded to a multiple of 8;
//   * every thread builds A in shared memory from the tile's Dhat (FP32,
//     written by the element kernel) and the staged Phi, split into a TF32
//     high part (round to nearest) and the FP32 remainder;
//   * one thread issues 3 x K/8 tcgen05.mma.kind::tf32 (128 x 32 x 8) into a
//     TMEM accumulator: A_hi B_hi + A_hi B_lo + A_lo B_hi (the "3xTF32"
//     split, ~2^-21 relative per product, FP32 accumulation), commits to an
//     mbarrier;
//   * warps 0-3 read their 32 TMEM lanes (tcgen05.ld 32x32b.x32) and store
//     J_e rows to the element-matrix buffer (FP32).
//
// Shared-memory operands are K-major without swizzle: core matrices of 8 rows
// x 16 bytes; element (r, k) of an R-row operand at byte
//   (k / 4) * (R * 16) + (r / 8) * 128 + (r % 8) * 16 + (k % 4) * 4,
// so the descriptor's leading-dimension offset (between core matrices along
// K) is R * 16 bytes and its stride-dimension offset (between 8-row groups)
// 128 bytes.
//
// Waits are bounded: an mbarrier wait that exceeds its iteration limit sets
// status bit FE_TC_TIMEOUT, waits once more (bounded), frees the TMEM columns
// and returns.
#ifndef FE_TC_CUH
#define FE_TC_CUH

#include <cstdint>

#define FE_TC_ROWS 128        // M of one MMA (tile rows)
#define FE_TC_N 32            // N of one MMA (test functions, padded)
#define FE_TC_EPT 4           // elements per tile (32 rows each)
#define FE_TC_THREADS 256
#define FE_TC_MAXK 128        // padded K at most (knots x active components)
#define FE_TC_MAXQ 32         // knots at most
#define FE_TC_MAXP 32         // Dhat pairs per knot at most
#define FE_TC_MAXC 4          // reference components (value + dim derivatives)
#define FE_TC_TIMEOUT 8       // status bit: an mbarrier wait gave up
#define FE_TC_SPIN_LIMIT (1u << 26)

struct FeTcArgs {
  const float *dhat;      // [n_elem][nq][npair] pulled-back derivatives (element kernel output)
  const float *phi;       // [nq][nc][FE_TC_N] reference basis, zero beyond the n local functions
  const float *b_hi;      // B operand, high TF32 part, already in the shared-memory layout: [kp/4][32][4]
  const float *b_lo;      // B operand, FP32 remainder, same layout
  float *jbuf;            // [n_elem][n][n] element matrices (FP32)
  int *status;            // status word of the problem
  long long n_elem;
  int n;                  // local functions (<= 32)
  int nq;                 // knots
  int nc;                 // reference components per knot
  int npair;              // Dhat entries per knot
  int nact;               // active test components (K = nq * nact)
  int kp;                 // K padded to a multiple of 8
  int act_of[FE_TC_MAXC]; // active test component index of component a (-1: none)
  int pa[FE_TC_MAXP];     // test component a_p of pair p
  int pb[FE_TC_MAXP];     // trial component b_p of pair p
};

namespace fe_tc {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor (tcgen05): start, leading/stride byte
// offsets (>> 4), descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor: D FP32, A and B TF32, both K-major, N and M
__host__ __device__ constexpr uint32_t idesc_tf32(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ float tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}

__device__ __forceinline__ void mma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}"
      :
      : "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

__device__ __forceinline__ void commit(uint64_t *mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

// bounded wait for the completion of `phase`; false when the limit ran out
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t phase) {
  const uint32_t a = smem_u32(mbar);
  for (uint32_t it = 0; it < FE_TC_SPIN_LIMIT; ++it) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(a), "r"(phase)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 32 lanes x 32 columns of FP32 from TMEM (this warp's lane quarter)
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

// shared-memory plan of one CTA (bytes): the B operand pieces, the A operand
// pieces, the tile's Dhat, Phi, the mbarrier and the TMEM address word; the
// A/B regions carry FE_TC_GUARD bytes of slack behind them
#define FE_TC_GUARD (48 * 1024)
struct Plan {
  uint32_t b_hi, b_lo, a_hi, a_lo, dh, ph, bar, total;
};

__host__ __device__ inline Plan plan(int kp, int nq, int npair, int nc) {
  Plan p;
  const uint32_t bbytes = (uint32_t)kp * FE_TC_N * 4, abytes = (uint32_t)kp * FE_TC_ROWS * 4;
  p.b_hi = 0;
  p.b_lo = p.b_hi + bbytes;
  p.a_hi = p.b_lo + bbytes;
  p.a_lo = p.a_hi + abytes;
  p.dh = p.a_lo + abytes + FE_TC_GUARD;
  p.ph = p.dh + (uint32_t)FE_TC_EPT * nq * npair * 4;
  p.bar = ((p.ph + (uint32_t)nq * nc * FE_TC_N * 4) + 15u) & ~15u;
  p.total = p.bar + 16;
  return p;
}

} // namespace fe_tc

__global__ void __launch_bounds__(FE_TC_THREADS, 1) k_tc_contract(const FeTcArgs a) {
  using namespace fe_tc;
  extern __shared__ __align__(1024) unsigned char tsm[];
  const Plan pl = plan(a.kp, a.nq, a.npair, a.nc);
  float *sBhi = reinterpret_cast<float *>(tsm + pl.b_hi);
  float *sBlo = reinterpret_cast<float *>(tsm + pl.b_lo);
  float *sAhi = reinterpret_cast<float *>(tsm + pl.a_hi);
  float *sAlo = reinterpret_cast<float *>(tsm + pl.a_lo);
  float *sDh = reinterpret_cast<float *>(tsm + pl.dh);
  float *sPh = reinterpret_cast<float *>(tsm + pl.ph);
  uint64_t *bar = reinterpret_cast<uint64_t *>(tsm + pl.bar);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(tsm + pl.bar + 8);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int kq = a.kp >> 2;                       // K chunks of 4
  const int dper = a.nq * a.npair;                // Dhat floats per element

  // stage B and Phi; set up the mbarrier; warp 0 allocates 32 TMEM columns
  for (int k = tid; k < a.kp * FE_TC_N; k += FE_TC_THREADS) {
    sBhi[k] = a.b_hi[k];
    sBlo[k] = a.b_lo[k];
  }
  for (int k = tid; k < a.nq * a.nc * FE_TC_N; k += FE_TC_THREADS) sPh[k] = a.phi[k];
  if (tid == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(smem_u32(tslot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = idesc_tf32(FE_TC_ROWS, FE_TC_N);
  const long long ntiles = (a.n_elem + FE_TC_EPT - 1) / FE_TC_EPT;
  uint32_t phase = 0;
  bool ok = true;

  for (long long t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
    const long long e0 = t * FE_TC_EPT;
    const int nel = (int)min((long long)FE_TC_EPT, a.n_elem - e0);
    // the tile's Dhat (contiguous in global memory)
    for (int k = tid; k < FE_TC_EPT * dper; k += FE_TC_THREADS)
      sDh[k] = k < nel * dper ? a.dhat[e0 * dper + k] : 0.0f;
    __syncthreads();
    // A[m = (element, j)][k = (q, active a)] = sum_{p: a_p = a} Dhat[q][p] Phi[q][b_p][j]
    for (int it = tid; it < FE_TC_ROWS * kq; it += FE_TC_THREADS) {
      const int m = it & (FE_TC_ROWS - 1), kc = it >> 7;
      const int el = m >> 5, j = m & 31;
      float v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int k = kc * 4 + u;
        const int q = k / a.nact, ai = k - q * a.nact;
        float s = 0.0f;
        if (el < nel && j < a.n && q < a.nq) {
          const float *dq = sDh + el * dper + q * a.npair;
          const float *pq = sPh + q * a.nc * FE_TC_N + j;
          for (int p = 0; p < a.npair; ++p)
            if (a.act_of[a.pa[p]] == ai) s = fmaf(dq[p], pq[a.pb[p] * FE_TC_N], s);
        }
        v[u] = s;
      }
      float4 hi, lo;
      hi.x = tf32_rna(v[0]);
      hi.y = tf32_rna(v[1]);
      hi.z = tf32_rna(v[2]);
      hi.w = tf32_rna(v[3]);
      lo.x = v[0] - hi.x;
      lo.y = v[1] - hi.y;
      lo.z = v[2] - hi.z;
      lo.w = v[3] - hi.w;
      const int off = kc * (FE_TC_ROWS * 4) + (m >> 3) * 32 + (m & 7) * 4;   // floats
      *reinterpret_cast<float4 *>(sAhi + off) = hi;
      *reinterpret_cast<float4 *>(sAlo + off) = lo;
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    if (tid == 0) {
      const uint32_t ahi = smem_u32(sAhi), alo = smem_u32(sAlo), bhi = smem_u32(sBhi), blo = smem_u32(sBlo);
      const uint32_t albo = FE_TC_ROWS * 16, blbo = FE_TC_N * 16;
      for (int s = 0; s < a.kp / 8; ++s) {
        const uint32_t ao = (uint32_t)s * 2 * albo, bo = (uint32_t)s * 2 * blbo;
        mma_tf32(tmem, desc(ahi + ao, albo, 128), desc(bhi + bo, blbo, 128), idesc, s > 0 ? 1u : 0u);
        mma_tf32(tmem, desc(ahi + ao, albo, 128), desc(blo + bo, blbo, 128), idesc, 1u);
        mma_tf32(tmem, desc(alo + ao, albo, 128), desc(bhi + bo, blbo, 128), idesc, 1u);
      }
      commit(bar);
    }
    ok = mbar_wait(bar, phase);
    phase ^= 1u;
    fence_after();
    if (ok && warp < 4 && warp < nel) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16), v);
      const int j = lane;
      if (j < a.n) {
        float *out = a.jbuf + (e0 + warp) * (long long)a.n * a.n + j;
#pragma unroll
        for (int i = 0; i < 32; ++i)
          if (i < a.n) out[(long long)i * a.n] = v[i];
      }
    }
    fence_before();
    __syncthreads();
  }
  if (!ok) {
    if (tid == 0) atomicOr(a.status, FE_TC_TIMEOUT);
    mbar_wait(bar, phase ^ 1u);      // the MMAs still in flight, bounded
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(tmem) : "memory");
}

#endif
