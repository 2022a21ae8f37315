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
//     J_e rows to the element-matrix buffer (FP32);
//   * two A buffers and two TMEM accumulators: building tile t overlaps the
//     MMAs of tile t - 1, whose results are stored after tile t's are issued.
//
// Shared-memory operands are K-major without swizzle: core matrices of 8 rows
// x 16 bytes; element (r, k) of an R-row operand at byte
//   (k / 4) * (R * 16) + (r / 8) * 128 + (r % 8) * 16 + (k % 4) * 4,
// so the descriptor's leading-dimension offset (between core matrices along
// K) is R * 16 bytes and its stride-dimension offset (between 8-row groups)
// 128 bytes.
//
// Waits are bounded: an mbarrier wait that exceeds its iteration limit sets
// status bit FE_TC_TIMEOUT, waits once more (bounded) for the MMAs still in
// flight, frees the TMEM columns and returns.
#ifndef FE_TC_CUH
#define FE_TC_CUH

#include <cstdint>

#define FE_TC_ROWS 128        // M of one MMA (tile rows)
#define FE_TC_N 32            // N of one MMA (test functions, padded)
#define FE_TC_EPT 4           // elements per tile (32 rows each)
#define FE_TC_THREADS 512
#define FE_TC_MAXK 128        // padded K at most (knots x active components)
#define FE_TC_MAXQ 32         // knots at most
#define FE_TC_MAXP 32         // Dhat pairs per knot at most
#define FE_TC_MAXC 4          // reference components (value + dim derivatives)
#define FE_TC_TIMEOUT 8       // status bit: an mbarrier wait gave up
#define FE_TC_SPIN_LIMIT (1u << 22)

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
  int nterm[FE_TC_MAXC];  // per active test component: its pairs ...
  int tp[FE_TC_MAXC][FE_TC_MAXP]; // ... Dhat index p
  int tb[FE_TC_MAXC][FE_TC_MAXP]; // ... and trial component b_p
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

// one contiguous global -> shared copy on the async proxy, completing on an
// mbarrier that expects `bytes` (16-byte aligned addresses, size a multiple
// of 16)
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *mbar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(mbar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(mbar))
               : "memory");
}

// 32 lanes x 8 columns of FP32 from TMEM (this warp's lane quarter)
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 8; ++k) v[k] = __uint_as_float(r[k]);
}

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

// shared-memory plan of one CTA (bytes): the B operand pieces, two A
// operand buffers (hi and lo each), two Dhat buffers, Phi, two mbarriers and
// the TMEM address word
struct Plan {
  uint32_t b_hi, b_lo, a[2], abytes, dh[2], ph, kinfo, bar, total;
};

__host__ __device__ inline Plan plan(int kp, int nq, int npair, int nc) {
  Plan p;
  const uint32_t bbytes = (uint32_t)kp * FE_TC_N * 4;
  p.abytes = (uint32_t)kp * FE_TC_ROWS * 4;
  p.b_hi = 0;
  p.b_lo = p.b_hi + bbytes;
  p.a[0] = p.b_lo + bbytes;                  // a[b]: hi part, lo part right after it
  p.a[1] = p.a[0] + 2 * p.abytes;
  const uint32_t dbytes = ((uint32_t)FE_TC_EPT * nq * npair * 4 + 15u) & ~15u;
  p.dh[0] = p.a[1] + 2 * p.abytes;
  p.dh[1] = p.dh[0] + dbytes;
  p.ph = p.dh[1] + dbytes;
  p.kinfo = ((p.ph + (uint32_t)(nq * nc + 1) * FE_TC_N * 4) + 15u) & ~15u;   // Phi and a zero row
  p.bar = ((p.kinfo + (uint32_t)kp * FE_TC_MAXC * 8) + 15u) & ~15u;
  p.total = p.bar + 48;
  return p;
}

} // namespace fe_tc

// One CTA per SM, persistent over tiles of FE_TC_EPT elements.  Iteration t
// (buffer b = t & 1): the next tile's Dhat is requested (bulk copy into
// buffer b ^ 1), tile t's A operand is built into buffer b and its MMAs
// issued into TMEM columns [32 b, 32 b + 32); meanwhile the MMAs of tile
// t - 1 (buffer b ^ 1) run, and after issuing, every warp waits for them and
// stores 8 test rows of one element of tile t - 1 (16 warps: 4 elements x 4
// column groups).
__global__ void __launch_bounds__(FE_TC_THREADS, 1) k_tc_contract(const FeTcArgs a) {
  using namespace fe_tc;
  extern __shared__ __align__(1024) unsigned char tsm[];
  const Plan pl = plan(a.kp, a.nq, a.npair, a.nc);
  float *sBhi = reinterpret_cast<float *>(tsm + pl.b_hi);
  float *sBlo = reinterpret_cast<float *>(tsm + pl.b_lo);
  float *sPh = reinterpret_cast<float *>(tsm + pl.ph);
  int2 *sKT = reinterpret_cast<int2 *>(tsm + pl.kinfo);            // [kp][4] terms: (Dhat index, Phi row)
  uint64_t *bar = reinterpret_cast<uint64_t *>(tsm + pl.bar);      // [0,1]: MMAs, [2,3]: Dhat loads
  uint32_t *tslot = reinterpret_cast<uint32_t *>(tsm + pl.bar + 32);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int kq = a.kp >> 2;                       // K chunks of 4
  const int dper = a.nq * a.npair;                // Dhat floats per element
  const long long ntiles = (a.n_elem + FE_TC_EPT - 1) / FE_TC_EPT;
  // Dhat rows of whole elements are 16-byte multiples: bulk copies; else plain loads
  const bool bulk = (dper % 4) == 0 && ((reinterpret_cast<uintptr_t>(a.dhat) & 15u) == 0);

  // stage B, Phi and the K table; set up the mbarriers; warp 0 allocates 64 TMEM columns
  for (int k = tid; k < a.kp * FE_TC_N; k += FE_TC_THREADS) {
    sBhi[k] = a.b_hi[k];
    sBlo[k] = a.b_lo[k];
  }
  const int zrow = a.nq * a.nc * FE_TC_N;          // a row of zeros after Phi
  for (int k = tid; k < zrow + FE_TC_N; k += FE_TC_THREADS) sPh[k] = k < zrow ? a.phi[k] : 0.0f;
  // the terms of each K index (knot q, active test component ai): Dhat
  // entries q * npair + p and Phi rows (q, trial component b) * 32; unused
  // terms read the zero row
  for (int k = tid; k < a.kp * FE_TC_MAXC; k += FE_TC_THREADS) {
    const int kk = k / FE_TC_MAXC, tt = k - kk * FE_TC_MAXC;
    const int q = kk / a.nact, ai = kk - q * a.nact;
    int2 e = make_int2(0, zrow);
    if (q < a.nq && tt < a.nterm[ai]) e = make_int2(q * a.npair + a.tp[ai][tt], (q * a.nc + a.tb[ai][tt]) * FE_TC_N);
    sKT[k] = e;
  }
  if (tid == 0) {
    for (int k = 0; k < 4; ++k) mbar_init(bar + k, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(smem_u32(tslot))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tslot;
  const uint32_t idesc = idesc_tf32(FE_TC_ROWS, FE_TC_N);
  // the first tile's Dhat
  uint32_t loads = 0u;         // bit 2 + x: a Dhat copy into buffer x is in flight (every thread tracks it)
  if (bulk && (long long)blockIdx.x < ntiles) {
    if (tid == 0) {
      const long long e0 = (long long)blockIdx.x * FE_TC_EPT;
      const int nel = (int)min((long long)FE_TC_EPT, a.n_elem - e0);
      bulk_load(tsm + pl.dh[0], a.dhat + e0 * dper, (uint32_t)(nel * dper * 4), bar + 2);
    }
    loads |= 1u << 2;
  }
  uint32_t phases = 0u;        // bit k: the phase of mbarrier k's next completion
  bool ok = true;
  int failed = -1;             // MMA buffer whose wait gave up
  int pending = -1;            // MMA buffer issued and not yet waited for
  long long prev_tile = -1;

  for (long long t = blockIdx.x, it = 0;; t += gridDim.x, ++it) {
    const bool have = t < ntiles;
    const int b = (int)(it & 1);
    float *sDh = reinterpret_cast<float *>(tsm + pl.dh[b]);
    float *sAhi = reinterpret_cast<float *>(tsm + pl.a[b]);
    float *sAlo = reinterpret_cast<float *>(tsm + pl.a[b] + pl.abytes);
    const long long e0 = t * FE_TC_EPT;
    const int nel = have ? (int)min((long long)FE_TC_EPT, a.n_elem - e0) : 0;
    if (have) {
      const long long tn = t + gridDim.x;
      if (bulk && tn < ntiles) {
        if (tid == 0) {
          // buffer b ^ 1 was last read by the previous iteration's build (a barrier ago)
          fence_async_smem();
          const int nn_ = (int)min((long long)FE_TC_EPT, a.n_elem - tn * FE_TC_EPT);
          bulk_load(tsm + pl.dh[b ^ 1], a.dhat + tn * FE_TC_EPT * dper, (uint32_t)(nn_ * dper * 4),
                    bar + 2 + (b ^ 1));
        }
        loads |= 1u << (2 + (b ^ 1));
      }
      if (bulk) {
        if (mbar_wait(bar + 2 + b, (phases >> (2 + b)) & 1u)) {
          phases ^= 1u << (2 + b);
          loads &= ~(1u << (2 + b));
        } else {
          ok = false;
        }
      } else {
        for (int k = tid; k < nel * dper; k += FE_TC_THREADS) sDh[k] = a.dhat[e0 * dper + k];
        __syncthreads();
      }
      // A[m = (element, j)][k = (q, active a)] = sum over a's terms of Dhat[q][p] Phi[q][b][j]
      // (rows of elements beyond the tile's last read stale Dhat: their
      // output rows are never stored; Phi is zero for j >= n)
      for (int item = tid; item < FE_TC_ROWS * kq; item += FE_TC_THREADS) {
        const int m = item & (FE_TC_ROWS - 1), kc = item >> 7;
        const float *dE = sDh + (m >> 5) * dper;
        const float *pJ = sPh + (m & 31);
        const int2 *kt = sKT + kc * 4 * FE_TC_MAXC;
        float v[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          float s = 0.0f;
#pragma unroll
          for (int tt = 0; tt < FE_TC_MAXC; ++tt) {
            const int2 e = kt[u * FE_TC_MAXC + tt];
            s = fmaf(dE[e.x], pJ[e.y], s);
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
        const int off = kc * (FE_TC_ROWS * 4) + m * 4;   // floats: (k/4) * R*4 + (r/8)*32 + (r%8)*4
        *reinterpret_cast<float4 *>(sAhi + off) = hi;
        *reinterpret_cast<float4 *>(sAlo + off) = lo;
      }
      fence_async_smem();
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (have && ok && tid == 0) {
      const uint32_t ahi = smem_u32(sAhi), alo = smem_u32(sAlo), bhi = smem_u32(sBhi), blo = smem_u32(sBlo);
      const uint32_t albo = FE_TC_ROWS * 16, blbo = FE_TC_N * 16;
      const uint32_t d = tmem + (uint32_t)(b * FE_TC_N);
      for (int s = 0; s < a.kp / 8; ++s) {
        const uint32_t ao = (uint32_t)s * 2 * albo, bo = (uint32_t)s * 2 * blbo;
        mma_tf32(d, desc(ahi + ao, albo, 128), desc(bhi + bo, blbo, 128), idesc, s > 0 ? 1u : 0u);
        mma_tf32(d, desc(ahi + ao, albo, 128), desc(blo + bo, blbo, 128), idesc, 1u);
        mma_tf32(d, desc(alo + ao, albo, 128), desc(bhi + bo, blbo, 128), idesc, 1u);
      }
      commit(bar + b);
    }
    // the previous tile: wait for its MMAs, store its element matrices
    if (pending >= 0 && ok) {
      const int pb = pending;
      if (mbar_wait(bar + pb, (phases >> pb) & 1u)) {
        phases ^= 1u << pb;
      } else {
        ok = false;
        failed = pb;
      }
      fence_after();
      const int pnel = (int)min((long long)FE_TC_EPT, a.n_elem - prev_tile * FE_TC_EPT);
      const int q4 = warp & 3, cg = warp >> 2;      // lane quarter = element; column group of 8
      if (ok && q4 < pnel) {
        float v[8];
        tmem_ld8(tmem + ((uint32_t)(q4 * 32) << 16) + (uint32_t)(pb * FE_TC_N + cg * 8), v);
        const int j = lane;
        if (j < a.n) {
          float *out = a.jbuf + (prev_tile * FE_TC_EPT + q4) * (long long)a.n * a.n + j;
#pragma unroll
          for (int i = 0; i < 8; ++i)
            if (cg * 8 + i < a.n) out[(long long)(cg * 8 + i) * a.n] = v[i];
        }
      }
    }
    pending = (have && ok) ? b : pending;
    prev_tile = t;
    fence_before();
    __syncthreads();
    if (!have || !ok) break;
  }
  if (!ok) {
    if (tid == 0) atomicOr(a.status, FE_TC_TIMEOUT);
    // MMAs and Dhat copies that may still run (bounded waits)
    if (failed >= 0) mbar_wait(bar + failed, (phases >> failed) & 1u);
    if (pending >= 0 && pending != failed) mbar_wait(bar + pending, (phases >> pending) & 1u);
    for (int k = 2; k < 4; ++k)
      if (loads & (1u << k)) mbar_wait(bar + k, (phases >> k) & 1u);
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem) : "memory");
}

#endif
