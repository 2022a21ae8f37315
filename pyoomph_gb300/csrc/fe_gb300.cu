// fe_gb300.cu -- runtime of the GB300 finite-element assembly engine.
//
// Implements the C-ABI of include/fe_gb300.h:
//   * element code JIT (nvrtc -> cubin for sm_103a -> cudaLibraryLoadData),
//     the device counterpart of pyoomph's C compiler + dlopen path
//     (pyoomph/generic/ccompiler.py:207-242, src/ccompiler.cpp:191-213);
//   * the resident problem: nodal positions/values, connectivity and
//     equation numbers in HBM;
//   * the CSR pattern of oomph's vectors-of-pairs assembler
//     (problem.cc:5332-5666): rows in equation order, columns in order of
//     first insertion over (element, local i, local j), built once per mesh;
//   * the deterministic scatter: every CSR slot (and every residual entry)
//     owns the list of element contributions that reach it, in element
//     order, so a slot is summed by one thread in exactly the order the
//     reference accumulates it (problem.cc:5500-5560) -- no atomics;
//   * Newton helpers: dof -> nodal value scatter, residual max-norm with
//     NaN -> inf (double_vector.cc:611-629), x -= dx.
#include <cuda_runtime.h>
#include <nvrtc.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fe_gb300.h"
#include "fe_abi.h"
#include "fe_df64.cuh"
#include "fe_tc.cuh"

#define FE_VERSION "fe_gb300 0.1.0 (sm_103a)"

namespace {

thread_local std::string g_err;

int fail(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CUDA_TRY(expr)                                                                      \
  do {                                                                                      \
    cudaError_t _e = (expr);                                                                \
    if (_e != cudaSuccess)                                                                  \
      return fail(_e == cudaErrorMemoryAllocation ? FE_ERR_NOMEM : FE_ERR_CUDA, "%s: %s (%s:%d)", \
                  #expr, cudaGetErrorString(_e), __FILE__, __LINE__);                       \
  } while (0)


// ---------------------------------------------------------------------------
// device buffers
// ---------------------------------------------------------------------------
// Owning device allocation: movable, not copyable (a copy would free the
// same pointer twice).
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept : p(o.p), bytes(o.bytes) {
    o.p = nullptr;
    o.bytes = 0;
  }
  DevBuf &operator=(DevBuf &&o) noexcept {
    if (this != &o) {
      if (p) cudaFree(p);
      p = o.p;
      bytes = o.bytes;
      o.p = nullptr;
      o.bytes = 0;
    }
    return *this;
  }
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  int alloc(size_t n) {
    if (p) {
      cudaFree(p);
      p = nullptr;
    }
    bytes = n;
    if (n == 0) return FE_OK;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
      p = nullptr;
      return fail(FE_ERR_NOMEM, "cudaMalloc(%zu) failed: %s", n, cudaGetErrorString(e));
    }
    return FE_OK;
  }
  int upload(const void *h, size_t n) {
    int rc = alloc(n);
    if (rc) return rc;
    if (n) CUDA_TRY(cudaMemcpy(p, h, n, cudaMemcpyHostToDevice));
    return FE_OK;
  }
  template <class T> T *as() const { return reinterpret_cast<T *>(p); }
};

// ---------------------------------------------------------------------------
// kernels of the runtime (element kernels come from nvrtc)
// ---------------------------------------------------------------------------

// dofs -> nodal values (the Data values a Newton update writes)
__global__ void k_scatter_dofs(const double *__restrict__ dofs, const int *__restrict__ eqn,
                               double *__restrict__ values, long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    int e = eqn[k];
    if (e >= 0) values[k] = dofs[e];
  }
}

// CSR slot s = sum of its element contributions in element order.  With
// U > 1 each thread takes U slots at once (a grid stride apart, so every
// load stays coalesced across the warp) and issues their range, index and
// value loads together -- the first two contributions of every slot in one
// go, the rest after -- so a warp keeps U dependent chains in flight
// instead of one; each slot still sums its contributions in order.
// With `list`, slot list[i] for i < nnz instead of slot i (the rows one
// chunk of the pipelined assembly completes).  With ROWS, each thread first
// sums its residual rows (grid-stride, row rows.list[i] when given) in the
// order of k_gather_rows: R and J in one launch, the rows' dependent loads
// overlapping the slots' instead of a launch of their own.
struct GatherRows {
  const unsigned *rptr, *ridx;
  const double *rbuf;
  double *R;
  long long n;
  const int *list;
};

template <typename T, int U, bool LIST, bool ROWS = false>
__global__ void k_gather_slots(const unsigned *__restrict__ cptr, const unsigned *__restrict__ cidx,
                               const T *__restrict__ jbuf, T *__restrict__ vals, long long nnz,
                               const int *__restrict__ list, GatherRows rows = GatherRows{}) {
  const long long nthr = (long long)gridDim.x * blockDim.x;
  if constexpr (ROWS) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < rows.n; i += nthr) {
      const long long r = rows.list ? (long long)rows.list[i] : i;
      const unsigned b = rows.rptr[r], e = rows.rptr[r + 1];
      double acc = 0.0;
      for (unsigned k = b; k < e; k++) acc += rows.rbuf[rows.ridx[k]];
      rows.R[r] = acc;
    }
  }
  if constexpr (U == 1) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nnz; i += nthr) {
      const long long s = LIST ? (long long)list[i] : i;
      const unsigned b = cptr[s], e = cptr[s + 1];
      T acc = jbuf[cidx[b]];
      for (unsigned k = b + 1; k < e; k++) acc += jbuf[cidx[k]];
      vals[s] = acc;
    }
  } else
  for (long long s0 = blockIdx.x * (long long)blockDim.x + threadIdx.x; s0 < nnz; s0 += U * nthr) {
    unsigned b[U], e[U];
    long long sl[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const long long i = s0 + u * nthr;
      b[u] = e[u] = 0;
      if constexpr (LIST) {
        sl[u] = -1;
        if (i < nnz) {
          sl[u] = (long long)list[i];
          b[u] = cptr[sl[u]];
          e[u] = cptr[sl[u] + 1];
        }
      } else {
        sl[u] = i;
        if (i < nnz) {
          b[u] = cptr[i];
          e[u] = cptr[i + 1];
        }
      }
    }
    unsigned i0[U], i1[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      i0[u] = b[u] < e[u] ? cidx[b[u]] : 0u;
      i1[u] = b[u] + 1 < e[u] ? cidx[b[u] + 1] : i0[u];
    }
    T acc[U], v1[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      acc[u] = b[u] < e[u] ? jbuf[i0[u]] : (T)0;
      v1[u] = b[u] + 1 < e[u] ? jbuf[i1[u]] : (T)0;
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      if (LIST ? sl[u] < 0 : s0 + u * nthr >= nnz) continue;
      if (b[u] + 1 < e[u]) acc[u] += v1[u];
      for (unsigned k = b[u] + 2; k < e[u]; k++) acc[u] += jbuf[cidx[k]];
      if constexpr (LIST)
        vals[sl[u]] = acc[u];
      else
        vals[s0 + u * nthr] = acc[u];
    }
  }
}

// several slots per thread over patterns large enough to fill the GPU with
// fewer threads: four for FP32 values, two for FP64 (measured on GB300, NS
// 256^2: FP64 0.138 -> 0.129 ms with two, four cost more occupancy than the
// extra loads in flight gain; FP32 0.107 -> 0.084 ms with four, eight were
// slower again at 0.112)
int grid_for(long long n, int threads, int sms);

template <typename T, bool ROWS>
void launch_gather_slots_(const unsigned *cptr, const unsigned *cidx, const T *jbuf, T *vals, long long nnz, int sms,
                          cudaStream_t st, const int *list, const GatherRows &rows) {
  const bool big = nnz >= (1LL << 22);
  constexpr int UU = sizeof(T) == 4 ? 4 : 2;
  long long work = big ? (nnz + UU - 1) / UU : nnz;
  if (ROWS && rows.n > work) work = rows.n;
  const int g = grid_for(work, 256, sms);
  if (big && list)
    k_gather_slots<T, UU, true, ROWS><<<g, 256, 0, st>>>(cptr, cidx, jbuf, vals, nnz, list, rows);
  else if (big)
    k_gather_slots<T, UU, false, ROWS><<<g, 256, 0, st>>>(cptr, cidx, jbuf, vals, nnz, list, rows);
  else if (list)
    k_gather_slots<T, 1, true, ROWS><<<g, 256, 0, st>>>(cptr, cidx, jbuf, vals, nnz, list, rows);
  else
    k_gather_slots<T, 1, false, ROWS><<<g, 256, 0, st>>>(cptr, cidx, jbuf, vals, nnz, list, rows);
}

template <typename T>
void launch_gather_slots(const unsigned *cptr, const unsigned *cidx, const T *jbuf, T *vals, long long nnz, int sms,
                         cudaStream_t st, const int *list = nullptr) {
  launch_gather_slots_<T, false>(cptr, cidx, jbuf, vals, nnz, sms, st, list, GatherRows{});
}

// R rows and CSR slots in one launch (ROWS prologue of k_gather_slots)
template <typename T>
void launch_gather_rows_slots(const GatherRows &rows, const unsigned *cptr, const unsigned *cidx, const T *jbuf,
                              T *vals, long long nnz, int sms, cudaStream_t st, const int *list = nullptr) {
  launch_gather_slots_<T, true>(cptr, cidx, jbuf, vals, nnz, sms, st, list, rows);
}

// residual entry r = sum of its element contributions in element order
// (with `list`, row list[i] for i < n)
__global__ void k_gather_rows(const unsigned *__restrict__ rptr, const unsigned *__restrict__ ridx,
                              const double *__restrict__ rbuf, double *__restrict__ R, long long n,
                              const int *__restrict__ list = nullptr) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long r = list ? (long long)list[i] : i;
    const unsigned b = rptr[r], e = rptr[r + 1];
    double acc = 0.0;
    for (unsigned k = b; k < e; k++) acc += rbuf[ridx[k]];
    R[r] = acc;
  }
}

// Tile gather: R (when R) and the CSR values of whole rows, each entry the
// sum of its element contributions in element order -- the order of
// k_gather_rows / k_gather_slots, so all give the same bits.  One warp per
// tile: consecutive rows whose incidences (element e, local row i; ranked
// in element order within a row) fit KT records.  The records of a tile are
// rank-major -- every row's rank-0 incidence, then every rank-1 incidence,
// ... -- each rank padded to whole passes of PG incidences, so a pass never
// holds two incidences of one row.  Record (16 bytes): first entry of the
// element-matrix row e,i in jbuf; offset of its column positions in gpos;
// its residual entry in rbuf (bits 0-25) and local values (26-31; 0 marks
// padding); the slot base of its row within the tile (bits 0-10), its row
// within the tile (11-15), its rank (16-20) and the first column position
// it introduces (21-28).  A row's columns are in order of first insertion,
// so a contribution at position p >= that first position is the first of
// its slot: it is stored, every later one added.  Tile (16 bytes): first
// row, first slot, slots, rows.  Two dependent loads per tile: the records,
// then every value, position and residual entry of the tile at once (lanes
// j of G-lane groups, PG incidences per pass).  The sums build in shared
// memory pass after pass (positions within one incidence are distinct, the
// incidences of a pass belong to different rows), so every slot receives
// its contributions in element order.
template <typename T, int G>
__global__ void __launch_bounds__(256, 3) k_gather_tiles(const uint4 *__restrict__ tmeta,
                                                         const uint4 *__restrict__ tinfo,
                                                         const unsigned char *__restrict__ gpos,
                                                         const double *__restrict__ rbuf, const T *__restrict__ jbuf,
                                                         double *__restrict__ R, T *__restrict__ vals, long long t0,
                                                         long long t1, int acc_stride) {
  constexpr int KT = G == 32 ? 16 : 32; // records per tile
  constexpr int PG = 32 / G;            // incidences per pass
  constexpr int NP = KT / PG;           // passes
  extern __shared__ __align__(16) unsigned char g_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane / G, j = lane % G;
  double *racc = reinterpret_cast<double *>(g_smem) + warp * 32;
  T *acc = reinterpret_cast<T *>(g_smem + (blockDim.x >> 5) * 32 * sizeof(double)) + (size_t)warp * acc_stride;
  const long long step = (long long)gridDim.x * (blockDim.x >> 5);
  for (long long t = t0 + (long long)blockIdx.x * (blockDim.x >> 5) + warp; t < t1; t += step) {
    uint4 m = make_uint4(0u, 0u, 0u, 0u);
    if (lane < KT) m = tmeta[(size_t)t * KT + lane];
    const uint4 ti = tinfo[t];
    const bool live = (m.z >> 26) != 0;
    double rv = 0.0;
    if (R && live) rv = rbuf[m.z & 0x3FFFFFFu];
    T v[NP];
    unsigned sq[NP]; // accumulator slot | first << 16, or ~0u: nothing to add
#pragma unroll
    for (int q = 0; q < NP; q++) {
      const int i = q * PG + sub;
      const unsigned jr = __shfl_sync(0xffffffffu, m.x, i), go = __shfl_sync(0xffffffffu, m.y, i);
      const unsigned nl = __shfl_sync(0xffffffffu, m.z, i) >> 26, w = __shfl_sync(0xffffffffu, m.w, i);
      v[q] = (T)0;
      sq[q] = ~0u;
      if ((unsigned)j < nl) {
        const unsigned pos = gpos[go + j];
        v[q] = jbuf[(size_t)jr + j];
        if (pos != 0xFFu) sq[q] = ((w & 0x7FFu) + pos) | ((pos >= ((w >> 21) & 0xFFu)) ? (1u << 16) : 0u);
      }
    }
#pragma unroll
    for (int q = 0; q < NP; q++) {
      if (sq[q] != ~0u) {
        const unsigned s = sq[q] & 0xFFFFu;
        acc[s] = (sq[q] >> 16) ? v[q] : acc[s] + v[q];
      }
      __syncwarp();
    }
    if (R) {
      // each row's residual entries in rank order, from 0.0
      racc[lane] = 0.0;
      unsigned rk = live ? (m.w >> 16) & 31u : 0u;
#pragma unroll
      for (int o = 16; o; o >>= 1) rk = max(rk, __shfl_xor_sync(0xffffffffu, rk, o));
      __syncwarp();
      for (unsigned r = 0; r <= rk; r++) {
        if (live && ((m.w >> 16) & 31u) == r) racc[(m.w >> 11) & 31u] += rv;
        __syncwarp();
      }
      if (lane < (int)ti.w) R[ti.x + lane] = racc[lane];
    }
    const int ns = (int)ti.z;
    for (int s = lane; s < ns; s += 32) vals[ti.y + s] = acc[s];
    __syncwarp();
  }
}

// hanging values: values[slot] = sum_m w_m values[master_m]
__global__ void k_hang_interp(const long long *__restrict__ slot, const long long *__restrict__ ptr,
                              const long long *__restrict__ master, const double *__restrict__ w,
                              double *__restrict__ values, long long n) {
  for (long long h = blockIdx.x * (long long)blockDim.x + threadIdx.x; h < n; h += (long long)gridDim.x * blockDim.x) {
    double v = 0.0;
    for (long long m = ptr[h]; m < ptr[h + 1]; m++) v += w[m] * values[master[m]];
    values[slot[h]] = v;
  }
}

// weighted scatter (meshes with hanging values): the same fixed order, each
// contribution times its weight
template <typename T>
__global__ void k_gather_slots_w(const unsigned *__restrict__ cptr, const unsigned *__restrict__ cidx,
                                 const double *__restrict__ cw, const T *__restrict__ jbuf, T *__restrict__ out,
                                 long long nnz) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < nnz;
       s += (long long)gridDim.x * blockDim.x) {
    const unsigned b = cptr[s], e = cptr[s + 1];
    T acc = (T)0;
    for (unsigned k = b; k < e; k++) acc += (T)cw[k] * jbuf[cidx[k]];
    out[s] = acc;
  }
}

__global__ void k_gather_rows_w(const unsigned *__restrict__ rptr, const unsigned *__restrict__ ridx,
                                const double *__restrict__ rw, const double *__restrict__ rbuf, double *__restrict__ R,
                                long long n) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n;
       r += (long long)gridDim.x * blockDim.x) {
    const unsigned b = rptr[r], e = rptr[r + 1];
    double acc = 0.0;
    for (unsigned k = b; k < e; k++) acc += rw[k] * rbuf[ridx[k]];
    R[r] = acc;
  }
}

// ---------------------------------------------------------------------------
// oomph's zero filter (Problem::Numerical_zero_for_sparse_assembly,
// problem.cc:110, 5520-5560): an element entry with |J_e(i,j)| <= thr is not
// inserted, so a slot holds the sum of its surviving contributions, a row's
// columns come in the order of their first surviving insertion, and a slot
// with none is absent.  The contributions of a slot are numbered in
// (domain, element, local i, local j) order, the reference's insertion
// order, so within a row the index of a slot's first surviving contribution
// orders the slots as the reference inserts them.
// ---------------------------------------------------------------------------
#define FE_ZF_DEAD 0xffffffffu

template <typename T>
__global__ void k_gather_slots_zf(const unsigned *__restrict__ cptr, const unsigned *__restrict__ cidx,
                                  const T *__restrict__ jbuf, T *__restrict__ vals, unsigned *__restrict__ key,
                                  long long nnz, double thr) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < nnz;
       s += (long long)gridDim.x * blockDim.x) {
    const unsigned b = cptr[s], e = cptr[s + 1];
    T acc = (T)0;
    unsigned k = FE_ZF_DEAD;
    for (unsigned c = b; c < e; c++) {
      const unsigned at = cidx[c];
      const T v = jbuf[at];
      if (fabs((double)v) > thr) {   // NaN fails the test: dropped, as in the reference
        acc = (k == FE_ZF_DEAD) ? v : acc + v;
        if (k == FE_ZF_DEAD) k = at;
      }
    }
    vals[s] = acc;
    key[s] = k;
  }
}

// one warp per row: the rank of each surviving slot among the row's
// surviving slots (by first insertion), -1 for a dropped slot, and the
// row's surviving count
__global__ void k_zf_rank(const int *__restrict__ rowptr, const unsigned *__restrict__ key, int *__restrict__ rank,
                          int *__restrict__ rowcnt, long long n) {
  const int lane = threadIdx.x & 31;
  const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
    const int b = rowptr[r], e = rowptr[r + 1];
    int live = 0;
    for (int t = b + lane; t < e; t += 32) {
      const unsigned kt = key[t];
      int rk = -1;
      if (kt != FE_ZF_DEAD) {
        rk = 0;
        for (int u = b; u < e; u++) rk += key[u] < kt;
        live++;
      }
      rank[t] = rk;
    }
    for (int o = 16; o; o >>= 1) live += __shfl_xor_sync(0xffffffffu, live, o);
    if (lane == 0) rowcnt[r] = live;
  }
}

// one warp per row: surviving slots to their filtered positions
template <typename T>
__global__ void k_zf_scatter(const int *__restrict__ rowptr, const int *__restrict__ rank,
                             const int *__restrict__ rowptr_zf, const int *__restrict__ colidx,
                             const T *__restrict__ vals_st, int *__restrict__ colidx_zf, T *__restrict__ vals_zf,
                             long long n) {
  const int lane = threadIdx.x & 31;
  const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += warps) {
    const int b = rowptr[r], e = rowptr[r + 1], o = rowptr_zf[r];
    for (int t = b + lane; t < e; t += 32) {
      const int rk = rank[t];
      if (rk >= 0) {
        colidx_zf[o + rk] = colidx[t];
        vals_zf[o + rk] = vals_st[t];
      }
    }
  }
}

// exclusive scan of cnt[0..n) into out[0..n) with out[n] = the total, in
// three launches: block scans with block totals, a scan of the totals (one
// block, in chunks), the block offsets added
#define FE_SCAN_THREADS 1024
#define FE_SCAN_ITEMS 4

__device__ __forceinline__ int block_inclusive_scan(int v, int *sh) {
  const int t = threadIdx.x;
  sh[t] = v;
  __syncthreads();
  for (int off = 1; off < FE_SCAN_THREADS; off <<= 1) {
    const int x = t >= off ? sh[t - off] : 0;
    __syncthreads();
    sh[t] += x;
    __syncthreads();
  }
  const int r = sh[t];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(FE_SCAN_THREADS) k_scan_blocks(const int *__restrict__ cnt, int *__restrict__ out,
                                                                 int *__restrict__ bsum, long long n) {
  __shared__ int sh[FE_SCAN_THREADS];
  const long long base = ((long long)blockIdx.x * FE_SCAN_THREADS + threadIdx.x) * FE_SCAN_ITEMS;
  int v[FE_SCAN_ITEMS], tot = 0;
  for (int i = 0; i < FE_SCAN_ITEMS; i++) {
    v[i] = base + i < n ? cnt[base + i] : 0;
    tot += v[i];
  }
  const int incl = block_inclusive_scan(tot, sh);
  int run = incl - tot;
  for (int i = 0; i < FE_SCAN_ITEMS; i++) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
  if (threadIdx.x == FE_SCAN_THREADS - 1) bsum[blockIdx.x] = incl;
}

__global__ void __launch_bounds__(FE_SCAN_THREADS) k_scan_totals(int *__restrict__ bsum, long long nb,
                                                                 int *__restrict__ total) {
  __shared__ int sh[FE_SCAN_THREADS];
  int carry = 0;
  for (long long c0 = 0; c0 < nb; c0 += FE_SCAN_THREADS) {
    const long long i = c0 + threadIdx.x;
    const int v = i < nb ? bsum[i] : 0;
    const int incl = block_inclusive_scan(v, sh);
    if (i < nb) bsum[i] = carry + incl - v;
    sh[threadIdx.x] = incl;
    __syncthreads();
    carry += sh[FE_SCAN_THREADS - 1];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(int *__restrict__ out, const int *__restrict__ bsum, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] += bsum[i / (FE_SCAN_THREADS * FE_SCAN_ITEMS)];
}

// max |R| with NaN -> inf; one block per chunk, then a single finishing block
__device__ __forceinline__ double absnan(double v) { return (v != v) ? __longlong_as_double(0x7ff0000000000000LL) : fabs(v); }

__global__ void k_absmax_partial(const double *__restrict__ R, long long n, double *__restrict__ part) {
  __shared__ double sm[32];
  double m = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    m = fmax(m, absnan(R[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) part[blockIdx.x] = m;
  }
}

__global__ void k_dof_update(double *__restrict__ x, const double *__restrict__ dx, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    x[i] -= dx[i];
}

// y = A x for a CSR matrix (FP64 or FP32 values, FP64 vectors): one warp
// per row, lanes stride the row, a fixed shuffle tree sums them
// (deterministic).  The Krylov solver of the device Newton path calls it.
// fe_widen: exact FP32 -> FP64 on the integer pipe (fe_df64.cuh)

// y = A x with L lanes per row.  GB300 issues FP64 at ~1/64 of the FP32
// rate, so the kernel is shaped to spend one FMA per stored entry and as
// little else as possible on the FP64 pipe: L = 4 lanes per row (a lane
// group's load of 4 consecutive entries fills a 32-byte sector for FP64
// values) accumulate with FMAs into two partial sums, and only log2(L) = 2
// adds per lane fold the group (a 32-lane group would spend 5 adds on every
// lane for every row, more than the row's own FMAs).  The matrix streams
// through once (evict-first loads), x stays in L2; four entries per lane
// are loaded before they are used.  Rows are assigned to lane groups in a
// grid-stride loop; a group's lanes share the row, so the shuffle mask is
// the group's own lanes.  With bstate, only the rows of diagonal blocks (of
// nb rows) whose state word is `want` are computed (the batched solver skips
// blocks that stopped).  The summation order depends on the row alone.
template <typename T, int L>
__global__ void __launch_bounds__(256) k_csr_spmv(const int *__restrict__ rowptr, const int *__restrict__ colidx,
                                                  const T *__restrict__ vals, const double *__restrict__ x,
                                                  double *__restrict__ y, long long n,
                                                  const int *__restrict__ bstate = nullptr, int want = 0,
                                                  long long nb = 1) {
  const int sub = threadIdx.x & (L - 1);
  const unsigned gmask = L == 32 ? 0xffffffffu : (((1u << L) - 1u) << ((threadIdx.x & 31) & ~(L - 1)));
  const long long ng = ((long long)gridDim.x * blockDim.x) / L;
  for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / L; r < n; r += ng) {
    if (bstate && bstate[r / nb] != want) continue;
    const int e = rowptr[r + 1];
    int k = rowptr[r] + sub;
    double a0 = 0.0, a1 = 0.0;
    for (; k + 3 * L < e; k += 4 * L) {
      const T v0 = __ldcs(vals + k), v1 = __ldcs(vals + k + L), v2 = __ldcs(vals + k + 2 * L),
              v3 = __ldcs(vals + k + 3 * L);
      const int c0 = __ldcs(colidx + k), c1 = __ldcs(colidx + k + L), c2 = __ldcs(colidx + k + 2 * L),
                c3 = __ldcs(colidx + k + 3 * L);
      const double x0 = x[c0], x1 = x[c1], x2 = x[c2], x3 = x[c3];
      a0 = fma(fe_widen(v0), x0, a0);
      a1 = fma(fe_widen(v1), x1, a1);
      a0 = fma(fe_widen(v2), x2, a0);
      a1 = fma(fe_widen(v3), x3, a1);
    }
    for (; k < e; k += L) a0 = fma(fe_widen(__ldcs(vals + k)), x[__ldcs(colidx + k)], a0);
    double acc = a0 + a1;
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(gmask, acc, o);
    if (sub == 0) y[r] = acc;
  }
}

// y = z + sc * w o (b - A x), each of z, b, w optional (0, 0, 1 when null):
// the updates of a multigrid cycle in one pass over the matrix -- a damped
// Jacobi step (z = x, w = 1/diag, sc = omega), a residual (z = w = null,
// sc = 1), a prolongation-and-add (b = w = null, z = the iterate, sc = -1,
// A = P).  The same 4-lane row groups and summation order as k_csr_spmv.
// T = float: the FP32 copy of the multigrid cycle (a preconditioner needs no
// FP64 accuracy; on GB300 the FP64 pipe bounds the FP64 variant).
template <int L, typename T>
__global__ void __launch_bounds__(256) k_csr_update(const int *__restrict__ rowptr, const int *__restrict__ colidx,
                                                    const T *__restrict__ vals, const T *__restrict__ x,
                                                    const T *__restrict__ b, const T *__restrict__ z,
                                                    const T *__restrict__ w, T sc, T *__restrict__ y, long long n) {
  const int sub = threadIdx.x & (L - 1);
  const unsigned gmask = L == 32 ? 0xffffffffu : (((1u << L) - 1u) << ((threadIdx.x & 31) & ~(L - 1)));
  const long long ng = ((long long)gridDim.x * blockDim.x) / L;
  for (long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / L; r < n; r += ng) {
    const int e = rowptr[r + 1];
    int k = rowptr[r] + sub;
    T a0 = (T)0, a1 = (T)0;
    for (; k + 3 * L < e; k += 4 * L) {
      a0 = fma(__ldcs(vals + k), x[__ldcs(colidx + k)], a0);
      a1 = fma(__ldcs(vals + k + L), x[__ldcs(colidx + k + L)], a1);
      a0 = fma(__ldcs(vals + k + 2 * L), x[__ldcs(colidx + k + 2 * L)], a0);
      a1 = fma(__ldcs(vals + k + 3 * L), x[__ldcs(colidx + k + 3 * L)], a1);
    }
    for (; k < e; k += L) a0 = fma(__ldcs(vals + k), x[__ldcs(colidx + k)], a0);
    T acc = a0 + a1;
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(gmask, acc, o);
    if (sub == 0) {
      const T br = b ? b[r] : (T)0, wr = w ? w[r] : (T)1, zr = z ? z[r] : (T)0;
      y[r] = fma(sc * wr, br - acc, zr);
    }
  }
}

template <typename T>
__global__ void k_csr_diagonal(const int *__restrict__ rowptr, const int *__restrict__ colidx,
                               const T *__restrict__ vals, double *__restrict__ diag, long long n) {
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x) {
    double v = 0.0;
    for (int k = rowptr[r]; k < rowptr[r + 1]; k++)
      if (colidx[k] == r) v += (double)vals[k];
    diag[r] = v;
  }
}

int grid_for(long long n, int threads, int sms) {
  long long g = (n + threads - 1) / threads;
  long long cap = (long long)sms * 16;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

int sm_count_cached();

// y = A x (rows of blocks whose state word is `want` only, with bstate):
// 4 lanes per row (32 for rows averaging over 128 entries), so the
// summation order depends only on the row and that choice.
void launch_csr_spmv(const int *rowptr, const int *colidx, const void *vals, int prec, const double *x, double *y,
                     long long n, long long nnz, const int *bstate, int want, long long nb, cudaStream_t st) {
  const int L = (double)nnz > 128.0 * (double)n ? 32 : 4;
  const int g = grid_for(n * L, 256, sm_count_cached());
#define FE_SPMV_LAUNCH(T)                                                                                      \
  if (L == 4)                                                                                                  \
    k_csr_spmv<T, 4><<<g, 256, 0, st>>>(rowptr, colidx, (const T *)vals, x, y, n, bstate, want, nb);           \
  else                                                                                                         \
    k_csr_spmv<T, 32><<<g, 256, 0, st>>>(rowptr, colidx, (const T *)vals, x, y, n, bstate, want, nb);
  if (prec == FE_JAC_F64) {
    FE_SPMV_LAUNCH(double)
  } else {
    FE_SPMV_LAUNCH(float)
  }
#undef FE_SPMV_LAUNCH
}

// ---------------------------------------------------------------------------
// JIT
// ---------------------------------------------------------------------------
uint64_t fnv1a(const std::string &s) {
  uint64_t h = 1469598103934665603ULL;
  for (unsigned char c : s) {
    h ^= c;
    h *= 1099511628211ULL;
  }
  return h;
}

bool read_file(const std::string &path, std::string &out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::ostringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return true;
}

int ensure_context() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return fail(FE_ERR_NOGPU, "no CUDA device: %s", cudaGetErrorString(e));
  CUDA_TRY(cudaFree(0)); // creates / binds the primary context
  return FE_OK;
}

int sm_count_cached() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (!sms) sms = 1;
  }
  return sms;
}

} // namespace

// A loaded element kernel.  The runtime's library-management API
// (cudaLibraryLoadData / cudaLibraryGetKernel) is used instead of the driver
// API so that the library links only against cudart and nvrtc.
struct fe_code {
  cudaLibrary_t lib = nullptr;
  cudaKernel_t func = nullptr;
  std::string name;
  ~fe_code() {
    if (lib) cudaLibraryUnload(lib);
  }
};

struct Domain {
  fe_code_t *code = nullptr;
  int nnode = 0, nlocal = 0;
  long long n_elem = 0;
  int epb = 1, threads = 128, smem = 0;
  long long replica_elems = 0;
  DevBuf conn, tables, rbuf, jbuf;
  long long jbase = 0; // flat offset of this domain's entries in the global contribution space
  long long rbase = 0;
  std::vector<int32_t> local_node, local_val;
  // tensor-core contraction of the Jacobian (fe_problem_set_tensor_contraction)
  bool tc = false;
  FeTcArgs tca;
  DevBuf tc_dhat, tc_phi, tc_bhi, tc_blo;
};

struct fe_problem {
  int dim = 0, nval = 0, jac_prec = FE_JAC_F64;
  long long n_nodes = 0, n_dof = 0, nnz = 0;
  int n_params = 0, params_stride = 0, n_hist = 0, fused = 0, dparam = 0;
  int fused_grid_cap = 0; // resident blocks of the fused kernel (persistent launch)
  int persistent = 0;
  std::vector<Domain> domains;
  DevBuf x, values, eqn, params, status, hist, x0, dir;
  long long n_hang = 0;
  DevBuf hang_slot, hang_ptr, hang_master, hang_weight, cw, rw; // weighted scatter when n_hang > 0
  DevBuf rowptr, colidx, cptr, cidx, rptr, ridx;
  // tile gather (k_gather_tiles): positions, records, tiles; lanes per
  // incidence, accumulator stride; gather_mode FE_GATHER_TILES selects it
  DevBuf gpos, tmeta, tinfo;
  bool g_ok = false;
  int g_G = 0, g_acc = 0, gather_mode = 0;
  long long g_ntiles = 0;
  DevBuf partial;
  // zero-filtered assembly (FE_ASSEMBLE_ZERO_FILTER): threshold, structural
  // values, per-slot keys and ranks, per-row counts, the filtered pattern
  double zf_thr = 0.0;
  bool zf_done = false;
  DevBuf zf_vals, zf_key, zf_rank, zf_cnt, zf_rowptr, zf_colidx, zf_bsum;
  // the domain buffers are one allocation per kind, addressed by offsets:
  DevBuf jbuf_all, rbuf_all;
  std::vector<int32_t> h_rowptr, h_colidx;
  // stage timing (tracing): events recorded around the stages of fe_assemble
  bool timing = false;
  std::vector<std::vector<cudaEvent_t>> pending; // per call: 6 events
  double stage_ms[5] = {0, 0, 0, 0, 0};
  long long stage_calls = 0;
  // one recorded assembly (fe_problem_graph_capture), replayed by fe_problem_graph_launch
  cudaGraphExec_t graph = nullptr;
  // pipelined host-buffer assembly (fe_assemble_pipelined): the last element
  // touching each row (single-domain problems), the chunk plan, device
  // staging buffers, a copy stream and one event per chunk
  std::vector<int32_t> row_last;
  int pipe_chunks = 0, pipe_requested = 0;
  std::vector<long long> pipe_elem;
  std::vector<std::vector<std::pair<long long, long long>>> pipe_runs; // per chunk: row ranges it completes
  // per chunk, the rows and the CSR slots it completes as index lists (one
  // gather launch each), at pipe_row_off[k] / pipe_slot_off[k]
  DevBuf pipe_rowlist, pipe_slotlist;
  std::vector<long long> pipe_row_off, pipe_slot_off;
  DevBuf pipe_dofs, pipe_R, pipe_J;
  cudaStream_t pipe_copy = nullptr;
  // the gathers run on a stream of their own: chunk k's gather overlaps
  // chunk k+1's element kernel (memory-bound beside compute-bound work)
  cudaStream_t pipe_gather = nullptr;
  // the element chunks alternate between pipe_nes streams (1 or 2; 0:
  // automatic): chunk k+1 may start while chunk k's last blocks drain (they
  // write disjoint element buffers)
  cudaStream_t pipe_es[2] = {nullptr, nullptr};
  int pipe_nes = 0;
  std::vector<cudaEvent_t> pipe_ev;  // per chunk: its gathers done (+1: all copies done)
  std::vector<cudaEvent_t> pipe_eev; // per chunk: its element kernel done (+1: all gathers done)
  // with stage timing: the last pipelined call's timeline (start; per chunk
  // the end of its element kernel, of its gathers and of its copies)
  std::vector<cudaEvent_t> pipe_tev;
  int pipe_timed = 0; // chunks of the recorded timeline (0: none)
  void pipe_release() {
    for (auto e : pipe_ev) cudaEventDestroy(e);
    pipe_ev.clear();
    for (auto e : pipe_eev) cudaEventDestroy(e);
    pipe_eev.clear();
    if (pipe_gather) cudaStreamDestroy(pipe_gather);
    pipe_gather = nullptr;
    for (auto &e : pipe_es) {
      if (e) cudaStreamDestroy(e);
      e = nullptr;
    }
    for (auto e : pipe_tev) cudaEventDestroy(e);
    pipe_tev.clear();
    pipe_timed = 0;
    if (pipe_copy) cudaStreamDestroy(pipe_copy);
    pipe_copy = nullptr;
    pipe_chunks = 0;
    pipe_requested = 0;
  }
  ~fe_problem() {
    for (auto &v : pending)
      for (auto e : v) cudaEventDestroy(e);
    if (graph) cudaGraphExecDestroy(graph);
    pipe_release();
  }
};

// ---------------------------------------------------------------------------
// CSR pattern in the reference's insertion order + contribution lists
// ---------------------------------------------------------------------------
namespace {

struct Incident {
  int dom;
  long long e;
  int i;
  double w; // weight of the row's master (1 without hanging nodes)
};

// Host description of the element blocks the pattern is built from.
struct PatDomain {
  const int32_t *conn;
  int nnode, nlocal;
  long long n_elem;
  const int32_t *local_node, *local_val;
  long long jbase, rbase; // offsets in the element-matrix / element-residual buffers
};

struct PatternOut {
  std::vector<int32_t> rowptr, colidx;
  std::vector<long long> cptr; // [nnz+1] per-slot contribution ranges
  std::vector<unsigned> cidx;  // element-matrix entry of each contribution
  std::vector<long long> rptr; // [n_dof+1] per-row residual contributions
  std::vector<unsigned> ridx;
  std::vector<double> cw, rw;  // contribution weights (hanging nodes), empty if all 1
  // tile gather (k_gather_tiles): column positions of every (incidence,
  // local value) (0xFF: pinned), the tiles' records and descriptors (4 u32
  // each), lanes per incidence, records per tile, the most slots of a tile
  std::vector<unsigned char> gpos;
  std::vector<uint32_t> tmeta, tinfo;
  int gG = 0, gKT = 0;
  long long gacc = 0;
  bool gok = false;
};

// Hanging values (oomph's HangInfo, nodes.h; constrained values have no
// equation): slot = node * nval + value, its masters and weights.
struct HangMap {
  std::vector<long long> slot_of;             // sorted hanging slots
  const int64_t *ptr = nullptr, *master = nullptr;
  const double *weight = nullptr;
  long long find(long long slot) const {
    auto it = std::lower_bound(slot_of.begin(), slot_of.end(), slot);
    return (it != slot_of.end() && *it == slot) ? (long long)(it - slot_of.begin()) : -1;
  }
};

// The CSR pattern of Problem::sparse_assemble_row_or_column_compressed_with_
// vectors_of_pairs (problem.cc:5459-5660) with every structural coupling kept:
// row r lists, in order of first insertion over (element, local equation i,
// local equation j), the columns of the elements that contain equation r.
// An element's local equations are oomph's: its own values' equations in
// local order, then -- with hanging values -- the equations of their masters
// that are not values of the element, in order of first appearance over
// (hanging value, master) (RefineableElement::assign_hanging_local_eqn_numbers,
// refineable_elements.cc:312-450).  Rows are built independently (in
// parallel): the incidence of each equation (its elements, in element order,
// with the local index) is gathered first, then each row walks its incidence
// with a marker array for O(1) membership.
struct PatternBuilder {
  long long n_dof;
  int nval;
  const int32_t *eqn;
  const std::vector<PatDomain> *doms;
  const HangMap *hang = nullptr;
  std::vector<long long> inc_ptr;
  std::vector<Incident> inc;

  // the element-residual entry of incidence k
  long long ridx_of(long long k) const {
    const Incident &I = inc[k];
    const PatDomain &d = (*doms)[I.dom];
    return d.rbase + I.e * d.nlocal + I.i;
  }

  // the equations (and weights) a local value of an element stands for: its
  // own equation, or the equations of its masters if it hangs
  template <typename F> void expand(const PatDomain &d, long long e, int k, F &&f) const {
    const long long node = d.conn[e * d.nnode + d.local_node[k]];
    const long long slot = node * nval + d.local_val[k];
    if (hang) {
      const long long h = hang->find(slot);
      if (h >= 0) {
        for (long long m = hang->ptr[h]; m < hang->ptr[h + 1]; m++) {
          const int32_t c = eqn[hang->master[m]];
          if (c >= 0) f(c, hang->weight[m]);
        }
        return;
      }
    }
    const int32_t c = eqn[slot];
    if (c >= 0) f(c, 1.0);
  }

  // the element's local equations in oomph's order (see above)
  template <typename F> void element_dofs(const PatDomain &d, long long e, F &&f) const {
    const bool hanging = hang && !hang->slot_of.empty();
    for (int k = 0; k < d.nlocal; k++) {
      const long long slot = (long long)d.conn[e * d.nnode + d.local_node[k]] * nval + d.local_val[k];
      if (hanging && hang->find(slot) >= 0) continue;
      if (eqn[slot] >= 0) f(eqn[slot]);
    }
    if (!hanging) return;
    // (a master met twice is passed twice: the caller keeps the first)
    for (int k = 0; k < d.nlocal; k++) {
      const long long slot = (long long)d.conn[e * d.nnode + d.local_node[k]] * nval + d.local_val[k];
      const long long h = hang->find(slot);
      if (h < 0) continue;
      for (long long m = hang->ptr[h]; m < hang->ptr[h + 1]; m++) {
        const long long ms = hang->master[m];
        bool own = false;   // a value of this element: numbered in the first pass (or pinned)
        for (int k2 = 0; k2 < d.nlocal && !own; k2++)
          own = (long long)d.conn[e * d.nnode + d.local_node[k2]] * nval + d.local_val[k2] == ms;
        const int32_t c = eqn[ms];
        if (!own && c >= 0) f(c);
      }
    }
  }

  void build_incidence() {
    const long long n = n_dof;
    std::vector<long long> cnt(n + 1, 0);
    for (const PatDomain &d : *doms)
      for (long long e = 0; e < d.n_elem; e++)
        for (int i = 0; i < d.nlocal; i++) expand(d, e, i, [&](int32_t r, double) { cnt[r + 1]++; });
    for (long long r = 0; r < n; r++) cnt[r + 1] += cnt[r];
    inc_ptr = cnt;
    inc.resize(cnt[n]);
    std::vector<long long> pos(cnt.begin(), cnt.end() - 1);
    for (size_t di = 0; di < doms->size(); di++) {
      const PatDomain &d = (*doms)[di];
      for (long long e = 0; e < d.n_elem; e++)
        for (int i = 0; i < d.nlocal; i++)
          expand(d, e, i, [&](int32_t r, double w) { inc[pos[r]++] = Incident{(int)di, e, i, w}; });
    }
  }

  void row(long long r, std::vector<int32_t> &marker, std::vector<int32_t> &cols,
           std::vector<long long> &slot_cnt, bool fill, int32_t *colidx_out, long long *cptr_out,
           unsigned *cidx_out, double *cw_out, long long cbase, long long *row_len, long long *row_contrib) const {
    cols.clear();
    slot_cnt.clear();
    long long ncontrib = 0;
    for (long long k = inc_ptr[r]; k < inc_ptr[r + 1]; k++) {
      const Incident &I = inc[k];
      const PatDomain &d = (*doms)[I.dom];
      // columns in the element's local-equation order (new ones appended)
      element_dofs(d, I.e, [&](int32_t c) {
        if (marker[c] < 0) {
          marker[c] = (int32_t)cols.size();
          cols.push_back(c);
          slot_cnt.push_back(0);
        }
      });
      // contributions of this incidence: every (local j, master) of the element
      for (int j = 0; j < d.nlocal; j++)
        expand(d, I.e, j, [&](int32_t c, double) {
          slot_cnt[marker[c]]++;
          ncontrib++;
        });
    }
    *row_len = (long long)cols.size();
    *row_contrib = ncontrib;
    if (fill) {
      long long acc = cbase;
      for (size_t s = 0; s < cols.size(); s++) {
        colidx_out[s] = cols[s];
        cptr_out[s] = acc;
        acc += slot_cnt[s];
      }
      std::vector<long long> wpos(cols.size());
      for (size_t s = 0; s < cols.size(); s++) wpos[s] = cptr_out[s];
      for (long long k = inc_ptr[r]; k < inc_ptr[r + 1]; k++) {
        const Incident &I = inc[k];
        const PatDomain &d = (*doms)[I.dom];
        const long long base = d.jbase + (I.e * d.nlocal + I.i) * (long long)d.nlocal;
        for (int j = 0; j < d.nlocal; j++)
          expand(d, I.e, j, [&](int32_t c, double w) {
            const long long at = wpos[marker[c]]++;
            cidx_out[at] = (unsigned)(base + j);
            if (cw_out) cw_out[at] = I.w * w;
          });
      }
    }
    for (int32_t c : cols) marker[c] = -1;
  }
};

// The tile gather's tables (k_gather_tiles) from the finished pattern.
// out.gok stays false, and the per-slot gather is used, where an element
// has more than 32 local values, a row more than 255 slots or more
// incidences than a tile holds, the tables more than 2^32 entries, or one
// incidence meets a column twice.
void build_tile_gather(const PatternBuilder &B, PatternOut &out, unsigned nthreads) {
  const long long n = B.n_dof, ninc = (long long)B.inc.size();
  out.gok = false;
  int maxnl = 1;
  for (const PatDomain &d : *B.doms) maxnl = std::max(maxnl, d.nlocal);
  long long maxrow = 0;
  for (long long r = 0; r < n; r++) maxrow = std::max(maxrow, (long long)(out.rowptr[r + 1] - out.rowptr[r]));
  if (maxnl > 32 || maxrow > 255) return;
  int G = 4;
  while (G < maxnl) G *= 2;
  const int KT = G == 32 ? 16 : 32;
  // accumulators of one warp: 8 warps x (32 residual + (704 | 1) FP64
  // slots) fit the 48 KB of dynamic shared memory a launch gets without
  // opting in
  const long long max_slots = 704;
  std::vector<long long> goff(ninc + 1, 0);
  for (long long k = 0; k < ninc; k++) goff[k + 1] = goff[k] + (*B.doms)[B.inc[k].dom].nlocal;
  if (goff[ninc] > 0xffffffffLL) return;
  std::vector<uint32_t> jrow(ninc);
  std::vector<unsigned char> cfirst(ninc);
  out.gpos.assign(goff[ninc], (unsigned char)0xFF);
  std::atomic<bool> bad{false};
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nthreads; t++) {
    th.emplace_back([&, t]() {
      std::vector<int32_t> marker(n > 0 ? n : 1, -1);
      std::vector<long long> stamp(256, -1);
      const long long lo = n * t / nthreads, hi = n * (t + 1) / nthreads;
      for (long long r = lo; r < hi; r++) {
        const int32_t s0 = out.rowptr[r], len = out.rowptr[r + 1] - s0;
        for (int32_t s = 0; s < len; s++) marker[out.colidx[s0 + s]] = s;
        int32_t seen = 0; // columns introduced by the row's incidences so far
        for (long long k = B.inc_ptr[r]; k < B.inc_ptr[r + 1]; k++) {
          const Incident &I = B.inc[k];
          const PatDomain &d = (*B.doms)[I.dom];
          const long long jr = d.jbase + (I.e * d.nlocal + I.i) * (long long)d.nlocal;
          if (jr + d.nlocal > 0xffffffffLL || B.ridx_of(k) >= (1LL << 26)) bad = true;
          jrow[k] = (uint32_t)jr;
          for (int j = 0; j < d.nlocal; j++) {
            int cnt = 0;
            int32_t pos = -1;
            B.expand(d, I.e, j, [&](int32_t c, double) {
              cnt++;
              pos = marker[c];
            });
            if (cnt == 0) continue; // pinned
            if (cnt > 1 || pos < 0 || stamp[pos] == k) {
              bad = true;
              continue;
            }
            stamp[pos] = k;
            out.gpos[goff[k] + j] = (unsigned char)pos;
          }
          // the columns this incidence introduces follow those of the
          // incidences before it (first-insertion order): cfirst, cfirst+1, ...
          int32_t nnew = 0, top = seen;
          for (int j = 0; j < d.nlocal; j++) {
            const unsigned char p = out.gpos[goff[k] + j];
            if (p == 0xFF || p < seen) continue;
            nnew++;
            top = std::max(top, (int32_t)p + 1);
          }
          if (top - seen != nnew) bad = true;
          cfirst[k] = (unsigned char)seen;
          seen = top;
        }
        for (int32_t s = 0; s < len; s++) marker[out.colidx[s0 + s]] = -1;
      }
    });
  }
  for (auto &x : th) x.join();
  if (bad) return;
  // tiles: consecutive rows while their records, rank-major with each rank
  // padded to whole passes, fit KT, their slots the accumulator and their
  // count a warp
  const int PG = 32 / G;
  out.tmeta.clear();
  out.tinfo.clear();
  long long gacc = 0;
  std::vector<long long> cnt(KT + 1), sbase;
  for (long long r = 0; r < n;) {
    const long long r0 = r;
    long long nsl = 0;
    std::fill(cnt.begin(), cnt.end(), 0);
    sbase.clear();
    while (r < n && r - r0 < 32) {
      const long long ki = B.inc_ptr[r + 1] - B.inc_ptr[r], si = out.rowptr[r + 1] - out.rowptr[r];
      if (ki * PG > KT || si > max_slots) return;
      long long padded = 0;
      for (int t = 0; t < KT; t++) padded += (cnt[t] + (t < ki) + PG - 1) / PG * PG;
      if (padded > KT || nsl + si > max_slots) break;
      for (long long t = 0; t < ki; t++) cnt[t]++;
      sbase.push_back(nsl);
      nsl += si;
      r++;
    }
    const size_t first = out.tmeta.size();
    for (int t = 0; t < KT && cnt[t]; t++) {
      long long emitted = 0;
      for (long long q = r0; q < r; q++) {
        if (B.inc_ptr[q + 1] - B.inc_ptr[q] <= t) continue;
        const long long k = B.inc_ptr[q] + t;
        const uint32_t nl = (uint32_t)(*B.doms)[B.inc[k].dom].nlocal;
        const uint32_t w = (uint32_t)sbase[q - r0] | ((uint32_t)(q - r0) << 11) | ((uint32_t)t << 16) |
                           ((uint32_t)cfirst[k] << 21);
        const uint32_t one[4] = {jrow[k], (uint32_t)goff[k], (uint32_t)B.ridx_of(k) | (nl << 26), w};
        out.tmeta.insert(out.tmeta.end(), one, one + 4);
        emitted++;
      }
      out.tmeta.resize(out.tmeta.size() + 4 * ((PG - emitted % PG) % PG), 0u);
    }
    out.tmeta.resize(first + 4 * (size_t)KT, 0u);
    const uint32_t info[4] = {(uint32_t)r0, (uint32_t)out.rowptr[r0], (uint32_t)nsl, (uint32_t)(r - r0)};
    out.tinfo.insert(out.tinfo.end(), info, info + 4);
    gacc = std::max(gacc, nsl);
  }
  out.gG = G;
  out.gKT = KT;
  out.gacc = gacc;
  out.gok = true;
}

int build_pattern_host(long long n_dof, int nval, const int32_t *eqn, const std::vector<PatDomain> &doms,
                       bool with_contributions, PatternOut &out, const HangMap *hang = nullptr) {
  PatternBuilder B;
  B.n_dof = n_dof;
  B.nval = nval;
  B.eqn = eqn;
  B.doms = &doms;
  B.hang = hang;
  const bool weighted = hang && !hang->slot_of.empty();
  B.build_incidence();
  const long long n = n_dof;
  unsigned nthreads = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  if (n < 4096) nthreads = 1;
  std::vector<long long> row_len(n), row_con(n);
  std::vector<long long> rp(n + 1, 0), cp(n + 1, 0);
  auto pass = [&](bool fill) {
    std::vector<std::thread> th;
    for (unsigned t = 0; t < nthreads; t++) {
      th.emplace_back([&, t]() {
        std::vector<int32_t> marker(n > 0 ? n : 1, -1), cols;
        std::vector<long long> slot_cnt;
        long long lo = n * t / nthreads, hi = n * (t + 1) / nthreads;
        for (long long r = lo; r < hi; r++) {
          long long rl, rc;
          if (!fill) {
            B.row(r, marker, cols, slot_cnt, false, nullptr, nullptr, nullptr, nullptr, 0, &rl, &rc);
            row_len[r] = rl;
            row_con[r] = rc;
          } else {
            long long o = rp[r];
            B.row(r, marker, cols, slot_cnt, with_contributions, out.colidx.data() + o,
                  with_contributions ? out.cptr.data() + o : nullptr,
                  with_contributions ? out.cidx.data() : nullptr,
                  (with_contributions && weighted) ? out.cw.data() : nullptr, cp[r], &rl, &rc);
            if (!with_contributions) {
              // columns only: recompute cols for this row
              for (size_t s = 0; s < cols.size(); s++) out.colidx[o + s] = cols[s];
            }
          }
        }
      });
    }
    for (auto &x : th) x.join();
  };
  pass(false);
  for (long long r = 0; r < n; r++) {
    rp[r + 1] = rp[r] + row_len[r];
    cp[r + 1] = cp[r] + row_con[r];
  }
  const long long nnz = rp[n];
  if (nnz > 0x7fffffffLL) return fail(FE_ERR_ARG, "nnz %lld exceeds int32 CSR", nnz);
  out.colidx.assign(nnz, 0);
  if (with_contributions) {
    out.cptr.assign(nnz + 1, 0);
    out.cidx.assign(cp[n], 0);
    if (weighted) out.cw.assign(cp[n], 0.0);
  }
  pass(true);
  if (with_contributions) out.cptr[nnz] = cp[n];
  out.rowptr.resize(n + 1);
  for (long long r = 0; r <= n; r++) out.rowptr[r] = (int32_t)rp[r];
  if (with_contributions) {
    out.rptr.assign(B.inc_ptr.begin(), B.inc_ptr.end());
    out.ridx.resize(B.inc.size());
    for (size_t k = 0; k < B.inc.size(); k++) {
      const Incident &I = B.inc[k];
      const PatDomain &d = doms[I.dom];
      out.ridx[k] = (unsigned)(d.rbase + I.e * d.nlocal + I.i);
    }
    if (weighted) {
      out.rw.resize(B.inc.size());
      for (size_t k = 0; k < B.inc.size(); k++) out.rw[k] = B.inc[k].w;
    }
    if (!weighted) build_tile_gather(B, out, nthreads);
  }
  return FE_OK;
}

int build_pattern(fe_problem *P, const std::vector<const int32_t *> &conn_h, const int32_t *eqn_h,
                  const HangMap *hang) {
  std::vector<PatDomain> doms;
  for (size_t di = 0; di < P->domains.size(); di++) {
    const Domain &d = P->domains[di];
    doms.push_back(PatDomain{conn_h[di], d.nnode, d.nlocal, d.n_elem, d.local_node.data(), d.local_val.data(),
                             d.jbase, d.rbase});
  }
  PatternOut out;
  int rc = build_pattern_host(P->n_dof, P->nval, eqn_h, doms, true, out, hang);
  if (rc) return rc;
  if (!out.cw.empty()) {
    if ((rc = P->cw.upload(out.cw.data(), sizeof(double) * out.cw.size()))) return rc;
    if ((rc = P->rw.upload(out.rw.data(), sizeof(double) * out.rw.size()))) return rc;
  }
  const long long n = P->n_dof;
  const long long nnz = (long long)out.colidx.size();
  P->nnz = nnz;
  P->h_rowptr = out.rowptr;
  P->h_colidx = out.colidx;
  if ((rc = P->rowptr.upload(out.rowptr.data(), sizeof(int32_t) * (n + 1)))) return rc;
  if ((rc = P->colidx.upload(out.colidx.data(), sizeof(int32_t) * nnz))) return rc;
  // contribution ranges as u32 (the lists index the element buffers, whose
  // entries are counted in u32 as well)
  if (out.cptr[nnz] > 0xffffffffLL || out.rptr[n] > 0xffffffffLL)
    return fail(FE_ERR_ARG, "more than 2^32 element contributions");
  {
    std::vector<unsigned> c32(out.cptr.begin(), out.cptr.end()), r32(out.rptr.begin(), out.rptr.end());
    if ((rc = P->cptr.upload(c32.data(), sizeof(unsigned) * (nnz + 1)))) return rc;
    if ((rc = P->rptr.upload(r32.data(), sizeof(unsigned) * (n + 1)))) return rc;
  }
  if ((rc = P->cidx.upload(out.cidx.data(), sizeof(unsigned) * out.cidx.size()))) return rc;
  if ((rc = P->ridx.upload(out.ridx.data(), sizeof(unsigned) * out.ridx.size()))) return rc;
  P->g_ok = false;
  if (out.gok && !out.tinfo.empty() && !out.gpos.empty()) {
    P->g_G = out.gG;
    P->g_acc = (int)(out.gacc | 1);
    P->g_ntiles = (long long)out.tinfo.size() / 4;
    if ((rc = P->gpos.upload(out.gpos.data(), out.gpos.size()))) return rc;
    if ((rc = P->tmeta.upload(out.tmeta.data(), sizeof(uint32_t) * out.tmeta.size()))) return rc;
    if ((rc = P->tinfo.upload(out.tinfo.data(), sizeof(uint32_t) * out.tinfo.size()))) return rc;
    P->g_ok = true;
  }
  return FE_OK;
}

// checks the hanging values of a description and indexes them
int hang_map(const fe_problem_desc_t *desc, HangMap &h) {
  h.slot_of.clear();
  if (desc->n_hang <= 0) return FE_OK;
  if (!desc->hang_slot || !desc->hang_ptr || !desc->hang_master || !desc->hang_weight)
    return fail(FE_ERR_ARG, "hanging values: null arrays");
  const long long nslots = desc->n_nodes * desc->nval;
  h.slot_of.assign(desc->hang_slot, desc->hang_slot + desc->n_hang);
  for (long long k = 0; k < desc->n_hang; k++) {
    const long long s = h.slot_of[k];
    if (s < 0 || s >= nslots || (k > 0 && s <= h.slot_of[k - 1]))
      return fail(FE_ERR_ARG, "hanging values: slots must be sorted, unique and in range (entry %lld)", k);
    if (desc->eqn[s] >= 0) return fail(FE_ERR_ARG, "hanging value %lld has an equation number", s);
    if (desc->hang_ptr[k + 1] < desc->hang_ptr[k]) return fail(FE_ERR_ARG, "hanging values: bad hang_ptr");
  }
  if (desc->hang_ptr[0] != 0) return fail(FE_ERR_ARG, "hanging values: hang_ptr[0] != 0");
  h.ptr = desc->hang_ptr;
  h.master = desc->hang_master;
  h.weight = desc->hang_weight;
  for (long long m = 0; m < desc->hang_ptr[desc->n_hang]; m++) {
    const long long s = desc->hang_master[m];
    if (s < 0 || s >= nslots) return fail(FE_ERR_ARG, "hanging values: master %lld out of range", m);
    if (h.find(s) >= 0) return fail(FE_ERR_ARG, "hanging values: master slot %lld hangs itself", s);
    if (!(desc->hang_weight[m] == desc->hang_weight[m])) return fail(FE_ERR_ARG, "hanging values: NaN weight");
  }
  return FE_OK;
}

// validates the host parts of a problem description
int validate_desc(const fe_problem_desc_t *desc, bool need_code) {
  if (!desc) return fail(FE_ERR_ARG, "null problem description");
  if (desc->dim < 1 || desc->dim > 3 || desc->nval < 1 || desc->n_nodes < 0 || desc->n_dof < 0 ||
      desc->n_domains < 1 || !desc->domains || !desc->eqn)
    return fail(FE_ERR_ARG, "problem description: bad sizes");
  for (long long k = 0; k < desc->n_nodes * desc->nval; k++)
    if (desc->eqn[k] >= desc->n_dof || desc->eqn[k] < -1)
      return fail(FE_ERR_ARG, "eqn[%lld]=%d out of range", k, desc->eqn[k]);
  for (int di = 0; di < desc->n_domains; di++) {
    const fe_domain_desc_t &dd = desc->domains[di];
    if ((need_code && !dd.code) || dd.nnode_el < 1 || dd.nlocal < 1 || dd.n_elem < 0 ||
        (!dd.conn && dd.n_elem) || !dd.local_node || !dd.local_val)
      return fail(FE_ERR_ARG, "bad domain %d", di);
    for (long long k = 0; k < dd.n_elem * dd.nnode_el; k++)
      if (dd.conn[k] < 0 || dd.conn[k] >= desc->n_nodes)
        return fail(FE_ERR_ARG, "domain %d: conn[%lld]=%d out of range", di, k, dd.conn[k]);
    for (int k = 0; k < dd.nlocal; k++)
      if (dd.local_node[k] < 0 || dd.local_node[k] >= dd.nnode_el || dd.local_val[k] < 0 ||
          dd.local_val[k] >= desc->nval)
        return fail(FE_ERR_ARG, "domain %d: bad local layout at %d", di, k);
  }
  return FE_OK;
}

FeElemArgs domain_args(fe_problem *p, Domain &d, int flag) {
  FeElemArgs a;
  a.x = p->x.as<double>();
  a.conn = d.conn.as<int>();
  a.values = p->values.as<double>();
  a.params = p->params.as<double>();
  a.tables = d.tables.as<double>();
  a.rbuf = p->rbuf_all.as<double>() + d.rbase;
  if (p->jac_prec == FE_JAC_F64)
    a.jbuf = (void *)(p->jbuf_all.as<double>() + d.jbase);
  else
    a.jbuf = (void *)(p->jbuf_all.as<float>() + d.jbase);
  a.n_elem = d.n_elem;
  a.nval = p->nval;
  a.flag = flag;
  a.status = p->status.as<int>();
  a.replica_elems = d.replica_elems;
  a.params_stride = p->params_stride;
  a.hist = p->hist.as<double>();
  a.x0 = p->x0.p ? p->x0.as<double>() : p->x.as<double>();
  a.n_hist = p->n_hist;
  a.hist_stride = (long long)p->n_nodes * p->nval;
  a.aux = p->dparam;
  a.n_nodes = p->n_nodes;
  a.dir = p->dir.p ? p->dir.as<double>() : p->values.as<double>();
  a.dhat = d.tc ? d.tc_dhat.as<float>() : nullptr;
  return a;
}

// ---------------------------------------------------------------------------
// tensor-core contraction (fe_tc.cuh): tables and launch
// ---------------------------------------------------------------------------
// nearest TF32 (ties away from zero) of a float: the high part of the split
float tf32_round_host(float x) {
  uint32_t b;
  memcpy(&b, &x, 4);
  b = (b + 0x1000u) & 0xFFFFE000u;
  float r;
  memcpy(&r, &b, 4);
  return r;
}

// validates the description and fills the arguments: phi [nq][nc][n] (local
// order) becomes the staged table [nq][nc][32] and the B operand pieces in
// the shared-memory layout [kp/4][32][4]
int tc_setup(FeTcArgs &A, DevBuf &phi_d, DevBuf &bhi_d, DevBuf &blo_d, int n, int nq, int nc, const double *phi,
             int npair, const int32_t *pa, const int32_t *pb) {
  if (n < 1 || n > FE_TC_N || nq < 1 || nq > FE_TC_MAXQ || nc < 1 || nc > FE_TC_MAXC || npair < 1 ||
      npair > FE_TC_MAXP || !phi || !pa || !pb)
    return fail(FE_ERR_ARG, "tensor contraction: sizes out of range (n %d, nq %d, nc %d, npair %d)", n, nq, nc, npair);
  memset(&A, 0, sizeof(A));
  for (int p_ = 0; p_ < npair; p_++)
    if (pa[p_] < 0 || pa[p_] >= nc || pb[p_] < 0 || pb[p_] >= nc)
      return fail(FE_ERR_ARG, "tensor contraction: pair %d has components out of range", p_);
  // the active test components (those some pair tests with), each with its
  // pairs (Dhat index, trial component)
  int nact = 0;
  std::vector<int> act;
  for (int c = 0; c < nc; c++) {
    int nt = 0;
    for (int p_ = 0; p_ < npair; p_++)
      if (pa[p_] == c) {
        A.tp[nact][nt] = p_;
        A.tb[nact][nt] = pb[p_];
        nt++;
      }
    if (nt) {
      A.nterm[nact++] = nt;
      act.push_back(c);
    }
  }
  const int K = nq * nact, kp = (K + 7) / 8 * 8;
  if (kp > FE_TC_MAXK) return fail(FE_ERR_ARG, "tensor contraction: K = %d exceeds %d", K, FE_TC_MAXK);
  A.n = n;
  A.nq = nq;
  A.nc = nc;
  A.npair = npair;
  A.nact = nact;
  A.kp = kp;
  std::vector<float> ph((size_t)nq * nc * FE_TC_N, 0.0f), bhi((size_t)kp * FE_TC_N, 0.0f), blo(bhi.size(), 0.0f);
  for (int q = 0; q < nq; q++)
    for (int c = 0; c < nc; c++)
      for (int i = 0; i < n; i++) ph[((size_t)q * nc + c) * FE_TC_N + i] = (float)phi[((size_t)q * nc + c) * n + i];
  for (int k = 0; k < K; k++) {
    const int q = k / nact, c = act[k % nact];
    for (int i = 0; i < n; i++) {
      const double v = phi[((size_t)q * nc + c) * n + i];
      const float hi = tf32_round_host((float)v);
      const size_t at = (size_t)(k / 4) * (FE_TC_N * 4) + (size_t)i * 4 + (k % 4);
      bhi[at] = hi;
      blo[at] = (float)(v - (double)hi);
    }
  }
  int rc;
  if ((rc = phi_d.upload(ph.data(), sizeof(float) * ph.size())) || (rc = bhi_d.upload(bhi.data(), sizeof(float) * bhi.size())) ||
      (rc = blo_d.upload(blo.data(), sizeof(float) * blo.size())))
    return rc;
  A.phi = phi_d.as<float>();
  A.b_hi = bhi_d.as<float>();
  A.b_lo = blo_d.as<float>();
  const fe_tc::Plan pl = fe_tc::plan(kp, nq, npair, nc);
  if (pl.total > 227 * 1024) return fail(FE_ERR_ARG, "tensor contraction: %u bytes of shared memory", pl.total);
  CUDA_TRY(cudaFuncSetAttribute((const void *)k_tc_contract, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)pl.total));
  return FE_OK;
}

int tc_launch(const FeTcArgs &A, cudaStream_t st) {
  if (A.n_elem <= 0) return FE_OK;
  const long long tiles = (A.n_elem + FE_TC_EPT - 1) / FE_TC_EPT;
  const int grid = (int)std::min<long long>(tiles, sm_count_cached());
  const fe_tc::Plan pl = fe_tc::plan(A.kp, A.nq, A.npair, A.nc);
  k_tc_contract<<<grid, FE_TC_THREADS, pl.total, st>>>(A);
  CUDA_TRY(cudaGetLastError());
  return FE_OK;
}

// the tensor-core contraction of domain d over elements [e0, e1)
int tc_domain(fe_problem *p, Domain &d, long long e0, long long e1, cudaStream_t st) {
  FeTcArgs A = d.tca;
  A.dhat = d.tc_dhat.as<float>() + e0 * (long long)A.nq * A.npair;
  A.jbuf = p->jbuf_all.as<float>() + d.jbase + e0 * (long long)d.nlocal * d.nlocal;
  A.status = p->status.as<int>();
  A.n_elem = e1 - e0;
  return tc_launch(A, st);
}

// the tile gather is used for the Jacobian (and the residual with it) where
// it is asked for and its tables exist
bool tile_gather(const fe_problem *p) { return p->g_ok && p->gather_mode == FE_GATHER_TILES && !p->cw.p; }

// every tile: R when given, the CSR values
template <typename T>
int launch_tile_gather(const fe_problem *p, double *R, T *vals, cudaStream_t st) {
  if (p->g_ntiles <= 0) return FE_OK;
  const int warps = 8;
  const size_t smem = (size_t)warps * (32 * sizeof(double) + p->g_acc * sizeof(T));
  const long long need = (p->g_ntiles + warps - 1) / warps;
  const unsigned grid = (unsigned)std::max(1LL, std::min(need, 8LL * sm_count_cached()));
  const uint4 *tm = p->tmeta.as<uint4>(), *ti = p->tinfo.as<uint4>();
  const unsigned char *gp = p->gpos.as<unsigned char>();
  const double *rb = p->rbuf_all.as<double>();
  const T *jb = p->jbuf_all.as<T>();
  switch (p->g_G) {
  case 4: k_gather_tiles<T, 4><<<grid, 32 * warps, smem, st>>>(tm, ti, gp, rb, jb, R, vals, 0, p->g_ntiles, p->g_acc); break;
  case 8: k_gather_tiles<T, 8><<<grid, 32 * warps, smem, st>>>(tm, ti, gp, rb, jb, R, vals, 0, p->g_ntiles, p->g_acc); break;
  case 16: k_gather_tiles<T, 16><<<grid, 32 * warps, smem, st>>>(tm, ti, gp, rb, jb, R, vals, 0, p->g_ntiles, p->g_acc); break;
  case 32: k_gather_tiles<T, 32><<<grid, 32 * warps, smem, st>>>(tm, ti, gp, rb, jb, R, vals, 0, p->g_ntiles, p->g_acc); break;
  default: return fail(FE_ERR_STATE, "tile gather: no kernel for %d lanes", p->g_G);
  }
  CUDA_TRY(cudaGetLastError());
  return FE_OK;
}

int launch_elements(fe_problem *p, int flag, cudaStream_t st) {
  if (p->fused) {
    FeFusedArgs fa;
    memset(&fa, 0, sizeof(fa));
    int threads = 32, smem = 0, nb = 0, k = 0;
    for (Domain &d : p->domains) {
      fa.d[k] = domain_args(p, d, flag);
      fa.block_start[k] = nb;
      nb += (int)((d.n_elem + d.epb - 1) / d.epb);
      threads = std::max(threads, d.threads);
      smem = std::max(smem, d.smem);
      k++;
    }
    fa.block_start[k] = nb;
    fa.n_domains = k;
    if (nb == 0) return FE_OK;
    // persistent launch (optional): as many blocks as the SMs hold at once, the
    // kernel striding over the element blocks of all domains; otherwise one
    // block per element block (the stride loop then runs once)
    if (p->persistent && p->fused_grid_cap == 0) {
      int per_sm = 1;
      CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)p->domains[0].code->func, threads,
                                                             (size_t)smem));
      p->fused_grid_cap = std::max(1, per_sm) * sm_count_cached();
    }
    const int grid = p->persistent ? std::min(nb, p->fused_grid_cap) : nb;
    void *kp[] = {&fa};
    CUDA_TRY(cudaLaunchKernel((const void *)p->domains[0].code->func, dim3(grid), dim3(threads), kp, (size_t)smem, st));
    return FE_OK;
  }
  for (Domain &d : p->domains) {
    if (d.n_elem == 0) continue;
    FeElemArgs a = domain_args(p, d, flag);
    void *kp[] = {&a};
    unsigned grid = (unsigned)((d.n_elem + d.epb - 1) / d.epb);
    CUDA_TRY(cudaLaunchKernel((const void *)d.code->func, dim3(grid), dim3(d.threads), kp, (size_t)d.smem, st));
  }
  return FE_OK;
}

} // namespace

// ---------------------------------------------------------------------------
// Allocation-free residual max-norm (fe_residual_max_noalloc).
//
// Its scratch (per-block partial maxima plus the result slot) is this
// file-scope device array, so the call itself allocates nothing.  Every GPU
// that loads the library holds these 256 KiB until the process exits.  All
// calls share the array: calls that overlap on the GPU race on it.  The
// kernels overwrite every partial they later read, so nothing has to be
// cleared between calls.
// ---------------------------------------------------------------------------
#define FE_NOALLOC_SLOTS 32768             // doubles in the scratch array (256 KiB)
#define FE_NOALLOC_ITEMS 8192              // residual entries reduced by one block
#define FE_NOALLOC_MAX_N ((long long)(FE_NOALLOC_SLOTS - 1) * FE_NOALLOC_ITEMS)

static __device__ __align__(256) double g_noalloc_scratch[FE_NOALLOC_SLOTS];

__global__ void k_absmax_noalloc_blocks(const double *__restrict__ R, long long n, double *__restrict__ part) {
  __shared__ double sm[32];
  const long long b0 = (long long)blockIdx.x * FE_NOALLOC_ITEMS;
  const long long b1 = b0 + FE_NOALLOC_ITEMS < n ? b0 + FE_NOALLOC_ITEMS : n;
  double m = 0.0;
  for (long long i = b0 + threadIdx.x; i < b1; i += blockDim.x) m = fmax(m, absnan(R[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) part[blockIdx.x] = m;
  }
}

__global__ void k_absmax_noalloc_final(const double *__restrict__ part, int nb, double *__restrict__ result) {
  __shared__ double sm[32];
  double m = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) m = fmax(m, part[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = (threadIdx.x < (blockDim.x >> 5)) ? sm[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (threadIdx.x == 0) *result = m;
  }
}

namespace {
// Device address of g_noalloc_scratch, looked up once per device with that
// device current.  In host code the symbol itself is only a host-side
// stand-in, never a device address.
constexpr int kMaxDevices = 64;
std::mutex g_noalloc_mu;
double *g_noalloc_ptr[kMaxDevices] = {nullptr};

int noalloc_scratch(double **ptr) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(FE_ERR_NOGPU, "no CUDA device: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(FE_ERR_ARG, "device %d out of range", dev);
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fail(FE_ERR_CUDA, "cudaGetSymbolAddress(g_noalloc_scratch) on device %d: %s", dev,
                  cudaGetErrorString(e));
    g_noalloc_ptr[dev] = static_cast<double *>(p);
  }
  *ptr = g_noalloc_ptr[dev];
  return FE_OK;
}
} // namespace

// ---------------------------------------------------------------------------
// C-ABI
// ---------------------------------------------------------------------------
extern "C" {

const char *fe_last_error(void) { return g_err.c_str(); }
const char *fe_version(void) { return FE_VERSION; }

int fe_device_info(int *sm_count, int *cc_major, int *cc_minor, size_t *free_bytes, size_t *total_bytes) {
  int rc = ensure_context();
  if (rc) return rc;
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  if (sm_count) CUDA_TRY(cudaDeviceGetAttribute(sm_count, cudaDevAttrMultiProcessorCount, dev));
  if (cc_major) CUDA_TRY(cudaDeviceGetAttribute(cc_major, cudaDevAttrComputeCapabilityMajor, dev));
  if (cc_minor) CUDA_TRY(cudaDeviceGetAttribute(cc_minor, cudaDevAttrComputeCapabilityMinor, dev));
  size_t f = 0, t = 0;
  CUDA_TRY(cudaMemGetInfo(&f, &t));
  if (free_bytes) *free_bytes = f;
  if (total_bytes) *total_bytes = t;
  return FE_OK;
}

namespace {
// nvrtc -> cubin (cached by source hash); no device needed.
int build_cubin(const char *source, const char *kernel_name, const char *include_dir, const char *cache_dir,
                std::string &cubin, char *log, size_t log_cap) {
  if (log && log_cap) log[0] = 0;
  const std::string arch = "--gpu-architecture=sm_103a";
  std::string inc = std::string("--include-path=") + (include_dir ? include_dir : ".");
  // compiler options: the defaults, or PYOOMPH_GB300_NVRTC_OPTS (space separated)
  std::vector<std::string> optv = {"--std=c++17", "-default-device", "-lineinfo", "--fmad=true", "-DFE_NVRTC=1"};
  if (const char *env = getenv("PYOOMPH_GB300_NVRTC_OPTS")) {
    optv.clear();
    std::istringstream is(env);
    std::string o;
    while (is >> o) optv.push_back(o);
  }
  std::string optkey;
  for (auto &o : optv) optkey += o + " ";
  const std::string key_src = std::string(source) + "\n//" + kernel_name + arch + FE_VERSION + optkey;
  char keyhex[32];
  snprintf(keyhex, sizeof(keyhex), "%016llx", (unsigned long long)fnv1a(key_src));
  std::string cache_path;
  cubin.clear();
  if (cache_dir && cache_dir[0]) {
    cache_path = std::string(cache_dir) + "/" + kernel_name + "_" + keyhex + ".cubin";
    read_file(cache_path, cubin);
  }
  if (!cubin.empty()) return FE_OK;
  nvrtcProgram prog;
  if (nvrtcCreateProgram(&prog, source, "fe_element.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS)
    return fail(FE_ERR_COMPILE, "nvrtcCreateProgram failed");
  std::vector<const char *> opts = {arch.c_str(), inc.c_str()};
  for (auto &o : optv) opts.push_back(o.c_str());
  nvrtcResult r = nvrtcCompileProgram(prog, (int)opts.size(), opts.data());
  size_t lsz = 0;
  nvrtcGetProgramLogSize(prog, &lsz);
  std::string lg(lsz, '\0');
  if (lsz) nvrtcGetProgramLog(prog, &lg[0]);
  if (log && log_cap) {
    size_t n = std::min(log_cap - 1, lg.size());
    memcpy(log, lg.data(), n);
    log[n] = 0;
  }
  if (r != NVRTC_SUCCESS) {
    nvrtcDestroyProgram(&prog);
    return fail(FE_ERR_COMPILE, "nvrtc: %s\n%s", nvrtcGetErrorString(r), lg.substr(0, 800).c_str());
  }
  size_t csz = 0;
  nvrtcGetCUBINSize(prog, &csz);
  cubin.resize(csz);
  nvrtcGetCUBIN(prog, &cubin[0]);
  nvrtcDestroyProgram(&prog);
  if (!cache_path.empty()) {
    std::string tmp = cache_path + ".tmp" +
                      std::to_string((unsigned long long)std::hash<std::thread::id>()(std::this_thread::get_id()));
    std::ofstream f(tmp, std::ios::binary);
    if (f) {
      f.write(cubin.data(), (std::streamsize)cubin.size());
      f.close();
      std::rename(tmp.c_str(), cache_path.c_str());
    }
  }
  return FE_OK;
}
} // namespace

int fe_code_build(const char *source, const char *kernel_name, const char *include_dir, const char *cache_dir,
                  size_t *cubin_bytes, char *log, size_t log_cap) {
  if (!source || !kernel_name) return fail(FE_ERR_ARG, "fe_code_build: null argument");
  std::string cubin;
  int rc = build_cubin(source, kernel_name, include_dir, cache_dir, cubin, log, log_cap);
  if (rc) return rc;
  if (cubin_bytes) *cubin_bytes = cubin.size();
  return FE_OK;
}

int fe_code_compile(const char *source, const char *kernel_name, const char *include_dir,
                    const char *cache_dir, fe_code_t **out, char *log, size_t log_cap) {
  if (!source || !kernel_name || !out) return fail(FE_ERR_ARG, "fe_code_compile: null argument");
  *out = nullptr;
  std::string cubin;
  int rc = build_cubin(source, kernel_name, include_dir, cache_dir, cubin, log, log_cap);
  if (rc) return rc;
  rc = ensure_context();
  if (rc) return rc;
  std::unique_ptr<fe_code> c(new fe_code());
  CUDA_TRY(cudaLibraryLoadData(&c->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0));
  CUDA_TRY(cudaLibraryGetKernel(&c->func, c->lib, kernel_name));
  c->name = kernel_name;
  *out = c.release();
  return FE_OK;
}

void fe_code_destroy(fe_code_t *code) { delete code; }

int fe_problem_create(const fe_problem_desc_t *desc, fe_problem_t **out) {
  if (!desc || !out) return fail(FE_ERR_ARG, "fe_problem_create: null argument");
  *out = nullptr;
  int rc0 = validate_desc(desc, true);
  if (rc0) return rc0;
  if (!desc->x) return fail(FE_ERR_ARG, "fe_problem_create: null positions");
  if (desc->jac_precision != FE_JAC_F64 && desc->jac_precision != FE_JAC_F32)
    return fail(FE_ERR_ARG, "fe_problem_create: bad jac_precision %d", desc->jac_precision);
  int rc = ensure_context();
  if (rc) return rc;
  std::unique_ptr<fe_problem> P(new fe_problem());
  P->dim = desc->dim;
  P->nval = desc->nval;
  P->n_nodes = desc->n_nodes;
  P->n_dof = desc->n_dof;
  P->jac_prec = desc->jac_precision;
  P->n_params = desc->n_params;
  P->params_stride = desc->params_stride;
  P->n_hist = std::max(0, desc->n_history);
  P->fused = desc->fused ? 1 : 0;
  if (P->fused) {
    if (desc->n_domains > FE_MAX_FUSED) return fail(FE_ERR_ARG, "at most %d fused domains", FE_MAX_FUSED);
    for (int di = 1; di < desc->n_domains; di++)
      if (desc->domains[di].code != desc->domains[0].code)
        return fail(FE_ERR_ARG, "fused domains must share one code");
  }
  std::vector<const int32_t *> conn_h;
  long long jtot = 0, rtot = 0;
  for (int di = 0; di < desc->n_domains; di++) {
    const fe_domain_desc_t &dd = desc->domains[di];
    if (dd.elems_per_block < 1 || dd.threads_per_block < 32 || dd.threads_per_block > 1024 || dd.smem_bytes < 0 ||
        dd.smem_bytes > 227 * 1024)
      return fail(FE_ERR_ARG, "fe_problem_create: bad launch shape in domain %d", di);
    Domain d;
    d.code = dd.code;
    d.nnode = dd.nnode_el;
    d.nlocal = dd.nlocal;
    d.n_elem = dd.n_elem;
    d.epb = dd.elems_per_block;
    d.threads = dd.threads_per_block;
    d.smem = dd.smem_bytes;
    d.replica_elems = dd.replica_elems > 0 ? dd.replica_elems : 0;
    if (d.replica_elems && (desc->params_stride < 0 ||
                            (dd.n_elem / d.replica_elems) * (long long)desc->params_stride > desc->n_params))
      return fail(FE_ERR_ARG, "domain %d: replica parameters exceed the parameter array", di);
    d.local_node.assign(dd.local_node, dd.local_node + dd.nlocal);
    d.local_val.assign(dd.local_val, dd.local_val + dd.nlocal);
    d.jbase = jtot;
    d.rbase = rtot;
    jtot += dd.n_elem * (long long)dd.nlocal * dd.nlocal;
    rtot += dd.n_elem * (long long)dd.nlocal;
    if ((rc = d.conn.upload(dd.conn, sizeof(int32_t) * dd.n_elem * dd.nnode_el))) return rc;
    if (dd.n_tables > 0 && (rc = d.tables.upload(dd.tables, sizeof(double) * dd.n_tables))) return rc;
    if (d.smem > 48 * 1024 && !P->fused)
      CUDA_TRY(cudaFuncSetAttribute((const void *)d.code->func, cudaFuncAttributeMaxDynamicSharedMemorySize, d.smem));
    conn_h.push_back(dd.conn);
    P->domains.push_back(std::move(d));
  }
  if (jtot > 0xffffffffLL) return fail(FE_ERR_ARG, "element Jacobian space %lld exceeds 2^32 entries", jtot);
  if (P->fused) {
    int smem = 0;
    for (Domain &d : P->domains) smem = std::max(smem, d.smem);
    if (smem > 48 * 1024)
      CUDA_TRY(cudaFuncSetAttribute((const void *)P->domains[0].code->func, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    smem));
  }
  if ((rc = P->x.upload(desc->x, sizeof(double) * desc->n_nodes * desc->dim))) return rc;
  if (desc->x0 && (rc = P->x0.upload(desc->x0, sizeof(double) * desc->n_nodes * desc->dim))) return rc;
  if (P->n_hist > 0) {
    if ((rc = P->hist.alloc(sizeof(double) * P->n_hist * desc->n_nodes * desc->nval))) return rc;
    CUDA_TRY(cudaMemset(P->hist.p, 0, P->hist.bytes));
  }
  if ((rc = P->eqn.upload(desc->eqn, sizeof(int32_t) * desc->n_nodes * desc->nval))) return rc;
  if ((rc = P->values.alloc(sizeof(double) * desc->n_nodes * desc->nval))) return rc;
  CUDA_TRY(cudaMemset(P->values.p, 0, P->values.bytes));
  if ((rc = P->params.alloc(sizeof(double) * std::max(1, desc->n_params)))) return rc;
  if (desc->n_params > 0)
    CUDA_TRY(cudaMemcpy(P->params.p, desc->params, sizeof(double) * desc->n_params, cudaMemcpyHostToDevice));
  if ((rc = P->status.alloc(sizeof(int) * 4))) return rc;
  CUDA_TRY(cudaMemset(P->status.p, 0, P->status.bytes));
  const size_t jel = P->jac_prec == FE_JAC_F64 ? sizeof(double) : sizeof(float);
  if ((rc = P->jbuf_all.alloc(jel * std::max(1LL, jtot)))) return rc;
  if ((rc = P->rbuf_all.alloc(sizeof(double) * std::max(1LL, rtot)))) return rc;
  if ((rc = P->partial.alloc(sizeof(double) * 4096))) return rc;
  HangMap hang;
  if ((rc = hang_map(desc, hang))) return rc;
  if ((rc = build_pattern(P.get(), conn_h, desc->eqn, &hang))) return rc;
  P->n_hang = desc->n_hang;
  if (P->n_hang > 0) {
    const long long nm = desc->hang_ptr[desc->n_hang];
    if ((rc = P->hang_slot.upload(desc->hang_slot, sizeof(int64_t) * P->n_hang)) ||
        (rc = P->hang_ptr.upload(desc->hang_ptr, sizeof(int64_t) * (P->n_hang + 1))) ||
        (rc = P->hang_master.upload(desc->hang_master, sizeof(int64_t) * std::max(1LL, nm))) ||
        (rc = P->hang_weight.upload(desc->hang_weight, sizeof(double) * std::max(1LL, nm))))
      return rc;
  }
  if (!P->fused && P->domains.size() == 1 && P->domains[0].replica_elems == 0 && desc->n_hang == 0) {
    // last element (in element order) contributing to each row
    const Domain &d = P->domains[0];
    const fe_domain_desc_t &dd = desc->domains[0];
    P->row_last.assign((size_t)P->n_dof, -1);
    for (long long e = 0; e < d.n_elem; e++)
      for (int i = 0; i < d.nlocal; i++) {
        const long long node = dd.conn[e * d.nnode + d.local_node[i]];
        const int eq = desc->eqn[node * desc->nval + d.local_val[i]];
        if (eq >= 0) P->row_last[eq] = (int32_t)e;
      }
  }
  *out = P.release();
  return FE_OK;
}

void fe_problem_destroy(fe_problem_t *p) { delete p; }

int fe_pattern_host(const fe_problem_desc_t *desc, int64_t *nnz, int32_t *rowptr, int32_t *colidx) {
  int rc = validate_desc(desc, false);
  if (rc) return rc;
  std::vector<PatDomain> doms;
  long long jb = 0, rb = 0;
  for (int di = 0; di < desc->n_domains; di++) {
    const fe_domain_desc_t &dd = desc->domains[di];
    doms.push_back(PatDomain{dd.conn, dd.nnode_el, dd.nlocal, dd.n_elem, dd.local_node, dd.local_val, jb, rb});
    jb += dd.n_elem * (long long)dd.nlocal * dd.nlocal;
    rb += dd.n_elem * (long long)dd.nlocal;
  }
  PatternOut out;
  HangMap hang;
  if ((rc = hang_map(desc, hang))) return rc;
  if ((rc = build_pattern_host(desc->n_dof, desc->nval, desc->eqn, doms, false, out, &hang))) return rc;
  if (nnz) *nnz = (int64_t)out.colidx.size();
  if (rowptr) memcpy(rowptr, out.rowptr.data(), sizeof(int32_t) * out.rowptr.size());
  if (colidx) memcpy(colidx, out.colidx.data(), sizeof(int32_t) * out.colidx.size());
  return FE_OK;
}

int fe_problem_sizes(const fe_problem_t *p, int64_t *n_dof, int64_t *nnz) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  if (n_dof) *n_dof = p->n_dof;
  if (nnz) *nnz = p->nnz;
  return FE_OK;
}

int fe_problem_pattern(const fe_problem_t *p, int32_t *rowptr, int32_t *colidx) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  if (rowptr) memcpy(rowptr, p->h_rowptr.data(), sizeof(int32_t) * (p->n_dof + 1));
  if (colidx) memcpy(colidx, p->h_colidx.data(), sizeof(int32_t) * p->nnz);
  return FE_OK;
}

int fe_problem_pattern_device(const fe_problem_t *p, const int32_t **rowptr, const int32_t **colidx) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  if (rowptr) *rowptr = p->rowptr.as<int32_t>();
  if (colidx) *colidx = p->colidx.as<int32_t>();
  return FE_OK;
}

int fe_problem_set_values(fe_problem_t *p, const double *values_host) {
  if (!p || !values_host) return fail(FE_ERR_ARG, "null argument");
  CUDA_TRY(cudaMemcpy(p->values.p, values_host, p->values.bytes, cudaMemcpyHostToDevice));
  return FE_OK;
}

int fe_problem_get_values(const fe_problem_t *p, double *values_host) {
  if (!p || !values_host) return fail(FE_ERR_ARG, "null argument");
  CUDA_TRY(cudaMemcpy(values_host, p->values.p, p->values.bytes, cudaMemcpyDeviceToHost));
  return FE_OK;
}

int fe_problem_set_history(fe_problem_t *p, int level, const double *values_host) {
  if (!p || !values_host || level < 0 || level >= p->n_hist) return fail(FE_ERR_ARG, "bad history level");
  const size_t n = sizeof(double) * p->n_nodes * p->nval;
  CUDA_TRY(cudaMemcpy(p->hist.as<char>() + n * level, values_host, n, cudaMemcpyHostToDevice));
  return FE_OK;
}

int fe_problem_get_history(const fe_problem_t *p, int level, double *values_host) {
  if (!p || !values_host || level < 0 || level >= p->n_hist) return fail(FE_ERR_ARG, "bad history level");
  const size_t n = sizeof(double) * p->n_nodes * p->nval;
  CUDA_TRY(cudaMemcpy(values_host, p->hist.as<const char>() + n * level, n, cudaMemcpyDeviceToHost));
  return FE_OK;
}

int fe_problem_shift_history(fe_problem_t *p) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  if (p->n_hist == 0) return FE_OK;
  const size_t n = sizeof(double) * p->n_nodes * p->nval;
  for (int k = p->n_hist - 1; k >= 1; k--)
    CUDA_TRY(cudaMemcpy(p->hist.as<char>() + n * k, p->hist.as<char>() + n * (k - 1), n, cudaMemcpyDeviceToDevice));
  CUDA_TRY(cudaMemcpy(p->hist.p, p->values.p, n, cudaMemcpyDeviceToDevice));
  return FE_OK;
}

int fe_problem_set_positions(fe_problem_t *p, const double *x_host) {
  if (!p || !x_host) return fail(FE_ERR_ARG, "null argument");
  CUDA_TRY(cudaMemcpy(p->x.p, x_host, p->x.bytes, cudaMemcpyHostToDevice));
  return FE_OK;
}

int fe_problem_set_params(fe_problem_t *p, const double *params_host) {
  if (!p || (!params_host && p->n_params)) return fail(FE_ERR_ARG, "null argument");
  if (p->n_params)
    CUDA_TRY(cudaMemcpy(p->params.p, params_host, sizeof(double) * p->n_params, cudaMemcpyHostToDevice));
  return FE_OK;
}

} // extern "C"

namespace {
// the zero-filtered matrix (FE_ASSEMBLE_ZERO_FILTER) from the element
// buffers: filtered gather, ranks, scan of the row counts, scatter
template <typename T>
int assemble_zero_filtered(fe_problem *p, T *J_vals, cudaStream_t st) {
  const long long n = p->n_dof, nnz = p->nnz;
  const int sms = sm_count_cached();
  const long long nb = (n + FE_SCAN_THREADS * FE_SCAN_ITEMS - 1) / (FE_SCAN_THREADS * FE_SCAN_ITEMS);
  int rc;
  if (p->zf_vals.bytes != sizeof(T) * nnz) {
    if ((rc = p->zf_vals.alloc(sizeof(T) * nnz)) || (rc = p->zf_key.alloc(sizeof(unsigned) * nnz)) ||
        (rc = p->zf_rank.alloc(sizeof(int) * nnz)) || (rc = p->zf_cnt.alloc(sizeof(int) * std::max(1LL, n))) ||
        (rc = p->zf_rowptr.alloc(sizeof(int) * (n + 1))) || (rc = p->zf_colidx.alloc(sizeof(int) * nnz)) ||
        (rc = p->zf_bsum.alloc(sizeof(int) * std::max(1LL, nb))))
      return rc;
  }
  k_gather_slots_zf<T><<<grid_for(nnz, 256, sms), 256, 0, st>>>(p->cptr.as<unsigned>(), p->cidx.as<unsigned>(),
                                                               p->jbuf_all.as<T>(), p->zf_vals.as<T>(),
                                                               p->zf_key.as<unsigned>(), nnz, p->zf_thr);
  CUDA_TRY(cudaGetLastError());
  const int wgrid = grid_for(n * 32, 256, sms);
  k_zf_rank<<<wgrid, 256, 0, st>>>(p->rowptr.as<int>(), p->zf_key.as<unsigned>(), p->zf_rank.as<int>(),
                                   p->zf_cnt.as<int>(), n);
  CUDA_TRY(cudaGetLastError());
  k_scan_blocks<<<(unsigned)nb, FE_SCAN_THREADS, 0, st>>>(p->zf_cnt.as<int>(), p->zf_rowptr.as<int>(),
                                                          p->zf_bsum.as<int>(), n);
  CUDA_TRY(cudaGetLastError());
  k_scan_totals<<<1, FE_SCAN_THREADS, 0, st>>>(p->zf_bsum.as<int>(), nb, p->zf_rowptr.as<int>() + n);
  CUDA_TRY(cudaGetLastError());
  k_scan_add<<<grid_for(n, 256, sms), 256, 0, st>>>(p->zf_rowptr.as<int>(), p->zf_bsum.as<int>(), n);
  CUDA_TRY(cudaGetLastError());
  k_zf_scatter<T><<<wgrid, 256, 0, st>>>(p->rowptr.as<int>(), p->zf_rank.as<int>(), p->zf_rowptr.as<int>(),
                                         p->colidx.as<int>(), p->zf_vals.as<T>(), p->zf_colidx.as<int>(), J_vals, n);
  CUDA_TRY(cudaGetLastError());
  p->zf_done = true;
  return FE_OK;
}
} // namespace

extern "C" {

int fe_assemble(fe_problem_t *p, const double *dofs, double *R, void *J_vals, int flags, void *stream) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  cudaStream_t st = (cudaStream_t)stream;
  const bool want_m = flags & FE_ASSEMBLE_MASS, want_p = flags & FE_ASSEMBLE_DPARAM;
  const bool want_h = flags & FE_ASSEMBLE_HVP;
  const bool want_zf = flags & FE_ASSEMBLE_ZERO_FILTER;
  if (want_zf && (want_h || !(flags & (FE_ASSEMBLE_JACOBIAN | FE_ASSEMBLE_MASS))))
    return fail(FE_ERR_ARG, "fe_assemble: the zero filter applies to a Jacobian or mass-matrix assembly");
  if (want_zf && p->cw.p)
    return fail(FE_ERR_ARG, "fe_assemble: the zero filter is not available on meshes with hanging values");
  const bool want_r = (flags & FE_ASSEMBLE_RESIDUAL) || want_p;
  const bool want_j = (flags & FE_ASSEMBLE_JACOBIAN) || want_m || want_h;
  if (want_h && (p->fused || !p->dir.p || (flags & (FE_ASSEMBLE_JACOBIAN | FE_ASSEMBLE_MASS | FE_ASSEMBLE_DPARAM))))
    return fail(FE_ERR_ARG, "fe_assemble: the Hessian-vector product needs fixed-mesh code, a direction "
                            "(fe_problem_set_direction) and a call of its own");
  if ((want_r && !R && p->n_dof > 0) || (want_j && !J_vals && p->nnz > 0))
    return fail(FE_ERR_ARG, "fe_assemble: missing output");
  if (want_m && !p->fused && p->n_hist == 0)
    return fail(FE_ERR_ARG, "fe_assemble: a mass matrix needs code of a transient form (fused code, or "
                            "fixed-mesh code with history levels, n_history > 0)");
  if ((want_m && (flags & FE_ASSEMBLE_JACOBIAN)) || (want_p && (flags & (FE_ASSEMBLE_JACOBIAN | FE_ASSEMBLE_MASS))))
    return fail(FE_ERR_ARG, "fe_assemble: Jacobian, mass matrix and parameter derivative are separate calls");
  const int eflag = want_h ? 4 : want_p ? 3 : want_m ? 2 : want_j ? 1 : 0;
  const int sms = sm_count_cached();
  std::vector<cudaEvent_t> ev;
  if (p->timing) {
    // 0 start, 1 after the dof scatter, 5 after the element kernels, 2 after
    // the tensor-core contraction, 3 after the residual gather, 4 at the end
    ev.resize(6);
    for (auto &e : ev) CUDA_TRY(cudaEventCreate(&e));
    CUDA_TRY(cudaEventRecord(ev[0], st));
  }
  if (flags & FE_ASSEMBLE_VALUES_FROM_DOFS) {
    if (!dofs && p->n_dof > 0) return fail(FE_ERR_ARG, "fe_assemble: missing dofs");
    long long n = p->n_nodes * p->nval;
    k_scatter_dofs<<<grid_for(n, 256, sms), 256, 0, st>>>(dofs, p->eqn.as<int>(), p->values.as<double>(), n);
    CUDA_TRY(cudaGetLastError());
  }
  if (p->n_hang > 0) {
    k_hang_interp<<<grid_for(p->n_hang, 256, sms), 256, 0, st>>>(
        p->hang_slot.as<long long>(), p->hang_ptr.as<long long>(), p->hang_master.as<long long>(),
        p->hang_weight.as<double>(), p->values.as<double>(), p->n_hang);
    CUDA_TRY(cudaGetLastError());
  }
  if (p->timing) CUDA_TRY(cudaEventRecord(ev[1], st));
  int rc = launch_elements(p, eflag, st);
  if (rc) return rc;
  if (p->timing) CUDA_TRY(cudaEventRecord(ev[5], st));
  if (eflag == 1 || eflag == 4)
    for (Domain &d : p->domains)
      if (d.tc && (rc = tc_domain(p, d, 0, d.n_elem, st))) return rc;
  if (p->timing) CUDA_TRY(cudaEventRecord(ev[2], st));
  // the tile gather sums the residual in the Jacobian's launch, and so does
  // the per-slot gather (a row prologue) where neither carries hang weights
  const bool rowg = want_j && p->nnz > 0 && !want_zf && tile_gather(p);
  const bool fused_r = want_r && want_j && p->nnz > 0 && !want_zf && !rowg && !p->rw.p && !p->cw.p;
  if (rowg || fused_r) {
  } else if (want_r && p->rw.p) {
    k_gather_rows_w<<<grid_for(p->n_dof, 256, sms), 256, 0, st>>>(p->rptr.as<unsigned>(), p->ridx.as<unsigned>(),
                                                                 p->rw.as<double>(), p->rbuf_all.as<double>(), R,
                                                                 p->n_dof);
    CUDA_TRY(cudaGetLastError());
  } else if (want_r) {
    k_gather_rows<<<grid_for(p->n_dof, 256, sms), 256, 0, st>>>(p->rptr.as<unsigned>(), p->ridx.as<unsigned>(),
                                                               p->rbuf_all.as<double>(), R, p->n_dof);
    CUDA_TRY(cudaGetLastError());
  }
  if (p->timing) CUDA_TRY(cudaEventRecord(ev[3], st));
  if (want_j && p->nnz > 0 && p->cw.p) {
    if (p->jac_prec == FE_JAC_F64)
      k_gather_slots_w<double><<<grid_for(p->nnz, 256, sms), 256, 0, st>>>(
          p->cptr.as<unsigned>(), p->cidx.as<unsigned>(), p->cw.as<double>(), p->jbuf_all.as<double>(),
          (double *)J_vals, p->nnz);
    else
      k_gather_slots_w<float><<<grid_for(p->nnz, 256, sms), 256, 0, st>>>(
          p->cptr.as<unsigned>(), p->cidx.as<unsigned>(), p->cw.as<double>(), p->jbuf_all.as<float>(),
          (float *)J_vals, p->nnz);
    CUDA_TRY(cudaGetLastError());
  } else if (want_j && p->nnz > 0 && want_zf) {
    rc = p->jac_prec == FE_JAC_F64 ? assemble_zero_filtered<double>(p, (double *)J_vals, st)
                                   : assemble_zero_filtered<float>(p, (float *)J_vals, st);
    if (rc) return rc;
  } else if (rowg) {
    rc = p->jac_prec == FE_JAC_F64 ? launch_tile_gather<double>(p, want_r ? R : nullptr, (double *)J_vals, st)
                                   : launch_tile_gather<float>(p, want_r ? R : nullptr, (float *)J_vals, st);
    if (rc) return rc;
  } else if (fused_r) {
    const GatherRows rows{p->rptr.as<unsigned>(), p->ridx.as<unsigned>(), p->rbuf_all.as<double>(), R, p->n_dof,
                          nullptr};
    if (p->jac_prec == FE_JAC_F64)
      launch_gather_rows_slots<double>(rows, p->cptr.as<unsigned>(), p->cidx.as<unsigned>(),
                                       p->jbuf_all.as<double>(), (double *)J_vals, p->nnz, sms, st);
    else
      launch_gather_rows_slots<float>(rows, p->cptr.as<unsigned>(), p->cidx.as<unsigned>(), p->jbuf_all.as<float>(),
                                      (float *)J_vals, p->nnz, sms, st);
    CUDA_TRY(cudaGetLastError());
  } else if (want_j && p->nnz > 0) {
    if (p->jac_prec == FE_JAC_F64)
      launch_gather_slots<double>(p->cptr.as<unsigned>(), p->cidx.as<unsigned>(), p->jbuf_all.as<double>(),
                                  (double *)J_vals, p->nnz, sms, st);
    else
      launch_gather_slots<float>(p->cptr.as<unsigned>(), p->cidx.as<unsigned>(), p->jbuf_all.as<float>(),
                                 (float *)J_vals, p->nnz, sms, st);
    CUDA_TRY(cudaGetLastError());
  }
  if (p->timing) {
    CUDA_TRY(cudaEventRecord(ev[4], st));
    p->pending.push_back(ev);
  }
  return FE_OK;
}

int fe_problem_graph_capture(fe_problem_t *p, const double *dofs, double *R, void *J_vals, int flags) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  if (p->graph) {
    CUDA_TRY(cudaGraphExecDestroy(p->graph));
    p->graph = nullptr;
  }
  cudaStream_t s;
  CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  const bool timing = p->timing;
  p->timing = false; // no events inside the recorded graph
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  int rc = FE_OK;
  if (e == cudaSuccess) {
    rc = fe_assemble(p, dofs, R, J_vals, flags, (void *)s);
    cudaGraph_t g = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(s, &g);
    if (rc == FE_OK && e2 == cudaSuccess) {
      e = cudaGraphInstantiate(&p->graph, g, 0);
      if (e != cudaSuccess) p->graph = nullptr;
    } else if (rc == FE_OK) {
      e = e2;
    }
    if (g) cudaGraphDestroy(g);
  }
  p->timing = timing;
  cudaStreamDestroy(s);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(FE_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
  return FE_OK;
}

int fe_problem_graph_launch(fe_problem_t *p, void *stream) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  if (!p->graph) return fail(FE_ERR_ARG, "no recorded assembly (call fe_problem_graph_capture first)");
  CUDA_TRY(cudaGraphLaunch(p->graph, (cudaStream_t)stream));
  return FE_OK;
}

namespace {
int plan_pipeline(fe_problem *p, int nchunks) {
  const int requested = nchunks;
  const Domain &d = p->domains[0];
  // chunks hold whole waves of blocks (all SMs busy), so only the last one has a tail
  int per_sm = 1;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)d.code->func, d.threads, d.smem));
  const long long wave = (long long)std::max(1, per_sm) * sm_count_cached(); // blocks per wave
  const long long blocks = (d.n_elem + d.epb - 1) / d.epb;
  const long long waves = (blocks + wave - 1) / wave;
  nchunks = (int)std::max(1LL, std::min<long long>(nchunks, waves));
  // decreasing chunks (waves in proportion to n, n-1, ..., 1): the copy of
  // each chunk's rows overlaps the next chunk's elements, and the last
  // chunk's copy, left exposed at the end, is the smallest
  std::vector<long long> wv(nchunks, 1);
  {
    const long long wsum = (long long)nchunks * (nchunks + 1) / 2;
    long long given = 0;
    for (int k = 0; k < nchunks; k++) {
      wv[k] = std::max(1LL, (waves * (nchunks - k) + wsum / 2) / wsum);
      given += wv[k];
    }
    // whole waves: the difference goes to (or comes from) the first chunks
    // (nchunks <= waves, so a chunk above one wave exists while given > waves)
    for (int k = 0; waves > 0 && given != waves; k = (k + 1) % nchunks) {
      if (given < waves) {
        wv[k]++;
        given++;
      } else if (wv[k] > 1) {
        wv[k]--;
        given--;
      }
    }
  }
  const long long units = blocks;
  if (p->pipe_copy) CUDA_TRY(cudaStreamSynchronize(p->pipe_copy)); // copies of the old plan
  if (p->pipe_gather) CUDA_TRY(cudaStreamSynchronize(p->pipe_gather));
  for (auto e : p->pipe_es)
    if (e) CUDA_TRY(cudaStreamSynchronize(e));
  p->pipe_release();
  p->pipe_elem.assign(nchunks + 1, 0);
  {
    long long w_at = 0;
    for (int k = 0; k <= nchunks; k++) {
      p->pipe_elem[k] = std::min(d.n_elem, std::min(units, w_at * wave) * d.epb);
      if (k < nchunks) w_at += wv[k];
    }
  }
  p->pipe_elem[nchunks] = d.n_elem;
  // a row is complete after the chunk holding its last contributing element;
  // maximal runs of consecutive rows completed by the same chunk become one
  // gather + copy each (structured meshes give a few runs per chunk: the
  // vertex rows and the rows of the nodes added for the quadratic space)
  std::vector<int> chunk_of(p->n_dof);
  for (long long r = 0; r < p->n_dof; r++) {
    const long long e = p->row_last[r];
    int k = 0;
    while (k + 1 < nchunks && e >= p->pipe_elem[k + 1]) k++;
    chunk_of[r] = e < 0 ? 0 : k;
  }
  std::vector<std::array<long long, 3>> runs; // chunk, r0, r1
  for (long long r = 0; r < p->n_dof;) {
    long long r1 = r + 1;
    while (r1 < p->n_dof && chunk_of[r1] == chunk_of[r]) r1++;
    runs.push_back({chunk_of[r], r, r1});
    r = r1;
  }
  // short runs (the alternating rows of the element column a chunk boundary
  // cuts) join the following run when that one completes no earlier: a row
  // may always be gathered late, never early
  {
    const long long thr = std::max(1LL, p->n_dof / (16LL * nchunks));
    std::vector<std::array<long long, 3>> m;
    for (auto it = runs.rbegin(); it != runs.rend(); ++it) {
      if (!m.empty() && (*it)[2] - (*it)[1] < thr && m.back()[0] >= (*it)[0])
        m.back()[1] = (*it)[1];
      else
        m.push_back(*it);
    }
    runs.assign(m.rbegin(), m.rend());
  }
  // still too many runs: pairwise merges into the later chunk (safety net)
  while ((long long)runs.size() > 8LL * nchunks) {
    std::vector<std::array<long long, 3>> m;
    for (size_t i = 0; i < runs.size(); i += 2) {
      if (i + 1 < runs.size())
        m.push_back({std::max(runs[i][0], runs[i + 1][0]), runs[i][1], runs[i + 1][2]});
      else
        m.push_back(runs[i]);
    }
    runs.swap(m);
  }
  p->pipe_runs.assign(nchunks, {});
  for (auto &q : runs) p->pipe_runs[q[0]].push_back({q[1], q[2]});
  {
    // the chunks' rows and slots as index lists, chunk by chunk
    const int32_t *rp = p->h_rowptr.data();
    std::vector<int32_t> rl, sl;
    rl.reserve((size_t)p->n_dof);
    sl.reserve((size_t)p->nnz);
    p->pipe_row_off.assign(nchunks + 1, 0);
    p->pipe_slot_off.assign(nchunks + 1, 0);
    for (int k = 0; k < nchunks; k++) {
      for (const auto &run : p->pipe_runs[k])
        for (long long r = run.first; r < run.second; r++) {
          rl.push_back((int32_t)r);
          for (int32_t q = rp[r]; q < rp[r + 1]; q++) sl.push_back(q);
        }
      p->pipe_row_off[k + 1] = (long long)rl.size();
      p->pipe_slot_off[k + 1] = (long long)sl.size();
    }
    int rc;
    if (!rl.empty() && (rc = p->pipe_rowlist.upload(rl.data(), sizeof(int32_t) * rl.size()))) return rc;
    if (!sl.empty() && (rc = p->pipe_slotlist.upload(sl.data(), sizeof(int32_t) * sl.size()))) return rc;
  }
  CUDA_TRY(cudaStreamCreateWithFlags(&p->pipe_copy, cudaStreamNonBlocking));
  CUDA_TRY(cudaStreamCreateWithFlags(&p->pipe_gather, cudaStreamNonBlocking));
  for (auto &e : p->pipe_es) CUDA_TRY(cudaStreamCreateWithFlags(&e, cudaStreamNonBlocking));
  p->pipe_ev.resize(nchunks + 1);
  for (auto &e : p->pipe_ev) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  p->pipe_eev.resize(nchunks + 2); // + the fork of the element streams
  for (auto &e : p->pipe_eev) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  p->pipe_chunks = nchunks;
  p->pipe_requested = requested;
  return FE_OK;
}
} // namespace

// element streams of the pipelined assembly; automatic: one.  Measured on
// GB300, NS 256^2 (ms per call, best chunk count): two streams run
// consecutive chunks concurrently rather than only across their tails;
// FP64 J 1.72 -> 1.63-1.87 depending on the chunk count and the run, df64
// J 1.15 -> 1.39, FP32 J 0.60 -> 0.67 (its copies start later)
static int pipe_streams(const fe_problem *p) {
  return p->pipe_nes == 2 ? 2 : 1;
}

int fe_problem_set_pipeline_streams(fe_problem_t *p, int n) {
  if (!p || n < 0 || n > 2) return fail(FE_ERR_ARG, "fe_problem_set_pipeline_streams: n must be 0, 1 or 2");
  p->pipe_nes = n;
  return FE_OK;
}

int fe_assemble_pipelined(fe_problem_t *p, const double *dofs, double *R, void *J_vals, int flags, int nchunks,
                          void *stream) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  if (p->row_last.empty() && p->n_dof > 0)
    return fail(FE_ERR_ARG, "fe_assemble_pipelined: single-domain problems without replicas only");
  const bool want_r = flags & FE_ASSEMBLE_RESIDUAL, want_j = flags & FE_ASSEMBLE_JACOBIAN;
  if (flags & ~(FE_ASSEMBLE_RESIDUAL | FE_ASSEMBLE_JACOBIAN | FE_ASSEMBLE_VALUES_FROM_DOFS))
    return fail(FE_ERR_ARG, "fe_assemble_pipelined: residual and Jacobian flags only");
  if ((want_r && !R && p->n_dof > 0) || (want_j && !J_vals && p->nnz > 0) ||
      ((flags & FE_ASSEMBLE_VALUES_FROM_DOFS) && !dofs && p->n_dof > 0))
    return fail(FE_ERR_ARG, "fe_assemble_pipelined: missing buffer");
  cudaStream_t st = (cudaStream_t)stream;
  int rc;
  if (p->pipe_requested != std::max(1, nchunks) && (rc = plan_pipeline(p, std::max(1, nchunks)))) return rc;
  const size_t jel = p->jac_prec == FE_JAC_F64 ? sizeof(double) : sizeof(float);
  if (!p->pipe_dofs.p && ((rc = p->pipe_dofs.alloc(sizeof(double) * std::max(1LL, p->n_dof))) ||
                          (rc = p->pipe_R.alloc(sizeof(double) * std::max(1LL, p->n_dof))) ||
                          (rc = p->pipe_J.alloc(jel * std::max(1LL, p->nnz)))))
    return rc;
  const int sms = sm_count_cached();
  // the previous call's copies read the staging buffers: finish them first
  CUDA_TRY(cudaStreamWaitEvent(st, p->pipe_ev[p->pipe_chunks], 0));
  cudaEvent_t *tev = nullptr;
  if (p->timing) {
    if (p->pipe_tev.size() != (size_t)(1 + 3 * p->pipe_chunks)) {
      for (auto e : p->pipe_tev) cudaEventDestroy(e);
      p->pipe_tev.assign(1 + 3 * p->pipe_chunks, nullptr);
      for (auto &e : p->pipe_tev) CUDA_TRY(cudaEventCreate(&e));
    }
    tev = p->pipe_tev.data();
    CUDA_TRY(cudaEventRecord(tev[0], st));
    p->pipe_timed = p->pipe_chunks;
  }
  if (flags & FE_ASSEMBLE_VALUES_FROM_DOFS) {
    CUDA_TRY(cudaMemcpyAsync(p->pipe_dofs.p, dofs, sizeof(double) * p->n_dof, cudaMemcpyHostToDevice, st));
    long long n = p->n_nodes * p->nval;
    k_scatter_dofs<<<grid_for(n, 256, sms), 256, 0, st>>>(p->pipe_dofs.as<double>(), p->eqn.as<int>(),
                                                          p->values.as<double>(), n);
    CUDA_TRY(cudaGetLastError());
  }
  Domain &d = p->domains[0];
  const int32_t *h_rp = p->h_rowptr.data();
  cudaStream_t gs = p->pipe_gather;
  const int nes = pipe_streams(p);
  if (nes == 2) {
    // fork: both element streams start after the caller's work so far
    CUDA_TRY(cudaEventRecord(p->pipe_eev[p->pipe_chunks + 1], st));
    for (auto e : p->pipe_es) CUDA_TRY(cudaStreamWaitEvent(e, p->pipe_eev[p->pipe_chunks + 1], 0));
  }
  for (int k = 0; k < p->pipe_chunks; k++) {
    const long long e0 = p->pipe_elem[k], e1 = p->pipe_elem[k + 1];
    cudaStream_t es = nes == 2 ? p->pipe_es[k & 1] : st; // one stream: the caller's
    if (e1 > e0) {
      FeElemArgs a = domain_args(p, d, want_j ? 1 : 0);
      a.conn += e0 * d.nnode;
      a.rbuf += e0 * d.nlocal;
      a.jbuf = (char *)a.jbuf + jel * (size_t)(e0 * (long long)d.nlocal * d.nlocal);
      a.n_elem = e1 - e0;
      if (d.tc) a.dhat += e0 * (long long)d.tca.nq * d.tca.npair;
      void *kp[] = {&a};
      unsigned grid = (unsigned)((a.n_elem + d.epb - 1) / d.epb);
      CUDA_TRY(cudaLaunchKernel((const void *)d.code->func, dim3(grid), dim3(d.threads), kp, (size_t)d.smem, es));
      if (want_j && d.tc && (rc = tc_domain(p, d, e0, e1, es))) return rc;
    }
    if (tev) CUDA_TRY(cudaEventRecord(tev[1 + 3 * k], es));
    // the rows and slots this chunk completes, on the gather stream once the
    // chunk's elements are done (the next chunk's elements, writing other
    // element buffers, run meanwhile): one gather launch
    CUDA_TRY(cudaEventRecord(p->pipe_eev[k], es));
    CUDA_TRY(cudaStreamWaitEvent(gs, p->pipe_eev[k], 0));
    {
      const long long q0 = p->pipe_row_off[k], q1 = p->pipe_row_off[k + 1];
      const long long z0 = p->pipe_slot_off[k], z1 = p->pipe_slot_off[k + 1];
      const GatherRows rows{p->rptr.as<unsigned>(), p->ridx.as<unsigned>(), p->rbuf_all.as<double>(),
                            p->pipe_R.as<double>(), q1 - q0, p->pipe_rowlist.as<int>() + q0};
      if (want_r && want_j && q1 > q0 && z1 > z0) {
        // R rows and J slots of the chunk in one launch
        if (p->jac_prec == FE_JAC_F64)
          launch_gather_rows_slots<double>(rows, p->cptr.as<unsigned>(), p->cidx.as<unsigned>(),
                                           p->jbuf_all.as<double>(), p->pipe_J.as<double>(), z1 - z0, sms, gs,
                                           p->pipe_slotlist.as<int>() + z0);
        else
          launch_gather_rows_slots<float>(rows, p->cptr.as<unsigned>(), p->cidx.as<unsigned>(),
                                          p->jbuf_all.as<float>(), p->pipe_J.as<float>(), z1 - z0, sms, gs,
                                          p->pipe_slotlist.as<int>() + z0);
        CUDA_TRY(cudaGetLastError());
      } else if (want_r && q1 > q0) {
        k_gather_rows<<<grid_for(q1 - q0, 256, sms), 256, 0, gs>>>(
            p->rptr.as<unsigned>(), p->ridx.as<unsigned>(), p->rbuf_all.as<double>(), p->pipe_R.as<double>(),
            q1 - q0, p->pipe_rowlist.as<int>() + q0);
        CUDA_TRY(cudaGetLastError());
      }
      if (want_j && z1 > z0 && !(want_r && q1 > q0)) {
        if (p->jac_prec == FE_JAC_F64)
          launch_gather_slots<double>(p->cptr.as<unsigned>(), p->cidx.as<unsigned>(), p->jbuf_all.as<double>(),
                                      p->pipe_J.as<double>(), z1 - z0, sms, gs, p->pipe_slotlist.as<int>() + z0);
        else
          launch_gather_slots<float>(p->cptr.as<unsigned>(), p->cidx.as<unsigned>(), p->jbuf_all.as<float>(),
                                     p->pipe_J.as<float>(), z1 - z0, sms, gs, p->pipe_slotlist.as<int>() + z0);
        CUDA_TRY(cudaGetLastError());
      }
    }
    if (tev) CUDA_TRY(cudaEventRecord(tev[2 + 3 * k], gs));
    if (p->pipe_runs[k].empty()) {
      if (tev) CUDA_TRY(cudaEventRecord(tev[3 + 3 * k], gs));
      continue;
    }
    // copy the finished rows to the host while the next chunk computes
    CUDA_TRY(cudaEventRecord(p->pipe_ev[k], gs));
    CUDA_TRY(cudaStreamWaitEvent(p->pipe_copy, p->pipe_ev[k], 0));
    for (const auto &run : p->pipe_runs[k]) {
      const long long r0 = run.first, r1 = run.second;
      const long long s0 = h_rp[r0], s1 = h_rp[r1];
      if (want_r)
        CUDA_TRY(cudaMemcpyAsync(R + r0, p->pipe_R.as<double>() + r0, sizeof(double) * (r1 - r0),
                                 cudaMemcpyDeviceToHost, p->pipe_copy));
      if (want_j && s1 > s0)
        CUDA_TRY(cudaMemcpyAsync((char *)J_vals + jel * s0, (const char *)p->pipe_J.p + jel * s0, jel * (s1 - s0),
                                 cudaMemcpyDeviceToHost, p->pipe_copy));
    }
    if (tev) CUDA_TRY(cudaEventRecord(tev[3 + 3 * k], p->pipe_copy));
  }
  // the caller's stream completes only after the gathers and the copies
  CUDA_TRY(cudaEventRecord(p->pipe_eev[p->pipe_chunks], gs));
  CUDA_TRY(cudaStreamWaitEvent(p->pipe_copy, p->pipe_eev[p->pipe_chunks], 0));
  CUDA_TRY(cudaEventRecord(p->pipe_ev[p->pipe_chunks], p->pipe_copy));
  CUDA_TRY(cudaStreamWaitEvent(st, p->pipe_ev[p->pipe_chunks], 0));
  return FE_OK;
}

int fe_problem_set_direction(fe_problem_t *p, const double *y, void *stream) {
  if (!p || (!y && p->n_dof > 0)) return fail(FE_ERR_ARG, "null argument");
  int rc;
  const long long n = p->n_nodes * p->nval;
  if (!p->dir.p && (rc = p->dir.alloc(sizeof(double) * std::max(1LL, n)))) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  CUDA_TRY(cudaMemsetAsync(p->dir.p, 0, sizeof(double) * n, st)); // pinned values: zero direction
  k_scatter_dofs<<<grid_for(n, 256, sm_count_cached()), 256, 0, st>>>(y, p->eqn.as<int>(), p->dir.as<double>(), n);
  CUDA_TRY(cudaGetLastError());
  return FE_OK;
}

int fe_problem_set_tensor_contraction(fe_problem_t *p, int domain, int n, int nq, int nc, const double *phi, int npair,
                                      const int32_t *pa, const int32_t *pb) {
  if (!p || domain < 0 || domain >= (int)p->domains.size()) return fail(FE_ERR_ARG, "bad problem or domain");
  if (p->jac_prec != FE_JAC_F32) return fail(FE_ERR_ARG, "tensor contraction: FP32 Jacobians only");
  if (p->fused) return fail(FE_ERR_ARG, "tensor contraction: fixed-mesh (unfused) code only");
  Domain &d = p->domains[domain];
  if (n != d.nlocal) return fail(FE_ERR_ARG, "tensor contraction: n %d != the domain's %d local values", n, d.nlocal);
  int rc;
  if ((rc = tc_setup(d.tca, d.tc_phi, d.tc_bhi, d.tc_blo, n, nq, nc, phi, npair, pa, pb))) return rc;
  if ((rc = d.tc_dhat.alloc(sizeof(float) * std::max(1LL, d.n_elem * (long long)nq * npair)))) return rc;
  CUDA_TRY(cudaMemset(d.tc_dhat.p, 0, d.tc_dhat.bytes));
  d.tc = true;
  return FE_OK;
}

int fe_tc_contract(const float *dhat, float *jbuf, int64_t n_elem, int n, int nq, int nc, const double *phi, int npair,
                   const int32_t *pa, const int32_t *pb, void *stream) {
  if ((!dhat || !jbuf) && n_elem > 0) return fail(FE_ERR_ARG, "fe_tc_contract: null buffer");
  int rc = ensure_context();
  if (rc) return rc;
  FeTcArgs A;
  DevBuf ph, bhi, blo, status;
  if ((rc = tc_setup(A, ph, bhi, blo, n, nq, nc, phi, npair, pa, pb))) return rc;
  if ((rc = status.alloc(sizeof(int)))) return rc;
  CUDA_TRY(cudaMemset(status.p, 0, sizeof(int)));
  A.dhat = dhat;
  A.jbuf = jbuf;
  A.status = status.as<int>();
  A.n_elem = n_elem;
  cudaStream_t st = (cudaStream_t)stream;
  if ((rc = tc_launch(A, st))) return rc;
  CUDA_TRY(cudaStreamSynchronize(st));
  int sw = 0;
  CUDA_TRY(cudaMemcpy(&sw, status.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (sw) return fail(FE_ERR_DEVICE, "fe_tc_contract: status word %d (a bounded wait gave up)", sw);
  return FE_OK;
}

int fe_problem_set_zero_threshold(fe_problem_t *p, double threshold) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  if (!(threshold >= 0.0)) return fail(FE_ERR_ARG, "zero threshold must be >= 0");
  p->zf_thr = threshold;
  return FE_OK;
}

int fe_problem_set_gather(fe_problem_t *p, int mode) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  if (mode != FE_GATHER_SLOTS && mode != FE_GATHER_TILES) return fail(FE_ERR_ARG, "unknown gather mode %d", mode);
  p->gather_mode = mode;
  return FE_OK;
}

int fe_problem_gather_lanes(const fe_problem_t *p) {
  if (!p) return -1;
  return tile_gather(p) ? p->g_G : 0;
}

int fe_problem_filtered_pattern(fe_problem_t *p, int64_t *nnz, int32_t *rowptr, int32_t *colidx, void *stream) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  if (!p->zf_done) return fail(FE_ERR_STATE, "no zero-filtered assembly yet");
  CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  int32_t m = 0;
  CUDA_TRY(cudaMemcpy(&m, p->zf_rowptr.as<int32_t>() + p->n_dof, sizeof(int32_t), cudaMemcpyDeviceToHost));
  if (nnz) *nnz = m;
  if (rowptr) CUDA_TRY(cudaMemcpy(rowptr, p->zf_rowptr.p, sizeof(int32_t) * (p->n_dof + 1), cudaMemcpyDefault));
  if (colidx && m > 0) CUDA_TRY(cudaMemcpy(colidx, p->zf_colidx.p, sizeof(int32_t) * m, cudaMemcpyDefault));
  return FE_OK;
}

int fe_problem_set_persistent(fe_problem_t *p, int enable) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  p->persistent = enable != 0;
  return FE_OK;
}

int fe_problem_set_dparam(fe_problem_t *p, int index) {
  if (!p || index < 0 || index >= std::max(1, p->n_params)) return fail(FE_ERR_ARG, "bad parameter index");
  p->dparam = index;
  return FE_OK;
}

int fe_problem_set_timing(fe_problem_t *p, int enable) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  p->timing = enable != 0;
  return FE_OK;
}

int fe_problem_stage_times(fe_problem_t *p, double *ms, int64_t *calls) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  for (auto &v : p->pending) {
    CUDA_TRY(cudaEventSynchronize(v[4]));
    const int from[5] = {0, 1, 2, 3, 5}, to[5] = {1, 5, 3, 4, 2};
    for (int k = 0; k < 5; k++) {
      float t = 0.f;
      CUDA_TRY(cudaEventElapsedTime(&t, v[from[k]], v[to[k]]));
      p->stage_ms[k] += t;
    }
    for (auto e : v) cudaEventDestroy(e);
    p->stage_calls++;
  }
  p->pending.clear();
  if (ms)
    for (int k = 0; k < 5; k++) ms[k] = p->stage_ms[k];
  if (calls) *calls = p->stage_calls;
  for (int k = 0; k < 5; k++) p->stage_ms[k] = 0;
  p->stage_calls = 0;
  return FE_OK;
}

int fe_problem_pipeline_times(fe_problem_t *p, float *ms, int cap) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  const int n = p->pipe_timed;
  if (n <= 0) return 0;
  if (!ms || cap < 3 * n) return fail(FE_ERR_ARG, "fe_problem_pipeline_times: buffer shorter than 3 x chunks");
  for (int i = 1; i <= 3 * n; i++) {
    CUDA_TRY(cudaEventSynchronize(p->pipe_tev[i]));
    CUDA_TRY(cudaEventElapsedTime(ms + (i - 1), p->pipe_tev[0], p->pipe_tev[i]));
  }
  return n;
}

int fe_assemble_host(fe_problem_t *p, const double *dofs, double *R, void *J_vals, int flags) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  DevBuf d_dofs, d_R, d_J;
  int rc;
  const size_t jel = p->jac_prec == FE_JAC_F64 ? sizeof(double) : sizeof(float);
  if (flags & FE_ASSEMBLE_VALUES_FROM_DOFS) {
    if (!dofs) return fail(FE_ERR_ARG, "missing dofs");
    if ((rc = d_dofs.upload(dofs, sizeof(double) * p->n_dof))) return rc;
  }
  if ((flags & FE_ASSEMBLE_RESIDUAL) && (rc = d_R.alloc(sizeof(double) * std::max(1LL, p->n_dof)))) return rc;
  if ((flags & FE_ASSEMBLE_JACOBIAN) && (rc = d_J.alloc(jel * std::max(1LL, p->nnz)))) return rc;
  if ((rc = fe_assemble(p, d_dofs.as<double>(), d_R.as<double>(), d_J.p, flags, nullptr))) return rc;
  if ((rc = fe_problem_check(p))) return rc;
  if (flags & FE_ASSEMBLE_RESIDUAL) CUDA_TRY(cudaMemcpy(R, d_R.p, sizeof(double) * p->n_dof, cudaMemcpyDeviceToHost));
  if (flags & FE_ASSEMBLE_JACOBIAN) CUDA_TRY(cudaMemcpy(J_vals, d_J.p, jel * p->nnz, cudaMemcpyDeviceToHost));
  return FE_OK;
}

int fe_residual_max(fe_problem_t *p, const double *R, int64_t n, double *out, void *stream) {
  if (!p || !out || (n > 0 && !R)) return fail(FE_ERR_ARG, "null argument");
  cudaStream_t st = (cudaStream_t)stream;
  if (n <= 0) {
    *out = 0.0;
    return FE_OK;
  }
  const int sms = sm_count_cached();
  int g = std::min(grid_for(n, 256, sms), 4000);
  k_absmax_partial<<<g, 256, 0, st>>>(R, n, p->partial.as<double>());
  k_absmax_partial<<<1, 1024, 0, st>>>(p->partial.as<double>(), g, p->partial.as<double>() + 4095);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(out, p->partial.as<double>() + 4095, sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return FE_OK;
}

int fe_residual_max_noalloc(const double *R, int64_t n, double *out, void *stream) {
  if (!out || (n > 0 && !R)) return fail(FE_ERR_ARG, "fe_residual_max_noalloc: null argument");
  if (n < 0) return fail(FE_ERR_ARG, "fe_residual_max_noalloc: negative length %lld", (long long)n);
  if (n > FE_NOALLOC_MAX_N)
    return fail(FE_ERR_ARG,
                "fe_residual_max_noalloc: n=%lld exceeds the maximum %lld of the static scratch; "
                "use fe_residual_max",
                (long long)n, FE_NOALLOC_MAX_N);
  if (n == 0) {
    *out = 0.0;
    return FE_OK;
  }
  double *scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  const int nb = (int)((n + FE_NOALLOC_ITEMS - 1) / FE_NOALLOC_ITEMS);
  double *result = scratch + (FE_NOALLOC_SLOTS - 1);
  k_absmax_noalloc_blocks<<<nb, 256, 0, st>>>(R, n, scratch);
  k_absmax_noalloc_final<<<1, 1024, 0, st>>>(scratch, nb, result);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(out, result, sizeof(double), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  return FE_OK;
}

int64_t fe_residual_max_noalloc_limit(void) { return (int64_t)FE_NOALLOC_MAX_N; }

int fe_csr_spmv(const int32_t *rowptr, const int32_t *colidx, const void *vals, int val_precision, const double *x,
                double *y, int64_t n, int64_t nnz, void *stream) {
  if (n <= 0) return FE_OK;
  if (!rowptr || !colidx || !vals || !x || !y || nnz < 0) return fail(FE_ERR_ARG, "fe_csr_spmv: null argument");
  launch_csr_spmv(rowptr, colidx, vals, val_precision, x, y, n, nnz, nullptr, 0, 1, (cudaStream_t)stream);
  CUDA_TRY(cudaGetLastError());
  return FE_OK;
}

int fe_csr_update(const int32_t *rowptr, const int32_t *colidx, const double *vals, const double *x, const double *b,
                  const double *z, const double *w, double sc, double *y, int64_t n, int64_t nnz, void *stream) {
  if (n < 0 || nnz < 0 || (n > 0 && (!rowptr || !y || (nnz > 0 && (!colidx || !vals || !x)))))
    return fail(FE_ERR_ARG, "fe_csr_update: bad arguments");
  if (n == 0) return FE_OK;
  const int L = (double)nnz > 128.0 * (double)n ? 32 : 4;
  const int g = grid_for(n * L, 256, sm_count_cached());
  cudaStream_t st = (cudaStream_t)stream;
  if (L == 4)
    k_csr_update<4, double><<<g, 256, 0, st>>>(rowptr, colidx, vals, x, b, z, w, sc, y, n);
  else
    k_csr_update<32, double><<<g, 256, 0, st>>>(rowptr, colidx, vals, x, b, z, w, sc, y, n);
  CUDA_TRY(cudaGetLastError());
  return FE_OK;
}

int fe_csr_update_f32(const int32_t *rowptr, const int32_t *colidx, const float *vals, const float *x, const float *b,
                      const float *z, const float *w, float sc, float *y, int64_t n, int64_t nnz, void *stream) {
  if (n < 0 || nnz < 0 || (n > 0 && (!rowptr || !y || (nnz > 0 && (!colidx || !vals || !x)))))
    return fail(FE_ERR_ARG, "fe_csr_update_f32: bad arguments");
  if (n == 0) return FE_OK;
  const int L = (double)nnz > 128.0 * (double)n ? 32 : 4;
  const int g = grid_for(n * L, 256, sm_count_cached());
  cudaStream_t st = (cudaStream_t)stream;
  if (L == 4)
    k_csr_update<4, float><<<g, 256, 0, st>>>(rowptr, colidx, vals, x, b, z, w, sc, y, n);
  else
    k_csr_update<32, float><<<g, 256, 0, st>>>(rowptr, colidx, vals, x, b, z, w, sc, y, n);
  CUDA_TRY(cudaGetLastError());
  return FE_OK;
}

int fe_csr_diagonal(const int32_t *rowptr, const int32_t *colidx, const void *vals, int val_precision, double *diag,
                    int64_t n, void *stream) {
  if (n <= 0) return FE_OK;
  if (!rowptr || !colidx || !vals || !diag) return fail(FE_ERR_ARG, "fe_csr_diagonal: null argument");
  const int g = grid_for(n, 256, sm_count_cached());
  if (val_precision == FE_JAC_F64)
    k_csr_diagonal<double><<<g, 256, 0, (cudaStream_t)stream>>>(rowptr, colidx, (const double *)vals, diag, n);
  else
    k_csr_diagonal<float><<<g, 256, 0, (cudaStream_t)stream>>>(rowptr, colidx, (const float *)vals, diag, n);
  CUDA_TRY(cudaGetLastError());
  return FE_OK;
}

int fe_dof_update(fe_problem_t *p, double *x, const double *dx, int64_t n, void *stream) {
  if (!p || (n > 0 && (!x || !dx))) return fail(FE_ERR_ARG, "null argument");
  if (n <= 0) return FE_OK;
  k_dof_update<<<grid_for(n, 256, sm_count_cached()), 256, 0, (cudaStream_t)stream>>>(x, dx, n);
  CUDA_TRY(cudaGetLastError());
  return FE_OK;
}

int fe_problem_element_buffers(fe_problem_t *p, int domain, double *R_e, void *J_e) {
  if (!p || domain < 0 || domain >= (int)p->domains.size()) return fail(FE_ERR_ARG, "bad problem/domain");
  CUDA_TRY(cudaDeviceSynchronize());
  const Domain &d = p->domains[domain];
  const size_t jel = p->jac_prec == FE_JAC_F64 ? sizeof(double) : sizeof(float);
  if (R_e)
    CUDA_TRY(cudaMemcpy(R_e, p->rbuf_all.as<double>() + d.rbase, sizeof(double) * d.n_elem * d.nlocal,
                        cudaMemcpyDeviceToHost));
  if (J_e)
    CUDA_TRY(cudaMemcpy(J_e, (const char *)p->jbuf_all.p + jel * d.jbase, jel * d.n_elem * d.nlocal * d.nlocal,
                        cudaMemcpyDeviceToHost));
  return FE_OK;
}

int fe_problem_check(fe_problem_t *p) {
  if (!p) return fail(FE_ERR_ARG, "null problem");
  CUDA_TRY(cudaDeviceSynchronize());
  int st[4] = {0, 0, 0, 0};
  CUDA_TRY(cudaMemcpy(st, p->status.p, sizeof(st), cudaMemcpyDeviceToHost));
  if (st[0]) return fail(FE_ERR_DEVICE, "element kernel status %d (detail %d %d %d)", st[0], st[1], st[2], st[3]);
  return FE_OK;
}

int fe_problem_launch_count(const fe_problem_t *p, int flags) {
  if (!p) return -1;
  int n = 0;
  if (flags & FE_ASSEMBLE_VALUES_FROM_DOFS) n++;
  if (p->fused) {
    for (const Domain &d : p->domains)
      if (d.n_elem) { n++; break; }
  } else {
    for (const Domain &d : p->domains)
      if (d.n_elem) n++;
  }
  const bool want_j = (flags & (FE_ASSEMBLE_JACOBIAN | FE_ASSEMBLE_MASS | FE_ASSEMBLE_HVP)) && p->nnz > 0;
  const bool zf = flags & FE_ASSEMBLE_ZERO_FILTER;
  // the tile gather and the per-slot gather without hang weights sum the
  // residual in the Jacobian's launch
  const bool r_in_j = want_j && !zf && (tile_gather(p) || (!p->rw.p && !p->cw.p));
  if ((flags & (FE_ASSEMBLE_RESIDUAL | FE_ASSEMBLE_DPARAM)) && !r_in_j) n++;
  if (flags & (FE_ASSEMBLE_JACOBIAN | FE_ASSEMBLE_HVP))
    for (const Domain &d : p->domains)
      if (d.tc && d.n_elem) n++;
  if (want_j) n += zf ? 6 : 1;   // filtered gather, ranks, three scan launches, scatter
  if (p->n_hang > 0) n++;
  return n;
}

} // extern "C"

#include "fe_krylov.cuh"
#include "fe_sa_level.cuh"
#include "fe_gmres.cuh"
