// One Arnoldi step of the saddle-point solver's GMRES on the device:
// classical Gram-Schmidt applied twice (fe_gmres_cgs2).  Included by
// fe_gb300.cu after its extern "C" block.
//
// For the basis rows V[0..k] (each n doubles, row stride ldv) and w = A z:
//   h  = V w,  w -= V^T h,  h2 = V w,  w -= V^T h2,
//   hcol[j] = h[j] + h2[j] (j <= k), hcol[k+1] = |w|, V[k+1] = w / |w|.
// Three passes over V: the first dot products; the first update fused with
// the second dot products (the dots re-read the block's rows of V just
// loaded, from L1/L2); the second update fused with the norm.  Every reduction is over
// fixed chunks of rows, summed chunk by chunk in order, so the result does
// not depend on the stream or on how many blocks run at once.

#pragma once

namespace fe_gm {

constexpr int NT = 256;      // threads per block
constexpr int RPT = 4;       // rows per thread
constexpr int CHUNK = NT * RPT;
constexpr int MAXK = 128;    // basis rows

__device__ __forceinline__ double block_sum(double v, double *red) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int q = 0; q < NT / 32; q++) s += red[q];
  return s;   // thread 0 only
}

// part[b * (k + 1) + j] = sum over chunk b of V[j][i] x[i]   (x = w)
// with `h`: first x[i] -= sum_j V[j][i] h[j] (written back), then the dots.
// The chunk's x is staged in shared memory; each warp then takes basis rows
// j = warp, warp + 8, ...: 32 independent loads per lane, a shuffle
// reduction, no barrier in the loop (lane-strided sums, then the xor tree:
// a fixed order)
__global__ void __launch_bounds__(NT) k_cgs_pass(const double *__restrict__ V, long long ldv, long long n, int k,
                                                 double *__restrict__ w, const double *__restrict__ h,
                                                 double *__restrict__ part) {
  __shared__ double xs[CHUNK];
  __shared__ double hs[MAXK];
  const long long base = (long long)blockIdx.x * CHUNK;
  if (h)
    for (int j = threadIdx.x; j <= k; j += NT) hs[j] = h[j];
  __syncthreads();
#pragma unroll
  for (int q = 0; q < RPT; q++) {
    const long long i = base + q * NT + threadIdx.x;
    double x = i < n ? w[i] : 0.0;
    if (h && i < n) {
      double s0 = 0.0, s1 = 0.0;
      int j = 0;
      for (; j + 1 <= k; j += 2) {
        s0 = fma(V[(long long)j * ldv + i], hs[j], s0);
        s1 = fma(V[(long long)(j + 1) * ldv + i], hs[j + 1], s1);
      }
      if (j <= k) s0 = fma(V[(long long)j * ldv + i], hs[j], s0);
      x -= s0 + s1;
      w[i] = x;
    }
    xs[q * NT + threadIdx.x] = x;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int lim = (int)min((long long)CHUNK, n - base);
  for (int j = warp; j <= k; j += NT / 32) {
    const double *vj = V + (long long)j * ldv + base;
    double s = 0.0;
#pragma unroll 8
    for (int t = lane; t < lim; t += 32) s = fma(vj[t], xs[t], s);
#pragma unroll
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) part[(long long)blockIdx.x * (k + 1) + j] = s;
  }
}

// out[j] = sum over blocks of part[b * (k + 1) + j] (+ add[j]): one block
// per j, thread t summing blocks t, t + NT, ... in order, then the block's
// fixed tree (block_sum)
__global__ void __launch_bounds__(NT) k_cgs_reduce(const double *__restrict__ part, int nb, int k,
                                                   double *__restrict__ out, const double *__restrict__ add) {
  __shared__ double red[NT / 32];
  const int j = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += NT) s += part[(long long)b * (k + 1) + j];
  s = block_sum(s, red);
  if (threadIdx.x == 0) out[j] = add ? add[j] + s : s;
}

// w -= V^T h2 and the chunks' sums of w^2
__global__ void __launch_bounds__(NT) k_cgs_update_norm(const double *__restrict__ V, long long ldv, long long n,
                                                        int k, double *__restrict__ w, const double *__restrict__ h,
                                                        double *__restrict__ part) {
  __shared__ double red[NT / 32];
  __shared__ double hs[MAXK];
  const long long base = (long long)blockIdx.x * CHUNK;
  for (int j = threadIdx.x; j <= k; j += NT) hs[j] = h[j];
  __syncthreads();
  double ss = 0.0;
#pragma unroll
  for (int q = 0; q < RPT; q++) {
    const long long i = base + q * NT + threadIdx.x;
    if (i >= n) continue;
    double s0 = 0.0, s1 = 0.0;
    int j = 0;
    for (; j + 1 <= k; j += 2) {
      s0 = fma(V[(long long)j * ldv + i], hs[j], s0);
      s1 = fma(V[(long long)(j + 1) * ldv + i], hs[j + 1], s1);
    }
    if (j <= k) s0 = fma(V[(long long)j * ldv + i], hs[j], s0);
    const double x = w[i] - (s0 + s1);
    w[i] = x;
    ss = fma(x, x, ss);
  }
  ss = block_sum(ss, red);
  if (threadIdx.x == 0) part[blockIdx.x] = ss;
}

// hcol[k+1] = |w| from the chunks' sums (the reduction of k_cgs_reduce);
// then V[k+1] = w / |w| (0 if |w| = 0)
__global__ void __launch_bounds__(NT) k_cgs_norm(const double *__restrict__ part, int nb,
                                                 double *__restrict__ hcol, int k) {
  __shared__ double red[NT / 32];
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += NT) s += part[b];
  s = block_sum(s, red);
  if (threadIdx.x == 0) hcol[k + 1] = sqrt(s);
}

__global__ void k_cgs_scale(const double *__restrict__ w, const double *__restrict__ hcol, int k,
                            double *__restrict__ vnext, long long n) {
  const double nw = hcol[k + 1];
  const double inv = nw > 1e-300 ? 1.0 / nw : 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    vnext[i] = w[i] * inv;
}

// the FP32 preconditioner's vector steps (the library's own kernels: torch's
// FP32 kernels cost seconds at their first use in a process on this machine)
__global__ void k_gather_cast_f32(const double *__restrict__ src, const int64_t *__restrict__ idx, long long n,
                                  const float *__restrict__ scale, float *__restrict__ dst) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float v = (float)src[idx[i]];
    dst[i] = scale ? scale[i] * v : v;
  }
}

__global__ void k_sub_mul_f32(const float *__restrict__ a, const float *__restrict__ b,
                              const float *__restrict__ d, float *__restrict__ c, float *__restrict__ x,
                              long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float t = b ? a[i] - b[i] : a[i];
    if (c) c[i] = t;
    x[i] = d[i] * t;
  }
}

__global__ void k_scatter_cast_f64(const float *__restrict__ src, const int64_t *__restrict__ idx, long long n,
                                   double *__restrict__ dst) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[idx[i]] = (double)src[i];
}

} // namespace fe_gm

extern "C" {

int fe_gather_cast_f32(const double *src, const int64_t *idx, int64_t n, const float *scale, float *dst,
                       void *stream) {
  if (n < 0 || (n > 0 && (!src || !idx || !dst))) return fail(FE_ERR_ARG, "fe_gather_cast_f32: bad arguments");
  if (n == 0) return FE_OK;
  fe_gm::k_gather_cast_f32<<<grid_for(n, 256, sm_count_cached()), 256, 0, (cudaStream_t)stream>>>(src, idx, n, scale,
                                                                                                  dst);
  CUDA_TRY(cudaGetLastError());
  return FE_OK;
}

int fe_sub_mul_f32(const float *a, const float *b, const float *d, float *c, float *x, int64_t n, void *stream) {
  if (n < 0 || (n > 0 && (!a || !d || !x))) return fail(FE_ERR_ARG, "fe_sub_mul_f32: bad arguments");
  if (n == 0) return FE_OK;
  fe_gm::k_sub_mul_f32<<<grid_for(n, 256, sm_count_cached()), 256, 0, (cudaStream_t)stream>>>(a, b, d, c, x, n);
  CUDA_TRY(cudaGetLastError());
  return FE_OK;
}

int fe_scatter_cast_f64(const float *src, const int64_t *idx, int64_t n, double *dst, void *stream) {
  if (n < 0 || (n > 0 && (!src || !idx || !dst))) return fail(FE_ERR_ARG, "fe_scatter_cast_f64: bad arguments");
  if (n == 0) return FE_OK;
  fe_gm::k_scatter_cast_f64<<<grid_for(n, 256, sm_count_cached()), 256, 0, (cudaStream_t)stream>>>(src, idx, n, dst);
  CUDA_TRY(cudaGetLastError());
  return FE_OK;
}

int64_t fe_gmres_cgs2_scratch(int64_t n, int kmax) {
  const int64_t nb = (n + fe_gm::CHUNK - 1) / fe_gm::CHUNK;
  return nb * (int64_t)(kmax + 2) + 2 * (int64_t)(kmax + 2);
}

int fe_gmres_cgs2(double *V, int64_t ldv, int64_t n, int k, double *w, double *hcol, double *work, void *stream) {
  using namespace fe_gm;
  if (!V || !w || !hcol || !work || n <= 0 || k < 0 || k + 2 > MAXK || ldv < n)
    return fail(FE_ERR_ARG, "fe_gmres_cgs2: bad arguments (k + 2 <= %d rows)", MAXK);
  cudaStream_t st = (cudaStream_t)stream;
  const long long nb = (n + CHUNK - 1) / CHUNK;
  if (nb > 0x7fffffffLL) return fail(FE_ERR_ARG, "fe_gmres_cgs2: vector too long");
  double *part = work, *h = work + nb * (k + 2), *h2 = h + (k + 2);
  const unsigned rb = (unsigned)(k + 1);
  // h = V w
  k_cgs_pass<<<(unsigned)nb, NT, 0, st>>>(V, ldv, n, k, w, nullptr, part);
  k_cgs_reduce<<<rb, NT, 0, st>>>(part, (int)nb, k, h, nullptr);
  // w -= V^T h; h2 = V w
  k_cgs_pass<<<(unsigned)nb, NT, 0, st>>>(V, ldv, n, k, w, h, part);
  k_cgs_reduce<<<rb, NT, 0, st>>>(part, (int)nb, k, h2, nullptr);
  // w -= V^T h2, |w|
  k_cgs_update_norm<<<(unsigned)nb, NT, 0, st>>>(V, ldv, n, k, w, h2, part);
  k_cgs_norm<<<1, NT, 0, st>>>(part, (int)nb, hcol, k);
  // hcol[j] = h[j] + h2[j]; V[k+1] = w / |w|
  k_cgs_reduce<<<rb, NT, 0, st>>>(h2, 1, k, hcol, h);
  k_cgs_scale<<<grid_for(n, 256, sm_count_cached()), 256, 0, st>>>(w, hcol, k, V + (long long)(k + 1) * ldv, n);
  CUDA_TRY(cudaGetLastError());
  return FE_OK;
}

} // extern "C"
