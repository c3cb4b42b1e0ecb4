// Jacobi-preconditioned conjugate gradients on the GPU: the potential-flow
// estimate of the warm start's features solves a cell Laplacian per case
// (all held-out cases together as one block-diagonal system).  No
// counterpart in the reference.
//
// Vectors are float32.  Every dot product is summed by each thread in
// float32 (multiply-adds; the rows of a thread are few) and then in double
// over the block and over the blocks in block order by one block, so an
// iteration is bitwise reproducible (float64 arithmetic is slow on this GPU,
// so it is kept to the reductions).  The scalars of the recurrence (alpha,
// beta, r.z) stay on the device; the host reads ||r||^2 every check_every
// iterations to stop.
//
// Recurrence (Saad, Iterative Methods for Sparse Linear Systems, 2nd ed.,
// Algorithm 9.1, with M = diag(A)):
//   r = b - A x, z = M^-1 r, p = z
//   repeat: q = A p; alpha = (r.z)/(p.q); x += alpha p; r -= alpha q;
//           z = M^-1 r; beta = (r.z)_new/(r.z); p = z + beta p
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "fvdbm.h"
#include "fvdbm_mpnn.h"

namespace {

constexpr int PT = 256;       // threads per block
constexpr int PB_MAX = 1216;  // blocks of the vector kernels (8 per SM of a 152-SM GB300, at most)

// scalar slots (double) at the start of the work buffer
enum { S_RZ = 0, S_RR, S_BB, S_PQ, S_ALPHA, S_BETA, S_COUNT = 8 };

// Row i of A times x, in entry order (column indices outside [0, n) are
// skipped, so a malformed matrix cannot read out of bounds).
__device__ __forceinline__ float row_dot(int n, const int* __restrict__ ip, const int* __restrict__ ix,
                                         const float* __restrict__ v, const float* __restrict__ x, int i) {
  float s = 0.0f;
  for (int e = ip[i]; e < ip[i + 1]; ++e) {
    const int c = ix[e];
    if (unsigned(c) < unsigned(n)) s += v[e] * x[c];
  }
  return s;
}

// Sum of up to 3 doubles over the block in a fixed order; thread 0 writes them.
template <int K>
__device__ __forceinline__ void block_sum_store(double v[K], double* __restrict__ out) {
  __shared__ double sh[PT / 32][K];
#pragma unroll
  for (int k = 0; k < K; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) sh[w][k] = v[k];
  __syncthreads();
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double s = sh[0][k];
      for (int j = 1; j < PT / 32; ++j) s += sh[j][k];
      out[k] = s;
    }
}

// diag^-1 (1 where the row has no positive diagonal), r = b - A x, z = r/diag,
// p = z; partials (r.z, r.r, b.b)
__global__ void __launch_bounds__(PT) k_init(int n, const int* __restrict__ ip, const int* __restrict__ ix,
                                            const float* __restrict__ v, const float* __restrict__ b,
                                            const float* __restrict__ x, float* __restrict__ dinv,
                                            float* __restrict__ r, float* __restrict__ z, float* __restrict__ p,
                                            double* __restrict__ part) {
  float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
  for (int i = blockIdx.x * PT + threadIdx.x; i < n; i += gridDim.x * PT) {
    float d = 0.0f;
    for (int e = ip[i]; e < ip[i + 1]; ++e)
      if (ix[e] == i) d += v[e];
    const float di = d > 0.0f ? 1.0f / d : 1.0f;
    const float ri = b[i] - row_dot(n, ip, ix, v, x, i);
    const float zi = ri * di;
    dinv[i] = di;
    r[i] = ri;
    z[i] = zi;
    p[i] = zi;
    a0 = __fmaf_rn(ri, zi, a0);
    a1 = __fmaf_rn(ri, ri, a1);
    a2 = __fmaf_rn(b[i], b[i], a2);
  }
  double acc[3] = {a0, a1, a2};
  block_sum_store<3>(acc, part + size_t(blockIdx.x) * 3);
}

// q = A p; partial p.q
__global__ void __launch_bounds__(PT) k_spmv(int n, const int* __restrict__ ip, const int* __restrict__ ix,
                                            const float* __restrict__ v, const float* __restrict__ p,
                                            float* __restrict__ q, double* __restrict__ part) {
  float a0 = 0.0f;
  for (int i = blockIdx.x * PT + threadIdx.x; i < n; i += gridDim.x * PT) {
    const float qi = row_dot(n, ip, ix, v, p, i);
    q[i] = qi;
    a0 = __fmaf_rn(p[i], qi, a0);
  }
  double acc[1] = {a0};
  block_sum_store<1>(acc, part + size_t(blockIdx.x) * 3);
}

// One block: sums the k-th partial of every block in block order.
// mode 0 (after init): rz, rr, bb.  mode 1: pq and alpha = rz / pq.
// mode 2: beta = rz_new / rz, rz = rz_new, rr.
__global__ void __launch_bounds__(PT) k_scalars(int nblk, const double* __restrict__ part, double* __restrict__ s,
                                               int mode) {
  double acc[3] = {0.0, 0.0, 0.0};
  for (int j = threadIdx.x; j < nblk; j += PT)
#pragma unroll
    for (int k = 0; k < 3; ++k) acc[k] += part[size_t(j) * 3 + k];
  __shared__ double tot[3];
  block_sum_store<3>(acc, tot);
  __syncthreads();
  if (threadIdx.x != 0) return;
  if (mode == 0) {
    s[S_RZ] = tot[0];
    s[S_RR] = tot[1];
    s[S_BB] = tot[2];
  } else if (mode == 1) {
    s[S_PQ] = tot[0];
    s[S_ALPHA] = tot[0] != 0.0 ? s[S_RZ] / tot[0] : 0.0;
  } else {
    s[S_BETA] = s[S_RZ] != 0.0 ? tot[0] / s[S_RZ] : 0.0;
    s[S_RZ] = tot[0];
    s[S_RR] = tot[1];
  }
}

// x += alpha p; r -= alpha q; z = r/diag; partials (r.z, r.r)
__global__ void __launch_bounds__(PT) k_update(int n, const double* __restrict__ s, const float* __restrict__ p,
                                              const float* __restrict__ q, const float* __restrict__ dinv,
                                              float* __restrict__ x, float* __restrict__ r, float* __restrict__ z,
                                              double* __restrict__ part) {
  const float a = float(s[S_ALPHA]);
  float a0 = 0.0f, a1 = 0.0f;
  for (int i = blockIdx.x * PT + threadIdx.x; i < n; i += gridDim.x * PT) {
    x[i] = __fmaf_rn(a, p[i], x[i]);
    const float ri = __fmaf_rn(-a, q[i], r[i]);
    const float zi = ri * dinv[i];
    r[i] = ri;
    z[i] = zi;
    a0 = __fmaf_rn(ri, zi, a0);
    a1 = __fmaf_rn(ri, ri, a1);
  }
  double acc[3] = {a0, a1, 0.0};
  block_sum_store<3>(acc, part + size_t(blockIdx.x) * 3);
}

// p = z + beta p
__global__ void __launch_bounds__(PT) k_direction(int n, const double* __restrict__ s, const float* __restrict__ z,
                                                 float* __restrict__ p) {
  const float bt = float(s[S_BETA]);
  for (int i = blockIdx.x * PT + threadIdx.x; i < n; i += gridDim.x * PT) p[i] = __fmaf_rn(bt, p[i], z[i]);
}

int grid_blocks(int n) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int g = (n + PT - 1) / PT;
  const int cap = sms > 0 ? sms * 8 : PB_MAX;
  if (g > cap) g = cap;
  if (g > PB_MAX) g = PB_MAX;
  return g < 1 ? 1 : g;
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

extern "C" size_t fvdbm_pcg_work_bytes(int32_t n) {
  if (n < 0) return 0;
  return align256(S_COUNT * sizeof(double)) + align256(size_t(PB_MAX) * 3 * sizeof(double)) +
         5 * align256(size_t(n) * sizeof(float));
}

extern "C" int fvdbm_pcg(int32_t n, const int32_t* indptr, const int32_t* indices, const float* values,
                         const float* b, float* x, int32_t max_iter, double rtol, int32_t check_every, void* work,
                         size_t work_bytes, void* stream, int32_t* iters, double* rel_res) {
  if (iters) *iters = 0;
  if (rel_res) *rel_res = 0.0;
  if (n < 0 || max_iter < 0 || check_every <= 0 || !(rtol >= 0.0)) return FVDBM_EINVAL;
  if (n == 0) return FVDBM_OK;
  if (!indptr || !indices || !values || !b || !x || !work || work_bytes < fvdbm_pcg_work_bytes(n))
    return FVDBM_EINVAL;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* w = static_cast<char*>(work);
  double* s = reinterpret_cast<double*>(w);
  w += align256(S_COUNT * sizeof(double));
  double* part = reinterpret_cast<double*>(w);
  w += align256(size_t(PB_MAX) * 3 * sizeof(double));
  float* vec[5];
  for (int k = 0; k < 5; ++k) {
    vec[k] = reinterpret_cast<float*>(w);
    w += align256(size_t(n) * sizeof(float));
  }
  float *dinv = vec[0], *r = vec[1], *z = vec[2], *p = vec[3], *q = vec[4];
  const int g = grid_blocks(n);
  double* hs = nullptr;
  if (cudaMallocHost(reinterpret_cast<void**>(&hs), 3 * sizeof(double)) != cudaSuccess) return FVDBM_ECUDA;
  int rc = FVDBM_OK;
  int it = 0;
  double rel = 0.0;
  auto read_rr = [&]() -> bool {
    if (cudaMemcpyAsync(hs, s, 3 * sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess) return false;
    return cudaStreamSynchronize(st) == cudaSuccess;
  };
  k_init<<<g, PT, 0, st>>>(n, indptr, indices, values, b, x, dinv, r, z, p, part);
  k_scalars<<<1, PT, 0, st>>>(g, part, s, 0);
  if (cudaGetLastError() != cudaSuccess || !read_rr()) {
    rc = FVDBM_ECUDA;
  } else {
    const double bn = hs[S_BB] > 0.0 ? hs[S_BB] : 1.0;
    rel = hs[S_RR] > 0.0 ? std::sqrt(hs[S_RR] / bn) : 0.0;
    while (it < max_iter && rel > rtol) {
      const int k = (max_iter - it) < check_every ? (max_iter - it) : check_every;
      for (int j = 0; j < k; ++j) {
        k_spmv<<<g, PT, 0, st>>>(n, indptr, indices, values, p, q, part);
        k_scalars<<<1, PT, 0, st>>>(g, part, s, 1);
        k_update<<<g, PT, 0, st>>>(n, s, p, q, dinv, x, r, z, part);
        k_scalars<<<1, PT, 0, st>>>(g, part, s, 2);
        k_direction<<<g, PT, 0, st>>>(n, s, z, p);
      }
      it += k;
      if (cudaGetLastError() != cudaSuccess || !read_rr()) {
        rc = FVDBM_ECUDA;
        break;
      }
      rel = hs[S_RR] > 0.0 ? std::sqrt(hs[S_RR] / bn) : 0.0;
      if (!(rel == rel)) break;  // NaN: not SPD or bad input; reported through rel_res
    }
  }
  cudaFreeHost(hs);
  if (iters) *iters = it;
  if (rel_res) *rel_res = rel;
  return rc;
}
