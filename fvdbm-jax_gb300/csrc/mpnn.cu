// Message-passing network kernels for the learned warm start: a small graph
// network over the cells of a mesh (cells adjacent through interior faces)
// that predicts steady rho and u from per-cell geometry features.
//
// Weights are bfloat16 (a fp32 master copy lives with the optimiser);
// activations, accumulations and gradients are float32.  Every reduction has
// a fixed order (per-block partials combined in block order), so training is
// bitwise reproducible run to run.  The layers are small (64 hidden units):
// the work is bound by reading the activations, so the kernels stage
// activation tiles and the (converted) weights in shared memory and use FP32
// FMAs.
#include <cuda_bf16.h>

#include <algorithm>

#include "../../include/fvdbm_mpnn.h"

namespace fvdbm {
namespace {

constexpr int DT = 256;       // threads per block of the dense kernels
constexpr int TC = 32;        // cells per tile
constexpr int GROUPS = DT / TC;  // threads per cell
constexpr int MAXK = 128;     // input width limit
constexpr int MAXO = 128;     // output width limit
constexpr int WG_MAX_ENTRIES = 64 * 128 + 64;  // weight-gradient entries per block (+ bias)

__device__ __forceinline__ float bf16f(uint16_t w) { return __uint_as_float(uint32_t(w) << 16); }

static int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  }
  return n;
}

// Out[c][o] = sum_k In[c][k] * Wm[k][o] (+ bias[o]), In = [Xa | Xb].  Wm is
// W^T (forward, W [O][K]) or W itself (backward data, W [K][O]).  Epilogue:
// z = pre-activation (optional store), y = act(z) (+ residual).
// Backward-data form: out columns [0, split) go to ya (accumulated when
// acc_a), the rest to yb.
template <bool TRANS>
__global__ void __launch_bounds__(DT) k_dense(const float* __restrict__ xa, int da, const float* __restrict__ xb,
                                              int db, int n, const uint16_t* __restrict__ w,
                                              const float* __restrict__ bias, int dout, int relu,
                                              const float* __restrict__ residual, float* __restrict__ z,
                                              float* __restrict__ ya, int split, int acc_a,
                                              float* __restrict__ yb) {
  extern __shared__ float sm[];
  const int K = da + db;
  float* wm = sm;                       // [K][dout]
  float* xs = sm + K * dout;            // [TC][K + 1]
  for (int e = threadIdx.x; e < K * dout; e += DT) {
    const int k = e / dout, o = e % dout;
    wm[e] = TRANS ? bf16f(w[size_t(o) * K + k]) : bf16f(w[size_t(k) * dout + o]);
  }
  const int c = threadIdx.x / GROUPS, g = threadIdx.x % GROUPS;
  const int ntile = (n + TC - 1) / TC;
  for (int t = blockIdx.x; t < ntile; t += gridDim.x) {
    __syncthreads();  // weights ready / previous tile consumed
    const int c0 = t * TC;
    for (int e = threadIdx.x; e < TC * K; e += DT) {
      const int cc = e / K, k = e % K;
      const int i = c0 + cc;
      float v = 0.0f;
      if (i < n) v = k < da ? xa[size_t(i) * da + k] : xb[size_t(i) * db + (k - da)];
      xs[cc * (K + 1) + k] = v;
    }
    __syncthreads();
    const int i = c0 + c;
    float acc[MAXO / GROUPS];
#pragma unroll
    for (int j = 0; j < MAXO / GROUPS; ++j) acc[j] = 0.0f;
    const float* xr = xs + c * (K + 1);
    for (int k = 0; k < K; ++k) {
      const float a = xr[k];
      const float* wr = wm + k * dout;
#pragma unroll
      for (int j = 0; j < MAXO / GROUPS; ++j) {
        const int o = g + GROUPS * j;
        if (o < dout) acc[j] = fmaf(a, wr[o], acc[j]);
      }
    }
    if (i >= n) continue;
#pragma unroll
    for (int j = 0; j < MAXO / GROUPS; ++j) {
      const int o = g + GROUPS * j;
      if (o >= dout) break;
      if (TRANS) {
        const float zz = acc[j] + (bias ? bias[o] : 0.0f);
        if (z) z[size_t(i) * dout + o] = zz;
        float yy = relu ? fmaxf(zz, 0.0f) : zz;
        if (residual) yy += residual[size_t(i) * dout + o];
        ya[size_t(i) * dout + o] = yy;
      } else if (o < split) {
        float* p = ya + size_t(i) * split + o;
        *p = acc_a ? *p + acc[j] : acc[j];
      } else {
        yb[size_t(i) * (dout - split) + (o - split)] = acc[j];
      }
    }
  }
}

// Per block (a fixed range of `chunk` cells): partial dW[o][k] = sum dz[c][o]
// x[c][k] and db[o] = sum dz[c][o], entries strided over the threads.
__global__ void __launch_bounds__(DT) k_dense_wgrad(const float* __restrict__ dz, int n, int dout,
                                                    const float* __restrict__ xa, int da,
                                                    const float* __restrict__ xb, int db, int chunk,
                                                    float* __restrict__ part) {
  extern __shared__ float sm[];
  const int K = da + db;
  float* zs = sm;                 // [TC][dout]
  float* xs = sm + TC * dout;     // [TC][K]
  const int E = dout * K + dout;  // weight entries, then bias entries
  constexpr int PER = (WG_MAX_ENTRIES + DT - 1) / DT;
  float acc[PER];
#pragma unroll
  for (int j = 0; j < PER; ++j) acc[j] = 0.0f;
  const int b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
  for (int c0 = b0; c0 < b1; c0 += TC) {
    __syncthreads();
    for (int e = threadIdx.x; e < TC * dout; e += DT) {
      const int cc = e / dout, o = e % dout, i = c0 + cc;
      zs[e] = (i < b1) ? dz[size_t(i) * dout + o] : 0.0f;
    }
    for (int e = threadIdx.x; e < TC * K; e += DT) {
      const int cc = e / K, k = e % K, i = c0 + cc;
      float v = 0.0f;
      if (i < b1) v = k < da ? xa[size_t(i) * da + k] : xb[size_t(i) * db + (k - da)];
      xs[e] = v;
    }
    __syncthreads();
    const int nc = min(TC, b1 - c0);
#pragma unroll
    for (int j = 0; j < PER; ++j) {
      const int e = threadIdx.x + DT * j;
      if (e >= E) break;
      const int o = e < dout * K ? e / K : e - dout * K;
      const int k = e < dout * K ? e % K : -1;
      float s = acc[j];
      for (int cc = 0; cc < nc; ++cc) s = fmaf(zs[cc * dout + o], k >= 0 ? xs[cc * K + k] : 1.0f, s);
      acc[j] = s;
    }
  }
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int e = threadIdx.x + DT * j;
    if (e < E) part[size_t(blockIdx.x) * E + e] = acc[j];
  }
}

// Sum of the block partials in block order.
__global__ void k_sum_parts(const float* __restrict__ part, int nparts, int E, float* __restrict__ dw,
                            float* __restrict__ dbias, int wentries) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= E) return;
  float s = 0.0f;
  for (int b = 0; b < nparts; ++b) s += part[size_t(b) * E + e];
  if (e < wentries)
    dw[e] = s;
  else if (dbias)
    dbias[e - wentries] = s;
}

__global__ void k_relu_bwd(const float* __restrict__ dy, const float* __restrict__ z, float* __restrict__ dz,
                           size_t count) {
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t < count) dz[t] = z[t] > 0.0f ? dy[t] : 0.0f;
}

// out[i][d] (+)= sum_e wt[e] * h[col[e]][d] over the row's entries in order
__global__ void k_spmm(const int* __restrict__ row_ptr, const int* __restrict__ col,
                       const float* __restrict__ wt, int n, const float* __restrict__ h, int d,
                       float* __restrict__ out, int accumulate) {
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int i = int(t / d), f = int(t % d);
  if (i >= n) return;
  float s = 0.0f;
  for (int e = row_ptr[i]; e < row_ptr[i + 1]; ++e) s = fmaf(wt[e], h[size_t(col[e]) * d + f], s);
  float* o = out + size_t(i) * d + f;
  *o = accumulate ? *o + s : s;
}

// dy = 2 (y - t) m / count_m; per-block partial sums of m (y - t)^2
__global__ void k_mse(const float* __restrict__ y, const float* __restrict__ tg, const float* __restrict__ mask,
                      size_t count, float scale, float* __restrict__ dy, double* __restrict__ part) {
  __shared__ double sh[DT];
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (t < count) {
    const float m = mask ? mask[t] : 1.0f;
    const float r = y[t] - tg[t];
    dy[t] = 2.0f * r * m * scale;
    v = double(r) * double(r) * double(m);
  }
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = DT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void k_sum_double(const double* __restrict__ part, int nparts, double scale, double* __restrict__ out) {
  __shared__ double sh[DT];
  double v = 0.0;
  for (int b = threadIdx.x; b < nparts; b += DT) v += part[b];
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = DT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0] * scale;
}

// Adam on the fp32 master weights; the bf16 copy is rounded to nearest even.
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                       uint16_t* __restrict__ wb, const float* __restrict__ g, size_t count, float lr, float b1,
                       float b2, float eps, float c1, float c2) {
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const float gg = g[t];
  const float mm = b1 * m[t] + (1.0f - b1) * gg;
  const float vv = b2 * v[t] + (1.0f - b2) * gg * gg;
  m[t] = mm;
  v[t] = vv;
  const float ww = w[t] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
  w[t] = ww;
  if (wb) {
    const __nv_bfloat16 h = __float2bfloat16_rn(ww);
    wb[t] = *reinterpret_cast<const uint16_t*>(&h);
  }
}

__global__ void k_to_bf16(const float* __restrict__ x, uint16_t* __restrict__ y, size_t count) {
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const __nv_bfloat16 h = __float2bfloat16_rn(x[t]);
  y[t] = *reinterpret_cast<const uint16_t*>(&h);
}

inline int nblk(size_t n, int t) { return int((n + t - 1) / t); }

}  // namespace
}  // namespace fvdbm

using namespace fvdbm;

extern "C" {

int fvdbm_mp_dense_fwd(const float* xa, int32_t da, const float* xb, int32_t db, int32_t n, const uint16_t* w,
                       const float* bias, int32_t dout, int32_t relu, const float* residual, float* z, float* y,
                       void* stream) {
  if (n < 0 || da <= 0 || db < 0 || da + db > MAXK || dout <= 0 || dout > MAXO || (db > 0 && !xb) || !xa || !w ||
      !y)
    return -1;
  if (n == 0) return 0;
  const int K = da + db;
  const size_t smem = sizeof(float) * (size_t(K) * dout + size_t(TC) * (K + 1));
  auto kern = k_dense<true>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) return -2;
  const int g = std::min(nblk(n, TC), sm_count() * 4);
  kern<<<g, DT, smem, static_cast<cudaStream_t>(stream)>>>(xa, da, xb, db, n, w, bias, dout, relu, residual, z,
                                                           y, 0, 0, nullptr);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int fvdbm_mp_dense_bwd_data(const float* dz, int32_t n, int32_t dout, const uint16_t* w, int32_t da, int32_t db,
                            float* dxa, int32_t acc_a, float* dxb, void* stream) {
  if (n < 0 || dout <= 0 || dout > MAXK || da <= 0 || db < 0 || da + db > MAXO || !dz || !w || !dxa ||
      (db > 0 && !dxb))
    return -1;
  if (n == 0) return 0;
  const int K = dout, O = da + db;
  const size_t smem = sizeof(float) * (size_t(K) * O + size_t(TC) * (K + 1));
  auto kern = k_dense<false>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) return -2;
  const int g = std::min(nblk(n, TC), sm_count() * 4);
  kern<<<g, DT, smem, static_cast<cudaStream_t>(stream)>>>(dz, dout, nullptr, 0, n, w, nullptr, O, 0, nullptr,
                                                           nullptr, dxa, da, acc_a, dxb);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

size_t fvdbm_mp_wgrad_scratch(int32_t n, int32_t dout, int32_t din) {
  const int chunk = 4096;
  const size_t parts = size_t((n + chunk - 1) / chunk);
  return sizeof(float) * std::max<size_t>(parts, 1) * (size_t(dout) * din + dout);
}

int fvdbm_mp_dense_bwd_weight(const float* dz, int32_t n, int32_t dout, const float* xa, int32_t da,
                              const float* xb, int32_t db, float* dw, float* dbias, float* scratch,
                              size_t scratch_bytes, void* stream) {
  const int K = da + db;
  if (n <= 0 || dout <= 0 || dout * K + dout > WG_MAX_ENTRIES || da <= 0 || db < 0 || K > MAXK || !dz || !xa ||
      (db > 0 && !xb) || !dw || !scratch || scratch_bytes < fvdbm_mp_wgrad_scratch(n, dout, K))
    return -1;
  const int chunk = 4096;
  const int parts = (n + chunk - 1) / chunk;
  const int E = dout * K + dout;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t smem = sizeof(float) * size_t(TC) * (dout + K);
  k_dense_wgrad<<<parts, DT, smem, s>>>(dz, n, dout, xa, da, xb, db, chunk, scratch);
  k_sum_parts<<<nblk(E, 256), 256, 0, s>>>(scratch, parts, E, dw, dbias, dout * K);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int fvdbm_mp_relu_bwd(const float* dy, const float* z, float* dz, size_t count, void* stream) {
  if (!dy || !z || !dz) return -1;
  if (count == 0) return 0;
  k_relu_bwd<<<nblk(count, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(dy, z, dz, count);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int fvdbm_mp_spmm(const int32_t* row_ptr, const int32_t* col, const float* wt, int32_t n, const float* h,
                  int32_t d, float* out, int32_t accumulate, void* stream) {
  if (n < 0 || d <= 0 || !row_ptr || !col || !wt || !h || !out) return -1;
  if (n == 0) return 0;
  k_spmm<<<nblk(size_t(n) * d, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(row_ptr, col, wt, n, h, d, out,
                                                                                 accumulate);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

size_t fvdbm_mp_mse_scratch(size_t count) { return sizeof(double) * (nblk(count, DT) + 1); }

int fvdbm_mp_mse(const float* y, const float* t, const float* mask, size_t count, float mask_total, float* dy,
                 double* scratch, size_t scratch_bytes, void* stream) {
  if (!y || !t || !dy || !scratch || count == 0 || mask_total <= 0.0f ||
      scratch_bytes < fvdbm_mp_mse_scratch(count))
    return -1;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nb = nblk(count, DT);
  k_mse<<<nb, DT, 0, s>>>(y, t, mask, count, 1.0f / mask_total, dy, scratch + 1);
  k_sum_double<<<1, DT, 0, s>>>(scratch + 1, nb, 1.0 / double(mask_total), scratch);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int fvdbm_mp_adam(float* w, float* m, float* v, uint16_t* wb, const float* g, size_t count, float lr, float b1,
                  float b2, float eps, int32_t step, void* stream) {
  if (!w || !m || !v || !g || step <= 0) return -1;
  if (count == 0) return 0;
  const float c1 = 1.0f - powf(b1, float(step)), c2 = 1.0f - powf(b2, float(step));
  k_adam<<<nblk(count, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(w, m, v, wb, g, count, lr, b1, b2, eps,
                                                                        c1, c2);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int fvdbm_mp_to_bf16(const float* x, uint16_t* y, size_t count, void* stream) {
  if (!x || !y) return -1;
  if (count == 0) return 0;
  k_to_bf16<<<nblk(count, 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(x, y, count);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

}  // extern "C"
