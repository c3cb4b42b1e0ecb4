// Message-passing network kernels for the learned warm start: a small graph
// network over the cells of a mesh (cells adjacent through interior faces)
// that predicts steady rho and u from per-cell geometry features.
//
// Weights are bfloat16 (a fp32 master copy lives with the optimiser);
// activations, accumulations and gradients are float32.  Every reduction has
// a fixed order (per-block partials combined in block order, the tensor
// core's own fixed summation inside a tile), so training is bitwise
// reproducible run to run.
//
// The dense layers and their weight gradients run on the tensor cores as
// warp-level mma.sync m16n8k8 TF32 products with FP32 accumulation.  A bf16
// weight is exact in TF32 (8 of TF32's 10 mantissa bits).  An FP32 operand x
// is split into hi = tf32(x) and lo = tf32(x - hi), which together carry 21
// of its 24 mantissa bits, and its products are formed as hi*w + lo*w (and
// hi*y + hi*yl + lo*y when both operands are FP32: the weight gradient), the
// split-precision scheme of Markidis et al., "NVIDIA Tensor Core
// Programmability, Performance & Precision" (IPDPSW 2018), restated here for
// TF32.  The result agrees with FP32 FMA accumulation to about 1e-6 relative.
#include <cuda_bf16.h>

#include <algorithm>

#include "../../include/fvdbm_mpnn.h"

namespace fvdbm {
namespace {

constexpr int DT = 256;       // threads per block of the dense kernels
constexpr int MAXK = 128;     // input width limit
constexpr int MAXO = 128;     // output width limit
constexpr int WG_MAX_ENTRIES = 64 * 128 + 64;  // weight-gradient entries per block (+ bias)

// TF32 helpers: round to nearest (ties away, cvt.rna) and the hi/lo split.
__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ void split_tf32(float x, uint32_t& hi, uint32_t& lo) {
  hi = to_tf32(x);
  lo = to_tf32(x - __uint_as_float(hi));
}

// D += A (16x8, row) * B (8x8, col), TF32 inputs, FP32 accumulators.
// Fragments (lane = 4*g + t): a0 (g, t), a1 (g+8, t), a2 (g, t+4),
// a3 (g+8, t+4); b0 (k t, n g), b1 (k t+4, n g); c0 (g, 2t), c1 (g, 2t+1),
// c2 (g+8, 2t), c3 (g+8, 2t+1).
__device__ __forceinline__ void mma_tf32(float c[4], const uint32_t a[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

constexpr int TCW = 8;               // warps per block of the tensor-core dense kernels
constexpr int TCM = 16 * TCW;        // cells per tile (16 rows per warp)
constexpr int TCO = MAXO;            // padded output width limit (multiple of 8)

// Asynchronous 16-byte global -> shared copies (cp.async.cg: through L2).
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const uint32_t d = uint32_t(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Rows [c0, c0 + TCM) of In = [Xa | Xb] into a tile [TCM][xsd]: 16-byte
// asynchronous copies when both parts' rows are 16-byte aligned (da, db
// multiples of 4 and aligned bases), else plain loads.  Rows past n are not
// written (their outputs are never stored); the pad columns [K, Kp) are
// zeroed once by the caller.
__device__ __forceinline__ bool rows_vec4(const float* xa, int da, const float* xb, int db) {
  return (da % 4 == 0) && (db % 4 == 0) && ((reinterpret_cast<uintptr_t>(xa) & 15) == 0) &&
         (db == 0 || (reinterpret_cast<uintptr_t>(xb) & 15) == 0);
}
__device__ __forceinline__ void load_rows(float* xs, int xsd, const float* __restrict__ xa, int da,
                                          const float* __restrict__ xb, int db, int c0, int rows, int n,
                                          bool vec) {
  const int K = da + db;
  if (vec) {
    const int K4 = K / 4;
    for (int e = threadIdx.x; e < rows * K4; e += blockDim.x) {
      const int cc = e / K4, k = (e % K4) * 4, i = c0 + cc;
      if (i >= n) continue;
      const float* src = k < da ? xa + size_t(i) * da + k : xb + size_t(i) * db + (k - da);
      cp_async16(xs + cc * xsd + k, src);
    }
  } else {
    for (int e = threadIdx.x; e < rows * K; e += blockDim.x) {
      const int cc = e / K, k = e % K, i = c0 + cc;
      if (i >= n) continue;
      xs[cc * xsd + k] = k < da ? xa[size_t(i) * da + k] : xb[size_t(i) * db + (k - da)];
    }
  }
}

// Out[c][o] = sum_k In[c][k] * Wm[k][o] on the tensor cores; same arguments
// and epilogue as the dense layer above.  Shared memory: the weights as bf16
// bits [Kp][Op + 8] (zero padded) and two activation tiles [TCM][Kp + 4]
// (padded strides keep the fragment loads free of bank conflicts): the next
// tile streams in by cp.async while the warps multiply the current one.
// Each warp owns 16 cells of a tile and all Op/8 output column blocks.
template <bool TRANS>
__global__ void __launch_bounds__(TCW * 32) k_dense_tc(const float* __restrict__ xa, int da,
                                                       const float* __restrict__ xb, int db, int n,
                                                       const uint16_t* __restrict__ w,
                                                       const float* __restrict__ bias, int dout, int relu,
                                                       const float* __restrict__ residual, float* __restrict__ z,
                                                       float* __restrict__ ya, int split, int acc_a,
                                                       float* __restrict__ yb) {
  extern __shared__ float sm[];
  const int K = da + db;
  const int Kp = (K + 7) & ~7, Op = (dout + 7) & ~7;
  const int ws = Op + 8, xsd = Kp + 4;
  uint16_t* wm = reinterpret_cast<uint16_t*>(sm);                          // [Kp][ws]
  float* xbuf = sm + ((size_t(Kp) * ws + 1) / 2 + 3) / 4 * 4;               // [2][TCM][xsd]
  const size_t tile_floats = size_t(TCM) * xsd;
  const bool vec = rows_vec4(xa, da, xb, db);
  const int ntile = (n + TCM - 1) / TCM;
  int tile = blockIdx.x;
  // first tile in flight while the weights are staged
  if (tile < ntile) load_rows(xbuf, xsd, xa, da, xb, db, tile * TCM, TCM, n, vec);
  cp_async_commit();
  for (int e = threadIdx.x; e < Kp * ws; e += blockDim.x) {
    const int k = e / ws, o = e % ws;
    uint16_t v = 0;
    if (k < K && o < dout) v = TRANS ? w[size_t(o) * K + k] : w[size_t(k) * dout + o];
    wm[e] = v;
  }
  if (Kp > K)  // pad columns of both tiles: zero, never copied over
    for (int e = threadIdx.x; e < 2 * TCM * (Kp - K); e += blockDim.x) {
      const int r = e / (Kp - K), k = K + e % (Kp - K);
      xbuf[size_t(r) * xsd + k] = 0.0f;
    }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int NB = Op / 8;
  for (int it = 0; tile < ntile; tile += gridDim.x, ++it) {
    float* xs = xbuf + (it & 1) * tile_floats;
    const int next = tile + int(gridDim.x);
    if (next < ntile) load_rows(xbuf + ((it + 1) & 1) * tile_floats, xsd, xa, da, xb, db, next * TCM, TCM, n, vec);
    cp_async_commit();
    cp_async_wait<1>();  // this tile's copies have landed (the next one's may still fly)
    __syncthreads();
    const int c0 = tile * TCM;
    float acc[TCO / 8][4];
#pragma unroll
    for (int j = 0; j < TCO / 8; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[j][r] = 0.0f;
    const float* xr = xs + (warp * 16) * xsd;
    for (int k0 = 0; k0 < Kp; k0 += 8) {
      uint32_t ah[4], al[4];
      split_tf32(xr[g * xsd + k0 + t], ah[0], al[0]);
      split_tf32(xr[(g + 8) * xsd + k0 + t], ah[1], al[1]);
      split_tf32(xr[g * xsd + k0 + t + 4], ah[2], al[2]);
      split_tf32(xr[(g + 8) * xsd + k0 + t + 4], ah[3], al[3]);
      const uint16_t* w0 = wm + (k0 + t) * ws + g;
      const uint16_t* w1 = wm + (k0 + t + 4) * ws + g;
#pragma unroll
      for (int j = 0; j < TCO / 8; ++j) {
        if (j < NB) {
          const uint32_t b0 = uint32_t(w0[8 * j]) << 16, b1 = uint32_t(w1[8 * j]) << 16;
          mma_tf32(acc[j], al, b0, b1);
          mma_tf32(acc[j], ah, b0, b1);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < TCO / 8; ++j) {
      if (j >= NB) break;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int i = c0 + warp * 16 + g + (r >= 2 ? 8 : 0);
        const int o = 8 * j + 2 * t + (r & 1);
        if (i >= n || o >= dout) continue;
        const float a = acc[j][r];
        if (TRANS) {
          const float zz = a + (bias ? bias[o] : 0.0f);
          if (z) z[size_t(i) * dout + o] = zz;
          float yy = relu ? fmaxf(zz, 0.0f) : zz;
          if (residual) yy += residual[size_t(i) * dout + o];
          ya[size_t(i) * dout + o] = yy;
        } else if (o < split) {
          float* p = ya + size_t(i) * split + o;
          *p = acc_a ? *p + a : a;
        } else {
          yb[size_t(i) * (dout - split) + (o - split)] = a;
        }
      }
    }
    __syncthreads();  // the tile is consumed before the buffer is refilled
  }
  cp_async_wait<0>();
}

size_t dense_tc_smem(int K, int dout) {
  const int Kp = (K + 7) & ~7, Op = (dout + 7) & ~7;
  const size_t wfl = ((size_t(Kp) * (Op + 8) + 1) / 2 + 3) / 4 * 4;
  return sizeof(float) * (wfl + 2 * size_t(TCM) * (Kp + 4));
}

// Weight gradient on the tensor cores: per block (a fixed range of `chunk`
// cells) partial dW[o][k] = sum_c dz[c][o] x[c][k] and db[o] = sum_c dz[c][o]
// (the bias as a column of ones appended to x).  M = dout (padded to 16s),
// N = K + 1 (padded to 8s), reduction over the cells in steps of 8; both
// operands FP32, split hi/lo: hi*hi + hi*lo + lo*hi.  Warp w owns m-tile
// (w % MT) and the n-blocks w / MT, w / MT + NW, ...
constexpr int WCT = 64;  // cells per staged slab
__global__ void __launch_bounds__(TCW * 32) k_dense_wgrad_tc(const float* __restrict__ dz, int n, int dout,
                                                            const float* __restrict__ xa, int da,
                                                            const float* __restrict__ xb, int db, int chunk,
                                                            float* __restrict__ part) {
  extern __shared__ float sm[];
  const int K = da + db;
  const int Mp = (dout + 15) & ~15, Np = (K + 1 + 7) & ~7;
  const int zsd = Mp + 4, xsd = Np + 8;
  const size_t slab = size_t(WCT) * (zsd + xsd);  // one buffer: dz slab, then x slab
  // two buffers [zs | xs]: cells x outputs, cells x inputs (+ ones column)
  for (int e = threadIdx.x; e < int(2 * slab); e += blockDim.x) {
    const int bsel = e / int(slab), r = e % int(slab);  // buffer, offset in it
    float v = 0.0f;
    if (r >= WCT * zsd && (r - WCT * zsd) % xsd == K) v = 1.0f;  // the bias column of ones
    (void)bsel;
    sm[e] = v;
  }
  __syncthreads();  // initialised before any copy lands on top of it
  const bool zvec = (dout % 4 == 0) && ((reinterpret_cast<uintptr_t>(dz) & 15) == 0);
  const bool xvec = rows_vec4(xa, da, xb, db);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int MT = Mp / 16, NBk = Np / 8;
  const int mt = warp % MT, NW = TCW / MT > 0 ? TCW / MT : 1;
  const bool active = warp < MT * NW;
  constexpr int MAXJ = (TCO + 8) / 8;  // n-blocks per warp, at most
  float acc[MAXJ][4];
#pragma unroll
  for (int j = 0; j < MAXJ; ++j)
#pragma unroll
    for (int r = 0; r < 4; ++r) acc[j][r] = 0.0f;
  const int b0 = blockIdx.x * chunk, b1 = min(n, b0 + chunk);
  // one slab of cells [s0, s0 + WCT) into buffer bsel; rows past b1 of the
  // dz slab are zeroed (they are summed over), x rows keep finite old values
  auto stage = [&](int s0, int bsel) {
    float* zs = sm + bsel * slab;
    float* xs = zs + WCT * zsd;
    const int rows = min(WCT, b1 - s0);
    if (zvec) {
      const int O4 = dout / 4;
      for (int e = threadIdx.x; e < rows * O4; e += blockDim.x) {
        const int cc = e / O4, o = (e % O4) * 4;
        cp_async16(zs + cc * zsd + o, dz + size_t(s0 + cc) * dout + o);
      }
    } else {
      for (int e = threadIdx.x; e < rows * dout; e += blockDim.x) {
        const int cc = e / dout, o = e % dout;
        zs[cc * zsd + o] = dz[size_t(s0 + cc) * dout + o];
      }
    }
    for (int e = threadIdx.x; e < (WCT - rows) * dout; e += blockDim.x) {
      const int cc = rows + e / dout, o = e % dout;
      zs[cc * zsd + o] = 0.0f;
    }
    load_rows(xs, xsd, xa, da, xb, db, s0, rows, b1, xvec);
  };
  int it = 0;
  if (b0 < b1) stage(b0, 0);
  cp_async_commit();
  for (int s0 = b0; s0 < b1; s0 += WCT, ++it) {
    if (s0 + WCT < b1) stage(s0 + WCT, (it + 1) & 1);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const float* zs = sm + (it & 1) * slab;
    const float* xs = zs + WCT * zsd;
    if (active) {
      for (int c8 = 0; c8 < WCT; c8 += 8) {
        // A = dz^T: rows o (m-tile), cols = cells c8..c8+7
        uint32_t ah[4], al[4];
        const int o0 = mt * 16;
        split_tf32(zs[(c8 + t) * zsd + o0 + g], ah[0], al[0]);
        split_tf32(zs[(c8 + t) * zsd + o0 + g + 8], ah[1], al[1]);
        split_tf32(zs[(c8 + t + 4) * zsd + o0 + g], ah[2], al[2]);
        split_tf32(zs[(c8 + t + 4) * zsd + o0 + g + 8], ah[3], al[3]);
#pragma unroll
        for (int j = 0; j < MAXJ; ++j) {
          const int nb = warp / MT + j * NW;
          if (nb < NBk) {
            uint32_t bh0, bl0, bh1, bl1;
            split_tf32(xs[(c8 + t) * xsd + nb * 8 + g], bh0, bl0);
            split_tf32(xs[(c8 + t + 4) * xsd + nb * 8 + g], bh1, bl1);
            mma_tf32(acc[j], al, bh0, bh1);
            mma_tf32(acc[j], ah, bl0, bl1);
            mma_tf32(acc[j], ah, bh0, bh1);
          }
        }
      }
    }
    __syncthreads();  // the slab is consumed before its buffer is refilled
  }
  cp_async_wait<0>();
  if (!active) return;
  const int E = dout * K + dout;
#pragma unroll
  for (int j = 0; j < MAXJ; ++j) {
    const int nb = warp / MT + j * NW;
    if (nb >= NBk) break;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int o = mt * 16 + g + (r >= 2 ? 8 : 0);
      const int k = nb * 8 + 2 * t + (r & 1);
      if (o >= dout || k > K) continue;
      const int e = k < K ? o * K + k : dout * K + o;
      part[size_t(blockIdx.x) * E + e] = acc[j][r];
    }
  }
}

size_t wgrad_tc_smem(int K, int dout) {
  const int Mp = (dout + 15) & ~15, Np = (K + 1 + 7) & ~7;
  return 2 * sizeof(float) * size_t(WCT) * ((Mp + 4) + (Np + 8));
}

static int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  }
  return n;
}

// Dense layer semantics (k_dense_tc): Out[c][o] = sum_k In[c][k] * Wm[k][o]
// (+ bias[o]), In = [Xa | Xb].  Wm is W^T (forward, W [O][K]) or W itself
// (backward data, W [K][O]).  Epilogue: z = pre-activation (optional store),
// y = act(z) (+ residual).  Backward-data form: out columns [0, split) go to
// ya (accumulated when acc_a), the rest to yb.

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

// Long rows in chunks: pass 1 folds each chunk's entries (at most a few
// dozen, in order) per feature into partial[chunk][f]; pass 2 folds a row's
// chunk partials in chunk order.  Fixed order throughout: reproducible.
__global__ void k_spmm_chunks(const int* __restrict__ chunk_start, const int* __restrict__ col,
                              const float* __restrict__ wt, int nchunks, const float* __restrict__ h, int d,
                              float* __restrict__ partial) {
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int c = int(t / d), f = int(t % d);
  if (c >= nchunks) return;
  float s = 0.0f;
  for (int e = chunk_start[c]; e < chunk_start[c + 1]; ++e) s = fmaf(wt[e], h[size_t(col[e]) * d + f], s);
  partial[size_t(c) * d + f] = s;
}

__global__ void k_spmm_rows(const int* __restrict__ chunk_ptr, int n, const float* __restrict__ partial, int d,
                            float* __restrict__ out, int accumulate) {
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int i = int(t / d), f = int(t % d);
  if (i >= n) return;
  float s = 0.0f;
  for (int c = chunk_ptr[i]; c < chunk_ptr[i + 1]; ++c) s += partial[size_t(c) * d + f];
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
  const size_t smem = dense_tc_smem(K, dout);
  auto kern = k_dense_tc<true>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) return -2;
  const int g = std::min(nblk(n, TCM), sm_count() * 2);
  kern<<<g, TCW * 32, smem, static_cast<cudaStream_t>(stream)>>>(xa, da, xb, db, n, w, bias, dout, relu, residual,
                                                                 z, y, 0, 0, nullptr);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int fvdbm_mp_dense_bwd_data(const float* dz, int32_t n, int32_t dout, const uint16_t* w, int32_t da, int32_t db,
                            float* dxa, int32_t acc_a, float* dxb, void* stream) {
  if (n < 0 || dout <= 0 || dout > MAXK || da <= 0 || db < 0 || da + db > MAXO || !dz || !w || !dxa ||
      (db > 0 && !dxb))
    return -1;
  if (n == 0) return 0;
  const int K = dout, O = da + db;
  const size_t smem = dense_tc_smem(K, O);
  auto kern = k_dense_tc<false>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess) return -2;
  const int g = std::min(nblk(n, TCM), sm_count() * 2);
  kern<<<g, TCW * 32, smem, static_cast<cudaStream_t>(stream)>>>(dz, dout, nullptr, 0, n, w, nullptr, O, 0, nullptr,
                                                                 nullptr, dxa, da, acc_a, dxb);
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

size_t fvdbm_mp_wgrad_scratch(int32_t n, int32_t dout, int32_t din) {
  const int chunk = 1024;  // cells per block of the weight gradient
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
  const int chunk = 1024;  // cells per block of the weight gradient
  const int parts = (n + chunk - 1) / chunk;
  const int E = dout * K + dout;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t smem = wgrad_tc_smem(K, dout);
  if (cudaFuncSetAttribute(k_dense_wgrad_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) != cudaSuccess)
    return -2;
  k_dense_wgrad_tc<<<parts, TCW * 32, smem, s>>>(dz, n, dout, xa, da, xb, db, chunk, scratch);
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

int fvdbm_mp_spmm_chunked(const int32_t* chunk_start, const int32_t* chunk_ptr, int32_t nchunks, const int32_t* col,
                          const float* wt, int32_t n, const float* h, int32_t d, float* out, int32_t accumulate,
                          float* partial, void* stream) {
  if (n < 0 || nchunks < 0 || d <= 0 || !chunk_start || !chunk_ptr || !col || !wt || !h || !out ||
      (nchunks > 0 && !partial))
    return -1;
  if (n == 0) return 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (nchunks > 0)
    k_spmm_chunks<<<nblk(size_t(nchunks) * d, 256), 256, 0, s>>>(chunk_start, col, wt, nchunks, h, d, partial);
  k_spmm_rows<<<nblk(size_t(n) * d, 256), 256, 0, s>>>(chunk_ptr, n, partial, d, out, accumulate);
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
