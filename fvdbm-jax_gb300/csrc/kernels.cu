// FVDBM step kernels for sm_103a (GB300): boundary nodes, the fused cell
// kernel, the staged face/gather pair, read-back helpers and the division
// self-check.  Arithmetic helpers live in fvdbm_math.cuh.
//
// Layout: cell pdfs are SoA [9][Np] float32 in device (renumbered) cell
// order; node state is SoA [9][Mp]; per-cell face slots are SoA [K][Np].
#include "fvdbm_math.cuh"

namespace fvdbm {

// ---------------------------------------------------------------------------
// Boundary nodes: Nodes.calc_pdfs (src/containers.py:339-404).  One group of
// 8 lanes per node: each lane evaluates one of the node's cells (macros, feq,
// the IDW products), then every lane folds the products in the reference's
// entry order through shuffles.  Velocity nodes (type 1) take rho =
// IDW(cell rho); density nodes (type 2) take u = IDW(cell u); both set pdf =
// feq(rho, u) + IDW(f - feq).
constexpr int NODE_LANES = 8;

__global__ void __launch_bounds__(128) k_nodes(DevPlan p, const float* __restrict__ f) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int m = tid / NODE_LANES;
  const int lane = threadIdx.x % NODE_LANES;
  if (m >= p.Mc) return;  // whole 8-lane group leaves together
  const unsigned mask = 0xFFu << (threadIdx.x & 24);
  const int b = __ldg(p.nd_ptr + m), e = __ldg(p.nd_ptr + m + 1);
  const size_t Np = p.Np;
  float ar = 0.0f, ax = 0.0f, ay = 0.0f, an[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) an[q] = 0.0f;
  bool first = true;
  for (int base = b; base < e; base += NODE_LANES) {
    const int j = base + lane;
    float xr = 0.0f, xx = 0.0f, xy = 0.0f, xn[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) xn[q] = 0.0f;
    if (j < e) {
      const unsigned code = __ldg(p.nd_cell + j);
      const int c = int(code & ~ND_NEQ_ZERO);
      const float w = __ldg(p.nd_w + j);
      float fc[Q], eq[Q];
#pragma unroll
      for (int q = 0; q < Q; ++q) fc[q] = __ldg(f + q * Np + c);
      float rho, ux, uy;
      macros(fc, rho, ux, uy);
      feq9(rho, ux, uy, p, eq);
      const bool zero = (code & ND_NEQ_ZERO) != 0;
      xr = rho * w;
      xx = ux * w;
      xy = uy * w;
#pragma unroll
      for (int q = 0; q < Q; ++q) xn[q] = (zero ? 0.0f : fc[q] - eq[q]) * w;
    }
    const int cnt = min(NODE_LANES, e - base);
    for (int t = 0; t < cnt; ++t) {
      const float vr = __shfl_sync(mask, xr, t, NODE_LANES);
      const float vx = __shfl_sync(mask, xx, t, NODE_LANES);
      const float vy = __shfl_sync(mask, xy, t, NODE_LANES);
      if (first) {
        ar = vr;
        ax = vx;
        ay = vy;
      } else {
        ar = ar + vr;
        ax = ax + vx;
        ay = ay + vy;
      }
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const float vn = __shfl_sync(mask, xn[q], t, NODE_LANES);
        an[q] = first ? vn : an[q] + vn;
      }
      first = false;
    }
  }
  if (__ldg(p.nd_npad + m) > 0) {
    // padded (-1, weight 0) entries gather the last cell: rho*0, u*0
    float fc[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) fc[q] = __ldg(f + q * Np + p.last_cell);
    float rho, ux, uy;
    macros(fc, rho, ux, uy);
    ar = first ? rho * 0.0f : ar + rho * 0.0f;
    ax = first ? ux * 0.0f : ax + ux * 0.0f;
    ay = first ? uy * 0.0f : ay + uy * 0.0f;
  }
  if (lane != 0) return;
  const float sw = __ldg(p.nd_sumw + m);
  const int type = __ldg(p.nd_type + m);
  float rho_p, ux_p, uy_p;
  if (type == 1) {
    rho_p = ar / sw;
    ux_p = p.node_vel[m];
    uy_p = p.node_vel[p.Mp + m];
    p.node_rho[m] = rho_p;
  } else {
    rho_p = p.node_rho[m];
    ux_p = ax / sw;
    uy_p = ay / sw;
    p.node_vel[m] = ux_p;
    p.node_vel[p.Mp + m] = uy_p;
  }
  float eqn[Q];
  feq9(rho_p, ux_p, uy_p, p, eqn);
#pragma unroll
  for (int q = 0; q < Q; ++q) p.node_pdf[size_t(q) * p.Mp + m] = eqn[q] + an[q] / sw;
}

// ---------------------------------------------------------------------------
// Fused cell kernel: macros, feq, the flux of each of the cell's faces
// (recomputed from the canonical slot-0/slot-1 pair, so both neighbours get
// bit-identical fluxes without a flux array or atomics), the signed flux sum
// and the BGK/explicit-Euler update (src/containers.py:107-121).
template <int SCHEME, int VARIANT, bool FIRST>
__device__ __forceinline__ void fused_face(const DevPlan& p, const float* __restrict__ fin, size_t Np,
                                           int i, int k, const float f[Q], float acc[Q]) {
  const size_t s = size_t(k) * Np + i;
  const int code = __ldg(p.hf_code + s);
  const float nx = __ldg(p.hf_nx + s), ny = __ldg(p.hf_ny + s);
  const float Ls = __ldg(p.hf_L + s);  // L * sigma
  const int other = code >> HF_SHIFT;
  const bool slot1 = (code & HF_SLOT1) != 0;
  float o[Q];
  if (code & HF_GHOST) {
    // ghost = m + (m - f_known)*(d_ghost/d_known), m = mean of the face's two
    // end-node pdfs (src/containers.py:280-287, utils/utils.py:153)
    const int a = __ldg(p.gh_a + other), b = __ldg(p.gh_b + other);
    const float rg = __ldg(p.gh_r + other);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const float mq = (__ldg(p.node_pdf + size_t(q) * p.Mp + a) +
                        __ldg(p.node_pdf + size_t(q) * p.Mp + b)) / 2.0f;
      o[q] = mq + (mq - f[q]) * rg;
    }
  } else {
#pragma unroll
    for (int q = 0; q < Q; ++q) o[q] = __ldg(fin + q * Np + other);
  }
  float v[Q];
  xi_dot_n(nx, ny, p.finite_n != 0, v);
  float w[Q];
  if (SCHEME == 1) lw_interp(v, __ldg(p.hf_r + s), __ldg(p.hf_D2 + s), p.dt, p.finite_n != 0, w);
  const float scale = (VARIANT == 1) ? __ldg(p.hf_scale + s) : 1.0f;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    float phi;
    if (SCHEME == 0) {
      // upwind: slot 0 when xi.n >= 0, else slot 1
      phi = ((v[q] >= 0.0f) != slot1) ? f[q] : o[q];
    } else {
      const float lq = slot1 ? o[q] : f[q], rq = slot1 ? f[q] : o[q];
      phi = lq + (rq - lq) * w[q];
    }
    float x = (phi * v[q]) * Ls;
    if (VARIANT == 1) x = x * scale;
    acc[q] = FIRST ? x : acc[q] + x;
  }
}

template <int SCHEME, int VARIANT, bool FV, int KT>
__global__ void __launch_bounds__(256) k_fused(DevPlan p, const float* __restrict__ fin,
                                               float* __restrict__ fout) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.N) return;
  const size_t Np = p.Np;
  float f[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) f[q] = __ldg(fin + q * Np + i);
  float rho, ux, uy, eq[Q];
  macros(f, rho, ux, uy);
  feq9(rho, ux, uy, p, eq);

  float acc[Q];
  const int K = KT > 0 ? KT : p.K;
  if (K == 0) {
#pragma unroll
    for (int q = 0; q < Q; ++q) acc[q] = 0.0f;
  } else {
    fused_face<SCHEME, VARIANT, true>(p, fin, Np, i, 0, f, acc);
    if (KT > 0) {
#pragma unroll
      for (int k = 1; k < KT; ++k) fused_face<SCHEME, VARIANT, false>(p, fin, Np, i, k, f, acc);
    } else {
      for (int k = 1; k < K; ++k) fused_face<SCHEME, VARIANT, false>(p, fin, Np, i, k, f, acc);
    }
  }
  if (FV) {
    const float ia = __ldg(p.inv_area + i);
#pragma unroll
    for (int q = 0; q < Q; ++q) acc[q] = acc[q] * ia;
  }
#pragma unroll
  for (int q = 0; q < Q; ++q) fout[q * Np + i] = f[q] + p.dt * (p.inv_tau * (eq[q] - f[q]) - acc[q]);
}

// ---------------------------------------------------------------------------
// Staged form, kernel 2: one thread per face writes the face flux
// (Faces.calc_fluxes, src/containers.py:191-278) into [9][Fp].
template <int SCHEME, int VARIANT>
__global__ void __launch_bounds__(256) k_face(DevPlan p, const float* __restrict__ f,
                                              float* __restrict__ flux) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p.F) return;
  const size_t Np = p.Np;
  const int s0 = p.fs0[j], s1 = p.fs1[j];
  float lf[Q], rf[Q];
  if (s0 >= 0 && s1 >= 0) {
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      lf[q] = __ldg(f + q * Np + s0);
      rf[q] = __ldg(f + q * Np + s1);
    }
  } else {
    const int a = p.fna[j], b = p.fnb[j];
    float mq[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q)
      mq[q] = (p.node_pdf[size_t(q) * p.Mp + a] + p.node_pdf[size_t(q) * p.Mp + b]) / 2.0f;
    if (s0 >= 0) {
#pragma unroll
      for (int q = 0; q < Q; ++q) lf[q] = __ldg(f + q * Np + s0);
    } else {
      const int kn = p.fkl[j];
      const float rg = p.frl[j];
#pragma unroll
      for (int q = 0; q < Q; ++q) lf[q] = mq[q] + (mq[q] - __ldg(f + q * Np + kn)) * rg;
    }
    if (s1 >= 0) {
#pragma unroll
      for (int q = 0; q < Q; ++q) rf[q] = __ldg(f + q * Np + s1);
    } else {
      const int kn = p.fkr[j];
      const float rg = p.frr[j];
#pragma unroll
      for (int q = 0; q < Q; ++q) rf[q] = mq[q] + (mq[q] - __ldg(f + q * Np + kn)) * rg;
    }
  }
  float v[Q], w[Q];
  xi_dot_n(p.fnx[j], p.fny[j], p.finite_n != 0, v);
  if (SCHEME == 1) lw_interp(v, p.fr[j], p.fD2[j], p.dt, p.finite_n != 0, w);
  const float L = p.fL[j];
  const float scale = (VARIANT == 1) ? p.fscale[j] : 1.0f;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    const float phi = (SCHEME == 0) ? (v[q] >= 0.0f ? lf[q] : rf[q]) : lf[q] + (rf[q] - lf[q]) * w[q];
    float x = (phi * v[q]) * L;
    if (VARIANT == 1) x = x * scale;
    if (VARIANT == 2) x = x * p.fscale[size_t(q) * p.Fp + j];
    flux[size_t(q) * p.Fp + j] = x;
  }
}

// Staged form, kernel 3: cell-centric gather of the signed face fluxes over
// each cell's face list (no atomics) fused with macros, feq and the update.
template <bool FV>
__global__ void __launch_bounds__(256) k_gather(DevPlan p, const float* __restrict__ fin,
                                                const float* __restrict__ flux,
                                                float* __restrict__ fout) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.N) return;
  const size_t Np = p.Np;
  float f[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) f[q] = __ldg(fin + q * Np + i);
  float rho, ux, uy, eq[Q];
  macros(f, rho, ux, uy);
  feq9(rho, ux, uy, p, eq);
  float acc[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) acc[q] = 0.0f;
  for (int k = 0; k < p.K; ++k) {
    const int fi = __ldg(p.cf_face + k * Np + i);
    const float sg = __ldg(p.cf_sign + k * Np + i);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const float x = __ldg(flux + size_t(q) * p.Fp + fi) * sg;
      acc[q] = (k == 0) ? x : acc[q] + x;
    }
  }
  if (FV) {
    const float ia = __ldg(p.inv_area + i);
#pragma unroll
    for (int q = 0; q < Q; ++q) acc[q] = acc[q] * ia;
  }
#pragma unroll
  for (int q = 0; q < Q; ++q) fout[q * Np + i] = f[q] + p.dt * (p.inv_tau * (eq[q] - f[q]) - acc[q]);
}

// Cells.rho/vel/pdf_eq of a pdf buffer (Cells.calc_macros/calc_eqs,
// src/containers.py:93-105).  rho [Np], vel [2][Np], feq [9][Np].
__global__ void __launch_bounds__(256) k_macros(DevPlan p, const float* __restrict__ f,
                                                float* __restrict__ rho_o, float* __restrict__ vel_o,
                                                float* __restrict__ feq_o) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.N) return;
  const size_t Np = p.Np;
  float fc[Q], eq[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) fc[q] = f[q * Np + i];
  float rho, ux, uy;
  macros(fc, rho, ux, uy);
  feq9(rho, ux, uy, p, eq);
  rho_o[i] = rho;
  vel_o[i] = ux;
  vel_o[Np + i] = uy;
#pragma unroll
  for (int q = 0; q < Q; ++q) feq_o[q * Np + i] = eq[q];
}

// [N][9] reference order -> [9][Np] device order.
__global__ void k_aos_to_soa(const float* __restrict__ src, float* __restrict__ dst,
                             const int* __restrict__ cell_new, int N, int Np) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  const int d = cell_new[c];
#pragma unroll
  for (int q = 0; q < Q; ++q) dst[size_t(q) * Np + d] = src[size_t(c) * Q + q];
}

// Exhaustive check of cdiv against IEEE division: every float32 bit pattern
// as dividend; counts the dividends whose quotients differ in value (NaN
// matches NaN).  Not on the step path; runs once per divisor per process.
__global__ void __launch_bounds__(256) k_cdiv_check(float y, float zr, unsigned long long* bad,
                                                    unsigned* example) {
  const CDiv d{y, zr, 1};
  unsigned long long local = 0;
  unsigned ex = 0xFFFFFFFFu;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  for (unsigned long long u = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
       u < (1ull << 32); u += stride) {
    const float x = __uint_as_float(unsigned(u));
    const float a = cdiv(x, d);
    const float b = x / y;
    if (!(a == b || (a != a && b != b))) {
      ++local;
      ex = min(ex, unsigned(u));
    }
  }
  for (int off = 16; off > 0; off >>= 1) {
    local += __shfl_down_sync(0xFFFFFFFFu, local, off);
    ex = min(ex, __shfl_down_sync(0xFFFFFFFFu, ex, off));
  }
  if ((threadIdx.x & 31) == 0 && local) {
    atomicAdd(bad, local);
    atomicMin(example, ex);
  }
}

// ---------------------------------------------------------------------------
static inline int blocks(long long n, int t) { return int((n + t - 1) / t); }

cudaError_t launch_nodes(const DevPlan& p, const float* f, cudaStream_t s) {
  if (p.Mc == 0) return cudaSuccess;
  k_nodes<<<blocks((long long)p.Mc * NODE_LANES, 128), 128, 0, s>>>(p, f);
  return cudaGetLastError();
}

template <int S, int V>
static void fused_dispatch(const DevPlan& p, const float* fin, float* fout, cudaStream_t s) {
  const int g = blocks(p.N, 256);
  if (p.K == 3) {
    if (p.fv) k_fused<S, V, true, 3><<<g, 256, 0, s>>>(p, fin, fout);
    else k_fused<S, V, false, 3><<<g, 256, 0, s>>>(p, fin, fout);
  } else {
    if (p.fv) k_fused<S, V, true, 0><<<g, 256, 0, s>>>(p, fin, fout);
    else k_fused<S, V, false, 0><<<g, 256, 0, s>>>(p, fin, fout);
  }
}

cudaError_t launch_fused(const DevPlan& p, const float* fin, float* fout, cudaStream_t s) {
  if (p.N == 0) return cudaSuccess;
  if (p.scheme == 0 && p.variant == 0) fused_dispatch<0, 0>(p, fin, fout, s);
  else if (p.scheme == 1 && p.variant == 0) fused_dispatch<1, 0>(p, fin, fout, s);
  else if (p.scheme == 0 && p.variant == 1) fused_dispatch<0, 1>(p, fin, fout, s);
  else if (p.scheme == 1 && p.variant == 1) fused_dispatch<1, 1>(p, fin, fout, s);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_face_flux(const DevPlan& p, const float* f, float* flux, cudaStream_t s) {
  if (p.F == 0) return cudaSuccess;
  const int g = blocks(p.F, 256);
  if (p.scheme == 0 && p.variant == 0) k_face<0, 0><<<g, 256, 0, s>>>(p, f, flux);
  else if (p.scheme == 1 && p.variant == 0) k_face<1, 0><<<g, 256, 0, s>>>(p, f, flux);
  else if (p.scheme == 0 && p.variant == 1) k_face<0, 1><<<g, 256, 0, s>>>(p, f, flux);
  else if (p.scheme == 1 && p.variant == 1) k_face<1, 1><<<g, 256, 0, s>>>(p, f, flux);
  else if (p.scheme == 0 && p.variant == 2) k_face<0, 2><<<g, 256, 0, s>>>(p, f, flux);
  else if (p.scheme == 1 && p.variant == 2) k_face<1, 2><<<g, 256, 0, s>>>(p, f, flux);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_gather(const DevPlan& p, const float* fin, const float* flux, float* fout,
                          cudaStream_t s) {
  if (p.N == 0) return cudaSuccess;
  if (p.fv)
    k_gather<true><<<blocks(p.N, 256), 256, 0, s>>>(p, fin, flux, fout);
  else
    k_gather<false><<<blocks(p.N, 256), 256, 0, s>>>(p, fin, flux, fout);
  return cudaGetLastError();
}

cudaError_t launch_macros(const DevPlan& p, const float* f, float* rho, float* vel, float* feq,
                          cudaStream_t s) {
  if (p.N == 0) return cudaSuccess;
  k_macros<<<blocks(p.N, 256), 256, 0, s>>>(p, f, rho, vel, feq);
  return cudaGetLastError();
}

cudaError_t launch_cdiv_check(float y, float zr, unsigned long long* bad, unsigned* example,
                              cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  k_cdiv_check<<<sms * 8, 256, 0, s>>>(y, zr, bad, example);
  return cudaGetLastError();
}

cudaError_t launch_scatter_cells(const float* src_aos, float* dst_soa, const int* cell_new, int N,
                                 int Np, cudaStream_t s) {
  if (N == 0) return cudaSuccess;
  k_aos_to_soa<<<blocks(N, 256), 256, 0, s>>>(src_aos, dst_soa, cell_new, N, Np);
  return cudaGetLastError();
}

}  // namespace fvdbm
