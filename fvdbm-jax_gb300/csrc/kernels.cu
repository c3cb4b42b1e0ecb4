// FVDBM step kernels for sm_103a (GB300).
//
// Every kernel restates the reference's float32 arithmetic operation by
// operation (MADALERAU/FVDBM-JAX src/dynamics.py, src/containers.py,
// utils/utils.py): sums are left folds in the reference's index order, the
// 0*x terms of its integer-lattice dot products are kept, and the library is
// compiled with --fmad=false so no multiply-add is contracted.  The result is
// bitwise equal to the CPU oracle.
//
// Layout: cell pdfs are SoA [9][Np] float32 in device (renumbered) cell
// order; node state is SoA [9][Mp]; per-cell face slots are SoA [K][Np].
#include "fvdbm_internal.h"

namespace fvdbm {

__constant__ float c_W[Q] = {(float)(4.0 / 9.0),  (float)(1.0 / 9.0),  (float)(1.0 / 9.0),
                             (float)(1.0 / 9.0),  (float)(1.0 / 9.0),  (float)(1.0 / 36.0),
                             (float)(1.0 / 36.0), (float)(1.0 / 36.0), (float)(1.0 / 36.0)};

// rho = sum_q f_q; u = (KSI^T f) / rho   (src/dynamics.py:35-47)
__device__ __forceinline__ void macros(const float f[Q], float& rho, float& ux, float& uy) {
  float r = f[0] + f[1];
  r = r + f[2];
  r = r + f[3];
  r = r + f[4];
  r = r + f[5];
  r = r + f[6];
  r = r + f[7];
  r = r + f[8];
  // KSI x column: 0 1 0 -1 0 1 -1 -1 1
  float mx = 0.0f * f[0];
  mx = mx + f[1];
  mx = mx + 0.0f * f[2];
  mx = mx + (-f[3]);
  mx = mx + 0.0f * f[4];
  mx = mx + f[5];
  mx = mx + (-f[6]);
  mx = mx + (-f[7]);
  mx = mx + f[8];
  // KSI y column: 0 0 1 0 -1 1 1 -1 -1
  float my = 0.0f * f[0];
  my = my + 0.0f * f[1];
  my = my + f[2];
  my = my + 0.0f * f[3];
  my = my + (-f[4]);
  my = my + f[5];
  my = my + f[6];
  my = my + (-f[7]);
  my = my + (-f[8]);
  rho = r;
  ux = mx / r;
  uy = my / r;
}

// xi_q . (x, y) folded over the two components (src/dynamics.py:72)
__device__ __forceinline__ void xi_dot(float x, float y, float a[Q]) {
  const float zx = 0.0f * x, zy = 0.0f * y;
  a[0] = zx + zy;
  a[1] = x + zy;
  a[2] = zx + y;
  a[3] = (-x) + zy;
  a[4] = zx + (-y);
  a[5] = x + y;
  a[6] = (-x) + y;
  a[7] = (-x) + (-y);
  a[8] = x + (-y);
}

// feq = (W*rho) * (((1 + a/C^2) + a^2/(2C^4)) - u.u/(2C^2))  (src/dynamics.py:70-74)
__device__ __forceinline__ void feq9(float rho, float ux, float uy, float c2, float c4x2,
                                     float c2x2, float out[Q]) {
  float a[Q];
  xi_dot(ux, uy, a);
  const float uu = ux * ux + uy * uy;
  const float t = uu / c2x2;
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    float s = 1.0f + a[q] / c2;
    s = s + (a[q] * a[q]) / c4x2;
    s = s - t;
    out[q] = (c_W[q] * rho) * s;
  }
}

// Face flux from the pdfs on the slot-0 (left) and slot-1 (right) sides
// (src/containers.py:215-278, src/faces.py:54-74,119-141).
template <int SCHEME, int VARIANT>
__device__ __forceinline__ void face_flux(const float lf[Q], const float rf[Q], float nx, float ny,
                                          float L, float r, float D2, float dt, float scale,
                                          const float* qscale, int qstride, float out[Q]) {
  float v[Q];
  xi_dot(nx, ny, v);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    float phi;
    if (SCHEME == 0) {
      phi = v[q] >= 0.0f ? lf[q] : rf[q];
    } else {
      const float interp = r - (v[q] * dt) / D2;
      phi = lf[q] + (rf[q] - lf[q]) * interp;
    }
    float fl = (phi * v[q]) * L;
    if (VARIANT == 1) fl = fl * scale;
    if (VARIANT == 2) fl = fl * qscale[q * qstride];
    out[q] = fl;
  }
}

// ---------------------------------------------------------------------------
// Boundary nodes: Nodes.calc_pdfs (src/containers.py:339-404).  Velocity
// nodes (type 1) take rho = IDW(cell rho); density nodes (type 2) take
// u = IDW(cell u); both set pdf = feq(rho,u) + IDW(f - feq).  Cell macros are
// recomputed from f with the same arithmetic as the cell kernels.
__global__ void __launch_bounds__(128) k_nodes(DevPlan p, const float* __restrict__ f) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= p.Mc) return;
  const int type = p.nd_type[m];
  const int b = p.nd_ptr[m], e = p.nd_ptr[m + 1];
  float ar = 0.0f, ax = 0.0f, ay = 0.0f, an[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) an[q] = 0.0f;
  bool first = true;
  for (int j = b; j < e; ++j) {
    const unsigned code = p.nd_cell[j];
    const int c = int(code & ~ND_NEQ_ZERO);
    const float w = p.nd_w[j];
    float fc[Q], eq[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) fc[q] = __ldg(f + size_t(q) * p.Np + c);
    float rho, ux, uy;
    macros(fc, rho, ux, uy);
    feq9(rho, ux, uy, p.c2, p.c4x2, p.c2x2, eq);
    const bool zero = (code & ND_NEQ_ZERO) != 0;
    if (first) {
      ar = rho * w;
      ax = ux * w;
      ay = uy * w;
#pragma unroll
      for (int q = 0; q < Q; ++q) an[q] = (zero ? 0.0f : fc[q] - eq[q]) * w;
      first = false;
    } else {
      ar = ar + rho * w;
      ax = ax + ux * w;
      ay = ay + uy * w;
#pragma unroll
      for (int q = 0; q < Q; ++q) an[q] = an[q] + (zero ? 0.0f : fc[q] - eq[q]) * w;
    }
  }
  if (p.nd_npad[m] > 0) {
    // padded (-1, weight 0) entries gather the last cell: rho*0, u*0
    float fc[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) fc[q] = __ldg(f + size_t(q) * p.Np + p.last_cell);
    float rho, ux, uy;
    macros(fc, rho, ux, uy);
    if (first) {
      ar = rho * 0.0f;
      ax = ux * 0.0f;
      ay = uy * 0.0f;
    } else {
      ar = ar + rho * 0.0f;
      ax = ax + ux * 0.0f;
      ay = ay + uy * 0.0f;
    }
  }
  const float sw = p.nd_sumw[m];
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
  feq9(rho_p, ux_p, uy_p, p.c2, p.c4x2, p.c2x2, eqn);
#pragma unroll
  for (int q = 0; q < Q; ++q) p.node_pdf[size_t(q) * p.Mp + m] = eqn[q] + an[q] / sw;
}

// ---------------------------------------------------------------------------
// Fused cell kernel: macros, feq, the flux of each of the cell's faces
// (recomputed from the canonical slot-0/slot-1 pair, so both neighbours get
// bit-identical fluxes without a flux array or atomics), the signed flux sum
// and the BGK/explicit-Euler update (src/containers.py:107-121).
template <int SCHEME, int VARIANT, bool FV>
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
  feq9(rho, ux, uy, p.c2, p.c4x2, p.c2x2, eq);

  float acc[Q];
  for (int k = 0; k < p.K; ++k) {
    const size_t s = k * Np + i;
    const int code = __ldg(p.hf_code + s);
    const float nx = __ldg(p.hf_nx + s), ny = __ldg(p.hf_ny + s), L = __ldg(p.hf_L + s);
    float r = 0.0f, D2 = 1.0f, scale = 1.0f;
    if (SCHEME == 1) {
      r = __ldg(p.hf_r + s);
      D2 = __ldg(p.hf_D2 + s);
    }
    if (VARIANT == 1) scale = __ldg(p.hf_scale + s);
    const int other = code >> HF_SHIFT;
    float o[Q];
    if (code & HF_GHOST) {
      // ghost = m + (m - f_known)*(d_ghost/d_known), m = mean of the face's
      // two end-node pdfs (src/containers.py:280-287, utils/utils.py:153)
      const int a = __ldg(p.gh_a + other), b = __ldg(p.gh_b + other);
      const float rg = __ldg(p.gh_r + other);
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const float mq = (p.node_pdf[size_t(q) * p.Mp + a] + p.node_pdf[size_t(q) * p.Mp + b]) / 2.0f;
        o[q] = mq + (mq - f[q]) * rg;
      }
    } else {
#pragma unroll
      for (int q = 0; q < Q; ++q) o[q] = __ldg(fin + q * Np + other);
    }
    float fl[Q];
    if (code & HF_SLOT1)
      face_flux<SCHEME, VARIANT>(o, f, nx, ny, L, r, D2, p.dt, scale, nullptr, 0, fl);
    else
      face_flux<SCHEME, VARIANT>(f, o, nx, ny, L, r, D2, p.dt, scale, nullptr, 0, fl);
    const float sg = float((code & 3) - 1);
    if (k == 0) {
#pragma unroll
      for (int q = 0; q < Q; ++q) acc[q] = fl[q] * sg;
    } else {
#pragma unroll
      for (int q = 0; q < Q; ++q) acc[q] = acc[q] + fl[q] * sg;
    }
  }
  if (p.K == 0) {
#pragma unroll
    for (int q = 0; q < Q; ++q) acc[q] = 0.0f;
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
  float r = 0.0f, D2 = 1.0f, scale = 1.0f;
  if (SCHEME == 1) {
    r = p.fr[j];
    D2 = p.fD2[j];
  }
  if (VARIANT == 1) scale = p.fscale[j];
  float fl[Q];
  face_flux<SCHEME, VARIANT>(lf, rf, p.fnx[j], p.fny[j], p.fL[j], r, D2, p.dt, scale,
                             VARIANT == 2 ? p.fscale + j : nullptr, p.Fp, fl);
#pragma unroll
  for (int q = 0; q < Q; ++q) flux[size_t(q) * p.Fp + j] = fl[q];
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
  feq9(rho, ux, uy, p.c2, p.c4x2, p.c2x2, eq);
  float acc[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) acc[q] = 0.0f;
  for (int k = 0; k < p.K; ++k) {
    const int fi = __ldg(p.cf_face + k * Np + i);
    const float sg = __ldg(p.cf_sign + k * Np + i);
    if (k == 0) {
#pragma unroll
      for (int q = 0; q < Q; ++q) acc[q] = __ldg(flux + size_t(q) * p.Fp + fi) * sg;
    } else {
#pragma unroll
      for (int q = 0; q < Q; ++q) acc[q] = acc[q] + __ldg(flux + size_t(q) * p.Fp + fi) * sg;
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
  feq9(rho, ux, uy, p.c2, p.c4x2, p.c2x2, eq);
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

// ---------------------------------------------------------------------------
static inline int blocks(int n, int t) { return (n + t - 1) / t; }

cudaError_t launch_nodes(const DevPlan& p, const float* f, cudaStream_t s) {
  if (p.Mc == 0) return cudaSuccess;
  k_nodes<<<blocks(p.Mc, 128), 128, 0, s>>>(p, f);
  return cudaGetLastError();
}

template <int S, int V>
static void fused_dispatch_fv(const DevPlan& p, const float* fin, float* fout, cudaStream_t s) {
  if (p.fv)
    k_fused<S, V, true><<<blocks(p.N, 256), 256, 0, s>>>(p, fin, fout);
  else
    k_fused<S, V, false><<<blocks(p.N, 256), 256, 0, s>>>(p, fin, fout);
}

cudaError_t launch_fused(const DevPlan& p, const float* fin, float* fout, cudaStream_t s) {
  if (p.N == 0) return cudaSuccess;
  if (p.scheme == 0 && p.variant == 0) fused_dispatch_fv<0, 0>(p, fin, fout, s);
  else if (p.scheme == 1 && p.variant == 0) fused_dispatch_fv<1, 0>(p, fin, fout, s);
  else if (p.scheme == 0 && p.variant == 1) fused_dispatch_fv<0, 1>(p, fin, fout, s);
  else if (p.scheme == 1 && p.variant == 1) fused_dispatch_fv<1, 1>(p, fin, fout, s);
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

cudaError_t launch_scatter_cells(const float* src_aos, float* dst_soa, const int* cell_new, int N,
                                 int Np, cudaStream_t s) {
  if (N == 0) return cudaSuccess;
  k_aos_to_soa<<<blocks(N, 256), 256, 0, s>>>(src_aos, dst_soa, cell_new, N, Np);
  return cudaGetLastError();
}

}  // namespace fvdbm
