// D2Q13 lattice (src/dynamics.py:77-102): the staged step (boundary nodes,
// per-face fluxes, per-cell gather and update), the fused cell update for
// triangle meshes (boundary nodes, then one cell kernel) and the read-back
// helpers
// with 13 velocities, including the (+-2, 0), (0, +-2) ones, and the
// third-order equilibrium
//   feq_q = (W_q rho) * (((((1 + a/C^2) + a^2/(2C^4)) - u.u/(2C^2))
//                          + a^3/(2C^6)) - 3 a u.u/(2C^4)),   a = xi_q . u,
// evaluated in that order with a^3 = a*(a*a) (jax's integer_pow), so that
// results equal the reference's float32 step bit for bit.  The float32
// lattice constants come from the host (C = 1/sqrt(2) in float32).
//
// Layouts as the D2Q9 kernels: cell pdfs AoSoA [Np/32][13][32], face fluxes
// [13][Fp], node state [13][Mp] / [Mp] / [2][Mp].
#include "fvdbm_math.cuh"

namespace fvdbm {

namespace {

constexpr int Q13 = 13;
__constant__ float c_kx13[Q13] = {0, 1, 0, -1, 0, 1, -1, -1, 1, 2, 0, -2, 0};
__constant__ float c_ky13[Q13] = {0, 0, 1, 0, -1, 1, 1, -1, -1, 0, 2, 0, -2};
__constant__ float c_w13[Q13] = {(float)(3.0 / 8.0),   (float)(1.0 / 12.0), (float)(1.0 / 12.0),
                                 (float)(1.0 / 12.0),  (float)(1.0 / 12.0), (float)(1.0 / 16.0),
                                 (float)(1.0 / 16.0),  (float)(1.0 / 16.0), (float)(1.0 / 16.0),
                                 (float)(1.0 / 96.0),  (float)(1.0 / 96.0), (float)(1.0 / 96.0),
                                 (float)(1.0 / 96.0)};

__device__ __forceinline__ size_t base13(int c) { return size_t(c >> 5) * (Q13 * 32) + size_t(c & 31); }

__device__ __forceinline__ void load13(const float* __restrict__ f, int c, float out[Q13]) {
  const float* b = f + base13(c);
#pragma unroll
  for (int q = 0; q < Q13; ++q) out[q] = __ldg(b + q * 32);
}

// rho = sum_q f_q; u = (xi^T f)/rho (src/dynamics.py:35-47).  For finite
// rho every f_q is finite: the 0*f_q terms of the literal fold are +-0 and
// leave the sum's value unchanged, +-1*f_q is +-f_q and 2*f_q is exact, so
// the fold runs over the nonzero directions only; otherwise every product is
// kept.
__device__ __forceinline__ void macros13(const float f[Q13], float& rho, float& ux, float& uy) {
  float r = f[0];
#pragma unroll
  for (int q = 1; q < Q13; ++q) r = r + f[q];
  float mx, my;
  if (fabsf(r) <= FLT_MAX) {
    mx = ((((((f[1] - f[3]) + f[5]) - f[6]) - f[7]) + f[8]) + 2.0f * f[9]) - 2.0f * f[11];
    my = ((((((f[2] - f[4]) + f[5]) + f[6]) - f[7]) - f[8]) + 2.0f * f[10]) - 2.0f * f[12];
  } else {
    mx = c_kx13[0] * f[0];
    my = c_ky13[0] * f[0];
#pragma unroll
    for (int q = 1; q < Q13; ++q) {
      mx = mx + c_kx13[q] * f[q];
      my = my + c_ky13[q] * f[q];
    }
  }
  rho = r;
  ux = mx / r;
  uy = my / r;
}

// v_q = xi_q . n (src/containers.py:235); for a finite normal the symmetric
// form (+-nx, +-ny, +-(nx+ny), +-(ny-nx), +-2nx, +-2ny), whose values equal
// the literal dot products'
__device__ __forceinline__ void xi13_dot_n(float nx, float ny, bool finite_n, float v[Q13]) {
  if (!finite_n) {
#pragma unroll
    for (int q = 0; q < Q13; ++q) v[q] = c_kx13[q] * nx + c_ky13[q] * ny;
    return;
  }
  const float s = nx + ny, d = ny - nx, x2 = 2.0f * nx, y2 = 2.0f * ny;
  v[0] = 0.0f;
  v[1] = nx;
  v[2] = ny;
  v[3] = -nx;
  v[4] = -ny;
  v[5] = s;
  v[6] = d;
  v[7] = -s;
  v[8] = -d;
  v[9] = x2;
  v[10] = y2;
  v[11] = -x2;
  v[12] = -y2;
}

// x == 0 or 2^-30 <= |x| <= 2^30: then x^2, x*x^2, 3x*u.u and their
// scalings by 2, 4, 8 stay in the normal range, where binary scaling commutes
// with rounding, and every dividend is one the known-divisor check covers.
__device__ __forceinline__ bool dom13(float x) {
  const float a = fabsf(x);
  return (a >= 0x1p-30f && a <= 0x1p30f) || x == 0.0f;
}

__device__ __forceinline__ float kdiv(float x, const CDiv& d, bool two) {
  return two ? cdiv_two(x, d.zr, d.zl) : cdiv_fast(x, d.y, d.zr);
}

__device__ __forceinline__ void feq13(float rho, float ux, float uy, const DevPlan& p, float out[Q13]) {
  const float uu = ux * ux + uy * uy;
  const float a5 = ux + uy, a6 = uy - ux;
  if (p.cdiv_mode != 0 && dom13(ux) && dom13(uy) && dom13(a5) && dom13(a6)) {
    // a_q = +-x or +-2x for x in (ux, uy, ux+uy, uy-ux) (a_0 = 0; the 0*u
    // terms of the literal dot product only change the sign of a zero a,
    // which leaves s unchanged).  Per x: t1 = x/C^2, t2 = x^2/(2C^4),
    // t4 = x*x^2/(2C^6), t5 = 3x*u.u/(2C^4); for -x the odd ones change sign
    // (RN(-y) = -RN(y)), for 2x they scale by 2, 4, 8, 2 exactly.  17
    // divisions instead of 65, each the known-divisor form.
    const bool two = p.cdiv_mode == 2;
    const float t3 = kdiv(uu, p.d_c2x2, two);
    const float b[4] = {ux, uy, a5, a6};
    float t1[4], t2[4], t4[4], t5[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float x = b[j], xx = x * x;
      t1[j] = kdiv(x, p.d_c2, two);
      t2[j] = kdiv(xx, p.d_c4x2, two);
      t4[j] = kdiv(x * xx, p.d_c6x2, two);
      t5[j] = kdiv((3.0f * x) * uu, p.d_c4x2, two);
    }
    auto S = [t3](float a1, float a2, float a4, float a5_) {
      float s = 1.0f + a1;
      s = s + a2;
      s = s - t3;
      s = s + a4;
      return s - a5_;
    };
    const float w0 = c_w13[0] * rho, w1 = c_w13[1] * rho, w5 = c_w13[5] * rho, w9 = c_w13[9] * rho;
    out[0] = w0 * S(0.0f, 0.0f, 0.0f, 0.0f);
    out[1] = w1 * S(t1[0], t2[0], t4[0], t5[0]);
    out[3] = w1 * S(-t1[0], t2[0], -t4[0], -t5[0]);
    out[2] = w1 * S(t1[1], t2[1], t4[1], t5[1]);
    out[4] = w1 * S(-t1[1], t2[1], -t4[1], -t5[1]);
    out[5] = w5 * S(t1[2], t2[2], t4[2], t5[2]);
    out[7] = w5 * S(-t1[2], t2[2], -t4[2], -t5[2]);
    out[6] = w5 * S(t1[3], t2[3], t4[3], t5[3]);
    out[8] = w5 * S(-t1[3], t2[3], -t4[3], -t5[3]);
    out[9] = w9 * S(2.0f * t1[0], 4.0f * t2[0], 8.0f * t4[0], 2.0f * t5[0]);
    out[11] = w9 * S(-2.0f * t1[0], 4.0f * t2[0], -8.0f * t4[0], -2.0f * t5[0]);
    out[10] = w9 * S(2.0f * t1[1], 4.0f * t2[1], 8.0f * t4[1], 2.0f * t5[1]);
    out[12] = w9 * S(-2.0f * t1[1], 4.0f * t2[1], -8.0f * t4[1], -2.0f * t5[1]);
    return;
  }
#pragma unroll
  for (int q = 0; q < Q13; ++q) {
    const float a = c_kx13[q] * ux + c_ky13[q] * uy;
    float s = 1.0f + a / p.c2;
    s = s + (a * a) / p.c4x2;
    s = s - uu / p.c2x2;
    s = s + (a * (a * a)) / p.c6x2;
    s = s - ((3.0f * a) * uu) / p.c4x2;
    out[q] = (c_w13[q] * rho) * s;
  }
}

// Boundary nodes (src/containers.py:339-404, utils/utils.py:34-60), one
// thread per computed node, its stencil entries folded in order.
__global__ void k13_nodes(DevPlan p, const float* __restrict__ f) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= p.Mc) return;
  const int type = p.nd_type[m];
  const int e0 = p.nd_ptr[m], e1 = p.nd_ptr[m + 1];
  float ar = 0.0f, ax = 0.0f, ay = 0.0f, an[Q13];
#pragma unroll
  for (int q = 0; q < Q13; ++q) an[q] = 0.0f;
  for (int e = e0; e < e1; ++e) {
    const unsigned code = p.nd_cell[e];
    const float w = p.nd_w[e];
    float fc[Q13], eq[Q13];
    load13(f, int(code & ~ND_NEQ_ZERO), fc);
    float rho, ux, uy;
    macros13(fc, rho, ux, uy);
    feq13(rho, ux, uy, p, eq);
    const bool zero = (code & ND_NEQ_ZERO) != 0;
    const bool first = e == e0;
    ar = first ? rho * w : ar + rho * w;
    ax = first ? ux * w : ax + ux * w;
    ay = first ? uy * w : ay + uy * w;
#pragma unroll
    for (int q = 0; q < Q13; ++q) {
      const float x = (zero ? 0.0f : fc[q] - eq[q]) * w;
      an[q] = first ? x : an[q] + x;
    }
  }
  if (p.nd_npad[m] > 0) {
    // padded (-1, weight 0) entries gather the last cell
    float fc[Q13];
    load13(f, p.last_cell, fc);
    float rho, ux, uy;
    macros13(fc, rho, ux, uy);
    const bool none = e1 == e0;
    ar = none ? rho * 0.0f : ar + rho * 0.0f;
    ax = none ? ux * 0.0f : ax + ux * 0.0f;
    ay = none ? uy * 0.0f : ay + uy * 0.0f;
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
  float eqn[Q13];
  feq13(rho_p, ux_p, uy_p, p, eqn);
#pragma unroll
  for (int q = 0; q < Q13; ++q) p.node_pdf[size_t(q) * p.Mp + m] = eqn[q] + an[q] / sw;
}

// Face fluxes (src/containers.py:191-287), one thread per face.
__global__ void k13_face(DevPlan p, const float* __restrict__ f, float* __restrict__ flux) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p.F) return;
  const int s0 = p.fs0[j], s1 = p.fs1[j];
  float lf[Q13], rf[Q13];
  if (s0 >= 0 && s1 >= 0) {
    load13(f, s0, lf);
    load13(f, s1, rf);
  } else {
    const int a = p.fna[j], b = p.fnb[j];
    float mq[Q13];
#pragma unroll
    for (int q = 0; q < Q13; ++q)
      mq[q] = (p.node_pdf[size_t(q) * p.Mp + a] + p.node_pdf[size_t(q) * p.Mp + b]) / 2.0f;
    if (s0 >= 0) {
      load13(f, s0, lf);
    } else {
      float kf[Q13];
      load13(f, p.fkl[j], kf);
#pragma unroll
      for (int q = 0; q < Q13; ++q) lf[q] = mq[q] + (mq[q] - kf[q]) * p.frl[j];
    }
    if (s1 >= 0) {
      load13(f, s1, rf);
    } else {
      float kf[Q13];
      load13(f, p.fkr[j], kf);
#pragma unroll
      for (int q = 0; q < Q13; ++q) rf[q] = mq[q] + (mq[q] - kf[q]) * p.frr[j];
    }
  }
  const float nx = p.fnx[j], ny = p.fny[j], L = p.fL[j];
#pragma unroll
  for (int q = 0; q < Q13; ++q) {
    const float v = c_kx13[q] * nx + c_ky13[q] * ny;
    float phi;
    if (p.scheme == 0) {
      phi = v >= 0.0f ? lf[q] : rf[q];
    } else {
      const float w = p.fr[j] - (v * p.dt) / p.fD2[j];
      phi = lf[q] + (rf[q] - lf[q]) * w;
    }
    flux[size_t(q) * p.Fp + j] = (phi * v) * L;
  }
}

// Cell update (src/containers.py:107-121), one thread per cell.
__global__ void k13_gather(DevPlan p, const float* __restrict__ fin, const float* __restrict__ flux,
                           float* __restrict__ fout) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.N) return;
  const size_t Np = p.Np;
  float f[Q13], eq[Q13], acc[Q13];
  load13(fin, i, f);
  float rho, ux, uy;
  macros13(f, rho, ux, uy);
  feq13(rho, ux, uy, p, eq);
#pragma unroll
  for (int q = 0; q < Q13; ++q) acc[q] = 0.0f;
  for (int k = 0; k < p.K; ++k) {
    const int fi = p.cf_face[k * Np + i];
    const float sg = p.cf_sign[k * Np + i];
#pragma unroll
    for (int q = 0; q < Q13; ++q) {
      const float x = flux[size_t(q) * p.Fp + fi] * sg;
      acc[q] = (k == 0) ? x : acc[q] + x;
    }
  }
  if (p.fv) {
    const float ia = p.inv_area[i];
#pragma unroll
    for (int q = 0; q < Q13; ++q) acc[q] = acc[q] * ia;
  }
  float* o = fout + base13(i);
#pragma unroll
  for (int q = 0; q < Q13; ++q) o[q * 32] = f[q] + p.dt * (p.inv_tau * (eq[q] - f[q]) - acc[q]);
}

// Fused cell update (k13_face + k13_gather in one pass), one thread per
// cell: macros, feq, the flux of each of the cell's three face slots from
// the canonical slot-0/slot-1 pair (both neighbours compute identical
// values), the signed sum and the update, with the per-cell face slots of
// the D2Q9 fused kernel ([Np/32][rows][32]: code, n, L*sigma, LW r and D2).
// ((phi*v)*L)*sigma == (phi*v)*(L*sigma) exactly for sigma = +-1.
template <int SCHEME>
__global__ void __launch_bounds__(256) k13_fused(DevPlan p, const float* __restrict__ fin,
                                                 float* __restrict__ fout) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.N) return;
  const HfRows HR{3, SCHEME, 0};
  const unsigned* hb = p.hf + size_t(i >> 5) * (HR.rows() * 32) + (i & 31);
  float f[Q13], eq[Q13], acc[Q13];
  load13(fin, i, f);
  float rho, ux, uy;
  macros13(f, rho, ux, uy);
  feq13(rho, ux, uy, p, eq);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int code = int(__ldg(hb + HR.code(k) * 32));
    const float nx = __uint_as_float(__ldg(hb + HR.nx(k) * 32));
    const float ny = __uint_as_float(__ldg(hb + HR.ny(k) * 32));
    const float Ls = __uint_as_float(__ldg(hb + HR.ls(k) * 32));
    const int other = code >> HF_SHIFT;
    const bool slot1 = (code & HF_SLOT1) != 0;
    float o[Q13];
    if (code & HF_GHOST) {
      // ghost = m + (m - f_known)*(d_ghost/d_known), the known cell this one
      const int a = __ldg(p.gh_a + other), b = __ldg(p.gh_b + other);
      const float rg = __ldg(p.gh_r + other);
#pragma unroll
      for (int q = 0; q < Q13; ++q) {
        const float mq = (p.node_pdf[size_t(q) * p.Mp + a] + p.node_pdf[size_t(q) * p.Mp + b]) / 2.0f;
        o[q] = mq + (mq - f[q]) * rg;
      }
    } else {
      load13(fin, other, o);
    }
    float r = 0.0f, D2 = 1.0f;
    if (SCHEME == 1) {
      r = __uint_as_float(__ldg(hb + HR.r(k) * 32));
      D2 = __uint_as_float(__ldg(hb + HR.d2(k) * 32));
    }
    float vq[Q13];
    xi13_dot_n(nx, ny, p.finite_n != 0, vq);
    float w[Q13];
    if (SCHEME == 1) {
      // interp_q = d0/(d0+d1) - (v_q dt)/(2(d0+d1)) (src/containers.py:274);
      // for a finite normal v_{q'} = -v_q pairs share one quotient:
      // (-v dt)/D2 == -((v dt)/D2), and r - (-t) == r + t
      if (p.finite_n) {
        const float t1 = (vq[1] * p.dt) / D2, t2 = (vq[2] * p.dt) / D2, t5 = (vq[5] * p.dt) / D2;
        const float t6 = (vq[6] * p.dt) / D2, t9 = (vq[9] * p.dt) / D2, t10 = (vq[10] * p.dt) / D2;
        w[0] = r - (vq[0] * p.dt) / D2;
        w[1] = r - t1;
        w[3] = r + t1;
        w[2] = r - t2;
        w[4] = r + t2;
        w[5] = r - t5;
        w[7] = r + t5;
        w[6] = r - t6;
        w[8] = r + t6;
        w[9] = r - t9;
        w[11] = r + t9;
        w[10] = r - t10;
        w[12] = r + t10;
      } else {
#pragma unroll
        for (int q = 0; q < Q13; ++q) w[q] = r - (vq[q] * p.dt) / D2;
      }
    }
    float phi[Q13];
#pragma unroll
    for (int q = 0; q < Q13; ++q) {
      const float lq = slot1 ? o[q] : f[q], rq = slot1 ? f[q] : o[q];
      phi[q] = (SCHEME == 0) ? (vq[q] >= 0.0f ? lq : rq) : lq + (rq - lq) * w[q];
    }
#if FVDBM_PAIRED
    // paired products; a sum that takes one is the multiply-add acc*one + x
    const float2 L2 = make_float2(Ls, Ls), one2 = make_float2(p.one, p.one);
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const float2 x = mul2(mul2(make_float2(phi[2 * j], phi[2 * j + 1]), make_float2(vq[2 * j], vq[2 * j + 1])), L2);
      const float2 a = (k == 0) ? x : fold2(make_float2(acc[2 * j], acc[2 * j + 1]), one2, x);
      acc[2 * j] = a.x;
      acc[2 * j + 1] = a.y;
    }
    {
      const float x = (phi[12] * vq[12]) * Ls;
      acc[12] = (k == 0) ? x : acc[12] + x;
    }
#else
#pragma unroll
    for (int q = 0; q < Q13; ++q) {
      const float x = (phi[q] * vq[q]) * Ls;
      acc[q] = (k == 0) ? x : acc[q] + x;
    }
#endif
  }
  if (p.fv) {
    const float ia = p.inv_area[i];
#pragma unroll
    for (int q = 0; q < Q13; ++q) acc[q] = acc[q] * ia;
  }
  float* o = fout + base13(i);
#if FVDBM_PAIRED
  // f + dt*(inv_tau*(eq - f) - acc), pairwise
  const float2 it2 = make_float2(p.inv_tau, p.inv_tau), dt2 = make_float2(p.dt, p.dt);
  const float2 one2 = make_float2(p.one, p.one), m12 = make_float2(p.neg_one, p.neg_one);
#pragma unroll
  for (int j = 0; j < 6; ++j) {
    const float2 f2 = make_float2(f[2 * j], f[2 * j + 1]);
    const float2 d = fold2(f2, m12, make_float2(eq[2 * j], eq[2 * j + 1]));
    const float2 u = fold2(make_float2(acc[2 * j], acc[2 * j + 1]), m12, mul2(it2, d));
    const float2 r = fold2(f2, one2, mul2(dt2, u));
    o[(2 * j) * 32] = r.x;
    o[(2 * j + 1) * 32] = r.y;
  }
  o[12 * 32] = f[12] + p.dt * (p.inv_tau * (eq[12] - f[12]) - acc[12]);
#else
#pragma unroll
  for (int q = 0; q < Q13; ++q) o[q * 32] = f[q] + p.dt * (p.inv_tau * (eq[q] - f[q]) - acc[q]);
#endif
}

// rho [Np], vel [2][Np], feq AoSoA of a pdf buffer (read-back)
__global__ void k13_macros(DevPlan p, const float* __restrict__ f, float* __restrict__ rho_o,
                           float* __restrict__ vel_o, float* __restrict__ feq_o) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.N) return;
  float fc[Q13], eq[Q13];
  load13(f, i, fc);
  float rho, ux, uy;
  macros13(fc, rho, ux, uy);
  feq13(rho, ux, uy, p, eq);
  rho_o[i] = rho;
  vel_o[i] = ux;
  vel_o[size_t(p.Np) + i] = uy;
  float* o = feq_o + base13(i);
#pragma unroll
  for (int q = 0; q < Q13; ++q) o[q * 32] = eq[q];
}

inline int nblk(long long n, int t) { return int((n + t - 1) / t); }

}  // namespace

cudaError_t launch13_step(const DevPlan& p, const float* fin, float* flux, float* fout, cudaStream_t s) {
  if (p.Mc > 0) k13_nodes<<<nblk(p.Mc, 128), 128, 0, s>>>(p, fin);
  if (p.F > 0) k13_face<<<nblk(p.F, 256), 256, 0, s>>>(p, fin, flux);
  if (p.N > 0) k13_gather<<<nblk(p.N, 256), 256, 0, s>>>(p, fin, flux, fout);
  return cudaGetLastError();
}

cudaError_t launch13_fused(const DevPlan& p, const float* fin, float* fout, cudaStream_t s) {
  if (p.Mc > 0) k13_nodes<<<nblk(p.Mc, 128), 128, 0, s>>>(p, fin);
  if (p.N > 0) {
    if (p.scheme == 1)
      k13_fused<1><<<nblk(p.N, 256), 256, 0, s>>>(p, fin, fout);
    else
      k13_fused<0><<<nblk(p.N, 256), 256, 0, s>>>(p, fin, fout);
  }
  return cudaGetLastError();
}

cudaError_t launch13_nodes(const DevPlan& p, const float* fin, cudaStream_t s) {
  if (p.Mc > 0) k13_nodes<<<nblk(p.Mc, 128), 128, 0, s>>>(p, fin);
  return cudaGetLastError();
}

cudaError_t launch13_cells(const DevPlan& p, const float* fin, float* fout, cudaStream_t s) {
  if (p.N > 0) {
    if (p.scheme == 1)
      k13_fused<1><<<nblk(p.N, 256), 256, 0, s>>>(p, fin, fout);
    else
      k13_fused<0><<<nblk(p.N, 256), 256, 0, s>>>(p, fin, fout);
  }
  return cudaGetLastError();
}

cudaError_t launch13_face_flux(const DevPlan& p, const float* f, float* flux, cudaStream_t s) {
  if (p.F > 0) k13_face<<<nblk(p.F, 256), 256, 0, s>>>(p, f, flux);
  return cudaGetLastError();
}

cudaError_t launch13_macros(const DevPlan& p, const float* f, float* rho, float* vel, float* feq,
                            cudaStream_t s) {
  if (p.N > 0) k13_macros<<<nblk(p.N, 256), 256, 0, s>>>(p, f, rho, vel, feq);
  return cudaGetLastError();
}

}  // namespace fvdbm
