// Device arithmetic shared by the step kernels (kernels.cu, tile.cu).
//
// Every helper restates the reference's float32 arithmetic (MADALERAU/
// FVDBM-JAX src/dynamics.py, src/containers.py, utils/utils.py) so that the
// results are bitwise equal to the CPU oracle:
//   * sums are left folds in the reference's index order;
//   * the library is compiled with --fmad=false, so no multiply-add is
//     contracted; the only FMAs are the explicit ones of cdiv();
//   * rewrites are value-identical: the 0*x terms of the integer-lattice dot
//     products only matter for non-finite inputs, and such inputs take the
//     literal path; the +-symmetric lattice directions reuse one quotient
//     (RN(-a/c) == -RN(a/c)).
#pragma once
#include <cfloat>

#include "fvdbm_internal.h"

namespace fvdbm {

static __constant__ float c_W[Q] = {(float)(4.0 / 9.0),  (float)(1.0 / 9.0),  (float)(1.0 / 9.0),
                             (float)(1.0 / 9.0),  (float)(1.0 / 9.0),  (float)(1.0 / 36.0),
                             (float)(1.0 / 36.0), (float)(1.0 / 36.0), (float)(1.0 / 36.0)};

__device__ __forceinline__ bool finite(float x) { return fabsf(x) <= FLT_MAX; }

// Paired float32 arithmetic (sm_100+ f32x2 instructions): each lane is the
// IEEE round-to-nearest operation of the scalar form, so paired and scalar
// evaluation give identical bits; the pairs halve the issued instructions.
// One rule keeps it so: a paired product never feeds a paired add.  The
// compiler contracts that pair into a fused multiply-add (one rounding)
// despite --fmad=false and the _rn forms (and rewrites a*1 + x with a
// literal 1 into an add first).  A sum that takes a paired product is
// written as the multiply-add a*one + x with one = 1 held in a run-time
// value: a*one is exact, so it rounds as a + x does, signed zeros included,
// and a multiply-add has no product left to contract.
#ifndef FVDBM_PAIRED
#define FVDBM_PAIRED 1
#endif
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
// a - b == a + (-b) exactly (signed zeros included)
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
// a*s + x for s = (1, 1) or (-1, -1) given at run time: x + a or x - a,
// where x may be a paired product
__device__ __forceinline__ float2 fold2(float2 a, float2 s, float2 x) { return __ffma2_rn(a, s, x); }

// Programmatic dependent launch: wait until the previous kernel in the
// stream has completed and its writes are visible (a no-op when the kernel
// was launched without the attribute); let the next kernel start launching.
__device__ __forceinline__ void grid_dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void grid_dep_launch() { asm volatile("griddepcontrol.launch_dependents;"); }

// Cell arrays are AoSoA: blocks of 32 cells, [block][row][32].  A cell's
// row r sits at cell_base(i) + r*32, a constant offset from one base.
__device__ __forceinline__ size_t cell_base(int i, int rows) {
  return size_t(i >> 5) * size_t(rows * 32) + size_t(i & 31);
}

__device__ __forceinline__ void load_cell(const float* __restrict__ f, int c, float out[Q]) {
  const float* b = f + cell_base(c, Q);
#pragma unroll
  for (int q = 0; q < Q; ++q) out[q] = __ldg(b + q * 32);
}

// The same through L2 (ld.global.cg): for pdfs that other blocks wrote
// earlier in the same launch, which the non-coherent path may hold stale.
__device__ __forceinline__ void load_cell_cg(const float* f, int c, float out[Q]) {
  const float* b = f + cell_base(c, Q);
#pragma unroll
  for (int q = 0; q < Q; ++q) out[q] = __ldcg(b + q * 32);
}

// Correctly rounded x/y for a divisor known in advance.  With zr = RN(1/y):
// q0 = RN(x*zr) is within 1.5 ulp of x/y; one correction
// q1 = RN(q0 + RN(x - q0*y)*zr) (remainder exact through an FMA) makes it
// faithful; by Markstein's theorem (P. Markstein, "Computation of elementary
// functions on the IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1),
// 1990) a second correction q2 = RN(q1 + (x - q1*y)*zr) is then the correctly
// rounded quotient (Brisebarre, Muller and Raina, IEEE Trans. Computers 53(8),
// 2004, show that the first correction alone fails for some divisors).
// Whether this equals x/y for every float32 x is checked exhaustively on the
// device (k_cdiv_check) before the kernels are allowed to use it.
__device__ __forceinline__ float cdiv_fast(float x, float y, float zr) {
  const float q0 = __fmul_rn(x, zr);
  const float r0 = __fmaf_rn(-q0, y, x);
  const float q1 = __fmaf_rn(r0, zr, q0);
  const float r1 = __fmaf_rn(-q1, y, x);
  return __fmaf_rn(r1, zr, q1);
}

// Brisebarre, Muller and Raina (same paper, Algorithm 1): with zh = RN(1/y)
// and zl = RN(1/y - zh), RN(x*zh + RN(x*zl)) equals RN(x/y) for every x for
// many divisors y (not all); k_cdiv_check decides for the divisor at hand.
__device__ __forceinline__ float cdiv_two(float x, float zh, float zl) {
  return __fmaf_rn(x, zh, __fmul_rn(x, zl));
}

// The remainders are exact only while they stay above the subnormal range,
// so tiny dividends (|x| < 2^-100) and quotients outside the normal range
// take x/y; x == 0 gives +-0 either way.  The same domain serves the
// two-operation form (x*zl stays normal there).
__device__ __forceinline__ float cdiv(float x, const CDiv& d) {
  if (d.ok) {
    const float q = d.two ? cdiv_two(x, d.zr, d.zl) : cdiv_fast(x, d.y, d.zr);
    const float a = fabsf(q);
    if ((fabsf(x) >= 0x1p-100f && a >= FLT_MIN && a <= FLT_MAX) || x == 0.0f) return q;
  }
  return x / d.y;
}

// ---------------------------------------------------------------------------
// Literal forms (src/dynamics.py:35-47,70-74), used for non-finite inputs.
__device__ __forceinline__ void macros_literal(const float f[Q], float& mx, float& my) {
  mx = 0.0f * f[0];
  mx = mx + f[1];
  mx = mx + 0.0f * f[2];
  mx = mx + (-f[3]);
  mx = mx + 0.0f * f[4];
  mx = mx + f[5];
  mx = mx + (-f[6]);
  mx = mx + (-f[7]);
  mx = mx + f[8];
  my = 0.0f * f[0];
  my = my + 0.0f * f[1];
  my = my + f[2];
  my = my + 0.0f * f[3];
  my = my + (-f[4]);
  my = my + f[5];
  my = my + f[6];
  my = my + (-f[7]);
  my = my + (-f[8]);
}

// xi_q . (x, y) folded over the two components, 0*x terms kept
__device__ __forceinline__ void xi_dot_literal(float x, float y, float a[Q]) {
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

__device__ __forceinline__ void feq9_literal(float rho, float ux, float uy, const DevPlan& p,
                                          float out[Q]) {
  float a[Q];
  xi_dot_literal(ux, uy, a);
  const float uu = ux * ux + uy * uy;
  const float t = uu / p.c2x2;
  for (int q = 0; q < Q; ++q) {
    float s = 1.0f + a[q] / p.c2;
    s = s + (a[q] * a[q]) / p.c4x2;
    s = s - t;
    out[q] = (c_W[q] * rho) * s;
  }
}

// rho = sum_q f_q; u = (KSI^T f)/rho.  For finite rho every f_q is finite and
// the 0*f_q terms of the literal fold are +-0, which leave the sum unchanged.
__device__ __forceinline__ void macros(const float f[Q], float& rho, float& ux, float& uy) {
  float r = f[0] + f[1];
  r = r + f[2];
  r = r + f[3];
  r = r + f[4];
  r = r + f[5];
  r = r + f[6];
  r = r + f[7];
  r = r + f[8];
  float mx, my;
  if (finite(r)) {
#if FVDBM_PAIRED
    // (mx, my) folded side by side
    float2 m = sub2(make_float2(f[1], f[2]), make_float2(f[3], f[4]));
    m = add2(m, make_float2(f[5], f[5]));
    m = add2(m, make_float2(-f[6], f[6]));
    m = sub2(m, make_float2(f[7], f[7]));
    m = add2(m, make_float2(f[8], -f[8]));
    mx = m.x;
    my = m.y;
#else
    mx = ((((f[1] - f[3]) + f[5]) - f[6]) - f[7]) + f[8];
    my = ((((f[2] - f[4]) + f[5]) + f[6]) - f[7]) - f[8];
#endif
  } else {
    macros_literal(f, mx, my);
  }
  rho = r;
  ux = mx / r;
  uy = my / r;
}

// x == 0 or 2^-50 <= |x| <= 2^50: then x, x*x and sums of two such squares
// are dividends for which the known-divisor division is exact (the
// exhaustive check covers |x| >= 2^-100 with normal quotients).
__device__ __forceinline__ bool cdiv_domain(float x) {
  const float a = fabsf(x);
  return (a >= 0x1p-50f && a <= 0x1p50f) || x == 0.0f;
}

// feq_q = (W_q rho) * (((1 + a_q/C^2) + a_q^2/(2C^4)) - u.u/(2C^2)).
// With finite u: a_3 = -a_1, a_4 = -a_2, a_7 = -a_5, a_8 = -a_6 exactly, and
// a_0 = +-0 gives s_0 = 1 - u.u/(2C^2).  One range check per call decides
// whether all nine divisions take the three-operation form.
__device__ __forceinline__ void feq9(float rho, float ux, float uy, const DevPlan& p, float out[Q]) {
  if (!(finite(ux) && finite(uy))) {
    feq9_literal(rho, ux, uy, p, out);
    return;
  }
  const float uu = ux * ux + uy * uy;
  const float a5 = ux + uy, a6 = uy - ux;
  float t, x1, y1, x2, y2, x5, y5, x6, y6;
  const bool dom = cdiv_domain(ux) && cdiv_domain(uy) && cdiv_domain(a5) && cdiv_domain(a6);
  if (p.cdiv_mode == 2 && dom) {
    t = cdiv_two(uu, p.d_c2x2.zr, p.d_c2x2.zl);
    x1 = cdiv_two(ux, p.d_c2.zr, p.d_c2.zl);
    y1 = cdiv_two(ux * ux, p.d_c4x2.zr, p.d_c4x2.zl);
    x2 = cdiv_two(uy, p.d_c2.zr, p.d_c2.zl);
    y2 = cdiv_two(uy * uy, p.d_c4x2.zr, p.d_c4x2.zl);
    x5 = cdiv_two(a5, p.d_c2.zr, p.d_c2.zl);
    y5 = cdiv_two(a5 * a5, p.d_c4x2.zr, p.d_c4x2.zl);
    x6 = cdiv_two(a6, p.d_c2.zr, p.d_c2.zl);
    y6 = cdiv_two(a6 * a6, p.d_c4x2.zr, p.d_c4x2.zl);
  } else if (p.cdiv_mode == 1 && dom) {
    t = cdiv_fast(uu, p.d_c2x2.y, p.d_c2x2.zr);
    x1 = cdiv_fast(ux, p.d_c2.y, p.d_c2.zr);
    y1 = cdiv_fast(ux * ux, p.d_c4x2.y, p.d_c4x2.zr);
    x2 = cdiv_fast(uy, p.d_c2.y, p.d_c2.zr);
    y2 = cdiv_fast(uy * uy, p.d_c4x2.y, p.d_c4x2.zr);
    x5 = cdiv_fast(a5, p.d_c2.y, p.d_c2.zr);
    y5 = cdiv_fast(a5 * a5, p.d_c4x2.y, p.d_c4x2.zr);
    x6 = cdiv_fast(a6, p.d_c2.y, p.d_c2.zr);
    y6 = cdiv_fast(a6 * a6, p.d_c4x2.y, p.d_c4x2.zr);
  } else {
    t = cdiv(uu, p.d_c2x2);
    x1 = cdiv(ux, p.d_c2);
    y1 = cdiv(ux * ux, p.d_c4x2);
    x2 = cdiv(uy, p.d_c2);
    y2 = cdiv(uy * uy, p.d_c4x2);
    x5 = cdiv(a5, p.d_c2);
    y5 = cdiv(a5 * a5, p.d_c4x2);
    x6 = cdiv(a6, p.d_c2);
    y6 = cdiv(a6 * a6, p.d_c4x2);
  }
#if FVDBM_PAIRED
  // (s_1, s_3), (s_2, s_4), (s_5, s_7), (s_6, s_8) share x, y: one pair each
  const float2 one = make_float2(1.0f, 1.0f), tt = make_float2(t, t);
  const float2 s13 = sub2(add2(add2(one, make_float2(x1, -x1)), make_float2(y1, y1)), tt);
  const float2 s24 = sub2(add2(add2(one, make_float2(x2, -x2)), make_float2(y2, y2)), tt);
  const float2 s57 = sub2(add2(add2(one, make_float2(x5, -x5)), make_float2(y5, y5)), tt);
  const float2 s68 = sub2(add2(add2(one, make_float2(x6, -x6)), make_float2(y6, y6)), tt);
  const float w0 = c_W[0] * rho, w1 = c_W[1] * rho, w5 = c_W[5] * rho;
  const float2 w11 = make_float2(w1, w1), w55 = make_float2(w5, w5);
  const float2 o13 = mul2(w11, s13), o24 = mul2(w11, s24), o57 = mul2(w55, s57), o68 = mul2(w55, s68);
  out[0] = w0 * (1.0f - t);
  out[1] = o13.x;
  out[3] = o13.y;
  out[2] = o24.x;
  out[4] = o24.y;
  out[5] = o57.x;
  out[7] = o57.y;
  out[6] = o68.x;
  out[8] = o68.y;
#else
  float s[Q];
  s[0] = 1.0f - t;
  s[1] = ((1.0f + x1) + y1) - t;
  s[3] = ((1.0f - x1) + y1) - t;
  s[2] = ((1.0f + x2) + y2) - t;
  s[4] = ((1.0f - x2) + y2) - t;
  s[5] = ((1.0f + x5) + y5) - t;
  s[7] = ((1.0f - x5) + y5) - t;
  s[6] = ((1.0f + x6) + y6) - t;
  s[8] = ((1.0f - x6) + y6) - t;
#pragma unroll
  for (int q = 0; q < Q; ++q) out[q] = (c_W[q] * rho) * s[q];
#endif
}

// One component q of feq9, bitwise equal to feq9(...)[q].
__device__ __forceinline__ float feq_one(float rho, float ux, float uy, int q, const DevPlan& p) {
  if (!(finite(ux) && finite(uy))) {
    float a[Q];
    xi_dot_literal(ux, uy, a);
    const float uu = ux * ux + uy * uy;
    float s = 1.0f + a[q] / p.c2;
    s = s + (a[q] * a[q]) / p.c4x2;
    s = s - uu / p.c2x2;
    return (c_W[q] * rho) * s;
  }
  const float uu = ux * ux + uy * uy;
  const float t = cdiv(uu, p.d_c2x2);
  if (q == 0) return (c_W[0] * rho) * (1.0f - t);
  // a_q for q = 1..8 in the symmetric form: (+-) of ux, uy, ux+uy, uy-ux
  const int base = (q <= 4) ? ((q - 1) & 1) : 2 + ((q - 5) & 1);
  const float ab = base == 0 ? ux : base == 1 ? uy : base == 2 ? ux + uy : uy - ux;
  const bool neg = (q == 3 || q == 4 || q == 7 || q == 8);
  const float x = cdiv(ab, p.d_c2);
  const float y = cdiv(ab * ab, p.d_c4x2);
  const float s = ((neg ? 1.0f - x : 1.0f + x) + y) - t;
  return (c_W[q] * rho) * s;
}

// ---------------------------------------------------------------------------
// Contracted forms for the fast family (FVDBM_KERNEL_FAST).  Not the
// reference's rounding: explicit multiply-adds, multiplications by the
// rounded reciprocals of the lattice constants, an approximate reciprocal of
// rho, and no literal paths for non-finite values (NaN/inf propagate, but not
// with the reference's signs).  The evaluation order is fixed, so a step is
// still bitwise reproducible run to run; against the reference the step
// differs by a few float32 ulps per cell.

// rho = sum_q f_q (pairwise), u = (KSI^T f) * (1/rho)
__device__ __forceinline__ void macros_fast(const float f[Q], float& rho, float& ux, float& uy) {
  rho = ((f[0] + f[1]) + (f[2] + f[3])) + ((f[4] + f[5]) + (f[6] + f[7])) + f[8];
  const float mx = ((f[1] - f[3]) + (f[5] - f[6])) + (f[8] - f[7]);
  const float my = ((f[2] - f[4]) + (f[5] + f[6])) - (f[7] + f[8]);
  const float ir = __fdividef(1.0f, rho);
  ux = mx * ir;
  uy = my * ir;
}

// feq_q = W_q rho (1 - u.u/(2C^2) + a_q/C^2 + a_q^2/(2C^4)), a_q = xi_q . u,
// with the constants' reciprocals ic2 = 1/C^2, ic4x2 = 1/(2C^4), ic2x2 = 1/(2C^2)
__device__ __forceinline__ void feq9_fast(float rho, float ux, float uy, float ic2, float ic4x2, float ic2x2,
                                          float out[Q]) {
  const float base = __fmaf_rn(-__fmaf_rn(ux, ux, __fmul_rn(uy, uy)), ic2x2, 1.0f);
  const float w0 = c_W[0] * rho, w1 = c_W[1] * rho, w5 = c_W[5] * rho;
  const float a[4] = {ux, uy, ux + uy, uy - ux};
  out[0] = w0 * base;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float b = __fmaf_rn(__fmul_rn(a[j], a[j]), ic4x2, base);
    const float c = __fmul_rn(a[j], ic2);
    const float w = j < 2 ? w1 : w5;
    // directions (1, 3), (2, 4), (5, 7), (6, 8): +a and -a
    const int qp = j < 2 ? 1 + j : 5 + (j - 2);
    out[qp] = w * (b + c);
    out[qp + 2] = w * (b - c);
  }
}

// v_q = xi_q . n (src/containers.py:235); symmetric form for finite n
__device__ __forceinline__ void xi_dot_n(float nx, float ny, bool finite_n, float v[Q]) {
  if (!finite_n) {
    xi_dot_literal(nx, ny, v);
    return;
  }
  const float s = nx + ny, d = ny - nx;
  v[0] = 0.0f;
  v[1] = nx;
  v[2] = ny;
  v[3] = -nx;
  v[4] = -ny;
  v[5] = s;
  v[6] = d;
  v[7] = -s;
  v[8] = -d;
}

// Lax-Wendroff weights interp_q = d0/(d0+d1) - (v_q*dt)/(2(d0+d1))
// (src/containers.py:274); (-v*dt)/D2 == -((v*dt)/D2).
__device__ __forceinline__ void lw_interp(const float v[Q], float r, float D2, float dt,
                                          bool finite_n, float w[Q]) {
  if (!finite_n) {
    for (int q = 0; q < Q; ++q) w[q] = r - (v[q] * dt) / D2;
    return;
  }
  const float t1 = (v[1] * dt) / D2, t2 = (v[2] * dt) / D2;
  const float t5 = (v[5] * dt) / D2, t6 = (v[6] * dt) / D2;
  w[0] = r - (v[0] * dt) / D2;
  w[1] = r - t1;
  w[3] = r + t1;
  w[2] = r - t2;
  w[4] = r + t2;
  w[5] = r - t5;
  w[7] = r + t5;
  w[6] = r - t6;
  w[8] = r + t6;
}

}  // namespace fvdbm
