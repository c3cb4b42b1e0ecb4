// FVDBM step kernels for sm_103a (GB300): boundary nodes, the fused cell
// kernel, the staged face/gather pair, read-back helpers and the division
// self-check.  Arithmetic helpers live in fvdbm_math.cuh.
//
// Layout: cell pdfs are AoSoA [Np/32][9][32] float32 in device (renumbered)
// cell order; the fused kernel's per-cell face slots are AoSoA
// [Np/32][hrows][32]; node state is SoA [9][Mp].
#include <algorithm>
#include <utility>

#include "fvdbm_math.cuh"

namespace fvdbm {

// Acquire load of a flag written by other blocks of the same launch.
__device__ __forceinline__ int ld_acquire_gpu(const int* ptr) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(ptr) : "memory");
  return v;
}

// Bounded wait (one thread): spin until *ctr >= target with an acquire load,
// sleeping ns between polls, at most iters polls.  Returns false when the
// limit ran out; the caller then records STATUS_WAIT_TIMEOUT and skips the
// work that needed the wait, so the launch still ends.
__device__ __forceinline__ bool wait_at_least(const int* ctr, int target, int iters, unsigned ns) {
  for (int it = 0; it < iters; ++it) {
    if (ld_acquire_gpu(ctr) >= target) return true;
    __nanosleep(ns);
  }
  return false;
}

// Macros of a node-stencil cell for the next step's node kernel:
// rho, ux, uy, f_q - feq_q (src/containers.py:93-105,388-390).
__device__ __forceinline__ void record_stencil(const DevPlan& p, int i, const float fn[Q]) {
  float rho, ux, uy, eq[Q];
  macros(fn, rho, ux, uy);
  feq9(rho, ux, uy, p, eq);
  float* c = p.cprod + (i - p.stencil_start);
  c[0] = rho;
  c[size_t(p.Sp)] = ux;
  c[2 * size_t(p.Sp)] = uy;
#pragma unroll
  for (int q = 0; q < Q; ++q) c[(3 + q) * size_t(p.Sp)] = fn[q] - eq[q];
}

// ---------------------------------------------------------------------------
// Boundary nodes: Nodes.calc_pdfs (src/containers.py:339-404).  A block holds
// whole nodes with at most NODE_BLOCK_ENTRIES stencil entries:
//   1. one thread per entry: that cell's macros, feq and the IDW products
//      rho*w, u*w, (f - feq)*w (utils/utils.py:34-60) into shared memory;
//   2. one thread per node: the ordered folds over the node's entries (the
//      reference's sum order), then velocity nodes (type 1) take rho =
//      IDW(cell rho), density nodes (type 2) take u = IDW(cell u), and
//      pdf = feq(rho, u) + IDW(f - feq).
// WAIT: call grid_dep_wait() before reading f (false when the caller did).
template <bool WAIT>
__device__ __forceinline__ void node_block(const DevPlan& p, const float* __restrict__ f, int blk,
                                           float (*prod)[NODE_BLOCK_ENTRIES], float* lastm) {
  const int4 meta = __ldg(reinterpret_cast<const int4*>(p.nb_meta) + blk);  // n0, n1, e0, e1
  const int n0 = meta.x, nn = meta.y - meta.x, e0 = meta.z, ne = meta.w - meta.z;
  const int tid = threadIdx.x;
  // static tables first (they do not depend on the previous kernel)
  int b = 0, cnt = 0, npad = 0, type = 0;
  float sw = 0.0f, set0 = 0.0f, set1 = 0.0f;
  if (tid < nn) {
    const int m = n0 + tid;
    b = __ldg(p.nd_ptr + m) - e0;
    cnt = __ldg(p.nd_ptr + m + 1) - e0 - b;
    npad = __ldg(p.nd_npad + m);
    sw = __ldg(p.nd_sumw + m);
    type = __ldg(p.nd_type + m);
    if (type == 1) {
      set0 = p.node_vel[m];
      set1 = p.node_vel[p.Mp + m];
    } else {
      set0 = p.node_rho[m];
    }
  }
  unsigned code = 0;
  float w = 0.0f;
  if (tid < ne) {
    code = __ldg(p.nd_cell + e0 + tid);
    w = __ldg(p.nd_w + e0 + tid);
  }
  if (WAIT) grid_dep_wait();  // f comes from the previous cell kernel
  if (tid < ne) {
    float fc[Q], eq[Q];
    load_cell(f, int(code & ~ND_NEQ_ZERO), fc);
    float rho, ux, uy;
    macros(fc, rho, ux, uy);
    feq9(rho, ux, uy, p, eq);
    const bool zero = (code & ND_NEQ_ZERO) != 0;
    prod[0][tid] = rho * w;
    prod[1][tid] = ux * w;
    prod[2][tid] = uy * w;
#pragma unroll
    for (int q = 0; q < Q; ++q) prod[3 + q][tid] = (zero ? 0.0f : fc[q] - eq[q]) * w;
  }
  if (tid == NODE_BLOCK_ENTRIES - 1) {
    // padded (-1, weight 0) entries gather the last cell
    float fc[Q];
    load_cell(f, p.last_cell, fc);
    float rho, ux, uy;
    macros(fc, rho, ux, uy);
    lastm[0] = rho;
    lastm[1] = ux;
    lastm[2] = uy;
  }
  __syncthreads();
  if (tid >= nn) return;  // (callers do not synchronise after this)
  float acc[12];
#pragma unroll
  for (int r = 0; r < 12; ++r) acc[r] = 0.0f;
  for (int k = 0; k < cnt; ++k) {
#pragma unroll
    for (int r = 0; r < 12; ++r) acc[r] = k ? acc[r] + prod[r][b + k] : prod[r][b + k];
  }
  if (npad > 0) {
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const float z = lastm[r] * 0.0f;
      acc[r] = cnt ? acc[r] + z : z;
    }
  }
  const int m = n0 + tid;
  float rho_p, ux_p, uy_p;
  if (type == 1) {
    rho_p = acc[0] / sw;
    ux_p = set0;
    uy_p = set1;
    p.node_rho[m] = rho_p;
  } else {
    rho_p = set0;
    ux_p = acc[1] / sw;
    uy_p = acc[2] / sw;
    p.node_vel[m] = ux_p;
    p.node_vel[p.Mp + m] = uy_p;
  }
  float eqn[Q];
  feq9(rho_p, ux_p, uy_p, p, eqn);
#pragma unroll
  for (int q = 0; q < Q; ++q) p.node_pdf[size_t(q) * p.Mp + m] = eqn[q] + acc[3 + q] / sw;
}

__global__ void __launch_bounds__(NODE_BLOCK_ENTRIES) k_nodes(DevPlan p, const float* __restrict__ f) {
  __shared__ float prod[12][NODE_BLOCK_ENTRIES];
  __shared__ float lastm[3];
  grid_dep_launch();
  node_block<true>(p, f, blockIdx.x, prod, lastm);
}

// The same node evaluation, fed by the stencil macros that the previous
// fused kernel recorded (cprod) instead of re-reading the stencil pdfs.  The
// padded tables put a thread's entry and node record at blk*256 + tid, so the
// first loads do not depend on one another.  Results go to npdf/nrho/nvel,
// which also hold the set values (velocity of type-1, density of type-2
// nodes).  Padded entries read the last cell's macros from f, or from cprod
// when LAST_CPROD (the last cell is then a stencil cell).  WAIT: wait for the
// previous kernel before reading cprod.
template <bool WAIT, bool LAST_CPROD, bool F_CG = false>
__device__ __forceinline__ void node_block_cp(const DevPlan& p, int blk, const float* __restrict__ f,
                                              float* __restrict__ npdf, float* __restrict__ nrho,
                                              float* __restrict__ nvel, float (*prod)[NODE_BLOCK_ENTRIES],
                                              float* lastm) {
  const int tid = threadIdx.x;
  const size_t s = size_t(blk) * NODE_BLOCK_ENTRIES + tid;
  const unsigned slot = __ldg(p.pe_slot + s);
  const float w = __ldg(p.pe_w + s);
  const int4 nm = __ldg(reinterpret_cast<const int4*>(p.pn_meta) + s);  // node, first, count, type|npad
  const float sw = __ldg(p.pn_sumw + s);
  const int type = nm.w & 3;
  float set0 = 0.0f, set1 = 0.0f;
  if (type == 1) {
    set0 = nvel[nm.x];
    set1 = nvel[p.Mp + nm.x];
  } else if (type == 2) {
    set0 = nrho[nm.x];
  }
  if (WAIT) grid_dep_wait();  // cprod comes from the previous fused kernel
  if (slot != ~0u) {
    const float* c = p.cprod + (slot & ~ND_NEQ_ZERO);
    const bool zero = (slot & ND_NEQ_ZERO) != 0;
#pragma unroll
    for (int r = 0; r < 3; ++r) prod[r][tid] = __ldcg(c + r * size_t(p.Sp)) * w;
#pragma unroll
    for (int q = 0; q < Q; ++q) prod[3 + q][tid] = (zero ? 0.0f : __ldcg(c + (3 + q) * size_t(p.Sp))) * w;
  }
  if (tid == NODE_BLOCK_ENTRIES - 1) {
    // padded (-1, weight 0) entries gather the last cell
    if (LAST_CPROD) {
      if (p.last_slot >= 0)
#pragma unroll
        for (int r = 0; r < 3; ++r) lastm[r] = __ldcg(p.cprod + p.last_slot + r * size_t(p.Sp));
    } else {
      float fc[Q];
      if (F_CG)
        load_cell_cg(f, p.last_cell, fc);
      else
        load_cell(f, p.last_cell, fc);
      float rho, ux, uy;
      macros(fc, rho, ux, uy);
      lastm[0] = rho;
      lastm[1] = ux;
      lastm[2] = uy;
    }
  }
  __syncthreads();
  if (type != 0) {  // (no early return: callers may synchronise after this)
    const int b = nm.y, cnt = nm.z;
    float acc[12];
#pragma unroll
    for (int r = 0; r < 12; ++r) acc[r] = 0.0f;
    for (int k = 0; k < cnt; ++k) {
#pragma unroll
      for (int r = 0; r < 12; ++r) acc[r] = k ? acc[r] + prod[r][b + k] : prod[r][b + k];
    }
    if (nm.w & 4) {
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        const float z = lastm[r] * 0.0f;
        acc[r] = cnt ? acc[r] + z : z;
      }
    }
    const int m = nm.x;
    float rho_p, ux_p, uy_p;
    if (type == 1) {
      rho_p = acc[0] / sw;
      ux_p = set0;
      uy_p = set1;
      nrho[m] = rho_p;
    } else {
      rho_p = set0;
      ux_p = acc[1] / sw;
      uy_p = acc[2] / sw;
      nvel[m] = ux_p;
      nvel[p.Mp + m] = uy_p;
    }
    float eqn[Q];
    feq9(rho_p, ux_p, uy_p, p, eqn);
#pragma unroll
    for (int q = 0; q < Q; ++q) npdf[size_t(q) * p.Mp + m] = eqn[q] + acc[3 + q] / sw;
  }
}

__global__ void __launch_bounds__(NODE_BLOCK_ENTRIES) k_nodes_cp(DevPlan p, const float* __restrict__ f) {
  __shared__ float prod[12][NODE_BLOCK_ENTRIES];
  __shared__ float lastm[3];
  grid_dep_launch();
  if (p.stencil_first)
    node_block_cp<true, true>(p, blockIdx.x, f, p.node_pdf, p.node_rho, p.node_vel, prod, lastm);
  else
    node_block_cp<true, false>(p, blockIdx.x, f, p.node_pdf, p.node_rho, p.node_vel, prod, lastm);
}

__global__ void __launch_bounds__(256) k_stencil_macros(DevPlan p, const float* __restrict__ f) {
  const int i = p.stencil_start + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.stencil_end) return;
  float fc[Q];
  load_cell(f, i, fc);
  record_stencil(p, i, fc);
}

// ---------------------------------------------------------------------------
// Fused cell kernel: macros, feq, the flux of each of the cell's faces
// (recomputed from the canonical slot-0/slot-1 pair, so both neighbours get
// bit-identical fluxes without a flux array or atomics), the signed flux sum
// and the BGK/explicit-Euler update (src/containers.py:107-121).
// The pdfs across face slot `code`: the neighbour cell's, or the ghost value
// m + (m - f_known)*(d_ghost/d_known), m = mean of the face's two end-node
// pdfs (src/containers.py:280-287, utils/utils.py:153).
template <bool GHOST_CG>
__device__ __forceinline__ void face_other(const DevPlan& p, const float* __restrict__ fin, int code,
                                           const float f[Q], float o[Q]) {
  const int other = code >> HF_SHIFT;
  if (code & HF_GHOST) {
    const int a = __ldg(p.gh_a + other), b = __ldg(p.gh_b + other);
    const float rg = __ldg(p.gh_r + other);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const float* pa = p.node_pdf + size_t(q) * p.Mp + a;
      const float* pb = p.node_pdf + size_t(q) * p.Mp + b;
      const float mq = (GHOST_CG ? (__ldcg(pa) + __ldcg(pb)) : (__ldg(pa) + __ldg(pb))) / 2.0f;
      o[q] = mq + (mq - f[q]) * rg;
    }
  } else if (GHOST_CG) {
    load_cell_cg(fin, other, o);
  } else {
    load_cell(fin, other, o);
  }
}

// Flux of face slot k from this cell's pdfs f and the pdfs o across it,
// signed for this cell, into acc (first slot: assigned).
template <int SCHEME, int VARIANT, bool FIRST>
__device__ __forceinline__ void face_flux(const DevPlan& p, const unsigned* __restrict__ hb, int k, int code,
                                          float nx, float ny, float Ls, float dt, const float f[Q],
                                          const float o[Q], float acc[Q]) {
  const HfRows HR{3, SCHEME, VARIANT};
  const bool slot1 = (code & HF_SLOT1) != 0;
  float v[Q];
  xi_dot_n(nx, ny, p.finite_n != 0, v);
  float w[Q];
  if (SCHEME == 1)
    lw_interp(v, __uint_as_float(__ldg(hb + HR.r(k) * 32)), __uint_as_float(__ldg(hb + HR.d2(k) * 32)),
              dt, p.finite_n != 0, w);
  const float scale = (VARIANT == 1) ? __uint_as_float(__ldg(hb + HR.sc(k) * 32)) : 1.0f;
#if FVDBM_PAIRED
  if constexpr (SCHEME == 0 && VARIANT == 0) {
    float phi[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q) phi[q] = ((v[q] >= 0.0f) != slot1) ? f[q] : o[q];
    const float2 L2 = make_float2(Ls, Ls), one2 = make_float2(p.one, p.one);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const float2 x = mul2(mul2(make_float2(phi[2 * j], phi[2 * j + 1]), make_float2(v[2 * j], v[2 * j + 1])), L2);
      const float2 a = FIRST ? x : fold2(make_float2(acc[2 * j], acc[2 * j + 1]), one2, x);
      acc[2 * j] = a.x;
      acc[2 * j + 1] = a.y;
    }
    const float x8 = (phi[8] * v[8]) * Ls;
    acc[8] = FIRST ? x8 : acc[8] + x8;
  } else
#endif
  {
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
}

template <int SCHEME, int VARIANT, bool FIRST, bool GHOST_CG>
__device__ __forceinline__ void fused_face(const DevPlan& p, const float* __restrict__ fin,
                                           const unsigned* __restrict__ hb, int k, int code, float nx,
                                           float ny, float Ls, float dt, const float f[Q], float acc[Q]) {
  float o[Q];
  face_other<GHOST_CG>(p, fin, code, f, o);
  face_flux<SCHEME, VARIANT, FIRST>(p, hb, k, code, nx, ny, Ls, dt, f, o, acc);
}

__device__ __forceinline__ void prefetch_l2(const void* ptr, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(ptr), "r"(bytes) : "memory");
}

// One cell of the fused update.  GHOST_CG: read node pdfs, and the cell
// pdfs, through L2 (for data written earlier in the same launch).  RECORD: node-stencil cells also
// record the macros of their new pdfs.  inv_tau and dt are the cell's case's.
template <int SCHEME, int VARIANT, bool FV, bool GHOST_CG, bool RECORD = false>
__device__ __forceinline__ void fused_cell_f(const DevPlan& p, const float* __restrict__ fin,
                                             float* __restrict__ fout, int i, const float f[Q],
                                             const int code[3], const float nx[3], const float ny[3],
                                             const float Ls[3], const unsigned* __restrict__ hb,
                                             float inv_tau, float dt) {
  float acc[Q];
  fused_face<SCHEME, VARIANT, true, GHOST_CG>(p, fin, hb, 0, code[0], nx[0], ny[0], Ls[0], dt, f, acc);
  fused_face<SCHEME, VARIANT, false, GHOST_CG>(p, fin, hb, 1, code[1], nx[1], ny[1], Ls[1], dt, f, acc);
  fused_face<SCHEME, VARIANT, false, GHOST_CG>(p, fin, hb, 2, code[2], nx[2], ny[2], Ls[2], dt, f, acc);
  float rho, ux, uy, eq[Q];
  macros(f, rho, ux, uy);
  feq9(rho, ux, uy, p, eq);
  if (FV) {
    const float ia = __ldg(p.inv_area + i);
#pragma unroll
    for (int q = 0; q < Q; ++q) acc[q] = acc[q] * ia;
  }
  float* o = fout + cell_base(i, Q);
  float fn[Q];
#if FVDBM_PAIRED
  // f + dt*(inv_tau*(eq - f) - acc), pairwise
  const float2 it2 = make_float2(inv_tau, inv_tau), dt2 = make_float2(dt, dt);
  const float2 one2 = make_float2(p.one, p.one), m12 = make_float2(p.neg_one, p.neg_one);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const float2 f2 = make_float2(f[2 * j], f[2 * j + 1]);
    const float2 d = fold2(f2, m12, make_float2(eq[2 * j], eq[2 * j + 1]));    // eq - f
    const float2 u = fold2(make_float2(acc[2 * j], acc[2 * j + 1]), m12, mul2(it2, d));  // - acc
    const float2 r = fold2(f2, one2, mul2(dt2, u));                               // f + ...
    fn[2 * j] = r.x;
    fn[2 * j + 1] = r.y;
  }
  fn[8] = f[8] + dt * (inv_tau * (eq[8] - f[8]) - acc[8]);
#pragma unroll
  for (int q = 0; q < Q; ++q) o[q * 32] = fn[q];
#else
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    fn[q] = f[q] + dt * (inv_tau * (eq[q] - f[q]) - acc[q]);
    o[q * 32] = fn[q];
  }
#endif
  if (RECORD && i >= p.stencil_start && i < p.stencil_end) record_stencil(p, i, fn);
}

template <int SCHEME, int VARIANT, bool FV, bool GHOST_CG, bool RECORD = false>
__device__ __forceinline__ void fused_cell(const DevPlan& p, const float* __restrict__ fin,
                                           float* __restrict__ fout, int i, const int code[3],
                                           const float nx[3], const float ny[3], const float Ls[3],
                                           const unsigned* __restrict__ hb) {
  float f[Q];
  if (GHOST_CG)
    load_cell_cg(fin, i, f);
  else
    load_cell(fin, i, f);
  fused_cell_f<SCHEME, VARIANT, FV, GHOST_CG, RECORD>(p, fin, fout, i, f, code, nx, ny, Ls, hb, p.inv_tau, p.dt);
}

// ---------------------------------------------------------------------------
// The fast family's cell update (FVDBM_KERNEL_FAST): the same step with
// contracted arithmetic (fvdbm_math.cuh, "contracted forms") on compact face
// slots: a = n * (L*sigma [*scale] [/area]) per face slot (HfFastRows), so
// that xi_q . a is the flux coefficient of direction q.  Direction q = 0 has
// xi.n = 0 and carries no flux; the pairs (1, 3), (2, 4), (5, 7), (6, 8)
// share |xi.a|.
//
// All nine pdfs across face slot `code` (Lax-Wendroff): the neighbour's, or
// the ghost value m + (m - f) * rg as a multiply-add.
__device__ __forceinline__ void face_other_fast(const DevPlan& p, const float* __restrict__ fin, int code,
                                                const float f[Q], float o[Q]) {
  const int other = code >> HF_SHIFT;
  if (code & HF_GHOST) {
    const int a = __ldg(p.gh_a + other), b = __ldg(p.gh_b + other);
    const float rg = __ldg(p.gh_r + other);
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      const float mq = (__ldg(p.node_pdf + size_t(q) * p.Mp + a) + __ldg(p.node_pdf + size_t(q) * p.Mp + b)) * 0.5f;
      o[q] = __fmaf_rn(mq - f[q], rg, mq);
    }
  } else {
    load_cell(fin, other, o);
  }
}

// Lax-Wendroff flux of one compact face slot:
// phi = l + (r - l) * (d0/(d0+d1) - (xi.n) dt/(2(d0+d1))), where
// (xi.n) dt/(2(d0+d1)) = (xi.a) * g.
__device__ __forceinline__ void face_lw_fast(int code, float ax, float ay, float r, float g, const float f[Q],
                                             const float o[Q], float acc[Q]) {
  const bool slot1 = (code & HF_SLOT1) != 0;
  const float a4[4] = {ax, ay, ax + ay, ay - ax};
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int qp = j < 2 ? 1 + j : 5 + (j - 2), qm = qp + 2;  // xi.a = +a4[j], -a4[j]
    const float lp = slot1 ? o[qp] : f[qp], rp = slot1 ? f[qp] : o[qp];
    const float lm = slot1 ? o[qm] : f[qm], rm = slot1 ? f[qm] : o[qm];
    const float pp = __fmaf_rn(rp - lp, __fmaf_rn(-a4[j], g, r), lp);
    const float pm = __fmaf_rn(rm - lm, __fmaf_rn(a4[j], g, r), lm);
    acc[qp] = __fmaf_rn(pp, a4[j], acc[qp]);
    acc[qm] = __fmaf_rn(-pm, a4[j], acc[qm]);
  }
}

// Upwind flux of one compact face slot, reading only the pdfs it uses: of
// each direction pair (q, opposite q) with xi.a = +a, -a exactly one takes
// the value across the face (the inflow one), so a face needs 4 values of
// the neighbour (or of the ghost), not 9, at a row that varies by lane.
__device__ __forceinline__ void face_upwind_fast(const DevPlan& p, const float* __restrict__ fin, int code,
                                                 float ax, float ay, const float f[Q], float acc[Q]) {
  const int other = code >> HF_SHIFT;
  const bool slot1 = (code & HF_SLOT1) != 0;
  const float a4[4] = {ax, ay, ax + ay, ay - ax};
  bool up[4];
  int qn[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int qp = j < 2 ? 1 + j : 5 + (j - 2);
    up[j] = (a4[j] >= 0.0f) != slot1;  // qp flows out (this cell's value), qp + 2 flows in
    qn[j] = up[j] ? qp + 2 : qp;
  }
  float o4[4];
  if (code & HF_GHOST) {
    const int a = __ldg(p.gh_a + other), b = __ldg(p.gh_b + other);
    const float rg = __ldg(p.gh_r + other);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int qp = j < 2 ? 1 + j : 5 + (j - 2);
      const float fq = up[j] ? f[qp + 2] : f[qp];
      const float* np_ = p.node_pdf + size_t(qn[j]) * p.Mp;
      const float mq = (__ldg(np_ + a) + __ldg(np_ + b)) * 0.5f;
      o4[j] = __fmaf_rn(mq - fq, rg, mq);
    }
  } else {
    const float* b = fin + cell_base(other, Q);
#pragma unroll
    for (int j = 0; j < 4; ++j) o4[j] = __ldg(b + qn[j] * 32);
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int qp = j < 2 ? 1 + j : 5 + (j - 2), qm = qp + 2;
    const float pp = up[j] ? f[qp] : o4[j];
    const float pm = up[j] ? o4[j] : f[qm];
    acc[qp] = __fmaf_rn(pp, a4[j], acc[qp]);
    acc[qm] = __fmaf_rn(-pm, a4[j], acc[qm]);
  }
}

template <int SCHEME>
__device__ __forceinline__ void load_slots_fast(const DevPlan& p, int i, const unsigned*& hb, int code[3],
                                                float ax[3], float ay[3]) {
  constexpr int HROWS = (3 + (SCHEME == 1 ? 2 : 0)) * 3;
  const HfFastRows HX{3, SCHEME};
  hb = p.hf + cell_base(i < p.N ? i : 0, HROWS);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    code[k] = int(__ldg(hb + HX.code(k) * 32));
    ax[k] = __uint_as_float(__ldg(hb + HX.ax(k) * 32));
    ay[k] = __uint_as_float(__ldg(hb + HX.ay(k) * 32));
  }
}

template <int SCHEME>
__device__ __forceinline__ void fused_cell_fast(const DevPlan& p, const float* __restrict__ fin,
                                                float* __restrict__ fout, int i, const int code[3],
                                                const float ax[3], const float ay[3],
                                                const unsigned* __restrict__ hb) {
  const HfFastRows HX{3, SCHEME};
  float f[Q];
  load_cell(fin, i, f);
  float acc[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) acc[q] = 0.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (SCHEME == 0) {
      face_upwind_fast(p, fin, code[k], ax[k], ay[k], f, acc);
    } else {
      float o[Q];
      face_other_fast(p, fin, code[k], f, o);
      const float r = __uint_as_float(__ldg(hb + HX.r(k) * 32));
      const float g = __uint_as_float(__ldg(hb + HX.g(k) * 32));
      face_lw_fast(code[k], ax[k], ay[k], r, g, f, o, acc);
    }
  }
  float rho, ux, uy, eq[Q];
  macros_fast(f, rho, ux, uy);
  feq9_fast(rho, ux, uy, p.d_c2.zr, p.d_c4x2.zr, p.d_c2x2.zr, eq);
  // f + dt*(inv_tau*(eq - f) - acc) (acc already carries 1/area in
  // finite-volume mode)
  const float om = p.dt * p.inv_tau;
  float* out = fout + cell_base(i, Q);
  float fn[Q];
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    fn[q] = __fmaf_rn(-p.dt, acc[q], __fmaf_rn(om, eq[q] - f[q], f[q]));
    out[q * 32] = fn[q];
  }
  if (i >= p.stencil_start && i < p.stencil_end) record_stencil(p, i, fn);
}

template <int SCHEME, int VARIANT>
__device__ __forceinline__ void load_slots(const DevPlan& p, int i, const unsigned*& hb, int code[3],
                                           float nx[3], float ny[3], float Ls[3]) {
  constexpr int HROWS = (4 + (SCHEME == 1 ? 2 : 0) + (VARIANT == 1 ? 1 : 0)) * 3;
  const HfRows HR{3, SCHEME, VARIANT};
  hb = p.hf + cell_base(i < p.N ? i : 0, HROWS);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    code[k] = int(__ldg(hb + HR.code(k) * 32));
    nx[k] = __uint_as_float(__ldg(hb + HR.nx(k) * 32));
    ny[k] = __uint_as_float(__ldg(hb + HR.ny(k) * 32));
    Ls[k] = __uint_as_float(__ldg(hb + HR.ls(k) * 32));  // L * sigma
  }
}

template <int SCHEME, int VARIANT, bool FV>
__global__ void __launch_bounds__(256) k_fused(DevPlan p, const float* __restrict__ fin,
                                               float* __restrict__ fout, int prefetch_blocks) {
  constexpr int HROWS = (4 + (SCHEME == 1 ? 2 : 0) + (VARIANT == 1 ? 1 : 0)) * 3;
  grid_dep_launch();
  // the block about one wave ahead streams into L2 while this one computes
  const int ahead = blockIdx.x + prefetch_blocks;
  const bool do_prefetch = threadIdx.x == 0 && prefetch_blocks > 0 && ahead < int(gridDim.x);
  // cells [ahead*256, min(+256, Np)): whole 32-cell groups, a multiple of 16 bytes
  const int pf_cells = do_prefetch ? min(256, p.Np - ahead * 256) : 0;
  if (pf_cells > 0) prefetch_l2(p.hf + size_t(ahead) * 256 * HROWS, pf_cells * HROWS * sizeof(unsigned));
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const unsigned* hb;
  int code[3];
  float nx[3], ny[3], Ls[3];
  load_slots<SCHEME, VARIANT>(p, i, hb, code, nx, ny, Ls);
  grid_dep_wait();  // fin and the node pdfs come from the previous kernels
  if (pf_cells > 0) prefetch_l2(fin + size_t(ahead) * 256 * Q, pf_cells * Q * sizeof(float));
  if (i >= p.N) return;
  fused_cell<SCHEME, VARIANT, FV, false, true>(p, fin, fout, i, code, nx, ny, Ls, hb);
}



// The fused cell kernel with the next step's boundary-node update in the same
// launch.  The node-stencil cells come first (cell blocks [0, R) record their
// new macros); the NB node blocks sit at grid position node_at.  A node block
// waits (bounded; on timeout it sets the status word and skips its nodes)
// until the R recording blocks have published, then evaluates its nodes from
// the recorded macros into the next step's node buffers, while the remaining
// cell blocks still run.  This step's ghost faces read the current node
// buffers, written by the previous launch.  The last node block to finish
// resets the two counters for the next launch.  At most NB blocks wait, far
// fewer than the resident blocks, so the recording blocks always get an SM.
template <int SCHEME, int VARIANT, bool FV, bool FAST>
__device__ __forceinline__ void fused_nodes_block(const DevPlan& p, const float* __restrict__ fin,
                                                  float* __restrict__ fout, int R, int node_at,
                                                  int prefetch_blocks) {
  constexpr int HROWS = FAST ? (3 + (SCHEME == 1 ? 2 : 0)) * 3 : (4 + (SCHEME == 1 ? 2 : 0) + (VARIANT == 1 ? 1 : 0)) * 3;
  static_assert(NODE_BLOCK_ENTRIES == 256, "node blocks use the whole CTA");
  __shared__ float prod[12][NODE_BLOCK_ENTRIES];
  __shared__ float lastm[3];
  __shared__ int s_ok;
  grid_dep_launch();
  const int b = blockIdx.x;
  int* ctr = p.step_ctr;  // [0] recording blocks published, [1] node blocks finished
  if (b >= node_at && b < node_at + p.NB) {
    grid_dep_wait();  // counters and set values of the previous launch
    if (threadIdx.x == 0) {
      const bool ok = wait_at_least(&ctr[0], R, 1 << 22, 128);
      if (!ok) atomicExch(p.status, STATUS_WAIT_TIMEOUT);
      s_ok = ok;
    }
    __syncthreads();
    if (s_ok) node_block_cp<false, true>(p, b - node_at, fin, p.node_pdf_nx, p.node_rho_nx, p.node_vel_nx, prod, lastm);
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      if (atomicAdd(&ctr[1], 1) == p.NB - 1) {
        ctr[0] = 0;
        ctr[1] = 0;
        __threadfence();
      }
    }
    return;
  }
  const int cb = b < node_at ? b : b - p.NB;
  const int ncb = int(gridDim.x) - p.NB;
  const int ahead = cb + prefetch_blocks;
  const bool do_prefetch = threadIdx.x == 0 && prefetch_blocks > 0 && ahead < ncb;
  const int pf_cells = do_prefetch ? min(256, p.Np - ahead * 256) : 0;
  if (pf_cells > 0) prefetch_l2(p.hf + size_t(ahead) * 256 * HROWS, pf_cells * HROWS * sizeof(unsigned));
  const int i = cb * 256 + threadIdx.x;
  const unsigned* hb;
  int code[3];
  if constexpr (FAST) {
    float ax[3], ay[3];
    load_slots_fast<SCHEME>(p, i, hb, code, ax, ay);
    grid_dep_wait();  // fin and the node pdfs come from the previous launch
    if (pf_cells > 0) prefetch_l2(fin + size_t(ahead) * 256 * Q, pf_cells * Q * sizeof(float));
    if (i < p.N) fused_cell_fast<SCHEME>(p, fin, fout, i, code, ax, ay, hb);
  } else {
    float nx[3], ny[3], Ls[3];
    load_slots<SCHEME, VARIANT>(p, i, hb, code, nx, ny, Ls);
    grid_dep_wait();  // fin and the node pdfs come from the previous launch
    if (pf_cells > 0) prefetch_l2(fin + size_t(ahead) * 256 * Q, pf_cells * Q * sizeof(float));
    if (i < p.N) fused_cell<SCHEME, VARIANT, FV, false, true>(p, fin, fout, i, code, nx, ny, Ls, hb);
  }
  if (cb < R) {
    __syncthreads();
    if (threadIdx.x == 0) {
      __threadfence();
      atomicAdd(&ctr[0], 1);
    }
  }
}

template <int SCHEME, int VARIANT, bool FV>
__global__ void __launch_bounds__(256) k_fused_nodes(DevPlan p, const float* __restrict__ fin,
                                                     float* __restrict__ fout, int R, int node_at,
                                                     int prefetch_blocks) {
  fused_nodes_block<SCHEME, VARIANT, FV, false>(p, fin, fout, R, node_at, prefetch_blocks);
}

// The fast family's launch: the same blocks with the contracted cell update
// on the compact half faces (the face scale and 1/area are folded into them,
// so only the flux scheme is a template parameter).  On the 1M step five
// resident blocks per SM (48 registers) measured 26.9 us per launch, four
// 28.8 us and six (40 registers, with spills) 27.8 us; the L2 prefetch
// distance of the bit-exact kernel (two blocks per SM ahead) 26.9 us against
// 27.2 (none), 27.9 (four) and 28.5 us (six).
#ifndef FVDBM_FAST_MIN_BLOCKS
#define FVDBM_FAST_MIN_BLOCKS 5
#endif
template <int SCHEME>
__global__ void __launch_bounds__(256, FVDBM_FAST_MIN_BLOCKS)
    k_fused_nodes_fast(DevPlan p, const float* __restrict__ fin, float* __restrict__ fout, int R, int node_at,
                       int prefetch_blocks) {
  fused_nodes_block<SCHEME, 0, false, true>(p, fin, fout, R, node_at, prefetch_blocks);
}

// ---------------------------------------------------------------------------
// Persistent multi-step kernel (cooperative launch: every block resident).
// Step s is the two-launch family's step: the boundary nodes from the
// recorded stencil macros (cprod), the node kernel's blocks, then the fused cell
// update of every cell from buffer f[s & 1] into f[(s + 1) & 1], which
// records cprod for the next step.  A grid barrier separates the phases, so
// each step costs two barriers instead of two launches.  The barrier is a
// monotonic arrival counter (zeroed by the host before the launch) with a
// bounded wait; a wait that runs out sets the status word and every block
// leaves at its next barrier.

// Grid barrier number k (k = 1, 2, ...): arrive, then wait (thread 0,
// bounded) until every block has arrived k times.  Returns false, with the
// status word set, when the wait ran out or another block already gave up.
__device__ __forceinline__ bool grid_barrier(const DevPlan& p, int* bar, int k, int* s_ok) {
  __threadfence();  // this thread's writes before the arrival
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(bar, 1);
    // a tight spin (no sleep between polls: a barrier lasts about a
    // microsecond), bounded to 2^24 polls
    const int target = k * int(gridDim.x);
    bool ok = false;
    for (int it = 0; it < (1 << 24); ++it)
      if (ld_acquire_gpu(bar) >= target) {
        ok = true;
        break;
      }
    if (!ok) atomicExch(p.status, STATUS_WAIT_TIMEOUT);
    *s_ok = ok && ld_acquire_gpu(p.status) == 0;
  }
  __syncthreads();
  return *s_ok != 0;
}

template <int SCHEME, int VARIANT, bool FV>
__global__ void __launch_bounds__(256) k_persist(DevPlan p, float* f0, float* f1, int n_steps, int* bar) {
  __shared__ int s_ok;
  __shared__ float prod[12][NODE_BLOCK_ENTRIES];
  __shared__ float lastm[3];
  const int ncb = (p.N + 255) / 256;
  int k = 0;
  for (int s = 0; s < n_steps; ++s) {
    const float* fin = (s & 1) ? f1 : f0;
    float* fout = (s & 1) ? f0 : f1;
    // boundary nodes of step s from the macros of fin (cprod): the node
    // kernel's entry-parallel blocks, spread over the grid
    for (int nb = blockIdx.x; nb < p.NB; nb += gridDim.x) {
      node_block_cp<false, false, true>(p, nb, fin, p.node_pdf, p.node_rho, p.node_vel, prod, lastm);
      __syncthreads();  // prod is reused by the block's next node block
    }
    if (!grid_barrier(p, bar, ++k, &s_ok)) return;
    // cells of step s
    for (int cb = blockIdx.x; cb < ncb; cb += gridDim.x) {
      const int i = cb * 256 + threadIdx.x;
      const unsigned* hb;
      int code[3];
      float nx[3], ny[3], Ls[3];
      load_slots<SCHEME, VARIANT>(p, i, hb, code, nx, ny, Ls);
      if (i < p.N) fused_cell<SCHEME, VARIANT, FV, true, 1>(p, fin, fout, i, code, nx, ny, Ls, hb);
    }
    if (!grid_barrier(p, bar, ++k, &s_ok)) return;
  }
}

template <int S, int V>
static cudaError_t persist_dispatch(const DevPlan& p, float* f0, float* f1, int n_steps, int* bar,
                                    cudaStream_t s) {
  void (*kern)(DevPlan, float*, float*, int, int*) = p.fv ? k_persist<S, V, true> : k_persist<S, V, false>;
  int dev = 0, sms = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, 0);
  if (e != cudaSuccess) return e;
  if (per_sm < 1) return cudaErrorInvalidConfiguration;
  const int ncb = (p.N + 255) / 256;
  const int grid = std::max(1, std::min(std::max(ncb, p.NB), per_sm * sms));
  e = cudaMemsetAsync(bar, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  DevPlan pp = p;
  void* args[] = {&pp, &f0, &f1, &n_steps, &bar};
  return cudaLaunchCooperativeKernel(reinterpret_cast<const void*>(kern), dim3(grid), dim3(256), args, 0, s);
}

cudaError_t launch_persist(const DevPlan& p, float* f0, float* f1, int n_steps, int* bar, cudaStream_t s) {
  if (p.N == 0 || n_steps <= 0) return cudaSuccess;
  if (p.K != 3) return cudaErrorInvalidValue;
  if (p.scheme == 0 && p.variant == 0) return persist_dispatch<0, 0>(p, f0, f1, n_steps, bar, s);
  if (p.scheme == 1 && p.variant == 0) return persist_dispatch<1, 0>(p, f0, f1, n_steps, bar, s);
  if (p.scheme == 0 && p.variant == 1) return persist_dispatch<0, 1>(p, f0, f1, n_steps, bar, s);
  if (p.scheme == 1 && p.variant == 1) return persist_dispatch<1, 1>(p, f0, f1, n_steps, bar, s);
  return cudaErrorInvalidValue;
}

// Packed batch of independent cases: the same cell update with the cell's
// case's 1/tau and dt; cells of retired cases are neither read nor written
// (both pdf buffers hold their final state).  Block size 128 or 256; the
// block `prefetch_blocks` ahead streams into L2.
template <int SCHEME, int VARIANT, bool FV>
__global__ void __launch_bounds__(256) k_fused_batch(DevPlan p, const float* __restrict__ fin,
                                                     float* __restrict__ fout, int prefetch_blocks) {
  constexpr int HROWS = (4 + (SCHEME == 1 ? 2 : 0) + (VARIANT == 1 ? 1 : 0)) * 3;
  grid_dep_launch();
  const int T = blockDim.x;
  const int blk = p.blk_list ? __ldg(p.blk_list + blockIdx.x) : int(blockIdx.x);
  const int i = blk * T + threadIdx.x;
  const int cs = __ldg(p.cell_case + min(i, p.Np - 1));
  const int ahead_idx = blockIdx.x + prefetch_blocks;
  const bool do_prefetch = threadIdx.x == 0 && prefetch_blocks > 0 && ahead_idx < int(gridDim.x);
  const int ahead = do_prefetch ? (p.blk_list ? __ldg(p.blk_list + ahead_idx) : ahead_idx) : 0;
  const int pf_cells = do_prefetch ? min(T, p.Np - ahead * T) : 0;
  if (pf_cells > 0) prefetch_l2(p.hf + size_t(ahead) * T * HROWS, pf_cells * HROWS * sizeof(unsigned));
  const unsigned* hb;
  int code[3];
  float nx[3], ny[3], Ls[3];
  load_slots<SCHEME, VARIANT>(p, i, hb, code, nx, ny, Ls);
  const float inv_tau = __ldg(p.case_inv_tau + cs), dt = __ldg(p.case_dt + cs);
  grid_dep_wait();  // fin, the node pdfs and the active flags come from earlier work
  if (pf_cells > 0) prefetch_l2(fin + size_t(ahead) * T * Q, pf_cells * Q * sizeof(float));
  if (i >= p.N || !p.case_active[cs]) return;
  float f[Q];
  load_cell(fin, i, f);
  fused_cell_f<SCHEME, VARIANT, FV, false, false>(p, fin, fout, i, f, code, nx, ny, Ls, hb, inv_tau, dt);
}

// ---------------------------------------------------------------------------
// Whole step in one launch.  Blocks take tickets in the order they start
// (atomicAdd after griddepcontrol.wait); a static schedule maps each ticket
// to a node block or a 256-cell block.  Node blocks are interleaved with the
// ghost-free cell blocks (their latency overlaps cell work) and publish their
// results (nodes_done); the cell blocks with ghost faces come last and wait
// (bounded) until every node block has published.  Tickets follow start
// order, so every node ticket before a waiting block belongs to a block that
// is already running: the wait cannot starve.  The last block to finish
// resets the counters for the next launch.

template <int SCHEME, int VARIANT, bool FV>
__global__ void __launch_bounds__(256) k_step(DevPlan p, const float* __restrict__ fin,
                                              float* __restrict__ fout, int n_cell_blocks,
                                              int prefetch_blocks) {
  static_assert(NODE_BLOCK_ENTRIES == 256, "node blocks use the whole CTA");
  __shared__ float prod[12][NODE_BLOCK_ENTRIES];
  __shared__ float lastm[3];
  __shared__ int s_ticket, s_ok;
  grid_dep_launch();
  grid_dep_wait();  // fin, and the counters reset by the previous launch
  int* ctr = p.step_ctr;  // [0] ticket, [1] nodes published, [2] blocks finished
  if (threadIdx.x == 0) s_ticket = atomicAdd(&ctr[0], 1);
  __syncthreads();
  const int t = s_ticket;
  const int work = __ldg(p.sched + t);
  if (work < 0) {
    node_block<false>(p, fin, -work - 1, prod, lastm);
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(&ctr[1], 1);
  } else {
    constexpr int HROWS = (4 + (SCHEME == 1 ? 2 : 0) + (VARIANT == 1 ? 1 : 0)) * 3;
    const int cb = work;
    // the cell block about one wave ahead in ticket order streams into L2
    const int ta = t + prefetch_blocks;
    if (threadIdx.x == 0 && ta < p.NB + n_cell_blocks) {
      const int wa = __ldg(p.sched + ta);
      if (wa >= 0) {
        const size_t c0 = size_t(wa) * 256;
        prefetch_l2(fin + c0 * Q, 256 * Q * sizeof(float));
        prefetch_l2(p.hf + c0 * HROWS, 256 * HROWS * sizeof(unsigned));
      }
    }
    const int i = cb * 256 + threadIdx.x;
    const unsigned* hb;
    int code[3];
    float nx[3], ny[3], Ls[3];
    load_slots<SCHEME, VARIANT>(p, i, hb, code, nx, ny, Ls);
    if (__ldg(p.cblk_ghost + cb)) {
      if (threadIdx.x == 0) {
        const bool ok = wait_at_least(&ctr[1], p.NB, 1 << 24, 64);
        if (!ok) atomicExch(p.status, STATUS_WAIT_TIMEOUT);
        s_ok = ok;
      }
      __syncthreads();
      if (s_ok && i < p.N) fused_cell<SCHEME, VARIANT, FV, true>(p, fin, fout, i, code, nx, ny, Ls, hb);
    } else if (i < p.N) {
      fused_cell<SCHEME, VARIANT, FV, false>(p, fin, fout, i, code, nx, ny, Ls, hb);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&ctr[2], 1) == p.NB + n_cell_blocks - 1) {
      ctr[0] = 0;
      ctr[1] = 0;
      ctr[2] = 0;
      __threadfence();
    }
  }
}

// ---------------------------------------------------------------------------
// Staged form, kernel 2: one thread per face writes the face flux
// (Faces.calc_fluxes, src/containers.py:191-278) into [9][Fp].
template <int SCHEME, int VARIANT>
__global__ void __launch_bounds__(256) k_face(DevPlan p, const float* __restrict__ f,
                                              float* __restrict__ flux) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= p.F) return;
  const int s0 = p.fs0[j], s1 = p.fs1[j];
  float lf[Q], rf[Q];
  if (s0 >= 0 && s1 >= 0) {
    load_cell(f, s0, lf);
    load_cell(f, s1, rf);
  } else {
    const int a = p.fna[j], b = p.fnb[j];
    float mq[Q];
#pragma unroll
    for (int q = 0; q < Q; ++q)
      mq[q] = (p.node_pdf[size_t(q) * p.Mp + a] + p.node_pdf[size_t(q) * p.Mp + b]) / 2.0f;
    if (s0 >= 0) {
      load_cell(f, s0, lf);
    } else {
      float kf[Q];
      load_cell(f, p.fkl[j], kf);
      const float rg = p.frl[j];
#pragma unroll
      for (int q = 0; q < Q; ++q) lf[q] = mq[q] + (mq[q] - kf[q]) * rg;
    }
    if (s1 >= 0) {
      load_cell(f, s1, rf);
    } else {
      float kf[Q];
      load_cell(f, p.fkr[j], kf);
      const float rg = p.frr[j];
#pragma unroll
      for (int q = 0; q < Q; ++q) rf[q] = mq[q] + (mq[q] - kf[q]) * rg;
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
  load_cell(fin, i, f);
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
  float* o = fout + cell_base(i, Q);
#pragma unroll
  for (int q = 0; q < Q; ++q) o[q * 32] = f[q] + p.dt * (p.inv_tau * (eq[q] - f[q]) - acc[q]);
}

// Cells.rho/vel/pdf_eq of a pdf buffer (Cells.calc_macros/calc_eqs,
// src/containers.py:93-105).  rho [Np], vel [2][Np] (SoA), feq AoSoA like f.
__global__ void __launch_bounds__(256) k_macros(DevPlan p, const float* __restrict__ f,
                                                float* __restrict__ rho_o, float* __restrict__ vel_o,
                                                float* __restrict__ feq_o) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= p.N) return;
  float fc[Q], eq[Q];
  load_cell(f, i, fc);
  float rho, ux, uy;
  macros(fc, rho, ux, uy);
  feq9(rho, ux, uy, p, eq);
  rho_o[i] = rho;
  vel_o[i] = ux;
  vel_o[size_t(p.Np) + i] = uy;
  float* o = feq_o + cell_base(i, Q);
#pragma unroll
  for (int q = 0; q < Q; ++q) o[q * 32] = eq[q];
}

// rho [N] and vel [N][2] of a pdf buffer, written directly in reference
// order (cell_new: reference -> device).
// rho_o / vel_o may be null, or host memory the device addresses directly
// (each warp then writes whole contiguous spans); vel2: vel_o is 8-byte
// aligned and (ux, uy) go out as one 8-byte store.
__global__ void __launch_bounds__(256) k_macros_ref(DevPlan p, const float* __restrict__ f,
                                                    const int* __restrict__ cell_new, float* __restrict__ rho_o,
                                                    float* __restrict__ vel_o, int vel2) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < p.N; c += gridDim.x * blockDim.x) {
    float fc[Q];
    load_cell(f, cell_new[c], fc);
    float rho, ux, uy;
    macros(fc, rho, ux, uy);
    if (rho_o) rho_o[c] = rho;
    if (vel_o) {
      if (vel2) {
        reinterpret_cast<float2*>(vel_o)[c] = make_float2(ux, uy);
      } else {
        vel_o[2 * size_t(c)] = ux;
        vel_o[2 * size_t(c) + 1] = uy;
      }
    }
  }
}

cudaError_t launch_macros_ref(const DevPlan& p, const float* f, const int* cell_new, float* rho, float* vel,
                              cudaStream_t s, bool grid_cap) {
  if (p.N == 0) return cudaSuccess;
  const int vel2 = (reinterpret_cast<uintptr_t>(vel) & 7) == 0 ? 1 : 0;
  int grid = (p.N + 255) / 256;
  if (grid_cap) {  // a few blocks per SM are enough to keep the host link busy
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    grid = std::min(grid, 2 * sms);
  }
  k_macros_ref<<<grid, 256, 0, s>>>(p, f, cell_new, rho, vel, vel2);
  return cudaGetLastError();
}

// [N][QQ] reference order read straight from page-locked host memory (the
// source must be 16-byte aligned): each block copies its 256 cells'
// contiguous bytes with 16-byte loads into shared memory, so every byte
// crosses the host link once, then scatters them to the AoSoA layout.
template <int QQ>
__global__ void __launch_bounds__(256) k_host_to_cells(const float* __restrict__ src, float* __restrict__ dst,
                                                       const int* __restrict__ cell_new, int N) {
  __shared__ float4 sm[(256 * QQ + 3) / 4];
  float* smf = reinterpret_cast<float*>(sm);
  const int c0 = blockIdx.x * 256;
  const int cells = min(256, N - c0);
  const int nf = cells * QQ, n4 = nf >> 2;
  const float* s = src + size_t(c0) * QQ;  // 16-byte aligned: c0 * QQ * 4 is a multiple of 1024
  for (int k = threadIdx.x; k < n4; k += 256) sm[k] = reinterpret_cast<const float4*>(s)[k];
  for (int k = (n4 << 2) + threadIdx.x; k < nf; k += 256) smf[k] = s[k];
  __syncthreads();
  if (int(threadIdx.x) < cells) {
    float* o = dst + cell_base(cell_new[c0 + threadIdx.x], QQ);
#pragma unroll
    for (int q = 0; q < QQ; ++q) o[q * 32] = smf[threadIdx.x * QQ + q];
  }
}

// [N][9] reference order -> AoSoA device order.
template <int QQ>
__global__ void k_aos_to_cells(const float* __restrict__ src, float* __restrict__ dst,
                               const int* __restrict__ cell_new, int N) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  float* o = dst + cell_base(cell_new[c], QQ);
#pragma unroll
  for (int q = 0; q < QQ; ++q) o[q * 32] = src[size_t(c) * QQ + q];
}

// AoSoA device order -> [N][Q] reference order.
template <int QQ>
__global__ void k_cells_to_aos(const float* __restrict__ src, float* __restrict__ dst,
                               const int* __restrict__ cell_new, int N) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  const float* b = src + cell_base(cell_new[c], QQ);
#pragma unroll
  for (int q = 0; q < QQ; ++q) dst[size_t(c) * QQ + q] = b[q * 32];
}

// Halo exchange of a domain decomposition: rows idx[k] (reference order) of
// the AoSoA pdf to / from a packed [n][QQ] buffer (coalesced on the buffer).
template <int QQ>
__global__ void k_pack_rows(const float* __restrict__ f, const int* __restrict__ cell_new,
                            const int* __restrict__ idx, int n, float* __restrict__ buf) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * QQ) return;
  const int k = int(t / QQ), q = int(t % QQ);
  buf[t] = f[cell_base(cell_new[idx[k]], QQ) + size_t(q) * 32];
}

template <int QQ>
__global__ void k_unpack_rows(float* __restrict__ f, const int* __restrict__ cell_new,
                              const int* __restrict__ idx, int n, const float* __restrict__ buf) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * QQ) return;
  const int k = int(t / QQ), q = int(t % QQ);
  f[cell_base(cell_new[idx[k]], QQ) + size_t(q) * 32] = buf[t];
}

// SoA [rows][Np] device order -> [N][rows] reference order.
__global__ void k_soa_to_aos(const float* __restrict__ src, float* __restrict__ dst,
                             const int* __restrict__ cell_new, int N, int Np, int rows) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= N) return;
  const int d = cell_new[c];
  for (int q = 0; q < rows; ++q) dst[size_t(c) * rows + q] = src[size_t(q) * Np + d];
}

// Self-test of the bounded wait the step kernels use: one thread waits for
// *flag >= 1 at most iters polls; a wait that runs out records
// STATUS_WAIT_TIMEOUT in *status, as the step kernels do.
__global__ void k_wait_selftest(const int* flag, int iters, int* status) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && !wait_at_least(flag, 1, iters, 128))
    atomicExch(status, STATUS_WAIT_TIMEOUT);
}

// Exhaustive check of cdiv (five-operation form, or the two-operation form
// when two is set) against IEEE division: every float32 bit pattern as
// dividend; counts the dividends whose quotients differ in value (NaN matches
// NaN).  Not on the step path; runs once per divisor and form per process.
__global__ void __launch_bounds__(256) k_cdiv_check(float y, float zr, float zl, int two, unsigned long long* bad,
                                                    unsigned* example) {
  const CDiv d{y, zr, zl, 1, two};
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

// Launch with programmatic stream serialization when pdl is set: the kernel
// may start while its predecessor drains; it synchronises with
// griddepcontrol.wait before touching the predecessor's output.
template <typename... KArgs, typename... Args>
static cudaError_t launch_ex(void (*kern)(KArgs...), int grid, int block, size_t smem, cudaStream_t s,
                             bool pdl, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

cudaError_t launch_nodes(const DevPlan& p, const float* f, cudaStream_t s, bool pdl) {
  if (p.NB == 0) return cudaSuccess;
  return launch_ex(k_nodes, p.NB, NODE_BLOCK_ENTRIES, 0, s, pdl, p, f);
}

cudaError_t launch_nodes_cp(const DevPlan& p, const float* f, cudaStream_t s, bool pdl) {
  if (p.NB == 0) return cudaSuccess;
  return launch_ex(k_nodes_cp, p.NB, NODE_BLOCK_ENTRIES, 0, s, pdl, p, f);
}

cudaError_t launch_stencil_macros(const DevPlan& p, const float* f, cudaStream_t s) {
  const int S = p.stencil_end - p.stencil_start;
  if (S <= 0) return cudaSuccess;
  k_stencil_macros<<<blocks(S, 256), 256, 0, s>>>(p, f);
  return cudaGetLastError();
}

static int fused_prefetch_blocks() {
  static int cached = -1;
  if (cached < 0) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cached = sms * 2;  // half a wave of 256-thread blocks (measured best on the 1M step)
  }
  return cached;
}

template <int S, int V>
static cudaError_t fused_dispatch(const DevPlan& p, const float* fin, float* fout, cudaStream_t s,
                                  bool pdl) {
  const int g = blocks(p.N, 256);
  const int pf = fused_prefetch_blocks();
  if (p.fv) return launch_ex(k_fused<S, V, true>, g, 256, 0, s, pdl, p, fin, fout, pf);
  return launch_ex(k_fused<S, V, false>, g, 256, 0, s, pdl, p, fin, fout, pf);
}

template <int S, int V>
static cudaError_t fused_nodes_dispatch(const DevPlan& p, const float* fin, float* fout, cudaStream_t s,
                                        bool pdl) {
  const int ncb = blocks(p.N, 256);
  const int R = p.NB > 0 ? blocks(p.stencil_end, 256) : 0;  // no node blocks: nothing to publish
  // node blocks three quarters into the grid: the recording blocks are long
  // done, and the node work overlaps the remaining cell blocks (measured on
  // the 1M porous step: 35.3 us at 3/4 against 37.5 us one wave after the
  // recording blocks and 37.4 us at the end)
  const int node_at = std::min(ncb, std::max(R, ncb * 3 / 4));
  const int pf = fused_prefetch_blocks();
  const int g = ncb + p.NB;
  if (p.fast) return launch_ex(k_fused_nodes_fast<S>, g, 256, 0, s, pdl, p, fin, fout, R, node_at, pf);
  if (p.fv) return launch_ex(k_fused_nodes<S, V, true>, g, 256, 0, s, pdl, p, fin, fout, R, node_at, pf);
  return launch_ex(k_fused_nodes<S, V, false>, g, 256, 0, s, pdl, p, fin, fout, R, node_at, pf);
}

cudaError_t launch_fused_nodes(const DevPlan& p, const float* fin, float* fout, cudaStream_t s, bool pdl) {
  if (p.N == 0) return cudaSuccess;
  if (p.K != 3 || !p.stencil_first) return cudaErrorInvalidValue;
  if (p.scheme == 0 && p.variant == 0) return fused_nodes_dispatch<0, 0>(p, fin, fout, s, pdl);
  if (p.scheme == 1 && p.variant == 0) return fused_nodes_dispatch<1, 0>(p, fin, fout, s, pdl);
  if (p.scheme == 0 && p.variant == 1) return fused_nodes_dispatch<0, 1>(p, fin, fout, s, pdl);
  if (p.scheme == 1 && p.variant == 1) return fused_nodes_dispatch<1, 1>(p, fin, fout, s, pdl);
  return cudaErrorInvalidValue;
}

template <int S, int V>
static cudaError_t fused_batch_dispatch(const DevPlan& p, const float* fin, float* fout, cudaStream_t s,
                                        bool pdl, int block, int waves) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int g = p.blk_list ? p.n_blk : blocks(p.N, block);
  if (g == 0) return cudaSuccess;
  const int pf = waves * sms * (2048 / block) / 2;  // about `waves` waves at half occupancy
  if (p.fv) return launch_ex(k_fused_batch<S, V, true>, g, block, 0, s, pdl, p, fin, fout, pf);
  return launch_ex(k_fused_batch<S, V, false>, g, block, 0, s, pdl, p, fin, fout, pf);
}

cudaError_t launch_fused_batch(const DevPlan& p, const float* fin, float* fout, cudaStream_t s, bool pdl,
                               int block, int prefetch_waves) {
  if (p.N == 0) return cudaSuccess;
  if (p.K != 3 || (block != 128 && block != 256) || prefetch_waves < 0) return cudaErrorInvalidValue;
  if (p.scheme == 0 && p.variant == 0) return fused_batch_dispatch<0, 0>(p, fin, fout, s, pdl, block, prefetch_waves);
  if (p.scheme == 1 && p.variant == 0) return fused_batch_dispatch<1, 0>(p, fin, fout, s, pdl, block, prefetch_waves);
  if (p.scheme == 0 && p.variant == 1) return fused_batch_dispatch<0, 1>(p, fin, fout, s, pdl, block, prefetch_waves);
  if (p.scheme == 1 && p.variant == 1) return fused_batch_dispatch<1, 1>(p, fin, fout, s, pdl, block, prefetch_waves);
  return cudaErrorInvalidValue;
}

__global__ void k_copy_cells(const float* __restrict__ src, float* __restrict__ dst, int c0, int c1) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = c0 + t / Q, q = t % Q;
  if (c >= c1) return;
  const size_t o = cell_base(c, Q) + size_t(q) * 32;
  dst[o] = src[o];
}

// Cell pdfs = feq(rho, u) (src/dynamics.py:70-74) from reference-order
// rho [N] and vel [N][2].
__global__ void k_cells_eq(DevPlan p, const float* __restrict__ rho, const float* __restrict__ vel,
                           const int* __restrict__ cell_new, float* __restrict__ f) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= p.N) return;
  float eq[Q];
  feq9(rho[c], vel[2 * size_t(c)], vel[2 * size_t(c) + 1], p, eq);
  float* o = f + cell_base(cell_new[c], Q);
#pragma unroll
  for (int q = 0; q < Q; ++q) o[q * 32] = eq[q];
}

cudaError_t launch_cells_eq(const DevPlan& p, const float* rho, const float* vel, const int* cell_new, float* f,
                            cudaStream_t s) {
  if (p.N == 0) return cudaSuccess;
  k_cells_eq<<<blocks(p.N, 256), 256, 0, s>>>(p, rho, vel, cell_new, f);
  return cudaGetLastError();
}

cudaError_t launch_copy_cells(const float* src, float* dst, int c0, int c1, cudaStream_t s) {
  if (c1 <= c0) return cudaSuccess;
  k_copy_cells<<<blocks(int64_t(c1 - c0) * Q, 256), 256, 0, s>>>(src, dst, c0, c1);
  return cudaGetLastError();
}

cudaError_t launch_fused(const DevPlan& p, const float* fin, float* fout, cudaStream_t s, bool pdl) {
  if (p.N == 0) return cudaSuccess;
  if (p.K != 3) return cudaErrorInvalidValue;
  if (p.scheme == 0 && p.variant == 0) return fused_dispatch<0, 0>(p, fin, fout, s, pdl);
  if (p.scheme == 1 && p.variant == 0) return fused_dispatch<1, 0>(p, fin, fout, s, pdl);
  if (p.scheme == 0 && p.variant == 1) return fused_dispatch<0, 1>(p, fin, fout, s, pdl);
  if (p.scheme == 1 && p.variant == 1) return fused_dispatch<1, 1>(p, fin, fout, s, pdl);
  return cudaErrorInvalidValue;
}

template <int S, int V>
static cudaError_t step_dispatch(const DevPlan& p, const float* fin, float* fout, cudaStream_t s,
                                 bool pdl) {
  const int ncb = blocks(p.N, 256);
  const int g = p.NB + ncb;
  const int pf = fused_prefetch_blocks();
  if (p.fv) return launch_ex(k_step<S, V, true>, g, 256, 0, s, pdl, p, fin, fout, ncb, pf);
  return launch_ex(k_step<S, V, false>, g, 256, 0, s, pdl, p, fin, fout, ncb, pf);
}

cudaError_t launch_step(const DevPlan& p, const float* fin, float* fout, cudaStream_t s, bool pdl) {
  if (p.N == 0) return cudaSuccess;
  if (p.K != 3) return cudaErrorInvalidValue;
  if (p.scheme == 0 && p.variant == 0) return step_dispatch<0, 0>(p, fin, fout, s, pdl);
  if (p.scheme == 1 && p.variant == 0) return step_dispatch<1, 0>(p, fin, fout, s, pdl);
  if (p.scheme == 0 && p.variant == 1) return step_dispatch<0, 1>(p, fin, fout, s, pdl);
  if (p.scheme == 1 && p.variant == 1) return step_dispatch<1, 1>(p, fin, fout, s, pdl);
  return cudaErrorInvalidValue;
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

cudaError_t launch_cdiv_check(float y, float zr, float zl, int two, unsigned long long* bad, unsigned* example,
                              cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  k_cdiv_check<<<sms * 8, 256, 0, s>>>(y, zr, zl, two, bad, example);
  return cudaGetLastError();
}

cudaError_t launch_scatter_cells(const float* src_aos, float* dst, const int* cell_new, int N,
                                 cudaStream_t s, int q) {
  if (N == 0) return cudaSuccess;
  if (q == 13)
    k_aos_to_cells<13><<<blocks(N, 256), 256, 0, s>>>(src_aos, dst, cell_new, N);
  else
    k_aos_to_cells<Q><<<blocks(N, 256), 256, 0, s>>>(src_aos, dst, cell_new, N);
  return cudaGetLastError();
}

cudaError_t launch_pack_rows(const float* f, const int* cell_new, const int* idx, int n, float* buf,
                             cudaStream_t s, int q) {
  if (n <= 0) return cudaSuccess;
  const int g = blocks((long long)n * q, 256);
  if (q == 13)
    k_pack_rows<13><<<g, 256, 0, s>>>(f, cell_new, idx, n, buf);
  else
    k_pack_rows<Q><<<g, 256, 0, s>>>(f, cell_new, idx, n, buf);
  return cudaGetLastError();
}

cudaError_t launch_unpack_rows(float* f, const int* cell_new, const int* idx, int n, const float* buf,
                               cudaStream_t s, int q) {
  if (n <= 0) return cudaSuccess;
  const int g = blocks((long long)n * q, 256);
  if (q == 13)
    k_unpack_rows<13><<<g, 256, 0, s>>>(f, cell_new, idx, n, buf);
  else
    k_unpack_rows<Q><<<g, 256, 0, s>>>(f, cell_new, idx, n, buf);
  return cudaGetLastError();
}

cudaError_t launch_wait_selftest(const int* flag, int iters, int* status, cudaStream_t s) {
  k_wait_selftest<<<1, 32, 0, s>>>(flag, iters, status);
  return cudaGetLastError();
}

cudaError_t launch_host_to_cells(const float* src_host, float* dst, const int* cell_new, int N,
                                 cudaStream_t s, int q) {
  if (N == 0) return cudaSuccess;
  if (q == 13)
    k_host_to_cells<13><<<blocks(N, 256), 256, 0, s>>>(src_host, dst, cell_new, N);
  else
    k_host_to_cells<Q><<<blocks(N, 256), 256, 0, s>>>(src_host, dst, cell_new, N);
  return cudaGetLastError();
}

cudaError_t launch_gather_cells(const float* src, float* dst_aos, const int* cell_new, int N,
                                cudaStream_t s, int q) {
  if (N == 0) return cudaSuccess;
  if (q == 13)
    k_cells_to_aos<13><<<blocks(N, 256), 256, 0, s>>>(src, dst_aos, cell_new, N);
  else
    k_cells_to_aos<Q><<<blocks(N, 256), 256, 0, s>>>(src, dst_aos, cell_new, N);
  return cudaGetLastError();
}

cudaError_t launch_soa_to_aos(const float* src, float* dst, const int* cell_new, int N, int Np,
                              int rows, cudaStream_t s) {
  if (N == 0) return cudaSuccess;
  k_soa_to_aos<<<blocks(N, 256), 256, 0, s>>>(src, dst, cell_new, N, Np, rows);
  return cudaGetLastError();
}

}  // namespace fvdbm
