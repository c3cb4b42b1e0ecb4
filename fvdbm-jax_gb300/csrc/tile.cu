// Persistent tile kernel: one launch per FVDBM step (sm_103a).
//
// The cells are cut into tiles of TILE consecutive cells (device order, which
// is Morton order when centroids are known).  Each CTA walks its tiles; for
// each tile one thread issues two bulk async copies (cp.async.bulk,
// completion counted on an mbarrier): the tile's pdfs and its per-face-slot
// words (neighbour code, normal, signed length, and the Lax-Wendroff /
// stencil scale rows when used), both contiguous in the AoSoA layout, into
// shared memory, double-buffered so that the next tile streams in while this
// one computes.  Then:
//   phase A  the boundary nodes that the tile's ghost faces need
//            (Nodes.calc_pdfs, src/containers.py:339-404): one thread per
//            node-stencil entry evaluates that cell's macros, equilibrium and
//            IDW products into shared memory; one thread per node folds them
//            in the reference's entry order.  The tile that owns a node also
//            writes its state to global memory for read-back;
//   phase B  one thread per cell: macros, equilibrium, the three face fluxes
//            (neighbour pdfs from shared memory when inside the tile) and the
//            update (src/containers.py:107-121, :191-291).
// Arithmetic is that of fvdbm_math.cuh, so the result is bitwise equal to the
// CPU oracle and to the two-kernel path.
//
// Every mbarrier wait is bounded; a wait that gives up sets p.status, waits
// (bounded) for the CTA's copies still in flight and returns.
#include "fvdbm_math.cuh"

namespace fvdbm {

namespace {

__device__ __forceinline__ uint32_t smem_u32(const void* ptr) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(ptr));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity), "r"(1000u)
      : "memory");
  return done != 0;
}

// Bounded wait: ~1000 ns suspend hint per try, 2^21 tries.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int i = 0; i < (1 << 21); ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

template <int SCHEME, int VARIANT>
struct TileRows {
  static constexpr int K = 3;
  static constexpr int HROWS = (4 + (SCHEME == 1 ? 2 : 0) + (VARIANT == 1 ? 1 : 0)) * K;
  static constexpr int FWORDS = TILE * Q;      // the tile's pdfs, AoSoA
  static constexpr int HWORDS = TILE * HROWS;  // the tile's face slots, AoSoA
  static constexpr int WORDS = FWORDS + HWORDS;
};

// A tile is TILE/32 consecutive AoSoA blocks, so its pdfs and its face slots
// are two contiguous ranges: one bulk copy each (lane 0 of warp 0).
template <int SCHEME, int VARIANT>
__device__ __forceinline__ void issue_tile(const DevPlan& p, const float* fin, int tile, float* stage,
                                           uint32_t bar, int lane) {
  using RW = TileRows<SCHEME, VARIANT>;
  if (lane != 0) return;
  mbar_expect_tx(bar, RW::WORDS * 4);
  bulk_g2s(smem_u32(stage), fin + size_t(tile) * RW::FWORDS, RW::FWORDS * 4, bar);
  bulk_g2s(smem_u32(stage + RW::FWORDS), p.hf + size_t(tile) * RW::HWORDS, RW::HWORDS * 4, bar);
}

}  // namespace

template <int SCHEME, int VARIANT>
constexpr size_t tile_smem_bytes() {
  return (size_t(2) * TileRows<SCHEME, VARIANT>::WORDS + size_t(Q) * TILE_MAX_NODES +
          size_t(12) * TILE_MAX_ENTRIES) * sizeof(float) + 2 * sizeof(uint64_t);
}

template <int SCHEME, int VARIANT, bool FV, bool NODES>
__global__ void __launch_bounds__(TILE, 2) k_tile(DevPlan p, const float* __restrict__ fin,
                                                  float* __restrict__ fout) {
  using RW = TileRows<SCHEME, VARIANT>;
  constexpr int K = RW::K;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  float* stage0 = reinterpret_cast<float*>(smem_raw);
  float* npdf = stage0 + 2 * RW::WORDS;            // [9][TILE_MAX_NODES]
  float* prod = npdf + Q * TILE_MAX_NODES;          // [12][TILE_MAX_ENTRIES]
  uint64_t* bars = reinterpret_cast<uint64_t*>(prod + 12 * TILE_MAX_ENTRIES);
  const int tid = threadIdx.x;
  const int first = blockIdx.x, stride = gridDim.x;
  if (first >= p.NT) return;
  const uint32_t bar0 = smem_u32(&bars[0]), bar1 = smem_u32(&bars[1]);

  if (tid == 0) {
    mbar_init(bar0, 1);
    mbar_init(bar1, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (tid < 32) {
    issue_tile<SCHEME, VARIANT>(p, fin, first, stage0, bar0, tid);
    if (first + stride < p.NT)
      issue_tile<SCHEME, VARIANT>(p, fin, first + stride, stage0 + RW::WORDS, bar1, tid);
  }

  int it = 0;
  for (int t = first; t < p.NT; t += stride, ++it) {
    const int s = it & 1;
    const uint32_t bar = s ? bar1 : bar0;
    const uint32_t parity = (it >> 1) & 1;
    const bool timed_out = !mbar_wait(bar, parity);
    if (__syncthreads_or(timed_out)) {
      // give up: report, let the copies still in flight land, return
      if (tid == 0) {
        atomicExch(p.status, STATUS_WAIT_TIMEOUT);
        mbar_wait(bar, parity);                                 // this tile's copies
        if (it == 0 && first + stride < p.NT) mbar_wait(bar1, 0);  // the pre-issued second tile
      }
      __syncthreads();
      return;
    }
    // every thread has finished the previous tile: refill its stage with
    // the tile two iterations ahead of that one
    if (it > 0 && tid < 32) {
      const int tn = t + stride;
      if (tn < p.NT) {
        if (tid == 0) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncwarp();
        issue_tile<SCHEME, VARIANT>(p, fin, tn, stage0 + (s ^ 1) * RW::WORDS, s ? bar0 : bar1, tid);
      }
    }
    const float* SF = stage0 + s * RW::WORDS;  // pdfs, AoSoA
    const unsigned* SH = reinterpret_cast<const unsigned*>(SF + RW::FWORDS);  // face slots, AoSoA
    const int tile_start = t * TILE;

    // ---- phase A: boundary nodes needed by this tile
    const int nb = NODES ? __ldg(p.tn_ptr + t) : 0;
    const int nn = NODES ? __ldg(p.tn_ptr + t + 1) - nb : 0;
    if (NODES && nn > 0) {
      const int eb = __ldg(p.te_ptr + t), ne = __ldg(p.te_ptr + t + 1) - eb;
      if (tid < ne) {
        const unsigned code = __ldg(p.te_cell + eb + tid);
        const int c = int(code & ~ND_NEQ_ZERO);
        const float w = __ldg(p.te_w + eb + tid);
        float fc[Q], eq[Q];
        const unsigned lc = unsigned(c - tile_start);
        if (lc < unsigned(TILE)) {
          const float* b = SF + cell_base(int(lc), Q);
#pragma unroll
          for (int q = 0; q < Q; ++q) fc[q] = b[q * 32];
        } else {
          load_cell(fin, c, fc);
        }
        float rho, ux, uy;
        macros(fc, rho, ux, uy);
        feq9(rho, ux, uy, p, eq);
        const bool zero = (code & ND_NEQ_ZERO) != 0;
        prod[0 * TILE_MAX_ENTRIES + tid] = rho * w;
        prod[1 * TILE_MAX_ENTRIES + tid] = ux * w;
        prod[2 * TILE_MAX_ENTRIES + tid] = uy * w;
#pragma unroll
        for (int q = 0; q < Q; ++q)
          prod[(3 + q) * TILE_MAX_ENTRIES + tid] = (zero ? 0.0f : fc[q] - eq[q]) * w;
      }
      __syncthreads();
      if (tid < nn) {
        const int kind = __ldg(p.tn_kind + nb + tid);
        const int d = __ldg(p.tn_dev + nb + tid);
        const int type = kind & 3;
        float g[Q];
        if (type == 0) {
#pragma unroll
          for (int q = 0; q < Q; ++q) g[q] = p.node_pdf[size_t(q) * p.Mp + d];
        } else {
          const int e0 = __ldg(p.tn_e0 + nb + tid), cnt = __ldg(p.tn_ecnt + nb + tid);
          float ar = 0.0f, ax = 0.0f, ay = 0.0f, an[Q];
#pragma unroll
          for (int q = 0; q < Q; ++q) an[q] = 0.0f;
          for (int j = 0; j < cnt; ++j) {
            const int e = e0 + j;
            const float vr = prod[0 * TILE_MAX_ENTRIES + e];
            const float vx = prod[1 * TILE_MAX_ENTRIES + e];
            const float vy = prod[2 * TILE_MAX_ENTRIES + e];
            ar = j ? ar + vr : vr;
            ax = j ? ax + vx : vx;
            ay = j ? ay + vy : vy;
#pragma unroll
            for (int q = 0; q < Q; ++q) {
              const float vn = prod[(3 + q) * TILE_MAX_ENTRIES + e];
              an[q] = j ? an[q] + vn : vn;
            }
          }
          if (__ldg(p.tn_npad + nb + tid) > 0) {
            // padded (-1, weight 0) entries gather the last cell: rho*0, u*0
            float fc[Q];
            load_cell(fin, p.last_cell, fc);
            float rho, ux, uy;
            macros(fc, rho, ux, uy);
            ar = cnt ? ar + rho * 0.0f : rho * 0.0f;
            ax = cnt ? ax + ux * 0.0f : ux * 0.0f;
            ay = cnt ? ay + uy * 0.0f : uy * 0.0f;
          }
          const float sw = __ldg(p.tn_sumw + nb + tid);
          float rho_p, ux_p, uy_p;
          if (type == 1) {
            rho_p = ar / sw;
            ux_p = p.node_vel[d];
            uy_p = p.node_vel[p.Mp + d];
          } else {
            rho_p = p.node_rho[d];
            ux_p = ax / sw;
            uy_p = ay / sw;
          }
          float eqn[Q];
          feq9(rho_p, ux_p, uy_p, p, eqn);
#pragma unroll
          for (int q = 0; q < Q; ++q) g[q] = eqn[q] + an[q] / sw;
          if (kind & TN_OWNER) {
#pragma unroll
            for (int q = 0; q < Q; ++q) p.node_pdf[size_t(q) * p.Mp + d] = g[q];
            if (type == 1) {
              p.node_rho[d] = rho_p;
            } else {
              p.node_vel[d] = ux_p;
              p.node_vel[p.Mp + d] = uy_p;
            }
          }
        }
#pragma unroll
        for (int q = 0; q < Q; ++q) npdf[q * TILE_MAX_NODES + tid] = g[q];
      }
      __syncthreads();
    }

    // ---- phase B: the tile's cells
    const int i = tile_start + tid;
    if (i < p.N) {
      float f[Q];
      {
        const float* b = SF + cell_base(tid, Q);
#pragma unroll
        for (int q = 0; q < Q; ++q) f[q] = b[q * 32];
      }
      const unsigned* hb = SH + cell_base(tid, RW::HROWS);
      const HfRows HR{K, SCHEME, VARIANT};
      float rho, ux, uy, eq[Q];
      macros(f, rho, ux, uy);
      feq9(rho, ux, uy, p, eq);
      float acc[Q];
#pragma unroll
      for (int k = 0; k < K; ++k) {
        const int code = int(hb[HR.code(k) * 32]);
        const float nx = __uint_as_float(hb[HR.nx(k) * 32]);
        const float ny = __uint_as_float(hb[HR.ny(k) * 32]);
        const float Ls = __uint_as_float(hb[HR.ls(k) * 32]);
        const int other = code >> HF_SHIFT;
        const bool slot1 = (code & HF_SLOT1) != 0;
        float o[Q];
        if (code & HF_GHOST) {
          const float rg = __ldg(p.gh_r + other);
          if (NODES) {
            const int la = __ldg(p.tgh_a + other), lb = __ldg(p.tgh_b + other);
#pragma unroll
            for (int q = 0; q < Q; ++q) {
              const float mq = (npdf[q * TILE_MAX_NODES + la] + npdf[q * TILE_MAX_NODES + lb]) / 2.0f;
              o[q] = mq + (mq - f[q]) * rg;
            }
          } else {
            const int a = __ldg(p.gh_a + other), b = __ldg(p.gh_b + other);
#pragma unroll
            for (int q = 0; q < Q; ++q) {
              const float mq = (__ldg(p.node_pdf + size_t(q) * p.Mp + a) +
                                __ldg(p.node_pdf + size_t(q) * p.Mp + b)) / 2.0f;
              o[q] = mq + (mq - f[q]) * rg;
            }
          }
        } else {
          const unsigned lo = unsigned(other - tile_start);
          if (lo < unsigned(TILE)) {
            const float* b = SF + cell_base(int(lo), Q);
#pragma unroll
            for (int q = 0; q < Q; ++q) o[q] = b[q * 32];
          } else {
            load_cell(fin, other, o);
          }
        }
        float v[Q], w[Q];
        xi_dot_n(nx, ny, p.finite_n != 0, v);
        if (SCHEME == 1)
          lw_interp(v, __uint_as_float(hb[HR.r(k) * 32]), __uint_as_float(hb[HR.d2(k) * 32]), p.dt,
                    p.finite_n != 0, w);
        const float scale = (VARIANT == 1) ? __uint_as_float(hb[HR.sc(k) * 32]) : 1.0f;
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          float phi;
          if (SCHEME == 0) {
            phi = ((v[q] >= 0.0f) != slot1) ? f[q] : o[q];
          } else {
            const float lq = slot1 ? o[q] : f[q], rq = slot1 ? f[q] : o[q];
            phi = lq + (rq - lq) * w[q];
          }
          float x = (phi * v[q]) * Ls;
          if (VARIANT == 1) x = x * scale;
          acc[q] = (k == 0) ? x : acc[q] + x;
        }
      }
      if (FV) {
        const float ia = __ldg(p.inv_area + i);
#pragma unroll
        for (int q = 0; q < Q; ++q) acc[q] = acc[q] * ia;
      }
      float* ob = fout + cell_base(i, Q);
#pragma unroll
      for (int q = 0; q < Q; ++q) ob[q * 32] = f[q] + p.dt * (p.inv_tau * (eq[q] - f[q]) - acc[q]);
    }

  }
}

namespace {

// Grid = SMs x resident CTAs per SM, per instantiation and device.
template <int S, int V, bool FV, bool NODES>
struct TileLaunch {
  static int grid[64];

  static cudaError_t prepare() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    if (grid[dev] > 0) return cudaSuccess;
    constexpr size_t smem = tile_smem_bytes<S, V>();
    e = cudaFuncSetAttribute(k_tile<S, V, FV, NODES>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    // the whole unified L1/shared array as shared memory: several CTAs per SM
    e = cudaFuncSetAttribute(k_tile<S, V, FV, NODES>, cudaFuncAttributePreferredSharedMemoryCarveout,
                             int(cudaSharedmemCarveoutMaxShared));
    if (e != cudaSuccess) return e;
    int sms = 0, per_sm = 0;
    e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tile<S, V, FV, NODES>, TILE, smem);
    if (e != cudaSuccess) return e;
    grid[dev] = sms * (per_sm > 0 ? per_sm : 1);
    per_sm_[dev] = per_sm;
    return cudaSuccess;
  }
  static int per_sm_[64];

  static cudaError_t launch(const DevPlan& p, const float* fin, float* fout, cudaStream_t st) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64 || grid[dev] <= 0) return cudaErrorNotReady;
    const int g = grid[dev] < p.NT ? grid[dev] : p.NT;
    k_tile<S, V, FV, NODES><<<g, TILE, tile_smem_bytes<S, V>(), st>>>(p, fin, fout);
    return cudaGetLastError();
  }
};

template <int S, int V, bool FV, bool NODES>
int TileLaunch<S, V, FV, NODES>::grid[64] = {0};
template <int S, int V, bool FV, bool NODES>
int TileLaunch<S, V, FV, NODES>::per_sm_[64] = {0};

template <bool NODES, class Fn>
cudaError_t dispatch_n(const DevPlan& p, Fn&& fn) {
  if (p.scheme == 0 && p.variant == 0)
    return p.fv ? fn(TileLaunch<0, 0, true, NODES>{}) : fn(TileLaunch<0, 0, false, NODES>{});
  if (p.scheme == 1 && p.variant == 0)
    return p.fv ? fn(TileLaunch<1, 0, true, NODES>{}) : fn(TileLaunch<1, 0, false, NODES>{});
  if (p.scheme == 0 && p.variant == 1)
    return p.fv ? fn(TileLaunch<0, 1, true, NODES>{}) : fn(TileLaunch<0, 1, false, NODES>{});
  if (p.scheme == 1 && p.variant == 1)
    return p.fv ? fn(TileLaunch<1, 1, true, NODES>{}) : fn(TileLaunch<1, 1, false, NODES>{});
  return cudaErrorInvalidValue;
}

template <class Fn>
cudaError_t dispatch(const DevPlan& p, Fn&& fn) {
  return p.tile_nodes ? dispatch_n<true>(p, fn) : dispatch_n<false>(p, fn);
}

}  // namespace

cudaError_t prepare_tile(const DevPlan& p) {
  if (p.K != 3) return cudaErrorInvalidValue;
  return dispatch(p, [](auto L) { return decltype(L)::prepare(); });
}

int tile_ctas_per_sm(const DevPlan& p) {
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 0;
  int out = 0;
  dispatch(p, [&](auto L) {
    out = decltype(L)::per_sm_[dev];
    return cudaSuccess;
  });
  return out;
}

cudaError_t launch_tile(const DevPlan& p, const float* fin, float* fout, cudaStream_t st) {
  if (p.N == 0 || p.NT == 0) return cudaSuccess;
  if (p.K != 3) return cudaErrorInvalidValue;
  return dispatch(p, [&](auto L) { return decltype(L)::launch(p, fin, fout, st); });
}

}  // namespace fvdbm
