// Convergence monitor: FP64 velocity residual and total mass of the current
// pdf buffer.  The reference has no residual; the quantities are
//   res  = ||u^now - u^snap||_2 / (K * dt * max(||u^snap||_2, eps))
//   mass = sum_i rho_i * A_i
// with u, rho the float32 macros of each cell (src/dynamics.py:35-47) and the
// sums taken in double.  Partial sums are formed per fixed chunk of cells and
// combined in a fixed order, so the result is bitwise reproducible run to run
// (no atomics, no dependence on block scheduling).
#include "fvdbm_internal.h"
#include "fvdbm_math.cuh"

namespace fvdbm {

namespace {

constexpr int RT = 256;  // threads per block of both kernels

// Sum of 4 doubles over the block in a fixed tree order; thread 0 gets it.
__device__ __forceinline__ void block_sum4(double v[4]) {
  __shared__ double sh[RT / 32][4];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0)
#pragma unroll
    for (int k = 0; k < 4; ++k) sh[w][k] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      double s = sh[0][k];
      for (int j = 1; j < RT / 32; ++j) s += sh[j][k];
      v[k] = s;
    }
  }
  __syncthreads();
}

// Block b covers cells [b*chunk, (b+1)*chunk) (or [chunk_start[b],
// chunk_start[b+1]) when a table is given) in a fixed per-thread order and
// writes {sum |du|^2, sum |u_snap|^2, sum rho*A, non-finite cells}.  The
// snapshot is replaced by the current velocity.  With chunk_case/case_take,
// a chunk whose case is not taken writes zeros and keeps its snapshot.
__global__ void __launch_bounds__(RT) k_residual_part(DevPlan p, const float* __restrict__ f,
                                                     float* __restrict__ usnap,
                                                     const float* __restrict__ area, int have_snap,
                                                     int chunk, const int* __restrict__ chunk_start,
                                                     const int* __restrict__ chunk_case,
                                                     const int* __restrict__ case_take,
                                                     double* __restrict__ part) {
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  if (chunk_case && !case_take[chunk_case[blockIdx.x]]) {
    if (threadIdx.x < 4) part[size_t(blockIdx.x) * 4 + threadIdx.x] = 0.0;
    return;
  }
  const int c0 = chunk_start ? chunk_start[blockIdx.x] : blockIdx.x * chunk;
  const int c1 = chunk_start ? chunk_start[blockIdx.x + 1] : min(p.N, c0 + chunk);
  const size_t Np = p.Np;
  for (int i = c0 + threadIdx.x; i < c1; i += RT) {
    float fc[Q];
    load_cell(f, i, fc);
    float rho, ux, uy;
    macros(fc, rho, ux, uy);
    if (!(finite(rho) && finite(ux) && finite(uy))) v[3] += 1.0;
    v[2] += double(rho) * (area ? double(area[i]) : 1.0);
    if (have_snap) {
      const double sx = usnap[i], sy = usnap[Np + i];
      const double dx = double(ux) - sx, dy = double(uy) - sy;
      v[0] += dx * dx + dy * dy;
      v[1] += sx * sx + sy * sy;
    }
    usnap[i] = ux;
    usnap[Np + i] = uy;
  }
  block_sum4(v);
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < 4; ++k) part[size_t(blockIdx.x) * 4 + k] = v[k];
}

// Segment s sums the partials of chunks [seg[s], seg[s+1]) in a fixed order.
__global__ void __launch_bounds__(RT) k_residual_final(const double* __restrict__ part,
                                                      const int* __restrict__ seg, int nseg_default,
                                                      double* __restrict__ out) {
  const int s = blockIdx.x;
  const int b0 = seg ? seg[s] : 0, b1 = seg ? seg[s + 1] : nseg_default;
  double v[4] = {0.0, 0.0, 0.0, 0.0};
  for (int b = b0 + threadIdx.x; b < b1; b += RT)
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] += part[size_t(b) * 4 + k];
  block_sum4(v);
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < 4; ++k) out[size_t(s) * 4 + k] = v[k];
}

}  // namespace

int residual_chunks(int N, int chunk) { return N > 0 ? (N + chunk - 1) / chunk : 0; }

cudaError_t launch_residual(const DevPlan& p, const float* f, float* usnap, const float* area,
                            bool have_snap, int chunk, const int* chunk_start, int nchunks,
                            double* part, const int* seg, int nseg, double* out, cudaStream_t s,
                            const int* chunk_case, const int* case_take) {
  const int nb = chunk_start ? nchunks : residual_chunks(p.N, chunk);
  if (nb > 0)
    k_residual_part<<<nb, RT, 0, s>>>(p, f, usnap, area, have_snap ? 1 : 0, chunk, chunk_start, chunk_case,
                                      case_take, part);
  k_residual_final<<<seg ? nseg : 1, RT, 0, s>>>(part, seg, nb, out);
  return cudaGetLastError();
}

}  // namespace fvdbm
