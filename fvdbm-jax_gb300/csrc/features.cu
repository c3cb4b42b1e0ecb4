// Network inputs of the learned warm start built on the GPU, one case per
// call: the same quantities as the host path of fvdbm-jax_gb300/warmstart.py
// (wall distance, the potential-flow system and its gradient, the mesh-mean
// and coarse-bin aggregation stages), so that a prediction costs no host
// sparse-matrix work.  No counterpart in the reference.
//
// Face kinds: 0 interior (both stencil cells), 1 wall (one cell, not open),
// 2 open (one cell, both end nodes density nodes).  Cell and face indices are
// the case's own; col_off shifts the column indices a case writes, so that
// several cases form one block-diagonal matrix.
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>

#include "fvdbm.h"
#include "fvdbm_mpnn.h"

namespace {

constexpr int FT = 256;
constexpr int WALL_TILE = 1024;  // wall points staged in shared memory per pass

int nblk(long long n) { return int((n + FT - 1) / FT); }

// Distance from each cell centre to the nearest wall point (brute force over
// the case's wall-face midpoints, tiled through shared memory).
__global__ void __launch_bounds__(FT) k_wall_distance(int n, const float* __restrict__ cx,
                                                     const float* __restrict__ cy, int nw,
                                                     const float* __restrict__ wx, const float* __restrict__ wy,
                                                     float* __restrict__ out) {
  __shared__ float sx[WALL_TILE], sy[WALL_TILE];
  const int i = blockIdx.x * FT + threadIdx.x;
  const float px = i < n ? cx[i] : 0.0f, py = i < n ? cy[i] : 0.0f;
  float best = FLT_MAX;
  for (int w0 = 0; w0 < nw; w0 += WALL_TILE) {
    const int m = min(WALL_TILE, nw - w0);
    __syncthreads();
    for (int k = threadIdx.x; k < m; k += FT) {
      sx[k] = wx[w0 + k];
      sy[k] = wy[w0 + k];
    }
    __syncthreads();
    for (int k = 0; k < m; ++k) {
      const float dx = px - sx[k], dy = py - sy[k];
      best = fminf(best, dx * dx + dy * dy);
    }
  }
  if (i < n) out[i] = nw > 0 ? sqrtf(best) : 1.0f;
}

// The other cell across face slot k of cell c, or -1 (boundary or self).
__device__ __forceinline__ int other_cell(const int* __restrict__ fcell, int f, int c) {
  const int a = fcell[2 * f], b = fcell[2 * f + 1];
  if (a < 0 || b < 0) return -1;
  const int o = a == c ? b : a;
  return o == c ? -1 : o;
}

// Potential system, four entries per row (row c: diagonal first, then its
// three face slots; a slot without an interior neighbour holds a zero on the
// diagonal's column), and the right-hand side.
__global__ void __launch_bounds__(FT) k_potential_rows(int n, const int* __restrict__ cf,
                                                      const int* __restrict__ fcell, const float* __restrict__ fd,
                                                      const float* __restrict__ fL, const uint8_t* __restrict__ kind,
                                                      const float* __restrict__ phib, int col_off,
                                                      int* __restrict__ col, float* __restrict__ val,
                                                      float* __restrict__ rhs) {
  const int c = blockIdx.x * FT + threadIdx.x;
  if (c >= n) return;
  double diag = 0.0, b = 0.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int f = cf[3 * c + k];
    int oc = -1;
    float w = 0.0f;
    if (f >= 0) {
      if (kind[f] == 0) {
        oc = other_cell(fcell, f, c);
        if (oc >= 0) {
          const double den = fmax(double(fd[2 * f]) + double(fd[2 * f + 1]), 1e-30);
          const double wd = double(fL[f]) / den;
          diag += wd;
          w = float(-wd);
        }
      } else if (kind[f] == 2) {
        const double wb = double(fL[f]) / fmax(double(fd[2 * f]), 1e-30);
        diag += wb;
        b += wb * double(phib[f]);
      }
    }
    col[4 * c + 1 + k] = col_off + (oc >= 0 ? oc : c);
    val[4 * c + 1 + k] = oc >= 0 ? w : 0.0f;
  }
  col[4 * c] = col_off + c;
  val[4 * c] = float(diag);
  rhs[c] = float(b);
}

// Green-Gauss gradient of phi: face values linear between the two cells, the
// boundary value on open faces, the owner's value on walls; then
// sum_k sign_k phi_f n_f L_f / area.  Writes -grad (the flow direction).
__global__ void __launch_bounds__(FT) k_potential_grad(int n, const int* __restrict__ cf,
                                                      const float* __restrict__ cs, const int* __restrict__ fcell,
                                                      const float* __restrict__ fd, const float* __restrict__ fL,
                                                      const float* __restrict__ fn, const uint8_t* __restrict__ kind,
                                                      const float* __restrict__ phib, const float* __restrict__ phi,
                                                      const float* __restrict__ area, float* __restrict__ ngx,
                                                      float* __restrict__ ngy) {
  const int c = blockIdx.x * FT + threadIdx.x;
  if (c >= n) return;
  double gx = 0.0, gy = 0.0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int f = cf[3 * c + k];
    if (f < 0) continue;
    double pf;
    if (kind[f] == 0) {
      const int a = fcell[2 * f], b = fcell[2 * f + 1];
      const double d0 = fd[2 * f], d1 = fd[2 * f + 1];
      pf = (double(phi[a]) * d1 + double(phi[b]) * d0) / fmax(d0 + d1, 1e-30);
    } else if (kind[f] == 2) {
      pf = phib[f];
    } else {
      pf = phi[c];
    }
    const double s = double(cs[3 * c + k]) * pf * double(fL[f]);
    gx += s * double(fn[2 * f]);
    gy += s * double(fn[2 * f + 1]);
  }
  const double A = area[c];
  ngx[c] = float(-gx / A);
  ngy[c] = float(-gy / A);
}

// Mesh mean, three entries per row: the interior neighbours in ascending
// order with weight 1/degree, then zero-weight entries on the row's own cell.
__global__ void __launch_bounds__(FT) k_mesh_mean(int n, const int* __restrict__ cf,
                                                 const int* __restrict__ fcell, int col_off,
                                                 int* __restrict__ col, float* __restrict__ wt) {
  const int c = blockIdx.x * FT + threadIdx.x;
  if (c >= n) return;
  int nb[3];
  int deg = 0;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int f = cf[3 * c + k];
    const int o = f >= 0 ? other_cell(fcell, f, c) : -1;
    if (o >= 0) {
      bool dup = false;
      for (int j = 0; j < deg; ++j) dup |= nb[j] == o;
      if (!dup) nb[deg++] = o;
    }
  }
  // ascending
  for (int a = 1; a < deg; ++a)
    for (int j = a; j > 0 && nb[j - 1] > nb[j]; --j) {
      const int t = nb[j];
      nb[j] = nb[j - 1];
      nb[j - 1] = t;
    }
  const float w = deg > 0 ? float(1.0 / double(deg)) : 0.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    col[3 * c + k] = col_off + (k < deg ? nb[k] : c);
    wt[3 * c + k] = k < deg ? w : 0.0f;
  }
}

// Bin of each cell on a g x g grid over [lo, hi] (double, as the host's
// bin assignment), and the bins' populations.
__global__ void __launch_bounds__(FT) k_bin_ids(int n, const double* __restrict__ cxy, double lox, double loy,
                                               double spx, double spy, int g, int* __restrict__ bin,
                                               int* __restrict__ count) {
  const int c = blockIdx.x * FT + threadIdx.x;
  if (c >= n) return;
  const long long i = (long long)(((cxy[2 * c] - lox) / spx) * g);
  const long long j = (long long)(((cxy[2 * c + 1] - loy) / spy) * g);
  const int bi = int(i < 0 ? 0 : (i > g - 1 ? g - 1 : i)), bj = int(j < 0 ? 0 : (j > g - 1 ? g - 1 : j));
  const int b = bi * g + bj;
  bin[c] = b;
  atomicAdd(count + b, 1);
}

// Rows of the bin stage P (one thread per bin, cells in ascending order):
// col = cell, weight wbin[bin].  start: each bin's first entry.  The stage U
// (cell -> its bin, weight 1) is written by the same pass.
__global__ void __launch_bounds__(FT) k_bin_rows(int n, int nbins, const int* __restrict__ bin,
                                                const int* __restrict__ start, const float* __restrict__ wbin,
                                                int cell_off, int bin_off, int* __restrict__ pcol,
                                                float* __restrict__ pwt, int* __restrict__ ucol) {
  const int b = blockIdx.x * FT + threadIdx.x;
  if (b < nbins) {
    const float w = wbin[b];
    int pos = start[b];
    for (int c = 0; c < n; ++c)
      if (bin[c] == b) {
        pcol[pos] = cell_off + c;
        pwt[pos] = w;
        ++pos;
      }
  }
  for (int c = blockIdx.x * FT + threadIdx.x; c < n; c += gridDim.x * FT) ucol[c] = bin_off + bin[c];
}

}  // namespace

extern "C" int fvdbm_ws_wall_distance(int32_t n, const float* cx, const float* cy, int32_t n_wall, const float* wx,
                                      const float* wy, float* out, void* stream) {
  if (n < 0 || n_wall < 0 || (n > 0 && (!cx || !cy || !out)) || (n_wall > 0 && (!wx || !wy))) return FVDBM_EINVAL;
  if (n == 0) return FVDBM_OK;
  k_wall_distance<<<nblk(n), FT, 0, static_cast<cudaStream_t>(stream)>>>(n, cx, cy, n_wall, wx, wy, out);
  return cudaGetLastError() == cudaSuccess ? FVDBM_OK : FVDBM_ECUDA;
}

extern "C" int fvdbm_ws_potential_rows(int32_t n, const int32_t* cell_faces, const int32_t* face_cells,
                                       const float* face_dists, const float* face_L, const uint8_t* face_kind,
                                       const float* face_phib, int32_t col_off, int32_t* col, float* val,
                                       float* rhs, void* stream) {
  if (n < 0 || col_off < 0) return FVDBM_EINVAL;
  if (n == 0) return FVDBM_OK;
  k_potential_rows<<<nblk(n), FT, 0, static_cast<cudaStream_t>(stream)>>>(n, cell_faces, face_cells, face_dists,
                                                                          face_L, face_kind, face_phib, col_off, col,
                                                                          val, rhs);
  return cudaGetLastError() == cudaSuccess ? FVDBM_OK : FVDBM_ECUDA;
}

extern "C" int fvdbm_ws_potential_grad(int32_t n, const int32_t* cell_faces, const float* cell_signs,
                                       const int32_t* face_cells, const float* face_dists, const float* face_L,
                                       const float* face_n, const uint8_t* face_kind, const float* face_phib,
                                       const float* phi, const float* area, float* ngx, float* ngy, void* stream) {
  if (n < 0) return FVDBM_EINVAL;
  if (n == 0) return FVDBM_OK;
  k_potential_grad<<<nblk(n), FT, 0, static_cast<cudaStream_t>(stream)>>>(
      n, cell_faces, cell_signs, face_cells, face_dists, face_L, face_n, face_kind, face_phib, phi, area, ngx, ngy);
  return cudaGetLastError() == cudaSuccess ? FVDBM_OK : FVDBM_ECUDA;
}

extern "C" int fvdbm_ws_mesh_mean(int32_t n, const int32_t* cell_faces, const int32_t* face_cells, int32_t col_off,
                                  int32_t* col, float* wt, void* stream) {
  if (n < 0 || col_off < 0) return FVDBM_EINVAL;
  if (n == 0) return FVDBM_OK;
  k_mesh_mean<<<nblk(n), FT, 0, static_cast<cudaStream_t>(stream)>>>(n, cell_faces, face_cells, col_off, col, wt);
  return cudaGetLastError() == cudaSuccess ? FVDBM_OK : FVDBM_ECUDA;
}

extern "C" int fvdbm_ws_bin_ids(int32_t n, const double* cell_xy, double lo_x, double lo_y, double span_x,
                                double span_y, int32_t g, int32_t* bin, int32_t* count, void* stream) {
  if (n < 0 || g <= 0 || !(span_x > 0.0) || !(span_y > 0.0)) return FVDBM_EINVAL;
  if (n == 0) return FVDBM_OK;
  k_bin_ids<<<nblk(n), FT, 0, static_cast<cudaStream_t>(stream)>>>(n, cell_xy, lo_x, lo_y, span_x, span_y, g, bin,
                                                                   count);
  return cudaGetLastError() == cudaSuccess ? FVDBM_OK : FVDBM_ECUDA;
}

extern "C" int fvdbm_ws_bin_rows(int32_t n, int32_t n_bins, const int32_t* bin, const int32_t* start,
                                 const float* wbin, int32_t cell_off, int32_t bin_off, int32_t* pcol, float* pwt,
                                 int32_t* ucol, void* stream) {
  if (n < 0 || n_bins <= 0 || cell_off < 0 || bin_off < 0) return FVDBM_EINVAL;
  if (n == 0) return FVDBM_OK;
  k_bin_rows<<<nblk(n_bins), FT, 0, static_cast<cudaStream_t>(stream)>>>(n, n_bins, bin, start, wbin, cell_off,
                                                                         bin_off, pcol, pwt, ucol);
  return cudaGetLastError() == cudaSuccess ? FVDBM_OK : FVDBM_ECUDA;
}
