/*
 * fvdbm_mpnn.h - kernels of the learned warm start (libfvdbm.so).
 *
 * No counterpart in the reference, which initialises every case uniformly
 * (every pdf = feq(1, 0), src/containers.py:24-30).  A small message-passing
 * network predicts the steady rho and u of a case from per-cell geometry; the
 * solver then starts from f = feq(rho, u) (fvdbm_set_cells_eq) and still runs
 * to its residual threshold.
 *
 * Conventions: all array pointers are DEVICE pointers; activations are
 * row-major float32 [n][width]; weights are bfloat16 bit patterns (uint16_t)
 * row-major [out][in]; `stream` is a cudaStream_t (NULL = default stream).
 * Calls are asynchronous on that stream.  Return 0, -1 for an invalid
 * argument, -2 for a CUDA error.  Every sum runs in a fixed order, so the
 * results are bitwise reproducible.
 */
#ifndef FVDBM_MPNN_H
#define FVDBM_MPNN_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Dense layer, forward: z = [xa | xb] W^T + bias; y = relu(z) if relu else z,
 * plus residual when given.  da + db <= 128, dout <= 128.  z (pre-activation)
 * is stored when non-NULL; xb/bias/residual may be NULL (db = 0). */
int fvdbm_mp_dense_fwd(const float *xa, int32_t da, const float *xb, int32_t db, int32_t n, const uint16_t *w,
                       const float *bias, int32_t dout, int32_t relu, const float *residual, float *z, float *y,
                       void *stream);

/* Dense layer, backward to the inputs: [dxa | dxb] = dz W.  dxa is
 * accumulated into when acc_a, else overwritten; dxb is overwritten. */
int fvdbm_mp_dense_bwd_data(const float *dz, int32_t n, int32_t dout, const uint16_t *w, int32_t da, int32_t db,
                            float *dxa, int32_t acc_a, float *dxb, void *stream);

/* Dense layer, backward to the parameters: dw = dz^T [xa | xb] (float32
 * [dout][da+db]) and dbias = column sums of dz (may be NULL).  scratch holds
 * per-block partials: at least fvdbm_mp_wgrad_scratch(n, dout, da + db) bytes.
 * dout * (da + db) + dout <= 8256. */
size_t fvdbm_mp_wgrad_scratch(int32_t n, int32_t dout, int32_t din);
int fvdbm_mp_dense_bwd_weight(const float *dz, int32_t n, int32_t dout, const float *xa, int32_t da,
                              const float *xb, int32_t db, float *dw, float *dbias, float *scratch,
                              size_t scratch_bytes, void *stream);

/* dz = dy where z > 0, else 0 (count elements). */
int fvdbm_mp_relu_bwd(const float *dy, const float *z, float *dz, size_t count, void *stream);

/* Neighbour aggregation: out[i][:] (+)= sum_e wt[e] h[col[e]][:] over the CSR
 * row i (row_ptr [n+1]), in entry order. */
int fvdbm_mp_spmm(const int32_t *row_ptr, const int32_t *col, const float *wt, int32_t n, const float *h,
                  int32_t d, float *out, int32_t accumulate, void *stream);

/* The same for long rows (the coarse-bin means): the entries of each row are
 * cut into chunks (chunk_start [nchunks+1] entry offsets, chunks never
 * crossing a row; chunk_ptr [n+1] first chunk of each row); each chunk is
 * folded in entry order into partial [nchunks][d] (caller's scratch), then
 * each row folds its chunks in order. */
int fvdbm_mp_spmm_chunked(const int32_t *chunk_start, const int32_t *chunk_ptr, int32_t nchunks,
                          const int32_t *col, const float *wt, int32_t n, const float *h, int32_t d, float *out,
                          int32_t accumulate, float *partial, void *stream);

/* Masked mean squared error: loss = sum mask (y - t)^2 / mask_total into
 * scratch[0] (double, device); dy = 2 mask (y - t) / mask_total.  mask may be
 * NULL (all ones).  scratch: at least fvdbm_mp_mse_scratch(count) bytes. */
size_t fvdbm_mp_mse_scratch(size_t count);
int fvdbm_mp_mse(const float *y, const float *t, const float *mask, size_t count, float mask_total, float *dy,
                 double *scratch, size_t scratch_bytes, void *stream);

/* Adam step `step` (1-based) on float32 master weights w with moments m, v;
 * wb (may be NULL) receives w rounded to bfloat16 (nearest even). */
int fvdbm_mp_adam(float *w, float *m, float *v, uint16_t *wb, const float *g, size_t count, float lr, float b1,
                  float b2, float eps, int32_t step, void *stream);

/* y = x rounded to bfloat16 (nearest even). */
int fvdbm_mp_to_bf16(const float *x, uint16_t *y, size_t count, void *stream);

/* Features: Jacobi-preconditioned conjugate gradients for A x = b, A
 * symmetric positive definite in CSR (indptr [n+1], indices in [0, n),
 * float32 values; the warm start's potential-flow estimate solves one cell
 * Laplacian per case, many cases as one block-diagonal system).  x holds the
 * initial guess on entry and the solution on return.  Iterates until
 * ||r|| <= rtol ||b|| (tested every check_every iterations, where the call
 * synchronises the stream) or max_iter.  Dot products are summed per thread
 * in float32, then in double over blocks, in a fixed order: bitwise
 * reproducible.  work: device scratch of at least
 * fvdbm_pcg_work_bytes(n) bytes.  *iters and *rel_res report the end state
 * (rel_res NaN: A was not positive definite or the input not finite). */
size_t fvdbm_pcg_work_bytes(int32_t n);
int fvdbm_pcg(int32_t n, const int32_t *indptr, const int32_t *indices, const float *values, const float *b,
              float *x, int32_t max_iter, double rtol, int32_t check_every, void *work, size_t work_bytes,
              void *stream, int32_t *iters, double *rel_res);

/* Features built on the GPU, one case per call (the host path of
 * fvdbm-jax_gb300/warmstart.py computes the same quantities).  Cell and face
 * indices are the case's own; col_off / cell_off / bin_off shift the column
 * indices a case writes, so that several cases form one block-diagonal
 * matrix.  face_kind: 0 interior, 1 wall, 2 open (both end nodes density
 * nodes); face_phib: the potential on open faces. */
/* Distance from each cell centre to the nearest of n_wall wall points. */
int fvdbm_ws_wall_distance(int32_t n, const float *cx, const float *cy, int32_t n_wall, const float *wx,
                           const float *wy, float *out, void *stream);
/* The potential-flow system in rows of four entries (diagonal, then the three
 * face slots; zero entries on the diagonal's column where a slot has no
 * interior neighbour): col [4n], val [4n], rhs [n]. */
int fvdbm_ws_potential_rows(int32_t n, const int32_t *cell_faces, const int32_t *face_cells,
                            const float *face_dists, const float *face_L, const uint8_t *face_kind,
                            const float *face_phib, int32_t col_off, int32_t *col, float *val, float *rhs,
                            void *stream);
/* -grad phi per cell (Green-Gauss over the face values). */
int fvdbm_ws_potential_grad(int32_t n, const int32_t *cell_faces, const float *cell_signs,
                            const int32_t *face_cells, const float *face_dists, const float *face_L,
                            const float *face_n, const uint8_t *face_kind, const float *face_phib,
                            const float *phi, const float *area, float *ngx, float *ngy, void *stream);
/* Mesh-mean stage in rows of three entries: the interior neighbours in
 * ascending order with weight 1/degree, then zero weights on the own cell. */
int fvdbm_ws_mesh_mean(int32_t n, const int32_t *cell_faces, const int32_t *face_cells, int32_t col_off,
                       int32_t *col, float *wt, void *stream);
/* Bin of each cell on a g x g grid over [lo, lo + span] (double), and the
 * bins' populations added into count [g*g]. */
int fvdbm_ws_bin_ids(int32_t n, const double *cell_xy, double lo_x, double lo_y, double span_x, double span_y,
                     int32_t g, int32_t *bin, int32_t *count, void *stream);
/* The bin stage's rows (cells of each bin in ascending order, weight
 * wbin[bin], from start[bin]) and each cell's bin column (ucol). */
int fvdbm_ws_bin_rows(int32_t n, int32_t n_bins, const int32_t *bin, const int32_t *start, const float *wbin,
                      int32_t cell_off, int32_t bin_off, int32_t *pcol, float *pwt, int32_t *ucol, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* FVDBM_MPNN_H */
