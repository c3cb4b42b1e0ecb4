/*
 * ORACLE (test infrastructure only).  A C restatement of the reference's
 * FVDBM time step (MADALERAU/FVDBM-JAX), used as the checker for the CUDA
 * path at sizes the numpy oracle is too slow for, and timed as the CPU
 * baseline.  Only tests/, __graft_entry__.smoke() and bench.py's CPU legs may
 * load it; the product never does.
 *
 * It follows oracle/oracle_np.py statement for statement (which the golden
 * vectors pin to the reference bit for bit): float32 arithmetic in the
 * reference's order, sums as left folds, the 0*x terms of the integer-lattice
 * dot products kept, -1 gather indices wrapping to the last row.  Build with
 * -ffp-contract=off so no multiply-add is fused.
 *
 * Layout is the reference's: cell_pdf [N][9], node_pdf [P][9], node_rho [P],
 * node_vel [P][2], face arrays [F][2] / [F].
 *
 * Compiled with -DORACLE_F64 the same statements run in float64 (state,
 * lattice constants, 1/tau and dt in double; the float32 geometry of the
 * containers promoted exactly), exported as oracle_step_f64: the reference
 * the float32 rounding error of a step sequence is measured against.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define Q 9

#ifdef ORACLE_F64
typedef double real;
#define ORACLE_FN(name) name##_f64
#else
typedef float real;
#define ORACLE_FN(name) name
#endif

typedef struct {
  int32_t N, F, P, K, Kn;
  const int32_t *face_indices; /* [N][K]  Cells.face_indices */
  const int32_t *face_signs;   /* [N][K]  Cells.face_normals */
  const int32_t *face_cells;   /* [F][2]  Faces.stencil_cells_index */
  const float *face_dists;     /* [F][2]  Faces.stencil_dists */
  const int32_t *face_nodes;   /* [F][2]  Faces.nodes_index */
  const float *face_n;         /* [F][2]  Faces.n */
  const float *face_L;         /* [F]     Faces.L */
  const float *face_scale;     /* [F] (variant 1) or [F][9] (variant 2) */
  const int32_t *node_type;    /* [P]     Nodes.type */
  const int32_t *node_cells;   /* [P][Kn] Nodes.cells_index */
  const float *node_dists;     /* [P][Kn] Nodes.cell_dists */
  const float *inv_area;       /* [N] or NULL */
  int32_t scheme, variant;
  real inv_tau, dt, c2, c4x2, c2x2;
} oracle_mesh_t;

static const real W[Q] = {(real)(4.0 / 9.0),  (real)(1.0 / 9.0),  (real)(1.0 / 9.0),
                          (real)(1.0 / 9.0),  (real)(1.0 / 9.0),  (real)(1.0 / 36.0),
                          (real)(1.0 / 36.0), (real)(1.0 / 36.0), (real)(1.0 / 36.0)};
static const real KX[Q] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const real KY[Q] = {0, 0, 1, 0, -1, 1, 1, -1, -1};

static inline int32_t wrap(int32_t i, int32_t n) { return i < 0 ? i + n : i; }

/* src/dynamics.py:35-47 */
static inline void macros(const real *f, real *rho, real *ux, real *uy) {
  real r = f[0], mx = KX[0] * f[0], my = KY[0] * f[0];
  for (int q = 1; q < Q; ++q) {
    r = r + f[q];
    mx = mx + KX[q] * f[q];
    my = my + KY[q] * f[q];
  }
  *rho = r;
  *ux = mx / r;
  *uy = my / r;
}

/* src/dynamics.py:70-74 */
static inline void feq9(const oracle_mesh_t *m, real rho, real ux, real uy, real *out) {
  const real uu = ux * ux + uy * uy;
  for (int q = 0; q < Q; ++q) {
    const real a = KX[q] * ux + KY[q] * uy;
    real s = (real)1 + a / m->c2;
    s = s + (a * a) / m->c4x2;
    s = s - uu / m->c2x2;
    out[q] = (W[q] * rho) * s;
  }
}

/* One Environment.step (src/environment.py:55-65).  Scratch: rho [N],
 * vel [N][2], feq [N][9], flux [F][9], fnew [N][9]. */
static void step_once(const oracle_mesh_t *m, real *pdf, real *npdf, real *nrho, real *nvel,
                      real *rho, real *vel, real *feq, real *flux, real *fnew, int nt) {
  const int N = m->N, F = m->F, P = m->P, K = m->K, Kn = m->Kn;
  (void)nt;
  /* cells: macros and equilibria (src/containers.py:93-105) */
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int i = 0; i < N; ++i) {
    macros(pdf + (size_t)i * Q, rho + i, vel + 2 * (size_t)i, vel + 2 * (size_t)i + 1);
    feq9(m, rho[i], vel[2 * i], vel[2 * i + 1], feq + (size_t)i * Q);
  }
  /* nodes (src/containers.py:339-404, utils/utils.py:34-60) */
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int p = 0; p < P; ++p) {
    const int t = m->node_type[p];
    if (t != 1 && t != 2) continue;
    real sw = 0, ar = 0, ax = 0, ay = 0, an[Q] = {0};
    for (int k = 0; k < Kn; ++k) {
      const int32_t c = m->node_cells[(size_t)p * Kn + k];
      real w = (real)1 / (real)m->node_dists[(size_t)p * Kn + k];
      if (w < (real)0) w = (real)0;
      const int32_t cw = wrap(c, N);
      real x_r = rho[cw] * w, x_x = vel[2 * (size_t)cw] * w, x_y = vel[2 * (size_t)cw + 1] * w;
      real x_n[Q];
      for (int q = 0; q < Q; ++q) {
        const real neq = (c == -1) ? (real)0 : pdf[(size_t)cw * Q + q] - feq[(size_t)cw * Q + q];
        x_n[q] = neq * w;
      }
      if (k == 0) {
        sw = w;
        ar = x_r;
        ax = x_x;
        ay = x_y;
        for (int q = 0; q < Q; ++q) an[q] = x_n[q];
      } else {
        sw = sw + w;
        ar = ar + x_r;
        ax = ax + x_x;
        ay = ay + x_y;
        for (int q = 0; q < Q; ++q) an[q] = an[q] + x_n[q];
      }
    }
    real rp, uxp, uyp;
    if (t == 1) {
      rp = ar / sw;
      nrho[p] = rp;
      uxp = nvel[2 * (size_t)p];
      uyp = nvel[2 * (size_t)p + 1];
    } else {
      rp = nrho[p];
      uxp = ax / sw;
      uyp = ay / sw;
      nvel[2 * (size_t)p] = uxp;
      nvel[2 * (size_t)p + 1] = uyp;
    }
    real eq[Q];
    feq9(m, rp, uxp, uyp, eq);
    for (int q = 0; q < Q; ++q) npdf[(size_t)p * Q + q] = eq[q] + an[q] / sw;
  }
  /* faces (src/containers.py:191-287, src/faces.py:54-74,119-141) */
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int j = 0; j < F; ++j) {
    const int32_t s0 = m->face_cells[2 * j], s1 = m->face_cells[2 * j + 1];
    const real d0 = m->face_dists[2 * j], d1 = m->face_dists[2 * j + 1];
    const real nx = m->face_n[2 * j], ny = m->face_n[2 * j + 1], L = m->face_L[j];
    real lf[Q], rf[Q];
    if (s0 == -1 || s1 == -1) {
      const real *ga = npdf + (size_t)wrap(m->face_nodes[2 * j], P) * Q;
      const real *gb = npdf + (size_t)wrap(m->face_nodes[2 * j + 1], P) * Q;
      for (int q = 0; q < Q; ++q) {
        const real mq = (ga[q] + gb[q]) / (real)2;
        if (s0 == -1) lf[q] = mq + (mq - pdf[(size_t)wrap(s1, N) * Q + q]) * (d0 / d1);
        if (s1 == -1) rf[q] = mq + (mq - pdf[(size_t)wrap(s0, N) * Q + q]) * (d1 / d0);
      }
    }
    for (int q = 0; q < Q; ++q) {
      if (s0 != -1) lf[q] = pdf[(size_t)s0 * Q + q];
      if (s1 != -1) rf[q] = pdf[(size_t)s1 * Q + q];
    }
    for (int q = 0; q < Q; ++q) {
      const real v = KX[q] * nx + KY[q] * ny;
      real phi;
      if (m->scheme == 0) {
        phi = v >= (real)0 ? lf[q] : rf[q];
      } else {
        const real D = d0 + d1;
        const real interp = (d0 / D) - (v * m->dt) / ((real)2 * D);
        phi = lf[q] + (rf[q] - lf[q]) * interp;
      }
      real fl = (phi * v) * L;
      if (m->variant == 1) fl = fl * (real)m->face_scale[j];
      if (m->variant == 2) fl = fl * (real)m->face_scale[(size_t)j * Q + q];
      flux[(size_t)j * Q + q] = fl;
    }
  }
  /* cells: signed flux sum and update (src/containers.py:107-121) */
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int i = 0; i < N; ++i) {
    real acc[Q] = {0};
    for (int k = 0; k < K; ++k) {
      const int32_t fi = wrap(m->face_indices[(size_t)i * K + k], F);
      const real sg = (real)m->face_signs[(size_t)i * K + k];
      for (int q = 0; q < Q; ++q) {
        const real x = flux[(size_t)fi * Q + q] * sg;
        acc[q] = (k == 0) ? x : acc[q] + x;
      }
    }
    for (int q = 0; q < Q; ++q) {
      real s = acc[q];
      if (m->inv_area) s = s * (real)m->inv_area[i];
      const real fq = pdf[(size_t)i * Q + q];
      fnew[(size_t)i * Q + q] = fq + m->dt * (m->inv_tau * (feq[(size_t)i * Q + q] - fq) - s);
    }
  }
  memcpy(pdf, fnew, sizeof(real) * (size_t)N * Q);
}

/* n_steps steps in place.  Optional outputs (may be NULL) receive the
 * reference's post-step Cells.rho/vel/pdf_eq and Faces.pdf of the last step.
 * Returns 0, or -1 when scratch memory cannot be allocated. */
int ORACLE_FN(oracle_step)(const oracle_mesh_t *m, real *cell_pdf, real *node_pdf, real *node_rho,
                real *node_vel, int n_steps, int n_threads, real *out_rho, real *out_vel,
                real *out_eq, real *out_flux) {
  const size_t N = (size_t)m->N, F = (size_t)m->F;
  real *rho = malloc(sizeof(real) * (N ? N : 1));
  real *vel = malloc(sizeof(real) * 2 * (N ? N : 1));
  real *feq = malloc(sizeof(real) * Q * (N ? N : 1));
  real *flux = malloc(sizeof(real) * Q * (F ? F : 1));
  real *fnew = malloc(sizeof(real) * Q * (N ? N : 1));
  if (!rho || !vel || !feq || !flux || !fnew) {
    free(rho), free(vel), free(feq), free(flux), free(fnew);
    return -1;
  }
  int nt = n_threads;
#ifdef _OPENMP
  if (nt <= 0) nt = omp_get_max_threads();
#else
  nt = 1;
#endif
  for (int s = 0; s < n_steps; ++s)
    step_once(m, cell_pdf, node_pdf, node_rho, node_vel, rho, vel, feq, flux, fnew, nt);
  if (n_steps > 0) {
    if (out_rho) memcpy(out_rho, rho, sizeof(real) * N);
    if (out_vel) memcpy(out_vel, vel, sizeof(real) * 2 * N);
    if (out_eq) memcpy(out_eq, feq, sizeof(real) * Q * N);
    if (out_flux) memcpy(out_flux, flux, sizeof(real) * Q * F);
  }
  free(rho), free(vel), free(feq), free(flux), free(fnew);
  return 0;
}

int ORACLE_FN(oracle_max_threads)(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
