/*
 * fvdbm.h - C ABI of the GB300 FVDBM time stepper (libfvdbm.so).
 *
 * This is the drop-in boundary for the reference's Environment.init/step
 * (MADALERAU/FVDBM-JAX src/environment.py:38-42 and :55-65) acting on the
 * Cells/Faces/Nodes containers that Mesher.to_env builds
 * (src/mesher.py:610-693) and set_vel_node/set_rho_node mutate
 * (src/mesher.py:697-742).  The reference binds this path from Python, so the
 * binding is ctypes (fvdbm-jax_gb300/_native.py); every argument is a plain
 * pointer or size.
 *
 * Conventions
 *   - Return codes: 0 ok, negative on error (FVDBM_E*); the message is in
 *     fvdbm_last_error(handle) (or fvdbm_last_error(NULL) for create).
 *   - Host arrays are read during the call and never retained.  The handle
 *     owns its device memory and its CUDA stream.  One handle is driven from
 *     one host thread at a time.
 *   - Arrays are in the reference's element order and row-major layout; the
 *     library renumbers cells internally and undoes it on every read-back.
 *   - fvdbm_step is stream-ordered and returns before the GPU finishes; the
 *     read-back calls synchronise.
 *   - No atomics on the step path: results are bitwise run-to-run stable and
 *     match the CPU oracle bit for bit.
 */
#ifndef FVDBM_H
#define FVDBM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FVDBM_ABI_VERSION 4

#define FVDBM_OK 0
#define FVDBM_EINVAL (-1)  /* invalid argument or inconsistent mesh */
#define FVDBM_ECUDA (-2)   /* CUDA runtime error */
#define FVDBM_ENOMEM (-3)  /* allocation failed */
#define FVDBM_EDEVICE (-4) /* device-side status word set */
#define FVDBM_ENONFINITE (-5) /* fvdbm_run_to_steady: the state turned non-finite
                                 (NaN residual): the run diverged */

/* Faces.flux_scheme (src/containers.py:197-203) */
#define FVDBM_UPWIND 0
#define FVDBM_LAX_WENDROFF 1

/* Flux multipliers of the cell-centre stencil face classes:
 * FACE_SCALE   = CCStencilFaces, flux * cos(alpha)      (src/faces.py:54-74)
 * FACE_Q_SCALE = CCStencilKsiFaces, flux * (xi.n)/(xi.npq), q0 -> 0
 *                                                       (src/faces.py:119-141) */
#define FVDBM_VARIANT_NONE 0
#define FVDBM_VARIANT_FACE_SCALE 1
#define FVDBM_VARIANT_FACE_Q_SCALE 2

/* Cell numbering used on the device (results are always returned in the
 * caller's order). */
#define FVDBM_ORDER_NONE 0
#define FVDBM_ORDER_RCM 1    /* reverse Cuthill-McKee on the face graph */
#define FVDBM_ORDER_MORTON 2 /* Z-order of cell_xy (needs cell_xy) */

/* Kernel family for the step. */
#define FVDBM_KERNEL_AUTO 0       /* fastest family the mesh allows (FUSED_NODES from 2^18 cells,
                                     FUSED below and for D2Q13, STAGED when the fused kernels
                                     cannot run: not triangles, padded or foreign face slots,
                                     per-q flux scale) */
#define FVDBM_KERNEL_STAGED 1     /* node BC + face flux + cell gather (3 kernels) */
#define FVDBM_KERNEL_FUSED 2      /* node BC + fused cell kernel (2 kernels; triangles) */
#define FVDBM_KERNEL_TILE 3       /* persistent tile kernel, nodes evaluated in-tile (1 kernel) */
#define FVDBM_KERNEL_TILE_SPLIT 4 /* node BC kernel + persistent tile kernel (2 kernels) */
#define FVDBM_KERNEL_ONE 5        /* node and cell blocks in one launch (1 kernel) */
#define FVDBM_KERNEL_BATCH 6      /* (reported by fvdbm_get_info) packed batch: node BC + fused cell kernel */
#define FVDBM_KERNEL_FUSED_NODES 7 /* fused cell kernel that also updates the boundary nodes of the
                                      next step (1 kernel) */
#define FVDBM_KERNEL_PERSIST 8    /* all the steps of one fvdbm_step call in one cooperative launch:
                                     nodes, grid barrier, cells, grid barrier per step (triangles;
                                     for meshes whose launches are short) */
#define FVDBM_KERNEL_FAST 9       /* FUSED_NODES with contracted float32 arithmetic (multiply-adds,
                                     reciprocals of the lattice constants, no literal paths for
                                     non-finite values): bitwise reproducible run to run, within a
                                     few float32 ulps per step of the reference's rounding, not
                                     bitwise equal to it (D2Q9 triangles; never picked by AUTO) */

/* Reference-layout mesh (host pointers).  N cells, F faces, P nodes. */
typedef struct fvdbm_mesh {
  int32_t n_cells;
  int32_t n_faces;
  int32_t n_nodes;
  int32_t cell_face_stride;          /* K: columns of Cells.face_indices */
  int32_t node_cell_stride;          /* Kn: columns of Nodes.cells_index */
  const int32_t *cell_face_indices;  /* [N][K] Cells.face_indices, -1 padded */
  const int32_t *cell_face_signs;    /* [N][K] Cells.face_normals (-1,0,1) */
  const int32_t *face_cells;         /* [F][2] Faces.stencil_cells_index, -1 = ghost */
  const float *face_dists;           /* [F][2] Faces.stencil_dists */
  const int32_t *face_nodes;         /* [F][2] Faces.nodes_index */
  const float *face_n;               /* [F][2] Faces.n */
  const float *face_L;               /* [F]    Faces.L */
  const float *face_scale;           /* [F] (FACE_SCALE) or [F][9] (FACE_Q_SCALE), else NULL */
  const int32_t *node_type;          /* [P] Nodes.type: 0 none, 1 velocity, 2 density */
  const int32_t *node_cells;         /* [P][Kn] Nodes.cells_index, -1 padded */
  const float *node_dists;           /* [P][Kn] Nodes.cell_dists, -1 padded */
  const float *cell_xy;              /* [N][2] cell centroids for MORTON, or NULL */
  const float *cell_inv_area;        /* [N] 1/area to scale the flux sum, or NULL
                                        (NULL = the reference's update, no area) */
  const float *cell_area;            /* [N] cell areas weighting the mass of
                                        fvdbm_residual, or NULL (weight 1) */
} fvdbm_mesh_t;

/* Step parameters, all float32 as the reference evaluates them
 * (src/dynamics.py:64-74, src/containers.py:121). */
typedef struct fvdbm_params {
  int32_t flux_scheme; /* FVDBM_UPWIND | FVDBM_LAX_WENDROFF */
  int32_t variant;     /* FVDBM_VARIANT_* */
  float inv_tau;       /* float32(1/tau), 1/tau taken in double */
  float delta_t;       /* float32(delta_t) */
  float c2;            /* C*C with C = 1/sqrt(3) in float32 */
  float c4x2;          /* 2*((C*C)*(C*C)) */
  float c2x2;          /* 2*(C*C) */
  int32_t ordering;    /* FVDBM_ORDER_* */
  int32_t kernel;      /* FVDBM_KERNEL_* */
  int32_t device;      /* CUDA device ordinal */
  int32_t lattice;     /* velocities: 9 (D2Q9, also when 0) or 13 (D2Q13,
                          src/dynamics.py:77-102: staged or fused kernels, no
                          flux-scale variant; c2, c4x2, c2x2 are then those of
                          C = 1/sqrt(2)) */
  float c6x2;          /* D2Q13: 2*C^6 with C^6 = (C*C)*((C*C)*(C*C)) */
} fvdbm_params_t;

/* Sizes and the algorithmic traffic of one step, for reporting. */
typedef struct fvdbm_info {
  int32_t n_cells, n_faces, n_nodes;
  int32_t n_bc_nodes;       /* type 1/2 nodes updated each step */
  int32_t n_ghost_faces;    /* faces with a ghost slot */
  int32_t kernel;           /* family actually used */
  int32_t launches_per_step;
  int32_t padded_cells;     /* row stride of the [9][Np] pdf */
  int32_t ctas_per_sm;      /* resident CTAs per SM of the tile kernel (0 if unused) */
  int32_t const_division;   /* divisions by the lattice constants use a
                               known-divisor form verified on this device to
                               equal IEEE division for every float32 dividend:
                               2 the two-operation form, 1 the five-operation
                               form, 0 neither (IEEE division) */
  double bytes_per_step;    /* algorithmic bytes of one step */
  double device_bytes;      /* device memory held by the handle */
} fvdbm_info_t;

/* Environment.init (src/environment.py:38-42): validate the containers,
 * renumber, build the device tables and upload the rest state
 * (every pdf = feq(1,0) = W, src/containers.py:29).  Replaces the jit
 * trace of the first Environment.step. */
int fvdbm_create(const fvdbm_mesh_t *mesh, const fvdbm_params_t *params, void **handle);

/* The dynamic pytree leaves (Cells.pdf, Nodes.pdf/rho/vel,
 * src/containers.py:33-36,75,321).  NULL leaves are left unchanged.
 * cell_pdf [N][9], node_pdf [P][9], node_rho [P], node_vel [P][2].  The
 * arrays are read before the call returns; a page-locked cell_pdf is read
 * by the device directly over the host link. */
int fvdbm_set_state(void *handle, const float *cell_pdf, const float *node_pdf,
                    const float *node_rho, const float *node_vel);

/* Halo exchange of a domain decomposition (no counterpart in the
 * reference, which steps one domain).  A rank's handle holds its owned cells
 * plus a one-ring halo of read-only cells (fvdbm-jax_gb300/partition.py
 * builds the sub-meshes); after each step it packs the owned rows its
 * neighbours read, the buffers move to the neighbours (peer copy, NCCL
 * send/recv, or through the host), and each neighbour unpacks them over its
 * halo rows.  buf is [n][Q] float32 rows of Cells.pdf for cells[0..n) (this
 * handle's own, reference-order cell indices), in memory the device
 * addresses (device memory or page-locked host memory).  Stream-ordered on
 * fvdbm_stream(handle); cells is read before the call returns.  Unpacking
 * counts as an upload of cell pdfs: boundary nodes are recomputed before the
 * next step.  FVDBM_EINVAL for an index outside [0, n_cells) or a batch
 * handle. */
int fvdbm_pack_cells(void *handle, const int32_t *cells, int32_t n, float *buf);
int fvdbm_unpack_cells(void *handle, const int32_t *cells, int32_t n, const float *buf);

/* Cell pdfs set to the equilibrium of given macros, f = feq(rho, u)
 * (src/dynamics.py:70-74, the form Container.__init__ uses for its default
 * state, src/containers.py:24-30): the warm start.  rho [N], vel [N][2]. */
int fvdbm_set_cells_eq(void *handle, const float *rho, const float *vel);

/* n_steps applications of Environment.step (src/environment.py:55-65). */
int fvdbm_step(void *handle, int32_t n_steps);

/* One step split at its kernel boundary so a caller can time each kernel
 * with events on fvdbm_stream(): phase 1 launches the boundary-node kernel
 * (Nodes.calc_pdfs), phase 2 the cell kernel(s) (Faces.calc_fluxes +
 * Cells.calc_pdfs) and completes the step.  Phase 1 then phase 2 is exactly
 * fvdbm_step(handle, 1). */
int fvdbm_step_phase(void *handle, int32_t phase);

/* Cells.pdf after the last step, and Cells.rho/vel/pdf_eq as the reference
 * leaves them: the macros of the pdf before the last update
 * (src/environment.py:60-64).  Any pointer may be NULL.  Synchronises.
 * pdf [N][9], rho [N], vel [N][2], pdf_eq [N][9].  Page-locked rho and vel
 * arrays are written by the device directly over the host link. */
int fvdbm_get_cells(void *handle, float *pdf, float *rho, float *vel, float *pdf_eq);

/* Nodes.pdf/rho/vel after the last step.  pdf [P][9], rho [P], vel [P][2]. */
int fvdbm_get_nodes(void *handle, float *pdf, float *rho, float *vel);

/* Faces.pdf after the last step: the face fluxes of the last update
 * (src/containers.py:205-213).  flux [F][9]. */
int fvdbm_get_face_fluxes(void *handle, float *flux);

/* Self-test of the bounded wait that the step kernels use (the node blocks
 * of the single-launch step wait for the blocks that record the stencil
 * macros): one device thread waits for a flag, set beforehand when flag_set
 * is nonzero and never set otherwise, polling at most `iterations` times
 * (1 .. 2^24, each poll followed by a ~128 ns sleep).  *status receives the
 * device status word: 0, or FVDBM_STATUS_WAIT_TIMEOUT when the wait ran out;
 * the context stays usable either way.  No counterpart in the reference. */
#define FVDBM_STATUS_WAIT_TIMEOUT 1
int fvdbm_wait_selftest(int32_t device, int32_t flag_set, int32_t iterations, int32_t *status);

/* Self-test of the division by a known divisor that the kernels use for the
 * lattice constants C^2, 2C^4 and 2C^2: counts, over all 2^32 float32
 * dividends, those whose quotient differs in value from IEEE x / divisor on
 * this device, and reports the lowest such bit pattern (0xFFFFFFFF if none).
 * No counterpart in the reference (it divides with XLA's division). */
int fvdbm_const_div_check(int32_t device, float divisor, uint64_t *mismatches,
                          uint32_t *first_mismatch);

/* The same check for one form: form 5 is the five-operation correction form
 * (what fvdbm_const_div_check checks), form 2 the two-operation form
 * RN(x*zh + RN(x*zl)) with zh = RN(1/divisor), zl = RN(1/divisor - zh)
 * (Brisebarre, Muller and Raina, IEEE Trans. Computers 53(8), 2004).  The
 * kernels use form 2 only for divisors that pass both checks.  No
 * counterpart in the reference. */
int fvdbm_const_div_check_form(int32_t device, float divisor, int32_t form, uint64_t *mismatches,
                               uint32_t *first_mismatch);

/* Block until the handle's stream is idle.  Returns FVDBM_EDEVICE when a
 * kernel reported a failure on the device status word (a bounded wait that
 * gave up), else 0 or a CUDA error. */
int fvdbm_sync(void *handle);

/* The handle's cudaStream_t (for event timing by the caller). */
void *fvdbm_stream(void *handle);

int fvdbm_get_info(void *handle, fvdbm_info_t *info);

/* Message of the last failure on this handle (or of the last failed create
 * when handle is NULL). */
const char *fvdbm_last_error(void *handle);

int fvdbm_destroy(void *handle);

int fvdbm_abi_version(void);

/* Convergence monitor (the reference has none; it steps a fixed count).
 * Velocity residual and total mass of the current cell pdfs, in double:
 *   res_u = ||u - u_prev||_2 / (K * delta_t * max(||u_prev||_2, 1e-30))
 *   mass  = sum_i rho_i * area_i     (area 1 when the mesh gave no cell_area)
 * u, rho are the float32 macros of each cell (src/dynamics.py:35-47); u_prev
 * is the velocity at the previous fvdbm_residual call, K the steps taken
 * since then.  res_u is +inf on the first call, after fvdbm_set_state of the
 * cell pdfs, or when no step was taken since the previous call; NaN when a
 * cell's rho or u is not finite.  Sums are formed in a fixed order: results
 * are bitwise reproducible.  Synchronises the handle's stream. */
int fvdbm_residual(void *handle, double *res_u, double *mass);

/* Steps in chunks of check_every until res_u < threshold, or max_steps
 * steps were taken.  steps_taken and res_u receive the outcome (res_u of the
 * last check).  The first residual snapshot is taken before the first chunk
 * when none is current.  res_u == 0 means that no cell's velocity changed
 * over the last chunk: the float32 state is frozen (a fixed point of the
 * float32 step, which it will not leave), whether or not the flow developed;
 * the run stops there.  A NaN residual (a cell's rho or u not finite: the
 * run diverged) stops the run and returns FVDBM_ENONFINITE, with
 * steps_taken and res_u filled. */
int fvdbm_run_to_steady(void *handle, double threshold, int32_t check_every, int64_t max_steps,
                        int64_t *steps_taken, double *res_u);

/* ---- Packed batch (no counterpart in the reference, which steps one
 * Environment at a time).  n_cases independent cases in one handle: their
 * meshes are joined into one device mesh (cells of a case stay contiguous,
 * ordered within the case), so each step is one node launch and one cell
 * launch for all cases, with each case's own 1/tau and delta_t.  Every case
 * evolves bit for bit as it would in its own handle.  Cases that converge
 * retire: their cells are no longer read or written.  Needs triangles (3
 * face slots per cell) and no flux-scale variant; params[s] may differ only in
 * inv_tau and delta_t.  fvdbm_step / fvdbm_get_cells / fvdbm_get_nodes /
 * fvdbm_residual act on the union (cells, nodes in case order). */
int fvdbm_batch_create(const fvdbm_mesh_t *meshes, const fvdbm_params_t *params, int32_t n_cases,
                       void **handle);

/* Launch shape of the batch cell kernel: threads per block (128 or 256) and
 * the L2 prefetch distance in waves (0 = none).  The autotuner sets these. */
int fvdbm_batch_config(void *handle, int32_t block, int32_t prefetch_waves);

/* Per-case residual and mass (as fvdbm_residual, per case).  [n_cases]. */
int fvdbm_batch_residual(void *handle, double *res_u, double *mass);

/* The same for the cases with take[s] != 0 only: each over the steps that
 * case took since its own last residual, whose snapshot is then renewed;
 * other cases keep their snapshots and their res_u/mass entries are left
 * as they were.  (The first call after creation or an upload takes every
 * case.)  [n_cases]. */
int fvdbm_batch_residual_cases(void *handle, const int32_t *take, double *res_u, double *mass);

/* Mark cases active (1) or retired (0).  A retired case's cells keep their
 * current state in both buffers and are skipped by the step.  [n_cases]. */
int fvdbm_batch_set_active(void *handle, const int32_t *active);

/* Steps every active case, checking the residuals every check_every steps.
 * A case retires with
 *   FVDBM_CASE_CONVERGED  its residual fell below threshold, or reached exactly
 *                         0 (an exact float32 fixed point) from a previous
 *                         residual below 100 * threshold,
 *   FVDBM_CASE_NONFINITE  its residual turned NaN (the case diverged),
 *   FVDBM_CASE_FROZEN     its residual is exactly 0 (no cell's velocity
 *                         changed over the last check interval) while the
 *                         previous one was not below 100 * threshold: the
 *                         float32 state stopped changing far from
 *                         convergence (typically a flow that float32 keeps
 *                         from developing),
 *   FVDBM_CASE_STALLED    its residual set no new minimum in
 *                         FVDBM_STALL_CHECKS consecutive checks,
 *   FVDBM_CASE_CAPPED     it took max_steps[s] steps.
 * Returns when no case is active.  steps [n_cases] = steps each case took,
 * res_u = its last residual, status as above.  Arrays are [n_cases]. */
#define FVDBM_CASE_CAPPED 0
#define FVDBM_CASE_CONVERGED 1
#define FVDBM_CASE_NONFINITE 2
#define FVDBM_CASE_FROZEN 3
#define FVDBM_CASE_STALLED 4
#define FVDBM_STALL_CHECKS 50

/* The same with each case's check window in its own time: the cases step
 * together in chunks of check_every steps, and a case's residual is taken
 * once it has advanced at least check_time time units (ceil(check_time /
 * delta_t_s) steps, rounded up to whole chunks) since its last check, or at
 * its step cap; res_u then measures the change over that window (K is the
 * case's own step count).  A float32 state keeps rounding-level changes in u
 * after it has converged; measured over a window of K steps their residual
 * is about 2e-6 / (K * delta_t), so a window of a few time units keeps that
 * floor below a 1e-6 threshold for every case whatever its delta_t.
 * check_time 0 is fvdbm_batch_run_to_steady. */
int fvdbm_batch_run_to_steady_time(void *handle, double threshold, int32_t check_every, double check_time,
                                   const int64_t *max_steps, int64_t *steps, double *res_u,
                                   int32_t *status);
int fvdbm_batch_run_to_steady(void *handle, double threshold, int32_t check_every,
                              const int64_t *max_steps, int64_t *steps, double *res_u,
                              int32_t *status);

/* Largest padded face count (faces rounded up to a multiple of 128, at least
 * 128) that fvdbm_step_static_scratch takes: its face-flux scratch is a fixed
 * device array of 9 x 131072 float32 = 4.5 MiB per device. */
#define FVDBM_STATIC_SCRATCH_MAX_FACES 131072

/* No counterpart in the reference.  n_steps steps of the staged kernels
 * (boundary nodes, per-face fluxes, per-cell gather and update) like
 * fvdbm_step on a handle created with FVDBM_KERNEL_STAGED, with the same
 * results, but with the per-step face fluxes in a fixed device array of the
 * library instead of the handle's buffer, and with no device memory
 * allocated or freed during the call: for callers that cannot allocate
 * device memory while they step, because another allocator owns the
 * device's memory (JAX/XLA preallocates most of it by default, so the
 * reference's own process has little left) or because a cudaMalloc or
 * cudaFree there would stall the device (cudaFree synchronises it).
 * Only single-mesh handles created with FVDBM_KERNEL_STAGED (or that the
 * fused kernels refused) are accepted, not batch handles; meshes whose
 * padded face count exceeds FVDBM_STATIC_SCRATCH_MAX_FACES are rejected with
 * FVDBM_EINVAL and a message, before any work is queued.  The first call on
 * a device looks up the array's device address (once per device and CUDA
 * context, under a lock: again after the context was re-created, e.g. by
 * cudaDeviceReset); make that first call before any stream capture.  Every call on a device shares the
 * one array and leaves its last fluxes there (no part of it needs to start
 * at zero: each step writes every face before it reads one); calls whose
 * kernels overlap on the GPU (other streams, other handles, other threads)
 * race on it, so order them on one stream or with events.  Asynchronous,
 * like fvdbm_step. */
int fvdbm_step_static_scratch(void *handle, int32_t n_steps);

#ifdef __cplusplus
}
#endif

#endif /* FVDBM_H */
