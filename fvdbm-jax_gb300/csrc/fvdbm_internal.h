// Internal structures of libfvdbm: the host-side plan built from the
// reference-layout containers and the device view the kernels read.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/fvdbm.h"

namespace fvdbm {

constexpr int Q = 9;

// Half-face code of the fused kernel (one per cell and face slot):
//   bits 0-1  sigma + 1   (sigma in {-1,0,1}: Cells.face_normals)
//   bit  2    this cell is the face's slot 1 (else slot 0)
//   bit  3    the other slot is a ghost (other = ghost-table index)
//   bits 4-31 the other cell (device numbering) or the ghost index
constexpr int HF_SLOT1 = 1 << 2;
constexpr int HF_GHOST = 1 << 3;
constexpr int HF_SHIFT = 4;
constexpr int64_t HF_MAX_INDEX = (int64_t(1) << 27) - 1;

// Persistent tile kernel: TILE consecutive cells per CTA iteration; the
// boundary nodes a tile's ghost faces need are evaluated inside the tile.
constexpr int TILE = 256;
constexpr int TILE_MAX_NODES = 128;    // nodes evaluated per tile
constexpr int TILE_MAX_ENTRIES = 256;  // node-stencil cells per tile
constexpr int TN_OWNER = 1 << 4;       // tn_kind flag: this tile writes the node state
constexpr int NODE_BLOCK_ENTRIES = 256; // node blocks: entries (= threads) per block

// rows of the half-face array for K face slots
struct HfRows {
  int K, scheme, variant;
  __host__ __device__ constexpr int code(int k) const { return k; }
  __host__ __device__ constexpr int nx(int k) const { return K + k; }
  __host__ __device__ constexpr int ny(int k) const { return 2 * K + k; }
  __host__ __device__ constexpr int ls(int k) const { return 3 * K + k; }
  __host__ __device__ constexpr int r(int k) const { return 4 * K + k; }
  __host__ __device__ constexpr int d2(int k) const { return (scheme == 1 ? 5 : 4) * K + k; }
  __host__ __device__ constexpr int sc(int k) const { return (scheme == 1 ? 6 : 4) * K + k; }
  __host__ __device__ constexpr int rows() const { return (4 + (scheme == 1 ? 2 : 0) + (variant == 1 ? 1 : 0)) * K; }
};

// Rows of the fast family's compact half faces (FVDBM_KERNEL_FAST): per slot
// the code word, a = n * (L*sigma) (times the face scale of FACE_SCALE, times
// 1/area in finite-volume mode) as two rows, and for Lax-Wendroff the
// interpolation weight r and g = dt / (D2 * L*sigma [* scale] [/ area]).  In
// the upwind code word HF_SLOT1 is then slot1 XOR (L*sigma < 0): the upwind
// side of direction q is this cell's exactly when xi_q . a >= 0 (xi_q . a == 0
// carries no flux).
struct HfFastRows {
  int K, scheme;
  __host__ __device__ constexpr int code(int k) const { return k; }
  __host__ __device__ constexpr int ax(int k) const { return K + k; }
  __host__ __device__ constexpr int ay(int k) const { return 2 * K + k; }
  __host__ __device__ constexpr int r(int k) const { return 3 * K + k; }
  __host__ __device__ constexpr int g(int k) const { return 4 * K + k; }
  __host__ __device__ constexpr int rows() const { return (3 + (scheme == 1 ? 2 : 0)) * K; }
};

// Node-cell entry: cell index (device numbering); bit 31 marks an entry whose
// reference index was -1 (its rho/vel gather wraps to the last cell but its
// non-equilibrium part is zero, src/containers.py:388-390).
constexpr uint32_t ND_NEQ_ZERO = 0x80000000u;

struct HostPlan {
  int N = 0, F = 0, P = 0, K = 0, Kn = 0;
  int Np = 0;  // padded row stride of [9][Np] cell arrays
  int Fp = 0;  // padded row stride of [9][Fp] face arrays
  int scheme = 0, variant = 0;
  int q = 9;  // lattice velocities
  bool fv = false;
  bool fast = false;  // compact half faces of the fast family
  bool fusable = false;
  int ordering = 0;

  std::vector<int32_t> cell_new;  // old -> new
  std::vector<int32_t> cell_old;  // new -> old
  int32_t last_cell_new = 0;      // device id of the reference's cell N-1

  // faces in device order
  std::vector<int32_t> face_old;  // new -> old
  std::vector<int32_t> face_new;  // old -> new
  std::vector<int32_t> fs0, fs1;  // slot cells (device ids) or -1
  std::vector<float> fnx, fny, fL;
  std::vector<float> fr, fD2;     // Lax-Wendroff: d0/(d0+d1), 2*(d0+d1)
  std::vector<int32_t> fna, fnb;  // end nodes (device node ids) for ghosts
  std::vector<float> frl, frr;    // ghost ratios d0/d1 (slot 0 ghost), d1/d0 (slot 1 ghost)
  std::vector<int32_t> fkl, fkr;  // known cells of those ghosts
  std::vector<float> fscale;      // [F] or [9][Fp]
  int n_ghost_faces = 0;

  // staged gather: [K][Np]
  std::vector<int32_t> cf_face;
  std::vector<float> cf_sign;

  // fused half faces, AoSoA [Np/32][hrows][32] of 32-bit words; rows are
  // code (K), nx (K), ny (K), L*sigma (K), then d0/(d0+d1) (K), 2(d0+d1) (K)
  // for Lax-Wendroff, then the stencil scale (K) for the cos variant
  int hrows = 0;
  std::vector<uint32_t> hf;
  std::vector<int32_t> gh_a, gh_b;
  std::vector<float> gh_r;
  // node blocks of the node kernel: contiguous computed nodes with at most
  // NODE_BLOCK_ENTRIES stencil entries each; nb_meta = 4 ints per block
  std::vector<int32_t> nb_ptr, nb_meta;
  std::vector<uint32_t> pe_slot;  // padded node-block tables (see plan.cpp)
  std::vector<float> pe_w, pn_sumw;
  std::vector<int32_t> pn_meta;
  int stencil_start = 0;  // device cells [stencil_start, stencil_end) are node-stencil cells
  int stencil_end = 0;    // (last: [., N); first, for the in-kernel node update: [0, .))
  bool stencil_first = false;
  int last_slot = -1;     // cprod slot of the reference's last cell (stencil_first, padded nodes)
  std::vector<uint8_t> cblk_ghost;  // per 256-cell block: any ghost face
  std::vector<int32_t> sched;       // single-launch tickets: cell block >= 0, node block -(b+1)

  // nodes on the device: computed (type 1/2) first, then frozen ghost ends
  int M = 0, Mc = 0, Mp = 0;
  std::vector<int32_t> node_dev;   // reference node -> device id or -1
  std::vector<int32_t> node_orig;  // device id -> reference node
  std::vector<int32_t> nd_type, nd_ptr, nd_npad;
  std::vector<uint32_t> nd_cell;
  std::vector<float> nd_w, nd_sumw;

  std::vector<float> inv_area;  // [Np] when fv
  std::vector<float> area;      // [Np] when the mesh gives cell areas (mass weights)

  // tile tables (valid when tile_ok)
  bool tile_ok = false;
  int NT = 0;
  std::vector<int32_t> tn_ptr, tn_dev, tn_kind, tn_npad, tn_e0, tn_ecnt;
  std::vector<float> tn_sumw;
  std::vector<int32_t> te_ptr;
  std::vector<uint32_t> te_cell;
  std::vector<float> te_w;
  std::vector<int32_t> tgh_a, tgh_b;  // ghost end nodes as tile-local indices

  bool finite_n = true;
  double bytes_per_step = 0.0;

  // packed batch of independent cases (S > 0): case s owns device cells
  // [case_cell[s], case_cell[s+1]); cell_case[i] is the case of device cell i
  int S = 0;
  std::vector<int32_t> case_cell;
  std::vector<int32_t> cell_case;  // [Np]
};

// Segments of a union mesh: case s owns cells [cell_ptr[s], cell_ptr[s+1]),
// faces [face_ptr[s], ..) and nodes [node_ptr[s], ..).  A padded -1 node
// stencil entry of a case wraps to that case's last cell.
struct BatchSegs {
  int S;
  const int32_t* cell_ptr;
  const int32_t* face_ptr;
  const int32_t* node_ptr;
};

// Build the plan; returns an empty string on success, else the reason.
std::string build_plan(const void* mesh, const void* params, HostPlan& hp,
                       const BatchSegs* segs = nullptr);

// The union of S cases' meshes (batch.cpp); `mesh` points into the vectors.
struct UnionMesh {
  int K = 0, Kn = 0;
  std::vector<int32_t> cfi, cfs, fc, fnd, nt, nc, cell_ptr, face_ptr, node_ptr;
  std::vector<float> fd, fn, fL, nd, xy, ia, area;
  fvdbm_mesh_t mesh{};
  BatchSegs segs{};
};
std::string build_union(const fvdbm_mesh_t* meshes, int S, UnionMesh& u);

// Division by a divisor known in advance: y, zr = RN(1/y) and
// zl = RN(1/y - zr).  ok says the correction form (five operations) was
// verified against IEEE division for every float32 dividend on this device
// (else the kernels divide with '/'); two says the same of the two-operation
// form, which is then used instead.
struct CDiv {
  float y, zr, zl;
  int ok, two;
};

struct DevPlan {
  int N, Np, F, Fp, K, M, Mp, Mc;
  int scheme, variant, fv;
  int last_cell;
  int finite_n;  // every face normal is finite (enables the symmetric xi.n form)
  float inv_tau, dt, c2, c4x2, c2x2;
  float one, neg_one;  // 1 and -1 as run-time values (paired sums of paired products)
  float c6x2;  // D2Q13: 2 C^6
  int q;       // lattice velocities: 9 or 13
  CDiv d_c2, d_c4x2, d_c2x2, d_c6x2;  // d_c6x2: D2Q13 only
  int cdiv_mode;  // 2: the lattice's divisors' two-operation forms verified, 1: five-operation, 0: neither
  int fast;       // FVDBM_KERNEL_FAST: contracted arithmetic in the fused cell update
  // staged faces
  const int* fs0;
  const int* fs1;
  const float* fnx;
  const float* fny;
  const float* fL;
  const float* fr;
  const float* fD2;
  const int* fna;
  const int* fnb;
  const float* frl;
  const float* frr;
  const int* fkl;
  const int* fkr;
  const float* fscale;
  const int* cf_face;
  const float* cf_sign;
  // fused half faces (AoSoA, hrows rows)
  const unsigned* hf;
  int hrows;
  const int* gh_a;
  const int* gh_b;
  const float* gh_r;
  // nodes
  const int* nd_type;
  const int* nd_ptr;
  const int* nd_npad;
  const unsigned* nd_cell;
  const float* nd_w;
  const float* nd_sumw;
  const int* nb_meta;  // node blocks: {first node, end node, first entry, end entry}
  int NB;
  // macros of the node-stencil cells [stencil_start, N): cprod[r][Sp] with
  // r = rho, ux, uy, f_q - feq_q; written by the fused kernel for the next step
  int stencil_start, stencil_end, Sp;
  int last_slot;
  int stencil_first;
  // in-kernel node update (k_fused_nodes): the next step's node buffers
  float* node_pdf_nx;
  float* node_rho_nx;
  float* node_vel_nx;
  float* cprod;
  const unsigned* pe_slot;
  const float* pe_w;
  const int* pn_meta;
  const float* pn_sumw;
  float* node_pdf;  // [9][Mp]
  float* node_rho;  // [Mp]
  float* node_vel;  // [2][Mp]
  const float* inv_area;
  // tile kernel
  int NT;
  int tile_nodes;  // boundary nodes evaluated inside the tile kernel (else by k_nodes)
  const int* tn_ptr;
  const int* tn_dev;
  const int* tn_kind;
  const int* tn_npad;
  const int* tn_e0;
  const int* tn_ecnt;
  const float* tn_sumw;
  const int* te_ptr;
  const unsigned* te_cell;
  const float* te_w;
  const int* tgh_a;
  const int* tgh_b;
  int* status;  // device status word (0 ok); set when a bounded wait gives up
  int* step_ctr;  // single-launch step: ticket, node blocks published, blocks finished
  const unsigned char* cblk_ghost;  // per 256-cell block: has a ghost face
  const int* sched;                 // single-launch tickets: cell block >= 0, node block -(b+1)
  // packed batch: per-cell case, per-case 1/tau, dt and active flag
  const int* cell_case;
  const float* case_inv_tau;
  const float* case_dt;
  const int* case_active;
  // cell blocks of the active cases (block size of the batch launch); all
  // blocks when null
  const int* blk_list;
  int n_blk;
};

constexpr int STATUS_WAIT_TIMEOUT = 1;

// kernel launchers (kernels.cu)
// pdl: launch with programmatic dependent launch after a step kernel
cudaError_t launch_nodes(const DevPlan& p, const float* f, cudaStream_t s, bool pdl = false);
cudaError_t launch_fused(const DevPlan& p, const float* fin, float* fout, cudaStream_t s,
                         bool pdl = false);
// node kernel fed by the stencil macros the previous fused kernel recorded
cudaError_t launch_nodes_cp(const DevPlan& p, const float* f, cudaStream_t s, bool pdl);
// fused cell kernel that also computes the next step's boundary nodes (node
// blocks in the grid wait, bounded, for the stencil cells' blocks)
cudaError_t launch_fused_nodes(const DevPlan& p, const float* fin, float* fout, cudaStream_t s, bool pdl);
// n_steps steps in one cooperative launch; f0 is the current buffer; bar is
// one device int (zeroed by the launch)
cudaError_t launch_persist(const DevPlan& p, float* f0, float* f1, int n_steps, int* bar, cudaStream_t s);
// record the stencil macros of f (after an upload of the cell pdfs)
cudaError_t launch_stencil_macros(const DevPlan& p, const float* f, cudaStream_t s);
// the whole step in one launch (node blocks then cell blocks, see kernels.cu)
cudaError_t launch_step(const DevPlan& p, const float* fin, float* fout, cudaStream_t s, bool pdl);
cudaError_t launch_face_flux(const DevPlan& p, const float* f, float* flux, cudaStream_t s);
// Persistent tile kernel (tile.cu): one launch per step.  prepare_tile sets
// the kernel's shared-memory attribute and grid size; call it outside any
// stream capture before the first launch_tile.
cudaError_t prepare_tile(const DevPlan& p);
int tile_ctas_per_sm(const DevPlan& p);
cudaError_t launch_tile(const DevPlan& p, const float* fin, float* fout, cudaStream_t s);
cudaError_t launch_gather(const DevPlan& p, const float* fin, const float* flux, float* fout,
                          cudaStream_t s);
cudaError_t launch_macros(const DevPlan& p, const float* f, float* rho, float* vel, float* feq,
                          cudaStream_t s);
// FP64 residual / mass partial sums (monitor.cu): one block per chunk of
// cells, then one block per segment of chunks (seg == nullptr: all chunks,
// one segment).  out[4*s..] = {sum |du|^2, sum |u_prev|^2, sum rho*A, bad cells}.
// chunk_start (nullable): chunk b covers cells [chunk_start[b], chunk_start[b+1]).
int residual_chunks(int N, int chunk);
cudaError_t launch_residual(const DevPlan& p, const float* f, float* usnap, const float* area,
                            bool have_snap, int chunk, const int* chunk_start, int nchunks,
                            double* part, const int* seg, int nseg, double* out, cudaStream_t s,
                            const int* chunk_case = nullptr, const int* case_take = nullptr);
// packed batch: the fused cell kernel with per-case 1/tau, dt and retirement
// (threads per block 128 or 256; L2 prefetch distance in waves)
cudaError_t launch_fused_batch(const DevPlan& p, const float* fin, float* fout, cudaStream_t s, bool pdl,
                               int block, int prefetch_waves);
// cell pdfs = feq(rho, vel) from reference-order device arrays
cudaError_t launch_cells_eq(const DevPlan& p, const float* rho, const float* vel, const int* cell_new, float* f,
                            cudaStream_t s);
// copy device cells [c0, c1) of an AoSoA pdf buffer
cudaError_t launch_copy_cells(const float* src, float* dst, int c0, int c1, cudaStream_t s);
// Counts the float32 dividends x (all 2^32 bit patterns) for which the
// known-divisor division differs from x / y, and the lowest such bit pattern;
// *bad must be zeroed and *example set to 0xFFFFFFFF.
cudaError_t launch_cdiv_check(float y, float zr, float zl, int two, unsigned long long* bad, unsigned* example,
                              cudaStream_t s);
// [N][q] reference order <-> AoSoA device order (cell_new: reference -> device)
cudaError_t launch_scatter_cells(const float* src_aos, float* dst, const int* cell_new, int N,
                                 cudaStream_t s, int q = Q);
cudaError_t launch_gather_cells(const float* src, float* dst_aos, const int* cell_new, int N,
                                cudaStream_t s, int q = Q);
// the bounded-wait self-test (fvdbm_wait_selftest)
cudaError_t launch_wait_selftest(const int* flag, int iters, int* status, cudaStream_t s);
cudaError_t launch_pack_rows(const float* f, const int* cell_new, const int* idx, int n, float* buf,
                             cudaStream_t s, int q);
cudaError_t launch_unpack_rows(float* f, const int* cell_new, const int* idx, int n, const float* buf,
                               cudaStream_t s, int q);
// the scatter reading page-locked host memory directly (src 16-byte aligned)
cudaError_t launch_host_to_cells(const float* src_host, float* dst, const int* cell_new, int N,
                                 cudaStream_t s, int q = Q);
// D2Q9 rho [N] and vel [N][2] of a pdf buffer in reference order (either
// may be null; both may be page-locked host memory)
// grid_cap: at most two blocks per SM, looping over the cells
cudaError_t launch_macros_ref(const DevPlan& p, const float* f, const int* cell_new, float* rho, float* vel,
                              cudaStream_t s, bool grid_cap = false);
// D2Q13 (d2q13.cu): the staged step, the face fluxes alone, read-back macros
cudaError_t launch13_step(const DevPlan& p, const float* fin, float* flux, float* fout, cudaStream_t s);
cudaError_t launch13_face_flux(const DevPlan& p, const float* f, float* flux, cudaStream_t s);
// D2Q13 fused family (triangles): the node kernel, then one cell kernel;
// and the two halves separately (step phases)
cudaError_t launch13_fused(const DevPlan& p, const float* fin, float* fout, cudaStream_t s);
cudaError_t launch13_nodes(const DevPlan& p, const float* fin, cudaStream_t s);
cudaError_t launch13_cells(const DevPlan& p, const float* fin, float* fout, cudaStream_t s);
cudaError_t launch13_macros(const DevPlan& p, const float* f, float* rho, float* vel, float* feq,
                            cudaStream_t s);
// SoA [rows][Np] device order -> [N][rows] reference order
cudaError_t launch_soa_to_aos(const float* src, float* dst, const int* cell_new, int N, int Np,
                              int rows, cudaStream_t s);

}  // namespace fvdbm
