// C ABI of libfvdbm (declared in include/fvdbm.h).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/fvdbm.h"
#include "fvdbm_internal.h"

namespace fvdbm {

namespace {

std::mutex g_err_mu;
std::string g_create_err;

constexpr int kGraphSteps = 32;  // steps per captured graph (even)

struct Handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  HostPlan hp;
  DevPlan dp{};
  fvdbm_params_t params{};
  std::vector<void*> allocs;
  double device_bytes = 0;
  float* f[2] = {nullptr, nullptr};
  int cur = 0;
  float* flux = nullptr;
  float* stage = nullptr;  // [N][9] staging (reference order)
  int* d_cell_new = nullptr;
  float* mac = nullptr;  // rho [Np], vel [2][Np], feq [9][Np]
  long long steps_done = 0;
  bool fused = false;
  bool tile = false;
  bool one = false;  // node and cell blocks in one launch
  bool persist = false;  // FVDBM_KERNEL_PERSIST: one cooperative launch per fvdbm_step call
  int* bar = nullptr;    // its grid-barrier counter
  // packed batch of independent cases (fvdbm_batch_create)
  bool batch = false;
  int batch_block = 256, batch_waves = 1;
  std::vector<int> active;          // per case, host copy of case_active
  std::vector<long long> case_steps; // steps each case has taken
  int* d_active = nullptr;
  int* d_chunk_start = nullptr;  // residual chunks inside the case ranges
  int* d_case_chunk = nullptr;   // first chunk of each case
  int* d_chunk_case = nullptr;   // case of each chunk
  int* d_case_take = nullptr;    // [S] cases whose residual a check takes
  std::vector<long long> case_snap;  // case_steps at each case's snapshot, -1 = none
  bool usnap_init = false;           // every case's snapshot was written once
  int n_chunks = 0;
  std::vector<float> case_dt_host;
  int* d_blk = nullptr;  // active cell blocks of the batch launch
  std::vector<int> blk_host;
  bool blk_valid = false;
  double* bred = nullptr;  // batch residual partials, then 4 totals per case
  int* status = nullptr;
  std::vector<float> node_pdf, node_rho, node_vel;  // reference-order host truth
  cudaGraphExec_t graph[4] = {nullptr, nullptr, nullptr, nullptr};  // [cur + 2 * node_cur]
  // in-kernel node update (FVDBM_KERNEL_FUSED_NODES): two node buffers; the
  // next step reads buffer node_cur and its kernel writes node_cur ^ 1;
  // node_last holds the node state of the last step (or the upload)
  bool fnodes = false;
  float* nbuf[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
  int node_cur = 0, node_last = 1;
  bool nodes_ready = false;
  // convergence monitor (fvdbm_residual)
  float* usnap = nullptr;   // [2][Np] velocity at the previous residual call
  double* red = nullptr;    // chunk partials, then the 4 totals
  float* d_area = nullptr;  // [Np] cell areas (mass weights) or null
  long long snap_step = -1; // steps_done at the snapshot, -1 = none
  // read-back beside the step: rho/vel of the last step's input buffer do not
  // depend on the step, so fvdbm_get_cells computes them on a side stream that
  // waits only for in_ready, recorded just before a single fvdbm_step(h, 1);
  // in_ok is cleared by every call that enqueues other work on the state
  cudaStream_t side = nullptr;  // highest priority: its blocks take SM slots as the step's retire
  cudaEvent_t in_ready = nullptr;
  bool in_ok = false;
  int* status_host = nullptr;  // page-locked copy of *status, filled on the stream before a sync
  int* d_rows = nullptr;       // [N] cell indices of a halo pack/unpack
  std::string err;
};

constexpr int kResidualChunk = 1024;  // cells per partial sum of the monitor

// Known-divisor division (see cdiv in kernels.cu) is used only for divisors
// whose exhaustive check on this device found no dividend that it rounds
// differently from IEEE division; results are cached per device and divisor.
std::mutex g_cdiv_mu;
std::map<std::pair<int, uint32_t>, std::pair<bool, bool>> g_cdiv_ok;  // (five-op ok, two-op ok)

// zl = RN(1/y - RN(1/y)): 1/y in double carries 53 bits, the difference is
// exact in double, and its float rounding is the low word.
float cdiv_low(float y, float zr) { return float(1.0 / double(y) - double(zr)); }

cudaError_t run_cdiv_check(float y, float zr, float zl, int two, cudaStream_t s, unsigned long long* bad,
                           unsigned* example) {
  unsigned long long* d_bad = nullptr;
  unsigned* d_ex = nullptr;
  cudaError_t e = cudaMalloc(&d_bad, sizeof(unsigned long long));
  if (e != cudaSuccess) return e;
  e = cudaMalloc(&d_ex, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0, sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_ex, 0xFF, sizeof(unsigned), s);
  if (e == cudaSuccess) e = launch_cdiv_check(y, zr, zl, two, d_bad, d_ex, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(bad, d_bad, sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(example, d_ex, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(d_bad);
  if (d_ex) cudaFree(d_ex);
  return e;
}

cudaError_t make_cdiv(int device, float y, cudaStream_t s, CDiv* out) {
  const float zr = 1.0f / y;
  out->y = y;
  out->zr = zr;
  out->zl = 0.0f;
  out->ok = 0;
  out->two = 0;
  uint32_t bits;
  std::memcpy(&bits, &y, 4);
  const auto key = std::make_pair(device, bits);
  if (!(std::fabs(y) > 0.0f) || !std::isfinite(y) || !std::isfinite(zr)) return cudaSuccess;
  out->zl = cdiv_low(y, zr);
  {
    std::lock_guard<std::mutex> lk(g_cdiv_mu);
    auto it = g_cdiv_ok.find(key);
    if (it != g_cdiv_ok.end()) {
      out->ok = it->second.first ? 1 : 0;
      out->two = it->second.second ? 1 : 0;
      return cudaSuccess;
    }
  }
  unsigned long long bad = ~0ull, bad2 = ~0ull;
  unsigned example = 0;
  cudaError_t e = run_cdiv_check(y, zr, out->zl, 0, s, &bad, &example);
  if (e == cudaSuccess && bad == 0 && std::isfinite(out->zl)) e = run_cdiv_check(y, zr, out->zl, 1, s, &bad2, &example);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(g_cdiv_mu);
  g_cdiv_ok[key] = std::make_pair(bad == 0, bad == 0 && bad2 == 0);
  out->ok = (bad == 0) ? 1 : 0;
  out->two = (bad == 0 && bad2 == 0) ? 1 : 0;
  return cudaSuccess;
}

// Device address of host memory the device reads and writes directly
// (page-locked memory known to CUDA), or null for any other pointer.
void* host_mapped(const void* ptr) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return (a.type == cudaMemoryTypeHost && a.devicePointer) ? a.devicePointer : nullptr;
}

int fail(Handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

#define CK(call)                                                                      \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      return fail(h, FVDBM_ECUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <class T>
int dalloc(Handle* h, T** out, size_t n, const std::vector<T>* init = nullptr) {
  *out = nullptr;
  if (n == 0) n = 1;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, n * sizeof(T));
  if (e != cudaSuccess) return fail(h, FVDBM_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  h->allocs.push_back(p);
  h->device_bytes += double(n * sizeof(T));
  *out = static_cast<T*>(p);
  if (init && !init->empty()) {
    e = cudaMemcpyAsync(p, init->data(), init->size() * sizeof(T), cudaMemcpyHostToDevice, h->stream);
    if (e != cudaSuccess) return fail(h, FVDBM_ECUDA, std::string("upload: ") + cudaGetErrorString(e));
  }
  return FVDBM_OK;
}

#define DA(ptr, n, init)                                  \
  do {                                                    \
    int rc_ = dalloc(h, &(ptr), (n), (init));             \
    if (rc_ != FVDBM_OK) return rc_;                      \
  } while (0)

int upload_nodes(Handle* h) {
  const HostPlan& hp = h->hp;
  if (hp.M == 0) return FVDBM_OK;
  const int Qh = hp.q;
  std::vector<float> pdf(size_t(Qh) * hp.Mp, 0.0f), rho(hp.Mp, 0.0f), vel(size_t(2) * hp.Mp, 0.0f);
  for (int d = 0; d < hp.M; ++d) {
    const int p = hp.node_orig[d];
    for (int q = 0; q < Qh; ++q) pdf[size_t(q) * hp.Mp + d] = h->node_pdf[size_t(p) * Qh + q];
    rho[d] = h->node_rho[p];
    vel[d] = h->node_vel[size_t(p) * 2];
    vel[hp.Mp + d] = h->node_vel[size_t(p) * 2 + 1];
  }
  CK(cudaMemcpyAsync(h->dp.node_pdf, pdf.data(), pdf.size() * 4, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->dp.node_rho, rho.data(), rho.size() * 4, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->dp.node_vel, vel.data(), vel.size() * 4, cudaMemcpyHostToDevice, h->stream));
  if (h->fnodes) {
    // both buffers hold the upload (and the set values of the computed nodes)
    for (int b = 0; b < 2; ++b) {
      CK(cudaMemcpyAsync(h->nbuf[b][0], pdf.data(), pdf.size() * 4, cudaMemcpyHostToDevice, h->stream));
      CK(cudaMemcpyAsync(h->nbuf[b][1], rho.data(), rho.size() * 4, cudaMemcpyHostToDevice, h->stream));
      CK(cudaMemcpyAsync(h->nbuf[b][2], vel.data(), vel.size() * 4, cudaMemcpyHostToDevice, h->stream));
    }
    h->nodes_ready = false;
    h->node_last = h->node_cur ^ 1;
  }
  // pageable sources: make sure the copies finished before the vectors die
  CK(cudaStreamSynchronize(h->stream));
  return FVDBM_OK;
}

// Back-to-back steps use programmatic dependent launch between the node and
// cell kernels (each waits for its predecessor before reading its output);
// the first launch of a call follows whatever preceded it in the stream.
// The plan with the node pointers of buffer a (read) and b (written).
DevPlan with_nodes(const Handle* h, int a, int b) {
  DevPlan q = h->dp;
  q.node_pdf = h->nbuf[a][0];
  q.node_rho = h->nbuf[a][1];
  q.node_vel = h->nbuf[a][2];
  q.node_pdf_nx = h->nbuf[b][0];
  q.node_rho_nx = h->nbuf[b][1];
  q.node_vel_nx = h->nbuf[b][2];
  return q;
}

// In-kernel node update: the boundary nodes of the next step, computed once
// from the recorded stencil macros after an upload (the step kernels then
// keep them current).
int ensure_nodes(Handle* h) {
  if (!h->fnodes || h->nodes_ready) return FVDBM_OK;
  CK(launch_nodes_cp(with_nodes(h, h->node_cur, h->node_cur), h->f[h->cur], h->stream, false));
  h->nodes_ready = true;
  return FVDBM_OK;
}

constexpr int kPersistSteps = 4096;  // steps per cooperative launch, at most

int enqueue_steps(Handle* h, int n) {
  if (h->persist) {
    for (int done = 0; done < n;) {
      const int k = std::min(n - done, kPersistSteps);
      CK(launch_persist(h->dp, h->f[h->cur], h->f[h->cur ^ 1], k, h->bar, h->stream));
      if (k & 1) h->cur ^= 1;
      done += k;
    }
    return FVDBM_OK;
  }
  if (h->fnodes) {
    int rc = ensure_nodes(h);
    if (rc != FVDBM_OK) return rc;
  }
  for (int s = 0; s < n; ++s) {
    const float* fin = h->f[h->cur];
    float* fout = h->f[h->cur ^ 1];
    if (h->hp.q == 13) {
      if (h->fused)
        CK(launch13_fused(h->dp, fin, fout, h->stream));
      else
        CK(launch13_step(h->dp, fin, h->flux, fout, h->stream));
    } else if (h->fnodes) {
      CK(launch_fused_nodes(with_nodes(h, h->node_cur, h->node_cur ^ 1), fin, fout, h->stream, /*pdl=*/true));
      h->node_last = h->node_cur;
      h->node_cur ^= 1;
    } else if (h->batch) {
      CK(launch_nodes(h->dp, fin, h->stream, /*pdl=*/s > 0));
      CK(launch_fused_batch(h->dp, fin, fout, h->stream, /*pdl=*/h->dp.NB > 0 || s > 0, h->batch_block,
                            h->batch_waves));
    } else if (h->one) {
      CK(launch_step(h->dp, fin, fout, h->stream, /*pdl=*/s > 0));
    } else if (h->tile) {
      if (!h->dp.tile_nodes) CK(launch_nodes(h->dp, fin, h->stream));
      CK(launch_tile(h->dp, fin, fout, h->stream));
    } else {
      if (h->fused)
        CK(launch_nodes_cp(h->dp, fin, h->stream, /*pdl=*/s > 0));
      else
        CK(launch_nodes(h->dp, fin, h->stream, /*pdl=*/s > 0));
      if (h->fused) {
        CK(launch_fused(h->dp, fin, fout, h->stream, /*pdl=*/h->dp.NB > 0 || s > 0));
      } else {
        CK(launch_face_flux(h->dp, fin, h->flux, h->stream));
        CK(launch_gather(h->dp, fin, h->flux, fout, h->stream));
      }
    }
    h->cur ^= 1;
  }
  return FVDBM_OK;
}

std::string status_message(int st) {
  return "device status " + std::to_string(st) +
         ": a bounded wait in a step kernel (tile kernel, or node blocks of a single-launch step) gave up";
}

int check_status(Handle* h) {
  int st = 0;
  CK(cudaMemcpy(&st, h->status, sizeof(int), cudaMemcpyDeviceToHost));
  if (st != 0) return fail(h, FVDBM_EDEVICE, status_message(st));
  return FVDBM_OK;
}

// check_status without a second round trip: the status word is copied on
// the stream before the synchronisation the caller needs anyway.
int sync_and_check(Handle* h) {
  CK(cudaMemcpyAsync(h->status_host, h->status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  if (*h->status_host != 0) return fail(h, FVDBM_EDEVICE, status_message(*h->status_host));
  return FVDBM_OK;
}

int get_graph(Handle* h, int parity, cudaGraphExec_t* out) {
  parity += 2 * (h->fnodes ? h->node_cur : 0);
  if (h->graph[parity]) {
    *out = h->graph[parity];
    return FVDBM_OK;
  }
  const int save = h->cur, save_nc = h->node_cur, save_nl = h->node_last;
  cudaGraph_t g = nullptr;
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_steps(h, kGraphSteps);
  cudaError_t e = cudaStreamEndCapture(h->stream, &g);
  h->cur = save;
  h->node_cur = save_nc;
  h->node_last = save_nl;
  if (rc != FVDBM_OK) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return fail(h, FVDBM_ECUDA, std::string("capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&h->graph[parity], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(h, FVDBM_ECUDA, std::string("instantiate: ") + cudaGetErrorString(e));
  *out = h->graph[parity];
  return FVDBM_OK;
}

// Cell blocks (of the batch launch's block size) holding cells of active
// cases; the launch covers only those.  The grid size changes, so captured
// graphs are dropped.
int update_batch_blocks(Handle* h) {
  const HostPlan& hp = h->hp;
  const int T = h->batch_block;
  std::vector<int> list;
  for (int s = 0; s < hp.S; ++s) {
    if (!h->active[s]) continue;
    const int b0 = hp.case_cell[s] / T, b1 = (hp.case_cell[s + 1] - 1) / T;
    for (int b = std::max(b0, list.empty() ? 0 : list.back() + 1); b <= b1; ++b) list.push_back(b);
  }
  if (h->blk_valid && list == h->blk_host) return FVDBM_OK;
  if (!list.empty())
    CK(cudaMemcpyAsync(h->d_blk, list.data(), list.size() * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->dp.blk_list = h->d_blk;
  h->dp.n_blk = int(list.size());
  h->blk_host = list;
  h->blk_valid = true;
  for (auto& g : h->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  return FVDBM_OK;
}

}  // namespace
}  // namespace fvdbm

using namespace fvdbm;

extern "C" {

int fvdbm_abi_version(void) { return FVDBM_ABI_VERSION; }

const char* fvdbm_last_error(void* handle) {
  if (!handle) {
    std::lock_guard<std::mutex> lk(g_err_mu);
    return g_create_err.c_str();
  }
  return static_cast<Handle*>(handle)->err.c_str();
}

int fvdbm_destroy(void* handle) {
  if (!handle) return FVDBM_OK;
  Handle* h = static_cast<Handle*>(handle);
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (auto& g : h->graph)
    if (g) cudaGraphExecDestroy(g);
  for (void* p : h->allocs) cudaFree(p);
  if (h->side) cudaStreamSynchronize(h->side);
  if (h->status_host) cudaFreeHost(h->status_host);
  if (h->in_ready) cudaEventDestroy(h->in_ready);
  if (h->side) cudaStreamDestroy(h->side);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return FVDBM_OK;
}

static int create_impl(const fvdbm_mesh_t* mesh, const fvdbm_params_t* params, const BatchSegs* segs,
                       const float* case_inv_tau, const float* case_dt, void** handle) {
  auto create_fail = [&](Handle* h, int code) {
    {
      std::lock_guard<std::mutex> lk(g_err_mu);
      g_create_err = h ? h->err : "invalid arguments";
    }
    if (h) fvdbm_destroy(h);
    return code;
  };
  if (!mesh || !params || !handle) return create_fail(nullptr, FVDBM_EINVAL);
  *handle = nullptr;
  Handle* h = new Handle();
  h->params = *params;
  h->device = params->device;
  // AUTO: the fused kernels when the mesh allows them, else the staged ones.
  // From 2^18 cells on, the single-launch step (node update inside the cell
  // kernel; measured 29.6 against 34.8 us per step at 1M cells); below, the
  // two-launch step, whose short launches do not wait inside (8.7 against
  // 9.9 us at 3.2k cells, 10.0 against 11.5 us at 60k)
  const bool auto_family = params->kernel == FVDBM_KERNEL_AUTO && !segs;
  fvdbm_params_t pplan = *params;
  if (auto_family && mesh->n_cells >= (1 << 18)) pplan.kernel = FVDBM_KERNEL_FUSED_NODES;
  std::string why = build_plan(mesh, &pplan, h->hp, segs);
  if (!why.empty()) {
    h->err = why;
    return create_fail(h, FVDBM_EINVAL);
  }
  int rc;
#define CR(call)                                                                   \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess) {                                                       \
      h->err = std::string(#call) + ": " + cudaGetErrorString(e_);                 \
      return create_fail(h, FVDBM_ECUDA);                                          \
    }                                                                              \
  } while (0)
  CR(cudaSetDevice(h->device));
  CR(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  {
    int lo = 0, hi = 0;
    CR(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    CR(cudaStreamCreateWithPriority(&h->side, cudaStreamNonBlocking, hi));
  }
  CR(cudaHostAlloc(reinterpret_cast<void**>(&h->status_host), sizeof(int), cudaHostAllocDefault));
  CR(cudaEventCreateWithFlags(&h->in_ready, cudaEventDisableTiming));
  const HostPlan& hp = h->hp;
  DevPlan& p = h->dp;
  // the fused kernels take three face slots per cell (triangles)
  h->fused = hp.fusable && hp.K == 3 && params->kernel != FVDBM_KERNEL_STAGED;
  const bool want_fnodes = params->kernel == FVDBM_KERNEL_FUSED_NODES || params->kernel == FVDBM_KERNEL_FAST;
  if (want_fnodes && !(hp.fusable && hp.K == 3 && hp.stencil_first)) {
    h->err = "the in-kernel node update needs triangles (3 face slots per cell), every cell face slot "
             "naming a face of that cell, and no per-q flux scale";
    return create_fail(h, FVDBM_EINVAL);
  }
  h->fnodes = want_fnodes ||
              (auto_family && pplan.kernel == FVDBM_KERNEL_FUSED_NODES && hp.fusable && hp.K == 3 && hp.stencil_first);
  if (hp.q == 13) {
    // D2Q13 (d2q13.cu): the staged kernels, or on triangles the node kernel
    // and one fused cell kernel
    if (segs || (params->kernel != FVDBM_KERNEL_AUTO && params->kernel != FVDBM_KERNEL_STAGED &&
                 params->kernel != FVDBM_KERNEL_FUSED)) {
      h->err = "D2Q13 runs on the staged or fused kernels (FVDBM_KERNEL_AUTO, FVDBM_KERNEL_STAGED or "
               "FVDBM_KERNEL_FUSED), not in a batch";
      return create_fail(h, FVDBM_EINVAL);
    }
    h->fnodes = false;
  }
  const bool want_tile = params->kernel == FVDBM_KERNEL_TILE || params->kernel == FVDBM_KERNEL_TILE_SPLIT;
  if ((params->kernel == FVDBM_KERNEL_FUSED || want_tile) && !(hp.fusable && hp.K == 3)) {
    h->err = "the fused kernels need triangles (3 face slots per cell), every cell face slot naming a "
             "face of that cell, and no per-q flux scale";
    return create_fail(h, FVDBM_EINVAL);
  }
  const bool tile_possible = hp.fusable && hp.K == 3 && hp.N > 0 &&
                             (params->kernel != FVDBM_KERNEL_TILE || hp.tile_ok);
  if (want_tile && !tile_possible) {
    h->err = "the tile kernel needs triangles (3 face slots per cell) and at most " +
             std::to_string(TILE_MAX_NODES) + " boundary nodes / " + std::to_string(TILE_MAX_ENTRIES) +
             " node-stencil cells per tile of " + std::to_string(TILE) + " cells";
    return create_fail(h, FVDBM_EINVAL);
  }
  h->tile = tile_possible && want_tile;
  const bool one_possible = hp.fusable && hp.K == 3 && hp.N > 0;
  if (params->kernel == FVDBM_KERNEL_ONE && !one_possible) {
    h->err = "the single-launch step needs triangles (3 face slots per cell), every cell face slot "
             "naming a face of that cell, and no per-q flux scale";
    return create_fail(h, FVDBM_EINVAL);
  }
  h->one = one_possible && params->kernel == FVDBM_KERNEL_ONE;
  if (params->kernel == FVDBM_KERNEL_PERSIST && !(hp.fusable && hp.K == 3 && hp.N > 0 && hp.q == 9 && !segs)) {
    h->err = "the persistent step needs D2Q9 triangles (3 face slots per cell), every cell face slot "
             "naming a face of that cell, and no per-q flux scale";
    return create_fail(h, FVDBM_EINVAL);
  }
  h->persist = params->kernel == FVDBM_KERNEL_PERSIST;
  if (hp.q == 13) h->tile = h->one = false;
  if (segs) {
    if (!(hp.fusable && hp.K == 3)) {
      h->err = "a batch needs triangles (3 face slots per cell), every cell face slot naming a face of "
               "that cell, and no per-q flux scale";
      return create_fail(h, FVDBM_EINVAL);
    }
    h->batch = true;
    h->fused = h->tile = h->one = false;
  }
  h->dp.tile_nodes = (params->kernel == FVDBM_KERNEL_TILE) ? 1 : 0;
  p.N = hp.N;
  p.Np = hp.Np;
  p.F = hp.F;
  p.Fp = hp.Fp;
  p.K = hp.K;
  p.M = hp.M;
  p.Mp = hp.Mp;
  p.Mc = hp.Mc;
  p.scheme = hp.scheme;
  p.variant = hp.variant;
  p.fv = hp.fv ? 1 : 0;
  p.last_cell = hp.last_cell_new;
  p.inv_tau = params->inv_tau;
  p.dt = params->delta_t;
  p.c2 = params->c2;
  p.c4x2 = params->c4x2;
  p.c2x2 = params->c2x2;
  p.c6x2 = params->c6x2;
  p.one = 1.0f;
  p.neg_one = -1.0f;
  p.q = hp.q;
  p.finite_n = hp.finite_n ? 1 : 0;
  CR(make_cdiv(h->device, p.c2, h->stream, &p.d_c2));
  CR(make_cdiv(h->device, p.c4x2, h->stream, &p.d_c4x2));
  CR(make_cdiv(h->device, p.c2x2, h->stream, &p.d_c2x2));
  if (hp.q == 13) {
    CR(make_cdiv(h->device, p.c6x2, h->stream, &p.d_c6x2));
  } else {
    p.d_c6x2 = p.d_c2x2;  // (unused by D2Q9; keeps the conditions below uniform)
  }
  p.fast = hp.fast ? 1 : 0;
  p.cdiv_mode = (p.d_c2.ok && p.d_c4x2.ok && p.d_c2x2.ok && p.d_c6x2.ok)
                    ? ((p.d_c2.two && p.d_c4x2.two && p.d_c2x2.two && p.d_c6x2.two) ? 2 : 1)
                    : 0;

#define UP(field, vec)                                                        \
  do {                                                                        \
    decltype(vec)::value_type* d_ = nullptr;                                  \
    if ((rc = dalloc(h, &d_, (vec).size(), &(vec))) != FVDBM_OK)              \
      return create_fail(h, rc);                                              \
    p.field = d_;                                                             \
  } while (0)
  UP(fs0, hp.fs0);
  UP(fs1, hp.fs1);
  UP(fnx, hp.fnx);
  UP(fny, hp.fny);
  UP(fL, hp.fL);
  UP(fr, hp.fr);
  UP(fD2, hp.fD2);
  UP(fna, hp.fna);
  UP(fnb, hp.fnb);
  UP(frl, hp.frl);
  UP(frr, hp.frr);
  UP(fkl, hp.fkl);
  UP(fkr, hp.fkr);
  UP(fscale, hp.fscale);
  UP(cf_face, hp.cf_face);
  UP(cf_sign, hp.cf_sign);
  p.hrows = hp.hrows;
  if (h->fused || h->batch) {
    UP(hf, hp.hf);
    UP(gh_a, hp.gh_a);
    UP(gh_b, hp.gh_b);
    UP(gh_r, hp.gh_r);
  }
  UP(nd_type, hp.nd_type);
  UP(nd_ptr, hp.nd_ptr);
  UP(nd_npad, hp.nd_npad);
  UP(nd_cell, hp.nd_cell);
  UP(nd_w, hp.nd_w);
  UP(nd_sumw, hp.nd_sumw);
  UP(nb_meta, hp.nb_meta);
  p.NB = int(hp.nb_meta.size() / 4);
  UP(pe_slot, hp.pe_slot);
  UP(pe_w, hp.pe_w);
  UP(pn_meta, hp.pn_meta);
  UP(pn_sumw, hp.pn_sumw);
  p.stencil_start = hp.stencil_start;
  p.stencil_end = hp.stencil_end;
  p.stencil_first = hp.stencil_first ? 1 : 0;
  p.last_slot = hp.last_slot;
  p.Sp = std::max(32, (hp.stencil_end - hp.stencil_start + 31) / 32 * 32);
  {
    float* d = nullptr;
    if ((rc = dalloc<float>(h, &d, size_t(12) * p.Sp)) != FVDBM_OK) return create_fail(h, rc);
    p.cprod = d;
  }
  UP(inv_area, hp.inv_area);
  p.NT = hp.NT;
  if (h->tile) {
    UP(tn_ptr, hp.tn_ptr);
    UP(tn_dev, hp.tn_dev);
    UP(tn_kind, hp.tn_kind);
    UP(tn_npad, hp.tn_npad);
    UP(tn_e0, hp.tn_e0);
    UP(tn_ecnt, hp.tn_ecnt);
    UP(tn_sumw, hp.tn_sumw);
    UP(te_ptr, hp.te_ptr);
    UP(te_cell, hp.te_cell);
    UP(te_w, hp.te_w);
    UP(tgh_a, hp.tgh_a);
    UP(tgh_b, hp.tgh_b);
  }
  if ((rc = dalloc<int>(h, &h->status, 4)) != FVDBM_OK) return create_fail(h, rc);
  if (h->persist && (rc = dalloc<int>(h, &h->bar, 1)) != FVDBM_OK) return create_fail(h, rc);
  CR(cudaMemsetAsync(h->status, 0, 4 * sizeof(int), h->stream));
  p.status = h->status;
  p.step_ctr = h->status + 1;
  if (h->fused) {
    UP(cblk_ghost, hp.cblk_ghost);
    UP(sched, hp.sched);
  }
  if (h->tile) CR(prepare_tile(p));
  if (!hp.area.empty())
    if ((rc = dalloc(h, &h->d_area, hp.area.size(), &hp.area)) != FVDBM_OK) return create_fail(h, rc);
  {
    float* d = nullptr;
    if ((rc = dalloc<float>(h, &d, size_t(hp.q) * hp.Mp)) != FVDBM_OK) return create_fail(h, rc);
    p.node_pdf = d;
    if ((rc = dalloc<float>(h, &d, hp.Mp)) != FVDBM_OK) return create_fail(h, rc);
    p.node_rho = d;
    if ((rc = dalloc<float>(h, &d, size_t(2) * hp.Mp)) != FVDBM_OK) return create_fail(h, rc);
    p.node_vel = d;
    h->nbuf[0][0] = p.node_pdf;
    h->nbuf[0][1] = p.node_rho;
    h->nbuf[0][2] = p.node_vel;
    if (h->fnodes) {
      const size_t sz[3] = {size_t(hp.q) * hp.Mp, size_t(hp.Mp), size_t(2) * hp.Mp};
      for (int k = 0; k < 3; ++k)
        if ((rc = dalloc<float>(h, &h->nbuf[1][k], sz[k])) != FVDBM_OK) return create_fail(h, rc);
    }
  }
  for (int b = 0; b < 2; ++b) {
    if ((rc = dalloc<float>(h, &h->f[b], size_t(hp.q) * hp.Np)) != FVDBM_OK) return create_fail(h, rc);
    CR(cudaMemsetAsync(h->f[b], 0, size_t(hp.q) * hp.Np * 4, h->stream));
  }
  if (!h->fused && !h->batch)
    if ((rc = dalloc<float>(h, &h->flux, size_t(hp.q) * hp.Fp)) != FVDBM_OK) return create_fail(h, rc);
  if (h->batch) {
    const std::vector<float> it(case_inv_tau, case_inv_tau + hp.S), dt(case_dt, case_dt + hp.S);
    h->case_dt_host = dt;
    h->active.assign(hp.S, 1);
    h->case_steps.assign(hp.S, 0);
    UP(cell_case, hp.cell_case);
    UP(case_inv_tau, it);
    UP(case_dt, dt);
    if ((rc = dalloc(h, &h->d_active, h->active.size(), &h->active)) != FVDBM_OK) return create_fail(h, rc);
    p.case_active = h->d_active;
    if ((rc = dalloc<int>(h, &h->d_blk, size_t(hp.N + 127) / 128)) != FVDBM_OK) return create_fail(h, rc);
    if ((rc = update_batch_blocks(h)) != FVDBM_OK) return create_fail(h, rc);
    // residual chunks of at most kResidualChunk cells inside each case
    std::vector<int> cs, cc;
    for (int s = 0; s < hp.S; ++s) {
      cc.push_back(int(cs.size()));
      for (int c = hp.case_cell[s]; c < hp.case_cell[s + 1]; c += kResidualChunk) cs.push_back(c);
    }
    cc.push_back(int(cs.size()));
    h->n_chunks = int(cs.size());
    cs.push_back(hp.N);
    if ((rc = dalloc(h, &h->d_chunk_start, cs.size(), &cs)) != FVDBM_OK) return create_fail(h, rc);
    if ((rc = dalloc(h, &h->d_case_chunk, cc.size(), &cc)) != FVDBM_OK) return create_fail(h, rc);
    std::vector<int> chc(h->n_chunks);
    for (int s = 0; s < hp.S; ++s)
      for (int k = cc[s]; k < cc[s + 1]; ++k) chc[k] = s;
    if ((rc = dalloc(h, &h->d_chunk_case, chc.size(), &chc)) != FVDBM_OK) return create_fail(h, rc);
    if ((rc = dalloc<int>(h, &h->d_case_take, size_t(hp.S))) != FVDBM_OK) return create_fail(h, rc);
    h->case_snap.assign(hp.S, -1);
  }
  if ((rc = dalloc<float>(h, &h->stage, size_t(hp.q) * std::max(hp.N, hp.F))) != FVDBM_OK)
    return create_fail(h, rc);
  if ((rc = dalloc(h, &h->d_cell_new, hp.cell_new.size(), &hp.cell_new)) != FVDBM_OK)
    return create_fail(h, rc);

  // rest state: every pdf = feq(1, 0) = W (src/containers.py:29)
  // (D2Q13: src/dynamics.py:96)
  const float W9[9] = {(float)(4.0 / 9.0),  (float)(1.0 / 9.0),  (float)(1.0 / 9.0),
                       (float)(1.0 / 9.0),  (float)(1.0 / 9.0),  (float)(1.0 / 36.0),
                       (float)(1.0 / 36.0), (float)(1.0 / 36.0), (float)(1.0 / 36.0)};
  const float W13[13] = {(float)(3.0 / 8.0),  (float)(1.0 / 12.0), (float)(1.0 / 12.0), (float)(1.0 / 12.0),
                         (float)(1.0 / 12.0), (float)(1.0 / 16.0), (float)(1.0 / 16.0), (float)(1.0 / 16.0),
                         (float)(1.0 / 16.0), (float)(1.0 / 96.0), (float)(1.0 / 96.0), (float)(1.0 / 96.0),
                         (float)(1.0 / 96.0)};
  const float* W = hp.q == 13 ? W13 : W9;
  const int Qh = hp.q;
  h->node_pdf.resize(size_t(Qh) * hp.P);
  for (int pp = 0; pp < hp.P; ++pp)
    for (int q = 0; q < Qh; ++q) h->node_pdf[size_t(pp) * Qh + q] = W[q];
  h->node_rho.assign(hp.P, 0.0f);
  h->node_vel.assign(size_t(2) * hp.P, 0.0f);
  if ((rc = upload_nodes(h)) != FVDBM_OK) return create_fail(h, rc);
  {
    std::vector<float> cells(size_t(Qh) * hp.N);
    for (int c = 0; c < hp.N; ++c)
      for (int q = 0; q < Qh; ++q) cells[size_t(c) * Qh + q] = W[q];
    if ((rc = fvdbm_set_state(h, cells.data(), nullptr, nullptr, nullptr)) != FVDBM_OK)
      return create_fail(h, rc);
  }
  CR(cudaStreamSynchronize(h->stream));
  *handle = h;
  return FVDBM_OK;
#undef CR
#undef UP
}

int fvdbm_create(const fvdbm_mesh_t* mesh, const fvdbm_params_t* params, void** handle) {
  return create_impl(mesh, params, nullptr, nullptr, nullptr, handle);
}

int fvdbm_batch_create(const fvdbm_mesh_t* meshes, const fvdbm_params_t* params, int32_t n_cases,
                       void** handle) {
  auto bad = [](const std::string& why) {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_create_err = why;
    return FVDBM_EINVAL;
  };
  if (!meshes || !params || !handle || n_cases <= 0) return bad("invalid arguments");
  *handle = nullptr;
  for (int s = 1; s < n_cases; ++s) {
    const fvdbm_params_t &a = params[0], &b = params[s];
    if (a.flux_scheme != b.flux_scheme || a.variant != b.variant || a.c2 != b.c2 || a.c4x2 != b.c4x2 ||
        a.c2x2 != b.c2x2 || a.ordering != b.ordering || a.device != b.device)
      return bad("batch case " + std::to_string(s) + ": parameters other than inv_tau and delta_t differ");
  }
  if (params[0].variant != FVDBM_VARIANT_NONE) return bad("a batch takes no flux-scale variant");
  UnionMesh u;
  std::string why = build_union(meshes, n_cases, u);
  if (!why.empty()) return bad(why);
  std::vector<float> it(n_cases), dt(n_cases);
  for (int s = 0; s < n_cases; ++s) {
    it[s] = params[s].inv_tau;
    dt[s] = params[s].delta_t;
  }
  fvdbm_params_t p0 = params[0];
  p0.kernel = FVDBM_KERNEL_FUSED;
  return create_impl(&u.mesh, &p0, &u.segs, it.data(), dt.data(), handle);
}

int fvdbm_batch_config(void* handle, int32_t block, int32_t prefetch_waves) {
  if (!handle) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  h->in_ok = false;
  if (!h->batch) return fail(h, FVDBM_EINVAL, "not a batch handle");
  if ((block != 128 && block != 256) || prefetch_waves < 0 || prefetch_waves > 8)
    return fail(h, FVDBM_EINVAL, "block must be 128 or 256 and prefetch_waves 0..8");
  if (block == h->batch_block && prefetch_waves == h->batch_waves) return FVDBM_OK;
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  for (auto& g : h->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  h->batch_block = block;
  h->batch_waves = prefetch_waves;
  h->blk_valid = false;  // rebuild for the new block size
  return update_batch_blocks(h);
}

// Residual and mass of the cases with take[s] != 0 (all when take is null):
// each over the steps that case took since its own snapshot, which is then
// renewed; other cases keep their snapshots (res_u and mass untouched).
static int batch_residual_take(Handle* h, const int32_t* take, double* res_u, double* mass) {
  const HostPlan& hp = h->hp;
  const int S = hp.S;
  CK(cudaSetDevice(h->device));
  int rc;
  if (!h->usnap && (rc = dalloc<float>(h, &h->usnap, size_t(2) * hp.Np)) != FVDBM_OK) return rc;
  if (!h->bred && (rc = dalloc<double>(h, &h->bred, size_t(4) * (h->n_chunks + S))) != FVDBM_OK) return rc;
  std::vector<int> tk(S, 1);
  if (take && h->usnap_init)
    for (int s = 0; s < S; ++s) tk[s] = take[s] ? 1 : 0;
  CK(cudaMemcpyAsync(h->d_case_take, tk.data(), S * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  double* out = h->bred + size_t(4) * h->n_chunks;
  CK(launch_residual(h->dp, h->f[h->cur], h->usnap, h->d_area, h->usnap_init, kResidualChunk, h->d_chunk_start,
                     h->n_chunks, h->bred, h->d_case_chunk, S, out, h->stream, h->d_chunk_case, h->d_case_take));
  std::vector<double> tot(size_t(4) * S);
  CK(cudaMemcpyAsync(tot.data(), out, tot.size() * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));  // (also: tk is read before it goes out of scope)
  if ((rc = check_status(h)) != FVDBM_OK) return rc;
  for (int s = 0; s < S; ++s) {
    if (!tk[s]) continue;
    const double* t = &tot[size_t(4) * s];
    const long long K = h->case_snap[s] >= 0 ? h->case_steps[s] - h->case_snap[s] : 0;
    mass[s] = t[2];
    if (t[3] > 0.0)
      res_u[s] = std::nan("");
    else if (!h->usnap_init || h->case_snap[s] < 0 || K <= 0)
      res_u[s] = HUGE_VAL;
    else
      res_u[s] = std::sqrt(t[0]) / (double(K) * double(h->case_dt_host[s]) * std::max(std::sqrt(t[1]), 1e-30));
    h->case_snap[s] = h->case_steps[s];
  }
  h->usnap_init = true;
  h->snap_step = h->steps_done;
  return FVDBM_OK;
}

int fvdbm_batch_residual(void* handle, double* res_u, double* mass) {
  if (!handle || !res_u || !mass) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  if (!h->batch) return fail(h, FVDBM_EINVAL, "not a batch handle");
  return batch_residual_take(h, nullptr, res_u, mass);
}

int fvdbm_batch_residual_cases(void* handle, const int32_t* take, double* res_u, double* mass) {
  if (!handle || !take || !res_u || !mass) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  if (!h->batch) return fail(h, FVDBM_EINVAL, "not a batch handle");
  return batch_residual_take(h, take, res_u, mass);
}

int fvdbm_batch_set_active(void* handle, const int32_t* active) {
  if (!handle || !active) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  h->in_ok = false;
  if (!h->batch) return fail(h, FVDBM_EINVAL, "not a batch handle");
  const HostPlan& hp = h->hp;
  CK(cudaSetDevice(h->device));
  bool changed = false;
  for (int s = 0; s < hp.S; ++s) {
    const int a = active[s] ? 1 : 0;
    if (a == h->active[s]) continue;
    changed = true;
    // both buffers must hold the final state of a retired case
    if (!a) CK(launch_copy_cells(h->f[h->cur], h->f[h->cur ^ 1], hp.case_cell[s], hp.case_cell[s + 1], h->stream));
    h->active[s] = a;
  }
  if (changed) {
    CK(cudaMemcpyAsync(h->d_active, h->active.data(), h->active.size() * sizeof(int), cudaMemcpyHostToDevice,
                       h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return update_batch_blocks(h);
  }
  return FVDBM_OK;
}

int fvdbm_batch_run_to_steady_time(void* handle, double threshold, int32_t check_every, double check_time,
                                   const int64_t* max_steps, int64_t* steps, double* res_u, int32_t* status) {
  if (!handle || !max_steps || !steps || !res_u || !status) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  h->in_ok = false;
  if (!h->batch) return fail(h, FVDBM_EINVAL, "not a batch handle");
  if (check_every <= 0) return fail(h, FVDBM_EINVAL, "check_every <= 0");
  if (!(check_time >= 0.0)) return fail(h, FVDBM_EINVAL, "check_time must be >= 0");
  const int S = h->hp.S;
  std::vector<int32_t> act(S), since_best(S, 0), take(S, 0);
  std::vector<double> r(S, HUGE_VAL), m(S), best(S, HUGE_VAL), prev(S, HUGE_VAL);
  std::vector<int64_t> window(S, check_every);
  for (int s = 0; s < S; ++s) {
    if (max_steps[s] < 0) return fail(h, FVDBM_EINVAL, "max_steps < 0");
    steps[s] = 0;
    res_u[s] = HUGE_VAL;
    status[s] = FVDBM_CASE_CAPPED;
    act[s] = max_steps[s] > 0;
    // a check covers at least check_time units of the case's own time
    if (check_time > 0.0)
      window[s] = std::max<int64_t>(1, int64_t(std::ceil(check_time / double(h->case_dt_host[s]))));
  }
  int rc = fvdbm_batch_set_active(h, act.data());
  if (rc != FVDBM_OK) return rc;
  if ((rc = batch_residual_take(h, nullptr, r.data(), m.data())) != FVDBM_OK) return rc;  // snapshots
  std::vector<int64_t> since(S, 0);  // steps since the case's snapshot
  for (;;) {
    int64_t n = check_every;
    bool any = false;
    for (int s = 0; s < S; ++s)
      if (act[s]) {
        any = true;
        n = std::min<int64_t>(n, max_steps[s] - steps[s]);
      }
    if (!any) break;
    if ((rc = fvdbm_step(h, int32_t(n))) != FVDBM_OK) return rc;
    bool check = false;
    for (int s = 0; s < S; ++s) {
      take[s] = 0;
      if (!act[s]) continue;
      steps[s] += n;
      since[s] += n;
      if (since[s] >= window[s] || steps[s] >= max_steps[s]) {
        take[s] = 1;
        check = true;
      }
    }
    if (!check) continue;
    if ((rc = batch_residual_take(h, take.data(), r.data(), m.data())) != FVDBM_OK) return rc;
    for (int s = 0; s < S; ++s) {
      if (!take[s]) continue;
      since[s] = 0;
      prev[s] = res_u[s];
      res_u[s] = r[s];
      if (r[s] < best[s]) {
        best[s] = r[s];
        since_best[s] = 0;
      } else {
        ++since_best[s];
      }
      if (std::isnan(r[s])) {
        status[s] = FVDBM_CASE_NONFINITE;
        act[s] = 0;
      } else if (r[s] == 0.0) {
        // an exact float32 fixed point: converged when the case was already
        // within two decades of the threshold, else frozen
        status[s] = prev[s] < 100.0 * threshold ? FVDBM_CASE_CONVERGED : FVDBM_CASE_FROZEN;
        act[s] = 0;
      } else if (r[s] < threshold) {
        status[s] = FVDBM_CASE_CONVERGED;
        act[s] = 0;
      } else if (since_best[s] >= FVDBM_STALL_CHECKS) {
        status[s] = FVDBM_CASE_STALLED;
        act[s] = 0;
      } else if (steps[s] >= max_steps[s]) {
        act[s] = 0;
      }
    }
    if ((rc = fvdbm_batch_set_active(h, act.data())) != FVDBM_OK) return rc;
  }
  return FVDBM_OK;
}

int fvdbm_batch_run_to_steady(void* handle, double threshold, int32_t check_every, const int64_t* max_steps,
                              int64_t* steps, double* res_u, int32_t* status) {
  return fvdbm_batch_run_to_steady_time(handle, threshold, check_every, 0.0, max_steps, steps, res_u, status);
}

int fvdbm_set_state(void* handle, const float* cell_pdf, const float* node_pdf, const float* node_rho,
                    const float* node_vel) {
  if (!handle) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  h->in_ok = false;
  const HostPlan& hp = h->hp;
  CK(cudaSetDevice(h->device));
  bool read_later = false;  // a page-locked source is read by the stream after this returns
  if (cell_pdf && hp.N > 0) {
    const float* mapped = static_cast<const float*>(host_mapped(cell_pdf));
    if (mapped && (reinterpret_cast<uintptr_t>(mapped) & 15) == 0) {
      // one pass over the host link, scattered on arrival
      CK(launch_host_to_cells(mapped, h->f[h->cur], h->d_cell_new, hp.N, h->stream, hp.q));
    } else {
      CK(cudaMemcpyAsync(h->stage, cell_pdf, size_t(hp.q) * hp.N * 4, cudaMemcpyHostToDevice, h->stream));
      CK(launch_scatter_cells(h->stage, h->f[h->cur], h->d_cell_new, hp.N, h->stream, hp.q));
    }
    read_later = mapped != nullptr;
    if (h->fused && hp.q == 9) CK(launch_stencil_macros(h->dp, h->f[h->cur], h->stream));
    // a retired batch case keeps its state in both buffers
    for (size_t s = 0; s < h->active.size(); ++s)
      if (!h->active[s])
        CK(launch_copy_cells(h->f[h->cur], h->f[h->cur ^ 1], hp.case_cell[s], hp.case_cell[s + 1], h->stream));
    h->snap_step = -1;
    if (!h->case_snap.empty()) h->case_snap.assign(h->case_snap.size(), -1);
    h->nodes_ready = false;
  }
  if (node_pdf || node_rho || node_vel) {
    if (node_pdf) std::memcpy(h->node_pdf.data(), node_pdf, size_t(hp.q) * hp.P * 4);
    if (node_rho) std::memcpy(h->node_rho.data(), node_rho, size_t(hp.P) * 4);
    if (node_vel) std::memcpy(h->node_vel.data(), node_vel, size_t(2) * hp.P * 4);
    int rc = upload_nodes(h);
    if (rc != FVDBM_OK) return rc;
  }
  if (read_later) CK(cudaStreamSynchronize(h->stream));  // the caller may reuse its arrays on return
  return FVDBM_OK;
}

// Halo rows of a domain decomposition (fvdbm_pack_cells / fvdbm_unpack_cells):
// checks the cell list and stages it on the device.
static int stage_rows(Handle* h, const int32_t* cells, int32_t n, const void* buf, const char* who) {
  const HostPlan& hp = h->hp;
  if (n < 0 || n > hp.N || (n > 0 && (!cells || !buf)))
    return fail(h, FVDBM_EINVAL, std::string(who) + ": need 0 <= n <= n_cells, a cell list and a buffer");
  if (h->batch) return fail(h, FVDBM_EINVAL, std::string(who) + ": not for batch handles");
  for (int32_t k = 0; k < n; ++k)
    if (cells[k] < 0 || cells[k] >= hp.N)
      return fail(h, FVDBM_EINVAL, std::string(who) + ": cell index " + std::to_string(cells[k]) +
                                       " at position " + std::to_string(k) + " out of range");
  CK(cudaSetDevice(h->device));
  if (n == 0) return FVDBM_OK;
  if (!h->d_rows) {
    int rc = dalloc<int>(h, &h->d_rows, size_t(hp.N));
    if (rc != FVDBM_OK) return rc;
  }
  // pageable source: the copy has finished reading it when the call returns
  CK(cudaMemcpyAsync(h->d_rows, cells, size_t(n) * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  return FVDBM_OK;
}

int fvdbm_pack_cells(void* handle, const int32_t* cells, int32_t n, float* buf) {
  if (!handle) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  h->in_ok = false;
  int rc = stage_rows(h, cells, n, buf, "fvdbm_pack_cells");
  if (rc != FVDBM_OK || n == 0) return rc;
  CK(launch_pack_rows(h->f[h->cur], h->d_cell_new, h->d_rows, n, buf, h->stream, h->hp.q));
  return FVDBM_OK;
}

int fvdbm_unpack_cells(void* handle, const int32_t* cells, int32_t n, const float* buf) {
  if (!handle) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  h->in_ok = false;
  int rc = stage_rows(h, cells, n, buf, "fvdbm_unpack_cells");
  if (rc != FVDBM_OK || n == 0) return rc;
  CK(launch_unpack_rows(h->f[h->cur], h->d_cell_new, h->d_rows, n, buf, h->stream, h->hp.q));
  // an upload of cell pdfs: the node stencils' macros and nodes follow them
  if (h->fused && h->hp.q == 9) CK(launch_stencil_macros(h->dp, h->f[h->cur], h->stream));
  h->snap_step = -1;
    if (!h->case_snap.empty()) h->case_snap.assign(h->case_snap.size(), -1);
  h->nodes_ready = false;
  return FVDBM_OK;
}

int fvdbm_set_cells_eq(void* handle, const float* rho, const float* vel) {
  if (!handle || !rho || !vel) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  h->in_ok = false;
  if (h->hp.q != 9) return fail(h, FVDBM_EINVAL, "fvdbm_set_cells_eq supports D2Q9");
  const HostPlan& hp = h->hp;
  CK(cudaSetDevice(h->device));
  if (hp.N == 0) return FVDBM_OK;
  // stage: rho [N] then vel [N][2] (the staging buffer holds 9 max(N, F) floats)
  CK(cudaMemcpyAsync(h->stage, rho, size_t(hp.N) * 4, cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->stage + hp.N, vel, size_t(2) * hp.N * 4, cudaMemcpyHostToDevice, h->stream));
  CK(launch_cells_eq(h->dp, h->stage, h->stage + hp.N, h->d_cell_new, h->f[h->cur], h->stream));
  if (h->fused) CK(launch_stencil_macros(h->dp, h->f[h->cur], h->stream));
  for (size_t s = 0; s < h->active.size(); ++s)
    if (!h->active[s])
      CK(launch_copy_cells(h->f[h->cur], h->f[h->cur ^ 1], hp.case_cell[s], hp.case_cell[s + 1], h->stream));
  h->snap_step = -1;
    if (!h->case_snap.empty()) h->case_snap.assign(h->case_snap.size(), -1);
  h->nodes_ready = false;
  CK(cudaStreamSynchronize(h->stream));
  return FVDBM_OK;
}

int fvdbm_step(void* handle, int32_t n_steps) {
  if (!handle) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  if (n_steps < 0) return fail(h, FVDBM_EINVAL, "n_steps < 0");
  CK(cudaSetDevice(h->device));
  h->in_ok = false;
  if (n_steps == 1 && h->hp.N > 0) CK(cudaEventRecord(h->in_ready, h->stream));
  int n = n_steps;
  if (n >= kGraphSteps && h->hp.N > 0 && !h->persist) {
    int rc = ensure_nodes(h);  // outside the capture
    if (rc != FVDBM_OK) return rc;
    while (n >= kGraphSteps) {
      cudaGraphExec_t g;
      rc = get_graph(h, h->cur, &g);
      if (rc != FVDBM_OK) return rc;
      CK(cudaGraphLaunch(g, h->stream));
      n -= kGraphSteps;  // even: the current buffers are unchanged
      if (h->fnodes) h->node_last = h->node_cur ^ 1;
    }
  }
  int rc = enqueue_steps(h, n);
  if (rc != FVDBM_OK) return rc;
  h->in_ok = n_steps == 1 && h->hp.N > 0;
  h->steps_done += n_steps;
  for (size_t s = 0; s < h->active.size(); ++s)
    if (h->active[s]) h->case_steps[s] += n_steps;
  return FVDBM_OK;
}

int fvdbm_wait_selftest(int32_t device, int32_t flag_set, int32_t iterations, int32_t* status) {
  if (!status || iterations < 1 || iterations > (1 << 24)) return FVDBM_EINVAL;
  cudaError_t e = cudaSetDevice(device);
  cudaStream_t s = nullptr;
  int* d = nullptr;  // [0] flag, [1] status
  int host[2] = {flag_set ? 1 : 0, 0};
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&d, 2 * sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpyAsync(d, host, 2 * sizeof(int), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = launch_wait_selftest(d, iterations, d + 1, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(host, d, 2 * sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (d) cudaFree(d);
  if (s) cudaStreamDestroy(s);
  if (e != cudaSuccess) {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_create_err = std::string("fvdbm_wait_selftest: ") + cudaGetErrorString(e);
    return FVDBM_ECUDA;
  }
  *status = host[1];
  return FVDBM_OK;
}

int fvdbm_const_div_check(int32_t device, float divisor, uint64_t* mismatches,
                          uint32_t* first_mismatch) {
  return fvdbm_const_div_check_form(device, divisor, 5, mismatches, first_mismatch);
}

int fvdbm_const_div_check_form(int32_t device, float divisor, int32_t form, uint64_t* mismatches,
                               uint32_t* first_mismatch) {
  if (!mismatches || !first_mismatch || (form != 5 && form != 2)) return FVDBM_EINVAL;
  cudaError_t e = cudaSetDevice(device);
  cudaStream_t s = nullptr;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  unsigned long long bad = 0;
  unsigned ex = 0xFFFFFFFFu;
  if (e == cudaSuccess) e = run_cdiv_check(divisor, 1.0f / divisor, cdiv_low(divisor, 1.0f / divisor), form == 2, s, &bad, &ex);
  if (s) cudaStreamDestroy(s);
  if (e != cudaSuccess) {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_create_err = std::string("fvdbm_const_div_check: ") + cudaGetErrorString(e);
    return FVDBM_ECUDA;
  }
  *mismatches = bad;
  *first_mismatch = ex;
  return FVDBM_OK;
}

int fvdbm_step_phase(void* handle, int32_t phase) {
  if (!handle) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  h->in_ok = false;
  CK(cudaSetDevice(h->device));
  const float* fin = h->f[h->cur];
  float* fout = h->f[h->cur ^ 1];
  if (h->hp.q == 13) {  // fused: nodes in phase 1; staged: nodes, faces and cells in phase 2
    if (phase != 1 && phase != 2) return fail(h, FVDBM_EINVAL, "phase must be 1 or 2");
    if (phase == 1) {
      if (h->fused) CK(launch13_nodes(h->dp, fin, h->stream));
      return FVDBM_OK;
    }
    if (h->fused)
      CK(launch13_cells(h->dp, fin, fout, h->stream));
    else
      CK(launch13_step(h->dp, fin, h->flux, fout, h->stream));
    h->cur ^= 1;
    h->steps_done += 1;
    return FVDBM_OK;
  }
  if (h->fnodes) {
    // one launch per step: phase 1 only brings the nodes up to date
    if (phase == 1) return ensure_nodes(h);
    if (phase != 2) return fail(h, FVDBM_EINVAL, "phase must be 1 or 2");
    int rc = ensure_nodes(h);
    if (rc != FVDBM_OK) return rc;
    CK(launch_fused_nodes(with_nodes(h, h->node_cur, h->node_cur ^ 1), fin, fout, h->stream, false));
    h->node_last = h->node_cur;
    h->node_cur ^= 1;
    h->cur ^= 1;
    h->steps_done += 1;
    return FVDBM_OK;
  }
  if (h->persist) {  // one launch per step: phase 1 is empty
    if (phase != 1 && phase != 2) return fail(h, FVDBM_EINVAL, "phase must be 1 or 2");
    if (phase == 2) {
      int rc = enqueue_steps(h, 1);
      if (rc != FVDBM_OK) return rc;
      h->steps_done += 1;
    }
    return FVDBM_OK;
  }
  if (phase == 1) {
    if (h->fused && !h->one && !h->tile)
      CK(launch_nodes_cp(h->dp, fin, h->stream, false));
    else if (!h->one && (!h->tile || !h->dp.tile_nodes))
      CK(launch_nodes(h->dp, fin, h->stream));
  } else if (phase == 2) {
    if (h->batch) {
      CK(launch_fused_batch(h->dp, fin, fout, h->stream, false, h->batch_block, h->batch_waves));
    } else if (h->one) {
      CK(launch_step(h->dp, fin, fout, h->stream, false));
    } else if (h->tile) {
      CK(launch_tile(h->dp, fin, fout, h->stream));
    } else if (h->fused) {
      CK(launch_fused(h->dp, fin, fout, h->stream));
    } else {
      CK(launch_face_flux(h->dp, fin, h->flux, h->stream));
      CK(launch_gather(h->dp, fin, h->flux, fout, h->stream));
    }
    h->cur ^= 1;
    h->steps_done += 1;
  } else {
    return fail(h, FVDBM_EINVAL, "phase must be 1 or 2");
  }
  return FVDBM_OK;
}

int fvdbm_sync(void* handle) {
  if (!handle) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  CK(cudaSetDevice(h->device));
  CK(cudaStreamSynchronize(h->stream));
  return check_status(h);
}

int fvdbm_get_cells(void* handle, float* pdf, float* rho, float* vel, float* pdf_eq) {
  if (!handle) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  const HostPlan& hp = h->hp;
  CK(cudaSetDevice(h->device));
  const int N = hp.N;
  if (pdf && N > 0) {
    CK(launch_gather_cells(h->f[h->cur], h->stage, h->d_cell_new, N, h->stream, hp.q));
    CK(cudaMemcpyAsync(pdf, h->stage, size_t(hp.q) * N * 4, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  }
  if ((rho || vel) && !pdf_eq && N > 0 && hp.q == 9 && h->steps_done > 0) {
    // rho and vel only: one kernel writes both in reference order, straight
    // into page-locked host arrays when both are, else into the staging
    // buffer (9N >= 3N floats) with two copies; one synchronisation
    float* hr = rho ? static_cast<float*>(host_mapped(rho)) : nullptr;
    float* hv = vel ? static_cast<float*>(host_mapped(vel)) : nullptr;
    if ((!rho || hr) && (!vel || hv)) {
      // after a single step, beside it: its input buffer is read-only to it
      cudaStream_t s = h->in_ok ? h->side : h->stream;
      if (h->in_ok) CK(cudaStreamWaitEvent(h->side, h->in_ready, 0));
      CK(launch_macros_ref(h->dp, h->f[h->cur ^ 1], h->d_cell_new, hr, hv, s, /*grid_cap=*/h->in_ok));
      if (h->in_ok) CK(cudaStreamSynchronize(h->side));
      return sync_and_check(h);
    }
    float* sr = h->stage;
    float* sv = h->stage + N;
    CK(launch_macros_ref(h->dp, h->f[h->cur ^ 1], h->d_cell_new, sr, sv, h->stream));
    if (rho) CK(cudaMemcpyAsync(rho, sr, size_t(N) * 4, cudaMemcpyDeviceToHost, h->stream));
    if (vel) CK(cudaMemcpyAsync(vel, sv, size_t(2) * N * 4, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return check_status(h);
  }
  if ((rho || vel || pdf_eq) && N > 0) {
    if (h->steps_done == 0) {
      if (rho) std::memset(rho, 0, size_t(N) * 4);
      if (vel) std::memset(vel, 0, size_t(2) * N * 4);
      if (pdf_eq) std::memset(pdf_eq, 0, size_t(hp.q) * N * 4);
    } else {
      if (!h->mac) {
        int rc = dalloc<float>(h, &h->mac, size_t(3 + hp.q) * hp.Np);
        if (rc != FVDBM_OK) return rc;
      }
      float* mr = h->mac;
      float* mv = h->mac + hp.Np;
      float* me = h->mac + size_t(3) * hp.Np;
      if (hp.q == 13)
        CK(launch13_macros(h->dp, h->f[h->cur ^ 1], mr, mv, me, h->stream));
      else
        CK(launch_macros(h->dp, h->f[h->cur ^ 1], mr, mv, me, h->stream));
      if (rho) {
        CK(launch_soa_to_aos(mr, h->stage, h->d_cell_new, N, hp.Np, 1, h->stream));
        CK(cudaMemcpyAsync(rho, h->stage, size_t(N) * 4, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
      }
      if (vel) {
        CK(launch_soa_to_aos(mv, h->stage, h->d_cell_new, N, hp.Np, 2, h->stream));
        CK(cudaMemcpyAsync(vel, h->stage, size_t(2) * N * 4, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
      }
      if (pdf_eq) {
        CK(launch_gather_cells(me, h->stage, h->d_cell_new, N, h->stream, hp.q));
        CK(cudaMemcpyAsync(pdf_eq, h->stage, size_t(hp.q) * N * 4, cudaMemcpyDeviceToHost, h->stream));
        CK(cudaStreamSynchronize(h->stream));
      }
    }
  }
  CK(cudaStreamSynchronize(h->stream));
  return check_status(h);
}

int fvdbm_get_nodes(void* handle, float* pdf, float* rho, float* vel) {
  if (!handle) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  const HostPlan& hp = h->hp;
  CK(cudaSetDevice(h->device));
  if (hp.M > 0) {
    std::vector<float> dp(size_t(hp.q) * hp.Mp), dr(hp.Mp), dv(size_t(2) * hp.Mp);
    const DevPlan q = h->fnodes ? with_nodes(h, h->node_last, h->node_last) : h->dp;
    CK(cudaMemcpyAsync(dp.data(), q.node_pdf, dp.size() * 4, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(dr.data(), q.node_rho, dr.size() * 4, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(dv.data(), q.node_vel, dv.size() * 4, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int d = 0; d < hp.M; ++d) {
      const int p = hp.node_orig[d];
      for (int q = 0; q < hp.q; ++q) h->node_pdf[size_t(p) * hp.q + q] = dp[size_t(q) * hp.Mp + d];
      h->node_rho[p] = dr[d];
      h->node_vel[size_t(p) * 2] = dv[d];
      h->node_vel[size_t(p) * 2 + 1] = dv[hp.Mp + d];
    }
  }
  if (pdf) std::memcpy(pdf, h->node_pdf.data(), size_t(hp.q) * hp.P * 4);
  if (rho) std::memcpy(rho, h->node_rho.data(), size_t(hp.P) * 4);
  if (vel) std::memcpy(vel, h->node_vel.data(), size_t(2) * hp.P * 4);
  return FVDBM_OK;
}

int fvdbm_get_face_fluxes(void* handle, float* flux) {
  if (!handle || !flux) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  const HostPlan& hp = h->hp;
  CK(cudaSetDevice(h->device));
  if (hp.F == 0) return FVDBM_OK;
  if (!h->flux) {
    int rc = dalloc<float>(h, &h->flux, size_t(hp.q) * hp.Fp);
    if (rc != FVDBM_OK) return rc;
  }
  if (hp.q == 13)
    CK(launch13_face_flux(h->dp, h->f[h->cur ^ 1], h->flux, h->stream));
  else
    CK(launch_face_flux(h->fnodes ? with_nodes(h, h->node_last, h->node_last) : h->dp, h->f[h->cur ^ 1], h->flux,
                        h->stream));
  std::vector<float> soa(size_t(hp.q) * hp.Fp);
  CK(cudaMemcpyAsync(soa.data(), h->flux, soa.size() * 4, cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  for (int j = 0; j < hp.F; ++j) {
    const int f = hp.face_old[j];
    for (int q = 0; q < hp.q; ++q) flux[size_t(f) * hp.q + q] = soa[size_t(q) * hp.Fp + j];
  }
  return FVDBM_OK;
}

int fvdbm_residual(void* handle, double* res_u, double* mass) {
  if (!handle || !res_u || !mass) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  if (h->hp.q != 9) return fail(h, FVDBM_EINVAL, "the convergence monitor supports D2Q9");
  const HostPlan& hp = h->hp;
  CK(cudaSetDevice(h->device));
  const int nb = residual_chunks(hp.N, kResidualChunk);
  if (!h->usnap) {
    int rc = dalloc<float>(h, &h->usnap, size_t(2) * hp.Np);
    if (rc != FVDBM_OK) return rc;
    if ((rc = dalloc<double>(h, &h->red, size_t(4) * (nb + 1))) != FVDBM_OK) return rc;
  }
  const bool have = h->snap_step >= 0;
  double* out = h->red + size_t(4) * nb;
  CK(launch_residual(h->dp, h->f[h->cur], h->usnap, h->d_area, have, kResidualChunk, nullptr, 0, h->red,
                     nullptr, 1, out, h->stream));
  double tot[4];
  CK(cudaMemcpyAsync(tot, out, sizeof(tot), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  int rc = check_status(h);
  if (rc != FVDBM_OK) return rc;
  const long long K = h->steps_done - h->snap_step;
  *mass = tot[2];
  if (tot[3] > 0.0)
    *res_u = std::nan("");
  else if (!have || K <= 0)
    *res_u = HUGE_VAL;
  else
    *res_u = std::sqrt(tot[0]) / (double(K) * double(h->params.delta_t) * std::max(std::sqrt(tot[1]), 1e-30));
  h->snap_step = h->steps_done;
  return FVDBM_OK;
}

int fvdbm_run_to_steady(void* handle, double threshold, int32_t check_every, int64_t max_steps,
                        int64_t* steps_taken, double* res_u) {
  if (!handle || !steps_taken || !res_u) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  h->in_ok = false;
  if (check_every <= 0 || max_steps < 0) return fail(h, FVDBM_EINVAL, "check_every <= 0 or max_steps < 0");
  double r = HUGE_VAL, m = 0.0;
  int rc;
  if (h->snap_step != h->steps_done && (rc = fvdbm_residual(h, &r, &m)) != FVDBM_OK) return rc;
  r = HUGE_VAL;
  int64_t taken = 0;
  while (taken < max_steps) {
    const int n = int(std::min<int64_t>(check_every, max_steps - taken));
    if ((rc = fvdbm_step(h, n)) != FVDBM_OK) return rc;
    taken += n;
    if ((rc = fvdbm_residual(h, &r, &m)) != FVDBM_OK) return rc;
    if (std::isnan(r) || r < threshold) break;
  }
  *steps_taken = taken;
  *res_u = r;
  if (std::isnan(r))
    return fail(h, FVDBM_ENONFINITE, "fvdbm_run_to_steady: the residual turned NaN after " + std::to_string(taken) +
                                         " steps (a cell's rho or u is not finite: the run diverged)");
  return FVDBM_OK;
}

void* fvdbm_stream(void* handle) { return handle ? static_cast<Handle*>(handle)->stream : nullptr; }

int fvdbm_get_info(void* handle, fvdbm_info_t* info) {
  if (!handle || !info) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  const HostPlan& hp = h->hp;
  info->n_cells = hp.N;
  info->n_faces = hp.F;
  info->n_nodes = hp.P;
  info->n_bc_nodes = hp.Mc;
  info->n_ghost_faces = hp.n_ghost_faces;
  info->kernel = h->persist ? FVDBM_KERNEL_PERSIST
               : h->fnodes ? (h->dp.fast ? FVDBM_KERNEL_FAST : FVDBM_KERNEL_FUSED_NODES)
               : h->batch ? FVDBM_KERNEL_BATCH : h->one ? FVDBM_KERNEL_ONE
                         : h->tile ? (h->dp.tile_nodes ? FVDBM_KERNEL_TILE : FVDBM_KERNEL_TILE_SPLIT)
                                   : (h->fused ? FVDBM_KERNEL_FUSED : FVDBM_KERNEL_STAGED);
  const int node_launch = (hp.Mc > 0 && !h->one && !h->fnodes && !(h->tile && h->dp.tile_nodes)) ? 1 : 0;
  info->launches_per_step = h->persist ? 1 : node_launch + (h->one || h->tile || h->batch ? 1 : (h->fused ? 1 : 2));
  info->padded_cells = hp.Np;
  info->ctas_per_sm = h->tile ? tile_ctas_per_sm(h->dp) : 0;
  info->const_division = h->dp.cdiv_mode;
  info->bytes_per_step = hp.bytes_per_step;
  info->device_bytes = h->device_bytes;
  return FVDBM_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Staged step with a fixed face-flux scratch array.  For callers that cannot
// allocate device memory while they step: a host framework that owns the
// device's memory (JAX/XLA preallocates most of it by default), or a loop in
// which a cudaMalloc/cudaFree would stall the device.  The array is shared by
// every call on a device and keeps the last call's fluxes; nothing in it needs
// to start at zero, because each step's face kernel writes all 9 x F fluxes
// before the gather reads any of them.  Calls whose kernels overlap on the GPU
// race on the array.

static __device__ __align__(256) float g_face_flux_scratch[size_t(Q) * FVDBM_STATIC_SCRATCH_MAX_FACES];

namespace {

constexpr int kScratchDevices = 64;
std::mutex g_scratch_mu;
// Per device: the array's address and the id of the CUDA context it was
// looked up in (0 when the id could not be read).
float* g_scratch_addr[kScratchDevices] = {};
unsigned long long g_scratch_ctx[kScratchDevices] = {};

// Id of the current CUDA context (unique for the life of the process, so a
// context re-created after cudaDeviceReset gets a new one), through the
// driver entry points the runtime hands out (no link-time dependency on the
// driver library); 0 when unavailable.
unsigned long long current_context_id() {
  using GetCurrent = int (*)(void**);
  using GetId = int (*)(void*, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    void* a = nullptr;
    void* b = nullptr;
    cudaDriverEntryPointQueryResult qa{}, qb{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
        qa == cudaDriverEntryPointSuccess && qb == cudaDriverEntryPointSuccess) {
      get_current = reinterpret_cast<GetCurrent>(a);
      get_id = reinterpret_cast<GetId>(b);
    }
    cudaGetLastError();
    looked_up = true;
  }
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
  return id;
}

// Device address of the scratch array on h's device (current on entry).
// Set-up once per device and context: the first call on a device (and the
// first call after the device's context was re-created, e.g. by
// cudaDeviceReset) looks the address up with cudaGetSymbolAddress; later
// calls reuse it.  When the context id cannot be read, every call looks the
// address up again.
int scratch_address(Handle* h, float** out) {
  if (h->device < 0 || h->device >= kScratchDevices)
    return fail(h, FVDBM_EINVAL, "fvdbm_step_static_scratch: device index " + std::to_string(h->device) +
                                     " out of range");
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  const unsigned long long ctx = current_context_id();
  if (!g_scratch_addr[h->device] || ctx == 0 || g_scratch_ctx[h->device] != ctx) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_face_flux_scratch);
    if (e != cudaSuccess)
      return fail(h, FVDBM_ECUDA, std::string("cudaGetSymbolAddress(face flux scratch): ") +
                                      cudaGetErrorString(e));
    g_scratch_addr[h->device] = static_cast<float*>(p);
    g_scratch_ctx[h->device] = ctx;
  }
  *out = g_scratch_addr[h->device];
  return FVDBM_OK;
}

}  // namespace

extern "C" int fvdbm_step_static_scratch(void* handle, int32_t n_steps) {
  if (!handle) return FVDBM_EINVAL;
  Handle* h = static_cast<Handle*>(handle);
  h->in_ok = false;
  const HostPlan& hp = h->hp;
  if (n_steps < 0) return fail(h, FVDBM_EINVAL, "n_steps < 0");
  if (h->fused || h->tile || h->one || h->batch)
    return fail(h, FVDBM_EINVAL,
                "fvdbm_step_static_scratch steps the staged kernels of a single mesh only: create the "
                "handle with fvdbm_create and FVDBM_KERNEL_STAGED (not a batch)");
  if (hp.q != 9) return fail(h, FVDBM_EINVAL, "fvdbm_step_static_scratch steps D2Q9 meshes only");
  if (hp.Fp > FVDBM_STATIC_SCRATCH_MAX_FACES)
    return fail(h, FVDBM_EINVAL,
                "fvdbm_step_static_scratch: the mesh has " + std::to_string(hp.F) + " faces (" +
                    std::to_string(hp.Fp) + " padded); the static face-flux scratch holds at most " +
                    std::to_string(FVDBM_STATIC_SCRATCH_MAX_FACES) + " padded faces (" +
                    std::to_string(size_t(Q) * FVDBM_STATIC_SCRATCH_MAX_FACES * 4) +
                    " bytes); use fvdbm_step");
  CK(cudaSetDevice(h->device));
  float* scratch = nullptr;
  int rc = scratch_address(h, &scratch);
  if (rc != FVDBM_OK) return rc;
  for (int s = 0; s < n_steps; ++s) {
    const float* fin = h->f[h->cur];
    float* fout = h->f[h->cur ^ 1];
    CK(launch_nodes(h->dp, fin, h->stream));
    CK(launch_face_flux(h->dp, fin, scratch, h->stream));
    CK(launch_gather(h->dp, fin, scratch, fout, h->stream));
    h->cur ^= 1;
  }
  h->steps_done += n_steps;
  return FVDBM_OK;
}
