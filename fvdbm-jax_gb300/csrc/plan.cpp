// Host-side plan: validates the reference-layout containers, renumbers the
// cells for locality and builds every device table.  Float32 quantities that
// the reference evaluates inside the step but that depend only on static
// data (IDW weights 1/d, their sum, the Lax-Wendroff d0/(d0+d1), the ghost
// distance ratios) are evaluated here once with the same float32 operations,
// so the kernels stay bitwise equal to the per-step evaluation.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <queue>
#include <sstream>

#include "../../include/fvdbm.h"
#include "fvdbm_internal.h"

namespace fvdbm {

namespace {

int round_up(int x, int m) { return (x + m - 1) / m * m; }

// JAX gathers wrap index -1 to the last row (the reference pads with -1).
inline int32_t wrap(int32_t idx, int32_t n) { return idx < 0 ? idx + n : idx; }

uint32_t spread16(uint32_t x) {
  x &= 0xffff;
  x = (x | (x << 8)) & 0x00ff00ff;
  x = (x | (x << 4)) & 0x0f0f0f0f;
  x = (x | (x << 2)) & 0x33333333;
  x = (x | (x << 1)) & 0x55555555;
  return x;
}

std::vector<int32_t> morton_order(const float* xy, int N) {
  float x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
  for (int i = 0; i < N; ++i) {
    x0 = std::min(x0, xy[2 * i]);
    x1 = std::max(x1, xy[2 * i]);
    y0 = std::min(y0, xy[2 * i + 1]);
    y1 = std::max(y1, xy[2 * i + 1]);
  }
  const double span = std::max(double(x1 - x0), double(y1 - y0));
  const double s = span > 0 ? 65535.0 / span : 0.0;
  std::vector<std::pair<uint32_t, int32_t>> key(N);
  for (int i = 0; i < N; ++i) {
    uint32_t qx = uint32_t(std::min(65535.0, std::max(0.0, (xy[2 * i] - x0) * s)));
    uint32_t qy = uint32_t(std::min(65535.0, std::max(0.0, (xy[2 * i + 1] - y0) * s)));
    key[i] = {spread16(qx) | (spread16(qy) << 1), i};
  }
  std::sort(key.begin(), key.end());
  std::vector<int32_t> order(N);
  for (int i = 0; i < N; ++i) order[i] = key[i].second;
  return order;
}

// Reverse Cuthill-McKee over the cell adjacency given by interior faces.
std::vector<int32_t> rcm_order(int N, int F, const int32_t* fc) {
  std::vector<int32_t> deg(N, 0);
  for (int f = 0; f < F; ++f) {
    const int a = fc[2 * f], b = fc[2 * f + 1];
    if (a >= 0 && b >= 0 && a != b) {
      deg[a]++;
      deg[b]++;
    }
  }
  std::vector<int32_t> ptr(N + 1, 0);
  for (int i = 0; i < N; ++i) ptr[i + 1] = ptr[i] + deg[i];
  std::vector<int32_t> adj(ptr[N]);
  std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
  for (int f = 0; f < F; ++f) {
    const int a = fc[2 * f], b = fc[2 * f + 1];
    if (a >= 0 && b >= 0 && a != b) {
      adj[fill[a]++] = b;
      adj[fill[b]++] = a;
    }
  }
  for (int i = 0; i < N; ++i)
    std::sort(adj.begin() + ptr[i], adj.begin() + ptr[i + 1],
              [&](int x, int y) { return deg[x] != deg[y] ? deg[x] < deg[y] : x < y; });
  std::vector<int32_t> order;
  order.reserve(N);
  std::vector<char> seen(N, 0);
  std::vector<int32_t> by_deg(N);
  std::iota(by_deg.begin(), by_deg.end(), 0);
  std::stable_sort(by_deg.begin(), by_deg.end(), [&](int x, int y) { return deg[x] < deg[y]; });
  for (int start : by_deg) {
    if (seen[start]) continue;
    // pseudo-peripheral start: last node of a BFS from the min-degree node
    int s = start;
    {
      std::vector<int32_t> lvl;
      std::queue<int32_t> qq;
      std::vector<char> vis(0);
      qq.push(s);
      std::vector<int32_t> visited{ s };
      seen[s] = 2;
      int last = s;
      while (!qq.empty()) {
        int u = qq.front();
        qq.pop();
        last = u;
        for (int e = ptr[u]; e < ptr[u + 1]; ++e)
          if (!seen[adj[e]]) {
            seen[adj[e]] = 2;
            visited.push_back(adj[e]);
            qq.push(adj[e]);
          }
      }
      for (int v : visited) seen[v] = 0;
      s = last;
    }
    std::queue<int32_t> qq;
    qq.push(s);
    seen[s] = 1;
    while (!qq.empty()) {
      int u = qq.front();
      qq.pop();
      order.push_back(u);
      for (int e = ptr[u]; e < ptr[u + 1]; ++e)
        if (!seen[adj[e]]) {
          seen[adj[e]] = 1;
          qq.push(adj[e]);
        }
    }
  }
  std::reverse(order.begin(), order.end());
  return order;
}

}  // namespace

// Order of the cells of one case (segment [a, b) of a union mesh whose faces
// [fa, fb) belong to it): Morton when centroids are given, else RCM.
std::vector<int32_t> segment_order(const fvdbm_mesh_t& m, int ordering, int a, int b, int fa, int fb) {
  const int n = b - a;
  std::vector<int32_t> loc;
  if (ordering == FVDBM_ORDER_MORTON && m.cell_xy) {
    loc = morton_order(m.cell_xy + 2 * int64_t(a), n);
  } else if (ordering == FVDBM_ORDER_RCM) {
    std::vector<int32_t> fc(2 * size_t(fb - fa));
    for (int f = fa; f < fb; ++f)
      for (int k = 0; k < 2; ++k) {
        const int32_t c = m.face_cells[2 * f + k];
        fc[2 * size_t(f - fa) + k] = c < 0 ? -1 : c - a;
      }
    loc = rcm_order(n, fb - fa, fc.data());
  } else {
    loc.resize(n);
    std::iota(loc.begin(), loc.end(), 0);
  }
  for (auto& c : loc) c += a;
  return loc;
}

std::string build_plan(const void* mesh_v, const void* params_v, HostPlan& hp, const BatchSegs* segs) {
  const fvdbm_mesh_t& m = *static_cast<const fvdbm_mesh_t*>(mesh_v);
  const fvdbm_params_t& pr = *static_cast<const fvdbm_params_t*>(params_v);
  std::ostringstream err;
  const int N = m.n_cells, F = m.n_faces, P = m.n_nodes, K = m.cell_face_stride,
            Kn = m.node_cell_stride;
  if (N < 0 || F < 0 || P < 0 || K < 0 || Kn < 0) return "negative size";
  if (int64_t(N) > HF_MAX_INDEX || int64_t(F) > HF_MAX_INDEX) return "mesh too large (max 2^27 cells/faces)";
  if (pr.flux_scheme != FVDBM_UPWIND && pr.flux_scheme != FVDBM_LAX_WENDROFF)
    return "Unknown flux scheme";
  if (pr.variant < 0 || pr.variant > 2) return "unknown flux variant";
  if (pr.kernel < FVDBM_KERNEL_AUTO || pr.kernel > FVDBM_KERNEL_FAST || pr.kernel == FVDBM_KERNEL_BATCH)
    return "unknown kernel family";
  hp.q = pr.lattice == 0 ? 9 : pr.lattice;
  if (hp.q != 9 && hp.q != 13) return "lattice must be 9 (D2Q9) or 13 (D2Q13)";
  if (hp.q == 13 && pr.variant != 0) return "D2Q13 takes no flux-scale variant";
  if (N > 0 && K > 0 && (!m.cell_face_indices || !m.cell_face_signs)) return "cell face arrays missing";
  if (F > 0 && (!m.face_cells || !m.face_dists || !m.face_nodes || !m.face_n || !m.face_L))
    return "face arrays missing";
  if (P > 0 && (!m.node_type || (Kn > 0 && (!m.node_cells || !m.node_dists))))
    return "node arrays missing";
  if (pr.variant != 0 && F > 0 && !m.face_scale) return "face_scale missing for the flux variant";
  if (K > 0 && N > 0 && F == 0) return "cells reference faces but there are none";

  hp.N = N;
  hp.F = F;
  hp.P = P;
  hp.K = K;
  hp.Kn = Kn;
  hp.Np = std::max(TILE, round_up(N, TILE));
  hp.Fp = std::max(128, round_up(F, 128));
  hp.scheme = pr.flux_scheme;
  hp.variant = pr.variant;
  hp.fv = m.cell_inv_area != nullptr;

  // ---- validation (reference semantics: -1 wraps to the last row)
  for (int64_t t = 0; t < int64_t(N) * K; ++t) {
    const int32_t fi = m.cell_face_indices[t], sg = m.cell_face_signs[t];
    if (fi < -1 || fi >= F) {
      err << "Cells.face_indices[" << t / K << "," << t % K << "]=" << fi << " out of range";
      return err.str();
    }
    if (sg < -1 || sg > 1) {
      err << "Cells.face_normals[" << t / K << "," << t % K << "]=" << sg << " is not -1, 0 or 1";
      return err.str();
    }
  }
  for (int64_t t = 0; t < int64_t(F) * 2; ++t) {
    if (m.face_cells[t] < -1 || m.face_cells[t] >= N) {
      err << "Faces.stencil_cells_index[" << t / 2 << "," << t % 2 << "] out of range";
      return err.str();
    }
    if (m.face_nodes[t] < -1 || m.face_nodes[t] >= P) {
      err << "Faces.nodes_index[" << t / 2 << "," << t % 2 << "] out of range";
      return err.str();
    }
  }
  for (int p = 0; p < P; ++p) {
    const int t = m.node_type[p];
    if (t < 0 || t > 2) {
      err << "Nodes.type[" << p << "]=" << t << " is not 0, 1 or 2";
      return err.str();
    }
    for (int k = 0; k < Kn; ++k)
      if (m.node_cells[int64_t(p) * Kn + k] < -1 || m.node_cells[int64_t(p) * Kn + k] >= N) {
        err << "Nodes.cells_index[" << p << "," << k << "] out of range";
        return err.str();
      }
  }

  // ---- packed batch: every reference stays inside its own case
  std::vector<int32_t> node_seg;
  if (segs) {
    const int S = segs->S;
    if (S <= 0 || segs->cell_ptr[0] != 0 || segs->cell_ptr[S] != N || segs->face_ptr[0] != 0 ||
        segs->face_ptr[S] != F || segs->node_ptr[0] != 0 || segs->node_ptr[S] != P)
      return "batch segments do not cover the union mesh";
    node_seg.assign(P, 0);
    for (int s = 0; s < S; ++s) {
      const int c0 = segs->cell_ptr[s], c1 = segs->cell_ptr[s + 1];
      const int f0 = segs->face_ptr[s], f1 = segs->face_ptr[s + 1];
      const int n0 = segs->node_ptr[s], n1 = segs->node_ptr[s + 1];
      if (c1 <= c0 || f1 < f0 || n1 < n0) return "batch case " + std::to_string(s) + " is empty or inverted";
      auto inside = [](int32_t x, int lo, int hi) { return x >= lo && x < hi; };
      for (int c = c0; c < c1; ++c)
        for (int k = 0; k < K; ++k)
          if (!inside(m.cell_face_indices[int64_t(c) * K + k], f0, f1))
            return "batch case " + std::to_string(s) + ": a cell names a face of another case";
      for (int f = f0; f < f1; ++f)
        for (int k = 0; k < 2; ++k) {
          const int32_t c = m.face_cells[2 * f + k], nd = m.face_nodes[2 * f + k];
          if ((c != -1 && !inside(c, c0, c1)) || !inside(nd, n0, n1))
            return "batch case " + std::to_string(s) + ": a face names a cell or node of another case";
        }
      for (int p_ = n0; p_ < n1; ++p_) {
        node_seg[p_] = s;
        for (int k = 0; k < Kn; ++k) {
          const int32_t c = m.node_cells[int64_t(p_) * Kn + k];
          if (c != -1 && !inside(c, c0, c1))
            return "batch case " + std::to_string(s) + ": a node names a cell of another case";
        }
      }
    }
  }

  // ---- cell order
  hp.ordering = pr.ordering;
  if (segs && N > 0) {
    hp.cell_old.clear();
    for (int s = 0; s < segs->S; ++s) {
      auto o = segment_order(m, pr.ordering, segs->cell_ptr[s], segs->cell_ptr[s + 1], segs->face_ptr[s],
                             segs->face_ptr[s + 1]);
      hp.cell_old.insert(hp.cell_old.end(), o.begin(), o.end());
    }
    if (pr.ordering == FVDBM_ORDER_MORTON && !m.cell_xy) hp.ordering = FVDBM_ORDER_NONE;
  } else if (pr.ordering == FVDBM_ORDER_MORTON && m.cell_xy && N > 0)
    hp.cell_old = morton_order(m.cell_xy, N);
  else if (pr.ordering == FVDBM_ORDER_RCM && N > 0)
    hp.cell_old = rcm_order(N, F, m.face_cells);
  else {
    hp.cell_old.resize(N);
    std::iota(hp.cell_old.begin(), hp.cell_old.end(), 0);
    if (pr.ordering == FVDBM_ORDER_MORTON) hp.ordering = FVDBM_ORDER_NONE;
  }
  // the stencil cells of the computed boundary nodes go last (stable): the
  // fused kernel's tail blocks then also record their macros for the next
  // step's node kernel, and the blocks that need boundary nodes in the
  // single-launch step form the tail of its grid.  (Not for the in-tile node
  // kernel, whose tiles must stay compact.)
  // With the node update inside the fused kernel (KERNEL_FUSED_NODES) the
  // stencil cells go first instead: their blocks finish early and the node
  // blocks can run while the other cell blocks still compute.  The last
  // reference cell then joins them when a node has padded entries (those
  // read its macros).
  hp.stencil_start = N;
  hp.stencil_end = N;
  hp.stencil_first = (pr.kernel == FVDBM_KERNEL_FUSED_NODES || pr.kernel == FVDBM_KERNEL_FAST) && !segs;
  if (N > 0 && Kn > 0 && pr.kernel != FVDBM_KERNEL_TILE && !segs) {
    std::vector<char> member(N, 0);
    bool padded = false;
    for (int p_ = 0; p_ < P; ++p_) {
      if (m.node_type[p_] == 0) continue;
      for (int k = 0; k < Kn; ++k) {
        const int32_t c = m.node_cells[int64_t(p_) * Kn + k];
        float w = 1.0f / m.node_dists[int64_t(p_) * Kn + k];
        if (w < 0.0f) w = 0.0f;
        if (c == -1 && w == 0.0f) {  // padding: evaluated from the last cell directly
          padded = true;
          continue;
        }
        member[wrap(c, N)] = 1;
      }
    }
    if (hp.stencil_first) {
      if (padded) member[N - 1] = 1;
      auto it = std::stable_partition(hp.cell_old.begin(), hp.cell_old.end(),
                                      [&](int32_t c) { return member[c] != 0; });
      hp.stencil_start = 0;
      hp.stencil_end = int(it - hp.cell_old.begin());
    } else {
      auto it = std::stable_partition(hp.cell_old.begin(), hp.cell_old.end(),
                                      [&](int32_t c) { return !member[c]; });
      hp.stencil_start = int(it - hp.cell_old.begin());
    }
  }
  hp.cell_new.assign(N, -1);
  for (int i = 0; i < N; ++i) hp.cell_new[hp.cell_old[i]] = i;
  hp.last_cell_new = N > 0 ? hp.cell_new[N - 1] : 0;
  if (hp.stencil_first && hp.last_cell_new < hp.stencil_end) hp.last_slot = hp.last_cell_new - hp.stencil_start;
  auto cnew = [&](int32_t c) { return c < 0 ? -1 : hp.cell_new[c]; };
  auto cnew_wrap = [&](int32_t c) { return N > 0 ? hp.cell_new[wrap(c, N)] : 0; };

  // ---- which faces need ghosts, which nodes live on the device
  std::vector<char> ghost_face(F, 0);
  for (int f = 0; f < F; ++f)
    ghost_face[f] = (m.face_cells[2 * f] == -1 || m.face_cells[2 * f + 1] == -1);
  hp.n_ghost_faces = int(std::count(ghost_face.begin(), ghost_face.end(), 1));
  std::vector<char> needed(P, 0);
  for (int f = 0; f < F; ++f)
    if (ghost_face[f] && P > 0) {
      needed[wrap(m.face_nodes[2 * f], P)] = 1;
      needed[wrap(m.face_nodes[2 * f + 1], P)] = 1;
    }
  if (hp.n_ghost_faces > 0 && P == 0) return "faces need ghost nodes but there are no nodes";

  // computed nodes first, ordered by their lowest neighbour cell
  std::vector<std::pair<int64_t, int32_t>> comp;
  std::vector<int32_t> frozen;
  for (int p = 0; p < P; ++p) {
    if (m.node_type[p] != 0) {
      int64_t key = int64_t(1) << 40;
      for (int k = 0; k < Kn; ++k) {
        const int32_t c = m.node_cells[int64_t(p) * Kn + k];
        if (c >= 0) key = std::min<int64_t>(key, hp.cell_new[c]);
      }
      comp.push_back({key * (int64_t(P) + 1) + p, p});
    } else if (needed[p]) {
      frozen.push_back(p);
    }
  }
  std::sort(comp.begin(), comp.end());
  hp.Mc = int(comp.size());
  hp.M = hp.Mc + int(frozen.size());
  hp.Mp = std::max(32, round_up(hp.M, 32));
  hp.node_dev.assign(P, -1);
  hp.node_orig.clear();
  for (auto& c : comp) hp.node_orig.push_back(c.second);
  for (int p : frozen) hp.node_orig.push_back(p);
  for (int d = 0; d < hp.M; ++d) hp.node_dev[hp.node_orig[d]] = d;

  // node IDW tables: w = 1/d with negative weights zeroed, sum(w) folded
  // over all Kn entries in order (utils/utils.py:34-60)
  hp.nd_type.resize(hp.Mc);
  hp.nd_ptr.assign(hp.Mc + 1, 0);
  hp.nd_npad.assign(hp.Mc, 0);
  hp.nd_sumw.resize(hp.Mc);
  hp.nd_cell.clear();
  hp.nd_w.clear();
  for (int d = 0; d < hp.Mc; ++d) {
    const int p = hp.node_orig[d];
    hp.nd_type[d] = m.node_type[p];
    float sumw = 0.0f;
    for (int k = 0; k < Kn; ++k) {
      const int32_t c = m.node_cells[int64_t(p) * Kn + k];
      const float dist = m.node_dists[int64_t(p) * Kn + k];
      float w = 1.0f / dist;
      if (w < 0.0f) w = 0.0f;
      sumw = (k == 0) ? w : sumw + w;
      if (c == -1 && w == 0.0f && !segs) {
        hp.nd_npad[d]++;
        continue;
      }
      if (N == 0) return "nodes reference cells but there are none";
      // a batch case's -1 entries wrap to that case's last cell
      uint32_t code = uint32_t(segs && c == -1 ? hp.cell_new[segs->cell_ptr[node_seg[p] + 1] - 1] : cnew_wrap(c));
      if (c == -1) code |= ND_NEQ_ZERO;
      hp.nd_cell.push_back(code);
      hp.nd_w.push_back(w);
    }
    hp.nd_sumw[d] = sumw;
    hp.nd_ptr[d + 1] = int(hp.nd_cell.size());
  }

  // node blocks: whole nodes, at most NODE_BLOCK_ENTRIES entries per block
  hp.nb_ptr.assign(1, 0);
  for (int d = 0; d < hp.Mc; ++d) {
    const int cnt = hp.nd_ptr[d + 1] - hp.nd_ptr[d];
    if (cnt > NODE_BLOCK_ENTRIES) return "a boundary node has more than 128 stencil cells";
    if (hp.nd_ptr[d + 1] - hp.nd_ptr[hp.nb_ptr.back()] > NODE_BLOCK_ENTRIES ||
        d - hp.nb_ptr.back() >= NODE_BLOCK_ENTRIES)
      hp.nb_ptr.push_back(d);
  }
  if (hp.Mc > 0) hp.nb_ptr.push_back(hp.Mc);
  hp.nb_meta.clear();
  for (size_t b = 0; b + 1 < hp.nb_ptr.size(); ++b) {
    hp.nb_meta.push_back(hp.nb_ptr[b]);
    hp.nb_meta.push_back(hp.nb_ptr[b + 1]);
    hp.nb_meta.push_back(hp.nd_ptr[hp.nb_ptr[b]]);
    hp.nb_meta.push_back(hp.nd_ptr[hp.nb_ptr[b + 1]]);
  }
  // the same blocks, padded to NODE_BLOCK_ENTRIES slots so that a thread's
  // entry and node record sit at blk*NODE_BLOCK_ENTRIES + tid:
  //   pe_slot  stencil slot of the entry's cell (| ND_NEQ_ZERO), or ~0u
  //   pe_w     weight
  //   pn_meta  {node, first local entry, entry count, type | npad << 2}, type 0 = empty
  //   pn_sumw  sum of weights
  {
    const int NBk = int(hp.nb_meta.size() / 4);
    hp.pe_slot.assign(size_t(NBk) * NODE_BLOCK_ENTRIES, ~0u);
    hp.pe_w.assign(size_t(NBk) * NODE_BLOCK_ENTRIES, 0.0f);
    hp.pn_meta.assign(size_t(NBk) * NODE_BLOCK_ENTRIES * 4, 0);
    hp.pn_sumw.assign(size_t(NBk) * NODE_BLOCK_ENTRIES, 0.0f);
    for (int b = 0; b < NBk; ++b) {
      const int n0 = hp.nb_meta[4 * b], n1 = hp.nb_meta[4 * b + 1], e0 = hp.nb_meta[4 * b + 2];
      for (int j = 0; j < n1 - n0; ++j) {
        const int d = n0 + j;
        const size_t s = size_t(b) * NODE_BLOCK_ENTRIES + j;
        hp.pn_meta[4 * s + 0] = d;
        hp.pn_meta[4 * s + 1] = hp.nd_ptr[d] - e0;
        hp.pn_meta[4 * s + 2] = hp.nd_ptr[d + 1] - hp.nd_ptr[d];
        hp.pn_meta[4 * s + 3] = hp.nd_type[d] | (hp.nd_npad[d] > 0 ? 4 : 0);
        hp.pn_sumw[s] = hp.nd_sumw[d];
      }
      for (int e = hp.nd_ptr[n0]; e < hp.nd_ptr[n1]; ++e) {
        const size_t s = size_t(b) * NODE_BLOCK_ENTRIES + (e - e0);
        const uint32_t code = hp.nd_cell[e];
        const int32_t cell = int32_t(code & ~ND_NEQ_ZERO);
        hp.pe_slot[s] = uint32_t(cell - hp.stencil_start) | (code & ND_NEQ_ZERO);
        hp.pe_w[s] = hp.nd_w[e];
      }
    }
  }

  // ---- faces in device order (by lowest slot cell)
  {
    std::vector<std::pair<int64_t, int32_t>> fk(F);
    for (int f = 0; f < F; ++f) {
      int64_t a = cnew(m.face_cells[2 * f]), b = cnew(m.face_cells[2 * f + 1]);
      int64_t lo = (a < 0) ? b : (b < 0 ? a : std::min(a, b));
      if (lo < 0) lo = int64_t(1) << 40;
      fk[f] = {lo * (int64_t(F) + 1) + f, f};
    }
    std::sort(fk.begin(), fk.end());
    hp.face_old.resize(F);
    hp.face_new.resize(F);
    for (int j = 0; j < F; ++j) {
      hp.face_old[j] = fk[j].second;
      hp.face_new[fk[j].second] = j;
    }
  }
  hp.fs0.resize(F);
  hp.fs1.resize(F);
  hp.fnx.resize(F);
  hp.fny.resize(F);
  hp.fL.resize(F);
  hp.fr.assign(F, 0.0f);
  hp.fD2.assign(F, 1.0f);
  hp.fna.assign(F, 0);
  hp.fnb.assign(F, 0);
  hp.frl.assign(F, 0.0f);
  hp.frr.assign(F, 0.0f);
  hp.fkl.assign(F, 0);
  hp.fkr.assign(F, 0);
  if (pr.variant == 1) hp.fscale.assign(F, 1.0f);
  if (pr.variant == 2) hp.fscale.assign(size_t(Q) * hp.Fp, 1.0f);
  for (int j = 0; j < F; ++j) {
    const int f = hp.face_old[j];
    const int32_t s0 = m.face_cells[2 * f], s1 = m.face_cells[2 * f + 1];
    const float d0 = m.face_dists[2 * f], d1 = m.face_dists[2 * f + 1];
    hp.fs0[j] = cnew(s0);
    hp.fs1[j] = cnew(s1);
    hp.fnx[j] = m.face_n[2 * f];
    hp.fny[j] = m.face_n[2 * f + 1];
    if (!std::isfinite(hp.fnx[j]) || !std::isfinite(hp.fny[j])) hp.finite_n = false;
    hp.fL[j] = m.face_L[f];
    const float D = d0 + d1;
    hp.fr[j] = d0 / D;
    hp.fD2[j] = 2.0f * D;
    if (ghost_face[f]) {
      hp.fna[j] = hp.node_dev[wrap(m.face_nodes[2 * f], P)];
      hp.fnb[j] = hp.node_dev[wrap(m.face_nodes[2 * f + 1], P)];
      hp.frl[j] = d0 / d1;
      hp.frr[j] = d1 / d0;
      hp.fkl[j] = cnew_wrap(s1);
      hp.fkr[j] = cnew_wrap(s0);
    }
    if (pr.variant == 1) hp.fscale[j] = m.face_scale[f];
    if (pr.variant == 2)
      for (int q = 0; q < Q; ++q) hp.fscale[size_t(q) * hp.Fp + j] = m.face_scale[size_t(f) * Q + q];
  }

  // ---- per-cell face slots: staged gather and fused half faces
  hp.cf_face.assign(size_t(K) * hp.Np, 0);
  hp.cf_sign.assign(size_t(K) * hp.Np, 0.0f);
  hp.fusable = (pr.variant != 2);
  for (int c = 0; c < N && hp.fusable; ++c)
    for (int k = 0; k < K; ++k) {
      const int f = wrap(m.cell_face_indices[int64_t(c) * K + k], F);
      const int32_t s0 = m.face_cells[2 * f], s1 = m.face_cells[2 * f + 1];
      if (!((s0 == c) ^ (s1 == c))) {
        hp.fusable = false;
        break;
      }
    }
  const HfRows HR{K, pr.flux_scheme, pr.variant};
  const HfFastRows HX{K, pr.flux_scheme};
  hp.fast = pr.kernel == FVDBM_KERNEL_FAST && !segs;
  hp.hrows = hp.fast ? HX.rows() : HR.rows();
  auto hfi = [&](int i, int row) { return size_t(i >> 5) * size_t(hp.hrows) * 32 + size_t(row) * 32 + (i & 31); };
  auto fbits = [](float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    return u;
  };
  if (hp.fusable) {
    hp.hf.assign(size_t(hp.Np / 32) * hp.hrows * 32, 0u);
    if (pr.flux_scheme == FVDBM_LAX_WENDROFF && !hp.fast)
      for (int i = 0; i < hp.Np; ++i)
        for (int k = 0; k < K; ++k) hp.hf[hfi(i, HR.d2(k))] = fbits(1.0f);
  }
  for (int i = 0; i < N; ++i) {
    const int c = hp.cell_old[i];
    for (int k = 0; k < K; ++k) {
      const int f = wrap(m.cell_face_indices[int64_t(c) * K + k], F);
      const int32_t sg = m.cell_face_signs[int64_t(c) * K + k];
      const size_t s = size_t(k) * hp.Np + i;
      const int j = hp.face_new[f];
      hp.cf_face[s] = j;
      hp.cf_sign[s] = float(sg);
      if (!hp.fusable) continue;
      const int32_t s0 = m.face_cells[2 * f], s1 = m.face_cells[2 * f + 1];
      const bool slot1 = (s1 == c);
      const int32_t oth = slot1 ? s0 : s1;
      int32_t code = (sg + 1) | (slot1 ? HF_SLOT1 : 0);
      if (oth == -1) {
        const int g = int(hp.gh_a.size());
        hp.gh_a.push_back(hp.fna[j]);
        hp.gh_b.push_back(hp.fnb[j]);
        hp.gh_r.push_back(slot1 ? hp.frl[j] : hp.frr[j]);
        code |= HF_GHOST | (g << HF_SHIFT);
      } else {
        code |= hp.cell_new[oth] << HF_SHIFT;
      }
      if (hp.fast) {
        // a = n * (L*sigma [*scale] [/area]), rounded once from double
        double s = double(hp.fL[j]) * double(sg);
        if (pr.variant == 1) s *= double(hp.fscale[j]);
        if (hp.fv) s *= double(m.cell_inv_area[c]);
        if (pr.flux_scheme == FVDBM_UPWIND) code = (code & ~HF_SLOT1) | (slot1 != (s < 0.0) ? HF_SLOT1 : 0);
        hp.hf[hfi(i, HX.code(k))] = uint32_t(code);
        hp.hf[hfi(i, HX.ax(k))] = fbits(float(double(hp.fnx[j]) * s));
        hp.hf[hfi(i, HX.ay(k))] = fbits(float(double(hp.fny[j]) * s));
        if (pr.flux_scheme == FVDBM_LAX_WENDROFF) {
          hp.hf[hfi(i, HX.r(k))] = fbits(hp.fr[j]);
          const double den = double(hp.fD2[j]) * s;
          hp.hf[hfi(i, HX.g(k))] = fbits(den != 0.0 ? float(double(pr.delta_t) / den) : 0.0f);
        }
        continue;
      }
      hp.hf[hfi(i, HR.code(k))] = uint32_t(code);
      hp.hf[hfi(i, HR.nx(k))] = fbits(hp.fnx[j]);
      hp.hf[hfi(i, HR.ny(k))] = fbits(hp.fny[j]);
      // ((phi*v)*L)*sigma == (phi*v)*(L*sigma) exactly for sigma in {-1,0,1}
      hp.hf[hfi(i, HR.ls(k))] = fbits(hp.fL[j] * float(sg));
      if (pr.flux_scheme == FVDBM_LAX_WENDROFF) {
        hp.hf[hfi(i, HR.r(k))] = fbits(hp.fr[j]);
        hp.hf[hfi(i, HR.d2(k))] = fbits(hp.fD2[j]);
      }
      if (pr.variant == 1) hp.hf[hfi(i, HR.sc(k))] = fbits(hp.fscale[j]);
    }
  }
  if (hp.fusable) {
    hp.cblk_ghost.assign((N + 255) / 256, 0);
    for (int i = 0; i < N; ++i)
      for (int k = 0; k < K; ++k)
        if (hp.hf[hfi(i, HR.code(k))] & HF_GHOST) hp.cblk_ghost[i / 256] = 1;
  }

  // ---- tile tables: per tile the nodes its ghost faces need (plus owner-only
  // computed nodes that no ghost face uses), their stencil entries, and the
  // ghost end nodes as tile-local indices
  if (hp.fusable && N > 0) {
    const int NT = (N + TILE - 1) / TILE;
    const int G = int(hp.gh_a.size());
    std::vector<char> referenced(hp.M, 0);
    for (int g = 0; g < G; ++g) referenced[hp.gh_a[g]] = referenced[hp.gh_b[g]] = 1;
    std::vector<std::vector<int32_t>> extra(NT);
    for (int d = 0; d < hp.Mc; ++d)
      if (!referenced[d]) {
        int t = 0;
        if (hp.nd_ptr[d + 1] > hp.nd_ptr[d]) t = int(hp.nd_cell[hp.nd_ptr[d]] & ~ND_NEQ_ZERO) / TILE;
        extra[t].push_back(d);
      }
    std::vector<int32_t> mark(hp.M, -1), local(hp.M, -1);
    std::vector<char> owned(hp.M, 0);
    hp.tgh_a.assign(G, 0);
    hp.tgh_b.assign(G, 0);
    hp.tn_ptr.assign(1, 0);
    hp.te_ptr.assign(1, 0);
    bool ok = true;
    for (int t = 0; t < NT && ok; ++t) {
      std::vector<int32_t> list;
      auto add = [&](int32_t d) {
        if (mark[d] != t) {
          mark[d] = t;
          local[d] = int(list.size());
          list.push_back(d);
        }
      };
      const int i1 = std::min(N, (t + 1) * TILE);
      for (int i = t * TILE; i < i1; ++i)
        for (int k = 0; k < K; ++k) {
          const int32_t code = int32_t(hp.hf[hfi(i, HR.code(k))]);
          if (!(code & HF_GHOST)) continue;
          const int g = code >> HF_SHIFT;
          add(hp.gh_a[g]);
          add(hp.gh_b[g]);
          hp.tgh_a[g] = local[hp.gh_a[g]];
          hp.tgh_b[g] = local[hp.gh_b[g]];
        }
      for (int32_t d : extra[t]) add(d);
      const int e_start = int(hp.te_cell.size());
      for (int32_t d : list) {
        int kind = 0, npad = 0, e0 = 0, ecnt = 0;
        float sumw = 0.0f;
        if (d < hp.Mc) {
          kind = hp.nd_type[d];
          if (!owned[d]) {
            owned[d] = 1;
            kind |= TN_OWNER;
          }
          sumw = hp.nd_sumw[d];
          npad = hp.nd_npad[d];
          e0 = int(hp.te_cell.size()) - e_start;
          for (int j = hp.nd_ptr[d]; j < hp.nd_ptr[d + 1]; ++j) {
            hp.te_cell.push_back(hp.nd_cell[j]);
            hp.te_w.push_back(hp.nd_w[j]);
          }
          ecnt = hp.nd_ptr[d + 1] - hp.nd_ptr[d];
        }
        hp.tn_dev.push_back(d);
        hp.tn_kind.push_back(kind);
        hp.tn_npad.push_back(npad);
        hp.tn_e0.push_back(e0);
        hp.tn_ecnt.push_back(ecnt);
        hp.tn_sumw.push_back(sumw);
      }
      if (int(list.size()) > TILE_MAX_NODES || int(hp.te_cell.size()) - e_start > TILE_MAX_ENTRIES)
        ok = false;
      hp.tn_ptr.push_back(int(hp.tn_dev.size()));
      hp.te_ptr.push_back(int(hp.te_cell.size()));
    }
    hp.NT = NT;
    hp.tile_ok = ok;
  }

  // single-launch schedule: ticket -> work item (>= 0 cell block, < 0 node
  // block -(b+1)).  Node blocks are spread evenly over the first two thirds of
  // the ghost-free cell blocks; the cell blocks with ghost faces come last.
  if (hp.fusable && N > 0) {
    std::vector<int32_t> free_blocks, ghost_blocks;
    for (int b = 0; b < int(hp.cblk_ghost.size()); ++b)
      (hp.cblk_ghost[b] ? ghost_blocks : free_blocks).push_back(b);
    const int NBk = int(hp.nb_meta.size() / 4);
    const int64_t span = std::max<int64_t>(1, (int64_t(free_blocks.size()) * 2) / 3);
    hp.sched.clear();
    int nb_next = 0;
    for (size_t j = 0; j < free_blocks.size(); ++j) {
      // node blocks due before this cell block
      const int64_t due = std::min<int64_t>(NBk, (int64_t(j) * NBk + span - 1) / span);
      while (nb_next < due) hp.sched.push_back(-(nb_next++ + 1));
      hp.sched.push_back(free_blocks[j]);
    }
    while (nb_next < NBk) hp.sched.push_back(-(nb_next++ + 1));
    for (int32_t b : ghost_blocks) hp.sched.push_back(b);
  }

  if (hp.fv) {
    hp.inv_area.assign(hp.Np, 0.0f);
    for (int i = 0; i < N; ++i) hp.inv_area[i] = m.cell_inv_area[hp.cell_old[i]];
  }
  if (m.cell_area) {
    hp.area.assign(hp.Np, 0.0f);
    for (int i = 0; i < N; ++i) hp.area[i] = m.cell_area[hp.cell_old[i]];
  }
  if (segs) {
    // cases keep their ranges: the order is a permutation within each case
    hp.S = segs->S;
    hp.case_cell.assign(segs->cell_ptr, segs->cell_ptr + segs->S + 1);
    hp.cell_case.assign(hp.Np, 0);
    for (int s = 0; s < segs->S; ++s)
      for (int i = segs->cell_ptr[s]; i < segs->cell_ptr[s + 1]; ++i) hp.cell_case[i] = s;
    for (int i = N; i < hp.Np; ++i) hp.cell_case[i] = segs->S - 1;
  }

  // algorithmic bytes of one step: pdf read+write, cell->face slots, face
  // geometry (2 slot ints + n + L, + 2 distances for Lax-Wendroff) and the
  // boundary-node pdf write + read
  hp.bytes_per_step = 8.0 * hp.q * N + 4.0 * K * N + 20.0 * F +
                      (pr.flux_scheme == FVDBM_LAX_WENDROFF ? 8.0 * F : 0.0) + 8.0 * hp.q * hp.Mc;
  return "";
}

}  // namespace fvdbm
