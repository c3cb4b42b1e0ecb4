// Packed batch: the disjoint union of independent cases' meshes, so that one
// launch per kernel steps all of them.  The reference steps one Environment
// at a time; a case of the union evolves exactly as it would alone:
//   * indices are offset into the union, so nothing refers across cases;
//   * the reference's padded -1 entries keep their per-case meaning: a -1
//     face slot or face node names the case's last face / node (explicitly),
//     and a -1 node-stencil entry stays -1 and is wrapped to the case's last
//     cell by the plan (it still contributes no non-equilibrium part);
//   * node stencils of a case with fewer columns than the widest case are
//     padded with (-1, -1) entries, which carry weight 0.
#include <string>
#include <vector>

#include "../../include/fvdbm.h"
#include "fvdbm_internal.h"

namespace fvdbm {

std::string build_union(const fvdbm_mesh_t* meshes, int S, UnionMesh& u) {
  if (S <= 0) return "a batch needs at least one case";
  const int K = meshes[0].cell_face_stride;
  int Kn = 0;
  bool xy = true, ia = true, area = true;
  int64_t N = 0, F = 0, P = 0;
  for (int s = 0; s < S; ++s) {
    const fvdbm_mesh_t& m = meshes[s];
    if (m.n_cells <= 0) return "batch case " + std::to_string(s) + " has no cells";
    if (m.cell_face_stride != K) return "batch cases must have the same number of face slots per cell";
    if (m.face_scale) return "a batch takes no flux-scale variant";
    if (!m.cell_face_indices || !m.cell_face_signs || (m.n_faces > 0 && (!m.face_cells || !m.face_dists ||
        !m.face_nodes || !m.face_n || !m.face_L)) || (m.n_nodes > 0 && !m.node_type))
      return "batch case " + std::to_string(s) + ": arrays missing";
    if (m.n_nodes > 0 && m.node_cell_stride > 0 && (!m.node_cells || !m.node_dists))
      return "batch case " + std::to_string(s) + ": node stencil arrays missing";
    Kn = std::max(Kn, m.node_cell_stride);
    xy = xy && m.cell_xy;
    ia = ia && m.cell_inv_area;
    area = area && m.cell_area;
    if (s > 0 && (m.cell_inv_area != nullptr) != (meshes[0].cell_inv_area != nullptr))
      return "batch cases must all give cell_inv_area or none";
    N += m.n_cells;
    F += m.n_faces;
    P += m.n_nodes;
  }
  if (N > HF_MAX_INDEX || F > HF_MAX_INDEX || P > HF_MAX_INDEX) return "batch too large";
  u.K = K;
  u.Kn = Kn;
  u.cell_ptr.assign(1, 0);
  u.face_ptr.assign(1, 0);
  u.node_ptr.assign(1, 0);
  u.cfi.clear();
  u.cfs.clear();
  u.fc.clear();
  u.fnd.clear();
  u.fd.clear();
  u.fn.clear();
  u.fL.clear();
  u.nt.clear();
  u.nc.clear();
  u.nd.clear();
  u.xy.clear();
  u.ia.clear();
  u.area.clear();
  for (int s = 0; s < S; ++s) {
    const fvdbm_mesh_t& m = meshes[s];
    const int c0 = u.cell_ptr.back(), f0 = u.face_ptr.back(), n0 = u.node_ptr.back();
    const int n = m.n_cells, f = m.n_faces, p = m.n_nodes;
    for (int64_t t = 0; t < int64_t(n) * K; ++t) {
      const int32_t fi = m.cell_face_indices[t];
      if (fi < -1 || fi >= f) return "batch case " + std::to_string(s) + ": a face index is out of range";
      u.cfi.push_back(f0 + (fi < 0 ? f - 1 : fi));
      u.cfs.push_back(m.cell_face_signs[t]);
    }
    for (int64_t t = 0; t < int64_t(f) * 2; ++t) {
      const int32_t c = m.face_cells[t], nd = m.face_nodes[t];
      if (c < -1 || c >= n || nd < -1 || nd >= p || p == 0)
        return "batch case " + std::to_string(s) + ": a face index is out of range";
      u.fc.push_back(c < 0 ? -1 : c0 + c);
      u.fnd.push_back(n0 + (nd < 0 ? p - 1 : nd));
      u.fd.push_back(m.face_dists[t]);
      u.fn.push_back(m.face_n[t]);
    }
    for (int j = 0; j < f; ++j) u.fL.push_back(m.face_L[j]);
    for (int q = 0; q < p; ++q) {
      u.nt.push_back(m.node_type[q]);
      for (int k = 0; k < Kn; ++k) {
        if (k < m.node_cell_stride) {
          const int32_t c = m.node_cells[int64_t(q) * m.node_cell_stride + k];
          if (c < -1 || c >= n) return "batch case " + std::to_string(s) + ": a node index is out of range";
          u.nc.push_back(c < 0 ? -1 : c0 + c);
          u.nd.push_back(m.node_dists[int64_t(q) * m.node_cell_stride + k]);
        } else {
          u.nc.push_back(-1);
          u.nd.push_back(-1.0f);
        }
      }
    }
    for (int i = 0; i < n; ++i) {
      if (xy) {
        u.xy.push_back(m.cell_xy[2 * i]);
        u.xy.push_back(m.cell_xy[2 * i + 1]);
      }
      if (ia) u.ia.push_back(m.cell_inv_area[i]);
      if (area) u.area.push_back(m.cell_area[i]);
    }
    u.cell_ptr.push_back(c0 + n);
    u.face_ptr.push_back(f0 + f);
    u.node_ptr.push_back(n0 + p);
  }
  fvdbm_mesh_t& m = u.mesh;
  m = fvdbm_mesh_t{};
  m.n_cells = int(N);
  m.n_faces = int(F);
  m.n_nodes = int(P);
  m.cell_face_stride = K;
  m.node_cell_stride = Kn;
  m.cell_face_indices = u.cfi.data();
  m.cell_face_signs = u.cfs.data();
  m.face_cells = u.fc.data();
  m.face_dists = u.fd.data();
  m.face_nodes = u.fnd.data();
  m.face_n = u.fn.data();
  m.face_L = u.fL.data();
  m.face_scale = nullptr;
  m.node_type = u.nt.data();
  m.node_cells = u.nc.data();
  m.node_dists = u.nd.data();
  m.cell_xy = xy ? u.xy.data() : nullptr;
  m.cell_inv_area = ia ? u.ia.data() : nullptr;
  m.cell_area = area ? u.area.data() : nullptr;
  u.segs = BatchSegs{S, u.cell_ptr.data(), u.face_ptr.data(), u.node_ptr.data()};
  return "";
}

}  // namespace fvdbm
