// tdy_mesh.cpp -- z-extruded mesh construction and geometry.
//
// Restates, for meshes extruded in z from a surface of triangles or
// quadrilaterals, what TDyMeshCreateFromPlex (src/fv/share/tdymeshplex.c:3685)
// derives from a DMPlex: cell/face/vertex connectivity, face normals, face and
// cell centroids, areas and volumes, and the face orientation convention of
// UpdateCellOrientationAroundAFace (tdymeshplex.c:3061-3172):
//   * the face normal points from face_cell0 ("up") to face_cell1 ("dn");
//   * a boundary face has face_cell0 = -(b+1) (boundary index b, numbered in
//     face order as in IdentifyLocalFaces, tdymeshplex.c:405-424) and an
//     inward normal.
// Face normals use the reference formulas TDyUnitNormalToTriangle and
// TDyNormalToQuadrilateral (src/tdyutils.c:400-440).  Areas, centroids and
// volumes (computed by PETSc's DMPlexComputeCellGeometryFVM in the reference)
// come from a fan triangulation about the vertex average: exact for planar
// faces and planar-faced cells.
#include <algorithm>
#include <cmath>
#include <map>

#include "tdy_internal.h"

namespace tdy {

namespace {

inline void sub3(const double *a, const double *b, double *c) {
  c[0] = a[0] - b[0];
  c[1] = a[1] - b[1];
  c[2] = a[2] - b[2];
}
inline void cross3(const double *a, const double *b, double *c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
inline double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// TDyUnitNormalToTriangle (src/tdyutils.c:400): ((n2-n1) x (n3-n1)) / |.|
void unit_normal_tri(const double *n1, const double *n2, const double *n3, double *nrm) {
  double a[3], b[3];
  sub3(n2, n1, a);
  sub3(n3, n1, b);
  cross3(a, b, nrm);
  double s = 0.0;
  for (int d = 0; d < 3; d++) s += nrm[d] * nrm[d];
  s = std::sqrt(s);
  for (int d = 0; d < 3; d++) nrm[d] = nrm[d] / s;
}

// TDyNormalToQuadrilateral (src/tdyutils.c:414): mean of the four unit normals
// of the triangles formed with the vertex average.
void normal_quad(const double *v1, const double *v2, const double *v3, const double *v4, double *nrm) {
  double c[3], n12[3], n23[3], n34[3], n41[3];
  for (int d = 0; d < 3; d++) c[d] = (v1[d] + v2[d] + v3[d] + v4[d]) / 4.0;
  unit_normal_tri(c, v1, v2, n12);
  unit_normal_tri(c, v2, v3, n23);
  unit_normal_tri(c, v3, v4, n34);
  unit_normal_tri(c, v4, v1, n41);
  for (int d = 0; d < 3; d++) nrm[d] = (n12[d] + n23[d] + n34[d] + n41[d]) / 4.0;
}

// Area and centroid of a (possibly non-planar) polygon from the fan of
// triangles about its vertex average.
void polygon_geometry(int n, const double *const *p, double *area, double *cen) {
  double c0[3] = {0, 0, 0};
  for (int i = 0; i < n; i++)
    for (int d = 0; d < 3; d++) c0[d] += p[i][d];
  for (int d = 0; d < 3; d++) c0[d] /= n;
  double asum = 0.0, csum[3] = {0, 0, 0};
  for (int i = 0; i < n; i++) {
    const double *a = p[i], *b = p[(i + 1) % n];
    double u[3], v[3], w[3];
    sub3(a, c0, u);
    sub3(b, c0, v);
    cross3(u, v, w);
    double at = 0.5 * std::sqrt(dot3(w, w));
    asum += at;
    for (int d = 0; d < 3; d++) csum[d] += at * (c0[d] + a[d] + b[d]) / 3.0;
  }
  *area = asum;
  for (int d = 0; d < 3; d++) cen[d] = csum[d] / asum;
}

}  // namespace

int build_extruded_mesh(const ExtrudedInput &in, Mesh &m) {
  const int nv2 = in.nv2, nc2 = in.nc2, nvpc = in.nvpc, nl = in.nlayers;
  if (nv2 <= 0 || nc2 <= 0 || nl <= 0) return set_error(TDY_ERR_ARG_OUTOFRANGE, "empty extruded mesh");
  if (nvpc != 3 && nvpc != 4) return set_error(TDY_ERR_SUP, "surface polygons must have 3 or 4 vertices");

  m = Mesh();
  m.nv = (nl + 1) * nv2;
  m.nc = nl * nc2;
  m.vx.resize(3 * (size_t)m.nv);
  for (int l = 0; l <= nl; l++)
    for (int v = 0; v < nv2; v++) {
      size_t id = (size_t)l * nv2 + v;
      m.vx[3 * id + 0] = in.xy[2 * v + 0];
      m.vx[3 * id + 1] = in.xy[2 * v + 1];
      m.vx[3 * id + 2] = in.z[id];
    }

  // Surface edges, their adjacent surface polygons, and polygon -> edges.
  std::map<std::pair<int, int>, int> edge_id;
  std::vector<std::pair<int, int>> edges;
  std::vector<std::vector<int>> edge_cells;
  std::vector<int> poly_edges((size_t)nc2 * nvpc);
  for (int c = 0; c < nc2; c++) {
    for (int k = 0; k < nvpc; k++) {
      int a = in.cells2d[(size_t)c * nvpc + k], b = in.cells2d[(size_t)c * nvpc + (k + 1) % nvpc];
      if (a < 0 || a >= nv2 || b < 0 || b >= nv2 || a == b)
        return set_error(TDY_ERR_ARG_OUTOFRANGE, "surface polygon %d has an invalid vertex", c);
      auto key = std::make_pair(std::min(a, b), std::max(a, b));
      auto it = edge_id.find(key);
      int e;
      if (it == edge_id.end()) {
        e = (int)edges.size();
        edge_id[key] = e;
        edges.push_back({a, b});
        edge_cells.emplace_back();
      } else {
        e = it->second;
      }
      edge_cells[e].push_back(c);
      if (edge_cells[e].size() > 2) return set_error(TDY_ERR_ARG_WRONG, "surface edge shared by >2 polygons");
      poly_edges[(size_t)c * nvpc + k] = e;
    }
  }
  const int ne2 = (int)edges.size();

  // Faces: horizontal faces (level l, polygon c) first, then vertical faces
  // (layer k, edge e).
  const int nfh = (nl + 1) * nc2;
  m.nf = nfh + nl * ne2;
  m.face_vert_off.assign(m.nf + 1, 0);
  std::vector<std::vector<int>> fcells(m.nf);
  for (int l = 0; l <= nl; l++)
    for (int c = 0; c < nc2; c++) {
      int f = l * nc2 + c;
      m.face_vert_off[f + 1] = nvpc;
      if (l >= 1) fcells[f].push_back((l - 1) * nc2 + c);
      if (l < nl) fcells[f].push_back(l * nc2 + c);
    }
  for (int k = 0; k < nl; k++)
    for (int e = 0; e < ne2; e++) {
      int f = nfh + k * ne2 + e;
      m.face_vert_off[f + 1] = 4;
      for (int c : edge_cells[e]) fcells[f].push_back(k * nc2 + c);
      std::sort(fcells[f].begin(), fcells[f].end());
    }
  for (int f = 0; f < m.nf; f++) m.face_vert_off[f + 1] += m.face_vert_off[f];
  m.face_verts.resize(m.face_vert_off[m.nf]);
  for (int l = 0; l <= nl; l++)
    for (int c = 0; c < nc2; c++) {
      int f = l * nc2 + c, o = m.face_vert_off[f];
      for (int k = 0; k < nvpc; k++) m.face_verts[o + k] = l * nv2 + in.cells2d[(size_t)c * nvpc + k];
    }
  for (int k = 0; k < nl; k++)
    for (int e = 0; e < ne2; e++) {
      int f = nfh + k * ne2 + e, o = m.face_vert_off[f];
      int a = edges[e].first, b = edges[e].second;
      m.face_verts[o + 0] = k * nv2 + a;
      m.face_verts[o + 1] = k * nv2 + b;
      m.face_verts[o + 2] = (k + 1) * nv2 + b;
      m.face_verts[o + 3] = (k + 1) * nv2 + a;
    }

  // Cells: vertices (bottom polygon then top polygon) and faces.
  const int nfpc = 2 + nvpc;
  m.cell_vert_off.resize(m.nc + 1);
  m.cell_face_off.resize(m.nc + 1);
  for (int i = 0; i <= m.nc; i++) {
    m.cell_vert_off[i] = 2 * nvpc * i;
    m.cell_face_off[i] = nfpc * i;
  }
  m.cell_verts.resize((size_t)2 * nvpc * m.nc);
  m.cell_faces.resize((size_t)nfpc * m.nc);
  for (int k = 0; k < nl; k++)
    for (int c = 0; c < nc2; c++) {
      int cell = k * nc2 + c;
      for (int j = 0; j < nvpc; j++) {
        int v2 = in.cells2d[(size_t)c * nvpc + j];
        m.cell_verts[(size_t)cell * 2 * nvpc + j] = k * nv2 + v2;
        m.cell_verts[(size_t)cell * 2 * nvpc + nvpc + j] = (k + 1) * nv2 + v2;
      }
      int *cf = &m.cell_faces[(size_t)cell * nfpc];
      cf[0] = k * nc2 + c;
      cf[1] = (k + 1) * nc2 + c;
      for (int j = 0; j < nvpc; j++) cf[2 + j] = nfh + k * ne2 + poly_edges[(size_t)c * nvpc + j];
    }

  // Face geometry.
  m.face_cen.resize(3 * (size_t)m.nf);
  m.face_nrm.resize(3 * (size_t)m.nf);
  m.face_area.resize(m.nf);
  for (int f = 0; f < m.nf; f++) {
    int o = m.face_vert_off[f], n = m.face_vert_off[f + 1] - o;
    const double *p[4];
    for (int k = 0; k < n; k++) p[k] = &m.vx[3 * (size_t)m.face_verts[o + k]];
    polygon_geometry(n, p, &m.face_area[f], &m.face_cen[3 * (size_t)f]);
    if (n == 3)
      unit_normal_tri(p[0], p[1], p[2], &m.face_nrm[3 * (size_t)f]);
    else
      normal_quad(p[0], p[1], p[2], p[3], &m.face_nrm[3 * (size_t)f]);
  }

  // Cell geometry: tetrahedra from the cell vertex average to the fan
  // triangles of every face.
  m.cell_cen.resize(3 * (size_t)m.nc);
  m.cell_vol.resize(m.nc);
  for (int c = 0; c < m.nc; c++) {
    double apex[3] = {0, 0, 0};
    int vo = m.cell_vert_off[c], vn = m.cell_vert_off[c + 1] - vo;
    for (int k = 0; k < vn; k++)
      for (int d = 0; d < 3; d++) apex[d] += m.vx[3 * (size_t)m.cell_verts[vo + k] + d];
    for (int d = 0; d < 3; d++) apex[d] /= vn;
    double vsum = 0.0, csum[3] = {0, 0, 0};
    for (int j = m.cell_face_off[c]; j < m.cell_face_off[c + 1]; j++) {
      int f = m.cell_faces[j], o = m.face_vert_off[f], n = m.face_vert_off[f + 1] - o;
      double c0[3] = {0, 0, 0};
      for (int k = 0; k < n; k++)
        for (int d = 0; d < 3; d++) c0[d] += m.vx[3 * (size_t)m.face_verts[o + k] + d];
      for (int d = 0; d < 3; d++) c0[d] /= n;
      for (int k = 0; k < n; k++) {
        const double *a = &m.vx[3 * (size_t)m.face_verts[o + k]];
        const double *b = &m.vx[3 * (size_t)m.face_verts[o + (k + 1) % n]];
        double u[3], v[3], w[3], x[3];
        sub3(a, apex, u);
        sub3(b, apex, v);
        sub3(c0, apex, w);
        cross3(u, v, x);
        double vol = std::fabs(dot3(x, w)) / 6.0;
        vsum += vol;
        for (int d = 0; d < 3; d++) csum[d] += vol * (apex[d] + c0[d] + a[d] + b[d]) / 4.0;
      }
    }
    m.cell_vol[c] = vsum;
    for (int d = 0; d < 3; d++) m.cell_cen[3 * (size_t)c + d] = csum[d] / vsum;
  }

  // Orientation: normal from cell0 to cell1; boundary side first, inward.
  m.face_cell0.assign(m.nf, 0);
  m.face_cell1.assign(m.nf, 0);
  m.face_bnd.assign(m.nf, -1);
  m.nb = 0;
  for (int f = 0; f < m.nf; f++) {
    double *nrm = &m.face_nrm[3 * (size_t)f];
    const double *fc = &m.face_cen[3 * (size_t)f];
    bool flip;
    if (fcells[f].size() == 2) {
      int c0 = fcells[f][0], c1 = fcells[f][1];
      double d[3];
      sub3(&m.cell_cen[3 * (size_t)c1], &m.cell_cen[3 * (size_t)c0], d);
      flip = dot3(nrm, d) < 0.0;
      m.face_cell0[f] = c0;
      m.face_cell1[f] = c1;
    } else if (fcells[f].size() == 1) {
      int c = fcells[f][0];
      double d[3];
      sub3(&m.cell_cen[3 * (size_t)c], fc, d);
      flip = dot3(nrm, d) < 0.0;
      m.face_bnd[f] = m.nb;
      m.face_cell0[f] = -(m.nb + 1);
      m.face_cell1[f] = c;
      m.bnd_face.push_back(f);
      m.nb++;
    } else {
      return set_error(TDY_ERR_ARG_WRONG, "face %d has no cell", f);
    }
    if (flip) {
      for (int d = 0; d < 3; d++) nrm[d] = -nrm[d];
      std::reverse(m.face_verts.begin() + m.face_vert_off[f], m.face_verts.begin() + m.face_vert_off[f + 1]);
    }
  }

  // Vertex -> cells (ascending) and vertex -> faces (internal first).
  std::vector<std::vector<int>> vc(m.nv), vfi(m.nv), vfb(m.nv);
  for (int c = 0; c < m.nc; c++)
    for (int j = m.cell_vert_off[c]; j < m.cell_vert_off[c + 1]; j++) vc[m.cell_verts[j]].push_back(c);
  for (int f = 0; f < m.nf; f++)
    for (int j = m.face_vert_off[f]; j < m.face_vert_off[f + 1]; j++)
      (m.face_bnd[f] < 0 ? vfi : vfb)[m.face_verts[j]].push_back(f);
  m.vert_cell_off.assign(m.nv + 1, 0);
  m.vert_face_off.assign(m.nv + 1, 0);
  for (int v = 0; v < m.nv; v++) {
    std::sort(vc[v].begin(), vc[v].end());
    std::sort(vfi[v].begin(), vfi[v].end());
    std::sort(vfb[v].begin(), vfb[v].end());
    m.vert_cell_off[v + 1] = m.vert_cell_off[v] + (int)vc[v].size();
    m.vert_face_off[v + 1] = m.vert_face_off[v] + (int)(vfi[v].size() + vfb[v].size());
  }
  m.vert_cells.reserve(m.vert_cell_off[m.nv]);
  m.vert_faces.reserve(m.vert_face_off[m.nv]);
  for (int v = 0; v < m.nv; v++) {
    m.vert_cells.insert(m.vert_cells.end(), vc[v].begin(), vc[v].end());
    m.vert_faces.insert(m.vert_faces.end(), vfi[v].begin(), vfi[v].end());
    m.vert_faces.insert(m.vert_faces.end(), vfb[v].begin(), vfb[v].end());
  }
  return 0;
}

void merge_meshes(const std::vector<Mesh> &parts, Mesh &m) {
  m = Mesh();
  m.cell_vert_off.push_back(0);
  m.cell_face_off.push_back(0);
  m.face_vert_off.push_back(0);
  m.vert_cell_off.push_back(0);
  m.vert_face_off.push_back(0);
  for (const Mesh &p : parts) {
    const int v0 = m.nv, c0 = m.nc, f0 = m.nf, b0 = m.nb;
    auto append = [](std::vector<int> &dst, const std::vector<int> &src, int add) {
      for (int x : src) dst.push_back(x + add);
    };
    auto append_off = [](std::vector<int> &dst, const std::vector<int> &src) {
      const int base = dst.back();
      for (size_t i = 1; i < src.size(); i++) dst.push_back(src[i] + base);
    };
    m.vx.insert(m.vx.end(), p.vx.begin(), p.vx.end());
    append_off(m.cell_vert_off, p.cell_vert_off);
    append(m.cell_verts, p.cell_verts, v0);
    append_off(m.cell_face_off, p.cell_face_off);
    append(m.cell_faces, p.cell_faces, f0);
    m.cell_cen.insert(m.cell_cen.end(), p.cell_cen.begin(), p.cell_cen.end());
    m.cell_vol.insert(m.cell_vol.end(), p.cell_vol.begin(), p.cell_vol.end());
    append_off(m.face_vert_off, p.face_vert_off);
    append(m.face_verts, p.face_verts, v0);
    // reference encoding: cell id, or -(boundary index + 1)
    for (int x : p.face_cell0) m.face_cell0.push_back(x >= 0 ? x + c0 : x - b0);
    for (int x : p.face_cell1) m.face_cell1.push_back(x >= 0 ? x + c0 : x - b0);
    m.face_cen.insert(m.face_cen.end(), p.face_cen.begin(), p.face_cen.end());
    m.face_nrm.insert(m.face_nrm.end(), p.face_nrm.begin(), p.face_nrm.end());
    m.face_area.insert(m.face_area.end(), p.face_area.begin(), p.face_area.end());
    for (int x : p.face_bnd) m.face_bnd.push_back(x >= 0 ? x + b0 : x);
    append(m.bnd_face, p.bnd_face, f0);
    append_off(m.vert_cell_off, p.vert_cell_off);
    append(m.vert_cells, p.vert_cells, c0);
    append_off(m.vert_face_off, p.vert_face_off);
    append(m.vert_faces, p.vert_faces, f0);
    m.nv += p.nv;
    m.nc += p.nc;
    m.nf += p.nf;
    m.nb += p.nb;
  }
}

}  // namespace tdy
