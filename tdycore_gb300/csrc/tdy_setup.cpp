// tdy_setup.cpp -- MPFA-O setup on the host, run once by TDySetup.
//
// Restates the reference's setup chain (src/fv/mpfao/tdympfao.c):
//   SetupSubcells (tdymeshplex.c:2829-3059)      -> subcell faces, nu vectors, T
//   ComputeGMatrix_MPFAO / _TPF (tdympfao.c:39-274)
//   ComputeTransmissibilityMatrix (tdympfao.c:1126-1860)
//   ComputeGravityDiscretization (tdympfao.c:2169-2274)
//   DMCreateMatrix FVM++ adjacency (src/tdydiscretization.c:156-170)
// and lays the results out for the device kernels.
//
// The per-vertex interaction-region system is formed directly from flux
// continuity: for an internal subface the flux computed from the subcell of
// face_cell0 equals the flux computed from the subcell of face_cell1; for a
// Neumann subface the flux is zero; Dirichlet/seepage subfaces are known
// pressures.  This is the same linear system the reference assembles through
// its Cup/Cdn/Fup/Fdn blocks (tdympfao.c:1000-1449), with rows and columns in
// a different (equivalent) order, so Trans agrees with the reference's to
// rounding.  The flux of an internal subface is taken from the face_cell0
// subcell; the reference picks one of the two subcells by its traversal
// order (tdymeshplex.c:1531-1622), which is equal at the solution.
#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <cstring>

#include "tdy_internal.h"

namespace tdy {

namespace {

inline double dot3(const double *a, const double *b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline void cross3(const double *a, const double *b, double *c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
// TDyComputeLength (src/tdyutils.c:239)
inline double length3(const double *a, const double *b) {
  double s = 0.0;
  for (int d = 0; d < 3; d++) s += (a[d] - b[d]) * (a[d] - b[d]);
  return std::sqrt(s);
}
// TDyUnitNormalVectorJoiningTwoVertices (src/tdyutils.c:370): (to - from)/|to - from|
inline void unit_from_to(const double *from, const double *to, double *u) {
  double s = 0.0;
  for (int d = 0; d < 3; d++) {
    u[d] = to[d] - from[d];
    s += u[d] * u[d];
  }
  s = std::sqrt(s);
  for (int d = 0; d < 3; d++) u[d] = u[d] / s;
}

// ComputeInverseOf3by3Matrix (src/tdyutils.c:683-718).
void inverse3(const double a[9], double inv[9]) {
  double det = a[0] * (a[4] * a[8] - a[5] * a[7]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
               a[2] * (a[3] * a[7] - a[4] * a[6]);
  inv[0] = +1.0 / det * (a[4] * a[8] - a[7] * a[5]);
  inv[1] = -1.0 / det * (a[1] * a[8] - a[7] * a[2]);
  inv[2] = +1.0 / det * (a[1] * a[5] - a[4] * a[2]);
  inv[3] = -1.0 / det * (a[3] * a[8] - a[6] * a[5]);
  inv[4] = +1.0 / det * (a[0] * a[8] - a[6] * a[2]);
  inv[5] = -1.0 / det * (a[0] * a[5] - a[3] * a[2]);
  inv[6] = +1.0 / det * (a[3] * a[7] - a[6] * a[4]);
  inv[7] = -1.0 / det * (a[0] * a[7] - a[6] * a[1]);
  inv[8] = +1.0 / det * (a[0] * a[4] - a[3] * a[1]);
}

// Dense LU with partial pivoting (first maximal |pivot|, as LAPACK dgetrf)
// solving A X = B in place; A is n x n row-major, B is n x m row-major.
bool lu_solve(int n, int m, std::vector<double> &A, std::vector<double> &B) {
  for (int k = 0; k < n; k++) {
    int p = k;
    double best = std::fabs(A[(size_t)k * n + k]);
    for (int i = k + 1; i < n; i++) {
      double v = std::fabs(A[(size_t)i * n + k]);
      if (v > best) {
        best = v;
        p = i;
      }
    }
    if (best == 0.0) return false;
    if (p != k) {
      for (int j = 0; j < n; j++) std::swap(A[(size_t)k * n + j], A[(size_t)p * n + j]);
      for (int j = 0; j < m; j++) std::swap(B[(size_t)k * m + j], B[(size_t)p * m + j]);
    }
    double piv = A[(size_t)k * n + k];
    for (int i = k + 1; i < n; i++) {
      double l = A[(size_t)i * n + k] / piv;
      if (l == 0.0) continue;
      A[(size_t)i * n + k] = l;
      for (int j = k + 1; j < n; j++) A[(size_t)i * n + j] -= l * A[(size_t)k * n + j];
      for (int j = 0; j < m; j++) B[(size_t)i * m + j] -= l * B[(size_t)k * m + j];
    }
  }
  for (int k = n - 1; k >= 0; k--) {
    double piv = A[(size_t)k * n + k];
    for (int j = 0; j < m; j++) {
      double s = B[(size_t)k * m + j];
      for (int i = k + 1; i < n; i++) s -= A[(size_t)k * n + i] * B[(size_t)i * m + j];
      B[(size_t)k * m + j] = s / piv;
    }
  }
  return true;
}

// Subcell of cell c at its vertex v: three faces meeting at v, ordered so that
// the normal of the plane through their centroids points toward the cell
// centroid (UpdateFaceOrientationAroundAVertex, tdymeshplex.c:1384-1412).
struct Subcell {
  int face[3];
  double nu[3][3];
  double T;
  double area[3];
};

int build_subcell(const Mesh &m, int c, int v, Subcell &sc) {
  int nfound = 0;
  for (int j = m.vert_face_off[v]; j < m.vert_face_off[v + 1]; j++) {
    int f = m.vert_faces[j];
    bool mine = (m.face_cell0[f] == c || m.face_cell1[f] == c);
    if (!mine) continue;
    if (nfound == 3) return set_error(TDY_ERR_SUP, "cell %d has more than 3 faces at vertex %d", c, v);
    sc.face[nfound++] = f;
  }
  if (nfound != 3) return set_error(TDY_ERR_SUP, "cell %d has %d faces at vertex %d (need 3)", c, nfound, v);
  const double *xc = &m.cell_cen[3 * (size_t)c];
  const double *xv = &m.vx[3 * (size_t)v];
  {
    const double *f0 = &m.face_cen[3 * (size_t)sc.face[0]];
    const double *f1 = &m.face_cen[3 * (size_t)sc.face[1]];
    const double *f2 = &m.face_cen[3 * (size_t)sc.face[2]];
    double a[3], b[3], cc[3], axb[3];
    for (int d = 0; d < 3; d++) {
      a[d] = f1[d] - f0[d];
      b[d] = f2[d] - f0[d];
      cc[d] = xc[d] - xv[d];
    }
    cross3(a, b, axb);
    if (dot3(axb, cc) < 0) std::swap(sc.face[1], sc.face[2]);
  }
  const double *fc[3];
  for (int i = 0; i < 3; i++) fc[i] = &m.face_cen[3 * (size_t)sc.face[i]];
  // T = 6 * volume of the tetrahedron (cell centroid, three face centroids)
  // (TDyComputeVolumeOfTetrahedron, src/tdyutils.c:442).
  {
    double a[3], b[3], cc[3], axb[3];
    for (int d = 0; d < 3; d++) {
      a[d] = fc[0][d] - xc[d];
      b[d] = fc[1][d] - xc[d];
      cc[d] = fc[2][d] - xc[d];
    }
    cross3(a, b, axb);
    double vol = std::fabs(dot3(axb, cc)) / 6.0;
    sc.T = vol * 6.0;
  }
  // nu_i = (x_{f(i+1)} - x_c) x (x_{f(i+2)} - x_c)  (tdymeshplex.c:2957-2989)
  static const int nxt[3][2] = {{1, 2}, {2, 0}, {0, 1}};
  for (int i = 0; i < 3; i++) {
    double a[3], b[3];
    for (int d = 0; d < 3; d++) {
      a[d] = fc[nxt[i][0]][d] - xc[d];
      b[d] = fc[nxt[i][1]][d] - xc[d];
    }
    cross3(a, b, sc.nu[i]);
    int f = sc.face[i];
    int nvf = m.face_vert_off[f + 1] - m.face_vert_off[f];
    sc.area[i] = m.face_area[f] / nvf;  // subface area (tdymeshplex.c:2943)
  }
  return 0;
}

// G matrix of a subcell.  MPFA-O: G_ij = (n_i . K nu_j) * A_i / T
// (ComputeEntryOfGMatrix, tdympfao.c:13-37).  TPF: diagonal two-point form
// (ComputeGMatrix_TPF, tdympfao.c:128-274).
void gmatrix(const Mesh &m, const Materials &mat, int method, int c, const Subcell &sc, double G[3][3]) {
  const double *K = &mat.K0[9 * (size_t)c];
  for (int i = 0; i < 3; i++) {
    int f = sc.face[i];
    const double *n = &m.face_nrm[3 * (size_t)f];
    for (int j = 0; j < 3; j++) {
      if (method == MPFAO_GMATRIX_DEFAULT) {
        double Kv[3];
        for (int a = 0; a < 3; a++) {
          Kv[a] = 0.0;
          for (int b = 0; b < 3; b++) Kv[a] += K[a * 3 + b] * sc.nu[j][b];
        }
        double g = 0.0;
        for (int a = 0; a < 3; a++) g += n[a] * Kv[a];
        g *= 1.0 / (sc.T) * sc.area[i];
        G[i][j] = g;
      } else {
        if (i != j) {
          G[i][j] = 0.0;
          continue;
        }
        const double *xc = &m.cell_cen[3 * (size_t)c];
        int nb = (m.face_cell0[f] == c) ? m.face_cell1[f] : m.face_cell0[f];
        const double *xn;
        const double *Kn;
        double dist;
        if (nb >= 0) {
          xn = &m.cell_cen[3 * (size_t)nb];
          dist = length3(xn, xc) * 0.50;
          Kn = &mat.K0[9 * (size_t)nb];
        } else {
          xn = &m.face_cen[3 * (size_t)f];
          dist = length3(xn, xc);
          Kn = K;
        }
        double u[3];
        unit_from_to(xn, xc, u);
        double dp = dot3(n, u);
        double knv = 0.0, kv = 0.0;
        for (int k = 0; k < 3; k++) {
          knv += u[k] * u[k] / Kn[k * 3 + k];
          kv += u[k] * u[k] / K[k * 3 + k];
        }
        knv = 1.0 / knv;
        kv = 1.0 / kv;
        double kav = 0.5 * kv + 0.5 * knv;
        G[i][j] = sc.area[i] * (dp)*kav / (dist);
      }
    }
  }
}

// Face permeability value for the gravity term (tdympfao.c:2008-2143).
double face_perm_value(const Mesh &m, const Materials &mat, int method, int f, const double u[3]) {
  int up = m.face_cell0[f], dn = m.face_cell1[f];
  const double *fc = &m.face_cen[3 * (size_t)f];
  double dup = (up >= 0) ? length3(&m.cell_cen[3 * (size_t)up], fc) : 0.0;
  double ddn = (dn >= 0) ? length3(&m.cell_cen[3 * (size_t)dn], fc) : 0.0;
  double wt_up = dup / (dup + ddn);
  // ExtractUpAndDownPermeabilityTensors stores the transpose.
  double Kup[9], Kdn[9];
  const double *Ku = &mat.K0[9 * (size_t)(up >= 0 ? up : dn)];
  const double *Kd = &mat.K0[9 * (size_t)(dn >= 0 ? dn : up)];
  for (int kk = 0; kk < 3; kk++)
    for (int mm = 0; mm < 3; mm++) {
      Kup[mm * 3 + kk] = Ku[kk * 3 + mm];
      Kdn[mm * 3 + kk] = Kd[kk * 3 + mm];
    }
  if (method == MPFAO_GMATRIX_DEFAULT) {
    double KupInv[9], KdnInv[9], KfInv[9], Kf[9];
    inverse3(Kup, KupInv);
    inverse3(Kdn, KdnInv);
    for (int i = 0; i < 9; i++) KfInv[i] = wt_up * KupInv[i] + (1.0 - wt_up) * KdnInv[i];
    inverse3(KfInv, Kf);
    for (int i = 0; i < 9; i++)
      if (Kf[i] < 0.0 || std::fabs(Kf[i]) < DBL_EPSILON) Kf[i] = 0.0;
    double Kuv[3];
    for (int a = 0; a < 3; a++) {
      Kuv[a] = 0.0;
      for (int b = 0; b < 3; b++) Kuv[a] += Kf[a * 3 + b] * u[b];
    }
    return dot3(&m.face_nrm[3 * (size_t)f], Kuv);
  }
  double kup = 0.0, kdn = 0.0;
  for (int k = 0; k < 3; k++) {
    kup += u[k] * u[k] / Kup[k * 3 + k];
    kdn += u[k] * u[k] / Kdn[k * 3 + k];
  }
  kup = 1.0 / kup;
  kdn = 1.0 / kdn;
  return (kup * kdn) / (wt_up * kdn + (1.0 - wt_up) * kup);
}

}  // namespace

// Octant layout of a vertex with 8 cells and 12 flux rows: the octant of each
// local cell from its centroid relative to the vertex (bit 0 x, bit 1 y,
// bit 2 z) and the canonical row (kCanonUp/kCanonDn) of each vertex row.
// False when the vertex does not fit: two cells in one octant, a boundary
// row, a row joining octants that differ in more than one bit, or a row whose
// first cell is not on the lower side.
bool canonical_layout(const Mesh &m, int v, const int *cells, const int *lup, const int *ldn,
                      std::array<int, 8> &oc, std::array<int, 12> &cr) {
  const double *xv = &m.vx[3 * (size_t)v];
  oc.fill(-1);
  cr.fill(-1);
  int oct_of[8];
  for (int a = 0; a < 8; a++) {
    const double *xc = &m.cell_cen[3 * (size_t)cells[a]];
    int o = (xc[0] > xv[0] ? 1 : 0) | (xc[1] > xv[1] ? 2 : 0) | (xc[2] > xv[2] ? 4 : 0);
    if (oc[o] >= 0) return false;
    oc[o] = a;
    oct_of[a] = o;
  }
  for (int r = 0; r < 12; r++) {
    if (lup[r] < 0 || ldn[r] < 0) return false;
    int ou = oct_of[lup[r]], od = oct_of[ldn[r]];
    int diff = ou ^ od;
    if (diff != 1 && diff != 2 && diff != 4) return false;
    if (ou & diff) return false;  // the face's first cell must be on the lower side
    int k = (diff == 1) ? 0 : (diff == 2) ? 1 : 2;
    int rc = -1;
    for (int j = 0; j < 4; j++)
      if (kCanonUp[4 * k + j] == ou) rc = 4 * k + j;
    if (rc < 0 || cr[rc] >= 0) return false;
    cr[rc] = r;
  }
  return true;
}


int mpfao_setup(const Options &opt, const Mesh &m, const Materials &mat, const Boundary &bnd, MPFAOSetup &s) {
  s = MPFAOSetup();
  const int nc = m.nc, nv = m.nv;
  auto is_neumann = [&](int f) { return m.face_bnd[f] >= 0 && bnd.type[m.face_bnd[f]] == NEUMANN_BC; };
  auto is_dirichlet = [&](int f) { return m.face_bnd[f] >= 0 && bnd.type[m.face_bnd[f]] != NEUMANN_BC; };

  // ---- per-vertex local systems ----
  s.v_row_off.assign(nv + 1, 0);
  s.v_col_off.assign(nv + 1, 0);
  s.v_nint.assign(nv, 0);
  s.v_trans_off.assign(nv + 1, 0);

  std::vector<int> fidx;  // face -> position at the current vertex (scratch)
  std::vector<int> fpos(m.nf, -1);
  for (int v = 0; v < nv; v++) {
    const int c0 = m.vert_cell_off[v], nint = m.vert_cell_off[v + 1] - c0;
    const int f0 = m.vert_face_off[v], nfv = m.vert_face_off[v + 1] - f0;
    if (nint == 0) {
      s.v_row_off[v + 1] = s.v_row_off[v];
      s.v_col_off[v + 1] = s.v_col_off[v];
      s.v_trans_off[v + 1] = s.v_trans_off[v];
      continue;
    }
    // unknown / known numbering of the subfaces at v
    std::vector<int> unk(nfv, -1), knw(nfv, -1), rows;
    int nunk = 0, nknw = 0;
    for (int j = 0; j < nfv; j++) {
      int f = m.vert_faces[f0 + j];
      fpos[f] = j;
      if (is_dirichlet(f))
        knw[j] = nknw++;
      else
        unk[j] = nunk++;
      if (!is_neumann(f)) rows.push_back(j);
    }
    const int ncol = nint + nknw;
    const int nrow = (int)rows.size();
    auto local_cell = [&](int c) {
      for (int a = 0; a < nint; a++)
        if (m.vert_cells[c0 + a] == c) return a;
      return -1;
    };
    // row metadata: face, local up/down cell
    const size_t rbase = s.row_face.size();
    for (int r = 0; r < nrow; r++) {
      int f = m.vert_faces[f0 + rows[r]];
      s.row_face.push_back(f);
      s.row_lup.push_back(m.face_cell0[f] >= 0 ? local_cell(m.face_cell0[f]) : -1);
      s.row_ldn.push_back(m.face_cell1[f] >= 0 ? local_cell(m.face_cell1[f]) : -1);
    }
    s.v_nint[v] = nint;
    s.v_row_off[v + 1] = s.v_row_off[v] + nrow;
    s.v_col_off[v + 1] = s.v_col_off[v] + ncol;
    s.v_trans_off[v + 1] = s.v_trans_off[v] + (long long)nrow * ncol;
    for (int a = 0; a < nint; a++) s.col_ext.push_back(m.vert_cells[c0 + a]);
    for (int j = 0; j < nfv; j++)
      if (knw[j] >= 0) s.col_ext.push_back(nc + m.face_bnd[m.vert_faces[f0 + j]]);
    // interior hexahedral vertices whose Trans the device builds
    if (opt.setup_on_device && nint == 8 && nknw == 0 && nrow == 12) {
      std::array<int, 8> oc;
      std::array<int, 12> cr;
      if (canonical_layout(m, v, &m.vert_cells[c0], &s.row_lup[rbase], &s.row_ldn[rbase], oc, cr)) {
        s.trans.insert(s.trans.end(), (size_t)nrow * ncol, 0.0);
        for (int j = 0; j < nfv; j++) fpos[m.vert_faces[f0 + j]] = -1;
        s.max_nint = std::max(s.max_nint, nint);
        s.max_nrow = std::max(s.max_nrow, nrow);
        s.max_ncol = std::max(s.max_ncol, ncol);
        continue;
      }
    }
    // other vertices whose system fits one warp's shared memory: built on the
    // device too (a placeholder here)
    // (the launch sizes every warp's shared memory by the largest cells,
    // faces, unknowns and columns over these vertices: the bound holds for
    // the running maxima)
    if (opt.setup_on_device && nint <= kDevGenMaxCells && nfv <= kDevGenMaxFaces &&
        dev_gen_smem_bytes(std::max(nint, s.dev_gen_max_cells), std::max(nfv, s.dev_gen_max_faces),
                           std::max(nunk, s.dev_gen_max_unk), std::max(ncol, s.dev_gen_max_col)) <= kDevGenMaxSmem) {
      s.trans.insert(s.trans.end(), (size_t)nrow * ncol, 0.0);
      s.dev_gen_vertex.push_back(v);
      s.dev_gen_max_cells = std::max(s.dev_gen_max_cells, nint);
      s.dev_gen_max_faces = std::max(s.dev_gen_max_faces, nfv);
      s.dev_gen_max_unk = std::max(s.dev_gen_max_unk, nunk);
      s.dev_gen_max_col = std::max(s.dev_gen_max_col, ncol);
      for (int j = 0; j < nfv; j++) fpos[m.vert_faces[f0 + j]] = -1;
      s.max_nint = std::max(s.max_nint, nint);
      s.max_nrow = std::max(s.max_nrow, nrow);
      s.max_ncol = std::max(s.max_ncol, ncol);
      continue;
    }
    // subcells and their flux coefficients
    // flux_{a,i} = sum_u cu[u] Pi_u + sum_k ck[k] P_D,k + ccell * P_a
    struct Flux {
      std::vector<double> cu, ck;
      double ccell;
    };
    std::vector<Subcell> sc(nint);
    std::vector<std::array<Flux, 3>> fl(nint);
    for (int a = 0; a < nint; a++) {
      int c = m.vert_cells[c0 + a];
      int ierr = build_subcell(m, c, v, sc[a]);
      if (ierr) return ierr;
      double G[3][3];
      gmatrix(m, mat, opt.gmatrix_method, c, sc[a], G);
      for (int i = 0; i < 3; i++) {
        Flux &F = fl[a][i];
        F.cu.assign(nunk, 0.0);
        F.ck.assign(nknw, 0.0);
        F.ccell = -(-G[i][0] - G[i][1] - G[i][2]);
        for (int j = 0; j < 3; j++) {
          int p = fpos[sc[a].face[j]];
          if (unk[p] >= 0)
            F.cu[unk[p]] += -G[i][j];
          else
            F.ck[knw[p]] += -G[i][j];
        }
      }
    }
    auto subcell_face = [&](int a, int f) {
      for (int i = 0; i < 3; i++)
        if (sc[a].face[i] == f) return i;
      return -1;
    };
    // Assemble A Pi = B [P_cells; P_D]
    std::vector<double> A((size_t)nunk * nunk, 0.0), B((size_t)nunk * ncol, 0.0);
    for (int j = 0; j < nfv; j++) {
      if (unk[j] < 0) continue;
      int e = unk[j];
      int f = m.vert_faces[f0 + j];
      if (m.face_bnd[f] < 0) {
        int au = local_cell(m.face_cell0[f]), ad = local_cell(m.face_cell1[f]);
        if (au < 0 || ad < 0) return set_error(TDY_ERR_SUP, "internal face %d not shared at vertex %d", f, v);
        const Flux &Fu = fl[au][subcell_face(au, f)];
        const Flux &Fd = fl[ad][subcell_face(ad, f)];
        for (int u = 0; u < nunk; u++) A[(size_t)e * nunk + u] = -Fu.cu[u] + Fd.cu[u];
        B[(size_t)e * ncol + au] += Fu.ccell;
        B[(size_t)e * ncol + ad] += -Fd.ccell;
        for (int k = 0; k < nknw; k++) B[(size_t)e * ncol + nint + k] = Fu.ck[k] - Fd.ck[k];
      } else {  // Neumann: zero flux from its only subcell
        int a = local_cell(m.face_cell1[f]);
        const Flux &Fa = fl[a][subcell_face(a, f)];
        for (int u = 0; u < nunk; u++) A[(size_t)e * nunk + u] = -Fa.cu[u];
        B[(size_t)e * ncol + a] += Fa.ccell;
        for (int k = 0; k < nknw; k++) B[(size_t)e * ncol + nint + k] = Fa.ck[k];
      }
    }
    if (nunk > 0 && !lu_solve(nunk, ncol, A, B))
      return set_error(TDY_ERR_LIB, "singular interaction-region system at vertex %d", v);
    // B now holds M = A^-1 B.  Trans rows.
    for (int r = 0; r < nrow; r++) {
      int f = m.vert_faces[f0 + rows[r]];
      int a = (m.face_bnd[f] < 0) ? local_cell(m.face_cell0[f]) : local_cell(m.face_cell1[f]);
      const Flux &F = fl[a][subcell_face(a, f)];
      std::vector<double> t(ncol, 0.0);
      for (int c = 0; c < ncol; c++) {
        double acc = 0.0;
        for (int u = 0; u < nunk; u++) acc += F.cu[u] * B[(size_t)u * ncol + c];
        t[c] = acc;
      }
      t[a] += F.ccell;
      for (int k = 0; k < nknw; k++) t[nint + k] += F.ck[k];
      s.trans.insert(s.trans.end(), t.begin(), t.end());
    }
    for (int j = 0; j < nfv; j++) fpos[m.vert_faces[f0 + j]] = -1;
    s.max_nint = std::max(s.max_nint, nint);
    s.max_nrow = std::max(s.max_nrow, nrow);
    s.max_ncol = std::max(s.max_ncol, ncol);
  }
  s.nrows = s.v_row_off[nv];
  s.ncols = s.v_col_off[nv];
  s.ntrans = s.v_trans_off[nv];

  // ---- gravity discretization per face ----
  s.gravdis.assign(m.nf, 0.0);
  for (int f = 0; f < m.nf; f++) {
    if (is_neumann(f)) continue;
    int up = m.face_cell0[f], dn = m.face_cell1[f];
    const double *fc = &m.face_cen[3 * (size_t)f];
    const double *xu = (up >= 0) ? &m.cell_cen[3 * (size_t)up] : fc;
    const double *xd = (dn >= 0) ? &m.cell_cen[3 * (size_t)dn] : fc;
    double u[3];
    unit_from_to(xu, xd, u);
    int nvf = m.face_vert_off[f + 1] - m.face_vert_off[f];
    double area = m.face_area[f] / nvf;
    double kval = face_perm_value(m, mat, opt.gmatrix_method, f, u);
    if (opt.gmatrix_method == MPFAO_GMATRIX_TPF) area *= dot3(&m.face_nrm[3 * (size_t)f], u);
    const double grav[3] = {0.0, 0.0, opt.gravity};
    double gu = 0.0;
    for (int d = 0; d < 3; d++) gu += std::fabs(grav[d]) * u[d];
    s.gravdis[f] = area * kval * gu;
  }

  // ---- Jacobian pattern: cells sharing a vertex, sorted ----
  s.rowptr.assign(nc + 1, 0);
  {
    std::vector<int> mark(nc, -1), cols;
    for (int c = 0; c < nc; c++) {
      cols.clear();
      for (int j = m.cell_vert_off[c]; j < m.cell_vert_off[c + 1]; j++) {
        int v = m.cell_verts[j];
        for (int k = m.vert_cell_off[v]; k < m.vert_cell_off[v + 1]; k++) {
          int c2 = m.vert_cells[k];
          if (mark[c2] != c) {
            mark[c2] = c;
            cols.push_back(c2);
          }
        }
      }
      std::sort(cols.begin(), cols.end());
      s.colidx.insert(s.colidx.end(), cols.begin(), cols.end());
      s.rowptr[c + 1] = (int)s.colidx.size();
      s.max_row_nnz = std::max(s.max_row_nnz, (int)cols.size());
    }
  }
  if (s.max_row_nnz > 255) return set_error(TDY_ERR_SUP, "Jacobian row with %d entries (max 255)", s.max_row_nnz);

  // ---- canonical interior-hex vertices ----
  std::vector<int> canon_idx(nv, -1);
  std::vector<std::array<int, 8>> octant_col;  // octant -> vertex column, per canonical vertex
  std::vector<std::array<int, 12>> canon_row;  // canonical row -> vertex row
  for (int v = 0; v < nv; v++) {
    const int nint = s.v_nint[v];
    const int r0 = s.v_row_off[v], nrow = s.v_row_off[v + 1] - r0;
    const int c0 = s.v_col_off[v], ncol = s.v_col_off[v + 1] - c0;
    if (nint != 8 || nrow != 12 || ncol != 8) continue;
    std::array<int, 8> oc;
    std::array<int, 12> cr;
    if (!canonical_layout(m, v, &s.col_ext[c0], &s.row_lup[r0], &s.row_ldn[r0], oc, cr)) continue;
    canon_idx[v] = (int)s.canon_vertex.size();
    s.canon_vertex.push_back(v);
    octant_col.push_back(oc);
    canon_row.push_back(cr);
  }
  s.nC = (int)s.canon_vertex.size();
  s.nCpad = ((s.nC + 31) / 32) * 32;
  const long long P = s.nCpad;
  if (!opt.setup_on_device) s.Tc.assign(96 * (size_t)P, 0.0);  // else built on the device
  s.cellc.assign(8 * (size_t)P, 0);
  s.facec.assign(12 * (size_t)P, 0);
  for (int k = 0; k < s.nC; k++) {
    const int v = s.canon_vertex[k];
    const int r0 = s.v_row_off[v], c0 = s.v_col_off[v];
    const double *T = &s.trans[s.v_trans_off[v]];
    for (int o = 0; o < 8; o++) s.cellc[o * P + k] = s.col_ext[c0 + octant_col[k][o]];
    for (int rc = 0; rc < 12; rc++) {
      const int r = canon_row[k][rc];
      s.facec[rc * P + k] = s.row_face[r0 + r];
      if (!opt.setup_on_device)
        for (int o = 0; o < 8; o++) s.Tc[(rc * 8 + o) * P + k] = T[r * 8 + octant_col[k][o]];
    }
  }
  // scratch layout
  s.v_jv_off.assign(nv, -1);
  long long off = 72 * P;
  for (int v = 0; v < nv; v++) {
    if (s.v_nint[v] == 0) continue;
    if (canon_idx[v] >= 0) {
      s.v_jv_off[v] = canon_idx[v];
    } else {
      s.gen_vertex.push_back(v);
      s.v_jv_off[v] = off;
      off += (long long)s.v_nint[v] * s.v_nint[v] + s.v_nint[v];
    }
  }
  s.scratch_size = off;

  // ---- cell gather program ----
  s.cv_off.assign(nc + 1, 0);
  for (int c = 0; c < nc; c++) {
    const int *row = &s.colidx[s.rowptr[c]];
    const int rn = s.rowptr[c + 1] - s.rowptr[c];
    for (int j = m.cell_vert_off[c]; j < m.cell_vert_off[c + 1]; j++) {
      int v = m.cell_verts[j];
      const int c0 = s.v_col_off[v], nint = s.v_nint[v];
      std::vector<int> cols(nint);
      if (canon_idx[v] >= 0) {
        for (int o = 0; o < 8; o++) cols[o] = s.col_ext[c0 + octant_col[canon_idx[v]][o]];
      } else {
        for (int k = 0; k < nint; k++) cols[k] = s.col_ext[c0 + k];
      }
      int a = -1;
      for (int k = 0; k < nint; k++)
        if (cols[k] == c) a = k;
      if (a < 0) return set_error(TDY_ERR_LIB, "cell %d missing at its vertex %d", c, v);
      if (canon_idx[v] >= 0) {
        s.cv_jbase.push_back(((long long)a * P + canon_idx[v]) * 8);
        s.cv_rbase.push_back(64 * P + (long long)a * P + canon_idx[v]);
        s.cv_stride.push_back(1);
      } else {
        s.cv_jbase.push_back(s.v_jv_off[v] + (long long)a * nint);
        s.cv_rbase.push_back(s.v_jv_off[v] + (long long)nint * nint + a);
        s.cv_stride.push_back(1);
      }
      s.cv_nint.push_back(nint);
      s.cv_local.push_back(a);
      s.cv_slot_off.push_back((int)s.cv_slots.size());
      for (int k = 0; k < nint; k++) {
        int pos = (int)(std::lower_bound(row, row + rn, cols[k]) - row);
        s.cv_slots.push_back((uint8_t)pos);
      }
    }
    s.cv_off[c + 1] = (int)s.cv_jbase.size();
  }

  // ---- structured interior cells ----
  std::vector<std::array<int, 8>> svc;
  for (int c = 0; c < nc; c++) {
    bool ok = (s.rowptr[c + 1] - s.rowptr[c] == 27) && (s.cv_off[c + 1] - s.cv_off[c] == 8);
    std::array<int, 8> vcs;
    for (int j = 0; ok && j < 8; j++) {
      const int k = s.cv_off[c] + j;
      const int v = m.cell_verts[m.cell_vert_off[c] + j];
      if (canon_idx[v] < 0 || s.cv_local[k] != struct_octant(j)) {
        ok = false;
        break;
      }
      for (int b = 0; b < 8; b++)
        if (s.cv_slots[s.cv_slot_off[k] + b] != struct_slot(j, b)) ok = false;
      vcs[j] = canon_idx[v];
    }
    if (ok) {
      s.sc_cells.push_back(c);
      svc.push_back(vcs);
    } else {
      s.gc_cells.push_back(c);
    }
  }
  s.nS = (int)s.sc_cells.size();
  s.nSpad = ((s.nS + 31) / 32) * 32;
  s.sc_vc.assign(8 * (size_t)s.nSpad, 0);
  for (int k = 0; k < s.nS; k++)
    for (int j = 0; j < 8; j++) s.sc_vc[(size_t)j * s.nSpad + k] = svc[k][j];
  return 0;
}

}  // namespace tdy
