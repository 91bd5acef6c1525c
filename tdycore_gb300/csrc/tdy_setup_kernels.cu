// tdy_setup_kernels.cu -- MPFA-O transmissibility of interior hexahedral
// vertices built on the device (-tdy_mpfao_setup_on_device).
//
// One thread per canonical vertex (8 cells in octant order, 12 internal faces
// in the canonical row order of kCanonUp/kCanonDn).  It restates the host
// setup chain for that vertex:
//   SetupSubcells (src/mesh/tdymeshplex.c:2829-3059): the three faces of each
//     subcell, oriented so the plane through their centroids faces the cell
//     centroid (UpdateFaceOrientationAroundAVertex, :1384-1412); T = 6 times
//     the tetrahedron volume; nu_i = (x_f(i+1) - x_c) x (x_f(i+2) - x_c);
//     subface area = face area / face vertices;
//   ComputeGMatrix_MPFAO / _TPF (src/fv/mpfao/tdympfao.c:13-274);
//   the interaction-region system (tdympfao.c:1000-1124): flux continuity on
//     the 12 subfaces, A Pi = B P, solved by LU with partial pivoting (first
//     maximal pivot, as LAPACK dgetrf), Trans = (flux of the face's first
//     subcell) applied to A^-1 B (ComputeCtimesAinvB, :1109-1124);
// and writes Trans straight into the structure-of-arrays layout the vertex
// kernel reads (Tc[(row * 8 + octant) * nCpad + vertex]).  Results equal the
// host's to rounding (the unknowns are eliminated in another order).
#include <cuda_runtime.h>

#include "tdy_arena.h"
#include "tdy_device.h"

namespace tdy {

namespace {

struct SetupGeom {
  int nC, nCpad, method;
  const int *canon_vertex, *cellc, *facec;
  const int *face_cell0, *face_cell1;
  const double *vx, *cell_cen, *face_cen, *face_nrm, *subface_area, *K0;
};

__device__ __forceinline__ void cross3d(const double a[3], const double b[3], double c[3]) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}
__device__ __forceinline__ double dot3d(const double a[3], const double b[3]) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

// canonical row joining octant o with its neighbour across axis k
__device__ __forceinline__ int crow(int o, int k) {
  return k == 0 ? ((o & ~1) >> 1) : k == 1 ? 4 + (((o & ~2) & 1) | (((o & ~2) >> 2) << 1)) : 8 + (o & ~4);
}
__device__ __forceinline__ int cup(int r) { return r < 4 ? 2 * r : r < 8 ? (((r - 4) & 1) | (((r - 4) >> 1) << 2)) : r - 8; }
__device__ __forceinline__ int cdn(int r) { return cup(r) | (1 << (r / 4)); }

__global__ void __launch_bounds__(64) canon_trans_kernel(SetupGeom g, double *Tc, int *status) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= g.nC) return;
  const long long P = g.nCpad;
  const int v = g.canon_vertex[k];
  const double xv[3] = {g.vx[3 * (size_t)v], g.vx[3 * (size_t)v + 1], g.vx[3 * (size_t)v + 2]};
  // flux of subcell o through its face at canonical row r:
  //   sum_j cf[o][i][j] * Pi_{row[o][j]} + cc[o][i] * P_o
  double cf[8][3][3], cc[8][3];
  int row[8][3];
  for (int o = 0; o < 8; o++) {
    const int c = g.cellc[o * P + k];
    const double xc[3] = {g.cell_cen[3 * (size_t)c], g.cell_cen[3 * (size_t)c + 1], g.cell_cen[3 * (size_t)c + 2]};
    int f[3];
    for (int a = 0; a < 3; a++) {
      row[o][a] = crow(o, a);
      f[a] = g.facec[row[o][a] * P + k];
    }
    double fc[3][3];
    for (int a = 0; a < 3; a++)
      for (int d = 0; d < 3; d++) fc[a][d] = g.face_cen[3 * (size_t)f[a] + d];
    {
      double a1[3], b1[3], c1[3], axb[3];
      for (int d = 0; d < 3; d++) {
        a1[d] = fc[1][d] - fc[0][d];
        b1[d] = fc[2][d] - fc[0][d];
        c1[d] = xc[d] - xv[d];
      }
      cross3d(a1, b1, axb);
      if (dot3d(axb, c1) < 0) {
        int t = f[1];
        f[1] = f[2];
        f[2] = t;
        t = row[o][1];
        row[o][1] = row[o][2];
        row[o][2] = t;
        for (int d = 0; d < 3; d++) {
          double x = fc[1][d];
          fc[1][d] = fc[2][d];
          fc[2][d] = x;
        }
      }
    }
    double T;
    {
      double a1[3], b1[3], c1[3], axb[3];
      for (int d = 0; d < 3; d++) {
        a1[d] = fc[0][d] - xc[d];
        b1[d] = fc[1][d] - xc[d];
        c1[d] = fc[2][d] - xc[d];
      }
      cross3d(a1, b1, axb);
      T = fabs(dot3d(axb, c1)) / 6.0 * 6.0;
    }
    double nu[3][3];
    for (int i = 0; i < 3; i++) {
      const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
      double a1[3], b1[3];
      for (int d = 0; d < 3; d++) {
        a1[d] = fc[i1][d] - xc[d];
        b1[d] = fc[i2][d] - xc[d];
      }
      cross3d(a1, b1, nu[i]);
    }
    const double *K = g.K0 + 9 * (size_t)c;
    for (int i = 0; i < 3; i++) {
      const double *n = g.face_nrm + 3 * (size_t)f[i];
      const double area = g.subface_area[f[i]];
      double G[3];
      for (int j = 0; j < 3; j++) {
        if (g.method == MPFAO_GMATRIX_DEFAULT) {
          double Kv[3];
          for (int a = 0; a < 3; a++) {
            Kv[a] = 0.0;
            for (int b = 0; b < 3; b++) Kv[a] += K[a * 3 + b] * nu[j][b];
          }
          double gg = 0.0;
          for (int a = 0; a < 3; a++) gg += n[a] * Kv[a];
          gg *= 1.0 / T * area;
          G[j] = gg;
        } else if (i != j) {
          G[j] = 0.0;
        } else {
          const int nb = (g.face_cell0[f[i]] == c) ? g.face_cell1[f[i]] : g.face_cell0[f[i]];
          const double *xn = g.cell_cen + 3 * (size_t)nb;
          const double *Kn = g.K0 + 9 * (size_t)nb;
          double dd[3];
          for (int d = 0; d < 3; d++) dd[d] = xc[d] - xn[d];
          const double dist = sqrt(dot3d(dd, dd)) * 0.50;
          const double len = sqrt(dot3d(dd, dd));
          double u[3];
          for (int d = 0; d < 3; d++) u[d] = dd[d] / len;
          const double dp = dot3d(n, u);
          double knv = 0.0, kv = 0.0;
          for (int q = 0; q < 3; q++) {
            knv += u[q] * u[q] / Kn[q * 3 + q];
            kv += u[q] * u[q] / K[q * 3 + q];
          }
          knv = 1.0 / knv;
          kv = 1.0 / kv;
          const double kav = 0.5 * kv + 0.5 * knv;
          G[j] = area * (dp)*kav / (dist);
        }
      }
      for (int j = 0; j < 3; j++) cf[o][i][j] = -G[j];
      cc[o][i] = -(-G[0] - G[1] - G[2]);
    }
  }
  // local index (0..2) of canonical row r among the faces of octant o
  auto slot = [&](int o, int r) { return row[o][0] == r ? 0 : row[o][1] == r ? 1 : 2; };
  double A[12][12], M[12][8];
  for (int r = 0; r < 12; r++) {
    for (int q = 0; q < 12; q++) A[r][q] = 0.0;
    for (int q = 0; q < 8; q++) M[r][q] = 0.0;
  }
  for (int r = 0; r < 12; r++) {
    const int u = cup(r), d = cdn(r);
    const int iu = slot(u, r), id = slot(d, r);
    for (int j = 0; j < 3; j++) A[r][row[u][j]] -= cf[u][iu][j];
    for (int j = 0; j < 3; j++) A[r][row[d][j]] += cf[d][id][j];
    M[r][u] += cc[u][iu];
    M[r][d] += -cc[d][id];
  }
  // LU with partial pivoting, solving A X = M in place
  for (int p = 0; p < 12; p++) {
    int piv = p;
    double best = fabs(A[p][p]);
    for (int r = p + 1; r < 12; r++)
      if (fabs(A[r][p]) > best) {
        best = fabs(A[r][p]);
        piv = r;
      }
    if (best == 0.0) {
      atomicExch(status, 1);
      return;
    }
    if (piv != p) {
      for (int q = 0; q < 12; q++) {
        double t = A[p][q];
        A[p][q] = A[piv][q];
        A[piv][q] = t;
      }
      for (int q = 0; q < 8; q++) {
        double t = M[p][q];
        M[p][q] = M[piv][q];
        M[piv][q] = t;
      }
    }
    for (int r = p + 1; r < 12; r++) {
      const double l = A[r][p] / A[p][p];
      if (l == 0.0) continue;
      for (int q = p + 1; q < 12; q++) A[r][q] -= l * A[p][q];
      for (int q = 0; q < 8; q++) M[r][q] -= l * M[p][q];
    }
  }
  for (int p = 11; p >= 0; p--) {
    for (int q = 0; q < 8; q++) {
      double s = M[p][q];
      for (int r = p + 1; r < 12; r++) s -= A[p][r] * M[r][q];
      M[p][q] = s / A[p][p];
    }
  }
  // Trans row r: flux of the face's first (up) subcell
  for (int r = 0; r < 12; r++) {
    const int u = cup(r), iu = slot(u, r);
    for (int o = 0; o < 8; o++) {
      double t = 0.0;
      for (int j = 0; j < 3; j++) t += cf[u][iu][j] * M[row[u][j]][o];
      if (o == u) t += cc[u][iu];
      Tc[(r * 8 + o) * P + k] = t;
    }
  }
}

// stream-ordered temporary (v must stay alive until the stream is synchronised)
// ---------------------------------------------------------------------------
// Other vertices (boundary, prismatic, irregular): one warp per vertex
// restates the host's per-vertex system (tdy_setup.cpp: subcells, G matrices,
// flux continuity A Pi = B [P; P_D], LU with partial pivoting, Trans rows as
// the flux of the subface's cell applied to A^-1 B; the reference's
// ComputeTransmissibilityMatrix_ForNonCornerVertex and _ForBoundaryVertex,
// tdympfao.c:1126-1756) with the system in the warp's shared memory, and
// writes the vertex's Trans block (rows: its non-Neumann faces in order;
// columns: its cells, then its Dirichlet faces) in place.
struct GenGeom {
  int n, method, NI, NF, NU, NC;  // vertices; limits of the launch
  const int *vert;                // the vertices
  const long long *trans_off;     // Trans block offset per vertex (all vertices)
  const int *vert_cell_off, *vert_cells, *vert_face_off, *vert_faces;
  const int *face_cell0, *face_cell1, *face_bnd, *bnd_type;
  const double *vx, *cell_cen, *face_cen, *face_nrm, *subface_area, *K0;
};

constexpr int kGenTransWarps = 2;

// face roles at a vertex
enum { GF_INTERNAL = 0, GF_DIRICHLET = 1, GF_NEUMANN = 2 };

__global__ void __launch_bounds__(32 * kGenTransWarps) gen_trans_kernel(GenGeom g, double *trans, int *status) {
  extern __shared__ double gsm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = blockIdx.x * kGenTransWarps + warp;
  if (k >= g.n) return;  // whole warp
  const size_t ndbl = (size_t)12 * g.NI + (size_t)g.NU * g.NU + (size_t)g.NU * g.NC;
  const size_t nint_words = (size_t)3 * g.NI + 3 * (size_t)g.NF;
  const size_t per_warp = ndbl + (nint_words + 1) / 2;  // in doubles
  double *Gm = gsm + per_warp * warp;    // [NI][3][3]
  double *cc = Gm + 9 * g.NI;            // [NI][3]
  double *A = cc + 3 * g.NI;             // [NU][NU] (nunk stride)
  double *B = A + (size_t)g.NU * g.NU;   // [NU][NC] (ncol stride)
  int *fp = reinterpret_cast<int *>(B + (size_t)g.NU * g.NC);  // [NI][3] face positions
  int *role = fp + 3 * g.NI;                                   // [NF]
  int *idx = role + g.NF;                                      // [NF] unknown or known index
  const int v = g.vert[k];
  const int c0 = g.vert_cell_off[v], nint = g.vert_cell_off[v + 1] - c0;
  const int f0 = g.vert_face_off[v], nfv = g.vert_face_off[v + 1] - f0;
  const double xv[3] = {g.vx[3 * (size_t)v], g.vx[3 * (size_t)v + 1], g.vx[3 * (size_t)v + 2]};
  auto local_cell = [&](int c) {
    for (int a = 0; a < nint; a++)
      if (g.vert_cells[c0 + a] == c) return a;
    return -1;
  };
  // face roles and the unknown / known numbering (in face order)
  int nunk = 0, nknw = 0;
  if (lane == 0) {
    for (int j = 0; j < nfv; j++) {
      const int f = g.vert_faces[f0 + j];
      const int b = g.face_bnd[f];
      const int r = b < 0 ? GF_INTERNAL : (g.bnd_type[b] == NEUMANN_BC ? GF_NEUMANN : GF_DIRICHLET);
      role[j] = r;
      idx[j] = r == GF_DIRICHLET ? nknw++ : nunk++;
    }
  }
  nunk = __shfl_sync(0xffffffffu, nunk, 0);
  nknw = __shfl_sync(0xffffffffu, nknw, 0);
  const int ncol = nint + nknw;
  __syncwarp();
  // subcells: the cell's three faces at v in face order, oriented to the cell
  // centroid; T, nu, subface areas; the G matrix row per face
  for (int a = lane; a < nint; a += 32) {
    const int c = g.vert_cells[c0 + a];
    int jf[3], n = 0;
    for (int j = 0; j < nfv && n <= 3; j++) {
      const int f = g.vert_faces[f0 + j];
      if (g.face_cell0[f] == c || g.face_cell1[f] == c) {
        if (n < 3) jf[n] = j;
        n++;
      }
    }
    if (n != 3) {
      atomicExch(status, 2);
      jf[0] = jf[1] = jf[2] = 0;
    }
    const double xc[3] = {g.cell_cen[3 * (size_t)c], g.cell_cen[3 * (size_t)c + 1], g.cell_cen[3 * (size_t)c + 2]};
    int f[3];
    double fc[3][3];
    for (int i = 0; i < 3; i++) {
      f[i] = g.vert_faces[f0 + jf[i]];
      for (int d = 0; d < 3; d++) fc[i][d] = g.face_cen[3 * (size_t)f[i] + d];
    }
    {
      double a1[3], b1[3], c1[3], axb[3];
      for (int d = 0; d < 3; d++) {
        a1[d] = fc[1][d] - fc[0][d];
        b1[d] = fc[2][d] - fc[0][d];
        c1[d] = xc[d] - xv[d];
      }
      cross3d(a1, b1, axb);
      if (dot3d(axb, c1) < 0) {
        int t = f[1];
        f[1] = f[2];
        f[2] = t;
        t = jf[1];
        jf[1] = jf[2];
        jf[2] = t;
        for (int d = 0; d < 3; d++) {
          double x = fc[1][d];
          fc[1][d] = fc[2][d];
          fc[2][d] = x;
        }
      }
    }
    double T;
    {
      double a1[3], b1[3], c1[3], axb[3];
      for (int d = 0; d < 3; d++) {
        a1[d] = fc[0][d] - xc[d];
        b1[d] = fc[1][d] - xc[d];
        c1[d] = fc[2][d] - xc[d];
      }
      cross3d(a1, b1, axb);
      T = fabs(dot3d(axb, c1)) / 6.0 * 6.0;
    }
    double nu[3][3];
    for (int i = 0; i < 3; i++) {
      const int i1 = (i + 1) % 3, i2 = (i + 2) % 3;
      double a1[3], b1[3];
      for (int d = 0; d < 3; d++) {
        a1[d] = fc[i1][d] - xc[d];
        b1[d] = fc[i2][d] - xc[d];
      }
      cross3d(a1, b1, nu[i]);
    }
    const double *K = g.K0 + 9 * (size_t)c;
    for (int i = 0; i < 3; i++) {
      const double *nrm = g.face_nrm + 3 * (size_t)f[i];
      const double area = g.subface_area[f[i]];
      double G[3];
      for (int j = 0; j < 3; j++) {
        if (g.method == MPFAO_GMATRIX_DEFAULT) {
          double Kv[3];
          for (int q = 0; q < 3; q++) {
            Kv[q] = 0.0;
            for (int b = 0; b < 3; b++) Kv[q] += K[q * 3 + b] * nu[j][b];
          }
          double gg = 0.0;
          for (int q = 0; q < 3; q++) gg += nrm[q] * Kv[q];
          gg *= 1.0 / T * area;
          G[j] = gg;
        } else if (i != j) {
          G[j] = 0.0;
        } else {
          const int nb = (g.face_cell0[f[i]] == c) ? g.face_cell1[f[i]] : g.face_cell0[f[i]];
          const double *xn;
          const double *Kn;
          double dist;
          double dd[3];
          if (nb >= 0) {
            xn = g.cell_cen + 3 * (size_t)nb;
            Kn = g.K0 + 9 * (size_t)nb;
            for (int d = 0; d < 3; d++) dd[d] = xc[d] - xn[d];
            dist = sqrt(dot3d(dd, dd)) * 0.50;
          } else {
            xn = g.face_cen + 3 * (size_t)f[i];
            Kn = K;
            for (int d = 0; d < 3; d++) dd[d] = xc[d] - xn[d];
            dist = sqrt(dot3d(dd, dd));
          }
          const double len = sqrt(dot3d(dd, dd));
          double u[3];
          for (int d = 0; d < 3; d++) u[d] = dd[d] / len;
          const double dp = dot3d(nrm, u);
          double knv = 0.0, kv = 0.0;
          for (int q = 0; q < 3; q++) {
            knv += u[q] * u[q] / Kn[q * 3 + q];
            kv += u[q] * u[q] / K[q * 3 + q];
          }
          knv = 1.0 / knv;
          kv = 1.0 / kv;
          const double kav = 0.5 * kv + 0.5 * knv;
          G[j] = area * (dp)*kav / (dist);
        }
      }
      for (int j = 0; j < 3; j++) Gm[(a * 3 + i) * 3 + j] = G[j];
      cc[a * 3 + i] = -(-G[0] - G[1] - G[2]);
      fp[a * 3 + i] = jf[i];
    }
  }
  for (int e = lane; e < nunk * nunk; e += 32) A[e] = 0.0;
  for (int e = lane; e < nunk * ncol; e += 32) B[e] = 0.0;
  __syncwarp();
  // position (0..2) of vertex face j in the subcell of local cell a
  auto slot = [&](int a, int j) { return fp[a * 3] == j ? 0 : fp[a * 3 + 1] == j ? 1 : 2; };
  // flux of subcell (a, i): sum_q -G[i][q] Pi_{face q} + cc P_a; rows of A
  // and B per unknown face, as the host assembles them
  for (int j = lane; j < nfv; j += 32) {
    if (role[j] == GF_DIRICHLET) continue;
    const int e = idx[j];
    const int f = g.vert_faces[f0 + j];
    if (role[j] == GF_INTERNAL) {
      const int au = local_cell(g.face_cell0[f]), ad = local_cell(g.face_cell1[f]);
      if (au < 0 || ad < 0) {
        atomicExch(status, 2);
        continue;
      }
      const int iu = slot(au, j), id = slot(ad, j);
      for (int q = 0; q < 3; q++) {  // -Fu.cu
        const int jq = fp[au * 3 + q];
        if (role[jq] != GF_DIRICHLET) A[e * nunk + idx[jq]] = -(-Gm[(au * 3 + iu) * 3 + q]);
      }
      for (int q = 0; q < 3; q++) {  // + Fd.cu
        const int jq = fp[ad * 3 + q];
        if (role[jq] != GF_DIRICHLET) A[e * nunk + idx[jq]] += -Gm[(ad * 3 + id) * 3 + q];
      }
      B[e * ncol + au] += cc[au * 3 + iu];
      B[e * ncol + ad] += -cc[ad * 3 + id];
      for (int q = 0; q < 3; q++) {  // Fu.ck - Fd.ck
        const int jq = fp[au * 3 + q];
        if (role[jq] == GF_DIRICHLET) B[e * ncol + nint + idx[jq]] = -Gm[(au * 3 + iu) * 3 + q];
      }
      for (int q = 0; q < 3; q++) {
        const int jq = fp[ad * 3 + q];
        if (role[jq] == GF_DIRICHLET) B[e * ncol + nint + idx[jq]] -= -Gm[(ad * 3 + id) * 3 + q];
      }
    } else {  // Neumann: zero flux from its only subcell
      const int a = local_cell(g.face_cell1[f]);
      if (a < 0) {
        atomicExch(status, 2);
        continue;
      }
      const int ia = slot(a, j);
      for (int q = 0; q < 3; q++) {
        const int jq = fp[a * 3 + q];
        if (role[jq] != GF_DIRICHLET) A[e * nunk + idx[jq]] = -(-Gm[(a * 3 + ia) * 3 + q]);
      }
      B[e * ncol + a] += cc[a * 3 + ia];
      for (int q = 0; q < 3; q++) {
        const int jq = fp[a * 3 + q];
        if (role[jq] == GF_DIRICHLET) B[e * ncol + nint + idx[jq]] = -Gm[(a * 3 + ia) * 3 + q];
      }
    }
  }
  __syncwarp();
  // LU with partial pivoting (first maximal |pivot|), A X = B in place
  for (int p = 0; p < nunk; p++) {
    double best = -1.0;
    int pr = p;
    for (int r = p + lane; r < nunk; r += 32) {
      const double x = fabs(A[r * nunk + p]);
      if (x > best) {
        best = x;
        pr = r;
      }
    }
    for (int off = 16; off > 0; off >>= 1) {
      const double ob = __shfl_down_sync(0xffffffffu, best, off);
      const int orr = __shfl_down_sync(0xffffffffu, pr, off);
      if (ob > best || (ob == best && orr < pr)) {
        best = ob;
        pr = orr;
      }
    }
    best = __shfl_sync(0xffffffffu, best, 0);
    pr = __shfl_sync(0xffffffffu, pr, 0);
    if (best == 0.0) {
      if (lane == 0) atomicExch(status, 1);
      return;
    }
    if (pr != p) {
      for (int q = lane; q < nunk; q += 32) {
        const double t = A[p * nunk + q];
        A[p * nunk + q] = A[pr * nunk + q];
        A[pr * nunk + q] = t;
      }
      for (int q = lane; q < ncol; q += 32) {
        const double t = B[p * ncol + q];
        B[p * ncol + q] = B[pr * ncol + q];
        B[pr * ncol + q] = t;
      }
    }
    __syncwarp();
    const double piv = A[p * nunk + p];
    // rows r > p: l = A[r][p] / piv, then the rest of the row and of B
    const int w = (nunk - p - 1) + ncol;  // columns to update per row
    for (int e = lane; e < (nunk - p - 1) * w; e += 32) {
      const int r = p + 1 + e / w, q = e % w;
      const double l = A[r * nunk + p] / piv;
      if (l == 0.0) continue;
      if (q < nunk - p - 1)
        A[r * nunk + p + 1 + q] -= l * A[p * nunk + p + 1 + q];
      else
        B[r * ncol + (q - (nunk - p - 1))] -= l * B[p * ncol + (q - (nunk - p - 1))];
    }
    __syncwarp();
    for (int r = p + 1 + lane; r < nunk; r += 32) A[r * nunk + p] = A[r * nunk + p] / piv;
    __syncwarp();
  }
  for (int kk = nunk - 1; kk >= 0; kk--) {
    const double piv = A[kk * nunk + kk];
    for (int j = lane; j < ncol; j += 32) {
      double sv = B[kk * ncol + j];
      for (int i = kk + 1; i < nunk; i++) sv -= A[kk * nunk + i] * B[i * ncol + j];
      B[kk * ncol + j] = sv / piv;
    }
    __syncwarp();
  }
  // Trans rows: the flux of the face's subcell (its first cell for internal
  // faces, its cell for boundary faces) applied to A^-1 B
  double *Tv = trans + g.trans_off[v];
  int r = 0;
  for (int j = 0; j < nfv; j++) {
    if (role[j] == GF_NEUMANN) continue;
    const int f = g.vert_faces[f0 + j];
    const int a = role[j] == GF_INTERNAL ? local_cell(g.face_cell0[f]) : local_cell(g.face_cell1[f]);
    if (a >= 0) {
      const int ia = slot(a, j);
      for (int c = lane; c < ncol; c += 32) {
        double acc = 0.0;
        // the subcell's unknown faces in ascending unknown order (the host's
        // dense loop adds only these terms)
        int qs[3] = {0, 1, 2}, key[3];
        for (int x = 0; x < 3; x++) {
          const int jq = fp[a * 3 + x];
          key[x] = role[jq] == GF_DIRICHLET ? 0x7fffffff : idx[jq];
        }
        for (int x = 0; x < 2; x++)
          for (int y = 0; y < 2 - x; y++)
            if (key[qs[y]] > key[qs[y + 1]]) {
              const int t = qs[y];
              qs[y] = qs[y + 1];
              qs[y + 1] = t;
            }
        for (int x = 0; x < 3; x++) {
          const int jq = fp[a * 3 + qs[x]];
          if (role[jq] != GF_DIRICHLET) acc += -Gm[(a * 3 + ia) * 3 + qs[x]] * B[idx[jq] * ncol + c];
        }
        if (c == a) acc += cc[a * 3 + ia];
        if (c >= nint)
          for (int x = 0; x < 3; x++) {
            const int jq = fp[a * 3 + x];
            if (role[jq] == GF_DIRICHLET && nint + idx[jq] == c) acc += -Gm[(a * 3 + ia) * 3 + x];
          }
        Tv[(size_t)r * ncol + c] = acc;
      }
    }
    r++;
  }
}

template <class T>
int upload(std::vector<void *> &owned, T **p, const std::vector<T> &v, cudaStream_t st) {
  int ierr = dmem_alloc((void **)p, v.size() * sizeof(T) + 1, st);
  if (ierr) return ierr;
  owned.push_back(*p);
  if (v.empty()) return 0;
  cudaError_t e = cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return set_error(TDY_ERR_GPU, "cudaMemcpyAsync: %s", cudaGetErrorString(e));
  return 0;
}

}  // namespace

int device_canon_trans(const _p_TDy *t, const int *d_cellc, const int *d_facec, double *d_Tc, void *stream) {
  cudaStream_t cs = (cudaStream_t)stream;
  const Mesh &m = t->mesh;
  const MPFAOSetup &s = t->setup;
  if (s.nC == 0) return 0;
  std::vector<void *> owned;
  int ierr = 0;
  SetupGeom g;
  g.nC = s.nC;
  g.nCpad = s.nCpad;
  g.method = t->opt.gmatrix_method;
  g.cellc = d_cellc;
  g.facec = d_facec;
  std::vector<double> sub(m.nf);
  for (int f = 0; f < m.nf; f++) sub[f] = m.face_area[f] / (m.face_vert_off[f + 1] - m.face_vert_off[f]);
  int *st = nullptr;
  const std::vector<int> zero(1, 0);
  {
    int *p;
    double *q;
    if ((ierr = upload(owned, &p, s.canon_vertex, cs))) goto done;
    g.canon_vertex = p;
    if ((ierr = upload(owned, &p, m.face_cell0, cs))) goto done;
    g.face_cell0 = p;
    if ((ierr = upload(owned, &p, m.face_cell1, cs))) goto done;
    g.face_cell1 = p;
    if ((ierr = upload(owned, &q, m.vx, cs))) goto done;
    g.vx = q;
    if ((ierr = upload(owned, &q, m.cell_cen, cs))) goto done;
    g.cell_cen = q;
    if ((ierr = upload(owned, &q, m.face_cen, cs))) goto done;
    g.face_cen = q;
    if ((ierr = upload(owned, &q, m.face_nrm, cs))) goto done;
    g.face_nrm = q;
    if ((ierr = upload(owned, &q, sub, cs))) goto done;
    g.subface_area = q;
    if ((ierr = upload(owned, &q, t->mat.K0, cs))) goto done;
    g.K0 = q;
    if ((ierr = upload(owned, &st, zero, cs))) goto done;
  }
  {
    const int bs = 64;
    canon_trans_kernel<<<(s.nC + bs - 1) / bs, bs, 0, cs>>>(g, d_Tc, st);
    int hs = 0;
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, st, sizeof(int), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    if (e != cudaSuccess) {
      ierr = set_error(TDY_ERR_GPU, "canon_trans_kernel: %s", cudaGetErrorString(e));
      goto done;
    }
    if (hs) ierr = set_error(TDY_ERR_LIB, "singular interaction-region system at an interior hexahedral vertex");
  }
done:
  cudaStreamSynchronize(cs);  // the uploads have read their host vectors
  for (void *p : owned) dmem_free(p, cs);
  return ierr;
}

// Trans of the other vertices that TDySetup marked for the device (one warp
// each), written in place into d_trans on `stream`.
int device_gen_trans(const _p_TDy *t, double *d_trans, void *stream) {
  const Mesh &m = t->mesh;
  const MPFAOSetup &s = t->setup;
  if (s.dev_gen_vertex.empty()) return 0;
  cudaStream_t cs = (cudaStream_t)stream;
  std::vector<double> sub(m.nf);
  for (int f = 0; f < m.nf; f++) sub[f] = m.face_area[f] / (m.face_vert_off[f + 1] - m.face_vert_off[f]);
  GenGeom g;
  g.n = (int)s.dev_gen_vertex.size();
  g.method = t->opt.gmatrix_method;
  g.NI = s.dev_gen_max_cells;
  g.NF = s.dev_gen_max_faces;
  g.NU = std::max(s.dev_gen_max_unk, 1);
  g.NC = std::max(s.dev_gen_max_col, 1);
  Arena ar;
  ar.up(&g.vert, s.dev_gen_vertex);
  ar.up(&g.trans_off, s.v_trans_off);
  ar.up(&g.vert_cell_off, m.vert_cell_off);
  ar.up(&g.vert_cells, m.vert_cells);
  ar.up(&g.vert_face_off, m.vert_face_off);
  ar.up(&g.vert_faces, m.vert_faces);
  ar.up(&g.face_cell0, m.face_cell0);
  ar.up(&g.face_cell1, m.face_cell1);
  ar.up(&g.face_bnd, m.face_bnd);
  ar.up(&g.bnd_type, t->bnd.type);
  ar.up(&g.vx, m.vx);
  ar.up(&g.cell_cen, m.cell_cen);
  ar.up(&g.face_cen, m.face_cen);
  ar.up(&g.face_nrm, m.face_nrm);
  ar.up(&g.subface_area, sub);
  ar.up(&g.K0, t->mat.K0);
  int *status = nullptr;
  ar.work(&status, 1);
  int ierr = ar.commit(cs);
  if (ierr) return ierr;
  const size_t per_warp = 8 * ((size_t)12 * g.NI + (size_t)g.NU * g.NU + (size_t)g.NU * g.NC) +
                          8 * (((size_t)3 * g.NI + 3 * (size_t)g.NF + 1) / 2);
  const size_t smem = per_warp * kGenTransWarps;  // at most 2 x 48 KB (the set-up bounds the maxima)
  if (smem > 2 * kDevGenMaxSmem + 1024) {
    cudaStreamSynchronize(cs);
    dmem_free(ar.base, cs);
    return set_error(TDY_ERR_LIB, "device Trans: %zu bytes of shared memory per block", smem);
  }
  cudaError_t e = cudaMemsetAsync(status, 0, sizeof(int), cs);
  if (e == cudaSuccess && smem > 48 * 1024)
    e = cudaFuncSetAttribute(gen_trans_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int hs = 0;
  if (e == cudaSuccess) {
    gen_trans_kernel<<<(g.n + kGenTransWarps - 1) / kGenTransWarps, 32 * kGenTransWarps, smem, cs>>>(g, d_trans,
                                                                                                  status);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, cs);
  if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
  cudaStreamSynchronize(cs);  // the staging buffer and `sub` outlive the uploads
  dmem_free(ar.base, cs);
  if (e != cudaSuccess) return set_error(TDY_ERR_GPU, "gen_trans_kernel: %s", cudaGetErrorString(e));
  if (hs == 1) return set_error(TDY_ERR_LIB, "singular interaction-region system at a vertex (device set-up)");
  if (hs == 2) return set_error(TDY_ERR_SUP, "a cell without exactly three faces at one of its vertices (device set-up)");
  return 0;
}

}  // namespace tdy
