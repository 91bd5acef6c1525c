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

}  // namespace tdy
