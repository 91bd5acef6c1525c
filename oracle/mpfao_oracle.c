/*
 * mpfao_oracle.c -- TEST INFRASTRUCTURE ONLY (see mpfao_oracle.h).
 *
 * Serial C restatement of the reference's MPFA-O Richards residual and
 * Jacobian.  Each function names the reference lines it follows; loops run in
 * the reference order (vertex, then row, then column) and arithmetic keeps
 * the reference's operation order, so the results are what the reference
 * computes on the same setup arrays up to the summation order of its sparse
 * kernels, which are emulated here:
 *   - MatMult(Trans_mat, P_vec): each row's entries summed in ascending
 *     column order, as PETSc's SeqAIJ stores them;
 *   - MatSetValuesLocal(..., ADD_VALUES): binary search of the column in the
 *     sorted CSR row, then add.
 * Parity status: restatement checked against the reference's regression
 * golden files through a Newton driver (tests/test_golden_regression.py).
 */
#include "mpfao_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { DIRICHLET = 0, NEUMANN = 1, SEEPAGE = 2 };
enum { SAT_GARDNER = 0, SAT_VG = 1 };
enum { KR_IRMAY = 0, KR_MUALEM = 1 };
enum { RHO_CONST = 0, RHO_EXP = 1, RHO_BW = 2 };
enum { MU_CONST = 0, MU_BW = 1 };

struct OracleCtx {
  OracleInput in;
  int nc, nb, nv, nrows;
  /* per-cell aux state (tdympfaoimpl.h:76-108) */
  double *S, *dS_dP, *d2S_dP2, *Kr, *dKr_dS, *rho, *drho_dP, *d2rho_dP2, *vis, *dvis_dP;
  /* boundary state */
  double *P_bnd, *S_bnd, *Kr_bnd, *dKr_dS_bnd;
  /* P_vec, TtimesP_vec, and sum_c |T_rc P_c| (error scale of each row) */
  double *P_vec, *TtimesP, *TPabs;
  /* Trans_mat as CSR over vertex rows, columns ascending */
  int *tm_rowptr, *tm_col;
  double *tm_val;
  /* Jacobian pattern */
  int *rowptr, *colidx, nnz;
  /* accumulation_prev and dtime (tdympfao_snes.c:19-64) */
  double *accum_prev, dtime;
  /* vertex colours for the threaded baseline */
  int ncolors, *color_off, *color_vert;
  /* owned copies of the input arrays */
  void *owned[32];
  int nowned;
};

static void *own_copy(OracleCtx *c, const void *src, size_t bytes) {
  void *p = malloc(bytes ? bytes : 1);
  if (bytes) memcpy(p, src, bytes);
  c->owned[c->nowned++] = p;
  return p;
}

/* ---------------------------------------------------------------------------
 * Characteristic curves: src/materials/tdycharacteristiccurves.c */

/* PressureSaturation_VanGenuchten (tdycharacteristiccurves.c:692-717) */
static void sat_vg(double m, double alpha, double Sr, double Pc, double *S, double *dS_dP, double *d2S_dP2) {
  double pc_alpha, pc_alpha_n, one_plus_pc_alpha_n, n;
  if (Pc <= 0) {
    *S = 1;
    *dS_dP = 0;
    *d2S_dP2 = 0.0;
  } else {
    double Se, dSe_dPc, d2Se_dPc2;
    n = 1 / (1 - m);
    pc_alpha = Pc * alpha;
    pc_alpha_n = pow(pc_alpha, n);
    one_plus_pc_alpha_n = 1 + pc_alpha_n;
    Se = pow(one_plus_pc_alpha_n, -m);
    *S = (1.0 - Sr) * Se + Sr;
    dSe_dPc = -m * n * alpha * pc_alpha_n / (pc_alpha * pow(one_plus_pc_alpha_n, m + 1));
    *dS_dP = -dSe_dPc * (1.0 - Sr);
    d2Se_dPc2 = m * n * (pc_alpha_n)*pow(one_plus_pc_alpha_n, -m - 2.0) * ((m * n + 1.0) * pc_alpha_n - n + 1) /
                pow(Pc, 2.0);
    *d2S_dP2 = (1.0 - Sr) * d2Se_dPc2;
  }
}

/* PressureSaturation_Gardner (tdycharacteristiccurves.c:641-667) */
static void sat_gardner(double n, double m, double alpha, double Sr, double Pc, double *S, double *dS_dP,
                        double *d2S_dP2) {
  (void)n;
  if (Pc < 0) {
    *S = 1;
    *dS_dP = 0;
    *d2S_dP2 = 0.0;
  } else {
    double Se, dSe_dPc, d2Se_dPc2;
    Se = exp(-alpha * Pc / m);
    *S = (1.0 - Sr) * Se + Sr;
    dSe_dPc = -alpha / m * exp(-alpha * Pc / m);
    *dS_dP = -dSe_dPc * (1.0 - Sr);
    d2Se_dPc2 = -alpha / m * dSe_dPc;
    *d2S_dP2 = (1.0 - Sr) * d2Se_dPc2;
  }
}

/* SaturationCompute dispatch (tdycharacteristiccurves.c:125-157) */
static void saturation(const OracleInput *in, int c, double Sr, double Pc, double *S, double *dS, double *d2S) {
  const double *p = in->sat_param + 3 * (size_t)c;
  if (in->sat_type[c] == SAT_VG)
    sat_vg(p[0], p[1], Sr, Pc, S, dS, d2S);
  else
    sat_gardner(p[0], p[1], p[2], Sr, Pc, S, dS, d2S);
}

/* RelativePermeability_Mualem_Unsmoothed (tdycharacteristiccurves.c:468-485) */
static void kr_mualem_unsmoothed(double m, double Se, double *Kr, double *dKr_dSe) {
  double Se_one_over_m, tmp;
  *Kr = 1.0;
  *dKr_dSe = 0.0;
  if (Se >= 1.0) return;
  Se_one_over_m = pow(Se, 1 / m);
  tmp = pow(1 - Se_one_over_m, m);
  (*Kr) = sqrt(Se);
  (*Kr) *= (1 - tmp) * (1 - tmp);
  (*dKr_dSe) = 0.5 * (*Kr) / Se;
  (*dKr_dSe) += 2 * pow(Se, 1 / m - 0.5) * pow(1 - Se_one_over_m, m - 1) * (1 - pow(1 - Se_one_over_m, m));
}

/* RelativePermeability_Mualem (tdycharacteristiccurves.c:607-614) with
 * CubicPolynomialEvaluate (:551-562) */
static void kr_mualem(const double *p, double Se, double *Kr, double *dKr_dSe) {
  double m = p[0], x0 = p[1], x1 = p[2], dx = p[4];
  const double *coeffs = p + 5;
  if (Se > x1) {
    double xt = (Se - x0) / dx;
    *Kr = coeffs[0] + xt * (coeffs[1] + xt * (coeffs[2] + xt * coeffs[3]));
    *dKr_dSe = (coeffs[1] + xt * (2.0 * coeffs[2] + xt * 3.0 * coeffs[3])) / dx;
  } else {
    kr_mualem_unsmoothed(m, Se, Kr, dKr_dSe);
  }
}

/* RelativePermeability_Irmay (tdycharacteristiccurves.c:451-460) */
static void kr_irmay(double m, double Se, double *Kr, double *dKr_dSe) {
  *Kr = 1.0;
  *dKr_dSe = 0.0;
  if (Se >= 1.0) return;
  *Kr = pow(Se, m);
  *dKr_dSe = pow(Se, m - 1) * m;
}

static void relperm(const OracleInput *in, int c, double Se, double *Kr, double *dKr) {
  const double *p = in->relperm_param + 9 * (size_t)c;
  if (in->relperm_type[c] == KR_MUALEM)
    kr_mualem(p, Se, Kr, dKr);
  else
    kr_irmay(p[0], Se, Kr, dKr);
}

/* ---------------------------------------------------------------------------
 * EOS: src/materials/tdyeos.c:5-136 (T = Tref = 25, zero salinity) */
static void eos_density(int type, double p, double *den, double *dden_dP, double *d2den_dP2) {
  if (type == RHO_CONST) {
    *den = 998.0;
    *dden_dP = 0.0;
    *d2den_dP2 = 0.0;
  } else if (type == RHO_EXP) {
    double ReferenceDensity = 997.16e0, ReferencePressure = 101325.e0, WaterCompressibility = 1.e-8;
    if (p < ReferencePressure) {
      *den = ReferenceDensity;
      *dden_dP = 0.0;
      *d2den_dP2 = 0.0;
    } else {
      *den = ReferenceDensity * exp(WaterCompressibility * (p - ReferencePressure));
      *dden_dP = WaterCompressibility * (*den);
      *d2den_dP2 = WaterCompressibility * (*dden_dP);
    }
  } else {
    double T = 25.0, S = 0.0, P = p, Pa_to_MPa = 1.e-6, pw;
    pw = 1 + 1.e-6 * (-80. * T - 3.3 * pow(T, 2) + 0.00175 * pow(T, 3) + 489. * P * Pa_to_MPa - 2. * T * P * Pa_to_MPa +
                      0.016 * P * Pa_to_MPa * pow(T, 2) - 1.3e-5 * pow(T, 3) * P * Pa_to_MPa -
                      0.333 * pow(P * Pa_to_MPa, 2) - 0.002 * T * pow(P * Pa_to_MPa, 2));
    pw *= 1000.;
    *den = pw + S * (0.668 + 0.44 * S +
                     1e-6 * (300. * P * Pa_to_MPa - 2400. * P * Pa_to_MPa * S +
                             T * (80. * 3. * T - 3300. * S - 13. * P * Pa_to_MPa + 47. * P * Pa_to_MPa * S))) *
                    1000.;
    /* the reference leaves the derivatives untouched (zero-initialised) */
    *dden_dP = 0.0;
    *d2den_dP2 = 0.0;
  }
}

static void eos_viscosity(int type, double *vis, double *dvis_dP) {
  if (type == MU_CONST) {
    *vis = 9.94e-4;
  } else {
    double T = 25.0, S = 0.0;
    *vis = 0.1 + 0.333 * S + (1.65 + 91.9 * pow(S, 3)) * exp((-0.42 * pow((pow(S, 0.8) - 0.17), 2) + 0.045) * pow(T, 0.8));
    *vis *= 1e-3;
  }
  *dvis_dP = 0.0;
}

/* ---------------------------------------------------------------------------
 * Context */

static int cmp_int(const void *a, const void *b) {
  int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

typedef struct {
  int col;
  double val;
} ColVal;
static int cmp_colval(const void *a, const void *b) {
  int x = ((const ColVal *)a)->col, y = ((const ColVal *)b)->col;
  return (x > y) - (x < y);
}

OracleCtx *oracle_create(const OracleInput *in) {
  OracleCtx *c = (OracleCtx *)calloc(1, sizeof(OracleCtx));
  c->in = *in;
  const int nc = in->ncells, nb = in->nbnd, nv = in->nverts, nf = in->nfaces;
  c->nc = nc;
  c->nb = nb;
  c->nv = nv;
  const int nrows = in->v_row_off[nv], ncols = in->v_col_off[nv];
  const long long ntr = in->v_trans_off[nv];
  c->nrows = nrows;
  OracleInput *o = &c->in;
  o->volume = own_copy(c, in->volume, sizeof(double) * nc);
  o->porosity = own_copy(c, in->porosity, sizeof(double) * nc);
  o->Sr = own_copy(c, in->Sr, sizeof(double) * nc);
  o->sat_type = own_copy(c, in->sat_type, sizeof(int) * nc);
  o->sat_param = own_copy(c, in->sat_param, sizeof(double) * 3 * nc);
  o->relperm_type = own_copy(c, in->relperm_type, sizeof(int) * nc);
  o->relperm_param = own_copy(c, in->relperm_param, sizeof(double) * 9 * nc);
  o->source_sink = own_copy(c, in->source_sink, sizeof(double) * nc);
  o->face_up = own_copy(c, in->face_up, sizeof(int) * nf);
  o->face_dn = own_copy(c, in->face_dn, sizeof(int) * nf);
  o->gravdis = own_copy(c, in->gravdis, sizeof(double) * nf);
  o->bnd_face = own_copy(c, in->bnd_face, sizeof(int) * nb);
  o->bnd_type = own_copy(c, in->bnd_type, sizeof(int) * nb);
  o->bnd_has_value = own_copy(c, in->bnd_has_value, sizeof(int) * nb);
  o->bnd_value = own_copy(c, in->bnd_value, sizeof(double) * nb);
  o->rho_bnd = own_copy(c, in->rho_bnd, sizeof(double) * nb);
  o->vis_bnd = own_copy(c, in->vis_bnd, sizeof(double) * nb);
  o->v_row_off = own_copy(c, in->v_row_off, sizeof(int) * (nv + 1));
  o->v_col_off = own_copy(c, in->v_col_off, sizeof(int) * (nv + 1));
  o->v_nint = own_copy(c, in->v_nint, sizeof(int) * nv);
  o->v_trans_off = own_copy(c, in->v_trans_off, sizeof(long long) * (nv + 1));
  o->row_face = own_copy(c, in->row_face, sizeof(int) * nrows);
  o->col_ext = own_copy(c, in->col_ext, sizeof(int) * ncols);
  o->trans = own_copy(c, in->trans, sizeof(double) * ntr);

#define ALLOC(p, n) p = (double *)calloc((n) ? (n) : 1, sizeof(double))
  ALLOC(c->S, nc);
  ALLOC(c->dS_dP, nc);
  ALLOC(c->d2S_dP2, nc);
  ALLOC(c->Kr, nc);
  ALLOC(c->dKr_dS, nc);
  ALLOC(c->rho, nc);
  ALLOC(c->drho_dP, nc);
  ALLOC(c->d2rho_dP2, nc);
  ALLOC(c->vis, nc);
  ALLOC(c->dvis_dP, nc);
  ALLOC(c->P_bnd, nb);
  ALLOC(c->S_bnd, nb);
  ALLOC(c->Kr_bnd, nb);
  ALLOC(c->dKr_dS_bnd, nb);
  ALLOC(c->P_vec, nc + nb);
  ALLOC(c->TtimesP, nrows);
  ALLOC(c->TPabs, nrows);
  ALLOC(c->accum_prev, nc);
#undef ALLOC

  /* Trans_mat: one row per (vertex, row), ascending columns
   * (tdympfao.c:1451-1466 inserts with MatSetValues; SeqAIJ sorts). */
  c->tm_rowptr = (int *)calloc(nrows + 1, sizeof(int));
  c->tm_col = (int *)malloc(sizeof(int) * (ntr ? ntr : 1));
  c->tm_val = (double *)malloc(sizeof(double) * (ntr ? ntr : 1));
  {
    long long k = 0;
    ColVal *tmp = (ColVal *)malloc(sizeof(ColVal) * 256);
    int cap = 256;
    for (int v = 0; v < nv; v++) {
      int r0 = o->v_row_off[v], nr = o->v_row_off[v + 1] - r0;
      int c0 = o->v_col_off[v], ncl = o->v_col_off[v + 1] - c0;
      if (ncl > cap) {
        cap = ncl;
        tmp = (ColVal *)realloc(tmp, sizeof(ColVal) * cap);
      }
      for (int r = 0; r < nr; r++) {
        const double *T = o->trans + o->v_trans_off[v] + (long long)r * ncl;
        for (int j = 0; j < ncl; j++) {
          tmp[j].col = o->col_ext[c0 + j];
          tmp[j].val = T[j];
        }
        qsort(tmp, ncl, sizeof(ColVal), cmp_colval);
        for (int j = 0; j < ncl; j++) {
          c->tm_col[k] = tmp[j].col;
          c->tm_val[k] = tmp[j].val;
          k++;
        }
        c->tm_rowptr[r0 + r + 1] = (int)k;
      }
    }
    free(tmp);
  }

  /* Jacobian pattern: cells sharing a vertex (DMPlex FVM++ adjacency,
   * tdympfao.c:808 + tdydiscretization.c:156-170), sorted columns. */
  {
    int *deg = (int *)calloc(nc, sizeof(int));
    int **lists = (int **)calloc(nc, sizeof(int *));
    int *cap = (int *)calloc(nc, sizeof(int));
    for (int v = 0; v < nv; v++) {
      int c0 = o->v_col_off[v], ni = o->v_nint[v];
      for (int a = 0; a < ni; a++) {
        int ca = o->col_ext[c0 + a];
        for (int b = 0; b < ni; b++) {
          int cb = o->col_ext[c0 + b];
          if (deg[ca] == cap[ca]) {
            cap[ca] = cap[ca] ? 2 * cap[ca] : 32;
            lists[ca] = (int *)realloc(lists[ca], sizeof(int) * cap[ca]);
          }
          lists[ca][deg[ca]++] = cb;
        }
      }
    }
    c->rowptr = (int *)calloc(nc + 1, sizeof(int));
    int total = 0;
    for (int i = 0; i < nc; i++) {
      if (deg[i]) qsort(lists[i], deg[i], sizeof(int), cmp_int);
      int u = 0;
      for (int j = 0; j < deg[i]; j++)
        if (j == 0 || lists[i][j] != lists[i][j - 1]) lists[i][u++] = lists[i][j];
      deg[i] = u;
      total += u;
      c->rowptr[i + 1] = total;
    }
    c->nnz = total;
    c->colidx = (int *)malloc(sizeof(int) * (total ? total : 1));
    for (int i = 0; i < nc; i++) {
      memcpy(c->colidx + c->rowptr[i], lists[i], sizeof(int) * deg[i]);
      free(lists[i]);
    }
    free(lists);
    free(deg);
    free(cap);
  }

  /* Greedy vertex colouring: vertices sharing a cell get different colours. */
  {
    int *vcolor = (int *)malloc(sizeof(int) * (nv ? nv : 1));
    /* cell -> vertices */
    int *cdeg = (int *)calloc(nc + 1, sizeof(int));
    for (int v = 0; v < nv; v++)
      for (int a = 0; a < o->v_nint[v]; a++) cdeg[o->col_ext[o->v_col_off[v] + a] + 1]++;
    for (int i = 0; i < nc; i++) cdeg[i + 1] += cdeg[i];
    int *cv = (int *)malloc(sizeof(int) * (cdeg[nc] ? cdeg[nc] : 1));
    int *fill = (int *)calloc(nc, sizeof(int));
    for (int v = 0; v < nv; v++)
      for (int a = 0; a < o->v_nint[v]; a++) {
        int cc = o->col_ext[o->v_col_off[v] + a];
        cv[cdeg[cc] + fill[cc]++] = v;
      }
    int maxc = 0;
    unsigned char *used = (unsigned char *)calloc(1024, 1);
    for (int v = 0; v < nv; v++) {
      memset(used, 0, 1024);
      for (int a = 0; a < o->v_nint[v]; a++) {
        int cc = o->col_ext[o->v_col_off[v] + a];
        for (int k = cdeg[cc]; k < cdeg[cc + 1]; k++) {
          int w = cv[k];
          if (w < v) used[vcolor[w]] = 1;
        }
      }
      int col = 0;
      while (used[col]) col++;
      vcolor[v] = col;
      if (col + 1 > maxc) maxc = col + 1;
    }
    c->ncolors = maxc;
    c->color_off = (int *)calloc(maxc + 1, sizeof(int));
    c->color_vert = (int *)malloc(sizeof(int) * (nv ? nv : 1));
    for (int v = 0; v < nv; v++) c->color_off[vcolor[v] + 1]++;
    for (int k = 0; k < maxc; k++) c->color_off[k + 1] += c->color_off[k];
    int *pos = (int *)calloc(maxc, sizeof(int));
    for (int v = 0; v < nv; v++) c->color_vert[c->color_off[vcolor[v]] + pos[vcolor[v]]++] = v;
    free(pos);
    free(used);
    free(fill);
    free(cv);
    free(cdeg);
    free(vcolor);
  }
  return c;
}

void oracle_destroy(OracleCtx *c) {
  if (!c) return;
  double *arr[] = {c->S, c->dS_dP, c->d2S_dP2, c->Kr, c->dKr_dS, c->rho, c->drho_dP, c->d2rho_dP2, c->vis,
                   c->dvis_dP, c->P_bnd, c->S_bnd, c->Kr_bnd, c->dKr_dS_bnd, c->P_vec, c->TtimesP, c->TPabs, c->accum_prev,
                   c->tm_val};
  for (size_t i = 0; i < sizeof(arr) / sizeof(arr[0]); i++) free(arr[i]);
  free(c->tm_rowptr);
  free(c->tm_col);
  free(c->rowptr);
  free(c->colidx);
  free(c->color_off);
  free(c->color_vert);
  for (int i = 0; i < c->nowned; i++) free(c->owned[i]);
  free(c);
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int oracle_pattern_nnz(OracleCtx *c) { return c->nnz; }
void oracle_pattern(OracleCtx *c, int *rowptr, int *colidx) {
  memcpy(rowptr, c->rowptr, sizeof(int) * (c->nc + 1));
  memcpy(colidx, c->colidx, sizeof(int) * c->nnz);
}

void oracle_get_state(OracleCtx *c, double *S, double *rho, double *Kr) {
  if (S) memcpy(S, c->S, sizeof(double) * c->nc);
  if (rho) memcpy(rho, c->rho, sizeof(double) * c->nc);
  if (Kr) memcpy(Kr, c->Kr, sizeof(double) * c->nc);
}

/* ---------------------------------------------------------------------------
 * State updates */

/* TDyUpdateState_Richards_MPFAO (tdympfao.c:2527-2594), cells lo..hi-1 */
static void update_state_range(OracleCtx *c, const double *U, int lo, int hi) {
  const OracleInput *in = &c->in;
  for (int i = lo; i < hi; i++) {
    double Pc = in->Pref - U[i];
    saturation(in, i, in->Sr[i], Pc, &c->S[i], &c->dS_dP[i], &c->d2S_dP2[i]);
    double Se = (c->S[i] - in->Sr[i]) / (1.0 - in->Sr[i]);
    relperm(in, i, Se, &c->Kr[i], &c->dKr_dS[i]);
    double dSe_dS = 1.0 / (1.0 - in->Sr[i]);
    c->dKr_dS[i] *= dSe_dS;
    double P = in->Pref - Pc;
    eos_density(in->rho_type, P, &c->rho[i], &c->drho_dP[i], &c->d2rho_dP2[i]);
    eos_viscosity(in->mu_type, &c->vis[i], &c->dvis_dP[i]);
    c->P_vec[i] = P;
  }
}

/* TDyMPFAO_SetBoundaryPressure (tdympfao_utils.c:690-759) followed by
 * TDyMPFAOUpdateBoundaryState (tdympfao_utils.c:24-99); boundary faces lo..hi-1
 * in face order. */
static void update_boundary_range(OracleCtx *c, const double *U, int lo, int hi) {
  const OracleInput *in = &c->in;
  for (int b = lo; b < hi; b++) {
    int f = in->bnd_face[b];
    int cell = in->face_up[f] >= 0 ? in->face_up[f] : in->face_dn[f];
    if (in->bnd_has_value[b])
      c->P_bnd[b] = in->bnd_value[b];
    else
      c->P_bnd[b] = U[cell];
    c->P_vec[b + c->nc] = c->P_bnd[b];
    double Sr = in->Sr[cell];
    double Pc = in->Pref - c->P_bnd[b];
    double S, dS, d2S;
    saturation(in, cell, Sr, Pc, &S, &dS, &d2S);
    double Se = (S - Sr) / (1.0 - Sr);
    double dSe_dS = 1.0 / (1.0 - Sr);
    double Kr, dKr_dSe;
    relperm(in, cell, Se, &Kr, &dKr_dSe);
    c->S_bnd[b] = S;
    c->Kr_bnd[b] = Kr;
    c->dKr_dS_bnd[b] = dKr_dSe * dSe_dS;
  }
}

/* MatMult(Trans_mat, P_vec, TtimesP_vec) (tdympfao_ts.c:184) */
static void matmult_range(OracleCtx *c, int lo, int hi) {
  for (int r = lo; r < hi; r++) {
    double s = 0.0, a = 0.0;
    for (int k = c->tm_rowptr[r]; k < c->tm_rowptr[r + 1]; k++) {
      s += c->tm_val[k] * c->P_vec[c->tm_col[k]];
      a += fabs(c->tm_val[k] * c->P_vec[c->tm_col[k]]);
    }
    c->TtimesP[r] = s;
    c->TPabs[r] = a;
  }
}

static void update_all(OracleCtx *c, const double *U) {
  update_state_range(c, U, 0, c->nc);
  update_boundary_range(c, U, 0, c->nb);
  matmult_range(c, 0, c->nrows);
}

/* ---------------------------------------------------------------------------
 * Residual */

static inline double cell_or_bnd(const double *cellv, const double *bndv, int id) {
  return id >= 0 ? cellv[id] : bndv[-id - 1];
}

/* TDyMPFAOIFunction_Vertices (tdympfao_ts.c:12-150) for one vertex */
static void ifunction_vertex(OracleCtx *c, int v, double *r, double *rmag) {
  const OracleInput *in = &c->in;
  int r0 = in->v_row_off[v], nr = in->v_row_off[v + 1] - r0;
  for (int irow = 0; irow < nr; irow++) {
    int set_flow_to_zero = 0;
    int face_id = in->row_face[r0 + irow];
    double TtimesP = c->TtimesP[r0 + irow];
    int cell_id_up = in->face_up[face_id];
    int cell_id_dn = in->face_dn[face_id];
    double den_aveg = 0.0;
    den_aveg += cell_or_bnd(c->rho, in->rho_bnd, cell_id_up);
    den_aveg += cell_or_bnd(c->rho, in->rho_bnd, cell_id_dn);
    den_aveg *= 0.5;
    double G = in->gravdis[face_id];
    double ukvr = 0.0;
    if (TtimesP + den_aveg * G < 0.0) {
      if (cell_id_up >= 0) {
        ukvr = c->Kr[cell_id_up] / c->vis[cell_id_up];
      } else {
        int b = -cell_id_up - 1;
        ukvr = c->Kr_bnd[b] / in->vis_bnd[b];
        if (in->bnd_type[b] == SEEPAGE && c->P_bnd[b] <= in->Pref) set_flow_to_zero = 1;
      }
    } else {
      if (cell_id_dn >= 0) {
        ukvr = c->Kr[cell_id_dn] / c->vis[cell_id_dn];
      } else {
        int b = -cell_id_dn - 1;
        ukvr = c->Kr_bnd[b] / in->vis_bnd[b];
        if (in->bnd_type[b] == SEEPAGE && c->P_bnd[b] <= in->Pref) set_flow_to_zero = 1;
      }
    }
    double fluxm = 0.0;
    if (!set_flow_to_zero) {
      fluxm = den_aveg * ukvr * (-TtimesP);
      fluxm += -pow(den_aveg, 2.0) * ukvr * G;
    }
    /* error scale of fluxm: |rho ukvr| (sum_c |T_c P_c| + |rho G|) */
    double fmag = set_flow_to_zero ? 0.0 : fabs(den_aveg * ukvr) * (c->TPabs[r0 + irow] + fabs(den_aveg * G));
    if (cell_id_up >= 0) {
      r[cell_id_up] += fluxm;
      if (rmag) rmag[cell_id_up] += fmag;
    }
    if (cell_id_dn >= 0) {
      r[cell_id_dn] -= fluxm;
      if (rmag) rmag[cell_id_dn] += fmag;
    }
  }
}

/* TDyMPFAOSNESAccumulation (tdympfao_snes.c:19-30) */
static inline double snes_accum(OracleCtx *c, int i) {
  const OracleInput *in = &c->in;
  return c->rho[i] * in->porosity[i] * c->S[i] * in->volume[i] / c->dtime;
}

void oracle_snes_presolve(OracleCtx *c, const double *Uprev, double dt) {
  c->dtime = dt;
  update_state_range(c, Uprev, 0, c->nc);
  for (int i = 0; i < c->nc; i++) c->accum_prev[i] = snes_accum(c, i);
}

/* TDyMPFAOSNESFunction (tdympfao_snes.c:67-140) */
void oracle_snes_function(OracleCtx *c, const double *U, double *R, double *Rmag) {
  memset(R, 0, sizeof(double) * c->nc);
  if (Rmag) memset(Rmag, 0, sizeof(double) * c->nc);
  update_all(c, U);
  for (int v = 0; v < c->nv; v++) ifunction_vertex(c, v, R, Rmag);
  for (int i = 0; i < c->nc; i++) {
    double accum_current = snes_accum(c, i);
    R[i] += accum_current - c->accum_prev[i];
    R[i] -= c->in.source_sink[i];
    if (Rmag) Rmag[i] += fabs(accum_current) + fabs(c->accum_prev[i]) + fabs(c->in.source_sink[i]);
  }
}

/* TDyMPFAOIFunction (tdympfao_ts.c:153-227) */
void oracle_ts_ifunction(OracleCtx *c, const double *U, const double *Ut, double *R, double *Rmag) {
  const OracleInput *in = &c->in;
  memset(R, 0, sizeof(double) * c->nc);
  if (Rmag) memset(Rmag, 0, sizeof(double) * c->nc);
  update_all(c, U);
  for (int v = 0; v < c->nv; v++) ifunction_vertex(c, v, R, Rmag);
  for (int i = 0; i < c->nc; i++) {
    double rho = c->rho[i], drho_dP = c->drho_dP[i], porosity = in->porosity[i], dporosity_dP = 0.0;
    double S = c->S[i], dS_dP = c->dS_dP[i];
    double dmass_dP = rho * dporosity_dP * S + drho_dP * porosity * S + rho * porosity * dS_dP;
    double volume = in->volume[i];
    double t1 = dmass_dP * Ut[i] * volume, t2 = in->source_sink[i] * volume;
    R[i] += t1;
    R[i] -= t2;
    if (Rmag) Rmag[i] += fabs(t1) + fabs(t2);
  }
}

/* dmass/dP of one cell, mass = rho * porosity * S (tdympfao_ts.c:470-480) */
static inline double dmass_dP_cell(OracleCtx *c, int i) {
  const double dporosity_dP = 0.0;
  return c->rho[i] * dporosity_dP * c->S[i] + c->drho_dP[i] * c->in.porosity[i] * c->S[i] +
         c->rho[i] * c->in.porosity[i] * c->dS_dP[i];
}

/* TDyMPFAOTransientVariable (tdympfao_ts_transientvar.c:13-47): C = rho phi S V;
 * dC (optional) = d(rho phi S)/dP V. */
void oracle_transient_variable(OracleCtx *c, const double *U, double *C, double *dC) {
  const OracleInput *in = &c->in;
  update_state_range(c, U, 0, c->nc);
  for (int i = 0; i < c->nc; i++) {
    C[i] = c->rho[i] * in->porosity[i] * c->S[i] * in->volume[i];
    if (dC) dC[i] = dmass_dP_cell(c, i) * in->volume[i];
  }
}

/* TDyMPFAOIFunction_TransientVariable (tdympfao_ts_transientvar.c:50-101):
 * R = fluxes + dM/dt V - source V. */
void oracle_tv_ifunction(OracleCtx *c, const double *U, const double *Mdot, double *R, double *Rmag) {
  const OracleInput *in = &c->in;
  memset(R, 0, sizeof(double) * c->nc);
  if (Rmag) memset(Rmag, 0, sizeof(double) * c->nc);
  update_all(c, U);
  for (int v = 0; v < c->nv; v++) ifunction_vertex(c, v, R, Rmag);
  for (int i = 0; i < c->nc; i++) {
    double t1 = Mdot[i] * in->volume[i], t2 = in->source_sink[i] * in->volume[i];
    R[i] += t1;
    R[i] -= t2;
    if (Rmag) Rmag[i] += fabs(t1) + fabs(t2);
  }
}

/* TDyMPFAOIFunction_DAE (tdympfao_ts_dae.c:13-84): U, U_t and R hold [P, M]
 * interleaved per cell; R_P = M_t V - source V + fluxes, R_M = M - rho phi S V. */
void oracle_dae_ifunction(OracleCtx *c, const double *U, const double *Ut, double *R, double *Rmag) {
  const OracleInput *in = &c->in;
  const int n = c->nc;
  double *P = (double *)malloc(sizeof(double) * n), *rp = (double *)calloc(n, sizeof(double));
  double *rpm = Rmag ? (double *)calloc(n, sizeof(double)) : NULL;
  for (int i = 0; i < n; i++) P[i] = U[2 * i];
  update_all(c, P);
  for (int v = 0; v < c->nv; v++) ifunction_vertex(c, v, rp, rpm);
  for (int i = 0; i < n; i++) {
    const double vol = in->volume[i];
    R[2 * i] = Ut[2 * i + 1] * vol - in->source_sink[i] * vol + rp[i];
    const double mass = c->rho[i] * in->porosity[i] * c->S[i] * vol;
    R[2 * i + 1] = U[2 * i + 1] - mass;
    if (Rmag) {
      Rmag[2 * i] = fabs(Ut[2 * i + 1] * vol) + fabs(in->source_sink[i] * vol) + rpm[i];
      Rmag[2 * i + 1] = fabs(U[2 * i + 1]) + fabs(mass);
    }
  }
  free(P);
  free(rp);
  free(rpm);
}

/* ---------------------------------------------------------------------------
 * Jacobian */

/* MatSetValuesLocal(A, 1, &row, n, cols, vals, ADD_VALUES) */
static inline void mat_add_row(OracleCtx *c, double *J, double *Jmag, int row, int n, const int *cols,
                               const double *vals, const double *mags) {
  const int *rc = c->colidx + c->rowptr[row];
  int rn = c->rowptr[row + 1] - c->rowptr[row];
  for (int j = 0; j < n; j++) {
    if (cols[j] < 0) continue;
    int lo = 0, hi = rn - 1, pos = -1;
    while (lo <= hi) {
      int mid = (lo + hi) >> 1;
      if (rc[mid] == cols[j]) {
        pos = mid;
        break;
      }
      if (rc[mid] < cols[j])
        lo = mid + 1;
      else
        hi = mid - 1;
    }
    if (pos < 0) abort(); /* column outside the preallocated pattern */
    J[c->rowptr[row] + pos] += vals[j];
    if (Jmag) Jmag[c->rowptr[row] + pos] += mags ? mags[j] : fabs(vals[j]);
  }
}

/* TDyMPFAOIJacobian_Vertices (tdympfao_ts.c:235-456) for one vertex */
static void ijacobian_vertex(OracleCtx *c, int v, double *J, double *Jmag) {
  const OracleInput *in = &c->in;
  int r0 = in->v_row_off[v], nr = in->v_row_off[v + 1] - r0;
  int c0 = in->v_col_off[v], ncl = in->v_col_off[v + 1] - c0;
  int num_int_cells = in->v_nint[v];
  const double *Tv = in->trans + in->v_trans_off[v];
  int up_cols[256], dn_cols[256];
  double up_Jac[256], dn_Jac[256], mag[256];
  for (int irow = 0; irow < nr; irow++) {
    int set_jac_to_zero = 0;
    int face_id = in->row_face[r0 + irow];
    double TtimesP = c->TtimesP[r0 + irow];
    int cell_id_up = in->face_up[face_id];
    int cell_id_dn = in->face_dn[face_id];
    /* Neumann boundary faces carry no row (tdympfao_ts.c:310) */
    if ((cell_id_up < 0 && in->bnd_type[-cell_id_up - 1] == NEUMANN) ||
        (cell_id_dn < 0 && in->bnd_type[-cell_id_dn - 1] == NEUMANN))
      continue;
    double dukvr_dPup = 0.0, dukvr_dPdn = 0.0, ukvr;
    double den_aveg = 0.0, dden_aveg_dPup = 0.0, dden_aveg_dPdn = 0.0;
    if (cell_id_up >= 0) {
      den_aveg += 0.5 * c->rho[cell_id_up];
      dden_aveg_dPup = 0.5 * c->drho_dP[cell_id_up];
    } else {
      den_aveg += 0.5 * in->rho_bnd[-cell_id_up - 1];
      dden_aveg_dPup = 0.0;
    }
    if (cell_id_dn >= 0) {
      den_aveg += 0.5 * c->rho[cell_id_dn];
      dden_aveg_dPdn = 0.5 * c->drho_dP[cell_id_dn];
    } else {
      den_aveg += 0.5 * in->rho_bnd[-cell_id_dn - 1];
      dden_aveg_dPdn = 0.0;
    }
    double G = in->gravdis[face_id];
    if (TtimesP + den_aveg * G < 0.0) {
      if (cell_id_up >= 0) {
        double Kr = c->Kr[cell_id_up], dKr_dS = c->dKr_dS[cell_id_up], vis = c->vis[cell_id_up];
        double dvis_dP = c->dvis_dP[cell_id_up], dS_dP = c->dS_dP[cell_id_up];
        ukvr = Kr / vis;
        dukvr_dPup = dKr_dS * dS_dP / vis - Kr / (vis * vis) * dvis_dP;
      } else {
        int b = -cell_id_up - 1;
        ukvr = c->Kr_bnd[b] / in->vis_bnd[b];
        dukvr_dPup = 0.0;
        if (in->bnd_type[b] == SEEPAGE && c->P_bnd[b] <= in->Pref) set_jac_to_zero = 1;
      }
    } else {
      if (cell_id_dn >= 0) {
        double Kr = c->Kr[cell_id_dn], dKr_dS = c->dKr_dS[cell_id_dn], vis = c->vis[cell_id_dn];
        double dvis_dP = c->dvis_dP[cell_id_dn], dS_dP = c->dS_dP[cell_id_dn];
        ukvr = Kr / vis;
        dukvr_dPdn = dKr_dS * dS_dP / vis - Kr / (vis * vis) * dvis_dP;
      } else {
        int b = -cell_id_dn - 1;
        ukvr = c->Kr_bnd[b] / in->vis_bnd[b];
        dukvr_dPdn = 0.0;
        if (in->bnd_type[b] == SEEPAGE && c->P_bnd[b] <= in->Pref) set_jac_to_zero = 1;
      }
    }
    for (int icol = 0; icol < num_int_cells; ++icol) {
      up_cols[icol] = -1;
      dn_cols[icol] = -1;
      int cell_id = in->col_ext[c0 + icol];
      double T = Tv[(long long)irow * ncl + icol];
      double Jac;
      const double tpa = c->TPabs[r0 + irow];
      if (set_jac_to_zero) {
        Jac = 0.0;
        mag[icol] = 0.0;
      } else if (cell_id_up > -1 && cell_id == cell_id_up) {
        Jac = dden_aveg_dPup * ukvr * TtimesP + den_aveg * dukvr_dPup * TtimesP + den_aveg * ukvr * T +
              2 * den_aveg * dden_aveg_dPup * ukvr * G + pow(den_aveg, 2.0) * dukvr_dPup * G;
        mag[icol] = fabs(dden_aveg_dPup * ukvr) * tpa + fabs(den_aveg * dukvr_dPup) * tpa + fabs(den_aveg * ukvr * T) +
                    fabs(2 * den_aveg * dden_aveg_dPup * ukvr * G) + fabs(pow(den_aveg, 2.0) * dukvr_dPup * G);
      } else if (cell_id_dn > -1 && cell_id == cell_id_dn) {
        Jac = dden_aveg_dPdn * ukvr * TtimesP + den_aveg * dukvr_dPdn * TtimesP + den_aveg * ukvr * T +
              2 * den_aveg * dden_aveg_dPdn * ukvr * G + pow(den_aveg, 2.0) * dukvr_dPdn * G;
        mag[icol] = fabs(dden_aveg_dPdn * ukvr) * tpa + fabs(den_aveg * dukvr_dPdn) * tpa + fabs(den_aveg * ukvr * T) +
                    fabs(2 * den_aveg * dden_aveg_dPdn * ukvr * G) + fabs(pow(den_aveg, 2.0) * dukvr_dPdn * G);
      } else {
        Jac = den_aveg * ukvr * T;
        mag[icol] = fabs(Jac);
      }
      Jac = -Jac;
      if (cell_id_up >= 0) {
        up_cols[icol] = cell_id;
        up_Jac[icol] = Jac;
      }
      if (cell_id_dn >= 0) {
        dn_cols[icol] = cell_id;
        dn_Jac[icol] = -Jac;
      }
    }
    if (cell_id_up >= 0) mat_add_row(c, J, Jmag, cell_id_up, num_int_cells, up_cols, up_Jac, mag);
    if (cell_id_dn >= 0) mat_add_row(c, J, Jmag, cell_id_dn, num_int_cells, dn_cols, dn_Jac, mag);
  }
}

/* TDyMPFAOSNESJacobian (tdympfao_snes.c:143-203).  The reference reads the
 * aux state left by the preceding TDyMPFAOSNESFunction at the same U; the
 * oracle recomputes it from U first, which is the same state. */
void oracle_snes_jacobian(OracleCtx *c, const double *U, double *J, double *Jmag) {
  const OracleInput *in = &c->in;
  memset(J, 0, sizeof(double) * c->nnz);
  if (Jmag) memset(Jmag, 0, sizeof(double) * c->nnz);
  update_all(c, U);
  for (int v = 0; v < c->nv; v++) ijacobian_vertex(c, v, J, Jmag);
  double dtInv = 1.0 / c->dtime;
  double dporosity_dP = 0.0;
  for (int i = 0; i < c->nc; i++) {
    double dmass_dP = c->rho[i] * dporosity_dP * c->S[i] + c->drho_dP[i] * in->porosity[i] * c->S[i] +
                      c->rho[i] * in->porosity[i] * c->dS_dP[i];
    double Jac = dmass_dP * in->volume[i] * dtInv;
    mat_add_row(c, J, Jmag, i, 1, &i, &Jac, NULL);
  }
}

/* TDyMPFAOIJacobian (tdympfao_ts.c:520-561) with
 * TDyMPFAOIJacobian_Accumulation (:459-517) */
void oracle_ts_ijacobian(OracleCtx *c, const double *U, const double *Ut, double shift, double *J, double *Jmag) {
  const OracleInput *in = &c->in;
  memset(J, 0, sizeof(double) * c->nnz);
  if (Jmag) memset(Jmag, 0, sizeof(double) * c->nnz);
  update_all(c, U);
  for (int v = 0; v < c->nv; v++) ijacobian_vertex(c, v, J, Jmag);
  double dporosity_dP = 0.0, d2porosity_dP2 = 0.0;
  for (int icell = 0; icell < c->nc; icell++) {
    double drho_dP = c->drho_dP[icell], d2rho_dP2 = c->d2rho_dP2[icell];
    double rho = c->rho[icell], S = c->S[icell], dS = c->dS_dP[icell], d2S = c->d2S_dP2[icell];
    double poro = in->porosity[icell];
    double dmass_dP = rho * dporosity_dP * S + drho_dP * poro * S + rho * poro * dS;
    double d2mass_dP2 = (dS * rho * dporosity_dP + S * drho_dP * dporosity_dP + S * rho * d2porosity_dP2 +
                         dS * drho_dP * poro + S * d2rho_dP2 * poro + S * drho_dP * dporosity_dP +
                         d2S * rho * poro + dS * drho_dP * poro + dS * rho * dporosity_dP);
    double value = (shift * dmass_dP + d2mass_dP2 * Ut[icell]) * in->volume[icell];
    mat_add_row(c, J, Jmag, icell, 1, &icell, &value, NULL);
  }
}

/* Jacobian of the transient-variable residual R(U, shift C(U) + const):
 * fluxes plus shift dC/dP on the diagonal.  The reference registers no
 * IJacobian for this form (src/tdycore.c:1956-1958) and leaves it to PETSc's
 * finite differences; this is the exact derivative of the same residual. */
void oracle_tv_ijacobian(OracleCtx *c, const double *U, double shift, double *J, double *Jmag) {
  const OracleInput *in = &c->in;
  memset(J, 0, sizeof(double) * c->nnz);
  if (Jmag) memset(Jmag, 0, sizeof(double) * c->nnz);
  update_all(c, U);
  for (int v = 0; v < c->nv; v++) ijacobian_vertex(c, v, J, Jmag);
  for (int i = 0; i < c->nc; i++) {
    double value = shift * dmass_dP_cell(c, i) * in->volume[i];
    mat_add_row(c, J, Jmag, i, 1, &i, &value, NULL);
  }
}

/* ---------------------------------------------------------------------------
 * Threaded residual only (per-step checks of long runs on large meshes): the
 * state, boundary and Trans.P stages in parallel, the vertex loop over
 * vertex colours.  The same terms as oracle_snes_function, summed in colour
 * order, so the result differs from it only by rounding. */
void oracle_snes_function_parallel(OracleCtx *c, const double *U, double *R, int nthreads) {
  const OracleInput *in = &c->in;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  (void)nthreads;
#endif
#pragma omp parallel num_threads(nthreads)
  {
#pragma omp for schedule(static)
    for (int i = 0; i < c->nc; i++) R[i] = 0.0;
#pragma omp for schedule(static)
    for (int i = 0; i < c->nc; i++) update_state_range(c, U, i, i + 1);
#pragma omp for schedule(static)
    for (int b = 0; b < c->nb; b++) update_boundary_range(c, U, b, b + 1);
#pragma omp for schedule(static)
    for (int r = 0; r < c->nrows; r++) matmult_range(c, r, r + 1);
    for (int col = 0; col < c->ncolors; col++) {
#pragma omp for schedule(static)
      for (int k = c->color_off[col]; k < c->color_off[col + 1]; k++) ifunction_vertex(c, c->color_vert[k], R, NULL);
    }
#pragma omp for schedule(static)
    for (int i = 0; i < c->nc; i++) {
      R[i] += snes_accum(c, i) - c->accum_prev[i];
      R[i] -= in->source_sink[i];
    }
  }
}

/* ---------------------------------------------------------------------------
 * Threaded fused F+J for the CPU baseline. */
void oracle_snes_function_jacobian_parallel(OracleCtx *c, const double *U, double *R, double *J, int nthreads) {
  const OracleInput *in = &c->in;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
  (void)nthreads;
#endif
#pragma omp parallel num_threads(nthreads)
  {
#pragma omp for schedule(static)
    for (int i = 0; i < c->nc; i++) R[i] = 0.0;
#pragma omp for schedule(static)
    for (int k = 0; k < c->nnz; k++) J[k] = 0.0;
#pragma omp for schedule(static)
    for (int i = 0; i < c->nc; i++) update_state_range(c, U, i, i + 1);
#pragma omp for schedule(static)
    for (int b = 0; b < c->nb; b++) update_boundary_range(c, U, b, b + 1);
#pragma omp for schedule(static)
    for (int r = 0; r < c->nrows; r++) matmult_range(c, r, r + 1);
    for (int col = 0; col < c->ncolors; col++) {
#pragma omp for schedule(static)
      for (int k = c->color_off[col]; k < c->color_off[col + 1]; k++) {
        int v = c->color_vert[k];
        ifunction_vertex(c, v, R, NULL);
        ijacobian_vertex(c, v, J, NULL);
      }
    }
    double dtInv = 1.0 / c->dtime;
#pragma omp for schedule(static)
    for (int i = 0; i < c->nc; i++) {
      double accum_current = snes_accum(c, i);
      R[i] += accum_current - c->accum_prev[i];
      R[i] -= in->source_sink[i];
      double dmass_dP = c->rho[i] * 0.0 * c->S[i] + c->drho_dP[i] * in->porosity[i] * c->S[i] +
                        c->rho[i] * in->porosity[i] * c->dS_dP[i];
      double Jac = dmass_dP * in->volume[i] * dtInv;
      mat_add_row(c, J, NULL, i, 1, &i, &Jac, NULL);
    }
  }
}
