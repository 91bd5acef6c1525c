/*
 * tdycore_gb300_setup.h -- read-only view of the MPFA-O setup arrays built by
 * TDySetup, exported for test harnesses and CPU baselines.
 *
 * The view restates the fields of the reference's TDyMPFAO context
 * (include/private/tdympfaoimpl.h:13-117) and TDyMesh
 * (include/private/tdymeshimpl.h:35-219) that the residual/Jacobian path
 * reads, in flat arrays:
 *
 *   - ext index: cells are 0..ncells-1; boundary face b is ncells+b.  The
 *     reference encodes a boundary side of a face as cell id -(b+1)
 *     (src/fv/share/tdymeshplex.c:405-424); face_up/face_dn keep that encoding.
 *   - per vertex v: rows v_row_off[v]..v_row_off[v+1]-1 (one per subface at v
 *     that carries a flux: internal, Dirichlet or seepage faces; Neumann
 *     boundary faces carry none), columns v_col_off[v]..v_col_off[v+1]-1 (the
 *     v_nint[v] internal cells first, then Dirichlet/seepage boundary faces),
 *     and a dense row-major block trans[v_trans_off[v] + r*ncol + c]: the
 *     reference's Trans[v][row][col] (tdympfao.c:2310, :1417-1449).
 *   - gravdis per face: the reference's GravDisVec entry, identical for every
 *     subface of a face (tdympfao.c:2169-2274).
 */
#ifndef TDYCORE_GB300_SETUP_H
#define TDYCORE_GB300_SETUP_H

#ifdef __cplusplus
extern "C" {
#endif

struct TDyMPFAOSetupView {
  int ncells, nfaces, nbnd, nverts;
  int nrows_total;          /* sum over vertices of rows */
  int ncols_total;          /* sum over vertices of columns */
  long long ntrans_total;   /* sum over vertices of rows*cols */
  int bc_type;              /* global TDyBoundaryConditionType */
  int gmatrix_method;
  int rho_type, mu_type;
  double gravity;           /* magnitude, gravity vector is (0,0,gravity) */
  double Pref;
  /* cells */
  const double *volume;        /* [ncells] */
  const double *centroid;      /* [3*ncells] */
  const double *porosity;      /* [ncells] */
  const double *Sr;            /* [ncells] */
  const double *K0;            /* [9*ncells], row major */
  const int *sat_type;         /* [ncells] TDySaturationType */
  const double *sat_param;     /* [3*ncells]: VG (m, alpha, -), Gardner (n, m, alpha) */
  const int *relperm_type;     /* [ncells] TDyRelativePermeabilityType */
  const double *relperm_param; /* [9*ncells]: Mualem (m,x0,x1,x2,dx,c0,c1,c2,c3), Irmay (m,...) */
  const double *source_sink;   /* [ncells] */
  /* faces */
  const int *face_up;          /* [nfaces] reference encoding */
  const int *face_dn;          /* [nfaces] */
  const double *gravdis;       /* [nfaces] */
  const double *face_centroid; /* [3*nfaces] */
  const double *face_area;     /* [nfaces] */
  const double *face_normal;   /* [3*nfaces] */
  const int *face_nverts;      /* [nfaces] */
  /* boundary faces */
  const int *bnd_face;         /* [nbnd] face id of boundary face b */
  const int *bnd_type;         /* [nbnd] TDyBoundaryConditionType */
  const int *bnd_has_value;    /* [nbnd] 1 if P_bnd comes from the BC function */
  const double *bnd_value;     /* [nbnd] BC function value at the face centroid */
  const double *rho_bnd;       /* [nbnd] density at Pref */
  const double *vis_bnd;       /* [nbnd] viscosity at Pref */
  /* vertices */
  const int *v_row_off;        /* [nverts+1] */
  const int *v_col_off;        /* [nverts+1] */
  const int *v_nint;           /* [nverts] */
  const long long *v_trans_off;/* [nverts+1] */
  const int *row_face;         /* [nrows_total] */
  const int *col_ext;          /* [ncols_total] */
  const double *trans;         /* [ntrans_total] */
  /* Jacobian pattern */
  const int *rowptr;           /* [ncells+1] */
  const int *colidx;           /* [nnz] */
  int nnz;
};

#ifdef __cplusplus
}
#endif
#endif
