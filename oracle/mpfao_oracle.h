/*
 * mpfao_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of TDycore's MPFA-O Richards residual and Jacobian
 * (src/fv/mpfao/tdympfao_ts.c, tdympfao_snes.c, tdympfao.c:2527-2594,
 * tdympfao_utils.c:24-99,690-759, src/materials/tdycharacteristiccurves.c,
 * src/materials/tdyeos.c), used by the test-suite and by the CPU baseline of
 * bench.py as the checker.  The product library never links or calls it.
 *
 * The oracle takes the setup arrays (per-vertex transmissibility blocks,
 * gravity discretization, face connectivity, cell parameters) as input and
 * evaluates F and J with the reference's loop structure and operation order,
 * including a sorted-column CSR product standing in for MatMult on Trans_mat
 * and a binary-search ADD standing in for MatSetValuesLocal.
 */
#ifndef MPFAO_ORACLE_H
#define MPFAO_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int ncells, nfaces, nbnd, nverts;
  int bc_type, rho_type, mu_type;
  double Pref;
  /* cells */
  const double *volume, *porosity, *Sr;
  const int *sat_type;
  const double *sat_param;     /* 3 per cell */
  const int *relperm_type;
  const double *relperm_param; /* 9 per cell */
  const double *source_sink;
  /* faces: reference encoding (>=0 cell, <0 -(b+1)) */
  const int *face_up, *face_dn;
  const double *gravdis;
  /* boundary */
  const int *bnd_face, *bnd_type, *bnd_has_value;
  const double *bnd_value, *rho_bnd, *vis_bnd;
  /* vertices */
  const int *v_row_off, *v_col_off, *v_nint;
  const long long *v_trans_off;
  const int *row_face, *col_ext;
  const double *trans;
} OracleInput;

typedef struct OracleCtx OracleCtx;

OracleCtx *oracle_create(const OracleInput *in);
void oracle_destroy(OracleCtx *ctx);
/* Number of threads for the *_parallel entry points (OpenMP). */
int oracle_max_threads(void);

/* Jacobian pattern computed independently from the vertex cell lists. */
int oracle_pattern_nnz(OracleCtx *ctx);
void oracle_pattern(OracleCtx *ctx, int *rowptr, int *colidx);

/* TDyMPFAOSNESPreSolve (tdympfao_snes.c:32-64) */
void oracle_snes_presolve(OracleCtx *ctx, const double *Uprev, double dt);
/* TDyMPFAOSNESFunction (tdympfao_snes.c:67-140); Rmag (may be NULL) receives
 * the floating-point error scale of R[i]: for each flux added into R[i],
 * |rho ukvr| (sum_c |T_c P_c| + |rho G|), plus the absolute accumulation
 * terms.  Jmag likewise holds, per entry, the sum of the error scales of the
 * contributions (products evaluated in absolute value). */
void oracle_snes_function(OracleCtx *ctx, const double *U, double *R, double *Rmag);
/* TDyMPFAOSNESJacobian (tdympfao_snes.c:143-203); J in pattern order. */
void oracle_snes_jacobian(OracleCtx *ctx, const double *U, double *J, double *Jmag);
/* TDyMPFAOIFunction / TDyMPFAOIJacobian (tdympfao_ts.c:153-227, 520-561) */
void oracle_ts_ifunction(OracleCtx *ctx, const double *U, const double *Ut, double *R, double *Rmag);
void oracle_ts_ijacobian(OracleCtx *ctx, const double *U, const double *Ut, double shift, double *J, double *Jmag);
/* transient-variable and DAE forms (tdympfao_ts_transientvar.c, tdympfao_ts_dae.c) */
void oracle_transient_variable(OracleCtx *ctx, const double *U, double *C, double *dC);
void oracle_tv_ifunction(OracleCtx *ctx, const double *U, const double *Mdot, double *R, double *Rmag);
void oracle_tv_ijacobian(OracleCtx *ctx, const double *U, double shift, double *J, double *Jmag);
void oracle_dae_ifunction(OracleCtx *ctx, const double *U, const double *Ut, double *R, double *Rmag);
/* Fused SNES F+J over all host threads, vertices processed by colour (used
 * for the CPU baseline timing; same arithmetic, different summation order). */
void oracle_snes_function_parallel(OracleCtx *c, const double *U, double *R, int nthreads);
void oracle_snes_function_jacobian_parallel(OracleCtx *ctx, const double *U, double *R, double *J, int nthreads);
/* Per-cell state after the last evaluation (for diagnostics tests). */
void oracle_get_state(OracleCtx *ctx, double *S, double *rho, double *Kr);

#ifdef __cplusplus
}
#endif
#endif
