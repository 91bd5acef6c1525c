/*
 * tdycore_gb300.h -- C-ABI drop-in for TDycore's MPFA-O Richards residual and
 * Jacobian path, evaluated on one GB300 (sm_103a).
 *
 * Every entry point returns a TDyErrorCode (0 = success), mirroring the
 * PetscErrorCode convention of the reference (include/tdycore.h:137-256).
 * The last error message of the calling thread is available through
 * TDyGetErrorMessage().
 *
 * Arrays are plain pointers with sizes; no PETSc, MPI or torch types appear.
 * Host-pointer entry points copy to and from the device inside the call;
 * the "...Device" variants take device pointers and a cudaStream_t (passed as
 * void*; NULL means the handle's own stream) and return after enqueueing work.
 *
 * Each declaration cites the reference interface it replaces (file:line in
 * the TDycore source tree).
 */
#ifndef TDYCORE_GB300_H
#define TDYCORE_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int TDyErrorCode;
typedef struct _p_TDy *TDy;

/* Error codes: numeric values follow PETSc's (petscerror.h) so callers that
 * test PETSC_ERR_* constants keep working. */
#define TDY_SUCCESS              0
#define TDY_ERR_MEM             55
#define TDY_ERR_SUP             56
#define TDY_ERR_ARG_WRONG       62
#define TDY_ERR_ARG_OUTOFRANGE  63
#define TDY_ERR_LIB             76
#define TDY_ERR_USER            83
#define TDY_ERR_ARG_NULL        85
#define TDY_ERR_NOT_CONVERGED   91
#define TDY_ERR_GPU             97

/* Enumerations: identical names and values to include/tdycore.h:8-99 and
 * include/tdycore.h:63-72 (MPFA-O options). */
typedef enum { RICHARDS = 0, TH, SALINITY } TDyMode;
typedef enum { MPFA_O = 0, MPFA_O_DAE, MPFA_O_TRANSIENTVAR, BDM, WY, FV_TPF } TDyDiscretization;
typedef enum { MPFAO_GMATRIX_DEFAULT = 0, MPFAO_GMATRIX_TPF } TDyMPFAOGmatrixMethod;
typedef enum { DIRICHLET_BC = 0, NEUMANN_BC, SEEPAGE_BC } TDyBoundaryConditionType;
typedef enum {
  WATER_DENSITY_CONSTANT = 0,
  WATER_DENSITY_EXPONENTIAL = 1,
  WATER_DENSITY_BATZLE_AND_WANG = 2
} TDyWaterDensityType;
typedef enum { WATER_VISCOSITY_CONSTANT = 0, WATER_VISCOSITY_BATZLE_AND_WANG = 1 } TDyWaterViscosityType;
/* Characteristic-curve families (include/private/tdycharacteristiccurvesimpl.h:7-38). */
typedef enum { SAT_FUNC_GARDNER = 0, SAT_FUNC_VAN_GENUCHTEN = 1 } TDySaturationType;
typedef enum { REL_PERM_FUNC_IRMAY = 0, REL_PERM_FUNC_MUALEM = 1 } TDyRelativePermeabilityType;

/* Spatial callbacks: same shape as include/tdycore.h:74-99 with
 * PetscInt = int and PetscReal = double (32-bit-index PETSc build). */
typedef void (*TDyScalarSpatialFunction)(int n, double *x, double *f);
typedef void (*TDyVectorSpatialFunction)(int n, double *x, double *f);
typedef void (*TDyTensorSpatialFunction)(int n, double *x, double *f);
typedef void (*TDyScalarSpatialIntegerFunction)(int n, double *x, int *f);

/* ---------------------------------------------------------------------- */
/* Process-level setup: replaces TDyInit/TDyFinalize (include/tdycore.h:126-130).
 * argv is scanned for -tdy_* options read later by TDySetFromOptions. */
TDyErrorCode TDyInit(int argc, char **argv);
TDyErrorCode TDyInitNoArguments(void);
TDyErrorCode TDyFinalize(void);
/* Appends options given as one string ("-tdy_gravity 9.8 -tdy_water_density
 * EXPONENTIAL"); stands in for PetscOptionsInsertString. */
TDyErrorCode TDyOptionsInsertString(const char *options);
TDyErrorCode TDyOptionsClear(void);
const char *TDyGetErrorMessage(void);
/* Queries of the same options database, standing in for PetscOptionsGetReal,
 * PetscOptionsGetInt, PetscOptionsGetString and PetscOptionsHasName (used by
 * the reference's driver, src/tdyti.c:28-44, and its demos). *set is 1 when
 * the option is present; the value is left unchanged otherwise. A malformed
 * number returns TDY_ERR_ARG_WRONG. */
TDyErrorCode TDyOptionsGetReal(const char *name, double *value, int *set);
TDyErrorCode TDyOptionsGetInt(const char *name, int *value, int *set);
TDyErrorCode TDyOptionsGetString(const char *name, char *value, int len, int *set);
TDyErrorCode TDyOptionsHasName(const char *name, int *set);

/* Lifecycle: include/tdycore.h:137-143 (TDyCreate ... TDyDestroy).
 * comm is accepted for signature compatibility and must describe a single
 * process (pass NULL). */
TDyErrorCode TDyCreate(void *comm, TDy *tdy);
TDyErrorCode TDySetMode(TDy tdy, TDyMode mode);
TDyErrorCode TDySetDiscretization(TDy tdy, TDyDiscretization discretization);
/* Alias used by demo/SPE10/steady.c:109. */
TDyErrorCode TDySetDiscretizationMethod(TDy tdy, TDyDiscretization discretization);
TDyErrorCode TDySetFromOptions(TDy tdy);
TDyErrorCode TDySetup(TDy tdy);
/* Host half of TDySetup only (mesh, materials, transmissibility, pattern):
 * for consumers of the setup arrays; entry points that evaluate on the GPU
 * then return TDY_ERR_GPU. */
TDyErrorCode TDySetupHost(TDy tdy);
TDyErrorCode TDyDestroy(TDy *tdy);

/* Mesh construction: replaces TDySetDMConstructor + DMPlexCreateBoxMesh
 * (include/tdycore.h:140; demo/transient/transient_mpfaof90.F90:47).
 * TDySetBoxMesh builds nx*ny*nz hexahedra over [lower, upper] with cells
 * numbered x fastest, then y, then z, as DMPlexCreateBoxMesh does.
 * TDySetExtrudedMesh builds a z-extruded mesh from a surface mesh of nc2
 * polygons with nvpc (3 or 4) counter-clockwise vertices each, over nv2
 * surface vertices (xy[2*nv2]) and nlayers layers whose vertex elevations are
 * z[(nlayers+1)*nv2] (level-major).  Cells are numbered layer*nc2 + c2. */
TDyErrorCode TDySetBoxMesh(TDy tdy, int nx, int ny, int nz, const double lower[3], const double upper[3]);
TDyErrorCode TDySetExtrudedMesh(TDy tdy, int nv2, const double *xy, int nc2, int nvpc, const int *cells2d,
                                int nlayers, const double *z);
/* Extension: a batch of independent extruded meshes (instances) in one
 * handle, for batched evaluation and solves.  Block b has nv2[b] surface
 * vertices, nc2[b] polygons of nvpc vertices and nlayers[b] layers; xy,
 * cells2d (indices local to the block) and z hold the blocks one after the
 * other in the layout of TDySetExtrudedMesh.  Cells, vertices, faces and
 * boundary faces are numbered block by block, so instance b owns a contiguous
 * cell range; no face joins two blocks. */
TDyErrorCode TDySetExtrudedMeshes(TDy tdy, int nblocks, const int *nv2, const double *xy, const int *nc2, int nvpc,
                                  const int *cells2d, const int *nlayers, const double *z);

/* Material properties: include/tdycore.h:150-171. */
TDyErrorCode TDySetWaterDensityType(TDy tdy, TDyWaterDensityType type);
TDyErrorCode TDySetWaterViscosityType(TDy tdy, TDyWaterViscosityType type);
TDyErrorCode TDySetConstantPorosity(TDy tdy, double porosity);
TDyErrorCode TDySetPorosityFunction(TDy tdy, TDyScalarSpatialFunction f);
TDyErrorCode TDySetConstantIsotropicPermeability(TDy tdy, double k);
TDyErrorCode TDySetIsotropicPermeabilityFunction(TDy tdy, TDyScalarSpatialFunction f);
TDyErrorCode TDySetConstantDiagonalPermeability(TDy tdy, const double k[3]);
TDyErrorCode TDySetDiagonalPermeabilityFunction(TDy tdy, TDyVectorSpatialFunction f);
TDyErrorCode TDySetConstantTensorPermeability(TDy tdy, const double k[9]);
TDyErrorCode TDySetTensorPermeabilityFunction(TDy tdy, TDyTensorSpatialFunction f);
TDyErrorCode TDySetConstantResidualSaturation(TDy tdy, double sr);
TDyErrorCode TDySetResidualSaturationFunction(TDy tdy, TDyScalarSpatialFunction f);
/* Per-cell values (extension; the reference sets per-point parameters through
 * SaturationSetType/RelativePermeabilitySetType,
 * src/materials/tdycharacteristiccurves.c:72-113,271-316). cells may be NULL
 * to mean 0..n-1. */
TDyErrorCode TDySetPorosityValuesLocal(TDy tdy, int n, const int *cells, const double *phi);
TDyErrorCode TDySetPermeabilityValuesLocal(TDy tdy, int n, const int *cells, const double *k9);
TDyErrorCode TDySetResidualSaturationValuesLocal(TDy tdy, int n, const int *cells, const double *sr);
TDyErrorCode TDySetCharacteristicCurveVanGenuchtenValuesLocal(TDy tdy, int n, const int *cells, const double *m,
                                                               const double *alpha);
TDyErrorCode TDySetCharacteristicCurveMualemValuesLocal(TDy tdy, int n, const int *cells, const double *m);
/* Switch the saturation family to Gardner for the given cells (n, m, alpha per
 * cell) or the relative permeability family to Irmay (m per cell);
 * src/materials/tdycharacteristiccurves.c:641-667 and :451-460. */
TDyErrorCode TDySetCharacteristicCurveGardnerValuesLocal(TDy tdy, int n, const int *cells, const double *gn,
                                                          const double *gm, const double *alpha);
TDyErrorCode TDySetCharacteristicCurveIrmayValuesLocal(TDy tdy, int n, const int *cells, const double *m);

/* Boundary conditions and sources: include/tdycore.h:190-197 and
 * src/fv/mpfao/tdympfao.c:408-426 (MPFA-O options). */
TDyErrorCode TDySetBoundaryPressureFunction(TDy tdy, TDyScalarSpatialFunction f);
/* The reference's MPFA-O applies one boundary type to every boundary face;
 * when this per-face function is set (reference: tdycore.c:1350), faces take
 * the returned TDyBoundaryConditionType instead (extension). */
TDyErrorCode TDySetBoundaryPressureTypeFunction(TDy tdy, TDyScalarSpatialIntegerFunction f);
TDyErrorCode TDyMPFAOSetGmatrixMethod(TDy tdy, TDyMPFAOGmatrixMethod method);
TDyErrorCode TDyMPFAOSetBoundaryConditionType(TDy tdy, TDyBoundaryConditionType bctype);
/* Mass source per cell in kg/s (SNES form) or kg/s/m^3 (TS form); the
 * reference's source_sink array (src/fv/mpfao/tdympfao.c:364-384), which it
 * never fills, so the default of zero keeps parity. */
TDyErrorCode TDySetSourceSinkValuesLocal(TDy tdy, int n, const int *cells, const double *q);

/* Queries. */
TDyErrorCode TDyGetNumCells(TDy tdy, int *ncells);
TDyErrorCode TDyGetNumBoundaryFaces(TDy tdy, int *nbnd);
TDyErrorCode TDyGetCellCentroids(TDy tdy, double *xyz);
TDyErrorCode TDyGetCellVolumes(TDy tdy, double *vol);
/* Fixed CSR pattern of the Jacobian (cells sharing a vertex, sorted columns):
 * replaces TDyCreateJacobian (src/tdycore.c:2187) and the DMCreateMatrix
 * FVM++ adjacency (src/tdydiscretization.c:156-170). Pointers stay valid
 * until TDyDestroy. */
TDyErrorCode TDyGetJacobianPattern(TDy tdy, int *nrows, int *nnz, const int **rowptr, const int **colidx);
/* Vector/matrix creation are no-ops kept for call-sequence compatibility
 * (src/tdycore.c:2166, :2187). */
TDyErrorCode TDyCreateVectors(TDy tdy);
TDyErrorCode TDyCreateJacobian(TDy tdy);

/* ---------------------------------------------------------------------- */
/* Backward-Euler (SNES) form: src/fv/mpfao/tdympfao_snes.c:19-203. */
TDyErrorCode TDySetDtimeForSNESSolver(TDy tdy, double dt);                    /* include/tdycore.h:237 */
TDyErrorCode TDySetPreviousSolutionForSNESSolver(TDy tdy, const double *U);   /* include/tdycore.h:240 */
TDyErrorCode TDyPreSolveSNESSolver(TDy tdy);                                 /* src/tdycore.c:2074 */
TDyErrorCode TDyPostSolve(TDy tdy, const double *U);                         /* src/tdycore.c:2056 */
/* TDyOutputRegression (src/tdycore.c:1564, src/tdyregression.c:8-250): when
 * -tdy_regression_test was given to TDySetFromOptions, writes
 * "<-tdy_regression_test_filename>.regression" with the max, min and mean of
 * U and U at -tdy_regression_test_num_cells_per_process (default 2) cells
 * spaced floor(ncells / count) apart, in the reference's text format; a no-op
 * otherwise. TDySetup fails with TDY_ERR_USER when -tdy_regression_test is
 * set without a filename, as TDyRegressionInitialize does. */
TDyErrorCode TDyOutputRegression(TDy tdy, const double *U);
/* TDyMPFAOSNESFunction (tdympfao_snes.c:67): R[ncells] from U[ncells]. */
TDyErrorCode TDyMPFAOSNESFunction(TDy tdy, const double *U, double *R);
/* TDyMPFAOSNESJacobian (tdympfao_snes.c:143): J values in pattern order. */
TDyErrorCode TDyMPFAOSNESJacobian(TDy tdy, const double *U, double *J);
/* Fused residual + Jacobian at the same U (one state update). */
TDyErrorCode TDyMPFAOSNESFunctionJacobian(TDy tdy, const double *U, double *R, double *J);

/* TS (implicit, IFunction/IJacobian) form: src/fv/mpfao/tdympfao_ts.c:153,520. */
TDyErrorCode TDyMPFAOIFunction(TDy tdy, double t, const double *U, const double *U_t, double *R);
TDyErrorCode TDyMPFAOIJacobian(TDy tdy, double t, const double *U, const double *U_t, double shift, double *J);
TDyErrorCode TDyMPFAOIFunctionIJacobian(TDy tdy, double t, const double *U, const double *U_t, double shift,
                                        double *R, double *J);
/* ---------------------------------------------------------------------- */
/* Extension: device-resident backward-Euler Newton solve (no reference
 * counterpart: the reference hands F and J to PETSc's SNES and KSP).  One
 * call advances every instance of the handle (each block of
 * TDySetExtrudedMeshes, or the single mesh) by dt: presolve at dU, then Newton
 * with the FP64 residual until ||F|| <= rtol ||F_0|| (or <= atol) per
 * instance (or until the Newton step is below stol ||U||, PETSc's step test),
 * with a backtracking line search per instance; each Newton system solved by BiCGStab preconditioned with exact
 * solves of the vertical lines of the extruded blocks or of strong-coupling
 * clusters (TDyNewtonOptions.precond), in FP32 (the Jacobian is rounded to
 * FP32) or FP64.  dU (device, ncells) holds U_n on entry and
 * U_{n+1} on return. */
typedef struct {
  double rtol;         /* relative FP64 residual per instance (default 1e-8) */
  double atol;         /* absolute residual (default 0) */
  int max_it;          /* Newton iterations (default 50, as PETSc SNES) */
  int linear_fp32;     /* 1: FP32 Jacobian and inner solve (default); 0: FP64 */
  double linear_rtol;  /* BiCGStab relative tolerance per instance (default 1e-6) */
  int linear_max_it;   /* BiCGStab iterations per Newton iteration (default 400); an FP32 inner
                          solve stops after a quarter of them (at least 20) and, if not converged
                          by then, that instance's solve is redone in FP64 */
  double stol;         /* step tolerance: converged when ||step|| < stol ||U|| per instance
                          (PETSc's CONVERGED_SNORM_RELATIVE; default 1e-8) */
  int precond;         /* TDY_PRECOND_LINES (default) or TDY_PRECOND_CLUSTERS */
  double cluster_threshold; /* clusters: a coupling with |a_ij| >= threshold sqrt(|a_ii a_jj|)
                               joins cells i and j (default 0.05) */
  int schedule;        /* inner-solve schedule with the line preconditioner: TDY_SCHEDULE_AUTO
                          (default), _TILE or _BLOCK; every schedule gives the same bits */
  int fp32_max_it;     /* with linear_fp32: Newton iterations with the FP32 inner solve, FP64 after
                          (an instance still iterating then stalls on FP32 directions; default 8,
                          negative: FP32 throughout) */
  int spmv_threads;    /* threads per row of the inner solve's sparse products: 0 (default) timed
                          on the process's first solve; 1, 2, 4 or 8.  Every choice gives the same
                          bits (each row is summed in 8 phases added by a fixed tree) */
} TDyNewtonOptions;
/* Inner-solve schedules.  TILE: every kernel of a BiCGStab iteration runs over
 * all cells of the batch, instances masked as they converge (one iteration is
 * a CUDA graph).  BLOCK: one CTA per instance runs the instance's whole
 * BiCGStab loop (CTAs take instances from a counter, largest first).  AUTO:
 * an autotuner times the tile, block and split schedules (instances up to
 * 4096, 16384 or 65536 cells on the block schedule, the rest on the tile
 * schedule) on the first solve of a size class and keeps the fastest for the
 * process.  The cluster preconditioner runs on the tile schedule. */
#define TDY_SCHEDULE_AUTO 0
#define TDY_SCHEDULE_TILE 1
#define TDY_SCHEDULE_BLOCK 2
/* Inner-solve preconditioners.  LINES: exact solves of the vertical lines of
 * the extruded blocks.  CLUSTERS: exact solves of the connected clusters of
 * strong couplings (up to 64 cells each; cells of larger clusters take their
 * diagonal), for meshes whose lateral couplings are not monotone (MPFA-O
 * with anisotropic K on obtuse prisms), where line solves diverge. */
#define TDY_PRECOND_LINES 0
#define TDY_PRECOND_CLUSTERS 1
typedef struct {
  int newton_iterations;        /* largest over the instances */
  long long linear_iterations;  /* BiCGStab iterations, summed over instances and Newton iterations */
  int converged;                /* instances whose FP64 residual met rtol (or atol) */
  int ninstances;
  double max_rel_residual;      /* largest final ||F|| / ||F_0|| */
  int step_converged;           /* instances ended by the step test (stol) above rtol: not in `converged` */
  int precond_used;             /* preconditioner of the last inner solve (TDY_PRECOND_*); CLUSTERS falls
                                   back to LINES when the cluster labels do not settle */
  int clusters;                 /* last inner solve: clusters of 2..64 cells factored */
  int cluster_cells;            /* last inner solve: cells in those clusters */
  int cluster_cells_diagonal;   /* last inner solve: cells of clusters larger than 64 (they take their diagonal) */
  int block_instances;          /* last inner solve: instances on the block schedule */
  long long block_max_cells;    /* last inner solve: the split (instances up to this many cells on the block
                                   schedule; -1 none) */
  int fp64_fallback;            /* 1 if Newton went past fp32_max_it and finished with FP64 inner solves */
  int eval_schedule;            /* evaluation of every instance: 0 three-stage launches, 1 one CTA per
                                   instance (timed on the handle's first evaluation; the same bits) */
  double eval_s;                /* seconds on the solve's stream in F+J evaluations (line-search trials
                                   included) */
  double precond_s;             /* ... in Jacobian copies to the inner solve's precision and
                                   preconditioner set-ups */
  double krylov_s;              /* ... in BiCGStab iterations (schedule tuning on a size class's first
                                   solve included) */
  int fp64_inner_redo;          /* FP32 inner solves that ran out of iterations and were redone in FP64
                                   (instances x Newton iterations) */
} TDyNewtonStats;
TDyErrorCode TDyNewtonOptionsDefault(TDyNewtonOptions *o);
TDyErrorCode TDyGetNumInstances(TDy tdy, int *n);
/* Extension for batched handles (no reference counterpart): which instances
 * the next TDyBackwardEulerStepDevice calls advance (host array of
 * ninstances flags; NULL: all).  An inactive instance keeps its state and
 * costs no evaluation or inner solve; it is reported with 0 iterations and
 * not counted as converged.  For a caller that retires some instances of a
 * batch (a server whose request failed) and goes on with the others. */
TDyErrorCode TDySetActiveInstances(TDy tdy, int ninstances, const int *active);
/* Per-instance outcome of the last TDyBackwardEulerStepDevice call (host
 * array of ninstances): TDY_INSTANCE_CONVERGED (FP64 residual met the
 * tolerance), _STEP_TEST (ended by the step test above it), _NOT_CONVERGED,
 * _INACTIVE (not advanced). */
#define TDY_INSTANCE_NOT_CONVERGED 0
#define TDY_INSTANCE_CONVERGED 1
#define TDY_INSTANCE_STEP_TEST 2
#define TDY_INSTANCE_INACTIVE 3
TDyErrorCode TDyGetInstanceStatus(TDy tdy, int ninstances, int *status);
/* inst_iterations and inst_rel_residual (host, ninstances entries) may be NULL. */
TDyErrorCode TDyBackwardEulerStepDevice(TDy tdy, double dt, double *dU, const TDyNewtonOptions *opt,
                                        TDyNewtonStats *stats, int *inst_iterations, double *inst_rel_residual,
                                        void *stream);

/* ---------------------------------------------------------------------- */
/* TS variants with the same flux kernels (TDySetDiscretization MPFA_O_TRANSIENTVAR
 * or MPFA_O_DAE; src/tdycore.c:1902-1908). */
/* TDyMPFAOTransientVariable (tdympfao_ts_transientvar.c:13-47): the conserved
 * variable C = rho * porosity * S * volume per cell. */
TDyErrorCode TDyMPFAOTransientVariable(TDy tdy, const double *U, double *C);
/* Extension: dC/dP per cell (d(rho porosity S)/dP * volume). */
TDyErrorCode TDyMPFAOTransientVariableDerivative(TDy tdy, const double *U, double *dC);
/* TDyMPFAOIFunction_TransientVariable (tdympfao_ts_transientvar.c:50-101):
 * R = fluxes + M_t * volume - source * volume, M_t the rate of C. */
TDyErrorCode TDyMPFAOIFunctionTransientVariable(TDy tdy, double t, const double *U, const double *M_t, double *R);
/* Extension: the Jacobian of that residual when M_t = shift * C(U) + const
 * (fluxes + shift * dC/dP on the diagonal), in pattern order.  The reference
 * registers no IJacobian for this form and lets PETSc difference it. */
TDyErrorCode TDyMPFAOIJacobianTransientVariable(TDy tdy, double t, const double *U, double shift, double *J);
/* TDyMPFAOIFunction_DAE (tdympfao_ts_dae.c:13-84): U, U_t and R hold
 * [P, M] interleaved per cell (2 * ncells values); R_P = M_t * volume -
 * source * volume + fluxes, R_M = M - rho * porosity * S * volume.  The
 * reference registers no IJacobian for this form either. */
TDyErrorCode TDyMPFAOIFunctionDAE(TDy tdy, double t, const double *U, const double *U_t, double *R);

/* Device-pointer variants (HBM-resident operands). R or J may be NULL to
 * skip that output. stream is a cudaStream_t or NULL. */
TDyErrorCode TDyMPFAOSNESFunctionJacobianDevice(TDy tdy, const double *dU, double *dR, double *dJ, void *stream);
TDyErrorCode TDyMPFAOIFunctionIJacobianDevice(TDy tdy, double t, const double *dU, const double *dU_t, double shift,
                                              double *dR, double *dJ, void *stream);
TDyErrorCode TDyPreSolveSNESSolverDevice(TDy tdy, const double *dU_prev, void *stream);
/* Extension for batched handles (TDySetExtrudedMeshes; no reference
 * counterpart): the SNES residual and Jacobian of the listed instances only
 * (host array of ninst instance indices), in one launch with one CTA per
 * instance at a time; the other instances' rows of dR and dJ are left as they
 * are.  Each listed instance gets the same bits as from
 * TDyMPFAOSNESFunctionJacobianDevice.  For Newton loops in which only some
 * instances still iterate.  TDY_ERR_SUP when the handle's rows are longer
 * than 96 entries. */
TDyErrorCode TDyMPFAOSNESFunctionJacobianDeviceInstances(TDy tdy, const double *dU, double *dR, double *dJ,
                                                         int ninst, const int *instances, void *stream);
/* Same result as TDyMPFAOSNESFunctionJacobianDevice, but the call allocates
 * no device memory at all: its partial-sum scratch is a fixed 64 MiB array
 * built into the library (8,388,608 doubles; every GPU that loads the library
 * keeps it until the process exits) rather than memory belonging to the
 * handle.  Meant for callers that are not allowed to allocate on the device
 * while they run, such as a host application whose device memory is handed
 * out by its own pool and must not change behind its back, or a time-critical
 * loop that cannot afford the device-wide synchronisation cudaMalloc and
 * cudaFree may cause.  The caller passes inputs and outputs as device
 * pointers.  Meshes whose scratch would exceed the array (about 110,000
 * interior hexahedral vertices) are rejected with TDY_ERR_ARG_OUTOFRANGE.
 * TDySetup looks up the array's device address once per device, so the call
 * itself loads nothing and allocates nothing, even the first time.  All
 * calls share the array:
 * calls that overlap on the GPU race and must be serialised by the caller.
 * This entry point has no counterpart in the reference. */
TDyErrorCode TDyMPFAOSNESFunctionJacobianDeviceNoAlloc(TDy tdy, const double *dU, double *dR, double *dJ,
                                                       void *stream);
/* Number of hot-path kernel launches one ...Device call enqueues. */
TDyErrorCode TDyGetLaunchesPerEvaluation(TDy tdy, int *nlaunch);
TDyErrorCode TDySynchronize(TDy tdy);

/* Per-kernel timers, the analogue of the reference's TDY_START_FUNCTION_TIMER
 * event log (include/tdytimers.h; -tdy_timers).  While enabled every
 * evaluation records CUDA events between its kernels and waits for them, so
 * enable timers for measurement runs only.  TDyGetTimers fills up to *n
 * entries (kernel name, total milliseconds, launch count) and sets *n to the
 * number of timed kernels. */
TDyErrorCode TDySetTimersEnabled(TDy tdy, int on);
TDyErrorCode TDyGetTimers(TDy tdy, int *n, const char **names, double *ms_total, long long *calls);
/* Achieved FP64 FMA throughput of the current device (TFLOP/s), the
 * denominator of the FP64 roofline fraction reported beside HBM. */
TDyErrorCode TDyDeviceFP64Throughput(double *tflops);

/* State and diagnostics: TDyUpdateState (src/tdycore.c:1461) and
 * TDyGetLiquidSaturation/TDyGetLiquidMass (include/tdycore.h:213-215).
 * Outputs are host arrays of ncells values. */
TDyErrorCode TDyUpdateState(TDy tdy, const double *U, int ncells);
TDyErrorCode TDyGetLiquidSaturation(TDy tdy, double *S);
TDyErrorCode TDyGetLiquidMass(TDy tdy, double *mass);

/* Setup export for test harnesses (host arrays owned by the handle); the
 * layout is described in tdycore_gb300_setup.h. */
struct TDyMPFAOSetupView;
/* With -tdy_mpfao_setup_on_device the interior vertices' Trans is built on
 * the device; the first call copies it into the host arrays of the view. */
TDyErrorCode TDyMPFAOGetSetupView(TDy tdy, struct TDyMPFAOSetupView *view);

#ifdef __cplusplus
}
#endif
#endif
