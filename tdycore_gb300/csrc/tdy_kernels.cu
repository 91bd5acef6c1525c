// tdy_kernels.cu -- sm_103a kernels of the MPFA-O Richards residual and
// Jacobian, and their host-side launch code.
//
// One evaluation is three stages on one stream:
//   1. state_kernel   (cells, then boundary faces)
//        TDyUpdateState_Richards_MPFAO (src/fv/mpfao/tdympfao.c:2527-2594),
//        TDyMPFAO_SetBoundaryPressure + TDyMPFAOUpdateBoundaryState
//        (src/fv/mpfao/tdympfao_utils.c:24-99, 690-759) and the accumulation
//        terms of TDyMPFAOSNESFunction/Jacobian (tdympfao_snes.c:19-30,
//        112-123, 166-179) or TDyMPFAOIFunction/IJacobian_Accumulation
//        (tdympfao_ts.c:191-212, 459-517).
//   2. vertices: MatMult(Trans_mat, P_vec) (tdympfao_ts.c:184) restricted to
//        the vertex's rows, the upwinded flux of TDyMPFAOIFunction_Vertices
//        (tdympfao_ts.c:12-150) and the Jacobian entries of
//        TDyMPFAOIJacobian_Vertices (tdympfao_ts.c:235-456).  Each vertex
//        writes its partial residual R_v[nint] and partial Jacobian block
//        J_v[nint][nint] (rows and columns: the vertex's internal cells) to a
//        scratch area it alone owns.  Interior hexahedral vertices use a fixed
//        octant layout (rows and columns known at compile time, structure-of-
//        arrays storage read with coalesced loads, one thread each, in
//        vertex_kernel); the others use per-vertex blocks, one thread each in
//        the first blocks of vertex_kernel when canonical vertices dominate,
//        else one warp each in generic_vertex_kernel (a launch of its own).
//   3. cells: sum, in a fixed order, the partials of the cell's vertices into
//        R[cell] and into the cell's row of the fixed CSR pattern, then add
//        the accumulation terms (cell_kernel: structured cells, and the
//        others one thread each when structured cells dominate; else the
//        others one warp each in generic_cell_kernel).  No atomics, and the
//        thread and warp forms sum in the same order: results are bitwise
//        reproducible run to run and independent of the form.
//
// Per row the flux is evaluated as -w*(T.P + rho_avg*G) with w = rho_avg*kr/mu
// and the Jacobian entry as -(w*T + E) with E the derivative terms of the
// up/down cell, the same quantities as the reference's
// rho*kr/mu*(-T.P) - rho^2*kr/mu*G and its five-term derivative
// (tdympfao_ts.c:116-118, 404-417) regrouped to need fewer FP64 operations.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

#include "tdy_arena.h"
#include "tdy_device.h"
#include "tdy_emit.h"
#include "tdy_ff.h"

namespace tdy {

#define TDY_MAX_ROWS 64
#define TDY_MAX_NINT 64
// Jacobian row length: the gather program stores slots in 8 bits (the
// generic cell kernel stages one row per warp in shared memory)
#define TDY_MAX_ROW_NNZ 255

struct DevArgs {
  int nc, nb, nv;
  int form;
  int rho_type, mu_type;
  int needR, needJ;
  double Pref, dt, shift;
  // inputs
  const double *U, *Ut;
  // cells
  const double *vol, *poro, *Sr, *sat_param, *rp_param, *ss, *accum_prev;
  const double *lam_sat;  // kr(Se = 1) / mu per cell (saturated cells)
  double vis;             // water viscosity (constant at Tref and zero salinity)
  const int *sat_type, *rp_type;
  // boundary faces
  const int *bnd_cell, *bnd_type, *bnd_has;
  const double *bnd_val, *bnd_rho, *bnd_vis;
  // extended state (cells then boundary faces): P, rho/2, (drho/dP)/2, kr/mu,
  // d(kr/mu)/dP, seepage flag
  double *P, *hr, *hdr, *lam, *dlam;
  unsigned char *seep;
  double *acc_a, *acc_b, *jdiag;
  // faces
  const int *f_up, *f_dn;
  const double *G;
  // canonical interior-hex vertices (SoA, stride nCpad); a launch takes those in [vc0, vc1)
  int nC, nCpad, vc0, vc1;
  const double *Tc;
  int jac_ff;  // Jacobian products of canonical vertices in double-float
  const int *cellc, *facec;
  // generic vertices
  int ngen;
  int gen_warp_doubles;  // shared memory of one generic-vertex warp (doubles)
  const int *gen_vertex;
  const int *v_row_off, *v_col_off, *v_nint;
  const long long *v_trans_off, *v_jv_off;
  const int *row_face, *row_lup, *row_ldn, *col_ext;
  const double *trans;
  double *scratch;
  // cell gather
  const int *rowptr, *cv_off, *cv_stride, *cv_nint, *cv_local, *cv_slot_off;
  const long long *cv_jbase, *cv_rbase;
  const unsigned char *cv_slots;
  int max_row_nnz;
  int nS, nSpad, ngc;
  const int *sc_cells, *sc_vc, *gc_cells;
  // outputs
  double *R, *J;
};

// The entities of one instance (block of a batched handle): cells [c0, c1),
// boundary faces [b0, b1), canonical vertices [vc0, vc1), other vertices
// gen_vertex[g0, g1), structured cells sc_cells[s0, s1), other cells
// gc_cells[gc0, gc1).
struct InstRange {
  int c0, c1, b0, b1, vc0, vc1, g0, g1, s0, s1, gc0, gc1;
};

// timer groups: the state kernel, the vertex kernels, the cell kernels
static const char *const kKernelNames[3] = {"state_kernel", "vertex_kernel", "cell_kernel"};

struct DeviceState {
  cudaStream_t stream = nullptr;
  DevArgs a;
  // per-kernel timers (TDY_START_FUNCTION_TIMER analogue, include/tdytimers.h)
  bool timers = false;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  double t_ms[3] = {0, 0, 0};
  long long t_calls[3] = {0, 0, 0};
  int device = 0;  // CUDA device current at TDySetup
  // owned allocations
  std::vector<void *> allocs;
  double *dU = nullptr, *dUt = nullptr, *dR = nullptr, *dJ = nullptr;
  double *diagS = nullptr, *diagMass = nullptr;
  double *dae = nullptr;  // DAE form: U, U_t, R interleaved (6 * nc), on first use
  int nnz = 0;
  // host-pointer evaluations in slabs of cells (see build_slabs): each slab's
  // rows of R and J go to host memory while the next slabs are evaluated
  struct Slab {
    int e0, e1;        // cells whose state this slab computes (its vertices read up to e1)
    int c0, c1;        // cells
    int vc0, vc1;      // canonical vertices
    int g0, g1;        // other vertices (indices into gen_vertex)
    int s0, s1;        // structured cells (indices into sc_cells)
    int gc0, gc1;      // other cells (indices into gc_cells)
    long long j0, j1;  // Jacobian values
  };
  std::vector<Slab> slabs;
  cudaStream_t copy_stream = nullptr;
  std::vector<cudaEvent_t> slab_ev;
  // the slab pipeline as one graph for pinned host buffers, with what its
  // nodes bake in (rebuilt when a call differs)
  struct SlabKey {
    int form = -1;
    double dt = 0.0, shift = 0.0;
    const double *U = nullptr, *Ut = nullptr;
    double *R = nullptr, *J = nullptr;
    bool operator==(const SlabKey &o) const {
      return form == o.form && dt == o.dt && shift == o.shift && U == o.U && Ut == o.Ut && R == o.R && J == o.J;
    }
  };
  cudaGraphExec_t slab_exec = nullptr;
  SlabKey slab_key;
  // callers' streams that enqueued work on this handle, each with an event
  // recorded after its last enqueue: TDyDestroy waits for them before the
  // stream-ordered frees (which do not synchronise the device)
  std::vector<std::pair<cudaStream_t, cudaEvent_t>> user_streams;
  // instance schedule (handles whose blocks are laid out contiguously):
  // per-instance ranges, the list of a call, its ticket; smem bytes per CTA
  InstRange *inst_rng = nullptr;
  int *inst_list = nullptr, *inst_ticket = nullptr;
  std::vector<InstRange> h_inst_rng;
  std::vector<long long> h_inst_cells;
  std::vector<int> h_list;
  size_t inst_smem = 0;
  bool inst_ok = false;
  // recorded after every allocation-free evaluation (created at set-up, so
  // that call creates nothing); such calls never overlap, so the last one
  // covers them all
  cudaEvent_t noalloc_ev = nullptr;
};

#define CUDA_TRY(call)                                                                          \
  do {                                                                                          \
    cudaError_t e_ = (call);                                                                    \
    if (e_ != cudaSuccess)                                                                      \
      return set_error(TDY_ERR_GPU, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

// ---------------------------------------------------------------------------
// Constitutive relations, restated from src/materials/tdycharacteristiccurves.c
// and src/materials/tdyeos.c with the reference's operation order.

// PressureSaturation_VanGenuchten (tdycharacteristiccurves.c:692-717) and
// PressureSaturation_Gardner (:641-667).
__device__ __forceinline__ void saturation(int type, const double *par, double Sr, double Pc, double *S, double *dS,
                                           double *d2S) {
  if (type == SAT_FUNC_VAN_GENUCHTEN) {
    const double m = par[0], alpha = par[1];
    if (Pc <= 0) {
      *S = 1;
      *dS = 0;
      *d2S = 0.0;
    } else {
      // PressureSaturation_VanGenuchten (tdycharacteristiccurves.c:692-717)
      // with two powers instead of four: (1 + x^n)^(m+1) = (1 + x^n) / Se and
      // (1 + x^n)^(-m-2) = Se / (1 + x^n)^2 (FP64 pow is the cost here)
      double n = 1 / (1 - m);
      double pc_alpha = Pc * alpha;
      double pc_alpha_n = pow(pc_alpha, n);
      double one_plus = 1 + pc_alpha_n;
      double Se = pow(one_plus, -m);
      *S = (1.0 - Sr) * Se + Sr;
      double dSe_dPc = -m * n * alpha * pc_alpha_n * Se / (pc_alpha * one_plus);
      *dS = -dSe_dPc * (1.0 - Sr);
      double d2Se = m * n * pc_alpha_n * (Se / (one_plus * one_plus)) * ((m * n + 1.0) * pc_alpha_n - n + 1) / (Pc * Pc);
      *d2S = (1.0 - Sr) * d2Se;
    }
  } else {
    const double m = par[1], alpha = par[2];
    if (Pc < 0) {
      *S = 1;
      *dS = 0;
      *d2S = 0.0;
    } else {
      double Se = exp(-alpha * Pc / m);
      *S = (1.0 - Sr) * Se + Sr;
      double dSe_dPc = -alpha / m * exp(-alpha * Pc / m);
      *dS = -dSe_dPc * (1.0 - Sr);
      double d2Se = -alpha / m * dSe_dPc;
      *d2S = (1.0 - Sr) * d2Se;
    }
  }
}

// RelativePermeability_Mualem (tdycharacteristiccurves.c:468-485, 551-562,
// 607-614) and RelativePermeability_Irmay (:451-460).
__device__ __forceinline__ void relperm(int type, const double *p, double Se, double *Kr, double *dKr) {
  if (type == REL_PERM_FUNC_MUALEM) {
    const double m = p[0], x0 = p[1], x1 = p[2], dx = p[4];
    if (Se > x1) {
      double xt = (Se - x0) / dx;
      *Kr = p[5] + xt * (p[6] + xt * (p[7] + xt * p[8]));
      *dKr = (p[6] + xt * (2.0 * p[7] + xt * 3.0 * p[8])) / dx;
    } else {
      *Kr = 1.0;
      *dKr = 0.0;
      if (Se >= 1.0) return;
      // two powers instead of five: Se^(1/m - 1/2) = so / sqrt(Se),
      // (1 - so)^(m-1) = tmp / (1 - so), (1 - so)^m = tmp
      double so = pow(Se, 1 / m);
      double oms = 1 - so;
      double tmp = pow(oms, m);
      double sq = sqrt(Se);
      double kr = sq * ((1 - tmp) * (1 - tmp));
      *Kr = kr;
      double d = 0.5 * kr / Se;
      d += 2 * (so / sq) * (tmp / oms) * (1 - tmp);
      *dKr = d;
    }
  } else {
    const double m = p[0];
    *Kr = 1.0;
    *dKr = 0.0;
    if (Se >= 1.0) return;
    *Kr = pow(Se, m);
    *dKr = pow(Se, m - 1) * m;
  }
}

// EOSComputeWaterDensity / EOSComputeWaterViscosity (tdyeos.c:5-136) at
// T = Tref and zero salinity.
// EOSComputeWaterDensity_Constant (tdyeos.c:5-14)
constexpr double kRhoConst = 998.0;

__device__ __forceinline__ void density(int type, double p, double *rho, double *drho, double *d2rho) {
  if (type == WATER_DENSITY_CONSTANT) {
    *rho = kRhoConst;
    *drho = 0.0;
    *d2rho = 0.0;
  } else if (type == WATER_DENSITY_EXPONENTIAL) {
    if (p < 101325.e0) {
      *rho = 997.16e0;
      *drho = 0.0;
      *d2rho = 0.0;
    } else {
      double r = 997.16e0 * exp(1.e-8 * (p - 101325.e0));
      *rho = r;
      *drho = 1.e-8 * r;
      *d2rho = 1.e-8 * (1.e-8 * r);
    }
  } else {
    const double T = 25.0, P = p * 1.e-6;
    double pw = 1 + 1.e-6 * (-80. * T - 3.3 * (T * T) + 0.00175 * (T * T * T) + 489. * P - 2. * T * P +
                             0.016 * P * (T * T) - 1.3e-5 * (T * T * T) * P - 0.333 * (P * P) - 0.002 * T * (P * P));
    *rho = pw * 1000.;
    *drho = 0.0;
    *d2rho = 0.0;
  }
}

__device__ __forceinline__ void viscosity(int type, double *vis, double *dvis) {
  if (type == WATER_VISCOSITY_CONSTANT) {
    *vis = 9.94e-4;
  } else {
    const double T = 25.0;
    *vis = (0.1 + 1.65 * exp((-0.42 * (0.17 * 0.17) + 0.045) * pow(T, 0.8))) * 1e-3;
  }
  *dvis = 0.0;
}

// ---------------------------------------------------------------------------
// 1. cell and boundary-face state
// Warps take 32-entity chunks in the order chunk = (warp * chunk_mul) mod
// nchunks (chunk_mul coprime to nchunks): loads stay coalesced within a warp
// while the unsaturated cells, which cost ~50x more and cluster in space
// (and therefore in cell numbering), spread over every SM instead of forming
// a tail of a few slow blocks.
// entity i: cell i < nc, else boundary face i - nc
__device__ __forceinline__ void state_entity(const DevArgs &a, int i) {
  if (i < a.nc) {
    const double U = a.U[i];
    const double Pc = a.Pref - U;
    const double P = a.Pref - Pc;
    const int st = a.sat_type[i];
    // Saturated cells (van Genuchten Pc <= 0, Gardner Pc < 0): S = 1, dS = 0,
    // Se = (1 - Sr)/(1 - Sr) = 1 exactly, so kr/mu is the per-cell constant
    // lam_sat and its pressure derivative is zero.
    const bool saturated = (st == SAT_FUNC_VAN_GENUCHTEN) ? (Pc <= 0) : (Pc < 0);
    double S, dS, d2S, lam, dlam;
    if (saturated) {
      S = 1.0;
      dS = 0.0;
      d2S = 0.0;
      lam = a.lam_sat[i];
      dlam = 0.0;
    } else {
      const double Sr = a.Sr[i];
      saturation(st, a.sat_param + 3 * (size_t)i, Sr, Pc, &S, &dS, &d2S);
      double Se = (S - Sr) / (1.0 - Sr);
      double Kr, dKr_dSe;
      relperm(a.rp_type[i], a.rp_param + 9 * (size_t)i, Se, &Kr, &dKr_dSe);
      double dSe_dS = 1.0 / (1.0 - Sr);
      double dKr_dS = dKr_dSe * dSe_dS;
      lam = Kr / a.vis;
      dlam = dKr_dS * dS / a.vis;  // the viscosity does not depend on pressure here
    }
    double rho, drho, d2rho;
    density(a.rho_type, P, &rho, &drho, &d2rho);
    a.P[i] = P;
    a.hr[i] = 0.5 * rho;
    a.hdr[i] = 0.5 * drho;
    a.lam[i] = lam;
    a.dlam[i] = dlam;
    a.seep[i] = 0;
    const double poro = a.poro[i], vol = a.vol[i];
    const double dporo = 0.0;
    double dmass = rho * dporo * S + drho * poro * S + rho * poro * dS;
    if (a.form == FORM_SNES) {
      const double dtInv = a.shift;  // 1/dt, computed on the host
      double acc = rho * poro * S * vol * dtInv;
      a.acc_a[i] = acc - a.accum_prev[i];
      a.acc_b[i] = a.ss[i];
      a.jdiag[i] = dmass * vol * dtInv;
    } else if (a.form == FORM_TV) {
      // TDyMPFAOIFunction_TransientVariable (tdympfao_ts_transientvar.c:89-95):
      // Ut holds dM/dt; the Jacobian adds shift * dM/dP * V.
      a.acc_a[i] = a.Ut[i] * vol;
      a.acc_b[i] = a.ss[i] * vol;
      a.jdiag[i] = a.shift * dmass * vol;
    } else {
      const double Ut = a.Ut[i];
      const double d2poro = 0.0;
      double d2mass = (dS * rho * dporo + S * drho * dporo + S * rho * d2poro + dS * drho * poro + S * d2rho * poro +
                       S * drho * dporo + d2S * rho * poro + dS * drho * poro + dS * rho * dporo);
      a.acc_a[i] = dmass * Ut * vol;
      a.acc_b[i] = a.ss[i] * vol;
      a.jdiag[i] = (a.shift * dmass + d2mass * Ut) * vol;
    }
  } else if (i < a.nc + a.nb) {
    const int b = i - a.nc;
    const int c = a.bnd_cell[b];
    const double p = a.bnd_has[b] ? a.bnd_val[b] : a.U[c];
    const double Pc = a.Pref - p;
    const int st = a.sat_type[c];
    const bool saturated = (st == SAT_FUNC_VAN_GENUCHTEN) ? (Pc <= 0) : (Pc < 0);
    double lam;
    if (saturated) {
      lam = a.lam_sat[c];  // kr(1) / mu with the boundary viscosity (the same constant)
    } else {
      const double Sr = a.Sr[c];
      double S, dS, d2S;
      saturation(st, a.sat_param + 3 * (size_t)c, Sr, Pc, &S, &dS, &d2S);
      double Se = (S - Sr) / (1.0 - Sr);
      double Kr, dKr;
      relperm(a.rp_type[c], a.rp_param + 9 * (size_t)c, Se, &Kr, &dKr);
      lam = Kr / a.bnd_vis[b];
    }
    a.P[i] = p;
    a.hr[i] = 0.5 * a.bnd_rho[b];
    a.hdr[i] = 0.0;
    a.lam[i] = lam;
    a.dlam[i] = 0.0;
    a.seep[i] = (a.bnd_type[b] == SEEPAGE_BC && p <= a.Pref) ? 1 : 0;
  }
}

// entities [e0, e1) (cells below nc, then boundary faces)
__global__ void __launch_bounds__(256) state_kernel(DevArgs a, int e0, int e1, int nchunks, int chunk_mul) {
  const int gw = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (gw >= nchunks) return;
  const int i = e0 + (int)(((long long)gw * chunk_mul) % nchunks) * 32 + (int)(threadIdx.x & 31);
  if (i < e1) state_entity(a, i);
}

// Accumulation at the previous solution (TDyMPFAOSNESPreSolve,
// tdympfao_snes.c:19-64).
__global__ void __launch_bounds__(256) presolve_kernel(DevArgs a, const double *Uprev, double *accum_prev) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.nc) return;
  const double Sr = a.Sr[i];
  const double Pc = a.Pref - Uprev[i];
  double S, dS, d2S;
  saturation(a.sat_type[i], a.sat_param + 3 * (size_t)i, Sr, Pc, &S, &dS, &d2S);
  double rho, drho, d2rho;
  density(a.rho_type, a.Pref - Pc, &rho, &drho, &d2rho);
  accum_prev[i] = rho * a.poro[i] * S * a.vol[i] / a.dt;
}

// Transient variable (TDyMPFAOTransientVariable, tdympfao_ts_transientvar.c:
// 13-47): C = rho phi S V, and its pressure derivative.
__global__ void __launch_bounds__(256) tv_kernel(DevArgs a, const double *U, double *C, double *dC) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.nc) return;
  const double Sr = a.Sr[i];
  const double Pc = a.Pref - U[i];
  double S, dS, d2S;
  saturation(a.sat_type[i], a.sat_param + 3 * (size_t)i, Sr, Pc, &S, &dS, &d2S);
  double rho, drho, d2rho;
  density(a.rho_type, a.Pref - Pc, &rho, &drho, &d2rho);
  const double poro = a.poro[i], vol = a.vol[i];
  if (C) C[i] = rho * poro * S * vol;
  if (dC) dC[i] = (rho * 0.0 * S + drho * poro * S + rho * poro * dS) * vol;
}

// DAE form (TDyMPFAOIFunction_DAE, tdympfao_ts_dae.c:13-84): split the
// interleaved [P, M] unknowns, then combine R_P (the transient-variable
// residual with dM/dt) and R_M = M - rho phi S V.
__global__ void __launch_bounds__(256) dae_split_kernel(int n, const double *U2, const double *Ut2, double *P,
                                                        double *Mdot) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  P[i] = U2[2 * i];
  Mdot[i] = Ut2[2 * i + 1];
}
__global__ void __launch_bounds__(256) dae_merge_kernel(int n, const double *U2, const double *Rp, const double *C,
                                                        double *R2) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  R2[2 * i] = Rp[i];
  R2[2 * i + 1] = U2[2 * i + 1] - C[i];
}

// Diagnostics (TDyUpdateDiagnostics_MPFAO, tdympfao.c:2780-2806): saturation
// and rho*V per cell.
__global__ void __launch_bounds__(256) diag_kernel(DevArgs a, double *Sout, double *mass) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.nc) return;
  const double Sr = a.Sr[i];
  const double Pc = a.Pref - a.U[i];
  double S, dS, d2S;
  saturation(a.sat_type[i], a.sat_param + 3 * (size_t)i, Sr, Pc, &S, &dS, &d2S);
  double rho, drho, d2rho;
  density(a.rho_type, a.Pref - Pc, &rho, &drho, &d2rho);
  Sout[i] = S;
  mass[i] = rho * a.vol[i];
}

// ---------------------------------------------------------------------------
// 2. interior hexahedral vertices, octant layout

// Octants joined by canonical row r (kCanonUp/kCanonDn in tdy_internal.h).
__host__ __device__ constexpr int canon_up(int r) {
  return r < 4 ? 2 * r : r < 8 ? (((r - 4) & 1) | (((r - 4) >> 1) << 2)) : r - 8;
}
__host__ __device__ constexpr int canon_dn(int r) { return canon_up(r) | (1 << (r / 4)); }
static_assert(canon_up(5) == kCanonUp[5] && canon_dn(5) == kCanonDn[5] && canon_up(10) == kCanonUp[10] &&
                  canon_dn(10) == kCanonDn[10] && canon_up(2) == kCanonUp[2] && canon_dn(7) == kCanonDn[7],
              "canonical row tables disagree");

// Corner offsets, octants and slots of structured cells (kCornerOffset,
// struct_octant, struct_slot in tdy_internal.h) without host tables.
__host__ __device__ constexpr int corner_offset(int j) { return j ^ ((j >> 1) & 1); }
__host__ __device__ constexpr int d_struct_octant(int j) { return 7 ^ corner_offset(j); }
__host__ __device__ constexpr int d_struct_slot(int j, int b) {
  return ((((corner_offset(j) >> 2) & 1) - 1 + ((b >> 2) & 1)) + 1) * 9 +
         ((((corner_offset(j) >> 1) & 1) - 1 + ((b >> 1) & 1)) + 1) * 3 + (((corner_offset(j) & 1) - 1 + (b & 1)) + 1);
}
static_assert(corner_offset(2) == kCornerOffset[2] && corner_offset(7) == kCornerOffset[7] &&
                  d_struct_slot(0, 7) == struct_slot(0, 7) && d_struct_slot(6, 0) == struct_slot(6, 0) &&
                  d_struct_slot(3, 5) == struct_slot(3, 5),
              "structured-cell tables disagree");

// Row of the canonical layout that joins octant c with its neighbour across
// axis k, and whether c is that row's first ("up") cell.
__host__ __device__ constexpr int canon_row(int c, int k) {
  return k == 0 ? ((c & ~1) >> 1) : k == 1 ? 4 + (((c & ~2) & 1) | (((c & ~2) >> 2) << 1)) : 8 + (c & ~4);
}
__host__ __device__ constexpr bool canon_is_up(int c, int k) { return ((c >> k) & 1) == 0; }

// x < 0.0 by integer operations (the FP64 pipe is this kernel's bound):
// the sign bit set, and neither a zero nor a NaN
__device__ __forceinline__ bool dneg(double x) {
  const long long b = __double_as_longlong(x), m = b & 0x7fffffffffffffffLL;
  return b < 0 && m != 0 && m <= 0x7ff0000000000000LL;
}

// first canonical row that touches octant o
__host__ __device__ constexpr int canon_first_row(int o) {
  for (int r = 0; r < 12; r++)
    if (canon_up(r) == o || canon_dn(r) == o) return r;
  return -1;
}

// Density modes of the canonical vertex: RHO_CONST (constant density: the
// face average 2 (rho/2) is the constant itself, rho/2 is not gathered),
// RHO_NODERIV (density without a pressure derivative), RHO_EXP (exponential,
// with its derivative).
enum { RHO_CONST = 0, RHO_NODERIV = 1, RHO_EXP = 2 };

// canonical vertex vc; tid: its slot of the block's shared rows
template <int RHO, bool FFJ>
__device__ __forceinline__ void canon_vertex_at(const DevArgs &a, int vc, int tid) {
  constexpr bool CONST_RHO = RHO != RHO_EXP;
  extern __shared__ double sh[];  // [36][blockDim]: w, E_up, E_dn per row
  const int bs = blockDim.x;
  const long long P = a.nCpad;
  double p[8], hr[8], lam[8], dlam[8], hdr[8];
#pragma unroll
  for (int o = 0; o < 8; o++) {
    const int cell = a.cellc[o * P + vc];
    p[o] = a.P[cell];
    hr[o] = RHO == RHO_CONST ? 0.5 * kRhoConst : a.hr[cell];
    lam[o] = a.lam[cell];
    dlam[o] = a.dlam[cell];
    hdr[o] = CONST_RHO ? 0.0 : a.hdr[cell];
  }
  double Rv[8];
#pragma unroll
  for (int r = 0; r < 12; r++) {
    const int u = canon_up(r), d = canon_dn(r);
    const double *T = a.Tc + (long long)(r * 8) * P + vc;
    // explicit roundings: the same bits whichever outputs a call requests
    double TP = __dmul_rn(T[0], p[0]);
#pragma unroll
    for (int c = 1; c < 8; c++) TP = __fma_rn(T[c * P], p[c], TP);
    const double G = a.G[a.facec[r * P + vc]];
    // (constant density: 499 + 499, exactly the constant)
    const double den = RHO == RHO_CONST ? kRhoConst : __dadd_rn(hr[u], hr[d]);
    const double q = __fma_rn(den, G, TP);
    const bool fdn = dneg(q);
    const double lm = fdn ? lam[u] : lam[d];
    const double w = __dmul_rn(den, lm);
    const double flux = -__dmul_rn(w, q);
    // an octant's partial residual starts from its first row's flux
    if (r == canon_first_row(u))
      Rv[u] = flux;
    else
      Rv[u] += flux;
    if (r == canon_first_row(d))
      Rv[d] = -flux;
    else
      Rv[d] -= flux;
    if (a.needJ) {
      // derivative of the flux with respect to the up and down cell pressures
      // beyond w*T: d(rho_avg)/dP and d(kr/mu)/dP of the upwind cell
      double eu, ed;
      if (CONST_RHO) {
        const double e = __dmul_rn(__dmul_rn(den, q), fdn ? dlam[u] : dlam[d]);
        eu = fdn ? e : 0.0;
        ed = fdn ? 0.0 : e;
      } else {
        const double dlu = fdn ? dlam[u] : 0.0, dld = fdn ? 0.0 : dlam[d];
        const double g2 = __fma_rn(den, G, q);
        eu = __fma_rn(__dmul_rn(hdr[u], lm), g2, __dmul_rn(__dmul_rn(den, dlu), q));
        ed = __fma_rn(__dmul_rn(hdr[d], lm), g2, __dmul_rn(__dmul_rn(den, dld), q));
      }
      sh[r * bs + tid] = w;
      sh[(12 + r) * bs + tid] = eu;
      sh[(24 + r) * bs + tid] = ed;
    }
  }
  double *S = a.scratch;
  if (a.needR) {
#pragma unroll
    for (int c = 0; c < 8; c++) S[64 * P + c * P + vc] = Rv[c];
  }
  if (!a.needJ) return;
  // J_v[c][b] = sum over the three rows k of octant c of
  //   -+ w_r T_rb  (minus when c is the row's up cell)  -+ E terms
  if (FFJ) {
    // Octants in a runtime loop (keeps the code small enough for the
    // instruction cache); entries are indexed relative to the octant,
    // j = b ^ c, so the row of axis k touches entries 0 (c itself) and 1 << k
    // at compile-time register indices.
#pragma unroll 1
    for (int c = 0; c < 8; c++) {
      // Each entry is accumulated at its own power-of-two scale, chosen from
      // the exponent fields of its terms so that its largest term is O(1):
      // entries of rows upwinded from nearly dry cells (kr ~ 1e-30 and
      // below) keep full relative accuracy next to O(1) entries.
      double wk[3], es[3], en[3], Tk[3][8];
      int bw[3], mb[8];
#pragma unroll
      for (int j = 0; j < 8; j++) mb[j] = 0;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const int r = canon_row(c, k);
        const bool up = canon_is_up(c, k);
        wk[k] = sh[r * bs + tid];
        bw[k] = d_bexp(wk[k]);
        const double eu = sh[(12 + r) * bs + tid], ed = sh[(24 + r) * bs + tid];
        es[k] = up ? eu : ed;  // E term of c itself
        en[k] = up ? ed : eu;  // E term of the neighbour c ^ (1 << k)
        const double *T = a.Tc + (long long)(r * 8) * P + vc;
#pragma unroll
        for (int j = 0; j < 8; j++) {
          Tk[k][j] = T[(j ^ c) * P];
          // biased exponent of |w T| (a zero factor gives a negligible value)
          mb[j] = max(mb[j], bw[k] + d_bexp(Tk[k][j]) - 1023);
        }
        mb[0] = max(mb[0], d_bexp(es[k]));
        mb[1 << k] = max(mb[1 << k], d_bexp(en[k]));
      }
      ff acc[8];
#pragma unroll
      for (int j = 0; j < 8; j++) acc[j] = ff{0.0f, 0.0f};
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const bool up = canon_is_up(c, k);
        // w normalised to [1, 2); T carries the rest of the entry's scale
        ff wf = ff_split_scaled(wk[k], bw[k], 1023 - bw[k]);
        ff ef = ff_split_scaled(es[k], d_bexp(es[k]), 1023 - mb[0]);
        ff nf = ff_split_scaled(en[k], d_bexp(en[k]), 1023 - mb[1 << k]);
        if (up) {
          wf = ff_neg(wf);
          ef = ff_neg(ef);
          nf = ff_neg(nf);
        }
#pragma unroll
        for (int j = 0; j < 8; j++)
          ff_acc(acc[j], ff_mul(wf, ff_split_scaled(Tk[k][j], d_bexp(Tk[k][j]), bw[k] - mb[j])));
        ff_acc(acc[0], ef);
        ff_acc(acc[1 << k], nf);
      }
      double *dst = S + ((long long)c * P + vc) * 8;
#pragma unroll
      for (int j = 0; j < 8; j++) dst[j ^ c] = ff_to_d(acc[j], mb[j] - 1023);
    }
  } else {
#pragma unroll
    for (int c = 0; c < 8; c++) {
      double out[8];
#pragma unroll
      for (int b = 0; b < 8; b++) out[b] = 0.0;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        const int r = canon_row(c, k);
        const bool up = canon_is_up(c, k);
        const double wr = sh[r * bs + tid];
        const double sw = up ? -wr : wr;
        const double *T = a.Tc + (long long)(r * 8) * P + vc;
#pragma unroll
        for (int b = 0; b < 8; b++) out[b] = __fma_rn(sw, T[b * P], out[b]);
        const double eu = sh[(12 + r) * bs + tid], ed = sh[(24 + r) * bs + tid];
        const int u = canon_up(r), d = canon_dn(r);
        out[u] = __dadd_rn(out[u], up ? -eu : eu);
        out[d] = __dadd_rn(out[d], up ? -ed : ed);
      }
      // J_v[c][0..7] is 64 contiguous bytes at [c][vc][b]
      double2 *dst = reinterpret_cast<double2 *>(S + ((long long)c * P + vc) * 8);
      dst[0] = make_double2(out[0], out[1]);
      dst[1] = make_double2(out[2], out[3]);
      dst[2] = make_double2(out[4], out[5]);
      dst[3] = make_double2(out[6], out[7]);
    }
  }
}

// Canonical vertex vc by a lane pair (h = lane parity; slot: the pair's
// column of the block's ns shared rows), double-float Jacobian products.
// Lane h computes rows 2h+i (x), 4+2h+i (y) and 8+2h+i (z), i = 0, 1: the x
// and y rows of octants 4h..4h+3 and half of their z rows (the other half
// comes from the partner by a shuffle); it writes R_v of octants 4h..4h+3 and
// entries 4h..4h+3 (relative to the octant, column j ^ c) of every octant's
// J_v.  Every value is formed by the operations of canon_vertex_at<RHO, true>
// in the same order, so both give the same bits.  A pair holds half the live
// state of one thread (the upwind cell data sit in shared memory), which
// doubles the warps that hide the FP64 latency.
constexpr int pair_shared_rows(int rho) { return 36 + 16 + (rho == 0 ? 0 : 8) + (rho == 2 ? 8 : 0); }
template <int RHO>
__device__ __forceinline__ void canon_vertex_pair(const DevArgs &a, int vc, int slot, int h, int ns) {
  constexpr bool CONST_RHO = RHO != RHO_EXP;
  // [36][ns]: w, E_up, E_dn per row; [8][ns] kr/mu and d(kr/mu)/dP per
  // octant; rho/2 and d(rho/2)/dP per octant where the density varies
  extern __shared__ double sh[];
  double *s_lam = sh + 36 * ns, *s_dlam = s_lam + 8 * ns, *s_hr = s_dlam + 8 * ns, *s_hdr = s_hr + 8 * ns;
  const unsigned pm = 3u << ((threadIdx.x & 31) & ~1);
  const long long P = a.nCpad;
  double p[8];
#pragma unroll
  for (int o = 0; o < 8; o++) {
    const int cell = a.cellc[o * P + vc];
    p[o] = a.P[cell];
    if ((o >> 2) == h) {
      s_lam[o * ns + slot] = a.lam[cell];
      s_dlam[o * ns + slot] = a.dlam[cell];
      if (RHO != RHO_CONST) s_hr[o * ns + slot] = a.hr[cell];
      if (!CONST_RHO) s_hdr[o * ns + slot] = a.hdr[cell];
    }
  }
  __syncwarp(pm);
  double fx[2], fy[2], fz[2];
#pragma unroll
  for (int t = 0; t < 6; t++) {
    const int axis = t >> 1, i = t & 1;
    const int r = 4 * axis + 2 * h + i;
    // octants of row r (canon_up, canon_dn) for this lane
    const int u = h ? (axis == 0 ? 4 + 2 * i : axis == 1 ? 4 + i : 2 + i) : (axis == 0 ? 2 * i : i);
    const int d = u + (1 << axis);
    const double *T = a.Tc + (long long)(r * 8) * P + vc;
    double TP = __dmul_rn(T[0], p[0]);
#pragma unroll
    for (int c = 1; c < 8; c++) TP = __fma_rn(T[c * P], p[c], TP);
    const double G = a.G[a.facec[r * P + vc]];
    const double den = RHO == RHO_CONST ? kRhoConst : __dadd_rn(s_hr[u * ns + slot], s_hr[d * ns + slot]);
    const double q = __fma_rn(den, G, TP);
    const bool fdn = dneg(q);
    const int uw = fdn ? u : d;  // upwind octant
    const double lm = s_lam[uw * ns + slot];
    const double w = __dmul_rn(den, lm);
    const double flux = -__dmul_rn(w, q);
    (axis == 0 ? fx : axis == 1 ? fy : fz)[i] = flux;
    if (a.needJ) {
      const double dl = s_dlam[uw * ns + slot];
      double eu, ed;
      if (CONST_RHO) {
        const double e = __dmul_rn(__dmul_rn(den, q), dl);
        eu = fdn ? e : 0.0;
        ed = fdn ? 0.0 : e;
      } else {
        const double dlu = fdn ? dl : 0.0, dld = fdn ? 0.0 : dl;
        const double g2 = __fma_rn(den, G, q);
        eu = __fma_rn(__dmul_rn(s_hdr[u * ns + slot], lm), g2, __dmul_rn(__dmul_rn(den, dlu), q));
        ed = __fma_rn(__dmul_rn(s_hdr[d * ns + slot], lm), g2, __dmul_rn(__dmul_rn(den, dld), q));
      }
      sh[r * ns + slot] = w;
      sh[(12 + r) * ns + slot] = eu;
      sh[(24 + r) * ns + slot] = ed;
    }
  }
  // z rows 8 + 2(1 - h) + i from the partner
  double pz[2];
#pragma unroll
  for (int i = 0; i < 2; i++) pz[i] = __shfl_xor_sync(pm, fz[i], 1);
  double *S = a.scratch;
  if (a.needR) {
    // octant o = 4h + ol: x row 2h + (ol >> 1), y row 4 + 2h + (ol & 1),
    // z row 8 + ol; first touch from the x row, then y, then z (row order)
#pragma unroll
    for (int ol = 0; ol < 4; ol++) {
      const double f1 = fx[ol >> 1], f2 = fy[ol & 1];
      const double f3 = ((ol >> 1) == h) ? fz[ol & 1] : pz[ol & 1];
      double Rv = (ol & 1) ? -f1 : f1;
      Rv = (ol & 2) ? Rv - f2 : Rv + f2;
      Rv = h ? Rv - f3 : Rv + f3;
      S[64 * P + (4 * h + ol) * P + vc] = Rv;
    }
  }
  if (!a.needJ) return;
  __syncwarp(pm);
#pragma unroll 1
  for (int c = 0; c < 8; c++) {
    // entries jj = 0..3 of this lane are entries j = 4h + jj of octant c
    double wk[3], es[3], en[3], Tk[3][4];
    int bw[3], mb[4];
#pragma unroll
    for (int jj = 0; jj < 4; jj++) mb[jj] = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int r = canon_row(c, k);
      const bool up = canon_is_up(c, k);
      wk[k] = sh[r * ns + slot];
      bw[k] = d_bexp(wk[k]);
      const double eu = sh[(12 + r) * ns + slot], ed = sh[(24 + r) * ns + slot];
      es[k] = up ? eu : ed;  // E term of c itself (entry 0)
      en[k] = up ? ed : eu;  // E term of the neighbour c ^ (1 << k) (entry 1 << k)
      const double *T = a.Tc + (long long)(r * 8) * P + vc;
#pragma unroll
      for (int jj = 0; jj < 4; jj++) {
        Tk[k][jj] = T[((4 * h + jj) ^ c) * P];
        mb[jj] = max(mb[jj], bw[k] + d_bexp(Tk[k][jj]) - 1023);
      }
      if (k < 2) {
        if (h == 0) {
          mb[0] = max(mb[0], d_bexp(es[k]));
          mb[1 << k] = max(mb[1 << k], d_bexp(en[k]));
        }
      } else {
        mb[0] = max(mb[0], d_bexp(h ? en[2] : es[2]));  // entry 4 gets en[2]
      }
    }
    ff acc[4];
#pragma unroll
    for (int jj = 0; jj < 4; jj++) acc[jj] = ff{0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const bool up = canon_is_up(c, k);
      ff wf = ff_split_scaled(wk[k], bw[k], 1023 - bw[k]);
      const double e0 = h ? en[k] : es[k];
      ff ef = ff_split_scaled(e0, d_bexp(e0), 1023 - mb[0]);
      ff nf = k < 2 ? ff_split_scaled(en[k], d_bexp(en[k]), 1023 - mb[(1 << k) & 3]) : ff{0.0f, 0.0f};
      if (up) {
        wf = ff_neg(wf);
        ef = ff_neg(ef);
        nf = ff_neg(nf);
      }
#pragma unroll
      for (int jj = 0; jj < 4; jj++)
        ff_acc(acc[jj], ff_mul(wf, ff_split_scaled(Tk[k][jj], d_bexp(Tk[k][jj]), bw[k] - mb[jj])));
      if (h == 0 || k == 2) ff_acc(acc[0], ef);
      if (k < 2 && h == 0) ff_acc(acc[(1 << k) & 3], nf);
    }
    double *dst = S + ((long long)c * P + vc) * 8;
#pragma unroll
    for (int jj = 0; jj < 4; jj++) dst[(4 * h + jj) ^ c] = ff_to_d(acc[jj], mb[jj] - 1023);
  }
}

// Entry (c, b) of another vertex's J_v in double-float: the rows r of
// local cell c, in row order, each add -+w_r T_rb and, where b is the row's
// up or down cell, -+E; every product at the entry's own power-of-two scale
// (the largest exponent among its terms), as for the canonical vertices.
// row_of(k), k < kn, lists the rows to scan; rows not touching c are skipped.
template <class RowOf>
__device__ __forceinline__ double gen_entry_ff(int c, int b, int kn, RowOf row_of, const int *lup, const int *ldn,
                                               const double *w, const double *Eu, const double *Ed, const double *T,
                                               int ncol) {
  int mb = 0;
  for (int k = 0; k < kn; k++) {
    const int r = row_of(k), lu = lup[r], ld = ldn[r];
    if (lu != c && ld != c) continue;
    mb = max(mb, d_bexp(w[r]) + d_bexp(T[(size_t)r * ncol + b]) - 1023);
    if (b == lu) mb = max(mb, d_bexp(Eu[r]));
    if (b == ld) mb = max(mb, d_bexp(Ed[r]));
  }
  ff acc = {0.0f, 0.0f};
  for (int k = 0; k < kn; k++) {
    const int r = row_of(k), lu = lup[r], ld = ldn[r];
    if (lu != c && ld != c) continue;
    const bool isup = lu == c;
    const double wr = w[r], t = T[(size_t)r * ncol + b];
    const int bw = d_bexp(wr);
    const ff p = ff_mul(ff_split_scaled(wr, bw, 1023 - bw), ff_split_scaled(t, d_bexp(t), bw - mb));
    ff_acc(acc, isup ? ff_neg(p) : p);
    if (b == lu || b == ld) {
      const double et = b == lu ? Eu[r] : Ed[r];
      const ff ef = ff_split_scaled(et, d_bexp(et), 1023 - mb);
      ff_acc(acc, isup ? ff_neg(ef) : ef);
    }
  }
  return ff_to_d(acc, mb - 1023);
}

// ---------------------------------------------------------------------------
// 3. other vertices.  Both forms below sum every Jacobian entry (c, b) of a
// vertex block over the rows whose faces touch local cell c in row order,
// each row's T term before its upwind-derivative terms, so they give the
// same bits.
//
// (a) one thread per vertex, for meshes that are mostly canonical hexahedra
// (their other vertices are few and small, and share the canonical launch)
// other vertex gen_vertex[g], one thread
__device__ __forceinline__ void generic_vertex_one(const DevArgs &a, int g) {
  const int v = a.gen_vertex[g];
  const int nint = a.v_nint[v];
  const int r0 = a.v_row_off[v], nrow = a.v_row_off[v + 1] - r0;
  const int c0 = a.v_col_off[v], ncol = a.v_col_off[v + 1] - c0;
  const double *T = a.trans + a.v_trans_off[v];
  double *Jv = a.scratch + a.v_jv_off[v];
  double *Rv = Jv + nint * nint;

  double w[TDY_MAX_ROWS], Eu[TDY_MAX_ROWS], Ed[TDY_MAX_ROWS], fl[TDY_MAX_ROWS];
  for (int r = 0; r < nrow; r++) {
    const double *Tr = T + (size_t)r * ncol;
    double TP = 0.0;
    for (int c = 0; c < ncol; c++) TP = __fma_rn(Tr[c], a.P[a.col_ext[c0 + c]], TP);
    const int f = a.row_face[r0 + r];
    const int up = a.f_up[f], dn = a.f_dn[f];
    const double G = a.G[f];
    const double den = __dadd_rn(a.hr[up], a.hr[dn]);
    const double q = __fma_rn(den, G, TP);
    const bool flowdn = q < 0.0;
    const int u = flowdn ? up : dn;
    const double lm = a.lam[u];
    const bool zero = a.seep[u] != 0;
    const double wr = zero ? 0.0 : __dmul_rn(den, lm);
    fl[r] = -__dmul_rn(wr, q);
    if (a.needJ) {
      w[r] = wr;
      if (zero) {
        Eu[r] = 0.0;
        Ed[r] = 0.0;
      } else {
        const double dlu = flowdn ? a.dlam[up] : 0.0, dld = flowdn ? 0.0 : a.dlam[dn];
        const double g2 = q + den * G;
        Eu[r] = a.hdr[up] * lm * g2 + den * dlu * q;
        Ed[r] = a.hdr[dn] * lm * g2 + den * dld * q;
      }
    }
  }
  if (a.needR) {
    for (int c = 0; c < nint; c++) {
      double s = 0.0;
      for (int r = 0; r < nrow; r++) {
        if (a.row_lup[r0 + r] == c) s += fl[r];
        if (a.row_ldn[r0 + r] == c) s -= fl[r];
      }
      Rv[c] = s;
    }
  }
  if (a.needJ && a.jac_ff) {
    for (int c = 0; c < nint; c++)
      for (int b = 0; b < nint; b++)
        Jv[c * nint + b] = gen_entry_ff(c, b, nrow, [](int k) { return k; }, a.row_lup + r0, a.row_ldn + r0, w, Eu, Ed,
                                        T, ncol);
  } else if (a.needJ) {
    for (int c = 0; c < nint; c++) {
      for (int b = 0; b < nint; b++) Jv[c * nint + b] = 0.0;
      for (int r = 0; r < nrow; r++) {
        const int lu = a.row_lup[r0 + r], ld = a.row_ldn[r0 + r];
        if (lu != c && ld != c) continue;
        const double sw = (lu == c) ? -w[r] : w[r];
        const double *Tr = T + (size_t)r * ncol;
        for (int b = 0; b < nint; b++) Jv[c * nint + b] = fma(sw, Tr[b], Jv[c * nint + b]);
        const double s = (lu == c) ? -1.0 : 1.0;
        if (lu >= 0) Jv[c * nint + lu] += s * Eu[r];
        if (ld >= 0) Jv[c * nint + ld] += s * Ed[r];
      }
    }
  }
}

// (b) one warp per vertex, for meshes without canonical vertices.  Lanes
// take the rows for the transmissibility products and upwinding, then the
// entries of the block; the rows of each local cell come from a list built
// in shared memory, so the lanes of an entry pass stay in step.
constexpr int kGenWarps = 4;     // warps (vertices) per 128-thread block
constexpr int kGenCellRows = 8;  // rows per local cell in the list; more take the scan

__device__ __forceinline__ void generic_vertex_warp(const DevArgs &a, int block) {
  extern __shared__ double gsh[];  // [kGenWarps][gen_warp_doubles]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = block * kGenWarps + warp;
  if (g >= a.ngen) return;  // whole warp
  const int v = a.gen_vertex[g];
  const int nint = a.v_nint[v];
  const int r0 = a.v_row_off[v], nrow = a.v_row_off[v + 1] - r0;
  const int c0 = a.v_col_off[v], ncol = a.v_col_off[v + 1] - c0;
  const double *T = a.trans + a.v_trans_off[v];
  double *Jv = a.scratch + a.v_jv_off[v];
  double *Rv = Jv + nint * nint;
  double *w = gsh + (size_t)warp * a.gen_warp_doubles;
  double *Eu = w + TDY_MAX_ROWS, *Ed = Eu + TDY_MAX_ROWS, *fl = Ed + TDY_MAX_ROWS;
  int *lup = reinterpret_cast<int *>(fl + TDY_MAX_ROWS), *ldn = lup + TDY_MAX_ROWS;
  unsigned char *cnt = reinterpret_cast<unsigned char *>(ldn + TDY_MAX_ROWS);  // [TDY_MAX_NINT]
  unsigned char *lst = cnt + TDY_MAX_NINT;                                    // [TDY_MAX_NINT][kGenCellRows]

  for (int r = lane; r < nrow; r += 32) {
    const double *Tr = T + (size_t)r * ncol;
    double TP = 0.0;
    for (int c = 0; c < ncol; c++) TP = __fma_rn(Tr[c], a.P[a.col_ext[c0 + c]], TP);
    const int f = a.row_face[r0 + r];
    const int up = a.f_up[f], dn = a.f_dn[f];
    const double G = a.G[f];
    const double den = __dadd_rn(a.hr[up], a.hr[dn]);
    const double q = __fma_rn(den, G, TP);
    const bool flowdn = q < 0.0;
    const int u = flowdn ? up : dn;
    const double lm = a.lam[u];
    const bool zero = a.seep[u] != 0;
    const double wr = zero ? 0.0 : __dmul_rn(den, lm);
    fl[r] = -__dmul_rn(wr, q);
    w[r] = wr;
    if (zero) {
      Eu[r] = 0.0;
      Ed[r] = 0.0;
    } else {
      const double dlu = flowdn ? a.dlam[up] : 0.0, dld = flowdn ? 0.0 : a.dlam[dn];
      const double g2 = q + den * G;
      Eu[r] = a.hdr[up] * lm * g2 + den * dlu * q;
      Ed[r] = a.hdr[dn] * lm * g2 + den * dld * q;
    }
    lup[r] = a.row_lup[r0 + r];
    ldn[r] = a.row_ldn[r0 + r];
  }
  __syncwarp();
  // rows of each local cell, in row order (count 255: more than the list holds)
  for (int c = lane; c < nint; c += 32) {
    int k = 0;
    for (int r = 0; r < nrow; r++)
      if (lup[r] == c || ldn[r] == c) {
        if (k < kGenCellRows) lst[c * kGenCellRows + k] = (unsigned char)r;
        k++;
      }
    cnt[c] = (unsigned char)(k <= kGenCellRows ? k : 255);
  }
  __syncwarp();
  // The FP64 pipe is the bound here (a warp-wide FP64 instruction costs as
  // many issue slots as it has lanes, active or not): walk only each cell's
  // own rows, and pick signs and upwind terms by integer selects.
  if (a.needR) {
    for (int c = lane; c < nint; c += 32) {
      const int kc = cnt[c];
      const int kn = kc == 255 ? nrow : kc;
      double s = 0.0;
      for (int k = 0; k < kn; k++) {
        const int r = kc == 255 ? k : lst[c * kGenCellRows + k];
        if (lup[r] == c) s += fl[r];
        if (ldn[r] == c) s -= fl[r];
      }
      Rv[c] = s;
    }
  }
  if (!a.needJ) return;
  const int nn = nint * nint;
  if (a.jac_ff) {
    for (int e = lane; e < nn; e += 32) {
      const int c = e / nint, b = e - c * nint;
      const int kc = cnt[c];
      const unsigned char *lc = lst + c * kGenCellRows;
      Jv[e] = gen_entry_ff(c, b, kc == 255 ? nrow : kc, [&](int k) { return kc == 255 ? k : (int)lc[k]; }, lup, ldn,
                           w, Eu, Ed, T, ncol);
    }
    return;
  }
  for (int e = lane; e < nn; e += 32) {
    const int c = e / nint, b = e - c * nint;
    const int kc = cnt[c];
    const int kn = kc == 255 ? nrow : kc;
    double J = 0.0;
    for (int k = 0; k < kn; k++) {
      const int r = kc == 255 ? k : lst[c * kGenCellRows + k];
      const int lu = lup[r], ld = ldn[r];
      if (lu != c && ld != c) continue;  // only in the scan
      const bool isup = lu == c;
      const double wr = w[r], eu = Eu[r], ed = Ed[r];
      J = fma(isup ? -wr : wr, T[(size_t)r * ncol + b], J);
      // at most one of b == lu, b == ld holds
      const double et = (b == lu) ? eu : ((b == ld) ? ed : 0.0);
      J += isup ? -et : et;
    }
    Jv[e] = J;
  }
}

// Canonical vertices (one thread each, register-heavy) share their launch
// with the thread form of the other vertices, which take the first blocks so
// they overlap the canonical ones; meshes without canonical vertices launch
// the warp form on its own (a light kernel with high occupancy for its
// latency-bound gathers).
template <int RHO, bool FFJ>
__global__ void __launch_bounds__(128) vertex_kernel(DevArgs a, int gen_blocks) {
  if ((int)blockIdx.x >= gen_blocks) {
    const int vc = a.vc0 + ((int)blockIdx.x - gen_blocks) * blockDim.x + threadIdx.x;
    if (vc < a.vc1) canon_vertex_at<RHO, FFJ>(a, vc, threadIdx.x);
  } else {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < a.ngen) generic_vertex_one(a, g);
  }
}

// The same with a lane pair per canonical vertex (double-float Jacobian
// products): a block of kPairThreads threads takes kPairThreads / 2 vertices.
constexpr int kPairThreads = 128;
template <int RHO>
__global__ void __launch_bounds__(kPairThreads, 7) vertex_pair_kernel(DevArgs a, int gen_blocks) {
  if ((int)blockIdx.x >= gen_blocks) {
    const int slot = threadIdx.x >> 1, h = threadIdx.x & 1;
    const int vc = a.vc0 + ((int)blockIdx.x - gen_blocks) * (kPairThreads / 2) + slot;
    if (vc < a.vc1) canon_vertex_pair<RHO>(a, vc, slot, h, kPairThreads / 2);
  } else {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < a.ngen) generic_vertex_one(a, g);
  }
}

__global__ void __launch_bounds__(128) generic_vertex_kernel(DevArgs a) { generic_vertex_warp(a, blockIdx.x); }

// ---------------------------------------------------------------------------
// 4. per-cell deterministic gather into R and the CSR row.
//
// Structured interior cells (all vertices canonical, 27-point row) read their
// eight vertices' partials at compile-time slots.  Other cells follow their
// gather program; each warp stages its rows in shared memory and writes them
// with coalesced stores.  Both sum the vertices in the cell's corner order, so
// a cell gets the same bits on either path.

// structured cell sc_cells[sidx]; the 32 lanes of a warp call it together
// with consecutive sidx (those at or past s_end do nothing)
__device__ __forceinline__ void struct_cell_at(const DevArgs &a, int sidx, int s_end) {
  extern __shared__ double rowbuf[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (sidx - lane >= s_end) return;  // whole warp out of range
  const bool active = sidx < s_end;
  const int i = active ? a.sc_cells[sidx] : 0;
  const long long P = a.nCpad, Q = a.nSpad;
  const double *S = a.scratch;
  double row[27];
  if (active) {
    int vc[8];
#pragma unroll
    for (int j = 0; j < 8; j++) vc[j] = a.sc_vc[j * Q + sidx];
    if (a.needR) {
      double s = 0.0;
#pragma unroll
      for (int j = 0; j < 8; j++) s += S[64 * P + d_struct_octant(j) * P + vc[j]];
      s += a.acc_a[i];
      s -= a.acc_b[i];
      a.R[i] = s;
    }
    if (a.needJ) {
#pragma unroll
      for (int k = 0; k < 27; k++) row[k] = 0.0;
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const double2 *blk = reinterpret_cast<const double2 *>(S + ((long long)d_struct_octant(j) * P + vc[j]) * 8);
        const double2 v0 = blk[0], v1 = blk[1], v2 = blk[2], v3 = blk[3];
        row[d_struct_slot(j, 0)] += v0.x;
        row[d_struct_slot(j, 1)] += v0.y;
        row[d_struct_slot(j, 2)] += v1.x;
        row[d_struct_slot(j, 3)] += v1.y;
        row[d_struct_slot(j, 4)] += v2.x;
        row[d_struct_slot(j, 5)] += v2.y;
        row[d_struct_slot(j, 6)] += v3.x;
        row[d_struct_slot(j, 7)] += v3.y;
      }
      row[13] += a.jdiag[i];
    }
  }
  if (!a.needJ) return;
  // rows of the warp contiguous in the CSR value array: stage and store
  // coalesced; otherwise every thread stores its own row
  const int rp = active ? a.rowptr[i] : 0;
  const int rp0 = __shfl_sync(0xffffffffu, rp, 0);
  const bool contig = __all_sync(0xffffffffu, active && rp == rp0 + 27 * lane);
  if (contig) {
    double *buf = rowbuf + (size_t)warp * 32 * 27;
#pragma unroll
    for (int k = 0; k < 27; k++) buf[lane * 27 + k] = row[k];
    __syncwarp();
    double *out = a.J + rp0;
    for (int j = lane; j < 32 * 27; j += 32) out[j] = buf[j];
  } else if (active) {
    double *out = a.J + rp;
#pragma unroll
    for (int k = 0; k < 27; k++) out[k] = row[k];
  }
}

// Other cells, thread form (meshes with structured cells).
// other cell gc_cells[gidx], one thread
__device__ __forceinline__ void generic_cell_at(const DevArgs &a, int gidx, int g_end) {
  extern __shared__ double rowbuf[];  // [warps][32 * max_row_nnz]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g0 = gidx - lane;
  if (g0 >= g_end) return;  // whole warp out of range
  const bool active = gidx < g_end;
  const int i = active ? a.gc_cells[gidx] : -1;
  if (a.needR && active) {
    const int k0 = a.cv_off[i], k1 = a.cv_off[i + 1];
    double s = 0.0;
    for (int k = k0; k < k1; k++) s += a.scratch[a.cv_rbase[k]];
    s += a.acc_a[i];
    s -= a.acc_b[i];
    a.R[i] = s;
  }
  if (!a.needJ) return;
  double *row = rowbuf + ((size_t)warp * 32 + lane) * a.max_row_nnz;
  int p0 = 0, rn = 0;
  if (active) {
    p0 = a.rowptr[i];
    rn = a.rowptr[i + 1] - p0;
    for (int j = 0; j < rn; j++) row[j] = 0.0;
    const int k0 = a.cv_off[i], k1 = a.cv_off[i + 1];
    int diag = -1;
    for (int k = k0; k < k1; k++) {
      const int nint = a.cv_nint[k], stride = a.cv_stride[k];
      const long long jb = a.cv_jbase[k];
      const unsigned char *sl = a.cv_slots + a.cv_slot_off[k];
      for (int b = 0; b < nint; b++) row[sl[b]] += a.scratch[jb + (long long)b * stride];
      diag = sl[a.cv_local[k]];
    }
    if (diag >= 0) row[diag] += a.jdiag[i];
    double *out = a.J + p0;
    for (int j = 0; j < rn; j++) out[j] = row[j];
  }
}

// Other cells, warp form (meshes without structured cells): one half-warp
// per cell (vertex blocks of such meshes have about 12 columns, so 16 lanes
// keep the FP64 adds, this kernel's bound, mostly full).  The row is staged
// in shared memory; the lanes take the columns of each vertex block (distinct
// columns land in distinct slots) and the vertices are added in the cell's
// corner order, as in the thread form.
constexpr int kCellWarps = 4;  // warps per generic-cell block (two cells each)

__device__ __forceinline__ void generic_cell_warp(const DevArgs &a, int block) {
  extern __shared__ double rowbuf[];  // [2 * kCellWarps][max_row_nnz]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int half = lane >> 4, hl = lane & 15;
  const int pair = block * kCellWarps + warp;
  if (2 * pair >= a.ngc) return;  // whole warp
  const int gidx = 2 * pair + half;
  if (gidx >= a.ngc) return;  // the second half of the last warp
  const unsigned mask = 0xffffu << (16 * half);
  const int i = a.gc_cells[gidx];
  const int k0 = a.cv_off[i], k1 = a.cv_off[i + 1];
  if (a.needR && hl == 0) {
    double s = 0.0;
    for (int k = k0; k < k1; k++) s += a.scratch[a.cv_rbase[k]];
    s += a.acc_a[i];
    s -= a.acc_b[i];
    a.R[i] = s;
  }
  if (!a.needJ) return;
  double *row = rowbuf + (size_t)(2 * warp + half) * a.max_row_nnz;
  const int p0 = a.rowptr[i], rn = a.rowptr[i + 1] - p0;
  for (int j = hl; j < rn; j += 16) row[j] = 0.0;
  __syncwarp(mask);
  int diag = -1;
  for (int k = k0; k < k1; k++) {
    const int nint = a.cv_nint[k], stride = a.cv_stride[k];
    const long long jb = a.cv_jbase[k];
    const unsigned char *sl = a.cv_slots + a.cv_slot_off[k];
    for (int b = hl; b < nint; b += 16) row[sl[b]] += a.scratch[jb + (long long)b * stride];
    diag = sl[a.cv_local[k]];
    __syncwarp(mask);
  }
  if (hl == 0 && diag >= 0) row[diag] += a.jdiag[i];
  __syncwarp(mask);
  double *out = a.J + p0;
  for (int j = hl; j < rn; j += 16) out[j] = row[j];
}

__global__ void __launch_bounds__(64) cell_kernel(DevArgs a, int struct_blocks) {
  if ((int)blockIdx.x < struct_blocks)
    struct_cell_at(a, blockIdx.x * blockDim.x + threadIdx.x, a.nS);
  else
    generic_cell_at(a, ((int)blockIdx.x - struct_blocks) * blockDim.x + threadIdx.x, a.ngc);
}

__global__ void __launch_bounds__(32 * kCellWarps) generic_cell_kernel(DevArgs a) { generic_cell_warp(a, blockIdx.x); }

// ---------------------------------------------------------------------------
// 5. instance schedule: one launch evaluates a list of instances (the blocks
// of a batched handle), one CTA per instance at a time, taken from a ticket
// counter; the CTA runs the instance's state, vertex and cell stages with
// block barriers between them.  Every entity goes through the same device
// function as in the three-stage launches (vertices and other cells in their
// thread forms, which give the warp forms' bits), so an instance gets the same
// bits from either schedule.  The instances not in the list keep their
// previous R and J.  256 threads with at most 128 registers each (a little
// spilling in the heaviest stage): measured on 4096 config-4 instances,
// 11.8 ms for all of them and 2.2 ms for 64, against 14.5 and 3.0 ms with 128
// threads at 251 registers, and 17.5 ms for the three-stage launches.
constexpr int kInstThreads = 256;

template <int RHO, bool FFJ>
__global__ void __launch_bounds__(kInstThreads, 2) instance_eval_kernel(DevArgs a, const InstRange *rng, const int *list,
                                                                     int nlist, int *ticket) {
  __shared__ int cur;
  const int tid = threadIdx.x, bs = blockDim.x;
  for (;;) {
    if (tid == 0) cur = atomicAdd(ticket, 1);
    __syncthreads();
    const int k = cur;
    __syncthreads();  // every thread has read the ticket before the next one is drawn
    if (k >= nlist) return;
    const InstRange R = rng[list[k]];
    for (int i = R.c0 + tid; i < R.c1; i += bs) state_entity(a, i);
    for (int b = R.b0 + tid; b < R.b1; b += bs) state_entity(a, a.nc + b);
    __syncthreads();
    for (int vc = R.vc0 + tid; vc < R.vc1; vc += bs) canon_vertex_at<RHO, FFJ>(a, vc, tid);
    for (int g = R.g0 + tid; g < R.g1; g += bs) generic_vertex_one(a, g);
    __syncthreads();
    for (int base = R.s0; base < R.s1; base += bs) struct_cell_at(a, base + tid, R.s1);
    for (int base = R.gc0; base < R.gc1; base += bs) generic_cell_at(a, base + tid, R.gc1);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Host side

// Stream-ordered device memory; the pool keeps up to kPoolKeep bytes of
// freed memory for reuse instead of returning it to the driver at every
// synchronisation (a server sets up and destroys handles continuously).
static constexpr unsigned long long kPoolKeep = 8ull << 30;
static constexpr int kMaxDevices = 64;
static std::mutex g_dev_mutex;  // per-device one-time set-up below
static bool g_pool_set[kMaxDevices] = {};

int dmem_alloc(void **p, size_t bytes, void *stream) {
  *p = nullptr;
  int dev = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  if (dev >= 0 && dev < kMaxDevices) {
    std::lock_guard<std::mutex> lk(g_dev_mutex);
    if (!g_pool_set[dev]) {
      cudaMemPool_t pool;
      CUDA_TRY(cudaDeviceGetDefaultMemPool(&pool, dev));
      unsigned long long keep = kPoolKeep;
      CUDA_TRY(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
      g_pool_set[dev] = true;
    }
  }
  cudaError_t e = cudaMallocAsync(p, bytes ? bytes : 1, (cudaStream_t)stream);
  if (e != cudaSuccess) {
    *p = nullptr;
    return set_error(TDY_ERR_GPU, "cudaMallocAsync(%zu bytes): %s", bytes, cudaGetErrorString(e));
  }
  return 0;
}

void dmem_free(void *p, void *stream) {
  if (p) cudaFreeAsync(p, (cudaStream_t)stream);
}

template <class T>
static int dalloc(DeviceState *d, T **p, size_t n) {
  int ierr = dmem_alloc((void **)p, (n ? n : 1) * sizeof(T), d->stream);
  if (ierr) return ierr;
  d->allocs.push_back(*p);
  return 0;
}

static int pool_event(cudaEvent_t *ev);

// Records that a caller's stream enqueued work on this handle.
static int note_stream(DeviceState *d, cudaStream_t st) {
  if (st == d->stream) return 0;
  for (auto &u : d->user_streams)
    if (u.first == st) {
      CUDA_TRY(cudaEventRecord(u.second, st));
      return 0;
    }
  cudaEvent_t e;
  int ierr = pool_event(&e);
  if (ierr) return ierr;
  d->user_streams.emplace_back(st, e);
  CUDA_TRY(cudaEventRecord(e, st));
  return 0;
}

// Slabs of the host-pointer evaluation, for a single extruded block (cells
// numbered layer by layer): cells split at layer boundaries, the first slab
// 1/kSlabFirst of the layers, each next one kSlabGrowth times the previous
// up to 1/kSlabCap (a remainder below half a slab joins the last one).  The
// copies of R and J to host memory run about 1.2x slower than the
// evaluation, so once the first slab is evaluated the copy engine stays
// busy; slabs much thinner than this cost more than they save, since every
// launch lasts at least the latency of one block (about 30 us for the vertex
// stage).  A vertex belongs to the slab of the first cell that uses it, so
// the cells of slab k need only vertices of slabs <= k.  The vertex and cell
// lists (ascending indices) must then run through the slabs in order, which
// is checked: any other numbering leaves one slab (no pipelining).  Slab k
// also computes the state of the cells its vertices read beyond its own (the
// layer above), up to e1.
constexpr double kSlabFirst = 16, kSlabGrowth = 1.25, kSlabCap = 8;
static void build_slabs(_p_TDy *t, DeviceState *d) {
  d->slabs.clear();
  if (t->mesh_blocks.size() != 1) return;
  const ExtrudedInput &blk = t->mesh_blocks[0];
  const Mesh &m = t->mesh;
  const MPFAOSetup &s = t->setup;
  const int nl = blk.nlayers, nc2 = blk.nc2;
  if (nl < 8 || m.nc != nl * nc2) return;
  const double cap = nl / kSlabCap;
  std::vector<int> cut = {0};
  int step = 1;
  for (double size = nl / kSlabFirst, layer = 0; layer < nl; size = std::min(cap, size * kSlabGrowth)) {
    step = std::max(1, (int)std::lround(size));
    layer = std::min<double>(nl, layer + step);
    cut.push_back((int)layer * nc2);
  }
  if (cut.size() > 2 && 2 * (cut[cut.size() - 1] - cut[cut.size() - 2]) < step * nc2) cut.erase(cut.end() - 2);
  const int K = (int)cut.size() - 1;
  if (K < 2) return;
  auto slab_of_cell = [&](int c) { return (int)(std::upper_bound(cut.begin(), cut.end(), c) - cut.begin()) - 1; };
  auto slab_of_vertex = [&](int v) { return slab_of_cell(m.vert_cells[m.vert_cell_off[v]]); };
  // b[k] = first list index in slab k or later; false if the slab decreases
  auto bounds = [&](const std::vector<int> &list, auto slab_of, std::vector<int> &b) {
    b.assign(K + 1, (int)list.size());
    b[0] = 0;
    int cur = 0;
    for (int i = 0; i < (int)list.size(); i++) {
      const int sk = slab_of(list[i]);
      if (sk < cur) return false;
      while (cur < sk) b[++cur] = i;
    }
    return true;
  };
  std::vector<int> bc, bg, bs, bgc;
  if (!bounds(s.canon_vertex, slab_of_vertex, bc) || !bounds(s.gen_vertex, slab_of_vertex, bg) ||
      !bounds(s.sc_cells, slab_of_cell, bs) || !bounds(s.gc_cells, slab_of_cell, bgc))
    return;
  int e_prev = 0;
  for (int k = 0; k < K; k++) {
    DeviceState::Slab sl;
    int need = cut[k + 1];
    auto reach = [&](const std::vector<int> &list, int b0, int b1) {
      for (int i = b0; i < b1; i++) {
        const int v = list[i];
        for (int q = m.vert_cell_off[v]; q < m.vert_cell_off[v + 1]; q++) need = std::max(need, m.vert_cells[q] + 1);
      }
    };
    reach(s.canon_vertex, bc[k], bc[k + 1]);
    reach(s.gen_vertex, bg[k], bg[k + 1]);
    sl.e0 = e_prev;
    sl.e1 = k == K - 1 ? m.nc : std::max(std::min(need, m.nc), e_prev);
    e_prev = sl.e1;
    sl.c0 = cut[k];
    sl.c1 = cut[k + 1];
    sl.vc0 = bc[k];
    sl.vc1 = bc[k + 1];
    sl.g0 = bg[k];
    sl.g1 = bg[k + 1];
    sl.s0 = bs[k];
    sl.s1 = bs[k + 1];
    sl.gc0 = bgc[k];
    sl.gc1 = bgc[k + 1];
    sl.j0 = s.rowptr[cut[k]];
    sl.j1 = s.rowptr[cut[k + 1]];
    d->slabs.push_back(sl);
  }
}

// Entity ranges of each block of the handle for the instance schedule; false
// when some list does not run through the blocks in order (then the handle
// evaluates with the three-stage launches only).
static bool build_inst_ranges(const _p_TDy *t, std::vector<InstRange> &out, std::vector<long long> &cells) {
  const Mesh &m = t->mesh;
  const MPFAOSetup &s = t->setup;
  const int nblk = (int)t->mesh_blocks.size();
  std::vector<int> cb(nblk + 1, 0), vb(nblk + 1, 0);
  for (int b = 0; b < nblk; b++) {
    const ExtrudedInput &e = t->mesh_blocks[b];
    cb[b + 1] = cb[b] + e.nc2 * e.nlayers;
    vb[b + 1] = vb[b] + e.nv2 * (e.nlayers + 1);
  }
  if (cb[nblk] != m.nc || vb[nblk] != m.nv) return false;
  auto block_of = [](const std::vector<int> &bounds, int x) {
    return (int)(std::upper_bound(bounds.begin(), bounds.end(), x) - bounds.begin()) - 1;
  };
  // [first, last) position in `list` of the items of each block; false if unordered
  auto ranges = [&](const std::vector<int> &list, const std::vector<int> &bounds, std::vector<int> &lo,
                    std::vector<int> &hi, auto key) {
    lo.assign(nblk, 0);
    hi.assign(nblk, 0);
    int prev = 0;
    std::vector<int> first(nblk, -1), last(nblk, -1);
    for (int i = 0; i < (int)list.size(); i++) {
      const int b = block_of(bounds, key(list[i]));
      if (b < prev) return false;
      prev = b;
      if (first[b] < 0) first[b] = i;
      last[b] = i + 1;
    }
    int pos = 0;
    for (int b = 0; b < nblk; b++) {
      lo[b] = first[b] < 0 ? pos : first[b];
      hi[b] = first[b] < 0 ? pos : last[b];
      pos = hi[b];
    }
    return true;
  };
  auto ident = [](int x) { return x; };
  std::vector<int> bcell(m.nb);
  for (int b = 0; b < m.nb; b++) bcell[b] = m.face_cell1[m.bnd_face[b]];
  std::vector<int> bidx(m.nb);
  for (int b = 0; b < m.nb; b++) bidx[b] = b;
  std::vector<int> blo, bhi, clo, chi, glo, ghi, slo, shi, gclo, gchi;
  if (!ranges(bidx, cb, blo, bhi, [&](int b) { return bcell[b]; })) return false;
  if (!ranges(s.canon_vertex, vb, clo, chi, ident)) return false;
  if (!ranges(s.gen_vertex, vb, glo, ghi, ident)) return false;
  if (!ranges(s.sc_cells, cb, slo, shi, ident)) return false;
  if (!ranges(s.gc_cells, cb, gclo, gchi, ident)) return false;
  out.resize(nblk);
  cells.resize(nblk);
  for (int b = 0; b < nblk; b++) {
    out[b] = InstRange{cb[b], cb[b + 1], blo[b], bhi[b], clo[b], chi[b], glo[b], ghi[b], slo[b], shi[b], gclo[b], gchi[b]};
    cells[b] = cb[b + 1] - cb[b];
  }
  return true;
}

static int noalloc_resolve(int dev);
static size_t cell_smem_bytes(const DevArgs &a, bool gen_warp);
static bool cell_warp_form(const DevArgs &a);

// Dynamic shared memory above 48 KB is an opt-in per kernel and device; it
// is made at set-up with the device current (and only ever raised).
static size_t g_cell_smem_granted[kMaxDevices] = {};
static int cell_smem_optin(int dev, size_t bytes) {
  if (bytes <= 48 * 1024) return 0;
  if (dev < 0 || dev >= kMaxDevices) return set_error(TDY_ERR_SUP, "device ordinal %d not supported", dev);
  std::lock_guard<std::mutex> lk(g_dev_mutex);
  if (bytes > g_cell_smem_granted[dev]) {
    CUDA_TRY(cudaFuncSetAttribute(cell_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    g_cell_smem_granted[dev] = bytes;
  }
  return 0;
}

// Streams and events of handles come from per-device pools and go back to
// them when the handle is destroyed (after their work has completed):
// creating and destroying them waits on the driver, and a server sets up and
// destroys handles on many threads at once.
static std::vector<cudaStream_t> g_stream_pool[kMaxDevices];
static std::vector<cudaEvent_t> g_event_pool[kMaxDevices];

static int pool_device(int *dev) {
  CUDA_TRY(cudaGetDevice(dev));
  if (*dev < 0 || *dev >= kMaxDevices) return set_error(TDY_ERR_SUP, "device ordinal %d not supported", *dev);
  return 0;
}
static int pool_stream(cudaStream_t *st) {
  int dev, ierr;
  if ((ierr = pool_device(&dev))) return ierr;
  {
    std::lock_guard<std::mutex> lk(g_dev_mutex);
    if (!g_stream_pool[dev].empty()) {
      *st = g_stream_pool[dev].back();
      g_stream_pool[dev].pop_back();
      return 0;
    }
  }
  CUDA_TRY(cudaStreamCreateWithFlags(st, cudaStreamNonBlocking));
  return 0;
}
static int pool_event(cudaEvent_t *ev) {
  int dev, ierr;
  if ((ierr = pool_device(&dev))) return ierr;
  {
    std::lock_guard<std::mutex> lk(g_dev_mutex);
    if (!g_event_pool[dev].empty()) {
      *ev = g_event_pool[dev].back();
      g_event_pool[dev].pop_back();
      return 0;
    }
  }
  CUDA_TRY(cudaEventCreateWithFlags(ev, cudaEventDisableTiming));
  return 0;
}
// (dev: the device the stream or event was made on; its work has completed)
static void pool_release(int dev, cudaStream_t st, cudaEvent_t ev) {
  if (dev < 0 || dev >= kMaxDevices) return;
  std::lock_guard<std::mutex> lk(g_dev_mutex);
  if (st) g_stream_pool[dev].push_back(st);
  if (ev) g_event_pool[dev].push_back(ev);
}

int device_setup(_p_TDy *t) {
  const Mesh &m = t->mesh;
  const MPFAOSetup &s = t->setup;
  if (s.max_nrow > TDY_MAX_ROWS || s.max_nint > TDY_MAX_NINT || s.max_row_nnz > TDY_MAX_ROW_NNZ)
    return set_error(TDY_ERR_SUP,
                     "mesh exceeds kernel limits (rows/vertex %d, cells/vertex %d, row nnz %d; max %d, %d, %d)",
                     s.max_nrow, s.max_nint, s.max_row_nnz, TDY_MAX_ROWS, TDY_MAX_NINT, TDY_MAX_ROW_NNZ);
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0)
    return set_error(TDY_ERR_GPU, "no CUDA device available: %s", e != cudaSuccess ? cudaGetErrorString(e) : "0 devices");
  DeviceState *d = new DeviceState();
  t->dev = d;
  CUDA_TRY(cudaGetDevice(&d->device));
  int ierr = 0;
  if ((ierr = pool_stream(&d->stream))) return ierr;
  DevArgs &a = d->a;
  memset(&a, 0, sizeof(a));
  a.nc = m.nc;
  a.nb = m.nb;
  a.nv = m.nv;
  a.Pref = t->opt.Pref;
  a.rho_type = t->opt.rho_type;
  a.mu_type = t->opt.mu_type;
  const int next = m.nc + m.nb;
  // every array of the handle in one allocation, uploaded with one copy
  Arena ar;
  ar.up(&a.vol, m.cell_vol);
  ar.up(&a.poro, t->mat.porosity);
  ar.up(&a.Sr, t->mat.Sr);
  ar.up(&a.sat_param, t->mat.sat_param);
  ar.up(&a.rp_param, t->mat.relperm_param);
  ar.up(&a.ss, t->mat.source_sink);
  ar.up(&a.sat_type, t->mat.sat_type);
  ar.up(&a.rp_type, t->mat.relperm_type);
  ar.up(&a.lam_sat, t->mat.lam_sat);
  a.vis = t->mat.vis;
  std::vector<int> bnd_cell(m.nb);
  for (int b = 0; b < m.nb; b++) bnd_cell[b] = m.face_cell1[m.bnd_face[b]];
  ar.up(&a.bnd_cell, bnd_cell);
  ar.up(&a.bnd_type, t->bnd.type);
  ar.up(&a.bnd_has, t->bnd.has_value);
  ar.up(&a.bnd_val, t->bnd.value);
  ar.up(&a.bnd_rho, t->bnd.rho);
  ar.up(&a.bnd_vis, t->bnd.vis);
  std::vector<int> fup(m.nf), fdn(m.nf);
  for (int f = 0; f < m.nf; f++) {
    int u = m.face_cell0[f], w = m.face_cell1[f];
    fup[f] = u >= 0 ? u : m.nc + (-u - 1);
    fdn[f] = w >= 0 ? w : m.nc + (-w - 1);
  }
  ar.up(&a.f_up, fup);
  ar.up(&a.f_dn, fdn);
  ar.up(&a.G, s.gravdis);
  a.nC = s.nC;
  a.vc0 = 0;
  a.vc1 = s.nC;
  a.nCpad = s.nCpad;
  if (t->opt.setup_on_device)
    ar.work(&a.Tc, 96 * (size_t)s.nCpad);
  else
    ar.up(&a.Tc, s.Tc);
  a.jac_ff = t->opt.jacobian_arithmetic == JACOBIAN_DOUBLE_FLOAT;
  ar.up(&a.cellc, s.cellc);
  ar.up(&a.facec, s.facec);
  a.ngen = (int)s.gen_vertex.size();
  // per row: w, E_up, E_dn, flux (doubles) and the two local-cell indices
  // (ints); per local cell: a row count and a list of kGenCellRows rows (bytes)
  a.gen_warp_doubles = 5 * TDY_MAX_ROWS + (TDY_MAX_NINT * (1 + kGenCellRows) + 7) / 8;
  ar.up(&a.gen_vertex, s.gen_vertex);
  ar.up(&a.v_row_off, s.v_row_off);
  ar.up(&a.v_col_off, s.v_col_off);
  ar.up(&a.v_nint, s.v_nint);
  ar.up(&a.v_trans_off, s.v_trans_off);
  ar.up(&a.v_jv_off, s.v_jv_off);
  ar.up(&a.row_face, s.row_face);
  ar.up(&a.row_lup, s.row_lup);
  ar.up(&a.row_ldn, s.row_ldn);
  ar.up(&a.col_ext, s.col_ext);
  ar.up(&a.trans, s.trans);
  ar.up(&a.rowptr, s.rowptr);
  ar.up(&a.cv_off, s.cv_off);
  ar.up(&a.cv_jbase, s.cv_jbase);
  ar.up(&a.cv_rbase, s.cv_rbase);
  ar.up(&a.cv_stride, s.cv_stride);
  ar.up(&a.cv_nint, s.cv_nint);
  ar.up(&a.cv_local, s.cv_local);
  ar.up(&a.cv_slot_off, s.cv_slot_off);
  ar.up(&a.cv_slots, s.cv_slots);
  a.max_row_nnz = s.max_row_nnz;
  a.nS = s.nS;
  a.nSpad = s.nSpad;
  a.ngc = (int)s.gc_cells.size();
  ar.up(&a.sc_cells, s.sc_cells);
  ar.up(&a.sc_vc, s.sc_vc);
  ar.up(&a.gc_cells, s.gc_cells);
  ar.work(&a.P, next);
  ar.work(&a.hr, next);
  ar.work(&a.hdr, next);
  ar.work(&a.lam, next);
  ar.work(&a.dlam, next);
  ar.work(&a.seep, next);
  ar.work(&a.acc_a, m.nc);
  ar.work(&a.acc_b, m.nc);
  ar.work(&a.jdiag, m.nc);
  double *accum_prev = nullptr;
  ar.work(&accum_prev, m.nc);
  ar.work(&a.scratch, (size_t)s.scratch_size);
  d->nnz = (int)s.colidx.size();
  ar.work(&d->dU, m.nc);
  ar.work(&d->dUt, m.nc);
  ar.work(&d->dR, m.nc);
  ar.work(&d->dJ, d->nnz);
  ar.work(&d->diagS, m.nc);
  ar.work(&d->diagMass, m.nc);
  // instance schedule: contiguous blocks and rows short enough for one CTA's
  // shared rows (canonical vertices' 36 per thread, the cell rows)
  d->inst_smem = (size_t)std::max(36, std::max(27, s.max_row_nnz)) * kInstThreads * sizeof(double);
  d->inst_ok = s.max_row_nnz <= 96 && build_inst_ranges(t, d->h_inst_rng, d->h_inst_cells);
  if (d->inst_ok) {
    ar.up(&d->inst_rng, d->h_inst_rng);
    ar.work(&d->inst_list, d->h_inst_rng.size());
    ar.work(&d->inst_ticket, 1);
  }
  if ((ierr = ar.commit(d->stream))) return ierr;
  d->allocs.push_back(ar.base);
  CUDA_TRY(cudaMemsetAsync(accum_prev, 0, sizeof(double) * m.nc, d->stream));
  a.accum_prev = accum_prev;
  if (t->opt.setup_on_device &&
      (ierr = device_canon_trans(t, a.cellc, a.facec, const_cast<double *>(a.Tc), d->stream)))
    return ierr;
  if (t->opt.setup_on_device && (ierr = device_gen_trans(t, const_cast<double *>(a.trans), d->stream))) return ierr;
  build_slabs(t, d);  // their copy stream and events are taken on first use
  if ((ierr = cell_smem_optin(d->device, cell_smem_bytes(a, cell_warp_form(a))))) return ierr;
  if ((ierr = noalloc_resolve(d->device))) return ierr;
  if ((ierr = pool_event(&d->noalloc_ev))) return ierr;
  // the uploads (and the device-built Trans) are complete before any other
  // stream uses them, and the staging buffer and host vectors above outlive
  // them; only this handle's stream is waited for
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  return 0;
}

// Waits for the work this handle has in flight (its own streams and the
// callers' streams it has seen), frees its memory stream-ordered (no
// device-wide synchronisation, so other handles keep running) and returns its
// streams and events to the pools.
void device_destroy(_p_TDy *t) {
  DeviceState *d = t->dev;
  if (!d) return;
  if (d->stream) cudaStreamSynchronize(d->stream);
  for (auto &u : d->user_streams) {
    cudaEventSynchronize(u.second);
    pool_release(d->device, nullptr, u.second);
  }
  if (d->noalloc_ev) {
    cudaEventSynchronize(d->noalloc_ev);
    pool_release(d->device, nullptr, d->noalloc_ev);
  }
  for (int k = 0; k < 4; k++)
    if (d->ev[k]) cudaEventDestroy(d->ev[k]);
  if (d->slab_exec) cudaGraphExecDestroy(d->slab_exec);
  if (d->copy_stream) {
    cudaStreamSynchronize(d->copy_stream);
    pool_release(d->device, d->copy_stream, nullptr);
  }
  for (cudaEvent_t e : d->slab_ev) pool_release(d->device, nullptr, e);
  if (d->stream) {
    for (void *p : d->allocs) dmem_free(p, d->stream);
    cudaStreamSynchronize(d->stream);
    pool_release(d->device, d->stream, nullptr);
  }
  delete d;
  t->dev = nullptr;
}

int device_upload_source_sink(_p_TDy *t) {
  DeviceState *d = t->dev;
  CUDA_TRY(cudaMemcpyAsync((void *)d->a.ss, t->mat.source_sink.data(), sizeof(double) * t->mesh.nc,
                           cudaMemcpyHostToDevice, d->stream));
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  return 0;
}

static inline unsigned nblocks(long long n, int bs) { return (unsigned)((n + bs - 1) / bs); }

// A multiplier coprime to n near 0.618 n (golden-ratio stride), so that
// chunk -> chunk * m mod n is a permutation that scatters neighbouring chunks.
static int chunk_multiplier(int n) {
  if (n <= 2) return 1;
  long long m = (long long)(0.6180339887 * n) | 1;
  auto gcd = [](long long x, long long y) {
    while (y) {
      long long t = x % y;
      x = y;
      y = t;
    }
    return x;
  };
  while (gcd(m, n) != 1) m += 2;
  return (int)(m % n);
}

int device_presolve(_p_TDy *t, const double *dUprev, void *stream) {
  DeviceState *d = t->dev;
  cudaStream_t st = stream ? (cudaStream_t)stream : d->stream;
  DevArgs a = d->a;
  a.dt = t->dtime;
  presolve_kernel<<<nblocks(a.nc, 256), 256, 0, st>>>(a, dUprev, (double *)a.accum_prev);
  CUDA_TRY(cudaGetLastError());
  return note_stream(d, st);
}

int device_presolve_host(_p_TDy *t, const double *Uprev) {
  DeviceState *d = t->dev;
  CUDA_TRY(cudaMemcpyAsync(d->dU, Uprev, sizeof(double) * t->mesh.nc, cudaMemcpyHostToDevice, d->stream));
  int ierr = device_presolve(t, d->dU, d->stream);
  if (ierr) return ierr;
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  return 0;
}

// The four launches of one evaluation; events[] (5 entries, or null) bracket
// them for the per-kernel timers.
static void launch_state_range(const DevArgs &a, int e0, int e1, Emit &e) {
  if (e1 <= e0) return;
  const int nchunks = (int)nblocks(e1 - e0, 32);
  e(state_kernel, nblocks((long long)nchunks * 32, 256), 256, 0, a, e0, e1, nchunks, chunk_multiplier(nchunks));
}
static void launch_state(const DevArgs &a, Emit &e) { launch_state_range(a, 0, a.nc + a.nb, e); }

// Vertex stage over the vertices a names (gen_vertex/ngen, [vc0, vc1)).
// gen_warp: mostly other vertices (e.g. prisms, whose valence-4 vertices are
// canonical): the warp form in its own launch, then the canonical ones; else
// one launch with the thread form in the first blocks.  The choice is made
// once per mesh, so a slab launches the same form as the whole evaluation.
static int rho_mode(const DevArgs &a) {
  return a.rho_type == WATER_DENSITY_CONSTANT ? RHO_CONST
         : a.rho_type == WATER_DENSITY_EXPONENTIAL ? RHO_EXP
                                                   : RHO_NODERIV;
}

static void launch_vertices(const DevArgs &a, bool gen_warp, Emit &e) {
  if (gen_warp && a.ngen > 0)
    e(generic_vertex_kernel, nblocks(a.ngen, kGenWarps), 128, (size_t)kGenWarps * a.gen_warp_doubles * sizeof(double),
      a);
  const int rho = rho_mode(a);
  if (a.jac_ff) {
    const size_t smem = (size_t)pair_shared_rows(rho) * (kPairThreads / 2) * sizeof(double);
    const int pb = (int)nblocks(a.vc1 - a.vc0, kPairThreads / 2), gb = gen_warp ? 0 : (int)nblocks(a.ngen, kPairThreads);
    auto k = rho == RHO_CONST ? vertex_pair_kernel<RHO_CONST>
             : rho == RHO_NODERIV ? vertex_pair_kernel<RHO_NODERIV>
                                  : vertex_pair_kernel<RHO_EXP>;
    e(k, pb + gb, kPairThreads, smem, a, gb);
    return;
  }
  const size_t smem = 36 * 128 * sizeof(double);
  const int cb = (int)nblocks(a.vc1 - a.vc0, 128), gb = gen_warp ? 0 : (int)nblocks(a.ngen, 128);
  auto k = rho == RHO_CONST ? vertex_kernel<RHO_CONST, false>
           : rho == RHO_NODERIV ? vertex_kernel<RHO_NODERIV, false>
                                : vertex_kernel<RHO_EXP, false>;
  e(k, cb + gb, 128, smem, a, gb);
}

// Cell stage over the cells a names (sc_cells/nS, gc_cells/ngc); gen_warp:
// mostly other cells take the warp form.
static size_t cell_smem_bytes(const DevArgs &a, bool gen_warp) {
  return 64 * (size_t)(gen_warp || a.max_row_nnz < 27 ? 27 : a.max_row_nnz) * sizeof(double);
}

// (rows longer than 96 entries need more than 48 KB of dynamic shared
// memory: device_setup opts in for the handle's device)
static void launch_cells(const DevArgs &a, bool gen_warp, Emit &e) {
  const int sb = (int)nblocks(a.nS, 64), gcb = gen_warp ? 0 : (int)nblocks(a.ngc, 64);
  e(cell_kernel, sb + gcb, 64, cell_smem_bytes(a, gen_warp), a, sb);
  if (gen_warp && a.ngc > 0)
    e(generic_cell_kernel, nblocks(a.ngc, 2 * kCellWarps), 32 * kCellWarps,
      (size_t)2 * kCellWarps * (size_t)a.max_row_nnz * sizeof(double), a);
}

static bool vertex_warp_form(const DevArgs &a) { return a.ngen > a.nC; }
static bool cell_warp_form(const DevArgs &a) { return a.ngc > a.nS; }

// The stages of one evaluation; events[] (4 entries, or null) bracket them
// for the per-kernel timers.
static int launch_eval(const DevArgs &a, cudaStream_t st, cudaEvent_t *events) {
  Emit e(st);
  if (events) CUDA_TRY(cudaEventRecord(events[0], st));
  launch_state(a, e);
  if (events) CUDA_TRY(cudaEventRecord(events[1], st));
  launch_vertices(a, vertex_warp_form(a), e);
  if (events) CUDA_TRY(cudaEventRecord(events[2], st));
  launch_cells(a, cell_warp_form(a), e);
  if (events) CUDA_TRY(cudaEventRecord(events[3], st));
  CUDA_TRY(cudaGetLastError());
  return 0;
}

// The arguments of one evaluation.
static int eval_args(_p_TDy *t, int form, const double *dU, const double *dUt, double shift, double *dR, double *dJ,
                     DevArgs *out) {
  DeviceState *d = t->dev;
  if (form == FORM_SNES && !(t->dtime > 0.0))
    return set_error(TDY_ERR_USER, "SNES form needs TDySetDtimeForSNESSolver before evaluation");
  DevArgs a = d->a;
  a.form = form;
  a.U = dU;
  a.Ut = dUt;
  a.dt = t->dtime;
  a.shift = form == FORM_SNES ? 1.0 / t->dtime : shift;
  a.needR = dR != nullptr;
  a.needJ = dJ != nullptr;
  a.R = dR;
  a.J = dJ;
  *out = a;
  return 0;
}

int device_eval(_p_TDy *t, int form, double time, const double *dU, const double *dUt, double shift, double *dR,
                double *dJ, void *stream) {
  (void)time;
  DeviceState *d = t->dev;
  cudaStream_t st = stream ? (cudaStream_t)stream : d->stream;
  DevArgs a;
  int ierr = eval_args(t, form, dU, dUt, shift, dR, dJ, &a);
  if (ierr) return ierr;
  ierr = launch_eval(a, st, d->timers ? d->ev : nullptr);
  if (ierr) return ierr;
  if ((ierr = note_stream(d, st))) return ierr;
  if (d->timers) {
    CUDA_TRY(cudaEventSynchronize(d->ev[3]));
    for (int k = 0; k < 3; k++) {
      float ms = 0.f;
      CUDA_TRY(cudaEventElapsedTime(&ms, d->ev[k], d->ev[k + 1]));
      d->t_ms[k] += ms;
      d->t_calls[k] += 1;
    }
  }
  return 0;
}

// Instance-schedule evaluation (SNES form) of the listed instances (blocks);
// the others keep their R and J.  TDY_ERR_SUP when the handle has no
// instance ranges (blocks not contiguous, or rows too long).
static size_t g_inst_smem_granted[kMaxDevices] = {};

int device_eval_instances(_p_TDy *t, const double *dU, double *dR, double *dJ, const int *list, int nlist,
                          void *stream) {
  DeviceState *d = t->dev;
  if (!d->inst_ok) return set_error(TDY_ERR_SUP, "instance schedule unavailable for this handle");
  if (nlist <= 0) return 0;
  cudaStream_t st = stream ? (cudaStream_t)stream : d->stream;
  DevArgs a;
  int ierr = eval_args(t, FORM_SNES, dU, nullptr, 0.0, dR, dJ, &a);
  if (ierr) return ierr;
  using Kern = void (*)(DevArgs, const InstRange *, const int *, int, int *);
  const Kern kerns[6] = {instance_eval_kernel<RHO_CONST, false>,   instance_eval_kernel<RHO_CONST, true>,
                         instance_eval_kernel<RHO_NODERIV, false>, instance_eval_kernel<RHO_NODERIV, true>,
                         instance_eval_kernel<RHO_EXP, false>,     instance_eval_kernel<RHO_EXP, true>};
  const Kern kern = kerns[2 * rho_mode(a) + (a.jac_ff ? 1 : 0)];
  if (d->inst_smem > 48 * 1024) {
    std::lock_guard<std::mutex> lk(g_dev_mutex);
    if (d->inst_smem > g_inst_smem_granted[d->device]) {
      for (Kern k : kerns)
        CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)d->inst_smem));
      g_inst_smem_granted[d->device] = d->inst_smem;
    }
  }
  int nsm = 0, per_sm = 0;
  CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, d->device));
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kInstThreads, d->inst_smem));
  const int grid = std::max(1, std::min(nlist, nsm * std::max(per_sm, 1)));
  d->h_list.assign(list, list + nlist);  // read by the copy before the caller's next synchronisation
  CUDA_TRY(cudaMemcpyAsync(d->inst_list, d->h_list.data(), sizeof(int) * nlist, cudaMemcpyHostToDevice, st));
  CUDA_TRY(cudaMemsetAsync(d->inst_ticket, 0, sizeof(int), st));
  kern<<<grid, kInstThreads, d->inst_smem, st>>>(a, d->inst_rng, d->inst_list, nlist, d->inst_ticket);
  CUDA_TRY(cudaGetLastError());
  return note_stream(d, st);
}

bool device_inst_ok(_p_TDy *t) { return t->dev && t->dev->inst_ok; }

void *device_default_stream(_p_TDy *t) { return t->dev ? (void *)t->dev->stream : nullptr; }

int device_download_trans(_p_TDy *t, std::vector<double> &trans) {
  const DeviceState *d = t->dev;
  trans.resize(t->setup.trans.size());
  if (!trans.empty())
    CUDA_TRY(cudaMemcpy(trans.data(), d->a.trans, sizeof(double) * trans.size(), cudaMemcpyDeviceToHost));
  return 0;
}

int device_download_tc(_p_TDy *t, std::vector<double> &Tc) {
  const DeviceState *d = t->dev;
  Tc.resize(96 * (size_t)t->setup.nCpad);
  CUDA_TRY(cudaMemcpy(Tc.data(), d->a.Tc, sizeof(double) * Tc.size(), cudaMemcpyDeviceToHost));
  return 0;
}

int device_set_timers(_p_TDy *t, int on) {
  DeviceState *d = t->dev;
  if (on && !d->ev[0])
    for (int k = 0; k < 4; k++) CUDA_TRY(cudaEventCreate(&d->ev[k]));
  d->timers = on != 0;
  for (int k = 0; k < 3; k++) {
    d->t_ms[k] = 0.0;
    d->t_calls[k] = 0;
  }
  return 0;
}

int device_get_timers(_p_TDy *t, int *n, const char **names, double *ms, long long *calls) {
  DeviceState *d = t->dev;
  int cap = *n;
  *n = 3;
  for (int k = 0; k < 3 && k < cap; k++) {
    if (names) names[k] = kKernelNames[k];
    if (ms) ms[k] = d->t_ms[k];
    if (calls) calls[k] = d->t_calls[k];
  }
  return 0;
}

// FP64 throughput probe: independent FMA chains per thread, enough blocks to
// fill every SM; reports achieved double-precision TFLOP/s on the device.
__global__ void __launch_bounds__(256) fp64_probe_kernel(double *out, int iters) {
  double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
  double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
  const double b = 0.999999999, c = 1e-12;
  for (int i = 0; i < iters; i++) {
    a0 = fma(a0, b, c);
    a1 = fma(a1, b, c);
    a2 = fma(a2, b, c);
    a3 = fma(a3, b, c);
    a4 = fma(a4, b, c);
    a5 = fma(a5, b, c);
    a6 = fma(a6, b, c);
    a7 = fma(a7, b, c);
  }
  double s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == 12345.678) out[blockIdx.x] = s;  // keep the chains live
}

int device_fp64_probe(double *tflops) {
  int dev = 0, nsm = 0;
  CUDA_TRY(cudaGetDevice(&dev));
  CUDA_TRY(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  double *out = nullptr;
  CUDA_TRY(cudaMalloc(&out, sizeof(double) * nsm * 8));
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  const int iters = 4096, blocks = nsm * 8, threads = 256;
  fp64_probe_kernel<<<blocks, threads>>>(out, iters);  // warm-up
  CUDA_TRY(cudaEventRecord(e0));
  const int reps = 5;
  for (int r = 0; r < reps; r++) fp64_probe_kernel<<<blocks, threads>>>(out, iters);
  CUDA_TRY(cudaEventRecord(e1));
  CUDA_TRY(cudaEventSynchronize(e1));
  float ms = 0.f;
  CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  double flops = 2.0 * 8.0 * iters * (double)blocks * threads * reps;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return 0;
}

int device_transient_variable_host(_p_TDy *t, const double *U, double *C, double *dC) {
  DeviceState *d = t->dev;
  const size_t n = (size_t)t->mesh.nc;
  CUDA_TRY(cudaMemcpyAsync(d->dU, U, sizeof(double) * n, cudaMemcpyHostToDevice, d->stream));
  tv_kernel<<<nblocks(n, 256), 256, 0, d->stream>>>(d->a, d->dU, C ? d->diagS : nullptr, dC ? d->diagMass : nullptr);
  CUDA_TRY(cudaGetLastError());
  if (C) CUDA_TRY(cudaMemcpyAsync(C, d->diagS, sizeof(double) * n, cudaMemcpyDeviceToHost, d->stream));
  if (dC) CUDA_TRY(cudaMemcpyAsync(dC, d->diagMass, sizeof(double) * n, cudaMemcpyDeviceToHost, d->stream));
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  return 0;
}

int device_eval_dae_host(_p_TDy *t, double time, const double *U2, const double *Ut2, double *R2) {
  DeviceState *d = t->dev;
  const int n = t->mesh.nc;
  if (!d->dae) {  // interleaved buffers, allocated on the first DAE call
    int ierr;
    if ((ierr = dalloc(d, &d->dae, 6 * (size_t)n))) return ierr;
  }
  double *dU2 = d->dae, *dUt2 = d->dae + 2 * (size_t)n, *dR2 = d->dae + 4 * (size_t)n;
  CUDA_TRY(cudaMemcpyAsync(dU2, U2, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, d->stream));
  CUDA_TRY(cudaMemcpyAsync(dUt2, Ut2, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, d->stream));
  dae_split_kernel<<<nblocks(n, 256), 256, 0, d->stream>>>(n, dU2, dUt2, d->dU, d->dUt);
  CUDA_TRY(cudaGetLastError());
  int ierr = device_eval(t, FORM_TV, time, d->dU, d->dUt, 0.0, d->dR, nullptr, d->stream);
  if (ierr) return ierr;
  tv_kernel<<<nblocks(n, 256), 256, 0, d->stream>>>(d->a, d->dU, d->diagS, nullptr);
  dae_merge_kernel<<<nblocks(n, 256), 256, 0, d->stream>>>(n, dU2, d->dR, d->diagS, dR2);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(R2, dR2, sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, d->stream));
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  return 0;
}

// The arguments of slab k: the vertices and cells of slab k only.
static DevArgs slab_args(const DevArgs &a, const DeviceState::Slab &sl) {
  DevArgs b = a;
  b.gen_vertex = a.gen_vertex + sl.g0;
  b.ngen = sl.g1 - sl.g0;
  b.vc0 = sl.vc0;
  b.vc1 = sl.vc1;
  b.sc_cells = a.sc_cells + sl.s0;
  b.sc_vc = a.sc_vc + sl.s0;  // structure of arrays, stride nSpad: the offset carries over
  b.nS = sl.s1 - sl.s0;
  b.gc_cells = a.gc_cells + sl.gc0;
  b.ngc = sl.gc1 - sl.gc0;
  return b;
}

static bool pinned(const void *p) {
  if (!p) return true;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

// The slab pipeline as a graph: U (and U_t) to the device, the boundary
// faces' state, then per slab the state of the cells its vertices read, its
// vertex and cell stages, and its rows of J and R to host memory.  The state
// of slab k waits for that of slab k-1 and, so that the first slab runs
// alone, for the vertex stage of slab k-1; the vertex stage of slab k waits
// for the state of slab k (so it sees every cell it reads); the cell stage of slab k waits
// for its vertex stage only, so it runs beside the state and vertex stages of
// slab k+1 (each stage writes entries no other running stage reads) and the
// tail of one launch overlaps the next; the copies form a chain of their
// own, each after its slab's cell stage, and run while the next slabs are
// evaluated.  One launch replaces about ten driver calls per slab.
static int build_slab_graph(_p_TDy *t, DeviceState *d, const DevArgs &a, const double *U, const double *Ut,
                            double *R, double *J, cudaGraphExec_t *out) {
  const size_t n = (size_t)t->mesh.nc;
  cudaGraph_t g = nullptr;
  CUDA_TRY(cudaGraphCreate(&g, 0));
  cudaError_t err = cudaSuccess;
  cudaGraphNode_t up[2] = {nullptr, nullptr}, join = nullptr, copy_last = nullptr;
  int nup = 0;
  err = cudaGraphAddMemcpyNode1D(&up[nup++], g, nullptr, 0, d->dU, U, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (err == cudaSuccess && Ut)
    err = cudaGraphAddMemcpyNode1D(&up[nup++], g, nullptr, 0, d->dUt, Ut, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (err == cudaSuccess) err = cudaGraphAddEmptyNode(&join, g, up, nup);
  Emit e(nullptr);
  e.g = g;
  e.last = join;
  if (err == cudaSuccess) {
    const bool vw = vertex_warp_form(a), cw = cell_warp_form(a);
    const size_t K = d->slabs.size();
    launch_state_range(a, a.nc, a.nc + a.nb, e);  // boundary faces
    cudaGraphNode_t sprev = e.last, vprev = nullptr;
    for (size_t k = 0; k < K && err == cudaSuccess && e.err == cudaSuccess; k++) {
      const DeviceState::Slab &sl = d->slabs[k];
      const DevArgs b = slab_args(a, sl);
      // the state of slab k after that of slab k-1 and the vertex stage of
      // slab k-1 (so the first slab runs alone), then its vertex stage
      cudaGraphNode_t sdeps[2] = {sprev, vprev}, sjoin = nullptr;
      err = cudaGraphAddEmptyNode(&sjoin, g, sdeps, vprev ? 2 : 1);
      if (err != cudaSuccess) break;
      e.last = sjoin;
      launch_state_range(a, sl.e0, sl.e1, e);
      sprev = e.last;
      launch_vertices(b, vw, e);
      vprev = e.last;
      launch_cells(b, cw, e);
      if (e.err != cudaSuccess) break;
      cudaGraphNode_t deps[2] = {e.last, copy_last}, nj = nullptr;
      err = cudaGraphAddMemcpyNode1D(&nj, g, deps, copy_last ? 2 : 1, J + sl.j0, d->dJ + sl.j0,
                                     sizeof(double) * (size_t)(sl.j1 - sl.j0), cudaMemcpyDeviceToHost);
      copy_last = nj;
      if (err == cudaSuccess && R) {
        cudaGraphNode_t dr[2] = {e.last, copy_last}, nr = nullptr;
        err = cudaGraphAddMemcpyNode1D(&nr, g, dr, 2, R + sl.c0, d->dR + sl.c0, sizeof(double) * (size_t)(sl.c1 - sl.c0),
                                       cudaMemcpyDeviceToHost);
        copy_last = nr;
      }
    }
  }
  if (err == cudaSuccess) err = e.err;
  if (err == cudaSuccess) err = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (err != cudaSuccess) return set_error(TDY_ERR_GPU, "slab graph: %s", cudaGetErrorString(err));
  return 0;
}

int device_eval_host(_p_TDy *t, int form, double time, const double *U, const double *Ut, double shift, double *R,
                     double *J) {
  DeviceState *d = t->dev;
  const size_t n = (size_t)t->mesh.nc;
  if (d->slabs.size() > 1 && J && !d->timers) {
    // slab by slab (build_slabs): the same launches, split; the same bits
    DevArgs a;
    int ierr = eval_args(t, form, d->dU, Ut ? d->dUt : nullptr, shift, R ? d->dR : nullptr, d->dJ, &a);
    if (ierr) return ierr;
    DeviceState::SlabKey key;
    key.form = form;
    key.dt = a.dt;
    key.shift = a.shift;
    key.U = U;
    key.Ut = Ut;
    key.R = R;
    key.J = J;
    if (d->slab_exec && !(key == d->slab_key)) {
      CUDA_TRY(cudaGraphExecDestroy(d->slab_exec));
      d->slab_exec = nullptr;
    }
    if (!d->slab_exec && pinned(U) && pinned(Ut) && pinned(R) && pinned(J)) {
      if ((ierr = build_slab_graph(t, d, a, U, Ut, R, J, &d->slab_exec))) return ierr;
      d->slab_key = key;
    }
    if (d->slab_exec) {
      CUDA_TRY(cudaGraphLaunch(d->slab_exec, d->stream));
      CUDA_TRY(cudaStreamSynchronize(d->stream));
      return 0;
    }
    // pageable host buffers: the same pipeline on two streams
    CUDA_TRY(cudaMemcpyAsync(d->dU, U, sizeof(double) * n, cudaMemcpyHostToDevice, d->stream));
    if (Ut) CUDA_TRY(cudaMemcpyAsync(d->dUt, Ut, sizeof(double) * n, cudaMemcpyHostToDevice, d->stream));
    if (!d->copy_stream) {  // first such call of this handle
      if ((ierr = pool_stream(&d->copy_stream))) return ierr;
      d->slab_ev.assign(d->slabs.size(), nullptr);
      for (cudaEvent_t &e : d->slab_ev)
        if ((ierr = pool_event(&e))) return ierr;
    }
    const bool vw = vertex_warp_form(a), cw = cell_warp_form(a);
    Emit e(d->stream);
    launch_state_range(a, a.nc, a.nc + a.nb, e);  // boundary faces
    for (size_t k = 0; k < d->slabs.size(); k++) {
      const DeviceState::Slab &sl = d->slabs[k];
      const DevArgs b = slab_args(a, sl);
      launch_state_range(a, sl.e0, sl.e1, e);
      launch_vertices(b, vw, e);
      launch_cells(b, cw, e);
      CUDA_TRY(cudaEventRecord(d->slab_ev[k], d->stream));
      CUDA_TRY(cudaStreamWaitEvent(d->copy_stream, d->slab_ev[k], 0));
      CUDA_TRY(cudaMemcpyAsync(J + sl.j0, d->dJ + sl.j0, sizeof(double) * (size_t)(sl.j1 - sl.j0),
                               cudaMemcpyDeviceToHost, d->copy_stream));
      if (R)
        CUDA_TRY(cudaMemcpyAsync(R + sl.c0, d->dR + sl.c0, sizeof(double) * (size_t)(sl.c1 - sl.c0),
                                 cudaMemcpyDeviceToHost, d->copy_stream));
    }
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(d->copy_stream));
    CUDA_TRY(cudaStreamSynchronize(d->stream));
    return 0;
  }
  CUDA_TRY(cudaMemcpyAsync(d->dU, U, sizeof(double) * n, cudaMemcpyHostToDevice, d->stream));
  if (Ut) CUDA_TRY(cudaMemcpyAsync(d->dUt, Ut, sizeof(double) * n, cudaMemcpyHostToDevice, d->stream));
  int ierr = device_eval(t, form, time, d->dU, Ut ? d->dUt : nullptr, shift, R ? d->dR : nullptr, J ? d->dJ : nullptr,
                         d->stream);
  if (ierr) return ierr;
  if (R) CUDA_TRY(cudaMemcpyAsync(R, d->dR, sizeof(double) * n, cudaMemcpyDeviceToHost, d->stream));
  if (J) CUDA_TRY(cudaMemcpyAsync(J, d->dJ, sizeof(double) * d->nnz, cudaMemcpyDeviceToHost, d->stream));
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  return 0;
}

// ---------------------------------------------------------------------------
// Evaluation without any device allocation of its own.
//
// The per-vertex partial sums (J_v, R_v) normally live in scratch that
// TDySetup allocates for the handle.  This variant takes them from a fixed
// array compiled into the library instead, so nothing in it allocates device
// memory.  The array is 64 MiB of doubles; every GPU that loads the library
// holds it until the process exits.  Host code never uses the array's name as
// an address (on the host it is only a stand-in for the symbol): the device
// address is looked up with cudaGetSymbolAddress once per device, while that
// device is current, by TDySetup (noalloc_resolve), so the call itself loads
// no module and allocates nothing, even the first time.
//
// All calls share the array and it keeps the last call's contents.  Nothing
// has to start at zero: vertex_kernel writes every partial that cell_kernel
// then reads in the same call.  Calls that overlap on the GPU (two streams, or
// two handles at once) race on the array and must be serialised by the caller.
#define TDY_NOALLOC_SCRATCH_DOUBLES (8ull << 20)
static __device__ __align__(256) double g_noalloc_scratch[TDY_NOALLOC_SCRATCH_DOUBLES];
static double *g_noalloc_ptr[kMaxDevices] = {};

static int noalloc_resolve(int dev) {
  if (dev < 0 || dev >= kMaxDevices) return set_error(TDY_ERR_SUP, "device ordinal %d not supported", dev);
  std::lock_guard<std::mutex> lk(g_dev_mutex);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_ptr[dev] = (double *)p;
  }
  return 0;
}

int device_eval_noalloc(_p_TDy *t, const double *dU, double *dR, double *dJ, void *stream) {
  DeviceState *d = t->dev;
  const long long need = t->setup.scratch_size;
  if (need > (long long)TDY_NOALLOC_SCRATCH_DOUBLES)
    return set_error(TDY_ERR_ARG_OUTOFRANGE,
                     "mesh needs %lld doubles of partial-sum scratch; the static scratch holds %llu (64 MiB). "
                     "Use TDyMPFAOSNESFunctionJacobianDevice for meshes this large",
                     need, (unsigned long long)TDY_NOALLOC_SCRATCH_DOUBLES);
  if (!(t->dtime > 0.0)) return set_error(TDY_ERR_USER, "SNES form needs TDySetDtimeForSNESSolver before evaluation");
  int dev = -1;
  CUDA_TRY(cudaGetDevice(&dev));
  if (dev != d->device)
    return set_error(TDY_ERR_USER, "current CUDA device %d is not the device %d this handle was set up on", dev,
                     d->device);
  double *scratch = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_dev_mutex);
    scratch = g_noalloc_ptr[dev];  // resolved by TDySetup on this device
  }
  if (!scratch) return set_error(TDY_ERR_LIB, "static scratch address of device %d was not resolved at set-up", dev);
  cudaStream_t st = stream ? (cudaStream_t)stream : d->stream;
  DevArgs a = d->a;
  a.form = FORM_SNES;
  a.U = dU;
  a.Ut = nullptr;
  a.dt = t->dtime;
  a.shift = 1.0 / t->dtime;
  a.needR = dR != nullptr;
  a.needJ = dJ != nullptr;
  a.R = dR;
  a.J = dJ;
  a.scratch = scratch;
  int ierr = launch_eval(a, st, nullptr);
  if (ierr) return ierr;
  CUDA_TRY(cudaEventRecord(d->noalloc_ev, st));
  return 0;
}

int device_launches_per_eval(_p_TDy *t) {
  const DevArgs &a = t->dev->a;
  const bool vw = a.ngen > a.nC, cw = a.ngc > a.nS;
  const int nvert = vw ? (a.ngen > 0) + (a.nC > 0) : ((a.nC + a.ngen) > 0 ? 1 : 0);
  const int ncell = cw ? (a.ngc > 0) + (a.nS > 0) : ((a.nS + a.ngc) > 0 ? 1 : 0);
  return 1 + nvert + ncell;
}

int device_synchronize(_p_TDy *t) {
  CUDA_TRY(cudaStreamSynchronize(t->dev->stream));
  return 0;
}

int device_update_state_host(_p_TDy *t, const double *U) {
  DeviceState *d = t->dev;
  CUDA_TRY(cudaMemcpyAsync(d->dU, U, sizeof(double) * t->mesh.nc, cudaMemcpyHostToDevice, d->stream));
  DevArgs a = d->a;
  a.U = d->dU;
  diag_kernel<<<nblocks(a.nc, 256), 256, 0, d->stream>>>(a, d->diagS, d->diagMass);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaStreamSynchronize(d->stream));
  return 0;
}

int device_get_diagnostic(_p_TDy *t, int which, double *out) {
  DeviceState *d = t->dev;
  CUDA_TRY(cudaMemcpy(out, which == 0 ? d->diagS : d->diagMass, sizeof(double) * t->mesh.nc, cudaMemcpyDeviceToHost));
  return 0;
}

}  // namespace tdy
