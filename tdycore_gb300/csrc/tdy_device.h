// tdy_device.h -- host-side interface of the CUDA translation unit.
#pragma once

#include "tdy_internal.h"

namespace tdy {

// accumulation terms: SNES backward Euler, TS (dm/dP U_t), TS with the mass
// as transient variable (M_t given)
enum { FORM_SNES = 0, FORM_TS = 1, FORM_TV = 2 };

// Device memory of handles and their solvers: stream-ordered allocation
// (cudaMallocAsync / cudaFreeAsync from the device's default pool) on the
// handle's stream, so that setting up or destroying a handle never
// synchronises the device and handles served by other threads keep running.
// A pointer from dmem_alloc is usable on other streams once `stream` has
// been synchronised.
int dmem_alloc(void **p, size_t bytes, void *stream);
void dmem_free(void *p, void *stream);

int device_setup(_p_TDy *t);
void device_destroy(_p_TDy *t);
int device_upload_source_sink(_p_TDy *t);
int device_presolve(_p_TDy *t, const double *dU_prev, void *stream);
int device_presolve_host(_p_TDy *t, const double *U_prev);
int device_eval(_p_TDy *t, int form, double time, const double *dU, const double *dUt, double shift, double *dR,
                double *dJ, void *stream);
int device_eval_host(_p_TDy *t, int form, double time, const double *U, const double *Ut, double shift, double *R,
                     double *J);
int device_launches_per_eval(_p_TDy *t);
// SNES-form evaluation of the listed instances (blocks) in one launch, one CTA
// per instance (the same bits as device_eval); the others keep their R and J.
int device_eval_instances(_p_TDy *t, const double *dU, double *dR, double *dJ, const int *list, int nlist,
                          void *stream);
bool device_inst_ok(_p_TDy *t);
int device_synchronize(_p_TDy *t);
int device_update_state_host(_p_TDy *t, const double *U);
int device_get_diagnostic(_p_TDy *t, int which, double *out);
int device_set_timers(_p_TDy *t, int on);
int device_get_timers(_p_TDy *t, int *n, const char **names, double *ms, long long *calls);
int device_fp64_probe(double *tflops);
int device_eval_noalloc(_p_TDy *t, const double *dU, double *dR, double *dJ, void *stream);
// C = rho phi S V and dC = d(rho phi S)/dP V per cell (either may be null).
int device_transient_variable_host(_p_TDy *t, const double *U, double *C, double *dC);
// DAE form: U, U_t, R interleaved [P, M] per cell (2 * ncells values).
int device_eval_dae_host(_p_TDy *t, double time, const double *U2, const double *Ut2, double *R2);
void *device_default_stream(_p_TDy *t);
// copies the device's canonical-vertex Trans (96 x nCpad) to the host
int device_download_tc(_p_TDy *t, std::vector<double> &Tc);
// Backward-Euler Newton solve of every instance (tdy_solver.cu).
int device_be_solve(_p_TDy *t, double dt, double *dU, const TDyNewtonOptions &o, TDyNewtonStats *stats,
                    int *inst_its, double *inst_rel, void *stream);
void device_solver_destroy(_p_TDy *t);
int device_num_instances(_p_TDy *t);
// Trans of the canonical vertices into d_Tc (-tdy_mpfao_setup_on_device).
int device_canon_trans(const _p_TDy *t, const int *d_cellc, const int *d_facec, double *d_Tc, void *stream);
// Trans of the other vertices marked by the set-up (setup.dev_gen_vertex), in
// place in the device Trans array (-tdy_mpfao_setup_on_device).
int device_gen_trans(const _p_TDy *t, double *d_trans, void *stream);
// copies the device's generic Trans array (setup.ntrans) to the host
int device_download_trans(_p_TDy *t, std::vector<double> &trans);

}  // namespace tdy
