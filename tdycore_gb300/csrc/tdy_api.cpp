// tdy_api.cpp -- C-ABI lifecycle, options, setters and host-pointer entry
// points of the GB300 MPFA-O Richards path.
//
// Call order and error behaviour follow src/tdycore.c: TDySetMode before
// TDySetDiscretization (:832-842), TDySetFromOptions before TDySetup
// (:627-639, :732-739).  Only RICHARDS + MPFA_O is provided; any other mode or
// discretization returns TDY_ERR_SUP.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "tdy_device.h"
#include "tdy_internal.h"

namespace tdy {

static thread_local std::string g_errmsg;

int set_error(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_errmsg = buf;
  return code;
}

// ---------------------------------------------------------------------------
// Options database: the -tdy_* subset of PETSc's options that this path reads.
static std::mutex g_opt_mutex;
static std::vector<std::string> g_opts;

static bool opt_find(const char *name, std::string *value) {
  std::lock_guard<std::mutex> lk(g_opt_mutex);
  bool found = false;
  for (size_t i = 0; i < g_opts.size(); i++) {
    if (g_opts[i] == name) {
      found = true;
      if (value) *value = (i + 1 < g_opts.size() && g_opts[i + 1][0] != '-') ? g_opts[i + 1] : std::string();
      if (value && i + 1 < g_opts.size()) {
        // negative numbers are values, not option names
        const std::string &nx = g_opts[i + 1];
        if (nx.size() > 1 && nx[0] == '-' && (isdigit((unsigned char)nx[1]) || nx[1] == '.')) *value = nx;
      }
    }
  }
  return found;
}

static int opt_real(const char *name, double *v) {
  std::string s;
  if (!opt_find(name, &s)) return 0;
  char *end = nullptr;
  double x = strtod(s.c_str(), &end);
  if (s.empty() || (end && *end)) return set_error(TDY_ERR_ARG_WRONG, "option %s expects a real, got '%s'", name, s.c_str());
  *v = x;
  return 0;
}

static int opt_int(const char *name, int *v) {
  std::string s;
  if (!opt_find(name, &s)) return 0;
  char *end = nullptr;
  long x = strtol(s.c_str(), &end, 10);
  if (s.empty() || (end && *end)) return set_error(TDY_ERR_ARG_WRONG, "option %s expects an integer, got '%s'", name, s.c_str());
  *v = (int)x;
  return 0;
}

static int opt_enum(const char *name, const char *const *names, int n, int *v) {
  std::string s;
  if (!opt_find(name, &s)) return 0;
  for (int i = 0; i < n; i++)
    if (strcasecmp(s.c_str(), names[i]) == 0) {
      *v = i;
      return 0;
    }
  return set_error(TDY_ERR_ARG_WRONG, "option %s: unknown value '%s'", name, s.c_str());
}

// Reference EOS (src/materials/tdyeos.c:5-136); the Batzle-Wang forms are
// evaluated at T = Tref and zero salinity and carry no pressure derivatives.
void eos_density(int type, double p, double *rho, double *drho, double *d2rho) {
  if (type == WATER_DENSITY_CONSTANT) {
    *rho = 998.0;
    *drho = 0.0;
    *d2rho = 0.0;
  } else if (type == WATER_DENSITY_EXPONENTIAL) {
    const double rho0 = 997.16e0, p0 = 101325.e0, c = 1.e-8;
    if (p < p0) {
      *rho = rho0;
      *drho = 0.0;
      *d2rho = 0.0;
    } else {
      *rho = rho0 * std::exp(c * (p - p0));
      *drho = c * (*rho);
      *d2rho = c * (*drho);
    }
  } else {
    const double T = 25.0, S = 0.0, P = p * 1.e-6;
    double pw = 1 + 1.e-6 * (-80. * T - 3.3 * std::pow(T, 2) + 0.00175 * std::pow(T, 3) + 489. * P - 2. * T * P +
                             0.016 * P * std::pow(T, 2) - 1.3e-5 * std::pow(T, 3) * P - 0.333 * std::pow(P, 2) -
                             0.002 * T * std::pow(P, 2));
    pw *= 1000.;
    *rho = pw + S * (0.668 + 0.44 * S + 1e-6 * (300. * P - 2400. * P * S + T * (80. * 3. * T - 3300. * S - 13. * P + 47. * P * S))) * 1000.;
    *drho = 0.0;
    *d2rho = 0.0;
  }
}

void eos_viscosity(int type, double p, double *vis, double *dvis, double *d2vis) {
  (void)p;
  if (type == WATER_VISCOSITY_CONSTANT) {
    *vis = 9.94e-4;
  } else {
    const double T = 25.0, S = 0.0;
    *vis = 0.1 + 0.333 * S +
           (1.65 + 91.9 * std::pow(S, 3)) * std::exp((-0.42 * std::pow((std::pow(S, 0.8) - 0.17), 2) + 0.045) * std::pow(T, 0.8));
    *vis *= 1e-3;
  }
  *dvis = 0.0;
  *d2vis = 0.0;
}

// Unsmoothed Mualem kr and dkr/dSe (tdycharacteristiccurves.c:468-485).
static void mualem_unsmoothed(double m, double Se, double *Kr, double *dKr) {
  *Kr = 1.0;
  *dKr = 0.0;
  if (Se >= 1.0) return;
  double so = std::pow(Se, 1 / m);
  double tmp = std::pow(1 - so, m);
  *Kr = std::sqrt(Se);
  *Kr *= (1 - tmp) * (1 - tmp);
  *dKr = 0.5 * (*Kr) / Se;
  *dKr += 2 * std::pow(Se, 1 / m - 0.5) * std::pow(1 - so, m - 1) * (1 - std::pow(1 - so, m));
}

// Cubic smoothing coefficients (tdycharacteristiccurves.c:509-535, 577-596):
// solves the same 4x4 system as the reference's dgesv call with partial
// pivoting.
int mualem_smoothing_coeffs(double m, double x0, double x1, double x2, double dx, double coeffs[4]) {
  double Kr, dKr;
  mualem_unsmoothed(m, x1, &Kr, &dKr);
  double rhs[4] = {1.0, Kr, 0.0, dKr};
  double xt1 = (x1 - x0) / dx, xt2 = (x2 - x0) / dx;
  double xt1_p2 = xt1 * xt1, xt2_p2 = xt2 * xt2, xt1_p3 = xt1 * xt1 * xt1, xt2_p3 = xt2 * xt2 * xt2;
  // column-major as in the reference, converted to row-major A[i][j]
  double cm[16] = {1.0, 1.0, 0.0, 0.0, xt2, xt1, 1.0 / dx, 1.0 / dx,
                   xt2_p2, xt1_p2, 2.0 * xt2 / dx, 2.0 * xt1 / dx, xt2_p3, xt1_p3, 3.0 * xt2_p2 / dx, 3.0 * xt1_p2 / dx};
  double A[4][4];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) A[i][j] = cm[j * 4 + i];
  for (int k = 0; k < 4; k++) {
    int p = k;
    for (int i = k + 1; i < 4; i++)
      if (std::fabs(A[i][k]) > std::fabs(A[p][k])) p = i;
    if (A[p][k] == 0.0) return set_error(TDY_ERR_USER, "CubicPolynomialSetup failed");
    if (p != k) {
      for (int j = 0; j < 4; j++) std::swap(A[k][j], A[p][j]);
      std::swap(rhs[k], rhs[p]);
    }
    for (int i = k + 1; i < 4; i++) {
      double l = A[i][k] / A[k][k];
      for (int j = k + 1; j < 4; j++) A[i][j] -= l * A[k][j];
      rhs[i] -= l * rhs[k];
    }
  }
  for (int k = 3; k >= 0; k--) {
    double s = rhs[k];
    for (int j = k + 1; j < 4; j++) s -= A[k][j] * rhs[j];
    rhs[k] = s / A[k][k];
  }
  for (int i = 0; i < 4; i++) coeffs[i] = rhs[i];
  return 0;
}

}  // namespace tdy

using namespace tdy;

#define TDY_CHECK_HANDLE(t)                                                        \
  do {                                                                             \
    if (!(t)) return set_error(TDY_ERR_ARG_NULL, "%s: null TDy handle", __func__); \
  } while (0)
#define TDY_CHECK_NOT_SETUP(t)                                                                    \
  do {                                                                                            \
    if ((t)->is_setup) return set_error(TDY_ERR_USER, "%s must be called before TDySetup", __func__); \
  } while (0)
#define TDY_CHECK_SETUP(t)                                                                       \
  do {                                                                                           \
    if (!(t)->is_setup) return set_error(TDY_ERR_USER, "%s requires TDySetup to have run", __func__); \
  } while (0)
#define TDY_CHECK_DEVICE(t)                                                                                 \
  do {                                                                                                      \
    TDY_CHECK_SETUP(t);                                                                                     \
    if (!(t)->dev) return set_error(TDY_ERR_GPU, "%s: no device state (TDySetupHost does not allocate HBM)", __func__); \
  } while (0)

extern "C" {

const char *TDyGetErrorMessage(void) { return g_errmsg.c_str(); }

TDyErrorCode TDyInit(int argc, char **argv) {
  std::lock_guard<std::mutex> lk(g_opt_mutex);
  g_opts.clear();
  for (int i = 1; i < argc; i++)
    if (argv && argv[i]) g_opts.emplace_back(argv[i]);
  return 0;
}
TDyErrorCode TDyInitNoArguments(void) { return TDyInit(0, nullptr); }
TDyErrorCode TDyFinalize(void) {
  std::lock_guard<std::mutex> lk(g_opt_mutex);
  g_opts.clear();
  return 0;
}
TDyErrorCode TDyOptionsInsertString(const char *options) {
  if (!options) return 0;
  std::istringstream ss(options);
  std::string w;
  std::lock_guard<std::mutex> lk(g_opt_mutex);
  while (ss >> w) g_opts.push_back(w);
  return 0;
}
TDyErrorCode TDyOptionsClear(void) { return TDyFinalize(); }

TDyErrorCode TDyOptionsGetReal(const char *name, double *value, int *set) {
  if (!name || !value) return set_error(TDY_ERR_ARG_NULL, "TDyOptionsGetReal: null argument");
  const int present = opt_find(name, nullptr) ? 1 : 0;
  if (set) *set = present;
  return present ? opt_real(name, value) : 0;
}
TDyErrorCode TDyOptionsGetInt(const char *name, int *value, int *set) {
  if (!name || !value) return set_error(TDY_ERR_ARG_NULL, "TDyOptionsGetInt: null argument");
  const int present = opt_find(name, nullptr) ? 1 : 0;
  if (set) *set = present;
  return present ? opt_int(name, value) : 0;
}
TDyErrorCode TDyOptionsGetString(const char *name, char *value, int len, int *set) {
  if (!name || !value || len <= 0) return set_error(TDY_ERR_ARG_NULL, "TDyOptionsGetString: null argument");
  std::string s;
  const bool present = opt_find(name, &s);
  if (set) *set = present ? 1 : 0;
  if (present) {
    if ((int)s.size() >= len) return set_error(TDY_ERR_ARG_OUTOFRANGE, "option %s: value longer than %d", name, len - 1);
    memcpy(value, s.c_str(), s.size() + 1);
  }
  return 0;
}
TDyErrorCode TDyOptionsHasName(const char *name, int *set) {
  if (!name || !set) return set_error(TDY_ERR_ARG_NULL, "TDyOptionsHasName: null argument");
  *set = opt_find(name, nullptr) ? 1 : 0;
  return 0;
}

TDyErrorCode TDyCreate(void *comm, TDy *tdy) {
  (void)comm;
  if (!tdy) return set_error(TDY_ERR_ARG_NULL, "TDyCreate: null output pointer");
  *tdy = new (std::nothrow) _p_TDy();
  if (!*tdy) return set_error(TDY_ERR_MEM, "TDyCreate: out of memory");
  return 0;
}

TDyErrorCode TDySetMode(TDy tdy, TDyMode mode) {
  TDY_CHECK_HANDLE(tdy);
  if (mode != RICHARDS) return set_error(TDY_ERR_SUP, "only the RICHARDS mode is provided on this path");
  tdy->mode = mode;
  tdy->flags |= TDY_FLAG_MODE;
  return 0;
}

TDyErrorCode TDySetDiscretization(TDy tdy, TDyDiscretization d) {
  TDY_CHECK_HANDLE(tdy);
  if (!(tdy->flags & TDY_FLAG_MODE)) return set_error(TDY_ERR_USER, "You must call TDySetMode before TDySetDiscretization");
  if (d != MPFA_O && d != MPFA_O_DAE && d != MPFA_O_TRANSIENTVAR)
    return set_error(TDY_ERR_SUP, "only the MPFA_O discretizations (MPFA_O, MPFA_O_DAE, MPFA_O_TRANSIENTVAR) are "
                                  "provided on this path");
  tdy->discretization = d;
  tdy->flags |= TDY_FLAG_DISC;
  return 0;
}
TDyErrorCode TDySetDiscretizationMethod(TDy tdy, TDyDiscretization d) { return TDySetDiscretization(tdy, d); }

TDyErrorCode TDySetFromOptions(TDy tdy) {
  TDY_CHECK_HANDLE(tdy);
  if (tdy->is_setup) return set_error(TDY_ERR_USER, "You must call TDySetFromOptions before TDySetup()");
  Options &o = tdy->opt;
  static const char *const modes[] = {"RICHARDS", "TH", "SALINITY"};
  static const char *const discs[] = {"MPFA_O", "MPFA_O_DAE", "MPFA_O_TRANSIENTVAR", "BDM", "WY", "FV_TPF"};
  static const char *const dens[] = {"CONSTANT", "EXPONENTIAL", "BATZLE_AND_WANG"};
  static const char *const visc[] = {"CONSTANT", "BATZLE_AND_WANG"};
  static const char *const gm[] = {"MPFAO_GMATRIX_DEFAULT", "MPFAO_GMATRIX_TPF"};
  static const char *const bct[] = {"DIRICHLET_BC", "NEUMANN_BC", "SEEPAGE_BC"};
  static const char *const jarith[] = {"DOUBLE_FLOAT", "FP64"};
  int ierr;
  // option names as spelled in src/tdycore.c:525-540 and tdympfao.c:584-596
  if ((ierr = opt_real("-tdy_porosity", &o.porosity))) return ierr;
  if ((ierr = opt_real("-tdy_permability", &o.permeability))) return ierr;
  if ((ierr = opt_real("-tdy_residual_satuaration", &o.residual_saturation))) return ierr;
  if ((ierr = opt_real("-tdy_gardner_param_n", &o.gardner_n))) return ierr;
  if ((ierr = opt_real("-tdy_vangenuchten_param_m", &o.vangenuchten_m))) return ierr;
  if ((ierr = opt_real("-tdy_vangenuchten_param_alpha", &o.vangenuchten_alpha))) return ierr;
  if ((ierr = opt_real("-tdy_gravity", &o.gravity))) return ierr;
  if ((ierr = opt_enum("-tdy_water_density", dens, 3, &o.rho_type))) return ierr;
  if ((ierr = opt_enum("-tdy_water_viscosity", visc, 2, &o.mu_type))) return ierr;
  if ((ierr = opt_enum("-tdy_mpfao_gmatrix_method", gm, 2, &o.gmatrix_method))) return ierr;
  if ((ierr = opt_enum("-tdy_mpfao_boundary_condition_type", bct, 3, &o.bc_type))) return ierr;
  // extension: arithmetic of the Jacobian products (FP64 residual either way)
  if ((ierr = opt_enum("-tdy_jacobian_arithmetic", jarith, 2, &o.jacobian_arithmetic))) return ierr;
  // extension: build the interior hexahedral vertices' Trans on the device
  if (opt_find("-tdy_mpfao_setup_on_device", nullptr)) o.setup_on_device = true;
  // regression output (src/tdycore.c:617, src/tdyregression.c:33-45)
  if (opt_find("-tdy_regression_test", nullptr)) o.regression_testing = true;
  if ((ierr = opt_int("-tdy_regression_test_num_cells_per_process", &o.regression_num_cells))) return ierr;
  {
    std::string fn;
    if (opt_find("-tdy_regression_test_filename", &fn)) o.regression_filename = fn;
  }
  double pbc;
  if (opt_find("-tdy_pressure_bc_value", nullptr)) {
    if ((ierr = opt_real("-tdy_pressure_bc_value", &pbc))) return ierr;
    o.has_pressure_bc_value = true;
    o.pressure_bc_value = pbc;
  }
  int mode = tdy->mode, disc = tdy->discretization;
  if ((ierr = opt_enum("-tdy_mode", modes, 3, &mode))) return ierr;
  if ((ierr = opt_enum("-tdy_discretization", discs, 6, &disc))) return ierr;
  if (mode != tdy->mode && (ierr = TDySetMode(tdy, (TDyMode)mode))) return ierr;
  if (disc != tdy->discretization && (ierr = TDySetDiscretization(tdy, (TDyDiscretization)disc))) return ierr;
  tdy->flags |= TDY_FLAG_OPTIONS;
  return 0;
}

// ---------------------------------------------------------------------------
// Mesh
TDyErrorCode TDySetExtrudedMesh(TDy tdy, int nv2, const double *xy, int nc2, int nvpc, const int *cells2d, int nlayers,
                                const double *z) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_NOT_SETUP(tdy);
  if (!xy || !cells2d || !z) return set_error(TDY_ERR_ARG_NULL, "TDySetExtrudedMesh: null array");
  if (nv2 <= 0 || nc2 <= 0 || nlayers <= 0) return set_error(TDY_ERR_ARG_OUTOFRANGE, "TDySetExtrudedMesh: empty mesh");
  if (nvpc != 3 && nvpc != 4) return set_error(TDY_ERR_SUP, "TDySetExtrudedMesh: polygons must have 3 or 4 vertices");
  ExtrudedInput in;
  in.set = true;
  in.nv2 = nv2;
  in.nc2 = nc2;
  in.nvpc = nvpc;
  in.nlayers = nlayers;
  in.xy.assign(xy, xy + 2 * (size_t)nv2);
  in.cells2d.assign(cells2d, cells2d + (size_t)nvpc * nc2);
  in.z.assign(z, z + (size_t)(nlayers + 1) * nv2);
  tdy->mesh_blocks.assign(1, std::move(in));
  return 0;
}

TDyErrorCode TDySetExtrudedMeshes(TDy tdy, int nblocks, const int *nv2, const double *xy, const int *nc2, int nvpc,
                                  const int *cells2d, const int *nlayers, const double *z) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_NOT_SETUP(tdy);
  if (nblocks <= 0) return set_error(TDY_ERR_ARG_OUTOFRANGE, "TDySetExtrudedMeshes: no blocks");
  if (!nv2 || !xy || !nc2 || !cells2d || !nlayers || !z) return set_error(TDY_ERR_ARG_NULL, "TDySetExtrudedMeshes: null array");
  if (nvpc != 3 && nvpc != 4) return set_error(TDY_ERR_SUP, "TDySetExtrudedMeshes: polygons must have 3 or 4 vertices");
  std::vector<ExtrudedInput> blocks(nblocks);
  size_t oxy = 0, oc = 0, oz = 0;
  for (int b = 0; b < nblocks; b++) {
    if (nv2[b] <= 0 || nc2[b] <= 0 || nlayers[b] <= 0)
      return set_error(TDY_ERR_ARG_OUTOFRANGE, "TDySetExtrudedMeshes: block %d is empty", b);
    ExtrudedInput &in = blocks[b];
    in.set = true;
    in.nv2 = nv2[b];
    in.nc2 = nc2[b];
    in.nvpc = nvpc;
    in.nlayers = nlayers[b];
    in.xy.assign(xy + oxy, xy + oxy + 2 * (size_t)nv2[b]);
    in.cells2d.assign(cells2d + oc, cells2d + oc + (size_t)nvpc * nc2[b]);
    in.z.assign(z + oz, z + oz + (size_t)(nlayers[b] + 1) * nv2[b]);
    for (int k : in.cells2d)
      if (k < 0 || k >= nv2[b]) return set_error(TDY_ERR_ARG_OUTOFRANGE, "TDySetExtrudedMeshes: block %d vertex index %d", b, k);
    oxy += 2 * (size_t)nv2[b];
    oc += (size_t)nvpc * nc2[b];
    oz += (size_t)(nlayers[b] + 1) * nv2[b];
  }
  tdy->mesh_blocks = std::move(blocks);
  return 0;
}

TDyErrorCode TDySetBoxMesh(TDy tdy, int nx, int ny, int nz, const double lower[3], const double upper[3]) {
  TDY_CHECK_HANDLE(tdy);
  if (nx <= 0 || ny <= 0 || nz <= 0) return set_error(TDY_ERR_ARG_OUTOFRANGE, "TDySetBoxMesh: nx, ny, nz must be > 0");
  double lo[3] = {0, 0, 0}, hi[3] = {1, 1, 1};
  if (lower) memcpy(lo, lower, sizeof(lo));
  if (upper) memcpy(hi, upper, sizeof(hi));
  int nv2 = (nx + 1) * (ny + 1), nc2 = nx * ny;
  std::vector<double> xy(2 * (size_t)nv2), zz((size_t)(nz + 1) * nv2);
  std::vector<int> c2(4 * (size_t)nc2);
  for (int j = 0; j <= ny; j++)
    for (int i = 0; i <= nx; i++) {
      xy[2 * ((size_t)j * (nx + 1) + i) + 0] = lo[0] + (hi[0] - lo[0]) * i / nx;
      xy[2 * ((size_t)j * (nx + 1) + i) + 1] = lo[1] + (hi[1] - lo[1]) * j / ny;
    }
  for (int k = 0; k <= nz; k++)
    for (int v = 0; v < nv2; v++) zz[(size_t)k * nv2 + v] = lo[2] + (hi[2] - lo[2]) * k / nz;
  for (int j = 0; j < ny; j++)
    for (int i = 0; i < nx; i++) {
      int c = j * nx + i;
      int v0 = j * (nx + 1) + i;
      c2[4 * (size_t)c + 0] = v0;
      c2[4 * (size_t)c + 1] = v0 + 1;
      c2[4 * (size_t)c + 2] = v0 + nx + 2;
      c2[4 * (size_t)c + 3] = v0 + nx + 1;
    }
  return TDySetExtrudedMesh(tdy, nv2, xy.data(), nc2, 4, c2.data(), nz, zz.data());
}

// ---------------------------------------------------------------------------
// Materials
TDyErrorCode TDySetWaterDensityType(TDy tdy, TDyWaterDensityType t) {
  TDY_CHECK_HANDLE(tdy);
  if (t < WATER_DENSITY_CONSTANT || t > WATER_DENSITY_BATZLE_AND_WANG) return set_error(TDY_ERR_ARG_OUTOFRANGE, "bad density type");
  tdy->opt.rho_type = t;
  return 0;
}
TDyErrorCode TDySetWaterViscosityType(TDy tdy, TDyWaterViscosityType t) {
  TDY_CHECK_HANDLE(tdy);
  if (t < WATER_VISCOSITY_CONSTANT || t > WATER_VISCOSITY_BATZLE_AND_WANG) return set_error(TDY_ERR_ARG_OUTOFRANGE, "bad viscosity type");
  tdy->opt.mu_type = t;
  return 0;
}
TDyErrorCode TDySetConstantPorosity(TDy tdy, double v) {
  TDY_CHECK_HANDLE(tdy);
  tdy->porosity.kind = ScalarSpec::CONSTANT;
  tdy->porosity.value = v;
  return 0;
}
TDyErrorCode TDySetPorosityFunction(TDy tdy, TDyScalarSpatialFunction f) {
  TDY_CHECK_HANDLE(tdy);
  if (!f) return set_error(TDY_ERR_ARG_NULL, "null function");
  tdy->porosity.kind = ScalarSpec::FUNCTION;
  tdy->porosity.func = f;
  return 0;
}
TDyErrorCode TDySetConstantResidualSaturation(TDy tdy, double v) {
  TDY_CHECK_HANDLE(tdy);
  tdy->sr.kind = ScalarSpec::CONSTANT;
  tdy->sr.value = v;
  return 0;
}
TDyErrorCode TDySetResidualSaturationFunction(TDy tdy, TDyScalarSpatialFunction f) {
  TDY_CHECK_HANDLE(tdy);
  if (!f) return set_error(TDY_ERR_ARG_NULL, "null function");
  tdy->sr.kind = ScalarSpec::FUNCTION;
  tdy->sr.func = f;
  return 0;
}
TDyErrorCode TDySetConstantIsotropicPermeability(TDy tdy, double k) {
  TDY_CHECK_HANDLE(tdy);
  tdy->perm.kind = PermSpec::ISO_CONST;
  for (int i = 0; i < 9; i++) tdy->perm.k[i] = 0.0;
  tdy->perm.k[0] = tdy->perm.k[4] = tdy->perm.k[8] = k;
  return 0;
}
TDyErrorCode TDySetIsotropicPermeabilityFunction(TDy tdy, TDyScalarSpatialFunction f) {
  TDY_CHECK_HANDLE(tdy);
  if (!f) return set_error(TDY_ERR_ARG_NULL, "null function");
  tdy->perm.kind = PermSpec::ISO_FUNC;
  tdy->perm.func = f;
  return 0;
}
TDyErrorCode TDySetConstantDiagonalPermeability(TDy tdy, const double k[3]) {
  TDY_CHECK_HANDLE(tdy);
  if (!k) return set_error(TDY_ERR_ARG_NULL, "null array");
  tdy->perm.kind = PermSpec::DIAG_CONST;
  for (int i = 0; i < 9; i++) tdy->perm.k[i] = 0.0;
  tdy->perm.k[0] = k[0];
  tdy->perm.k[4] = k[1];
  tdy->perm.k[8] = k[2];
  return 0;
}
TDyErrorCode TDySetDiagonalPermeabilityFunction(TDy tdy, TDyVectorSpatialFunction f) {
  TDY_CHECK_HANDLE(tdy);
  if (!f) return set_error(TDY_ERR_ARG_NULL, "null function");
  tdy->perm.kind = PermSpec::DIAG_FUNC;
  tdy->perm.func = f;
  return 0;
}
TDyErrorCode TDySetConstantTensorPermeability(TDy tdy, const double k[9]) {
  TDY_CHECK_HANDLE(tdy);
  if (!k) return set_error(TDY_ERR_ARG_NULL, "null array");
  tdy->perm.kind = PermSpec::TENSOR_CONST;
  for (int i = 0; i < 9; i++) tdy->perm.k[i] = k[i];
  return 0;
}
TDyErrorCode TDySetTensorPermeabilityFunction(TDy tdy, TDyTensorSpatialFunction f) {
  TDY_CHECK_HANDLE(tdy);
  if (!f) return set_error(TDY_ERR_ARG_NULL, "null function");
  tdy->perm.kind = PermSpec::TENSOR_FUNC;
  tdy->perm.func = f;
  return 0;
}

static int check_values(int n, const void *vals) {
  if (n < 0) return set_error(TDY_ERR_ARG_OUTOFRANGE, "negative count");
  if (n > 0 && !vals) return set_error(TDY_ERR_ARG_NULL, "null values");
  return 0;
}

TDyErrorCode TDySetPorosityValuesLocal(TDy tdy, int n, const int *cells, const double *v) {
  TDY_CHECK_HANDLE(tdy);
  if (int e = check_values(n, v)) return e;
  for (int i = 0; i < n; i++) tdy->porosity.overrides.push_back({cells ? cells[i] : i, v[i]});
  return 0;
}
TDyErrorCode TDySetResidualSaturationValuesLocal(TDy tdy, int n, const int *cells, const double *v) {
  TDY_CHECK_HANDLE(tdy);
  if (int e = check_values(n, v)) return e;
  for (int i = 0; i < n; i++) tdy->sr.overrides.push_back({cells ? cells[i] : i, v[i]});
  return 0;
}
TDyErrorCode TDySetPermeabilityValuesLocal(TDy tdy, int n, const int *cells, const double *k9) {
  TDY_CHECK_HANDLE(tdy);
  if (int e = check_values(n, k9)) return e;
  for (int i = 0; i < n; i++)
    tdy->perm.overrides.push_back({cells ? cells[i] : i, std::vector<double>(k9 + 9 * (size_t)i, k9 + 9 * (size_t)i + 9)});
  return 0;
}
TDyErrorCode TDySetCharacteristicCurveVanGenuchtenValuesLocal(TDy tdy, int n, const int *cells, const double *m,
                                                               const double *alpha) {
  TDY_CHECK_HANDLE(tdy);
  if (int e = check_values(n, m)) return e;
  if (int e = check_values(n, alpha)) return e;
  for (int i = 0; i < n; i++) tdy->vg_over.push_back({cells ? cells[i] : i, {m[i], alpha[i]}});
  return 0;
}
TDyErrorCode TDySetCharacteristicCurveMualemValuesLocal(TDy tdy, int n, const int *cells, const double *m) {
  TDY_CHECK_HANDLE(tdy);
  if (int e = check_values(n, m)) return e;
  for (int i = 0; i < n; i++) tdy->mualem_over.push_back({cells ? cells[i] : i, m[i]});
  return 0;
}
TDyErrorCode TDySetCharacteristicCurveGardnerValuesLocal(TDy tdy, int n, const int *cells, const double *gn,
                                                          const double *gm, const double *alpha) {
  TDY_CHECK_HANDLE(tdy);
  if (int e = check_values(n, gn)) return e;
  if (int e = check_values(n, gm)) return e;
  if (int e = check_values(n, alpha)) return e;
  for (int i = 0; i < n; i++) tdy->gardner_over.push_back({cells ? cells[i] : i, {gn[i], gm[i], alpha[i]}});
  return 0;
}
TDyErrorCode TDySetCharacteristicCurveIrmayValuesLocal(TDy tdy, int n, const int *cells, const double *m) {
  TDY_CHECK_HANDLE(tdy);
  if (int e = check_values(n, m)) return e;
  for (int i = 0; i < n; i++) tdy->irmay_over.push_back({cells ? cells[i] : i, m[i]});
  return 0;
}
TDyErrorCode TDySetSourceSinkValuesLocal(TDy tdy, int n, const int *cells, const double *q) {
  TDY_CHECK_HANDLE(tdy);
  if (int e = check_values(n, q)) return e;
  if (tdy->is_setup) {
    for (int i = 0; i < n; i++) {
      int c = cells ? cells[i] : i;
      if (c < 0 || c >= tdy->mesh.nc) return set_error(TDY_ERR_ARG_OUTOFRANGE, "cell %d out of range", c);
      tdy->mat.source_sink[c] = q[i];
    }
    return tdy->dev ? device_upload_source_sink(tdy) : 0;
  }
  for (int i = 0; i < n; i++) tdy->source_over.push_back({cells ? cells[i] : i, q[i]});
  return 0;
}

TDyErrorCode TDySetBoundaryPressureFunction(TDy tdy, TDyScalarSpatialFunction f) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_NOT_SETUP(tdy);
  tdy->bc_pressure_func = f;
  return 0;
}
TDyErrorCode TDySetBoundaryPressureTypeFunction(TDy tdy, TDyScalarSpatialIntegerFunction f) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_NOT_SETUP(tdy);
  tdy->bc_type_func = f;
  return 0;
}
TDyErrorCode TDyMPFAOSetGmatrixMethod(TDy tdy, TDyMPFAOGmatrixMethod m) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_NOT_SETUP(tdy);
  if (m != MPFAO_GMATRIX_DEFAULT && m != MPFAO_GMATRIX_TPF) return set_error(TDY_ERR_ARG_OUTOFRANGE, "bad gmatrix method");
  tdy->opt.gmatrix_method = m;
  return 0;
}
TDyErrorCode TDyMPFAOSetBoundaryConditionType(TDy tdy, TDyBoundaryConditionType t) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_NOT_SETUP(tdy);
  if (t < DIRICHLET_BC || t > SEEPAGE_BC) return set_error(TDY_ERR_ARG_OUTOFRANGE, "bad boundary condition type");
  tdy->opt.bc_type = t;
  return 0;
}

// ---------------------------------------------------------------------------
// Setup
static int eval_scalar(const ScalarSpec &s, double dflt, int nc, std::vector<double> &X, std::vector<double> &out) {
  out.assign(nc, dflt);
  if (s.kind == ScalarSpec::CONSTANT)
    out.assign(nc, s.value);
  else if (s.kind == ScalarSpec::FUNCTION)
    s.func(nc, X.data(), out.data());
  for (auto &ov : s.overrides) {
    if (ov.first < 0 || ov.first >= nc) return set_error(TDY_ERR_ARG_OUTOFRANGE, "cell %d out of range", ov.first);
    out[ov.first] = ov.second;
  }
  return 0;
}

static int build_materials(TDy t) {
  const int nc = t->mesh.nc;
  const Options &o = t->opt;
  Materials &mat = t->mat;
  std::vector<double> X(t->mesh.cell_cen);
  int ierr;
  if ((ierr = eval_scalar(t->porosity, o.porosity, nc, X, mat.porosity))) return ierr;
  if ((ierr = eval_scalar(t->sr, o.residual_saturation, nc, X, mat.Sr))) return ierr;
  mat.K0.assign(9 * (size_t)nc, 0.0);
  const PermSpec &p = t->perm;
  std::vector<double> buf;
  for (int c = 0; c < nc; c++) {
    double *K = &mat.K0[9 * (size_t)c];
    if (p.kind == PermSpec::DEFAULT) {
      K[0] = K[4] = K[8] = o.permeability;
    } else if (p.kind == PermSpec::ISO_CONST || p.kind == PermSpec::DIAG_CONST || p.kind == PermSpec::TENSOR_CONST) {
      for (int i = 0; i < 9; i++) K[i] = p.k[i];
    }
  }
  if (p.kind == PermSpec::ISO_FUNC) {
    buf.assign(nc, 0.0);
    p.func(nc, X.data(), buf.data());
    for (int c = 0; c < nc; c++) mat.K0[9 * (size_t)c] = mat.K0[9 * (size_t)c + 4] = mat.K0[9 * (size_t)c + 8] = buf[c];
  } else if (p.kind == PermSpec::DIAG_FUNC) {
    buf.assign(3 * (size_t)nc, 0.0);
    p.func(nc, X.data(), buf.data());
    for (int c = 0; c < nc; c++)
      for (int d = 0; d < 3; d++) mat.K0[9 * (size_t)c + 4 * d] = buf[3 * (size_t)c + d];
  } else if (p.kind == PermSpec::TENSOR_FUNC) {
    buf.assign(9 * (size_t)nc, 0.0);
    p.func(nc, X.data(), buf.data());
    mat.K0 = buf;
  }
  for (auto &ov : p.overrides) {
    if (ov.first < 0 || ov.first >= nc) return set_error(TDY_ERR_ARG_OUTOFRANGE, "cell %d out of range", ov.first);
    for (int i = 0; i < 9; i++) mat.K0[9 * (size_t)ov.first + i] = ov.second[i];
  }
  // Characteristic curves: van Genuchten + Mualem by default (InitMaterials,
  // tdympfao.c:699-738).
  mat.sat_type.assign(nc, SAT_FUNC_VAN_GENUCHTEN);
  mat.sat_param.assign(3 * (size_t)nc, 0.0);
  mat.relperm_type.assign(nc, REL_PERM_FUNC_MUALEM);
  mat.relperm_param.assign(9 * (size_t)nc, 0.0);
  std::vector<double> mualem_m(nc, o.vangenuchten_m);
  for (int c = 0; c < nc; c++) {
    mat.sat_param[3 * (size_t)c + 0] = o.vangenuchten_m;
    mat.sat_param[3 * (size_t)c + 1] = o.vangenuchten_alpha;
  }
  for (auto &ov : t->vg_over) {
    int c = ov.first;
    if (c < 0 || c >= nc) return set_error(TDY_ERR_ARG_OUTOFRANGE, "cell %d out of range", c);
    mat.sat_type[c] = SAT_FUNC_VAN_GENUCHTEN;
    mat.sat_param[3 * (size_t)c + 0] = ov.second[0];
    mat.sat_param[3 * (size_t)c + 1] = ov.second[1];
  }
  for (auto &ov : t->gardner_over) {
    int c = ov.first;
    if (c < 0 || c >= nc) return set_error(TDY_ERR_ARG_OUTOFRANGE, "cell %d out of range", c);
    mat.sat_type[c] = SAT_FUNC_GARDNER;
    for (int i = 0; i < 3; i++) mat.sat_param[3 * (size_t)c + i] = ov.second[i];
  }
  for (auto &ov : t->mualem_over) {
    if (ov.first < 0 || ov.first >= nc) return set_error(TDY_ERR_ARG_OUTOFRANGE, "cell %d out of range", ov.first);
    mualem_m[ov.first] = ov.second;
  }
  // Smoothing coefficients depend only on m: cache them across cells.
  double last_m = std::nan(""), last_coef[4] = {0, 0, 0, 0};
  for (int c = 0; c < nc; c++) {
    double *rp = &mat.relperm_param[9 * (size_t)c];
    double m = mualem_m[c];
    rp[0] = m;
    rp[1] = o.mualem_poly_x0;
    rp[2] = o.mualem_poly_x1;
    rp[3] = o.mualem_poly_x2;
    rp[4] = o.mualem_poly_dx;
    if (!(m == last_m)) {
      if ((ierr = mualem_smoothing_coeffs(m, rp[1], rp[2], rp[3], rp[4], last_coef))) return ierr;
      last_m = m;
    }
    for (int i = 0; i < 4; i++) rp[5 + i] = last_coef[i];
  }
  for (auto &ov : t->irmay_over) {
    int c = ov.first;
    if (c < 0 || c >= nc) return set_error(TDY_ERR_ARG_OUTOFRANGE, "cell %d out of range", c);
    mat.relperm_type[c] = REL_PERM_FUNC_IRMAY;
    mat.relperm_param[9 * (size_t)c] = ov.second;
  }
  // Saturated-cell mobility kr(Se = 1)/mu, evaluated with the reference's
  // expressions (tdycharacteristiccurves.c:451-460, 551-562, 607-614).
  {
    double d1, d2;
    eos_viscosity(o.mu_type, o.Pref, &mat.vis, &d1, &d2);
    mat.lam_sat.assign(nc, 0.0);
    for (int c = 0; c < nc; c++) {
      const double *rp = &mat.relperm_param[9 * (size_t)c];
      double Kr = 1.0;
      if (mat.relperm_type[c] == REL_PERM_FUNC_MUALEM && 1.0 > rp[2]) {
        double xt = (1.0 - rp[1]) / rp[4];
        Kr = rp[5] + xt * (rp[6] + xt * (rp[7] + xt * rp[8]));
      }
      mat.lam_sat[c] = Kr / mat.vis;
    }
  }
  mat.source_sink.assign(nc, 0.0);
  for (auto &ov : t->source_over) {
    if (ov.first < 0 || ov.first >= nc) return set_error(TDY_ERR_ARG_OUTOFRANGE, "cell %d out of range", ov.first);
    mat.source_sink[ov.first] = ov.second;
  }
  return 0;
}

static int build_boundary(TDy t) {
  const Mesh &m = t->mesh;
  Boundary &b = t->bnd;
  b.type.assign(m.nb, t->opt.bc_type);
  b.has_value.assign(m.nb, 0);
  b.value.assign(m.nb, 0.0);
  b.rho.assign(m.nb, 0.0);
  b.vis.assign(m.nb, 0.0);
  // the spatial functions take n points at once: one call for all faces
  std::vector<double> xs(3 * (size_t)m.nb);
  for (int i = 0; i < m.nb; i++)
    for (int d = 0; d < 3; d++) xs[3 * (size_t)i + d] = m.face_cen[3 * (size_t)m.bnd_face[i] + d];
  if (t->bc_type_func && m.nb > 0) {
    t->bc_type_func(m.nb, xs.data(), b.type.data());
    for (int i = 0; i < m.nb; i++)
      if (b.type[i] < DIRICHLET_BC || b.type[i] > SEEPAGE_BC)
        return set_error(TDY_ERR_ARG_OUTOFRANGE, "bad boundary type %d", b.type[i]);
  }
  if (t->bc_pressure_func && m.nb > 0) t->bc_pressure_func(m.nb, xs.data(), b.value.data());
  for (int i = 0; i < m.nb; i++) {
    if (t->bc_pressure_func) {
      b.has_value[i] = 1;
    } else if (t->opt.has_pressure_bc_value) {
      b.has_value[i] = 1;
      b.value[i] = t->opt.pressure_bc_value;
    }
    double d1, d2;
    eos_density(t->opt.rho_type, t->opt.Pref, &b.rho[i], &d1, &d2);
    eos_viscosity(t->opt.mu_type, t->opt.Pref, &b.vis[i], &d1, &d2);
  }
  return 0;
}

static int setup_host(TDy tdy) {
  if (!(tdy->flags & TDY_FLAG_DISC)) return set_error(TDY_ERR_USER, "You must call TDySetDiscretization before TDySetup()");
  if (!(tdy->flags & TDY_FLAG_OPTIONS)) return set_error(TDY_ERR_USER, "You must call TDySetFromOptions before TDySetup()");
  if (tdy->is_setup) return set_error(TDY_ERR_USER, "TDySetup called twice");
  if (tdy->mesh_blocks.empty())
    return set_error(TDY_ERR_USER, "no mesh: call TDySetBoxMesh, TDySetExtrudedMesh or TDySetExtrudedMeshes before TDySetup");
  // TDyRegressionInitialize (src/tdyregression.c:38-45)
  if (tdy->opt.regression_testing && tdy->opt.regression_filename.empty())
    return set_error(TDY_ERR_USER, "Need to specify a regression filename via -tdy_regression_test_filename");
  int ierr;
  if (tdy->mesh_blocks.size() == 1) {
    if ((ierr = build_extruded_mesh(tdy->mesh_blocks[0], tdy->mesh))) return ierr;
  } else {
    std::vector<Mesh> parts(tdy->mesh_blocks.size());
    for (size_t b = 0; b < parts.size(); b++)
      if ((ierr = build_extruded_mesh(tdy->mesh_blocks[b], parts[b]))) return ierr;
    merge_meshes(parts, tdy->mesh);
  }
  if ((ierr = build_materials(tdy))) return ierr;
  if ((ierr = build_boundary(tdy))) return ierr;
  if ((ierr = mpfao_setup(tdy->opt, tdy->mesh, tdy->mat, tdy->bnd, tdy->setup))) return ierr;
  tdy->is_setup = true;
  tdy->flags |= TDY_FLAG_SETUP;
  return 0;
}

TDyErrorCode TDySetup(TDy tdy) {
  TDY_CHECK_HANDLE(tdy);
  int ierr = setup_host(tdy);
  if (ierr) return ierr;
  if ((ierr = device_setup(tdy))) {
    device_destroy(tdy);
    tdy->is_setup = false;
    tdy->flags &= ~TDY_FLAG_SETUP;
    return ierr;
  }
  return 0;
}

TDyErrorCode TDySetupHost(TDy tdy) {
  TDY_CHECK_HANDLE(tdy);
  return setup_host(tdy);
}

TDyErrorCode TDyDestroy(TDy *tdy) {
  if (!tdy || !*tdy) return 0;
  device_solver_destroy(*tdy);
  device_destroy(*tdy);
  delete *tdy;
  *tdy = nullptr;
  return 0;
}

// ---------------------------------------------------------------------------
// Queries
TDyErrorCode TDyGetNumCells(TDy tdy, int *n) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_SETUP(tdy);
  if (!n) return set_error(TDY_ERR_ARG_NULL, "null output");
  *n = tdy->mesh.nc;
  return 0;
}
TDyErrorCode TDyGetNumBoundaryFaces(TDy tdy, int *n) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_SETUP(tdy);
  if (!n) return set_error(TDY_ERR_ARG_NULL, "null output");
  *n = tdy->mesh.nb;
  return 0;
}
TDyErrorCode TDyGetCellCentroids(TDy tdy, double *xyz) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_SETUP(tdy);
  if (!xyz) return set_error(TDY_ERR_ARG_NULL, "null output");
  memcpy(xyz, tdy->mesh.cell_cen.data(), tdy->mesh.cell_cen.size() * sizeof(double));
  return 0;
}
TDyErrorCode TDyGetCellVolumes(TDy tdy, double *vol) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_SETUP(tdy);
  if (!vol) return set_error(TDY_ERR_ARG_NULL, "null output");
  memcpy(vol, tdy->mesh.cell_vol.data(), tdy->mesh.cell_vol.size() * sizeof(double));
  return 0;
}
TDyErrorCode TDyGetJacobianPattern(TDy tdy, int *nrows, int *nnz, const int **rowptr, const int **colidx) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_SETUP(tdy);
  if (nrows) *nrows = tdy->mesh.nc;
  if (nnz) *nnz = (int)tdy->setup.colidx.size();
  if (rowptr) *rowptr = tdy->setup.rowptr.data();
  if (colidx) *colidx = tdy->setup.colidx.data();
  return 0;
}
TDyErrorCode TDyCreateVectors(TDy tdy) {
  TDY_CHECK_HANDLE(tdy);
  return 0;
}
TDyErrorCode TDyCreateJacobian(TDy tdy) {
  TDY_CHECK_HANDLE(tdy);
  return 0;
}

TDyErrorCode TDyMPFAOGetSetupView(TDy tdy, struct TDyMPFAOSetupView *v) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_SETUP(tdy);
  if (!v) return set_error(TDY_ERR_ARG_NULL, "null view");
  // With -tdy_mpfao_setup_on_device the interior vertices' Trans exists only
  // on the device: bring it into the host arrays the view points at, once.
  if (tdy->opt.setup_on_device && tdy->dev && !tdy->trans_on_host) {
    MPFAOSetup &su = tdy->setup;
    if (!su.dev_gen_vertex.empty()) {  // the other vertices built on the device
      std::vector<double> tr;
      int ierr = device_download_trans(tdy, tr);
      if (ierr) return ierr;
      for (int vtx : su.dev_gen_vertex)
        std::copy(tr.begin() + su.v_trans_off[vtx], tr.begin() + su.v_trans_off[vtx + 1],
                  su.trans.begin() + su.v_trans_off[vtx]);
    }
    std::vector<double> Tc;
    int ierr = device_download_tc(tdy, Tc);
    if (ierr) return ierr;
    const long long P = su.nCpad;
    for (int k = 0; k < su.nC; k++) {
      const int vtx = su.canon_vertex[k];
      const int r0 = su.v_row_off[vtx], c0 = su.v_col_off[vtx];
      std::array<int, 8> oc;
      std::array<int, 12> cr;
      if (!canonical_layout(tdy->mesh, vtx, &su.col_ext[c0], &su.row_lup[r0], &su.row_ldn[r0], oc, cr))
        return set_error(TDY_ERR_LIB, "vertex %d lost its canonical layout", vtx);
      double *T = &su.trans[su.v_trans_off[vtx]];
      for (int rc = 0; rc < 12; rc++)
        for (int o = 0; o < 8; o++) T[cr[rc] * 8 + oc[o]] = Tc[(rc * 8 + o) * P + k];
    }
    tdy->trans_on_host = true;
  }
  const Mesh &m = tdy->mesh;
  const MPFAOSetup &s = tdy->setup;
  static thread_local std::vector<int> face_nverts;
  memset(v, 0, sizeof(*v));
  v->ncells = m.nc;
  v->nfaces = m.nf;
  v->nbnd = m.nb;
  v->nverts = m.nv;
  v->nrows_total = s.nrows;
  v->ncols_total = s.ncols;
  v->ntrans_total = s.ntrans;
  v->bc_type = tdy->opt.bc_type;
  v->gmatrix_method = tdy->opt.gmatrix_method;
  v->rho_type = tdy->opt.rho_type;
  v->mu_type = tdy->opt.mu_type;
  v->gravity = tdy->opt.gravity;
  v->Pref = tdy->opt.Pref;
  v->volume = m.cell_vol.data();
  v->centroid = m.cell_cen.data();
  v->porosity = tdy->mat.porosity.data();
  v->Sr = tdy->mat.Sr.data();
  v->K0 = tdy->mat.K0.data();
  v->sat_type = tdy->mat.sat_type.data();
  v->sat_param = tdy->mat.sat_param.data();
  v->relperm_type = tdy->mat.relperm_type.data();
  v->relperm_param = tdy->mat.relperm_param.data();
  v->source_sink = tdy->mat.source_sink.data();
  v->face_up = m.face_cell0.data();
  v->face_dn = m.face_cell1.data();
  v->gravdis = s.gravdis.data();
  v->face_centroid = m.face_cen.data();
  v->face_area = m.face_area.data();
  v->face_normal = m.face_nrm.data();
  face_nverts.resize(m.nf);
  for (int f = 0; f < m.nf; f++) face_nverts[f] = m.face_vert_off[f + 1] - m.face_vert_off[f];
  v->face_nverts = face_nverts.data();
  v->bnd_face = m.bnd_face.data();
  v->bnd_type = tdy->bnd.type.data();
  v->bnd_has_value = tdy->bnd.has_value.data();
  v->bnd_value = tdy->bnd.value.data();
  v->rho_bnd = tdy->bnd.rho.data();
  v->vis_bnd = tdy->bnd.vis.data();
  v->v_row_off = s.v_row_off.data();
  v->v_col_off = s.v_col_off.data();
  v->v_nint = s.v_nint.data();
  v->v_trans_off = s.v_trans_off.data();
  v->row_face = s.row_face.data();
  v->col_ext = s.col_ext.data();
  v->trans = s.trans.data();
  v->rowptr = s.rowptr.data();
  v->colidx = s.colidx.data();
  v->nnz = (int)s.colidx.size();
  return 0;
}

// ---------------------------------------------------------------------------
// Host-pointer hot entry points: copy in, evaluate on the device, copy out.
TDyErrorCode TDySetDtimeForSNESSolver(TDy tdy, double dt) {
  TDY_CHECK_HANDLE(tdy);
  if (!(dt > 0.0)) return set_error(TDY_ERR_ARG_OUTOFRANGE, "time step must be > 0");
  tdy->dtime = dt;
  return 0;
}
TDyErrorCode TDySetPreviousSolutionForSNESSolver(TDy tdy, const double *U) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_SETUP(tdy);
  if (!U) return set_error(TDY_ERR_ARG_NULL, "null solution");
  tdy->U_prev.assign(U, U + tdy->mesh.nc);
  tdy->have_prev = true;
  return 0;
}
TDyErrorCode TDyPreSolveSNESSolver(TDy tdy) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!tdy->have_prev) return set_error(TDY_ERR_USER, "TDyPreSolveSNESSolver: no previous solution set");
  if (!(tdy->dtime > 0.0)) return set_error(TDY_ERR_USER, "TDyPreSolveSNESSolver: call TDySetDtimeForSNESSolver first");
  return device_presolve_host(tdy, tdy->U_prev.data());
}
TDyErrorCode TDyPostSolve(TDy tdy, const double *U) { return TDySetPreviousSolutionForSNESSolver(tdy, U); }

// TDyRegressionInitialize + TDyRegressionOutput (src/tdyregression.c:8-250)
// for one process: cells c * floor(n / count), c < count (count capped at n);
// mean = sum / n with the sum taken in cell order.
TDyErrorCode TDyOutputRegression(TDy tdy, const double *U) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_SETUP(tdy);
  if (!tdy->opt.regression_testing) return 0;
  if (!U) return set_error(TDY_ERR_ARG_NULL, "TDyOutputRegression: null array");
  const int n = tdy->mesh.nc;
  int count = tdy->opt.regression_num_cells;
  if (n < count) count = n;
  const int inc = count > 0 ? n / count : 0;
  double mx = U[0], mn = U[0], sum = 0.0;
  for (int i = 0; i < n; i++) {
    mx = U[i] > mx ? U[i] : mx;
    mn = U[i] < mn ? U[i] : mn;
    sum += U[i];
  }
  const std::string fname = tdy->opt.regression_filename + ".regression";
  FILE *fp = fopen(fname.c_str(), "w");
  if (!fp) return set_error(TDY_ERR_USER, "Unable to write regression file %s", fname.c_str());
  fprintf(fp, "-- PRESSURE: Liquid Pressure --\n");
  fprintf(fp, "      Max: %21.13e\n", mx);
  fprintf(fp, "      Min: %21.13e\n", mn);
  fprintf(fp, "     Mean: %21.13e\n", sum / n);
  for (int c = 0; c < count; c++) fprintf(fp, "%9d: %21.13e\n", c * inc, U[c * inc]);
  fclose(fp);
  return 0;
}

TDyErrorCode TDyMPFAOSNESFunction(TDy tdy, const double *U, double *R) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!U || !R) return set_error(TDY_ERR_ARG_NULL, "null array");
  return device_eval_host(tdy, FORM_SNES, 0.0, U, nullptr, 0.0, R, nullptr);
}
TDyErrorCode TDyMPFAOSNESJacobian(TDy tdy, const double *U, double *J) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!U || !J) return set_error(TDY_ERR_ARG_NULL, "null array");
  return device_eval_host(tdy, FORM_SNES, 0.0, U, nullptr, 0.0, nullptr, J);
}
TDyErrorCode TDyMPFAOSNESFunctionJacobian(TDy tdy, const double *U, double *R, double *J) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!U || (!R && !J)) return set_error(TDY_ERR_ARG_NULL, "null array");
  return device_eval_host(tdy, FORM_SNES, 0.0, U, nullptr, 0.0, R, J);
}
TDyErrorCode TDyMPFAOIFunction(TDy tdy, double t, const double *U, const double *U_t, double *R) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!U || !U_t || !R) return set_error(TDY_ERR_ARG_NULL, "null array");
  return device_eval_host(tdy, FORM_TS, t, U, U_t, 0.0, R, nullptr);
}
TDyErrorCode TDyMPFAOIJacobian(TDy tdy, double t, const double *U, const double *U_t, double shift, double *J) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!U || !U_t || !J) return set_error(TDY_ERR_ARG_NULL, "null array");
  return device_eval_host(tdy, FORM_TS, t, U, U_t, shift, nullptr, J);
}
TDyErrorCode TDyNewtonOptionsDefault(TDyNewtonOptions *o) {
  if (!o) return set_error(TDY_ERR_ARG_NULL, "TDyNewtonOptionsDefault: null");
  o->rtol = 1e-8;
  o->atol = 0.0;
  o->max_it = 50;
  o->linear_fp32 = 1;
  o->linear_rtol = 1e-6;
  o->linear_max_it = 400;
  o->stol = 1e-8;
  o->precond = TDY_PRECOND_LINES;
  o->cluster_threshold = 0.05;
  o->schedule = TDY_SCHEDULE_AUTO;
  o->fp32_max_it = 8;
  o->spmv_threads = 0;
  return 0;
}
TDyErrorCode TDySetActiveInstances(TDy tdy, int ninstances, const int *active) {
  TDY_CHECK_HANDLE(tdy);
  if (!active) {
    tdy->inst_active.clear();
    return 0;
  }
  if (ninstances != (int)tdy->mesh_blocks.size())
    return set_error(TDY_ERR_ARG_OUTOFRANGE, "TDySetActiveInstances: %d flags for %d instances", ninstances,
                     (int)tdy->mesh_blocks.size());
  tdy->inst_active.assign(active, active + ninstances);
  return 0;
}
TDyErrorCode TDyGetInstanceStatus(TDy tdy, int ninstances, int *status) {
  TDY_CHECK_HANDLE(tdy);
  if (!status) return set_error(TDY_ERR_ARG_NULL, "TDyGetInstanceStatus: null");
  if (ninstances != (int)tdy->mesh_blocks.size())
    return set_error(TDY_ERR_ARG_OUTOFRANGE, "TDyGetInstanceStatus: %d entries for %d instances", ninstances,
                     (int)tdy->mesh_blocks.size());
  if ((int)tdy->inst_status.size() != ninstances)
    return set_error(TDY_ERR_USER, "TDyGetInstanceStatus: no device Newton step yet");
  std::copy(tdy->inst_status.begin(), tdy->inst_status.end(), status);
  return 0;
}
TDyErrorCode TDyGetNumInstances(TDy tdy, int *n) {
  TDY_CHECK_HANDLE(tdy);
  if (!n) return set_error(TDY_ERR_ARG_NULL, "TDyGetNumInstances: null");
  *n = (int)tdy->mesh_blocks.size();
  return 0;
}
TDyErrorCode TDyBackwardEulerStepDevice(TDy tdy, double dt, double *dU, const TDyNewtonOptions *opt,
                                        TDyNewtonStats *stats, int *inst_iterations, double *inst_rel_residual,
                                        void *stream) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!dU) return set_error(TDY_ERR_ARG_NULL, "TDyBackwardEulerStepDevice: null dU");
  if (!(dt > 0.0)) return set_error(TDY_ERR_ARG_OUTOFRANGE, "TDyBackwardEulerStepDevice: dt must be > 0");
  TDyNewtonOptions o;
  TDyNewtonOptionsDefault(&o);
  if (opt) o = *opt;
  if (o.max_it < 0 || o.linear_max_it < 1 || !(o.rtol >= 0.0) || !(o.linear_rtol > 0.0) ||
      (o.precond != TDY_PRECOND_LINES && o.precond != TDY_PRECOND_CLUSTERS) ||
      (o.precond == TDY_PRECOND_CLUSTERS && !(o.cluster_threshold > 0.0)) ||
      (o.schedule != TDY_SCHEDULE_AUTO && o.schedule != TDY_SCHEDULE_TILE && o.schedule != TDY_SCHEDULE_BLOCK) ||
      (o.spmv_threads != 0 && o.spmv_threads != 1 && o.spmv_threads != 2 && o.spmv_threads != 4 &&
       o.spmv_threads != 8))
    return set_error(TDY_ERR_ARG_OUTOFRANGE, "TDyBackwardEulerStepDevice: invalid options");
  return device_be_solve(tdy, dt, dU, o, stats, inst_iterations, inst_rel_residual, stream);
}

TDyErrorCode TDyMPFAOTransientVariable(TDy tdy, const double *U, double *C) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!U || !C) return set_error(TDY_ERR_ARG_NULL, "null array");
  return device_transient_variable_host(tdy, U, C, nullptr);
}
TDyErrorCode TDyMPFAOTransientVariableDerivative(TDy tdy, const double *U, double *dC) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!U || !dC) return set_error(TDY_ERR_ARG_NULL, "null array");
  return device_transient_variable_host(tdy, U, nullptr, dC);
}
TDyErrorCode TDyMPFAOIFunctionTransientVariable(TDy tdy, double t, const double *U, const double *M_t, double *R) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!U || !M_t || !R) return set_error(TDY_ERR_ARG_NULL, "null array");
  return device_eval_host(tdy, FORM_TV, t, U, M_t, 0.0, R, nullptr);
}
TDyErrorCode TDyMPFAOIJacobianTransientVariable(TDy tdy, double t, const double *U, double shift, double *J) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!U || !J) return set_error(TDY_ERR_ARG_NULL, "null array");
  // the diagonal term does not depend on M_t; pass U as a placeholder rate
  return device_eval_host(tdy, FORM_TV, t, U, U, shift, nullptr, J);
}
TDyErrorCode TDyMPFAOIFunctionDAE(TDy tdy, double t, const double *U, const double *U_t, double *R) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!U || !U_t || !R) return set_error(TDY_ERR_ARG_NULL, "null array");
  return device_eval_dae_host(tdy, t, U, U_t, R);
}

TDyErrorCode TDyMPFAOIFunctionIJacobian(TDy tdy, double t, const double *U, const double *U_t, double shift, double *R,
                                        double *J) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!U || !U_t || (!R && !J)) return set_error(TDY_ERR_ARG_NULL, "null array");
  return device_eval_host(tdy, FORM_TS, t, U, U_t, shift, R, J);
}

TDyErrorCode TDyMPFAOSNESFunctionJacobianDevice(TDy tdy, const double *dU, double *dR, double *dJ, void *stream) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!dU || (!dR && !dJ)) return set_error(TDY_ERR_ARG_NULL, "null array");
  return device_eval(tdy, FORM_SNES, 0.0, dU, nullptr, 0.0, dR, dJ, stream);
}
TDyErrorCode TDyMPFAOSNESFunctionJacobianDeviceInstances(TDy tdy, const double *dU, double *dR, double *dJ,
                                                         int ninst, const int *instances, void *stream) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!dU || (!dR && !dJ) || (ninst > 0 && !instances)) return set_error(TDY_ERR_ARG_NULL, "null array");
  const int nblk = (int)tdy->mesh_blocks.size();
  for (int k = 0; k < ninst; k++)
    if (instances[k] < 0 || instances[k] >= nblk)
      return set_error(TDY_ERR_ARG_OUTOFRANGE, "instance %d out of range [0, %d)", instances[k], nblk);
  return device_eval_instances(tdy, dU, dR, dJ, instances, ninst, stream);
}
TDyErrorCode TDyMPFAOIFunctionIJacobianDevice(TDy tdy, double t, const double *dU, const double *dU_t, double shift,
                                              double *dR, double *dJ, void *stream) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!dU || !dU_t || (!dR && !dJ)) return set_error(TDY_ERR_ARG_NULL, "null array");
  return device_eval(tdy, FORM_TS, t, dU, dU_t, shift, dR, dJ, stream);
}
TDyErrorCode TDyMPFAOSNESFunctionJacobianDeviceNoAlloc(TDy tdy, const double *dU, double *dR, double *dJ,
                                                       void *stream) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!dU || (!dR && !dJ)) return set_error(TDY_ERR_ARG_NULL, "null array");
  return device_eval_noalloc(tdy, dU, dR, dJ, stream);
}
TDyErrorCode TDyPreSolveSNESSolverDevice(TDy tdy, const double *dU_prev, void *stream) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!dU_prev) return set_error(TDY_ERR_ARG_NULL, "null array");
  if (!(tdy->dtime > 0.0)) return set_error(TDY_ERR_USER, "call TDySetDtimeForSNESSolver first");
  return device_presolve(tdy, dU_prev, stream);
}
TDyErrorCode TDyGetLaunchesPerEvaluation(TDy tdy, int *n) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!n) return set_error(TDY_ERR_ARG_NULL, "null output");
  *n = device_launches_per_eval(tdy);
  return 0;
}
TDyErrorCode TDySynchronize(TDy tdy) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  return device_synchronize(tdy);
}

TDyErrorCode TDyUpdateState(TDy tdy, const double *U, int ncells) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!U) return set_error(TDY_ERR_ARG_NULL, "null array");
  if (ncells != tdy->mesh.nc) return set_error(TDY_ERR_ARG_WRONG, "TDyUpdateState: expected %d cells", tdy->mesh.nc);
  return device_update_state_host(tdy, U);
}
TDyErrorCode TDyGetLiquidSaturation(TDy tdy, double *S) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!S) return set_error(TDY_ERR_ARG_NULL, "null output");
  return device_get_diagnostic(tdy, 0, S);
}
TDyErrorCode TDyGetLiquidMass(TDy tdy, double *mass) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!mass) return set_error(TDY_ERR_ARG_NULL, "null output");
  return device_get_diagnostic(tdy, 1, mass);
}

TDyErrorCode TDySetTimersEnabled(TDy tdy, int on) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  return device_set_timers(tdy, on);
}
TDyErrorCode TDyGetTimers(TDy tdy, int *n, const char **names, double *ms_total, long long *calls) {
  TDY_CHECK_HANDLE(tdy);
  TDY_CHECK_DEVICE(tdy);
  if (!n) return set_error(TDY_ERR_ARG_NULL, "null count");
  return device_get_timers(tdy, n, names, ms_total, calls);
}
TDyErrorCode TDyDeviceFP64Throughput(double *tflops) {
  if (!tflops) return set_error(TDY_ERR_ARG_NULL, "null output");
  return device_fp64_probe(tflops);
}

}  // extern "C"
