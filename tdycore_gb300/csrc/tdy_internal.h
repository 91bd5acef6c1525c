// tdy_internal.h -- host-side data model of the GB300 MPFA-O Richards path.
//
// The structs here restate, for z-extruded hexahedral and prismatic meshes,
// the parts of the reference's TDyMesh (include/private/tdymeshimpl.h:35-219)
// and TDyMPFAO (include/private/tdympfaoimpl.h:13-117) that the residual and
// Jacobian evaluation needs.  They are built once on the host by TDySetup and
// uploaded to the device in flat structure-of-arrays form.
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/tdycore_gb300.h"
#include "../../include/tdycore_gb300_setup.h"

namespace tdy {

// Records an error message for the calling thread and returns the code.
int set_error(int code, const char *fmt, ...);

// ---------------------------------------------------------------------------
// Options (reference: src/tdycore.c:260-296 SetDefaultOptions and
// src/fv/mpfao/tdympfao.c:428-444 TDyCreate_MPFAO).
// -tdy_jacobian_arithmetic values (extension; the reference has FP64 only)
enum { JACOBIAN_DOUBLE_FLOAT = 0, JACOBIAN_FP64 = 1 };

struct Options {
  double gravity = 9.8068;
  double porosity = 0.25;
  double permeability = 1.e-12;
  double residual_saturation = 0.15;
  double gardner_n = 0.5;
  double vangenuchten_m = 0.8;
  double vangenuchten_alpha = 1.e-4;
  double mualem_poly_x0 = 0.995;
  double mualem_poly_x1 = 0.99;
  double mualem_poly_x2 = 1.00;
  double mualem_poly_dx = 0.005;
  int rho_type = WATER_DENSITY_CONSTANT;
  int mu_type = WATER_VISCOSITY_CONSTANT;
  int gmatrix_method = MPFAO_GMATRIX_DEFAULT;
  int bc_type = DIRICHLET_BC;
  double Pref = 101325.0;
  double Tref = 25.0;
  bool has_pressure_bc_value = false;
  double pressure_bc_value = 0.0;
  // arithmetic of the Jacobian products w*T at interior hexahedral vertices
  int jacobian_arithmetic = JACOBIAN_DOUBLE_FLOAT;
  // interior hexahedral vertices' Trans built on the device (extension)
  bool setup_on_device = false;
  // regression output (src/tdyregression.c)
  bool regression_testing = false;
  std::string regression_filename;
  int regression_num_cells = 2;
};

// How a per-cell property is specified by the user.
struct ScalarSpec {
  enum Kind { DEFAULT, CONSTANT, FUNCTION } kind = DEFAULT;
  double value = 0.0;
  TDyScalarSpatialFunction func = nullptr;
  std::vector<std::pair<int, double>> overrides;  // per-cell values
};

struct PermSpec {
  enum Kind { DEFAULT, ISO_CONST, DIAG_CONST, TENSOR_CONST, ISO_FUNC, DIAG_FUNC, TENSOR_FUNC } kind = DEFAULT;
  double k[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  void (*func)(int, double *, double *) = nullptr;
  std::vector<std::pair<int, std::vector<double>>> overrides;
};

// ---------------------------------------------------------------------------
// Mesh input: a surface mesh extruded in z.
struct ExtrudedInput {
  bool set = false;
  int nv2 = 0, nc2 = 0, nvpc = 0, nlayers = 0;
  std::vector<double> xy;      // 2*nv2
  std::vector<int> cells2d;    // nvpc*nc2, counter-clockwise
  std::vector<double> z;       // (nlayers+1)*nv2
};

// Unstructured 3-D mesh with the connectivity the MPFA-O setup needs.
struct Mesh {
  int nv = 0, nc = 0, nf = 0, nb = 0;
  std::vector<double> vx;                        // 3*nv vertex coordinates
  std::vector<int> cell_vert_off, cell_verts;    // cell -> vertices
  std::vector<int> cell_face_off, cell_faces;    // cell -> faces
  std::vector<double> cell_cen, cell_vol;        // 3*nc, nc
  std::vector<int> face_vert_off, face_verts;    // face -> vertices (oriented)
  std::vector<int> face_cell0, face_cell1;       // reference encoding (<0 -> boundary -(b+1))
  std::vector<double> face_cen, face_nrm, face_area;
  std::vector<int> face_bnd;                     // boundary index or -1
  std::vector<int> bnd_face;                     // nb -> face id
  std::vector<int> vert_cell_off, vert_cells;    // vertex -> cells (ascending)
  std::vector<int> vert_face_off, vert_faces;    // vertex -> faces (internal first, ascending)
};

// Builds the z-extruded mesh: connectivity, geometry and face orientation.
int build_extruded_mesh(const ExtrudedInput &in, Mesh &m);
// Disjoint union of block meshes: vertices, cells, faces and boundary faces
// numbered block by block (block b's entities follow those of blocks < b).
void merge_meshes(const std::vector<Mesh> &parts, Mesh &m);

// ---------------------------------------------------------------------------
// Cell material and characteristic-curve parameters (SoA).
struct Materials {
  std::vector<double> K0;          // 9*nc
  std::vector<double> porosity;    // nc
  std::vector<double> Sr;          // nc
  std::vector<int> sat_type;       // nc
  std::vector<double> sat_param;   // 3*nc
  std::vector<int> relperm_type;   // nc
  std::vector<double> relperm_param;  // 9*nc
  std::vector<double> source_sink; // nc
  std::vector<double> lam_sat;     // nc: kr(Se = 1) / mu
  double vis = 0.0;                // water viscosity (pressure independent)
};

// Per-boundary-face condition data.
struct Boundary {
  std::vector<int> type;           // nb
  std::vector<int> has_value;      // nb
  std::vector<double> value;       // nb
  std::vector<double> rho, vis;    // nb (EOS at Pref)
};

// Result of the MPFA-O setup (host copy; also the layout uploaded to HBM).
struct MPFAOSetup {
  int nrows = 0, ncols = 0;
  long long ntrans = 0;
  std::vector<int> v_row_off, v_col_off, v_nint;  // nv+1, nv+1, nv
  std::vector<long long> v_trans_off;             // nv+1
  std::vector<int> row_face;                      // nrows
  std::vector<int> row_lup, row_ldn;              // nrows: local internal-cell index or -1
  std::vector<int> col_ext;                       // ncols
  std::vector<double> trans;                      // ntrans
  std::vector<double> gravdis;                    // nf
  // Jacobian pattern
  std::vector<int> rowptr, colidx;
  // Canonical interior hexahedral vertices: 8 cells, 12 internal faces, no
  // boundary column, cells indexed by octant (bit0 x, bit1 y, bit2 z relative
  // to the vertex) and rows in the fixed order of kCanonUp/kCanonDn, with the
  // face's first cell on the lower side.  Stored structure-of-arrays with
  // stride nCpad so consecutive threads read consecutive vertices.
  int nC = 0, nCpad = 0;
  std::vector<int> canon_vertex;   // nC
  std::vector<double> Tc;          // 96 * nCpad, entry (row*8 + col)
  std::vector<int> cellc;          // 8 * nCpad
  std::vector<int> facec;          // 12 * nCpad
  std::vector<int> gen_vertex;     // other vertices with cells (generic path)
  // Scratch: canonical partials, J_v as [octant][nCpad][8] then R_v as
  // [octant][nCpad],
  // then generic per-vertex blocks J_v[nint][nint], R_v[nint].
  std::vector<long long> v_jv_off; // nv: generic block offset, or canonical column index
  long long scratch_size = 0;
  // cell -> (vertex) gather program
  std::vector<int> cv_off;         // nc+1
  std::vector<long long> cv_jbase; // offset of J_v[a][0] in scratch
  std::vector<long long> cv_rbase; // offset of R_v[a]
  std::vector<int> cv_stride;      // distance between J_v[a][b] and J_v[a][b+1]
  std::vector<int> cv_nint;        // columns of the vertex
  std::vector<int> cv_local;       // a: local index of the cell at the vertex
  std::vector<int> cv_slot_off;    // offset into cv_slots for this (cell, vertex)
  std::vector<uint8_t> cv_slots;   // CSR slot (within the row) of each vertex column
  // Structured interior cells: all 8 vertices canonical, 27-entry row in
  // (dz, dy, dx) order, vertices in corner order (see kCornerOffset).  Their
  // gather needs only the 8 canonical vertex indices (SoA, stride nSpad).
  int nS = 0, nSpad = 0;
  std::vector<int> sc_cells;       // nS
  std::vector<int> sc_vc;          // 8 * nSpad
  std::vector<int> gc_cells;       // the other cells
  int max_nint = 0, max_nrow = 0, max_ncol = 0, max_row_nnz = 0;
  // -tdy_mpfao_setup_on_device: other vertices whose Trans the device builds
  // (one warp each) and the largest of their systems
  std::vector<int> dev_gen_vertex;
  int dev_gen_max_cells = 0, dev_gen_max_faces = 0, dev_gen_max_unk = 0, dev_gen_max_col = 0;
};

// Device-built Trans of other vertices: the limits of one warp's system
// (cells, faces, shared-memory bytes: per cell 12 doubles and 3 ints, per
// face 3 ints, A nunk x nunk and B nunk x ncol doubles).
constexpr int kDevGenMaxCells = 48;
constexpr int kDevGenMaxFaces = 96;
constexpr size_t kDevGenMaxSmem = 48 * 1024;
inline size_t dev_gen_smem_bytes(int ncell, int nface, int nunk, int ncol) {
  return 8 * ((size_t)12 * ncell + (size_t)nunk * nunk + (size_t)nunk * ncol) + 4 * ((size_t)3 * ncell + 3 * nface);
}

int mpfao_setup(const Options &opt, const Mesh &m, const Materials &mat, const Boundary &bnd, MPFAOSetup &s);
// Octant of each local cell and canonical row of each vertex row of a vertex
// with 8 cells and 12 flux rows; false when it does not fit the layout.
bool canonical_layout(const Mesh &m, int v, const int *cells, const int *lup, const int *ldn,
                      std::array<int, 8> &oc, std::array<int, 12> &cr);

// Canonical interior-hex row order: row r joins octants kCanonUp[r] (lower
// side, the face's first cell) and kCanonDn[r] = kCanonUp[r] | (1 << (r / 4)).
constexpr int kCanonUp[12] = {0, 2, 4, 6, 0, 1, 4, 5, 0, 1, 2, 3};
constexpr int kCanonDn[12] = {1, 3, 5, 7, 2, 3, 6, 7, 4, 5, 6, 7};

// Hexahedron corner j (bottom face counter-clockwise, then top face) at
// offset (x, y, z) in {0,1}^3 from the cell's lowest corner; the cell lies in
// octant struct_octant(j) of that vertex, and octant b of that vertex holds
// the neighbour whose slot in a 27-entry (dz, dy, dx)-ordered row is
// struct_slot(j, b).
constexpr int kCornerOffset[8] = {0, 1, 3, 2, 4, 5, 7, 6};  // bit0 x, bit1 y, bit2 z
inline constexpr int struct_octant(int j) { return 7 ^ kCornerOffset[j]; }
inline constexpr int struct_slot(int j, int b) {
  return ((((kCornerOffset[j] >> 2) & 1) - 1 + ((b >> 2) & 1)) + 1) * 9 +
         ((((kCornerOffset[j] >> 1) & 1) - 1 + ((b >> 1) & 1)) + 1) * 3 + (((kCornerOffset[j] & 1) - 1 + (b & 1)) + 1);
}

// EOS at one pressure (src/materials/tdyeos.c:5-136).
void eos_density(int type, double p, double *rho, double *drho, double *d2rho);
void eos_viscosity(int type, double p, double *vis, double *dvis, double *d2vis);
// Mualem cubic smoothing coefficients (tdycharacteristiccurves.c:577-596).
int mualem_smoothing_coeffs(double m, double x0, double x1, double x2, double dx, double coeffs[4]);

struct DeviceState;  // defined in the CUDA translation unit
struct SolverState;  // tdy_solver.cu

}  // namespace tdy

// ---------------------------------------------------------------------------
// The handle.
struct _p_TDy {
  unsigned flags = 0;
  int mode = RICHARDS;
  int discretization = MPFA_O;
  tdy::Options opt;
  // one extruded block (TDySetBoxMesh, TDySetExtrudedMesh) or several
  // independent ones (TDySetExtrudedMeshes: a batch of instances)
  std::vector<tdy::ExtrudedInput> mesh_blocks;
  tdy::ScalarSpec porosity, sr;
  tdy::PermSpec perm;
  std::vector<std::pair<int, std::vector<double>>> vg_over, gardner_over;
  std::vector<std::pair<int, double>> mualem_over, irmay_over;
  std::vector<std::pair<int, double>> source_over;
  TDyScalarSpatialFunction bc_pressure_func = nullptr;
  TDyScalarSpatialIntegerFunction bc_type_func = nullptr;

  // built by TDySetup
  bool is_setup = false;
  tdy::Mesh mesh;
  tdy::Materials mat;
  tdy::Boundary bnd;
  tdy::MPFAOSetup setup;
  double dtime = 0.0;
  bool have_prev = false;
  std::vector<double> U_prev;
  tdy::DeviceState *dev = nullptr;
  tdy::SolverState *solver = nullptr;  // device Newton solver, on first use
  std::vector<int> inst_active;        // instances the device Newton advances (empty: all)
  std::vector<int> inst_status;        // outcome per instance of the last device Newton step
  bool trans_on_host = false;          // device-built Trans copied into setup.trans
};

enum : unsigned {
  TDY_FLAG_MODE = 1u << 1,
  TDY_FLAG_DISC = 1u << 2,
  TDY_FLAG_OPTIONS = 1u << 3,
  TDY_FLAG_SETUP = 1u << 4,
};
