// Host-side case description shared by host_case.cpp and the C ABI.
#pragma once
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace cycas {

constexpr int VOID_CELL_ON_BOUNDARY = -10;   // NS/navier.h:17
constexpr int VOID_CELL_ON_INTERFACE = -20;  // NS/navier.h:18
constexpr int INNER_FACE_BOUNDARY = -10;     // NS/navier.h:19

struct IoError : std::runtime_error { using std::runtime_error::runtime_error; };
struct ParamError : std::runtime_error { using std::runtime_error::runtime_error; };
struct MeshError : std::runtime_error { using std::runtime_error::runtime_error; };

struct Region {   // BdRegion (NS/BasicType.h:247-310): types and initial values
  int type1 = -1, type2 = -1;
  double fixed = 0.0;
  double init[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
};

struct HostCase {
  // options pool defaults (NS/navier.cpp:475-516)
  int steady = 1, max_step = 10000, turb_model = 0, density_model = 0, solve_energy = 0;
  int limiter = 0, restart = 0, noutput = 1, cell_pressure_ref = 0;
  int time_scheme = 1, max_outer = 50;  // TimeScheme, MaxOuterStep
  double dt = 1.0, total_time = 0.0;
  double residual_steady = 1.e-6, pressure_reference = 1.01325e5;
  double urf[8] = {0.6, 0.6, 0.6, 0.5, 0.8, 0.8, 0.8, 0.8};
  double gravity[3] = {0, 0, 0};
  std::string gridfile;
  std::string backup_path;  // res.sav read when restart is "yes" (beside param.in)
  std::map<int, Region> regions;

  int ncel = 0, nfac = 0, nbnd = 0, nvrt = 0;
  std::vector<double> vert;
  std::vector<int32_t> cell_vertices, cell_rid, cell_nface, cell_face, cell_cell;
  std::vector<int32_t> bnd_vertices, bnd_rid, bnd_face, bnd_type;
  std::vector<int32_t> face_cell1, face_cell2, face_bnd, face_vertices;

  // InitFlowField state
  std::vector<double> U, V, W, R, T, P, VisLam, VisTur, TE, ED;
  std::vector<double> BU, BV, BW, BRo, BTem, BTE, BED;
};

void load_params(HostCase& hc, const std::string& path);
void load_gmsh(HostCase& hc, const std::string& path, bool binary);
void build_faces(HostCase& hc);
void init_fields(HostCase& hc);
void load_case(HostCase& hc, const std::string& paramPath, bool msh_binary = false);

// ---------------------------------------------------------------- batches (union_mesh.cpp)
// Independent cases concatenated into one mesh.  Cells, boundaries and vertices are appended
// case by case; faces are renumbered so that the boundary faces of all cases come first (in
// case order) followed by all interior faces (in case order).  Each case keeps the reference's
// own numbering properties: boundary b is face b, and the faces of every cell keep their
// relative order.
struct UnionMesh {
  HostCase h;                            // topology + InitFlowField arrays of the union
  std::vector<int> cell0, bnd0, iface0;  // iface0: first interior face of each case (union index)
};
// Every case fills its own slices of the union on the host's threads.  Throws MeshError for the
// first case (in case order) that does not number its boundary faces first.
UnionMesh build_union(const std::vector<const HostCase*>& hs);

// ---------------------------------------------------------------- result files (result_io.cpp)
// The cell fields one case writes, each [ncel] on the host (TE and ED only read with k-epsilon).
struct CellFieldsView {
  long ncel = 0;
  int turb = 0;
  int density = 0;         // DensityModel: 1 writes the Mach number in the Ma column
  double pref = 1.01325e5; // PressureReference
  const double *P = nullptr, *U = nullptr, *V = nullptr, *W = nullptr, *R = nullptr, *T = nullptr;
  const double *VisLam = nullptr, *VisTur = nullptr, *TE = nullptr, *ED = nullptr;
};

std::string tecplot_text(const double* vert, long nvrt, const int32_t* cell_vertices, const CellFieldsView& f);
std::string grid_text(const HostCase& hc);
std::string geo_bytes(const HostCase& hc);
std::string data_bytes(const CellFieldsView& f);
std::string backup_text(const CellFieldsView& f);
// parses a backup file into out[0..10) = R U V W P T VisLam VisTur TE ED (each [ncel]; the last
// three only with k-epsilon)
void read_backup(const std::string& path, long ncel, int turb, double* const out[10]);
void write_file(const std::string& path, const std::string& bytes);

}  // namespace cycas
