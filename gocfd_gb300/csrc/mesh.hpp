// Host-side mesh topology for the DFR solver (set-up time); the geometry is
// built on the device from it (gcfd_geometry.cu).
//
// Reference behaviour followed (gocfd):
//   DG2D/triangulation.go:19-171   edge creation per element (edges v0v1, v1v2, v2v0),
//                                  first connected triangle = "left", orientation flag
//   types/elemental.go:12-46       EdgeKey = min | max<<32, GetVertices(rev)
//   DG2D/element_utils.go:163-175  CalculateElementLocalGeometry (x,y of points)
//   types/cfd.go:11-26             BCFLAG numbering
#pragma once
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "dfr_element.hpp"

namespace gcfd {

enum BCFlag : int {
  BC_None = 0,
  BC_In = 1,
  BC_Dirichlet = 2,
  BC_Slip = 3,
  BC_Far = 4,
  BC_Wall = 5,
  BC_Cyl = 6,
  BC_Neuman = 7,
  BC_Out = 8,
  BC_IVortex = 9,
  BC_Periodic = 10,
  BC_PeriodicReversed = 11,
};

struct Topology {
  int K = 0, Nv = 0, nEdges = 0;
  std::vector<uint64_t> key;            // packed vertex pair
  std::vector<uint64_t> keyR;           // the right side's own edge (differs from key on periodic pairs)
  std::vector<int> kL, eL, kR, eR;      // kR = eR = -1 on boundary edges
  std::vector<uint8_t> revL, revR;      // traversal direction flag per connection
  std::vector<int> bc;                  // BCFlag per edge
  std::vector<int> elemEdge;            // K*3: edge index of (k, local edge)
};

// Builds the edge table.  Returns an empty string on success, else a message.
// Boundary flags are BCFLAGs; periodic ones (10, 11) carry a group number in
// bits 8 and up (one group per periodic tag), and each group's edges are
// paired into shared edges (pair_periodic).
std::string build_topology(int Nv, int K, const int32_t* etov, int nbc, const int32_t* bc_v1,
                           const int32_t* bc_v2, const int32_t* bc_flag, Topology* topo);

std::string pair_periodic(const std::vector<std::pair<int, std::vector<int>>>& groups, Topology* t);

// Physical coordinates of the reference point (r, s) of element k
// (CalculateElementLocalGeometry, element_utils.go:163-175).
inline void element_point(const int32_t* etov, const double* vx, const double* vy, int k, double r, double s,
                          double* x, double* y) {
  const int va = etov[3 * k], vb = etov[3 * k + 1], vc = etov[3 * k + 2];
  const double a = -(r + s), b = r + 1.0, c = s + 1.0;
  *x = 0.5 * (a * vx[va] + b * vx[vb] + c * vx[vc]);
  *y = 0.5 * (a * vy[va] + b * vy[vb] + c * vy[vc]);
}

// A mesh file's vertices, triangles (0-based) and boundary edges with their
// BCFLAG, as the reference's readers produce them.
struct MeshFile {
  std::vector<double> vx, vy;
  std::vector<int32_t> etov;  // K x 3
  std::vector<int32_t> bc_v1, bc_v2, bc_flag;  // periodic flags carry their tag's group in bits 8..
  std::vector<std::string> periodicTags;       // group -> tag
};

// BC tag -> BCFLAG as types.BCNameMap (types/cfd.go:28-73): the part of the tag
// before a '-' selects the flag; -1 for an unknown name.
int bc_flag_of_tag(const std::string& tag);

// Gambit neutral (readfiles/readGambitGrid.go:21-165,223-363) or SU2
// (readfiles/readSU2Grid.go:27-177) 2D triangle mesh, chosen by the file
// extension as getFileTypeFromExtension (DG2D/dfr_startup.go:184-204).
// Returns an empty string on success, else the error.
std::string read_mesh_file(const std::string& path, MeshFile* out);

}  // namespace gcfd
