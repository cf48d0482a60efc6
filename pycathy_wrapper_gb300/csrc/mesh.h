// Host-side mesh and sparsity construction for one CATHY domain.
//
// Produces the same mesh as the reference's TRIANGOLI (triangoli.f:1-159),
// TPNODI2D, RIORD, AREA2D (area2d.f), GEN3D (gen3d.f:28-77) and, for the
// matrix pattern, the same nonzero set as STRPIC/STRNEW (strpic.f,
// strnew.f) -- but stored as one full 0-based CSR with sorted columns, which
// is what every device kernel uses.  On top of the pattern it derives what
// the GPU needs: node->element incidence (row-owned assembly), diagonal
// slots, IC(0)/ILU(0) level schedules and the vertical column structure of
// the extruded mesh.
#pragma once
#include <cstdint>
#include <vector>

#include "../../include/cathy_gb300.h"

namespace cathy {

struct HostMesh {
  int nrow = 0, ncol = 0, nnod = 0, ntri = 0, nstr = 0, n = 0, nt = 0, nzone = 1;
  int iopt = 1;
  std::vector<double> x, y, z;          // n
  std::vector<double> arenod;           // nnod
  std::vector<int32_t> triang;          // 4*ntri (3 nodes 1-based + zone)
  std::vector<int32_t> tetra;           // 5*nt (4 nodes 1-based + zone)
  std::vector<int32_t> tet_layer;       // nt, 1-based layer
  // full CSR (0-based)
  std::vector<int32_t> rowptr, cols, diag;   // n+1, nnz, n
  std::vector<int32_t> down;                 // n: slot of (i, i+nnod) or -1
  std::vector<int32_t> up;                   // n: slot of (i, i-nnod) or -1
  // node -> (element, local index) incidence, packed as elem*4+k
  std::vector<int32_t> inc_ptr, inc;
  // level schedules for lower (forward) and upper (backward) triangular
  // dependencies: rows grouped by level
  std::vector<int32_t> lev_f_ptr, lev_f_rows, lev_b_ptr, lev_b_rows;
  int64_t nnz() const { return (int64_t)cols.size(); }
};

// Build mesh + pattern from a DEM.  Returns false on an invalid mesh (a node
// without elements or a zero-area/zero-volume element).
bool build_mesh(const cathy_dem_t& dem, int iopt, HostMesh& m);

// Vegetation type of each surface node (datin.f:221-233): TRIANGOLI and
// TPNODI2D applied to a per-cell map -- the mean of FACTOR * map over the
// node's triangles -- truncated to an integer.  map == NULL gives 1.
// Returns false when the map is 0 on an active DEM cell (the reference would
// number the nodes of the two triangulations differently).
bool node_map_types(const cathy_dem_t& dem, const double* map, const HostMesh& m,
                    std::vector<int32_t>& out);

// Shared topology helpers (also used by the Fortran drop-ins):
// full CSR from a symmetric upper CSR (1-based TOPOL/JA, diag first).
void upper_to_full(int n, const int32_t* topol, const int32_t* ja,
                   std::vector<int32_t>& rowptr, std::vector<int32_t>& cols,
                   std::vector<int32_t>& up_slot_of_full);
// level schedules for a full CSR pattern
void level_schedule(int n, const std::vector<int32_t>& rowptr,
                    const std::vector<int32_t>& cols, bool lower,
                    std::vector<int32_t>& lev_ptr, std::vector<int32_t>& rows);

}  // namespace cathy
