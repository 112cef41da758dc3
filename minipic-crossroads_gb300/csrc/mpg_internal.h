// mpg_internal.h -- shared declarations of the GB300 PIC library (not installed).
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "minipic_gb300.h"

// ---------------------------------------------------------------------------
// Host mesh (built once per run; mesh.cpp:78-714 is the reference).
struct HostMesh {
  mpg_mesh_desc d{};
  int64_t T = 0, N = 0, n_bnodes = 0;
  std::vector<double> nodes;    // N*3
  std::vector<int32_t> tets;    // T*4
  std::vector<int32_t> nbrs;    // T*4, reference face order (0,1,3),(1,2,3),(0,3,2),(0,2,1); -1 wall
  std::vector<uint32_t> nbr_opp;  // T*4, face opposite local node k: (perm << 24) | nbr, nbr 0xFFFFFF = wall
  std::vector<double> jinv;     // T*9 row-major J^-1
  std::vector<double> detj;     // T
  std::vector<double> normals;  // T*12
  std::vector<double> grad;     // T*12, grad N_i (x,y,z) per local node
  std::vector<uint8_t> bnd;     // N
  std::vector<int8_t> fper;     // T*4, reference face order: +1 on both sides of an x = lo/hi face (periodic)
  std::vector<int32_t> pair;    // N: the x = lo node a periodic ghost node stands for, -1 otherwise
  int64_t nsolve = 0;           // unknowns of the symmetric system (N, or N minus the ghost plane)
};
// a periodic ghost node stands for its pair (ES.cpp:93-95, PIC.cpp:132-134)
static inline int32_t host_pmap(const HostMesh &m, int32_t g) { return m.pair[g] >= 0 ? m.pair[g] : g; }

// Returns 0 or an MPG_ERR_* code with err filled.
int host_mesh_generate(const mpg_mesh_desc &d, HostMesh &m, std::string &err);
// mode 0 = reference (identity Dirichlet rows, boundary columns kept),
// mode 1 = symmetric (boundary columns dropped).
// mode 1 on a periodic mesh assembles the nsolve rows of the x < hi planes (the
// ghost plane is the last plane in node order and is copied after a solve)
void host_csr_assemble(const HostMesh &m, int mode, std::vector<int32_t> &rowptr, std::vector<int32_t> &col,
                       std::vector<double> &val);
void host_background(const HostMesh &m, double rho_bg, std::vector<double> &bg);
// acceptance ratio vol/vol_max per tet for the volume-uniform fill
void host_fill_ratio(const HostMesh &m, std::vector<float> &ratio);
// fixed-point charge slots grouped by node: node i owns [off[i], off[i+1]),
// one slot per (tet, corner) that uses it, in tet order; c2n[4 t + k] is the
// slot of tet t's corner k
void host_charge_slots(const HostMesh &m, std::vector<int32_t> &off, std::vector<int32_t> &c2n);

// Geometric multigrid hierarchy of the structured node grid (mg_host.cpp):
// level 0 is the fine grid (its operator is the solver's own), levels >= 1
// hold Galerkin 27-point stencils [d][n], d = 9 (di+1) + 3 (dj+1) + (dk+1);
// the coarsest level is solved with a dense inverse over its interior nodes.
struct MgHostLevel {
  int gx = 0, gy = 0, gz = 0;   // nodes per axis (x slowest); x-planes on a periodic level
  bool px = false;              // periodic in x (indices wrap, no x walls)
  std::vector<float> val;       // 27 * n, levels >= 1
  std::vector<float> dinv;      // n: 1 / diagonal (1 on Dirichlet rows)
  std::vector<uint8_t> bnd;     // n
};
struct MgHostHierarchy {
  std::vector<MgHostLevel> lev;
  std::vector<int32_t> dense_idx;  // interior rows of the coarsest level
  std::vector<float> dense_inv;    // row-major inverse over them
};
// from the symmetric (mode 1) CSR of the mesh (periodic in x or not); false
// with a reason when the grid cannot be coarsened.  dense_max: interior
// unknowns of the coarsest level (0: the default, or MPG_MG_DENSE_MAX)
bool host_mg_build(const HostMesh &m, const std::vector<int32_t> &rp, const std::vector<int32_t> &col,
                   const std::vector<double> &val, MgHostHierarchy &H, std::string &why, int64_t dense_max = 0);

// The 6-type walk table of a uniform Kuhn mesh (see KuhnTable in
// mpg_kernels.h): jinv[k][9] and face[k][4] from the tets of one interior hex,
// then checked against every tet's J^-1 (as the FP32 walk record holds it)
// and neighbour word.  False when the mesh is not such a mesh or any tet
// differs (the walk then uses the per-tet records).
bool host_kuhn_table(const HostMesh &m, float jinv[6][9], uint32_t face[6][4], int32_t noff[6][4]);

// counter-based generator shared by the jitter and the fills (splitmix64 finaliser)
static inline uint64_t mpg_mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static const uint64_t MPG_SALT_JITTER = 0x6A09E667F3BCC908ULL;
static const uint64_t MPG_SALT_FILL = 0xBB67AE8584CAA73BULL;
