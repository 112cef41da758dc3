// mpg_kernels.h -- launch wrappers of the GB300 PIC kernels (host-callable).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpg_device.cuh"

// Plain FP64 particle state: component-major SoA, x[d*cap + p].
struct PlainParts {
  int32_t *cell;
  double *x, *xr, *v;
  double *w;
  int32_t *sp;
  int64_t *id;  // may be null
  int64_t cap;
};

// Mixed particle state: cellsp = species<<24 | cell, b = (b1,b2,b3,vx), v = (vy,vz).
struct MixedParts {
  uint32_t *c;
  float4 *b;
  float2 *v;
  int64_t *id;  // may be null
  int64_t cap;
};

// Uniform Kuhn meshes (unmapped, not periodic): every tet of type k = t % 6
// has the same J^-1, and its face neighbours sit at the same hex offsets
// with the same types and vertex permutations, so the mixed walk reads them
// from this 6-type table instead of per-tet records.  face word per type and
// opposite vertex: (di+1) | (dj+1) << 2 | (dk+1) << 4 | type' << 8 | perm << 16
// (di, dj, dk the neighbour hex's offset; the face is a wall when that hex
// lies outside the grid).
struct KuhnTable {
  float jinv[6][9];
  uint32_t face[6][4];
  int32_t noff[6][4];  // node index of each type's corners minus the hex's first node (i, j, k)
  int nx = 0, ny = 0, nz = 0;
  // ceil(2^40 / d) for d = nz and d = ny nz: exact division of hex indices
  // (< 2^24) by a multiply and a shift, for ny nz <= 2^16
  unsigned long long mz = 0, myz = 0;
};

struct DevMesh {
  int64_t T = 0, N = 0;
  int4 *tets = nullptr;      // T
  int4 *nbrs = nullptr;      // T, reference face order, -1 wall
  double *jinv = nullptr;    // T*9
  double *detj = nullptr;    // T
  double *normals = nullptr; // T*12
  double *grad = nullptr;    // T*12
  double *nodes = nullptr;   // N*3
  uint8_t *bnd = nullptr;    // N
  int8_t *fper = nullptr;    // T*4: periodic face flags (reference face order), null if not periodic
  double xflip = 0.0;        // lo + hi: a periodic crossing maps x to xflip - x (mirror-image x faces)
  double xshift = 0.0;       // > 0 (jittered periodic mesh, translated x faces): x moves by -+xshift
  int64_t nsolve = 0;        // unknowns of the symmetric system; < N on a periodic mesh
  int64_t plane = 0;         // nodes per x plane ((ny+1)(nz+1)); the ghost plane starts at nsolve
  float4 *mrec = nullptr;    // T*3: J^-1 (9 floats) then E (3 floats)
  uint4 *mnbr = nullptr;     // T: neighbour + permutation per face (indexed by opposite vertex)
  float *fill_ratio = nullptr;  // T: vol/vol_max
  // fixed-point charge slots of the mixed form, grouped by node: node i owns
  // slots [n2c_off[i], n2c_off[i+1]), one per (tet, corner) that uses it;
  // c2n[t] holds the slots of tet t's four corners
  int32_t *n2c_off = nullptr;   // N+1
  int4 *c2n = nullptr;          // T
  // uniform Kuhn meshes: the 6-type walk table, and E per tet as (Ex, Ey, Ez, 0)
  // (the E-field pass writes etet4 instead of the records' E)
  int kuhn = 0;
  KuhnTable ktab;
  float4 *etet4 = nullptr;      // T
};

// ---- plain FP64 path ------------------------------------------------------
void launch_plain_deposit(cudaStream_t s, const PlainParts &P, int64_t n, const DevMesh &M, const SpeciesTable &S,
                          int mode, double *rhs);
// rhs += background, Dirichlet rows zeroed; periodic ghost-plane charge folded into the pairs
void launch_rhs_finish(cudaStream_t s, const DevMesh &M, double *rhs, const double *bg);
// periodic meshes: the ghost plane of phi takes the values of the x = lo plane
void launch_periodic_copy(cudaStream_t s, const DevMesh &M, double *phi);
void launch_efield_plain(cudaStream_t s, const DevMesh &M, const double *phi, double *Etet);
void launch_plain_move(cudaStream_t s, const PlainParts &P, int64_t n, const DevMesh &M, const double *Etet,
                       const SpeciesTable &S, double dt, int kill, int max_cross, DevStats *st);
// stable compaction of live particles (cell >= 0) from P into Q; returns via *d_count (device)
void launch_compact_plain(cudaStream_t s, const PlainParts &P, int64_t n, const PlainParts &Q, uint32_t *scratch,
                          int64_t scratch_len, uint32_t *d_count);

// ---- mixed path -----------------------------------------------------------
// The fixed-point charge accumulator holds one slot per (cell, corner), 4T
// entries grouped by node (DevMesh::n2c_off, c2n); node i's quanta are the
// sum of its slot range.
void launch_mixed_deposit(cudaStream_t s, const MixedParts &P, int64_t n, const DevMesh &M, const SpeciesTable &S,
                          unsigned long long *acc);
// rhs from the slots (gathered per node; the slots stay unchanged, the
// caller zeroes them before the next deposit)
void launch_mixed_convert(cudaStream_t s, const DevMesh &M, unsigned long long *acc, double quantum, const double *bg,
                          double *rhs);
// per-node quanta (N) from the slots
void launch_node_quanta(cudaStream_t s, const DevMesh &M, const unsigned long long *acc, long long *out);
// zero (optional): nzero charge slots cleared alongside (by the E kernel
// itself on a uniform Kuhn mesh)
void launch_efield_mixed(cudaStream_t s, const DevMesh &M, const double *phi, unsigned long long *zero = nullptr,
                         int64_t nzero = 0);
// hist (optional, zeroed T entries): the moved live particles per cell are
// added to it, the counts the next cell sort needs (launch_mixed_sort_order
// with have_hist)
void launch_mixed_move(cudaStream_t s, const MixedParts &P, int64_t n, const DevMesh &M, const SpeciesTable &S,
                       float dt, int kill, int max_cross, unsigned long long *acc, DevStats *st,
                       uint32_t *hist = nullptr);
// the move fused with the gather of a cell sort (launch_mixed_sort_order):
// particle i of the result is input particle perm[i] of P, moved, written to
// Q; *d_count is the sorted count, Q's slots [count, n) are marked dead
void launch_mixed_move_sorted(cudaStream_t s, const MixedParts &P, int64_t n, const MixedParts &Q,
                              const uint32_t *perm, const uint32_t *d_count, const DevMesh &M, const SpeciesTable &S,
                              float dt, int kill, int max_cross, unsigned long long *acc, DevStats *st,
                              uint32_t *hist = nullptr);
// Scratch of the stable cell sort: per-cell counts and starts (start holds
// T + 1 entries: the first sorted position of every cell, start[T] = count),
// the permutation (one uint32 per particle slot), the lists of cells with
// medium and long ranges (list_len >= cap / 32 + 1 entries in all) and their
// two counters, the scan scratch.
struct SortWork {
  uint32_t *cnt = nullptr, *start = nullptr, *perm = nullptr, *long_list = nullptr, *long_count = nullptr;
  int64_t list_len = 0;
  uint32_t *scan_scratch = nullptr;
  int64_t scan_len = 0;
  int long_blocks = 1;
};
// Stable counting sort by cell (ParticleList::sort, particle_list.cpp:90-146):
// live particles of P in cell order, inside a cell in their input order, into
// Q; dead particles are dropped; *d_count receives the new count.  The mixed
// form marks the slots [count, n) of Q dead.  Particle slots must number
// fewer than 2^32.
void launch_mixed_sort(cudaStream_t s, const MixedParts &P, int64_t n, const MixedParts &Q, int64_t T,
                       const SortWork &w, uint32_t *d_count);
// the first four passes of launch_mixed_sort (permutation, starts, count;
// Q.c is their scratch) and its last one, the gather.  have_hist: w.cnt
// already holds the live particles per cell of P (counted by the move that
// wrote P), so the counting pass is left out.
void launch_mixed_sort_order(cudaStream_t s, const MixedParts &P, int64_t n, const MixedParts &Q, int64_t T,
                             const SortWork &w, uint32_t *d_count, bool have_hist = false);
void launch_mixed_gather(cudaStream_t s, const MixedParts &P, int64_t n, const MixedParts &Q, const uint32_t *perm,
                         const uint32_t *d_count);
void launch_plain_sort(cudaStream_t s, const PlainParts &P, int64_t n, const PlainParts &Q, int64_t T,
                       const SortWork &w, uint32_t *d_count);
// blocks of the long-range pass (two per SM)
int sort_long_blocks(int device);

// initial guess from the last solutions: phi <- 2 phi - prev (prev2 null) or
// phi <- 3 phi - 3 prev + prev2; the history shifts by one
void launch_extrapolate(cudaStream_t s, int64_t n, double *phi, double *prev, double *prev2);

// ---- fills, conversions ---------------------------------------------------
void launch_fill_uniform(cudaStream_t s, int mixed, const PlainParts &P, const MixedParts &X, int64_t n0, int64_t n,
                         uint64_t seed, int type, double weight, const double drift[3], double vth, const DevMesh &M,
                         int64_t id0);
void launch_fill_ref(cudaStream_t s, const PlainParts &P, int64_t n0, int nppe, int type, double density,
                     const double vel[3], double temp, double mass, const DevMesh &M, int64_t id0);
// row-major (n,3) staging <-> component-major plain arrays
void launch_rows_to_cols(cudaStream_t s, const double *rows, double *cols, int64_t n, int64_t cap);
void launch_cols_to_rows(cudaStream_t s, const double *cols, double *rows, int64_t n, int64_t cap);
void launch_mixed_pack(cudaStream_t s, const float *b, const float *v, MixedParts X, int64_t n);
// the pack with the cell words copied to X.c and checked as launch_mixed_check
// does; with acc (zeroed) also the deposit of launch_mixed_deposit
void launch_mixed_pack_checked(cudaStream_t s, const uint32_t *cs, const float *b, const float *v, MixedParts X,
                               int64_t n, int64_t T, uint32_t weight_mask, unsigned long long *out,
                               const DevMesh &M, const SpeciesTable &S, unsigned long long *acc);
// cs (optional): the cell words as well
void launch_mixed_unpack(cudaStream_t s, const MixedParts X, int64_t n, float *b, float *v, uint32_t *cs = nullptr);
// out[0] = lowest invalid index (caller sets it to all ones), out[1] += live entries
void launch_mixed_check(cudaStream_t s, const uint32_t *cs, int64_t n, int64_t T, uint32_t weight_mask,
                        unsigned long long *out);
// plain -> mixed conversion of a state (b = float(xref), v = float(v))
void launch_plain_to_mixed(cudaStream_t s, const PlainParts &P, int64_t n0, int64_t n, const MixedParts &X);
// mixed -> plain (x = ref_to_phys(cell, b), xref = b, w = species weight)
void launch_mixed_to_plain(cudaStream_t s, const MixedParts &X, int64_t n, const DevMesh &M, const SpeciesTable &S,
                           const PlainParts &P);
// exclusive scan of n uint32 values into out[0..n] (out[n] = total)
void scan_u32(cudaStream_t s, const uint32_t *in, uint32_t *out, int64_t n, uint32_t *scratch, int64_t scratch_len);
int64_t scan_scratch_len(int64_t n);

// ---- solvers (solver.cu) --------------------------------------------------
// Structured diagonal (DIA) form of the symmetric stiffness matrix: on the
// structured tet grid every column of row i is i + off[d] for at most 27
// offsets.  val[d*n + i] holds A(i, i+off[d]) (0 where absent); boundary
// rows are identity rows and are flagged in bnd.
struct DiaMatrix {
  int64_t n = 0;
  int64_t nwrap = 0;  // periodic mesh: neighbour indices are taken modulo nwrap (= n); 0 otherwise
  int ndiag = 0;
  int off[27] = {};
  double *val64 = nullptr;  // ndiag * n
  float *val32 = nullptr;   // ndiag * n; the FP32 inner operator (Jacobi-scaled when dis is set)
  double *dis = nullptr;    // n: D^-1/2 of the symmetric Jacobi scaling of val32, or null
  const uint8_t *bnd = nullptr;
  // Uniform meshes: every interior row holds the same coefficients (to FP32
  // precision), so the FP32 inner operator of the mixed solver can be this
  // stencil and read no matrix at all.  A missing entry of a row next to the
  // boundary multiplies a boundary entry of the inner vectors, which is
  // exactly zero, so the stencil gives the same products there.
  int constant = 0;
  float cst[27] = {};
};

struct CgWork {
  double *r = nullptr, *p0 = nullptr, *p1 = nullptr, *q = nullptr;  // FP64 vectors, n each
  float4 *v4 = nullptr;  // mixed inner vectors {r, p, q, z} per node, two copies (3n allocated; the
                         // multigrid PCG uses 10n floats of it)
  double *partials = nullptr;  // 8 * max_blocks
  int max_blocks = 0;
  // inner stop of the mixed solvers: the FP32 residual reduction also ends
  // once it is below inner_safety^2 * (tol^2 |b|^2 / |r64|^2), the reduction
  // the outer FP64 test needs (0: fixed inner_tol only)
  double inner_safety = 0.5;
  int threads = 512;  // block size of the cooperative solver kernels (256, 512 or 1024)
  int bar_mode = 0;   // grid barrier flavour (0: fence + volatile polling, 1: release/acquire)
  int bar_skip = 0;   // time-out test: block bar_skip - 1 skips its barrier arrivals (0 = none)
  unsigned bar_limit = 0;  // polls before a barrier wait gives up (0 = the default)
  int block_cap = 0;  // > 0: at most this many blocks in the mixed solver's grid
};
// Geometric multigrid preconditioner of the mixed solver (mg.cu, mg_host.cpp):
// device view of the levels.  Level 0 is the fine grid (operator: the solver's
// DiaMatrix; vectors r/e/t inside the solver's work buffer), levels >= 1 hold
// Galerkin 27-point stencils; levels [0, ngrid) are processed by the whole
// grid, the others and the dense coarsest solve by one block.
struct MgLevelDev {
  int64_t n = 0;
  int si = 0, sj = 0, gx = 0, gy = 0, gz = 0;  // strides and nodes per axis (x slowest)
  int px = 0;                                  // periodic in x: gx planes, x indices wrap
  const float *val = nullptr;                  // 27 * n (levels >= 1)
  const float *dinv = nullptr;                 // n
  const uint8_t *bnd = nullptr;                // n
  float *r = nullptr, *e = nullptr, *t = nullptr;
  float *t2 = nullptr;  // levels with two smoothing sweeps: the first residual, then the second iterate
};
constexpr int kMgMaxLevels = 8;
struct MgDev {
  int nlev = 0, ngrid = 0;
  MgLevelDev lev[kMgMaxLevels];
  const int32_t *dense_idx = nullptr;
  const float *dense_inv = nullptr;
  float *dense_r = nullptr;  // the coarsest level's right-hand side over its interior rows (dense_m)
  int dense_m = 0;
  float omega = 0.8f;
  int reliable = 1;  // keep the search direction across refinement sweeps (reliable updates)
  int fuse_update = 1;  // fuse the PCG update with the next pre-smoothing (level 0 up to ~1M rows)
  int nu0 = 2;          // Jacobi sweeps before and after the coarse correction on level 0 (1 or 2)
  int nu1 = 1;          // the same on the other grid-wide levels (1 or 2)
  float dinv0 = 1.f;    // level 0's D^-1 on a uniform mesh (constant stencil)
};
// mixed CG preconditioned by one V(1,1) cycle per iteration, one cooperative
// launch; `max_blocks` from mg_max_blocks
int run_cg_mg(cudaStream_t s, const DiaMatrix &A, const MgDev &mg, const double *b, double *x, double tol,
              double inner_tol, int max_iter, CgWork &w, int max_blocks, DevStats *st);
int mg_max_blocks(int device, int threads);

// plain FP64 CG on CSR (CG_solve.hpp:54-114), one cooperative launch; returns 0 or an MPG_ERR_*
int run_cg64(cudaStream_t s, int device, int64_t n, const int32_t *rowptr, const int32_t *col, const double *val,
             const double *b, double *x, double tol, int max_iter, CgWork &w, DevStats *st);
// plain FP64 CG on the DIA form (same arithmetic, same summation order as CSR)
int run_cg64_dia(cudaStream_t s, const DiaMatrix &A, const double *b, double *x, double tol, int max_iter, CgWork &w,
                 DevStats *st);
// mixed: FP32 CG inside FP64 iterative refinement on the DIA form, one cooperative launch
int run_cg_mixed(cudaStream_t s, const DiaMatrix &A, const double *b, double *x, double tol, double inner_tol,
                 int max_iter, CgWork &w, DevStats *st);
// reference BiCGStab (CG_solve.hpp:115-206), host-driven; returns iterations in *iters
int run_bicgstab(cudaStream_t s, int64_t n, const int32_t *rowptr, const int32_t *col, const double *val,
                 const double *b, double *x, double tol, int max_iter, double *work, double *red_dev,
                 double *red_host, int *iters, double *resid);
int cg_max_blocks(int device, int threads);
// zeroes the grid-barrier counter of st and sets its flavour and time-out
// test fields from w, on stream s, before a cooperative launch
int barrier_setup(cudaStream_t s, DevStats *st, const CgWork &w);
