/*
 * oracle.h -- CPU restatement of MiniPIC's electrostatic PIC step.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code.  It is used by tests/, by __graft_entry__.smoke() and by
 * the cpu_baseline / --impl reference legs of bench.py, always as the checker
 * or the CPU baseline, never as the thing measured or shipped.
 *
 * Parity status: PARTIALLY PINNED.  The reference ships no tests, fixtures or
 * golden vectors.  Its random-number generator (random.hpp) compiles
 * standalone and is pinned against golden vectors produced by the
 * reference's own code (oracle/ref_golden.cpp, built by oracle/Makefile into
 * oracle/_ref/; fixtures in tests/golden/ref_random.json): the LCG sequence,
 * drand(), and the per-particle seed and x_ref rejection of the reference
 * fill.  Everything that needs Kokkos / Trilinos / MPI (mesh generator,
 * assembly, solver, push, walk) cannot be built here and is "parity
 * unpinned": it restates the reference's operation order (file:line cited per
 * function in oracle.cpp) and is checked against the reference's own assert()
 * invariants and against closed-form answers.
 *
 * All arrays are caller-owned, row-major, double precision unless noted.
 */
#ifndef MINIPIC_ORACLE_H_
#define MINIPIC_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_mesh orc_mesh;

/* split: 5 = reference five-tet alternating-parity split (mesh.cpp:195-224)
 *        6 = six-tet Kuhn split along the (0,0,0)-(1,1,1) diagonal
 * mapping: 0..3 = reference node mappings (mesh.cpp:763-792)
 *          4    = interior-node jitter, uniform +-jitter*h per component   */
typedef struct {
  int nx, ny, nz;
  int split;
  double lo, hi;
  int mapping;
  double jitter;
  uint64_t seed;
  int periodic; /* periodic in x (mesh.cpp:61-76,178-189,369-392) */
} orc_mesh_desc;

orc_mesh *orc_mesh_create(const orc_mesh_desc *d, char *err, int errlen);
void orc_mesh_destroy(orc_mesh *m);
void orc_mesh_sizes(const orc_mesh *m, int64_t *T, int64_t *N, int64_t *n_faces,
                    int64_t *n_boundary_faces, int64_t *n_boundary_nodes);
/* any pointer may be NULL */
void orc_mesh_export(const orc_mesh *m, double *nodes, int32_t *tets, int32_t *nbrs,
                     double *jinv, double *detj, double *normals, double *grad,
                     uint8_t *boundary);
/* elem_face_periodic T*4 and node_pairs N (mesh.cpp:178-189,369-392) */
void orc_mesh_export_periodic(const orc_mesh *m, int8_t *face_periodic, int32_t *node_pairs);

/* CSR of the P1 stiffness matrix.  mode 0 = reference assembly (Dirichlet
 * rows are identity rows, interior rows keep boundary columns, ES.cpp:83-213);
 * mode 1 = symmetric form (boundary columns dropped from interior rows). */
int64_t orc_assemble(orc_mesh *m, int mode);
/* rows of the assembled system: N, or N minus the ghost plane for mode 1 on a periodic mesh */
int64_t orc_csr_rows(const orc_mesh *m);
void orc_csr_export(const orc_mesh *m, int32_t *rowptr, int32_t *col, double *val);
/* y = A x with the assembled matrix */
void orc_spmv(const orc_mesh *m, const double *x, double *y, int nthreads);

/* background term: bg[i] = -rho_bg * sum_{e ∋ i} vol_e/4 (0 on boundary) */
void orc_background(const orc_mesh *m, double rho_bg, double *bg);

/* ---- particles (plain FP64 state) --------------------------------------- */
/* deposit mode 0 = reference equal quarters via cubature (PIC.cpp:120-137),
 *              1 = linear barycentric scatter.
 * rhs is zeroed, filled, bg added (if non-NULL), Dirichlet rows zeroed. */
void orc_deposit(const orc_mesh *m, int mode, int64_t n, const int32_t *cell,
                 const double *xref, const double *w, const int32_t *sp,
                 const double *q_of_species, const double *bg, double *rhs,
                 int nthreads);

/* fixed-point deposit of the mixed form: acc[node] += quanta (int64),
 * b = barycentric (float, 3 per particle), cellsp = species<<24 | cell,
 * dead particles have cellsp == 0xFFFFFFFF. */
void orc_deposit_fixed(const orc_mesh *m, int64_t n, const uint32_t *cellsp,
                       const float *b, const int64_t *qfix_of_species,
                       int64_t *acc);

/* BiCGStab exactly as CG_solve.hpp:115-206 (x := 0 first).
 * Returns the iteration index at exit; *resid = sqrt(r.r/rho0). */
int orc_bicgstab(const orc_mesh *m, const double *rhs, double *x, double tol,
                 int max_iter, double *resid, int nthreads);
/* CG as CG_solve.hpp:54-114 (warm start from x). */
int orc_cg(const orc_mesh *m, const double *rhs, double *x, double tol,
           int max_iter, double *resid, int nthreads);

/* E per tet: E[t][d] = sum_i phi[n_i] * G_i[d] */
void orc_efield_tet(const orc_mesh *m, const double *phi, double *E_tet, int nthreads);
/* gather: mode 0 = reference 48-term loop (PIC.cpp:162-184),
 *         1 = per-tet E copied to the particle. */
void orc_gather(const orc_mesh *m, int mode, int64_t n, const int32_t *cell,
                const double *xref, const double *phi, const double *E_tet,
                double *E, int nthreads);

/* Boris push (particle_move.hpp:364-392) with B = 0, then v_ref = J^-1 v. */
void orc_push(const orc_mesh *m, int64_t n, const int32_t *cell, const double *E,
              double *v, double *vref, const int32_t *sp, const double *qm,
              double dt, int nthreads);

/* Tet walk (particle_move.hpp:72-124,135-225).  Killed particles get
 * cell = -1.  Returns number of particles that hit max_cross; *n_killed and
 * *n_cross receive counts. */
int64_t orc_walk(const orc_mesh *m, int64_t n, int32_t *cell, double *x,
                 double *xref, double *v, double *vref, double dt, int kill,
                 int max_cross, int64_t *n_killed, int64_t *n_cross, int nthreads);

/* compaction of dead particles (cell < 0).
 * mode 0 = reference tail fill (particle_list.cpp:148-191, Serial order),
 * mode 1 = stable (order-preserving).  Arrays: cell, x, xref, v (3/part),
 * w, sp, id (any of w/sp/id may be NULL).  Returns the new count. */
int64_t orc_compact(int mode, int64_t n, int32_t *cell, double *x, double *xref,
                    double *v, double *w, int32_t *sp, int64_t *id);

/* ParticleList::sort + compute_start_particles_by_element
 * (particle_list.cpp:90-146) with the order inside an element fixed to the
 * input order (stable sort by element), dead (cell < 0) dropped: perm[k] =
 * input index of sorted position k, start[T+1] = first position of each
 * element (start may be NULL).  Returns the count. */
int64_t orc_sort_by_cell(int64_t n, const int32_t *cell, int64_t T, int64_t *perm, int64_t *start);

double orc_kinetic(int64_t n, const double *v, const double *w, const int32_t *sp,
                   const double *m_of_species, int nthreads);

/* reference fill (particle_fill.hpp:100-164) in Serial order; returns the
 * number written (capacity checked like particle_fill.hpp:61-64: -1 if it
 * would not fit).  Arrays receive cell, x, xref, v, w; sp set to type. */
int64_t orc_fill_ref(const orc_mesh *m, int nppe, int type, double density,
                     const double vel[3], double temp, double mass,
                     int64_t capacity, int32_t *cell, double *x, double *xref,
                     double *v, double *w, int32_t *sp);

/* volume-uniform fill with counter-based draws (seeded). */
void orc_fill_uniform(const orc_mesh *m, int64_t n, uint64_t seed, int type,
                      double weight, const double drift[3], double vth,
                      int32_t *cell, double *x, double *xref, double *v,
                      double *w, int32_t *sp, int nthreads);

/* reference dRandom (random.hpp:43-87): n rand() values and n drand() values
 * from two generators seeded with `seed` */
void orc_ref_lcg(uint64_t seed, int n, uint64_t *rand_out, double *drand_out);

/* counter-based generator used by the fills and the jitter */
uint64_t orc_mix64(uint64_t z);
uint64_t orc_draw(uint64_t base, uint64_t ctr);

/* ---- whole step (PIC.cpp:245-267) ------------------------------------- */
typedef struct {
  int deposit_mode;   /* 0 ref quarters, 1 linear */
  int solver;         /* 0 BiCGStab (ref), 1 CG */
  double tol;
  int max_iter;
  int warm_start;     /* CG only: start from previous phi */
  int gather_mode;    /* 0 ref 48-term, 1 per-tet */
  int kill;           /* 1 absorbing walls, 0 specular */
  int max_cross;
  int compact_mode;   /* 0 tail fill, 1 stable */
  int nthreads;
} orc_step_cfg;

typedef struct {
  double ke;
  int64_t n_alive;
  int64_t n_killed;
  int64_t n_cross;
  int64_t n_walk_limit;
  int solver_iters;
  double solver_resid;
} orc_step_stats;

/* state arrays are updated in place; *n is the particle count.  phi (N)
 * and rhs (N) are work/output arrays; E (3n) scratch. */
int orc_step(orc_mesh *m, const orc_step_cfg *cfg, double dt, int64_t *n,
             int32_t *cell, double *x, double *xref, double *v, double *vref,
             double *w, int32_t *sp, int64_t *id, const double *q_of_species,
             const double *m_of_species, const double *bg, double *phi,
             double *rhs, double *E, orc_step_stats *st);

#ifdef __cplusplus
}
#endif
#endif
