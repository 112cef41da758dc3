/*
 * minipic_gb300.h -- C ABI of the GB300-native electrostatic PIC step.
 *
 * One mpg_ctx owns one CUDA stream on one GPU and the device-resident state
 * of one PIC run: the tet mesh, the particle list, the field (rhs, phi, E)
 * and the solver.  Calls on one ctx are serialised on its stream; separate
 * ctxs are independent.  Every entry point returns an int status (MPG_OK = 0,
 * negative = error class); mpg_last_error() returns the message.  No C++
 * exception crosses this boundary and no entry point takes torch types.
 *
 * Each entry point names the reference interface it replaces (MiniPIC file:line).
 * The reference is C++ only; include/minipic_gb300.hpp mirrors its classes
 * (DataWarehouse, Mesh, ParticleList, ES, PIC, ParticleFill, ParticleMove) on
 * top of these calls.
 */
#ifndef MINIPIC_GB300_H_
#define MINIPIC_GB300_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define MPG_OK 0
#define MPG_ERR_ARG (-1)           /* bad argument or size                              */
#define MPG_ERR_CUDA (-2)          /* a CUDA runtime call failed                        */
#define MPG_ERR_CAPACITY (-3)      /* particle capacity exceeded (particle_fill.hpp:61) */
#define MPG_ERR_WALK_LIMIT (-4)    /* a particle exceeded the face-crossing limit       */
#define MPG_ERR_NAN (-5)           /* non-finite value detected                         */
#define MPG_ERR_NOT_CONVERGED (-6) /* Krylov solve hit max_iter                         */
#define MPG_ERR_STATE (-7)         /* call order (e.g. no mesh yet)                     */
#define MPG_ERR_MESH (-8)          /* mesh generation failed (detJ <= 0, bad split)     */
#define MPG_ERR_TIMEOUT (-9)       /* a bounded device-side wait ran out                */

/* ---- enums ------------------------------------------------------------- */
#define MPG_PLAIN 0               /* FP64 throughout, reference semantics               */
#define MPG_MIXED 1               /* FP32 push/walk, int64 fixed-point deposit, FP32 CG in FP64 refinement */

#define MPG_DEPOSIT_REF_QUARTER 0 /* PIC.cpp:120-137: -w q/4 per node via cubature      */
#define MPG_DEPOSIT_LINEAR 1      /* -w q lambda_i (linear-basis scatter)               */

#define MPG_SOLVER_BICGSTAB 0     /* CG_solve.hpp:115-206 (x := 0, reference default)   */
#define MPG_SOLVER_CG 1           /* CG_solve.hpp:54-114                                 */
#define MPG_SOLVER_CG_MG 2        /* mixed form: CG preconditioned by a geometric        */
                                  /* multigrid V-cycle (not in the reference; grids of   */
                                  /* <= 1500 interior nodes: plain inner CG)             */

#define MPG_SPLIT_REF5 5          /* mesh.cpp:195-224 five-tet alternating split         */
#define MPG_SPLIT_KUHN6 6         /* six Kuhn tets per hex                               */

#define MPG_MAP_NONE 0            /* mesh.cpp:763-792 mappings 0..3                      */
#define MPG_MAP_JITTER 4          /* interior nodes jittered by U(-j,j)*h per component  */

#define MPG_FIELD_RHS 0
#define MPG_FIELD_PHI 1
#define MPG_FIELD_E_TET 2         /* T*3, constant per tet                               */
#define MPG_FIELD_BACKGROUND 3

typedef struct mpg_ctx mpg_ctx;

/* replaces the brick.txt read of Mesh::Mesh (mesh.cpp:85-89): nx ny nz mapping */
typedef struct {
  int nx, ny, nz;
  int split;       /* MPG_SPLIT_REF5 or MPG_SPLIT_KUHN6 */
  double lo, hi;   /* box [lo,hi]^3; the reference uses [-1,1] */
  int mapping;     /* MPG_MAP_* */
  double jitter;   /* fraction of h, MPG_MAP_JITTER only */
  uint64_t seed;   /* jitter seed */
  int periodic;    /* 1: periodic in x (Mesh::Mesh(..., periodic), mesh.cpp:61-76,178-189);
                      the x = hi plane nodes off the y/z walls are ghosts of the x = lo plane,
                      nx >= 2 (even for MPG_SPLIT_REF5, mesh.cpp:91-94) */
} mpg_mesh_desc;

typedef struct {
  int precision;         /* MPG_PLAIN / MPG_MIXED */
  int deposit;           /* MPG_DEPOSIT_*; the mixed form always deposits linearly */
  int solver;            /* MPG_SOLVER_*; the mixed form always uses refined CG */
  double tol;            /* relative residual |b-Ax|/|b| (PIC.cpp:251 uses 1e-6) */
  int max_iter;          /* CG_solve.hpp:144 uses 1000 */
  int warm_start;        /* CG initial guess: 0 zero, 1 the previous phi, 2 2*phi[n-1] - phi[n-2],
                            3 3*phi[n-1] - 3*phi[n-2] + phi[n-3] */
  int kill_on_wall;      /* DataWarehouse::set_kill_particles_on_wall_impact */
  int max_crossings;     /* face crossings per particle per step before MPG_ERR_WALK_LIMIT */
  int sort_interval;     /* cell sort every k steps, 0 = never (ParticleList::sort) */
  double rho_background; /* uniform background charge density (0 = none) */
  int track_ids;         /* keep a 64-bit id per particle (parity checks) */
} mpg_config;

typedef struct {
  double ke;             /* PIC.cpp:255-264 "Total KE" after the move */
  int64_t n_alive;
  int64_t n_killed;      /* removed at absorbing walls this step */
  int64_t n_crossings;   /* face crossings this step */
  int64_t n_walk_limit;  /* particles stopped by max_crossings */
  int solver_iters;
  double solver_resid;   /* relative residual at exit */
  int status;
  int steps;
  /* device time per phase (ms), summed over the steps of the call;
   * filled when mpg_set_timing(ctx, 1) */
  double ms_deposit, ms_solve, ms_efield, ms_move, ms_sort;
  int64_t n_launches;    /* kernels this library launched during the call */
} mpg_step_stats;

int mpg_version(void);
int mpg_device_count(int *n);

/* DataWarehouse::DataWarehouse (data_warehouse.cpp:46-48) */
int mpg_ctx_create(int device, mpg_ctx **out);
int mpg_ctx_destroy(mpg_ctx *ctx);
/* copies the last error message of ctx (or of the last failed create) */
int mpg_last_error(mpg_ctx *ctx, char *buf, int len);
int mpg_set_timing(mpg_ctx *ctx, int on);
/* device timer on the ctx stream (replaces the Kokkos::Impl::Timer pairs of
 * PIC.cpp:250-259): op 0 records the start event, op 1 records the stop
 * event, waits for it and returns the elapsed milliseconds in *ms. */
int mpg_timer(mpg_ctx *ctx, int op, double *ms);

/* DataWarehouse::create_mesh -> Mesh::Mesh (data_warehouse.cpp:50-54, mesh.cpp:78-714) */
int mpg_mesh_build(mpg_ctx *ctx, const mpg_mesh_desc *desc);
int mpg_mesh_sizes(mpg_ctx *ctx, int64_t *n_tets, int64_t *n_nodes, int64_t *n_boundary_nodes);
/* Mesh public arrays (mesh.hpp:109-154): nodes N*3, elem_to_node T*4,
 * elem_face_to_elem T*4 (-1 = wall, faces (0,1,3),(1,2,3),(0,3,2),(0,2,1)),
 * inverse_jacobian T*9, determinate_jacobian T, normals T*12, boundary N.
 * Host buffers; NULL skips an array. */
int mpg_mesh_download(mpg_ctx *ctx, double *nodes, int32_t *tets, int32_t *nbrs, double *jinv, double *detj,
                      double *normals, uint8_t *boundary);
/* Periodic meshes: Mesh::elem_face_periodic T*4 (+1 on both sides of an x = lo/hi
 * face, 0 elsewhere; mesh.cpp:369-392) and Mesh::node_pairs N (the x = lo node a
 * ghost node stands for, -1 otherwise; mesh.cpp:178-189).  NULL skips an array;
 * both are all zero / all -1 on a non-periodic mesh. */
int mpg_mesh_periodic_download(mpg_ctx *ctx, int8_t *face_periodic, int32_t *node_pairs);

/* ParticleTypeList::add_particle_type (particle_type.hpp:58-84); defaults
 * 0: e- (-1,1), 1: e+ (1,1), 2: H+ (1,1837); at most 16 species. */
int mpg_species_set(mpg_ctx *ctx, int index, double q, double m);

/* DataWarehouse::create_ES -> ES::ES (ES.cpp:47-213) plus the step options. */
int mpg_configure(mpg_ctx *ctx, const mpg_config *cfg);
/* CSR of the assembled stiffness matrix (Tpetra CrsMatrix of ES.cpp:114) */
int mpg_csr_sizes(mpg_ctx *ctx, int64_t *n_rows, int64_t *nnz);
int mpg_csr_download(mpg_ctx *ctx, int32_t *rowptr, int32_t *col, double *val);

/* DataWarehouse::create_particle_list -> ParticleList::ParticleList (particle_list.cpp:44-68) */
int mpg_particles_reserve(mpg_ctx *ctx, int64_t capacity);
/* ParticleFill (particle_fill.hpp:59-164): nppe particles per tet, seeded per (elem, i, type) */
int mpg_fill_ref(mpg_ctx *ctx, int nppe, int type, double density, const double vel[3], double temp);
/* n particles uniform in volume from a seed, Maxwellian velocities of per-component
 * sigma vth around drift; weight per particle given */
int mpg_fill_uniform(mpg_ctx *ctx, int64_t n, uint64_t seed, int type, double weight, const double drift[3],
                     double vth);
/* ParticleList accessors x/x_ref/v/ielement/weight/type (particle_list.hpp:68-91):
 * host arrays, (n,3) row-major for vectors; id may be NULL (ids = index). */
int mpg_particles_upload(mpg_ctx *ctx, int64_t n, const int32_t *cell, const double *x, const double *xref,
                         const double *v, const double *w, const int32_t *species, const int64_t *id);
int mpg_particles_download(mpg_ctx *ctx, int64_t cap, int64_t *n, int32_t *cell, double *x, double *xref, double *v,
                           double *w, int32_t *species, int64_t *id);
/* ParticleList::num_particles (particle_list.hpp:165) */
int mpg_particles_count(mpg_ctx *ctx, int64_t *n);
/* raw mixed-form state: cellsp = species<<24 | cell (0xFFFFFFFF = dead),
 * b = barycentric (3 floats), v (3 floats) */
int mpg_mixed_download(mpg_ctx *ctx, int64_t cap, int64_t *n, uint32_t *cellsp, float *b, float *v);
int mpg_mixed_upload(mpg_ctx *ctx, int64_t n, const uint32_t *cellsp, const float *b, const float *v);
/* fixed-point charge accumulator of the mixed form (N int64) and its quantum */
int mpg_charge_download(mpg_ctx *ctx, int64_t *acc, double *quantum, int64_t *qfix_of_species);

/* ---- the step and its phases (PIC.cpp:245-267) ------------------------- */
int mpg_weight_charge(mpg_ctx *ctx);                            /* PIC::weight_charge, PIC.cpp:139-160 */
int mpg_solve(mpg_ctx *ctx, int *iters, double *resid);         /* ES::solve, ES.cpp:216-231           */
int mpg_weight_efield(mpg_ctx *ctx);                            /* PIC::weight_Efield, PIC.cpp:186-189 */
int mpg_move(mpg_ctx *ctx, double dt, mpg_step_stats *st);      /* ParticleMove::move, particle_move.hpp:398-404, plus KE */
int mpg_step(mpg_ctx *ctx, double dt, int n_steps, mpg_step_stats *st); /* PIC::time_step x n_steps */
/* ParticleList::sort (particle_list.cpp:90-116): live particles in cell order;
 * inside a cell the previous list order is kept (a stable sort, the same on
 * every run; the reference's BinSort leaves that order open).  Dead particles
 * are dropped.  The mixed step also sorts every sort_interval steps; the
 * plain step never does (Serial list order, PIC.cpp:51-53). */
int mpg_sort(mpg_ctx *ctx);
/* ParticleList::compute_start_particles_by_element / start_by_element
 * (particle_list.cpp:118-146): start[e] = first list position of cell e's
 * particles, start[T] = count (len >= T + 1).  Valid after mpg_sort until
 * particles move, are added or are replaced (MPG_ERR_STATE otherwise). */
int mpg_cell_starts(mpg_ctx *ctx, int64_t len, int64_t *start);

/* Test of the failure path of the cooperative field solvers (no counterpart
 * in the reference, whose solves run on the host): in the solves of later
 * steps, block skip_block of the solver's grid does not arrive at its grid
 * barriers, and a barrier wait gives up after poll_limit polls (0: the
 * default of ~2^22, about a second).  The solve then ends without hanging:
 * every block leaves the kernel, the step returns MPG_ERR_TIMEOUT and the
 * ctx stays usable.  skip_block < 0 turns the test off. */
int mpg_set_barrier_test(mpg_ctx *ctx, int skip_block, unsigned poll_limit);

/* ES::rhs / ES::phi / set_analytic_RHS-style access (ES.hpp:53-71) */
int mpg_get_field(mpg_ctx *ctx, int which, double *host);
int mpg_set_field(mpg_ctx *ctx, int which, const double *host);

/* Stand-alone CSR solve on caller-owned DEVICE buffers: conjugate gradients
 * on A x = b (A n x n, CSR with int32 indices, FP64), x holds the start
 * vector and receives the result.  Scratch (4 n doubles + reduction slots)
 * is allocated on first use and kept in ctx.  Replaces CG_solve
 * (CG_solve.hpp:54-114) for callers that hold their own matrix. */
int mpg_cg_csr(mpg_ctx *ctx, int64_t n, const int32_t *d_rowptr, const int32_t *d_col, const double *d_val,
               const double *d_b, double *d_x, double tol, int max_iter, int *iters, double *resid);

/* ---- batched ensemble / serving (no counterpart in the reference) --------
 * Many independent runs (each: Kuhn-split unit cube n^3, uniform or with
 * jittered interior nodes, one species, volume-uniform fill, absorbing
 * walls, mixed precision) resident on one GPU
 * and advanced together: one persistent launch per step for all active runs
 * (charge conversion, field solve, E field, fused push/walk/deposit, with
 * grid barriers between them; mpg_batch_set_fused), the step captured in a
 * CUDA graph.  The field operator of a batched run is the 15-point Kuhn
 * stencil of its mesh (constant coefficients on a uniform mesh, per-row
 * coefficients on a jittered one; FP32 inside FP64 refinement), its inner
 * solve multigrid-preconditioned CG with a per-run hierarchy for meshes of
 * 9^3 cells and more, up to 2^20 nodes, and plain CG otherwise.  Runs are
 * admitted against a device-memory budget, step
 * until their requested step count and are retired to free their slot.
 * A run's results do not depend on which other runs share the batch. */
typedef struct mpg_batch mpg_batch;

typedef struct {
  int n_side;            /* mesh: n^3 cubes, 6 Kuhn tets each, unit cube */
  int64_t n_particles;   /* uniform in volume */
  uint64_t seed;         /* fill seed */
  double q, m;           /* species charge and mass */
  double weight;         /* weight per particle */
  double vth;            /* Maxwellian sigma per component */
  double drift[3];
  double rho_background; /* uniform background charge density */
  double dt;
  double tol;            /* relative residual of the field solve */
  int max_iter;
  int steps;             /* the run finishes after this many steps */
  double jitter;         /* interior nodes moved by up to +-jitter h per axis (0: uniform mesh, < 0.5) */
  uint64_t mesh_seed;    /* jitter seed */
} mpg_run_desc;

typedef struct {
  int active;            /* admitted and not finished */
  int finished;
  int steps_done;
  int64_t n_alive;
  double ke;             /* kinetic energy after the last step */
  int solver_iters;      /* of the last step */
  double solver_resid;
  int status;
  int64_t bytes;         /* device memory charged to the run */
} mpg_run_info;

typedef struct {
  int active_runs;       /* runs stepped by the last call */
  int64_t particle_steps;
  double ms;             /* device time of the call */
  double ms_last_step;   /* device time of its last step */
  int64_t n_launches;
  int graph;             /* 1 if the steps ran from a captured CUDA graph */
  int status;
} mpg_batch_stats;

/* max_runs <= 256 resident runs; particle_capacity < 2^32 for all runs together */
int mpg_batch_create(int device, int64_t budget_bytes, int max_runs, int64_t particle_capacity, mpg_batch **out);
int mpg_batch_destroy(mpg_batch *b);
int mpg_batch_last_error(mpg_batch *b, char *buf, int len);
/* block size of the batched solver (256, 512, 1024) and cell-sort interval */
int mpg_batch_set_tuning(mpg_batch *b, int cg_threads, int sort_interval);
/* on (the default): each batch step is one persistent cooperative launch
 * whose phases (charge -> rhs, field solves, E, push/walk/deposit) are
 * separated by grid barriers; off: one launch per phase.  Same results. */
int mpg_batch_set_fused(mpg_batch *b, int on);
/* MPG_ERR_CAPACITY when the budget, the particle capacity or the slots are exhausted */
int mpg_batch_admit(mpg_batch *b, const mpg_run_desc *desc, int *slot);
/* mpg_batch_admit in two parts, so that the host work of an admission can
 * overlap the batch's steps.  mpg_batch_prepare builds the run's mesh, field
 * stencil and tables on the host: it touches no device and no batch, so any
 * host thread may call it while another thread steps the batch.
 * mpg_batch_admit_prepared uploads a prepared run into a free slot and fills
 * its particles (between steps, on the thread that steps the batch); the prep
 * stays the caller's (it may be admitted again, e.g. into another batch) until
 * mpg_run_prep_destroy.  Same results as mpg_batch_admit. */
typedef struct mpg_run_prep mpg_run_prep;
int mpg_batch_prepare(const mpg_run_desc *desc, mpg_run_prep **out);
int mpg_batch_admit_prepared(mpg_batch *b, const mpg_run_prep *prep, int *slot);
int mpg_run_prep_destroy(mpg_run_prep *prep);
int mpg_batch_step(mpg_batch *b, int n_steps, mpg_batch_stats *st);
int mpg_batch_run_info(mpg_batch *b, int slot, mpg_run_info *info);
int mpg_batch_run_phi(mpg_batch *b, int slot, double *phi);
/* raw particle state of a run (local cell, barycentrics, velocity), any order */
int mpg_batch_run_particles(mpg_batch *b, int slot, int64_t cap, int64_t *n, uint32_t *cell, float *b3, float *v3);
int mpg_batch_retire(mpg_batch *b, int slot);

/* Multigrid hierarchy of MPG_SOLVER_CG_MG for a mesh, built on the host
 * only (no device; a check of the preconditioner's set-up).  *nlev = number
 * of levels; for `level`: extent[3] = node extents (x-planes on a periodic
 * mesh, x slowest) and, where the pointers are non-null, its 27-point FP32
 * stencil val27[d * n + row] (levels >= 1; d = 9 (dx+1) + 3 (dy+1) + (dz+1)),
 * D^-1 dinv[n] and Dirichlet flags bnd[n], n = extent product.  dense_max:
 * interior unknowns allowed on the coarsest level (0: the default).
 * MPG_ERR_ARG when the grid cannot be coarsened. */
int mpg_mg_hierarchy(const mpg_mesh_desc *mesh, int64_t dense_max, int level, int *nlev, int *extent, float *val27,
                     float *dinv, uint8_t *bnd);

/* Allocation-free variant of mpg_cg_csr.  No counterpart in the reference.
 *
 * For callers that cannot allocate device memory at the point of the call:
 * code that hands all device memory to its own pool or to another framework,
 * real-time loops that must not pay an allocation, or a host that only lends
 * out device pointers.  The call allocates nothing (no cudaMalloc, no
 * cudaFree, no allocating library routine) and needs no mpg_ctx: its scratch
 * (the CG vectors r, p, p', q, the per-block partial sums and the barrier
 * counters, 4 n doubles plus ~256 KB) is one file-scope static device array
 * of the library, sized for n <= MPG_NOALLOC_MAX_N rows (about 4.3 MB, held
 * on every GPU that loads the library until the process exits).  Larger n is
 * rejected with MPG_ERR_CAPACITY before anything runs.
 *
 * Same arguments and result as mpg_cg_csr, plus the stream to run on
 * (a cudaStream_t passed as void*, NULL = the default stream); the caller
 * owns and passes the CSR matrix, b and x (device pointers).  Every call looks
 * up the array's device address in the current context (so a context reset
 * between calls is harmless); the first call on a device also queries the
 * solver's co-residency limit for that device (the device current at the
 * call).  Make that first call before any stream capture.  All calls share the one array:
 * calls that overlap on the GPU (on different streams or host threads) race
 * and give wrong results; serialise them.  The array keeps the last call's
 * contents; the call clears the counters it needs at its start.  Status
 * only (it has no ctx to hold a message): MPG_ERR_CAPACITY n too large,
 * MPG_ERR_ARG bad argument, MPG_ERR_CUDA, MPG_ERR_TIMEOUT,
 * MPG_ERR_NOT_CONVERGED. */
#define MPG_NOALLOC_MAX_N 131072
int mpg_cg_csr_noalloc(void *stream, int64_t n, const int32_t *d_rowptr, const int32_t *d_col, const double *d_val,
                       const double *d_b, double *d_x, double tol, int max_iter, int *iters, double *resid);

#ifdef __cplusplus
}
#endif
#endif
