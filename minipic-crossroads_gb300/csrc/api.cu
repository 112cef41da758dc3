// api.cu -- C ABI of the GB300 PIC library (include/minipic_gb300.h).
//
// One mpg_ctx = one CUDA stream + the device-resident state of one run.  The
// orchestration follows PIC::time_step (PIC.cpp:245-267):
//   plain: deposit -> solve -> E per tet -> push+walk (+KE) -> compaction
//   mixed: [fixed-point charge -> rhs] -> refined CG -> E per tet ->
//          fused push+walk+deposit (+KE); cell sort every sort_interval steps
// No step path copies field or particle data to the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "mpg_internal.h"
#include "mpg_kernels.h"

struct mpg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  bool timing = false;
  cudaEvent_t ev[12] = {};

  bool has_mesh = false;
  HostMesh hm;
  DevMesh dm;

  SpeciesTable sp{};
  bool weight_set[MPG_MAX_SPECIES] = {};
  double quantum = 0.0;
  bool qfix_valid = false;

  bool configured = false;
  mpg_config cfg{};
  int csr_mode = -1;
  int csr_mg = 0;              // the multigrid hierarchy was built with the current CSR
  MgDev mg;                    // multigrid preconditioner of the mixed solver (MPG_SOLVER_CG_MG)
  bool mg_ok = false;
  std::vector<void *> mg_bufs;  // its device arrays
  int mg_max_blocks = 0;
  int64_t nnz = 0;
  int32_t *rowptr = nullptr, *col = nullptr;
  double *val = nullptr;
  float *val32 = nullptr;
  DiaMatrix dia;  // structured diagonal form of the symmetric matrix (CG paths)
  double *rhs = nullptr, *phi = nullptr, *bg = nullptr, *Etet = nullptr;
  double *phi_prev = nullptr;   // previous solution (warm_start 2, 3)
  double *phi_prev2 = nullptr;  // the one before (warm_start 3)
  int phi_hist = 0;             // solutions held in phi / phi_prev / phi_prev2 (0 .. 3)
  unsigned long long *acc = nullptr;  // fixed-point charge, one slot per (cell, corner), grouped by node (4T)
  long long *acc_node = nullptr;      // per-node quanta for downloads (N)
  bool acc_valid = false;
  bool needs_sort = false;  // particles added or replaced since the last cell sort
  // a cell sort's permutation (sort_perm) whose gather is left to the next
  // move, which reads the particles through it into the other buffer; the
  // list in mp[cur] then still has n_presort slots (n may already hold the
  // sorted count)
  bool gather_pending = false;
  int64_t n_presort = 0;
  double inner_tol = 1e-5;  // relative residual target of the mixed solver's FP32 inner CG

  int precision = MPG_PLAIN;  // precision of the allocated particle arrays
  bool parts_alloc = false;
  int64_t cap = 0, n = 0, want_cap = 0;
  int64_t n_live = 0;  // live particles (the mixed form leaves holes until the next sort)
  int cur = 0;
  PlainParts pp[2]{};
  MixedParts mp[2]{};
  int64_t id_next = 0;
  int64_t step_count = 0;

  CgWork cg;
  int64_t cg_n = 0;
  double *bicg_work = nullptr, *red_dev = nullptr, *red_host = nullptr;
  uint32_t *sort_cnt = nullptr, *sort_start = nullptr, *scan_scratch = nullptr;
  uint32_t *sort_perm = nullptr, *sort_long = nullptr;  // stable cell sort: permutation (cap), long-range list
  int64_t sort_perm_cap = 0;
  bool starts_valid = false;  // sort_start holds the start offsets of the current particle order
  int64_t scan_len = 0;
  uint32_t *d_count = nullptr, *h_count = nullptr;
  DevStats *d_stats = nullptr, *h_stats = nullptr;

  std::vector<void *> allocs;  // device allocations owned by the ctx
  int64_t launches = 0;        // kernels launched by this ctx (cumulative)
  int64_t csr_rows = 0;        // rows of the assembled CSR
};

static std::string g_last_create_error;

namespace {

int fail(mpg_ctx *c, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  return code;
}

#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) return fail(c, MPG_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));  \
  } while (0)

#define CKL()                                                                                      \
  do {                                                                                             \
    cudaError_t e_ = cudaGetLastError();                                                           \
    if (e_ != cudaSuccess) return fail(c, MPG_ERR_CUDA, "kernel launch: %s", cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
int dalloc(mpg_ctx *c, T **p, int64_t count) {
  *p = nullptr;
  if (count <= 0) count = 1;
  cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (size_t)count);
  if (e != cudaSuccess) return fail(c, MPG_ERR_CUDA, "cudaMalloc(%lld bytes): %s", (long long)(sizeof(T) * count),
                                    cudaGetErrorString(e));
  c->allocs.push_back(*p);
  return MPG_OK;
}

template <typename T>
void dfree(mpg_ctx *c, T *&p) {
  if (!p) return;
  auto it = std::find(c->allocs.begin(), c->allocs.end(), (void *)p);
  if (it != c->allocs.end()) c->allocs.erase(it);
  cudaFree(p);
  p = nullptr;
}

int check_ctx(mpg_ctx *c) {
  if (!c) return MPG_ERR_ARG;
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return fail(c, MPG_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  return MPG_OK;
}

#define ENTER(c)                 \
  do {                           \
    int rc_ = check_ctx(c);      \
    if (rc_) return rc_;         \
  } while (0)
#define TRY(x)                   \
  do {                           \
    int rc_ = (x);               \
    if (rc_) return rc_;         \
  } while (0)

void default_species(SpeciesTable &s) {
  // particle_type.hpp:65-74
  for (int i = 0; i < MPG_MAX_SPECIES; ++i) {
    s.q[i] = -1;
    s.m[i] = 1;
  }
  s.q[0] = -1, s.m[0] = 1;
  s.q[1] = 1, s.m[1] = 1;
  s.q[2] = 1, s.m[2] = 1837;
  for (int i = 0; i < MPG_MAX_SPECIES; ++i) {
    s.qm[i] = s.q[i] / s.m[i];
    s.qm_f[i] = (float)s.qm[i];
    s.w[i] = 0.0;
    s.qfix[i] = 0;
    s.half_wm_f[i] = 0.f;
  }
}

// scratch of the block scans (compaction over particles, sort over cells)
int ensure_scan_scratch(mpg_ctx *c) {
  const int64_t want = scan_scratch_len(std::max<int64_t>(std::max<int64_t>(c->cap, c->hm.T + 1), 1)) + 4;
  if (c->scan_scratch && c->scan_len >= want) return MPG_OK;
  dfree(c, c->scan_scratch);
  TRY(dalloc(c, &c->scan_scratch, want));
  c->scan_len = want;
  return MPG_OK;
}

void free_particles(mpg_ctx *c) {
  dfree(c, c->sort_perm);
  dfree(c, c->sort_long);
  c->sort_perm_cap = 0;
  c->starts_valid = false;
  for (int k = 0; k < 2; ++k) {
    dfree(c, c->pp[k].cell);
    dfree(c, c->pp[k].x);
    dfree(c, c->pp[k].xr);
    dfree(c, c->pp[k].v);
    dfree(c, c->pp[k].w);
    dfree(c, c->pp[k].sp);
    dfree(c, c->pp[k].id);
    dfree(c, c->mp[k].c);
    dfree(c, c->mp[k].b);
    dfree(c, c->mp[k].v);
    dfree(c, c->mp[k].id);
    c->pp[k] = PlainParts{};
    c->mp[k] = MixedParts{};
  }
  c->parts_alloc = false;
  c->cap = 0;
  c->n = 0;
}

int alloc_particles(mpg_ctx *c, int64_t cap) {
  free_particles(c);
  c->precision = c->cfg.precision;
  const bool ids = c->cfg.track_ids != 0;
  for (int k = 0; k < 2; ++k) {
    if (c->precision == MPG_PLAIN) {
      PlainParts &P = c->pp[k];
      TRY(dalloc(c, &P.cell, cap));
      TRY(dalloc(c, &P.x, 3 * cap));
      TRY(dalloc(c, &P.xr, 3 * cap));
      TRY(dalloc(c, &P.v, 3 * cap));
      TRY(dalloc(c, &P.w, cap));
      TRY(dalloc(c, &P.sp, cap));
      if (ids) TRY(dalloc(c, &P.id, cap));
      P.cap = cap;
    } else {
      MixedParts &X = c->mp[k];
      TRY(dalloc(c, &X.c, cap));
      TRY(dalloc(c, &X.b, cap));
      TRY(dalloc(c, &X.v, cap));
      if (ids) TRY(dalloc(c, &X.id, cap));
      X.cap = cap;
    }
  }
  c->cap = cap;
  c->n = 0;
  c->n_live = 0;
  c->cur = 0;
  c->parts_alloc = true;
  TRY(ensure_scan_scratch(c));
  c->acc_valid = false;
  return MPG_OK;
}

int ensure_particles(mpg_ctx *c) {
  if (!c->has_mesh) return fail(c, MPG_ERR_STATE, "no mesh: call mpg_mesh_build first");
  if (!c->configured) return fail(c, MPG_ERR_STATE, "not configured: call mpg_configure first");
  if (c->parts_alloc && c->precision == c->cfg.precision && c->cap >= c->want_cap) return MPG_OK;
  if (c->want_cap <= 0) return fail(c, MPG_ERR_STATE, "no particle capacity: call mpg_particles_reserve");
  return alloc_particles(c, c->want_cap);
}

// temporary plain buffers (stream-ordered allocations)
struct TempPlain {
  PlainParts P{};
  std::vector<void *> ptrs;
};
int temp_plain(mpg_ctx *c, int64_t n, bool ids, TempPlain &t) {
  auto get = [&](void **p, size_t bytes) -> int {
    cudaError_t e = cudaMallocAsync(p, bytes ? bytes : 8, c->stream);
    if (e != cudaSuccess) return fail(c, MPG_ERR_CUDA, "cudaMallocAsync: %s", cudaGetErrorString(e));
    t.ptrs.push_back(*p);
    return MPG_OK;
  };
  const int64_t m = n > 0 ? n : 1;
  TRY(get((void **)&t.P.cell, sizeof(int32_t) * m));
  TRY(get((void **)&t.P.x, sizeof(double) * 3 * m));
  TRY(get((void **)&t.P.xr, sizeof(double) * 3 * m));
  TRY(get((void **)&t.P.v, sizeof(double) * 3 * m));
  TRY(get((void **)&t.P.w, sizeof(double) * m));
  TRY(get((void **)&t.P.sp, sizeof(int32_t) * m));
  if (ids) TRY(get((void **)&t.P.id, sizeof(int64_t) * m));
  t.P.cap = m;
  return MPG_OK;
}
void temp_free(mpg_ctx *c, TempPlain &t) {
  for (void *p : t.ptrs) cudaFreeAsync(p, c->stream);
  t.ptrs.clear();
}

void upload_species_derived(mpg_ctx *c) {
  for (int i = 0; i < MPG_MAX_SPECIES; ++i) {
    c->sp.qm[i] = c->sp.q[i] / c->sp.m[i];
    c->sp.qm_f[i] = (float)c->sp.qm[i];
    c->sp.half_wm_f[i] = (float)(0.5 * c->sp.w[i] * c->sp.m[i]);
  }
}

// fixed-point quantum: the largest |w q| over species maps to 2^25 quanta
// (finer than the 24-bit barycentrics it multiplies; a warp's run of 32
// particles then sums to < 2^30 and is aggregated in int32)
void ensure_qfix(mpg_ctx *c) {
  if (c->qfix_valid) return;
  double mx = 0.0;
  for (int i = 0; i < MPG_MAX_SPECIES; ++i)
    if (c->weight_set[i]) mx = std::max(mx, fabs(c->sp.w[i] * c->sp.q[i]));
  c->quantum = mx > 0 ? mx / 33554432.0 : 1.0;
  for (int i = 0; i < MPG_MAX_SPECIES; ++i)
    c->sp.qfix[i] = c->weight_set[i] ? llround(c->sp.w[i] * c->sp.q[i] / c->quantum) : 0;
  c->qfix_valid = true;
}

int set_species_weight(mpg_ctx *c, int s, double w) {
  if (c->weight_set[s] && c->sp.w[s] != w) {
    if (c->cfg.precision == MPG_MIXED)
      return fail(c, MPG_ERR_ARG, "mixed form carries one weight per species (species %d: %g vs %g)", s, c->sp.w[s], w);
  }
  if (!c->weight_set[s] || c->sp.w[s] != w) {
    c->sp.w[s] = w;
    c->weight_set[s] = true;
    c->qfix_valid = false;
    c->acc_valid = false;
    upload_species_derived(c);
  }
  return MPG_OK;
}

int ensure_cg_work(mpg_ctx *c, int64_t n) {
  if (c->cg_n >= n && c->cg.r) return MPG_OK;
  dfree(c, c->cg.r);
  dfree(c, c->cg.p0);
  dfree(c, c->cg.p1);
  dfree(c, c->cg.q);
  dfree(c, c->cg.v4);
  dfree(c, c->cg.partials);
  // solver launch shape: tunable through MPG_CG_THREADS / MPG_CG_BARRIER
  if (const char *e = getenv("MPG_CG_THREADS")) c->cg.threads = atoi(e);
  if (const char *e = getenv("MPG_CG_BARRIER")) c->cg.bar_mode = atoi(e);
  if (const char *e = getenv("MPG_CG_BLOCKS")) c->cg.block_cap = atoi(e);
  if (const char *e = getenv("MPG_CG_INNER_TOL")) c->inner_tol = atof(e);
  if (const char *e = getenv("MPG_CG_INNER_SAFETY")) c->cg.inner_safety = atof(e);
  c->cg.max_blocks = cg_max_blocks(c->device, c->cg.threads == 256 || c->cg.threads == 1024 ? c->cg.threads : 512);
  c->mg_max_blocks = mg_max_blocks(c->device, c->cg.threads == 256 || c->cg.threads == 1024 ? c->cg.threads : 512);
  TRY(dalloc(c, &c->cg.r, n));
  TRY(dalloc(c, &c->cg.p0, n));
  TRY(dalloc(c, &c->cg.p1, n));
  TRY(dalloc(c, &c->cg.q, n));
  TRY(dalloc(c, &c->cg.v4, 3 * n));  // 8n floats for the mixed CG, 10n for the multigrid PCG
  if (c->cg.max_blocks < 1) return fail(c, MPG_ERR_CUDA, "solver kernels cannot be resident (occupancy 0)");
  TRY(dalloc(c, &c->cg.partials, 8 * (int64_t)std::max(c->cg.max_blocks, c->mg_max_blocks)));
  c->cg_n = n;
  return MPG_OK;
}

// device statistics to the host (no status check)
int fetch_stats(mpg_ctx *c) {
  CK(cudaMemcpyAsync(c->h_stats, c->d_stats, sizeof(DevStats), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return MPG_OK;
}

int sync_stats(mpg_ctx *c) {
  TRY(fetch_stats(c));
  if (c->h_stats->bar_error) return fail(c, MPG_ERR_TIMEOUT, "solver grid barrier timed out");
  return MPG_OK;
}

int zero_stats(mpg_ctx *c) {
  CK(cudaMemsetAsync(c->d_stats, 0, sizeof(DevStats), c->stream));
  return MPG_OK;
}

void ev_record(mpg_ctx *c, int i) {
  if (c->timing) cudaEventRecord(c->ev[i], c->stream);
}
double ev_ms(mpg_ctx *c, int a, int b) {
  float ms = 0.f;
  if (c->timing && cudaEventElapsedTime(&ms, c->ev[a], c->ev[b]) == cudaSuccess) return ms;
  return 0.0;
}

// ---- phases ---------------------------------------------------------------
int phase_deposit_plain(mpg_ctx *c) {
  CK(cudaMemsetAsync(c->rhs, 0, sizeof(double) * c->dm.N, c->stream));
  launch_plain_deposit(c->stream, c->pp[c->cur], c->n, c->dm, c->sp, c->cfg.deposit, c->rhs);
  launch_rhs_finish(c->stream, c->dm, c->rhs, c->bg);
  c->launches += 2;
  CKL();
  return MPG_OK;
}

int settle_sort(mpg_ctx *c);
int phase_deposit_mixed(mpg_ctx *c) {
  if (!c->acc_valid) {
    // the deposit does not depend on the order: with a gather pending it
    // reads the unsorted list (its dead slots deposit nothing)
    ensure_qfix(c);
    CK(cudaMemsetAsync(c->acc, 0, sizeof(unsigned long long) * 4 * c->dm.T, c->stream));
    launch_mixed_deposit(c->stream, c->mp[c->cur], c->gather_pending ? c->n_presort : c->n, c->dm, c->sp, c->acc);
    c->acc_valid = true;
    c->launches += 1;
  }
  launch_mixed_convert(c->stream, c->dm, c->acc, c->quantum, c->bg, c->rhs);
  c->launches += 1;
  CKL();
  return MPG_OK;
}

// Initial guess of the CG solves: zero (warm_start 0), the previous phi (1),
// the linear extrapolation 2 phi_{n-1} - phi_{n-2} of the last two solutions
// (2), or the quadratic one 3 phi_{n-1} - 3 phi_{n-2} + phi_{n-3} (3); the
// extrapolations use the lower orders until enough solutions exist.
int initial_guess(mpg_ctx *c, int64_t N) {
  const int ws = c->cfg.warm_start;
  if (ws != 2 && ws != 3) {
    // the history buffers are not kept up to date in these modes
    c->phi_hist = 0;
    if (!ws) CK(cudaMemsetAsync(c->phi, 0, sizeof(double) * N, c->stream));
    return MPG_OK;
  }
  if (!c->phi_prev) {
    TRY(dalloc(c, &c->phi_prev, N));
    c->phi_hist = c->phi_hist > 1 ? 1 : c->phi_hist;
  }
  if (ws == 3 && !c->phi_prev2) {
    TRY(dalloc(c, &c->phi_prev2, N));
    c->phi_hist = c->phi_hist > 2 ? 2 : c->phi_hist;
  }
  const int order = std::min(c->phi_hist, ws) - 1;  // 0: copy only, 1: linear, 2: quadratic
  if (order >= 1) {
    launch_extrapolate(c->stream, N, c->phi, c->phi_prev, order == 2 ? c->phi_prev2 : nullptr);
    c->launches += 1;
  } else if (c->phi_hist == 1) {
    CK(cudaMemcpyAsync(c->phi_prev, c->phi, sizeof(double) * N, cudaMemcpyDeviceToDevice, c->stream));
  }
  return MPG_OK;
}

int phase_solve(mpg_ctx *c) {
  const int64_t N = c->dm.N;
  if (c->cfg.precision == MPG_MIXED || c->cfg.solver != MPG_SOLVER_BICGSTAB) {
    TRY(ensure_cg_work(c, N));
    TRY(initial_guess(c, N));
    int rc;
    if (c->cfg.precision == MPG_MIXED && c->mg_ok)
      rc = run_cg_mg(c->stream, c->dia, c->mg, c->rhs, c->phi, c->cfg.tol, c->inner_tol, c->cfg.max_iter, c->cg,
                     c->mg_max_blocks, c->d_stats);
    else if (c->cfg.precision == MPG_MIXED)
      rc = run_cg_mixed(c->stream, c->dia, c->rhs, c->phi, c->cfg.tol, c->inner_tol, c->cfg.max_iter, c->cg,
                        c->d_stats);
    else
      rc = run_cg64_dia(c->stream, c->dia, c->rhs, c->phi, c->cfg.tol, c->cfg.max_iter, c->cg, c->d_stats);
    c->launches += 1;
    if (rc) return fail(c, rc, "CG launch failed: %s", cudaGetErrorString(cudaGetLastError()));
    if (c->dm.fper) {
      // the symmetric periodic system leaves the ghost plane out
      launch_periodic_copy(c->stream, c->dm, c->phi);
      c->launches += 1;
    }
    if (c->phi_hist < 3) ++c->phi_hist;
    return MPG_OK;
  }
  // reference BiCGStab (host-driven; parity mode)
  if (!c->bicg_work) TRY(dalloc(c, &c->bicg_work, 5 * N));
  int it = 0;
  double res = 0.0;
  int rc = run_bicgstab(c->stream, N, c->rowptr, c->col, c->val, c->rhs, c->phi, c->cfg.tol, c->cfg.max_iter,
                        c->bicg_work, c->red_dev, c->red_host, &it, &res);
  // 2 SpMV + 6 dot pairs + 6 updates per iteration, roughly
  c->launches += 4 + (int64_t)it * 20;
  if (rc == MPG_ERR_CUDA) return fail(c, rc, "BiCGStab: %s", cudaGetErrorString(cudaGetLastError()));
  // the reference system holds phi_ghost = phi_pair only to the solver
  // tolerance; the ghost plane takes the pair values exactly
  launch_periodic_copy(c->stream, c->dm, c->phi);
  // record into the device stats so both solver kinds report the same way
  DevStats tmp;
  CK(cudaMemcpyAsync(&tmp, c->d_stats, sizeof(DevStats), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  tmp.solver_iters = it;
  tmp.iters_total += it;
  tmp.solver_resid = res;
  tmp.solver_status = rc ? 1 : 0;
  if (rc) tmp.solver_fail = 1;
  CK(cudaMemcpyAsync(c->d_stats, &tmp, sizeof(DevStats), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return MPG_OK;
}

// zero_acc (mixed form): the charge slots are cleared alongside, for the
// move's deposit
int phase_efield(mpg_ctx *c, bool zero_acc) {
  if (c->cfg.precision == MPG_MIXED)
    launch_efield_mixed(c->stream, c->dm, c->phi, zero_acc ? c->acc : nullptr, zero_acc ? 4 * c->dm.T : 0);
  else
    launch_efield_plain(c->stream, c->dm, c->phi, c->Etet);
  c->launches += 1;
  CKL();
  return MPG_OK;
}

int compact_plain(mpg_ctx *c) {
  const int other = 1 - c->cur;
  launch_compact_plain(c->stream, c->pp[c->cur], c->n, c->pp[other], c->scan_scratch, c->scan_len, c->d_count);
  c->launches += 3;
  CKL();
  CK(cudaMemcpyAsync(c->h_count, c->d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->cur = other;
  c->n = *c->h_count;
  c->starts_valid = false;
  return MPG_OK;
}

// scratch of the stable cell sort for the current particle capacity
int sort_work(mpg_ctx *c, SortWork &w) {
  if (c->cap >= (int64_t)1 << 32) return fail(c, MPG_ERR_ARG, "the cell sort needs fewer than 2^32 particle slots");
  if (!c->sort_perm || c->sort_perm_cap < c->cap) {
    dfree(c, c->sort_perm);
    dfree(c, c->sort_long);
    TRY(dalloc(c, &c->sort_perm, std::max<int64_t>(c->cap, 1)));
    TRY(dalloc(c, &c->sort_long, c->cap / 32 + 3));
    c->sort_perm_cap = c->cap;
  }
  w.cnt = c->sort_cnt;
  w.start = c->sort_start;
  w.perm = c->sort_perm;
  w.long_count = c->sort_long;
  w.long_list = c->sort_long + 2;
  w.list_len = c->cap / 32 + 1;
  w.scan_scratch = c->scan_scratch;
  w.scan_len = c->scan_len;
  w.long_blocks = sort_long_blocks(c->device);
  return MPG_OK;
}

// Stable cell sort of the mixed form (drops dead particles).  The new count
// is read back at the next host sync; the slots [count, n) of the new buffer
// are dead, so the grid bound n stays valid until then.
int sort_mixed(mpg_ctx *c) {
  TRY(settle_sort(c));
  c->needs_sort = false;
  SortWork w;
  TRY(sort_work(c, w));
  const int other = 1 - c->cur;
  launch_mixed_sort(c->stream, c->mp[c->cur], c->n, c->mp[other], c->dm.T, w, c->d_count);
  c->launches += 10;
  CKL();
  c->cur = other;
  c->starts_valid = true;
  return MPG_OK;
}

// The cell sort of mpg_step: permutation, start offsets and count only; the
// gather is the next move's (launch_mixed_move_sorted), one pass over the
// particle records fewer.  Any other use of the particle list completes the
// gather first (settle_sort).  have_hist: the move that wrote the list
// counted its particles per cell into the sort's counters.
int sort_mixed_deferred(mpg_ctx *c, bool have_hist) {
  TRY(settle_sort(c));
  c->needs_sort = false;
  SortWork w;
  TRY(sort_work(c, w));
  launch_mixed_sort_order(c->stream, c->mp[c->cur], c->n, c->mp[1 - c->cur], c->dm.T, w, c->d_count, have_hist);
  c->launches += 9;
  CKL();
  c->gather_pending = true;
  c->n_presort = c->n;
  c->starts_valid = true;
  return MPG_OK;
}

int settle_sort(mpg_ctx *c) {
  if (!c->gather_pending) return MPG_OK;
  const int other = 1 - c->cur;
  launch_mixed_gather(c->stream, c->mp[c->cur], c->n, c->mp[other], c->sort_perm, c->d_count);
  c->launches += 1;
  CKL();
  c->cur = other;
  c->gather_pending = false;
  return MPG_OK;
}

// Stable cell sort of the plain form (mpg_sort only: the plain step keeps
// the reference's Serial list order, PIC.cpp:51-53)
int sort_plain(mpg_ctx *c) {
  SortWork w;
  TRY(sort_work(c, w));
  const int other = 1 - c->cur;
  launch_plain_sort(c->stream, c->pp[c->cur], c->n, c->pp[other], c->dm.T, w, c->d_count);
  c->launches += 10;
  CKL();
  CK(cudaMemcpyAsync(c->h_count, c->d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->cur = other;
  c->n = *c->h_count;
  c->starts_valid = true;
  return MPG_OK;
}

int finish_counts_mixed(mpg_ctx *c, bool sorted) {
  if (!sorted) return MPG_OK;
  CK(cudaMemcpyAsync(c->h_count, c->d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  c->n = *c->h_count;
  return MPG_OK;
}

int one_step(mpg_ctx *c, double dt, mpg_step_stats *acc_st, bool &sorted) {
  const bool mixed = c->cfg.precision == MPG_MIXED;
  if (mixed && c->cfg.sort_interval > 0 && c->needs_sort) {
    // freshly filled or uploaded particles are in arbitrary cell order: sort
    // before the first step instead of after sort_interval steps (its gather
    // is this step's move)
    TRY(sort_mixed_deferred(c, false));
    sorted = true;
  }
  ev_record(c, 0);
  TRY(mixed ? phase_deposit_mixed(c) : phase_deposit_plain(c));
  ev_record(c, 1);
  TRY(phase_solve(c));
  ev_record(c, 2);
  // the move deposits the new positions' charge into zeroed slots, cleared
  // by the E-field pass (timed with the E-field phase)
  TRY(phase_efield(c, mixed));
  CK(cudaMemsetAsync(&c->d_stats->ke, 0, sizeof(double), c->stream));
  c->starts_valid = false;
  // a step that ends with a cell sort has the move count the particles per
  // cell for it (its deposit runs are the sort's counting pass)
  const bool sort_after =
      mixed && c->cfg.sort_interval > 0 && (c->step_count + 1) % c->cfg.sort_interval == 0;
  uint32_t *hist = nullptr;
  if (sort_after) {
    SortWork w;
    TRY(sort_work(c, w));
    hist = w.cnt;
    CK(cudaMemsetAsync(hist, 0, sizeof(uint32_t) * c->dm.T, c->stream));
  }
  ev_record(c, 3);
  if (mixed && c->gather_pending) {
    // the last step's cell sort: read through its permutation, write sorted
    const int other = 1 - c->cur;
    launch_mixed_move_sorted(c->stream, c->mp[c->cur], c->n, c->mp[other], c->sort_perm, c->d_count, c->dm, c->sp,
                             (float)dt, c->cfg.kill_on_wall, c->cfg.max_crossings, c->acc, c->d_stats, hist);
    c->cur = other;
    c->gather_pending = false;
  } else if (mixed) {
    launch_mixed_move(c->stream, c->mp[c->cur], c->n, c->dm, c->sp, (float)dt, c->cfg.kill_on_wall,
                      c->cfg.max_crossings, c->acc, c->d_stats, hist);
  } else {
    launch_plain_move(c->stream, c->pp[c->cur], c->n, c->dm, c->Etet, c->sp, dt, c->cfg.kill_on_wall,
                      c->cfg.max_crossings, c->d_stats);
  }
  c->launches += 1;
  CKL();
  ev_record(c, 4);
  c->step_count++;
  if (mixed) {
    if (sort_after) {
      TRY(sort_mixed_deferred(c, true));
      sorted = true;
    }
  } else {
    // the plain form compacts whenever particles were removed (particle_list.cpp:148-164),
    // also after a failed solve, so that the list stays consistent
    TRY(fetch_stats(c));
    if (c->h_stats->n_killed > 0) {
      TRY(compact_plain(c));
      CK(cudaMemsetAsync(&c->d_stats->n_killed, 0, sizeof(unsigned long long), c->stream));
      acc_st->n_killed += (int64_t)c->h_stats->n_killed;
    }
    if (c->h_stats->bar_error) return fail(c, MPG_ERR_TIMEOUT, "solver grid barrier timed out");
  }
  ev_record(c, 5);
  if (c->timing) {
    CK(cudaEventSynchronize(c->ev[5]));
    acc_st->ms_deposit += ev_ms(c, 0, 1);
    acc_st->ms_solve += ev_ms(c, 1, 2);
    acc_st->ms_efield += ev_ms(c, 2, 3);
    acc_st->ms_move += ev_ms(c, 3, 4);
    acc_st->ms_sort += ev_ms(c, 4, 5);
  }
  return MPG_OK;
}

int upload_mesh(mpg_ctx *c) {
  HostMesh &h = c->hm;
  DevMesh &d = c->dm;
  d.T = h.T;
  d.N = h.N;
  d.nsolve = h.nsolve;
  d.plane = (int64_t)(h.d.ny + 1) * (h.d.nz + 1);
  d.xflip = h.d.lo + h.d.hi;
  d.xshift = (h.d.periodic && h.d.mapping == MPG_MAP_JITTER) ? h.d.hi - h.d.lo : 0.0;
  d.fper = nullptr;
  if (h.d.periodic) {
    TRY(dalloc(c, &d.fper, 4 * h.T));
    CK(cudaMemcpyAsync(d.fper, h.fper.data(), 4 * h.T, cudaMemcpyHostToDevice, c->stream));
  }
  TRY(dalloc(c, &d.tets, h.T));
  TRY(dalloc(c, &d.nbrs, h.T));
  TRY(dalloc(c, &d.jinv, 9 * h.T));
  TRY(dalloc(c, &d.detj, h.T));
  TRY(dalloc(c, &d.normals, 12 * h.T));
  TRY(dalloc(c, &d.grad, 12 * h.T));
  TRY(dalloc(c, &d.nodes, 3 * h.N));
  TRY(dalloc(c, &d.bnd, h.N));
  TRY(dalloc(c, &d.mrec, 3 * h.T));
  TRY(dalloc(c, &d.mnbr, h.T));
  TRY(dalloc(c, &d.fill_ratio, h.T));
  cudaStream_t s = c->stream;
  CK(cudaMemcpyAsync(d.tets, h.tets.data(), sizeof(int4) * h.T, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d.nbrs, h.nbrs.data(), sizeof(int4) * h.T, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d.jinv, h.jinv.data(), sizeof(double) * 9 * h.T, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d.detj, h.detj.data(), sizeof(double) * h.T, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d.normals, h.normals.data(), sizeof(double) * 12 * h.T, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d.grad, h.grad.data(), sizeof(double) * 12 * h.T, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d.nodes, h.nodes.data(), sizeof(double) * 3 * h.N, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d.bnd, h.bnd.data(), h.N, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d.mnbr, h.nbr_opp.data(), sizeof(uint4) * h.T, cudaMemcpyHostToDevice, s));
  // walk record per tet: J^-1 (9 floats), E (3 floats, written by the E-field pass)
  std::vector<float> rec(12 * h.T), ratio;
  for (int64_t t = 0; t < h.T; ++t) {
    for (int q = 0; q < 9; ++q) rec[12 * t + q] = (float)h.jinv[9 * t + q];
    rec[12 * t + 9] = rec[12 * t + 10] = rec[12 * t + 11] = 0.f;
  }
  CK(cudaMemcpyAsync(d.mrec, rec.data(), sizeof(float) * 12 * h.T, cudaMemcpyHostToDevice, s));
  host_fill_ratio(h, ratio);
  CK(cudaMemcpyAsync(d.fill_ratio, ratio.data(), sizeof(float) * h.T, cudaMemcpyHostToDevice, s));
  std::vector<int32_t> off, c2n;
  host_charge_slots(h, off, c2n);
  TRY(dalloc(c, &d.n2c_off, h.N + 1));
  TRY(dalloc(c, &d.c2n, h.T));
  CK(cudaMemcpyAsync(d.n2c_off, off.data(), sizeof(int32_t) * (h.N + 1), cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(d.c2n, c2n.data(), sizeof(int32_t) * 4 * h.T, cudaMemcpyHostToDevice, s));
  // uniform Kuhn meshes: the mixed walk reads the 6-type table (MPG_KUHN_WALK=0
  // keeps the per-tet records, for comparisons)
  d.kuhn = 0;
  const char *kw = getenv("MPG_KUHN_WALK");
  const int64_t nyz = (int64_t)h.d.ny * h.d.nz;
  if (!(kw && atoi(kw) == 0) && nyz <= (1 << 16) && host_kuhn_table(h, d.ktab.jinv, d.ktab.face, d.ktab.noff)) {
    d.ktab.nx = h.d.nx;
    d.ktab.ny = h.d.ny;
    d.ktab.nz = h.d.nz;
    d.ktab.mz = ((1ull << 40) + (unsigned long long)h.d.nz - 1) / (unsigned long long)h.d.nz;
    d.ktab.myz = ((1ull << 40) + (unsigned long long)nyz - 1) / (unsigned long long)nyz;
    TRY(dalloc(c, &d.etet4, h.T));
    CK(cudaMemsetAsync(d.etet4, 0, sizeof(float4) * h.T, s));
    d.kuhn = 1;
  }
  CK(cudaStreamSynchronize(s));
  return MPG_OK;
}

void free_mesh(mpg_ctx *c) {
  DevMesh &d = c->dm;
  dfree(c, d.fper);
  dfree(c, d.tets);
  dfree(c, d.nbrs);
  dfree(c, d.jinv);
  dfree(c, d.detj);
  dfree(c, d.normals);
  dfree(c, d.grad);
  dfree(c, d.nodes);
  dfree(c, d.bnd);
  dfree(c, d.mrec);
  dfree(c, d.mnbr);
  dfree(c, d.fill_ratio);
  dfree(c, d.n2c_off);
  dfree(c, d.c2n);
  dfree(c, d.etet4);
  d.kuhn = 0;
  d = DevMesh();
}

void free_mg(mpg_ctx *c) {
  for (void *p : c->mg_bufs) dfree(c, p);
  c->mg_bufs.clear();
  c->mg = MgDev();
  c->mg_ok = false;
}

// upload a host multigrid hierarchy; levels with more than kMgBlockRows rows
// (and always the fine one) are processed by the whole grid
int upload_mg(mpg_ctx *c, const MgHostHierarchy &H) {
  int64_t kMgBlockRows = 4096;
  if (const char *e = getenv("MPG_MG_BLOCK_ROWS")) kMgBlockRows = atoll(e);
  free_mg(c);
  MgDev &m = c->mg;
  m.nlev = (int)H.lev.size();
  for (int l = 0; l < m.nlev; ++l) {
    const MgHostLevel &h = H.lev[l];
    MgLevelDev &L = m.lev[l];
    L.gx = h.gx;
    L.gy = h.gy;
    L.gz = h.gz;
    L.px = h.px ? 1 : 0;
    L.sj = h.gz;
    L.si = h.gy * h.gz;
    L.n = (int64_t)h.gx * h.gy * h.gz;
    float *dinv;
    uint8_t *bnd;
    TRY(dalloc(c, &dinv, L.n));
    TRY(dalloc(c, &bnd, L.n));
    c->mg_bufs.push_back(dinv);
    c->mg_bufs.push_back(bnd);
    CK(cudaMemcpyAsync(dinv, h.dinv.data(), sizeof(float) * L.n, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(bnd, h.bnd.data(), L.n, cudaMemcpyHostToDevice, c->stream));
    L.dinv = dinv;
    L.bnd = bnd;
    if (l > 0) {
      float *val, *r, *e, *t;
      TRY(dalloc(c, &val, 27 * L.n));
      TRY(dalloc(c, &r, L.n));
      TRY(dalloc(c, &e, L.n));
      TRY(dalloc(c, &t, L.n));
      float *t2;
      TRY(dalloc(c, &t2, L.n));
      for (void *p : {(void *)val, (void *)r, (void *)e, (void *)t, (void *)t2}) c->mg_bufs.push_back(p);
      CK(cudaMemcpyAsync(val, h.val.data(), sizeof(float) * 27 * L.n, cudaMemcpyHostToDevice, c->stream));
      CK(cudaMemsetAsync(e, 0, sizeof(float) * L.n, c->stream));
      CK(cudaMemsetAsync(t, 0, sizeof(float) * L.n, c->stream));
      CK(cudaMemsetAsync(t2, 0, sizeof(float) * L.n, c->stream));
      L.val = val;
      L.r = r;
      L.e = e;
      L.t = t;
      L.t2 = t2;
    }
  }
  m.ngrid = 1;
  while (m.ngrid < m.nlev - 1 && m.lev[m.ngrid].n > kMgBlockRows) ++m.ngrid;
  int32_t *idx;
  float *inv;
  m.dense_m = (int)H.dense_idx.size();
  float *dr;
  TRY(dalloc(c, &idx, m.dense_m));
  TRY(dalloc(c, &inv, (int64_t)m.dense_m * m.dense_m));
  TRY(dalloc(c, &dr, m.dense_m));
  c->mg_bufs.push_back(idx);
  c->mg_bufs.push_back(inv);
  c->mg_bufs.push_back(dr);
  m.dense_r = dr;
  CK(cudaMemcpyAsync(idx, H.dense_idx.data(), sizeof(int32_t) * m.dense_m, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(inv, H.dense_inv.data(), sizeof(float) * H.dense_inv.size(), cudaMemcpyHostToDevice,
                     c->stream));
  CK(cudaStreamSynchronize(c->stream));
  m.dense_idx = idx;
  m.dense_inv = inv;
  if (const char *e = getenv("MPG_MG_OMEGA")) m.omega = (float)atof(e);
  if (const char *e = getenv("MPG_MG_RELIABLE")) m.reliable = atoi(e);
  if (const char *e = getenv("MPG_MG_NU0")) m.nu0 = atoi(e) == 2 ? 2 : 1;
  if (const char *e = getenv("MPG_MG_NU1")) m.nu1 = atoi(e) == 2 ? 2 : 1;
  int64_t fuse_rows = 1 << 20;
  if (const char *e = getenv("MPG_MG_FUSE_UPDATE_ROWS")) fuse_rows = atoll(e);
  m.fuse_update = m.lev[0].n <= fuse_rows ? 1 : 0;
  if (c->dia.constant)
    for (int d = 0; d < c->dia.ndiag; ++d)
      if (c->dia.off[d] == 0 && c->dia.cst[d] != 0.f) m.dinv0 = (float)(1.0 / (double)c->dia.cst[d]);
  c->mg_ok = true;
  return MPG_OK;
}

void free_field(mpg_ctx *c) {
  dfree(c, c->rowptr);
  dfree(c, c->col);
  dfree(c, c->val);
  dfree(c, c->val32);
  dfree(c, c->dia.val64);
  dfree(c, c->dia.val32);
  dfree(c, c->dia.dis);
  c->dia = DiaMatrix();
  dfree(c, c->rhs);
  dfree(c, c->phi);
  dfree(c, c->phi_prev);
  dfree(c, c->phi_prev2);
  c->phi_hist = 0;
  dfree(c, c->bg);
  dfree(c, c->Etet);
  dfree(c, c->acc);
  dfree(c, c->acc_node);
  dfree(c, c->sort_cnt);
  dfree(c, c->sort_start);
  c->starts_valid = false;
  dfree(c, c->scan_scratch);
  c->scan_len = 0;
  dfree(c, c->bicg_work);
  free_mg(c);
  c->configured = false;
  c->csr_mode = -1;
}

}  // namespace

// ===========================================================================
extern "C" {

int mpg_version(void) { return 1; }

int mpg_device_count(int *n) {
  if (!n) return MPG_ERR_ARG;
  cudaError_t e = cudaGetDeviceCount(n);
  if (e != cudaSuccess) {
    *n = 0;
    g_last_create_error = cudaGetErrorString(e);
    return MPG_ERR_CUDA;
  }
  return MPG_OK;
}

int mpg_ctx_create(int device, mpg_ctx **out) {
  if (!out) return MPG_ERR_ARG;
  *out = nullptr;
  int nd = 0;
  cudaError_t e = cudaGetDeviceCount(&nd);
  if (e != cudaSuccess || nd == 0) {
    g_last_create_error = std::string("no CUDA device: ") + cudaGetErrorString(e);
    return MPG_ERR_CUDA;
  }
  if (device < 0 || device >= nd) {
    g_last_create_error = "device index out of range";
    return MPG_ERR_ARG;
  }
  mpg_ctx *c = new (std::nothrow) mpg_ctx();
  if (!c) return MPG_ERR_ARG;
  c->device = device;
  auto bail = [&](const char *what, cudaError_t err) {
    g_last_create_error = std::string(what) + ": " + cudaGetErrorString(err);
    delete c;
    return MPG_ERR_CUDA;
  };
  if ((e = cudaSetDevice(device)) != cudaSuccess) return bail("cudaSetDevice", e);
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return bail("cudaStreamCreate", e);
  for (int i = 0; i < 12; ++i)
    if ((e = cudaEventCreate(&c->ev[i])) != cudaSuccess) return bail("cudaEventCreate", e);
  if ((e = cudaMalloc(&c->d_stats, sizeof(DevStats))) != cudaSuccess) return bail("cudaMalloc", e);
  if ((e = cudaMallocHost(&c->h_stats, sizeof(DevStats))) != cudaSuccess) return bail("cudaMallocHost", e);
  if ((e = cudaMalloc(&c->d_count, sizeof(uint32_t))) != cudaSuccess) return bail("cudaMalloc", e);
  if ((e = cudaMallocHost(&c->h_count, sizeof(uint32_t))) != cudaSuccess) return bail("cudaMallocHost", e);
  if ((e = cudaMalloc(&c->red_dev, sizeof(double) * 512)) != cudaSuccess) return bail("cudaMalloc", e);
  if ((e = cudaMallocHost(&c->red_host, sizeof(double) * 8)) != cudaSuccess) return bail("cudaMallocHost", e);
  cudaMemsetAsync(c->d_stats, 0, sizeof(DevStats), c->stream);
  default_species(c->sp);
  c->cfg.precision = MPG_PLAIN;
  c->cfg.deposit = MPG_DEPOSIT_REF_QUARTER;
  c->cfg.solver = MPG_SOLVER_BICGSTAB;
  c->cfg.tol = 1e-6;
  c->cfg.max_iter = 1000;
  c->cfg.max_crossings = 1000;
  *out = c;
  return MPG_OK;
}

int mpg_ctx_destroy(mpg_ctx *c) {
  if (!c) return MPG_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (void *p : c->allocs) cudaFree(p);
  c->allocs.clear();
  cudaFree(c->d_stats);
  cudaFreeHost(c->h_stats);
  cudaFree(c->d_count);
  cudaFreeHost(c->h_count);
  cudaFree(c->red_dev);
  cudaFreeHost(c->red_host);
  for (int i = 0; i < 12; ++i)
    if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  cudaStreamDestroy(c->stream);
  delete c;
  return MPG_OK;
}

int mpg_last_error(mpg_ctx *c, char *buf, int len) {
  if (!buf || len <= 0) return MPG_ERR_ARG;
  const std::string &m = c ? c->err : g_last_create_error;
  snprintf(buf, (size_t)len, "%s", m.c_str());
  return MPG_OK;
}

int mpg_set_timing(mpg_ctx *c, int on) {
  if (!c) return MPG_ERR_ARG;
  c->timing = on != 0;
  return MPG_OK;
}

int mpg_timer(mpg_ctx *c, int op, double *ms) {
  ENTER(c);
  if (op == 0) {
    CK(cudaEventRecord(c->ev[10], c->stream));
    return MPG_OK;
  }
  if (op != 1 || !ms) return fail(c, MPG_ERR_ARG, "mpg_timer: op must be 0 (start) or 1 (stop) with ms");
  CK(cudaEventRecord(c->ev[11], c->stream));
  CK(cudaEventSynchronize(c->ev[11]));
  float f = 0.f;
  CK(cudaEventElapsedTime(&f, c->ev[10], c->ev[11]));
  *ms = f;
  return MPG_OK;
}

int mpg_mg_hierarchy(const mpg_mesh_desc *mesh, int64_t dense_max, int level, int *nlev, int *extent, float *val27,
                     float *dinv, uint8_t *bnd) {
  if (!mesh || !nlev || !extent) return MPG_ERR_ARG;
  HostMesh hm;
  std::string err;
  int rc = host_mesh_generate(*mesh, hm, err);
  if (rc) return rc;
  std::vector<int32_t> rp, col;
  std::vector<double> val;
  host_csr_assemble(hm, 1, rp, col, val);
  MgHostHierarchy H;
  if (!host_mg_build(hm, rp, col, val, H, err, dense_max)) return MPG_ERR_ARG;
  *nlev = (int)H.lev.size();
  if (level < 0 || level >= *nlev) return MPG_ERR_ARG;
  const MgHostLevel &L = H.lev[level];
  extent[0] = L.gx;
  extent[1] = L.gy;
  extent[2] = L.gz;
  if (val27 && level > 0) std::copy(L.val.begin(), L.val.end(), val27);
  if (dinv) std::copy(L.dinv.begin(), L.dinv.end(), dinv);
  if (bnd) std::copy(L.bnd.begin(), L.bnd.end(), bnd);
  return MPG_OK;
}

int mpg_mesh_build(mpg_ctx *c, const mpg_mesh_desc *d) {
  ENTER(c);
  TRY(settle_sort(c));
  if (!d) return fail(c, MPG_ERR_ARG, "null mesh descriptor");
  CK(cudaStreamSynchronize(c->stream));
  free_particles(c);
  free_field(c);
  free_mesh(c);
  c->has_mesh = false;
  std::string err;
  int rc = host_mesh_generate(*d, c->hm, err);
  if (rc) return fail(c, rc, "%s", err.c_str());
  TRY(upload_mesh(c));
  c->has_mesh = true;
  c->step_count = 0;
  return MPG_OK;
}

int mpg_mesh_sizes(mpg_ctx *c, int64_t *T, int64_t *N, int64_t *nb) {
  if (!c) return MPG_ERR_ARG;
  if (!c->has_mesh) return fail(c, MPG_ERR_STATE, "no mesh");
  if (T) *T = c->hm.T;
  if (N) *N = c->hm.N;
  if (nb) *nb = c->hm.n_bnodes;
  return MPG_OK;
}

int mpg_mesh_download(mpg_ctx *c, double *nodes, int32_t *tets, int32_t *nbrs, double *jinv, double *detj,
                      double *normals, uint8_t *boundary) {
  ENTER(c);
  if (!c->has_mesh) return fail(c, MPG_ERR_STATE, "no mesh");
  const DevMesh &d = c->dm;
  cudaStream_t s = c->stream;
  if (nodes) CK(cudaMemcpyAsync(nodes, d.nodes, sizeof(double) * 3 * d.N, cudaMemcpyDeviceToHost, s));
  if (tets) CK(cudaMemcpyAsync(tets, d.tets, sizeof(int4) * d.T, cudaMemcpyDeviceToHost, s));
  if (nbrs) CK(cudaMemcpyAsync(nbrs, d.nbrs, sizeof(int4) * d.T, cudaMemcpyDeviceToHost, s));
  if (jinv) CK(cudaMemcpyAsync(jinv, d.jinv, sizeof(double) * 9 * d.T, cudaMemcpyDeviceToHost, s));
  if (detj) CK(cudaMemcpyAsync(detj, d.detj, sizeof(double) * d.T, cudaMemcpyDeviceToHost, s));
  if (normals) CK(cudaMemcpyAsync(normals, d.normals, sizeof(double) * 12 * d.T, cudaMemcpyDeviceToHost, s));
  if (boundary) CK(cudaMemcpyAsync(boundary, d.bnd, d.N, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  return MPG_OK;
}

int mpg_mesh_periodic_download(mpg_ctx *c, int8_t *face_periodic, int32_t *node_pairs) {
  ENTER(c);
  if (!c->has_mesh) return fail(c, MPG_ERR_STATE, "no mesh");
  const HostMesh &h = c->hm;
  // the face flags the device walk reads; the pairs live on the host only
  if (face_periodic) {
    if (c->dm.fper) {
      CK(cudaMemcpyAsync(face_periodic, c->dm.fper, 4 * c->dm.T, cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
    } else {
      memset(face_periodic, 0, 4 * c->dm.T);
    }
  }
  if (node_pairs) memcpy(node_pairs, h.pair.data(), sizeof(int32_t) * h.pair.size());
  return MPG_OK;
}

int mpg_species_set(mpg_ctx *c, int i, double q, double m) {
  if (!c) return MPG_ERR_ARG;
  if (i < 0 || i >= MPG_MAX_SPECIES) return fail(c, MPG_ERR_ARG, "species index %d out of range", i);
  if (!(m > 0)) return fail(c, MPG_ERR_ARG, "species mass must be positive");
  c->sp.q[i] = q;
  c->sp.m[i] = m;
  upload_species_derived(c);
  c->qfix_valid = false;
  c->acc_valid = false;
  return MPG_OK;
}

int mpg_configure(mpg_ctx *c, const mpg_config *cfg) {
  ENTER(c);
  TRY(settle_sort(c));
  if (!cfg) return fail(c, MPG_ERR_ARG, "null config");
  if (!c->has_mesh) return fail(c, MPG_ERR_STATE, "no mesh: call mpg_mesh_build first");
  if (cfg->precision != MPG_PLAIN && cfg->precision != MPG_MIXED) return fail(c, MPG_ERR_ARG, "bad precision");
  if (cfg->deposit != MPG_DEPOSIT_REF_QUARTER && cfg->deposit != MPG_DEPOSIT_LINEAR)
    return fail(c, MPG_ERR_ARG, "bad deposit mode");
  if (cfg->solver != MPG_SOLVER_BICGSTAB && cfg->solver != MPG_SOLVER_CG && cfg->solver != MPG_SOLVER_CG_MG)
    return fail(c, MPG_ERR_ARG, "bad solver");
  if (!(cfg->tol > 0) || cfg->max_iter < 1 || cfg->max_crossings < 1)
    return fail(c, MPG_ERR_ARG, "tol, max_iter and max_crossings must be positive");
  if (cfg->precision == MPG_MIXED && c->hm.T >= (int64_t)MPG_WALL)
    return fail(c, MPG_ERR_ARG, "mixed form holds cell ids in 24 bits (T < %u)", MPG_WALL);
  CK(cudaStreamSynchronize(c->stream));
  const bool realloc_parts = c->parts_alloc && (c->cfg.precision != cfg->precision ||
                                                (cfg->track_ids != 0) != (c->cfg.track_ids != 0));
  if (realloc_parts) free_particles(c);
  c->cfg = *cfg;
  // the mixed form always solves the symmetric system with refined CG
  const int mode = (cfg->precision == MPG_MIXED || cfg->solver != MPG_SOLVER_BICGSTAB) ? 1 : 0;
  const int64_t N = c->hm.N, T = c->hm.T;
  // rows of the assembled system: all nodes, or (symmetric form of a periodic
  // mesh) the nodes of the x < hi planes, the ghost plane being last in order
  const int64_t R = mode == 1 ? c->hm.nsolve : N;
  const bool per = c->hm.d.periodic != 0;
  // periodic stencils wrap around in x: an offset or index modulo R
  auto wrap_off = [&](int64_t o) -> int64_t {
    if (per) {
      if (o > R / 2) o -= R;
      else if (o < -R / 2) o += R;
    }
    return o;
  };
  auto wrap_idx = [&](int64_t j) -> int64_t {
    if (per) {
      if (j < 0) j += R;
      else if (j >= R) j -= R;
    }
    return j;
  };
  const int want_mg = (cfg->precision == MPG_MIXED && cfg->solver == MPG_SOLVER_CG_MG) ? 1 : 0;
  if (c->csr_mode != mode || c->csr_mg != want_mg) {
    dfree(c, c->rowptr);
    dfree(c, c->col);
    dfree(c, c->val);
    dfree(c, c->val32);
    std::vector<int32_t> rp, col;
    std::vector<double> val;
    host_csr_assemble(c->hm, mode, rp, col, val);
    c->nnz = (int64_t)val.size();
    c->csr_rows = R;
    TRY(dalloc(c, &c->rowptr, R + 1));
    TRY(dalloc(c, &c->col, c->nnz));
    TRY(dalloc(c, &c->val, c->nnz));
    TRY(dalloc(c, &c->val32, c->nnz));
    std::vector<float> v32(val.begin(), val.end());
    CK(cudaMemcpyAsync(c->rowptr, rp.data(), sizeof(int32_t) * (R + 1), cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->col, col.data(), sizeof(int32_t) * c->nnz, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->val, val.data(), sizeof(double) * c->nnz, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemcpyAsync(c->val32, v32.data(), sizeof(float) * c->nnz, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    dfree(c, c->dia.val64);
    dfree(c, c->dia.val32);
    dfree(c, c->dia.dis);
    c->dia = DiaMatrix();
    if (mode == 1) {
      // diagonal offsets present in the interior rows, in column order
      std::vector<int64_t> offs;
      for (int64_t r = 0; r < R; ++r) {
        if (c->hm.bnd[r]) continue;
        for (int32_t k = rp[r]; k < rp[r + 1]; ++k) offs.push_back(wrap_off((int64_t)col[k] - r));
      }
      std::sort(offs.begin(), offs.end());
      offs.erase(std::unique(offs.begin(), offs.end()), offs.end());
      if (offs.size() > 27) return fail(c, MPG_ERR_MESH, "matrix is not a structured stencil (%zu offsets)", offs.size());
      // pad to the kernel's diagonal count (15 or 27) with zero diagonals at offset 0
      const int nd = offs.size() <= 15 ? 15 : 27;
      std::vector<double> d64((size_t)nd * R, 0.0);
      for (int64_t r = 0; r < R; ++r) {
        if (c->hm.bnd[r]) continue;
        for (int32_t k = rp[r]; k < rp[r + 1]; ++k) {
          const int d =
              (int)(std::lower_bound(offs.begin(), offs.end(), wrap_off((int64_t)col[k] - r)) - offs.begin());
          d64[(size_t)d * R + r] = val[k];
        }
      }
      std::vector<float> d32(d64.begin(), d64.end());
      c->dia.n = R;
      c->dia.nwrap = per ? R : 0;
      c->dia.ndiag = nd;
      for (int d = 0; d < nd; ++d) c->dia.off[d] = d < (int)offs.size() ? (int)offs[d] : 0;
      TRY(dalloc(c, &c->dia.val64, (int64_t)nd * R));
      TRY(dalloc(c, &c->dia.val32, (int64_t)nd * R));
      CK(cudaMemcpyAsync(c->dia.val64, d64.data(), sizeof(double) * d64.size(), cudaMemcpyHostToDevice, c->stream));
      CK(cudaMemcpyAsync(c->dia.val32, d32.data(), sizeof(float) * d32.size(), cudaMemcpyHostToDevice, c->stream));
      c->dia.bnd = c->dm.bnd;
      // constant-stencil test: for every interior row, every entry whose
      // column is an interior node equals its diagonal's reference value to
      // within 1e-7 of the largest entry (couplings that are zero in exact
      // arithmetic come out as rounding noise of either sign); entries of
      // boundary columns are dropped, and the stencil multiplies them by the
      // exactly zero boundary entries of the inner vectors
      {
        double amax = 0.0;
        for (size_t k = 0; k < d64.size(); ++k) amax = std::max(amax, fabs(d64[k]));
        const double atol = 1e-7 * amax;
        std::vector<double> ref(nd, 0.0);
        std::vector<char> have(nd, 0);
        bool uniform = amax > 0.0;
        for (int64_t r = 0; r < R && uniform; ++r) {
          if (c->hm.bnd[r]) continue;
          for (int d = 0; d < (int)offs.size(); ++d) {
            if (c->hm.bnd[wrap_idx(r + offs[d])]) continue;
            const double v = d64[(size_t)d * R + r];
            if (!have[d]) {
              ref[d] = v;
              have[d] = 1;
            } else if (fabs(v - ref[d]) > atol) {
              uniform = false;
              break;
            }
          }
        }
        c->dia.constant = uniform ? 1 : 0;
        for (int d = 0; d < nd; ++d) c->dia.cst[d] = uniform ? (float)ref[d] : 0.f;
      }
      // Non-uniform meshes: the FP32 inner operator of the mixed solver is the
      // symmetrically Jacobi-scaled matrix D^-1/2 A D^-1/2 (unit diagonal; the
      // FP64 outer residual keeps A itself).  MPG_CG_JACOBI=0 turns it off.
      const char *jenv = getenv("MPG_CG_JACOBI");
      const int center = (int)(std::lower_bound(offs.begin(), offs.end(), (int64_t)0) - offs.begin());
      // with the multigrid preconditioner the inner operator stays A itself
      // (the V-cycle smooths with its own D^-1)
      free_mg(c);
      if (want_mg) {
        MgHostHierarchy H;
        std::string why;
        if (host_mg_build(c->hm, rp, col, val, H, why)) TRY(upload_mg(c, H));
      }
      if (!c->mg_ok && !c->dia.constant && !(jenv && atoi(jenv) == 0) && center < (int)offs.size() &&
          offs[center] == 0) {
        std::vector<double> dis(R, 1.0);
        for (int64_t r = 0; r < R; ++r) {
          const double dr = d64[(size_t)center * R + r];
          if (!c->hm.bnd[r] && dr > 0.0) dis[r] = 1.0 / std::sqrt(dr);
        }
        for (int64_t r = 0; r < R; ++r) {
          if (c->hm.bnd[r]) continue;
          for (int d = 0; d < (int)offs.size(); ++d) {
            const double v = d64[(size_t)d * R + r];
            if (v != 0.0) d32[(size_t)d * R + r] = (float)(v * dis[r] * dis[wrap_idx(r + offs[d])]);
          }
        }
        TRY(dalloc(c, &c->dia.dis, R));
        CK(cudaMemcpyAsync(c->dia.dis, dis.data(), sizeof(double) * R, cudaMemcpyHostToDevice, c->stream));
        CK(cudaMemcpyAsync(c->dia.val32, d32.data(), sizeof(float) * d32.size(), cudaMemcpyHostToDevice,
                           c->stream));
      }
      CK(cudaStreamSynchronize(c->stream));
    }
    c->csr_mode = mode;
    c->csr_mg = want_mg;
  }
  if (!c->rhs) {
    TRY(dalloc(c, &c->rhs, N));
    TRY(dalloc(c, &c->phi, N));
    TRY(dalloc(c, &c->Etet, 3 * T));
    TRY(dalloc(c, &c->acc, 4 * T));
    TRY(dalloc(c, &c->acc_node, N));
    CK(cudaMemsetAsync(c->acc, 0, sizeof(unsigned long long) * 4 * c->dm.T, c->stream));
    TRY(dalloc(c, &c->sort_cnt, T + 1));
    TRY(dalloc(c, &c->sort_start, T + 1));
    CK(cudaMemsetAsync(c->phi, 0, sizeof(double) * N, c->stream));
    CK(cudaMemsetAsync(c->Etet, 0, sizeof(double) * 3 * T, c->stream));
  }
  dfree(c, c->bg);
  if (cfg->rho_background != 0.0) {
    std::vector<double> bg;
    host_background(c->hm, cfg->rho_background, bg);
    TRY(dalloc(c, &c->bg, N));
    CK(cudaMemcpyAsync(c->bg, bg.data(), sizeof(double) * N, cudaMemcpyHostToDevice, c->stream));
  }
  c->configured = true;
  c->acc_valid = false;
  CK(cudaStreamSynchronize(c->stream));
  return MPG_OK;
}

int mpg_csr_sizes(mpg_ctx *c, int64_t *rows, int64_t *nnz) {
  if (!c) return MPG_ERR_ARG;
  if (!c->configured) return fail(c, MPG_ERR_STATE, "not configured");
  if (rows) *rows = c->csr_rows;
  if (nnz) *nnz = c->nnz;
  return MPG_OK;
}

int mpg_csr_download(mpg_ctx *c, int32_t *rowptr, int32_t *col, double *val) {
  ENTER(c);
  if (!c->configured) return fail(c, MPG_ERR_STATE, "not configured");
  if (rowptr)
    CK(cudaMemcpyAsync(rowptr, c->rowptr, sizeof(int32_t) * (c->csr_rows + 1), cudaMemcpyDeviceToHost, c->stream));
  if (col) CK(cudaMemcpyAsync(col, c->col, sizeof(int32_t) * c->nnz, cudaMemcpyDeviceToHost, c->stream));
  if (val) CK(cudaMemcpyAsync(val, c->val, sizeof(double) * c->nnz, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return MPG_OK;
}

int mpg_particles_reserve(mpg_ctx *c, int64_t capacity) {
  ENTER(c);
  TRY(settle_sort(c));
  if (capacity <= 0 || capacity >= (1LL << 31)) return fail(c, MPG_ERR_ARG, "capacity out of range");
  if (c->parts_alloc && c->n > 0 && !(c->cap == capacity && c->precision == c->cfg.precision))
    return fail(c, MPG_ERR_STATE, "cannot resize a non-empty particle list");
  c->want_cap = capacity;
  if (c->configured && !(c->parts_alloc && c->cap == capacity && c->precision == c->cfg.precision)) {
    CK(cudaStreamSynchronize(c->stream));
    return alloc_particles(c, capacity);
  }
  return MPG_OK;
}

int mpg_particles_count(mpg_ctx *c, int64_t *n) {
  if (!c || !n) return MPG_ERR_ARG;
  *n = c->parts_alloc ? c->n_live : 0;
  return MPG_OK;
}

int mpg_fill_ref(mpg_ctx *c, int nppe, int type, double density, const double vel[3], double temp) {
  ENTER(c);
  TRY(settle_sort(c));
  TRY(ensure_particles(c));
  if (nppe < 1 || type < 0 || type >= MPG_MAX_SPECIES) return fail(c, MPG_ERR_ARG, "bad nppe or type");
  const int64_t add = c->hm.T * (int64_t)nppe;
  if (c->n + add > c->cap)  // particle_fill.hpp:61-64 (the reference prints and skips)
    return fail(c, MPG_ERR_CAPACITY, "Cannot create that number of particles, no fill performed");
  const double v0[3] = {0, 0, 0};
  const double *vel3 = vel ? vel : v0;
  const double mass = c->sp.m[type];
  if (c->cfg.precision == MPG_PLAIN) {
    launch_fill_ref(c->stream, c->pp[c->cur], c->n, nppe, type, density, vel3, temp, mass, c->dm, c->id_next);
    CKL();
    c->weight_set[type] = true;
  } else {
    TempPlain t;
    TRY(temp_plain(c, add, c->cfg.track_ids != 0, t));
    launch_fill_ref(c->stream, t.P, 0, nppe, type, density, vel3, temp, mass, c->dm, c->id_next);
    MixedParts X = c->mp[c->cur];
    // shift the destination by n: convert into slots [n, n+add)
    X.c += c->n;
    X.b += c->n;
    X.v += c->n;
    if (X.id) X.id += c->n;
    launch_plain_to_mixed(c->stream, t.P, 0, add, X);
    CKL();
    temp_free(c, t);
    double vol = 0.0;
    for (int64_t i = 0; i < c->hm.T; ++i) vol += c->hm.detj[i] / 6.;
    TRY(set_species_weight(c, type, density * (vol / c->hm.T) / nppe));
  }
  c->n += add;
  c->n_live += add;
  c->id_next += add;
  c->acc_valid = false;
  c->needs_sort = true;
  c->starts_valid = false;
  CK(cudaStreamSynchronize(c->stream));
  return MPG_OK;
}

int mpg_fill_uniform(mpg_ctx *c, int64_t n, uint64_t seed, int type, double weight, const double drift[3],
                     double vth) {
  ENTER(c);
  TRY(settle_sort(c));
  TRY(ensure_particles(c));
  if (n < 0 || type < 0 || type >= MPG_MAX_SPECIES) return fail(c, MPG_ERR_ARG, "bad count or type");
  if (c->n + n > c->cap) return fail(c, MPG_ERR_CAPACITY, "fill of %lld exceeds capacity", (long long)n);
  if (c->cfg.precision == MPG_MIXED && c->n + n >= (1LL << 32))
    return fail(c, MPG_ERR_ARG, "too many particles");
  const double d0[3] = {0, 0, 0};
  TRY(set_species_weight(c, type, weight));
  launch_fill_uniform(c->stream, c->cfg.precision == MPG_MIXED, c->pp[c->cur], c->mp[c->cur], c->n, n, seed, type,
                      weight, drift ? drift : d0, vth, c->dm, c->id_next);
  CKL();
  c->n += n;
  c->n_live += n;
  c->id_next += n;
  c->acc_valid = false;
  c->needs_sort = true;
  c->starts_valid = false;
  CK(cudaStreamSynchronize(c->stream));
  return MPG_OK;
}

int mpg_particles_upload(mpg_ctx *c, int64_t n, const int32_t *cell, const double *x, const double *xref,
                         const double *v, const double *w, const int32_t *species, const int64_t *id) {
  ENTER(c);
  TRY(settle_sort(c));
  TRY(ensure_particles(c));
  if (n < 0 || n > c->cap) return fail(c, MPG_ERR_CAPACITY, "upload of %lld exceeds capacity", (long long)n);
  if (n > 0 && (!cell || !xref || !v)) return fail(c, MPG_ERR_ARG, "cell, xref and v are required");
  cudaStream_t s = c->stream;
  const bool mixed = c->cfg.precision == MPG_MIXED;
  // host-side validation of species and weights
  std::vector<int32_t> spv(n > 0 ? n : 1, 0);
  if (species)
    for (int64_t i = 0; i < n; ++i) {
      if (species[i] < 0 || species[i] >= MPG_MAX_SPECIES) return fail(c, MPG_ERR_ARG, "species out of range");
      spv[i] = species[i];
    }
  for (int64_t i = 0; i < n; ++i)
    if (cell[i] >= c->hm.T) return fail(c, MPG_ERR_ARG, "cell id %d out of range", cell[i]);
  std::vector<double> wv(n > 0 ? n : 1, 1.0);
  if (w)
    for (int64_t i = 0; i < n; ++i) wv[i] = w[i];
  if (mixed) {
    for (int64_t i = 0; i < n; ++i)
      if (cell[i] >= 0) TRY(set_species_weight(c, spv[i], wv[i]));
  } else {
    for (int64_t i = 0; i < n; ++i) c->weight_set[spv[i]] = true;
  }
  TempPlain t;
  TRY(temp_plain(c, n, true, t));
  double *stage;
  CK(cudaMallocAsync((void **)&stage, sizeof(double) * 3 * (n > 0 ? n : 1), s));
  if (n > 0) {
    CK(cudaMemcpyAsync(t.P.cell, cell, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(t.P.w, wv.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(t.P.sp, spv.data(), sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
    if (id) {
      CK(cudaMemcpyAsync(t.P.id, id, sizeof(int64_t) * n, cudaMemcpyHostToDevice, s));
    } else {
      std::vector<int64_t> ids(n);
      for (int64_t i = 0; i < n; ++i) ids[i] = i;
      CK(cudaMemcpyAsync(t.P.id, ids.data(), sizeof(int64_t) * n, cudaMemcpyHostToDevice, s));
      CK(cudaStreamSynchronize(s));
    }
    const double *srcs[3] = {x, xref, v};
    double *dsts[3] = {t.P.x, t.P.xr, t.P.v};
    for (int k = 0; k < 3; ++k) {
      if (!srcs[k]) {
        CK(cudaMemsetAsync(dsts[k], 0, sizeof(double) * 3 * n, s));
        continue;
      }
      CK(cudaMemcpyAsync(stage, srcs[k], sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s));
      launch_rows_to_cols(s, stage, dsts[k], n, t.P.cap);
    }
  }
  if (mixed) {
    launch_plain_to_mixed(s, t.P, 0, n, c->mp[c->cur]);
  } else {
    PlainParts &P = c->pp[c->cur];
    if (n > 0) {
      CK(cudaMemcpyAsync(P.cell, t.P.cell, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
      CK(cudaMemcpyAsync(P.w, t.P.w, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      CK(cudaMemcpyAsync(P.sp, t.P.sp, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
      if (P.id) CK(cudaMemcpyAsync(P.id, t.P.id, sizeof(int64_t) * n, cudaMemcpyDeviceToDevice, s));
      for (int d = 0; d < 3; ++d) {
        CK(cudaMemcpyAsync(P.x + d * P.cap, t.P.x + d * t.P.cap, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(P.xr + d * P.cap, t.P.xr + d * t.P.cap, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                           s));
        CK(cudaMemcpyAsync(P.v + d * P.cap, t.P.v + d * t.P.cap, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
      }
    }
  }
  CKL();
  CK(cudaFreeAsync(stage, s));
  temp_free(c, t);
  CK(cudaStreamSynchronize(s));
  c->n = n;
  c->n_live = 0;
  for (int64_t i = 0; i < n; ++i) c->n_live += cell[i] >= 0;
  c->id_next = n;
  c->acc_valid = false;
  c->needs_sort = true;
  c->starts_valid = false;
  return MPG_OK;
}

int mpg_particles_download(mpg_ctx *c, int64_t cap, int64_t *nout, int32_t *cell, double *x, double *xref, double *v,
                           double *w, int32_t *species, int64_t *id) {
  ENTER(c);
  TRY(settle_sort(c));
  if (!c->parts_alloc) {
    if (nout) *nout = 0;
    return MPG_OK;
  }
  const int64_t n = c->n;
  if (nout) *nout = n;
  if (cap < n) return fail(c, MPG_ERR_CAPACITY, "download buffer holds %lld < %lld", (long long)cap, (long long)n);
  cudaStream_t s = c->stream;
  PlainParts P = c->pp[c->cur];
  TempPlain t;
  if (c->precision == MPG_MIXED) {
    TRY(temp_plain(c, n, true, t));
    launch_mixed_to_plain(s, c->mp[c->cur], n, c->dm, c->sp, t.P);
    CKL();
    P = t.P;
  }
  double *stage;
  CK(cudaMallocAsync((void **)&stage, sizeof(double) * 3 * (n > 0 ? n : 1), s));
  if (n > 0) {
    if (cell) CK(cudaMemcpyAsync(cell, P.cell, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
    if (w) CK(cudaMemcpyAsync(w, P.w, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    if (species) CK(cudaMemcpyAsync(species, P.sp, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
    if (id && P.id) CK(cudaMemcpyAsync(id, P.id, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, s));
    double *outs[3] = {x, xref, v};
    double *srcs[3] = {P.x, P.xr, P.v};
    for (int k = 0; k < 3; ++k) {
      if (!outs[k]) continue;
      launch_cols_to_rows(s, srcs[k], stage, n, P.cap);
      CK(cudaMemcpyAsync(outs[k], stage, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
    }
  }
  CKL();
  CK(cudaFreeAsync(stage, s));
  temp_free(c, t);
  CK(cudaStreamSynchronize(s));
  if (id && !P.id)
    for (int64_t i = 0; i < n; ++i) id[i] = i;
  return MPG_OK;
}

// Device address of host memory that the device can read and write (page
// locked and mapped: cudaHostAlloc'ed or cudaHostRegister'ed), else null.
// Such buffers are read and written by the pack kernels directly over the
// host link, without a staging copy in device memory.
static void *mapped_host(const void *p) {
  if (!p) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

int mpg_mixed_download(mpg_ctx *c, int64_t cap, int64_t *nout, uint32_t *cellsp, float *b, float *v) {
  ENTER(c);
  TRY(settle_sort(c));
  if (!c->parts_alloc || c->precision != MPG_MIXED) return fail(c, MPG_ERR_STATE, "no mixed particle state");
  const int64_t n = c->n;
  if (nout) *nout = n;
  if (cap < n) return fail(c, MPG_ERR_CAPACITY, "download buffer too small");
  cudaStream_t s = c->stream;
  float *hb = static_cast<float *>(mapped_host(b)), *hv = static_cast<float *>(mapped_host(v));
  if (n > 0 && hb && hv) {
    uint32_t *hc = static_cast<uint32_t *>(mapped_host(cellsp));
    launch_mixed_unpack(s, c->mp[c->cur], n, hb, hv, hc);
    CKL();
    if (cellsp && !hc)
      CK(cudaMemcpyAsync(cellsp, c->mp[c->cur].c, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    return MPG_OK;
  }
  float *sb, *sv;
  CK(cudaMallocAsync((void **)&sb, sizeof(float) * 3 * (n > 0 ? n : 1), s));
  CK(cudaMallocAsync((void **)&sv, sizeof(float) * 3 * (n > 0 ? n : 1), s));
  if (n > 0) {
    launch_mixed_unpack(s, c->mp[c->cur], n, sb, sv);
    CKL();
    if (cellsp) CK(cudaMemcpyAsync(cellsp, c->mp[c->cur].c, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s));
    if (b) CK(cudaMemcpyAsync(b, sb, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, s));
    if (v) CK(cudaMemcpyAsync(v, sv, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaFreeAsync(sb, s));
  CK(cudaFreeAsync(sv, s));
  CK(cudaStreamSynchronize(s));
  return MPG_OK;
}

int mpg_mixed_upload(mpg_ctx *c, int64_t n, const uint32_t *cellsp, const float *b, const float *v) {
  ENTER(c);
  TRY(settle_sort(c));
  TRY(ensure_particles(c));
  if (c->precision != MPG_MIXED) return fail(c, MPG_ERR_STATE, "context is not in mixed precision");
  if (n < 0 || n > c->cap) return fail(c, MPG_ERR_CAPACITY, "upload exceeds capacity");
  // staged upload: the words are validated on the device before they replace
  // the resident state, so a rejected upload leaves the context unchanged
  // (mapped host buffers: validated and packed from host memory directly)
  cudaStream_t s = c->stream;
  const int64_t nn = n > 0 ? n : 1;
  const uint32_t *hc = static_cast<const uint32_t *>(mapped_host(cellsp));
  const float *hb = static_cast<const float *>(mapped_host(b)), *hv = static_cast<const float *>(mapped_host(v));
  const bool direct = n > 0 && hc && hb && hv;
  uint32_t *sc;
  float *sb, *sv;
  unsigned long long *chk;
  const int64_t ns = direct ? 1 : nn;
  CK(cudaMallocAsync((void **)&sc, sizeof(uint32_t) * ns, s));
  CK(cudaMallocAsync((void **)&sb, sizeof(float) * 3 * ns, s));
  CK(cudaMallocAsync((void **)&sv, sizeof(float) * 3 * ns, s));
  CK(cudaMallocAsync((void **)&chk, 2 * sizeof(unsigned long long), s));
  uint32_t wmask = 0;
  for (int k = 0; k < MPG_MAX_SPECIES; ++k)
    if (c->weight_set[k]) wmask |= 1u << k;
  unsigned long long h_chk[2] = {~0ull, 0ull};
  CK(cudaMemcpyAsync(chk, h_chk, sizeof(h_chk), cudaMemcpyHostToDevice, s));
  const int other = 1 - c->cur;
  if (direct) {
    // checked, packed into the free buffer and deposited in one pass over
    // the host arrays (the deposit costs nothing beside the reads over the
    // host link); it replaces the resident list only if every word passed
    ensure_qfix(c);
    CK(cudaMemsetAsync(c->acc, 0, sizeof(unsigned long long) * 4 * c->dm.T, s));
    launch_mixed_pack_checked(s, hc, hb, hv, c->mp[other], n, c->hm.T, wmask, chk, c->dm, c->sp, c->acc);
    CKL();
  } else if (n > 0) {
    CK(cudaMemcpyAsync(sc, cellsp, sizeof(uint32_t) * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(sb, b, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(sv, v, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, s));
    launch_mixed_check(s, sc, n, c->hm.T, wmask, chk);
    CKL();
  }
  CK(cudaMemcpyAsync(h_chk, chk, sizeof(h_chk), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  int rc = MPG_OK;
  if (h_chk[0] != ~0ull) {
    const int64_t i = (int64_t)h_chk[0];
    if ((int64_t)(cellsp[i] & 0xFFFFFFu) >= c->hm.T || (cellsp[i] >> 24) >= MPG_MAX_SPECIES)
      rc = fail(c, MPG_ERR_ARG, "cellsp[%lld] out of range", (long long)i);
    else
      rc = fail(c, MPG_ERR_STATE, "species %u has no weight (fill or upload it first)", cellsp[i] >> 24);
  } else if (direct) {
    if (c->mp[c->cur].id && c->mp[other].id)
      CK(cudaMemcpyAsync(c->mp[other].id, c->mp[c->cur].id, sizeof(int64_t) * n, cudaMemcpyDeviceToDevice, s));
    c->cur = other;
  } else if (n > 0) {
    CK(cudaMemcpyAsync(c->mp[c->cur].c, sc, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, s));
    launch_mixed_pack(s, sb, sv, c->mp[c->cur], n);
    CKL();
  }
  CK(cudaFreeAsync(sc, s));
  CK(cudaFreeAsync(sb, s));
  CK(cudaFreeAsync(sv, s));
  CK(cudaFreeAsync(chk, s));
  CK(cudaStreamSynchronize(s));
  if (rc != MPG_OK) {
    if (direct) c->acc_valid = false;  // the slots hold a partial deposit of the rejected list
    return rc;
  }
  c->n = n;
  c->n_live = (int64_t)h_chk[1];
  c->acc_valid = direct;  // the direct path deposited the new list
  c->needs_sort = true;
  c->starts_valid = false;
  return MPG_OK;
}

int mpg_charge_download(mpg_ctx *c, int64_t *acc, double *quantum, int64_t *qfix) {
  ENTER(c);
  TRY(settle_sort(c));
  if (!c->configured) return fail(c, MPG_ERR_STATE, "not configured");
  if (c->cfg.precision != MPG_MIXED) return fail(c, MPG_ERR_STATE, "charge accumulator exists in the mixed form only");
  ensure_qfix(c);
  if (!c->acc_valid && c->parts_alloc) {
    CK(cudaMemsetAsync(c->acc, 0, sizeof(unsigned long long) * 4 * c->dm.T, c->stream));
    launch_mixed_deposit(c->stream, c->mp[c->cur], c->n, c->dm, c->sp, c->acc);
    CKL();
    c->acc_valid = true;
  }
  if (acc) {
    launch_node_quanta(c->stream, c->dm, c->acc, c->acc_node);
    CKL();
    CK(cudaMemcpyAsync(acc, c->acc_node, sizeof(int64_t) * c->dm.N, cudaMemcpyDeviceToHost, c->stream));
  }
  CK(cudaStreamSynchronize(c->stream));
  if (quantum) *quantum = c->quantum;
  if (qfix)
    for (int i = 0; i < MPG_MAX_SPECIES; ++i) qfix[i] = c->sp.qfix[i];
  return MPG_OK;
}

int mpg_weight_charge(mpg_ctx *c) {
  ENTER(c);
  TRY(settle_sort(c));
  TRY(ensure_particles(c));
  if (c->cfg.precision == MPG_MIXED) {
    c->acc_valid = false;
    TRY(phase_deposit_mixed(c));
  } else {
    TRY(phase_deposit_plain(c));
  }
  CK(cudaStreamSynchronize(c->stream));
  return MPG_OK;
}

int mpg_solve(mpg_ctx *c, int *iters, double *resid) {
  ENTER(c);
  if (!c->configured) return fail(c, MPG_ERR_STATE, "not configured");
  TRY(zero_stats(c));
  TRY(phase_solve(c));
  TRY(sync_stats(c));
  if (iters) *iters = c->h_stats->solver_iters;
  if (resid) *resid = c->h_stats->solver_resid;
  if (c->h_stats->solver_status) return fail(c, MPG_ERR_NOT_CONVERGED, "solver reached max_iter");
  return MPG_OK;
}

int mpg_weight_efield(mpg_ctx *c) {
  ENTER(c);
  if (!c->configured) return fail(c, MPG_ERR_STATE, "not configured");
  TRY(phase_efield(c, false));
  CK(cudaStreamSynchronize(c->stream));
  return MPG_OK;
}

int mpg_move(mpg_ctx *c, double dt, mpg_step_stats *st) {
  ENTER(c);
  TRY(settle_sort(c));
  TRY(ensure_particles(c));
  mpg_step_stats acc{};
  TRY(zero_stats(c));
  c->starts_valid = false;
  if (c->cfg.precision == MPG_MIXED) {
    // the fused kernel also deposits; keep the accumulator consistent
    CK(cudaMemsetAsync(c->acc, 0, sizeof(unsigned long long) * 4 * c->dm.T, c->stream));
    ensure_qfix(c);
    launch_mixed_move(c->stream, c->mp[c->cur], c->n, c->dm, c->sp, (float)dt, c->cfg.kill_on_wall,
                      c->cfg.max_crossings, c->acc, c->d_stats);
    CKL();
    c->acc_valid = true;
    TRY(sync_stats(c));
  } else {
    launch_plain_move(c->stream, c->pp[c->cur], c->n, c->dm, c->Etet, c->sp, dt, c->cfg.kill_on_wall,
                      c->cfg.max_crossings, c->d_stats);
    CKL();
    TRY(sync_stats(c));
    if (c->h_stats->n_killed > 0) TRY(compact_plain(c));
  }
  const DevStats &h = *c->h_stats;
  acc.ke = h.ke;
  acc.n_killed = (int64_t)h.n_killed;
  acc.n_crossings = (int64_t)h.n_cross;
  acc.n_walk_limit = (int64_t)h.n_limit;
  if (c->cfg.precision == MPG_MIXED)
    c->n_live -= (int64_t)h.n_killed;
  else
    c->n_live = c->n;
  acc.n_alive = c->n_live;
  acc.steps = 1;
  if (st) *st = acc;
  if (h.n_limit) return fail(c, MPG_ERR_WALK_LIMIT, "%llu particles hit max_crossings", h.n_limit);
  return MPG_OK;
}

int mpg_step(mpg_ctx *c, double dt, int n_steps, mpg_step_stats *st) {
  ENTER(c);
  TRY(ensure_particles(c));
  if (n_steps < 0) return fail(c, MPG_ERR_ARG, "n_steps < 0");
  mpg_step_stats acc{};
  TRY(zero_stats(c));
  const int64_t launches0 = c->launches;
  bool sorted = false;
  int rc = MPG_OK;
  for (int i = 0; i < n_steps && rc == MPG_OK; ++i) rc = one_step(c, dt, &acc, sorted);
  // the counts are brought up to date after a failed step too
  TRY(fetch_stats(c));
  TRY(finish_counts_mixed(c, sorted));
  const DevStats &h = *c->h_stats;
  acc.ke = h.ke;
  if (c->cfg.precision == MPG_MIXED) {
    acc.n_killed = (int64_t)h.n_killed;
  } else {
    acc.n_killed += (int64_t)h.n_killed;
  }
  acc.n_crossings = (int64_t)h.n_cross;
  acc.n_walk_limit = (int64_t)h.n_limit;
  acc.solver_iters = h.iters_total;
  acc.solver_resid = h.solver_resid;
  acc.steps = n_steps;
  acc.n_launches = c->launches - launches0;
  if (c->cfg.precision == MPG_MIXED)
    c->n_live -= (int64_t)h.n_killed;
  else
    c->n_live = c->n;
  acc.n_alive = c->n_live;
  acc.status = rc ? rc
                  : h.bar_error ? MPG_ERR_TIMEOUT
                  : h.solver_fail ? MPG_ERR_NOT_CONVERGED
                  : (h.n_limit ? MPG_ERR_WALK_LIMIT : MPG_OK);
  if (st) *st = acc;
  if (rc) return rc;  // the failed step set the message
  if (h.bar_error) return fail(c, MPG_ERR_TIMEOUT, "solver grid barrier timed out");
  if (h.solver_fail) return fail(c, MPG_ERR_NOT_CONVERGED, "a field solve reached max_iter");
  if (h.n_limit) return fail(c, MPG_ERR_WALK_LIMIT, "%llu particles hit max_crossings", h.n_limit);
  return MPG_OK;
}

int mpg_sort(mpg_ctx *c) {
  ENTER(c);
  TRY(settle_sort(c));
  TRY(ensure_particles(c));
  if (c->cfg.precision == MPG_MIXED) {
    TRY(sort_mixed(c));
    TRY(finish_counts_mixed(c, true));
  } else {
    // on request only: the plain step keeps the reference's Serial list order
    TRY(sort_plain(c));
  }
  CK(cudaStreamSynchronize(c->stream));
  return MPG_OK;
}

int mpg_set_barrier_test(mpg_ctx *c, int skip_block, unsigned poll_limit) {
  ENTER(c);
  c->cg.bar_skip = skip_block >= 0 ? skip_block + 1 : 0;
  c->cg.bar_limit = poll_limit;
  return MPG_OK;
}

int mpg_cell_starts(mpg_ctx *c, int64_t len, int64_t *start) {
  ENTER(c);
  if (!c->has_mesh) return fail(c, MPG_ERR_STATE, "no mesh");
  const int64_t T = c->dm.T;
  if (!start || len < T + 1) return fail(c, MPG_ERR_ARG, "start needs T + 1 = %lld entries", (long long)(T + 1));
  if (!c->starts_valid || !c->sort_start)
    return fail(c, MPG_ERR_STATE, "particles changed since the last sort: call mpg_sort first");
  std::vector<uint32_t> tmp(T + 1);
  CK(cudaMemcpyAsync(tmp.data(), c->sort_start, sizeof(uint32_t) * (T + 1), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  for (int64_t e = 0; e <= T; ++e) start[e] = tmp[e];
  return MPG_OK;
}

int mpg_get_field(mpg_ctx *c, int which, double *host) {
  ENTER(c);
  if (!c->configured || !host) return fail(c, MPG_ERR_STATE, "not configured");
  const int64_t N = c->dm.N, T = c->dm.T;
  cudaStream_t s = c->stream;
  if (which == MPG_FIELD_RHS) {
    CK(cudaMemcpyAsync(host, c->rhs, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
  } else if (which == MPG_FIELD_PHI) {
    CK(cudaMemcpyAsync(host, c->phi, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
  } else if (which == MPG_FIELD_BACKGROUND) {
    if (c->bg)
      CK(cudaMemcpyAsync(host, c->bg, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
    else
      memset(host, 0, sizeof(double) * N);
  } else if (which == MPG_FIELD_E_TET) {
    if (c->cfg.precision == MPG_MIXED && c->dm.kuhn) {
      std::vector<float4> e4(T);
      CK(cudaMemcpyAsync(e4.data(), c->dm.etet4, sizeof(float4) * T, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      for (int64_t t = 0; t < T; ++t) {
        host[3 * t] = e4[t].x;
        host[3 * t + 1] = e4[t].y;
        host[3 * t + 2] = e4[t].z;
      }
    } else if (c->cfg.precision == MPG_MIXED) {
      std::vector<float> rec(12 * T);
      CK(cudaMemcpyAsync(rec.data(), c->dm.mrec, sizeof(float) * 12 * T, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      for (int64_t t = 0; t < T; ++t)
        for (int d = 0; d < 3; ++d) host[3 * t + d] = rec[12 * t + 9 + d];
    } else {
      CK(cudaMemcpyAsync(host, c->Etet, sizeof(double) * 3 * T, cudaMemcpyDeviceToHost, s));
    }
  } else {
    return fail(c, MPG_ERR_ARG, "unknown field %d", which);
  }
  CK(cudaStreamSynchronize(s));
  return MPG_OK;
}

int mpg_set_field(mpg_ctx *c, int which, const double *host) {
  ENTER(c);
  if (!c->configured || !host) return fail(c, MPG_ERR_STATE, "not configured");
  const int64_t N = c->dm.N;
  if (which == MPG_FIELD_RHS)
    CK(cudaMemcpyAsync(c->rhs, host, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream));
  else if (which == MPG_FIELD_PHI) {
    CK(cudaMemcpyAsync(c->phi, host, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream));
    c->phi_hist = 1;  // the given phi is the only history
  } else
    return fail(c, MPG_ERR_ARG, "field %d is not settable", which);
  CK(cudaStreamSynchronize(c->stream));
  return MPG_OK;
}

int mpg_cg_csr(mpg_ctx *c, int64_t n, const int32_t *d_rowptr, const int32_t *d_col, const double *d_val,
               const double *d_b, double *d_x, double tol, int max_iter, int *iters, double *resid) {
  ENTER(c);
  if (n <= 0 || !d_rowptr || !d_col || !d_val || !d_b || !d_x) return fail(c, MPG_ERR_ARG, "bad CSR arguments");
  if (!(tol > 0) || max_iter < 1) return fail(c, MPG_ERR_ARG, "tol and max_iter must be positive");
  TRY(ensure_cg_work(c, n));
  TRY(zero_stats(c));
  int rc = run_cg64(c->stream, c->device, n, d_rowptr, d_col, d_val, d_b, d_x, tol, max_iter, c->cg, c->d_stats);
  if (rc) return fail(c, rc, "CG launch failed: %s", cudaGetErrorString(cudaGetLastError()));
  TRY(sync_stats(c));
  if (iters) *iters = c->h_stats->solver_iters;
  if (resid) *resid = c->h_stats->solver_resid;
  if (c->h_stats->solver_status) return fail(c, MPG_ERR_NOT_CONVERGED, "CG reached max_iter");
  return MPG_OK;
}

}  // extern "C"
