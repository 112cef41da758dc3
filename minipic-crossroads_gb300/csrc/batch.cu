// batch.cu -- batched ensemble / serving engine (mpg_batch_*).
//
// Many independent runs stay resident on one GPU and advance together.  Every
// run owns its mesh tables, field vectors and solver vectors (separate device
// buffers, addressed through a per-slot table SlotDev in device memory); all
// runs share one particle array whose 8-bit species field holds the run slot
// (cellsp = slot << 24 | local cell).  One step of the whole batch is one
// launch per phase:
//   k_batch_convert  fixed-point charge -> rhs, per (run, node block)
//   k_batch_cg       mixed CG of every run: a cooperative grid in which each
//                    run gets its own group of CTAs and its own group barrier
//                    (small runs one CTA, no grid-wide barrier at all)
//   k_batch_efield   per (run, tet block)
//   k_batch_move     fused push/walk/deposit over the particle array, the same
//                    per-particle code as the single-run kernel (mpg_walk.cuh)
// plus a counting sort by (run, cell) every sort_interval steps, which also
// drops the particles of retired runs.  The steps run from a captured CUDA
// graph, re-captured when the set of runs or the particle count changes.
//
// The field operator of a batched run is the 15-point Kuhn stencil of its
// mesh (FP32 inner CG, FP64 outer residual): constant coefficients on a
// uniform mesh, so such a run carries no matrix; per-row coefficients (15
// diagonals, FP64 and FP32 copies) on a mesh with jittered interior nodes.  Nothing a kernel computes for one run reads another run's
// data, and every per-run reduction has a fixed order, so a run's field and
// particle state do not depend on which runs share the batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "minipic_gb300.h"
#include "mpg_internal.h"
#include "mpg_kernels.h"
#include "mpg_mg.cuh"
#include "mpg_walk.cuh"

namespace {

constexpr int kMaxSlots = 256;  // the 8-bit run field of cellsp
constexpr int kND = 15;      // Kuhn stencil
constexpr int kMaxParts = 64;  // CTAs of one run in the solver

struct SlotDev {
  const float4 *rec;
  const uint4 *nbr;
  const int4 *tets;
  const uint8_t *bnd;
  const float *fill_ratio;
  unsigned long long *acc;   // fixed-point charge slots, one per (tet, corner), grouped by node (4T)
  const int32_t *n2c_off;    // N+1: node i's slots are acc[n2c_off[i] .. n2c_off[i+1])
  const int4 *c2n;           // T: the slots of tet t's four corners
  double *rhs, *phi, *bg, *r64;
  float *r[2], *p[2], *q[2], *z;
  double *partials;  // 8 * kMaxParts slots (outer phases); inner phases: one 32-byte record per part
  double *phi_prev;  // previous solution (initial guess 2 phi[n-1] - phi[n-2])
  int *hist;         // solutions held in phi / phi_prev (0, 1, 2), kept on the device
  int64_t T, N;
  int off[kND];
  double s64[kND];
  float s32[kND];
  // jittered mesh: row i's coefficient of diagonal d at v64[d * N + i] (FP64)
  // and v32 (FP32); null on a uniform mesh (s64 / s32 for every row)
  const double *v64;
  const float *v32;
  // multigrid state of a run solved by one CTA (its inner solve is then the
  // multigrid-preconditioned CG of the single-run solver); null: plain inner CG
  const mgpass::CgMgArgs *mg;
  double quantum;
  int Q;
  float hk, dt;
  double tol2, inner_tol2, safety2;  // safety2: inner stop at safety2 * tol2 |b|^2 / |r64|^2 as well
  int max_iter, max_cross;
  int active;    // stepped
  int resident;  // particles kept
};

struct SlotStat {
  double ke;
  unsigned long long killed, cross, limit;
  double resid;
  int iters;
  int status;
  unsigned bar;
  int bar_error;
};

// ---------------------------------------------------------------------------
// also forms the solver's initial guess: 2 phi[n-1] - phi[n-2] once two
// solutions exist (the count is advanced by the solver after it finishes)
constexpr int kPlanChunk = 256;  // elements (nodes or tets) per plan entry

__device__ __forceinline__ void batch_convert_at(const SlotDev &S, int64_t i) {
  if (i >= S.N) return;
  const int h = *S.hist;
  if (h >= 2) {
    const double a = S.phi[i];
    S.phi[i] = 2.0 * a - S.phi_prev[i];
    S.phi_prev[i] = a;
  } else if (h == 1) {
    S.phi_prev[i] = S.phi[i];
  }
  const long long a = slot_sum(S.acc, S.n2c_off[i], S.n2c_off[i + 1]);
  double r = -((double)a * S.quantum);
  if (S.bg) r += S.bg[i];
  if (S.bnd[i]) r = 0.0;
  S.rhs[i] = r;
}

__global__ void k_batch_convert(const SlotDev *__restrict__ slots, const int2 *__restrict__ plan) {
  const int2 pl = plan[blockIdx.x];
  batch_convert_at(slots[pl.x], (int64_t)pl.y * kPlanChunk + threadIdx.x);
}

__device__ __forceinline__ void batch_efield_at(const SlotDev &S, int64_t t) {
  if (t >= S.T) return;
  const int4 nd = S.tets[t];
  const double f0 = S.phi[nd.x];
  const float d1 = (float)(S.phi[nd.y] - f0), d2 = (float)(S.phi[nd.z] - f0), d3 = (float)(S.phi[nd.w] - f0);
  float4 *rec = const_cast<float4 *>(S.rec);
  const float4 r0 = rec[3 * t], r1 = rec[3 * t + 1];
  float4 r2 = rec[3 * t + 2];
  r2.y = __fmaf_rn(d3, r1.z, __fmaf_rn(d2, r0.w, d1 * r0.x));
  r2.z = __fmaf_rn(d3, r1.w, __fmaf_rn(d2, r1.x, d1 * r0.y));
  r2.w = __fmaf_rn(d3, r2.x, __fmaf_rn(d2, r1.y, d1 * r0.z));
  rec[3 * t + 2] = r2;
  // the charge slots were read by k_batch_convert; zero them for the move
  ulonglong2 *a2 = reinterpret_cast<ulonglong2 *>(S.acc + 4 * t);
  a2[0] = make_ulonglong2(0ull, 0ull);
  a2[1] = make_ulonglong2(0ull, 0ull);
}

__global__ void k_batch_efield(const SlotDev *__restrict__ slots, const int2 *__restrict__ plan) {
  const int2 pl = plan[blockIdx.x];
  batch_efield_at(slots[pl.x], (int64_t)pl.y * kPlanChunk + threadIdx.x);
}

// warp-aggregated fixed-point deposit keyed by the full cellsp word (runs
// never merge); the tail lane of a run of equal keys issues the atomics
__device__ __forceinline__ void batch_deposit_warp(const SlotDev *__restrict__ slots, uint32_t key, float b1, float b2,
                                                   float b3, int Q) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const bool valid = key != MPG_DEAD;
  int c0 = 0, c1 = 0, c2 = 0, c3 = 0;
  if (valid) {
    const float Qf = (float)Q;
    c1 = __float2int_rn(b1 * Qf);
    c2 = __float2int_rn(b2 * Qf);
    c3 = __float2int_rn(b3 * Qf);
    c0 = Q - c1 - c2 - c3;
  }
  const uint32_t prev = __shfl_up_sync(FULL, key, 1);
  const bool head = lane == 0 || prev != key;
  const unsigned heads = __ballot_sync(FULL, head);
  if (heads == 1u) {
    // the whole warp holds one cell (typical after a sort): plain reductions
    c0 = __reduce_add_sync(FULL, c0);
    c1 = __reduce_add_sync(FULL, c1);
    c2 = __reduce_add_sync(FULL, c2);
    c3 = __reduce_add_sync(FULL, c3);
    if (lane == 0 && valid) {
      const SlotDev &S = slots[key >> 24];
      const int4 q = S.c2n[key & 0xFFFFFFu];
      atomicAdd(S.acc + q.x, (unsigned long long)(long long)c0);
      atomicAdd(S.acc + q.y, (unsigned long long)(long long)c1);
      atomicAdd(S.acc + q.z, (unsigned long long)(long long)c2);
      atomicAdd(S.acc + q.w, (unsigned long long)(long long)c3);
    }
    return;
  }
  const int seg = 31 - __clz(heads & (FULL >> (31 - lane)));
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int su = __shfl_up_sync(FULL, seg, o);
    const int u0 = __shfl_up_sync(FULL, c0, o);
    const int u1 = __shfl_up_sync(FULL, c1, o);
    const int u2 = __shfl_up_sync(FULL, c2, o);
    const int u3 = __shfl_up_sync(FULL, c3, o);
    if (lane >= o && su == seg) {
      c0 += u0;
      c1 += u1;
      c2 += u2;
      c3 += u3;
    }
  }
  const int sn = __shfl_down_sync(FULL, seg, 1);
  const bool tail = lane == 31 || sn != seg;
  if (tail && valid) {
    const SlotDev &S = slots[key >> 24];
    const int4 q = S.c2n[key & 0xFFFFFFu];
    atomicAdd(S.acc + q.x, (unsigned long long)(long long)c0);
    atomicAdd(S.acc + q.y, (unsigned long long)(long long)c1);
    atomicAdd(S.acc + q.z, (unsigned long long)(long long)c2);
    atomicAdd(S.acc + q.w, (unsigned long long)(long long)c3);
  }
}

constexpr int kMoveThreads = 256;

// Persistent: one wave of resident blocks; each warp walks a contiguous range
// of 32-particle chunks and loads the next chunk's records before it
// processes the current one.  After the (run, cell) sort a run's particles are
// contiguous, so a lane's particles mostly belong to one run: the lane keeps
// that run's statistics in registers (kinetic energy per unit mass in
// float-float) and adds them to the run's counters when its run changes.
__device__ __forceinline__ void batch_move_body(MixedParts P, int64_t n, const SlotDev *__restrict__ slots,
                                                SlotStat *stats, int kill) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nchunks = (n + 31) >> 5;
  const int64_t per = (nchunks + nw - 1) / nw;
  int64_t c = w * per;
  const int64_t cend = c + per < nchunks ? c + per : nchunks;
  int cur = -1;
  ff ke = {0.f, 0.f};
  unsigned kl = 0, cr = 0, lm = 0;
  auto flush = [&]() {
    if (cur >= 0) {
      const double e = (double)ke.hi + (double)ke.lo;
      if (e != 0.0) atomicAdd(&stats[cur].ke, e);
      if (kl) atomicAdd(&stats[cur].killed, (unsigned long long)kl);
      if (cr) atomicAdd(&stats[cur].cross, (unsigned long long)cr);
      if (lm) atomicAdd(&stats[cur].limit, (unsigned long long)lm);
    }
    ke = ff{0.f, 0.f};
    kl = cr = lm = 0;
  };
  uint32_t cs_n = MPG_DEAD;
  float4 bv_n = make_float4(0.f, 0.f, 0.f, 0.f);
  float2 vv_n = make_float2(0.f, 0.f);
  if (c < cend) {
    const int64_t p = c * 32 + lane;
    if (p < n) {
      cs_n = P.c[p];
      bv_n = P.b[p];
      vv_n = P.v[p];
    }
  }
  for (; c < cend; ++c) {
    const int64_t p = c * 32 + lane;
    const uint32_t cs = cs_n;
    const float4 bv = bv_n;
    const float2 vv = vv_n;
    cs_n = MPG_DEAD;
    if (c + 1 < cend) {
      const int64_t q = p + 32;
      if (q < n) {
        cs_n = P.c[q];
        bv_n = P.b[q];
        vv_n = P.v[q];
      }
    }
    uint32_t key = MPG_DEAD;
    float d1 = 0.f, d2 = 0.f, d3 = 0.f;
    int dq = 0;
    if (p < n && cs != MPG_DEAD) {
      const int slot = (int)(cs >> 24);
      const SlotDev &S = slots[slot];
      if (S.active) {
        if (slot != cur) {
          flush();
          cur = slot;
        }
        uint32_t e = cs & 0xFFFFFFu;
        float l1 = bv.x, l2 = bv.y, l3 = bv.z;
        float vx = bv.w, vy = vv.x, vz = vv.y;
        bool dead, lim;
        const int it = mixed_walk(S.rec, S.nbr, e, l1, l2, l3, vx, vy, vz, S.hk, S.dt, kill, S.max_cross, dead, lim);
        cr += (unsigned)it;
        lm += lim ? 1u : 0u;
        if (dead) {
          kl += 1;
          P.c[p] = MPG_DEAD;
        } else {
          if (e != (cs & 0xFFFFFFu)) P.c[p] = ((uint32_t)slot << 24) | e;
          P.b[p] = make_float4(l1, l2, l3, vx);
          P.v[p] = make_float2(vy, vz);
          // kinetic energy per unit mass; scaled by w m / 2 on the host
          ke = ff_add(ke, ff{__fmaf_rn(vz, vz, __fmaf_rn(vy, vy, vx * vx)), 0.f});
          key = ((uint32_t)slot << 24) | e;
          d1 = l1;
          d2 = l2;
          d3 = l3;
          dq = S.Q;
        }
      }
    }
    // every lane of the warp is here (c is uniform across the warp)
    batch_deposit_warp(slots, key, d1, d2, d3, dq);
  }
  flush();
}

__global__ void __launch_bounds__(kMoveThreads) k_batch_move(MixedParts P, int64_t n, const SlotDev *__restrict__ slots,
                                                             SlotStat *stats, int kill) {
  batch_move_body(P, n, slots, stats, kill);
}

// resident blocks of the persistent batch move on the current device (one wave)
unsigned batch_move_blocks(int device) {
  static int cached[64] = {0};
  if (device < 0 || device >= 64) device = 0;
  if (!cached[device]) {
    int sms = 0, occ = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_batch_move, kMoveThreads, 0);
    cached[device] = (sms > 0 ? sms : 1) * (occ > 0 ? occ : 1);
  }
  return (unsigned)cached[device];
}

// initial deposit of newly admitted particles [n0, n1)
__global__ void k_batch_deposit(MixedParts P, int64_t n0, int64_t n1, const SlotDev *__restrict__ slots) {
  const int64_t p = n0 + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t key = MPG_DEAD;
  float b1 = 0.f, b2 = 0.f, b3 = 0.f;
  int Q = 0;
  if (p < n1) {
    const uint32_t cs = P.c[p];
    if (cs != MPG_DEAD) {
      const float4 b = P.b[p];
      key = cs;
      b1 = b.x;
      b2 = b.y;
      b3 = b.z;
      Q = slots[cs >> 24].Q;
    }
  }
  batch_deposit_warp(slots, key, b1, b2, b3, Q);
}

__global__ void k_batch_kill_slot(uint32_t *c, int64_t n, int slot) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n && c[p] != MPG_DEAD && (int)(c[p] >> 24) == slot) c[p] = MPG_DEAD;
}

// counting sort by (run, cell): key = base[slot] + cell; particles of
// non-resident runs and dead particles are dropped
// Runs of equal (run, cell) words in a warp (particles stay nearly sorted
// between sorts): the run's first lane and the lane's rank within its run.
__device__ __forceinline__ void key_run(uint32_t key, int &first, int &rank, int &len) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const uint32_t prev = __shfl_up_sync(FULL, key, 1);
  const unsigned heads = __ballot_sync(FULL, lane == 0 || prev != key);
  first = 31 - __clz(heads & (FULL >> (31 - lane)));
  rank = lane - first;
  const unsigned after = heads & ~(FULL >> (31 - lane));
  len = (after ? __ffs(after) - 1 : 32) - first;
}

__global__ void k_batch_hist(const uint32_t *__restrict__ c, int64_t n, const int64_t *__restrict__ base,
                             uint32_t *__restrict__ cnt) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t cs = p < n ? c[p] : MPG_DEAD;
  if (cs != MPG_DEAD && base[cs >> 24] < 0) cs = MPG_DEAD;
  int first, rank, len;
  key_run(cs, first, rank, len);
  if (rank == 0 && cs != MPG_DEAD) atomicAdd(&cnt[base[cs >> 24] + (cs & 0xFFFFFFu)], (unsigned)len);
}

// one atomic per run of equal keys; lanes of a run keep their order
__global__ void k_batch_scatter(MixedParts P, int64_t n, MixedParts Q, const int64_t *__restrict__ base,
                                const uint32_t *__restrict__ start, uint32_t *__restrict__ fill) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t cs = p < n ? P.c[p] : MPG_DEAD;
  if (cs != MPG_DEAD && base[cs >> 24] < 0) cs = MPG_DEAD;
  int first, rank, len;
  key_run(cs, first, rank, len);
  const int64_t k = cs != MPG_DEAD ? base[cs >> 24] + (cs & 0xFFFFFFu) : 0;
  uint32_t off = 0;
  if (rank == 0 && cs != MPG_DEAD) off = atomicAdd(&fill[k], (unsigned)len);
  off = __shfl_sync(0xffffffffu, off, first);
  if (cs == MPG_DEAD) return;
  const uint32_t dst = start[k] + off + (uint32_t)rank;
  Q.c[dst] = cs;
  Q.b[dst] = P.b[p];
  Q.v[dst] = P.v[p];
}

__global__ void k_batch_copy_count(const uint32_t *start, int64_t k, uint32_t *out) { *out = start[k]; }

// ---------------------------------------------------------------------------
// batched mixed CG.  One work item = (slot, part, nparts): the rows
// [N*part/nparts, N*(part+1)/nparts) of one run, solved together with the
// other parts of that run through the run's group barrier.
__device__ __forceinline__ bool group_barrier(SlotStat *st, int nparts, unsigned &epoch) {
  if (nparts == 1) {
    __syncthreads();
    return true;
  }
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    ++epoch;
    const unsigned target = epoch * (unsigned)nparts;
    __threadfence();
    atomicAdd(&st->bar, 1u);
    unsigned spins = 0;
    for (;;) {
      const unsigned v = *(volatile unsigned *)&st->bar;
      if ((int)(v - target) >= 0) break;
      ++spins;
      if ((spins & 255u) == 0) {
        if (*(volatile int *)&st->bar_error) {
          ok = 0;
          break;
        }
        if (spins > (1u << 22)) {
          atomicExch(&st->bar_error, 1);
          ok = 0;
          break;
        }
      }
      if (spins > 64) __nanosleep(32);
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

// The run's CTA group: part `part` of `nparts` takes the rows
// [n part / nparts, n (part + 1) / nparts) of every level; `sync` is the
// group barrier (a block barrier for a one-CTA run).
struct GroupRows {
  int part, nparts;
  __device__ void of(int64_t n, int64_t &lo, int64_t &hi) const {
    lo = n * part / nparts;
    hi = n * (part + 1) / nparts;
  }
};

// u = M r: the single-run solver's V-cycle with every level on the run's
// CTA group (group barriers between dependent passes).  Level 0's first
// pre-smoothing residual (from rf) is in place on this part's rows.
template <bool CST, typename Sync>
__device__ bool batch_vcycle(const mgpass::CgMgArgs &a, const float *rf, const GroupRows g, Sync sync) {
  using namespace mgpass;
  const MgDev &mg = a.mg;
  const int nl = mg.nlev;
  int64_t lo, hi, clo, chi;
  if (!sync()) return false;
  g.of(mg.lev[0].n, lo, hi);
  if (mg.nu0 == 2) {
    const float *__restrict__ t1 = mg.lev[0].t2;
    presmooth_residual<kND, CST>(a, 0, lo, hi, [&](int64_t j) { return t1[j]; }, mg.lev[0].t);
    if (!sync()) return false;
  }
  g.of(mg.lev[1].n, clo, chi);
  restrict_rows(a, 0, clo, chi);
  if (!sync()) return false;
  for (int l = 1; l < nl - 1; ++l) {
    g.of(mg.lev[l].n, lo, hi);
    g.of(mg.lev[l + 1].n, clo, chi);
    const bool ok = mg.nu1 == 2 ? level_down_twice<kND, CST>(a, l, lo, hi, clo, chi, sync)
                                : level_down<kND, CST>(a, l, lo, hi, clo, chi, sync);
    if (!ok) return false;
  }
  const int nw = blockDim.x >> 5;
  dense_solve_rows(mg, g.part * nw + (threadIdx.x >> 5), g.nparts * nw);
  if (!sync()) return false;
  for (int l = nl - 2; l >= 1; --l) {
    g.of(mg.lev[l].n, lo, hi);
    const bool ok = mg.nu1 == 2 ? level_up_twice<kND, CST>(a, l, lo, hi, mg.lev[l].r, mg.lev[l + 1].t, sync)
                                : level_up<kND, CST>(a, l, lo, hi, mg.lev[l].r, mg.lev[l + 1].t, sync);
    if (!ok) return false;
  }
  g.of(mg.lev[0].n, lo, hi);
  return mg.nu0 == 2 ? level_up_twice<kND, CST>(a, 0, lo, hi, rf, mg.lev[1].t, sync)
                     : level_up<kND, CST>(a, 0, lo, hi, rf, mg.lev[1].t, sync);
}

// inner solve of one FP64 refinement sweep for a run with a multigrid
// hierarchy: PCG on A z = r64 / |r64| in the single-reduction form of the
// single-run solver (one all-reduce of four float-float dots per iteration,
// through the part records and the group barrier when the run has several
// CTAs, summed in part order), z starting at 0, the search direction
// restarted each sweep.  False when a group barrier timed out.
template <bool CST, typename Sync>
__device__ bool batch_mg_inner(const mgpass::CgMgArgs &a, const GroupRows g, Sync sync, double scale,
                               float stop_rel, int &total_inner, int max_iter, ff *smf, double *partials,
                               int &phase) {
  using namespace mgpass;
  float *__restrict__ r = a.r[0];
  float *__restrict__ s = a.s[0];
  float *__restrict__ p = a.p;
  float *__restrict__ z = a.z;
  float *__restrict__ w = a.w;
  const float *__restrict__ u = a.u;
  int64_t lo, hi;
  g.of(a.mg.lev[0].n, lo, hi);
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    r[i] = (float)(a.r64[i] * scale);
    z[i] = 0.f;
    p[i] = 0.f;
    s[i] = 0.f;
  }
  if (!sync()) return false;
  presmooth_residual<kND, CST>(a, 0, lo, hi, [&](int64_t j) { return r[j]; }, first_residual(a));
  ff gam0 = {0.f, 0.f}, gam_prev = {0.f, 0.f};
  bool have_dir = false;
  for (int k = 0;; ++k) {
    if (!batch_vcycle<CST>(a, r, g, sync)) return false;
    ff v[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const float ui = u[i];
      const float wi = level_apply<kND, CST>(a, 0, [&](int64_t j) { return u[j]; }, i);
      const float si = s[i];
      w[i] = wi;
      v[0] = ff_add(v[0], ff_prod(r[i], ui));
      v[1] = ff_add(v[1], ff_prod(wi, ui));
      v[2] = ff_add(v[2], ff_prod(ui, si));
      v[3] = ff_add(v[3], ff_prod(p[i], si));
    }
    block_sum_ff<4>(v, smf);
    if (g.nparts > 1) {
      // part records (two float4 per part, sets alternating by phase), then
      // every part sums them in part order
      float4 *rec = reinterpret_cast<float4 *>(partials + (size_t)(phase & 1) * 4 * kMaxParts);
      if (threadIdx.x == 0) {
        rec[2 * g.part] = make_float4(v[0].hi, v[0].lo, v[1].hi, v[1].lo);
        rec[2 * g.part + 1] = make_float4(v[2].hi, v[2].lo, v[3].hi, v[3].lo);
      }
      ++phase;
      if (!sync()) return false;
      ff t[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
      for (int q = 0; q < g.nparts; ++q) {
        const float4 x = rec[2 * q], y = rec[2 * q + 1];
        t[0] = ff_add(t[0], ff{x.x, x.y});
        t[1] = ff_add(t[1], ff{x.z, x.w});
        t[2] = ff_add(t[2], ff{y.x, y.y});
        t[3] = ff_add(t[3], ff{y.z, y.w});
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) v[q] = t[q];
    }
    const ff G = v[0];
    if (k == 0) gam0 = G;
    if (!(G.hi > 0.f) || G.hi <= stop_rel * gam0.hi || total_inner >= max_iter) break;
    const float beta = have_dir ? G.hi / gam_prev.hi : 0.f;
    const ff den = ff_add(ff_add(v[1], ff_mulf(v[2], 2.f * beta)), ff_mulf(ff_mulf(v[3], beta), beta));
    const float alpha = G.hi / den.hi;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const float pi = __fmaf_rn(beta, p[i], u[i]);
      const float si = __fmaf_rn(beta, s[i], w[i]);
      p[i] = pi;
      s[i] = si;
      z[i] = __fmaf_rn(alpha, pi, z[i]);
      r[i] = __fmaf_rn(-alpha, si, r[i]);
    }
    if (!sync()) return false;
    presmooth_residual<kND, CST>(a, 0, lo, hi, [&](int64_t j) { return r[j]; }, first_residual(a));
    gam_prev = G;
    have_dir = true;
    ++total_inner;
  }
  return true;
}

template <int TH>
__device__ void solve_run(const SlotDev &S, SlotStat *st, const int part, const int nparts) {
  __shared__ double red[32];
  __shared__ ff smf[4 * 32];
  __shared__ float smw[4 * 32];
  __shared__ ff smt[4];
  __shared__ double bc;
  unsigned epoch = 0;
  const int64_t n = S.N;
  const int64_t lo = n * part / nparts, hi = n * (part + 1) / nparts;
  const uint8_t *__restrict__ bnd = S.bnd;
  auto slot64 = [&](int set, int k) { return S.partials + (size_t)(set * 4 + k) * kMaxParts; };
  auto slotff = [&](int set, int k) { return reinterpret_cast<float2 *>(slot64(set, k)); };
  auto put_ff = [&](int set, const ff *v, int K) {
    if (threadIdx.x == 0)
      for (int k = 0; k < K; ++k) slotff(set, k)[part] = make_float2(v[k].hi, v[k].lo);
  };
  auto total_ff = [&](int set, ff *out, int K) {
    ff v[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    for (int i = threadIdx.x; i < nparts; i += blockDim.x)
      for (int k = 0; k < K; ++k) {
        const float2 t = slotff(set, k)[i];
        v[k] = ff_add(v[k], ff{t.x, t.y});
      }
    block_sum_ff<4>(v, smf);
    for (int k = 0; k < K; ++k) out[k] = v[k];
  };
  auto total64 = [&](const double *p) {
    double s = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += p[i];
    s = block_sum(s, red);
    if (threadIdx.x == 0) bc = s;
    __syncthreads();
    const double v = bc;
    __syncthreads();
    return v;
  };
  int phase = 0;
  double bb = 0.0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) bb += S.rhs[i] * S.rhs[i];
  double t = block_sum(bb, red);
  if (threadIdx.x == 0) slot64(1, 3)[part] = t;
  int total_inner = 0, status = 0, sweeps = 0;
  double rho64 = 0.0, rho0 = 0.0;
  for (;; ++sweeps) {
    double rr = 0.0;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      double s = 0.0;
      if (bnd[i]) {
        S.phi[i] = S.rhs[i];
        s = S.phi[i];
      } else {
#pragma unroll
        for (int d = 0; d < kND; ++d) s = __fma_rn(S.v64 ? S.v64[d * S.N + i] : S.s64[d], S.phi[i + S.off[d]], s);
      }
      const double ri = S.rhs[i] - s;
      S.r64[i] = ri;
      rr += ri * ri;
    }
    int set = phase & 1;
    t = block_sum(rr, red);
    if (threadIdx.x == 0) slot64(set, 0)[part] = t;
    if (!group_barrier(st, nparts, epoch)) return;
    if (sweeps == 0) rho0 = total64(slot64(1, 3));
    rho64 = total64(slot64(set, 0));
    ++phase;
    if (rho0 == 0.0) {
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) S.phi[i] = 0.0;
      rho64 = 0.0;
      break;
    }
    if (rho64 <= S.tol2 * rho0) break;
    if (total_inner >= S.max_iter) {
      status = 1;
      break;
    }
    const double scale = 1.0 / sqrt(rho64);
    if (S.mg) {
      const float stop_rel = (float)fmax(S.inner_tol2, S.safety2 * S.tol2 * rho0 / rho64);
      const GroupRows g{part, nparts};
      auto gsync = [&]() { return group_barrier(st, nparts, epoch); };
      const bool ok = S.v32 ? batch_mg_inner<false>(*S.mg, g, gsync, scale, stop_rel, total_inner, S.max_iter, smf,
                                                    S.partials, phase)
                            : batch_mg_inner<true>(*S.mg, g, gsync, scale, stop_rel, total_inner, S.max_iter, smf,
                                                   S.partials, phase);
      if (!ok) return;
      const double back = sqrt(rho64);
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) S.phi[i] += (double)S.z[i] * back;
      if (!group_barrier(st, nparts, epoch)) return;
      continue;
    }
    float *r0 = S.r[0], *p0 = S.p[0];
    ff rs = {0.f, 0.f};
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const float ri = (float)(S.r64[i] * scale);
      r0[i] = ri;
      p0[i] = ri;
      S.z[i] = 0.f;
      rs = ff_add(rs, ff_prod(ri, ri));
    }
    set = phase & 1;
    block_sum_ff<1>(&rs, smf);
    put_ff(set, &rs, 1);
    if (!group_barrier(st, nparts, epoch)) return;
    ff rin0;
    total_ff(set, &rin0, 1);
    ++phase;
    {
      float *q0 = S.q[0];
      ff pq = {0.f, 0.f}, qq = {0.f, 0.f};
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const float pi = p0[i];
        float s;
        if (bnd[i]) {
          s = pi;
        } else {
          s = 0.f;
#pragma unroll
          for (int d = 0; d < kND; ++d) s = __fmaf_rn(S.v32 ? S.v32[d * S.N + i] : S.s32[d], p0[i + S.off[d]], s);
        }
        q0[i] = s;
        pq = ff_add(pq, ff_prod(pi, s));
        qq = ff_add(qq, ff_prod(s, s));
      }
      set = phase & 1;
      ff v3[3] = {pq, pq, qq};
      block_sum_ff<3>(v3, smf);
      put_ff(set, v3, 3);
    }
    if (!group_barrier(st, nparts, epoch)) return;
    ff tot[4];
    total_ff(phase & 1, tot, 3);
    ff pq = tot[0], rq = tot[1], qq = tot[2], rho = rin0;
    ++phase;
    int cur = 0;
    const float stop = (float)fmax(S.inner_tol2, S.safety2 * S.tol2 * rho0 / rho64) * rin0.hi;
    for (;;) {
      if (rho.hi <= stop || total_inner >= S.max_iter || !(pq.hi > 0.f)) break;
      const float af = rho.hi / pq.hi;
      ff rn = ff_add(rho, ff_mulf(rq, -2.f * af));
      rn = ff_add(rn, ff_mulf(ff_mulf(qq, af), af));
      const float bf = rn.hi > 0.f ? rn.hi / rho.hi : 0.f;
      // separate r, p, q arrays here (not one float4 per node as in the
      // single-run solver): a batch CTA holds many rows per thread, where the
      // row loop is bound by L1 bytes rather than load latency
      const float *rk = S.r[cur], *pk = S.p[cur], *qk = S.q[cur];
      float *rnx = S.r[cur ^ 1], *pnx = S.p[cur ^ 1], *qnx = S.q[cur ^ 1];
      ff dpq = {0.f, 0.f}, drq = {0.f, 0.f}, dqq = {0.f, 0.f}, drr = {0.f, 0.f};
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const float ri = __fmaf_rn(-af, qk[i], rk[i]);
        const float pi = __fmaf_rn(bf, pk[i], ri);
        S.z[i] = __fmaf_rn(af, pk[i], S.z[i]);
        float s;
        if (bnd[i]) {
          s = pi;
        } else {
          s = 0.f;
#pragma unroll
          for (int d = 0; d < kND; ++d) {
            const int64_t j = i + S.off[d];
            const float rj = __fmaf_rn(-af, qk[j], rk[j]);
            s = __fmaf_rn(S.v32 ? S.v32[d * S.N + i] : S.s32[d], __fmaf_rn(bf, pk[j], rj), s);
          }
        }
        rnx[i] = ri;
        pnx[i] = pi;
        qnx[i] = s;
        dpq = ff_add(dpq, ff_prod(pi, s));
        drq = ff_add(drq, ff_prod(ri, s));
        dqq = ff_add(dqq, ff_prod(s, s));
        drr = ff_add(drr, ff_prod(ri, ri));
      }
      set = phase & 1;
      {
        // block partials: FP32 warp trees, one float-float pass over the warp sums
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        float w4[4] = {dpq.hi + dpq.lo, drq.hi + drq.lo, dqq.hi + dqq.lo, drr.hi + drr.lo};
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
          for (int k = 0; k < 4; ++k) w4[k] += __shfl_down_sync(0xffffffffu, w4[k], o);
        if (lane == 0)
#pragma unroll
          for (int k = 0; k < 4; ++k) smw[k * 32 + wid] = w4[k];
        __syncthreads();
        if (wid == 0) {
          ff tt[4];
#pragma unroll
          for (int k = 0; k < 4; ++k) {
            tt[k] = ff{lane < TH / 32 ? smw[k * 32 + lane] : 0.f, 0.f};
            for (int o = 16; o > 0; o >>= 1) tt[k] = ff_add(tt[k], ff_shfl_down(tt[k], o));
          }
          if (lane == 0) {
            if (nparts == 1) {
#pragma unroll
              for (int k = 0; k < 4; ++k) smt[k] = tt[k];
            } else {
              float4 *rec = reinterpret_cast<float4 *>(slot64(set, 0)) + 2 * part;
              rec[0] = make_float4(tt[0].hi, tt[0].lo, tt[1].hi, tt[1].lo);
              rec[1] = make_float4(tt[2].hi, tt[2].lo, tt[3].hi, tt[3].lo);
            }
          }
        }
        if (nparts > 1) {
          if (!group_barrier(st, nparts, epoch)) return;
          // run totals: warp 0 sums the part records (at most 64) in part order
          if (wid == 0) {
            const float4 *rec = reinterpret_cast<const float4 *>(slot64(set, 0));
            ff tt[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
            for (int j = 0; j < 2; ++j) {
              const int q = lane + 32 * j;
              if (q < nparts) {
                const float4 x = rec[2 * q], y = rec[2 * q + 1];
                tt[0] = ff_add(tt[0], ff{x.x, x.y});
                tt[1] = ff_add(tt[1], ff{x.z, x.w});
                tt[2] = ff_add(tt[2], ff{y.x, y.y});
                tt[3] = ff_add(tt[3], ff{y.z, y.w});
              }
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
              for (int o = 16; o > 0; o >>= 1) tt[k] = ff_add(tt[k], ff_shfl_down(tt[k], o));
              if (lane == 0) smt[k] = tt[k];
            }
          }
        }
        __syncthreads();
      }
      pq = smt[0];
      rq = smt[1];
      qq = smt[2];
      rho = smt[3];
      ++phase;
      cur ^= 1;
      ++total_inner;
    }
    const double back = sqrt(rho64);
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) S.phi[i] += (double)S.z[i] * back;
    if (!group_barrier(st, nparts, epoch)) return;
  }
  if (part == 0 && threadIdx.x == 0) {
    st->iters = total_inner;
    st->status = status;
    st->resid = rho0 > 0.0 ? sqrt(rho64 / rho0) : 0.0;
    if (*S.hist < 2) ++*S.hist;
  }
}

template <int TH>
__global__ void __launch_bounds__(TH, 1024 / TH) k_batch_cg(const SlotDev *__restrict__ slots, SlotStat *stats,
                                                            const int4 *__restrict__ items,
                                                            const int2 *__restrict__ block_items) {
  const int2 rng = block_items[blockIdx.x];
  for (int k = rng.x; k < rng.y; ++k) {
    const int4 w = items[k];
    solve_run<TH>(slots[w.x], &stats[w.x], w.y, w.z);
    __syncthreads();
  }
}

void *batch_cg_kernel(int th) {
  return th <= 256 ? (void *)k_batch_cg<256> : th <= 512 ? (void *)k_batch_cg<512> : (void *)k_batch_cg<1024>;
}

// One persistent cooperative launch per batch step: the four phases of the
// step separated by grid barriers (bounded waits, as in the single-run
// solvers; a time-out ends the launch in every block).
//   1 charge -> rhs and the initial guess, grid-stride over the node plan;
//   2 the runs' field solves: block b < n_cg_blocks works its solver items
//     (each run's CTA group synchronises on its own group barrier), the
//     other blocks go straight to the barrier;
//   3 E per tet (and zeroed charge slots), grid-stride over the tet plan;
//   4 the fused push/walk/deposit over the particle array.
struct BatchStepArgs {
  const SlotDev *slots;
  SlotStat *stats;
  const int2 *conv_plan, *ef_plan, *block_items;
  const int4 *items;
  int n_conv, n_ef, n_cg_blocks;
  MixedParts P;
  int64_t n;
  DevStats *gbar;
};

template <int TH>
__global__ void __launch_bounds__(TH, 1024 / TH) k_batch_step(BatchStepArgs a) {
  static_assert(TH % kPlanChunk == 0, "block size is a multiple of the plan chunk");
  constexpr int kPer = TH / kPlanChunk;  // plan entries per block and pass
  unsigned epoch = 0;
  const int sub = threadIdx.x / kPlanChunk, t = threadIdx.x % kPlanChunk;
  for (int e = blockIdx.x * kPer + sub; e < a.n_conv; e += gridDim.x * kPer) {
    const int2 pl = a.conv_plan[e];
    batch_convert_at(a.slots[pl.x], (int64_t)pl.y * kPlanChunk + t);
  }
  if (!grid_barrier(a.gbar, gridDim.x, epoch)) return;
  if ((int)blockIdx.x < a.n_cg_blocks) {
    const int2 rng = a.block_items[blockIdx.x];
    for (int k = rng.x; k < rng.y; ++k) {
      const int4 w = a.items[k];
      solve_run<TH>(a.slots[w.x], &a.stats[w.x], w.y, w.z);
      __syncthreads();
    }
  }
  if (!grid_barrier(a.gbar, gridDim.x, epoch)) return;
  for (int e = blockIdx.x * kPer + sub; e < a.n_ef; e += gridDim.x * kPer) {
    const int2 pl = a.ef_plan[e];
    batch_efield_at(a.slots[pl.x], (int64_t)pl.y * kPlanChunk + t);
  }
  if (!grid_barrier(a.gbar, gridDim.x, epoch)) return;
  if (a.n > 0) batch_move_body(a.P, a.n, a.slots, a.stats, 1);
}

void *batch_step_kernel(int th) {
  return th <= 256 ? (void *)k_batch_step<256> : th <= 512 ? (void *)k_batch_step<512> : (void *)k_batch_step<1024>;
}

// ---------------------------------------------------------------------------
struct Run {
  bool used = false, active = false, finished = false;
  mpg_run_desc d{};
  int64_t T = 0, N = 0, n_alive = 0, bytes = 0;
  int steps_done = 0;
  std::vector<void *> bufs;
  SlotDev dev{};
  mpg_run_info last{};
};

}  // namespace

// host-side part of an admission (mpg_batch_prepare): the run's mesh, its
// uniform stencil and the tables uploaded at admission
struct mpg_run_prep {
  mpg_run_desc d{};
  HostMesh hm;
  int off[kND] = {};
  double s64[kND] = {};
  std::vector<double> d64;  // jittered mesh: per-row coefficients by diagonal (kND x N), else empty
  std::vector<float> d32;   // the same in FP32
  std::vector<float> recv, ratio;
  std::vector<double> bg;
  std::vector<int32_t> n2c_off, c2n;
  // multigrid hierarchy of the run's operator (runs of at most kBatchMgMaxRows
  // nodes whose grid coarsens to at most kBatchDenseMax interior unknowns; the
  // others keep the plain inner CG)
  bool has_mg = false;
  MgHostHierarchy mg;
};

struct mpg_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  int64_t budget = 0, used = 0;
  int max_runs = 0;
  int cg_threads = 512, sort_interval = 10;
  int64_t cap = 0, n = 0;  // particle slots
  int cur = 0;
  MixedParts mp[2]{};
  Run runs[kMaxSlots];
  SlotDev *d_slots = nullptr;
  SlotStat *d_stats = nullptr, *h_stats = nullptr;
  int *d_hist = nullptr;  // per slot: solutions in the extrapolation history
  // plans
  int2 *d_conv_plan = nullptr, *d_ef_plan = nullptr, *d_block_items = nullptr;
  int4 *d_items = nullptr;
  int n_conv_blocks = 0, n_ef_blocks = 0, n_cg_blocks = 0;
  int64_t plan_cap_conv = 0, plan_cap_ef = 0, plan_cap_items = 0, plan_cap_blocks = 0;
  bool plan_dirty = true;
  int max_cg_blocks = 0;
  // one persistent launch per step (k_batch_step) or one launch per phase
  bool fused = true;
  int max_step_blocks = 0;   // co-resident blocks of k_batch_step at cg_threads
  DevStats *d_gbar = nullptr;  // grid barrier of k_batch_step
  DevStats *h_gbar = nullptr;
  // sort scratch
  int64_t *d_base = nullptr;
  uint32_t *d_cnt = nullptr, *d_start = nullptr, *d_scan = nullptr, *d_count = nullptr, *h_count = nullptr;
  int64_t keys_cap = 0, start_cap = 0, scan_cap = 0;
  int64_t steps_since_sort = 0;
  int64_t admitted_since_sort = 0;  // particles admitted since the last (run, cell) sort
  // graph
  cudaGraphExec_t gexec = nullptr;
  int64_t graph_n = -1;
  bool graph_ok = true, use_graph = true;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
  int64_t launches = 0;
};

namespace {

int bfail(mpg_batch *b, int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (b) b->err = buf;
  return code;
}

#define BCK(call)                                                                                     \
  do {                                                                                                \
    cudaError_t e_ = (call);                                                                          \
    if (e_ != cudaSuccess) return bfail(b, MPG_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));    \
  } while (0)

template <typename T>
int balloc(mpg_batch *b, Run *r, T **p, int64_t count) {
  *p = nullptr;
  const size_t bytes = sizeof(T) * (size_t)(count > 0 ? count : 1);
  cudaError_t e = cudaMalloc((void **)p, bytes);
  if (e != cudaSuccess) return bfail(b, MPG_ERR_CUDA, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
  if (r) {
    r->bufs.push_back(*p);
    r->bytes += (int64_t)bytes;
  }
  return MPG_OK;
}

#define BTRY(x)              \
  do {                       \
    int rc_ = (x);           \
    if (rc_) return rc_;     \
  } while (0)

void free_run(Run &r) {
  for (void *p : r.bufs) cudaFree(p);
  r.bufs.clear();
  r.bytes = 0;
}

constexpr int64_t kBatchDenseMax = 400;  // interior unknowns of a run's coarsest multigrid level
// runs up to this many nodes solve with multigrid (on a CTA group of
// rows_per_mg_cta nodes per CTA, at most kMaxParts CTAs)
constexpr int64_t kBatchMgMaxRows = 1 << 20;

int64_t run_bytes_estimate(const mpg_run_desc &d) {
  const int64_t n = d.n_side;
  const int64_t T = 6 * n * n * n, N = (n + 1) * (n + 1) * (n + 1);
  // per tet: walk record, neighbours, node ids, fill ratio, 4 charge slots, slot
  // indices; per node: flag, slot offset, rhs, phi, background, r64, previous
  // phi, 7 FP32 solver vectors
  // (+ 15 FP64 and 15 FP32 coefficients per node on a jittered mesh)
  // (+ a multigrid hierarchy: level-0 D^-1, flags and three vectors, the
  // coarser levels' stencils and vectors (< N / 7 nodes), the dense inverse)
  return T * (48 + 16 + 16 + 4 + 32 + 16) + N * (1 + 4 + 8 * 5 + 4 * 7 + (d.jitter > 0 ? kND * 12 : 0)) +
         8 * kMaxParts * 8 + d.n_particles * 56 + N * 40 + kBatchDenseMax * kBatchDenseMax * 4 + (16 << 10);
}

// device copy of a run's multigrid hierarchy, and the solver state
// (mgpass::CgMgArgs) pointing into the run's own vectors; one CTA runs the
// run's V-cycles (batch_vcycle)
int upload_run_mg(mpg_batch *b, Run &r, const mpg_run_prep &p, const SlotDev &v, mgpass::CgMgArgs **out) {
  const MgHostHierarchy &H = p.mg;
  cudaStream_t st = b->stream;
  mgpass::CgMgArgs a{};
  MgDev &m = a.mg;
  m.nlev = (int)H.lev.size();
  if (m.nlev < 2 || m.nlev > kMgMaxLevels) return bfail(b, MPG_ERR_ARG, "multigrid hierarchy of %d levels", m.nlev);
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
    float *dinv, *e, *t, *t2;
    uint8_t *bnd;
    BTRY(balloc(b, &r, &dinv, L.n));
    BTRY(balloc(b, &r, &bnd, L.n));
    BTRY(balloc(b, &r, &e, L.n));
    BTRY(balloc(b, &r, &t, L.n));
    BTRY(balloc(b, &r, &t2, L.n));
    BCK(cudaMemcpyAsync(dinv, h.dinv.data(), sizeof(float) * L.n, cudaMemcpyHostToDevice, st));
    BCK(cudaMemcpyAsync(bnd, h.bnd.data(), L.n, cudaMemcpyHostToDevice, st));
    BCK(cudaMemsetAsync(e, 0, sizeof(float) * L.n, st));
    BCK(cudaMemsetAsync(t, 0, sizeof(float) * L.n, st));
    BCK(cudaMemsetAsync(t2, 0, sizeof(float) * L.n, st));
    L.dinv = dinv;
    L.bnd = bnd;
    L.e = e;
    L.t = t;
    L.t2 = t2;
    L.r = nullptr;  // level 0's right-hand side is the PCG residual
    if (l > 0) {
      float *val, *rr;
      BTRY(balloc(b, &r, &val, 27 * L.n));
      BTRY(balloc(b, &r, &rr, L.n));
      BCK(cudaMemcpyAsync(val, h.val.data(), sizeof(float) * 27 * L.n, cudaMemcpyHostToDevice, st));
      BCK(cudaMemsetAsync(rr, 0, sizeof(float) * L.n, st));
      L.val = val;
      L.r = rr;
    }
  }
  m.ngrid = m.nlev - 1;
  m.dense_m = (int)H.dense_idx.size();
  int32_t *idx;
  float *inv, *dr;
  BTRY(balloc(b, &r, &idx, m.dense_m));
  BTRY(balloc(b, &r, &inv, (int64_t)m.dense_m * m.dense_m));
  BTRY(balloc(b, &r, &dr, m.dense_m));
  BCK(cudaMemcpyAsync(idx, H.dense_idx.data(), sizeof(int32_t) * m.dense_m, cudaMemcpyHostToDevice, st));
  BCK(cudaMemcpyAsync(inv, H.dense_inv.data(), sizeof(float) * H.dense_inv.size(), cudaMemcpyHostToDevice, st));
  BCK(cudaMemsetAsync(dr, 0, sizeof(float) * m.dense_m, st));
  m.dense_idx = idx;
  m.dense_inv = inv;
  m.dense_r = dr;
  m.omega = 0.8f;
  m.nu0 = 2;
  m.nu1 = 1;
  m.reliable = 0;
  m.fuse_update = 0;
  // level 0: the run's 15-point stencil, constant on a uniform mesh
  DiaMatrix &A = a.A;
  A.n = m.lev[0].n;
  A.nwrap = 0;
  A.ndiag = kND;
  A.constant = v.v32 ? 0 : 1;
  A.val32 = const_cast<float *>(v.v32);
  A.val64 = const_cast<double *>(v.v64);
  A.bnd = v.bnd;
  for (int k = 0; k < kND; ++k) {
    A.off[k] = p.off[k];
    A.cst[k] = (float)p.s64[k];
    if (p.off[k] == 0 && p.s64[k] != 0.0) m.dinv0 = (float)(1.0 / p.s64[k]);
  }
  a.b = v.rhs;
  a.x = v.phi;
  a.r64 = v.r64;
  a.r[0] = a.r[1] = v.r[0];
  a.s[0] = a.s[1] = v.q[1];
  a.w = v.q[0];
  a.p = v.p[0];
  a.z = v.z;
  a.u = m.lev[0].t;
  a.partials = v.partials;
  a.tol2 = v.tol2;
  a.inner_tol2 = v.inner_tol2;
  a.safety2 = v.safety2;
  a.max_iter = v.max_iter;
  a.st = nullptr;
  mgpass::CgMgArgs *d;
  BTRY(balloc(b, &r, &d, 1));
  BCK(cudaMemcpyAsync(d, &a, sizeof(a), cudaMemcpyHostToDevice, st));
  BCK(cudaStreamSynchronize(st));
  *out = d;
  return MPG_OK;
}

int upload_slots(mpg_batch *b) {
  std::vector<SlotDev> h(kMaxSlots);
  for (int s = 0; s < kMaxSlots; ++s) {
    h[s] = b->runs[s].dev;
    h[s].active = b->runs[s].used && b->runs[s].active;
    h[s].resident = b->runs[s].used;
  }
  BCK(cudaMemcpyAsync(b->d_slots, h.data(), sizeof(SlotDev) * kMaxSlots, cudaMemcpyHostToDevice, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return MPG_OK;
}

template <typename T>
int ensure_buf(mpg_batch *b, T **p, int64_t &cap, int64_t want) {
  if (*p && cap >= want) return MPG_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  const int64_t c = std::max<int64_t>(want, 16) * 2;
  BTRY(balloc(b, nullptr, p, c));
  cap = c;
  return MPG_OK;
}

// plans of the per-run kernels and of the batched solver
int build_plans(mpg_batch *b) {
  std::vector<int2> conv, ef;
  std::vector<int> act;
  for (int s = 0; s < kMaxSlots; ++s)
    if (b->runs[s].used && b->runs[s].active) act.push_back(s);
  for (int s : act) {
    const Run &r = b->runs[s];
    for (int64_t k = 0; k < (r.N + 255) / 256; ++k) conv.push_back(make_int2(s, (int)k));
    for (int64_t k = 0; k < (r.T + 255) / 256; ++k) ef.push_back(make_int2(s, (int)k));
  }
  // solver: runs bigger than rows_per_cta get several CTAs (their items come
  // first in each CTA's list, one multi-CTA item per CTA); the rest are dealt
  // to the least-loaded CTA
  const int G = std::max(1, b->fused ? b->max_step_blocks : b->max_cg_blocks);
  const int64_t rows_per_cta = 24 * 1024;
  // a multigrid run gets a CTA per (average nodes per CTA) of the whole batch,
  // at least 4096: the parts of the big runs then carry about the load the
  // small runs put on the other CTAs (256-run ensemble: 24k nodes per CTA,
  // step 7.59 ms, against 8.16 ms at 12k and 8.51 ms at 36k)
  int64_t total_rows = 0;
  for (int s : act) total_rows += b->runs[s].N;
  int64_t rows_per_mg_cta = std::max<int64_t>(4096, total_rows / std::max(1, b->fused ? b->max_step_blocks
                                                                                       : b->max_cg_blocks));
  if (const char *e = getenv("MPG_BATCH_MG_ROWS")) rows_per_mg_cta = std::max<int64_t>(1024, atoll(e));
  std::vector<std::vector<int4>> per(G);
  std::vector<int64_t> load(G, 0);
  int next = 0;
  std::vector<int> order = act;
  std::sort(order.begin(), order.end(), [&](int a, int c) { return b->runs[a].N > b->runs[c].N; });
  for (int s : order) {
    const int64_t N = b->runs[s].N;
    // a run with a multigrid hierarchy takes fewer rows per CTA: its
    // iterations are few and each is a dozen latency-bound passes
    const int64_t rows = b->runs[s].dev.mg ? rows_per_mg_cta : rows_per_cta;
    int parts = (int)std::min<int64_t>(kMaxParts, (N + rows - 1) / rows);
    if (parts > 1 && next + parts <= G) {
      for (int q = 0; q < parts; ++q) {
        per[next + q].insert(per[next + q].begin(), make_int4(s, q, parts, 0));
        load[next + q] += N / parts;
      }
      next += parts;
    } else {
      int best = 0;
      for (int g = 1; g < G; ++g)
        if (load[g] < load[best]) best = g;
      per[best].push_back(make_int4(s, 0, 1, 0));
      load[best] += N;
    }
  }
  std::vector<int4> items;
  std::vector<int2> bi;
  int used_blocks = 0;
  for (int g = 0; g < G; ++g) {
    if (per[g].empty()) continue;
    used_blocks = g + 1;
  }
  for (int g = 0; g < used_blocks; ++g) {
    const int start = (int)items.size();
    for (const int4 &w : per[g]) items.push_back(w);
    bi.push_back(make_int2(start, (int)items.size()));
  }
  BTRY(ensure_buf(b, &b->d_conv_plan, b->plan_cap_conv, (int64_t)conv.size()));
  BTRY(ensure_buf(b, &b->d_ef_plan, b->plan_cap_ef, (int64_t)ef.size()));
  BTRY(ensure_buf(b, &b->d_items, b->plan_cap_items, (int64_t)items.size()));
  BTRY(ensure_buf(b, &b->d_block_items, b->plan_cap_blocks, (int64_t)bi.size()));
  if (!conv.empty())
    BCK(cudaMemcpyAsync(b->d_conv_plan, conv.data(), sizeof(int2) * conv.size(), cudaMemcpyHostToDevice, b->stream));
  if (!ef.empty())
    BCK(cudaMemcpyAsync(b->d_ef_plan, ef.data(), sizeof(int2) * ef.size(), cudaMemcpyHostToDevice, b->stream));
  if (!items.empty())
    BCK(cudaMemcpyAsync(b->d_items, items.data(), sizeof(int4) * items.size(), cudaMemcpyHostToDevice, b->stream));
  if (!bi.empty())
    BCK(cudaMemcpyAsync(b->d_block_items, bi.data(), sizeof(int2) * bi.size(), cudaMemcpyHostToDevice, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  b->n_conv_blocks = (int)conv.size();
  b->n_ef_blocks = (int)ef.size();
  b->n_cg_blocks = (int)bi.size();
  b->plan_dirty = false;
  return MPG_OK;
}

int batch_sort(mpg_batch *b) {
  // per-slot key bases over resident runs
  std::vector<int64_t> base(kMaxSlots, -1);
  int64_t K = 0;
  for (int s = 0; s < kMaxSlots; ++s)
    if (b->runs[s].used) {
      base[s] = K;
      K += b->runs[s].T;
    }
  BTRY(ensure_buf(b, &b->d_cnt, b->keys_cap, K + 1));
  BTRY(ensure_buf(b, &b->d_start, b->start_cap, K + 1));
  const int64_t sl = scan_scratch_len(K + 1) + 4;
  BTRY(ensure_buf(b, &b->d_scan, b->scan_cap, sl));
  BCK(cudaMemcpyAsync(b->d_base, base.data(), sizeof(int64_t) * kMaxSlots, cudaMemcpyHostToDevice, b->stream));
  BCK(cudaMemsetAsync(b->d_cnt, 0, sizeof(uint32_t) * (K + 1), b->stream));
  const int other = 1 - b->cur;
  const unsigned g = (unsigned)std::max<int64_t>(1, (b->n + 255) / 256);
  if (b->n > 0) k_batch_hist<<<g, 256, 0, b->stream>>>(b->mp[b->cur].c, b->n, b->d_base, b->d_cnt);
  scan_u32(b->stream, b->d_cnt, b->d_start, K, b->d_scan, sl);
  BCK(cudaMemsetAsync(b->d_cnt, 0, sizeof(uint32_t) * (K + 1), b->stream));
  if (b->n > 0)
    k_batch_scatter<<<g, 256, 0, b->stream>>>(b->mp[b->cur], b->n, b->mp[other], b->d_base, b->d_start, b->d_cnt);
  k_batch_copy_count<<<1, 1, 0, b->stream>>>(b->d_start, K, b->d_count);
  b->launches += 6;
  BCK(cudaGetLastError());
  BCK(cudaMemcpyAsync(b->h_count, b->d_count, sizeof(uint32_t), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  b->cur = other;
  b->n = *b->h_count;
  b->steps_since_sort = 0;
  b->admitted_since_sort = 0;
  return MPG_OK;
}

// the launches of one step (eager, or recorded into a graph)
int enqueue_step(mpg_batch *b) {
  cudaStream_t s = b->stream;
  BCK(cudaMemsetAsync(b->d_stats, 0, sizeof(SlotStat) * kMaxSlots, s));
  if (b->fused) {
    // one persistent cooperative launch for all phases of the step
    BCK(cudaMemsetAsync(b->d_gbar, 0, sizeof(DevStats), s));
    BatchStepArgs a;
    a.slots = b->d_slots;
    a.stats = b->d_stats;
    a.conv_plan = b->d_conv_plan;
    a.ef_plan = b->d_ef_plan;
    a.block_items = b->d_block_items;
    a.items = b->d_items;
    a.n_conv = b->n_conv_blocks;
    a.n_ef = b->n_ef_blocks;
    a.n_cg_blocks = b->n_cg_blocks;
    a.P = b->mp[b->cur];
    a.n = b->n;
    a.gbar = b->d_gbar;
    void *args[] = {(void *)&a};
    BCK(cudaLaunchCooperativeKernel(batch_step_kernel(b->cg_threads), dim3(b->max_step_blocks),
                                    dim3(b->cg_threads), args, 0, s));
    return MPG_OK;
  }
  if (b->n_conv_blocks) k_batch_convert<<<b->n_conv_blocks, 256, 0, s>>>(b->d_slots, b->d_conv_plan);
  if (b->n_cg_blocks) {
    void *args[] = {(void *)&b->d_slots, (void *)&b->d_stats, (void *)&b->d_items, (void *)&b->d_block_items};
    BCK(cudaLaunchCooperativeKernel(batch_cg_kernel(b->cg_threads), dim3(b->n_cg_blocks), dim3(b->cg_threads), args,
                                    0, s));
  }
  if (b->n_ef_blocks) k_batch_efield<<<b->n_ef_blocks, 256, 0, s>>>(b->d_slots, b->d_ef_plan);
  if (b->n > 0) {
    const unsigned want = (unsigned)((b->n + kMoveThreads - 1) / kMoveThreads), wave = batch_move_blocks(b->device);
    k_batch_move<<<want < wave ? want : wave, kMoveThreads, 0, s>>>(b->mp[b->cur], b->n, b->d_slots, b->d_stats, 1);
  }
  BCK(cudaGetLastError());
  return MPG_OK;
}

int step_once(mpg_batch *b, double &ms) {
  if (b->plan_dirty) {
    BTRY(upload_slots(b));
    BTRY(build_plans(b));
    if (b->gexec) {
      cudaGraphExecDestroy(b->gexec);
      b->gexec = nullptr;
    }
  }
  const int n_launch = b->fused ? 1
                                : (b->n_conv_blocks ? 1 : 0) + (b->n_cg_blocks ? 1 : 0) + (b->n_ef_blocks ? 1 : 0) +
                                      (b->n > 0 ? 1 : 0);
  BCK(cudaEventRecord(b->ev0, b->stream));
  bool ran = false;
  if (b->use_graph && b->graph_ok) {
    if (!b->gexec || b->graph_n != b->n) {
      if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
      }
      cudaGraph_t g = nullptr;
      if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        int rc = enqueue_step(b);
        cudaError_t e = cudaStreamEndCapture(b->stream, &g);
        if (rc == MPG_OK && e == cudaSuccess && g &&
            cudaGraphInstantiate(&b->gexec, g, 0) == cudaSuccess) {
          b->graph_n = b->n;
        } else {
          b->graph_ok = false;
          b->gexec = nullptr;
        }
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
      } else {
        b->graph_ok = false;
        cudaGetLastError();
      }
    }
    if (b->gexec) {
      BCK(cudaGraphLaunch(b->gexec, b->stream));
      ran = true;
    }
  }
  if (!ran) BTRY(enqueue_step(b));
  b->launches += n_launch;
  BCK(cudaEventRecord(b->ev1, b->stream));
  BCK(cudaMemcpyAsync(b->h_stats, b->d_stats, sizeof(SlotStat) * kMaxSlots, cudaMemcpyDeviceToHost, b->stream));
  if (b->fused) BCK(cudaMemcpyAsync(b->h_gbar, b->d_gbar, sizeof(DevStats), cudaMemcpyDeviceToHost, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  if (b->fused && b->h_gbar->bar_error)
    for (int s = 0; s < kMaxSlots; ++s) b->h_stats[s].bar_error = 1;  // the step ended early for every run
  float f = 0.f;
  BCK(cudaEventElapsedTime(&f, b->ev0, b->ev1));
  ms = f;
  return MPG_OK;
}

}  // namespace

extern "C" {

int mpg_batch_create(int device, int64_t budget_bytes, int max_runs, int64_t particle_capacity, mpg_batch **out) {
  if (!out) return MPG_ERR_ARG;
  *out = nullptr;
  if (max_runs < 1 || max_runs > kMaxSlots || particle_capacity < 1 || particle_capacity >= (1LL << 32) ||
      budget_bytes <= 0)
    return MPG_ERR_ARG;
  mpg_batch *b = new (std::nothrow) mpg_batch();
  if (!b) return MPG_ERR_ARG;
  b->device = device;
  b->budget = budget_bytes;
  b->max_runs = max_runs;
  auto bail = [&](int rc) {
    mpg_batch_destroy(b);
    return rc;
  };
  if (cudaSetDevice(device) != cudaSuccess) return bail(MPG_ERR_CUDA);
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(MPG_ERR_CUDA);
  if (cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess ||
      cudaEventCreate(&b->ev2) != cudaSuccess)
    return bail(MPG_ERR_CUDA);
  for (int k = 0; k < 2; ++k) {
    if (balloc(b, nullptr, &b->mp[k].c, particle_capacity) || balloc(b, nullptr, &b->mp[k].b, particle_capacity) ||
        balloc(b, nullptr, &b->mp[k].v, particle_capacity))
      return bail(MPG_ERR_CUDA);
    b->mp[k].id = nullptr;
    b->mp[k].cap = particle_capacity;
  }
  b->cap = particle_capacity;
  b->used = particle_capacity * 56;
  if (balloc(b, nullptr, &b->d_slots, kMaxSlots) || balloc(b, nullptr, &b->d_stats, kMaxSlots) ||
      balloc(b, nullptr, &b->d_base, kMaxSlots) || balloc(b, nullptr, &b->d_count, 1) ||
      balloc(b, nullptr, &b->d_hist, kMaxSlots))
    return bail(MPG_ERR_CUDA);
  if (cudaMallocHost(&b->h_stats, sizeof(SlotStat) * kMaxSlots) != cudaSuccess ||
      cudaMallocHost(&b->h_count, sizeof(uint32_t)) != cudaSuccess ||
      cudaMallocHost(&b->h_gbar, sizeof(DevStats)) != cudaSuccess)
    return bail(MPG_ERR_CUDA);
  if (balloc(b, nullptr, &b->d_gbar, 1)) return bail(MPG_ERR_CUDA);
  int sms = 0, occ = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_cg_kernel(b->cg_threads), b->cg_threads, 0);
  b->max_cg_blocks = sms * occ;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_step_kernel(b->cg_threads), b->cg_threads, 0);
  b->max_step_blocks = sms * occ;
  if (b->max_cg_blocks < 1 || b->max_step_blocks < 1) return bail(MPG_ERR_CUDA);
  *out = b;
  return MPG_OK;
}

int mpg_batch_destroy(mpg_batch *b) {
  if (!b) return MPG_OK;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (int s = 0; s < kMaxSlots; ++s) free_run(b->runs[s]);
  for (int k = 0; k < 2; ++k) {
    cudaFree(b->mp[k].c);
    cudaFree(b->mp[k].b);
    cudaFree(b->mp[k].v);
  }
  void *ps[] = {b->d_slots, b->d_stats, b->d_base, b->d_count, b->d_hist, b->d_conv_plan, b->d_ef_plan,
                b->d_block_items, b->d_items, b->d_cnt, b->d_start, b->d_scan, b->d_gbar};
  for (void *p : ps)
    if (p) cudaFree(p);
  if (b->h_gbar) cudaFreeHost(b->h_gbar);
  if (b->h_stats) cudaFreeHost(b->h_stats);
  if (b->h_count) cudaFreeHost(b->h_count);
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  if (b->ev0) cudaEventDestroy(b->ev0);
  if (b->ev1) cudaEventDestroy(b->ev1);
  if (b->ev2) cudaEventDestroy(b->ev2);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return MPG_OK;
}

int mpg_batch_last_error(mpg_batch *b, char *buf, int len) {
  if (!b || !buf || len <= 0) return MPG_ERR_ARG;
  snprintf(buf, (size_t)len, "%s", b->err.c_str());
  return MPG_OK;
}

int mpg_batch_set_tuning(mpg_batch *b, int cg_threads, int sort_interval) {
  if (!b) return MPG_ERR_ARG;
  if (cg_threads != 256 && cg_threads != 512 && cg_threads != 1024)
    return bfail(b, MPG_ERR_ARG, "cg_threads must be 256, 512 or 1024");
  if (sort_interval < 0) return bfail(b, MPG_ERR_ARG, "sort_interval < 0");
  BCK(cudaSetDevice(b->device));
  int sms = 0, occ = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_cg_kernel(cg_threads), cg_threads, 0);
  if (sms * occ < 1) return bfail(b, MPG_ERR_ARG, "solver block size %d cannot be resident", cg_threads);
  int occ_step = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_step, batch_step_kernel(cg_threads), cg_threads, 0);
  if (sms * occ_step < 1) return bfail(b, MPG_ERR_ARG, "step block size %d cannot be resident", cg_threads);
  b->cg_threads = cg_threads;
  b->max_cg_blocks = sms * occ;
  b->max_step_blocks = sms * occ_step;
  b->sort_interval = sort_interval;
  b->plan_dirty = true;
  return MPG_OK;
}

int mpg_batch_prepare(const mpg_run_desc *d, mpg_run_prep **out) {
  if (!d || !out) return MPG_ERR_ARG;
  *out = nullptr;
  // n >= 4: the stencil is read off the centre node's row, whose 14
  // neighbours must all be interior nodes
  if (d->n_side < 4 || d->n_particles < 0 || !(d->m > 0) || !(d->dt > 0) || !(d->tol > 0) || d->max_iter < 1 ||
      d->steps < 0 || !(d->jitter >= 0.0 && d->jitter < 0.5))
    return MPG_ERR_ARG;
  if (6LL * d->n_side * d->n_side * d->n_side >= (int64_t)MPG_WALL) return MPG_ERR_ARG;
  mpg_run_prep *p = new (std::nothrow) mpg_run_prep();
  if (!p) return MPG_ERR_ARG;
  p->d = *d;
  // mesh and stencil on the host
  mpg_mesh_desc md{};
  md.nx = md.ny = md.nz = d->n_side;
  md.split = MPG_SPLIT_KUHN6;
  md.lo = 0.0;
  md.hi = 1.0;
  md.mapping = d->jitter > 0.0 ? MPG_MAP_JITTER : MPG_MAP_NONE;
  md.jitter = d->jitter;
  md.seed = d->mesh_seed;
  HostMesh &hm = p->hm;
  std::string err;
  int rc = host_mesh_generate(md, hm, err);
  if (rc) {
    delete p;
    return rc;
  }
  std::vector<int32_t> rp, col;
  std::vector<double> val;
  host_csr_assemble(hm, 1, rp, col, val);
  // stencil: the row of the centre node (all 15 neighbours interior for n >= 4)
  const int64_t c = (int64_t)(d->n_side / 2) * (d->n_side + 1) * (d->n_side + 1) +
                    (int64_t)(d->n_side / 2) * (d->n_side + 1) + d->n_side / 2;
  if (rp[c + 1] - rp[c] != kND) {
    delete p;
    return MPG_ERR_MESH;
  }
  for (int k = 0; k < kND; ++k) {
    p->off[k] = col[rp[c] + k] - (int32_t)c;
    p->s64[k] = val[rp[c] + k];
  }
  if (d->jitter > 0.0) {
    // every interior row has the centre row's 15 offsets (jittering moves
    // nodes, not the connectivity); boundary rows stay zero (identity rows)
    const int64_t N = hm.N;
    p->d64.assign((size_t)kND * N, 0.0);
    for (int64_t r = 0; r < N; ++r) {
      if (hm.bnd[r]) continue;
      for (int32_t k = rp[r]; k < rp[r + 1]; ++k) {
        int dd = 0;
        while (dd < kND && p->off[dd] != col[k] - (int32_t)r) ++dd;
        if (dd == kND) {
          delete p;
          return MPG_ERR_MESH;
        }
        p->d64[(size_t)dd * N + r] = val[k];
      }
    }
    p->d32.assign(p->d64.begin(), p->d64.end());
  }
  p->recv.resize(12 * hm.T);
  for (int64_t t = 0; t < hm.T; ++t) {
    for (int q = 0; q < 9; ++q) p->recv[12 * t + q] = (float)hm.jinv[9 * t + q];
    p->recv[12 * t + 9] = p->recv[12 * t + 10] = p->recv[12 * t + 11] = 0.f;
  }
  host_fill_ratio(hm, p->ratio);
  host_background(hm, d->rho_background, p->bg);
  host_charge_slots(hm, p->n2c_off, p->c2n);
  {
    const char *e = getenv("MPG_BATCH_MG");
    std::string why;
    if (!(e && atoi(e) == 0) && hm.N <= kBatchMgMaxRows)
      p->has_mg = host_mg_build(hm, rp, col, val, p->mg, why, kBatchDenseMax);
  }
  *out = p;
  return MPG_OK;
}

int mpg_run_prep_destroy(mpg_run_prep *p) {
  delete p;
  return MPG_OK;
}

int mpg_batch_set_fused(mpg_batch *b, int on) {
  if (!b) return MPG_ERR_ARG;
  b->fused = on != 0;
  b->plan_dirty = true;
  return MPG_OK;
}

int mpg_batch_admit(mpg_batch *b, const mpg_run_desc *d, int *slot) {
  if (!b || !d || !slot) return MPG_ERR_ARG;
  *slot = -1;
  mpg_run_prep *p = nullptr;
  const int rc = mpg_batch_prepare(d, &p);
  if (rc) return bfail(b, rc, rc == MPG_ERR_MESH ? "unexpected stencil size" : "bad run descriptor");
  const int rc2 = mpg_batch_admit_prepared(b, p, slot);
  mpg_run_prep_destroy(p);
  return rc2;
}

int mpg_batch_admit_prepared(mpg_batch *b, const mpg_run_prep *p, int *slot) {
  if (!b || !p || !slot) return MPG_ERR_ARG;
  BCK(cudaSetDevice(b->device));
  *slot = -1;
  const mpg_run_desc *d = &p->d;
  const HostMesh &hm = p->hm;
  int used_runs = 0, s = -1;
  for (int k = 0; k < kMaxSlots; ++k) {
    if (b->runs[k].used)
      ++used_runs;
    else if (s < 0)
      s = k;
  }
  if (used_runs >= b->max_runs || s < 0) return bfail(b, MPG_ERR_CAPACITY, "no free run slot");
  const int64_t need = run_bytes_estimate(*d) - d->n_particles * 56;
  if (b->used + need > b->budget) return bfail(b, MPG_ERR_CAPACITY, "device-memory budget exhausted");
  if (b->n + d->n_particles > b->cap && b->n > 0) BTRY(batch_sort(b));
  if (b->n + d->n_particles > b->cap) return bfail(b, MPG_ERR_CAPACITY, "particle capacity exhausted");
  Run &r = b->runs[s];
  r = Run();
  r.used = true;
  r.active = d->steps > 0;
  r.d = *d;
  r.T = hm.T;
  r.N = hm.N;
  SlotDev &v = r.dev;
  v = SlotDev();
  for (int k = 0; k < kND; ++k) {
    v.off[k] = p->off[k];
    v.s64[k] = p->s64[k];
    v.s32[k] = (float)p->s64[k];
  }
  v.T = hm.T;
  v.N = hm.N;
  v.tol2 = d->tol * d->tol;
  v.inner_tol2 = 1e-10;
  v.safety2 = 0.25;  // the reduction the outer test needs, halved (as the single-run solvers)
  if (const char *e = getenv("MPG_CG_INNER_SAFETY")) v.safety2 = atof(e) * atof(e);
  v.max_iter = d->max_iter;
  v.max_cross = 1000;
  v.dt = (float)d->dt;
  // same float expression as the single-run kernel: (0.5f * dt) * (q/m)
  v.hk = 0.5f * (float)d->dt * (float)(d->q / d->m);
  const double wq = fabs(d->weight * d->q);
  v.quantum = wq > 0 ? wq / 33554432.0 : 1.0;
  v.Q = (int)llround(d->weight * d->q / v.quantum);
  // device buffers of the run (freed again if an allocation fails)
  auto undo = [&](int rc) {
    free_run(r);
    r = Run();
    return rc;
  };
  float4 *rec;
  uint4 *nbr;
  int4 *tets;
  uint8_t *bnd;
  float *ratio;
  unsigned long long *acc;
  double *rhs, *phi, *bg, *r64;
  float *f[7];
  double *parts;
  int32_t *n2c_off;
  int4 *c2n;
  double *phi_prev;
  if (balloc(b, &r, &rec, 3 * hm.T) || balloc(b, &r, &nbr, hm.T) || balloc(b, &r, &tets, hm.T) ||
      balloc(b, &r, &bnd, hm.N) || balloc(b, &r, &ratio, hm.T) || balloc(b, &r, &acc, 4 * hm.T) ||
      balloc(b, &r, &n2c_off, hm.N + 1) || balloc(b, &r, &c2n, hm.T) || balloc(b, &r, &rhs, hm.N) ||
      balloc(b, &r, &phi, hm.N) || balloc(b, &r, &bg, hm.N) || balloc(b, &r, &r64, hm.N) ||
      balloc(b, &r, &parts, 8 * kMaxParts) || balloc(b, &r, &phi_prev, hm.N))
    return undo(MPG_ERR_CUDA);
  for (int k = 0; k < 7; ++k)
    if (balloc(b, &r, &f[k], hm.N)) return undo(MPG_ERR_CUDA);
  double *v64 = nullptr;
  float *v32 = nullptr;
  if (!p->d64.empty() && (balloc(b, &r, &v64, kND * hm.N) || balloc(b, &r, &v32, kND * hm.N)))
    return undo(MPG_ERR_CUDA);
  cudaStream_t st = b->stream;
  BCK(cudaMemcpyAsync(rec, p->recv.data(), sizeof(float) * 12 * hm.T, cudaMemcpyHostToDevice, st));
  BCK(cudaMemcpyAsync(nbr, hm.nbr_opp.data(), sizeof(uint4) * hm.T, cudaMemcpyHostToDevice, st));
  BCK(cudaMemcpyAsync(tets, hm.tets.data(), sizeof(int4) * hm.T, cudaMemcpyHostToDevice, st));
  BCK(cudaMemcpyAsync(bnd, hm.bnd.data(), hm.N, cudaMemcpyHostToDevice, st));
  BCK(cudaMemcpyAsync(ratio, p->ratio.data(), sizeof(float) * hm.T, cudaMemcpyHostToDevice, st));
  BCK(cudaMemcpyAsync(bg, p->bg.data(), sizeof(double) * hm.N, cudaMemcpyHostToDevice, st));
  BCK(cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * 4 * hm.T, st));
  BCK(cudaMemcpyAsync(n2c_off, p->n2c_off.data(), sizeof(int32_t) * (hm.N + 1), cudaMemcpyHostToDevice, st));
  BCK(cudaMemcpyAsync(c2n, p->c2n.data(), sizeof(int32_t) * 4 * hm.T, cudaMemcpyHostToDevice, st));
  BCK(cudaMemsetAsync(phi, 0, sizeof(double) * hm.N, st));
  if (v64) {
    BCK(cudaMemcpyAsync(v64, p->d64.data(), sizeof(double) * p->d64.size(), cudaMemcpyHostToDevice, st));
    BCK(cudaMemcpyAsync(v32, p->d32.data(), sizeof(float) * p->d32.size(), cudaMemcpyHostToDevice, st));
  }
  v.v64 = v64;
  v.v32 = v32;
  v.rec = rec;
  v.nbr = nbr;
  v.tets = tets;
  v.bnd = bnd;
  v.fill_ratio = ratio;
  v.acc = acc;
  v.n2c_off = n2c_off;
  v.c2n = c2n;
  v.rhs = rhs;
  v.phi = phi;
  v.bg = bg;
  v.r64 = r64;
  v.r[0] = f[0];
  v.r[1] = f[1];
  v.p[0] = f[2];
  v.p[1] = f[3];
  v.q[0] = f[4];
  v.q[1] = f[5];
  v.z = f[6];
  v.partials = parts;
  v.phi_prev = phi_prev;
  v.hist = b->d_hist + s;
  BCK(cudaMemsetAsync(v.hist, 0, sizeof(int), st));
  v.mg = nullptr;
  if (p->has_mg) {
    mgpass::CgMgArgs *dargs;
    if (upload_run_mg(b, r, *p, v, &dargs)) return undo(MPG_ERR_CUDA);
    v.mg = dargs;
  }
  // fill: append the run's particles, species field = slot
  DevMesh dm;
  dm.T = hm.T;
  dm.N = hm.N;
  dm.tets = tets;
  dm.fill_ratio = ratio;
  PlainParts none{};
  const int64_t n0 = b->n;
  launch_fill_uniform(st, 1, none, b->mp[b->cur], n0, d->n_particles, d->seed, s, d->weight, d->drift, d->vth, dm, 0);
  b->n += d->n_particles;
  r.n_alive = d->n_particles;
  b->used += r.bytes;
  // the slot table must hold this run before its first deposit
  BTRY(upload_slots(b));
  if (d->n_particles > 0)
    k_batch_deposit<<<(unsigned)((d->n_particles + 255) / 256), 256, 0, st>>>(b->mp[b->cur], n0, b->n, b->d_slots);
  BCK(cudaGetLastError());
  BCK(cudaStreamSynchronize(st));
  b->admitted_since_sort += d->n_particles;
  b->plan_dirty = true;
  r.last.active = r.active;
  r.last.n_alive = r.n_alive;
  r.last.bytes = r.bytes;
  *slot = s;
  return MPG_OK;
}

int mpg_batch_step(mpg_batch *b, int n_steps, mpg_batch_stats *st) {
  if (!b || n_steps < 0) return MPG_ERR_ARG;
  BCK(cudaSetDevice(b->device));
  mpg_batch_stats acc{};
  const int64_t l0 = b->launches;
  for (int k = 0; k < n_steps; ++k) {
    int nact = 0;
    int64_t parts = 0;
    for (int s = 0; s < kMaxSlots; ++s)
      if (b->runs[s].used && b->runs[s].active) {
        ++nact;
        parts += b->runs[s].n_alive;
      }
    if (nact == 0) break;
    // sort every sort_interval steps, and before a step when the particles
    // admitted since the last sort (in fill order) are a tenth of the batch
    if (b->sort_interval > 0 &&
        (b->steps_since_sort >= b->sort_interval || b->admitted_since_sort * 10 >= b->n))
      BTRY(batch_sort(b));
    double ms = 0.0;
    BTRY(step_once(b, ms));
    b->steps_since_sort++;
    acc.ms += ms;
    acc.ms_last_step = ms;
    acc.active_runs = nact;
    acc.particle_steps += parts;
    // per-run bookkeeping from the device statistics
    bool changed = false;
    for (int s = 0; s < kMaxSlots; ++s) {
      Run &r = b->runs[s];
      if (!r.used || !r.active) continue;
      const SlotStat &h = b->h_stats[s];
      r.steps_done++;
      r.n_alive -= (int64_t)h.killed;
      r.last.steps_done = r.steps_done;
      r.last.n_alive = r.n_alive;
      r.last.ke = 0.5 * r.d.weight * r.d.m * h.ke;
      r.last.solver_iters = h.iters;
      r.last.solver_resid = h.resid;
      r.last.status = h.bar_error ? MPG_ERR_TIMEOUT
                                  : h.status ? MPG_ERR_NOT_CONVERGED : h.limit ? MPG_ERR_WALK_LIMIT : MPG_OK;
      if (r.last.status && !acc.status) acc.status = r.last.status;
      if (r.steps_done >= r.d.steps) {
        r.active = false;
        r.finished = true;
        r.last.active = 0;
        r.last.finished = 1;
        changed = true;
      }
    }
    if (changed) b->plan_dirty = true;
  }
  acc.n_launches = b->launches - l0;
  acc.graph = (b->use_graph && b->graph_ok && b->gexec) ? 1 : 0;
  if (st) *st = acc;
  return acc.status;
}

int mpg_batch_run_info(mpg_batch *b, int slot, mpg_run_info *info) {
  if (!b || !info || slot < 0 || slot >= kMaxSlots) return MPG_ERR_ARG;
  if (!b->runs[slot].used) return bfail(b, MPG_ERR_STATE, "slot %d is empty", slot);
  *info = b->runs[slot].last;
  info->active = b->runs[slot].active;
  info->finished = b->runs[slot].finished;
  info->bytes = b->runs[slot].bytes;
  return MPG_OK;
}

int mpg_batch_run_phi(mpg_batch *b, int slot, double *phi) {
  if (!b || !phi || slot < 0 || slot >= kMaxSlots) return MPG_ERR_ARG;
  if (!b->runs[slot].used) return bfail(b, MPG_ERR_STATE, "slot %d is empty", slot);
  BCK(cudaSetDevice(b->device));
  BCK(cudaMemcpyAsync(phi, b->runs[slot].dev.phi, sizeof(double) * b->runs[slot].N, cudaMemcpyDeviceToHost,
                      b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  return MPG_OK;
}

int mpg_batch_run_particles(mpg_batch *b, int slot, int64_t cap, int64_t *nout, uint32_t *cell, float *b3,
                            float *v3) {
  if (!b || !nout || slot < 0 || slot >= kMaxSlots) return MPG_ERR_ARG;
  if (!b->runs[slot].used) return bfail(b, MPG_ERR_STATE, "slot %d is empty", slot);
  BCK(cudaSetDevice(b->device));
  const int64_t n = b->n;
  std::vector<uint32_t> c(n > 0 ? n : 1);
  std::vector<float> bb(3 * (n > 0 ? n : 1)), vv(3 * (n > 0 ? n : 1));
  float *db, *dv;
  BCK(cudaMallocAsync((void **)&db, sizeof(float) * 3 * (n > 0 ? n : 1), b->stream));
  BCK(cudaMallocAsync((void **)&dv, sizeof(float) * 3 * (n > 0 ? n : 1), b->stream));
  if (n > 0) {
    launch_mixed_unpack(b->stream, b->mp[b->cur], n, db, dv);
    BCK(cudaMemcpyAsync(c.data(), b->mp[b->cur].c, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaMemcpyAsync(bb.data(), db, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, b->stream));
    BCK(cudaMemcpyAsync(vv.data(), dv, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, b->stream));
  }
  BCK(cudaFreeAsync(db, b->stream));
  BCK(cudaFreeAsync(dv, b->stream));
  BCK(cudaStreamSynchronize(b->stream));
  int64_t k = 0;
  for (int64_t p = 0; p < n; ++p) {
    if (c[p] == MPG_DEAD || (int)(c[p] >> 24) != slot) continue;
    if (k < cap) {
      if (cell) cell[k] = c[p] & 0xFFFFFFu;
      for (int q = 0; q < 3; ++q) {
        if (b3) b3[3 * k + q] = bb[3 * p + q];
        if (v3) v3[3 * k + q] = vv[3 * p + q];
      }
    }
    ++k;
  }
  *nout = k;
  return k > cap ? bfail(b, MPG_ERR_CAPACITY, "buffer holds %lld < %lld", (long long)cap, (long long)k) : MPG_OK;
}

int mpg_batch_retire(mpg_batch *b, int slot) {
  if (!b || slot < 0 || slot >= kMaxSlots) return MPG_ERR_ARG;
  Run &r = b->runs[slot];
  if (!r.used) return bfail(b, MPG_ERR_STATE, "slot %d is empty", slot);
  BCK(cudaSetDevice(b->device));
  // drop the run's particles so that a later run can reuse the slot number
  if (b->n > 0)
    k_batch_kill_slot<<<(unsigned)((b->n + 255) / 256), 256, 0, b->stream>>>(b->mp[b->cur].c, b->n, slot);
  BCK(cudaGetLastError());
  BCK(cudaStreamSynchronize(b->stream));
  b->used -= r.bytes;
  free_run(r);
  r = Run();
  b->plan_dirty = true;
  return upload_slots(b);
}

}  // extern "C"
