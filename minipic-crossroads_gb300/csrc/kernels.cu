// kernels.cu -- particle and field kernels of the GB300 PIC step (sm_103a).
//
// Plain form (FP64, reference semantics): one thread per particle, state in
// component-major SoA so that every load and store of a warp is one coalesced
// 256-byte transaction per component.  Built with --fmad=false, so the Boris
// push and the tet walk round exactly like the reference's CPU build
// (particle_move.hpp:135-225,364-392).
//
// Mixed form: cell index + FP32 barycentric coordinates + FP32 velocity
// (28 bytes per particle), one fused kernel per step that gathers the per-tet
// E, pushes, walks across faces by carrying barycentrics through a per-face
// vertex permutation (no re-projection), removes particles at absorbing
// walls and deposits the new position into an int64 fixed-point node
// accumulator (order-independent, exact total charge).
#include <cuda_runtime.h>
#include <stdlib.h>

#include "mpg_internal.h"
#include "mpg_kernels.h"
#include "mpg_walk.cuh"

namespace {

constexpr int kThreads = 256;

inline unsigned grid_for(int64_t n, int threads = kThreads) {
  int64_t g = (n + threads - 1) / threads;
  return (unsigned)(g < 1 ? 1 : g);
}

// ---------------------------------------------------------------------------
// block-level exclusive scan of one uint32 per thread (blockDim = 1024)
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t *warp_tot, uint32_t &total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  __syncthreads();
  if (lane == 31) warp_tot[wid] = x;
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    uint32_t t = lane < nw ? warp_tot[lane] : 0u;
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < nw) warp_tot[lane] = t;  // inclusive warp prefix
  }
  __syncthreads();
  total = warp_tot[(blockDim.x >> 5) - 1];
  uint32_t before = wid > 0 ? warp_tot[wid - 1] : 0u;
  return before + x - v;
}

constexpr int kScanThreads = 1024;
constexpr int kScanPer = 4;
constexpr int kScanTile = kScanThreads * kScanPer;

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const uint32_t *__restrict__ in, int64_t n,
                                                             uint32_t *__restrict__ tile_sum) {
  __shared__ uint32_t wt[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
  uint32_t s = 0;
  for (int i = 0; i < kScanPer; ++i)
    if (base + i < n) s += in[base + i];
  uint32_t tot;
  block_exclusive_scan(s, wt, tot);
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sums(uint32_t *tile_sum, int64_t ntiles) {
  __shared__ uint32_t wt[32];
  uint32_t carry = 0;
  for (int64_t b0 = 0; b0 < ntiles; b0 += kScanThreads) {
    int64_t i = b0 + threadIdx.x;
    uint32_t v = i < ntiles ? tile_sum[i] : 0u;
    uint32_t tot;
    uint32_t ex = block_exclusive_scan(v, wt, tot);
    if (i < ntiles) tile_sum[i] = carry + ex;
    carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) tile_sum[ntiles] = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const uint32_t *__restrict__ in, int64_t n,
                                                             const uint32_t *__restrict__ tile_off,
                                                             uint32_t *__restrict__ out, int64_t ntiles) {
  __shared__ uint32_t wt[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPer;
  uint32_t v[kScanPer], s = 0;
  for (int i = 0; i < kScanPer; ++i) {
    v[i] = base + i < n ? in[base + i] : 0u;
    s += v[i];
  }
  uint32_t tot;
  uint32_t ex = block_exclusive_scan(s, wt, tot) + tile_off[blockIdx.x];
  for (int i = 0; i < kScanPer; ++i) {
    if (base + i < n) out[base + i] = ex;
    ex += v[i];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = tile_off[ntiles];
}

// ---------------------------------------------------------------------------
// plain FP64 kernels
__device__ __forceinline__ void jinv_apply(const double *__restrict__ I, const double a[3], double out[3]) {
  // mesh.hpp:244-250: ref_vec[i] = sum_j Jinv[i][j] * phys[j], accumulated from 0
  for (int r = 0; r < 3; ++r) {
    double s = 0.0;
    s += I[3 * r + 0] * a[0];
    s += I[3 * r + 1] * a[1];
    s += I[3 * r + 2] * a[2];
    out[r] = s;
  }
}

// Block totals without __syncthreads at the end: each warp reduces its lanes
// (kinetic energy in float-float, counters with integer reductions), lane 0
// stores the warp's share, and the last warp to finish sums the shares and
// pushes one set of device atomics per block.  Warps retire independently and
// no FP64 arithmetic runs per warp.
struct BlockTotals {
  ff ke[32];
  unsigned killed, cross, limit, done;
};
__device__ __forceinline__ void block_totals_init(BlockTotals *bt) {
  if (threadIdx.x < 32) bt->ke[threadIdx.x] = ff{0.f, 0.f};
  if (threadIdx.x == 0) bt->killed = bt->cross = bt->limit = bt->done = 0u;
  __syncthreads();
}
__device__ __forceinline__ void block_totals_push(BlockTotals *bt, ff ke, unsigned killed, unsigned cross,
                                                  unsigned limit, DevStats *st) {
  const unsigned FULL = 0xffffffffu;
  for (int o = 16; o > 0; o >>= 1) ke = ff_add(ke, ff_shfl_down(ke, o));
  killed = __reduce_add_sync(FULL, killed);
  cross = __reduce_add_sync(FULL, cross);
  limit = __reduce_add_sync(FULL, limit);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const unsigned nw = (blockDim.x + 31) >> 5;
  unsigned last = 0;
  if (lane == 0) {
    bt->ke[wid] = ke;
    if (killed) atomicAdd(&bt->killed, killed);
    if (cross) atomicAdd(&bt->cross, cross);
    if (limit) atomicAdd(&bt->limit, limit);
    __threadfence_block();
    last = atomicAdd(&bt->done, 1u) == nw - 1;
  }
  last = __shfl_sync(FULL, last, 0);
  if (!last) return;
  __threadfence_block();
  const volatile BlockTotals *v = bt;
  ff s = lane < (int)nw ? ff{v->ke[lane].hi, v->ke[lane].lo} : ff{0.f, 0.f};
  for (int o = 16; o > 0; o >>= 1) s = ff_add(s, ff_shfl_down(s, o));
  if (lane == 0) {
    const double e = (double)s.hi + (double)s.lo;
    if (e != 0.0) atomicAdd(&st->ke, e);
    if (v->killed) atomicAdd(&st->n_killed, (unsigned long long)v->killed);
    if (v->cross) atomicAdd(&st->n_cross, (unsigned long long)v->cross);
    if (v->limit) atomicAdd(&st->n_limit, (unsigned long long)v->limit);
  }
}

__global__ void __launch_bounds__(kThreads) k_plain_deposit(PlainParts P, int64_t n, const int4 *__restrict__ tets,
                                                            const double *__restrict__ detj, SpeciesTable S, int mode,
                                                            double *__restrict__ rhs) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int e = P.cell[p];
  if (e < 0) return;
  const int4 nd = tets[e];
  const int nodes[4] = {nd.x, nd.y, nd.z, nd.w};
  const double w = P.w[p], q = S.q[P.sp[p]];
  if (mode == 0) {
    // PIC.cpp:125-135: val = sum_c -tot_q * (detJ*w_c * N_i(c))
    const double A = 0.5854101966249685, B = 0.1381966011250105;
    const double Pc[4][3] = {{B, B, B}, {A, B, B}, {B, A, B}, {B, B, A}};
    const double dj = detj[e];
    const double tot_q = w * q * (6 / dj);
    const double wm = dj * (1.0 / 24.0);
    for (int i = 0; i < 4; ++i) {
      double val = 0;
      for (int c = 0; c < 4; ++c) {
        const double Ni = (i == 0) ? (1 - Pc[c][0] - Pc[c][1] - Pc[c][2]) : Pc[c][i - 1];
        val += -tot_q * (wm * Ni);
      }
      atomicAdd(&rhs[nodes[i]], val);
    }
  } else {
    const int64_t cap = P.cap;
    const double x0 = P.xr[p], x1 = P.xr[cap + p], x2 = P.xr[2 * cap + p];
    const double wq = w * q;
    const double lam[4] = {1 - x0 - x1 - x2, x0, x1, x2};
    for (int i = 0; i < 4; ++i) atomicAdd(&rhs[nodes[i]], -(wq * lam[i]));
  }
}

// Periodic meshes (plane > 0): charge deposited on a ghost node of the x = hi
// plane belongs to its pair on the x = lo plane (PIC.cpp:132-134); the pair's
// thread folds it in and clears the ghost plane.
__global__ void k_rhs_finish(int64_t N, double *__restrict__ rhs, const double *__restrict__ bg,
                             const uint8_t *__restrict__ bnd, int64_t nsolve, int64_t plane) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N || (plane && i >= nsolve)) return;
  double r = rhs[i];
  if (plane && i < plane) {
    r += rhs[nsolve + i];
    rhs[nsolve + i] = 0.0;
  }
  if (bg) r += bg[i];
  if (bnd[i]) r = 0.0;  // PIC.cpp:155-158
  rhs[i] = r;
}

__global__ void k_efield_plain(int64_t T, const int4 *__restrict__ tets, const double *__restrict__ grad,
                               const double *__restrict__ phi, double *__restrict__ E) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const int4 nd = tets[t];
  const double f[4] = {phi[nd.x], phi[nd.y], phi[nd.z], phi[nd.w]};
  const double *G = grad + 12 * t;
  for (int d = 0; d < 3; ++d) {
    double s = 0.0;
    for (int i = 0; i < 4; ++i) s += f[i] * G[3 * i + d];
    E[3 * t + d] = s;
  }
}

// find_intersection of particle_move.hpp:135-225 for one sub-step
__device__ __forceinline__ double plain_intersect(const DevMesh &M, int &e, double x[3], double xr[3], double v[3],
                                                  double vr[3], double dt, double time_remaining, int kill,
                                                  bool &killed) {
  const double span = dt * time_remaining;
  double frac = 1.0;
  int face = -1;
  double dlam[3], lend[3];
  for (int d = 0; d < 3; ++d) {
    dlam[d] = span * vr[d];
    lend[d] = xr[d] + dlam[d];
  }
  if (vr[2] < 0 && lend[2] < 0) {
    face = 3;
    frac = -xr[2] / (dlam[2]);
  }
  if (vr[1] < 0 && lend[1] < 0) {
    const double fy = -xr[1] / (dlam[1]);
    if (fy < frac) {
      face = 0;
      frac = fy;
    }
  }
  if (vr[0] < 0 && lend[0] < 0) {
    const double fx = -xr[0] / (dlam[0]);
    if (fx < frac) {
      face = 2;
      frac = fx;
    }
  }
  const double end_sum = lend[0] + lend[1] + lend[2];
  const double rate_sum = vr[0] + vr[1] + vr[2];
  if (rate_sum > 0 && end_sum > 1) {
    const double fs = (1 - xr[0] - xr[1] - xr[2]) / (dlam[0] + dlam[1] + dlam[2]);
    if (fs < frac) {
      face = 1;
      frac = fs;
    }
  }
  for (int d = 0; d < 3; ++d) {
    x[d] = x[d] + frac * span * v[d];
    xr[d] = xr[d] + frac * span * vr[d];
  }
  if (frac < 1) {
    const int4 nb4 = M.nbrs[e];
    const int nb = face == 0 ? nb4.x : face == 1 ? nb4.y : face == 2 ? nb4.z : nb4.w;
    if (nb >= 0) {
      // a periodic face wraps x to the other side of the box: lo + hi - x on
      // the reference's mirror-image meshes (particle_move.hpp:190-191 writes
      // x = -x on its [-1,1] box), a shift by the box length on jittered ones
      if (M.fper && M.fper[4 * (int64_t)e + face]) {
        if (M.xshift != 0.0)
          x[0] = (x[0] + x[0] > M.xflip) ? x[0] - M.xshift : x[0] + M.xshift;
        else
          x[0] = M.xflip - x[0];
      }
      e = nb;
      const int n0 = M.tets[e].x;
      const double delta[3] = {x[0] - M.nodes[3 * n0], x[1] - M.nodes[3 * n0 + 1], x[2] - M.nodes[3 * n0 + 2]};
      double dref[3];
      jinv_apply(M.jinv + 9 * (int64_t)e, delta, dref);
      for (int d = 0; d < 3; ++d) xr[d] = 0.0 + dref[d];
      jinv_apply(M.jinv + 9 * (int64_t)e, v, vr);
    } else {
      if (kill) {
        killed = true;
        return 1;
      }
      const double *nrm = M.normals + 12 * (int64_t)e + 3 * face;
      double vdn = 0;
      for (int d = 0; d < 3; ++d) vdn += v[d] * nrm[d];
      for (int d = 0; d < 3; ++d) v[d] -= 2 * vdn * nrm[d];
      jinv_apply(M.jinv + 9 * (int64_t)e, v, vr);
    }
  }
  return frac;
}

__global__ void __launch_bounds__(kThreads) k_plain_move(PlainParts P, int64_t n, DevMesh M,
                                                         const double *__restrict__ Etet, SpeciesTable S, double dt,
                                                         int kill, int max_cross, DevStats *st) {
  __shared__ BlockTotals bt;
  block_totals_init(&bt);
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double ke = 0.0;
  unsigned killed = 0, cross = 0, limit = 0;
  if (p < n) {
    int e = P.cell[p];
    if (e >= 0) {
      const int64_t cap = P.cap;
      double x[3] = {P.x[p], P.x[cap + p], P.x[2 * cap + p]};
      double xr[3] = {P.xr[p], P.xr[cap + p], P.xr[2 * cap + p]};
      double v[3] = {P.v[p], P.v[cap + p], P.v[2 * cap + p]};
      const int s = P.sp[p];
      const double E[3] = {Etet[3 * (int64_t)e], Etet[3 * (int64_t)e + 1], Etet[3 * (int64_t)e + 2]};
      // Boris push, particle_move.hpp:366-389 (B = 0, PIC.cpp:179)
      const double scaled_dt = dt * 1.0;
      const double q_over_m = S.qm[s];
      const double B[3] = {0.0, 0.0, 0.0};
      double t[3] = {q_over_m * 0.5 * B[0], q_over_m * 0.5 * B[1], q_over_m * 0.5 * B[2]};
      for (int d = 0; d < 3; ++d) v[d] += scaled_dt * E[d] * q_over_m * 0.5;
      double tmp[3] = {v[0], v[1], v[2]};
      tmp[0] += v[1] * t[2] - v[2] * t[1];
      tmp[1] += v[2] * t[0] - v[0] * t[2];
      tmp[2] += v[0] * t[1] - v[1] * t[0];
      const double t_sqr = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
      for (int d = 0; d < 3; ++d) t[d] *= 2. / (1 + t_sqr);
      v[0] += tmp[1] * t[2] - tmp[2] * t[1];
      v[1] += tmp[2] * t[0] - tmp[0] * t[2];
      v[2] += tmp[0] * t[1] - tmp[1] * t[0];
      for (int d = 0; d < 3; ++d) v[d] += scaled_dt * E[d] * q_over_m * 0.5;
      double vr[3];
      jinv_apply(M.jinv + 9 * (int64_t)e, v, vr);
      // walk, particle_move.hpp:110-121
      double tr = 1.0;
      int it = 0;
      bool dead = false;
      while (tr > 0) {
        if (it >= max_cross) {
          limit = 1;
          break;
        }
        const double sf = plain_intersect(M, e, x, xr, v, vr, dt, tr, kill, dead);
        tr -= sf * tr;
        ++it;
        if (dead) break;
      }
      cross = it > 0 ? (unsigned)(it - 1) : 0u;
      if (dead) {
        killed = 1;
        e = -1;
      } else {
        // PIC.cpp:193-199
        const double tot_m = P.w[p] * S.m[s];
        double v_sqr = 0;
        for (int d = 0; d < 3; ++d) v_sqr += v[d] * v[d];
        ke = 0.5 * tot_m * v_sqr;
      }
      P.cell[p] = e;
      P.x[p] = x[0];
      P.x[cap + p] = x[1];
      P.x[2 * cap + p] = x[2];
      P.xr[p] = xr[0];
      P.xr[cap + p] = xr[1];
      P.xr[2 * cap + p] = xr[2];
      P.v[p] = v[0];
      P.v[cap + p] = v[1];
      P.v[2 * cap + p] = v[2];
    }
  }
  // kinetic energy of this particle as float-float (exact split of the double)
  const float ke_hi = (float)ke;
  block_totals_push(&bt, ff{ke_hi, (float)(ke - (double)ke_hi)}, killed, cross, limit, st);
}

// Stable compaction by warp ballots over 4096-particle tiles.  A tile is
// four rounds of 1024 consecutive particles; in a round thread t holds
// particle t of the round, so every load and store of a warp covers
// consecutive particles.  A particle's destination is the tile's offset +
// the live particles of the tile's earlier rounds + those of earlier warps in
// its round (a scan of 32 warp counts) + those of lower lanes in its warp
// (popc of the ballot below the lane).
__global__ void __launch_bounds__(kScanThreads) k_count_live(const int32_t *__restrict__ cell, int64_t n,
                                                             uint32_t *__restrict__ tile_cnt) {
  __shared__ uint32_t wt[32];
  const int64_t base = (int64_t)blockIdx.x * kScanTile + threadIdx.x;
  uint32_t s = 0;
#pragma unroll
  for (int r = 0; r < kScanPer; ++r) {
    const int64_t e = base + (int64_t)r * kScanThreads;
    if (e < n && cell[e] >= 0) ++s;
  }
  uint32_t tot;
  block_exclusive_scan(s, wt, tot);
  if (threadIdx.x == 0) tile_cnt[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanThreads) k_compact_plain(PlainParts P, int64_t n, PlainParts Q,
                                                                const uint32_t *__restrict__ tile_off,
                                                                int64_t ntiles, uint32_t *d_count) {
  __shared__ uint32_t wcnt[32];
  __shared__ uint32_t round_total;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t base = (int64_t)blockIdx.x * kScanTile + threadIdx.x;
  uint32_t off = tile_off[blockIdx.x];
  for (int r = 0; r < kScanPer; ++r) {
    const int64_t e = base + (int64_t)r * kScanThreads;
    const bool live = e < n && P.cell[e] >= 0;
    const unsigned bal = __ballot_sync(0xffffffffu, live);
    if (lane == 0) wcnt[wid] = __popc(bal);
    __syncthreads();
    if (wid == 0) {
      const uint32_t c = lane < (kScanThreads >> 5) ? wcnt[lane] : 0u;
      uint32_t x = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      if (lane < (kScanThreads >> 5)) wcnt[lane] = x - c;  // exclusive
      if (lane == 31) round_total = x;
    }
    __syncthreads();
    if (live) {
      const uint32_t dst = off + wcnt[wid] + __popc(bal & ((1u << lane) - 1u));
      Q.cell[dst] = P.cell[e];
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        Q.x[d * Q.cap + dst] = P.x[d * P.cap + e];
        Q.xr[d * Q.cap + dst] = P.xr[d * P.cap + e];
        Q.v[d * Q.cap + dst] = P.v[d * P.cap + e];
      }
      Q.w[dst] = P.w[e];
      Q.sp[dst] = P.sp[e];
      if (P.id) Q.id[dst] = P.id[e];
    }
    off += round_total;
    __syncthreads();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) *d_count = tile_off[ntiles];
}

// ---------------------------------------------------------------------------
// mixed form
// Fixed-point charge of one particle split over its tet's four nodes:
// c_k = rint(b_k * Q) for k = 1..3 and c_0 = Q - c_1 - c_2 - c_3, so the four
// parts sum to the particle's charge exactly.
//
// Warp-aggregated: lanes that hold the same cell in a contiguous run (the
// usual case after a cell sort) add their contributions with a segmented warp
// scan, and the last lane of each run issues the four atomics.  Without this,
// a sorted warp sends 32 same-address atomics to one L2 slice, which
// serialise.  The atomics go to the cell's own four corner slots (not to
// the nodes, which 24 tets share), so distinct cells never contend: slot
// (t, k) sits at acc[c2n[t].k], inside node tets[t][k]'s contiguous slot
// range, and k_mixed_convert sums each node's range.  Integer addition is
// associative, so the result does not depend on the grouping.  Every lane of
// the warp must call this; lanes with key < 0 contribute nothing.
// `slots(key)` gives the four slot indices of cell `key`; it is called by
// the lanes that issue a run's atomics only.  With hist, the run's length is
// added to hist[key] as well: the particles per cell of the next cell sort
// (k_cell_hist's counts, taken from the deposit's runs at no extra pass).
template <class Slots>
__device__ __forceinline__ void deposit_fixed_warp_t(unsigned long long *__restrict__ acc, Slots slots, int key,
                                                     float b1, float b2, float b3, int Q,
                                                     uint32_t *__restrict__ hist) {
  // |Q| <= 2^25 quanta, so a run of up to 32 lanes sums to < 2^30 in int32
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  int c0 = 0, c1 = 0, c2 = 0, c3 = 0;
  if (key >= 0) {
    const float Qf = (float)Q;
    c1 = __float2int_rn(b1 * Qf);
    c2 = __float2int_rn(b2 * Qf);
    c3 = __float2int_rn(b3 * Qf);
    c0 = Q - c1 - c2 - c3;
  }
  const int prev = __shfl_up_sync(FULL, key, 1);
  const bool head = lane == 0 || prev != key;
  const unsigned heads = __ballot_sync(FULL, head);
  if (heads == 1u) {
    // the whole warp holds one cell (typical after a sort): plain reductions
    c0 = __reduce_add_sync(FULL, c0);
    c1 = __reduce_add_sync(FULL, c1);
    c2 = __reduce_add_sync(FULL, c2);
    c3 = __reduce_add_sync(FULL, c3);
    if (lane == 0 && key >= 0) {
      const int4 q = slots(key);
      atomicAdd(acc + q.x, (unsigned long long)(long long)c0);
      atomicAdd(acc + q.y, (unsigned long long)(long long)c1);
      atomicAdd(acc + q.z, (unsigned long long)(long long)c2);
      atomicAdd(acc + q.w, (unsigned long long)(long long)c3);
      if (hist) atomicAdd(hist + key, 32u);
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
  if (tail && key >= 0) {
    const int4 q = slots(key);
    atomicAdd(acc + q.x, (unsigned long long)(long long)c0);
    atomicAdd(acc + q.y, (unsigned long long)(long long)c1);
    atomicAdd(acc + q.z, (unsigned long long)(long long)c2);
    atomicAdd(acc + q.w, (unsigned long long)(long long)c3);
    if (hist) atomicAdd(hist + key, (unsigned)(lane - seg + 1));
  }
}

// slot indices from the tet table c2n (a load per run)
__device__ __forceinline__ void deposit_fixed_warp(unsigned long long *__restrict__ acc, const int4 *__restrict__ c2n,
                                                   int key, float b1, float b2, float b3, int Q,
                                                   uint32_t *__restrict__ hist = nullptr) {
  deposit_fixed_warp_t(acc, [&](int k) { return c2n[k]; }, key, b1, b2, b3, Q, hist);
}

// Walk tables of a uniform Kuhn mesh (KuhnTable, staged in shared memory):
// J^-1 by tet type t % 6, neighbours by hex offset.  A crossing needs no
// memory access at all; E of the start tet comes from etet4.
// Hex indices are split into (i, j, k) without a division instruction: for
// n < 2^24 and 1 <= d <= 2^16, m = ceil(2^40 / d) = (2^40 + e) / d with
// 0 <= e < d, and n m / 2^40 = n / d + n e / (d 2^40) exceeds n / d by less
// than 1 / d, so its floor is floor(n / d) (division by invariant integers
// using multiplication, Granlund and Montgomery, PLDI 1994).  At 128^3 the
// two divisions per crossing cost 0.3 ms of a 4.3 ms move.
__device__ __forceinline__ uint32_t div_magic40(uint32_t n, unsigned long long m) {
  return (uint32_t)(((unsigned long long)n * m) >> 40);
}

struct KuhnWalk {
  const float *__restrict__ jinv;   // 6 x 9
  const uint32_t *__restrict__ fw;  // 6 x 4 face words
  uint32_t nx, ny, nz;
  unsigned long long mz, myz;       // ceil(2^40 / nz), ceil(2^40 / (ny nz))
  __device__ __forceinline__ void load(uint32_t e, float4 &r0, float4 &r1, float4 &r2) const {
    const float *J = jinv + 9 * (e % 6u);
    r0 = make_float4(J[0], J[1], J[2], J[3]);
    r1 = make_float4(J[4], J[5], J[6], J[7]);
    r2.x = J[8];  // r2.yzw (E) is used by the kick at the start only
  }
  __device__ __forceinline__ uint32_t face(uint32_t e, int k) const {
    const uint32_t h = e / 6u, ty = e - 6u * h;
    const uint32_t f = fw[4 * ty + k];
    const uint32_t nyz = ny * nz, i = div_magic40(h, myz), rem = h - i * nyz, j = div_magic40(rem, mz),
                   kk = rem - j * nz;
    const int ni = (int)i + (int)(f & 3u) - 1, nj = (int)j + (int)((f >> 2) & 3u) - 1,
              nk = (int)kk + (int)((f >> 4) & 3u) - 1;
    if (ni < 0 || ni >= (int)nx || nj < 0 || nj >= (int)ny || nk < 0 || nk >= (int)nz) return MPG_WALL;
    return ((f >> 16) << 24) | (6u * (((uint32_t)ni * ny + (uint32_t)nj) * nz + (uint32_t)nk) + ((f >> 8) & 0xFFu));
  }
};

__global__ void __launch_bounds__(kThreads) k_mixed_deposit(MixedParts P, int64_t n, const int4 *__restrict__ c2n,
                                                            SpeciesTable S, unsigned long long *__restrict__ acc) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int key = -1;
  float b1 = 0.f, b2 = 0.f, b3 = 0.f;
  int Q = 0;
  if (p < n) {
    const uint32_t cs = P.c[p];
    if (cs != MPG_DEAD) {
      const float4 b = P.b[p];
      key = (int)(cs & 0xFFFFFFu);
      b1 = b.x;
      b2 = b.y;
      b3 = b.z;
      Q = (int)S.qfix[cs >> 24];
    }
  }
  // each lane converts its own charge Q, so runs may mix species
  deposit_fixed_warp(acc, c2n, key, b1, b2, b3, Q);
}

// charge quanta of node i: the sum of its slot range acc[off[i] .. off[i+1])
// (one thread per node; the slots are zeroed before the next deposit by the
// E-field pass or a memset, which is cheaper than zeroing them here, behind
// the reads)
__device__ __forceinline__ long long node_quanta(int64_t i, const int32_t *__restrict__ off,
                                                 const unsigned long long *__restrict__ acc) {
  return slot_sum(acc, off[i], off[i + 1]);
}

// Periodic meshes (plane > 0): the ghost plane's quanta are folded into
// their pairs by the pair's thread (integer sums: exact, order free).
__global__ void k_mixed_convert(int64_t N, const int32_t *__restrict__ off, const unsigned long long *__restrict__ acc,
                                double quantum, const double *__restrict__ bg, const uint8_t *__restrict__ bnd,
                                double *__restrict__ rhs, int64_t nsolve, int64_t plane) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N || (plane && i >= nsolve)) return;
  long long a = node_quanta(i, off, acc);
  if (plane && i < plane) {
    a += node_quanta(nsolve + i, off, acc);
    rhs[nsolve + i] = 0.0;
  }
  double r = -((double)a * quantum);
  if (bg) r += bg[i];
  if (bnd[i]) r = 0.0;
  rhs[i] = r;
}

// per-node quanta, for downloads
__global__ void k_node_quanta(int64_t N, const int32_t *__restrict__ off, const unsigned long long *__restrict__ acc,
                              long long *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) out[i] = node_quanta(i, off, acc);
}

// E per tet from phi: E = sum_k (phi_k - phi_0) * row_{k-1}(J^-1); the phi
// differences are formed in FP64, the products in FP32.
__global__ void k_efield_mixed(int64_t T, const int4 *__restrict__ tets, float4 *__restrict__ rec,
                               const double *__restrict__ phi) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= T) return;
  const int4 nd = tets[t];
  const double f0 = phi[nd.x];
  const float d1 = (float)(phi[nd.y] - f0), d2 = (float)(phi[nd.z] - f0), d3 = (float)(phi[nd.w] - f0);
  const float4 r0 = rec[3 * t], r1 = rec[3 * t + 1];
  float4 r2 = rec[3 * t + 2];
  // J^-1 rows: (r0.x r0.y r0.z) (r0.w r1.x r1.y) (r1.z r1.w r2.x)
  r2.y = __fmaf_rn(d3, r1.z, __fmaf_rn(d2, r0.w, d1 * r0.x));
  r2.z = __fmaf_rn(d3, r1.w, __fmaf_rn(d2, r1.x, d1 * r0.y));
  r2.w = __fmaf_rn(d3, r2.x, __fmaf_rn(d2, r1.y, d1 * r0.z));
  rec[3 * t + 2] = r2;
}

// E per tet of a uniform Kuhn mesh, one thread per hex: node ids come from
// the hex index and the table's corner offsets (no tet array is read).  All
// six tets of a hex have the hex's first node as their vertex 0, so the
// seven FP64 differences phi_c - phi_0 over the hex's other corners are
// formed and rounded to FP32 once per hex (the per-tet form needs eighteen
// on the narrow FP64 pipe, which bounded it), and each tet picks its three;
// the values are those of the per-tet formula bit for bit.  The block's
// 6 x 256 results are staged in shared memory and stored coalesced.  With
// zero, the block also clears its share of the nzero charge slots (the next
// move deposits into them), overlapping the stores with the FP64 work.
constexpr int kEfThreads = 256;
__global__ void __launch_bounds__(kEfThreads) k_efield_kuhn(int64_t T, KuhnTable kt, const double *__restrict__ phi,
                                                            float4 *__restrict__ etet4,
                                                            unsigned long long *__restrict__ zero, int64_t nzero) {
  __shared__ float sj[54];
  __shared__ int sc[24];                     // corner (4 di + 2 dj + dk) of vertex q of type ty
  __shared__ float sd[kEfThreads * 9];       // per thread: phi_c - phi_0 for c = 0..7 (stride 9)
  __shared__ float4 se[6 * kEfThreads];
  const int64_t SJ = kt.nz + 1, SI = (int64_t)(kt.ny + 1) * SJ;
  for (int i = threadIdx.x; i < 54; i += blockDim.x) sj[i] = kt.jinv[i / 9][i % 9];
  for (int i = threadIdx.x; i < 24; i += blockDim.x) {
    const int64_t o = kt.noff[i / 4][i % 4], di = o / SI, dj = (o - di * SI) / SJ, dk = o - di * SI - dj * SJ;
    sc[i] = (int)(4 * di + 2 * dj + dk);
  }
  __syncthreads();
  const int64_t H = T / 6, h0 = (int64_t)blockIdx.x * kEfThreads, h = h0 + threadIdx.x;
  if (h < H) {
    const uint32_t nyz = (uint32_t)(kt.ny * kt.nz), i = div_magic40((uint32_t)h, kt.myz),
                   rem = (uint32_t)h - i * nyz, j = div_magic40(rem, kt.mz), k = rem - j * (uint32_t)kt.nz;
    const int64_t base = ((int64_t)i * (kt.ny + 1) + j) * SJ + k;
    const double f0 = phi[base];
    float *d = sd + 9 * threadIdx.x;
    d[0] = 0.f;
    d[1] = (float)(phi[base + 1] - f0);
    d[2] = (float)(phi[base + SJ] - f0);
    d[3] = (float)(phi[base + SJ + 1] - f0);
    d[4] = (float)(phi[base + SI] - f0);
    d[5] = (float)(phi[base + SI + 1] - f0);
    d[6] = (float)(phi[base + SI + SJ] - f0);
    d[7] = (float)(phi[base + SI + SJ + 1] - f0);
#pragma unroll
    for (int ty = 0; ty < 6; ++ty) {
      const float d1 = d[sc[4 * ty + 1]], d2 = d[sc[4 * ty + 2]], d3 = d[sc[4 * ty + 3]];
      const float *J = sj + 9 * ty;
      se[6 * threadIdx.x + ty] = make_float4(__fmaf_rn(d3, J[6], __fmaf_rn(d2, J[3], d1 * J[0])),
                                             __fmaf_rn(d3, J[7], __fmaf_rn(d2, J[4], d1 * J[1])),
                                             __fmaf_rn(d3, J[8], __fmaf_rn(d2, J[5], d1 * J[2])), 0.f);
    }
  }
  __syncthreads();
  const int64_t t0 = 6 * h0, nt = T - t0 < 6 * kEfThreads ? T - t0 : 6 * kEfThreads;
  for (int q = threadIdx.x; q < nt; q += kEfThreads) etet4[t0 + q] = se[q];
  if (zero) {
    // this block's share [z0, z1) of the slots, in 16-byte stores where aligned
    const int64_t z0 = nzero * blockIdx.x / gridDim.x, z1 = nzero * (blockIdx.x + 1) / gridDim.x;
    int64_t a = z0;
    if (a & 1) {  // to a 16-byte boundary (the slots start on one)
      if (threadIdx.x == 0 && a < z1) zero[a] = 0ull;
      ++a;
    }
    if (a > z1) a = z1;
    const int64_t npair = (z1 - a) >> 1;
    uint4 *zp = reinterpret_cast<uint4 *>(zero + a);
    for (int64_t q = threadIdx.x; q < npair; q += kEfThreads) zp[q] = make_uint4(0u, 0u, 0u, 0u);
    if (threadIdx.x == 0 && ((z1 - a) & 1)) zero[z1 - 1] = 0ull;
  }
}

__global__ void __launch_bounds__(kThreads) k_mixed_move(MixedParts P, int64_t n, const float4 *__restrict__ rec,
                                                         const uint4 *__restrict__ nbr,
                                                         const int4 *__restrict__ c2n, SpeciesTable S, float dt,
                                                         int kill, int max_cross, unsigned long long *__restrict__ acc,
                                                         DevStats *st) {
  __shared__ BlockTotals bt;
  block_totals_init(&bt);
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float ke = 0.f;
  unsigned killed = 0, cross = 0, limit = 0;
  int dep_key = -1;
  float d1 = 0.f, d2 = 0.f, d3 = 0.f;
  int dq = 0;
  if (p < n) {
    uint32_t cs = P.c[p];
    if (cs != MPG_DEAD) {
      const int s = (int)(cs >> 24);
      uint32_t e = cs & 0xFFFFFFu;
      const float4 bv = P.b[p];
      const float2 vv = P.v[p];
      float l1 = bv.x, l2 = bv.y, l3 = bv.z;
      float vx = bv.w, vy = vv.x, vz = vv.y;
      bool dead, lim;
      const int it = mixed_walk(rec, nbr, e, l1, l2, l3, vx, vy, vz, 0.5f * dt * S.qm_f[s], dt, kill, max_cross,
                                dead, lim);
      limit = lim ? 1u : 0u;
      cross = (unsigned)it;
      if (dead) {
        killed = 1;
        P.c[p] = MPG_DEAD;
      } else {
        if (e != (cs & 0xFFFFFFu)) P.c[p] = ((uint32_t)s << 24) | e;
        P.b[p] = make_float4(l1, l2, l3, vx);
        P.v[p] = make_float2(vy, vz);
        ke = S.half_wm_f[s] * __fmaf_rn(vz, vz, __fmaf_rn(vy, vy, vx * vx));
        dep_key = (int)e;
        d1 = l1;
        d2 = l2;
        d3 = l3;
        dq = (int)S.qfix[s];
      }
    }
  }
  // deposit of the new position for the next step's field solve
  deposit_fixed_warp(acc, c2n, dep_key, d1, d2, d3, dq);
  block_totals_push(&bt, ff{ke, 0.f}, killed, cross, limit, st);
}

// Persistent form of the move: the grid is one wave of resident blocks and
// each warp walks 32-particle chunks c, c + W, c + 2W, ... (W = warps in the
// grid).  The next chunk's particle record is loaded before the current chunk
// is processed, so its DRAM latency overlaps the push, walk and deposit of
// the current one; block totals are formed once per block.  Per particle the
// arithmetic is that of k_mixed_move.  KUHN: the walk tables come from the
// 6-type table of a uniform Kuhn mesh (same values, bit for bit, as the
// per-tet records the table was checked against).
//
// Crossing particles walk in full warps: a chunk's lanes kick their particle
// and look for the first exit only; a particle that stays in its tet is
// finished and deposited with the chunk, one that leaves it goes, in its
// kicked state, to the warp's queue in shared memory.  Each time 32 are
// queued the warp walks them together from that state (the same operations
// as an uninterrupted walk, so the results are bit for bit those of walking
// every particle in its own chunk) and deposits them; the rest are walked
// after the last chunk.  Without the queue every chunk runs the crossing
// code about twice (some lane almost always crosses), with a third of the
// lanes active.
constexpr int kMoveWarps = kThreads / 32;
constexpr int kMoveQueue = 64;  // per warp: fewer than 32 wait, up to 32 join per chunk

template <bool KUHN>
__global__ void __launch_bounds__(kThreads, 4) k_mixed_move_persistent(MixedParts P, int64_t n, MixedParts Q,
                                                                    const uint32_t *__restrict__ perm,
                                                                    const uint32_t *__restrict__ d_count,
                                                                    const float4 *__restrict__ rec,
                                                                    const uint4 *__restrict__ nbr,
                                                                    const float4 *__restrict__ etet4, KuhnTable kt,
                                                                    const int4 *__restrict__ c2n, SpeciesTable S,
                                                                    float dt, int kill, int max_cross,
                                                                    unsigned long long *__restrict__ acc,
                                                                    uint32_t *__restrict__ hist, DevStats *st) {
  __shared__ BlockTotals bt;
  __shared__ float s_jinv[KUHN ? 54 : 1];
  __shared__ uint32_t s_face[KUHN ? 24 : 1];
  // queued particles of each warp: index (< 2^31, the particle capacity
  // bound), cellsp word, barycentrics, kicked velocity
  __shared__ uint32_t q_u[kMoveWarps][2][kMoveQueue];
  __shared__ float q_f[kMoveWarps][6][kMoveQueue];
  if (KUHN) {
    for (int i = threadIdx.x; i < 54; i += blockDim.x) s_jinv[i] = kt.jinv[i / 9][i % 9];
    for (int i = threadIdx.x; i < 24; i += blockDim.x) s_face[i] = kt.face[i / 4][i % 4];
  }
  block_totals_init(&bt);  // also the barrier after the table stores
  const KuhnWalk kw{s_jinv, s_face, (uint32_t)kt.nx, (uint32_t)kt.ny, (uint32_t)kt.nz, kt.mz, kt.myz};
  const RecTab3 rt{rec, nbr};
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  uint32_t *const qp = q_u[wib][0], *const qc = q_u[wib][1];
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int64_t nchunks = (n + 31) >> 5;
  const bool sorted_in = perm != nullptr;
  const int64_t cnt = sorted_in ? (int64_t)*d_count : n;
  ff ke = {0.f, 0.f};
  unsigned killed = 0, cross = 0, limit = 0;
  int qn = 0;  // queued particles of this warp (warp-uniform)
  // the walk tables of tet e
  auto load_rec = [&](uint32_t e, float4 &r0, float4 &r1, float4 &r2) {
    if (KUHN)
      kw.load(e, r0, r1, r2);
    else
      rt.load(e, r0, r1, r2);
  };
  // full walk of a kicked particle from (e, l), then its store, statistics
  // and deposit key; every lane of the warp calls it (live = has a particle)
  auto finish = [&](bool live, uint32_t p, uint32_t cs, float l1, float l2, float l3, float vx, float vy, float vz) {
    int dep_key = -1;
    float d1 = 0.f, d2 = 0.f, d3 = 0.f;
    int dq = 0;
    if (live) {
      const int s = (int)(cs >> 24);
      uint32_t e = cs & 0xFFFFFFu;
      float4 r0, r1, r2;
      load_rec(e, r0, r1, r2);
      bool dead, lim, stopped;
      int it;
      if (KUHN) {
        KuhnWalk tab = kw;
        it = mixed_walk_from<false>(tab, e, r0, r1, r2, l1, l2, l3, vx, vy, vz, dt, kill, max_cross, dead, lim,
                                    stopped);
      } else {
        RecTab3 tab = rt;
        it = mixed_walk_from<false>(tab, e, r0, r1, r2, l1, l2, l3, vx, vy, vz, dt, kill, max_cross, dead, lim,
                                    stopped);
      }
      limit += lim ? 1u : 0u;
      cross += (unsigned)it;
      if (dead) {
        killed += 1;
        Q.c[p] = MPG_DEAD;
      } else {
        if (sorted_in || e != (cs & 0xFFFFFFu)) Q.c[p] = ((uint32_t)s << 24) | e;
        Q.b[p] = make_float4(l1, l2, l3, vx);
        Q.v[p] = make_float2(vy, vz);
        ke = ff_add(ke, ff{S.half_wm_f[s] * __fmaf_rn(vz, vz, __fmaf_rn(vy, vy, vx * vx)), 0.f});
        dep_key = (int)e;
        d1 = l1;
        d2 = l2;
        d3 = l3;
        dq = (int)S.qfix[s];
      }
    }
    deposit_fixed_warp(acc, c2n, dep_key, d1, d2, d3, dq, hist);
  };
  // walk the queued particles [qn - m, qn) in lanes 0 .. m-1
  auto drain = [&](int m) {
    __syncwarp();
    const int slot = qn - m + lane;
    const bool live = lane < m;
    uint32_t p = 0, cs = MPG_DEAD;
    float l1 = 0.f, l2 = 0.f, l3 = 0.f, vx = 0.f, vy = 0.f, vz = 0.f;
    if (live) {
      p = qp[slot];
      cs = qc[slot];
      l1 = q_f[wib][0][slot];
      l2 = q_f[wib][1][slot];
      l3 = q_f[wib][2][slot];
      vx = q_f[wib][3][slot];
      vy = q_f[wib][4][slot];
      vz = q_f[wib][5][slot];
    }
    __syncwarp();
    qn -= m;
    finish(live, p, cs, l1, l2, l3, vx, vy, vz);
  };
  int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  // the record of particle i (input perm[i] when fused with a sort's
  // gather, whose slots [count, n) are dead in Q)
  auto fetch = [&](int64_t i, uint32_t &cs_, float4 &bv_, float2 &vv_) {
    cs_ = MPG_DEAD;
    if (i >= cnt) {
      if (sorted_in && i < n) Q.c[i] = MPG_DEAD;
      return;
    }
    const int64_t src = sorted_in ? (int64_t)perm[i] : i;
    cs_ = P.c[src];
    bv_ = P.b[src];
    vv_ = P.v[src];
    if (sorted_in && P.id) Q.id[i] = P.id[src];
  };
  // prefetched record of this lane's particle in chunk c
  uint32_t cs_n = MPG_DEAD;
  float4 bv_n = make_float4(0.f, 0.f, 0.f, 0.f);
  float2 vv_n = make_float2(0.f, 0.f);
  if (c < nchunks) fetch(c * 32 + lane, cs_n, bv_n, vv_n);
  for (; c < nchunks; c += nw) {
    const int64_t p = c * 32 + lane;
    const uint32_t cs = cs_n;
    const float4 bv = bv_n;
    const float2 vv = vv_n;
    cs_n = MPG_DEAD;
    if (c + nw < nchunks) fetch((c + nw) * 32 + lane, cs_n, bv_n, vv_n);
    int dep_key = -1;
    float d1 = 0.f, d2 = 0.f, d3 = 0.f;
    int dq = 0;
    bool queue = false;
    float l1 = bv.x, l2 = bv.y, l3 = bv.z;
    float vx = bv.w, vy = vv.x, vz = vv.y;
    if (p < cnt && cs != MPG_DEAD) {
      const int s = (int)(cs >> 24);
      uint32_t e = cs & 0xFFFFFFu;
      float4 r0, r1, r2;
      if (KUHN) {
        kw.load(e, r0, r1, r2);
        const float4 E = etet4[e];
        r2.y = E.x;
        r2.z = E.y;
        r2.w = E.z;
      } else {
        rt.load(e, r0, r1, r2);
      }
      mixed_kick(0.5f * dt * S.qm_f[s], r2, vx, vy, vz);
      bool dead, lim;
      if (KUHN) {
        KuhnWalk tab = kw;
        mixed_walk_from<true>(tab, e, r0, r1, r2, l1, l2, l3, vx, vy, vz, dt, kill, max_cross, dead, lim, queue);
      } else {
        RecTab3 tab = rt;
        mixed_walk_from<true>(tab, e, r0, r1, r2, l1, l2, l3, vx, vy, vz, dt, kill, max_cross, dead, lim, queue);
      }
      if (!queue) {
        // stays in its tet: l advanced by dt, nothing else changes
        if (sorted_in) Q.c[p] = cs;
        Q.b[p] = make_float4(l1, l2, l3, vx);
        Q.v[p] = make_float2(vy, vz);
        ke = ff_add(ke, ff{S.half_wm_f[s] * __fmaf_rn(vz, vz, __fmaf_rn(vy, vy, vx * vx)), 0.f});
        dep_key = (int)e;
        d1 = l1;
        d2 = l2;
        d3 = l3;
        dq = (int)S.qfix[s];
      }
    }
    // every lane of the warp is here (c is uniform across the warp)
    deposit_fixed_warp(acc, c2n, dep_key, d1, d2, d3, dq, hist);
    const unsigned qm = __ballot_sync(FULL, queue);
    if (queue) {
      const int slot = qn + __popc(qm & ((1u << lane) - 1u));
      qp[slot] = (uint32_t)p;
      qc[slot] = cs;
      q_f[wib][0][slot] = l1;
      q_f[wib][1][slot] = l2;
      q_f[wib][2][slot] = l3;
      q_f[wib][3][slot] = vx;
      q_f[wib][4][slot] = vy;
      q_f[wib][5][slot] = vz;
    }
    qn += __popc(qm);
    if (qn >= 32) drain(32);
  }
  if (qn > 0) drain(qn);
  block_totals_push(&bt, ke, killed, cross, limit, st);
}

// Runs of equal cells in a warp (particles stay nearly sorted between sorts):
// the run's first lane and the lane's rank within its run.
__device__ __forceinline__ void cell_run(uint32_t key, int &first, int &rank, int &len) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const uint32_t prev = __shfl_up_sync(FULL, key, 1);
  const unsigned heads = __ballot_sync(FULL, lane == 0 || prev != key);
  first = 31 - __clz(heads & (FULL >> (31 - lane)));
  rank = lane - first;
  const unsigned after = heads & ~(FULL >> (31 - lane));  // heads above this lane
  const int next = after ? __ffs(after) - 1 : 32;
  len = next - first;
}

// ---- stable cell sort (ParticleList::sort + compute_start_particles_by_element,
// particle_list.cpp:90-146) --------------------------------------------------
// 1. k_cell_hist: particles per cell (one atomic per warp run of equal cells);
// 2. exclusive scan: the first sorted position of every cell (start);
// 3. k_cell_slots: every live particle's input index goes to a slot of its
//    cell's range, claimed per warp run with one atomic (the order inside a
//    range depends on timing here);
// 4. k_cell_order / k_cell_order_long: each cell's range of input indices is
//    sorted ascending, so the order inside a cell is the input order: the
//    permutation is that of a stable sort by cell, the same on every run (the
//    reference's BinSort leaves it open);
// 5. k_sort_gather_*: sorted record i = input record perm[i] (coalesced
//    stores; the loads follow the input order cell by cell).
// Keys: mixed cellsp words (species << 24 | cell, MPG_DEAD = dead) or plain
// int32 cells (< 0 = dead); dead particles are dropped.
template <bool kMixed>
__device__ __forceinline__ uint32_t sort_key(const uint32_t *__restrict__ c, int64_t p, int64_t n) {
  if (p >= n) return MPG_DEAD;
  const uint32_t v = c[p];
  if (kMixed) return v == MPG_DEAD ? MPG_DEAD : (v & 0xFFFFFFu);
  return (int32_t)v < 0 ? MPG_DEAD : v;
}

template <bool kMixed>
__global__ void k_cell_hist(const uint32_t *__restrict__ c, int64_t n, uint32_t *__restrict__ cnt) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t key = sort_key<kMixed>(c, p, n);
  int first, rank, len;
  cell_run(key, first, rank, len);
  if (rank == 0 && key != MPG_DEAD) atomicAdd(&cnt[key], (unsigned)len);
}

// Each thread takes kSlotsPer particles, kThreads apart (each warp sees
// kSlotsPer runs of 32 consecutive particles), so that their slot claims and
// start loads are in flight together: one claim is an atomic whose result
// the thread waits for, and the pass is bound by that latency.
constexpr int kSlotsPer = 4;
template <bool kMixed>
__global__ void k_cell_slots(const uint32_t *__restrict__ c, int64_t n, const uint32_t *__restrict__ start,
                             uint32_t *__restrict__ fill, uint32_t *__restrict__ perm) {
  const int64_t p0 = (int64_t)blockIdx.x * blockDim.x * kSlotsPer + threadIdx.x;
  uint32_t key[kSlotsPer], base[kSlotsPer], st[kSlotsPer];
  int first[kSlotsPer], rank[kSlotsPer], len[kSlotsPer];
#pragma unroll
  for (int u = 0; u < kSlotsPer; ++u) {
    key[u] = sort_key<kMixed>(c, p0 + (int64_t)u * blockDim.x, n);
    cell_run(key[u], first[u], rank[u], len[u]);
  }
#pragma unroll
  for (int u = 0; u < kSlotsPer; ++u) {
    base[u] = 0;
    if (rank[u] == 0 && key[u] != MPG_DEAD) base[u] = atomicAdd(&fill[key[u]], (unsigned)len[u]);
    st[u] = key[u] != MPG_DEAD ? start[key[u]] : 0u;
  }
#pragma unroll
  for (int u = 0; u < kSlotsPer; ++u) {
    const uint32_t b = __shfl_sync(0xffffffffu, base[u], first[u]);
    if (key[u] != MPG_DEAD) perm[st[u] + b + (uint32_t)rank[u]] = (uint32_t)(p0 + (int64_t)u * blockDim.x);
  }
}

// ranges of up to kSortLocal entries are sorted by one thread (a sorting
// network in registers); ranges of up to kSortWarp entries are listed for
// k_cell_order_warp (one warp each), longer ones for k_cell_order_long (one
// block each).  The two lists share one buffer: medium ranges from the
// front (counter long_count[0]), long ones from the back (long_count[1]).
constexpr int kSortLocal = 32;
constexpr int kSortWarp = 1024;

// Ascending sort of a[0..m), m <= N (N a power of two), in registers: the
// entries padded to N with the largest key; a range found in order (most are:
// claimed by one warp run) is left as it is, any other goes through a bitonic
// sorting network whose loops unroll completely (every index a constant), so
// nothing goes through local memory, and is written back.
template <int N>
__device__ __forceinline__ void sort_range_net(uint32_t *__restrict__ a, uint32_t m) {
  uint32_t v[N];
#pragma unroll
  for (int k = 0; k < N; ++k) v[k] = (uint32_t)k < m ? a[k] : 0xFFFFFFFFu;
  bool in_order = true;
#pragma unroll
  for (int k = 0; k + 1 < N; ++k) in_order = in_order && v[k] <= v[k + 1];  // the padding is in order too
  if (in_order) return;
#pragma unroll
  for (int k = 2; k <= N; k <<= 1)
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const int l = i ^ j;
        if (l > i) {
          const uint32_t x = v[i], y = v[l];
          const bool up = (i & k) == 0;
          v[i] = up ? min(x, y) : max(x, y);
          v[l] = up ? max(x, y) : min(x, y);
        }
      }
#pragma unroll
  for (int k = 0; k < N; ++k)
    if ((uint32_t)k < m) a[k] = v[k];
}
__global__ void k_cell_order(const uint32_t *__restrict__ start, int64_t T, uint32_t *__restrict__ perm,
                             uint32_t *__restrict__ lists, int64_t list_len, uint32_t *__restrict__ long_count) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= T) return;
  const uint32_t lo = start[e], m = start[e + 1] - lo;
  if (m < 2) return;
  if (m > (uint32_t)kSortLocal) {
    if (m <= (uint32_t)kSortWarp)
      lists[atomicAdd(long_count, 1u)] = (uint32_t)e;
    else
      lists[list_len - 1 - atomicAdd(long_count + 1, 1u)] = (uint32_t)e;
    return;
  }
  if (m <= 16)
    sort_range_net<16>(perm + lo, m);
  else
    sort_range_net<32>(perm + lo, m);
}

// number of entries of a taken among the first d outputs of the merge of
// sorted runs a[0..la) and b[0..lb) (entries are distinct)
__device__ __forceinline__ uint32_t merge_split(const uint32_t *a, uint32_t la, const uint32_t *b, uint32_t lb,
                                                uint32_t d) {
  uint32_t lo = d > lb ? d - lb : 0u, hi = d < la ? d : la;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a[mid] <= b[d - 1 - mid])
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

// Medium ranges, one warp each (warp-stride over the list): a bitonic sort of
// the range padded to the next power of two, in the warp's shared-memory
// slice, with warp-level synchronisation only.
constexpr int kWarpSortThreads = 256;
__global__ void __launch_bounds__(kWarpSortThreads) k_cell_order_warp(const uint32_t *__restrict__ start,
                                                                     const uint32_t *__restrict__ lists,
                                                                     const uint32_t *__restrict__ long_count,
                                                                     uint32_t *__restrict__ perm) {
  __shared__ uint32_t sm[(kWarpSortThreads / 32) * kSortWarp];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t *a = sm + wid * kSortWarp;
  const uint32_t nl = long_count[0];
  const uint32_t nwarps = gridDim.x * (kWarpSortThreads / 32);
  for (uint32_t li = blockIdx.x * (kWarpSortThreads / 32) + wid; li < nl; li += nwarps) {
    const uint32_t e = lists[li];
    const uint32_t lo = start[e], m = start[e + 1] - lo;
    uint32_t P = 64;
    while (P < m) P <<= 1;
    for (uint32_t i = lane; i < P; i += 32) a[i] = i < m ? perm[lo + i] : 0xFFFFFFFFu;
    __syncwarp();
    for (uint32_t k = 2; k <= P; k <<= 1)
      for (uint32_t j = k >> 1; j > 0; j >>= 1) {
        for (uint32_t i = lane; i < P; i += 32) {
          const uint32_t ixj = i ^ j;
          if (ixj > i) {
            const uint32_t x = a[i], y = a[ixj];
            if ((x > y) == ((i & k) == 0)) {
              a[i] = y;
              a[ixj] = x;
            }
          }
        }
        __syncwarp();
      }
    for (uint32_t i = lane; i < m; i += 32) perm[lo + i] = a[i];
    __syncwarp();
  }
}

// Long ranges, one block each (grid-stride over the list): tiles of
// kLongTile entries are sorted in shared memory (bitonic), then runs are
// merged pairwise (merge path split over the block's threads) between the
// range and the same range of tmp, until one run is left.
constexpr int kLongThreads = 1024;
constexpr int kLongTile = 4096;
__global__ void __launch_bounds__(kLongThreads) k_cell_order_long(const uint32_t *__restrict__ start,
                                                                  const uint32_t *__restrict__ lists,
                                                                  int64_t list_len,
                                                                  const uint32_t *__restrict__ long_count,
                                                                  uint32_t *__restrict__ perm,
                                                                  uint32_t *__restrict__ tmp) {
  __shared__ uint32_t sm[kLongTile];
  const uint32_t nl = long_count[1];
  const int tid = threadIdx.x;
  for (uint32_t li = blockIdx.x; li < nl; li += gridDim.x) {
    const uint32_t e = lists[list_len - 1 - li];
    const uint32_t lo = start[e], m = start[e + 1] - lo;
    uint32_t *a = perm + lo;
    for (uint32_t t0 = 0; t0 < m; t0 += kLongTile) {
      const uint32_t len = min((uint32_t)kLongTile, m - t0);
      for (int i = tid; i < kLongTile; i += kLongThreads) sm[i] = (uint32_t)i < len ? a[t0 + i] : 0xFFFFFFFFu;
      __syncthreads();
      for (int k = 2; k <= kLongTile; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
          for (int i = tid; i < kLongTile; i += kLongThreads) {
            const int ixj = i ^ j;
            if (ixj > i) {
              const uint32_t x = sm[i], y = sm[ixj];
              if ((x > y) == ((i & k) == 0)) {
                sm[i] = y;
                sm[ixj] = x;
              }
            }
          }
          __syncthreads();
        }
      for (int i = tid; (uint32_t)i < len; i += kLongThreads) a[t0 + i] = sm[i];
      __syncthreads();
    }
    uint32_t *src = a, *dst = tmp + lo;
    for (uint32_t w = kLongTile; w < m; w <<= 1) {
      for (uint32_t p0 = 0; p0 < m; p0 += 2 * w) {
        const uint32_t l1 = min(w, m - p0), l2 = min(w, m - p0 - l1), L = l1 + l2;
        const uint32_t *A = src + p0, *B = src + p0 + l1;
        const uint32_t d0 = (uint32_t)(((uint64_t)L * tid) / kLongThreads);
        const uint32_t d1 = (uint32_t)(((uint64_t)L * (tid + 1)) / kLongThreads);
        uint32_t i = merge_split(A, l1, B, l2, d0), j = d0 - i;
        for (uint32_t d = d0; d < d1; ++d) {
          if (j >= l2 || (i < l1 && A[i] <= B[j]))
            dst[p0 + d] = A[i++];
          else
            dst[p0 + d] = B[j++];
        }
      }
      __syncthreads();
      uint32_t *t = src;
      src = dst;
      dst = t;
    }
    if (src != a)
      for (uint32_t i = tid; i < m; i += kLongThreads) a[i] = src[i];
    __syncthreads();
  }
}

// sorted slot i < count takes input record perm[i]; slots [count, n) are
// dead (the grid bound n stays the old count until the host reads the new one)
// four particles per thread (strided by the block), their permutation
// entries first, so that twelve record loads are in flight per thread
constexpr int kGatherPer = 4;
__global__ void k_sort_gather_mixed(MixedParts P, int64_t n, MixedParts Q, const uint32_t *__restrict__ perm,
                                    const uint32_t *__restrict__ count) {
  const int64_t cnt = (int64_t)*count;
  const int64_t base = (int64_t)blockIdx.x * blockDim.x * kGatherPer + threadIdx.x;
  uint32_t src[kGatherPer];
#pragma unroll
  for (int u = 0; u < kGatherPer; ++u) {
    const int64_t i = base + (int64_t)u * blockDim.x;
    src[u] = i < cnt ? perm[i] : 0u;
  }
  uint32_t c[kGatherPer];
  float4 b[kGatherPer];
  float2 v[kGatherPer];
#pragma unroll
  for (int u = 0; u < kGatherPer; ++u) {
    if (base + (int64_t)u * blockDim.x < cnt) {
      c[u] = P.c[src[u]];
      b[u] = P.b[src[u]];
      v[u] = P.v[src[u]];
    }
  }
#pragma unroll
  for (int u = 0; u < kGatherPer; ++u) {
    const int64_t i = base + (int64_t)u * blockDim.x;
    if (i < cnt) {
      Q.c[i] = c[u];
      Q.b[i] = b[u];
      Q.v[i] = v[u];
      if (P.id) Q.id[i] = P.id[src[u]];
    } else if (i < n) {
      Q.c[i] = MPG_DEAD;
    }
  }
}

__global__ void k_sort_gather_plain(PlainParts P, PlainParts Q, const uint32_t *__restrict__ perm,
                                    const uint32_t *__restrict__ count) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (int64_t)*count) return;
  const int64_t p = perm[i];
  Q.cell[i] = P.cell[p];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    Q.x[d * Q.cap + i] = P.x[d * P.cap + p];
    Q.xr[d * Q.cap + i] = P.xr[d * P.cap + p];
    Q.v[d * Q.cap + i] = P.v[d * P.cap + p];
  }
  Q.w[i] = P.w[p];
  Q.sp[i] = P.sp[p];
  if (P.id) Q.id[i] = P.id[p];
}

__global__ void k_copy_u32(const uint32_t *src, uint32_t *dst) { *dst = *src; }

// initial guess of the next solve from the last solutions (see launch_extrapolate)
__global__ void k_extrapolate(int64_t n, double *__restrict__ phi, double *__restrict__ prev,
                              double *__restrict__ prev2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double a = phi[i], b = prev[i];
  if (prev2) {
    phi[i] = 3.0 * (a - b) + prev2[i];
    prev2[i] = b;
  } else {
    phi[i] = 2.0 * a - b;
  }
  prev[i] = a;
}


// ---------------------------------------------------------------------------
// fills
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t draw(uint64_t base, uint64_t ctr) { return mix64(base + mix64(ctr)); }
__device__ __forceinline__ float f24(uint64_t h) { return (float)(h >> 40) * (1.0f / 16777216.0f); }

__device__ __forceinline__ void ref_to_phys(const DevMesh &M, int e, const double r[3], double out[3]) {
  // mesh.hpp:182-190
  const double w[4] = {1 - r[0] - r[1] - r[2], r[0], r[1], r[2]};
  const int4 nd = M.tets[e];
  const int ids[4] = {nd.x, nd.y, nd.z, nd.w};
  out[0] = out[1] = out[2] = 0.0;
  for (int i = 0; i < 4; ++i)
    for (int d = 0; d < 3; ++d) out[d] += w[i] * M.nodes[3 * ids[i] + d];
}

__global__ void k_fill_uniform(int mixed, PlainParts P, MixedParts X, int64_t n0, int64_t n, uint64_t base, int type,
                               double weight, double dr0, double dr1, double dr2, float vth, DevMesh M, int64_t id0) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint64_t c0 = (uint64_t)k << 8;
  const uint64_t T = (uint64_t)M.T;
  uint64_t e = 0;
  for (uint64_t j = 0; j < 128; j += 2) {
    e = ((draw(base, c0 | j) >> 32) * T) >> 32;
    if (f24(draw(base, c0 | (j + 1))) < M.fill_ratio[e]) break;
  }
  float s = f24(draw(base, c0 | 128));
  float t = f24(draw(base, c0 | 129));
  float u = f24(draw(base, c0 | 130));
  // Rocchini & Cignoni (2000): fold the unit cube onto the unit tet
  if (s + t > 1.0f) {
    s = 1.0f - s;
    t = 1.0f - t;
  }
  if (t + u > 1.0f) {
    const float tmp = u;
    u = 1.0f - s - t;
    t = 1.0f - tmp;
  } else if (s + t + u > 1.0f) {
    const float tmp = u;
    u = s + t + u - 1.0f;
    s = 1.0f - t - tmp;
  }
  const float a0 = f24(draw(base, c0 | 131)), a1 = f24(draw(base, c0 | 132));
  const float a2 = f24(draw(base, c0 | 133)), a3 = f24(draw(base, c0 | 134));
  const float twopi = 6.28318530717958648f;
  const float rr0 = sqrtf(-2.0f * logf(1.0f - a0)), rr1 = sqrtf(-2.0f * logf(1.0f - a2));
  const float g[3] = {rr0 * cosf(twopi * a1), rr0 * sinf(twopi * a1), rr1 * cosf(twopi * a3)};
  const float drift[3] = {(float)dr0, (float)dr1, (float)dr2};
  float vf[3];
  for (int d = 0; d < 3; ++d) vf[d] = drift[d] + vth * g[d];
  const int64_t dst = n0 + k;
  if (mixed) {
    X.c[dst] = ((uint32_t)type << 24) | (uint32_t)e;
    X.b[dst] = make_float4(s, t, u, vf[0]);
    X.v[dst] = make_float2(vf[1], vf[2]);
    if (X.id) X.id[dst] = id0 + k;
  } else {
    const double xr[3] = {(double)s, (double)t, (double)u};
    double xp[3];
    ref_to_phys(M, (int)e, xr, xp);
    P.cell[dst] = (int32_t)e;
    for (int d = 0; d < 3; ++d) {
      P.x[d * P.cap + dst] = xp[d];
      P.xr[d * P.cap + dst] = xr[d];
      P.v[d * P.cap + dst] = (double)vf[d];
    }
    P.w[dst] = weight;
    P.sp[dst] = type;
    if (P.id) P.id[dst] = id0 + k;
  }
}

// particle_fill.hpp:129-164 with the seed of :147 and set_vel of :100-124;
// particle (elem, ipart) lands at n0 + elem*nppe + ipart (Serial push order)
__global__ void k_fill_ref(PlainParts P, int64_t n0, int nppe, int type, double density, double v0, double v1,
                           double v2, double temp, double mass, DevMesh M, int64_t id0) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t total = M.T * (int64_t)nppe;
  if (k >= total) return;
  const int64_t elem = k / nppe;
  const uint64_t ipart = (uint64_t)(k % nppe);
  const int64_t NG = M.T;
  uint64_t sd = (uint64_t)elem + (34030 + ipart) * (uint64_t)NG + (uint64_t)(NG * 12345 * (int64_t)type);
  auto rnd = [&]() -> uint64_t {
    sd = 6364136223846793005ULL * sd + 1442695040888963407ULL;
    return sd;
  };
  const double dscale = 1. / static_cast<double>(18446744073709551615ULL);
  auto drand = [&]() -> double { return (double)rnd() * dscale; };
  for (int i = 0; i < 10; ++i) rnd();
  // rejection loops of the reference are unbounded; here they stop after
  // 2^20 tries (acceptance is 1/6 for x_ref and far above 1e-6 for the
  // Maxwellian at any sane temperature, so the cap is never reached)
  const int kMaxTries = 1 << 20;
  double xr[3];
  int tries = 0;
  do {
    xr[0] = drand();
    xr[1] = drand();
    xr[2] = drand();
  } while (xr[0] + xr[1] + xr[2] > 1.0 && ++tries < kMaxTries);
  double xp[3];
  ref_to_phys(M, (int)elem, xr, xp);
  const double vel[3] = {v0, v1, v2};
  double vp[3];
  if (temp == 0) {
    vp[0] = vel[0];
    vp[1] = vel[1];
    vp[2] = vel[2];
  } else if (temp < 0) {
    vp[0] = vel[0] * (1. + temp * sin(1. * 3.14159265358979323846 * xp[0]));
    vp[1] = vp[2] = 0.0;
  } else {
    for (int k = 0;; ++k) {
      const double r = drand();
      const double vmax = sqrt(6 * temp / mass);
      double vv[3];
      vv[0] = vmax * 2 * (-.5 + drand());
      vv[1] = vmax * 2 * (-.5 + drand());
      vv[2] = vmax * 2 * (-.5 + drand());
      const double prob = exp(-(vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2]) / temp);
      if (r < prob || k >= kMaxTries) {
        vp[0] = vel[0] + vv[0];
        vp[1] = vel[1] + vv[1];
        vp[2] = vel[2] + vv[2];
        break;
      }
    }
  }
  const double vol = M.detj[elem] / 6.;
  const int64_t dst = n0 + k;
  P.cell[dst] = (int32_t)elem;
  for (int d = 0; d < 3; ++d) {
    P.x[d * P.cap + dst] = xp[d];
    P.xr[d * P.cap + dst] = xr[d];
    P.v[d * P.cap + dst] = vp[d];
  }
  P.w[dst] = density * vol / nppe;
  P.sp[dst] = type;
  if (P.id) P.id[dst] = id0 + k;
}

__global__ void k_rows_to_cols(const double *__restrict__ rows, double *__restrict__ cols, int64_t n, int64_t cap) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  for (int d = 0; d < 3; ++d) cols[d * cap + p] = rows[3 * p + d];
}
__global__ void k_cols_to_rows(const double *__restrict__ cols, double *__restrict__ rows, int64_t n, int64_t cap) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  for (int d = 0; d < 3; ++d) rows[3 * p + d] = cols[d * cap + p];
}
// validation of uploaded cell/species words: out[0] = lowest index of an
// entry with a cell out of range, a species out of range or a species without
// weight (initialised to all ones), out[1] += live entries
__global__ void k_mixed_check(const uint32_t *__restrict__ cs, int64_t n, int64_t T, uint32_t weight_mask,
                              unsigned long long *__restrict__ out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned live = 0;
  if (i < n) {
    const uint32_t w = cs[i];
    if (w != MPG_DEAD) {
      const uint32_t sp = w >> 24;
      if ((int64_t)(w & 0xFFFFFFu) >= T || sp >= MPG_MAX_SPECIES || !((weight_mask >> sp) & 1u))
        atomicMin(&out[0], (unsigned long long)i);
      else
        live = 1;
    }
  }
  live = __reduce_add_sync(0xffffffffu, live);
  if ((threadIdx.x & 31) == 0 && live) atomicAdd(&out[1], (unsigned long long)live);
}

// Host layout (b and v as float[3] per particle) <-> device records.  A
// warp moves its 32 particles' 384-byte spans of b and v as 24 float4 each,
// through shared memory, so that every access to the host arrays (which may
// be mapped host memory, read and written over the host link) is a full
// 16-byte vector; arrays not 16-byte aligned, and the last partial warp, go
// element by element.
constexpr int kPackWarps = kThreads / 32;
// With cs (checked packing): the cell words go to X.c as well, each one
// checked as k_mixed_check does (first bad index and live count in out), and
// with acc the charge of every checked live particle is deposited as
// k_mixed_deposit does (the same integer sums; the slots are zeroed first).
__global__ void __launch_bounds__(kThreads) k_mixed_pack(const float *__restrict__ b, const float *__restrict__ v,
                                                         MixedParts X, int64_t n, const uint32_t *__restrict__ cs,
                                                         int64_t T, uint32_t weight_mask,
                                                         unsigned long long *__restrict__ out,
                                                         const int4 *__restrict__ c2n, SpeciesTable S,
                                                         unsigned long long *__restrict__ acc) {
  __shared__ float4 sm[kPackWarps][2][24];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t p0 = ((int64_t)blockIdx.x * blockDim.x) + 32 * wib, p = p0 + lane;
  int key = -1;  // the cell whose charge this lane deposits
  int Q = 0;
  if (cs) {
    unsigned live = 0;
    if (p < n) {
      const uint32_t w = cs[p];
      X.c[p] = w;
      if (w != MPG_DEAD) {
        const uint32_t sp = w >> 24;
        if ((int64_t)(w & 0xFFFFFFu) >= T || sp >= MPG_MAX_SPECIES || !((weight_mask >> sp) & 1u)) {
          atomicMin(&out[0], (unsigned long long)p);
        } else {
          live = 1;
          key = (int)(w & 0xFFFFFFu);
          Q = (int)S.qfix[sp];
        }
      }
    }
    live = __reduce_add_sync(0xffffffffu, live);
    if (lane == 0 && live) atomicAdd(&out[1], (unsigned long long)live);
  }
  const bool vec = ((reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(v)) & 15u) == 0 && p0 + 32 <= n;
  float4 bw = make_float4(0.f, 0.f, 0.f, 0.f);
  if (vec) {
    if (lane < 24) {
      sm[wib][0][lane] = reinterpret_cast<const float4 *>(b + 3 * p0)[lane];
      sm[wib][1][lane] = reinterpret_cast<const float4 *>(v + 3 * p0)[lane];
    }
    __syncwarp();
    const float *fb = reinterpret_cast<const float *>(sm[wib][0]), *fv = reinterpret_cast<const float *>(sm[wib][1]);
    bw = make_float4(fb[3 * lane], fb[3 * lane + 1], fb[3 * lane + 2], fv[3 * lane]);
    X.b[p] = bw;
    X.v[p] = make_float2(fv[3 * lane + 1], fv[3 * lane + 2]);
  } else if (p < n) {
    bw = make_float4(b[3 * p], b[3 * p + 1], b[3 * p + 2], v[3 * p]);
    X.b[p] = bw;
    X.v[p] = make_float2(v[3 * p + 1], v[3 * p + 2]);
  }
  // every lane of the warp is here (acc is uniform across the grid)
  if (acc) deposit_fixed_warp(acc, c2n, key, bw.x, bw.y, bw.z, Q);
}
__global__ void __launch_bounds__(kThreads) k_mixed_unpack(MixedParts X, int64_t n, float *__restrict__ b,
                                                           float *__restrict__ v, uint32_t *__restrict__ cs) {
  __shared__ float4 sm[kPackWarps][2][24];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int64_t p0 = ((int64_t)blockIdx.x * blockDim.x) + 32 * wib, p = p0 + lane;
  if (cs && p < n) cs[p] = X.c[p];
  const bool vec = ((reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(v)) & 15u) == 0 && p0 + 32 <= n;
  if (vec) {
    const float4 a = X.b[p];
    const float2 c = X.v[p];
    float *fb = reinterpret_cast<float *>(sm[wib][0]), *fv = reinterpret_cast<float *>(sm[wib][1]);
    fb[3 * lane] = a.x;
    fb[3 * lane + 1] = a.y;
    fb[3 * lane + 2] = a.z;
    fv[3 * lane] = a.w;
    fv[3 * lane + 1] = c.x;
    fv[3 * lane + 2] = c.y;
    __syncwarp();
    if (lane < 24) {
      reinterpret_cast<float4 *>(b + 3 * p0)[lane] = sm[wib][0][lane];
      reinterpret_cast<float4 *>(v + 3 * p0)[lane] = sm[wib][1][lane];
    }
    return;
  }
  if (p >= n) return;
  const float4 a = X.b[p];
  const float2 c = X.v[p];
  b[3 * p] = a.x;
  b[3 * p + 1] = a.y;
  b[3 * p + 2] = a.z;
  v[3 * p] = a.w;
  v[3 * p + 1] = c.x;
  v[3 * p + 2] = c.y;
}
__global__ void k_plain_to_mixed(PlainParts P, int64_t n0, int64_t n, MixedParts X) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int64_t p = n0 + k;
  const int32_t e = P.cell[p];
  X.c[p] = e < 0 ? MPG_DEAD : (((uint32_t)P.sp[p] << 24) | (uint32_t)e);
  X.b[p] = make_float4((float)P.xr[p], (float)P.xr[P.cap + p], (float)P.xr[2 * P.cap + p], (float)P.v[p]);
  X.v[p] = make_float2((float)P.v[P.cap + p], (float)P.v[2 * P.cap + p]);
  if (X.id) X.id[p] = P.id ? P.id[p] : p;
}
__global__ void k_mixed_to_plain(MixedParts X, int64_t n, DevMesh M, SpeciesTable S, PlainParts P) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const uint32_t cs = X.c[p];
  const float4 a = X.b[p];
  const float2 c = X.v[p];
  const double xr[3] = {(double)a.x, (double)a.y, (double)a.z};
  double xp[3] = {0.0, 0.0, 0.0};
  const int s = cs == MPG_DEAD ? 0 : (int)(cs >> 24);
  if (cs != MPG_DEAD) ref_to_phys(M, (int)(cs & 0xFFFFFFu), xr, xp);
  P.cell[p] = cs == MPG_DEAD ? -1 : (int32_t)(cs & 0xFFFFFFu);
  const double vv[3] = {(double)a.w, (double)c.x, (double)c.y};
  for (int d = 0; d < 3; ++d) {
    P.x[d * P.cap + p] = xp[d];
    P.xr[d * P.cap + p] = xr[d];
    P.v[d * P.cap + p] = vv[d];
  }
  P.w[p] = S.w[s];
  P.sp[p] = s;
  if (P.id) P.id[p] = X.id ? X.id[p] : p;
}

}  // namespace

// ---------------------------------------------------------------------------
// launch wrappers
int64_t scan_scratch_len(int64_t n) { return (n + kScanTile - 1) / kScanTile + 2; }

void scan_u32(cudaStream_t s, const uint32_t *in, uint32_t *out, int64_t n, uint32_t *scratch, int64_t) {
  const int64_t nt = (n + kScanTile - 1) / kScanTile;
  const unsigned g = (unsigned)(nt < 1 ? 1 : nt);
  k_scan_tiles<<<g, kScanThreads, 0, s>>>(in, n, scratch);
  k_scan_sums<<<1, kScanThreads, 0, s>>>(scratch, g);
  k_scan_apply<<<g, kScanThreads, 0, s>>>(in, n, scratch, out, g);
}

void launch_plain_deposit(cudaStream_t s, const PlainParts &P, int64_t n, const DevMesh &M, const SpeciesTable &S,
                          int mode, double *rhs) {
  if (n <= 0) return;
  k_plain_deposit<<<grid_for(n), kThreads, 0, s>>>(P, n, M.tets, M.detj, S, mode, rhs);
}
void launch_rhs_finish(cudaStream_t s, const DevMesh &M, double *rhs, const double *bg) {
  k_rhs_finish<<<grid_for(M.N), kThreads, 0, s>>>(M.N, rhs, bg, M.bnd, M.nsolve, M.fper ? M.plane : 0);
}
__global__ void k_periodic_copy(double *__restrict__ phi, int64_t nsolve, int64_t plane) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < plane) phi[nsolve + i] = phi[i];
}
void launch_periodic_copy(cudaStream_t s, const DevMesh &M, double *phi) {
  if (M.fper && M.plane > 0) k_periodic_copy<<<grid_for(M.plane), kThreads, 0, s>>>(phi, M.nsolve, M.plane);
}
void launch_efield_plain(cudaStream_t s, const DevMesh &M, const double *phi, double *Etet) {
  k_efield_plain<<<grid_for(M.T), kThreads, 0, s>>>(M.T, M.tets, M.grad, phi, Etet);
}
void launch_plain_move(cudaStream_t s, const PlainParts &P, int64_t n, const DevMesh &M, const double *Etet,
                       const SpeciesTable &S, double dt, int kill, int max_cross, DevStats *st) {
  if (n <= 0) return;
  k_plain_move<<<grid_for(n), kThreads, 0, s>>>(P, n, M, Etet, S, dt, kill, max_cross, st);
}
void launch_compact_plain(cudaStream_t s, const PlainParts &P, int64_t n, const PlainParts &Q, uint32_t *scratch,
                          int64_t, uint32_t *d_count) {
  const int64_t nt = (n + kScanTile - 1) / kScanTile;
  const unsigned g = (unsigned)(nt < 1 ? 1 : nt);
  k_count_live<<<g, kScanThreads, 0, s>>>(P.cell, n, scratch);
  k_scan_sums<<<1, kScanThreads, 0, s>>>(scratch, g);
  k_compact_plain<<<g, kScanThreads, 0, s>>>(P, n, Q, scratch, g, d_count);
}
void launch_mixed_deposit(cudaStream_t s, const MixedParts &P, int64_t n, const DevMesh &M, const SpeciesTable &S,
                          unsigned long long *acc) {
  if (n <= 0) return;
  k_mixed_deposit<<<grid_for(n), kThreads, 0, s>>>(P, n, M.c2n, S, acc);
}
void launch_mixed_convert(cudaStream_t s, const DevMesh &M, unsigned long long *acc, double quantum, const double *bg,
                          double *rhs) {
  k_mixed_convert<<<grid_for(M.N), kThreads, 0, s>>>(M.N, M.n2c_off, acc, quantum, bg, M.bnd, rhs,
                                                     M.nsolve, M.fper ? M.plane : 0);
}
void launch_node_quanta(cudaStream_t s, const DevMesh &M, const unsigned long long *acc, long long *out) {
  k_node_quanta<<<grid_for(M.N), kThreads, 0, s>>>(M.N, M.n2c_off, acc, out);
}
void launch_efield_mixed(cudaStream_t s, const DevMesh &M, const double *phi, unsigned long long *zero,
                         int64_t nzero) {
  if (M.kuhn) {
    k_efield_kuhn<<<(unsigned)((M.T / 6 + kEfThreads - 1) / kEfThreads), kEfThreads, 0, s>>>(M.T, M.ktab, phi,
                                                                                            M.etet4, zero, nzero);
  } else {
    k_efield_mixed<<<grid_for(M.T), kThreads, 0, s>>>(M.T, M.tets, M.mrec, phi);
    if (zero && nzero > 0) cudaMemsetAsync(zero, 0, sizeof(unsigned long long) * nzero, s);
  }
}
// resident blocks of a persistent move kernel on the current device (one wave)
template <bool KUHN>
static unsigned move_wave_blocks() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) dev = 0;
  if (!cached[dev]) {
    int sms = 0, occ = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_mixed_move_persistent<KUHN>, kThreads, 0);
    cached[dev] = (sms > 0 ? sms : 1) * (occ > 0 ? occ : 1);
  }
  return (unsigned)cached[dev];
}
static void move_persistent(cudaStream_t s, const MixedParts &P, int64_t n, const MixedParts &Q,
                            const uint32_t *perm, const uint32_t *d_count, const DevMesh &M, const SpeciesTable &S,
                            float dt, int kill, int max_cross, unsigned long long *acc, uint32_t *hist,
                            DevStats *st) {
  const unsigned want = grid_for(n);
  if (M.kuhn) {
    const unsigned wave = move_wave_blocks<true>();
    k_mixed_move_persistent<true><<<want < wave ? want : wave, kThreads, 0, s>>>(
        P, n, Q, perm, d_count, M.mrec, M.mnbr, M.etet4, M.ktab, M.c2n, S, dt, kill, max_cross, acc, hist, st);
  } else {
    const unsigned wave = move_wave_blocks<false>();
    k_mixed_move_persistent<false><<<want < wave ? want : wave, kThreads, 0, s>>>(
        P, n, Q, perm, d_count, M.mrec, M.mnbr, M.etet4, M.ktab, M.c2n, S, dt, kill, max_cross, acc, hist, st);
  }
}
void launch_mixed_move(cudaStream_t s, const MixedParts &P, int64_t n, const DevMesh &M, const SpeciesTable &S,
                       float dt, int kill, int max_cross, unsigned long long *acc, DevStats *st, uint32_t *hist) {
  if (n <= 0) return;
  static const char *env = getenv("MPG_MOVE_KERNEL");
  if (!M.kuhn && env && atoi(env) == 0 && !hist) {
    k_mixed_move<<<grid_for(n), kThreads, 0, s>>>(P, n, M.mrec, M.mnbr, M.c2n, S, dt, kill, max_cross, acc, st);
    return;
  }
  move_persistent(s, P, n, P, nullptr, nullptr, M, S, dt, kill, max_cross, acc, hist, st);
}
void launch_mixed_move_sorted(cudaStream_t s, const MixedParts &P, int64_t n, const MixedParts &Q,
                              const uint32_t *perm, const uint32_t *d_count, const DevMesh &M, const SpeciesTable &S,
                              float dt, int kill, int max_cross, unsigned long long *acc, DevStats *st,
                              uint32_t *hist) {
  if (n <= 0) return;
  move_persistent(s, P, n, Q, perm, d_count, M, S, dt, kill, max_cross, acc, hist, st);
}
// the five passes of the stable cell sort; leaves perm[0..count) and start
// (T + 1 entries) behind, and the count in *d_count
// (have_hist: w.cnt already holds the particles per cell, counted by the move)
template <bool kMixed>
static void cell_sort_order(cudaStream_t s, const uint32_t *keys, int64_t n, int64_t T, const SortWork &w,
                            uint32_t *tmp, uint32_t *d_count, bool have_hist = false) {
  cudaMemsetAsync(w.long_count, 0, 2 * sizeof(uint32_t), s);
  if (!have_hist) {
    cudaMemsetAsync(w.cnt, 0, sizeof(uint32_t) * T, s);
    if (n > 0) k_cell_hist<kMixed><<<grid_for(n), kThreads, 0, s>>>(keys, n, w.cnt);
  }
  scan_u32(s, w.cnt, w.start, T, w.scan_scratch, w.scan_len);
  cudaMemsetAsync(w.cnt, 0, sizeof(uint32_t) * T, s);
  if (n > 0)
    k_cell_slots<kMixed><<<grid_for((n + kSlotsPer - 1) / kSlotsPer), kThreads, 0, s>>>(keys, n, w.start, w.cnt,
                                                                                       w.perm);
  k_cell_order<<<grid_for(T), kThreads, 0, s>>>(w.start, T, w.perm, w.long_list, w.list_len, w.long_count);
  k_cell_order_warp<<<w.long_blocks * 4, kWarpSortThreads, 0, s>>>(w.start, w.long_list, w.long_count, w.perm);
  k_cell_order_long<<<w.long_blocks, kLongThreads, 0, s>>>(w.start, w.long_list, w.list_len, w.long_count, w.perm,
                                                            tmp);
  k_copy_u32<<<1, 1, 0, s>>>(w.start + T, d_count);
}
void launch_mixed_sort_order(cudaStream_t s, const MixedParts &P, int64_t n, const MixedParts &Q, int64_t T,
                             const SortWork &w, uint32_t *d_count, bool have_hist) {
  cell_sort_order<true>(s, P.c, n, T, w, Q.c, d_count, have_hist);
}
void launch_mixed_gather(cudaStream_t s, const MixedParts &P, int64_t n, const MixedParts &Q, const uint32_t *perm,
                         const uint32_t *d_count) {
  if (n > 0)
    k_sort_gather_mixed<<<grid_for((n + kGatherPer - 1) / kGatherPer), kThreads, 0, s>>>(P, n, Q, perm, d_count);
}
void launch_mixed_sort(cudaStream_t s, const MixedParts &P, int64_t n, const MixedParts &Q, int64_t T,
                       const SortWork &w, uint32_t *d_count) {
  launch_mixed_sort_order(s, P, n, Q, T, w, d_count);
  launch_mixed_gather(s, P, n, Q, w.perm, d_count);
}
void launch_plain_sort(cudaStream_t s, const PlainParts &P, int64_t n, const PlainParts &Q, int64_t T,
                       const SortWork &w, uint32_t *d_count) {
  cell_sort_order<false>(s, (const uint32_t *)P.cell, n, T, w, (uint32_t *)Q.cell, d_count);
  if (n > 0) k_sort_gather_plain<<<grid_for(n), kThreads, 0, s>>>(P, Q, w.perm, d_count);
}
int sort_long_blocks(int device) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  return 2 * (sms > 0 ? sms : 1);
}
void launch_extrapolate(cudaStream_t s, int64_t n, double *phi, double *prev, double *prev2) {
  if (n > 0) k_extrapolate<<<grid_for(n), kThreads, 0, s>>>(n, phi, prev, prev2);
}
void launch_fill_uniform(cudaStream_t s, int mixed, const PlainParts &P, const MixedParts &X, int64_t n0, int64_t n,
                         uint64_t seed, int type, double weight, const double drift[3], double vth, const DevMesh &M,
                         int64_t id0) {
  if (n <= 0) return;
  const uint64_t base = mpg_mix64(seed ^ MPG_SALT_FILL);
  k_fill_uniform<<<grid_for(n), kThreads, 0, s>>>(mixed, P, X, n0, n, base, type, weight, drift[0], drift[1],
                                                   drift[2], (float)vth, M, id0);
}
void launch_fill_ref(cudaStream_t s, const PlainParts &P, int64_t n0, int nppe, int type, double density,
                     const double vel[3], double temp, double mass, const DevMesh &M, int64_t id0) {
  const int64_t total = M.T * (int64_t)nppe;
  if (total <= 0) return;
  k_fill_ref<<<grid_for(total, 128), 128, 0, s>>>(P, n0, nppe, type, density, vel[0], vel[1], vel[2], temp, mass, M,
                                                   id0);
}
void launch_rows_to_cols(cudaStream_t s, const double *rows, double *cols, int64_t n, int64_t cap) {
  if (n > 0) k_rows_to_cols<<<grid_for(n), kThreads, 0, s>>>(rows, cols, n, cap);
}
void launch_cols_to_rows(cudaStream_t s, const double *cols, double *rows, int64_t n, int64_t cap) {
  if (n > 0) k_cols_to_rows<<<grid_for(n), kThreads, 0, s>>>(cols, rows, n, cap);
}
void launch_mixed_pack(cudaStream_t s, const float *b, const float *v, MixedParts X, int64_t n) {
  if (n > 0)
    k_mixed_pack<<<grid_for(n), kThreads, 0, s>>>(b, v, X, n, nullptr, 0, 0u, nullptr, nullptr, SpeciesTable{},
                                                  nullptr);
}
void launch_mixed_pack_checked(cudaStream_t s, const uint32_t *cs, const float *b, const float *v, MixedParts X,
                               int64_t n, int64_t T, uint32_t weight_mask, unsigned long long *out,
                               const DevMesh &M, const SpeciesTable &S, unsigned long long *acc) {
  if (n > 0) k_mixed_pack<<<grid_for(n), kThreads, 0, s>>>(b, v, X, n, cs, T, weight_mask, out, M.c2n, S, acc);
}
void launch_mixed_check(cudaStream_t s, const uint32_t *cs, int64_t n, int64_t T, uint32_t weight_mask,
                        unsigned long long *out) {
  if (n > 0) k_mixed_check<<<grid_for(n), kThreads, 0, s>>>(cs, n, T, weight_mask, out);
}
void launch_mixed_unpack(cudaStream_t s, const MixedParts X, int64_t n, float *b, float *v, uint32_t *cs) {
  if (n > 0) k_mixed_unpack<<<grid_for(n), kThreads, 0, s>>>(X, n, b, v, cs);
}
void launch_plain_to_mixed(cudaStream_t s, const PlainParts &P, int64_t n0, int64_t n, const MixedParts &X) {
  if (n > 0) k_plain_to_mixed<<<grid_for(n), kThreads, 0, s>>>(P, n0, n, X);
}
void launch_mixed_to_plain(cudaStream_t s, const MixedParts &X, int64_t n, const DevMesh &M, const SpeciesTable &S,
                           const PlainParts &P) {
  if (n > 0) k_mixed_to_plain<<<grid_for(n), kThreads, 0, s>>>(X, n, M, S, P);
}
