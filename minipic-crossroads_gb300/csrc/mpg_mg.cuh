// mpg_mg.cuh -- device side of the multigrid-preconditioned mixed CG:
// the solver state (CgMgArgs) and the level passes of the V-cycle (stencil
// products, damped Jacobi sweeps, restriction, prolongation).  Used by the
// single-run cooperative solver (mg.cu), whose levels run on the whole grid,
// and by the batch engine (batch.cu), where one CTA runs a whole V-cycle.
// Every pass works on the rows [lo, hi) given to it; `sync` is the caller's
// barrier between dependent passes.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpg_device.cuh"
#include "mpg_kernels.h"

namespace mgpass {

struct CgMgArgs {
  DiaMatrix A;
  MgDev mg;
  const double *__restrict__ b;
  double *x, *r64;
  float *r[2], *s[2];  // fine-level PCG residual and A p, double-buffered by iteration parity
  float *u, *w, *p, *z;  // u = M r is the V-cycle's output (mg.lev[0].t), w = A u
  double *partials;      // outer phases: [2 sets][4][nb]; inner: one 32-byte record per block
  double tol2, inner_tol2, safety2;
  int max_iter;
  DevStats *st;
};

// (A_l x)_i on level l, x given by the loader xv(j): the solver's
// 15/27-diagonal operator on level 0, the Galerkin 27-point stencil on the
// coarser levels; Dirichlet rows are identity rows
template <int ND, bool CST, typename X>
__device__ __forceinline__ float level_apply(const CgMgArgs &a, int l, X xv, int64_t i) {
  const MgLevelDev &L = a.mg.lev[l];
  if (L.bnd[i]) return xv(i);
  float s = 0.f;
  if (l == 0) {
    const int64_t n = a.A.n, nwrap = a.A.nwrap;
#pragma unroll
    for (int d = 0; d < ND; ++d)
      s = __fmaf_rn(CST ? a.A.cst[d] : a.A.val32[d * n + i], xv(dia_nb(i, a.A.off[d], nwrap)), s);
  } else {
    const int64_t n = L.n;
    // x-plane offsets of the -1 / +1 neighbours (wrapping on a periodic level)
    int64_t xm = -(int64_t)L.si, xp = L.si;
    if (L.px) {
      const int64_t I = i / L.si;
      if (I == 0) xm += (int64_t)L.gx * L.si;
      if (I == L.gx - 1) xp -= (int64_t)L.gx * L.si;
    }
#pragma unroll
    for (int d = 0; d < 27; ++d) {
      const int64_t off = (d / 9 == 0 ? xm : d / 9 == 2 ? xp : 0) + ((d / 3) % 3 - 1) * (int64_t)L.sj + (d % 3 - 1);
      s = __fmaf_rn(L.val[d * n + i], xv(i + off), s);
    }
  }
  return s;
}

// row index -> (i, j, k) on a level (row counts stay below 2^32)
__device__ __forceinline__ void level_ijk(const MgLevelDev &L, int64_t r, unsigned &i, unsigned &j, unsigned &k) {
  const unsigned rr = (unsigned)r, sj = (unsigned)L.sj, si = (unsigned)L.si;
  i = rr / si;
  const unsigned rem = rr - i * si;
  j = rem / sj;
  k = rem - j * sj;
}

// restriction r_{l+1}[C] = sum_delta w(delta) t_l[2C + delta] over the 27 fine
// nodes around 2C (w = 1/2 per non-zero component); zero on Dirichlet rows.
// The host's Galerkin product leaves Dirichlet fine nodes out of P (on an odd
// cell count the far boundary node 2C + 1 is one of the 27); this sum reads
// them, which is the same because t is exactly zero on every Dirichlet row of
// every level: the right-hand side r is zero there (the PCG residual of the
// identity rows, and restrict_at's own zero on coarse Dirichlet rows), so
// t = r - A (omega D^-1 r) = 0 - 1 * 0 on those rows.
__device__ __forceinline__ float restrict_at(const MgLevelDev &F, const MgLevelDev &Cl, int64_t C) {
  if (Cl.bnd[C]) return 0.f;
  unsigned I, J, K;
  level_ijk(Cl, C, I, J, K);
  const int64_t f0 = 2 * (int64_t)J * F.sj + 2 * (int64_t)K;
  float s = 0.f;
#pragma unroll
  for (int di = -1; di <= 1; ++di)
#pragma unroll
    for (int dj = -1; dj <= 1; ++dj) {
      const float wij = (di ? 0.5f : 1.f) * (dj ? 0.5f : 1.f);
      int64_t fi = 2 * (int64_t)I + di;  // fine x-plane, wrapping on a periodic level
      if (F.px) fi = fi < 0 ? fi + F.gx : fi >= F.gx ? fi - F.gx : fi;
      const float *row = F.t + fi * F.si + f0 + dj * (int64_t)F.sj;
      s = __fmaf_rn(wij * 0.5f, row[-1], s);
      s = __fmaf_rn(wij, row[0], s);
      s = __fmaf_rn(wij * 0.5f, row[1], s);
    }
  return s;
}

// prolongation (P c)_i: trilinear interpolation of the coarse result c, as
// the mean of the 8 corners (fi >> 1, (fi + 1) >> 1) x ... (a corner repeats
// along a direction where the fine index is even)
__device__ __forceinline__ float prolong_at(const MgLevelDev &F, const MgLevelDev &Cl, const float *__restrict__ c,
                                            int64_t i) {
  unsigned fi, fj, fk;
  level_ijk(F, i, fi, fj, fk);
  unsigned ci1 = (fi + 1) >> 1;
  if (Cl.px && ci1 == (unsigned)Cl.gx) ci1 = 0;  // the last fine plane sits between the last and first coarse ones
  const int64_t i0 = (int64_t)(fi >> 1) * Cl.si, i1 = (int64_t)ci1 * Cl.si;
  const int64_t j0 = (int64_t)(fj >> 1) * Cl.sj, j1 = (int64_t)((fj + 1) >> 1) * Cl.sj;
  const int64_t k0 = fk >> 1, k1 = (fk + 1) >> 1;
  const float s = ((c[i0 + j0 + k0] + c[i0 + j0 + k1]) + (c[i0 + j1 + k0] + c[i0 + j1 + k1])) +
                  ((c[i1 + j0 + k0] + c[i1 + j0 + k1]) + (c[i1 + j1 + k0] + c[i1 + j1 + k1]));
  return 0.125f * s;
}

// pre-smoothing residual on rows [lo, hi) of level l: t = r - A e with
// e = omega D^-1 r (one Jacobi sweep from zero).  e is not stored: A e reads
// it through a loader (rv(j) gives r at row j), and the ascending steps
// recompute it.
// D^-1 of row j on level l: one constant on level 0 of a uniform mesh (its
// Dirichlet rows carry r = 0, so their own D^-1 = 1 never matters)
template <bool CST>
__device__ __forceinline__ float dinv_at(const CgMgArgs &a, int l, const float *__restrict__ dinv, int64_t j) {
  return (CST && l == 0) ? a.mg.dinv0 : dinv[j];
}

// Invariant relied on by restrict_at: on a Dirichlet (identity) row r = 0,
// hence out = 0 there.
template <int ND, bool CST, typename R>
__device__ __forceinline__ void presmooth_residual(const CgMgArgs &a, int l, int64_t lo, int64_t hi, R rv,
                                                   float *__restrict__ out) {
  const MgLevelDev &L = a.mg.lev[l];
  const float om = a.mg.omega;
  const float *__restrict__ dinv = L.dinv;
  auto e0 = [&](int64_t j) { return om * dinv_at<CST>(a, l, dinv, j) * rv(j); };
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) out[i] = rv(i) - level_apply<ND, CST>(a, l, e0, i);
}

// where level 0's first pre-smoothing residual goes: t (one sweep), or t2
// when level 0 smooths twice (the second sweep then writes t)
__device__ __forceinline__ float *first_residual(const CgMgArgs &a) {
  return a.mg.nu0 == 2 ? a.mg.lev[0].t2 : a.mg.lev[0].t;
}

// restriction of level l's t onto the coarse rows [clo, chi) of level l + 1;
// the coarsest level keeps only its interior rows, in order (the dense
// solve's right-hand side)
__device__ __forceinline__ void restrict_rows(const CgMgArgs &a, int l, int64_t clo, int64_t chi) {
  const MgLevelDev &L = a.mg.lev[l], &C = a.mg.lev[l + 1];
  if (l + 1 < a.mg.nlev - 1) {
    for (int64_t i = clo + threadIdx.x; i < chi; i += blockDim.x) C.r[i] = restrict_at(L, C, i);
    return;
  }
  const int x0 = C.px ? 0 : 1, ny = C.gy - 2, nz = C.gz - 2;
  for (int64_t i = clo + threadIdx.x; i < chi; i += blockDim.x) {
    if (C.bnd[i]) continue;
    unsigned I, J, K;
    level_ijk(C, i, I, J, K);
    a.mg.dense_r[((int64_t)(I - x0) * ny + (J - 1)) * nz + (K - 1)] = restrict_at(L, C, i);
  }
}

// one coarse level's descending steps on rows [lo, hi) (coarse rows
// [clo, chi)), `sync` between dependent steps
template <int ND, bool CST, typename Sync>
__device__ __forceinline__ bool level_down(const CgMgArgs &a, int l, int64_t lo, int64_t hi, int64_t clo, int64_t chi,
                                           Sync sync) {
  const float *__restrict__ r = a.mg.lev[l].r;
  presmooth_residual<ND, CST>(a, l, lo, hi, [&](int64_t j) { return r[j]; }, a.mg.lev[l].t);
  if (!sync()) return false;
  restrict_rows(a, l, clo, chi);
  return sync();
}

// ascending steps: e = omega D^-1 r + P c, then t = e + omega D^-1 (r - A e)
// (the level's result); r is the level's right-hand side
template <int ND, bool CST, typename Sync>
__device__ __forceinline__ bool level_up(const CgMgArgs &a, int l, int64_t lo, int64_t hi, const float *r,
                                         const float *c, Sync sync) {
  const MgLevelDev &L = a.mg.lev[l];
  const MgLevelDev &C = a.mg.lev[l + 1];
  const float om = a.mg.omega;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    float e = om * dinv_at<CST>(a, l, L.dinv, i) * r[i];
    if (!L.bnd[i]) e += prolong_at(L, C, c, i);
    L.e[i] = e;
  }
  if (!sync()) return false;
  const float *__restrict__ ev = L.e;
  auto ld = [&](int64_t j) { return ev[j]; };
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x)
    L.t[i] = ev[i] + om * dinv_at<CST>(a, l, L.dinv, i) * (r[i] - level_apply<ND, CST>(a, l, ld, i));
  return sync();
}

// level 0 with two Jacobi sweeps on each side (V(2,2) there): the
// pre-smoothed error was e2 = omega D^-1 (r + t1) with t1 = r - A omega D^-1 r
// (in t2); e3 = e2 + P c, then two post-smoothing sweeps; the result is t
template <int ND, bool CST, typename Sync>
__device__ __forceinline__ bool level_up_twice(const CgMgArgs &a, int l, int64_t lo, int64_t hi, const float *r,
                                               const float *c, Sync sync) {
  const MgLevelDev &L = a.mg.lev[l];
  const MgLevelDev &C = a.mg.lev[l + 1];
  const float om = a.mg.omega;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    float e = om * dinv_at<CST>(a, l, L.dinv, i) * (r[i] + L.t2[i]);
    if (!L.bnd[i]) e += prolong_at(L, C, c, i);
    L.e[i] = e;
  }
  if (!sync()) return false;
  {
    const float *__restrict__ ev = L.e;
    auto ld = [&](int64_t j) { return ev[j]; };
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x)
      L.t2[i] = ev[i] + om * dinv_at<CST>(a, l, L.dinv, i) * (r[i] - level_apply<ND, CST>(a, l, ld, i));
  }
  if (!sync()) return false;
  const float *__restrict__ ev = L.t2;
  auto ld = [&](int64_t j) { return ev[j]; };
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x)
    L.t[i] = ev[i] + om * dinv_at<CST>(a, l, L.dinv, i) * (r[i] - level_apply<ND, CST>(a, l, ld, i));
  return sync();
}

// a grid level l >= 1 with two pre-smoothing sweeps: t1 (in t2), then t
template <int ND, bool CST, typename Sync>
__device__ __forceinline__ bool level_down_twice(const CgMgArgs &a, int l, int64_t lo, int64_t hi, int64_t clo,
                                                 int64_t chi, Sync sync) {
  const MgLevelDev &L = a.mg.lev[l];
  const float *__restrict__ r = L.r;
  presmooth_residual<ND, CST>(a, l, lo, hi, [&](int64_t j) { return r[j]; }, L.t2);
  if (!sync()) return false;
  const float *__restrict__ t1 = L.t2;
  presmooth_residual<ND, CST>(a, l, lo, hi, [&](int64_t j) { return t1[j]; }, L.t);
  if (!sync()) return false;
  restrict_rows(a, l, clo, chi);
  return sync();
}

// coarsest level: t = A_c^-1 r over its interior rows (r compact in
// dense_r), one warp per row of the dense inverse, warp w0 of nw taking
// rows w0, w0 + nw, ... (lanes over the row, four chains, fixed shuffle
// tree); the Dirichlet rows of t stay zero
__device__ __forceinline__ void dense_solve_rows(const MgDev &mg, int w0, int nw) {
  const MgLevelDev &Lc = mg.lev[mg.nlev - 1];
  const int m = mg.dense_m, lane = threadIdx.x & 31;
  for (int q = w0; q < m; q += nw) {
    const float *__restrict__ row = mg.dense_inv + (int64_t)q * m;
    const float *__restrict__ rc = mg.dense_r;
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;  // four independent chains
    int k = lane;
    for (; k + 96 < m; k += 128) {
      s0 = __fmaf_rn(row[k], rc[k], s0);
      s1 = __fmaf_rn(row[k + 32], rc[k + 32], s1);
      s2 = __fmaf_rn(row[k + 64], rc[k + 64], s2);
      s3 = __fmaf_rn(row[k + 96], rc[k + 96], s3);
    }
    for (; k < m; k += 32) s0 = __fmaf_rn(row[k], rc[k], s0);
    float s = (s0 + s1) + (s2 + s3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) Lc.t[mg.dense_idx[q]] = s;
  }
}

}  // namespace mgpass
