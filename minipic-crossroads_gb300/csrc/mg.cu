// mg.cu -- mixed-precision CG preconditioned by a geometric multigrid V-cycle.
//
// One cooperative launch per field solve, like k_cg_mixed: FP64 outer
// refinement (r64 = b - A64 x, stop at |r64| <= tol |b|) around an FP32 inner
// solve of A z = r64 / |r64|.  The inner solve is preconditioned CG in the
// single-reduction form of Chronopoulos and Gear (one grid-wide all-reduce
// of four dots per iteration), with u = M r one multigrid V-cycle: damped
// Jacobi smoothing (two sweeps per side on the fine level, one on the
// others), restriction P^T, Galerkin coarse operators (mg_host.cpp) and a
// dense solve on the coarsest level.  Levels with many rows are processed by
// the whole grid (a grid barrier between dependent steps); small ones by
// block 0 alone (block barriers) while the other blocks wait at the next grid
// barrier; the dense solve by the whole grid.  The search direction survives
// the FP64 refinement sweeps (reliable updates).
// Not part of the reference, whose CG (CG_solve.hpp:54-114) is
// unpreconditioned; the converged phi meets the same FP64 tolerance.
#include <cuda_runtime.h>

#include "minipic_gb300.h"
#include "mpg_device.cuh"
#include "mpg_kernels.h"
#include "mpg_mg.cuh"

namespace {
using namespace mgpass;

// grid barrier of the cooperative solve (epoch-counted, bounded wait)
struct MgSync {
  DevStats *st;
  unsigned epoch = 0;
  __device__ bool operator()() { return grid_barrier(st, gridDim.x, epoch); }
  __device__ void iteration() {}
};

constexpr int kRecMg = 5;  // block records each of the first 128 threads gathers (grids up to 640 blocks)


// row range of this block on a level processed by the whole grid
__device__ __forceinline__ void grid_rows(int64_t n, int64_t &lo, int64_t &hi) {
  lo = n * blockIdx.x / gridDim.x;
  hi = n * (blockIdx.x + 1) / gridDim.x;
}

// coarsest level: the dense solve across the whole grid
__device__ __forceinline__ void dense_solve(const MgDev &mg) {
  dense_solve_rows(mg, blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), (blockDim.x >> 5) * gridDim.x);
}

// rest of u = M r after level 0's first pre-smoothing residual has been
// written on this block's rows (first_residual); rf is level 0's right-hand
// side r and the result u is lev[0].t.  Levels [0, ngrid) run on the whole grid, levels
// [ngrid, nlev - 1) on block 0 alone, the dense coarsest solve on the whole
// grid again.
template <int ND, bool CST>
__device__ bool vcycle_rest(const CgMgArgs &a, const float *rf, MgSync &bar) {
  const int nl = a.mg.nlev, ng = a.mg.ngrid;
  auto gsync = [&]() { return bar(); };
  auto bsync = [&]() {
    __syncthreads();
    return true;
  };
  int64_t clo, chi;
  if (!gsync()) return false;
  if (a.mg.nu0 == 2) {
    // second pre-smoothing sweep on level 0: t = t1 - A omega D^-1 t1
    int64_t lo, hi;
    grid_rows(a.mg.lev[0].n, lo, hi);
    const float *__restrict__ t1 = a.mg.lev[0].t2;
    presmooth_residual<ND, CST>(a, 0, lo, hi, [&](int64_t j) { return t1[j]; }, a.mg.lev[0].t);
    if (!gsync()) return false;
  }
  grid_rows(a.mg.lev[1].n, clo, chi);
  restrict_rows(a, 0, clo, chi);
  if (!gsync()) return false;
  for (int l = 1; l < ng; ++l) {
    int64_t lo, hi;
    grid_rows(a.mg.lev[l].n, lo, hi);
    grid_rows(a.mg.lev[l + 1].n, clo, chi);
    if (a.mg.nu1 == 2) {
      if (!level_down_twice<ND, CST>(a, l, lo, hi, clo, chi, gsync)) return false;
    } else if (!level_down<ND, CST>(a, l, lo, hi, clo, chi, gsync)) {
      return false;
    }
  }
  const bool blk = ng < nl - 1;
  if (blk) {
    if (blockIdx.x == 0)
      for (int l = ng; l < nl - 1; ++l) level_down<ND, CST>(a, l, 0, a.mg.lev[l].n, 0, a.mg.lev[l + 1].n, bsync);
    if (!gsync()) return false;
  }
  dense_solve(a.mg);
  if (!gsync()) return false;
  if (blk) {
    if (blockIdx.x == 0)
      for (int l = nl - 2; l >= ng; --l)
        level_up<ND, CST>(a, l, 0, a.mg.lev[l].n, a.mg.lev[l].r, a.mg.lev[l + 1].t, bsync);
    if (!gsync()) return false;
  }
  for (int l = ng - 1; l >= 0; --l) {
    int64_t lo, hi;
    grid_rows(a.mg.lev[l].n, lo, hi);
    if (l > 0 && a.mg.nu1 == 2) {
      if (!level_up_twice<ND, CST>(a, l, lo, hi, a.mg.lev[l].r, a.mg.lev[l + 1].t, gsync)) return false;
    } else if (l == 0 && a.mg.nu0 == 2) {
      if (!level_up_twice<ND, CST>(a, 0, lo, hi, rf, a.mg.lev[1].t, gsync)) return false;
    } else if (!level_up<ND, CST>(a, l, lo, hi, l == 0 ? rf : a.mg.lev[l].r, a.mg.lev[l + 1].t, gsync)) {
      return false;
    }
  }
  return true;
}

template <int ND, int TH, bool CST>
__global__ void __launch_bounds__(TH, 1024 / TH) k_cg_mg(CgMgArgs a) {
  __shared__ double red[32];
  __shared__ float smw[4 * 32];
  __shared__ ff smf[4 * 32];
  __shared__ ff smt[4];
  __shared__ double bcast;
  MgSync bar;
  bar.st = a.st;
  const int nb = gridDim.x, bid = blockIdx.x;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t n = a.A.n;
  const int64_t lo = n * bid / nb, hi = n * (bid + 1) / nb;
  const uint8_t *__restrict__ bnd = a.A.bnd;
  const double *__restrict__ v64 = a.A.val64;
  auto slot64 = [&](int set, int k) { return a.partials + ((size_t)(set * 4 + k)) * nb; };
  // all-reduce of four float-float values per block (block record of two
  // float4, grid barrier, four warps gather every record in block order)
  auto allreduce4 = [&](int set, const ff (&v)[4], ff (&out)[4]) -> bool {
    float w4[4] = {v[0].hi + v[0].lo, v[1].hi + v[1].lo, v[2].hi + v[2].lo, v[3].hi + v[3].lo};
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int k = 0; k < 4; ++k) w4[k] += __shfl_down_sync(0xffffffffu, w4[k], o);
    if (lane == 0)
#pragma unroll
      for (int k = 0; k < 4; ++k) smw[k * 32 + wid] = w4[k];
    __syncthreads();
    if (wid == 0) {
      ff t[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        t[k] = ff{lane < TH / 32 ? smw[k * 32 + lane] : 0.f, 0.f};
        for (int o = 16; o > 0; o >>= 1) t[k] = ff_add(t[k], ff_shfl_down(t[k], o));
      }
      if (lane == 0) {
        float4 *rec = reinterpret_cast<float4 *>(slot64(set, 0)) + 2 * bid;
        rec[0] = make_float4(t[0].hi, t[0].lo, t[1].hi, t[1].lo);
        rec[1] = make_float4(t[2].hi, t[2].lo, t[3].hi, t[3].lo);
      }
    }
    if (!bar()) return false;
    if (wid < 4) {
      const float4 *rec = reinterpret_cast<const float4 *>(slot64(set, 0));
      float4 x[kRecMg], y[kRecMg];
#pragma unroll
      for (int j = 0; j < kRecMg; ++j) {
        const int i = threadIdx.x + 128 * j;
        x[j] = i < nb ? rec[2 * i] : make_float4(0.f, 0.f, 0.f, 0.f);
        y[j] = i < nb ? rec[2 * i + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
      }
      ff t[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
      for (int j = 0; j < kRecMg; ++j) {
        t[0] = ff_add(t[0], ff{x[j].x, x[j].y});
        t[1] = ff_add(t[1], ff{x[j].z, x[j].w});
        t[2] = ff_add(t[2], ff{y[j].x, y[j].y});
        t[3] = ff_add(t[3], ff{y[j].z, y[j].w});
      }
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        for (int o = 16; o > 0; o >>= 1) t[k] = ff_add(t[k], ff_shfl_down(t[k], o));
        if (lane == 0) smf[k * 32 + wid] = t[k];
      }
    }
    __syncthreads();
    if (wid == 0) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        ff u = lane < 4 ? smf[k * 32 + lane] : ff{0.f, 0.f};
        for (int o = 2; o > 0; o >>= 1) u = ff_add(u, ff_shfl_down(u, o));
        if (lane == 0) smt[k] = u;
      }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = smt[k];
    __syncthreads();
    return true;
  };
  double bb = 0.0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) bb = __fma_rn(a.b[i], a.b[i], bb);
  double t = block_sum(bb, red);
  if (threadIdx.x == 0) slot64(1, 3)[bid] = t;  // read after the first barrier
  int total_inner = 0, status = 0, sweeps = 0, phase = 0;
  double rho64 = 0.0, rho0 = 0.0, rho_prev64 = 0.0;
  // PCG state kept across refinement sweeps when reliable updates are on:
  // the search direction p (and s = A p) continues, rescaled to the new
  // right-hand side, instead of restarting from z = 0, p = 0
  ff gam_prev = {0.f, 0.f};
  int cur = 0;
  bool have_dir = false;
  for (;; ++sweeps) {
    // ---- FP64 residual with the FP64 matrix (identity rows: x = b there)
    double rr = 0.0;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      double s = 0.0;
      if (bnd[i]) {
        a.x[i] = a.b[i];
        s = a.x[i];
      } else {
#pragma unroll
        for (int d = 0; d < ND; ++d) s = __fma_rn(v64[d * n + i], a.x[dia_nb(i, a.A.off[d], a.A.nwrap)], s);
      }
      const double ri = a.b[i] - s;
      a.r64[i] = ri;
      rr = __fma_rn(ri, ri, rr);
    }
    int set = phase & 1;
    t = block_sum(rr, red);
    if (threadIdx.x == 0) slot64(set, 0)[bid] = t;
    if (!bar()) return;
    if (sweeps == 0) rho0 = grid_total(slot64(1, 3), nb, &bcast);
    rho64 = grid_total(slot64(set, 0), nb, &bcast);
    ++phase;
    if (rho0 == 0.0) {
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) a.x[i] = 0.0;
      rho64 = 0.0;
      break;
    }
    if (rho64 <= a.tol2 * rho0) break;
    if (total_inner >= a.max_iter) {
      status = 1;
      break;
    }
    // ---- inner PCG on A z = r64 / |r64| (FP32), z = 0
    const double scale = 1.0 / sqrt(rho64);
    const bool carry = have_dir && a.mg.reliable;
    // the old system's vectors in the new scale: r_new = r64_new / |r64_new|
    // is the old recursive residual times f = |r64_old| / |r64_new|
    const float f = carry ? (float)sqrt(rho_prev64 / rho64) : 0.f;
    if (carry) {
      gam_prev = ff_mulf(ff_mulf(gam_prev, f), f);
    } else {
      have_dir = false;
      cur = 0;
    }
    {
      float *__restrict__ rc = a.r[cur];
      float *__restrict__ sc = a.s[cur];
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        rc[i] = (float)(a.r64[i] * scale);
        a.z[i] = 0.f;
        a.p[i] = carry ? a.p[i] * f : 0.f;
        sc[i] = carry ? sc[i] * f : 0.f;
      }
    }
    if (!bar()) return;
    {
      const float *__restrict__ r0 = a.r[cur];
      presmooth_residual<ND, CST>(a, 0, lo, hi, [&](int64_t j) { return r0[j]; }, first_residual(a));
    }
    ff gam0 = {0.f, 0.f};
    const float stop_rel = (float)fmax(a.inner_tol2, a.safety2 * a.tol2 * rho0 / rho64);
    for (int k = 0;; ++k) {
      bar.iteration();
      if (!vcycle_rest<ND, CST>(a, a.r[cur], bar)) return;  // u = M r, visible everywhere
      const float *__restrict__ rc = a.r[cur];
      const float *__restrict__ sc = a.s[cur];
      // (r, u), (w, u), (u, s) and (p, s) with w = A u: the last two give the
      // exact (p_new, A p_new) = (w, u) + 2 beta (u, s) + beta^2 (p, s), which
      // stays valid when the residual was replaced by the true one
      ff v[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const float ui = a.u[i];
        const float wi = level_apply<ND, CST>(a, 0, [&](int64_t j) { return a.u[j]; }, i);
        const float si = sc[i];
        a.w[i] = wi;
        v[0] = ff_add(v[0], ff_prod(rc[i], ui));
        v[1] = ff_add(v[1], ff_prod(wi, ui));
        v[2] = ff_add(v[2], ff_prod(ui, si));
        v[3] = ff_add(v[3], ff_prod(a.p[i], si));
      }
      set = phase & 1;
      ff tot[4];
      if (!allreduce4(set, v, tot)) return;
      ++phase;
      const ff G = tot[0];
      if (k == 0) gam0 = G;
      if (!(G.hi > 0.f) || G.hi <= stop_rel * gam0.hi || total_inner >= a.max_iter) break;
      const float beta = have_dir ? G.hi / gam_prev.hi : 0.f;
      const ff den = ff_add(ff_add(tot[1], ff_mulf(tot[2], 2.f * beta)), ff_mulf(ff_mulf(tot[3], beta), beta));
      const float alpha = G.hi / den.hi;
      // update into the other buffers, fused (levels up to fuse_update rows)
      // with the next V-cycle's first step: that step reads the new residual
      // at neighbour rows, which it recomputes from the old buffers bit for
      // bit as their owners write it
      const int nx = cur ^ 1;
      const float *__restrict__ ro = a.r[cur];
      const float *__restrict__ so = a.s[cur];
      const float *__restrict__ wv = a.w;
      float *__restrict__ rn = a.r[nx];
      float *__restrict__ sn = a.s[nx];
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const float pi = __fmaf_rn(beta, a.p[i], a.u[i]);
        const float si = __fmaf_rn(beta, so[i], wv[i]);
        a.p[i] = pi;
        sn[i] = si;
        a.z[i] = __fmaf_rn(alpha, pi, a.z[i]);
        rn[i] = __fmaf_rn(-alpha, si, ro[i]);
      }
      if (a.mg.fuse_update) {
        presmooth_residual<ND, CST>(
            a, 0, lo, hi, [&](int64_t j) { return __fmaf_rn(-alpha, __fmaf_rn(beta, so[j], wv[j]), ro[j]); },
            first_residual(a));
      } else {
        // large levels: one barrier more, but the pre-smoothing then reads
        // one vector per neighbour instead of three
        if (!bar()) return;
        presmooth_residual<ND, CST>(a, 0, lo, hi, [&](int64_t j) { return rn[j]; }, first_residual(a));
      }
      cur = nx;
      gam_prev = G;
      have_dir = true;
      ++total_inner;
    }
    rho_prev64 = rho64;
    // ---- x += |r64| z  (FP64)
    const double back = sqrt(rho64);
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) a.x[i] = __fma_rn((double)a.z[i], back, a.x[i]);
    if (!bar()) return;
  }
  if (bid == 0 && threadIdx.x == 0) {
    a.st->solver_iters = total_inner;
    a.st->solver_status = status;
    a.st->iters_total += total_inner;
    if (status) a.st->solver_fail = 1;
    a.st->solver_resid = rho0 > 0.0 ? sqrt(rho64 / rho0) : 0.0;
  }
}

void *mg_kernel_of(int nd, bool cst, int th) {
  static void *tab[2][2][3] = {
      {{(void *)k_cg_mg<15, 256, false>, (void *)k_cg_mg<15, 512, false>, (void *)k_cg_mg<15, 1024, false>},
       {(void *)k_cg_mg<15, 256, true>, (void *)k_cg_mg<15, 512, true>, (void *)k_cg_mg<15, 1024, true>}},
      {{(void *)k_cg_mg<27, 256, false>, (void *)k_cg_mg<27, 512, false>, (void *)k_cg_mg<27, 1024, false>},
       {(void *)k_cg_mg<27, 256, true>, (void *)k_cg_mg<27, 512, true>, (void *)k_cg_mg<27, 1024, true>}}};
  return tab[nd > 15 ? 1 : 0][cst ? 1 : 0][th <= 256 ? 0 : th <= 512 ? 1 : 2];
}

}  // namespace

int mg_max_blocks(int device, int threads) {
  int sms = 0, occ = 1 << 30, o = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  for (int nd : {15, 27})
    for (int cst = 0; cst < 2; ++cst) {
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, mg_kernel_of(nd, cst != 0, threads), threads, 0);
      occ = o < occ ? o : occ;
    }
  int nbmax = sms * occ;
  return nbmax < 128 * kRecMg ? nbmax : 128 * kRecMg;
}

int run_cg_mg(cudaStream_t s, const DiaMatrix &A, const MgDev &mg, const double *b, double *x, double tol,
              double inner_tol, int max_iter, CgWork &w, int max_blocks, DevStats *st) {
  CgMgArgs a;
  a.A = A;
  a.mg = mg;
  a.b = b;
  a.x = x;
  a.r64 = w.r;
  // fine-level PCG vectors over the first 10n floats of the work buffer (12n)
  float *f = reinterpret_cast<float *>(w.v4);
  const int64_t n = A.n;
  a.w = f + 0 * n;
  a.p = f + 1 * n;
  a.z = f + 2 * n;
  a.r[0] = f + 3 * n;
  a.r[1] = f + 4 * n;
  a.s[0] = f + 5 * n;
  a.s[1] = f + 6 * n;
  a.mg.lev[0].r = nullptr;  // level 0's right-hand side is r[cur]
  a.mg.lev[0].e = f + 7 * n;
  a.mg.lev[0].t = f + 8 * n;
  a.mg.lev[0].t2 = f + 9 * n;
  a.u = a.mg.lev[0].t;
  if (!mg.fuse_update) {
    // without the fused update no pass reads a neighbour's old residual while
    // the new one is written, so r and s are updated in place: two fine-level
    // vectors fewer in the working set (L2)
    a.r[1] = a.r[0];
    a.s[1] = a.s[0];
  }
  a.partials = w.partials;
  a.tol2 = tol * tol;
  a.inner_tol2 = inner_tol * inner_tol;
  a.safety2 = w.inner_safety * w.inner_safety;
  a.max_iter = max_iter;
  a.st = st;
  const int th = w.threads == 256 || w.threads == 1024 ? w.threads : 512;
  int64_t want = (n + th - 1) / th;
  if (want < 1) want = 1;
  int cap = max_blocks;
  if (w.block_cap > 0 && w.block_cap < cap) cap = w.block_cap;
  const int nb = (int)(want < cap ? want : cap);
  CgWork wb = w;
  wb.bar_mode = 0;  // the multigrid solver uses the fence + volatile-polling barrier
  if (barrier_setup(s, st, wb)) return MPG_ERR_CUDA;
  void *args[] = {&a};
  cudaError_t e = cudaLaunchCooperativeKernel(mg_kernel_of(A.ndiag, A.constant != 0, th), dim3(nb), dim3(th), args, 0, s);
  return e == cudaSuccess ? MPG_OK : MPG_ERR_CUDA;
}
