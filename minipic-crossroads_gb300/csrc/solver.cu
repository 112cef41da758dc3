// solver.cu -- Krylov solvers of the field solve (ES::solve, ES.cpp:216-231).
//
// The reference runs BiCGStab/CG on the host through Tpetra with a
// device->host->device copy of rhs/phi every step (ES.cpp:217-222).  Here the
// matrix and the vectors stay in HBM and the whole solve is one cooperative
// (persistent) launch: the grid walks all iterations, with a bounded grid
// barrier between the phases that need a global reduction.
//
// CG needs two barriers per iteration: the search direction
// p_k = beta p_{k-1} + r is formed on the fly inside the SpMV (double-buffered
// p, so no block reads a value another block is overwriting), which folds the
// p-update into the SpMV pass.  Dot products are reduced deterministically:
// every block writes one partial, and after the barrier every block sums the
// partials in block order, so all blocks agree bit for bit on alpha/beta and
// on the stopping test.
//
// Mixed form: FP32 CSR SpMV and FP32 vectors inside FP64 iterative refinement;
// FP64 is kept for dot products, the residual recomputation r = b - A x with
// the FP64 matrix, and the update of phi.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cmath>

#include "minipic_gb300.h"
#include "mpg_kernels.h"

namespace {

constexpr int kCgThreads = 512;

struct Cg64Args {
  int64_t n;
  const int32_t *__restrict__ rowptr;
  const int32_t *__restrict__ col;
  const double *__restrict__ val;
  const double *__restrict__ b;
  double *x;
  double *r;
  double *p0;
  double *p1;
  double *q;
  double *partials;  // [4][nb]
  double tol2;
  int max_iter;
  DevStats *st;
};

// sum of partials[0..nb): every thread loads at most one partial (one L2
// round trip), then a fixed block reduction; all blocks compute the same
// value bit for bit.  nb <= blockDim.x * 4 is required (checked at launch).
__device__ __forceinline__ double grid_total(const double *partials, int nb, double *sh) {
  double s = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s += partials[i];
  __shared__ double red2[32];
  s = block_sum(s, red2);
  if (threadIdx.x == 0) *sh = s;
  __syncthreads();
  const double v = *sh;
  __syncthreads();
  return v;
}

__global__ void __launch_bounds__(kCgThreads) k_cg64(Cg64Args a) {
  __shared__ double red[32];
  __shared__ double bcast;
  const int nb = gridDim.x, bid = blockIdx.x;
  const int64_t lo = a.n * bid / nb, hi = a.n * (bid + 1) / nb;
  double *P0 = a.partials, *P1 = a.partials + nb, *P2 = a.partials + 2 * nb;
  // r = b - A x (CG_solve.hpp:62-63); rho0 = b.b, rho = r.r
  double rr = 0.0, bb = 0.0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    double s = 0.0;
    for (int32_t k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k) s += a.val[k] * a.x[a.col[k]];
    const double ri = -1.0 * s + 1.0 * a.b[i];
    a.r[i] = ri;
    rr += ri * ri;
    bb += a.b[i] * a.b[i];
  }
  double t = block_sum(rr, red);
  if (threadIdx.x == 0) P0[bid] = t;
  t = block_sum(bb, red);
  if (threadIdx.x == 0) P1[bid] = t;
  if (!grid_barrier(a.st, nb)) return;
  const double rho0 = grid_total(P1, nb, &bcast);
  double rho = grid_total(P0, nb, &bcast), rho_old = 0.0;
  int iter = 0, status = 0;
  if (rho0 == 0.0 || rho == 0.0) {
    if (rho0 == 0.0)
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) a.x[i] = 0.0;
  } else {
    for (;; ++iter) {
      if (iter >= a.max_iter) {
        status = 1;
        break;
      }
      const double beta = iter == 0 ? 0.0 : rho / rho_old;
      double *pk = (iter & 1) ? a.p1 : a.p0;
      const double *pp = (iter & 1) ? a.p0 : a.p1;
      // p_k = beta*p_{k-1} + 1.0*r (CG_solve.hpp:77-82), q = A p_k (:85), p.q (:87)
      double pq = 0.0;
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        double s = 0.0;
        if (iter == 0) {
          for (int32_t k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k) s += a.val[k] * a.r[a.col[k]];
          pk[i] = a.r[i];
        } else {
          for (int32_t k = a.rowptr[i]; k < a.rowptr[i + 1]; ++k) {
            const int32_t j = a.col[k];
            s += a.val[k] * (beta * pp[j] + 1.0 * a.r[j]);
          }
          pk[i] = beta * pp[i] + 1.0 * a.r[i];
        }
        a.q[i] = s;
        pq += pk[i] * s;
      }
      t = block_sum(pq, red);
      if (threadIdx.x == 0) P2[bid] = t;
      if (!grid_barrier(a.st, nb)) return;
      const double alpha = rho / grid_total(P2, nb, &bcast);
      // x += alpha p (:92), r -= alpha q (:96), rho = r.r (:100)
      rr = 0.0;
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        a.x[i] = 1.0 * a.x[i] + alpha * pk[i];
        const double ri = 1.0 * a.r[i] + -alpha * a.q[i];
        a.r[i] = ri;
        rr += ri * ri;
      }
      t = block_sum(rr, red);
      if (threadIdx.x == 0) P0[bid] = t;
      if (!grid_barrier(a.st, nb)) return;
      rho_old = rho;
      rho = grid_total(P0, nb, &bcast);
      if (rho / rho0 < a.tol2) {
        ++iter;
        break;
      }
    }
  }
  if (bid == 0 && threadIdx.x == 0) {
    a.st->solver_iters = iter;
    a.st->solver_status = status;
    a.st->iters_total += iter;
    if (status) a.st->solver_fail = 1;
    a.st->solver_resid = rho0 > 0.0 ? sqrt(rho / rho0) : 0.0;
  }
}

// ---------------------------------------------------------------------------
// DIA kernels.  ND is the compile-time upper bound of the diagonal count
// (15 for the Kuhn split, 27 in general); nd is the actual count.
struct Cg64DiaArgs {
  DiaMatrix A;
  const double *__restrict__ b;
  double *x;
  double *r;
  double *p0;
  double *p1;
  double *q;
  double *partials;
  double tol2;
  int max_iter;
  DevStats *st;
};

template <int ND>
__global__ void __launch_bounds__(kCgThreads) k_cg64_dia(Cg64DiaArgs a) {
  __shared__ double red[32];
  __shared__ double bcast;
  const int nb = gridDim.x, bid = blockIdx.x;
  const int64_t n = a.A.n;
  const int nd = a.A.ndiag;
  const int64_t lo = n * bid / nb, hi = n * (bid + 1) / nb;
  double *P0 = a.partials, *P1 = a.partials + nb, *P2 = a.partials + 2 * nb;
  const double *__restrict__ val = a.A.val64;
  const uint8_t *__restrict__ bnd = a.A.bnd;
  // r = b - A x (CG_solve.hpp:62-63)
  double rr = 0.0, bb = 0.0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    double s = 0.0;
    if (bnd[i]) {
      s += 1.0 * a.x[i];
    } else {
#pragma unroll
      for (int d = 0; d < ND; ++d) {
        if (d >= nd) break;
        s += val[d * n + i] * a.x[i + a.A.off[d]];
      }
    }
    const double ri = -1.0 * s + 1.0 * a.b[i];
    a.r[i] = ri;
    rr += ri * ri;
    bb += a.b[i] * a.b[i];
  }
  double t = block_sum(rr, red);
  if (threadIdx.x == 0) P0[bid] = t;
  t = block_sum(bb, red);
  if (threadIdx.x == 0) P1[bid] = t;
  if (!grid_barrier(a.st, nb)) return;
  const double rho0 = grid_total(P1, nb, &bcast);
  double rho = grid_total(P0, nb, &bcast), rho_old = 0.0;
  int iter = 0, status = 0;
  if (rho0 == 0.0 || rho == 0.0) {
    if (rho0 == 0.0)
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) a.x[i] = 0.0;
  } else {
    for (;; ++iter) {
      if (iter >= a.max_iter) {
        status = 1;
        break;
      }
      const double beta = iter == 0 ? 0.0 : rho / rho_old;
      double *pk = (iter & 1) ? a.p1 : a.p0;
      const double *pp = (iter & 1) ? a.p0 : a.p1;
      const bool first = iter == 0;
      double pq = 0.0;
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const double pki = first ? a.r[i] : beta * pp[i] + 1.0 * a.r[i];
        double s = 0.0;
        if (bnd[i]) {
          s += 1.0 * pki;
        } else {
#pragma unroll
          for (int d = 0; d < ND; ++d) {
            if (d >= nd) break;
            const int64_t j = i + a.A.off[d];
            const double pj = first ? a.r[j] : beta * pp[j] + 1.0 * a.r[j];
            s += val[d * n + i] * pj;
          }
        }
        pk[i] = pki;
        a.q[i] = s;
        pq += pki * s;
      }
      t = block_sum(pq, red);
      if (threadIdx.x == 0) P2[bid] = t;
      if (!grid_barrier(a.st, nb)) return;
      const double alpha = rho / grid_total(P2, nb, &bcast);
      rr = 0.0;
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        a.x[i] = 1.0 * a.x[i] + alpha * pk[i];
        const double ri = 1.0 * a.r[i] + -alpha * a.q[i];
        a.r[i] = ri;
        rr += ri * ri;
      }
      t = block_sum(rr, red);
      if (threadIdx.x == 0) P0[bid] = t;
      if (!grid_barrier(a.st, nb)) return;
      rho_old = rho;
      rho = grid_total(P0, nb, &bcast);
      if (rho / rho0 < a.tol2) {
        ++iter;
        break;
      }
    }
  }
  if (bid == 0 && threadIdx.x == 0) {
    a.st->solver_iters = iter;
    a.st->solver_status = status;
    a.st->iters_total += iter;
    if (status) a.st->solver_fail = 1;
    a.st->solver_resid = rho0 > 0.0 ? sqrt(rho / rho0) : 0.0;
  }
}

struct CgMixedArgs {
  DiaMatrix A;
  const double *__restrict__ b;
  double *x;
  double *r64;
  float *r;
  float *z;
  float *q;
  float *pa;
  float *pb;
  double *partials;
  double tol2;
  double inner_tol2;
  int max_iter;
  DevStats *st;
};

template <int ND>
__global__ void __launch_bounds__(kCgThreads) k_cg_mixed(CgMixedArgs a) {
  __shared__ double red[32];
  __shared__ double bcast;
  const int nb = gridDim.x, bid = blockIdx.x;
  const int64_t n = a.A.n;
  const int nd = a.A.ndiag;
  const int64_t lo = n * bid / nb, hi = n * (bid + 1) / nb;
  const uint8_t *__restrict__ bnd = a.A.bnd;
  const double *__restrict__ v64 = a.A.val64;
  const float *__restrict__ v32 = a.A.val32;
  // partial slots: a slot written in phase k is read after barrier k and may
  // only be rewritten in phase k+2 or later
  double *P0 = a.partials, *P1 = a.partials + nb, *P2 = a.partials + 2 * nb, *P3 = a.partials + 3 * nb;
  double bb = 0.0;
  for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) bb += a.b[i] * a.b[i];
  double t = block_sum(bb, red);
  if (threadIdx.x == 0) P1[bid] = t;
  int total_inner = 0, status = 0, sweeps = 0;
  double rho64 = 0.0, rho0 = 0.0;
  for (;; ++sweeps) {
    // FP64 residual with the FP64 matrix
    double rr = 0.0;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      double s = 0.0;
      if (bnd[i]) {
        s = a.x[i];
      } else {
#pragma unroll
        for (int d = 0; d < ND; ++d) {
          if (d >= nd) break;
          s += v64[d * n + i] * a.x[i + a.A.off[d]];
        }
      }
      const double ri = a.b[i] - s;
      a.r64[i] = ri;
      rr += ri * ri;
    }
    t = block_sum(rr, red);
    if (threadIdx.x == 0) P0[bid] = t;
    if (!grid_barrier(a.st, nb)) return;
    if (sweeps == 0) rho0 = grid_total(P1, nb, &bcast);
    rho64 = grid_total(P0, nb, &bcast);
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
    // inner FP32 CG on A z = r / |r|, from z = 0
    const double scale = 1.0 / sqrt(rho64);
    double rs = 0.0;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const float ri = (float)(a.r64[i] * scale);
      a.r[i] = ri;
      a.z[i] = 0.f;
      rs += (double)ri * (double)ri;
    }
    t = block_sum(rs, red);
    if (threadIdx.x == 0) P3[bid] = t;
    if (!grid_barrier(a.st, nb)) return;
    const double rin0 = grid_total(P3, nb, &bcast);
    double rho = rin0, rho_old = 0.0;
    for (int k = 0;; ++k) {
      const float beta = k == 0 ? 0.f : (float)(rho / rho_old);
      float *pk = (k & 1) ? a.pb : a.pa;
      const float *pp = (k & 1) ? a.pa : a.pb;
      const bool first = k == 0;
      double pq = 0.0;
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const float pki = first ? a.r[i] : __fmaf_rn(beta, pp[i], a.r[i]);
        float s = 0.f;
        if (bnd[i]) {
          s = pki;
        } else {
#pragma unroll
          for (int d = 0; d < ND; ++d) {
            if (d >= nd) break;
            const int64_t j = i + a.A.off[d];
            const float pj = first ? a.r[j] : __fmaf_rn(beta, pp[j], a.r[j]);
            s = __fmaf_rn(v32[d * n + i], pj, s);
          }
        }
        pk[i] = pki;
        a.q[i] = s;
        pq += (double)pki * (double)s;
      }
      t = block_sum(pq, red);
      if (threadIdx.x == 0) P2[bid] = t;
      if (!grid_barrier(a.st, nb)) return;
      const float alpha = (float)(rho / grid_total(P2, nb, &bcast));
      double rr2 = 0.0;
      for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        a.z[i] = __fmaf_rn(alpha, pk[i], a.z[i]);
        const float ri = __fmaf_rn(-alpha, a.q[i], a.r[i]);
        a.r[i] = ri;
        rr2 += (double)ri * (double)ri;
      }
      t = block_sum(rr2, red);
      if (threadIdx.x == 0) P0[bid] = t;
      if (!grid_barrier(a.st, nb)) return;
      rho_old = rho;
      rho = grid_total(P0, nb, &bcast);
      ++total_inner;
      if (rho <= a.inner_tol2 * rin0 || total_inner >= a.max_iter) break;
    }
    // x += z * |r|  (FP64)
    const double back = sqrt(rho64);
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) a.x[i] += (double)a.z[i] * back;
    if (!grid_barrier(a.st, nb)) return;
  }
  if (bid == 0 && threadIdx.x == 0) {
    a.st->solver_iters = total_inner;
    a.st->solver_status = status;
    a.st->iters_total += total_inner;
    if (status) a.st->solver_fail = 1;
    a.st->solver_resid = rho0 > 0.0 ? sqrt(rho64 / rho0) : 0.0;
  }
}

// ---- BiCGStab building blocks (host-driven loop) -------------------------
__global__ void k_spmv64(int64_t n, const int32_t *__restrict__ rp, const int32_t *__restrict__ col,
                         const double *__restrict__ val, const double *__restrict__ x, double *__restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int32_t k = rp[i]; k < rp[i + 1]; ++k) s += val[k] * x[col[k]];
  y[i] = s;
}
// y = alpha*x + beta*y  (Tpetra update(alpha, x, beta))
__global__ void k_update(int64_t n, double alpha, const double *__restrict__ x, double beta, double *__restrict__ y) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  y[i] = beta * y[i] + alpha * x[i];
}
__global__ void k_dot_partial(int64_t n, const double *__restrict__ a, const double *__restrict__ b,
                              double *__restrict__ part) {
  __shared__ double red[32];
  double s = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += a[i] * b[i];
  s = block_sum(s, red);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}
__global__ void k_dot_final(const double *__restrict__ part, int nb, double *out) {
  __shared__ double red[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) s += part[i];
  s = block_sum(s, red);
  if (threadIdx.x == 0) *out = s;
}

}  // namespace

int cg_max_blocks(int device) {
  int sms = 0, occ = 1 << 30, o = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_cg64, kCgThreads, 0);
  occ = o < occ ? o : occ;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_cg64_dia<15>, kCgThreads, 0);
  occ = o < occ ? o : occ;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_cg64_dia<27>, kCgThreads, 0);
  occ = o < occ ? o : occ;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_cg_mixed<15>, kCgThreads, 0);
  occ = o < occ ? o : occ;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_cg_mixed<27>, kCgThreads, 0);
  occ = o < occ ? o : occ;
  if (occ < 1) occ = 1;
  return sms * occ;
}

// one row per thread until every co-resident block is busy
static int grid_for_rows(int64_t n, int max_blocks) {
  int64_t want = (n + kCgThreads - 1) / kCgThreads;
  if (want < 1) want = 1;
  if (want > max_blocks) want = max_blocks;
  return (int)want;
}

int run_cg64(cudaStream_t s, int device, int64_t n, const int32_t *rowptr, const int32_t *col, const double *val,
             const double *b, double *x, double tol, int max_iter, CgWork &w, DevStats *st) {
  Cg64Args a;
  a.n = n;
  a.rowptr = rowptr;
  a.col = col;
  a.val = val;
  a.b = b;
  a.x = x;
  a.r = w.r;
  a.p0 = w.p0;
  a.p1 = w.p1;
  a.q = w.q;
  a.partials = w.partials;
  a.tol2 = tol * tol;
  a.max_iter = max_iter;
  a.st = st;
  (void)device;
  const int nb = grid_for_rows(n, w.max_blocks);
  void *args[] = {&a};
  cudaError_t e = cudaLaunchCooperativeKernel((void *)k_cg64, dim3(nb), dim3(kCgThreads), args, 0, s);
  return e == cudaSuccess ? MPG_OK : MPG_ERR_CUDA;
}

int run_cg64_dia(cudaStream_t s, const DiaMatrix &A, const double *b, double *x, double tol, int max_iter, CgWork &w,
                 DevStats *st) {
  Cg64DiaArgs a;
  a.A = A;
  a.b = b;
  a.x = x;
  a.r = w.r;
  a.p0 = w.p0;
  a.p1 = w.p1;
  a.q = w.q;
  a.partials = w.partials;
  a.tol2 = tol * tol;
  a.max_iter = max_iter;
  a.st = st;
  const int nb = grid_for_rows(A.n, w.max_blocks);
  void *args[] = {&a};
  void *fn = A.ndiag <= 15 ? (void *)k_cg64_dia<15> : (void *)k_cg64_dia<27>;
  cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(nb), dim3(kCgThreads), args, 0, s);
  return e == cudaSuccess ? MPG_OK : MPG_ERR_CUDA;
}

int run_cg_mixed(cudaStream_t s, const DiaMatrix &A, const double *b, double *x, double tol, double inner_tol,
                 int max_iter, CgWork &w, DevStats *st) {
  CgMixedArgs a;
  a.A = A;
  a.b = b;
  a.x = x;
  a.r64 = w.r;
  a.r = w.r32;
  a.z = w.z32;
  a.q = w.q32;
  a.pa = w.pa32;
  a.pb = w.pb32;
  a.partials = w.partials;
  a.tol2 = tol * tol;
  a.inner_tol2 = inner_tol * inner_tol;
  a.max_iter = max_iter;
  a.st = st;
  const int nb = grid_for_rows(A.n, w.max_blocks);
  void *args[] = {&a};
  void *fn = A.ndiag <= 15 ? (void *)k_cg_mixed<15> : (void *)k_cg_mixed<27>;
  cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(nb), dim3(kCgThreads), args, 0, s);
  return e == cudaSuccess ? MPG_OK : MPG_ERR_CUDA;
}

// CG_solve.hpp:115-206, one host round trip per dot product
int run_bicgstab(cudaStream_t s, int64_t n, const int32_t *rp, const int32_t *col, const double *val,
                 const double *rhs, double *x, double tol, int max_iter, double *work, double *red_dev,
                 double *red_host, int *iters_out, double *resid_out) {
  const int th = 256;
  const unsigned g = (unsigned)((n + th - 1) / th);
  const int nbd = 256;
  double *r = work, *rt = work + n, *p = work + 2 * n, *v = work + 3 * n, *t = work + 4 * n;
  double *part = red_dev + 8;
  auto dot = [&](const double *A, const double *B) -> double {
    k_dot_partial<<<nbd, th, 0, s>>>(n, A, B, part);
    k_dot_final<<<1, th, 0, s>>>(part, nbd, red_dev);
    cudaMemcpyAsync(red_host, red_dev, sizeof(double), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    return *red_host;
  };
  double rho0, rho, rho_old = 0.0, beta = 0.0, alpha = 0.0, omega = 0.0, resid = 0.0;
  rho0 = dot(rhs, rhs);
  cudaMemsetAsync(x, 0, sizeof(double) * n, s);  // x->scale(0.)
  k_spmv64<<<g, th, 0, s>>>(n, rp, col, val, x, r);
  k_update<<<g, th, 0, s>>>(n, 1.0, rhs, -1.0, r);
  cudaMemcpyAsync(rt, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
  rho = dot(rt, r);
  *iters_out = 0;
  *resid_out = 0.0;
  if (rho == 0) return cudaGetLastError() == cudaSuccess ? MPG_OK : MPG_ERR_CUDA;
  int iter = 0;
  for (; iter < max_iter; ++iter) {
    if (iter == 0) {
      cudaMemcpyAsync(p, r, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
    } else {
      rho = dot(rt, r);
      if (rho == 0) break;
      beta = rho / rho_old * alpha / omega;
      k_update<<<g, th, 0, s>>>(n, -omega, v, 1.0, p);
      k_update<<<g, th, 0, s>>>(n, 1.0, r, beta, p);
    }
    k_spmv64<<<g, th, 0, s>>>(n, rp, col, val, p, v);
    alpha = dot(rhs, v);
    alpha = rho / alpha;
    k_update<<<g, th, 0, s>>>(n, -alpha, v, 1.0, r);
    if ((resid = dot(r, r)) < rho0 * tol * tol) {
      k_update<<<g, th, 0, s>>>(n, alpha, p, 1.0, x);
      break;
    }
    k_spmv64<<<g, th, 0, s>>>(n, rp, col, val, r, t);
    const double tdott = dot(t, t);
    omega = dot(t, r) / tdott;
    if (omega == 0.0 || tdott == 0) break;
    k_update<<<g, th, 0, s>>>(n, alpha, p, 1.0, x);
    k_update<<<g, th, 0, s>>>(n, omega, r, 1.0, x);
    k_update<<<g, th, 0, s>>>(n, -omega, t, 1.0, r);
    rho_old = rho;
    resid = dot(r, r);
    if (resid / rho0 < tol * tol) break;
  }
  *iters_out = iter;
  *resid_out = rho0 > 0 ? sqrt(resid / rho0) : 0.0;
  if (cudaGetLastError() != cudaSuccess) return MPG_ERR_CUDA;
  return iter >= max_iter ? MPG_ERR_NOT_CONVERGED : MPG_OK;
}
