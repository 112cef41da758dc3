// mpg_device.cuh -- device-side layouts and helpers of the GB300 PIC library.
//
// All translation units are built with --fmad=false: every FP64 multiply and
// add rounds separately, like the reference's CPU build.  The single-precision
// kernels of the mixed form request fused multiply-adds explicitly
// (__fmaf_rn), so their results are reproducible too.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define MPG_MAX_SPECIES 16
#define MPG_DEAD 0xFFFFFFFFu
#define MPG_WALL 0xFFFFFFu

// per-species constants, uploaded with cudaMemcpyToSymbolAsync
struct SpeciesTable {
  double q[MPG_MAX_SPECIES];
  double m[MPG_MAX_SPECIES];
  double qm[MPG_MAX_SPECIES];
  double w[MPG_MAX_SPECIES];       // mixed form: weight per species
  long long qfix[MPG_MAX_SPECIES]; // mixed form: charge w*q in quanta
  float qm_f[MPG_MAX_SPECIES];
  float half_wm_f[MPG_MAX_SPECIES];  // 0.5 * w * m for the kinetic energy
};

// device-side counters of one step; zeroed by the host before a step batch
struct DevStats {
  unsigned long long n_killed;
  unsigned long long n_cross;
  unsigned long long n_limit;
  unsigned long long n_nan;
  double ke;
  int solver_iters;
  int solver_status;   // 0 ok, 1 not converged
  int solver_fail;     // sticky: some solve of the batch did not converge
  int iters_total;     // summed over the solves of a batch
  double solver_resid;
  unsigned int bar_count;
  unsigned int bar_gen;
  int bar_error;
  int bar_mode;  // 0: fence + volatile polling, 1: release/acquire
  // test of the time-out path (mpg_set_barrier_test): block bar_skip - 1
  // skips its arrivals (0 = none); bar_limit = polls before a wait gives up
  // (0 = the default 2^22)
  int bar_skip;
  unsigned int bar_limit;
};

// -------------------------------------------------------------------------
// grid-wide barrier for cooperative launches.  Every block of the grid is
// co-resident (cudaLaunchCooperativeKernel guarantees it).  bar_count only
// grows: the k-th barrier of a launch completes when it reaches k * nblocks
// (the host zeroes it before each launch).  Arrival is one release-reduction,
// the wait is an acquire load, so the block's writes before the barrier are
// visible to every block after it.  The wait is bounded: after ~2^22 polls
// (about a second with the back-off; bar_limit when set) the block raises
// bar_error and returns false; every later barrier sees the flag and returns
// false at once, so all blocks leave the kernel.  `epoch` is a per-block
// counter (thread 0 only).  A block named by bar_skip does not arrive (the
// host-set test of this time-out path).
__device__ __forceinline__ bool grid_barrier(DevStats *st, unsigned nblocks, unsigned &epoch) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    ok = 1;
    ++epoch;
    const unsigned target = epoch * nblocks;
    unsigned *cnt = &st->bar_count;
    const int mode = st->bar_mode;
    const unsigned limit = st->bar_limit ? st->bar_limit : (1u << 22);
    if (st->bar_skip == (int)blockIdx.x + 1) {
      // no arrival (time-out test)
    } else if (mode == 0) {
      // fence + relaxed arrival, volatile polling, fence
      __threadfence();
      atomicAdd(cnt, 1u);
    } else {
      asm volatile("red.release.gpu.global.add.u32 [%0], 1;" ::"l"(cnt) : "memory");
    }
    unsigned spins = 0, v;
    for (;;) {
      if (mode == 0)
        v = *(volatile unsigned *)cnt;
      else
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(cnt) : "memory");
      if ((int)(v - target) >= 0) break;
      ++spins;
      if ((spins & 255u) == 0) {
        if (*(volatile int *)&st->bar_error) {
          ok = 0;
          break;
        }
        if (spins > limit) {
          atomicExch(&st->bar_error, 1);
          ok = 0;
          break;
        }
      }
      if (spins > 64) __nanosleep(32);
    }
    if (mode == 0) __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

// sum of the fixed-point charge slots acc[lo .. hi) as a signed integer, in
// 16-byte loads, four slots per iteration into four partial sums (integer
// sums: the grouping does not change the result), so that a thread has
// several loads in flight; acc must start on a 16-byte boundary (a device
// allocation does), so an even slot index is one too
__device__ __forceinline__ long long slot_sum(const unsigned long long *__restrict__ acc, int32_t lo, int32_t hi) {
  int32_t q = lo;
  long long a0 = 0, a1 = 0, a2 = 0, a3 = 0;
  if ((q & 1) && q < hi) a0 += (long long)acc[q++];
  for (; q + 4 <= hi; q += 4) {
    const ulonglong2 x = *reinterpret_cast<const ulonglong2 *>(acc + q);
    const ulonglong2 y = *reinterpret_cast<const ulonglong2 *>(acc + q + 2);
    a0 += (long long)x.x;
    a1 += (long long)x.y;
    a2 += (long long)y.x;
    a3 += (long long)y.y;
  }
  for (; q < hi; ++q) a0 += (long long)acc[q];
  return (a0 + a1) + (a2 + a3);
}

// block-wide sum of one double per thread (blockDim.x multiple of 32, <= 1024);
// deterministic for a fixed block size.  Result valid in thread 0.  The last
// stage runs in warp 0 as a shuffle tree (FP64 is a slow pipe on this chip, so
// no thread sums serially).
__device__ __forceinline__ double block_sum(double v, double *smem32) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) smem32[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    s = lane < nw ? smem32[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  }
  return s;
}

// neighbour row of row i along a stencil offset; on a periodic mesh the rows
// are the x < hi planes and x wraps around, i.e. the index is taken modulo nwrap
__device__ __forceinline__ int64_t dia_nb(int64_t i, int off, int64_t nwrap) {
  int64_t j = i + off;
  if (nwrap) {
    if (j < 0)
      j += nwrap;
    else if (j >= nwrap)
      j -= nwrap;
  }
  return j;
}

// sum of partials[0..nb): every thread loads at most one partial (one L2
// round trip), then a fixed block reduction; all blocks compute the same
// value bit for bit.
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

// ---------------------------------------------------------------------------
// float-float ("double-single") arithmetic: a value is hi + lo with |lo| <=
// ulp(hi)/2, about 44 significant bits, built from FP32 operations only
// (Knuth's TwoSum and the FMA-based exact product).  Used for the dot products
// of the mixed solver, where FP64 would run on the slow FP64 pipe.  The
// translation unit is built with --fmad=false, so no operation below is
// contracted behind our back.
struct ff {
  float hi, lo;
};
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  e += a.lo + b.lo;
  const float hi = s + e;
  return {hi, e - (hi - s)};
}
__device__ __forceinline__ ff ff_prod(float a, float b) {
  const float p = a * b;
  return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ ff ff_mulf(ff a, float b) {
  const float p = a.hi * b;
  const float e = __fmaf_rn(a.hi, b, -p) + a.lo * b;
  const float hi = p + e;
  return {hi, e - (hi - p)};
}
__device__ __forceinline__ ff ff_shfl_down(ff a, int o) {
  return {__shfl_down_sync(0xffffffffu, a.hi, o), __shfl_down_sync(0xffffffffu, a.lo, o)};
}
// block-wide float-float sums of K values per thread; results valid in all
// threads (broadcast through shared memory).  sm must hold K*32 ff.
template <int K>
__device__ __forceinline__ void block_sum_ff(ff v[K], ff *sm) {
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = ff_add(v[k], ff_shfl_down(v[k], o));
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < K; ++k) sm[k * 32 + wid] = v[k];
  __syncthreads();
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      ff s = lane < nw ? sm[k * 32 + lane] : ff{0.f, 0.f};
      for (int o = 16; o > 0; o >>= 1) s = ff_add(s, ff_shfl_down(s, o));
      if (lane == 0) sm[k * 32] = s;
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; ++k) v[k] = sm[k * 32];
  __syncthreads();
}

__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long v, unsigned long long *smem32) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) smem32[wid] = v;
  __syncthreads();
  unsigned long long s = 0;
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    for (int i = 0; i < nw; ++i) s += smem32[i];
  }
  return s;
}
