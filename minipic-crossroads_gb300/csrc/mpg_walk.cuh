// mpg_walk.cuh -- push + tet walk of one particle in the mixed form.
//
// Shared by the single-run kernel (kernels.cu) and the batched kernel
// (batch.cu), so that a run advanced alone and a run advanced inside a batch
// execute the same arithmetic.  The per-tet tables are reached through a
// table policy `Tab` with
//   load(e, r0, r1, r2): the tet's record, J^-1 (9 floats) + E (3 floats),
//   face(e, k): the neighbour word of the face opposite vertex k of tet e
//               (neighbour | vertex permutation << 24, MPG_WALL = wall).
// RecTab3 reads the tables rec[3*e .. 3*e+2] and nbr[e] as needed (the
// neighbour word only when the particle reaches a face).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpg_device.cuh"

struct RecTab3 {
  const float4 *__restrict__ rec;
  const uint4 *__restrict__ nbr;
  __device__ __forceinline__ void load(uint32_t e, float4 &r0, float4 &r1, float4 &r2) const {
    r0 = rec[3 * e];
    r1 = rec[3 * e + 1];
    r2 = rec[3 * e + 2];
  }
  __device__ __forceinline__ uint32_t face(uint32_t e, int k) const {
    const uint4 nb4 = nbr[e];
    return k == 0 ? nb4.x : k == 1 ? nb4.y : k == 2 ? nb4.z : nb4.w;
  }
};

// Boris push with B = 0: the two half kicks of particle_move.hpp:376-387
// (hk = dt q/(2m)) with E of the start tet in r2.yzw
__device__ __forceinline__ void mixed_kick(const float hk, const float4 &r2, float &vx, float &vy, float &vz) {
  vx = __fmaf_rn(hk, r2.y, vx);
  vy = __fmaf_rn(hk, r2.z, vy);
  vz = __fmaf_rn(hk, r2.w, vz);
  vx = __fmaf_rn(hk, r2.y, vx);
  vy = __fmaf_rn(hk, r2.z, vy);
  vz = __fmaf_rn(hk, r2.w, vz);
}

// The walk of a kicked particle across faces until dt is used up
// (particle_move.hpp:110-121), from tet e with barycentrics (l1, l2, l3).
// Barycentrics are carried across each face through the vertex
// permutation; the entered face's coordinate is exactly 0.  Returns the
// number of face crossings; *dead is set when the particle left through an
// absorbing wall, *limit when max_cross was reached.  The record of the
// start tet e is given in (r0, r1, r2); on return they hold the record of
// the final tet.  STOP: return as soon as the first step finds an exit
// before dt, with *stopped set and nothing changed, so that the walk can be
// run again from the same state later (the move kernel gathers such
// particles to walk them in full warps).
template <bool STOP, class Tab>
__device__ __forceinline__ int mixed_walk_from(Tab &tab, uint32_t &e, float4 &r0, float4 &r1, float4 &r2, float &l1,
                                               float &l2, float &l3, float &vx, float &vy, float &vz, const float dt,
                                               const int kill, const int max_cross, bool &dead, bool &limit,
                                               bool &stopped) {
  dead = false;
  limit = false;
  stopped = false;
  float tleft = dt;
  int entry = -1;  // vertex opposite the face the particle entered through
  int it = 0;
  for (;;) {
    // barycentric velocity u_k = d lambda_k / dt; u_{1..3} = J^-1 v
    const float u1 = __fmaf_rn(r0.z, vz, __fmaf_rn(r0.y, vy, r0.x * vx));
    const float u2 = __fmaf_rn(r1.y, vz, __fmaf_rn(r1.x, vy, r0.w * vx));
    const float u3 = __fmaf_rn(r2.x, vz, __fmaf_rn(r1.w, vy, r1.z * vx));
    const float u0 = -(u1 + u2 + u3);
    const float l0 = 1.0f - l1 - l2 - l3;
    const float lam[4] = {l0, l1, l2, l3};
    const float uu[4] = {u0, u1, u2, u3};
    // earliest exit: face k is reached at t_k = lam_k / (-u_k) for u_k < 0.
    // Compare t_k < t_best as lam_k * w_best < lam_best * w_k (w = -u > 0),
    // so a division is needed only for the face actually crossed.
    int kmin = -1;
    float lbest = 0.f, wbest = 0.f;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (uu[k] < 0.f && k != entry) {
        const float lk = fmaxf(lam[k], 0.f), wk = -uu[k];
        // inside the remaining time?  lam_k < tleft * w_k
        if (lk < tleft * wk && (kmin < 0 || lk * wbest < lbest * wk)) {
          kmin = k;
          lbest = lk;
          wbest = wk;
        }
      }
    }
    if (kmin < 0) {
      l1 = __fmaf_rn(tleft, u1, l1);
      l2 = __fmaf_rn(tleft, u2, l2);
      l3 = __fmaf_rn(tleft, u3, l3);
      break;
    }
    if (STOP) {
      stopped = true;
      break;
    }
    if (it >= max_cross) {
      limit = true;
      break;
    }
    ++it;
    const float tmin = __fdiv_rn(lbest, wbest);
    float nl[4] = {__fmaf_rn(tmin, u0, l0), __fmaf_rn(tmin, u1, l1), __fmaf_rn(tmin, u2, l2),
                   __fmaf_rn(tmin, u3, l3)};
    nl[kmin] = 0.f;
    tleft = tleft - tmin;
    const uint32_t w = tab.face(e, kmin);
    const uint32_t nb = w & 0xFFFFFFu;
    if (nb == MPG_WALL) {
      if (kill) {
        dead = true;
        l1 = nl[1];
        l2 = nl[2];
        l3 = nl[3];
        break;
      }
      // specular reflection off the wall: outward normal is -grad(lambda_k)
      float gx, gy, gz;
      if (kmin == 1) {
        gx = r0.x; gy = r0.y; gz = r0.z;
      } else if (kmin == 2) {
        gx = r0.w; gy = r1.x; gz = r1.y;
      } else if (kmin == 3) {
        gx = r1.z; gy = r1.w; gz = r2.x;
      } else {
        gx = -(r0.x + r0.w + r1.z);
        gy = -(r0.y + r1.x + r1.w);
        gz = -(r0.z + r1.y + r2.x);
      }
      const float inv = rsqrtf(__fmaf_rn(gz, gz, __fmaf_rn(gy, gy, gx * gx)));
      gx *= inv;
      gy *= inv;
      gz *= inv;
      const float vdn2 = 2.f * __fmaf_rn(vz, gz, __fmaf_rn(vy, gy, vx * gx));
      vx = __fmaf_rn(-vdn2, gx, vx);
      vy = __fmaf_rn(-vdn2, gy, vy);
      vz = __fmaf_rn(-vdn2, gz, vz);
      l1 = nl[1];
      l2 = nl[2];
      l3 = nl[3];
      entry = kmin;
      continue;
    }
    const uint32_t perm = w >> 24;
    float ml[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) ml[(perm >> (2 * j)) & 3u] = nl[j];
    entry = (int)((perm >> (2 * kmin)) & 3u);
    ml[entry] = 0.f;
    e = nb;
    l1 = ml[1];
    l2 = ml[2];
    l3 = ml[3];
    tab.load(e, r0, r1, r2);
  }
  return it;
}

// kick and full walk from the start tet e (record in r0, r1, r2)
template <class Tab>
__device__ __forceinline__ int mixed_walk_t(Tab &tab, uint32_t &e, float4 &r0, float4 &r1, float4 &r2, float &l1,
                                            float &l2, float &l3, float &vx, float &vy, float &vz, const float hk,
                                            const float dt, const int kill, const int max_cross, bool &dead,
                                            bool &limit) {
  mixed_kick(hk, r2, vx, vy, vz);
  bool stopped;
  return mixed_walk_from<false>(tab, e, r0, r1, r2, l1, l2, l3, vx, vy, vz, dt, kill, max_cross, dead, limit,
                                stopped);
}

// the walk on run-local tables rec[3*e ..] / nbr[e] (batch engine)
__device__ __forceinline__ int mixed_walk(const float4 *__restrict__ rec, const uint4 *__restrict__ nbr, uint32_t &e,
                                          float &l1, float &l2, float &l3, float &vx, float &vy, float &vz,
                                          const float hk, const float dt, const int kill, const int max_cross,
                                          bool &dead, bool &limit) {
  RecTab3 tab{rec, nbr};
  float4 r0, r1, r2;
  tab.load(e, r0, r1, r2);
  return mixed_walk_t(tab, e, r0, r1, r2, l1, l2, l3, vx, vy, vz, hk, dt, kill, max_cross, dead, limit);
}
