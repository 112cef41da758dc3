// mg_host.cpp -- geometric multigrid hierarchy for the mixed solver's
// preconditioner, built once per configure on the host.
//
// The node grid of the structured tet mesh (gx * gy * gz nodes, x slowest)
// is coarsened by two in every direction: coarse node C sits on fine node 2C
// (with an even node extent the last coarse node is the far boundary node).  Prolongation P is trilinear interpolation in
// index space between interior nodes (Dirichlet nodes carry no error), the
// restriction is P^T, and the coarse operator is the Galerkin product
// A_c = P^T A P, a 27-point stencil on the coarse grid (Dirichlet rows are
// identity rows).  The coarsest level (at most kDenseMax interior unknowns)
// is solved with its dense inverse.  Not part of the reference: MiniPIC's
// solver is unpreconditioned CG / BiCGStab (CG_solve.hpp); the V-cycle only
// preconditions the FP32 inner iterations, the FP64 outer residual is the
// same as without it.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <string>
#include <vector>

#include "mpg_internal.h"

namespace {

constexpr int kDenseMaxDefault = 1500;  // interior unknowns of the coarsest level (11^3 = 1331, 12 x 11^2 = 1452)
constexpr int kMaxLevels = 8;

// row access to a level's FP64 operator: level 0 is the assembled CSR, the
// coarser ones are 27-point stencils [d][n] with d = 9 (di+1) + 3 (dj+1) + (dk+1).
// On a mesh periodic in x the levels hold the gx x-planes without the ghost
// plane, x indices wrap around and only the y/z walls are Dirichlet rows.
struct LevelOp {
  int gx, gy, gz;
  bool px = false;  // periodic in x
  const std::vector<int32_t> *rp = nullptr, *col = nullptr;
  const std::vector<double> *val = nullptr;
  std::vector<double> dia;  // 27 * n (coarse levels)
  int64_t n() const { return (int64_t)gx * gy * gz; }
  bool bnd(int64_t i, int64_t j, int64_t k) const {
    return (!px && (i == 0 || i == gx - 1)) || j == 0 || k == 0 || j == gy - 1 || k == gz - 1;
  }
  int64_t wrapx(int64_t i) const { return px ? (i % gx + gx) % gx : i; }
  // interior unknowns (rows that are not Dirichlet rows)
  int64_t interior() const { return (int64_t)(px ? gx : gx - 2) * (gy - 2) * (gz - 2); }
};

}  // namespace

bool host_mg_build(const HostMesh &m, const std::vector<int32_t> &rp, const std::vector<int32_t> &col,
                   const std::vector<double> &val, MgHostHierarchy &H, std::string &why, int64_t dense_max) {
  H = MgHostHierarchy();
  const bool px = m.d.periodic != 0;
  std::vector<LevelOp> ops(1);
  // level 0: the solver's rows (a periodic mesh solves the nx planes x < hi)
  ops[0].gx = px ? m.d.nx : m.d.nx + 1;
  ops[0].gy = m.d.ny + 1;
  ops[0].gz = m.d.nz + 1;
  ops[0].px = px;
  ops[0].rp = &rp;
  ops[0].col = &col;
  ops[0].val = &val;
  if ((int64_t)rp.size() != ops[0].n() + 1) {
    why = "system rows do not match the node grid";
    return false;
  }
  int64_t kDenseMax = kDenseMaxDefault;
  if (const char *e = getenv("MPG_MG_DENSE_MAX")) kDenseMax = atoll(e);
  if (dense_max > 0) kDenseMax = dense_max;
  while ((int)ops.size() < kMaxLevels && ops.back().interior() > kDenseMax) {
    const LevelOp &f = ops.back();
    // Dirichlet axes: coarse node C sits on fine node 2C; node extents 2m+1 ->
    // m+1, and an even extent 2m -> m+1 whose last coarse node is the far
    // boundary node 2m-1 (only that boundary interval is one fine cell long;
    // interior nodes interpolate as everywhere else).  A periodic x axis
    // needs an even plane count 2m -> m (m >= 4, so that the 27-point
    // stencil's x-1 and x+1 planes stay distinct).
    const bool okx = f.px ? (f.gx % 2 == 0 && f.gx / 2 >= 4) : f.gx >= 5;
    if (!okx || f.gy < 5 || f.gz < 5) break;
    LevelOp c;
    c.px = f.px;
    auto half = [](int g) { return g / 2 + 1; };  // (2m+1) -> m+1 and 2m -> m+1
    c.gx = f.px ? f.gx / 2 : half(f.gx);
    c.gy = half(f.gy);
    c.gz = half(f.gz);
    const int64_t nc = c.n();
    c.dia.assign(27 * nc, 0.0);
    const int64_t fsj = f.gz, fsi = (int64_t)f.gy * f.gz, csj = c.gz, csi = (int64_t)c.gy * c.gz;
    // A_c[C, C'] = sum_{f, f'} P[f, C] A[f, f'] P[f', C'] over interior f, f', C, C'
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t C = 0; C < nc; ++C) {
      const int64_t I = C / csi, J = (C / csj) % c.gy, K = C % csj;
      double acc[27] = {0};
      if (c.bnd(I, J, K)) {
        c.dia[13 * nc + C] = 1.0;  // identity row
        continue;
      }
      for (int di = -1; di <= 1; ++di)
        for (int dj = -1; dj <= 1; ++dj)
          for (int dk = -1; dk <= 1; ++dk) {
            const int64_t fi = f.wrapx(2 * I + di), fj = 2 * J + dj, fk = 2 * K + dk;
            if (f.bnd(fi, fj, fk)) continue;
            const double wf = (di ? 0.5 : 1.0) * (dj ? 0.5 : 1.0) * (dk ? 0.5 : 1.0);
            const int64_t frow = fi * fsi + fj * fsj + fk;
            auto visit = [&](int64_t fcol, double a) {
              const int64_t gi = fcol / fsi, gj = (fcol / fsj) % f.gy, gk = fcol % fsj;
              if (f.bnd(gi, gj, gk)) return;
              // coarse nodes interpolating fine node (gi, gj, gk)
              const int64_t ci0 = gi / 2, ci1 = c.wrapx((gi + 1) / 2), cj0 = gj / 2, cj1 = (gj + 1) / 2,
                            ck0 = gk / 2, ck1 = (gk + 1) / 2;
              const int ni = gi % 2 ? 2 : 1, nj = gj % 2 ? 2 : 1, nk = gk % 2 ? 2 : 1;
              const double wi = gi % 2 ? 0.5 : 1.0, wj = gj % 2 ? 0.5 : 1.0, wk = gk % 2 ? 0.5 : 1.0;
              for (int a1 = 0; a1 < ni; ++a1)
                for (int a2 = 0; a2 < nj; ++a2)
                  for (int a3 = 0; a3 < nk; ++a3) {
                    const int64_t CI = a1 ? ci1 : ci0, CJ = a2 ? cj1 : cj0, CK = a3 ? ck1 : ck0;
                    if (c.bnd(CI, CJ, CK)) continue;
                    int64_t dI = CI - I;
                    if (c.px) {
                      if (dI > 1) dI -= c.gx;
                      if (dI < -1) dI += c.gx;
                    }
                    const int d = 9 * (int)(dI + 1) + 3 * (int)(CJ - J + 1) + (int)(CK - K + 1);
                    acc[d] += wf * a * (wi * wj * wk);
                  }
            };
            if (f.rp) {
              for (int32_t q = (*f.rp)[frow]; q < (*f.rp)[frow + 1]; ++q) visit((*f.col)[q], (*f.val)[q]);
            } else {
              const int64_t nf = f.n();
              for (int d = 0; d < 27; ++d) {
                const double a = f.dia[d * nf + frow];
                if (a == 0.0) continue;
                const int64_t gi = f.wrapx(fi + d / 9 - 1), gj = fj + (d / 3) % 3 - 1, gk = fk + d % 3 - 1;
                visit(gi * fsi + gj * fsj + gk, a);
              }
            }
          }
      for (int d = 0; d < 27; ++d) c.dia[d * nc + C] = acc[d];
    }
    ops.push_back(std::move(c));
  }
  if (ops.size() < 2 || ops.back().interior() > kDenseMax) {
    why = "grid cannot be coarsened to a small enough level";
    return false;
  }
  // device-side level data
  H.lev.resize(ops.size());
  for (size_t l = 0; l < ops.size(); ++l) {
    const LevelOp &o = ops[l];
    MgHostLevel &L = H.lev[l];
    L.gx = o.gx;
    L.gy = o.gy;
    L.gz = o.gz;
    L.px = o.px;
    const int64_t n = o.n();
    L.dinv.assign(n, 1.0f);
    L.bnd.assign(n, 1);
    for (int64_t r = 0; r < n; ++r) {
      const int64_t i = r / ((int64_t)o.gy * o.gz), j = (r / o.gz) % o.gy, k = r % o.gz;
      L.bnd[r] = o.bnd(i, j, k) ? 1 : 0;
    }
    if (l == 0) {
      for (int64_t r = 0; r < n; ++r)
        for (int32_t q = rp[r]; q < rp[r + 1]; ++q)
          if (col[q] == r && val[q] != 0.0) L.dinv[r] = (float)(1.0 / val[q]);
    } else {
      L.val.resize(27 * n);
      for (int64_t q = 0; q < 27 * n; ++q) L.val[q] = (float)o.dia[q];
      for (int64_t r = 0; r < n; ++r) L.dinv[r] = (float)(1.0 / o.dia[13 * n + r]);
    }
  }
  // dense inverse of the coarsest level over its interior unknowns (Gauss-Jordan, FP64)
  const LevelOp &o = ops.back();
  const int64_t n = o.n();
  for (int64_t r = 0; r < n; ++r)
    if (!H.lev.back().bnd[r]) H.dense_idx.push_back((int32_t)r);
  const int mm = (int)H.dense_idx.size();
  std::vector<int> pos(n, -1);
  for (int a = 0; a < mm; ++a) pos[H.dense_idx[a]] = a;
  std::vector<double> M((size_t)mm * mm, 0.0), Inv((size_t)mm * mm, 0.0);
  const int64_t sj = o.gz, si = (int64_t)o.gy * o.gz;
  for (int a = 0; a < mm; ++a) {
    const int64_t r = H.dense_idx[a];
    const int64_t ri = r / si, rj = (r / sj) % o.gy, rk = r % sj;
    for (int d = 0; d < 27; ++d) {
      const int64_t ci = o.wrapx(ri + d / 9 - 1), cj = rj + (d / 3) % 3 - 1, ck = rk + d % 3 - 1;
      if (ci < 0 || ci >= o.gx || cj < 0 || cj >= o.gy || ck < 0 || ck >= o.gz) continue;
      const int64_t c = ci * si + cj * sj + ck;
      if (pos[c] < 0) continue;
      M[(size_t)a * mm + pos[c]] += o.dia[d * n + r];
    }
    Inv[(size_t)a * mm + a] = 1.0;
  }
  for (int p = 0; p < mm; ++p) {
    int piv = p;
    for (int q = p + 1; q < mm; ++q)
      if (std::fabs(M[(size_t)q * mm + p]) > std::fabs(M[(size_t)piv * mm + p])) piv = q;
    if (std::fabs(M[(size_t)piv * mm + p]) < 1e-300) {
      why = "singular coarsest operator";
      return false;
    }
    if (piv != p)
      for (int q = 0; q < mm; ++q) {
        std::swap(M[(size_t)p * mm + q], M[(size_t)piv * mm + q]);
        std::swap(Inv[(size_t)p * mm + q], Inv[(size_t)piv * mm + q]);
      }
    const double inv = 1.0 / M[(size_t)p * mm + p];
    // columns q < p of the pivot row are already exactly zero, so M's updates
    // start at column p; the rows are eliminated in parallel (each row's
    // arithmetic, and so the result, is that of the sequential loop)
    for (int q = p; q < mm; ++q) M[(size_t)p * mm + q] *= inv;
    for (int q = 0; q < mm; ++q) Inv[(size_t)p * mm + q] *= inv;
#pragma omp parallel for schedule(static)
    for (int r = 0; r < mm; ++r) {
      if (r == p) continue;
      const double f = M[(size_t)r * mm + p];
      if (f == 0.0) continue;
      for (int q = p; q < mm; ++q) M[(size_t)r * mm + q] -= f * M[(size_t)p * mm + q];
      for (int q = 0; q < mm; ++q) Inv[(size_t)r * mm + q] -= f * Inv[(size_t)p * mm + q];
    }
  }
  H.dense_inv.resize((size_t)mm * mm);
  for (size_t q = 0; q < Inv.size(); ++q) H.dense_inv[q] = (float)Inv[q];
  return true;
}
