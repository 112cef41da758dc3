/*
 * oracle.cpp -- CPU restatement of MiniPIC's electrostatic PIC step.
 *
 * TEST INFRASTRUCTURE ONLY (see oracle.h).  Compiled with
 * -ffp-contract=off so that every multiply and add rounds separately, the
 * same as the plain FP64 CUDA path built with --fmad=false.
 *
 * Each function names the reference file:line whose operation order it
 * follows.  Reference file names are relative to the MiniPIC source tree.
 */
#include "oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

struct orc_mesh {
  orc_mesh_desc d;
  int64_t T = 0, N = 0, n_faces = 0, n_bfaces = 0, n_bnodes = 0;
  std::vector<double> nodes;    // N*3
  std::vector<int32_t> tets;    // T*4
  std::vector<int32_t> nbrs;    // T*4, reference face order
  std::vector<double> jinv;     // T*9
  std::vector<double> detj;     // T
  std::vector<double> normals;  // T*12
  std::vector<double> grad;     // T*12
  std::vector<uint8_t> bnd;     // N
  std::vector<int8_t> fper;     // T*4, elem_face_periodic (mesh.cpp:369-392)
  std::vector<int32_t> pair;    // N, node_pairs (mesh.cpp:178-189), -1 = none
  int csr_mode = -1;
  int64_t nsolve = 0;           // rows of the assembled system
  std::vector<int32_t> rowptr, col;
  std::vector<double> val;
};

static inline int nthr(int n) {
#ifdef _OPENMP
  return n > 0 ? n : omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* counter-based draws: splitmix64 finaliser                                 */
extern "C" uint64_t orc_mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
extern "C" uint64_t orc_draw(uint64_t base, uint64_t ctr) { return orc_mix64(base + orc_mix64(ctr)); }
static inline double unit53(uint64_t u) { return (double)(u >> 11) * (1.0 / 9007199254740992.0); }

static const uint64_t SALT_JITTER = 0x6A09E667F3BCC908ULL;
static const uint64_t SALT_FILL = 0xBB67AE8584CAA73BULL;

/* ------------------------------------------------------------------------ */
/* reference LCG (random.hpp:43-87, dRandom): seed = A*seed + C mod 2^64,
 * drand = rand() * (1/(double)M) with M = 2^64-1.                          */
struct RefRand {
  uint64_t s;
  uint64_t rand() {
    s = 6364136223846793005ULL * s + 1442695040888963407ULL;
    return s;
  }
  double drand() {
    const double d = 1. / static_cast<double>(18446744073709551615ULL);
    return rand() * d;
  }
};

extern "C" void orc_ref_lcg(uint64_t seed, int n, uint64_t *rand_out, double *drand_out) {
  RefRand a{seed}, b{seed};
  for (int i = 0; i < n; ++i) {
    if (rand_out) rand_out[i] = a.rand();
    if (drand_out) drand_out[i] = b.drand();
  }
}

/* ------------------------------------------------------------------------ */
/* mesh generation: mesh.cpp:78-714 (single rank)                           */
static void apply_mapping(double &inx, double &iny, double &inz, int mapping) {
  // mesh.cpp:763-792
  double outx = inx, outy = iny, outz = inz;
  switch (mapping) {
    case 1: {
      double r = (1.0 - fabs(inx)) * (1.0 - fabs(iny));
      outx = inx * cos(r) - iny * sin(r);
      outy = inx * sin(r) + iny * cos(r);
      outz = inz;
    } break;
    case 2:
      outx = inx * sqrt(1 - .5 * iny * iny - .5 * inz * inz + iny * iny * inz * inz / 3.);
      outy = iny * sqrt(1 - .5 * inx * inx - .5 * inz * inz + inx * inx * inz * inz / 3.);
      outz = inz * sqrt(1 - .5 * iny * iny - .5 * inx * inx + iny * iny * inx * inx / 3.);
      break;
    case 3:
      outx = inx * inx;
      if (inx < 0) outx = -outx;
      break;
    default:
      return;
  }
  inx = outx;
  iny = outy;
  inz = outz;
}

extern "C" orc_mesh *orc_mesh_create(const orc_mesh_desc *d, char *err, int errlen) {
  auto fail = [&](const char *msg) -> orc_mesh * {
    if (err && errlen > 0) snprintf(err, errlen, "%s", msg);
    return nullptr;
  };
  if (d->nx < 1 || d->ny < 1 || d->nz < 1) return fail("mesh size must be >= 1");
  if (d->split != 5 && d->split != 6) return fail("split must be 5 or 6");
  if (d->periodic && d->nx < 2) return fail("periodic mesh needs nx >= 2");
  // mesh.cpp:91-94: the alternating five-tet split only matches across x when nx is even
  if (d->periodic && d->split == 5 && d->nx % 2 == 1) return fail("periodic five-tet mesh needs an even nx");
  orc_mesh *m = new orc_mesh();
  m->d = *d;
  const int64_t nx = d->nx, ny = d->ny, nz = d->nz;
  const int per = d->split;
  m->N = (nx + 1) * (ny + 1) * (nz + 1);
  m->T = per * nx * ny * nz;
  auto gid = [&](int64_t i, int64_t j, int64_t k) -> int32_t {
    return (int32_t)(i * (ny + 1) * (nz + 1) + j * (nz + 1) + k);  // mesh.cpp:52-54
  };
  // nodes: mesh.cpp:135-142 (x = lo + i*dx, reference lo=-1, dx=2/nx)
  const double dx = (d->hi - d->lo) / nx, dy = (d->hi - d->lo) / ny, dz = (d->hi - d->lo) / nz;
  m->nodes.resize(m->N * 3);
  m->bnd.assign(m->N, 0);
  for (int64_t i = 0; i <= nx; ++i)
    for (int64_t j = 0; j <= ny; ++j)
      for (int64_t k = 0; k <= nz; ++k) {
        int32_t g = gid(i, j, k);
        m->nodes[3 * g + 0] = d->lo + i * dx;
        m->nodes[3 * g + 1] = d->lo + j * dy;
        m->nodes[3 * g + 2] = d->lo + k * dz;
        // boundary nodeset (mesh.cpp:407-412), by grid index; a periodic
        // mesh has no x walls
        if ((!d->periodic && (i == 0 || i == nx)) || j == 0 || j == ny || k == 0 || k == nz) m->bnd[g] = 1;
      }
  // periodic node pairs (mesh.cpp:178-189): interior nodes of the x = hi plane
  m->pair.assign(m->N, -1);
  if (d->periodic)
    for (int64_t j = 1; j < ny; ++j)
      for (int64_t k = 1; k < nz; ++k) m->pair[gid(nx, j, k)] = gid(0, j, k);
  for (int64_t g = 0; g < m->N; ++g) m->n_bnodes += m->bnd[g];
  // tets: mesh.cpp:195-224 (5-split) or Kuhn 6-split
  m->tets.resize(m->T * 4);
  int64_t cnt = 0;
  for (int64_t i = 0; i < nx; ++i)
    for (int64_t j = 0; j < ny; ++j)
      for (int64_t k = 0; k < nz; ++k) {
        int32_t c[8];
        c[0] = gid(i, j, k);
        c[1] = gid(i, j, k + 1);
        c[2] = gid(i, j + 1, k);
        c[3] = gid(i, j + 1, k + 1);
        c[4] = gid(i + 1, j, k);
        c[5] = gid(i + 1, j, k + 1);
        c[6] = gid(i + 1, j + 1, k);
        c[7] = gid(i + 1, j + 1, k + 1);
        if (per == 5) {
          static const int odd[5][4] = {{3, 1, 0, 5}, {6, 4, 5, 0}, {6, 2, 0, 3}, {5, 7, 6, 3}, {5, 6, 0, 3}};
          static const int even[5][4] = {{2, 3, 1, 7}, {7, 6, 4, 2}, {2, 0, 4, 1}, {4, 5, 7, 1}, {2, 4, 7, 1}};
          const int(*tab)[4] = ((i + j + k) % 2 != 0) ? odd : even;
          for (int t = 0; t < 5; ++t, ++cnt)
            for (int q = 0; q < 4; ++q) m->tets[4 * cnt + q] = c[tab[t][q]];
        } else {
          // corner index of a displacement (di,dj,dk) is di*4 + dj*2 + dk (see c[] above)
          static const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
          static const int parity[6] = {+1, -1, -1, +1, +1, -1};
          static const int axbit[3] = {4, 2, 1};
          for (int t = 0; t < 6; ++t, ++cnt) {
            int v1 = axbit[perms[t][0]];
            int v2 = v1 + axbit[perms[t][1]];
            int v[4] = {0, v1, v2, 7};
            if (parity[t] < 0) std::swap(v[2], v[3]);
            for (int q = 0; q < 4; ++q) m->tets[4 * cnt + q] = c[v[q]];
          }
        }
      }
  // face matching (mesh.cpp:233-405): faces (0,1,3),(1,2,3),(0,3,2),(0,2,1)
  static const int fnodes[4][3] = {{0, 1, 3}, {1, 2, 3}, {0, 3, 2}, {0, 2, 1}};
  std::map<std::array<int32_t, 3>, std::vector<std::pair<int32_t, int>>> faces;
  const int64_t plane = (ny + 1) * (nz + 1);
  for (int64_t t = 0; t < m->T; ++t)
    for (int f = 0; f < 4; ++f) {
      std::array<int32_t, 3> key = {m->tets[4 * t + fnodes[f][0]], m->tets[4 * t + fnodes[f][1]],
                                    m->tets[4 * t + fnodes[f][2]]};
      // Mesh::periodic_face (mesh.cpp:61-76): a face with every node on the
      // x = hi plane is renamed onto the x = lo plane
      if (d->periodic && key[0] / plane == nx && key[1] / plane == nx && key[2] / plane == nx)
        for (int q = 0; q < 3; ++q) key[q] -= (int32_t)(nx * plane);
      std::sort(key.begin(), key.end());
      faces[key].push_back({(int32_t)t, f});
    }
  m->fper.assign(m->T * 4, 0);
  m->nbrs.assign(m->T * 4, INT32_MIN);
  auto tuple = [&](int32_t g, int64_t &i, int64_t &j, int64_t &k) {
    i = g / ((ny + 1) * (nz + 1));
    j = (g - i * (ny + 1) * (nz + 1)) / (nz + 1);
    k = g % (nz + 1);
  };
  m->n_faces = (int64_t)faces.size();
  for (auto &kv : faces) {
    auto &v = kv.second;
    if (d->periodic) {
      // mesh.cpp:369-378: a (renamed) face on the x = lo plane is periodic on both sides
      int64_t I[3], J[3], K[3];
      for (int q = 0; q < 3; ++q) tuple(kv.first[q], I[q], J[q], K[q]);
      if (I[0] == 0 && I[1] == 0 && I[2] == 0)
        for (auto &e : v) m->fper[4 * e.first + e.second] = +1;
    }
    if (v.size() == 2) {
      m->nbrs[4 * v[0].first + v[0].second] = v[1].first;
      m->nbrs[4 * v[1].first + v[1].second] = v[0].first;
    } else if (v.size() == 1) {
      // must lie on a wall: all three nodes on one boundary plane (mesh.cpp:367-394)
      int64_t I[3], J[3], K[3];
      for (int q = 0; q < 3; ++q) tuple(kv.first[q], I[q], J[q], K[q]);
      bool wall = (!d->periodic && ((I[0] == 0 && I[1] == 0 && I[2] == 0) || (I[0] == nx && I[1] == nx && I[2] == nx))) ||
                  (J[0] == 0 && J[1] == 0 && J[2] == 0) || (J[0] == ny && J[1] == ny && J[2] == ny) ||
                  (K[0] == 0 && K[1] == 0 && K[2] == 0) || (K[0] == nz && K[1] == nz && K[2] == nz);
      if (!wall) {
        delete m;
        return fail("unmatched interior face");
      }
      m->nbrs[4 * v[0].first + v[0].second] = -1;
      m->n_bfaces++;
    } else {
      delete m;
      return fail("face shared by more than two tets");
    }
  }
  // node mapping (mesh.cpp:587-588) or jitter of interior nodes
  if (d->mapping >= 1 && d->mapping <= 3) {
    for (int64_t g = 0; g < m->N; ++g)
      apply_mapping(m->nodes[3 * g], m->nodes[3 * g + 1], m->nodes[3 * g + 2], d->mapping);
  } else if (d->mapping == 4) {
    const uint64_t base = orc_mix64(d->seed ^ SALT_JITTER);
    const double h[3] = {dx, dy, dz};
    for (int64_t g = 0; g < m->N; ++g) {
      if (m->bnd[g]) continue;
      // a ghost node moves with its pair: the x = hi face is the x = lo face
      // translated by the box length (the periodic crossing is a translation)
      const int64_t src = m->pair[g] >= 0 ? m->pair[g] : g;
      for (int q = 0; q < 3; ++q) {
        double u = unit53(orc_draw(base, 3 * (uint64_t)src + q));
        m->nodes[3 * g + q] += (2.0 * u - 1.0) * d->jitter * h[q];
      }
    }
  }
  // normals (mesh.cpp:650-669), Jacobians (mesh.cpp:671-700), grads (PIC.cpp:203-242)
  m->normals.resize(m->T * 12);
  m->jinv.resize(m->T * 9);
  m->detj.resize(m->T);
  m->grad.resize(m->T * 12);
  static const double ghat[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  for (int64_t t = 0; t < m->T; ++t) {
    const double *X[4];
    for (int q = 0; q < 4; ++q) X[q] = &m->nodes[3 * m->tets[4 * t + q]];
    static const int nrm[4][3] = {{0, 1, 3}, {1, 2, 3}, {0, 3, 2}, {0, 2, 1}};
    for (int f = 0; f < 4; ++f) {
      // v1 = X[a]-X[b], v2 = X[c]-X[b], n = v2 x v1, normalise
      const double *A = X[nrm[f][0]], *B = X[nrm[f][1]], *C = X[nrm[f][2]];
      double v1[3] = {A[0] - B[0], A[1] - B[1], A[2] - B[2]};
      double v2[3] = {C[0] - B[0], C[1] - B[1], C[2] - B[2]};
      double n[3] = {v2[1] * v1[2] - v2[2] * v1[1], v2[2] * v1[0] - v2[0] * v1[2], v2[0] * v1[1] - v2[1] * v1[0]};
      double fac = 1. / sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      for (int q = 0; q < 3; ++q) m->normals[12 * t + 3 * f + q] = n[q] * fac;
    }
    double J[3][3];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) J[r][c] = X[c + 1][r] - X[0][r];
    double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                 J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    if (!(det > 0)) {
      delete m;
      return fail("non-positive Jacobian determinant");
    }
    double *I = &m->jinv[9 * t];
    I[0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
    I[1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    I[2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    I[3] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
    I[4] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    I[5] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    I[6] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
    I[7] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    I[8] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    m->detj[t] = det;
    for (int i = 0; i < 4; ++i)
      for (int dd = 0; dd < 3; ++dd) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s += I[3 * k + dd] * ghat[i][k];
        m->grad[12 * t + 3 * i + dd] = s;
      }
  }
  return m;
}

extern "C" void orc_mesh_destroy(orc_mesh *m) { delete m; }

extern "C" void orc_mesh_export_periodic(const orc_mesh *m, int8_t *face_periodic, int32_t *node_pairs) {
  if (face_periodic) memcpy(face_periodic, m->fper.data(), m->fper.size());
  if (node_pairs) memcpy(node_pairs, m->pair.data(), sizeof(int32_t) * m->pair.size());
}

extern "C" void orc_mesh_sizes(const orc_mesh *m, int64_t *T, int64_t *N, int64_t *n_faces, int64_t *n_bfaces,
                               int64_t *n_bnodes) {
  if (T) *T = m->T;
  if (N) *N = m->N;
  if (n_faces) *n_faces = m->n_faces;
  if (n_bfaces) *n_bfaces = m->n_bfaces;
  if (n_bnodes) *n_bnodes = m->n_bnodes;
}

extern "C" void orc_mesh_export(const orc_mesh *m, double *nodes, int32_t *tets, int32_t *nbrs, double *jinv,
                                double *detj, double *normals, double *grad, uint8_t *boundary) {
  if (nodes) memcpy(nodes, m->nodes.data(), m->nodes.size() * sizeof(double));
  if (tets) memcpy(tets, m->tets.data(), m->tets.size() * sizeof(int32_t));
  if (nbrs) memcpy(nbrs, m->nbrs.data(), m->nbrs.size() * sizeof(int32_t));
  if (jinv) memcpy(jinv, m->jinv.data(), m->jinv.size() * sizeof(double));
  if (detj) memcpy(detj, m->detj.data(), m->detj.size() * sizeof(double));
  if (normals) memcpy(normals, m->normals.data(), m->normals.size() * sizeof(double));
  if (grad) memcpy(grad, m->grad.data(), m->grad.size() * sizeof(double));
  if (boundary) memcpy(boundary, m->bnd.data(), m->bnd.size());
}

/* ------------------------------------------------------------------------ */
/* P1 stiffness assembly: ES.cpp:83-205.  K_e(i,j) = sum_c sum_d G_i[d] *
 * (wm_c * G_j[d]) with wm_c = detJ * (1/24) for the 4-point degree-2 rule.  */
// a periodic ghost node stands for its pair (ES.cpp:93-95,168-176; PIC.cpp:132-134)
static inline int32_t pmap(const orc_mesh *m, int32_t g) { return m->pair[g] >= 0 ? m->pair[g] : g; }

extern "C" int64_t orc_assemble(orc_mesh *m, int mode) {
  const int64_t N = m->N, T = m->T;
  // mode 1 on a periodic mesh solves for the nodes of the x < hi planes only;
  // the ghost plane (the last plane in gid order) is copied afterwards
  const int64_t plane = (int64_t)(m->d.ny + 1) * (m->d.nz + 1);
  const int64_t R = (mode == 1 && m->d.periodic) ? N - plane : N;
  std::vector<std::vector<int32_t>> cols(R);
  for (int64_t t = 0; t < T; ++t)
    for (int a = 0; a < 4; ++a) {
      int32_t r = pmap(m, m->tets[4 * t + a]);
      if (m->bnd[r]) continue;
      for (int b = 0; b < 4; ++b) {
        int32_t c = pmap(m, m->tets[4 * t + b]);
        if (mode == 1 && m->bnd[c]) continue;
        cols[r].push_back(c);
      }
    }
  m->rowptr.assign(R + 1, 0);
  for (int64_t r = 0; r < R; ++r) {
    if (m->bnd[r]) {
      cols[r].assign(1, (int32_t)r);
    } else if (m->pair[r] >= 0) {
      // ghost row of the reference system: -phi_ghost + phi_pair = 0 (ES.cpp:183-189)
      cols[r] = {m->pair[r], (int32_t)r};
    } else {
      std::sort(cols[r].begin(), cols[r].end());
      cols[r].erase(std::unique(cols[r].begin(), cols[r].end()), cols[r].end());
    }
    m->rowptr[r + 1] = m->rowptr[r] + (int32_t)cols[r].size();
  }
  const int64_t nnz = m->rowptr[R];
  m->col.resize(nnz);
  m->val.assign(nnz, 0.0);
  for (int64_t r = 0; r < R; ++r) std::copy(cols[r].begin(), cols[r].end(), m->col.begin() + m->rowptr[r]);
  const double wcub = 1.0 / 24.0;
  for (int64_t t = 0; t < T; ++t) {
    const double *G = &m->grad[12 * t];
    const double wm = m->detj[t] * wcub;
    for (int a = 0; a < 4; ++a) {
      int32_t r = pmap(m, m->tets[4 * t + a]);
      if (m->bnd[r]) continue;
      for (int b = 0; b < 4; ++b) {
        int32_t c = pmap(m, m->tets[4 * t + b]);
        if (mode == 1 && m->bnd[c]) continue;
        double k = 0.0;
        for (int cub = 0; cub < 4; ++cub)
          for (int dd = 0; dd < 3; ++dd) k += G[3 * a + dd] * (wm * G[3 * b + dd]);
        const int32_t *p = std::lower_bound(&m->col[m->rowptr[r]], &m->col[m->rowptr[r + 1]], c);
        m->val[p - m->col.data()] += k;
      }
    }
  }
  for (int64_t r = 0; r < R; ++r) {
    if (m->bnd[r]) m->val[m->rowptr[r]] = 1.0;  // ES.cpp:198-204
    if (m->pair[r] >= 0) {
      m->val[m->rowptr[r]] = 1.0;
      m->val[m->rowptr[r] + 1] = -1.0;
    }
  }
  m->csr_mode = mode;
  m->nsolve = R;
  return nnz;
}

// ghost nodes take their pair's value (the solve of mode 1 leaves them out)
static void periodic_copy(const orc_mesh *m, double *x) {
  if (!m->d.periodic) return;
  for (int64_t g = 0; g < m->N; ++g)
    if (m->pair[g] >= 0) x[g] = x[m->pair[g]];
}

extern "C" int64_t orc_csr_rows(const orc_mesh *m) { return m->nsolve; }

extern "C" void orc_csr_export(const orc_mesh *m, int32_t *rowptr, int32_t *col, double *val) {
  if (rowptr) memcpy(rowptr, m->rowptr.data(), m->rowptr.size() * sizeof(int32_t));
  if (col) memcpy(col, m->col.data(), m->col.size() * sizeof(int32_t));
  if (val) memcpy(val, m->val.data(), m->val.size() * sizeof(double));
}

extern "C" void orc_spmv(const orc_mesh *m, const double *x, double *y, int nthreads) {
  const int64_t N = m->nsolve;
#pragma omp parallel for num_threads(nthr(nthreads)) schedule(static)
  for (int64_t r = 0; r < N; ++r) {
    double s = 0.0;
    for (int32_t p = m->rowptr[r]; p < m->rowptr[r + 1]; ++p) s += m->val[p] * x[m->col[p]];
    y[r] = s;
  }
}

static double dot(const double *a, const double *b, int64_t n, int nthreads) {
  // Fixed chunking so that the result only depends on nthreads.
  int nt = nthr(nthreads);
  if (nt <= 1) {
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
  }
  std::vector<double> part(nt, 0.0);
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    int t = omp_get_thread_num();
#else
    int t = 0;
#endif
    int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
    double s = 0.0;
    for (int64_t i = lo; i < hi; ++i) s += a[i] * b[i];
    part[t] = s;
  }
  double s = 0.0;
  for (int t = 0; t < nt; ++t) s += part[t];
  return s;
}

extern "C" void orc_background(const orc_mesh *m, double rho_bg, double *bg) {
  std::fill(bg, bg + m->N, 0.0);
  for (int64_t t = 0; t < m->T; ++t) {
    double q = -(rho_bg * (m->detj[t] / 6.0)) * 0.25;
    for (int a = 0; a < 4; ++a) bg[pmap(m, m->tets[4 * t + a])] += q;
  }
  for (int64_t i = 0; i < m->N; ++i)
    if (m->bnd[i]) bg[i] = 0.0;
}

/* ------------------------------------------------------------------------ */
/* deposit: PIC.cpp:120-160 (Serial path, NOSORT_WEIGHTING)                  */
static const double CUB_A = 0.5854101966249685, CUB_B = 0.1381966011250105;

static void basis_at_cub(double N[4][4]) {
  // N[i][c]: P1 basis i at cubature point c; points (b,b,b),(a,b,b),(b,a,b),(b,b,a)
  const double P[4][3] = {{CUB_B, CUB_B, CUB_B}, {CUB_A, CUB_B, CUB_B}, {CUB_B, CUB_A, CUB_B}, {CUB_B, CUB_B, CUB_A}};
  for (int c = 0; c < 4; ++c) {
    N[0][c] = 1 - P[c][0] - P[c][1] - P[c][2];
    N[1][c] = P[c][0];
    N[2][c] = P[c][1];
    N[3][c] = P[c][2];
  }
}

static inline void deposit_one(const orc_mesh *m, int mode, int32_t e, const double *xr, double w, double q,
                               const double Nc[4][4], double *rhs) {
  if (mode == 0) {
    const double detj = m->detj[e];
    const double tot_q = w * q * (6 / detj);
    const double wm = detj * (1.0 / 24.0);
    for (int i = 0; i < 4; ++i) {
      double val = 0;
      for (int c = 0; c < 4; ++c) val += -tot_q * (wm * Nc[i][c]);
      rhs[pmap(m, m->tets[4 * e + i])] += val;
    }
  } else {
    const double wq = w * q;
    const double lam[4] = {1 - xr[0] - xr[1] - xr[2], xr[0], xr[1], xr[2]};
    for (int i = 0; i < 4; ++i) rhs[pmap(m, m->tets[4 * e + i])] += -(wq * lam[i]);
  }
}

extern "C" void orc_deposit(const orc_mesh *m, int mode, int64_t n, const int32_t *cell, const double *xref,
                            const double *w, const int32_t *sp, const double *q, const double *bg, double *rhs,
                            int nthreads) {
  double Nc[4][4];
  basis_at_cub(Nc);
  const int64_t N = m->N;
  std::fill(rhs, rhs + N, 0.0);
  int nt = nthr(nthreads);
  if (nt <= 1) {
    for (int64_t p = 0; p < n; ++p)
      if (cell[p] >= 0) deposit_one(m, mode, cell[p], &xref[3 * p], w[p], q[sp[p]], Nc, rhs);
  } else {
    std::vector<std::vector<double>> priv(nt, std::vector<double>());
#pragma omp parallel num_threads(nt)
    {
#ifdef _OPENMP
      int t = omp_get_thread_num();
#else
      int t = 0;
#endif
      priv[t].assign(N, 0.0);
      int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
      for (int64_t p = lo; p < hi; ++p)
        if (cell[p] >= 0) deposit_one(m, mode, cell[p], &xref[3 * p], w[p], q[sp[p]], Nc, priv[t].data());
    }
#pragma omp parallel for num_threads(nt) schedule(static)
    for (int64_t i = 0; i < N; ++i) {
      double s = 0.0;
      for (int t = 0; t < nt; ++t) s += priv[t][i];
      rhs[i] = s;
    }
  }
  if (bg)
    for (int64_t i = 0; i < N; ++i) rhs[i] += bg[i];
  for (int64_t i = 0; i < N; ++i)
    if (m->bnd[i]) rhs[i] = 0.0;  // PIC.cpp:155-158 (Serial semantics)
}

extern "C" void orc_deposit_fixed(const orc_mesh *m, int64_t n, const uint32_t *cellsp, const float *b,
                                  const int64_t *qfix, int64_t *acc) {
  for (int64_t p = 0; p < n; ++p) {
    uint32_t cs = cellsp[p];
    if (cs == 0xFFFFFFFFu) continue;
    int32_t e = (int32_t)(cs & 0xFFFFFFu);
    int s = (int)(cs >> 24);
    const int64_t Q = qfix[s];
    const float Qf = (float)Q;
    int64_t c1 = llrintf(b[3 * p + 0] * Qf);
    int64_t c2 = llrintf(b[3 * p + 1] * Qf);
    int64_t c3 = llrintf(b[3 * p + 2] * Qf);
    int64_t c0 = Q - c1 - c2 - c3;
    // unsigned adds: two's-complement wraparound, same as device atomics
    uint64_t *A = reinterpret_cast<uint64_t *>(acc);
    A[m->tets[4 * e + 0]] += (uint64_t)c0;
    A[m->tets[4 * e + 1]] += (uint64_t)c1;
    A[m->tets[4 * e + 2]] += (uint64_t)c2;
    A[m->tets[4 * e + 3]] += (uint64_t)c3;
  }
}

/* ------------------------------------------------------------------------ */
/* solvers                                                                   */
static int bicgstab_impl(const orc_mesh *m, const double *rhs, double *x, double tol, int max_iter, double *resid_out,
                         int nthreads) {
  // CG_solve.hpp:115-206, operation for operation, over the rows of the assembled system
  const int64_t N = m->nsolve;
  double rho0, rho, rho_old = 0.0, beta = 0.0, alpha = 0.0, omega = 0.0, resid = 0.0;
  rho0 = dot(rhs, rhs, N, nthreads);
  std::vector<double> r(N), rt(N), p(N), v(N), t(N);
  for (int64_t i = 0; i < N; ++i) x[i] = x[i] * 0.;
  orc_spmv(m, x, r.data(), nthreads);
  for (int64_t i = 0; i < N; ++i) r[i] = -1.0 * r[i] + 1.0 * rhs[i];
  rt = r;
  rho = dot(rt.data(), r.data(), N, nthreads);
  if (resid_out) *resid_out = 0.0;
  if (rho == 0) return 0;
  int iter = 0;
  for (; iter < max_iter; ++iter) {
    if (iter == 0) {
      p = r;
    } else {
      rho = dot(rt.data(), r.data(), N, nthreads);
      if (rho == 0) break;
      beta = rho / rho_old * alpha / omega;
      for (int64_t i = 0; i < N; ++i) p[i] = 1.0 * p[i] + -omega * v[i];
      for (int64_t i = 0; i < N; ++i) p[i] = beta * p[i] + 1.0 * r[i];
    }
    orc_spmv(m, p.data(), v.data(), nthreads);
    alpha = dot(rhs, v.data(), N, nthreads);
    alpha = rho / alpha;
    for (int64_t i = 0; i < N; ++i) r[i] = 1.0 * r[i] + -alpha * v[i];
    if ((resid = dot(r.data(), r.data(), N, nthreads)) < rho0 * tol * tol) {
      for (int64_t i = 0; i < N; ++i) x[i] = 1.0 * x[i] + alpha * p[i];
      break;
    }
    orc_spmv(m, r.data(), t.data(), nthreads);
    double tdott = dot(t.data(), t.data(), N, nthreads);
    omega = dot(t.data(), r.data(), N, nthreads) / tdott;
    if (omega == 0.0 || tdott == 0) break;
    for (int64_t i = 0; i < N; ++i) x[i] = 1.0 * x[i] + alpha * p[i];
    for (int64_t i = 0; i < N; ++i) x[i] = 1.0 * x[i] + omega * r[i];
    for (int64_t i = 0; i < N; ++i) r[i] = 1.0 * r[i] + -omega * t[i];
    rho_old = rho;
    resid = dot(r.data(), r.data(), N, nthreads);
    if (resid / rho0 < tol * tol) break;
  }
  if (resid_out) *resid_out = sqrt(resid / rho0);
  return iter;
}

extern "C" int orc_bicgstab(const orc_mesh *m, const double *rhs, double *x, double tol, int max_iter, double *resid_out,
                            int nthreads) {
  const int it = bicgstab_impl(m, rhs, x, tol, max_iter, resid_out, nthreads);
  periodic_copy(m, x);
  return it;
}

static int cg_impl(const orc_mesh *m, const double *rhs, double *x, double tol, int max_iter, double *resid_out,
                   int nthreads) {
  // CG_solve.hpp:54-114, over the rows of the assembled system
  const int64_t N = m->nsolve;
  double rho0, rho, rho_old = 0.0, beta, alpha;
  rho0 = dot(rhs, rhs, N, nthreads);
  std::vector<double> p(N), q(N), r(N);
  orc_spmv(m, x, r.data(), nthreads);
  for (int64_t i = 0; i < N; ++i) r[i] = -1.0 * r[i] + 1.0 * rhs[i];
  rho = dot(r.data(), r.data(), N, nthreads);
  if (resid_out) *resid_out = rho0 > 0 ? sqrt(rho / rho0) : 0.0;
  if (rho == 0) return 0;
  int iter = 0;
  // the vector updates are elementwise: the same result on any thread count
  const int nt = nthr(nthreads);
  for (; iter < max_iter; ++iter) {
    if (iter == 0) {
      p = r;
    } else {
      beta = rho / rho_old;
#pragma omp parallel for num_threads(nt) schedule(static) if (nt > 1)
      for (int64_t i = 0; i < N; ++i) p[i] = beta * p[i] + 1.0 * r[i];
    }
    orc_spmv(m, p.data(), q.data(), nthreads);
    alpha = dot(p.data(), q.data(), N, nthreads);
    alpha = rho / alpha;
#pragma omp parallel for num_threads(nt) schedule(static) if (nt > 1)
    for (int64_t i = 0; i < N; ++i) {
      x[i] = 1.0 * x[i] + alpha * p[i];
      r[i] = 1.0 * r[i] + -alpha * q[i];
    }
    rho_old = rho;
    rho = dot(r.data(), r.data(), N, nthreads);
    if (rho / rho0 < tol * tol) break;
  }
  if (resid_out) *resid_out = sqrt(rho / rho0);
  // number of iterations performed (the loop index at the break, plus one)
  return iter < max_iter ? iter + 1 : iter;
}

extern "C" int orc_cg(const orc_mesh *m, const double *rhs, double *x, double tol, int max_iter, double *resid_out,
                      int nthreads) {
  const int it = cg_impl(m, rhs, x, tol, max_iter, resid_out, nthreads);
  periodic_copy(m, x);
  return it;
}

/* ------------------------------------------------------------------------ */
/* gather: PIC.cpp:162-189                                                   */
extern "C" void orc_efield_tet(const orc_mesh *m, const double *phi, double *E, int nthreads) {
  const int64_t T = m->T;
#pragma omp parallel for num_threads(nthr(nthreads)) schedule(static)
  for (int64_t t = 0; t < T; ++t) {
    const double *G = &m->grad[12 * t];
    for (int dd = 0; dd < 3; ++dd) {
      double s = 0.0;
      for (int i = 0; i < 4; ++i) s += phi[m->tets[4 * t + i]] * G[3 * i + dd];
      E[3 * t + dd] = s;
    }
  }
}

extern "C" void orc_gather(const orc_mesh *m, int mode, int64_t n, const int32_t *cell, const double *xref,
                           const double *phi, const double *E_tet, double *E, int nthreads) {
#pragma omp parallel for num_threads(nthr(nthreads)) schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    int32_t e = cell[p];
    double *Ep = &E[3 * p];
    if (e < 0) {
      Ep[0] = Ep[1] = Ep[2] = 0.0;
      continue;
    }
    if (mode == 1) {
      for (int dd = 0; dd < 3; ++dd) Ep[dd] = E_tet[3 * e + dd];
      continue;
    }
    const double *xr = &xref[3 * p];
    double weights[4] = {1 - xr[0] - xr[1] - xr[2], xr[0], xr[1], xr[2]};  // mesh.hpp:169-176
    double dof[4];
    for (int i = 0; i < 4; ++i) dof[i] = phi[m->tets[4 * e + i]];
    Ep[0] = Ep[1] = Ep[2] = 0.0;
    const double *G = &m->grad[12 * e];
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j)
        for (int dd = 0; dd < 3; ++dd) Ep[dd] += dof[i] * weights[j] * G[3 * i + dd];
  }
}

/* ------------------------------------------------------------------------ */
/* push: particle_move.hpp:364-392 (B = 0 as set by PIC.cpp:179)              */
static inline void jinv_apply(const double *I, const double *a, double *out) {
  // mesh.hpp:244-250
  for (int r = 0; r < 3; ++r) {
    double s = 0.0;
    for (int c = 0; c < 3; ++c) s += I[3 * r + c] * a[c];
    out[r] = s;
  }
}

extern "C" void orc_push(const orc_mesh *m, int64_t n, const int32_t *cell, const double *E, double *v, double *vref,
                         const int32_t *sp, const double *qm, double dt, int nthreads) {
#pragma omp parallel for num_threads(nthr(nthreads)) schedule(static)
  for (int64_t p = 0; p < n; ++p) {
    int32_t e = cell[p];
    if (e < 0) continue;
    const double scaled_dt = dt * 1.0;
    double *vp = &v[3 * p];
    const double *Ep = &E[3 * p];
    const double B[3] = {0.0, 0.0, 0.0};
    const double q_over_m = qm[sp[p]];
    double t[3] = {q_over_m * 0.5 * B[0], q_over_m * 0.5 * B[1], q_over_m * 0.5 * B[2]};
    for (int d = 0; d < 3; ++d) vp[d] += scaled_dt * Ep[d] * q_over_m * 0.5;
    double tmp[3] = {vp[0], vp[1], vp[2]};
    // utils.hpp add_cross: tmp += v x t
    tmp[0] += vp[1] * t[2] - vp[2] * t[1];
    tmp[1] += vp[2] * t[0] - vp[0] * t[2];
    tmp[2] += vp[0] * t[1] - vp[1] * t[0];
    double t_sqr = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
    for (int d = 0; d < 3; ++d) t[d] *= 2. / (1 + t_sqr);
    vp[0] += tmp[1] * t[2] - tmp[2] * t[1];
    vp[1] += tmp[2] * t[0] - tmp[0] * t[2];
    vp[2] += tmp[0] * t[1] - tmp[1] * t[0];
    for (int d = 0; d < 3; ++d) vp[d] += scaled_dt * Ep[d] * q_over_m * 0.5;
    jinv_apply(&m->jinv[9 * e], vp, &vref[3 * p]);
  }
}

/* ------------------------------------------------------------------------ */
/* walk: particle_move.hpp:102-124 (loop) and :135-225 (find_intersection)   */
// returns the fraction of the sub-step used; *killed set when the particle left through an absorbing wall
static inline double find_intersection(const orc_mesh *m, int32_t &e, double *x, double *xr, double *v, double *vr,
                                       double dt, double time_remaining, int kill, bool &killed) {
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
    double fy = -xr[1] / (dlam[1]);
    if (fy < frac) {
      face = 0;
      frac = fy;
    }
  }
  if (vr[0] < 0 && lend[0] < 0) {
    double fx = -xr[0] / (dlam[0]);
    if (fx < frac) {
      face = 2;
      frac = fx;
    }
  }
  double end_sum = lend[0] + lend[1] + lend[2];
  double rate_sum = vr[0] + vr[1] + vr[2];
  if (rate_sum > 0 && end_sum > 1) {
    double fs = (1 - xr[0] - xr[1] - xr[2]) / (dlam[0] + dlam[1] + dlam[2]);
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
    int32_t nb = m->nbrs[4 * e + face];
    if (nb >= 0) {
      // a periodic face wraps x to the other side of the box.  The reference's
      // meshes have mirror-image x faces and it writes x = -x on its [-1,1]
      // box (particle_move.hpp:190-191), i.e. x -> lo + hi - x; a jittered
      // mesh has translated x faces, so x moves by the box length instead.
      if (m->fper[4 * e + face] != 0) {
        const double L = m->d.hi - m->d.lo;
        if (m->d.mapping == 4)
          x[0] = (x[0] + x[0] > m->d.lo + m->d.hi) ? x[0] - L : x[0] + L;
        else
          x[0] = (m->d.lo + m->d.hi) - x[0];
      }
      e = nb;
      // physToReference (mesh.hpp:196-211): ref = 0 + J^-1 (x - x0)
      const double *X0 = &m->nodes[3 * m->tets[4 * e]];
      double delta[3] = {x[0] - X0[0], x[1] - X0[1], x[2] - X0[2]};
      double dref[3];
      jinv_apply(&m->jinv[9 * e], delta, dref);
      for (int d = 0; d < 3; ++d) xr[d] = 0.0 + dref[d];
      jinv_apply(&m->jinv[9 * e], v, vr);
    } else {
      if (kill) {
        killed = true;
        return 1;
      }
      const double *nrm = &m->normals[12 * e + 3 * face];
      double vdn = 0;
      for (int d = 0; d < 3; ++d) vdn += v[d] * nrm[d];
      for (int d = 0; d < 3; ++d) v[d] -= 2 * vdn * nrm[d];
      jinv_apply(&m->jinv[9 * e], v, vr);
    }
  }
  return frac;
}

extern "C" int64_t orc_walk(const orc_mesh *m, int64_t n, int32_t *cell, double *x, double *xref, double *v,
                            double *vref, double dt, int kill, int max_cross, int64_t *n_killed, int64_t *n_cross,
                            int nthreads) {
  int64_t limit_hits = 0, killed_tot = 0, cross_tot = 0;
#pragma omp parallel for num_threads(nthr(nthreads)) schedule(dynamic, 4096) reduction(+ : limit_hits, killed_tot, cross_tot)
  for (int64_t p = 0; p < n; ++p) {
    int32_t e = cell[p];
    if (e < 0) continue;
    double tr = 1.0;  // particles_.set_time_remaining(1.0), particle_move.hpp:77
    int iters = 0;
    bool killed = false;
    while (tr > 0) {
      if (iters >= max_cross) {
        limit_hits++;
        break;
      }
      double s = find_intersection(m, e, &x[3 * p], &xref[3 * p], &v[3 * p], &vref[3 * p], dt, tr, kill, killed);
      tr -= s * tr;
      ++iters;
      if (killed) break;
    }
    cross_tot += iters - 1;
    if (killed) {
      killed_tot++;
      e = -1;
    }
    cell[p] = e;
  }
  if (n_killed) *n_killed = killed_tot;
  if (n_cross) *n_cross = cross_tot;
  return limit_hits;
}

/* ------------------------------------------------------------------------ */
/* compaction                                                                */
extern "C" int64_t orc_compact(int mode, int64_t n, int32_t *cell, double *x, double *xref, double *v, double *w,
                               int32_t *sp, int64_t *id) {
  auto move = [&](int64_t dst, int64_t src) {
    cell[dst] = cell[src];
    for (int d = 0; d < 3; ++d) {
      x[3 * dst + d] = x[3 * src + d];
      xref[3 * dst + d] = xref[3 * src + d];
      v[3 * dst + d] = v[3 * src + d];
    }
    if (w) w[dst] = w[src];
    if (sp) sp[dst] = sp[src];
    if (id) id[dst] = id[src];
  };
  if (mode == 1) {
    int64_t k = 0;
    for (int64_t p = 0; p < n; ++p)
      if (cell[p] >= 0) {
        if (k != p) move(k, p);
        ++k;
      }
    return k;
  }
  // particle_list.cpp:148-191: deleted list in Serial marking order (ascending
  // index), holes below the new count filled from the tail, skipping dead ones
  std::vector<int64_t> deleted;
  for (int64_t p = 0; p < n; ++p)
    if (cell[p] < 0) deleted.push_back(p);
  const int64_t nd = (int64_t)deleted.size();
  const int64_t nnew = n - nd;
  int64_t fill_from = n - 1;
  if (nnew > 0)
    for (int64_t i = 0; i < nd; ++i) {
      int64_t index = deleted[i];
      if (index >= nnew) continue;
      int64_t get_from = fill_from--;
      while (cell[get_from] < 0) get_from = fill_from--;
      move(index, get_from);
    }
  return nnew;
}

/* ------------------------------------------------------------------------ */
/* sort by element                                                           */
/* ParticleList::sort and compute_start_particles_by_element
 * (particle_list.cpp:90-146): the particle list ordered by element.  The
 * reference's Kokkos BinSort is built with sort_within_bins = false
 * (particle_list.cpp:100), which leaves the order inside an element open; here
 * it is the input order (std::stable_sort by element).  Entries with cell < 0
 * (dead) are dropped.  perm[k] = input index of the k-th particle of the
 * sorted list; start[e] = first sorted position whose element is >= e (the
 * bisection of particle_list.cpp:118-133, i.e. lower_bound), start[T] =
 * count.  Returns the count. */
extern "C" int64_t orc_sort_by_cell(int64_t n, const int32_t *cell, int64_t T, int64_t *perm, int64_t *start) {
  std::vector<int64_t> idx;
  idx.reserve(n);
  for (int64_t p = 0; p < n; ++p)
    if (cell[p] >= 0) idx.push_back(p);
  std::stable_sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) { return cell[a] < cell[b]; });
  const int64_t m = (int64_t)idx.size();
  for (int64_t k = 0; k < m; ++k) perm[k] = idx[k];
  if (start) {
    int64_t k = 0;
    for (int64_t e = 0; e <= T; ++e) {
      while (k < m && cell[idx[k]] < e) ++k;
      start[e] = k;
    }
  }
  return m;
}

/* Stable compaction (mode 1) on nt threads: the same order and values as the
 * serial loop.  Each thread stages its chunk's live particles, then writes
 * them at the chunk's offset (the live count of the chunks before it). */
static int64_t compact_stable_par(int64_t n, int32_t *cell, double *x, double *xref, double *v, double *w, int32_t *sp,
                                  int64_t *id, int nt) {
  std::vector<int64_t> cnt(nt + 1, 0);
  struct Stage {
    std::vector<int32_t> cell, sp;
    std::vector<double> x, xref, v, w;
    std::vector<int64_t> id;
  };
  std::vector<Stage> st(nt);
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    const int t = omp_get_thread_num();
#else
    const int t = 0;
#endif
    const int64_t lo = n * t / nt, hi = n * (t + 1) / nt;
    Stage &S = st[t];
    for (int64_t p = lo; p < hi; ++p) {
      if (cell[p] < 0) continue;
      S.cell.push_back(cell[p]);
      for (int d = 0; d < 3; ++d) {
        S.x.push_back(x[3 * p + d]);
        S.xref.push_back(xref[3 * p + d]);
        S.v.push_back(v[3 * p + d]);
      }
      if (w) S.w.push_back(w[p]);
      if (sp) S.sp.push_back(sp[p]);
      if (id) S.id.push_back(id[p]);
    }
    cnt[t + 1] = (int64_t)S.cell.size();
#pragma omp barrier
#pragma omp single
    for (int k = 0; k < nt; ++k) cnt[k + 1] += cnt[k];
    const int64_t o = cnt[t];
    const int64_t m = (int64_t)S.cell.size();
    for (int64_t k = 0; k < m; ++k) {
      cell[o + k] = S.cell[k];
      for (int d = 0; d < 3; ++d) {
        x[3 * (o + k) + d] = S.x[3 * k + d];
        xref[3 * (o + k) + d] = S.xref[3 * k + d];
        v[3 * (o + k) + d] = S.v[3 * k + d];
      }
      if (w) w[o + k] = S.w[k];
      if (sp) sp[o + k] = S.sp[k];
      if (id) id[o + k] = S.id[k];
    }
  }
  return cnt[nt];
}

extern "C" double orc_kinetic(int64_t n, const double *v, const double *w, const int32_t *sp, const double *mass,
                              int nthreads) {
  // PIC.cpp:191-200
  (void)nthreads;
  double sum = 0.0;
  for (int64_t p = 0; p < n; ++p) {
    double tot_m = w[p] * mass[sp[p]];
    double v_sqr = 0;
    for (int d = 0; d < 3; ++d) v_sqr += v[3 * p + d] * v[3 * p + d];
    sum += 0.5 * tot_m * v_sqr;
  }
  return sum;
}

/* ------------------------------------------------------------------------ */
/* fills                                                                     */
static inline void ref_to_phys(const orc_mesh *m, int32_t e, const double *ref, double *phys) {
  // mesh.hpp:182-190
  double w[4] = {1 - ref[0] - ref[1] - ref[2], ref[0], ref[1], ref[2]};
  phys[0] = phys[1] = phys[2] = 0.0;
  for (int i = 0; i < 4; ++i)
    for (int d = 0; d < 3; ++d) phys[d] += w[i] * m->nodes[3 * m->tets[4 * e + i] + d];
}

extern "C" int64_t orc_fill_ref(const orc_mesh *m, int nppe, int type, double density, const double vel[3], double temp,
                                double mass, int64_t capacity, int32_t *cell, double *x, double *xref, double *v,
                                double *w, int32_t *sp) {
  // particle_fill.hpp:59-68 capacity check, :129-164 per-element fill, :100-124 set_vel
  if (capacity < m->T * (int64_t)nppe) return -1;
  const int64_t NG = m->T;
  int64_t k = 0;
  for (int64_t elem = 0; elem < m->T; ++elem) {
    const double vol = m->detj[elem] / 6.;
    const double weight = density * vol / nppe;
    for (uint64_t ipart = 0; ipart < (uint64_t)nppe; ++ipart) {
      RefRand rr;
      rr.s = (uint64_t)elem + (34030 + ipart) * (uint64_t)NG + (uint64_t)(NG * 12345 * (int64_t)type);
      for (int i = 0; i < 10; ++i) rr.rand();
      double xr[3];
      do {
        xr[0] = rr.drand();
        xr[1] = rr.drand();
        xr[2] = rr.drand();
      } while (xr[0] + xr[1] + xr[2] > 1.0);
      double xp[3];
      ref_to_phys(m, (int32_t)elem, xr, xp);
      double vp[3];
      if (temp == 0) {
        vp[0] = vel[0];
        vp[1] = vel[1];
        vp[2] = vel[2];
      } else if (temp < 0) {
        vp[0] = vel[0] * (1. + temp * sin(1. * M_PI * xp[0]));
        vp[1] = vp[2] = 0.0;
      } else {
        do {
          double r = rr.drand();
          double vmax = sqrt(6 * temp / mass);
          double vv[3];
          vv[0] = vmax * 2 * (-.5 + rr.drand());
          vv[1] = vmax * 2 * (-.5 + rr.drand());
          vv[2] = vmax * 2 * (-.5 + rr.drand());
          double prob = exp(-(vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2]) / temp);
          if (r < prob) {
            vp[0] = vel[0] + vv[0];
            vp[1] = vel[1] + vv[1];
            vp[2] = vel[2] + vv[2];
            break;
          }
        } while (true);
      }
      cell[k] = (int32_t)elem;
      for (int d = 0; d < 3; ++d) {
        x[3 * k + d] = xp[d];
        xref[3 * k + d] = xr[d];
        v[3 * k + d] = vp[d];
      }
      w[k] = weight;
      sp[k] = type;
      ++k;
    }
  }
  return k;
}

static inline float f24(uint64_t h) { return (float)(h >> 40) * (1.0f / 16777216.0f); }

extern "C" void orc_fill_uniform(const orc_mesh *m, int64_t n, uint64_t seed, int type, double weight,
                                 const double drift[3], double vth, int32_t *cell, double *x, double *xref, double *v,
                                 double *w, int32_t *sp, int nthreads) {
  // tet chosen uniformly and accepted with probability vol/vol_max (uniform in volume)
  double dmax = 0.0;
  for (int64_t t = 0; t < m->T; ++t) dmax = std::max(dmax, m->detj[t]);
  std::vector<float> ratio(m->T);
  for (int64_t t = 0; t < m->T; ++t) ratio[t] = (float)(m->detj[t] / dmax);
  const uint64_t base = orc_mix64(seed ^ SALT_FILL);
  const uint64_t T = (uint64_t)m->T;
#pragma omp parallel for num_threads(nthr(nthreads)) schedule(static)
  for (int64_t k = 0; k < n; ++k) {
    const uint64_t c0 = (uint64_t)k << 8;
    uint64_t e = 0;
    for (uint64_t j = 0; j < 128; j += 2) {
      e = ((orc_draw(base, c0 | j) >> 32) * T) >> 32;
      if (f24(orc_draw(base, c0 | (j + 1))) < ratio[e]) break;
    }
    float s = f24(orc_draw(base, c0 | 128));
    float t = f24(orc_draw(base, c0 | 129));
    float u = f24(orc_draw(base, c0 | 130));
    // Rocchini & Cignoni (2000): fold the unit cube onto the unit tet
    if (s + t > 1.0f) {
      s = 1.0f - s;
      t = 1.0f - t;
    }
    if (t + u > 1.0f) {
      float tmp = u;
      u = 1.0f - s - t;
      t = 1.0f - tmp;
    } else if (s + t + u > 1.0f) {
      float tmp = u;
      u = s + t + u - 1.0f;
      s = 1.0f - t - tmp;
    }
    // Box-Muller in single precision
    float a0 = f24(orc_draw(base, c0 | 131)), a1 = f24(orc_draw(base, c0 | 132));
    float a2 = f24(orc_draw(base, c0 | 133)), a3 = f24(orc_draw(base, c0 | 134));
    const float twopi = 6.28318530717958648f;
    float r0 = sqrtf(-2.0f * logf(1.0f - a0)), r1 = sqrtf(-2.0f * logf(1.0f - a2));
    float g[3] = {r0 * cosf(twopi * a1), r0 * sinf(twopi * a1), r1 * cosf(twopi * a3)};
    float vf[3];
    for (int d = 0; d < 3; ++d) vf[d] = (float)drift[d] + (float)vth * g[d];
    double xr[3] = {(double)s, (double)t, (double)u};
    double xp[3];
    ref_to_phys(m, (int32_t)e, xr, xp);
    cell[k] = (int32_t)e;
    for (int d = 0; d < 3; ++d) {
      x[3 * k + d] = xp[d];
      xref[3 * k + d] = xr[d];
      v[3 * k + d] = (double)vf[d];
    }
    w[k] = weight;
    sp[k] = type;
  }
}

/* ------------------------------------------------------------------------ */
/* whole step: PIC.cpp:245-267                                               */
extern "C" int orc_step(orc_mesh *m, const orc_step_cfg *c, double dt, int64_t *n, int32_t *cell, double *x,
                        double *xref, double *v, double *vref, double *w, int32_t *sp, int64_t *id, const double *q,
                        const double *mass, const double *bg, double *phi, double *rhs, double *E,
                        orc_step_stats *st) {
  orc_step_stats s;
  memset(&s, 0, sizeof(s));
  int64_t np = *n;
  orc_deposit(m, c->deposit_mode, np, cell, xref, w, sp, q, bg, rhs, c->nthreads);
  if (c->solver == 0) {
    s.solver_iters = orc_bicgstab(m, rhs, phi, c->tol, c->max_iter, &s.solver_resid, c->nthreads);
  } else {
    if (!c->warm_start) std::fill(phi, phi + m->N, 0.0);
    s.solver_iters = orc_cg(m, rhs, phi, c->tol, c->max_iter, &s.solver_resid, c->nthreads);
  }
  std::vector<double> Et;
  if (c->gather_mode == 1) {
    Et.resize(3 * m->T);
    orc_efield_tet(m, phi, Et.data(), c->nthreads);
  }
  orc_gather(m, c->gather_mode, np, cell, xref, phi, Et.data(), E, c->nthreads);
  std::vector<double> qm(16, 0.0);
  for (int i = 0; i < 16; ++i) qm[i] = (mass[i] != 0.0) ? q[i] / mass[i] : 0.0;
  orc_push(m, np, cell, E, v, vref, sp, qm.data(), dt, c->nthreads);
  s.n_walk_limit = orc_walk(m, np, cell, x, xref, v, vref, dt, c->kill, c->max_cross, &s.n_killed, &s.n_cross,
                            c->nthreads);
  if (c->compact_mode == 1 && nthr(c->nthreads) > 1)
    np = compact_stable_par(np, cell, x, xref, v, w, sp, id, nthr(c->nthreads));
  else
    np = orc_compact(c->compact_mode, np, cell, x, xref, v, w, sp, id);
  // compaction does not carry vref: it is recomputed by the next push
  s.ke = orc_kinetic(np, v, w, sp, mass, c->nthreads);
  s.n_alive = np;
  *n = np;
  if (st) *st = s;
  return s.n_walk_limit ? -4 : 0;
}
