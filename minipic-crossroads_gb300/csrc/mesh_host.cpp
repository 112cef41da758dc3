// mesh_host.cpp -- structured tet mesh, connectivity and P1 stiffness assembly.
//
// Host-side setup of the GB300 PIC library (runs once per run, not per step).
// Replaces Mesh::Mesh (mesh.cpp:78-714) and the assembly of ES::ES
// (ES.cpp:83-205) for one rank.  Differences in method, not in result:
//  * face neighbours are found per hex (a tet face either lies inside its hex
//    or on one of the six hex faces, so the partner is among the <= 24 faces
//    of one hex) instead of through a std::multimap of all faces
//    (mesh.cpp:233-405);
//  * the CSR pattern of a row is a 27-bit mask over the {-1,0,1}^3 node
//    offsets of the structured grid, so rows come out sorted without a
//    sort.
// Node numbering (mesh.cpp:52-54), tet tables (mesh.cpp:211-223), face order
// (mesh.cpp:239-250), normals (mesh.cpp:650-669), Jacobians (mesh.cpp:671-700),
// gradients (PIC.cpp:229-241) and the element-order summation of element
// matrices follow the reference so that the arrays are bit-identical to the
// CPU restatement.  Built with -ffp-contract=off.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "mpg_internal.h"

namespace {

inline double unit53(uint64_t u) { return (double)(u >> 11) * (1.0 / 9007199254740992.0); }

void apply_mapping(double &x, double &y, double &z, int mapping) {
  // mesh.cpp:763-792
  double ox = x, oy = y, oz = z;
  if (mapping == 1) {
    double r = (1.0 - fabs(x)) * (1.0 - fabs(y));
    ox = x * cos(r) - y * sin(r);
    oy = x * sin(r) + y * cos(r);
  } else if (mapping == 2) {
    ox = x * sqrt(1 - .5 * y * y - .5 * z * z + y * y * z * z / 3.);
    oy = y * sqrt(1 - .5 * x * x - .5 * z * z + x * x * z * z / 3.);
    oz = z * sqrt(1 - .5 * y * y - .5 * x * x + y * y * x * x / 3.);
  } else if (mapping == 3) {
    ox = x * x;
    if (x < 0) ox = -ox;
  } else {
    return;
  }
  x = ox;
  y = oy;
  z = oz;
}

const int kFaceNodes[4][3] = {{0, 1, 3}, {1, 2, 3}, {0, 3, 2}, {0, 2, 1}};
const int kFaceOfOpposite[4] = {1, 2, 0, 3};  // face index whose opposite vertex is k

}  // namespace

int host_mesh_generate(const mpg_mesh_desc &d, HostMesh &m, std::string &err) {
  if (d.nx < 1 || d.ny < 1 || d.nz < 1) {
    err = "mesh: nx, ny, nz must be >= 1";
    return MPG_ERR_ARG;
  }
  if (d.split != MPG_SPLIT_REF5 && d.split != MPG_SPLIT_KUHN6) {
    err = "mesh: split must be 5 or 6";
    return MPG_ERR_ARG;
  }
  if (!(d.hi > d.lo)) {
    err = "mesh: hi must exceed lo";
    return MPG_ERR_ARG;
  }
  if (d.periodic && d.nx < 2) {
    err = "mesh: a periodic mesh needs nx >= 2";
    return MPG_ERR_ARG;
  }
  if (d.periodic && d.split == MPG_SPLIT_REF5 && d.nx % 2 == 1) {
    // mesh.cpp:91-94: the alternating five-tet split only matches across x for even nx
    err = "mesh: a periodic five-tet mesh needs an even nx";
    return MPG_ERR_ARG;
  }
  const int64_t nx = d.nx, ny = d.ny, nz = d.nz, per = d.split;
  const int64_t N = (nx + 1) * (ny + 1) * (nz + 1), T = per * nx * ny * nz;
  if (N >= (1LL << 31) || T >= (1LL << 31)) {
    err = "mesh: too large for 32-bit indices";
    return MPG_ERR_ARG;
  }
  m = HostMesh();
  m.d = d;
  m.N = N;
  m.T = T;
  const int64_t sj = nz + 1, si = (ny + 1) * (nz + 1);
  const double dx = (d.hi - d.lo) / nx, dy = (d.hi - d.lo) / ny, dz = (d.hi - d.lo) / nz;
  m.nodes.resize(N * 3);
  m.bnd.assign(N, 0);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i <= nx; ++i)
    for (int64_t j = 0; j <= ny; ++j)
      for (int64_t k = 0; k <= nz; ++k) {
        int64_t g = i * si + j * sj + k;
        m.nodes[3 * g + 0] = d.lo + i * dx;
        m.nodes[3 * g + 1] = d.lo + j * dy;
        m.nodes[3 * g + 2] = d.lo + k * dz;
        // a periodic mesh has no x walls (mesh.cpp:407-412)
        m.bnd[g] = ((!d.periodic && (i == 0 || i == nx)) || j == 0 || j == ny || k == 0 || k == nz) ? 1 : 0;
      }
  int64_t nb = 0;
  for (int64_t g = 0; g < N; ++g) nb += m.bnd[g];
  m.n_bnodes = nb;
  // periodic node pairs (mesh.cpp:178-189): interior nodes of the x = hi plane
  m.pair.assign(N, -1);
  if (d.periodic)
    for (int64_t j = 1; j < ny; ++j)
      for (int64_t k = 1; k < nz; ++k) m.pair[nx * si + j * sj + k] = (int32_t)(j * sj + k);
  m.nsolve = d.periodic ? N - si : N;

  // ---- tets, hex by hex in (i, j, k) order
  m.tets.resize(T * 4);
  static const int kOdd[5][4] = {{3, 1, 0, 5}, {6, 4, 5, 0}, {6, 2, 0, 3}, {5, 7, 6, 3}, {5, 6, 0, 3}};
  static const int kEven[5][4] = {{2, 3, 1, 7}, {7, 6, 4, 2}, {2, 0, 4, 1}, {4, 5, 7, 1}, {2, 4, 7, 1}};
  // Kuhn: tet (0, e_a, e_a+e_b, 1) for each axis order (a,b,c); corner bit of x=4, y=2, z=1;
  // odd orders swap the last two vertices so that detJ > 0.
  static const int kKuhn[6][4] = {{0, 4, 6, 7}, {0, 4, 7, 5}, {0, 2, 7, 6}, {0, 2, 3, 7}, {0, 1, 5, 7}, {0, 1, 7, 3}};
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < nx; ++i)
    for (int64_t j = 0; j < ny; ++j)
      for (int64_t k = 0; k < nz; ++k) {
        const int64_t base = i * si + j * sj + k;
        // corner c = 4*di + 2*dj + dk  (mesh.cpp:200-208 ordering)
        int32_t c[8];
        for (int q = 0; q < 8; ++q) c[q] = (int32_t)(base + ((q >> 2) & 1) * si + ((q >> 1) & 1) * sj + (q & 1));
        const int64_t h = (i * ny + j) * nz + k;
        const int(*tab)[4] = (per == 6) ? kKuhn : (((i + j + k) % 2 != 0) ? kOdd : kEven);
        for (int t = 0; t < per; ++t)
          for (int q = 0; q < 4; ++q) m.tets[4 * (h * per + t) + q] = c[tab[t][q]];
      }

  // ---- face neighbours, per hex.  On a periodic mesh a face on the x = hi
  // plane is renamed onto the x = lo plane (Mesh::periodic_face,
  // mesh.cpp:61-76), so the hexes at the two ends of x are neighbours.
  m.nbrs.assign(T * 4, -1);
  m.fper.assign(T * 4, 0);
  const int32_t ghost_shift = (int32_t)(nx * si);
  auto face_key = [&](const int32_t *g3, int32_t key[3]) {
    bool hi_plane = d.periodic != 0;
    for (int q = 0; q < 3; ++q) hi_plane = hi_plane && g3[q] / si == nx;
    for (int q = 0; q < 3; ++q) key[q] = hi_plane ? g3[q] - ghost_shift : g3[q];
    std::sort(key, key + 3);
  };
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
  for (int64_t t = 0; t < T; ++t) {
    const int64_t h = t / per;
    const int64_t hi_ = h / (ny * nz), hj = (h / nz) % ny, hk = h % nz;
    const int64_t corner = hi_ * si + hj * sj + hk;
    for (int f = 0; f < 4; ++f) {
      int32_t key[3], g3[3];
      int all[3][2] = {{1, 1}, {1, 1}, {1, 1}};  // [axis][offset 0/1] all nodes share it
      for (int q = 0; q < 3; ++q) {
        int32_t g = m.tets[4 * t + kFaceNodes[f][q]];
        g3[q] = g;
        int64_t r = g - corner;
        int di = (int)(r / si), dj = (int)((r % si) / sj), dk = (int)(r % sj);
        int off[3] = {di, dj, dk};
        for (int a = 0; a < 3; ++a) {
          all[a][0] &= (off[a] == 0);
          all[a][1] &= (off[a] == 1);
        }
      }
      face_key(g3, key);
      int64_t nh[3] = {hi_, hj, hk};
      const int64_t lim[3] = {nx, ny, nz};
      bool wall = false;
      for (int a = 0; a < 3; ++a) {
        const bool wrap = a == 0 && d.periodic;
        if (all[a][0]) {
          if (nh[a] == 0) {
            if (wrap) {
              nh[a] = lim[a] - 1;
              m.fper[4 * t + f] = 1;  // mesh.cpp:369-378
            } else {
              wall = true;
            }
          } else {
            nh[a] -= 1;
          }
        } else if (all[a][1]) {
          if (nh[a] == lim[a] - 1) {
            if (wrap) {
              nh[a] = 0;
              m.fper[4 * t + f] = 1;
            } else {
              wall = true;
            }
          } else {
            nh[a] += 1;
          }
        }
      }
      if (wall) {
        m.nbrs[4 * t + f] = -1;
        continue;
      }
      const int64_t h2 = (nh[0] * ny + nh[1]) * nz + nh[2];
      int32_t found = -1;
      for (int64_t t2 = h2 * per; t2 < (h2 + 1) * per && found < 0; ++t2) {
        if (t2 == t) continue;
        for (int f2 = 0; f2 < 4; ++f2) {
          const int32_t c3[3] = {m.tets[4 * t2 + kFaceNodes[f2][0]], m.tets[4 * t2 + kFaceNodes[f2][1]],
                                 m.tets[4 * t2 + kFaceNodes[f2][2]]};
          int32_t k2[3];
          face_key(c3, k2);
          if (k2[0] == key[0] && k2[1] == key[1] && k2[2] == key[2]) {
            found = (int32_t)t2;
            break;
          }
        }
      }
      if (found < 0) ++bad;
      m.nbrs[4 * t + f] = found;
    }
  }
  if (bad) {
    err = "mesh: unmatched interior face (non-conforming split)";
    return MPG_ERR_MESH;
  }

  // ---- node mapping / jitter (mesh.cpp:587-588)
  if (d.mapping >= 1 && d.mapping <= 3) {
    for (int64_t g = 0; g < N; ++g) apply_mapping(m.nodes[3 * g], m.nodes[3 * g + 1], m.nodes[3 * g + 2], d.mapping);
  } else if (d.mapping == MPG_MAP_JITTER) {
    const uint64_t base = mpg_mix64(d.seed ^ MPG_SALT_JITTER);
    const double h3[3] = {dx, dy, dz};
#pragma omp parallel for schedule(static)
    for (int64_t g = 0; g < N; ++g) {
      if (m.bnd[g]) continue;
      // a ghost node moves with its pair: the x = hi face is the x = lo face
      // translated by the box length (the periodic crossing is a translation)
      const uint64_t src = (uint64_t)host_pmap(m, (int32_t)g);
      for (int q = 0; q < 3; ++q) {
        double u = unit53(mpg_mix64(base + mpg_mix64(3 * src + q)));
        m.nodes[3 * g + q] += (2.0 * u - 1.0) * d.jitter * h3[q];
      }
    }
  } else if (d.mapping != MPG_MAP_NONE) {
    err = "mesh: unknown mapping";
    return MPG_ERR_ARG;
  }

  // ---- per-tet geometry
  m.normals.resize(T * 12);
  m.jinv.resize(T * 9);
  m.detj.resize(T);
  m.grad.resize(T * 12);
  static const double ghat[4][3] = {{-1, -1, -1}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  int nonpos = 0;
#pragma omp parallel for schedule(static) reduction(+ : nonpos)
  for (int64_t t = 0; t < T; ++t) {
    const double *X[4];
    for (int q = 0; q < 4; ++q) X[q] = &m.nodes[3 * m.tets[4 * t + q]];
    for (int f = 0; f < 4; ++f) {
      const double *A = X[kFaceNodes[f][0]], *B = X[kFaceNodes[f][1]], *C = X[kFaceNodes[f][2]];
      const double v1[3] = {A[0] - B[0], A[1] - B[1], A[2] - B[2]};
      const double v2[3] = {C[0] - B[0], C[1] - B[1], C[2] - B[2]};
      const double n[3] = {v2[1] * v1[2] - v2[2] * v1[1], v2[2] * v1[0] - v2[0] * v1[2],
                           v2[0] * v1[1] - v2[1] * v1[0]};
      const double fac = 1. / sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      for (int q = 0; q < 3; ++q) m.normals[12 * t + 3 * f + q] = n[q] * fac;
    }
    double J[3][3];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) J[r][c] = X[c + 1][r] - X[0][r];
    const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                       J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                       J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    if (!(det > 0)) ++nonpos;
    double *I = &m.jinv[9 * t];
    I[0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
    I[1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    I[2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
    I[3] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
    I[4] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
    I[5] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    I[6] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
    I[7] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    I[8] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    m.detj[t] = det;
    for (int i = 0; i < 4; ++i)
      for (int dd = 0; dd < 3; ++dd) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s += I[3 * k + dd] * ghat[i][k];
        m.grad[12 * t + 3 * i + dd] = s;
      }
  }
  if (nonpos) {
    err = "mesh: non-positive Jacobian determinant (mesh.cpp:692)";
    return MPG_ERR_MESH;
  }

  // ---- neighbour + vertex permutation per face, indexed by opposite vertex
  auto xmap = [&](int32_t g) -> int32_t { return (d.periodic && g / si == nx) ? g - ghost_shift : g; };
  m.nbr_opp.resize(T * 4);
#pragma omp parallel for schedule(static)
  for (int64_t t = 0; t < T; ++t)
    for (int k = 0; k < 4; ++k) {
      int32_t b = m.nbrs[4 * t + kFaceOfOpposite[k]];
      if (b < 0) {
        m.nbr_opp[4 * t + k] = 0xFFFFFFu;
        continue;
      }
      uint32_t perm = 0;
      int used = 0;
      for (int j = 0; j < 4; ++j) {
        if (j == k) continue;
        // across a periodic face a vertex of the x = hi plane is the vertex
        // with the same (j, k) on the x = lo plane -- every such vertex, the
        // ones on the y/z walls included (Mesh::periodic_face, mesh.cpp:61-76),
        // not only the ES node pairs
        const int32_t g = xmap(m.tets[4 * t + j]);
        int pos = 0;
        while (pos < 3 && xmap(m.tets[4 * (int64_t)b + pos]) != g) ++pos;
        perm |= (uint32_t)pos << (2 * j);
        used |= 1 << pos;
      }
      int miss = 0;
      while (used & (1 << miss)) ++miss;
      perm |= (uint32_t)miss << (2 * k);
      m.nbr_opp[4 * t + k] = (perm << 24) | ((uint32_t)b & 0xFFFFFFu);
    }
  return MPG_OK;
}

// Periodic meshes: rows and columns go through the node pairs (ES.cpp:93-95,
// 168-176).  Mode 0 keeps all N rows, a ghost row being -phi_ghost + phi_pair
// = 0 (ES.cpp:183-189); mode 1 keeps the nsolve rows of the x < hi planes.
// Columns sorted per row, element-order sums, as the oracle.
static void csr_assemble_periodic(const HostMesh &m, int mode, std::vector<int32_t> &rowptr,
                                  std::vector<int32_t> &col, std::vector<double> &val) {
  const int64_t T = m.T;
  const int64_t R = mode == 1 ? m.nsolve : m.N;
  std::vector<std::vector<int32_t>> cols(R);
  for (int64_t t = 0; t < T; ++t)
    for (int a = 0; a < 4; ++a) {
      const int32_t r = host_pmap(m, m.tets[4 * t + a]);
      if (m.bnd[r]) continue;
      for (int b = 0; b < 4; ++b) {
        const int32_t c = host_pmap(m, m.tets[4 * t + b]);
        if (mode == 1 && m.bnd[c]) continue;
        cols[r].push_back(c);
      }
    }
  rowptr.assign(R + 1, 0);
  for (int64_t r = 0; r < R; ++r) {
    if (m.bnd[r]) {
      cols[r].assign(1, (int32_t)r);
    } else if (m.pair[r] >= 0) {
      cols[r] = {m.pair[r], (int32_t)r};
    } else {
      std::sort(cols[r].begin(), cols[r].end());
      cols[r].erase(std::unique(cols[r].begin(), cols[r].end()), cols[r].end());
    }
    rowptr[r + 1] = rowptr[r] + (int32_t)cols[r].size();
  }
  col.resize(rowptr[R]);
  val.assign(rowptr[R], 0.0);
  for (int64_t r = 0; r < R; ++r) std::copy(cols[r].begin(), cols[r].end(), col.begin() + rowptr[r]);
  const double wcub = 1.0 / 24.0;
  for (int64_t t = 0; t < T; ++t) {
    const double *G = &m.grad[12 * t];
    const double wm = m.detj[t] * wcub;
    for (int a = 0; a < 4; ++a) {
      const int32_t r = host_pmap(m, m.tets[4 * t + a]);
      if (m.bnd[r]) continue;
      for (int b = 0; b < 4; ++b) {
        const int32_t c = host_pmap(m, m.tets[4 * t + b]);
        if (mode == 1 && m.bnd[c]) continue;
        double k = 0.0;
        for (int cub = 0; cub < 4; ++cub)
          for (int dd = 0; dd < 3; ++dd) k += G[3 * a + dd] * (wm * G[3 * b + dd]);
        const int32_t *p = std::lower_bound(&col[rowptr[r]], &col[0] + rowptr[r + 1], c);
        val[p - col.data()] += k;
      }
    }
  }
  for (int64_t r = 0; r < R; ++r) {
    if (m.bnd[r]) val[rowptr[r]] = 1.0;
    if (m.pair[r] >= 0) {
      val[rowptr[r]] = 1.0;
      val[rowptr[r] + 1] = -1.0;
    }
  }
}

void host_csr_assemble(const HostMesh &m, int mode, std::vector<int32_t> &rowptr, std::vector<int32_t> &col,
                       std::vector<double> &val) {
  if (m.d.periodic) {
    csr_assemble_periodic(m, mode, rowptr, col, val);
    return;
  }
  const int64_t N = m.N, T = m.T;
  const int64_t nz = m.d.nz, ny = m.d.ny;
  const int64_t sj = nz + 1, si = (ny + 1) * (nz + 1);
  auto offset_index = [&](int32_t r, int32_t c) -> int {
    // (di,dj,dk) in {-1,0,1}^3 between structured grid nodes
    int64_t ri = r / si, rj = (r % si) / sj, rk = r % sj;
    int64_t ci = c / si, cj = (c % si) / sj, ck = c % sj;
    return (int)((ci - ri + 1) * 9 + (cj - rj + 1) * 3 + (ck - rk + 1));
  };
  auto delta = [&](int o) -> int64_t { return (o / 9 - 1) * si + ((o / 3) % 3 - 1) * sj + (o % 3 - 1); };
  // rows are assembled in parallel, each from the (tet, corner) pairs that
  // use its node, in tet order: every entry sums its element contributions in
  // the order of the element loop (ES.cpp:83-213), so the values are those of
  // the sequential assembly bit for bit
  std::vector<int32_t> off, c2n;
  host_charge_slots(m, off, c2n);
  std::vector<int32_t> inc(4 * T);
  for (int64_t q = 0; q < 4 * T; ++q) inc[c2n[q]] = (int32_t)q;
  std::vector<uint32_t> mask(N, 0);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t r = 0; r < N; ++r) {
    if (m.bnd[r]) {
      mask[r] = 1u << 13;
      continue;
    }
    uint32_t mk = 0;
    for (int32_t q = off[r]; q < off[r + 1]; ++q) {
      const int64_t t = inc[q] >> 2;
      for (int b = 0; b < 4; ++b) {
        int32_t c = m.tets[4 * t + b];
        if (mode == 1 && m.bnd[c]) continue;
        mk |= 1u << offset_index((int32_t)r, c);
      }
    }
    mask[r] = mk;
  }
  rowptr.assign(N + 1, 0);
  for (int64_t r = 0; r < N; ++r) rowptr[r + 1] = rowptr[r] + __builtin_popcount(mask[r]);
  col.resize(rowptr[N]);
  val.assign(rowptr[N], 0.0);
#pragma omp parallel for schedule(static)
  for (int64_t r = 0; r < N; ++r) {
    int32_t p = rowptr[r];
    for (int o = 0; o < 27; ++o)
      if (mask[r] & (1u << o)) col[p++] = (int32_t)(r + delta(o));
  }
  const double wcub = 1.0 / 24.0;
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t r = 0; r < N; ++r) {
    if (m.bnd[r]) {
      val[rowptr[r]] = 1.0;
      continue;
    }
    for (int32_t q = off[r]; q < off[r + 1]; ++q) {
      const int64_t t = inc[q] >> 2;
      const int a = inc[q] & 3;
      const double *G = &m.grad[12 * t];
      const double wm = m.detj[t] * wcub;
      for (int b = 0; b < 4; ++b) {
        int32_t c = m.tets[4 * t + b];
        if (mode == 1 && m.bnd[c]) continue;
        double k = 0.0;
        for (int cub = 0; cub < 4; ++cub)
          for (int dd = 0; dd < 3; ++dd) k += G[3 * a + dd] * (wm * G[3 * b + dd]);
        int o = offset_index((int32_t)r, c);
        val[rowptr[r] + __builtin_popcount(mask[r] & ((1u << o) - 1u))] += k;
      }
    }
  }
}

void host_background(const HostMesh &m, double rho_bg, std::vector<double> &bg) {
  bg.assign(m.N, 0.0);
  for (int64_t t = 0; t < m.T; ++t) {
    const double q = -(rho_bg * (m.detj[t] / 6.0)) * 0.25;
    for (int a = 0; a < 4; ++a) bg[host_pmap(m, m.tets[4 * t + a])] += q;
  }
  for (int64_t i = 0; i < m.N; ++i)
    if (m.bnd[i]) bg[i] = 0.0;
}

void host_fill_ratio(const HostMesh &m, std::vector<float> &ratio) {
  double dmax = 0.0;
  for (int64_t t = 0; t < m.T; ++t) dmax = std::max(dmax, m.detj[t]);
  ratio.resize(m.T);
  for (int64_t t = 0; t < m.T; ++t) ratio[t] = (float)(m.detj[t] / dmax);
}

void host_charge_slots(const HostMesh &m, std::vector<int32_t> &off, std::vector<int32_t> &c2n) {
  off.assign(m.N + 1, 0);
  c2n.resize(4 * m.T);
  for (int64_t t = 0; t < m.T; ++t)
    for (int k = 0; k < 4; ++k) ++off[m.tets[4 * t + k] + 1];
  for (int64_t i = 0; i < m.N; ++i) off[i + 1] += off[i];
  std::vector<int32_t> fill(off.begin(), off.end() - 1);
  for (int64_t t = 0; t < m.T; ++t)
    for (int k = 0; k < 4; ++k) c2n[4 * t + k] = fill[m.tets[4 * t + k]]++;
}

bool host_kuhn_table(const HostMesh &m, float jinv[6][9], uint32_t face[6][4], int32_t noff[6][4]) {
  const mpg_mesh_desc &d = m.d;
  if (d.split != MPG_SPLIT_KUHN6 || d.mapping != MPG_MAP_NONE || d.periodic) return false;
  const int64_t nx = d.nx, ny = d.ny, nz = d.nz;
  if (nx < 3 || ny < 3 || nz < 3 || m.T != 6 * nx * ny * nz) return false;
  // reference hex (1, 1, 1): all its face neighbours are interior tets
  const int64_t h0 = (1 * ny + 1) * nz + 1;
  for (int k = 0; k < 6; ++k) {
    const int64_t t = 6 * h0 + k;
    for (int q = 0; q < 9; ++q) jinv[k][q] = (float)m.jinv[9 * t + q];
    for (int v = 0; v < 4; ++v) {
      const uint32_t w = m.nbr_opp[4 * t + v];
      const uint32_t nb = w & 0xFFFFFFu;
      if (nb == 0xFFFFFFu) return false;
      const int64_t h = nb / 6, di = h / (ny * nz) - 1, dj = (h / nz) % ny - 1, dk = h % nz - 1;
      if (di < -1 || di > 1 || dj < -1 || dj > 1 || dk < -1 || dk > 1) return false;
      face[k][v] = (uint32_t)(di + 1) | (uint32_t)(dj + 1) << 2 | (uint32_t)(dk + 1) << 4 | (nb % 6) << 8 |
                   (w >> 24) << 16;
    }
  }
  // the corner (x = 4, y = 2, z = 1) of each local vertex, to check the node
  // numbering of every tet as well
  const int64_t si = (ny + 1) * (nz + 1), sj = nz + 1;
  const int64_t base0 = 1 * si + 1 * sj + 1;
  int corner[6][4];
  for (int k = 0; k < 6; ++k)
    for (int q = 0; q < 4; ++q) {
      const int64_t r = m.tets[4 * (6 * h0 + k) + q] - base0;
      const int64_t di = r / si, dj = (r % si) / sj, dk = r % sj;
      if (r < 0 || di > 1 || dj > 1 || dk > 1) return false;
      corner[k][q] = (int)(4 * di + 2 * dj + dk);
      noff[k][q] = (int32_t)(di * si + dj * sj + dk);
    }
  // the per-hex E-field pass relies on vertex 0 of every type being the
  // hex's first node
  for (int k = 0; k < 6; ++k)
    if (corner[k][0] != 0) return false;
  // every tet must match its type's entries bit for bit
  int bad = 0;
#pragma omp parallel for schedule(static) reduction(+ : bad)
  for (int64_t t = 0; t < m.T; ++t) {
    const int k = (int)(t % 6);
    for (int q = 0; q < 9; ++q)
      if ((float)m.jinv[9 * t + q] != jinv[k][q]) ++bad;
    const int64_t h = t / 6, i = h / (ny * nz), j = (h / nz) % ny, kk = h % nz;
    const int64_t base = i * si + j * sj + kk;
    for (int q = 0; q < 4; ++q) {
      const int c = corner[k][q];
      if (m.tets[4 * t + q] != base + (c >> 2) * si + ((c >> 1) & 1) * sj + (c & 1)) ++bad;
    }
    for (int v = 0; v < 4; ++v) {
      const uint32_t f = face[k][v];
      const int64_t ni = i + (int64_t)(f & 3) - 1, nj = j + (int64_t)((f >> 2) & 3) - 1,
                    nk = kk + (int64_t)((f >> 4) & 3) - 1;
      uint32_t want;
      if (ni < 0 || ni >= nx || nj < 0 || nj >= ny || nk < 0 || nk >= nz)
        want = 0xFFFFFFu;
      else
        want = ((f >> 16) << 24) | (uint32_t)(6 * ((ni * ny + nj) * nz + nk) + ((f >> 8) & 0xFF));
      const uint32_t got = m.nbr_opp[4 * t + v];
      // a wall carries no permutation
      if ((got & 0xFFFFFFu) == 0xFFFFFFu ? want != 0xFFFFFFu : got != want) ++bad;
    }
  }
  return bad == 0;
}
