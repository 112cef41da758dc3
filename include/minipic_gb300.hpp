// minipic_gb300.hpp -- the reference's C++ classes, re-hosted on the GB300 C ABI.
//
// Header-only.  Same class names, methods and argument meanings as MiniPIC's
// DataWarehouse (data_warehouse.hpp:51-90), Mesh (mesh.hpp:59-267),
// ParticleList (particle_list.hpp:54-320), ParticleTypeList
// (particle_type.hpp:58-86), ParticleFill (particle_fill.hpp:53-68), ES
// (ES.hpp:48-116), PIC (PIC.hpp:54-106) and ParticleMove
// (particle_move.hpp:53-436), so a driver written against the reference
// (main.cpp:58-153) compiles against this with the include changed.  All
// state lives on the GPU behind one mpg_ctx; accessors that the reference
// serves from host-visible Views (x(i), v(i), nodes(i), ...) read a host
// snapshot that is refreshed on demand.  Errors the reference asserts on
// throw std::runtime_error here; ParticleFill keeps the reference's
// print-and-skip behaviour on over-capacity (particle_fill.hpp:61-64).
#pragma once

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "minipic_gb300.h"

namespace mpg {

typedef double FLOAT;   // types.hpp:52
typedef int LO;         // types.hpp:48
typedef long GO;        // types.hpp:49
typedef std::array<double, 3> VECTOR;

inline void check(mpg_ctx *c, int rc, const char *what) {
  if (rc != MPG_OK) {
    char buf[512];
    mpg_last_error(c, buf, sizeof(buf));
    throw std::runtime_error(std::string(what) + ": " + buf);
  }
}

// shared device context (the reference shares ref-counted Kokkos Views)
struct Context {
  mpg_ctx *ctx = nullptr;
  mpg_config cfg{};
  bool configured = false;
  explicit Context(int device = 0) {
    int rc = mpg_ctx_create(device, &ctx);
    if (rc) {
      char buf[512];
      mpg_last_error(nullptr, buf, sizeof(buf));
      throw std::runtime_error(std::string("mpg_ctx_create: ") + buf);
    }
    cfg.precision = MPG_PLAIN;
    cfg.deposit = MPG_DEPOSIT_REF_QUARTER;
    cfg.solver = MPG_SOLVER_BICGSTAB;
    cfg.tol = 1e-6;
    cfg.max_iter = 1000;
    cfg.max_crossings = 1000;
  }
  ~Context() { mpg_ctx_destroy(ctx); }
  Context(const Context &) = delete;
  Context &operator=(const Context &) = delete;
  void configure() {
    check(ctx, mpg_configure(ctx, &cfg), "mpg_configure");
    configured = true;
  }
};

class ParticleType {  // particle_type.hpp:44-54
 public:
  FLOAT q, m, q_over_m;
  ParticleType(FLOAT q_ = -1, FLOAT m_ = 1) : q(q_), m(m_), q_over_m(q_ / m_) {}
};

class ParticleTypeList {  // particle_type.hpp:58-86
 public:
  ParticleTypeList() {
    types_ = {ParticleType(-1, 1), ParticleType(1, 1), ParticleType(1, 1837)};
    names_ = {"e-", "e+", "H+"};
  }
  void add_particle_type(const ParticleType t, const std::string &name) {
    types_.push_back(t);
    names_.push_back(name);
    if (ctx_) push(ctx_);
  }
  ParticleType &particle_info(int i) { return types_.at(i); }
  int count() const { return (int)types_.size(); }
  void push(std::shared_ptr<Context> c) {
    ctx_ = c;
    for (int i = 0; i < (int)types_.size(); ++i)
      check(c->ctx, mpg_species_set(c->ctx, i, types_[i].q, types_[i].m), "mpg_species_set");
  }

 private:
  std::vector<ParticleType> types_;
  std::vector<std::string> names_;
  std::shared_ptr<Context> ctx_;
};

class Mesh {  // mesh.hpp:59-267 (single rank; node/elem gids == lids)
 public:
  LO num_elems = 0, num_nodes = 0, num_owned_nodes = 0;
  GO num_global_elems = 0;
  int num_nodes_per_elem = 4, num_faces_per_elem = 4, num_nodes_per_face = 3, dimension = 3;
  bool is_periodic = false;

  Mesh() = default;
  Mesh(std::shared_ptr<Context> c, const mpg_mesh_desc &d) : ctx_(c), desc_(d) {
    check(c->ctx, mpg_mesh_build(c->ctx, &d), "mpg_mesh_build");
    int64_t T, N, nb;
    check(c->ctx, mpg_mesh_sizes(c->ctx, &T, &N, &nb), "mpg_mesh_sizes");
    num_elems = (LO)T;
    num_global_elems = T;
    num_nodes = num_owned_nodes = (LO)N;
    nodes_.resize(3 * N);
    tets_.resize(4 * T);
    nbrs_.resize(4 * T);
    jinv_.resize(9 * T);
    detj_.resize(T);
    normals_.resize(12 * T);
    bnd_.resize(N);
    check(c->ctx, mpg_mesh_download(c->ctx, nodes_.data(), tets_.data(), nbrs_.data(), jinv_.data(), detj_.data(),
                                    normals_.data(), bnd_.data()),
          "mpg_mesh_download");
    is_periodic = d.periodic != 0;
    fper_.resize(4 * T);
    pairs_.resize(N);
    check(c->ctx, mpg_mesh_periodic_download(c->ctx, fper_.data(), pairs_.data()), "mpg_mesh_periodic_download");
  }
  // mesh.hpp:149-154 (periodic meshes): +1 on both sides of an x face, and
  // the x = lo node a ghost node of the x = hi plane stands for (-1 otherwise)
  int elem_face_periodic(LO e, int f) const { return fper_[4 * e + f]; }
  GO node_pairs(LO i) const { return pairs_[i]; }
  VECTOR nodes(LO i) const { return {nodes_[3 * i], nodes_[3 * i + 1], nodes_[3 * i + 2]}; }
  LO elem_to_node_lids(LO e, int i) const { return tets_[4 * e + i]; }
  GO elem_to_node_gids(LO e, int i) const { return tets_[4 * e + i]; }
  GO elem_face_to_elem_gids(LO e, int f) const { return nbrs_[4 * e + f]; }
  FLOAT determinate_jacobian(LO e) const { return detj_[e]; }
  FLOAT inverse_jacobian(LO e, int /*node*/, int i, int j) const { return jinv_[9 * e + 3 * i + j]; }
  VECTOR normals(LO e, int f) const {
    return {normals_[12 * e + 3 * f], normals_[12 * e + 3 * f + 1], normals_[12 * e + 3 * f + 2]};
  }
  bool is_boundary_node(LO i) const { return bnd_[i] != 0; }
  // mesh.hpp:169-176
  void getWeights(FLOAT *w, const VECTOR &ref) const {
    w[0] = 1 - ref[0] - ref[1] - ref[2];
    w[1] = ref[0];
    w[2] = ref[1];
    w[3] = ref[2];
  }
  // mesh.hpp:182-190
  void refToPhysical(VECTOR &phys, const VECTOR &ref, LO e) const {
    FLOAT w[4];
    getWeights(w, ref);
    phys = {0.0, 0.0, 0.0};
    for (int i = 0; i < 4; ++i)
      for (int d = 0; d < 3; ++d) phys[d] += w[i] * nodes_[3 * tets_[4 * e + i] + d];
  }
  // mesh.hpp:244-250
  void physToReferenceVector(VECTOR &ref_vec, const VECTOR &phys_vec, const VECTOR &, LO e) const {
    for (int i = 0; i < 3; ++i) {
      double s = 0.0;
      for (int j = 0; j < 3; ++j) s += jinv_[9 * e + 3 * i + j] * phys_vec[j];
      ref_vec[i] = s;
    }
  }
  // mesh.hpp:196-211
  void physToReference(VECTOR &ref, const VECTOR &phys, LO e) const {
    const LO n0 = tets_[4 * e];
    VECTOR delta = {phys[0] - nodes_[3 * n0], phys[1] - nodes_[3 * n0 + 1], phys[2] - nodes_[3 * n0 + 2]};
    VECTOR r;
    physToReferenceVector(r, delta, ref, e);
    ref = {0.0 + r[0], 0.0 + r[1], 0.0 + r[2]};
  }
  bool isPhysicalInElement(const VECTOR &phys, LO e) const {
    VECTOR ref;
    physToReference(ref, phys, e);
    return ref[0] >= 0 && ref[1] >= 0 && ref[2] >= 0 && ref[0] + ref[1] + ref[2] <= 1;
  }
  // Mesh::dump_data (mesh.cpp:794-910), one rank (file suffix 000): nodes,
  // elems, faces, edges, owned faces and edges, boundary faces and edges.
  // Faces and edges carry the reference's gids: their sorted node-gid tuples
  // in lexicographic order (mesh.cpp:271-303; on a periodic mesh a face on
  // the x = nx node plane is renamed to the x = 0 plane first, mesh.cpp:61-76;
  // edges are not renamed).  A face (edge) is on the boundary when the mean
  // of its node coordinates, mapped onto [-1,1], is within 1e-8 of -1 or +1
  // in some axis (mesh.cpp:602-625).  Numbers go out with the stream's
  // default precision, like the reference's.
  void dump_data() const {
    std::ofstream out("nodes-000.dat");
    for (LO i = 0; i < num_nodes; ++i)
      out << i << ' ' << nodes_[3 * i] << ' ' << nodes_[3 * i + 1] << ' ' << nodes_[3 * i + 2] << " \n";
    std::ofstream oe("elems-000.dat");
    for (LO e = 0; e < num_elems; ++e) {
      oe << e << ' ';
      for (int i = 0; i < 4; ++i) oe << tets_[4 * e + i] << ' ';
      oe << '\n';
    }
    const int64_t plane = (int64_t)(desc_.ny + 1) * (desc_.nz + 1);
    static const int fn[4][3] = {{0, 1, 3}, {1, 2, 3}, {0, 3, 2}, {0, 2, 1}};
    std::vector<std::array<int64_t, 3>> faces;
    faces.reserve(4 * (size_t)num_elems);
    for (LO e = 0; e < num_elems; ++e)
      for (int f = 0; f < 4; ++f) {
        std::array<int64_t, 3> t = {tets_[4 * e + fn[f][0]], tets_[4 * e + fn[f][1]], tets_[4 * e + fn[f][2]]};
        if (is_periodic && t[0] / plane == desc_.nx && t[1] / plane == desc_.nx && t[2] / plane == desc_.nx)
          for (auto &g : t) g -= (int64_t)desc_.nx * plane;
        std::sort(t.begin(), t.end());
        faces.push_back(t);
      }
    std::sort(faces.begin(), faces.end());
    faces.erase(std::unique(faces.begin(), faces.end()), faces.end());
    std::vector<std::array<int64_t, 2>> edges;
    edges.reserve(6 * (size_t)num_elems);
    for (LO e = 0; e < num_elems; ++e)
      for (int j = 0; j < 3; ++j)
        for (int k = j + 1; k < 4; ++k) {
          int64_t a = tets_[4 * e + j], b = tets_[4 * e + k];
          edges.push_back({std::min(a, b), std::max(a, b)});
        }
    std::sort(edges.begin(), edges.end());
    edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
    std::ofstream of("faces-000.dat"), oed("edges-000.dat"), oof("owned-faces-000.dat"),
        ooe("owned-edges-000.dat"), obf("boundary-faces-000.dat"), obe("boundary-edges-000.dat");
    const double almost_one = 0.99999999, mid = 0.5 * (desc_.lo + desc_.hi), half = 0.5 * (desc_.hi - desc_.lo);
    auto on_boundary = [&](const int64_t *g, int m) {
      for (int d = 0; d < 3; ++d) {
        double s = 0.0;
        for (int q = 0; q < m; ++q) s += nodes_[3 * g[q] + d];
        const double u = (s / m - mid) / half;
        if (u <= -almost_one || u >= almost_one) return true;
      }
      return false;
    };
    for (size_t i = 0; i < faces.size(); ++i) {
      of << i << ' ' << faces[i][0] << ' ' << faces[i][1] << ' ' << faces[i][2] << ' ' << '\n';
      oof << i << '\n';
      if (on_boundary(faces[i].data(), 3)) obf << i << '\n';
    }
    for (size_t i = 0; i < edges.size(); ++i) {
      oed << i << ' ' << edges[i][0] << ' ' << edges[i][1] << ' ' << '\n';
      ooe << i << '\n';
      if (on_boundary(edges[i].data(), 2)) obe << i << '\n';
    }
  }

 private:
  std::shared_ptr<Context> ctx_;
  mpg_mesh_desc desc_{};
  std::vector<double> nodes_, jinv_, detj_, normals_;
  std::vector<int32_t> tets_, nbrs_, pairs_;
  std::vector<int8_t> fper_;
  std::vector<uint8_t> bnd_;
};

class ParticleList {  // particle_list.hpp:54-320
 public:
  enum KILL_MIGRATE_FLAG { KILL_ONLY = -2, DO_NOTHING };
  ParticleList() = default;
  ParticleList(std::shared_ptr<Context> c, std::size_t max_capacity) : ctx_(c), cap_(max_capacity) {
    check(c->ctx, mpg_particles_reserve(c->ctx, (int64_t)max_capacity), "mpg_particles_reserve");
  }
  std::size_t num_particles() const {
    int64_t n = 0;
    check(ctx_->ctx, mpg_particles_count(ctx_->ctx, &n), "mpg_particles_count");
    return (std::size_t)n;
  }
  GO max_capacity() const { return (GO)cap_; }
  // host snapshot of the device list (ParticleList accessors, particle_list.hpp:68-91)
  void refresh() const {
    int64_t slots = 0;
    mpg_particles_download(ctx_->ctx, 0, &slots, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    const int64_t m = slots > 0 ? slots : 1;
    cell_.resize(m);
    x_.resize(3 * m);
    xr_.resize(3 * m);
    v_.resize(3 * m);
    w_.resize(m);
    sp_.resize(m);
    int64_t n = 0;
    check(ctx_->ctx,
          mpg_particles_download(ctx_->ctx, m, &n, cell_.data(), x_.data(), xr_.data(), v_.data(), w_.data(),
                                 sp_.data(), nullptr),
          "mpg_particles_download");
    snap_n_ = n;
  }
  GO ielement(std::size_t i) const { return cell_.at(i); }
  VECTOR x(std::size_t i) const { return {x_[3 * i], x_[3 * i + 1], x_[3 * i + 2]}; }
  VECTOR x_ref(std::size_t i) const { return {xr_[3 * i], xr_[3 * i + 1], xr_[3 * i + 2]}; }
  VECTOR v(std::size_t i) const { return {v_[3 * i], v_[3 * i + 1], v_[3 * i + 2]}; }
  FLOAT weight(std::size_t i) const { return w_.at(i); }
  int type(std::size_t i) const { return sp_.at(i); }
  bool is_dead(std::size_t i) const { return cell_.at(i) < 0; }
  std::size_t snapshot_size() const { return (std::size_t)snap_n_; }
  void sort() { check(ctx_->ctx, mpg_sort(ctx_->ctx), "mpg_sort"); }
  // particle_list.cpp:135-146: sort, then the first list position per element
  void compute_start_particles_by_element() {
    sort();
    int64_t T = 0, N = 0, nb = 0;
    check(ctx_->ctx, mpg_mesh_sizes(ctx_->ctx, &T, &N, &nb), "mpg_mesh_sizes");
    start_.resize(T + 1);
    check(ctx_->ctx, mpg_cell_starts(ctx_->ctx, T + 1, start_.data()), "mpg_cell_starts");
  }
  // particle_list.hpp:253-257 (start_by_element_ after compute_start_particles_by_element)
  LO start(LO elem) const { return (LO)start_.at(elem); }
  LO count_for_element(LO elem) const { return (LO)(start_.at(elem + 1) - start_.at(elem)); }
  void dump_particles(std::ostream &out) const {  // particle_list.hpp:221-226
    refresh();
    for (int64_t i = 0; i < snap_n_; ++i)
      out << cell_[i] << "(" << x_[3 * i] << ", " << x_[3 * i + 1] << ", " << x_[3 * i + 2] << ") (" << v_[3 * i]
          << ", " << v_[3 * i + 1] << ", " << v_[3 * i + 2] << ") " << sp_[i] << "\n";
  }

 private:
  std::shared_ptr<Context> ctx_;
  std::size_t cap_ = 0;
  mutable std::vector<int32_t> cell_, sp_;
  mutable std::vector<double> x_, xr_, v_, w_;
  mutable int64_t snap_n_ = 0;
  std::vector<int64_t> start_;
};

class ES {  // ES.hpp:48-116
 public:
  ES() = default;
  ES(std::shared_ptr<Context> c, const Mesh *mesh) : ctx_(c), mesh_(mesh) {
    c->configure();
    phi_.resize(mesh->num_nodes);
    rhs_.resize(mesh->num_nodes);
  }
  // ES.cpp:216-231: |r|/|rhs| < tol
  bool solve(FLOAT tol = 1.e-5) {
    if (ctx_->cfg.tol != tol) {
      ctx_->cfg.tol = tol;
      ctx_->configure();
    }
    int it = 0;
    double res = 0;
    int rc = mpg_solve(ctx_->ctx, &it, &res);
    if (rc != MPG_OK && rc != MPG_ERR_NOT_CONVERGED) check(ctx_->ctx, rc, "mpg_solve");
    fresh_ = false;
    return rc == MPG_OK;
  }
  FLOAT phi(LO lid) {
    pull();
    return phi_.at(lid);
  }
  FLOAT rhs(LO lid) {
    pull();
    return rhs_.at(lid);
  }
  // ES.cpp:235-257: rhs_i = -sum_c f(x_c) detJ w_c N_i(c), zero on the boundary
  void set_analytic_RHS(FLOAT (*f)(VECTOR &x)) {
    const double A = 0.5854101966249685, B = 0.1381966011250105;
    const double P[4][3] = {{B, B, B}, {A, B, B}, {B, A, B}, {B, B, A}};
    std::vector<double> r(mesh_->num_nodes, 0.0);
    for (LO e = 0; e < mesh_->num_elems; ++e) {
      double fc[4];
      for (int c = 0; c < 4; ++c) {
        VECTOR phys, ref = {P[c][0], P[c][1], P[c][2]};
        mesh_->refToPhysical(phys, ref, e);
        fc[c] = f(phys);
      }
      const double wm = mesh_->determinate_jacobian(e) * (1.0 / 24.0);
      for (int i = 0; i < 4; ++i) {
        double val = 0;
        for (int c = 0; c < 4; ++c) {
          const double Ni = i == 0 ? 1 - P[c][0] - P[c][1] - P[c][2] : P[c][i - 1];
          val += -fc[c] * (wm * Ni);
        }
        const LO row = mesh_->elem_to_node_lids(e, i);
        if (mesh_->is_boundary_node(row)) val = 0;
        r[row] += val;
      }
    }
    check(ctx_->ctx, mpg_set_field(ctx_->ctx, MPG_FIELD_RHS, r.data()), "mpg_set_field");
    fresh_ = false;
  }
  // ES.cpp:258-268
  void set_analytic_phi(FLOAT (*f)(VECTOR &x)) {
    std::vector<double> p(mesh_->num_nodes);
    for (LO i = 0; i < mesh_->num_nodes; ++i) {
      VECTOR x = mesh_->nodes(i);
      p[i] = f(x);
    }
    check(ctx_->ctx, mpg_set_field(ctx_->ctx, MPG_FIELD_PHI, p.data()), "mpg_set_field");
    fresh_ = false;
  }

 private:
  void pull() {
    if (fresh_) return;
    check(ctx_->ctx, mpg_get_field(ctx_->ctx, MPG_FIELD_PHI, phi_.data()), "mpg_get_field");
    check(ctx_->ctx, mpg_get_field(ctx_->ctx, MPG_FIELD_RHS, rhs_.data()), "mpg_get_field");
    fresh_ = true;
  }
  std::shared_ptr<Context> ctx_;
  const Mesh *mesh_ = nullptr;
  std::vector<double> phi_, rhs_;
  bool fresh_ = false;
};

class DataWarehouse {  // data_warehouse.hpp:51-90
 public:
  explicit DataWarehouse(int device = 0) : ctx_(std::make_shared<Context>(device)) { types_.push(ctx_); }
  DataWarehouse(const DataWarehouse &) = delete;
  DataWarehouse &operator=(const DataWarehouse &) = delete;

  // mesh.cpp:85-89 brick file: "nx ny nz mapping" -> five-tet split of [-1,1]^3;
  // periodic: x = -1 and x = 1 identified (mesh.cpp:61-76,178-189; even nx)
  void create_mesh(std::string &in_name, bool periodic = false) {
    std::ifstream in(in_name.c_str());
    mpg_mesh_desc d{};
    int mapping = 0;
    if (!(in >> d.nx >> d.ny >> d.nz)) throw std::runtime_error("cannot read mesh file " + in_name);
    in >> mapping;
    d.split = MPG_SPLIT_REF5;
    d.lo = -1.0;
    d.hi = 1.0;
    d.mapping = mapping;
    d.periodic = periodic ? 1 : 0;
    create_mesh(d);
  }
  void create_mesh(const mpg_mesh_desc &d) { mesh_ = std::make_unique<Mesh>(ctx_, d); }
  void dump_mesh_data() { mesh_->dump_data(); }
  void create_particle_list(std::size_t max_capacity = 32768 * 1024) {
    if (!ctx_->configured) ctx_->configure();
    particles_ = std::make_unique<ParticleList>(ctx_, max_capacity);
  }
  void create_ES() { es_ = std::make_unique<ES>(ctx_, mesh_.get()); }
  void set_kill_particles_on_wall_impact(bool flag) {
    ctx_->cfg.kill_on_wall = flag ? 1 : 0;
    if (ctx_->configured) ctx_->configure();
  }
  bool kill_particles_on_wall_impact() { return ctx_->cfg.kill_on_wall != 0; }
  // GB300 options not present in the reference: precision, deposit, solver, ...
  mpg_config &config() { return ctx_->cfg; }
  void apply_config() { ctx_->configure(); }

  Mesh &mesh_reference() { return *mesh_; }
  ParticleList &particles_reference() { return *particles_; }
  ParticleTypeList &particle_type_list_reference() { return types_; }
  class ES &ES_reference() { return *es_; }
  const Mesh &mesh() const { return *mesh_; }
  const ParticleList &particles() const { return *particles_; }
  mpg_ctx *raw() { return ctx_->ctx; }
  std::shared_ptr<Context> context() { return ctx_; }

 private:
  std::shared_ptr<Context> ctx_;
  std::unique_ptr<Mesh> mesh_;
  std::unique_ptr<ParticleList> particles_;
  ParticleTypeList types_;
  std::unique_ptr<class ES> es_;
};

class ParticleFill {  // particle_fill.hpp:53-68
 public:
  ParticleFill(DataWarehouse &data, int num_parts_per_element, int type, FLOAT density, VECTOR vel = VECTOR{0, 0, 0},
               FLOAT temp = 1.0) {
    int rc = mpg_fill_ref(data.raw(), num_parts_per_element, type, density, vel.data(), temp);
    if (rc == MPG_ERR_CAPACITY) {
      std::cout << "Cannot create that number of particles, no fill performed\n";
      return;
    }
    check(data.raw(), rc, "mpg_fill_ref");
  }
};

class ParticleMove {  // particle_move.hpp:53-436
 public:
  explicit ParticleMove(DataWarehouse &data) : data_(data) {}
  void move(double dt) {
    mpg_step_stats st{};
    int rc = mpg_move(data_.raw(), dt * scale_, &st);
    if (rc != MPG_OK && rc != MPG_ERR_WALK_LIMIT) check(data_.raw(), rc, "mpg_move");
  }
  void set_force_scale(FLOAT scale = 1) { scale_ = scale; }

 private:
  DataWarehouse &data_;
  FLOAT scale_ = 1.0;
};

class PIC {  // PIC.hpp:54-106
 public:
  explicit PIC(DataWarehouse &data) : data_(data) { mpg_set_timing(data.raw(), 1); }
  void weight_charge() {
    auto t0 = std::chrono::steady_clock::now();
    check(data_.raw(), mpg_weight_charge(data_.raw()), "mpg_weight_charge");
    weight_charge_timer_ += seconds_since(t0);
  }
  void weight_Efield() {
    auto t0 = std::chrono::steady_clock::now();
    check(data_.raw(), mpg_weight_efield(data_.raw()), "mpg_weight_efield");
    weight_field_timer_ += seconds_since(t0);
  }
  // PIC.cpp:245-267: one step; prints the total kinetic energy like PIC.cpp:263
  void time_step(double dt) {
    mpg_step_stats st{};
    int rc = mpg_step(data_.raw(), dt, 1, &st);
    if (rc != MPG_OK && rc != MPG_ERR_NOT_CONVERGED && rc != MPG_ERR_WALK_LIMIT)
      check(data_.raw(), rc, "mpg_step");
    move_timer_ += st.ms_move * 1e-3;
    weight_charge_timer_ += st.ms_deposit * 1e-3;
    solve_timer_ += st.ms_solve * 1e-3;
    weight_field_timer_ += st.ms_efield * 1e-3;
    sort_timer_ += st.ms_sort * 1e-3;
    last_ = st;
    if (print_ke_) std::cout << "Total KE is " << st.ke << std::endl;
  }
  void output_timers() {  // PIC.hpp:85-88
    std::cout << "Timers are:\nMove " << move_timer_ << " Weight charge " << weight_charge_timer_ << ", Sorting "
              << sort_timer_ << ", Solve " << solve_timer_ << ", Weight EField " << weight_field_timer_
              << ", and KE compute " << KE_timer_ << std::endl;
  }
  const mpg_step_stats &last_stats() const { return last_; }
  void set_print_ke(bool on) { print_ke_ = on; }

 private:
  static double seconds_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  DataWarehouse &data_;
  double move_timer_ = 0, weight_charge_timer_ = 0, sort_timer_ = 0, solve_timer_ = 0, weight_field_timer_ = 0,
         KE_timer_ = 0;
  mpg_step_stats last_{};
  bool print_ke_ = true;
};

}  // namespace mpg
