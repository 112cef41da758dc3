// main.cpp -- command-line driver of the GB300 PIC step, shaped like the
// reference driver (main.cpp:58-153): same flags, same problem set-up and the
// same printed lines ("Fill time", "Total KE is", "Move time ... updates/second",
// the timer summary).  Extra flags select the GB300 options.
//
//   minipic_gb300 --mesh=brick.txt --nparts=10 --dt=0.1 --tfinal=2.0
//                 [--kill-particles=1] [--density=...] [--output=k] [--dump_mesh=1]
//                 [--steps=N] [--precision=plain|mixed] [--solver=bicgstab|cg|cg-mg]
//                 [--deposit=quarter|linear] [--tol=1e-6]
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>

#include "minipic_gb300.hpp"

using namespace mpg;

static bool opt(const char *arg, const char *name, std::string &val) {
  const size_t n = strlen(name);
  if (strncmp(arg, "--", 2) || strncmp(arg + 2, name, n) || arg[2 + n] != '=') return false;
  val = arg + 3 + n;
  return true;
}

int main(int argc, char **argv) {
  std::string meshfile("brick.txt"), problem("none"), precision("plain"), solver("bicgstab"), deposit("quarter");
  int num_particles_per_element = 10000, part_kill = 0, output = 0, dump_mesh = 0, steps = -1;
  double dt = 0.1, t_final = 2.0, density = 2. / 3. * M_PI * M_PI, tol = 1e-6;
  for (int i = 1; i < argc; ++i) {
    std::string v;
    if (opt(argv[i], "nparts", v)) num_particles_per_element = atoi(v.c_str());
    else if (opt(argv[i], "mesh", v)) meshfile = v;
    else if (opt(argv[i], "dt", v)) dt = atof(v.c_str());
    else if (opt(argv[i], "tfinal", v)) t_final = atof(v.c_str());
    else if (opt(argv[i], "output", v)) output = atoi(v.c_str());
    else if (opt(argv[i], "kill-particles", v)) part_kill = atoi(v.c_str());
    else if (opt(argv[i], "problem", v)) problem = v;
    else if (opt(argv[i], "density", v)) density = atof(v.c_str());
    else if (opt(argv[i], "dump_mesh", v)) dump_mesh = atoi(v.c_str());
    else if (opt(argv[i], "steps", v)) steps = atoi(v.c_str());
    else if (opt(argv[i], "precision", v)) precision = v;
    else if (opt(argv[i], "solver", v)) solver = v;
    else if (opt(argv[i], "deposit", v)) deposit = v;
    else if (opt(argv[i], "tol", v)) tol = atof(v.c_str());
    else if (!strcmp(argv[i], "--help") || !strcmp(argv[i], "-h")) {
      std::cout << "usage: " << argv[0]
                << " [--nparts=N] [--mesh=file] [--dt=x] [--tfinal=x] [--output=k] [--kill-particles=0|1]"
                   " [--problem=none|two-stream] [--density=x] [--dump_mesh=0|1] [--steps=N] [--precision=plain|mixed]"
                   " [--solver=bicgstab|cg|cg-mg] [--deposit=quarter|linear] [--tol=x]\n";
      return 0;
    } else {
      std::cerr << "unknown option " << argv[i] << "\n";
      return 2;
    }
  }
  const bool two_stream = problem == "two-stream";
  try {
    DataWarehouse data;
    data.create_mesh(meshfile, two_stream);  // main.cpp:89-92: periodic for the two-stream problem
    mpg_config &cfg = data.config();
    cfg.precision = precision == "mixed" ? MPG_MIXED : MPG_PLAIN;
    cfg.solver = solver == "cg" ? MPG_SOLVER_CG : solver == "cg-mg" ? MPG_SOLVER_CG_MG : MPG_SOLVER_BICGSTAB;
    cfg.deposit = deposit == "linear" ? MPG_DEPOSIT_LINEAR : MPG_DEPOSIT_REF_QUARTER;
    cfg.tol = tol;
    cfg.kill_on_wall = part_kill == 1;
    data.apply_config();
    data.create_particle_list((size_t)data.mesh().num_elems * num_particles_per_element * 3 + 1000);
    data.create_ES();
    data.set_kill_particles_on_wall_impact(part_kill == 1);
    auto t0 = std::chrono::steady_clock::now();
    if (two_stream) {
      // main.cpp:98-106: two counter-streaming electron beams with a sinusoidal
      // velocity perturbation (temp < 0, particle_fill.hpp:106-110) over ions at rest
      VECTOR v{0.5, 0.0, 0.0};
      const FLOAT temp = -.05;
      ParticleFill fill1a(data, num_particles_per_element / 2, 0, density / 2, v, temp);
      v[0] *= -1;
      ParticleFill fill1b(data, num_particles_per_element / 2, 0, density / 2, v, temp);
      ParticleFill fill2(data, num_particles_per_element, 2, density, VECTOR{0, 0, 0}, 0);
    } else {
      ParticleFill fill1(data, num_particles_per_element, 0, density);
      ParticleFill fill2(data, num_particles_per_element, 1, density);
    }
    if (dump_mesh) data.dump_mesh_data();
    PIC pic(data);
    double fill_time = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    printf("Fill time %lf for %ld particles\n", fill_time, (long)data.particles().num_particles());
    auto t1 = std::chrono::steady_clock::now();
    int output_cnt = 0, nsteps = 0;
    const int max_steps = steps >= 0 ? steps : (int)ceil(t_final / dt - 1e-12);
    for (double t = 0; nsteps < max_steps; t += dt, ++nsteps) {
      if (output && (output_cnt++) % output == 0) {  // main.cpp:125-136
        char name[256];
        snprintf(name, sizeof(name), "output.%f", t);
        std::ofstream out(name);
        ParticleList &pl = data.particles_reference();
        pl.refresh();
        for (size_t i = 0; i < pl.snapshot_size(); i += num_particles_per_element)
          if (pl.type(i) == 0)
            out << pl.x(i)[0] << " " << pl.x(i)[1] << " " << pl.x(i)[2] << " " << pl.v(i)[0] << " " << pl.v(i)[1]
                << " " << pl.v(i)[2] << std::endl;
      }
      pic.time_step(dt);
    }
    double move_time = std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
    printf("Move time %lf for %d parts, or %5.1lfE6 updates/second \n", move_time,
           (int)data.particles().num_particles(),
           1e-6 * data.mesh().num_global_elems * num_particles_per_element * nsteps / move_time);
    pic.output_timers();
  } catch (const std::exception &e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
