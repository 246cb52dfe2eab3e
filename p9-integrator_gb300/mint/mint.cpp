// mint.cpp - drop-in replacement for the reference's `mint` executable.
//
// Same command line (src/simutils.cuh:138-175), same JSON system config
// (src/simutils.cuh:232-301), same batch loop and output files
// (src/mercurius.cu:179-252, src/simutils.cuh:177-230), driving the GPU
// integrator through the C ABI of libmerc.so.
//
//   mint -c <config.json> -t <T> [-i] [-p] [-o <file>] [-d <device>]
//        [--dump-precise <file>] [--checkpoint <file>] [--resume <file>] [--dry-run]
//
//  -t T      as in the reference: T > batch_size runs T / batch_size batches,
//            otherwise T batches, each of batch_size steps (src/mercurius.cu:179)
//  -o file   positions file (default output_<device>), appended every
//            CHECKPOINT_FREQUENCY = 20 batches with `#`, `$` and "x y z" lines
//  -i        print the system and per-batch progress
//  -p        accepted and ignored, as in the reference (src/mercurius.cu:251)
//  --dump-precise file   also write the positions with 17 significant digits,
//            and the elements file with 17 significant digits
//  --checkpoint file     write a binary checkpoint (merc_save_checkpoint) after
//            every CHECKPOINT_FREQUENCY-th batch and after the last one
//  --resume file         start from a checkpoint written by --checkpoint for
//            the same configuration, continuing with the batch after it
//  --dry-run parse the configuration, print it, run nothing
//
// Optional config keys (reference defaults in brackets): "dt" [0.8219],
// "batch_size" [1000000], "changeover_hill_factor" [1], "softening2" [1e-8],
// "kepler_iters" [8], "bs_rows" [3], "drift" ["elements"|"universal"],
// "compat_local_index" [false: a body excludes only itself; true: the
// reference's threadIdx.x comparison with block size N/16],
// "sweeps_per_device" [4].
//
// Sweeps: the reference reads sweeps[4 * device + k], k < 4, each replacing
// the elements (not the mass) of body 0 with mean anomaly 0
// (src/simutils.cuh:288-300, src/mercurius.cu:133-164).  Without a "sweeps"
// key the reference dereferences an unset pointer; here the bodies run as one
// system.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/merc.h"
#include "json_reader.h"

namespace {

constexpr int kCheckpointFrequency = 20;  // src/constants.cuh:13
constexpr double kMassiveThreshold = 1e-12;  // src/mercurius.cu:9
const char* kElementKeys[6] = {"inclination", "longitude_of_ascending_node", "argument_of_perihelion",
                               "mean_anomaly", "eccentricity", "semi_major_axis"};

struct Args {
  bool info = false, positions = false, dry_run = false;
  long long timesteps = 1;
  std::string config, output, precise, checkpoint, resume;
  int device = 0;
};

// src/simutils.cuh:138-175: flags anywhere, value in the next argument
Args parse_args(int argc, char** argv) {
  Args a;
  for (int i = 0; i < argc; i++) {
    std::string s = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) throw std::runtime_error("missing value after " + s);
      return argv[++i];
    };
    if (s == "-i") a.info = true;
    else if (s == "-p") a.positions = true;
    else if (s == "-t") a.timesteps = std::atoll(next().c_str());
    else if (s == "-c") a.config = next();
    else if (s == "-o") a.output = next();
    else if (s == "-d") a.device = std::atoi(next().c_str());
    else if (s == "--dump-precise") a.precise = next();
    else if (s == "--checkpoint") a.checkpoint = next();
    else if (s == "--resume") a.resume = next();
    else if (s == "--dry-run") a.dry_run = true;
  }
  if (a.config.empty()) throw std::runtime_error("no config file: use -c <config.json>");
  return a;
}

struct Body {
  std::string name;
  double mass;
  double el[6];
  double radius;  // optional "radius" key (AU); collisions are detected when any body has one
};

struct Config {
  std::vector<Body> bodies;
  std::vector<Body> sweeps;
  merc_params p;
  long long batch_size = 1000000;
  int sweeps_per_device = 4;
  bool compat_local_index = false;
};

Body read_body(const mintjson::Value& v) {
  Body b;
  b.name = v.string_or("name", "");
  b.mass = v.number("mass");
  for (int k = 0; k < 6; k++) b.el[k] = v.number(kElementKeys[k]);
  b.radius = v.number_or("radius", -1.0);
  return b;
}

Config read_config(const std::string& path) {
  mintjson::Value doc = mintjson::parse_file(path);
  Config c;
  merc_default_params(&c.p);
  const mintjson::Value* bodies = doc.get("bodies");
  if (!bodies || bodies->kind != mintjson::Value::Array || bodies->arr.empty())
    throw std::runtime_error("config has no \"bodies\" array");
  for (auto& b : bodies->arr) c.bodies.push_back(read_body(b));
  if (const mintjson::Value* sw = doc.get("sweeps"))
    for (auto& b : sw->arr) c.sweeps.push_back(read_body(b));
  c.p.dt = doc.number_or("dt", c.p.dt);
  c.batch_size = (long long)doc.number_or("batch_size", (double)c.batch_size);
  c.p.hill_factor = doc.number_or("changeover_hill_factor", c.p.hill_factor);
  c.p.softening2 = doc.number_or("softening2", c.p.softening2);
  c.p.kepler_iters = (int)doc.number_or("kepler_iters", c.p.kepler_iters);
  c.p.bs_rows = (int)doc.number_or("bs_rows", c.p.bs_rows);
  c.p.kepler_tol = doc.number_or("kepler_tol", c.p.kepler_tol);
  std::string drift = doc.string_or("drift", "elements");
  if (drift == "elements") c.p.drift = MERC_DRIFT_ELEMENTS;
  else if (drift == "universal") c.p.drift = MERC_DRIFT_UNIVERSAL;
  else throw std::runtime_error("unknown drift '" + drift + "'");
  c.compat_local_index = doc.bool_or("compat_local_index", false);
  c.sweeps_per_device = (int)doc.number_or("sweeps_per_device", 4);
  if (c.batch_size <= 0) throw std::runtime_error("batch_size must be positive");
  return c;
}

// dump_sim, src/simutils.cuh:118-136
void dump_system(const std::vector<Body>& b) {
  std::cout << "Simulation with " << b.size() << " bodies" << std::endl;
  for (size_t i = 0; i < b.size(); i++) {
    std::cout << "Body: " << i << std::endl;
    std::cout << "inclination: " << b[i].el[0] << std::endl;
    std::cout << "longitude of ascending node: " << b[i].el[1] << std::endl;
    std::cout << "argument of perihelion: " << b[i].el[2] << std::endl;
    std::cout << "mean anomaly: " << b[i].el[3] << std::endl;
    std::cout << "eccentricity: " << b[i].el[4] << std::endl;
    std::cout << "semi major axis: " << b[i].el[5] << std::endl;
    std::cout << "mass: " << b[i].mass << std::endl << std::endl;
  }
}

void check(int st, merc_ctx* ctx, const char* what) {
  if (st != MERC_OK) {
    throw std::runtime_error(std::string(what) + " failed (" + std::to_string(st) + "): " + merc_last_error(ctx));
  }
}

}  // namespace

int main(int argc, char** argv) {
  try {
    Args a = parse_args(argc, argv);
    Config c = read_config(a.config);
    const int nb = (int)c.bodies.size();
    int nm = 0;
    for (auto& b : c.bodies) nm += b.mass > kMassiveThreshold;
    for (int i = 0; i < nm; i++)
      if (!(c.bodies[i].mass > kMassiveThreshold))
        throw std::runtime_error("massive bodies must come first (body " + std::to_string(i) + ")");
    // systems of this device: one per sweep, or the bodies as given
    int nsys = 1;
    std::vector<const Body*> sweep_of;
    if (!c.sweeps.empty()) {
      nsys = c.sweeps_per_device;
      for (int k = 0; k < nsys; k++) {
        size_t idx = (size_t)c.sweeps_per_device * a.device + k;
        if (idx >= c.sweeps.size())
          throw std::runtime_error("config has " + std::to_string(c.sweeps.size()) + " sweeps; device " +
                                   std::to_string(a.device) + " needs sweep " + std::to_string(idx));
        sweep_of.push_back(&c.sweeps[idx]);
      }
    }
    if (c.compat_local_index) c.p.compat_block = std::max(1, nb / 16);
    const int64_t ntot = (int64_t)nb * nsys;
    std::vector<int64_t> off(nsys + 1);
    std::vector<int32_t> nmv(nsys, nm);
    std::vector<double> mass(ntot), el(6 * ntot), radius(ntot);
    bool radii = false;
    for (auto& b : c.bodies) radii = radii || b.radius >= 0.0;
    for (int s = 0; s < nsys; s++) {
      off[s + 1] = off[s] + nb;
      for (int j = 0; j < nb; j++) {
        int64_t g = off[s] + j;
        mass[g] = c.bodies[j].mass;
        radius[g] = std::max(0.0, c.bodies[j].radius);
        for (int k = 0; k < 6; k++) el[k * ntot + g] = c.bodies[j].el[k];
      }
      if (!sweep_of.empty()) {  // body 0 takes the sweep's elements, M = 0, mass unchanged
        for (int k = 0; k < 6; k++) el[k * ntot + off[s]] = sweep_of[s]->el[k];
        el[3 * ntot + off[s]] = 0.0;
      }
    }
    const long long iters = a.timesteps > c.batch_size ? a.timesteps / c.batch_size : a.timesteps;
    if (a.timesteps > c.batch_size && a.timesteps % c.batch_size != 0)
      throw std::runtime_error("-t must be a multiple of batch_size when larger than it");
    if (a.info || a.dry_run) {
      std::cout << "Systems: " << nsys << " x " << nb << " bodies (" << nm << " massive), dt " << c.p.dt
                << ", batch " << c.batch_size << " steps x " << iters << " batches, drift "
                << (c.p.drift == MERC_DRIFT_ELEMENTS ? "elements" : "universal") << std::endl;
      dump_system(c.bodies);
    }
    if (a.dry_run) return 0;

    merc_ctx* ctx = nullptr;
    int st = merc_create(a.device, &c.p, &ctx);
    if (st != MERC_OK) throw std::runtime_error("merc_create failed: status " + std::to_string(st));
    long long first_batch = 0;
    if (a.resume.empty()) {
      check(merc_load_elements(ctx, nsys, off.data(), nmv.data(), mass.data(), el.data()), ctx, "load");
      if (radii) check(merc_set_radii(ctx, radius.data()), ctx, "radii");
    } else {
      check(merc_load_checkpoint(ctx, a.resume.c_str()), ctx, "resume");
      merc_stats rs;
      check(merc_get_stats(ctx, &rs), ctx, "stats");
      if (rs.n_bodies != ntot || rs.n_systems != nsys || rs.steps_done % c.batch_size != 0)
        throw std::runtime_error("checkpoint " + a.resume + " does not belong to this configuration");
      first_batch = rs.steps_done / c.batch_size;
      if (a.info) std::cout << "Resuming after batch " << first_batch << std::endl;
    }
    std::string outname = a.output.empty() ? "output_" + std::to_string(a.device) : a.output;
    std::vector<double> pos(3 * ntot), elements(6 * ntot);
    for (long long batch = first_batch; batch < iters; batch++) {
      check(merc_step(ctx, c.batch_size), ctx, "step");
      if (a.info) std::cout << "Batch " << (batch + 1) << " Simulation Complete.\n";
      const bool checkpoint = batch % kCheckpointFrequency == 0;
      if (checkpoint) {
        check(merc_get_state(ctx, pos.data(), nullptr, nullptr), ctx, "get_state");
        check(merc_get_elements(ctx, elements.data()), ctx, "get_elements");
        // write_positions, src/simutils.cuh:186-230
        std::ofstream f(outname, std::ios::app);
        if (!f) {
          std::cerr << "Error opening file: " << outname << std::endl;
        } else {
          int nan_counter = 0;
          f << "#\n";
          for (int s = 0; s < nsys; s++) {
            f << "$\n";
            for (int j = 0; j < nb; j++) {
              int64_t g = off[s] + j;
              double x = pos[g], y = pos[ntot + g], z = pos[2 * ntot + g];
              if (std::isnan(x) || std::isnan(y) || std::isnan(z)) nan_counter++;
              f << x << " " << y << " " << z << std::endl;
            }
            f << std::endl;
          }
          f << std::endl;
          std::cout << "NaN counter for  " << (int)(c.batch_size * batch) + 1 << " timestep (mYrs): " << nan_counter
                    << std::endl;
        }
        if (!a.precise.empty()) {
          std::ofstream fp(a.precise, std::ios::app);
          fp << std::setprecision(17) << "#\n";
          for (int s = 0; s < nsys; s++) {
            fp << "$\n";
            for (int j = 0; j < nb; j++) {
              int64_t g = off[s] + j;
              fp << pos[g] << " " << pos[ntot + g] << " " << pos[2 * ntot + g] << "\n";
            }
            fp << "\n";
          }
          fp << "\n";
        }
        // elements file, src/mercurius.cu:210-248
        std::ofstream fe("elements_" + std::to_string(a.device) + ".txt");
        if (!a.precise.empty()) fe << std::setprecision(17);
        fe << "Timestep: " << batch * c.batch_size << std::endl;
        for (int s = 0; s < nsys; s++) {
          fe << "Experiment: " << s << std::endl;
          for (int j = 0; j < nb; j++) {
            int64_t g = off[s] + j;
            fe << elements[g] << " " << elements[ntot + g] << " " << elements[2 * ntot + g] << " "
               << elements[3 * ntot + g] << " " << elements[4 * ntot + g] << " " << elements[5 * ntot + g]
               << std::endl;
          }
          fe << std::endl;
        }
      }
      // the next batch restarts from the elements, as every kernel launch of
      // the reference does (src/sim.cuh:744-765 then :654-677)
      check(merc_roundtrip(ctx), ctx, "roundtrip");
      if (!a.checkpoint.empty() && (checkpoint || batch == iters - 1))
        check(merc_save_checkpoint(ctx, a.checkpoint.c_str()), ctx, "checkpoint");
    }
    if (radii && a.info) {
      int64_t ncol = 0;
      check(merc_get_collisions(ctx, nullptr, 0, &ncol), ctx, "collisions");
      std::cout << "Collisions: " << ncol << std::endl;
    }
    merc_destroy(ctx);
    return 0;
  } catch (const std::exception& e) {
    std::cerr << "mint: " << e.what() << std::endl;
    return 1;
  }
}
