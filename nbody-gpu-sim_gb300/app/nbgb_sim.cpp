// nbgb_sim.cpp -- headless simulation driver with the reference
// application's command line and its --benchmark JSON report.
//
// Mirrors nbody_sim's non-interactive path: option parsing and validation
// (src/core/app_cli.cpp:52-140), ParticleSystem::initialize with the
// spherical initial conditions (src/core/particle_system.cpp:62-105,
// src/cuda/particle_init.cu:188-209), --import / --export of the v1
// checkpoint format (src/utils/serialization.cpp), the benchmark loop and
// its BenchmarkRunRecord JSON (src/main.cpp:347-401,
// src/utils/performance_observability.cpp:97-139).  The interactive window
// is not built (no graphics stack on the GPU host): without --benchmark the
// driver reports that and exits 1.
//
// The loop runs on the device-resident FP64 system (nbgb_system_*): state
// stays on the GPU across all steps and a(0) is computed once, so the
// per-step cost is the force evaluation plus one fused kick-drift kernel.
//
// Extension beyond the reference CLI: --export-initial PATH writes the
// initial state (after --import, if given) before any GPU work.
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "nbgb.h"

namespace {

struct ValidationError : std::runtime_error {
  explicit ValidationError(const std::string& m) : std::runtime_error("Validation Error: " + m) {}
};
struct IoError : std::runtime_error {
  explicit IoError(const std::string& m) : std::runtime_error("I/O Error: " + m) {}
};
struct DeviceError : std::runtime_error {
  explicit DeviceError(const std::string& m) : std::runtime_error(m) {}
};

// AppCliOptions (include/nbody/app_cli.hpp:8-24) with its defaults.
struct Options {
  size_t particle_count = 10000;
  int force_method = NBGB_DIRECT_N2;
  float dt = 0.001f;
  float G = 1.0f;
  float softening = 0.1f;
  float theta = 0.5f;
  float cell_size = 2.0f;
  float cutoff = 2.0f;
  bool benchmark_mode = false;
  size_t benchmark_steps = 120;
  std::string benchmark_output_path;
  bool show_help = false;
  std::string export_path;
  std::string import_path;
  std::string export_initial_path;
  bool group_walk = false;  // extension: --bh-walk group
};

const char* method_name(int m) {  // forceMethodToString (types.hpp:39-49)
  switch (m) {
    case NBGB_DIRECT_N2: return "direct_n2";
    case NBGB_BARNES_HUT: return "barnes_hut";
    case NBGB_SPATIAL_HASH: return "spatial_hash";
  }
  return "unknown";
}

int parse_method(const std::string& v) {
  if (v == "direct-n2" || v == "direct_n2") return NBGB_DIRECT_N2;
  if (v == "barnes-hut" || v == "barnes_hut") return NBGB_BARNES_HUT;
  if (v == "spatial-hash" || v == "spatial_hash") return NBGB_SPATIAL_HASH;
  throw ValidationError("Unsupported force method: " + v);
}

std::string require_value(int argc, char** argv, int& i, const std::string& flag) {
  if (i + 1 >= argc) throw ValidationError("Missing value for " + flag);
  return argv[++i];
}

size_t parse_size(const std::string& v, const std::string& flag) {
  try {
    return static_cast<size_t>(std::stoull(v));
  } catch (const std::exception&) {
    throw ValidationError("Invalid numeric value for " + flag + ": " + v);
  }
}

float parse_float(const std::string& v, const std::string& flag) {
  try {
    return std::stof(v);
  } catch (const std::exception&) {
    throw ValidationError("Invalid numeric value for " + flag + ": " + v);
  }
}

// validateParticleCountRange / validateTimeStep / validateSoftening /
// validateTheta (src/utils/error_handling.cpp:89-137).
void validate_count(size_t n) {
  if (n == 0) throw ValidationError("Particle count must be greater than 0");
  if (n > 100000000ull) throw ValidationError("Particle count exceeds maximum supported (100M)");
}
void validate_dt(float dt) {
  if (dt <= 0) throw ValidationError("Time step must be positive");
  if (std::isnan(dt) || std::isinf(dt)) throw ValidationError("Time step must be a finite number");
  if (dt > 1.0f) throw ValidationError("Time step is too large (max 1.0)");
}
void validate_softening(float eps) {
  if (std::isnan(eps) || std::isinf(eps))
    throw ValidationError("Softening parameter must be a finite number");
  if (eps <= 0) throw ValidationError("Softening parameter must be positive");
}
void validate_theta(float t) {
  if (t < 0 || t > 2.0f) throw ValidationError("Barnes-Hut theta must be between 0 and 2");
  if (std::isnan(t) || std::isinf(t)) throw ValidationError("Barnes-Hut theta must be a finite number");
}

Options parse(int argc, char** argv) {
  Options o;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "--help" || a == "-h") {
      o.show_help = true;
    } else if (a == "--particles") {
      o.particle_count = parse_size(require_value(argc, argv, i, a), a);
    } else if (a == "--method") {
      o.force_method = parse_method(require_value(argc, argv, i, a));
    } else if (a == "--dt") {
      o.dt = parse_float(require_value(argc, argv, i, a), a);
    } else if (a == "--gravity") {
      o.G = parse_float(require_value(argc, argv, i, a), a);
    } else if (a == "--softening") {
      o.softening = parse_float(require_value(argc, argv, i, a), a);
    } else if (a == "--theta") {
      o.theta = parse_float(require_value(argc, argv, i, a), a);
    } else if (a == "--cell-size") {
      o.cell_size = parse_float(require_value(argc, argv, i, a), a);
    } else if (a == "--cutoff") {
      o.cutoff = parse_float(require_value(argc, argv, i, a), a);
    } else if (a == "--benchmark") {
      o.benchmark_mode = true;
    } else if (a == "--benchmark-steps") {
      o.benchmark_steps = parse_size(require_value(argc, argv, i, a), a);
      o.benchmark_mode = true;
    } else if (a == "--benchmark-output") {
      o.benchmark_output_path = require_value(argc, argv, i, a);
      o.benchmark_mode = true;
    } else if (a == "--export") {
      o.export_path = require_value(argc, argv, i, a);
    } else if (a == "--import") {
      o.import_path = require_value(argc, argv, i, a);
    } else if (a == "--export-initial") {
      o.export_initial_path = require_value(argc, argv, i, a);
    } else if (a == "--bh-walk") {
      const std::string v = require_value(argc, argv, i, a);
      if (v == "group")
        o.group_walk = true;
      else if (v == "reference")
        o.group_walk = false;
      else
        throw ValidationError("Unsupported Barnes-Hut walk: " + v);
    } else if (!a.empty() && a.front() == '-') {
      throw ValidationError("Unknown argument: " + a);
    } else {
      o.particle_count = parse_size(a, "particle count");
    }
  }
  validate_count(o.particle_count);
  validate_dt(o.dt);
  validate_softening(o.softening);
  validate_theta(o.theta);
  if (o.G <= 0.0f) throw ValidationError("Gravitational constant must be positive");
  if (o.cell_size <= 0.0f) throw ValidationError("Spatial hash cell size must be positive");
  if (o.cutoff <= 0.0f) throw ValidationError("Spatial hash cutoff must be positive");
  if (o.benchmark_steps == 0) throw ValidationError("Benchmark steps must be greater than zero");
  return o;
}

std::string usage() {
  std::ostringstream u;
  u << "Usage: nbgb_sim [particle_count] [options]\n\n"
    << "Simulation options:\n"
    << "  --particles N          Set particle count\n"
    << "  --method NAME          direct-n2 | barnes-hut | spatial-hash\n"
    << "  --dt VALUE             Set integration time step\n"
    << "  --gravity VALUE        Set gravitational constant\n"
    << "  --softening VALUE      Set softening parameter\n"
    << "  --theta VALUE          Set Barnes-Hut theta\n"
    << "  --cell-size VALUE      Set spatial hash cell size\n"
    << "  --cutoff VALUE         Set spatial hash cutoff radius\n"
    << "  --bh-walk NAME         reference | group (Barnes-Hut walk; default reference)\n"
    << "  --benchmark            Run a non-interactive benchmark and exit\n"
    << "  --benchmark-steps N    Set benchmark update steps\n"
    << "  --benchmark-output P   Write benchmark JSON to path P\n"
    << "\nData export/import:\n"
    << "  --export PATH          Export particle state to checkpoint file\n"
    << "  --import PATH          Import particle state from checkpoint file\n"
    << "  --export-initial PATH  Export the initial state before stepping\n"
    << "\n  --help                 Show this message\n";
  return u.str();
}

// SimulationState (include/nbody/simulation_state.hpp:10-27).
struct State {
  std::vector<float> a[7];  // pos x y z, vel x y z, mass
  size_t count = 0;
  float simulation_time = 0.0f;
  float dt = 0.0f;
  float G = 0.0f;
  float softening = 0.0f;
  int force_method = NBGB_DIRECT_N2;
};

// ParticleInitializer::initSpherical with SphericalDistParams{centre 0,
// radius 10, mass 1} and the default seed 42 (particle_init.cu:188-209):
// std::mt19937 and std::uniform_real_distribution<float>, draws in the
// order r, theta, phi, mass.
void init_spherical(State& s, size_t n) {
  std::mt19937 rng(42u);
  std::uniform_real_distribution<float> u01(0.0f, 1.0f);
  std::uniform_real_distribution<float> um(1.0f, 1.0f);
  const float radius = 10.0f;
  for (auto& v : s.a) v.assign(n, 0.0f);
  for (size_t i = 0; i < n; ++i) {
    const float r = std::cbrt(u01(rng)) * radius;
    const float th = u01(rng) * 2.0f * 3.14159265f;
    const float ph = std::acos(2.0f * u01(rng) - 1.0f);
    s.a[0][i] = 0.0f + r * std::sin(ph) * std::cos(th);
    s.a[1][i] = 0.0f + r * std::sin(ph) * std::sin(th);
    s.a[2][i] = 0.0f + r * std::cos(ph);
    s.a[6][i] = um(rng);
  }
  s.count = n;
}

// .nbody v1 (include/nbody/serialization.hpp, src/utils/serialization.cpp):
// 56-byte native header then seven float32 arrays.
struct FileHeader {
  uint32_t magic;
  uint32_t version;
  uint64_t particle_count;
  float simulation_time, dt, G, softening;
  uint32_t force_method;
  uint32_t reserved[4];
};
static_assert(sizeof(FileHeader) == 56, "v1 header is 56 bytes");
constexpr uint32_t kMagic = 0x4E424F44u;

void save(const std::string& path, const State& s) {
  std::ofstream f(path, std::ios::binary);
  if (!f) throw IoError("Failed to open file for writing: " + path);
  FileHeader h{};
  h.magic = kMagic;
  h.version = 1;
  h.particle_count = s.count;
  h.simulation_time = s.simulation_time;
  h.dt = s.dt;
  h.G = s.G;
  h.softening = s.softening;
  h.force_method = (uint32_t)s.force_method;
  f.write(reinterpret_cast<const char*>(&h), sizeof h);
  for (const auto& v : s.a) f.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * 4));
  if (!f) throw IoError("Failed to write particle data: " + path);
}

State load(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw IoError("Failed to open file for reading: " + path);
  FileHeader h{};
  if (!f.read(reinterpret_cast<char*>(&h), sizeof h))
    throw ValidationError("Failed to read file header: file may be truncated or corrupted");
  if (h.magic != kMagic) throw ValidationError("Invalid file format: wrong magic number");
  if (h.version != 1) throw ValidationError("Unsupported file version");
  if (h.particle_count > 100000000ull)
    throw ValidationError("Particle count (" + std::to_string(h.particle_count) +
                          ") exceeds maximum allowed (100000000)");
  if (h.force_method > 2)
    throw ValidationError("Invalid force method in file header: " + std::to_string(h.force_method));
  State s;
  s.count = (size_t)h.particle_count;
  s.simulation_time = h.simulation_time;
  s.dt = h.dt;
  s.G = h.G;
  s.softening = h.softening;
  s.force_method = (int)h.force_method;
  for (auto& v : s.a) {
    v.resize(s.count);
    if (!f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(s.count * 4)))
      throw ValidationError("Failed to read particle data: file may be truncated or corrupted");
  }
  return s;
}

void check(nbgb_status st) {
  if (st == NBGB_OK) return;
  const std::string msg = nbgb_last_error();
  if (st == NBGB_ERR_INVALID_ARG) throw std::runtime_error(msg);
  throw DeviceError(msg.empty() ? std::string("nbgb status ") + std::to_string((int)st) : msg);
}

nbgb_particle_data host_view(State& s) {
  nbgb_particle_data d{};
  d.pos_x = s.a[0].data();
  d.pos_y = s.a[1].data();
  d.pos_z = s.a[2].data();
  d.vel_x = s.a[3].data();
  d.vel_y = s.a[4].data();
  d.vel_z = s.a[5].data();
  d.mass = s.a[6].data();
  d.count = s.count;
  return d;
}

std::string json_escape(const std::string& v) {
  std::ostringstream e;
  for (char ch : v) {
    switch (ch) {
      case '\\': e << "\\\\"; break;
      case '"': e << "\\\""; break;
      case '\n': e << "\\n"; break;
      case '\r': e << "\\r"; break;
      case '\t': e << "\\t"; break;
      default: e << ch;
    }
  }
  return e.str();
}

void number_map(std::ostringstream& out, const std::map<std::string, double>& m) {
  out << "{";
  bool first = true;
  for (const auto& [k, v] : m) {
    if (!first) out << ",";
    first = false;
    out << "\"" << json_escape(k) << "\":" << v;
  }
  out << "}";
}

int run_benchmark(const Options& o) {
  // SimulationConfig from the options (the app's configFromOptions)
  State s;
  s.dt = o.dt;
  s.G = o.G;
  s.softening = o.softening;
  s.force_method = o.force_method;
  init_spherical(s, o.particle_count);
  if (!o.import_path.empty()) {
    std::cout << "Importing state from: " << o.import_path << std::endl;
    s = load(o.import_path);
    validate_count(s.count);
    validate_dt(s.dt);
    validate_softening(s.softening);
    if (!(s.G > 0) || std::isinf(s.G))
      throw ValidationError("Gravitational constant must be positive and finite");
    std::cout << "Imported " << s.count << " particles" << std::endl;
  }
  if (!o.export_initial_path.empty()) save(o.export_initial_path, s);

  nbgb_params p;
  nbgb_params_default(&p);
  p.G = s.G;
  p.softening = s.softening;
  p.theta = o.theta;
  p.cell_size = o.cell_size;
  p.cutoff = o.cutoff;
  if (o.group_walk && s.force_method == NBGB_BARNES_HUT) p.flags |= NBGB_FLAG_GROUP_WALK;
  p.flags |= NBGB_FLAG_STAGE_TIMINGS;  // device time per stage, for phase_timings
  nbgb_calculator* calc = nullptr;
  check(nbgb_calculator_create((nbgb_method)s.force_method, &p, &calc));
  nbgb_system* sys = nullptr;
  nbgb_particle_data h = host_view(s);
  nbgb_status st = nbgb_system_create(calc, &h, &sys);
  if (st != NBGB_OK) {
    nbgb_calculator_destroy(calc);
    check(st);
  }
  // the initial force evaluation is not part of the steps: its stages are
  // dropped from the totals
  int32_t n_stages = 0;
  if (st == NBGB_OK) st = nbgb_calculator_stage_times(calc, 0, nullptr, nullptr, nullptr, &n_stages, 1);
  const auto t0 = std::chrono::steady_clock::now();
  if (st == NBGB_OK) st = nbgb_system_step(sys, s.dt, (int32_t)o.benchmark_steps);
  const auto t1 = std::chrono::steady_clock::now();
  // device time per stage of the steps' force evaluations (CUDA events)
  constexpr int kMaxStages = 32;
  char stage_names[32 * kMaxStages] = {};
  double stage_ms[kMaxStages] = {};
  int64_t stage_runs[kMaxStages] = {};
  if (st == NBGB_OK)
    st = nbgb_calculator_stage_times(calc, kMaxStages, stage_names, stage_ms, stage_runs,
                                     &n_stages, 0);
  if (st == NBGB_OK) {
    for (size_t k = 0; k < o.benchmark_steps; ++k) s.simulation_time += s.dt;
    if (!o.export_path.empty()) st = nbgb_system_read(sys, &h);
  }
  nbgb_system_destroy(sys);
  nbgb_calculator_destroy(calc);
  check(st);
  if (!o.export_path.empty()) {
    std::cout << "Exporting checkpoint to: " << o.export_path << std::endl;
    save(o.export_path, s);
    std::cout << "Exported " << s.count << " particles" << std::endl;
  }

  // BenchmarkRunRecord: force method, count and parameters from the options
  std::map<std::string, double> metrics, params;
  const double ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  metrics["wall_time_ms"] = ms / (double)o.benchmark_steps;
  params["dt"] = o.dt;
  params["gravity"] = o.G;
  params["softening"] = o.softening;
  params["particle_count"] = (double)o.particle_count;
  if (o.force_method == NBGB_BARNES_HUT) {
    params["theta"] = o.theta;
    if (o.group_walk) params["group_walk"] = 1;
  } else if (o.force_method == NBGB_SPATIAL_HASH) {
    params["cell_size"] = o.cell_size;
    params["cutoff_radius"] = o.cutoff;
  }
  std::ostringstream out;
  out << "{\"benchmarks\":[{";
  out << "\"benchmark_name\":\"application.benchmark_mode\",";
  out << "\"force_method\":\"" << method_name(o.force_method) << "\",";
  out << "\"particle_count\":" << o.particle_count << ",";
  out << "\"iterations\":" << o.benchmark_steps << ",";
  out << "\"metrics\":";
  number_map(out, metrics);
  out << ",\"parameters\":";
  number_map(out, params);
  out << ",\"phase_timings\":[{\"name\":\"simulation.update\",\"total_duration_ms\":" << ms
      << ",\"samples\":" << o.benchmark_steps << "}";
  for (int32_t i = 0; i < std::min(n_stages, kMaxStages); ++i)
    out << ",{\"name\":\"" << (stage_names + 32 * i) << "\",\"total_duration_ms\":"
        << stage_ms[i] << ",\"samples\":" << stage_runs[i] << "}";
  out << "]";
  out << "}]}";
  std::cout << out.str() << std::endl;
  if (!o.benchmark_output_path.empty()) {
    std::ofstream f(o.benchmark_output_path);
    if (!f) throw IoError("Failed to open benchmark output file: " + o.benchmark_output_path);
    f << out.str() << "\n";
  }
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    const Options o = parse(argc, argv);
    if (o.show_help) {
      std::cout << usage();
      return 0;
    }
    if (!o.benchmark_mode) {
      std::cerr << "Error: interactive mode is not available in the headless build; pass "
                   "--benchmark\n";
      return 1;
    }
    return run_benchmark(o);
  } catch (const DeviceError& e) {
    const std::string m = e.what();
    std::cerr << (m.rfind("CUDA Error", 0) == 0 ? m : "CUDA Error: " + m) << std::endl;
    return 1;
  } catch (const std::exception& e) {
    std::cerr << "Error: " << e.what() << std::endl;
    return 1;
  }
}
