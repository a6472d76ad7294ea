// Runs the drop-in adapter's classes (the reference's declarations, defined
// in nbody-gpu-sim_gb300/adapter/nbody_adapter.cpp) against the fake C ABI of
// fake_nbgb.c and prints one line per check; tests/test_adapter_runtime.py
// compares the lines.  Host arrays stand in for device arrays: the fake
// reads nothing but the count.
#include <cstdio>
#include <cstdlib>
#include <new>
#include <stdexcept>
#include <string>

#include "nbody/barnes_hut_tree.hpp"
#include "nbody/error_handling.hpp"
#include "nbody/force_calculator.hpp"
#include "nbody/integrator.hpp"

extern "C" {
const char* fake_log(void);
void fake_clear(void);
void fake_fail_next(int status, const char* msg);
}

static void show(const char* what) {
  std::printf("%s: %s\n", what, fake_log());
  fake_clear();
}

// The reference exception type a failing call raises, with its message.
template <typename F>
static void raised(const char* what, F&& f) {
  try {
    f();
    std::printf("%s: no exception\n", what);
  } catch (const nbody::ValidationException& e) {
    std::printf("%s: ValidationException|%s\n", what, e.what());
  } catch (const nbody::ResourceException& e) {
    std::printf("%s: ResourceException|%s\n", what, e.what());
  } catch (const nbody::CudaException& e) {
    std::printf("%s: CudaException|%s\n", what, e.getErrorMsg());
  } catch (const std::runtime_error& e) {
    std::printf("%s: runtime_error|%s\n", what, e.what());
  }
  fake_clear();
}

int main() {
  float buf[13][4] = {};
  nbody::ParticleData d;
  d.pos_x = buf[0];
  d.pos_y = buf[1];
  d.pos_z = buf[2];
  d.vel_x = buf[3];
  d.vel_y = buf[4];
  d.vel_z = buf[5];
  d.acc_x = buf[6];
  d.acc_y = buf[7];
  d.acc_z = buf[8];
  d.acc_old_x = buf[9];
  d.acc_old_y = buf[10];
  d.acc_old_z = buf[11];
  d.mass = buf[12];
  d.count = 4;

  // 1. one library calculator per object, released by its destructor; a new
  //    object in the same storage gets a new calculator
  alignas(nbody::BarnesHutCalculator) unsigned char store[sizeof(nbody::BarnesHutCalculator)];
  auto* a = new (store) nbody::BarnesHutCalculator(0.5f);
  a->computeForces(&d);
  a->computeForces(&d);
  a->~BarnesHutCalculator();
  auto* b = new (store) nbody::BarnesHutCalculator(0.7f);
  b->computeForces(&d);
  b->~BarnesHutCalculator();
  show("bh_lifecycle");

  // 1b. the tree the reference's tests inspect is the reference's own tree
  //     (the build's scratch allocation needs a device, which a CPU run does
  //     not have: only the calculator it asked for is checked)
  {
    nbody::BarnesHutTree tree(4);
    try {
      tree.build(&d);
    } catch (const std::exception&) {
    }
  }
  show("tree_build");

  // 2. direct calculators share one library calculator
  {
    nbody::DirectForceCalculator d1(256), d2(128);
    d1.computeForces(&d);
    d2.computeForces(&d);
  }
  show("direct_shared");

  // 3. status codes -> the reference's exception types
  nbody::SpatialHashCalculator hash(2.0f, 2.0f);
  hash.computeForces(&d);
  fake_clear();
  fake_fail_next(1, "Validation Error: Particle count must be greater than 0");
  raised("invalid_arg", [&] { hash.computeForces(&d); });
  fake_fail_next(2, "out of device memory");
  raised("oom", [&] { hash.computeForces(&d); });
  fake_fail_next(5, "Spatial hash grid exceeds 1e8 cells");
  raised("overflow", [&] { hash.computeForces(&d); });
  fake_fail_next(4, "a bounded device wait ran out of iterations");
  raised("timeout", [&] { hash.computeForces(&d); });
  fake_fail_next(7, "no CUDA device");
  raised("no_device", [&] { hash.computeForces(&d); });
  raised("recovered", [&] { hash.computeForces(&d); });

  // 4. Integrator::integrate: FP64 state (kick-drift, forces, kick), the
  //    reference's FP32 kernels with NBGB_FP32_VERLET=1, and the state
  //    released with the integrator
  {
    nbody::Integrator integ(256);
    nbody::BarnesHutCalculator calc(0.5f);
    integ.integrate(&d, &calc, 0.01f);
    integ.integrate(&d, &calc, 0.01f);
    show("integrate_fp64");
    setenv("NBGB_FP32_VERLET", "1", 1);
    integ.integrate(&d, &calc, 0.01f);
    unsetenv("NBGB_FP32_VERLET");
    show("integrate_fp32");
    std::printf("energy: %.3f\n", integ.computeTotalEnergy(&d, 1.0f, 0.1f));
    fake_fail_next(1, "Validation Error: Time step must be positive and finite");
    raised("integrate_invalid", [&] { integ.integrate(&d, &calc, 0.01f); });
  }
  show("integrator_released");
  return 0;
}
