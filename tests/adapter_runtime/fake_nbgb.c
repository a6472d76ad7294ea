/* A stand-in for libnbgb.so with the entry points the drop-in adapter calls
 * (nbody-gpu-sim_gb300/adapter/nbody_adapter.cpp), for a CPU test of the
 * adapter's own logic: the per-object calculator handles, the mapping of
 * status codes to the reference's exceptions, and the call sequence of
 * Integrator::integrate.  Every call is appended to a log; fake_fail_next()
 * makes the next status-returning call fail with a given status and text.
 * No device work happens here. */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "nbgb.h"

struct nbgb_calculator {
  int id;
  int method;
};

static char g_log[16384];
static char g_err[512];
static int g_next_id = 1;
static int g_fail_status = 0;
static char g_fail_msg[512];

static void note(const char* fmt, ...) {
  char e[96];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(e, sizeof e, fmt, ap);
  va_end(ap);
  if (strlen(g_log) + strlen(e) + 2 < sizeof g_log) {
    strcat(g_log, e);
    strcat(g_log, " ");
  }
}

/* The status of the current call: a planted failure once, else success. */
static nbgb_status result(void) {
  if (g_fail_status) {
    nbgb_status s = (nbgb_status)g_fail_status;
    g_fail_status = 0;
    snprintf(g_err, sizeof g_err, "%s", g_fail_msg);
    return s;
  }
  g_err[0] = 0;
  return NBGB_OK;
}

const char* fake_log(void) { return g_log; }
void fake_clear(void) { g_log[0] = 0; }
void fake_fail_next(int status, const char* msg) {
  g_fail_status = status;
  snprintf(g_fail_msg, sizeof g_fail_msg, "%s", msg);
}

const char* nbgb_last_error(void) { return g_err; }

void nbgb_params_default(nbgb_params* p) {
  memset(p, 0, sizeof *p);
  p->G = 1.0f;
  p->softening = 0.1f;
  p->theta = 0.5f;
  p->cell_size = 2.0f;
  p->cutoff = 2.0f;
  p->block_size = 256;
  p->leaf_capacity = 1;
  p->flags = NBGB_FLAG_SYNC | NBGB_FLAG_COMPENSATED;
}

nbgb_status nbgb_calculator_create(nbgb_method method, const nbgb_params* params,
                                   nbgb_calculator** out) {
  nbgb_status s = result();
  if (s != NBGB_OK) return s;
  nbgb_calculator* c = (nbgb_calculator*)malloc(sizeof *c);
  c->id = g_next_id++;
  c->method = (int)method;
  *out = c;
  if (params->flags & NBGB_FLAG_REFERENCE_TREE)
    note("create:%d:%d:reftree", c->method, c->id);
  else
    note("create:%d:%d", c->method, c->id);
  return s;
}

nbgb_status nbgb_calculator_destroy(nbgb_calculator* calc) {
  note("destroy:%d", calc ? calc->id : -1);
  free(calc);
  return NBGB_OK;
}

nbgb_status nbgb_calculator_set_params(nbgb_calculator* calc, const nbgb_params* params) {
  (void)params;
  note("set_params:%d", calc->id);
  return result();
}

nbgb_status nbgb_compute_forces(nbgb_calculator* calc, const nbgb_particle_data* d) {
  note("compute:%d:%d", calc->id, (int)d->count);
  return result();
}

nbgb_status nbgb_bh_tree_stats(nbgb_calculator* calc, int32_t* node_count, int32_t* max_depth) {
  (void)calc;
  *node_count = 0;
  *max_depth = 0;
  return result();
}

nbgb_status nbgb_bh_copy_nodes(nbgb_calculator* calc, nbgb_octree_node* nodes, size_t capacity) {
  (void)calc;
  (void)nodes;
  (void)capacity;
  return result();
}

nbgb_status nbgb_hash_grid_info(nbgb_calculator* calc, int32_t dims[3], float bbox_min[3],
                                float* cell_size, int64_t* total_cells) {
  (void)calc;
  dims[0] = dims[1] = dims[2] = 0;
  bbox_min[0] = bbox_min[1] = bbox_min[2] = 0.f;
  *cell_size = 0.f;
  *total_cells = 0;
  return result();
}

nbgb_status nbgb_hash_copy_cells(nbgb_calculator* calc, int32_t* cell_start, int32_t* cell_end,
                                 int32_t* particle_cells, int32_t* sorted_indices) {
  (void)calc;
  (void)cell_start;
  (void)cell_end;
  (void)particle_cells;
  (void)sorted_indices;
  return result();
}

nbgb_status nbgb_update_positions(const nbgb_particle_data* d, float dt, void* stream) {
  (void)d;
  (void)dt;
  (void)stream;
  note("update_positions");
  return result();
}

nbgb_status nbgb_update_velocities(const nbgb_particle_data* d, float dt, void* stream) {
  (void)d;
  (void)dt;
  (void)stream;
  note("update_velocities");
  return result();
}

nbgb_status nbgb_store_old_accelerations(const nbgb_particle_data* d, void* stream) {
  (void)d;
  (void)stream;
  note("store_old");
  return result();
}

nbgb_status nbgb_state_kick_drift(const nbgb_particle_data* d, float dt, void* stream) {
  (void)dt;
  (void)stream;
  note("kick_drift:%d", (int)d->count);
  return result();
}

nbgb_status nbgb_state_kick(const nbgb_particle_data* d, float dt, void* stream) {
  (void)dt;
  (void)stream;
  note("kick:%d", (int)d->count);
  return result();
}

nbgb_status nbgb_state_release(const nbgb_particle_data* d) {
  note("release:%d", (int)d->count);
  return NBGB_OK;
}

nbgb_status nbgb_kinetic_energy(const nbgb_particle_data* d, double* ke, void* stream) {
  (void)d;
  (void)stream;
  *ke = 1.5;
  return result();
}

nbgb_status nbgb_potential_energy(const nbgb_particle_data* d, float G, float eps, double* pe,
                                  void* stream) {
  (void)d;
  (void)G;
  (void)eps;
  (void)stream;
  *pe = -2.0;
  return result();
}
