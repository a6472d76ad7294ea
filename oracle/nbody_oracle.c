/*
 * nbody_oracle.c -- CPU restatement of the reference force-and-integrate path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA
 * library in nbody-gpu-sim_gb300/csrc.  Only tests/, __graft_entry__.smoke()
 * and the cpu_baseline / --impl reference legs of bench.py may load it.  The
 * product path never calls it and has no CPU fallback.
 *
 * Every function cites the reference file:line it restates (paths are
 * relative to the reference project root).  The restatement is pinned in
 * tests/test_oracle_pins.py against (a) the reference's own known-answer
 * tests, (b) golden fixtures generated by the reference's own host code
 * (tests/golden/make_golden.py, which drives oracle/_ref built from the
 * reference sources), and (c) the reference's host octree build run on the
 * CPU through oracle/_ref.
 *
 * Build: gcc -O2 -ffp-contract=off -fopenmp -shared -fPIC (oracle/build.py).
 * -ffp-contract=off is load-bearing: the reference's host code was built for
 * x86-64 where GCC emits no FMA, so the host octree's float bits only match
 * when no multiply-add is contracted (this matters on the aarch64 GPU host).
 *
 * Where a device-side float expression decides a discrete outcome (the
 * spatial-hash cutoff test, the Barnes-Hut opening test), the oracle spells
 * the expression with the same explicit fmaf() the CUDA kernels use, so that
 * neighbour counts and interaction lists compare bit-exactly.  The expression
 * chosen is the contraction nvcc applies to the reference's left-to-right
 * source `dx*dx + dy*dy + dz*dz`: fma(dz,dz, fma(dy,dy, dx*dx)).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_OK 0
#define ORC_ERR_ARG 1
#define ORC_ERR_OVERFLOW 5

/* ------------------------------------------------------------------------ */
/* Pairwise law                                                             */
/* ------------------------------------------------------------------------ */

/* computeGravitationalAccelerationCPU, src/cuda/force_direct.cu:109-117:
 * r = p2 - p1; dist2 = |r|^2 + eps*eps; inv = 1/sqrtf(dist2);
 * f = G*m2*inv^3; return r*f.  Vec3::length2 is x*x + y*y + z*z
 * (include/nbody/types.hpp:83-84), evaluated left to right. */
void orc_pair_accel(const float p1[3], const float p2[3], float m2, float G, float eps,
                    float out[3]) {
  float rx = p2[0] - p1[0], ry = p2[1] - p1[1], rz = p2[2] - p1[2];
  float len2 = rx * rx + ry * ry + rz * rz;
  float dist2 = len2 + eps * eps;
  float inv = 1.0f / sqrtf(dist2);
  float inv3 = inv * inv * inv;
  float f = G * m2 * inv3;
  out[0] = rx * f;
  out[1] = ry * f;
  out[2] = rz * f;
}

/* The reference host CPU path for direct forces: for each target i, sum the
 * pair function over j = 0..N-1 ascending, skipping j == i, in FP32
 * (tests/test_force_calculation.cpp:131-139 is the reference's own loop;
 * src/cuda/force_direct.cu:56-75 is the kernel it stands for).  Targets are
 * independent, so they run in parallel; the per-target order is fixed. */
void orc_direct_f32(int64_t n, const float* x, const float* y, const float* z, const float* m,
                    float G, float eps, float* ax, float* ay, float* az, int64_t i_begin,
                    int64_t i_end) {
  if (i_end > n) i_end = n;
#pragma omp parallel for schedule(static)
  for (int64_t i = i_begin; i < i_end; i++) {
    float pi[3] = {x[i], y[i], z[i]};
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    for (int64_t j = 0; j < n; j++) {
      if (j == i) continue;
      float pj[3] = {x[j], y[j], z[j]};
      float a[3];
      orc_pair_accel(pi, pj, m[j], G, eps, a);
      sx += a[0];
      sy += a[1];
      sz += a[2];
    }
    ax[i - i_begin] = sx;
    ay[i - i_begin] = sy;
    az[i - i_begin] = sz;
  }
}

/* FP64 direct sum: the accuracy oracle for every force and energy result.
 * Same law as force_direct.cu:61-73 evaluated in double precision with
 * j ascending and j == i skipped.  Inputs are the FP32 positions/masses
 * widened exactly to double (or FP64 state when given). */
void orc_direct_f64(int64_t n, const double* x, const double* y, const double* z,
                    const double* m, double G, double eps, const int64_t* targets,
                    int64_t n_targets, double* ax, double* ay, double* az) {
  double eps2 = eps * eps;
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t t = 0; t < n_targets; t++) {
    int64_t i = targets ? targets[t] : t;
    double xi = x[i], yi = y[i], zi = z[i];
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int64_t j = 0; j < n; j++) {
      if (j == i) continue;
      double dx = x[j] - xi, dy = y[j] - yi, dz = z[j] - zi;
      double d2 = dx * dx + dy * dy + dz * dz + eps2;
      double inv = 1.0 / sqrt(d2);
      double f = G * m[j] * inv * inv * inv;
      sx += f * dx;
      sy += f * dy;
      sz += f * dz;
    }
    ax[t] = sx;
    ay[t] = sy;
    az[t] = sz;
  }
}

/* ------------------------------------------------------------------------ */
/* Velocity Verlet and energies                                             */
/* ------------------------------------------------------------------------ */

/* updatePositionsKernel, src/cuda/integrator.cu:12-22:
 * x += v*dt + a*(0.5*dt*dt).  dt2_half = 0.5f*dt*dt left to right. */
void orc_update_positions(int64_t n, float* x, float* y, float* z, const float* vx,
                          const float* vy, const float* vz, const float* ax, const float* ay,
                          const float* az, float dt) {
  float dt2_half = 0.5f * dt * dt;
  for (int64_t i = 0; i < n; i++) {
    x[i] += vx[i] * dt + ax[i] * dt2_half;
    y[i] += vy[i] * dt + ay[i] * dt2_half;
    z[i] += vz[i] * dt + az[i] * dt2_half;
  }
}

/* updateVelocitiesKernel, src/cuda/integrator.cu:25-37:
 * v += (a_old + a_new) * (0.5*dt). */
void orc_update_velocities(int64_t n, float* vx, float* vy, float* vz, const float* aox,
                           const float* aoy, const float* aoz, const float* anx,
                           const float* any, const float* anz, float dt) {
  float dt_half = 0.5f * dt;
  for (int64_t i = 0; i < n; i++) {
    vx[i] += (aox[i] + anx[i]) * dt_half;
    vy[i] += (aoy[i] + any[i]) * dt_half;
    vz[i] += (aoz[i] + anz[i]) * dt_half;
  }
}

/* computeKineticEnergyKernel + host sum, src/cuda/integrator.cu:52-79,203-220:
 * KE = sum 0.5*m*|v|^2, here accumulated in double (the reference sums
 * per-block FP32 partials; the FP64 reduction is the accuracy oracle). */
double orc_kinetic_energy(int64_t n, const double* vx, const double* vy, const double* vz,
                          const double* m) {
  double ke = 0.0;
  for (int64_t i = 0; i < n; i++) ke += 0.5 * m[i] * (vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i]);
  return ke;
}

/* computePotentialEnergyKernel, src/cuda/integrator.cu:82-120:
 * PE = -sum_{i<j} G m_i m_j / sqrt(r^2 + eps^2) (Plummer potential), in double. */
double orc_potential_energy(int64_t n, const double* x, const double* y, const double* z,
                            const double* m, double G, double eps) {
  double eps2 = eps * eps;
  double pe = 0.0;
#pragma omp parallel for reduction(+ : pe) schedule(dynamic, 8)
  for (int64_t i = 0; i < n; i++) {
    double part = 0.0;
    for (int64_t j = i + 1; j < n; j++) {
      double dx = x[j] - x[i], dy = y[j] - y[i], dz = z[j] - z[i];
      part -= G * m[i] * m[j] / sqrt(dx * dx + dy * dy + dz * dz + eps2);
    }
    pe += part;
  }
  return pe;
}

/* One Velocity-Verlet step in FP64 with an FP64 direct force (the trajectory
 * oracle).  Same update order as Integrator::integrate,
 * src/cuda/integrator.cu:175-189: a_old = a; x += v dt + a dt^2/2;
 * a = F(x); v += (a_old + a) dt/2.  a must hold F(x) on entry. */
void orc_vv_step_f64(int64_t n, double* x, double* y, double* z, double* vx, double* vy,
                     double* vz, double* ax, double* ay, double* az, const double* m, double G,
                     double eps, double dt) {
  double* aox = (double*)malloc(sizeof(double) * (size_t)n * 3);
  if (!aox) return;
  double* aoy = aox + n;
  double* aoz = aoy + n;
  for (int64_t i = 0; i < n; i++) {
    aox[i] = ax[i];
    aoy[i] = ay[i];
    aoz[i] = az[i];
    x[i] += vx[i] * dt + ax[i] * (0.5 * dt * dt);
    y[i] += vy[i] * dt + ay[i] * (0.5 * dt * dt);
    z[i] += vz[i] * dt + az[i] * (0.5 * dt * dt);
  }
  orc_direct_f64(n, x, y, z, m, G, eps, NULL, n, ax, ay, az);
  for (int64_t i = 0; i < n; i++) {
    vx[i] += (aox[i] + ax[i]) * (0.5 * dt);
    vy[i] += (aoy[i] + ay[i]) * (0.5 * dt);
    vz[i] += (aoz[i] + az[i]) * (0.5 * dt);
  }
  free(aox);
}

/* ------------------------------------------------------------------------ */
/* Bounding box, Morton keys, stable sort                                   */
/* ------------------------------------------------------------------------ */

/* computeBoundingBoxKernel, src/cuda/force_barnes_hut.cu:78-122: per-axis
 * min/max seeded with +-1e30f (:18-19).  fminf/fmaxf are exact, so the
 * result is order independent. */
void orc_bbox(int64_t n, const float* x, const float* y, const float* z, float out_min[3],
              float out_max[3]) {
  float mn[3] = {1e30f, 1e30f, 1e30f}, mx[3] = {-1e30f, -1e30f, -1e30f};
  for (int64_t i = 0; i < n; i++) {
    mn[0] = fminf(mn[0], x[i]);
    mn[1] = fminf(mn[1], y[i]);
    mn[2] = fminf(mn[2], z[i]);
    mx[0] = fmaxf(mx[0], x[i]);
    mx[1] = fmaxf(mx[1], y[i]);
    mx[2] = fmaxf(mx[2], z[i]);
  }
  memcpy(out_min, mn, sizeof mn);
  memcpy(out_max, mx, sizeof mx);
}

/* expandBits, src/cuda/force_barnes_hut.cu:34-40: spread 10 bits so that
 * bit k lands on bit 3k.  Restated with shifts (same mapping). */
static uint32_t orc_spread3(uint32_t v) {
  v &= 0x3FFu;
  v = (v | (v << 16)) & 0x030000FFu;
  v = (v | (v << 8)) & 0x0300F00Fu;
  v = (v | (v << 4)) & 0x030C30C3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}

/* computeMortonCode, src/cuda/force_barnes_hut.cu:42-50: clamp each
 * normalised coordinate to [0,1] in float, scale by 1023, truncate, and
 * interleave with x in the most significant bit of each triple. */
uint32_t orc_morton_code(float nx, float ny, float nz) {
  uint32_t ix = (uint32_t)(fminf(fmaxf(nx, 0.0f), 1.0f) * 1023.0f);
  uint32_t iy = (uint32_t)(fminf(fmaxf(ny, 0.0f), 1.0f) * 1023.0f);
  uint32_t iz = (uint32_t)(fminf(fmaxf(nz, 0.0f), 1.0f) * 1023.0f);
  return (orc_spread3(ix) << 2) | (orc_spread3(iy) << 1) | orc_spread3(iz);
}

/* BarnesHutTree::computeMortonCodes + computeMortonCodesKernel,
 * src/cuda/force_barnes_hut.cu:308-322,125-139: size = max - min + 0.001f
 * per axis, inv = 1.0f/size on the host, n = (p - min)*inv; idx = iota. */
void orc_morton_keys(int64_t n, const float* x, const float* y, const float* z,
                     const float bmin[3], const float bmax[3], uint32_t* keys, int32_t* idx) {
  float sx = bmax[0] - bmin[0] + 0.001f;
  float sy = bmax[1] - bmin[1] + 0.001f;
  float sz = bmax[2] - bmin[2] + 0.001f;
  float ix = 1.0f / sx, iy = 1.0f / sy, iz = 1.0f / sz;
  for (int64_t i = 0; i < n; i++) {
    float nx = (x[i] - bmin[0]) * ix;
    float ny = (y[i] - bmin[1]) * iy;
    float nz = (z[i] - bmin[2]) * iz;
    keys[i] = orc_morton_code(nx, ny, nz);
    idx[i] = (int32_t)i;
  }
}

/* thrust::sort_by_key on (u32 key, i32 value), src/cuda/force_barnes_hut.cu:324-328.
 * Thrust sorts primitive keys with a stable LSD radix sort, so equal keys keep
 * their input (index) order.  Restated as an LSD counting sort, 8 bits/pass. */
int orc_stable_sort_u32(int64_t n, uint32_t* keys, int32_t* vals) {
  uint32_t* k2 = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(n ? n : 1));
  int32_t* v2 = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n ? n : 1));
  if (!k2 || !v2) {
    free(k2);
    free(v2);
    return ORC_ERR_ARG;
  }
  for (int shift = 0; shift < 32; shift += 8) {
    int64_t cnt[257];
    memset(cnt, 0, sizeof cnt);
    for (int64_t i = 0; i < n; i++) cnt[((keys[i] >> shift) & 0xFFu) + 1]++;
    for (int d = 0; d < 256; d++) cnt[d + 1] += cnt[d];
    for (int64_t i = 0; i < n; i++) {
      int64_t p = cnt[(keys[i] >> shift) & 0xFFu]++;
      k2[p] = keys[i];
      v2[p] = vals[i];
    }
    memcpy(keys, k2, sizeof(uint32_t) * (size_t)n);
    memcpy(vals, v2, sizeof(int32_t) * (size_t)n);
  }
  free(k2);
  free(v2);
  return ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Barnes-Hut octree (host insertion build)                                 */
/* ------------------------------------------------------------------------ */

/* OctreeNode, include/nbody/barnes_hut_tree.hpp:9-30; 76 bytes, offsets
 * center 0, half 12, com 16, mass 28, children 32, particle_index 64,
 * is_leaf 68, particle_count 72.  Default: zeros, children -1,
 * particle_index -1, is_leaf true (:19-29). */
typedef struct {
  float cx, cy, cz;
  float half;
  float comx, comy, comz;
  float mass;
  int32_t children[8];
  int32_t particle_index;
  uint8_t is_leaf;
  uint8_t pad_[3];
  int32_t particle_count;
} orc_node;

#define ORC_BH_MAX_DEPTH 32 /* force_barnes_hut.cu:24 */

int orc_node_size(void) { return (int)sizeof(orc_node); }

static void orc_node_default(orc_node* n) {
  memset(n, 0, sizeof *n);
  for (int c = 0; c < 8; c++) n->children[c] = -1;
  n->particle_index = -1;
  n->is_leaf = 1;
}

/* octantOf, force_barnes_hut.cu:339-348. */
static int orc_octant(float px, float py, float pz, const orc_node* c) {
  int o = 0;
  if (px >= c->cx) o |= 1;
  if (py >= c->cy) o |= 2;
  if (pz >= c->cz) o |= 4;
  return o;
}

/* mergeParticleIntoLeaf, force_barnes_hut.cu:355-365. */
static void orc_merge(orc_node* n, int32_t pidx, float px, float py, float pz, float m) {
  float total = n->mass + m;
  float cx = (n->comx * n->mass + px * m) / total;
  float cy = (n->comy * n->mass + py * m) / total;
  float cz = (n->comz * n->mass + pz * m) / total;
  n->comx = cx;
  n->comy = cy;
  n->comz = cz;
  n->mass = total;
  n->particle_count += 1;
  if (n->particle_index < 0) n->particle_index = pidx;
}

/* allocateLeaf, force_barnes_hut.cu:368-389.  Returns -1 when the node
 * array is full (the reference would write past its vector). */
static int orc_alloc_leaf(orc_node* nodes, int64_t max_nodes, int* count, int parent, int oct,
                          int32_t pidx, float px, float py, float pz, float m) {
  if ((int64_t)*count >= max_nodes) return -1;
  int ni = (*count)++;
  orc_node* p = &nodes[parent];
  p->children[oct] = ni;
  p->is_leaf = 0;
  float hs = p->half * 0.5f;
  orc_node* c = &nodes[ni];
  orc_node_default(c);
  c->cx = p->cx + ((oct & 1) ? hs : -hs);
  c->cy = p->cy + ((oct & 2) ? hs : -hs);
  c->cz = p->cz + ((oct & 4) ? hs : -hs);
  c->half = hs;
  c->is_leaf = 1;
  c->particle_index = pidx;
  c->particle_count = 1;
  c->mass = m;
  c->comx = px;
  c->comy = py;
  c->comz = pz;
  return ni;
}

/* BarnesHutTree::buildTreeOnHost, force_barnes_hut.cu:391-543: root cube
 * from the unpadded bbox (:418-422), sequential insertion in the given
 * (Morton-sorted) order with leaf splitting (:431-510), node-budget merge
 * when node_count + 33 >= max_nodes (:449-453), depth-32 merge (:490-507),
 * then the bottom-up centre-of-mass pass in descending node index with
 * children in octant order (:514-538).  max_nodes is 2N in the reference
 * (:253).  Returns ORC_ERR_OVERFLOW if the node array would overflow. */
int orc_build_octree(int64_t n, const float* x, const float* y, const float* z, const float* m,
                     const int32_t* sorted_idx, const float bmin[3], const float bmax[3],
                     orc_node* nodes, int64_t max_nodes, int* node_count_out, int* max_depth_out,
                     int64_t* budget_merges_out) {
  if (max_nodes < 1) return ORC_ERR_ARG;
  for (int64_t i = 0; i < max_nodes; i++) orc_node_default(&nodes[i]);
  orc_node* root = &nodes[0];
  root->cx = (bmin[0] + bmax[0]) * 0.5f;
  root->cy = (bmin[1] + bmax[1]) * 0.5f;
  root->cz = (bmin[2] + bmax[2]) * 0.5f;
  float ex = bmax[0] - bmin[0], ey = bmax[1] - bmin[1], ez = bmax[2] - bmin[2];
  /* std::max({ex, ey, ez}) returns the first largest element. */
  float max_size = ex;
  if (max_size < ey) max_size = ey;
  if (max_size < ez) max_size = ez;
  root->half = max_size * 0.5f + 0.001f;
  root->is_leaf = 0;
  root->particle_index = -1;
  root->particle_count = (int32_t)n;
  int count = 1, max_depth = 0;
  int64_t budget_merges = 0;

  for (int64_t i = 0; i < n; i++) {
    int32_t idx = sorted_idx[i];
    float px = x[idx], py = y[idx], pz = z[idx], pm = m[idx];
    int current = 0, depth = 0, merged = 0;
    while (depth < ORC_BH_MAX_DEPTH) {
      orc_node* node = &nodes[current];
      if (node->is_leaf) {
        if ((int64_t)count + ORC_BH_MAX_DEPTH + 1 >= max_nodes) {
          orc_merge(node, idx, px, py, pz, pm);
          merged = 1;
          budget_merges++;
          break;
        }
        int32_t e_idx = node->particle_index;
        float ex_ = node->comx, ey_ = node->comy, ez_ = node->comz, em = node->mass;
        node->is_leaf = 0;
        node->particle_index = -1;
        node->particle_count = 0;
        node->mass = 0.0f;
        node->comx = node->comy = node->comz = 0.0f;
        int eo = orc_octant(ex_, ey_, ez_, node);
        if (node->children[eo] < 0) {
          if (orc_alloc_leaf(nodes, max_nodes, &count, current, eo, e_idx, ex_, ey_, ez_, em) < 0)
            return ORC_ERR_OVERFLOW;
        }
      }
      int oct = orc_octant(px, py, pz, node);
      int child = node->children[oct];
      if (child < 0) {
        if (orc_alloc_leaf(nodes, max_nodes, &count, current, oct, idx, px, py, pz, pm) < 0)
          return ORC_ERR_OVERFLOW;
        break;
      }
      current = child;
      depth++;
    }
    if (!merged && depth >= ORC_BH_MAX_DEPTH) {
      int leaf = current;
      while (!nodes[leaf].is_leaf) {
        for (int c = 0; c < 8; c++) {
          if (nodes[leaf].children[c] >= 0) {
            leaf = nodes[leaf].children[c];
            break;
          }
        }
      }
      orc_merge(&nodes[leaf], idx, px, py, pz, pm);
    }
    if (depth > max_depth) max_depth = depth;
  }

  for (int i = count - 1; i >= 0; i--) {
    orc_node* nd = &nodes[i];
    if (nd->is_leaf) continue;
    float tm = 0.0f, cx = 0.0f, cy = 0.0f, cz = 0.0f;
    int32_t cnt = 0;
    for (int c = 0; c < 8; c++) {
      int ci = nd->children[c];
      if (ci >= 0) {
        const orc_node* ch = &nodes[ci];
        tm += ch->mass;
        cx += ch->comx * ch->mass;
        cy += ch->comy * ch->mass;
        cz += ch->comz * ch->mass;
        cnt += ch->particle_count;
      }
    }
    nd->mass = tm;
    nd->particle_count = cnt;
    if (tm > 0.0f) {
      nd->comx = cx / tm;
      nd->comy = cy / tm;
      nd->comz = cz / tm;
    }
  }
  *node_count_out = count;
  *max_depth_out = max_depth;
  if (budget_merges_out) *budget_merges_out = budget_merges;
  return ORC_OK;
}

/* barnesHutForceKernel, force_barnes_hut.cu:142-249, one target at a time:
 * DFS with an explicit stack (children pushed in octant order 0..7, popped
 * last-first), contains_i test (:180-182), leaf self-subtraction
 * (:190-200), opening test !contains_i && 4h^2/(d^2+eps^2) < theta^2
 * (:218-224), stack guard sp+8 <= 256 (:234).  rsqrtf is replaced by
 * 1/sqrtf on the CPU; the opening test uses the contracted distance
 * expression shared with the CUDA walk (see file header).  Optionally
 * reports the number of accepted interactions per target.
 *
 * leaf_cap > 1 walks the same tree with every subtree of at most leaf_cap
 * bodies collapsed into one bucket (the bucket variant of the reference
 * walk; the reference itself has leaf_cap 1): an internal bucket node that
 * fails the opening test is replaced by the direct sum over its bodies in
 * octant order, skipping the target itself by index.  Returns ORC_ERR_ARG
 * when a bucket holds a multi-body (depth-32) leaf, whose bodies the node
 * records do not list. */
int orc_bh_forces(const orc_node* nodes, int num_nodes, int64_t n, const float* x,
                  const float* y, const float* z, const float* m, float theta, float G,
                  float eps, const int64_t* targets, int64_t n_targets, float* ax, float* ay,
                  float* az, int32_t* interactions, int leaf_cap) {
  float theta2 = theta * theta;
  float eps2 = eps * eps;
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(| : bad)
  for (int64_t t = 0; t < n_targets; t++) {
    int64_t i = targets ? targets[t] : t;
    float xi = x[i], yi = y[i], zi = z[i], mi = m[i];
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    int32_t inter = 0;
    int stack[256];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
      int ni = stack[--sp];
      if (ni < 0 || ni >= num_nodes) continue;
      const orc_node* nd = &nodes[ni];
      if (nd->mass == 0.0f) continue;
      int contains = fabsf(xi - nd->cx) <= nd->half && fabsf(yi - nd->cy) <= nd->half &&
                     fabsf(zi - nd->cz) <= nd->half;
      if (nd->is_leaf) {
        float me = nd->mass, cx = nd->comx, cy = nd->comy, cz = nd->comz;
        if (contains) {
          me -= mi;
          if (me <= 0.0f) continue;
          cx = (cx * nd->mass - xi * mi) / me;
          cy = (cy * nd->mass - yi * mi) / me;
          cz = (cz * nd->mass - zi * mi) / me;
        }
        float dx = cx - xi, dy = cy - yi, dz = cz - zi;
        float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx)) + eps2;
        float inv = 1.0f / sqrtf(d2);
        float f = G * me * (inv * inv * inv);
        sx += f * dx;
        sy += f * dy;
        sz += f * dz;
        inter++;
        continue;
      }
      float dx = nd->comx - xi, dy = nd->comy - yi, dz = nd->comz - zi;
      float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx)) + eps2;
      float size2 = 4.0f * nd->half * nd->half;
      if (!contains && size2 / d2 < theta2) {
        float inv = 1.0f / sqrtf(d2);
        float f = G * nd->mass * (inv * inv * inv);
        sx += f * dx;
        sy += f * dy;
        sz += f * dz;
        inter++;
      } else if (leaf_cap > 1 && nd->particle_count <= leaf_cap) {
        int bst[64];
        int bp = 0;
        bst[bp++] = ni;
        while (bp > 0) {
          const orc_node* b = &nodes[bst[--bp]];
          if (!b->is_leaf) {
            for (int c = 7; c >= 0; c--)
              if (b->children[c] >= 0 && bp < 64) bst[bp++] = b->children[c];
            continue;
          }
          if (b->particle_count != 1) {
            bad = 1;
            continue;
          }
          int64_t j = b->particle_index;
          if (j == i) continue;
          float ex = x[j] - xi, ey = y[j] - yi, ez = z[j] - zi;
          float e2 = fmaf(ez, ez, fmaf(ey, ey, ex * ex)) + eps2;
          float inv = 1.0f / sqrtf(e2);
          float f = G * m[j] * (inv * inv * inv);
          sx += f * ex;
          sy += f * ey;
          sz += f * ez;
          inter++;
        }
      } else if (sp + 8 <= 256) {
        for (int c = 0; c < 8; c++)
          if (nd->children[c] >= 0) stack[sp++] = nd->children[c];
      }
    }
    ax[t] = sx;
    ay[t] = sy;
    az[t] = sz;
    if (interactions) interactions[t] = inter;
  }
  return bad ? ORC_ERR_ARG : ORC_OK;
}

/* Group walk (the library's NBGB_FLAG_GROUP_WALK; the reference has no
 * such walk -- it restates the same tree and opening quantities, see
 * orc_bh_forces above).  Groups: the root if it holds at most group_max
 * bodies (32 or 64, the library's choice for the build's body count);
 * below a larger node, runs of consecutive children (octant order) holding
 * at most group_max bodies in total, merged only when the parent holds at
 * most 1024 bodies; a child of more than group_max bodies ends the run.  The group's box is
 * its bounding box as a centre b = (lo + hi) * 0.5 and half sizes
 * max(hi - b, b - lo) * (1 + 2^-22).  Each group walks the tree once from the
 * root: a node of zero mass is skipped, a leaf adds its body, an internal
 * node is accepted (its centre of mass added) unless its cube touches the
 * box (|c - b| <= h + half on every axis) and when
 * 4h^2 < theta^2 * fma(dz,dz, fma(dy,dy, fma(dx,dx, eps^2))), d the per-axis
 * distance max(|com - b| - half, 0) of the centre of mass outside the box;
 * otherwise its children are walked.  Every body of the group sums the whole list;
 * interactions per body = list length minus its own leaf.  With leaf_cap > 1
 * an internal node of at most leaf_cap bodies that is not accepted adds its
 * bodies (in octant order) instead of its children.  With eps = 0 a
 * zero-distance entry adds nothing.  Multi-body (depth-32) leaves are not
 * supported here (their bodies are not listed in the node records):
 * returns ORC_ERR_ARG. */
#define ORC_GROUP 64
#define ORC_GROUP_MERGE 1024

typedef struct {
  int nmem;
  int mem[8];
} orc_group;

/* Bodies of the subtree at ni in octant (path) order, at most cap. */
static void orc_subtree_bodies(const orc_node* nodes, int ni, int* out, int* nb, int cap,
                               int* bad) {
  const orc_node* nd = &nodes[ni];
  if (nd->is_leaf) {
    if (nd->particle_count != 1 || *nb >= cap) {
      *bad = 1;
      return;
    }
    out[(*nb)++] = nd->particle_index;
    return;
  }
  for (int c = 0; c < 8; c++)
    if (nd->children[c] >= 0) orc_subtree_bodies(nodes, nd->children[c], out, nb, cap, bad);
}

static void orc_group_bodies(const orc_node* nodes, int ni, int* out, int* nb, int cap, int* bad) {
  orc_subtree_bodies(nodes, ni, out, nb, cap, bad);
}

int orc_bh_group_forces(const orc_node* nodes, int num_nodes, int64_t n, const float* x,
                        const float* y, const float* z, const float* m, float theta, float G,
                        float eps, float* ax, float* ay, float* az, int32_t* interactions,
                        int leaf_cap, int group_max) {
  if (num_nodes < 1 || group_max < 1 || group_max > ORC_GROUP) return ORC_ERR_ARG;
  /* groups, by a pre-order pass over the nodes of more than ORC_GROUP bodies */
  orc_group* groups = (orc_group*)malloc(sizeof(orc_group) * (size_t)(n + 1));
  int* st = (int*)malloc(sizeof(int) * (size_t)(num_nodes + 8));
  int64_t ng = 0;
  int bad = 0, sp = 0;
  if (nodes[0].particle_count <= group_max) {
    groups[ng].nmem = 1;
    groups[ng++].mem[0] = 0;
  } else {
    st[sp++] = 0;
  }
  while (sp > 0) {
    const orc_node* nd = &nodes[st[--sp]];
    if (nd->is_leaf) {
      bad = 1; /* a leaf of more than group_max bodies */
      continue;
    }
    int merge = nd->particle_count <= ORC_GROUP_MERGE, gn = 0;
    for (int c = 0; c < 8; c++) {
      int ch = nd->children[c];
      if (ch < 0) continue;
      int cc = nodes[ch].particle_count;
      if (cc > group_max) {
        gn = 0;
        st[sp++] = ch;
      } else if (gn && merge && gn + cc <= group_max) {
        groups[ng - 1].mem[groups[ng - 1].nmem++] = ch;
        gn += cc;
      } else {
        groups[ng].nmem = 1;
        groups[ng++].mem[0] = ch;
        gn = cc;
      }
    }
  }
  free(st);
  float theta2 = theta * theta, eps2 = eps * eps;
#pragma omp parallel for schedule(dynamic, 16) reduction(| : bad)
  for (int64_t g = 0; g < ng; g++) {
    int body[ORC_GROUP], nb = 0, gbad = 0;
    for (int j = 0; j < groups[g].nmem; j++)
      orc_group_bodies(nodes, groups[g].mem[j], body, &nb, group_max, &gbad);
    if (gbad) {
      bad = 1;
      continue;
    }
    float lo[3] = {x[body[0]], y[body[0]], z[body[0]]}, hi[3] = {lo[0], lo[1], lo[2]};
    for (int j = 1; j < nb; j++) {
      const float p[3] = {x[body[j]], y[body[j]], z[body[j]]};
      for (int a = 0; a < 3; a++) {
        if (p[a] < lo[a]) lo[a] = p[a];
        if (p[a] > hi[a]) hi[a] = p[a];
      }
    }
    float bc[3], bh[3];
    for (int a = 0; a < 3; a++) {
      bc[a] = (lo[a] + hi[a]) * 0.5f;
      bh[a] = fmaxf(hi[a] - bc[a], bc[a] - lo[a]) * 0x1.000004p0f;
    }
    /* interaction list */
    int cap = 4096, len = 0, own[ORC_GROUP] = {0};
    float* list = (float*)malloc(sizeof(float) * 4 * (size_t)cap);
    int stk[512]; /* depth-first: at most 7 pending siblings per level, depth <= 32 */
    int s = 0;
    stk[s++] = 0;
    while (s > 0) {
      const orc_node* nd = &nodes[stk[--s]];
      if (nd->mass == 0.0f) continue;
      int entry = 0;
      if (nd->is_leaf) {
        entry = 1;
        for (int j = 0; j < nb; j++)
          if (body[j] == nd->particle_index) own[j] = 1;
      } else {
        int overlap = fabsf(nd->cx - bc[0]) <= nd->half + bh[0] &&
                      fabsf(nd->cy - bc[1]) <= nd->half + bh[1] &&
                      fabsf(nd->cz - bc[2]) <= nd->half + bh[2];
        float dx = fmaxf(fabsf(nd->comx - bc[0]) - bh[0], 0.0f);
        float dy = fmaxf(fabsf(nd->comy - bc[1]) - bh[1], 0.0f);
        float dz = fmaxf(fabsf(nd->comz - bc[2]) - bh[2], 0.0f);
        float d2 = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, eps2)));
        float size2 = 4.0f * nd->half * nd->half;
        entry = !overlap && size2 < theta2 * d2;
        if (!entry && leaf_cap > 1 && nd->particle_count <= leaf_cap) {
          /* an opened bucket: its bodies join the list */
          int bb[16], nbb = 0;
          orc_subtree_bodies(nodes, (int)(nd - nodes), bb, &nbb, 16, &bad);
          for (int q = 0; q < nbb; q++) {
            if (len == cap) {
              cap *= 2;
              list = (float*)realloc(list, sizeof(float) * 4 * (size_t)cap);
            }
            list[4 * len] = x[bb[q]];
            list[4 * len + 1] = y[bb[q]];
            list[4 * len + 2] = z[bb[q]];
            list[4 * len + 3] = m[bb[q]];
            len++;
            for (int j = 0; j < nb; j++)
              if (body[j] == bb[q]) own[j] = 1;
          }
          continue;
        }
        if (!entry) {
          if (s + 8 > 512) {
            bad = 1;
            continue;
          }
          for (int c = 7; c >= 0; c--)
            if (nd->children[c] >= 0) stk[s++] = nd->children[c];
        }
      }
      if (entry) {
        if (len == cap) {
          cap *= 2;
          list = (float*)realloc(list, sizeof(float) * 4 * (size_t)cap);
        }
        list[4 * len] = nd->comx;
        list[4 * len + 1] = nd->comy;
        list[4 * len + 2] = nd->comz;
        list[4 * len + 3] = nd->mass;
        len++;
      }
    }
    for (int j = 0; j < nb; j++) {
      int i = body[j];
      float sx = 0.0f, sy = 0.0f, sz = 0.0f;
      for (int e = 0; e < len; e++) {
        float ex = list[4 * e] - x[i], ey = list[4 * e + 1] - y[i], ez = list[4 * e + 2] - z[i];
        float e2 = fmaf(ez, ez, fmaf(ey, ey, ex * ex)) + eps2;
        if (e2 == 0.0f) continue;
        float inv = 1.0f / sqrtf(e2);
        float f = list[4 * e + 3] * (inv * inv * inv);
        sx += f * ex;
        sy += f * ey;
        sz += f * ez;
      }
      ax[i] = G * sx;
      ay[i] = G * sy;
      az[i] = G * sz;
      if (interactions) interactions[i] = len - own[j];
    }
    free(list);
  }
  free(groups);
  return bad ? ORC_ERR_ARG : ORC_OK;
}

/* ------------------------------------------------------------------------ */
/* Spatial hash                                                             */
/* ------------------------------------------------------------------------ */

/* SpatialHashGrid::computeBoundingBox + build dims,
 * src/cuda/force_spatial_hash.cu:190-239,249-261: bbox padded by 0.001f,
 * dims = (int)ceilf((max-min)/cell) + 1, cap of 1e8 cells.  Returns the
 * padded box in bmin/bmax and ORC_ERR_OVERFLOW above the cap. */
int orc_hash_dims(int64_t n, const float* x, const float* y, const float* z, float cell,
                  float bmin[3], float bmax[3], int dims[3], int64_t* total_cells) {
  orc_bbox(n, x, y, z, bmin, bmax);
  for (int a = 0; a < 3; a++) {
    bmin[a] -= 0.001f;
    bmax[a] += 0.001f;
  }
  for (int a = 0; a < 3; a++) dims[a] = (int)ceilf((bmax[a] - bmin[a]) / cell) + 1;
  int64_t tot = (int64_t)dims[0] * dims[1] * dims[2];
  *total_cells = tot;
  return tot > 100000000 ? ORC_ERR_OVERFLOW : ORC_OK;
}

/* Cell coordinates before the clamp: floor((p - min) / cell) per axis with
 * IEEE division (assignCellsKernel, force_spatial_hash.cu:36-42; with
 * min = 0 this is SpatialHashGrid::getCellIndex, :15-18). */
void orc_cell_coords(float px, float py, float pz, const float bmin[3], float cell,
                     int32_t out[3]) {
  out[0] = (int32_t)floorf((px - bmin[0]) / cell);
  out[1] = (int32_t)floorf((py - bmin[1]) / cell);
  out[2] = (int32_t)floorf((pz - bmin[2]) / cell);
}

/* assignCellsKernel, force_spatial_hash.cu:29-50: the coordinates above,
 * clamped to the grid, linear id x + y*gx + z*gx*gy. */
static int32_t orc_cell_of(float px, float py, float pz, const float bmin[3], float cell,
                           const int dims[3]) {
  int32_t c3[3];
  orc_cell_coords(px, py, pz, bmin, cell, c3);
  int cx = c3[0], cy = c3[1], cz = c3[2];
  cx = cx < 0 ? 0 : (cx > dims[0] - 1 ? dims[0] - 1 : cx);
  cy = cy < 0 ? 0 : (cy > dims[1] - 1 ? dims[1] - 1 : cy);
  cz = cz < 0 ? 0 : (cz > dims[2] - 1 ? dims[2] - 1 : cz);
  return cx + cy * dims[0] + cz * dims[0] * dims[1];
}

/* SpatialHashGrid::build, force_spatial_hash.cu:241-309: assign, count,
 * exclusive scan -> cell_start, end = start + count, scatter.  The reference
 * scatter order within a cell comes from atomicAdd (non-deterministic,
 * :79); the oracle fixes it to ascending particle index, which is also the
 * order the CUDA build produces.  Compare per-cell sets against the
 * reference, and exact order against the CUDA build. */
int orc_hash_build(int64_t n, const float* x, const float* y, const float* z, float cell,
                   const float bmin[3], const int dims[3], int32_t* particle_cell,
                   int32_t* cell_start, int32_t* cell_end, int32_t* sorted_indices) {
  int64_t tot = (int64_t)dims[0] * dims[1] * dims[2];
  for (int64_t c = 0; c < tot; c++) cell_start[c] = 0;
  for (int64_t i = 0; i < n; i++) {
    particle_cell[i] = orc_cell_of(x[i], y[i], z[i], bmin, cell, dims);
    cell_start[particle_cell[i]]++;
  }
  int64_t run = 0;
  for (int64_t c = 0; c < tot; c++) {
    int64_t cnt = cell_start[c];
    cell_start[c] = (int32_t)run;
    cell_end[c] = (int32_t)(run + cnt);
    run += cnt;
  }
  /* stable scatter: slot = start + rank among earlier particles of the cell */
  int32_t* fill = (int32_t*)malloc(sizeof(int32_t) * (size_t)(tot ? tot : 1));
  if (!fill) return ORC_ERR_ARG;
  memcpy(fill, cell_start, sizeof(int32_t) * (size_t)tot);
  for (int64_t i = 0; i < n; i++) sorted_indices[fill[particle_cell[i]]++] = (int32_t)i;
  free(fill);
  return ORC_OK;
}

/* spatialHashForceKernel, force_spatial_hash.cu:84-158: target cell with the
 * same clamp, 27 neighbours in dz, dy, dx order (no wrap), skip j == i,
 * accept if the unsoftened d^2 < cutoff^2, then add G m_j d (d^2+eps^2)^-3/2.
 * neighbours[t] counts accepted pairs (compared bit-exactly with the CUDA
 * kernel, which evaluates the same contracted d^2). */
void orc_hash_forces(int64_t n, const float* x, const float* y, const float* z, const float* m,
                     float cell, const float bmin[3], const int dims[3],
                     const int32_t* cell_start, const int32_t* cell_end,
                     const int32_t* sorted_indices, float cutoff, float G, float eps,
                     const int64_t* targets, int64_t n_targets, float* ax, float* ay, float* az,
                     int32_t* neighbours) {
  float cut2 = cutoff * cutoff;
  float eps2 = eps * eps;
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t t = 0; t < n_targets; t++) {
    int64_t i = targets ? targets[t] : t;
    float xi = x[i], yi = y[i], zi = z[i];
    int cx = (int)floorf((xi - bmin[0]) / cell);
    int cy = (int)floorf((yi - bmin[1]) / cell);
    int cz = (int)floorf((zi - bmin[2]) / cell);
    cx = cx < 0 ? 0 : (cx > dims[0] - 1 ? dims[0] - 1 : cx);
    cy = cy < 0 ? 0 : (cy > dims[1] - 1 ? dims[1] - 1 : cy);
    cz = cz < 0 ? 0 : (cz > dims[2] - 1 ? dims[2] - 1 : cz);
    float sx = 0.0f, sy = 0.0f, sz = 0.0f;
    int32_t acc = 0;
    for (int oz = -1; oz <= 1; oz++)
      for (int oy = -1; oy <= 1; oy++)
        for (int ox = -1; ox <= 1; ox++) {
          int nx = cx + ox, ny = cy + oy, nz = cz + oz;
          if (nx < 0 || nx >= dims[0] || ny < 0 || ny >= dims[1] || nz < 0 || nz >= dims[2])
            continue;
          int64_t c = nx + (int64_t)ny * dims[0] + (int64_t)nz * dims[0] * dims[1];
          for (int32_t k = cell_start[c]; k < cell_end[c]; k++) {
            int32_t j = sorted_indices[k];
            if (j == i) continue;
            float dx = x[j] - xi, dy = y[j] - yi, dz = z[j] - zi;
            float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
            if (d2 < cut2) {
              d2 += eps2;
              float inv = 1.0f / sqrtf(d2);
              float f = G * m[j] * (inv * inv * inv);
              sx += f * dx;
              sy += f * dy;
              sz += f * dz;
              acc++;
            }
          }
        }
    ax[t] = sx;
    ay[t] = sy;
    az[t] = sz;
    if (neighbours) neighbours[t] = acc;
  }
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Threads of the OpenMP loops above (timing on one core vs all cores). */
void orc_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
