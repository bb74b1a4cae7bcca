// The fused DiReBM step on a dense cell grid: device-side data structures and helpers.
//
// Geometry: a batch of instances, each a box of dims[0] x dims[1] (x dims[2]) cells of size
// `cell` (the thinning cell).  Cells of all instances are numbered globally, instance by
// instance, row-major (x fastest) inside each.  A moment is (global cell, offset in [0,1)^D in
// cell units) and the moments are kept sorted by global cell, with start[c] .. start[c+1] the
// moments of cell c -- the "hash grid built from sorted cell ranges", exact (no aliasing) because
// the grid is dense.  Components are never materialised: the component of moment m in direction
// k sits at S + off + cd_k (cd_k = c_k*dx/cell) and every kernel recomputes it with the same
// round-to-nearest operations, so each (m, k) makes the same integer decisions everywhere.
#pragma once

#include <type_traits>

#include "lattice.cuh"

namespace dbm {

struct InstK {
  uint32_t base;     // first global cell
  int32_t dims[3];
  int32_t origin[3];
  int32_t periodic;
  double tau;
  double rho_rest;
  int32_t has_obs;   // a solid sphere (disc in 2D) with bounce-back
  int32_t inflow_w;  // inflow layer: moments in local cell columns x < inflow_w are set to feq(rho, u_in)
  double obs_c[3];   // sphere center, instance-local cell units
  double obs_r2;     // squared radius, cell units
  double u_in[3];
  float near2;       // squared distance from the center beyond which no direction of a moment can be blocked
  float reach2;      // squared distance beyond which no bounced component lies within r of a point
};

struct PF64 {
  using real = double;
  static constexpr int id = DBM_FP64;
};
struct PF32 {
  using real = float;
  static constexpr int id = DBM_FP32DEV;
};

// A moment (or control point) packed for the untiled window loops: its offsets and its cell's x
// coordinate in the box (an exact small integer), one aligned load.
template <class real>
struct alignas(4 * sizeof(real)) PackItem {
  real x, y, z, cx;
};

template <class P>
struct StateP {
  using real = typename P::real;
  uint32_t* cell = nullptr;   // [cap]
  real* off = nullptr;        // [D][cap]
  PackItem<real>* pk = nullptr;  // [cap] packed copy for the untiled window kernels
  double* f64 = nullptr;      // FP64: [Q][cap]
  float* rho = nullptr;       // FP32DEV: [cap]
  float* dev = nullptr;       // FP32DEV: [Q][cap]
  uint32_t* start = nullptr;  // [ncells + 1]
  uint32_t* count = nullptr;  // device scalar
};

// A brick of cells of one instance (x0, y0, z0: its first cell) and the brick extent: the untiled
// window kernels map thread t of a block to cell t of a brick, x fastest.
struct Brick {
  int inst, x0, y0, z0;
};
struct BrickGeo {
  int bx, by, bz;  // bx * by * bz = threads per block
};
template <int D>
__device__ __forceinline__ bool brick_cell(const Brick& B, const InstK& I, const BrickGeo& g, int t, uint32_t* F) {
  const int lx = t % g.bx, ly = (t / g.bx) % g.by, lz = t / (g.bx * g.by);
  const int x = B.x0 + lx, y = B.y0 + ly, z = B.z0 + lz;
  if (lz >= g.bz || x >= I.dims[0] || y >= I.dims[1] || (D == 3 && z >= I.dims[2])) return false;
  *F = I.base + (uint32_t)x + (uint32_t)I.dims[0] * ((uint32_t)y + (D == 3 ? (uint32_t)I.dims[1] * (uint32_t)z : 0u));
  return true;
}

// (1/sw, f*_k) of one component: what a resampling hit reads, in one load.
template <class real>
struct alignas(2 * sizeof(real)) KV {
  real inv, f;
};

template <int Q, int D, class P>
struct Args {
  using real = typename P::real;
  LatK<Q, D> L;
  const InstK* inst;
  const uint32_t* inst_base;  // [n_inst + 1]
  int n_inst;
  uint32_t ncells;
  real R;          // r_res / cell
  real R2;         // largest d2 with rn_sqrt(d2) <= R (so d2 <= R2 <=> rn_sqrt(d2) <= R)
  real tiny;       // window safety margin (cell units)
  int kappa_hard;
  real eps;
  int64_t mcap;    // moment buffer capacity
  int64_t ccap;    // control-point buffer capacity (>= ncells; >= 2 ncells with the soft spawn)
  StateP<P> a;     // input moments (collided in place)
  StateP<P> b;     // output moments (= sorted control points)
  // scratch, per cell (occ and fkey have a second block of ncells slots for spawned CPs)
  uint32_t* occ;
  uint32_t* tcnt;
  real* cen;       // [D][ncells]
  uint32_t* mask;
  uint32_t* fkey;
  real* foff;      // [D][ncells]
  // soft-outer spawn: a CP with kappa_hard < kappa <= kappa_soft adds one CP soft_off cells along
  // the normalised sum of its components' directions (0: off)
  int kappa_soft;
  double soft_off;
  real* foff2;     // [D][ncells] offsets of the spawned CPs (slot ncells + F)
  // sort (keys_in/vals_in before, skeys/svals = the sorted result)
  uint32_t* skeys;
  uint32_t* svals;
  // resampling
  real* sw;        // [Q][mcap]
  KV<real>* kv;    // [Q][mcap] (1/sw, f*_k), written by the untiled weights kernel for the untiled gather
  real* wexp;      // [Q][mcap] exp(f*_k), written by the collision when want_wexp (untiled refine)
  int want_wexp;
  double* cpf64;   // FP64: [Q][ccap]
  float* cpfhi;    // FP32DEV: [Q][ccap]
  float* cpflo;    // FP32DEV: [Q][ccap]
  uint32_t* emask; // [ccap]
  uint32_t* bmask; // [mcap] blocked (bounced) directions of each input moment, bit k (obstacles only)
  int any_obstacle;
  uint32_t* status;
  uint32_t* d_P;
  int write_trace;
};

// ---- geometry helpers ---------------------------------------------------------------------------

__device__ __forceinline__ int find_instance(const uint32_t* __restrict__ base, int n, uint32_t g) {
  int lo = 0, hi = n;  // invariant: base[lo] <= g < base[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (__ldg(base + mid) <= g) lo = mid; else hi = mid;
  }
  return lo;
}

template <int D>
__device__ __forceinline__ void decode_cell(const InstK& I, uint32_t g, int (&c)[3]) {
  uint32_t local = g - I.base;
  c[0] = (int)(local % (uint32_t)I.dims[0]);
  local /= (uint32_t)I.dims[0];
  if (D == 3) {
    c[1] = (int)(local % (uint32_t)I.dims[1]);
    c[2] = (int)(local / (uint32_t)I.dims[1]);
  } else {
    c[1] = (int)local;
    c[2] = 0;
  }
}

// Global cell of unwrapped integer coordinates, or false if a bounded box has no such cell.
// Offsets are at most a few cells, far below the minimum box size, so one wrap suffices.
template <int D>
__device__ __forceinline__ bool cell_at(const InstK& I, int x, int y, int z, uint32_t* g) {
  const int nx = I.dims[0], ny = I.dims[1], nz = I.dims[2];
  if (I.periodic) {
    x = x < 0 ? x + nx : (x >= nx ? x - nx : x);
    y = y < 0 ? y + ny : (y >= ny ? y - ny : y);
    if (D == 3) z = z < 0 ? z + nz : (z >= nz ? z - nz : z);
  } else {
    if (x < 0 || x >= nx || y < 0 || y >= ny) return false;
    if (D == 3 && (z < 0 || z >= nz)) return false;
  }
  uint32_t lin = (uint32_t)x + (uint32_t)nx * ((uint32_t)y + (D == 3 ? (uint32_t)ny * (uint32_t)z : 0u));
  *g = I.base + lin;
  return true;
}

// The canonical displacement of a candidate from a reference point (the oracle's order, see
// oracle/grid_step.py): per window cell  c = (float(dS) + cd) - p,  per candidate  e = off + c,
// d2 = sum e*e, every step rounded to nearest with no contraction.  inside <=> sqrt(d2) <= R,
// which is decided as d2 <= R2 with R2 the largest value whose rounded square root is <= R
// (computed exactly on the host), so misses never pay for a square root.
template <class T>
__device__ __forceinline__ T canon_c(int dS, T cd, T p) {
  return rn_sub(rn_add((T)dS, cd), p);
}
template <int D, class T>
__device__ __forceinline__ T canon_d2(const T (&off)[3], const T (&c)[3], T (&e)[3]) {
  T s = 0;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    e[a] = rn_add(off[a], c[a]);
    const T e2 = rn_mul(e[a], e[a]);
    s = a == 0 ? e2 : rn_add(s, e2);
  }
  return s;
}
// Lower bound (rounded exactly like canon_d2) of d2 over all candidates of a window cell: every
// offset lies in [0, 1), so e_a lies in [c_a, fl(c_a + 1)] and rounding is monotonic.
template <int D, class T>
__device__ __forceinline__ T cell_d2_lower(const T (&c)[3]) {
  T s = 0;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const T hi = rn_add(c[a], (T)1);
    const T m = c[a] > (T)0 ? c[a] : (hi < (T)0 ? -hi : (T)0);
    const T m2 = rn_mul(m, m);
    s = a == 0 ? m2 : rn_add(s, m2);
  }
  return s;
}

template <class P>
__device__ __forceinline__ typename P::real floor_r(typename P::real x) { return floor(x); }

// One window row of cells (x0 + lo .. x0 + hi, unwrapped, at box row y, z) as at most two runs of
// consecutive cells of the box, in ascending unwrapped x: fn(first global cell, last global cell,
// shift) with unwrapped x = (cell x in the box) + shift.  Returns false if the row lies outside a
// bounded box.  Windows are narrower than every box, so a row wraps at most once.
template <int D, class Fn>
__device__ __forceinline__ bool row_runs(const InstK& I, int x0, int y, int z, int lo, int hi, Fn&& fn) {
  const int nx = I.dims[0], ny = I.dims[1], nz = I.dims[2];
  if (I.periodic) {
    y = y < 0 ? y + ny : (y >= ny ? y - ny : y);
    if (D == 3) z = z < 0 ? z + nz : (z >= nz ? z - nz : z);
  } else if (y < 0 || y >= ny || (D == 3 && (z < 0 || z >= nz))) {
    return false;
  }
  const uint32_t row = I.base + (uint32_t)nx * ((uint32_t)y + (D == 3 ? (uint32_t)ny * (uint32_t)z : 0u));
  int a = x0 + lo, b = x0 + hi;
  if (!I.periodic) {
    a = max(a, 0);
    b = min(b, nx - 1);
    if (a <= b) fn(row + (uint32_t)a, row + (uint32_t)b, 0);
    return true;
  }
  if (a < 0) {
    fn(row + (uint32_t)(a + nx), row + (uint32_t)(nx - 1), -nx);
    a = 0;
  }
  if (b >= nx) {
    if (a <= nx - 1) fn(row + (uint32_t)a, row + (uint32_t)(nx - 1), 0);
    fn(row, row + (uint32_t)(b - nx), nx);
  } else if (a <= b) {
    fn(row + (uint32_t)a, row + (uint32_t)b, 0);
  }
  return true;
}

// Half-width bound on |e_x| for a window row whose candidates have e_y^2 + e_z^2 >= lb2 (each
// square and the sum rounded): any hit has fl(e_x^2) + lb2 <= R2 up to a couple of roundings, so
// |e_x| <= sqrt(R2 - lb2 + R2 * 2^-20).  Returns < 0 if the row cannot hold a hit.
template <class real>
__device__ __forceinline__ real row_halfwidth2(real R2, real lb2) {
  const float rem = (float)(R2 - lb2);
  if (rem < -(float)R2 * 1e-6f) return (real)-1;
  const float x = fmaxf(rem, 0.f) + (float)R2 * 9.5367431640625e-07f;
  return (real)(bound_sqrt(x) * 1.0001f + 1e-6f);
}

// Lower bound of |e| on one axis over the candidates of a window cell whose e lies in
// [fl(c), fl(c + 1)] (offsets in [0, 1), rounding monotonic).
template <class real>
__device__ __forceinline__ real axis_lb(real c) {
  const real hi = rn_add(c, (real)1);
  return c > (real)0 ? c : (hi < (real)0 ? -hi : (real)0);
}

// Source-cell offsets (per axis) from which a component of displacement cd can land in a cell:
// floor(off + cd) over off in [0, 1), rounded in the working precision, takes only the values
// floor(cd) .. floor(rn(below1 + cd)) (monotone rounding), so so = -floor(...) lies in
// [lo, lo + n) with n = 1 or 2.  Cells outside this range hold no landing component.
template <class real>
__device__ __forceinline__ void thin_sources(real cd, int* lo, int* n) {
  const real below1 = std::is_same<real, double>::value ? (real)nextafter(1.0, 0.0) : (real)nextafterf(1.0f, 0.0f);
  const int fmin = (int)floor(cd), fmax = (int)floor(rn_add(below1, cd));
  *lo = -fmax;
  *n = fmax - fmin + 1;
}

// Squared distance (FP32, approximate) from the instance's sphere center to local cell S + o; used
// only against margins that are wider than its error, to skip exact tests far from the solid.
template <int D, class T>
__device__ __forceinline__ float sphere_dist2(const InstK& I, const int (&S)[3], const T (&o)[3]) {
  float d2 = 0.f;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const float e = (float)S[a] - (float)I.obs_c[a] + (float)o[a];
    d2 += e * e;
  }
  return d2;
}

// Whether the point (local integer cell S) + o (cell units, FP64) lies inside the instance's
// sphere: end_a = ((double)S_a - ctr_a) + o_a, inside <=> sum end_a^2 < r^2, each operation rounded
// in FP64 in this order (the oracle's order, oracle/grid_step.py: inside_obstacle).
template <int D>
__device__ __forceinline__ bool inside_sphere(const InstK& I, const int (&S)[3], const double (&o)[3]) {
  double d2 = 0;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    const double e = __dadd_rn(__dsub_rn((double)S[a], I.obs_c[a]), o[a]);
    const double e2 = __dmul_rn(e, e);
    d2 = a == 0 ? e2 : __dadd_rn(d2, e2);
  }
  return d2 < I.obs_r2;
}

// Called around one step by SimBase::step_hooked.  `before` sees the input state (args->a, not
// yet collided); `after` sees every buffer of the step (a = the collided input moments, b = the
// output moments, the per-cell thinning/refine scratch, the sorted pairs, 1/sw, the gathered f
// and the empty masks) before the two state buffers swap roles.  `args` is an Args<Q, D, P>.
struct StepHook {
  virtual ~StepHook() = default;
  virtual int before(const void* args, cudaStream_t s) = 0;
  virtual int after(const void* args, cudaStream_t s) = 0;
};

// Summation order of the window sums (refine, weights, gather).  2D FP32 (where dense stencils,
// shifted and plain row segments and the untiled kernels must agree bit for bit): per direction,
// the first item of every window cell in window order, then, if a window cell holds more, the
// other items in the same cell order.  Elsewhere (FP64, 3D) the items of each cell in order.
template <class P, int D>
constexpr bool kFirstItemsFirst = std::is_same<P, PF32>::value && D == 2;

// Type-erased simulator (SimImpl<Q, D, P> in sim.cu).
struct SimBase {
  virtual ~SimBase() = default;
  // Load m moments: positions (m, D) and f (m, Q) as double, or float with kLoadF32; kLoadPresorted
  // declares them in cell order (checked on the device) and skips the sort.
  enum { kLoadF32 = 1, kLoadPresorted = 2 };
  virtual int load(const int32_t* inst_of, const void* pos, const void* f, int64_t m, int flags, cudaStream_t) = 0;
  virtual int step(int, cudaStream_t) = 0;
  virtual int step_partial(int, cudaStream_t) = 0;
  virtual int step_hooked(StepHook*, cudaStream_t) = 0;
  virtual int profile_step(float*, cudaStream_t) = 0;
  virtual int count(int64_t*, cudaStream_t) = 0;
  virtual int get_state(int32_t*, void* pos, void* f, int f32, cudaStream_t) = 0;
  virtual int status(uint32_t*, int, cudaStream_t) = 0;
  virtual int conservation(double*, cudaStream_t) = 0;
  virtual int trace(int, void*, int64_t, int64_t*, cudaStream_t) = 0;
  virtual int set_tau(const double*, int) = 0;
  virtual int set_obstacle(int, const double*, double) = 0;
  virtual int set_inflow(int, const double*, int) = 0;
  virtual int snapshot(void*, int64_t, int64_t*, cudaStream_t) = 0;
  virtual int restore(const void*, int64_t, cudaStream_t) = 0;
  virtual int64_t device_bytes() const = 0;
  virtual void invalidate_graphs() = 0;
  virtual int tiling(int* tx, int* persistent) const = 0;
  virtual int set_tiling_v(int tx, int persistent) = 0;
  virtual int set_soft_spawn(int kappa_soft) = 0;
  virtual int ensure_untiled() = 0;
  virtual int set_brick(int bx) = 0;
  virtual int brick_width() const = 0;
  int kappa_soft = 0;  // soft-outer spawn threshold (0: off)
  int use_graphs = 1;
  int use_tiles = 1;
  int use_shift = 1;  // DBM_OPT_SHIFTED_WINDOWS
  int use_dense = 1;  // DBM_OPT_DENSE_STENCIL
  uint64_t version = 0;  // bumped by every change of the state (load, step, restore)
  int lattice = 0;
  int precision = 0;
  int n_inst = 0;
  uint32_t n_cells = 0;
};

}  // namespace dbm

struct dbm_sim {
  dbm::SimBase* impl;
};
