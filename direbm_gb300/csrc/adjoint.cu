// Reverse mode of the DiReBM step with its discrete structure held fixed.
//
// The reference has no derivative of its step (differentiation is future work in the reference,
// idea.md:250); this file adds one for the fused step of sim.cu (itself a restatement of
// direbm/warp/simulator.py:50-73 and direbm/warp/propagation.py:21-275).
//
// Held fixed per step (the "tape", recorded while the step runs): which components land in which
// thinning cell, which control points (CPs) refine moved and the components within r of their
// centroids, the CP sort order, the resampling pairs (component, CP) within r, the dropped
// components, the gap-filled directions and the CP pairs of the gap fill.  With those fixed the
// step is a smooth map of the input offsets x (cell units), the input f and tau:
//   f*    = f + (feq(rho, u) - f) / tau                                   (collision)
//   y_i   = x_m + cd_k                                                    (dispersion, i = (m, k))
//   cen_t = mean of y_i over the components thinned into cell t
//   p_t   = cen_t, or sum w_i y_i / sum w_i over its refine pairs, w_i = exp(f*_i)  (refine)
//   sw_i  = sum over resample pairs (i, j) of (r - |y_i - p_j|)
//   F_jk  = sum over resample pairs (i, j), k_i = k, of (r - |y_i - p_j|) / sw_i * f*_i
//   F_jk  = r rho_rest W_k / sum over gap pairs (j, l) of (r - |p_l - p_j|)      (filled entries)
// and the next state is (p_j, F_j).  dbm_tape_backward applies the transpose of its Jacobian,
// pair by pair, in fixed order (no float atomics): every accumulation is owned by one thread, and
// every neighbour list is recorded in both orientations (by control point and by component), each
// enumerated on its own side with the same canonical arithmetic, so scatters become gathers.
// |y - p| has the subgradient 0 at zero distance.
#include <algorithm>
#include <vector>

#include "sim.cuh"
#include "sortscan.cuh"

namespace dbm {

constexpr uint32_t kNone = 0xffffffffu;

// ---- device memory: a chunked bump allocator ----------------------------------------------------
struct DevArena {
  struct Chunk {
    char* p;
    size_t cap, used;
  };
  std::vector<Chunk> chunks;
  size_t total = 0;
  ~DevArena() {
    for (auto& c : chunks) cudaFree(c.p);
  }
  void reset() {
    for (auto& c : chunks) c.used = 0;
  }
  template <class T>
  int get(T** out, int64_t n) {
    const size_t b = (((size_t)std::max<int64_t>(n, 1) * sizeof(T)) + 255) & ~(size_t)255;
    for (auto& c : chunks)
      if (c.cap - c.used >= b) {
        *out = (T*)(c.p + c.used);
        c.used += b;
        return DBM_OK;
      }
    const size_t cap = std::max<size_t>(b, (size_t)64 << 20);
    void* p = nullptr;
    DBM_CUDA(cudaMalloc(&p, cap));
    chunks.push_back({(char*)p, cap, b});
    total += cap;
    *out = (T*)p;
    return DBM_OK;
  }
};

// ---- the recorded step ----------------------------------------------------------------------

// One recorded pair: the reference point (row: a CP), the other end (item: a component m*Q + k, or
// a neighbour CP in the gap fill) and the displacement e = other end - reference point exactly as
// the step computed it.  One record is one aligned store / load (16 bytes for FP32 in 2D).
template <class real, int D>
struct alignas((sizeof(real) * D + 8) <= 16 ? 16 : 8) PairRec {
  uint32_t row;
  uint32_t item;
  real e[D];
};

// A pair list: row r's pairs are rec[start[r] .. start[r] + cnt[r]).  Rows reserve their slots as
// they are enumerated, so where a row sits in rec varies from run to run; what it holds does not.
template <class real, int D>
struct PairList {
  int64_t rows = 0, n = 0, cap = 0;
  uint32_t* start = nullptr;         // [rows]
  uint32_t* cnt = nullptr;           // [rows]
  PairRec<real, D>* rec = nullptr;   // [cap]
  uint32_t* bits = nullptr;          // [cap] gap fill, CP side: directions empty in both CPs
};

// Both orientations of one neighbour relation: f by reference point (rows CP x direction; gap fill:
// the filled CP), t by the other end (rows component k*M + m; gap fill: the neighbour CP, whose
// records hold row = filled CP, item = the shared empty directions).
template <class real, int D>
struct PairCSR {
  PairList<real, D> f, t;
};

template <class real, int D>
struct StepRec {
  int64_t M = 0, P = 0;
  uint32_t* in_cell = nullptr;    // [M]
  uint32_t* in_start = nullptr;   // [ncells + 1] the input state's cell ranges (read by the lists)
  real* in_off = nullptr;         // [D][M]
  real* in_f = nullptr;           // FP64: f [Q][M]; FP32DEV: dev [Q][M]
  float* in_rho = nullptr;        // FP32DEV: rho [M]
  real* fs = nullptr;             // FP64: f* [Q][M]; FP32DEV: dev* [Q][M] (rho is unchanged)
  uint32_t* thin_cell = nullptr;  // [Q][M]
  real* inv_sw = nullptr;         // [Q][M]
  uint32_t* inst_start = nullptr; // [n_inst + 1]
  uint32_t* cp_thin = nullptr;    // [P]
  uint32_t* cp_n = nullptr;       // [P]
  uint32_t* cp_moved = nullptr;   // [P]
  real* cp_cen = nullptr;         // [D][P]
  uint32_t* out_cell = nullptr;   // [P]
  real* out_off = nullptr;        // [D][P]
  uint32_t* emask = nullptr;      // [P]
  PairCSR<real, D> ref, res, gap;
};

// Per component (m, k), from the gather's VJP to the control-point rows: f*·(1/sw) (0 for a
// dropped component) and G = sum over its pairs of a_ij fbar_jk.
template <class real>
struct alignas(2 * sizeof(real)) FsG {
  real fsi, g;
};

// Per moved control point, from its VJP to the component side's refine pairs: W = sum of the
// refine weights, the position cotangent and the move s, in one record (one pair reads it with
// two vector loads instead of five scalar ones).
template <class real>
struct alignas(16) CPBar {
  real W;
  real xb[3];
  real s[3];
  real pad;
};

// Everything a backward kernel reads, by value.
template <int Q, int D, class P>
struct RecK {
  using real = typename P::real;
  LatK<Q, D> L;
  const InstK* inst;
  const uint32_t* inst_base;
  int n_inst;
  real R;
  StepRec<real, D> r;
};

template <int Q, int D, class P>
__device__ __forceinline__ typename P::real rec_fstar(const RecK<Q, D, P>& K, int64_t m, int k) {
  if constexpr (std::is_same<P, PF64>::value) return K.r.fs[(int64_t)k * K.r.M + m];
  else return __fmaf_rn(K.r.in_rho[m], K.L.wf[k], K.r.fs[(int64_t)k * K.r.M + m]);
}

// Unit vector of a pair's displacement and its length (subgradient 0 at zero distance).
template <int D, class real>
__device__ __forceinline__ real unit_of(const PairRec<real, D>& pr, real (&u)[3]) {
  real d2 = 0;
#pragma unroll
  for (int a = 0; a < D; ++a) {
    u[a] = pr.e[a];
    d2 += u[a] * u[a];
  }
  if constexpr (std::is_same<real, float>::value) {
    // FP32 store: the hardware reciprocal square root (a few ulp), far inside the 2e-4 the FP32
    // backward is held to against the FP64 reference; one instruction instead of a correctly
    // rounded square root and a division
    const float r = d2 > 0.f ? rsqrtf(d2) : 0.f;
#pragma unroll
    for (int a = 0; a < D; ++a) u[a] *= r;
    return d2 * r;
  } else {
    const real d = sqrt(d2);
    const real inv = d > (real)0 ? (real)1 / d : (real)0;
#pragma unroll
    for (int a = 0; a < D; ++a) u[a] *= inv;
    return d;
  }
}

template <int D, class real>
__device__ __forceinline__ PairRec<real, D> make_rec(uint32_t row, uint32_t item, const real (&e)[3]) {
  PairRec<real, D> pr;
  pr.row = row;
  pr.item = item;
#pragma unroll
  for (int a = 0; a < D; ++a) pr.e[a] = e[a];
  return pr;
}

// ---- recording kernels (read the step's buffers through Args, see StepHook) --------------------

// Gather up to 8 device words into mapped pinned host memory: one launch instead of one small
// device-to-host copy per word at every recorded step's synchronisation.
struct FetchSrc {
  const uint32_t* p[8];
};
__global__ void k_fetch_words(FetchSrc src, int n, uint32_t* __restrict__ dst) {
  const int i = threadIdx.x;
  if (i < n) dst[i] = *src.p[i];
}

template <int Q, int D, class P>
__global__ void __launch_bounds__(256) k_rec_thin_cell(const __grid_constant__ Args<Q, D, P> A, int64_t M,
                                                       uint32_t* __restrict__ thin_cell) {
  using real = typename P::real;
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M; m += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t g = A.a.cell[m];
    const InstK I = A.inst[find_instance(A.inst_base, A.n_inst, g)];
    int Sc[3];
    decode_cell<D>(I, g, Sc);
#pragma unroll 1
    for (int k = 0; k < Q; ++k) {
      int x[3] = {Sc[0], Sc[1], Sc[2]};
#pragma unroll
      for (int a = 0; a < D; ++a) x[a] += (int)floor(rn_add(A.a.off[(int64_t)a * A.mcap + m], A.L.template cd_as<real>(k, a)));
      uint32_t F;
      thin_cell[(int64_t)k * M + m] = cell_at<D>(I, x[0], x[1], x[2], &F) ? F : kNone;
    }
  }
}

template <int Q, int D, class P>
__global__ void __launch_bounds__(256) k_rec_cp(const __grid_constant__ Args<Q, D, P> A,
                                                const __grid_constant__ StepRec<typename P::real, D> r,
                                                uint32_t* __restrict__ cp_of_cell) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < r.P; j += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t F = A.svals[j];
    r.cp_thin[j] = F;
    cp_of_cell[F] = (uint32_t)j;
    r.cp_n[j] = A.tcnt[F];
    r.cp_moved[j] = __popc(A.mask[F]) > A.kappa_hard ? 1u : 0u;
    r.out_cell[j] = A.b.cell[j];
    r.emask[j] = A.emask[j];
#pragma unroll
    for (int a = 0; a < D; ++a) {
      r.cp_cen[(int64_t)a * r.P + j] = A.cen[(int64_t)a * A.ncells + F];
      r.out_off[(int64_t)a * r.P + j] = A.b.off[(int64_t)a * A.ccap + j];
    }
  }
}

template <int Q, int D, class P>
__global__ void k_rec_inst_start(const __grid_constant__ Args<Q, D, P> A, uint32_t* __restrict__ inst_start) {
  for (int b = threadIdx.x; b <= A.n_inst; b += blockDim.x) inst_start[b] = A.a.start[A.inst_base[b]];
}

// ---- neighbour lists ---------------------------------------------------------------------------
// Each enumeration visits one row's pairs with exactly the arithmetic of the forward decision it
// restates (canonical displacement, inclusive radius test) and calls emit(other end, e) per pair.

// ---- 2D row runs -----------------------------------------------------------------------------
//
// The same enumerations in 2D with fewer dependent loads: a window row's candidate cells form at
// most two runs of consecutive cells (split at a periodic seam), so a row reads its item range
// with two loads instead of two per cell, and the row's x range is narrowed by its lower bound on
// |e_y| (row_halfwidth2 drops only cells that hold no hit).  Candidates are visited in the
// per-cell loops' order (rows ascending, x ascending, items in cell order), so every list is
// identical, pair for pair.  Windows are at most kListRows rows (R < 2 cells); taller ones use the
// per-cell loops.
constexpr int kListRows = 5;

struct RowRuns2 {
  int n;             // runs, 0..2, in x order
  uint32_t g0[2], g1[2];  // first and last cell of each run
  int sx0[2];        // window-relative x of the run's first cell
};

// Runs of one window row: grid row Gy + sy, unwrapped cells [Gx + lo, Gx + hi] (windows are
// narrower than every box, so a row wraps at most once).
__device__ __forceinline__ RowRuns2 row_runs2(const InstK& I, int Gx, int Gy, int sy, int lo, int hi) {
  RowRuns2 R;
  R.n = 0;
  const int nx = I.dims[0], ny = I.dims[1];
  int y = Gy + sy;
  if (I.periodic) y = y < 0 ? y + ny : (y >= ny ? y - ny : y);
  else if (y < 0 || y >= ny) return R;
  const uint32_t row = I.base + (uint32_t)nx * (uint32_t)y;
  int a = Gx + lo, b = Gx + hi;
  if (!I.periodic) {
    a = max(a, 0);
    b = min(b, nx - 1);
    lo = a - Gx;
  }
  if (a > b) return R;
  if (I.periodic && a < 0) {  // cells a + nx .. nx - 1, then 0 .. b
    R.g0[0] = row + (uint32_t)(a + nx);
    R.g1[0] = row + (uint32_t)(nx - 1);
    R.sx0[0] = lo;
    R.n = 1;
    if (b >= 0) {
      R.g0[1] = row;
      R.g1[1] = row + (uint32_t)b;
      R.sx0[1] = -Gx;
      R.n = 2;
    }
  } else if (I.periodic && b >= nx) {  // cells a .. nx - 1, then 0 .. b - nx
    if (a <= nx - 1) {
      R.g0[0] = row + (uint32_t)a;
      R.g1[0] = row + (uint32_t)(nx - 1);
      R.sx0[0] = lo;
      R.g0[1] = row;
      R.g1[1] = row + (uint32_t)(b - nx);
      R.sx0[1] = nx - Gx;
      R.n = 2;
    } else {
      R.g0[0] = row;
      R.g1[0] = row + (uint32_t)(b - nx);
      R.sx0[0] = nx - Gx;
      R.n = 1;
    }
  } else {
    R.g0[0] = row + (uint32_t)a;
    R.g1[0] = row + (uint32_t)b;
    R.sx0[0] = lo;
    R.n = 1;
  }
  return R;
}

// CP side (refine: reference = centroid, resampling: reference = control point), candidates the
// moments of A.a: emit(m * Q + k, e) for every component (m, k) within r of the reference p
// (offsets in the reference's cell Gc).  Returns the pair count, or -1 if the window is too tall.
template <int Q, class P, class Emit>
__device__ __forceinline__ int enum_cp_rows2(const Args<Q, 2, P>& A, const InstK& I, const int (&Gc)[3],
                                             typename P::real px, typename P::real py, int k, Emit&& emit) {
  using real = typename P::real;
  const real cdx = A.L.template cd_as<real>(k, 0), cdy = A.L.template cd_as<real>(k, 1);
  const real bxr = px - cdx, byr = py - cdy;
  const int ylo = (int)floor(byr - A.R - A.tiny), yhi = (int)floor(byr + A.R + A.tiny);
  if (yhi - ylo + 1 > kListRows) return -1;
  int cnt = 0;
#pragma unroll 1
  for (int sy = ylo; sy <= yhi; ++sy) {
    const real cy = canon_c<real>(sy, cdy, py);
    const real lb = axis_lb<real>(cy);
    const real hw = row_halfwidth2<real>(A.R2, rn_mul(lb, lb));
    if (hw < (real)0) continue;
    const RowRuns2 R = row_runs2(I, Gc[0], Gc[1], sy, (int)floor(bxr - hw - A.tiny), (int)floor(bxr + hw + A.tiny));
    uint32_t mb[2], me[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      mb[q] = q < R.n ? A.a.start[R.g0[q]] : 0u;
      me[q] = q < R.n ? A.a.start[R.g1[q] + 1] : 0u;
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (q >= R.n) break;
      for (uint32_t m = mb[q]; m < me[q]; ++m) {
        const real o[3] = {A.a.off[m], A.a.off[A.mcap + m], 0};
        const int sx = R.sx0[q] + (int)(A.a.cell[m] - R.g0[q]);
        const real c[3] = {canon_c<real>(sx, cdx, px), cy, 0};
        real e[3];
        if (canon_d2<2, real>(o, c, e) <= A.R2) {
          emit(m * (uint32_t)Q + (uint32_t)k, e);
          ++cnt;
        }
      }
    }
  }
  return cnt;
}

// Resampling, component side (row = component (m, k)), candidates the output control points; e in
// the CP side's operation order.  Returns the pair count, or -1 if the window is too tall.
template <int Q, class P, class Emit>
__device__ __forceinline__ int enum_comp_rows2(const Args<Q, 2, P>& A, const InstK& I, const int (&Sc)[3], uint32_t m,
                                               int k, Emit&& emit) {
  using real = typename P::real;
  const real o[3] = {A.a.off[m], A.a.off[A.mcap + m], 0};
  const real cdx = A.L.template cd_as<real>(k, 0), cdy = A.L.template cd_as<real>(k, 1);
  const real tx = rn_add(o[0], cdx), ty = rn_add(o[1], cdy);
  const int ylo = (int)floor(ty - A.R - A.tiny), yhi = (int)floor(ty + A.R + A.tiny);
  if (yhi - ylo + 1 > kListRows) return -1;
  int cnt = 0;
#pragma unroll 1
  for (int gy = ylo; gy <= yhi; ++gy) {
    // candidates have e_y in [fl(o_y + fl(base_y - 1)), fl(o_y + base_y)] (offsets in [0, 1))
    const real basey = rn_add((real)(-gy), cdy);
    const real ely = rn_add(o[1], rn_sub(basey, (real)1)), ehy = rn_add(o[1], basey);
    const real lb = ely > (real)0 ? ely : (ehy < (real)0 ? -ehy : (real)0);
    const real hw = row_halfwidth2<real>(A.R2, rn_mul(lb, lb));
    if (hw < (real)0) continue;
    const RowRuns2 R = row_runs2(I, Sc[0], Sc[1], gy, (int)floor(tx - hw - A.tiny), (int)floor(tx + hw + A.tiny));
    uint32_t cb[2], ce[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      cb[q] = q < R.n ? A.b.start[R.g0[q]] : 0u;
      ce[q] = q < R.n ? A.b.start[R.g1[q] + 1] : 0u;
    }
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      if (q >= R.n) break;
      for (uint32_t c = cb[q]; c < ce[q]; ++c) {
        const int gx = R.sx0[q] + (int)(A.b.cell[c] - R.g0[q]);
        const real cc[3] = {canon_c<real>(-gx, cdx, A.b.off[c]), canon_c<real>(-gy, cdy, A.b.off[A.ccap + c]), 0};
        real e[3];
        if (canon_d2<2, real>(o, cc, e) <= A.R2) {
          emit(c, e);
          ++cnt;
        }
      }
    }
  }
  return cnt;
}

// Refine, CP side, row (CP j, direction k): the components of direction k within r of the centroid
// of moved CP j (the forward refine's window around the thin cell).
template <int Q, int D, class P, class Emit>
__device__ __forceinline__ uint32_t enum_refine_cp(const Args<Q, D, P>& A, const StepRec<typename P::real, D>& r,
                                                   int64_t j, int k, Emit&& emit) {
  using real = typename P::real;
  if (!r.cp_moved[j]) return 0;
  const uint32_t F = r.cp_thin[j];
  const InstK I = A.inst[find_instance(A.inst_base, A.n_inst, F)];
  int Fc[3];
  decode_cell<D>(I, F, Fc);
  if constexpr (D == 2) {
    const int n = enum_cp_rows2<Q, P>(A, I, Fc, r.cp_cen[j], r.cp_cen[r.P + j], k, emit);
    if (n >= 0) return (uint32_t)n;
  }
  real cen[3] = {0, 0, 0}, cdk[3] = {0, 0, 0};
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) {
    cen[a] = r.cp_cen[(int64_t)a * r.P + j];
    cdk[a] = A.L.template cd_as<real>(k, a);
    const real base = cen[a] - cdk[a];
    lo[a] = (int)floor(base - A.R - A.tiny);
    hi[a] = (int)floor(base + A.R + A.tiny);
  }
  uint32_t cnt = 0;
#pragma unroll 1
  for (int sz = lo[2]; sz <= hi[2]; ++sz)
#pragma unroll 1
    for (int sy = lo[1]; sy <= hi[1]; ++sy)
#pragma unroll 1
      for (int sx = lo[0]; sx <= hi[0]; ++sx) {
        const int dS[3] = {sx, sy, sz};
        real c[3] = {0, 0, 0};
#pragma unroll
        for (int a = 0; a < D; ++a) c[a] = canon_c<real>(dS[a], cdk[a], cen[a]);
        if (cell_d2_lower<D, real>(c) > A.R2) continue;
        uint32_t Sg;
        if (!cell_at<D>(I, Fc[0] + sx, Fc[1] + sy, Fc[2] + sz, &Sg)) continue;
        const uint32_t m0 = A.a.start[Sg], m1 = A.a.start[Sg + 1];
        for (uint32_t m = m0; m < m1; ++m) {
          real o[3] = {0, 0, 0}, e[3];
#pragma unroll
          for (int a = 0; a < D; ++a) o[a] = A.a.off[(int64_t)a * A.mcap + m];
          if (canon_d2<D, real>(o, c, e) <= A.R2) {
            emit(m * (uint32_t)Q + (uint32_t)k, e);
            ++cnt;
          }
        }
      }
  return cnt;
}

// Resampling, CP side, row (CP j, direction k): the components of direction k within r of the CP
// (the forward gather's window).
template <int Q, int D, class P, class Emit>
__device__ __forceinline__ uint32_t enum_resample_cp(const Args<Q, D, P>& A, int64_t j, int k, Emit&& emit) {
  using real = typename P::real;
  const uint32_t G = A.b.cell[j];
  const InstK I = A.inst[find_instance(A.inst_base, A.n_inst, G)];
  int Gc[3];
  decode_cell<D>(I, G, Gc);
  if constexpr (D == 2) {
    const int n = enum_cp_rows2<Q, P>(A, I, Gc, A.b.off[j], A.b.off[A.ccap + j], k, emit);
    if (n >= 0) return (uint32_t)n;
  }
  real p[3] = {0, 0, 0}, cdk[3] = {0, 0, 0};
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) {
    p[a] = A.b.off[(int64_t)a * A.ccap + j];
    cdk[a] = A.L.template cd_as<real>(k, a);
    const real base = p[a] - cdk[a];
    lo[a] = (int)floor(base - A.R - A.tiny);
    hi[a] = (int)floor(base + A.R + A.tiny);
  }
  uint32_t cnt = 0;
#pragma unroll 1
  for (int sz = lo[2]; sz <= hi[2]; ++sz)
#pragma unroll 1
    for (int sy = lo[1]; sy <= hi[1]; ++sy)
#pragma unroll 1
      for (int sx = lo[0]; sx <= hi[0]; ++sx) {
        const int dS[3] = {sx, sy, sz};
        real c[3] = {0, 0, 0};
#pragma unroll
        for (int a = 0; a < D; ++a) c[a] = canon_c<real>(dS[a], cdk[a], p[a]);
        if (cell_d2_lower<D, real>(c) > A.R2) continue;
        uint32_t Sg;
        if (!cell_at<D>(I, Gc[0] + sx, Gc[1] + sy, Gc[2] + sz, &Sg)) continue;
        const uint32_t m0 = A.a.start[Sg], m1 = A.a.start[Sg + 1];
        for (uint32_t m = m0; m < m1; ++m) {
          real o[3] = {0, 0, 0}, e[3];
#pragma unroll
          for (int a = 0; a < D; ++a) o[a] = A.a.off[(int64_t)a * A.mcap + m];
          if (canon_d2<D, real>(o, c, e) <= A.R2) {
            emit(m * (uint32_t)Q + (uint32_t)k, e);
            ++cnt;
          }
        }
      }
  return cnt;
}

// Component side of both lists, row = component (m, k): the window around the component's landing
// point; CP candidates come from the output cells (resampling) or from the moved thin cells
// (refine, through cp_of_cell).  The displacement is computed in the CP side's operation order, so
// both sides decide the same pairs and record the same e.
template <int Q, int D, class P, bool REFINE, class Emit>
__device__ __forceinline__ uint32_t enum_comp(const Args<Q, D, P>& A, const StepRec<typename P::real, D>& r,
                                              const uint32_t* __restrict__ cp_of_cell, uint32_t m, int k, Emit&& emit) {
  using real = typename P::real;
  const uint32_t g = A.a.cell[m];
  const InstK I = A.inst[find_instance(A.inst_base, A.n_inst, g)];
  int Sc[3];
  decode_cell<D>(I, g, Sc);
  if constexpr (D == 2 && !REFINE) {  // (the refine side reads one centroid per cell: no item runs)
    const int n = enum_comp_rows2<Q, P>(A, I, Sc, m, k, emit);
    if (n >= 0) return (uint32_t)n;
  }
  real o[3] = {0, 0, 0}, cdk[3] = {0, 0, 0};
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) {
    o[a] = A.a.off[(int64_t)a * A.mcap + m];
    cdk[a] = A.L.template cd_as<real>(k, a);
    const real tt = rn_add(o[a], cdk[a]);
    lo[a] = (int)floor(tt - A.R - A.tiny);
    hi[a] = (int)floor(tt + A.R + A.tiny);
  }
  uint32_t cnt = 0;
#pragma unroll 1
  for (int gz = lo[2]; gz <= hi[2]; ++gz)
#pragma unroll 1
    for (int gy = lo[1]; gy <= hi[1]; ++gy)
#pragma unroll 1
      for (int gx = lo[0]; gx <= hi[0]; ++gx) {
        const int dG[3] = {gx, gy, gz};
        uint32_t Gg;
        if (!cell_at<D>(I, Sc[0] + gx, Sc[1] + gy, Sc[2] + gz, &Gg)) continue;
        if constexpr (REFINE) {
          const uint32_t j = cp_of_cell[Gg];
          if (j == kNone || !r.cp_moved[j]) continue;
          real c[3] = {0, 0, 0}, e[3];
#pragma unroll
          for (int a = 0; a < D; ++a) c[a] = canon_c<real>(-dG[a], cdk[a], r.cp_cen[(int64_t)a * r.P + j]);
          if (canon_d2<D, real>(o, c, e) <= A.R2) {
            emit(j, e);
            ++cnt;
          }
        } else {
          const uint32_t c0 = A.b.start[Gg], c1 = A.b.start[Gg + 1];
          for (uint32_t c = c0; c < c1; ++c) {
            real cc[3] = {0, 0, 0}, e[3];
#pragma unroll
            for (int a = 0; a < D; ++a) cc[a] = canon_c<real>(-dG[a], cdk[a], A.b.off[(int64_t)a * A.ccap + c]);
            if (canon_d2<D, real>(o, cc, e) <= A.R2) {
              emit(c, e);
              ++cnt;
            }
          }
        }
      }
  return cnt;
}

// Gap fill, row = CP j (T = false: the filled CP's side, emit(neighbour l, both, e)) or row = CP l
// (T = true: the neighbour's side, emit(filled CP j, both, e)).  e = p_l - p_j is computed from j's
// side in both cases, as the emit pass does.
template <int Q, int D, class P, bool T, class Emit>
__device__ __forceinline__ uint32_t enum_gap(const Args<Q, D, P>& A, int64_t x, Emit&& emit) {
  using real = typename P::real;
  const uint32_t em = A.emask[x];
  if (!em) return 0;
  const uint32_t G = A.b.cell[x];
  const InstK I = A.inst[find_instance(A.inst_base, A.n_inst, G)];
  int Gc[3];
  decode_cell<D>(I, G, Gc);
  real px[3] = {0, 0, 0};
  int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
#pragma unroll
  for (int a = 0; a < D; ++a) {
    px[a] = A.b.off[(int64_t)a * A.ccap + x];
    lo[a] = (int)floor(px[a] - A.R - A.tiny) - (T ? 1 : 0);
    hi[a] = (int)floor(px[a] + A.R + A.tiny) + (T ? 1 : 0);
  }
  uint32_t cnt = 0;
#pragma unroll 1
  for (int gz = lo[2]; gz <= hi[2]; ++gz)
#pragma unroll 1
    for (int gy = lo[1]; gy <= hi[1]; ++gy)
#pragma unroll 1
      for (int gx = lo[0]; gx <= hi[0]; ++gx) {
        const int dS[3] = {gx, gy, gz};
        uint32_t Hg;
        if (!cell_at<D>(I, Gc[0] + gx, Gc[1] + gy, Gc[2] + gz, &Hg)) continue;
        const uint32_t c0 = A.b.start[Hg], c1 = A.b.start[Hg + 1];
        for (uint32_t c = c0; c < c1; ++c) {
          const uint32_t both = A.emask[c] & em;
          if (!both) continue;
          real e[3], d2;
          if constexpr (!T) {  // j = x, l = c, window offset dS from j to l
            real cc[3] = {0, 0, 0}, o[3] = {0, 0, 0};
#pragma unroll
            for (int a = 0; a < D; ++a) {
              cc[a] = canon_c<real>(dS[a], (real)0, px[a]);
              o[a] = A.b.off[(int64_t)a * A.ccap + c];
            }
            d2 = canon_d2<D, real>(o, cc, e);
          } else {  // l = x, j = c: offset from j to l is -dS
            real cc[3] = {0, 0, 0};
#pragma unroll
            for (int a = 0; a < D; ++a) cc[a] = canon_c<real>(-dS[a], (real)0, A.b.off[(int64_t)a * A.ccap + c]);
            d2 = canon_d2<D, real>(px, cc, e);
          }
          if (d2 <= A.R2) {
            emit(c, both, e);
            ++cnt;
          }
        }
      }
  return cnt;
}

// Reserve cnt consecutive slots of a list for this lane: one atomicAdd per warp.  Every lane of the
// warp calls it (lanes without a row pass 0).
__device__ __forceinline__ uint32_t warp_reserve(uint32_t cnt, uint32_t* counter) {
  const int lane = threadIdx.x & 31;
  uint32_t incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
  uint32_t base = 0;
  if (lane == 31 && total) base = atomicAdd(counter, total);
  base = __shfl_sync(0xffffffffu, base, 31);
  return base + incl - cnt;
}

// One pass per list.  Each row enumerates its pairs once: it counts them all and stages the first
// kListStage records in shared memory (record i of thread t at i * blockDim + t, so a warp's
// accesses are conflict-free).  Then the row reserves its slots and copies the staged records out.
// Only a row with more pairs than that enumerates a second time, writing straight to the list.
// Within a row the order is the enumeration order either way.  A list whose capacity is too small
// writes nothing past it; the counter then holds the size needed and the host runs the kernel again.
enum ListKind { kRefineCP = 0, kRefineComp = 1, kResCP = 2, kResComp = 3, kGapCP = 4, kGapNb = 5 };
constexpr int kListStage = 12;

template <class real, int D, int KIND>
constexpr size_t list_smem_bytes(int threads) {
  return (size_t)kListStage * threads * (sizeof(PairRec<real, D>) + (KIND == kGapCP ? 4 : 0));
}

template <int Q, int D, class P, int KIND>
__global__ void __launch_bounds__(256) k_list(const __grid_constant__ Args<Q, D, P> A,
                                              const __grid_constant__ StepRec<typename P::real, D> r,
                                              const uint32_t* __restrict__ cp_of_cell, uint32_t* __restrict__ counter) {
  using real = typename P::real;
  using Rec = PairRec<real, D>;
  extern __shared__ __align__(16) unsigned char list_smem[];
  Rec* s_rec = reinterpret_cast<Rec*>(list_smem);
  uint32_t* s_bits = reinterpret_cast<uint32_t*>(s_rec + (size_t)kListStage * blockDim.x);  // kGapCP only
  const auto& Lst = KIND == kRefineCP ? r.ref.f : KIND == kRefineComp ? r.ref.t : KIND == kResCP ? r.res.f
                  : KIND == kResComp ? r.res.t : KIND == kGapCP ? r.gap.f : r.gap.t;
  const int64_t rows = Lst.rows;
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int64_t t0 = blockIdx.x * (int64_t)blockDim.x; t0 < rows; t0 += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = t0 + tid;
    const bool act = row < rows;
    uint32_t cnt = 0;
    int64_t j = 0, m = 0;
    int k = 0;
    uint32_t i_comp = 0;
    // stage: count every pair, keep the first kListStage
    const auto stage2 = [&](uint32_t row_id, uint32_t item, const real(&e)[3]) {
      if (cnt < (uint32_t)kListStage) s_rec[(size_t)cnt * nt + tid] = make_rec<D, real>(row_id, item, e);
      ++cnt;
    };
    if (act) {
      if constexpr (KIND == kRefineCP || KIND == kResCP) {
        j = row / Q;
        k = (int)(row - j * Q);
        const auto put = [&](uint32_t item, const real(&e)[3]) { stage2((uint32_t)j, item, e); };
        if constexpr (KIND == kRefineCP) enum_refine_cp<Q, D, P>(A, r, j, k, put);
        else enum_resample_cp<Q, D, P>(A, j, k, put);
      } else if constexpr (KIND == kRefineComp || KIND == kResComp) {
        k = (int)(row / r.M);
        m = row - (int64_t)k * r.M;
        i_comp = (uint32_t)m * (uint32_t)Q + (uint32_t)k;
        const auto put = [&](uint32_t cp, const real(&e)[3]) { stage2(cp, i_comp, e); };
        enum_comp<Q, D, P, KIND == kRefineComp>(A, r, cp_of_cell, (uint32_t)m, k, put);
      } else if constexpr (KIND == kGapCP) {
        const auto put = [&](uint32_t l, uint32_t both, const real(&e)[3]) {
          if (cnt < (uint32_t)kListStage) s_bits[(size_t)cnt * nt + tid] = both;
          stage2((uint32_t)row, l, e);
        };
        enum_gap<Q, D, P, false>(A, row, put);
      } else {
        const auto put = [&](uint32_t jj, uint32_t both, const real(&e)[3]) { stage2(jj, both, e); };
        enum_gap<Q, D, P, true>(A, row, put);
      }
    }
    const uint32_t pos = warp_reserve(cnt, counter);
    if (!act) continue;
    Lst.start[row] = pos;
    Lst.cnt[row] = cnt;
    if (!cnt || (int64_t)pos + cnt > Lst.cap) continue;
    if (cnt <= (uint32_t)kListStage) {
      for (uint32_t q = 0; q < cnt; ++q) {
        Lst.rec[pos + q] = s_rec[(size_t)q * nt + tid];
        if constexpr (KIND == kGapCP) Lst.bits[pos + q] = s_bits[(size_t)q * nt + tid];
      }
      continue;
    }
    uint32_t w = pos;  // a long row: enumerate again, writing straight to the list
    if constexpr (KIND == kRefineCP || KIND == kResCP) {
      const auto put = [&](uint32_t item, const real(&e)[3]) { Lst.rec[w++] = make_rec<D, real>((uint32_t)j, item, e); };
      if constexpr (KIND == kRefineCP) enum_refine_cp<Q, D, P>(A, r, j, k, put);
      else enum_resample_cp<Q, D, P>(A, j, k, put);
    } else if constexpr (KIND == kRefineComp || KIND == kResComp) {
      const auto put = [&](uint32_t cp, const real(&e)[3]) { Lst.rec[w++] = make_rec<D, real>(cp, i_comp, e); };
      enum_comp<Q, D, P, KIND == kRefineComp>(A, r, cp_of_cell, (uint32_t)m, k, put);
    } else if constexpr (KIND == kGapCP) {
      const auto put = [&](uint32_t l, uint32_t both, const real(&e)[3]) {
        Lst.bits[w] = both;
        Lst.rec[w++] = make_rec<D, real>((uint32_t)row, l, e);
      };
      enum_gap<Q, D, P, false>(A, row, put);
    } else {
      const auto put = [&](uint32_t jj, uint32_t both, const real(&e)[3]) { Lst.rec[w++] = make_rec<D, real>(jj, both, e); };
      enum_gap<Q, D, P, true>(A, row, put);
    }
  }
}

// ---- backward kernels ---------------------------------------------------------------------------

// Output cotangents into the working layout, then the gap fill, CP side: F_jk = r rho_rest W_k / s_jk
// for the filled entries.  d s_jk / d p_j = sum of
// unit vectors u_jl (e = p_l - p_j); the neighbours' share (-u_jl) comes from sbar (kept per CP and
// direction) in k_bwd_gap_t.  Filled entries do not depend on the gather: their cotangent is cleared.
template <int Q, int D, class P>
__global__ void __launch_bounds__(256) k_bwd_gap(const __grid_constant__ RecK<Q, D, P> K, const double* __restrict__ goff,
                                                 const double* __restrict__ gf, typename P::real* __restrict__ xbarP,
                                                 typename P::real* __restrict__ fbarG, typename P::real* __restrict__ sbarG) {
  using real = typename P::real;
  const int64_t Pn = K.r.P;
  const auto& L = K.r.gap.f;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < Pn; j += (int64_t)gridDim.x * blockDim.x) {
    // the output cotangents (row-major FP64) into the working layout [D][P], [Q][P]
#pragma unroll
    for (int a = 0; a < D; ++a) xbarP[(int64_t)a * Pn + j] = (real)goff[j * D + a];
#pragma unroll
    for (int k = 0; k < Q; ++k) fbarG[(int64_t)k * Pn + j] = (real)gf[j * Q + k];
    const uint32_t em = K.r.emask[j];
    real sbar[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) sbar[k] = 0;
    if (em) {
      const InstK I = K.inst[find_instance(K.inst_base, K.n_inst, K.r.out_cell[j])];
      const uint32_t p0 = L.start[j], p1 = p0 + L.cnt[j];
      real s[Q];
#pragma unroll
      for (int k = 0; k < Q; ++k) s[k] = 0;
      for (uint32_t p = p0; p < p1; ++p) {
        real u[3];
        const real w = K.R - unit_of<D, real>(L.rec[p], u);
        const uint32_t bits = L.bits[p];
#pragma unroll
        for (int k = 0; k < Q; ++k)
          if ((bits >> k) & 1u) s[k] += w;
      }
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        if (((em >> k) & 1u) && s[k] > (real)0) {
          const real Fk = (K.R / s[k]) * (real)(I.rho_rest * K.L.w[k]);
          sbar[k] = -fbarG[(int64_t)k * Pn + j] * Fk / s[k];
          fbarG[(int64_t)k * Pn + j] = 0;
        }
      }
      real xj[3] = {0, 0, 0};
      for (uint32_t p = p0; p < p1; ++p) {
        real u[3];
        unit_of<D, real>(L.rec[p], u);
        const uint32_t bits = L.bits[p];
        real c = 0;
#pragma unroll
        for (int k = 0; k < Q; ++k)
          if ((bits >> k) & 1u) c += sbar[k];
#pragma unroll
        for (int a = 0; a < D; ++a) xj[a] += c * u[a];
      }
#pragma unroll
      for (int a = 0; a < D; ++a) xbarP[(int64_t)a * Pn + j] += xj[a];
    }
#pragma unroll
    for (int k = 0; k < Q; ++k) sbarG[(int64_t)k * Pn + j] = sbar[k];
  }
}

// Gap fill, neighbour side: p_l receives -(sum over shared empty k of sbar_jk) u_jl from every
// filled CP j it is paired with.
template <int Q, int D, class P>
__global__ void __launch_bounds__(256) k_bwd_gap_t(const __grid_constant__ RecK<Q, D, P> K, const typename P::real* __restrict__ sbarG,
                                                   typename P::real* __restrict__ xbarP) {
  using real = typename P::real;
  const int64_t Pn = K.r.P;
  const auto& L = K.r.gap.t;
  for (int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; l < Pn; l += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t q0 = L.start[l], q1 = q0 + L.cnt[l];
    if (q0 == q1) continue;
    real xl[3] = {0, 0, 0};
    for (uint32_t q = q0; q < q1; ++q) {
      const auto pr = L.rec[q];
      real u[3];
      unit_of<D, real>(pr, u);
      real c = 0;
#pragma unroll
      for (int k = 0; k < Q; ++k)
        if ((pr.item >> k) & 1u) c += sbarG[(int64_t)k * Pn + pr.row];
#pragma unroll
      for (int a = 0; a < D; ++a) xl[a] -= c * u[a];
    }
#pragma unroll
    for (int a = 0; a < D; ++a) xbarP[(int64_t)a * Pn + l] += xl[a];
  }
}

// Gather + weights, component side (one thread per component i = (m, k), m fastest):
//   G_i = sum_j a_ij Fbar_jk,  a_ij = (r - d_ij)/sw_i                  -> f*bar_i
//   wbar_ij = f*_i / sw_i (Fbar_jk - G_i)   (cotangent of r - d_ij through F and sw)
//   ybar_i = -sum_j wbar_ij u_ij;  G_i is kept for the CP side
template <int Q, int D, class P>
__global__ void __launch_bounds__(256) k_bwd_gather(const __grid_constant__ RecK<Q, D, P> K,
                                                    const typename P::real* __restrict__ fbarG,
                                                    typename P::real* __restrict__ fsbar, typename P::real* __restrict__ ybar,
                                                    FsG<typename P::real>* __restrict__ fg, typename P::real* __restrict__ wexp) {
  using real = typename P::real;
  const int64_t M = K.r.M, Pn = K.r.P, QM = (int64_t)Q * M;
  const auto& L = K.r.res.t;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < QM; t += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(t / M);
    const int64_t m = t - (int64_t)k * M;
    const real inv = K.r.inv_sw[t];
    const uint32_t q0 = L.start[t], q1 = q0 + L.cnt[t];
    real G = 0;
    if (inv > (real)0) {
      for (uint32_t q = q0; q < q1; ++q) {
        const auto pr = L.rec[q];
        real u[3];
        const real d = unit_of<D, real>(pr, u);
        G += (K.R - d) * inv * fbarG[(int64_t)k * Pn + pr.row];
      }
    }
    fsbar[t] = G;
    const real fst = rec_fstar<Q, D, P>(K, m, k);
    wexp[t] = exp(fst);  // the refine weight, kept for the refine kernels
    const real fsi = fst * inv;
    fg[t] = FsG<real>{inv > (real)0 ? fsi : (real)0, G};
    real y[3] = {0, 0, 0};
    for (uint32_t q = q0; q < q1; ++q) {
      const auto pr = L.rec[q];
      real u[3];
      unit_of<D, real>(pr, u);
      const real wb = inv > (real)0 ? fsi * (fbarG[(int64_t)k * Pn + pr.row] - G) : (real)0;
#pragma unroll
      for (int a = 0; a < D; ++a) y[a] -= wb * u[a];
    }
#pragma unroll
    for (int a = 0; a < D; ++a) ybar[(int64_t)a * QM + t] = y[a];
  }
}

// Per row (CP j, direction k): the CP's share of the resampling pairs (+wbar u, wbar from G of the
// component side), and for a moved CP
// the row's part of W = sum w and sum w e over its refine pairs (w = exp(f*)).
template <int Q, int D, class P>
__global__ void __launch_bounds__(256) k_bwd_rows(const __grid_constant__ RecK<Q, D, P> K,
                                                  const FsG<typename P::real>* __restrict__ fg,
                                                  const typename P::real* __restrict__ wexp,
                                                  const typename P::real* __restrict__ fbarG,
                                                  typename P::real* __restrict__ xrow, typename P::real* __restrict__ Wrow,
                                                  typename P::real* __restrict__ sxrow) {
  using real = typename P::real;
  const int64_t M = K.r.M, Pn = K.r.P, PQ = Pn * Q;
  for (int64_t rw = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; rw < PQ; rw += (int64_t)gridDim.x * blockDim.x) {
    const auto& L = K.r.res.f;
    const int64_t j = rw / Q;
    const int k = (int)(rw - j * Q);
    const real fb = fbarG[(int64_t)k * Pn + j];
    real x[3] = {0, 0, 0};
    for (uint32_t p = L.start[rw], pe = p + L.cnt[rw]; p < pe; ++p) {
      const auto pr = L.rec[p];
      real u[3];
      unit_of<D, real>(pr, u);
      const int64_t m = pr.item / Q;
      // f*·(1/sw)·(fbar − G), the product formed in k_bwd_gather (0 for a dropped component: the
      // pair then adds ±0, which leaves x unchanged)
      const FsG<real> v = fg[(int64_t)k * M + m];
      const real wb = v.fsi * (fb - v.g);
#pragma unroll
      for (int a = 0; a < D; ++a) x[a] += wb * u[a];
    }
#pragma unroll
    for (int a = 0; a < D; ++a) xrow[(int64_t)a * PQ + rw] = x[a];
    const auto& R = K.r.ref.f;
    real W = 0, sx[3] = {0, 0, 0};
    for (uint32_t p = R.start[rw], pe = p + R.cnt[rw]; p < pe; ++p) {
      const auto pr = R.rec[p];
      const uint32_t i = pr.item;
      const real w = wexp[(int64_t)(i % Q) * M + i / Q];
      W += w;
#pragma unroll
      for (int a = 0; a < D; ++a) sx[a] += w * pr.e[a];
    }
    Wrow[rw] = W;
#pragma unroll
    for (int a = 0; a < D; ++a) sxrow[(int64_t)a * PQ + rw] = sx[a];
  }
}

// Per CP: total cotangent of its position; a moved CP is p = sum w_i y_i / W (its centroid cancels),
// so keep W and the move s = sum w_i e_i / W for the component side; an unmoved CP is its centroid,
// whose cotangent goes to the thin cell (already divided by the component count).
template <int Q, int D, class P>
__global__ void __launch_bounds__(256) k_bwd_cp(const __grid_constant__ RecK<Q, D, P> K,
                                                const typename P::real* __restrict__ xrow, const typename P::real* __restrict__ Wrow,
                                                const typename P::real* __restrict__ sxrow, typename P::real* __restrict__ xbarP,
                                                CPBar<typename P::real>* __restrict__ cpb,
                                                typename P::real* __restrict__ cenbar, int64_t ncells) {
  using real = typename P::real;
  const int64_t Pn = K.r.P, PQ = Pn * Q;
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < Pn; j += (int64_t)gridDim.x * blockDim.x) {
    real x[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; ++a) x[a] = xbarP[(int64_t)a * Pn + j];
#pragma unroll 1
    for (int k = 0; k < Q; ++k)
#pragma unroll
      for (int a = 0; a < D; ++a) x[a] += xrow[(int64_t)a * PQ + j * Q + k];
#pragma unroll
    for (int a = 0; a < D; ++a) xbarP[(int64_t)a * Pn + j] = x[a];
    if (K.r.cp_moved[j]) {
      real W = 0, sx[3] = {0, 0, 0};
#pragma unroll 1
      for (int k = 0; k < Q; ++k) {
        W += Wrow[j * Q + k];
#pragma unroll
        for (int a = 0; a < D; ++a) sx[a] += sxrow[(int64_t)a * PQ + j * Q + k];
      }
      CPBar<real> c{};
      c.W = W;
#pragma unroll
      for (int a = 0; a < D; ++a) {
        c.xb[a] = x[a];
        c.s[a] = W > (real)0 ? sx[a] / W : (real)0;
      }
      cpb[j] = c;
    } else {
      const uint32_t F = K.r.cp_thin[j];
      const real invn = (real)1 / (real)K.r.cp_n[j];
#pragma unroll
      for (int a = 0; a < D; ++a) cenbar[(int64_t)a * ncells + F] = x[a] * invn;
    }
  }
}

// Component side of refine and thinning (one thread per component, m fastest):
//   ybar_i += w_i/W_j pbar_j,  f*bar_i += w_i ((e_i - s_j) . pbar_j)/W_j   (refine pairs of i)
//   ybar_i += cenbar[thin cell of i]                                        (thinning)
template <int Q, int D, class P>
__global__ void __launch_bounds__(256) k_bwd_comp(const __grid_constant__ RecK<Q, D, P> K,
                                                  const CPBar<typename P::real>* __restrict__ cpb,
                                                  const typename P::real* __restrict__ cenbar, int64_t ncells,
                                                  const typename P::real* __restrict__ wexp,
                                                  typename P::real* __restrict__ fsbar, typename P::real* __restrict__ ybar) {
  using real = typename P::real;
  const int64_t QM = (int64_t)Q * K.r.M;
  const auto& L = K.r.ref.t;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < QM; t += (int64_t)gridDim.x * blockDim.x) {
    real y[3] = {0, 0, 0};
#pragma unroll
    for (int a = 0; a < D; ++a) y[a] = ybar[(int64_t)a * QM + t];
    real g = fsbar[t];
    const uint32_t F = K.r.thin_cell[t];
    if (F != kNone) {
#pragma unroll
      for (int a = 0; a < D; ++a) y[a] += cenbar[(int64_t)a * ncells + F];
    }
    const uint32_t q0 = L.start[t], q1 = q0 + L.cnt[t];
    if (q0 < q1) {
      const real w = wexp[t];
      for (uint32_t q = q0; q < q1; ++q) {
        const auto pr = L.rec[q];
        const CPBar<real> c = cpb[pr.row];  // a refine pair's control point has moved
        const real wW = w / c.W;
        real dot = 0;
#pragma unroll
        for (int a = 0; a < D; ++a) {
          const real pb = c.xb[a];
          y[a] += wW * pb;
          dot += (pr.e[a] - c.s[a]) * pb;
        }
        g += wW * dot;
      }
    }
    fsbar[t] = g;
#pragma unroll
    for (int a = 0; a < D; ++a) ybar[(int64_t)a * QM + t] = y[a];
  }
}

// Per moment: the dispersion sum over directions (y = x + cd_k) and the collision:
//   xbar_m = sum_k ybar_(m,k)
//   fbar   = (1 - 1/tau) f*bar + (1/tau) J_feq^T f*bar,  taubar_m = -(1/tau^2) f*bar . (feq - f)
template <int Q, int D, class P>
__global__ void __launch_bounds__(256) k_bwd_moment(const __grid_constant__ RecK<Q, D, P> K,
                                                    const typename P::real* __restrict__ fsbar,
                                                    const typename P::real* __restrict__ ybar,
                                                    double* __restrict__ goff_in, double* __restrict__ gf_in,
                                                    double* __restrict__ taupart) {
  using real = typename P::real;
  const int64_t M = K.r.M, QM = (int64_t)Q * M;
  for (int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; m < M; m += (int64_t)gridDim.x * blockDim.x) {
    real x[3] = {0, 0, 0}, g[Q];
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      g[k] = fsbar[(int64_t)k * M + m];
#pragma unroll
      for (int a = 0; a < D; ++a) x[a] += ybar[(int64_t)a * QM + (int64_t)k * M + m];
    }
    const InstK I = K.inst[find_instance(K.inst_base, K.n_inst, K.r.in_cell[m])];
    const real tau = (real)I.tau, itau = (real)1 / tau;
    const real inv = K.L.template inv_cs2_as<real>();
    real rho, u[D], fmfeq[Q], feqw[Q];  // fmfeq = feq - f;  feqw = feq / rho
    if constexpr (std::is_same<P, PF64>::value) {
      real f[Q], mom[D];
      rho = 0;
#pragma unroll
      for (int a = 0; a < D; ++a) mom[a] = 0;
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        f[k] = K.r.in_f[(int64_t)k * M + m];
        rho += f[k];
#pragma unroll
        for (int a = 0; a < D; ++a) mom[a] += f[k] * K.L.c[k][a];
      }
#pragma unroll
      for (int a = 0; a < D; ++a) u[a] = mom[a] / rho;
      real feq[Q];
      equilibrium_all<Q, D, real>(rho, u, K.L, feq);
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        fmfeq[k] = feq[k] - f[k];
        feqw[k] = feq[k] / rho;
      }
    } else {
      float dv[Q], mom[D];
      rho = K.r.in_rho[m];
#pragma unroll
      for (int a = 0; a < D; ++a) mom[a] = 0.f;
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        dv[k] = K.r.in_f[(int64_t)k * M + m];
#pragma unroll
        for (int a = 0; a < D; ++a) mom[a] += dv[k] * K.L.cf[k][a];
      }
#pragma unroll
      for (int a = 0; a < D; ++a) u[a] = mom[a] / rho;
      float deq[Q];
      eq_deviation_f32<Q, D>(rho, u, K.L, deq);
      float m0 = 0.f;  // the forward's projection onto the deviations' mass and momentum
#pragma unroll
      for (int k = 0; k < Q; ++k) m0 += dv[k];
      conserve_moments_f32<Q, D>(deq, m0, mom, K.L);
#pragma unroll
      for (int k = 0; k < Q; ++k) {
        fmfeq[k] = deq[k] - dv[k];
        feqw[k] = K.L.wf[k] + deq[k] / rho;
      }
    }
    real phi = 0, h[D], tb = 0;
#pragma unroll
    for (int a = 0; a < D; ++a) h[a] = 0;
#pragma unroll
    for (int k = 0; k < Q; ++k) {
      phi += g[k] * feqw[k];
      tb += g[k] * fmfeq[k];
      real cu = 0;
#pragma unroll
      for (int a = 0; a < D; ++a) cu += K.L.template c_as<real>(k, a) * u[a];
      const real gw = g[k] * K.L.template w_as<real>(k) * inv;
#pragma unroll
      for (int a = 0; a < D; ++a) h[a] += gw * (K.L.template c_as<real>(k, a) * ((real)1 + inv * cu) - u[a]);
    }
    real hu = 0;
#pragma unroll
    for (int a = 0; a < D; ++a) hu += h[a] * u[a];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
      real hc = 0;
#pragma unroll
      for (int a = 0; a < D; ++a) hc += h[a] * K.L.template c_as<real>(q, a);
      gf_in[m * Q + q] = (double)(((real)1 - itau) * g[q] + itau * (phi + hc - hu));
    }
#pragma unroll
    for (int a = 0; a < D; ++a) goff_in[m * D + a] = (double)x[a];
    taupart[m] = -(double)tb * (double)itau * (double)itau;
  }
}

// Per-instance sum of the tau partials in a fixed order: kTauSplit blocks per instance each sum a
// fixed strided subset (then a tree), and one thread per instance adds the block sums in order.
constexpr int kTauSplit = 32;
__global__ void __launch_bounds__(256) k_bwd_tau(const uint32_t* __restrict__ inst_start, const double* __restrict__ part,
                                                 double* __restrict__ blocksum) {
  __shared__ double sh[256];
  const int b = blockIdx.x / kTauSplit, sblk = blockIdx.x % kTauSplit;
  const uint32_t m0 = inst_start[b], m1 = inst_start[b + 1];
  double s = 0;
  for (uint32_t m = m0 + sblk * 256 + threadIdx.x; m < m1; m += 256 * kTauSplit) s += part[m];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) blocksum[blockIdx.x] = sh[0];
}
__global__ void k_bwd_tau_sum(const double* __restrict__ blocksum, int n_inst, double* __restrict__ gtau) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < n_inst; b += gridDim.x * blockDim.x) {
    double s = 0;
    for (int i = 0; i < kTauSplit; ++i) s += blocksum[b * kTauSplit + i];
    gtau[b] += s;
  }
}

// Export helpers: real -> double, FP32DEV f -> rho*W + dev.
template <class real>
__global__ void k_to_f64(const real* __restrict__ src, int64_t n, double* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (double)src[i];
}
template <int Q>
__global__ void k_dev_to_f64(const float* __restrict__ rho, const float* __restrict__ dev, const double* __restrict__ w, int64_t M,
                             double* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (int64_t)Q * M; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = i / M, m = i - k * M;
    dst[i] = (double)rho[m] * w[k] + (double)dev[i];
  }
}

// ---- the tape ------------------------------------------------------------------------------

struct TapeBase {
  virtual ~TapeBase() = default;
  virtual void set_estimate(double) = 0;
  virtual int clear() = 0;
  virtual int step(cudaStream_t) = 0;
  virtual int backward_all(const double*, const double*, double*, double*, double*, cudaStream_t) = 0;
  virtual int length() const = 0;
  virtual int counts(int, int64_t*) = 0;
  virtual int backward(int, const double*, const double*, double*, double*, double*, cudaStream_t) = 0;
  virtual int export_(int, int, void*, int64_t, int64_t*, cudaStream_t) = 0;
};

inline unsigned grid_for(int64_t n, int threads = 256) {
  return std::max(1u, std::min<unsigned>(div_up(std::max<int64_t>(n, 1), threads), (unsigned)sm_count() * 16));
}

// Canonical row-ordered copy of a list (export only): out[prefix[r] + q] = rec[start[r] + q].
template <class real, int D>
__global__ void k_rows_compact(PairList<real, D> L, const uint32_t* __restrict__ prefix, uint32_t* __restrict__ item,
                               uint32_t* __restrict__ bits, double* __restrict__ e, int64_t n) {
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < L.rows; r += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t o = prefix[r], s0 = L.start[r], c = L.cnt[r];
    for (uint32_t q = 0; q < c; ++q) {
      const PairRec<real, D> pr = L.rec[s0 + q];
      if (item) item[o + q] = pr.item;
      if (bits) bits[o + q] = L.bits[s0 + q];
      if (e) {
#pragma unroll
        for (int a = 0; a < D; ++a) e[(int64_t)a * n + o + q] = (double)pr.e[a];
      }
    }
  }
}

template <int Q, int D, class P>
struct TapeImpl : TapeBase, StepHook {
  using real = typename P::real;
  SimBase* sim;
  std::vector<StepRec<real, D>> steps;
  DevArena rec_mem, tmp_mem, bwd_mem;
  StepRec<real, D> cur{};
  LatK<Q, D> L{};
  const InstK* inst = nullptr;
  const uint32_t* inst_base = nullptr;
  int n_inst = 0;
  real R = 0;
  int64_t ncells = 0;
  double* wk = nullptr;        // W_k in FP64 (export of FP32DEV f); written once, at the first step
  bool wk_set = false;
  uint32_t* hbuf = nullptr;    // mapped pinned host words read back while recording
  uint32_t* hbuf_dev = nullptr;  // the same words as seen from the device
  uint32_t* d_count = nullptr; // slot counters of the six lists
  double per_row[6] = {16, 16, 16, 16, 4, 4};  // capacity estimate: pairs per row, grown as seen
  uint64_t known_version = ~0ull - 1;  // simulator state version right after this tape's last step
  uint32_t known_P = 0;                // and its moment count
  cudaEvent_t done = nullptr;
  cudaStream_t side = nullptr;   // second stream for the recording kernels
  double* io[1] = {nullptr};     // intermediate cotangents of backward_all
  int64_t io_cap = 0;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // The six lists of a recorded step run on two streams of their own (side: component side and gap
  // fill, side2: control-point side) and read only the tape and the step's output state, so they
  // overlap the simulator's next step.  Whatever reads their counters or lists, or could overwrite
  // what they read, first waits on lists_done.
  cudaStream_t side2 = nullptr;
  cudaEvent_t ev_join2 = nullptr, lists_done = nullptr;
  bool lists_pending = false;

  explicit TapeImpl(SimBase* s) : sim(s) {}
  ~TapeImpl() override {
    if (lists_pending) cudaEventSynchronize(lists_done);
    if (io[0]) cudaFree(io[0]);
    if (side) cudaStreamDestroy(side);
    if (side2) cudaStreamDestroy(side2);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (ev_join2) cudaEventDestroy(ev_join2);
    if (lists_done) cudaEventDestroy(lists_done);
    if (done) cudaEventDestroy(done);
    if (hbuf) cudaFreeHost(hbuf);
    if (d_count) cudaFree(d_count);
    if (wk) cudaFree(wk);
  }

  int init() {
    DBM_CUDA(cudaEventCreateWithFlags(&done, cudaEventDisableTiming));
    DBM_CUDA(cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking));
    DBM_CUDA(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
    DBM_CUDA(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    DBM_CUDA(cudaStreamCreateWithFlags(&side2, cudaStreamNonBlocking));
    DBM_CUDA(cudaEventCreateWithFlags(&ev_join2, cudaEventDisableTiming));
    DBM_CUDA(cudaEventCreateWithFlags(&lists_done, cudaEventDisableTiming));
    DBM_CUDA(cudaHostAlloc(&hbuf, 64, cudaHostAllocMapped));
    DBM_CUDA(cudaHostGetDevicePointer(&hbuf_dev, hbuf, 0));
    DBM_CUDA(cudaMalloc(&d_count, 6 * 4));
    DBM_CUDA(cudaMalloc(&wk, sizeof(double) * Q));
    return DBM_OK;
  }

  int clear() override {
    if (lists_pending) DBM_CUDA(cudaEventSynchronize(lists_done));  // their memory is about to be reused
    lists_pending = false;
    steps.clear();
    pending = -1;
    invalid = false;
    rec_mem.reset();
    return DBM_OK;
  }
  int length() const override { return (int)steps.size(); }
  void set_estimate(double per) override {
    for (auto& v : per_row) v = per;
  }
  int counts(int i, int64_t* c) override {
    if (i < 0 || i >= (int)steps.size()) { set_last_error("tape: no step %d", i); return DBM_ERR_INVALID; }
    DBM_TRY(settle(nullptr));
    const auto& r = steps[i];
    c[0] = r.M; c[1] = r.P; c[2] = r.ref.f.n; c[3] = r.res.f.n; c[4] = r.gap.f.n; c[5] = 0; c[6] = 0; c[7] = 0;
    return DBM_OK;
  }

  int step(cudaStream_t s) override {
    if (sim->kappa_soft > 0) {  // spawned control points have no recorded VJP
      set_last_error("tape: the adjoint does not cover the soft-outer spawn (DBM_OPT_KAPPA_SOFT)");
      return DBM_ERR_INVALID;
    }
    cur = StepRec<real, D>{};
    known_version = ~0ull - 1;
    DBM_TRY(sim->step_hooked(this, s));
    steps.push_back(cur);
    known_version = sim->version;
    known_P = (uint32_t)cur.P;
    return DBM_OK;
  }

  // Copy n device words into hbuf[0..n) and wait for them.
  int fetch(const uint32_t* const* src, int n, cudaStream_t s) {
    FetchSrc fs{};
    for (int i = 0; i < n && i < 8; ++i) fs.p[i] = src[i];
    k_fetch_words<<<1, 32, 0, s>>>(fs, n < 8 ? n : 8, hbuf_dev);
    DBM_LAUNCH_CHECK();
    DBM_CUDA(cudaStreamSynchronize(s));
    return DBM_OK;
  }

  int before(const void* av, cudaStream_t s) override {
    const Args<Q, D, P>& A = *(const Args<Q, D, P>*)av;
    if (A.any_obstacle) {
      set_last_error("tape: the adjoint does not cover obstacles (bounced components)");
      return DBM_ERR_INVALID;
    }
    L = A.L;
    inst = A.inst;
    inst_base = A.inst_base;
    n_inst = A.n_inst;
    R = A.R;
    ncells = A.ncells;
    uint32_t M;
    if (sim->version == known_version + 1) {  // the state is the output of this tape's last step
      M = known_P;
    } else {
      const uint32_t* src[1] = {A.a.count};
      DBM_TRY(fetch(src, 1, s));
      M = hbuf[0];
    }
    if (!wk_set) {  // a copy from pageable memory waits for the stream: once, not at every step
      DBM_CUDA(cudaMemcpyAsync(wk, L.w, sizeof(double) * Q, cudaMemcpyHostToDevice, s));
      wk_set = true;
    }
    StepRec<real, D>& r = cur;
    r.M = M;
    DBM_TRY(rec_mem.get(&r.in_cell, M));
    DBM_TRY(rec_mem.get(&r.in_off, (int64_t)D * M));
    DBM_TRY(rec_mem.get(&r.in_f, (int64_t)Q * M));
    DBM_TRY(rec_mem.get(&r.fs, (int64_t)Q * M));
    DBM_TRY(rec_mem.get(&r.thin_cell, (int64_t)Q * M));
    DBM_TRY(rec_mem.get(&r.inv_sw, (int64_t)Q * M));
    DBM_TRY(rec_mem.get(&r.inst_start, n_inst + 1));
    DBM_TRY(rec_mem.get(&r.in_start, ncells + 1));
    DBM_CUDA(cudaMemcpyAsync(r.in_start, A.a.start, (size_t)(ncells + 1) * 4, cudaMemcpyDeviceToDevice, s));
    if (M == 0) return DBM_OK;
    DBM_CUDA(cudaMemcpyAsync(r.in_cell, A.a.cell, (size_t)M * 4, cudaMemcpyDeviceToDevice, s));
    DBM_CUDA(cudaMemcpy2DAsync(r.in_off, (size_t)M * sizeof(real), A.a.off, (size_t)A.mcap * sizeof(real),
                               (size_t)M * sizeof(real), D, cudaMemcpyDeviceToDevice, s));
    if constexpr (std::is_same<P, PF64>::value) {
      DBM_CUDA(cudaMemcpy2DAsync(r.in_f, (size_t)M * 8, A.a.f64, (size_t)A.mcap * 8, (size_t)M * 8, Q,
                                 cudaMemcpyDeviceToDevice, s));
    } else {
      DBM_TRY(rec_mem.get(&r.in_rho, M));
      DBM_CUDA(cudaMemcpyAsync(r.in_rho, A.a.rho, (size_t)M * 4, cudaMemcpyDeviceToDevice, s));
      DBM_CUDA(cudaMemcpy2DAsync(r.in_f, (size_t)M * 4, A.a.dev, (size_t)A.mcap * 4, (size_t)M * 4, Q,
                                 cudaMemcpyDeviceToDevice, s));
    }
    return DBM_OK;
  }

  PairList<real, D>& list_of(StepRec<real, D>& r, int kind) {
    switch (kind) {
      case kRefineCP: return r.ref.f;
      case kRefineComp: return r.ref.t;
      case kResCP: return r.res.f;
      case kResComp: return r.res.t;
      case kGapCP: return r.gap.f;
      default: return r.gap.t;
    }
  }

  int alloc_list(PairList<real, D>& Lst, int64_t rows, int64_t cap, bool with_bits) {
    Lst.rows = rows;
    Lst.cap = cap;
    DBM_TRY(rec_mem.get(&Lst.start, rows));
    DBM_TRY(rec_mem.get(&Lst.cnt, rows));
    DBM_TRY(rec_mem.get(&Lst.rec, cap));
    if (with_bits) DBM_TRY(rec_mem.get(&Lst.bits, cap));
    return DBM_OK;
  }

  int launch_list(const Args<Q, D, P>& A, const StepRec<real, D>& r, int kind, const uint32_t* cp_of_cell,
                  cudaStream_t s) {
    const PairList<real, D>& Lst = list_of(const_cast<StepRec<real, D>&>(r), kind);
    DBM_CUDA(cudaMemsetAsync(d_count + kind, 0, 4, s));
    if (Lst.rows == 0) return DBM_OK;
    const unsigned g = grid_for(Lst.rows);
    switch (kind) {
      case kRefineCP: return launch_list_k<kRefineCP>(A, r, cp_of_cell, g, s);
      case kRefineComp: return launch_list_k<kRefineComp>(A, r, cp_of_cell, g, s);
      case kResCP: return launch_list_k<kResCP>(A, r, cp_of_cell, g, s);
      case kResComp: return launch_list_k<kResComp>(A, r, cp_of_cell, g, s);
      case kGapCP: return launch_list_k<kGapCP>(A, r, cp_of_cell, g, s);
      default: return launch_list_k<kGapNb>(A, r, cp_of_cell, g, s);
    }
  }

  bool list_attr_set[6] = {false, false, false, false, false, false};
  template <int KIND>
  int launch_list_k(const Args<Q, D, P>& A, const StepRec<real, D>& r, const uint32_t* cp_of_cell, unsigned g,
                    cudaStream_t s) {
    const size_t sm = list_smem_bytes<real, D, KIND>(256);
    if (!list_attr_set[KIND]) {
      DBM_CUDA(cudaFuncSetAttribute((const void*)k_list<Q, D, P, KIND>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)sm));
      list_attr_set[KIND] = true;
    }
    k_list<Q, D, P, KIND><<<g, 256, sm, s>>>(A, r, cp_of_cell, d_count + KIND);
    DBM_LAUNCH_CHECK();
    return DBM_OK;
  }

  int after(const void* av, cudaStream_t s) override {
    const Args<Q, D, P>& A = *(const Args<Q, D, P>*)av;
    StepRec<real, D>& r = cur;
    tmp_mem.reset();
    rec_stream = s;
    if (invalid) return DBM_ERR_CAPACITY;
    if (lists_pending) {  // the previous step's lists ran beside this step: wait for their counters
      DBM_CUDA(cudaStreamWaitEvent(s, lists_done, 0));
      lists_pending = false;
    }
    if (pending >= 0) {  // one synchronisation: this step's count and the previous step's counters
      const uint32_t* src[8] = {A.status, A.d_P, pending_counts, pending_counts + 1, pending_counts + 2,
                                pending_counts + 3, pending_counts + 4, pending_counts + 5};
      DBM_TRY(fetch(src, 8, s));
      const uint32_t st = hbuf[0], pn = hbuf[1];
      uint32_t need[6];
      for (int i = 0; i < 6; ++i) need[i] = hbuf[2 + i];
      DBM_TRY(settle_counts(need));
      hbuf[0] = st;
      hbuf[1] = pn;
    } else {
      const uint32_t* src[2] = {A.status, A.d_P};
      DBM_TRY(fetch(src, 2, s));
    }
    DBM_TRY(rec_mem.get(&cur_counts, 6));
    if (hbuf[0] & ST_NONFINITE) {
      set_last_error("tape: the step produced a non-finite refine move; it has no derivative");
      return DBM_ERR_INVALID;
    }
    r.P = hbuf[1];
    const int64_t M = r.M, Pn = r.P;
    if (M > 0) {
      if constexpr (std::is_same<P, PF64>::value) {
        DBM_CUDA(cudaMemcpy2DAsync(r.fs, (size_t)M * 8, A.a.f64, (size_t)A.mcap * 8, (size_t)M * 8, Q,
                                   cudaMemcpyDeviceToDevice, s));
      } else {
        DBM_CUDA(cudaMemcpy2DAsync(r.fs, (size_t)M * 4, A.a.dev, (size_t)A.mcap * 4, (size_t)M * 4, Q,
                                   cudaMemcpyDeviceToDevice, s));
      }
      DBM_CUDA(cudaMemcpy2DAsync(r.inv_sw, (size_t)M * sizeof(real), A.sw, (size_t)A.mcap * sizeof(real),
                                 (size_t)M * sizeof(real), Q, cudaMemcpyDeviceToDevice, s));
      k_rec_thin_cell<Q, D, P><<<grid_for(M), 256, 0, s>>>(A, M, r.thin_cell);
      DBM_LAUNCH_CHECK();
    }
    k_rec_inst_start<Q, D, P><<<1, 256, 0, s>>>(A, r.inst_start);
    DBM_LAUNCH_CHECK();
    DBM_TRY(rec_mem.get(&r.cp_thin, Pn));
    DBM_TRY(rec_mem.get(&r.cp_n, Pn));
    DBM_TRY(rec_mem.get(&r.cp_moved, Pn));
    DBM_TRY(rec_mem.get(&r.cp_cen, (int64_t)D * Pn));
    DBM_TRY(rec_mem.get(&r.out_cell, Pn));
    DBM_TRY(rec_mem.get(&r.out_off, (int64_t)D * Pn));
    DBM_TRY(rec_mem.get(&r.emask, Pn));
    uint32_t* cp_of_cell;  // kept with the step: its lists may still run during the next step
    DBM_TRY(rec_mem.get(&cp_of_cell, ncells));
    DBM_CUDA(cudaMemsetAsync(cp_of_cell, 0xff, (size_t)ncells * 4, s));
    if (Pn > 0) {
      k_rec_cp<Q, D, P><<<grid_for(Pn), 256, 0, s>>>(A, r, cp_of_cell);
      DBM_LAUNCH_CHECK();
    }
    // the six lists, in one pass each
    const int64_t rows[6] = {Pn * Q, (int64_t)Q * M, Pn * Q, (int64_t)Q * M, Pn, Pn};
    for (int kind = 0; kind < 6; ++kind) {
      const int64_t cap = (int64_t)(per_row[kind] * 1.25 * (double)rows[kind]) + 1024;
      DBM_TRY(alloc_list(list_of(r, kind), rows[kind], cap, kind == kGapCP));
    }
    // The lists read the input moments from the tape's copies (the next step overwrites the
    // simulator's input buffer), the emptiness masks from the tape, and the output state, which
    // the next step only reads (its collision changes f, which no list reads).  So they run on two
    // streams of their own beside the next step: control-point side on side2, component side and
    // gap fill on side.
    Args<Q, D, P> AL = A;
    AL.a.start = r.in_start;
    AL.a.cell = r.in_cell;
    AL.a.off = r.in_off;
    AL.mcap = M;
    AL.emask = r.emask;
    DBM_CUDA(cudaEventRecord(ev_fork, s));
    DBM_CUDA(cudaStreamWaitEvent(side, ev_fork, 0));
    DBM_CUDA(cudaStreamWaitEvent(side2, ev_fork, 0));
    for (int kind : {kRefineCP, kResCP}) DBM_TRY(launch_list(AL, r, kind, cp_of_cell, side2));
    for (int kind : {kRefineComp, kResComp, kGapCP, kGapNb}) DBM_TRY(launch_list(AL, r, kind, cp_of_cell, side));
    DBM_CUDA(cudaEventRecord(ev_join2, side2));
    DBM_CUDA(cudaStreamWaitEvent(side, ev_join2, 0));
    // the slot counters are read at the next synchronisation (see settle), after lists_done
    DBM_CUDA(cudaMemcpyAsync(r_counts_dev(), d_count, 6 * 4, cudaMemcpyDeviceToDevice, side));
    DBM_CUDA(cudaEventRecord(lists_done, side));
    lists_pending = true;
    pending = (int)steps.size();  // this step's index once step() appends it
    pending_counts = cur_counts;
    return DBM_OK;
  }

  // Per-step device copy of the six slot counters (in the tape's arena).
  uint32_t* cur_counts = nullptr;
  uint32_t* r_counts_dev() { return cur_counts; }
  int pending = -1;                 // step whose counters are not read yet
  cudaStream_t rec_stream = nullptr;  // the simulator's stream the recording kernels ran on
  uint32_t* pending_counts = nullptr;
  bool invalid = false;             // a list outgrew its capacity: the tape must be recorded again

  // Read the pending step's counters (the caller synchronises `s` or has just done so through
  // fetch): set the list sizes, grow the capacity estimates, and mark the tape invalid if a list
  // did not fit.  Returns DBM_ERR_CAPACITY then.
  int settle_counts(const uint32_t* need) {
    StepRec<real, D>& r = steps[pending];
    const int idx = pending;
    pending = -1;
    bool over = false;
    for (int kind = 0; kind < 6; ++kind) {
      PairList<real, D>& Lst = list_of(r, kind);
      Lst.n = need[kind];
      if (Lst.rows > 0) per_row[kind] = std::max(per_row[kind], (double)need[kind] / (double)Lst.rows);
      over |= (int64_t)need[kind] > Lst.cap;
    }
    if (over) {
      invalid = true;
      set_last_error("tape: a neighbour list of step %d outgrew its estimate; restore the state of the first "
                     "recorded step, clear the tape and record again (the estimate has grown)", idx);
      return DBM_ERR_CAPACITY;
    }
    if (need[kRefineCP] != need[kRefineComp] || need[kResCP] != need[kResComp] || need[kGapCP] != need[kGapNb]) {
      invalid = true;
      set_last_error("tape: the two orientations of a neighbour list disagree (%u/%u, %u/%u, %u/%u)",
                     need[0], need[1], need[2], need[3], need[4], need[5]);
      return DBM_ERR_STATE;
    }
    return DBM_OK;
  }

  // Settle the pending step now (one synchronisation of the stream the recording ran on); no-op
  // when nothing is pending.
  int settle(cudaStream_t) {
    if (invalid) return DBM_ERR_CAPACITY;
    if (pending < 0) return DBM_OK;
    cudaStream_t s = rec_stream;
    if (lists_pending) {
      DBM_CUDA(cudaStreamWaitEvent(s, lists_done, 0));
      lists_pending = false;
    }
    const uint32_t* src[6] = {pending_counts, pending_counts + 1, pending_counts + 2, pending_counts + 3,
                              pending_counts + 4, pending_counts + 5};
    DBM_TRY(fetch(src, 6, s));
    uint32_t need[6];
    for (int i = 0; i < 6; ++i) need[i] = hbuf[i];
    return settle_counts(need);
  }

  RecK<Q, D, P> reck(const StepRec<real, D>& r) const {
    RecK<Q, D, P> K;
    K.L = L;
    K.inst = inst;
    K.inst_base = inst_base;
    K.n_inst = n_inst;
    K.R = R;
    K.r = r;
    return K;
  }

  int backward(int idx, const double* goff_out, const double* gf_out, double* goff_in, double* gf_in, double* gtau,
               cudaStream_t s) override {
    if (idx < 0 || idx >= (int)steps.size()) { set_last_error("tape: no step %d", idx); return DBM_ERR_INVALID; }
    DBM_TRY(settle(s));
    const StepRec<real, D>& r = steps[idx];
    const int64_t M = r.M, Pn = r.P, QM = (int64_t)Q * M, PQ = Pn * Q;
    if ((Pn > 0 && (!goff_out || !gf_out)) || (M > 0 && (!goff_in || !gf_in)) || !gtau) {
      set_last_error("tape backward: null cotangent");
      return DBM_ERR_INVALID;
    }
    DBM_CUDA(cudaStreamWaitEvent(s, done, 0));  // the previous call's scratch is free
    bwd_mem.reset();
    real *xbarP, *fbarG, *sbarG, *fsbar, *ybar, *wexp, *xrow, *Wrow, *sxrow, *cenbar;
    CPBar<real>* cpb;
    FsG<real>* fg;
    double *taupart, *blocksum;
    DBM_TRY(bwd_mem.get(&xbarP, (int64_t)D * Pn));
    DBM_TRY(bwd_mem.get(&fbarG, (int64_t)Q * Pn));
    DBM_TRY(bwd_mem.get(&sbarG, (int64_t)Q * Pn));
    DBM_TRY(bwd_mem.get(&fsbar, QM));
    DBM_TRY(bwd_mem.get(&ybar, (int64_t)D * QM));
    DBM_TRY(bwd_mem.get(&fg, QM));
    DBM_TRY(bwd_mem.get(&wexp, QM));
    DBM_TRY(bwd_mem.get(&xrow, (int64_t)D * PQ));
    DBM_TRY(bwd_mem.get(&Wrow, PQ));
    DBM_TRY(bwd_mem.get(&sxrow, (int64_t)D * PQ));
    DBM_TRY(bwd_mem.get(&cpb, Pn));
    DBM_TRY(bwd_mem.get(&cenbar, (int64_t)D * ncells));
    DBM_TRY(bwd_mem.get(&taupart, M));
    DBM_TRY(bwd_mem.get(&blocksum, (int64_t)n_inst * kTauSplit));
    const RecK<Q, D, P> K = reck(r);
    DBM_CUDA(cudaMemsetAsync(cenbar, 0, sizeof(real) * (size_t)D * ncells, s));
    if (Pn > 0) {
      k_bwd_gap<Q, D, P><<<grid_for(Pn), 256, 0, s>>>(K, goff_out, gf_out, xbarP, fbarG, sbarG);
      DBM_LAUNCH_CHECK();
      if (r.gap.f.n > 0) {
        k_bwd_gap_t<Q, D, P><<<grid_for(Pn), 256, 0, s>>>(K, sbarG, xbarP);
        DBM_LAUNCH_CHECK();
      }
    }
    if (M > 0) {
      k_bwd_gather<Q, D, P><<<grid_for(QM), 256, 0, s>>>(K, fbarG, fsbar, ybar, fg, wexp);
      DBM_LAUNCH_CHECK();
    }
    if (Pn > 0) {
      k_bwd_rows<Q, D, P><<<grid_for(PQ), 256, 0, s>>>(K, fg, wexp, fbarG, xrow, Wrow, sxrow);
      DBM_LAUNCH_CHECK();
      k_bwd_cp<Q, D, P><<<grid_for(Pn), 256, 0, s>>>(K, xrow, Wrow, sxrow, xbarP, cpb, cenbar, ncells);
      DBM_LAUNCH_CHECK();
    }
    if (M > 0) {
      k_bwd_comp<Q, D, P><<<grid_for(QM), 256, 0, s>>>(K, cpb, cenbar, ncells, wexp, fsbar, ybar);
      DBM_LAUNCH_CHECK();
      k_bwd_moment<Q, D, P><<<grid_for(M), 256, 0, s>>>(K, fsbar, ybar, goff_in, gf_in, taupart);
      DBM_LAUNCH_CHECK();
      k_bwd_tau<<<n_inst * kTauSplit, 256, 0, s>>>(r.inst_start, taupart, blocksum);
      DBM_LAUNCH_CHECK();
      k_bwd_tau_sum<<<div_up(n_inst, 256), 256, 0, s>>>(blocksum, n_inst, gtau);
      DBM_LAUNCH_CHECK();
    }
    DBM_CUDA(cudaEventRecord(done, s));
    return DBM_OK;
  }

  // Every recorded step in reverse: the output cotangents of the last step in, the input
  // cotangents of the first step out, intermediate ones in two device buffers of the tape.
  int backward_all(const double* goff_out, const double* gf_out, double* goff_in, double* gf_in, double* gtau,
                   cudaStream_t s) override {
    const int n = (int)steps.size();
    if (n == 0) { set_last_error("tape: nothing recorded"); return DBM_ERR_INVALID; }
    DBM_TRY(settle(s));
    int64_t cap = 1;
    for (const auto& r : steps) cap = std::max(cap, std::max(r.M, r.P));
    if (cap > io_cap) {
      if (io[0]) cudaFree(io[0]);
      io[0] = nullptr;
      DBM_CUDA(cudaMalloc(&io[0], sizeof(double) * (size_t)cap * (D + Q) * 2));
      io_cap = cap;
    }
    double* buf[2] = {io[0], io[0] + (size_t)io_cap * (D + Q)};
    const double* go = goff_out;
    const double* gfo = gf_out;
    for (int i = n - 1; i >= 0; --i) {
      double* oo = i == 0 ? goff_in : buf[i & 1];
      double* of = i == 0 ? gf_in : buf[i & 1] + (size_t)io_cap * D;
      DBM_TRY(backward(i, go, gfo, oo, of, gtau, s));
      go = oo;
      gfo = of;
    }
    return DBM_OK;
  }

  // A list in canonical CSR form (rows ascending, each row's pairs in enumeration order):
  // what = 0 start u32[rows + 1], 1 items u32[n], 2 displacements f64[D][n], 3 bits u32[n].
  int export_list(const PairList<real, D>& Lst, int what, void* dst, int64_t nbytes, int64_t* needed, cudaStream_t s) {
    const int64_t n = Lst.n;
    const int64_t sz = what == 0 ? (Lst.rows + 1) * 4 : what == 2 ? n * 8 * D : n * 4;
    if (needed) *needed = sz;
    if (!dst) return DBM_OK;
    if (nbytes < sz) { set_last_error("tape export: destination too small"); return DBM_ERR_INVALID; }
    uint32_t* prefix;
    DBM_TRY(tmp_mem.get(&prefix, Lst.rows + 1));
    DBM_CUDA(cudaMemsetAsync(prefix + Lst.rows, 0, 4, s));
    if (Lst.rows > 0) DBM_CUDA(cudaMemcpyAsync(prefix, Lst.cnt, (size_t)Lst.rows * 4, cudaMemcpyDeviceToDevice, s));
    char* stmp;
    DBM_TRY(tmp_mem.get(&stmp, (int64_t)scan_tmp_bytes(Lst.rows + 1)));
    DBM_TRY(scan_exclusive_u32(prefix, prefix, Lst.rows + 1, nullptr, nullptr, stmp, s));
    if (what == 0) {
      DBM_CUDA(cudaMemcpyAsync(dst, prefix, (size_t)sz, cudaMemcpyDeviceToDevice, s));
    } else if (n > 0 && Lst.rows > 0) {
      k_rows_compact<real, D><<<grid_for(Lst.rows), 256, 0, s>>>(Lst, prefix, what == 1 ? (uint32_t*)dst : nullptr,
                                                                  what == 3 ? (uint32_t*)dst : nullptr,
                                                                  what == 2 ? (double*)dst : nullptr, n);
      DBM_LAUNCH_CHECK();
    }
    DBM_CUDA(cudaStreamSynchronize(s));  // tmp_mem may be reused by the next call
    return DBM_OK;
  }

  int export_(int idx, int what, void* dst, int64_t nbytes, int64_t* needed, cudaStream_t s) override {
    if (idx < 0 || idx >= (int)steps.size()) { set_last_error("tape: no step %d", idx); return DBM_ERR_INVALID; }
    DBM_TRY(settle(s));
    const StepRec<real, D>& r = steps[idx];
    const void* src = nullptr;
    int64_t n = 0;
    bool conv = false;  // real -> f64
    switch (what) {
      case DBM_TAPE_IN_CELL: src = r.in_cell; n = r.M; break;
      case DBM_TAPE_IN_OFF: src = r.in_off; n = (int64_t)D * r.M; conv = true; break;
      case DBM_TAPE_IN_F:
      case DBM_TAPE_FSTAR: src = what == DBM_TAPE_IN_F ? r.in_f : r.fs; n = (int64_t)Q * r.M; conv = true; break;
      case DBM_TAPE_THIN_CELL: src = r.thin_cell; n = (int64_t)Q * r.M; break;
      case DBM_TAPE_CP_THIN: src = r.cp_thin; n = r.P; break;
      case DBM_TAPE_CP_COUNT: src = r.cp_n; n = r.P; break;
      case DBM_TAPE_CP_CEN: src = r.cp_cen; n = (int64_t)D * r.P; conv = true; break;
      case DBM_TAPE_CP_MOVED: src = r.cp_moved; n = r.P; break;
      case DBM_TAPE_OUT_CELL: src = r.out_cell; n = r.P; break;
      case DBM_TAPE_OUT_OFF: src = r.out_off; n = (int64_t)D * r.P; conv = true; break;
      case DBM_TAPE_EMPTY: src = r.emask; n = r.P; break;
      case DBM_TAPE_INV_SW: src = r.inv_sw; n = (int64_t)Q * r.M; conv = true; break;
      case DBM_TAPE_REFINE_START: return export_list(r.ref.f, 0, dst, nbytes, needed, s);
      case DBM_TAPE_REFINE_ITEM: return export_list(r.ref.f, 1, dst, nbytes, needed, s);
      case DBM_TAPE_REFINE_E: return export_list(r.ref.f, 2, dst, nbytes, needed, s);
      case DBM_TAPE_RES_START: return export_list(r.res.f, 0, dst, nbytes, needed, s);
      case DBM_TAPE_RES_ITEM: return export_list(r.res.f, 1, dst, nbytes, needed, s);
      case DBM_TAPE_RES_E: return export_list(r.res.f, 2, dst, nbytes, needed, s);
      case DBM_TAPE_GAP_START: return export_list(r.gap.f, 0, dst, nbytes, needed, s);
      case DBM_TAPE_GAP_ITEM: return export_list(r.gap.f, 1, dst, nbytes, needed, s);
      case DBM_TAPE_GAP_BITS: return export_list(r.gap.f, 3, dst, nbytes, needed, s);
      case DBM_TAPE_GAP_E: return export_list(r.gap.f, 2, dst, nbytes, needed, s);
      case DBM_TAPE_INST_START: src = r.inst_start; n = n_inst + 1; break;
      default: set_last_error("tape export: unknown array %d", what); return DBM_ERR_INVALID;
    }
    const int64_t sz = n * (conv ? 8 : 4);
    if (needed) *needed = sz;
    if (!dst || n == 0) return DBM_OK;
    if (nbytes < sz) { set_last_error("tape export: destination too small"); return DBM_ERR_INVALID; }
    if (!conv) {
      DBM_CUDA(cudaMemcpyAsync(dst, src, (size_t)sz, cudaMemcpyDeviceToDevice, s));
    } else if (!std::is_same<P, PF64>::value && (what == DBM_TAPE_IN_F || what == DBM_TAPE_FSTAR)) {
      k_dev_to_f64<Q><<<grid_for(n), 256, 0, s>>>((const float*)r.in_rho, (const float*)src, wk, r.M, (double*)dst);
      DBM_LAUNCH_CHECK();
    } else {
      k_to_f64<real><<<grid_for(n), 256, 0, s>>>((const real*)src, n, (double*)dst);
      DBM_LAUNCH_CHECK();
    }
    return DBM_OK;
  }
};

}  // namespace dbm

using namespace dbm;

struct dbm_tape {
  TapeBase* impl;
};

template <class P>
static int make_tape(SimBase* sim, TapeBase** out) {
  return dispatch_lattice(sim->lattice, [&](auto tag) -> int {
    using LT = decltype(tag);
    auto* t = new TapeImpl<LT::Q, LT::D, P>(sim);
    int rc = t->init();
    if (rc != DBM_OK) { delete t; return rc; }
    *out = t;
    return DBM_OK;
  });
}

#define TAPE_CHECK(t)                        \
  if (!(t) || !(t)->impl) {                  \
    set_last_error("null tape handle");      \
    return DBM_ERR_INVALID;                  \
  }

extern "C" {

int dbm_tape_create(dbm_sim* sim, dbm_tape** out) {
  if (!sim || !sim->impl || !out) { set_last_error("dbm_tape_create: bad arguments"); return DBM_ERR_INVALID; }
  TapeBase* impl = nullptr;
  int rc = sim->impl->precision == DBM_FP64 ? make_tape<PF64>(sim->impl, &impl) : make_tape<PF32>(sim->impl, &impl);
  if (rc != DBM_OK) return rc;
  *out = new dbm_tape{impl};
  return DBM_OK;
}
int dbm_tape_destroy(dbm_tape* t) {
  if (!t) return DBM_OK;
  delete t->impl;
  delete t;
  return DBM_OK;
}
int dbm_tape_clear(dbm_tape* t) {
  TAPE_CHECK(t);
  return t->impl->clear();
}
int dbm_tape_step(dbm_tape* t, void* stream) {
  TAPE_CHECK(t);
  return t->impl->step((cudaStream_t)stream);
}
int dbm_tape_set_estimate(dbm_tape* t, double pairs_per_row) {
  TAPE_CHECK(t);
  if (!(pairs_per_row >= 0)) { set_last_error("dbm_tape_set_estimate: bad estimate"); return DBM_ERR_INVALID; }
  t->impl->set_estimate(pairs_per_row);
  return DBM_OK;
}
int dbm_tape_record(dbm_tape* t, int32_t steps, void* stream) {
  TAPE_CHECK(t);
  for (int i = 0; i < steps; ++i) DBM_TRY(t->impl->step((cudaStream_t)stream));
  return DBM_OK;
}
int dbm_tape_backward_all(dbm_tape* t, const double* goff_out, const double* gf_out, double* goff_in, double* gf_in,
                          double* gtau, void* stream) {
  TAPE_CHECK(t);
  return t->impl->backward_all(goff_out, gf_out, goff_in, gf_in, gtau, (cudaStream_t)stream);
}
int32_t dbm_tape_length(dbm_tape* t) {
  if (!t || !t->impl) return -1;
  return t->impl->length();
}
int dbm_tape_counts(dbm_tape* t, int32_t index, int64_t* counts) {
  TAPE_CHECK(t);
  if (!counts) return DBM_ERR_INVALID;
  return t->impl->counts(index, counts);
}
int dbm_tape_backward(dbm_tape* t, int32_t index, const double* goff_out, const double* gf_out, double* goff_in,
                      double* gf_in, double* gtau, void* stream) {
  TAPE_CHECK(t);
  return t->impl->backward(index, goff_out, gf_out, goff_in, gf_in, gtau, (cudaStream_t)stream);
}
int dbm_tape_export(dbm_tape* t, int32_t index, int32_t what, void* dst, int64_t bytes, int64_t* needed, void* stream) {
  TAPE_CHECK(t);
  return t->impl->export_(index, what, dst, bytes, needed, (cudaStream_t)stream);
}

}  // extern "C"
