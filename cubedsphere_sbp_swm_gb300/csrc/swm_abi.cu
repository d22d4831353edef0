// swm_abi.cu -- the C-ABI of include/swm_gpu.h: context (domain + operator +
// RK4 time scheme), device states and fields, the fused RK4 driver replayed
// as a CUDA graph, the unfused FP64 operator path and FP64 diagnostics.
#include "../../include/swm_gpu.h"
#include "swm_cgrid.h"
#include "swm_cube.h"
#include "swm_launch.h"
#include "swm_ops.cuh"

#include <nvtx3/nvToolsExt.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <set>
#include <tuple>
#include <string>
#include <utility>
#include <vector>

using namespace swm;

namespace {

thread_local std::string g_err;  // errors without a context

constexpr double kPi = 3.141592653589793238462643383279502884;

// ---------------------------------------------------------------------------
// Which neighbour side holds the duplicated nodes of each panel side, and the
// component map of the vector exchange: the halo placement of
// parallel/exchange_factory_mod.f90:157-299 (the neighbour's copy of a shared
// node sits in the 1-wide halo ring), through the index map of swm_cube.h.
// ---------------------------------------------------------------------------
using cube::map_index;
using cube::orientation;

bool build_topology(Topology& tp, std::string& why) {
  const int n = 9;  // the map is linear along a side; any size resolves it
  for (int p = 0; p < 6; ++p)
    for (int s = 0; s < 4; ++s) tp.link[p][s].q = -1;
  for (int p = 0; p < 6; ++p) {
    for (int q = 0; q < 6; ++q) {
      if (q == p) continue;
      int istep, jstep, dim_i;
      orientation(p, q, istep, jstep, dim_i);  // (receiver, sender)
      int k_first[4] = {-1, -1, -1, -1}, kq_first[4], kq_mid[4], sq_mid[4];
      for (int js = 1; js <= n; ++js)
        for (int is = 1; is <= n; ++is) {
          if (is != 1 && is != n && js != 1 && js != n) continue;
          int it, jt;
          map_index(q, is, js, p, n, n, it, jt);
          int side = -1, k = -1;
          if (it == 0 && jt >= 1 && jt <= n) { side = SIDE_L; k = jt - 1; }
          else if (it == n + 1 && jt >= 1 && jt <= n) { side = SIDE_R; k = jt - 1; }
          else if (jt == 0 && it >= 1 && it <= n) { side = SIDE_B; k = it - 1; }
          else if (jt == n + 1 && it >= 1 && it <= n) { side = SIDE_T; k = it - 1; }
          if (side < 0) continue;
          // side of q holding the node, and its along-side index
          int sq, kq;
          if (k == n / 2) {
            if (is == 1) { sq = SIDE_L; kq = js - 1; }
            else if (is == n) { sq = SIDE_R; kq = js - 1; }
            else if (js == 1) { sq = SIDE_B; kq = is - 1; }
            else { sq = SIDE_T; kq = is - 1; }
            sq_mid[side] = sq;
            kq_mid[side] = kq;
          }
          if (k == 0) {
            k_first[side] = 0;
            // remember q-node of k=0 (along-side index resolved below)
            kq_first[side] = (js - 1) * n + (is - 1);
          }
        }
      for (int s = 0; s < 4; ++s) {
        if (k_first[s] < 0) continue;
        EdgeLink L;
        L.q = q;
        L.side_q = sq_mid[s];
        const int node0 = kq_first[s];
        const int is0 = node0 % n, js0 = node0 / n;
        const int k0 = (L.side_q == SIDE_L || L.side_q == SIDE_R) ? js0 : is0;
        L.rev = (k0 == 0) ? 0 : 1;
        if (L.rev && k0 != n - 1) { why = "topology: non-linear side map"; return false; }
        if ((L.rev ? n - 1 - n / 2 : n / 2) != kq_mid[s]) { why = "topology: inconsistent side map"; return false; }
        L.dim_i = dim_i;
        L.istep = istep;
        L.jstep = jstep;
        tp.link[p][s] = L;
      }
    }
  }
  for (int p = 0; p < 6; ++p)
    for (int s = 0; s < 4; ++s)
      if (tp.link[p][s].q < 0) { why = "topology: panel side without neighbour"; return false; }
  return true;
}

const SbpC kTables[4] = SWM_SBP_TABLES;

}  // namespace

// ---------------------------------------------------------------------------
// handles
// ---------------------------------------------------------------------------
struct swm_state {
  swm_ctx* ctx;
  void* hi;     // 3 fields of the context precision
  float* lo;    // FP32 contexts: low parts of the compensated state
};

struct swm_field {
  swm_ctx* ctx;
  double* p;
  int mesh;  // SWM_MESH_*: the staggered mesh of a C-grid field (all one mesh on the Ah grid)
};

// Lat-lon interpolator of one context (regrid_factory_mod.f90:9-301): device
// copies of the per-point stencil offsets, weights and rotation, and output
// buffers of two planes (FP64 and FP32) with their page-locked host copies.
struct swm_latlon {
  swm_ctx* ctx;
  int nlon, nlat, w, contravariant;
  long long* base;
  double *wx, *wy, *rot;
  double* out;
  float* out32;
  double* hout;
  float* hout32;
};

struct GraphEntry {
  cudaGraphExec_t exec;
  long use;
};

struct swm_ctx {
  swm_config cfg{};
  int N = 0, n = 0, P = 0, order = 42, prec = SWM_FP64_PLAIN, elt = 8;
  long long ps = 0, fs = 0;
  double hx = 0.0, ghs = 0.0;
  cudaStream_t st = nullptr;
  std::string err;
  Topology topo{};
  FieldGeom g{};      // geometry of the context-precision fields
  FieldGeom g64{};    // geometry of FP64 fields (pitch for doubles)
  double* m64 = nullptr;   // FP64 metric, NMETRIC fields (g64)
  float* m32 = nullptr;    // FP32 metric copy (FP32 contexts)
  double* qw = nullptr;    // sync weights 4n
  double* Aw = nullptr;    // quadrature weights per line index (n)
  void* edge = nullptr;    // stage edge buffer (context precision)
  void* edge2 = nullptr;   // second edge buffer of the FP32 diffusion step (allocated on first use)
  double* edge64 = nullptr;
  void* ya = nullptr; void* yb = nullptr; void* acc = nullptr;  // RK work (3 fields)
  double* tmp = nullptr;   // 14 FP64 work fields (g64)
  double* hs64 = nullptr; void* hsT = nullptr;
  double* partial = nullptr; double* dres = nullptr; double* hres = nullptr;
  int* herr = nullptr;      // page-locked copy of the device error flag
  WorkUnit* units = nullptr; int nunits = 0;
  int* derr = nullptr;          // device error flag of the bounded waits
  int num_sms = 0;
  StageShape shape{};           // launch shape of the fused stage kernel
  int seg_rows = 0;             // rows per work unit (0: from the occupancy)
  int stage_grid = 0;           // persistent CTAs (0: one CTA per unit)
  // CUDA graphs of whole steps, keyed by (state, dt, kind): kind 0 RK4 step,
  // 1 RK4 step + diffusion step, 2 diffusion step
  std::map<std::tuple<void*, double, int>, GraphEntry> graphs;
  long graph_clock = 0;
  bool timing = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_stage, ev_edge;
  // live children: destroying the context releases their device memory and
  // detaches them, so a later swm_state_free / swm_field_free stays safe
  std::set<swm_state*> states;
  std::set<swm_field*> fields;
  std::set<swm_latlon*> latlons;
  // tangent-linear / adjoint workspace (FP64 contexts, allocated on first
  // use): 10 work fields, then 7 states of 3 fields; edge buffer of the
  // vector-sync transpose; transposed SBP table
  void* adw = nullptr;      // elements of the context precision
  void* adC = nullptr;
  SbpT sbpT{};
  // hyperdiffusion split step (swm_diffusion_set): narrow Laplacian orders
  // of the (u, v) and h operators (0: not configured), coefficients, the
  // coefficient tables per order ([0] 4/2, [1] 6/3), the Cartesian basis
  // vectors (6 fields) and 19 FP64 work fields, all allocated on first use
  int diff_uv = 0, diff_h = 0;
  double diff_uv_coeff = 0.0, diff_h_coeff = 0.0;
  void* ntab[3][5] = {};    // per narrow order (4/2, 6/3, 2/1): cx, cy, clx, cly, b (context precision)
  void* b12 = nullptr;
  void* dw = nullptr;
  // Asynchronous state transfers (swm_state_upload_async / _download_async),
  // allocated on first use: the copy engines move packed FP64 states
  // between the caller's host arrays and device staging buffers on one
  // stream per direction ([0] host to device, [1] device to host), two
  // buffers per direction; the context stream unpacks from / packs into
  // them.  ready[d][k]: buffer k filled; done[d][k]: its consumer finished.
  cudaStream_t xst[2] = {nullptr, nullptr};
  double* xbuf[2][2] = {};
  cudaEvent_t xready[2][2] = {}, xdone[2][2] = {};
  int xnext[2] = {0, 0};
  cudaGraphExec_t ad_graph = nullptr;   // rk4 adjoint step of the last (x, lx, dt)
  // C-grid contexts (the &shallow_water_model_c operator family): the
  // staggered-mesh operator; null on the Ah grid
  CGrid* cg = nullptr;
  // Ah contexts with a laplace_ch_halo4 hyperdiffusion: the corner-mesh
  // tables of the ECS_xy halo (the node mesh is the corner mesh)
  CGrid* xyg = nullptr;
  const void* ad_key[2] = {nullptr, nullptr};
  double ad_dt = 0.0;
};

namespace {

// Named range of a public call for profilers (NVTX; no-op without a tool).
struct TraceRange {
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

int fail(swm_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg; else g_err = msg;
  return code;
}
int cuda_fail(swm_ctx* c, cudaError_t e, const char* where) {
  return fail(c, SWM_E_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
// Makes the context's device current; a bad device index is reported here,
// not later as an unrelated CUDA error.
#define USE_DEVICE(c)                                                 \
  do {                                                                \
    cudaError_t e_ = cudaSetDevice((c)->cfg.device);                  \
    if (e_ != cudaSuccess) return cuda_fail((c), e_, "set device");   \
  } while (0)
#define CK(call, where)                                   \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, where); \
  } while (0)

long long round_up(long long a, long long b) { return (a + b - 1) / b * b; }

// Work units of the fused stage kernel: column strips x row segments, as
// many as fit on the GPU at once (target_ctas) so no CTA waits for a wave,
// or exactly nseg_fixed row segments per strip when that is > 0.
bool make_units(const SbpC& s, int n, int threads, int target_ctas, std::vector<WorkUnit>& out,
                std::string& why, int nseg_fixed = 0) {
  auto need_lo = [&](int k) {
    if (k < s.ne) return 0;
    if (k >= n - s.ne) return n - s.last[n - 1 - k];
    return k - s.H;
  };
  auto need_hi = [&](int k) {
    if (k < s.ne) return s.last[k] - 1;
    if (k >= n - s.ne) return n - 1;
    return k + s.H;
  };
  int nstrip = (n + (threads - 2 * s.rmax) - 1) / (threads - 2 * s.rmax);
  std::vector<int> cs;
  for (;; ++nstrip) {
    cs.assign(nstrip + 1, 0);
    for (int k = 0; k <= nstrip; ++k) cs[k] = (int)((long long)n * k / nstrip);
    bool ok = true;
    for (int k = 0; k < nstrip && ok; ++k) {
      int lo = n, hi = 0;
      for (int c = cs[k]; c < cs[k + 1]; ++c) { lo = std::min(lo, need_lo(c)); hi = std::max(hi, need_hi(c)); }
      ok = (hi + 1 - lo) <= threads && (cs[k + 1] - cs[k]) >= 1;
    }
    if (ok) break;
    if (nstrip > n) { why = "work split failed"; return false; }
  }
  // Row cuts of every strip, so that units carry about the same modelled
  // cost in row-equivalents.  The model is measured per unit on GB300: a
  // strip on a panel edge costs 1 + kStripEdge per row (its closure columns
  // make one warp diverge, and the per-row barrier makes the CTA wait for
  // it); a closure row at a panel end costs 1 + kRowClosure; every unit adds
  // 0.8 * rmax rows for its halo.  nseg_fixed > 0: inner strips get that many
  // units and edge strips (1 + kStripEdge) times as many when the panel also
  // has inner strips; otherwise the unit
  // counts fill one wave of target_ctas.  Each strip is cut at equal shares
  // of its row cost.
  std::vector<std::vector<int>> cuts(nstrip);
  const double kStripEdge = 0.3, kRowClosure = s.ne >= 6 ? 2.0 : 1.0, over = 0.8 * s.rmax;
  std::vector<double> pre(n + 1, 0.0);
  for (int j = 0; j < n; ++j)
    pre[j + 1] = pre[j] + ((j < s.ne || j >= n - s.ne) ? 1.0 + kRowClosure : 1.0);
  auto edge_strip = [&](int k) { return cs[k] == 0 || cs[k + 1] == n; };
  auto cut_equal = [&](int k, int m) {
    auto& c = cuts[k];
    c.assign(1, 0);
    int j = 0;
    for (int r = 1; r < m; ++r) {
      const double want = pre[n] * r / m;
      while (j < n && pre[j + 1] <= want) ++j;
      if (j > c.back()) c.push_back(j);
    }
    c.push_back(n);
  };
  if (nseg_fixed > 0) {
    // (with no inner strip every strip is an edge strip and none waits)
    for (int k = 0; k < nstrip; ++k) {
      const double m = nseg_fixed * (nstrip > 2 && edge_strip(k) ? 1.0 + kStripEdge : 1.0);
      cut_equal(k, std::max(1, std::min(n, (int)std::lround(m))));
    }
  } else {
    const int max_units = std::max(1, n / std::min(8, n));   // at least 8 rows a unit
    // units of strip k for a unit cost of at most tau: m units of a strip of
    // factor f cost f * (pre[n] + m * over) in total
    auto units_of = [&](int k, double tau) {
      const double f = edge_strip(k) ? 1.0 + kStripEdge : 1.0;
      const double per = tau - f * over;
      if (per <= 0.0) return max_units;
      return std::max(1, std::min(max_units, (int)std::ceil(f * pre[n] / per - 1e-9)));
    };
    auto total = [&](double tau) {
      int t = 0;
      for (int k = 0; k < nstrip; ++k) t += units_of(k, tau);
      return 6 * t;
    };
    // the smallest unit cost whose units fit the wave
    double lo = 0.0, hi = (1.0 + kStripEdge) * (pre[n] + over);
    const int budget = std::max(target_ctas, 6 * nstrip);
    for (int it = 0; it < 60; ++it) {
      const double mid = 0.5 * (lo + hi);
      if (total(mid) <= budget) hi = mid; else lo = mid;
    }
    for (int k = 0; k < nstrip; ++k) cut_equal(k, units_of(k, hi));
  }
  for (int p = 0; p < 6; ++p)
    for (int k = 0; k < nstrip; ++k)
      for (size_t r = 0; r + 1 < cuts[k].size(); ++r) {
        WorkUnit w;
        w.inst = 0; w.panel = (int16_t)p;
        w.i0 = (int16_t)cs[k]; w.i1 = (int16_t)cs[k + 1];
        w.j0 = (int16_t)cuts[k][r]; w.j1 = (int16_t)cuts[k][r + 1];
        if (w.j1 <= w.j0) continue;
        int lo = n, hi = 0;
        for (int c = w.i0; c < w.i1; ++c) { lo = std::min(lo, need_lo(c)); hi = std::max(hi, need_hi(c)); }
        w.cl0 = (int16_t)lo; w.cl1 = (int16_t)(hi + 1);
        lo = n; hi = 0;
        for (int c = w.j0; c < w.j1; ++c) { lo = std::min(lo, need_lo(c)); hi = std::max(hi, need_hi(c)); }
        w.rl0 = (int16_t)lo; w.rl1 = (int16_t)(hi + 1);
        out.push_back(w);
      }
  return true;
}

bool name_order(const std::string& nm, const char* prefix, const char* suffix, int& order) {
  const std::string pre(prefix), suf(suffix);
  if (nm.size() < pre.size() + suf.size() + 2) return false;
  if (nm.compare(0, pre.size(), pre) != 0) return false;
  if (nm.compare(nm.size() - suf.size(), suf.size(), suf) != 0) return false;
  const std::string mid = nm.substr(pre.size(), nm.size() - pre.size() - suf.size());
  if (mid == "21") order = 21;
  else if (mid == "42") order = 42;
  else if (mid == "43") order = 43;
  else if (mid == "63") order = 63;
  else return false;
  return true;
}

template <class T>
InstDev<T> base_inst(swm_ctx* c) {
  InstDev<T> I{};
  I.n = c->n; I.P = c->P; I.ps = c->ps; I.fs = c->fs;
  I.boxw = c->shape.boxw;
  I.metric = (c->prec == SWM_FP32_FUSED) ? (const T*)(const void*)c->m32 : (const T*)(const void*)c->m64;
  I.qw = c->qw;
  I.hs = (const T*)c->hsT;
  I.edge = (T*)c->edge;
  I.ghs = (T)c->ghs;
  I.grav = (T)c->cfg.grav;
  return I;
}

// cuTensorMapEncodeTiled, resolved once through the runtime's driver entry
// point query (no link-time dependency on libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  }
  return fn;
}

// Device address of a host array of `bytes` bytes that kernels may read and
// write in place, or nullptr.  Only an array whose first and last byte lie in
// the same page-locked CUDA allocation (cudaHostAlloc / cudaMallocHost /
// cudaHostRegister, same buffer id) mapped for the current device qualifies;
// pageable memory and anything the driver does not describe answer nullptr.
typedef CUresult (*PtrAttrsFn)(unsigned, CUpointer_attribute*, void**, CUdeviceptr);
void* mapped_host(const void* p, size_t bytes) {
  static PtrAttrsFn fn = nullptr;
  static bool looked = false;
  if (!looked) {
    void* q = nullptr;
    cudaDriverEntryPointQueryResult r;
    if (cudaGetDriverEntryPointByVersion("cuPointerGetAttributes", &q, 12000, cudaEnableDefault,
                                         &r) == cudaSuccess &&
        r == cudaDriverEntryPointSuccess)
      fn = (PtrAttrsFn)q;
    looked = true;
  }
  if (!fn || !p || bytes == 0) return nullptr;
  CUpointer_attribute at[3] = {CU_POINTER_ATTRIBUTE_MEMORY_TYPE, CU_POINTER_ATTRIBUTE_DEVICE_POINTER,
                               CU_POINTER_ATTRIBUTE_BUFFER_ID};
  unsigned mt[2] = {0, 0};
  CUdeviceptr dp[2] = {0, 0};
  unsigned long long id[2] = {0, 0};
  for (int e = 0; e < 2; ++e) {
    void* out[3] = {&mt[e], &dp[e], &id[e]};
    const char* a = (const char*)p + (e ? bytes - 1 : 0);
    if (fn(3, at, out, (CUdeviceptr)a) != CUDA_SUCCESS) {
      cudaGetLastError();
      return nullptr;
    }
  }
  if (mt[0] != CU_MEMORYTYPE_HOST || mt[1] != CU_MEMORYTYPE_HOST) return nullptr;
  if (!dp[0] || dp[1] - dp[0] != bytes - 1 || id[0] == 0 || id[0] != id[1]) return nullptr;
  return (void*)dp[0];
}

// 3-D map (column, row of the 6n panel rows, field) over nfields pitched
// fields starting at base; box {boxw, rps, boxf}.
template <class T>
bool encode_fields(swm_ctx* c, CUtensorMap* m, const void* base, int nfields, int boxf) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn || !base) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)c->P, (cuuint64_t)6 * c->n, (cuuint64_t)nfields};
  const cuuint64_t strides[2] = {(cuuint64_t)c->P * sizeof(T), (cuuint64_t)c->fs * sizeof(T)};
  const cuuint32_t box[3] = {(cuuint32_t)c->shape.boxw, (cuuint32_t)c->shape.rps, (cuuint32_t)boxf};
  const cuuint32_t es[3] = {1, 1, 1};
  return fn(m, sizeof(T) == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3,
            const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor maps of one stage launch on instance I in mode `mode`.
template <class T>
int make_maps(swm_ctx* ctx, const InstDev<T>& I, int mode, StageMaps* m) {
  std::memset(m, 0, sizeof(*m));
  if (!ctx->shape.tma) return SWM_OK;
  bool ok = encode_fields<T>(ctx, &m->met, I.metric, NMETRIC, 4);
  ok = ok && encode_fields<T>(ctx, &m->metf, I.metric, NMETRIC, ctx->shape.nf);
  ok = ok && encode_fields<T>(ctx, &m->in, I.in, 3, 3);
  if (!ok) return fail(ctx, SWM_E_CUDA, "cuTensorMapEncodeTiled failed");
  m->base = m->acc = m->lo = m->hs = m->met;
  const T* b = (sizeof(T) == 4 && mode == MODE_RK4) ? I.base_out : I.base;
  if (b && !encode_fields<T>(ctx, &m->base, b, 3, 3)) return fail(ctx, SWM_E_CUDA, "tensor map (base)");
  if (I.acc && !encode_fields<T>(ctx, &m->acc, I.acc, 3, 3)) return fail(ctx, SWM_E_CUDA, "tensor map (acc)");
  if (I.base_lo && !encode_fields<T>(ctx, &m->lo, I.base_lo, 3, 3)) return fail(ctx, SWM_E_CUDA, "tensor map (lo)");
  if (I.hs && !encode_fields<T>(ctx, &m->hs, I.hs, 1, 1)) return fail(ctx, SWM_E_CUDA, "tensor map (hs)");
  return SWM_OK;
}

template <class T>
int run_stage(swm_ctx* ctx, const InstDev<T>& I, int mode) {
  StageMaps maps;
  if (int rc = make_maps<T>(ctx, I, mode, &maps)) return rc;
  cudaEvent_t a = nullptr, b = nullptr;
  if (ctx->timing) {
    CK(cudaEventCreate(&a), "event"); CK(cudaEventCreate(&b), "event");
    CK(cudaEventRecord(a, ctx->st), "event record");
  }
  CK(launch_stage<T>(ctx->order, ctx->shape.cols, ctx->shape.fixbw != 0, &maps, I, nullptr, ctx->units,
                     ctx->nunits, mode, ctx->shape.boxw, ctx->stage_grid, ctx->derr, ctx->st),
     "stage kernel");
  if (ctx->timing) {
    CK(cudaEventRecord(b, ctx->st), "event record");
    ctx->ev_stage.emplace_back(a, b);
    CK(cudaEventCreate(&a), "event"); CK(cudaEventCreate(&b), "event");
    CK(cudaEventRecord(a, ctx->st), "event record");
  }
  CK(launch_edge<T>(I, nullptr, 1, ctx->n, ctx->topo, mode, ctx->st), "edge kernel");
  if (ctx->timing) {
    CK(cudaEventRecord(b, ctx->st), "event record");
    ctx->ev_edge.emplace_back(a, b);
  }
  return SWM_OK;
}

// One RK4 step of the fused path on state s (see rk4_mod.f90:20-42).
template <class T>
int enqueue_rk4(swm_ctx* ctx, swm_state* s, double dt) {
  T* v0 = (T*)s->hi;
  T* ya = (T*)ctx->ya;
  T* yb = (T*)ctx->yb;
  T* acc = (T*)ctx->acc;
  InstDev<T> I = base_inst<T>(ctx);
  int rc;
  // stage 1: k1 = A(v0); y = v0 + dt/2 k1; running sum from v0 + dt/6 k1
  I.in = v0; I.base = v0; I.out = ya; I.acc = acc;
  I.c_in = (T)(0.5 * dt); I.c_acc = (T)(dt / 6.0);
  if ((rc = run_stage<T>(ctx, I, MODE_RK1))) return rc;
  // stage 2: k2 = A(y); y = v0 + dt/2 k2; sum += dt/3 k2
  I.in = ya; I.out = yb; I.c_in = (T)(0.5 * dt); I.c_acc = (T)(dt / 3.0);
  if ((rc = run_stage<T>(ctx, I, MODE_RK2))) return rc;
  // stage 3: k3 = A(y); y = v0 + dt k3; sum += dt/3 k3
  I.in = yb; I.out = ya; I.c_in = (T)dt; I.c_acc = (T)(dt / 3.0);
  if ((rc = run_stage<T>(ctx, I, MODE_RK3))) return rc;
  // stage 4: k4 = A(y); v0 = sum + dt/6 k4
  I.in = ya; I.out = nullptr; I.base_out = v0; I.base_lo = s->lo ? (T*)(void*)s->lo : nullptr;
  I.c_acc = (T)(dt / 6.0);
  return run_stage<T>(ctx, I, MODE_RK4);
}

int check_state(swm_ctx* ctx, const swm_state* s) {
  if (!ctx) return fail(nullptr, SWM_E_INVALID, "null context");
  if (!s || s->ctx != ctx) return fail(ctx, SWM_E_INVALID, "state does not belong to this context");
  return SWM_OK;
}
int check_field(swm_ctx* ctx, const swm_field* f) {
  if (!ctx) return fail(nullptr, SWM_E_INVALID, "null context");
  if (!f || f->ctx != ctx) return fail(ctx, SWM_E_INVALID, "field does not belong to this context");
  return SWM_OK;
}

// Entry points of the Ah-grid path only: refuse a C-grid context.
#define AH_ONLY(ctx_, what_)                                                              \
  do {                                                                                    \
    if ((ctx_) && (ctx_)->cg)                                                             \
      return fail((ctx_), SWM_E_UNSUPPORTED, std::string(what_) + " is not provided on the C grid"); \
  } while (0)

// Points per panel row / column of a mesh of the context.
void mesh_dims(const swm_ctx* ctx, int mesh, int* nx, int* ny) {
  if (ctx->cg) { cgrid_mesh_dims(ctx->cg, mesh, nx, ny); return; }
  *nx = ctx->n; *ny = ctx->n;
}

int sync_check(swm_ctx* ctx, cudaStream_t st);

// Dense host field of a C-grid mesh (i fastest, then j, then panel) to or
// from its pitched device field: one 2-D copy per panel, then a sync.
int c_copy(swm_ctx* ctx, int mesh, double* dev, const double* host_in, double* host_out) {
  int nx, ny;
  mesh_dims(ctx, mesh, &nx, &ny);
  const size_t w = sizeof(double) * nx, dp = sizeof(double) * ctx->P;
  for (int p = 0; p < 6; ++p) {
    double* d = dev + (long long)p * ctx->ps;
    if (host_in)
      CK(cudaMemcpy2DAsync(d, dp, host_in + (size_t)p * nx * ny, w, w, ny, cudaMemcpyHostToDevice, ctx->st), "upload");
    else
      CK(cudaMemcpy2DAsync(host_out + (size_t)p * nx * ny, w, d, dp, w, ny, cudaMemcpyDeviceToHost, ctx->st), "download");
  }
  return sync_check(ctx, ctx->st);
}
int check_mesh(swm_ctx* ctx, const swm_field* f, int mesh, const char* what) {
  if (ctx->cg && f->mesh != mesh)
    return fail(ctx, SWM_E_INVALID, std::string(what) + ": field on the wrong C-grid mesh");
  return SWM_OK;
}

double* tmpf(swm_ctx* c, int k) { return c->tmp + (long long)k * c->g64.fs; }

// Work split of the fused stage kernel for consumer width cols (TMA kernel;
// the FP64 kernel keeps its own width): the column strips fix the narrowest
// TMA box that covers every strip from its aligned start; the box fixes the
// shared memory and so the resident CTAs per SM, which sets the number of
// row segments unless seg_rows > 0 fixes the rows per unit.  grid > 0 runs
// the kernel persistently on that many CTAs.  box selects the box mode:
// SWM_BOX_STRIP (that narrowest box, its width a kernel argument),
// SWM_BOX_WIDEST (the width's widest box, a compile-time constant of the
// kernel; needs a pitch of at least that box) or SWM_BOX_AUTO (the widest
// box where it fits and keeps the resident CTAs per SM).  Replaces the
// context's units and drops its captured graphs.
int stage_layout(swm_ctx* ctx, int cols, int seg_rows = 0, int grid = 0, int box = SWM_BOX_AUTO) {
  std::string why;
  StageShape sh = ctx->shape;
  const SbpC& tab = kTables[sbp_index(ctx->order)];
  if (sh.tma) {
    const int bmax = ctx->prec == SWM_FP32_FUSED ? stage_boxw_max<float>(cols) : stage_boxw_max<double>(cols);
    if (bmax <= 0) return fail(ctx, SWM_E_INVALID, "no stage kernel of that width");
    std::vector<WorkUnit> strips;
    if (!make_units(tab, ctx->n, cols, 1, strips, why)) return fail(ctx, SWM_E_INVALID, why);
    const int al = 16 / ctx->elt;
    int bw = al;
    for (const WorkUnit& w : strips) {
      const int cal = w.cl0 & ~(al - 1);
      bw = std::max(bw, (w.cl1 - cal + al - 1) / al * al);
    }
    if (bw > bmax) return fail(ctx, SWM_E_INVALID, "work split exceeds the TMA box");
    const bool f32 = ctx->prec == SWM_FP32_FUSED;
    auto occ = [&](int w, bool fixed) {
      return f32 ? stage_occupancy<float>(ctx->order, w, cols, fixed)
                 : stage_occupancy<double>(ctx->order, w, cols, fixed);
    };
    const bool fits = f32 && bmax <= ctx->P;
    if (box == SWM_BOX_WIDEST && !fits) return fail(ctx, SWM_E_INVALID, "the widest box exceeds the pitch");
    const int occ_strip = occ(bw, false);
    const bool fixed = box == SWM_BOX_WIDEST || (box == SWM_BOX_AUTO && fits && occ(bmax, true) >= occ_strip);
    sh.cols = cols;
    sh.fixbw = fixed ? 1 : 0;
    sh.boxw = fixed ? bmax : bw;
    sh.ctas_per_sm = fixed ? occ(bmax, true) : occ_strip;
  }
  std::vector<WorkUnit> units;
  const int nseg = seg_rows > 0 ? (ctx->n + seg_rows - 1) / seg_rows : 0;
  if (!make_units(tab, ctx->n, sh.cols, std::max(1, sh.ctas_per_sm) * ctx->num_sms, units, why, nseg))
    return fail(ctx, SWM_E_INVALID, why);
  CK(cudaStreamSynchronize(ctx->st), "sync");
  WorkUnit* d = nullptr;
  CK(cudaMalloc(&d, sizeof(WorkUnit) * units.size()), "alloc");
  cudaError_t e = cudaMemcpy(d, units.data(), sizeof(WorkUnit) * units.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { cudaFree(d); return cuda_fail(ctx, e, "copy units"); }
  if (ctx->units) cudaFree(ctx->units);
  ctx->units = d;
  ctx->nunits = (int)units.size();
  ctx->shape = sh;
  ctx->seg_rows = seg_rows;
  ctx->stage_grid = grid;
  for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second.exec);
  ctx->graphs.clear();
  if (ctx->ad_graph) { cudaGraphExecDestroy(ctx->ad_graph); ctx->ad_graph = nullptr; }
  return SWM_OK;
}

// metric fields of the context precision (NMETRIC fields)
template <class T>
const T* metric_of(swm_ctx* c) {
  return c->prec == SWM_FP32_FUSED ? (const T*)(const void*)c->m32 : (const T*)(const void*)c->m64;
}

// FP64 view of a state: the state itself (FP64) or its joined copy in the
// work fields 11..13 (FP32).
int state64(swm_ctx* ctx, const swm_state* s, const double** h, const double** u, const double** v) {
  if (ctx->prec == SWM_FP64_PLAIN) {
    const double* b = (const double*)s->hi;
    *h = b; *u = b + ctx->fs; *v = b + 2 * ctx->fs;
    return SWM_OK;
  }
  // FP32 fields share the FP64 geometry (same n, pitch in elements differs)
  double* d = tmpf(ctx, 11);
  for (int c = 0; c < 3; ++c) {
    // join row by row through a pitched 2D copy: same element pitch needed,
    // so the FP32 pitch is kept equal to the FP64 pitch (see ctx creation)
    CK(launch_join_f32pair(ctx->fs, (const float*)s->hi + c * ctx->fs, s->lo + c * ctx->fs,
                           d + c * ctx->g64.fs, ctx->st), "join");
  }
  *h = d; *u = d + ctx->g64.fs; *v = d + 2 * ctx->g64.fs;
  return SWM_OK;
}

// Whole-state transfers between packed FP64 arrays (6*n*n values per field,
// host or device) and a state.  One kernel scatters the packed fields into
// the pitched state (splitting them into the FP32 pair) and reads device
// arrays and page-locked host arrays in place, the latter over the
// host-device link; pageable host data first moves as one contiguous copy
// per field into the work fields 11..13.  Downloads run the mirror image.
int put_packed(swm_ctx* ctx, swm_state* s, const double* const src[3], cudaMemcpyKind kind) {
  const size_t bytes = sizeof(double) * 6 * (size_t)ctx->n * ctx->n;
  PackedFields pf;
  for (int c = 0; c < 3; ++c) {
    pf.f[c] = const_cast<double*>(src[c]);
    if (kind != cudaMemcpyHostToDevice) continue;
    if (void* d = mapped_host(src[c], bytes)) {
      pf.f[c] = (double*)d;
    } else {
      pf.f[c] = tmpf(ctx, 11 + c);
      CK(cudaMemcpyAsync(pf.f[c], src[c], bytes, cudaMemcpyHostToDevice, ctx->st), "upload");
    }
  }
  CK(launch_unpack_state(ctx->g64, 3, pf, s->hi, ctx->prec == SWM_FP32_FUSED ? s->lo : nullptr,
                         ctx->st),
     "unpack");
  return SWM_OK;
}

// one packed FP64 host field into a pitched FP64 field
int put_field(swm_ctx* ctx, double* dst, const double* host) {
  const size_t bytes = sizeof(double) * 6 * (size_t)ctx->n * ctx->n;
  PackedFields pf{{(double*)mapped_host(host, bytes), nullptr, nullptr}};
  if (!pf.f[0]) {
    pf.f[0] = tmpf(ctx, 11);
    CK(cudaMemcpyAsync(pf.f[0], host, bytes, cudaMemcpyHostToDevice, ctx->st), "upload");
  }
  CK(launch_unpack_state(ctx->g64, 1, pf, dst, nullptr, ctx->st), "unpack");
  return SWM_OK;
}

int get_packed(swm_ctx* ctx, const swm_state* s, double* const dst[3], cudaMemcpyKind kind) {
  const size_t bytes = sizeof(double) * 6 * (size_t)ctx->n * ctx->n;
  bool staged[3] = {false, false, false};
  PackedFields pf;
  for (int c = 0; c < 3; ++c) {
    pf.f[c] = dst[c];
    if (kind != cudaMemcpyDeviceToHost) continue;
    if (void* d = mapped_host(dst[c], bytes)) {
      pf.f[c] = (double*)d;
    } else {
      pf.f[c] = tmpf(ctx, 11 + c);
      staged[c] = true;
    }
  }
  CK(launch_pack_state(ctx->g64, 3, s->hi, ctx->prec == SWM_FP32_FUSED ? s->lo : nullptr, pf,
                       ctx->st),
     "pack");
  for (int c = 0; c < 3; ++c)
    if (staged[c])
      CK(cudaMemcpyAsync(dst[c], pf.f[c], bytes, cudaMemcpyDeviceToHost, ctx->st), "download");
  return SWM_OK;
}

int reduce(swm_ctx* ctx, int kind, const double* a, const double* b, int slot) {
  CK(launch_reduce(ctx->g64, kind, a, b, ctx->m64 + MJ * ctx->g64.fs, ctx->Aw, ctx->hx * ctx->hx,
                   ctx->partial, REDUCE_BLOCKS, ctx->dres + slot, ctx->st), "reduce");
  return SWM_OK;
}

// Synchronise stream st and report (and clear) the device error flag a
// kernel raises when one of its bounded waits expired; the flag is read by a
// copy queued on st behind the work it guards.
int sync_check(swm_ctx* ctx, cudaStream_t st) {
  CK(cudaMemcpyAsync(ctx->herr, ctx->derr, sizeof(int), cudaMemcpyDeviceToHost, st), "read error flag");
  CK(cudaStreamSynchronize(st), "sync");
  const int flag = *ctx->herr;
  if (flag != 0) {
    *ctx->herr = 0;
    CK(cudaMemsetAsync(ctx->derr, 0, sizeof(int), st), "clear error flag");
    CK(cudaStreamSynchronize(st), "sync");
    return fail(ctx, SWM_E_DEVICE, "a kernel gave up a bounded wait (code " + std::to_string(flag) +
                                       "); results of the affected calls are invalid");
  }
  return SWM_OK;
}

int fetch_results(swm_ctx* ctx, int count, double* out) {
  CK(cudaMemcpyAsync(ctx->hres, ctx->dres, sizeof(double) * count, cudaMemcpyDeviceToHost, ctx->st), "copy results");
  if (int rc_ = sync_check(ctx, ctx->st)) return rc_;
  std::memcpy(out, ctx->hres, sizeof(double) * count);
  return SWM_OK;
}

// unfused operator helpers on FP64 fields
int op_curl(swm_ctx* ctx, const double* u, const double* v, double* out) {
  CK(launch_div_presync(ctx->g64, ctx->order, ctx->hx * ctx->cfg.radius, ctx->m64, u, v, 1, out, ctx->st), "curl");
  CK(launch_sync_scalar(ctx->g64, ctx->topo, out, ctx->edge64, ctx->st), "sync");
  return SWM_OK;
}
int op_div(swm_ctx* ctx, const double* u, const double* v, double* out) {
  CK(launch_div_presync(ctx->g64, ctx->order, ctx->hx * ctx->cfg.radius, ctx->m64, u, v, 0, out, ctx->st), "div");
  CK(launch_sync_scalar(ctx->g64, ctx->topo, out, ctx->edge64, ctx->st), "sync");
  return SWM_OK;
}
int op_grad(swm_ctx* ctx, const double* f, double* gx, double* gy) {
  CK(launch_grad_presync(ctx->g64, ctx->order, ctx->ghs, f, gx, gy, ctx->st), "grad");
  CK(launch_sync_vector(ctx->g64, ctx->topo, ctx->qw, gx, gy, ctx->edge64, ctx->st), "sync");
  return SWM_OK;
}

void release_latlon(swm_latlon* r) {
  void* dev[] = {r->base, r->wx, r->wy, r->rot, r->out, r->out32};
  for (void* p : dev) if (p) cudaFree(p);
  if (r->hout) cudaFreeHost(r->hout);
  if (r->hout32) cudaFreeHost(r->hout32);
  r->base = nullptr; r->wx = r->wy = r->rot = r->out = r->hout = nullptr;
  r->out32 = r->hout32 = nullptr;
}

void free_ctx(swm_ctx* c) {
  if (!c) return;
  for (swm_state* s : c->states) {
    if (s->hi) cudaFree(s->hi);
    if (s->lo) cudaFree(s->lo);
    s->hi = nullptr; s->lo = nullptr; s->ctx = nullptr;
  }
  for (swm_field* f : c->fields) {
    if (f->p) cudaFree(f->p);
    f->p = nullptr; f->ctx = nullptr;
  }
  for (swm_latlon* r : c->latlons) {
    release_latlon(r);
    r->ctx = nullptr;
  }
  for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second.exec);
  for (auto& e : c->ev_stage) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
  for (auto& e : c->ev_edge) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
  // hsT aliases hs64 in FP64 contexts: free each allocation once
  void* hsT = (c->hsT == (void*)c->hs64) ? nullptr : c->hsT;
  if (c->ad_graph) cudaGraphExecDestroy(c->ad_graph);
  cgrid_destroy(c->cg);
  cgrid_destroy(c->xyg);
  void* ptrs[] = {c->m64, c->m32, c->qw, c->Aw, c->edge, c->edge2, c->edge64, c->ya, c->yb, c->acc,
                  c->tmp, c->hs64, hsT, c->partial, c->dres, c->units, c->derr, c->adw, c->adC};
  for (void* p : ptrs) if (p) cudaFree(p);
  for (auto& t : c->ntab)
    for (void* p : t) if (p) cudaFree(p);
  if (c->b12) cudaFree(c->b12);
  if (c->dw) cudaFree(c->dw);
  if (c->hres) cudaFreeHost(c->hres);
  if (c->herr) cudaFreeHost(c->herr);
  for (int d = 0; d < 2; ++d) {
    if (c->xst[d]) { cudaStreamSynchronize(c->xst[d]); cudaStreamDestroy(c->xst[d]); }
    for (int k = 0; k < 2; ++k) {
      if (c->xbuf[d][k]) cudaFree(c->xbuf[d][k]);
      if (c->xready[d][k]) cudaEventDestroy(c->xready[d][k]);
      if (c->xdone[d][k]) cudaEventDestroy(c->xdone[d][k]);
    }
  }
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
}

// Edge scratch of swm_sync_scalar_static: the context edge-buffer layout
// (6 panels x 4 sides x 4 value slots x n) for n <= SWM_SYNC_STATIC_MAX_N + 1,
// part of the module image so that no call allocates it.
constexpr int kStaticSyncScratch = 6 * 4 * 4 * (SWM_SYNC_STATIC_MAX_N + 1);
static __device__ __align__(256) double g_sync_scratch[kStaticSyncScratch];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
double* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_sync_scratch on the context's device, looked up once
// per device (the device is current: the caller has just selected it).
int static_sync_scratch(swm_ctx* ctx, double** out) {
  const int dev = ctx->cfg.device;
  if (dev < 0 || dev >= kMaxDevices) return fail(ctx, SWM_E_INVALID, "device index out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    CK(cudaGetSymbolAddress(&p, g_sync_scratch), "static scratch address");
    g_scratch_ptr[dev] = static_cast<double*>(p);
  }
  *out = g_scratch_ptr[dev];
  return SWM_OK;
}

}  // namespace

// ===========================================================================
// C-ABI
// ===========================================================================
extern "C" {

const char* swm_last_error(const swm_ctx* ctx) { return ctx ? ctx->err.c_str() : g_err.c_str(); }

int swm_ctx_create_named(const swm_config* cfg, const char* div_op_name, const char* grad_op_name,
                         const char* curl_op_name, const char* coriolis_op_name,
                         const char* KE_op_name, const char* co2contra_op_name,
                         const char* massflux_op_name, const char* quadrature_name,
                         swm_ctx** out) {
  swm_ctx* ctx = nullptr;
  if (!cfg || !out) return fail(nullptr, SWM_E_INVALID, "null argument");
  *out = nullptr;
  int od = 0, og = 0, oc = 0, oq = 0;
  // The C-grid family of &shallow_water_model_c (namelist_swm:80-102), all
  // operators of one SBP order: divergence_c_sbpNN, gradient_c_sbpNN,
  // curl_c_sbpNN, coriolis_Cgrid_sbpNN, KE_Cgrid_sbpNN, co2contra_c_sbpNN,
  // massflux_c_sbpNN, SBP_CNN_quadrature with NN 21 or 42.  co2contra_c_sbpNN_new
  // (co2contra_Cgrid_mod.f90:66-134: the same interpolate, J Qi12, interpolate
  // back, divide by J chain through the 2-D interpolators) is the same map.
  int cgrid_order = 0;
  if (div_op_name && std::strncmp(div_op_name, "divergence_c_sbp", 16) == 0) {
    if (!name_order(div_op_name, "divergence_c_sbp", "", od) || (od != 21 && od != 42))
      return fail(nullptr, SWM_E_UNSUPPORTED, std::string("unsupported div operator: ") + div_op_name);
    const std::string o = std::to_string(od);
    const char* want[7] = {grad_op_name, curl_op_name, coriolis_op_name, KE_op_name, co2contra_op_name,
                           massflux_op_name, quadrature_name};
    const std::string need[7] = {"gradient_c_sbp" + o, "curl_c_sbp" + o, "coriolis_Cgrid_sbp" + o, "KE_Cgrid_sbp" + o,
                                 "co2contra_c_sbp" + o, "massflux_c_sbp" + o, "SBP_C" + o + "_quadrature"};
    for (int k = 0; k < 7; ++k)
      if (!want[k] || (need[k] != want[k] && !(k == 4 && need[k] + "_new" == want[k])))
        return fail(nullptr, SWM_E_UNSUPPORTED,
                    std::string("C-grid family needs ") + need[k] + ", got " + (want[k] ? want[k] : "(null)"));
    cgrid_order = od;
  } else if (!div_op_name || !name_order(div_op_name, "divergence_ah", "_sbp", od))
    return fail(nullptr, SWM_E_UNSUPPORTED, std::string("unsupported div operator: ") + (div_op_name ? div_op_name : "(null)"));
  if (!cgrid_order && (!grad_op_name || !name_order(grad_op_name, "gradient_ah", "_sbp_ecs", og)))
    return fail(nullptr, SWM_E_UNSUPPORTED, std::string("unsupported grad operator: ") + (grad_op_name ? grad_op_name : "(null)"));
  if (!cgrid_order && (!curl_op_name || !name_order(curl_op_name, "curl_divergence_ah", "_sbp", oc)))
    return fail(nullptr, SWM_E_UNSUPPORTED, std::string("unsupported curl operator: ") + (curl_op_name ? curl_op_name : "(null)"));
  if (!cgrid_order) {
    if (od == 21 || oc == 21)
      return fail(nullptr, SWM_E_UNSUPPORTED, "divergence_ah21_sbp does not exist in the operator family");
    if (od != og || od != oc)
      return fail(nullptr, SWM_E_UNSUPPORTED, "fused path needs div, grad and curl of one SBP order");
    auto eq = [](const char* a, const char* b) { return a && std::strcmp(a, b) == 0; };
    if (!eq(coriolis_op_name, "coriolis_colocated")) return fail(nullptr, SWM_E_UNSUPPORTED, "unsupported coriolis operator");
    if (!eq(KE_op_name, "KE_colocated")) return fail(nullptr, SWM_E_UNSUPPORTED, "unsupported KE operator");
    if (!eq(co2contra_op_name, "co2contra_colocated")) return fail(nullptr, SWM_E_UNSUPPORTED, "unsupported co2contra operator");
    if (!eq(massflux_op_name, "massflux_colocated")) return fail(nullptr, SWM_E_UNSUPPORTED, "unsupported massflux operator");
    if (!quadrature_name || !name_order(quadrature_name, "SBP_Ah", "_quadrature", oq) || oq == 43)
      return fail(nullptr, SWM_E_UNSUPPORTED, "unsupported quadrature");
  }
  if (cfg->N < 16 || cfg->N > 8190) return fail(nullptr, SWM_E_INVALID, "N must be in [16, 8190]");
  if (cfg->precision != SWM_FP64_PLAIN && cfg->precision != SWM_FP32_FUSED)
    return fail(nullptr, SWM_E_UNSUPPORTED, "unknown precision");
  if (!(cfg->radius > 0.0) || !std::isfinite(cfg->grav) || !std::isfinite(cfg->omega))
    return fail(nullptr, SWM_E_INVALID, "bad physical constants");
  const double an = std::sqrt(cfg->rotation_axis[0] * cfg->rotation_axis[0] +
                              cfg->rotation_axis[1] * cfg->rotation_axis[1] +
                              cfg->rotation_axis[2] * cfg->rotation_axis[2]);
  if (!(an > 0.0)) return fail(nullptr, SWM_E_INVALID, "rotation axis must be non-zero");

  ctx = new swm_ctx();
  ctx->cfg = *cfg;
  ctx->N = cfg->N; ctx->n = cfg->N + 1; ctx->order = od; ctx->prec = cfg->precision;
  ctx->elt = ctx->prec == SWM_FP32_FUSED ? 4 : 8;
  // One element pitch for both precisions (a 128-byte multiple for doubles
  // and a 64-byte multiple for floats) so FP32 and FP64 fields share indexing.
  ctx->P = (int)round_up(ctx->n, 16);
  ctx->ps = (long long)ctx->n * ctx->P;
  ctx->fs = 6 * ctx->ps;
  ctx->hx = (0.25 * kPi - (-0.25 * kPi)) / (double)ctx->N;
  ctx->ghs = 1.0 / (ctx->hx * cfg->radius);
  ctx->g = FieldGeom{ctx->n, ctx->P, ctx->ps, ctx->fs};
  ctx->g64 = ctx->g;
  std::string why;
  if (!build_topology(ctx->topo, why)) { free_ctx(ctx); return fail(nullptr, SWM_E_INVALID, why); }
  cudaError_t e;
#define CKC(call, where)                                                              \
  do {                                                                                \
    e = (call);                                                                       \
    if (e != cudaSuccess) {                                                           \
      std::string m = std::string(where) + ": " + cudaGetErrorString(e);             \
      free_ctx(ctx);                                                                  \
      return fail(nullptr, e == cudaErrorMemoryAllocation ? SWM_E_NOMEM : SWM_E_CUDA, m); \
    }                                                                                 \
  } while (0)
  CKC(cudaSetDevice(cfg->device), "cudaSetDevice");
  (void)cudaGetLastError();  // drop a stale, non-sticky error of an earlier caller
  CKC(cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking), "stream");
  const size_t fbytes = sizeof(double) * ctx->fs;
  CKC(cudaMalloc(&ctx->m64, NMETRIC * fbytes), "alloc metric");
  CKC(cudaMemsetAsync(ctx->m64, 0, NMETRIC * fbytes, ctx->st), "memset");
  CKC(cudaMalloc(&ctx->qw, sizeof(double) * 4 * ctx->n), "alloc");
  CKC(cudaMalloc(&ctx->Aw, sizeof(double) * ctx->n), "alloc");
  CKC(cudaMalloc(&ctx->edge64, sizeof(double) * 16 * 6 * ctx->n), "alloc");
  CKC(cudaMalloc(&ctx->edge, (size_t)ctx->elt * 16 * 6 * ctx->n), "alloc");
  CKC(cudaMalloc(&ctx->ya, (size_t)ctx->elt * 3 * ctx->fs), "alloc");
  CKC(cudaMalloc(&ctx->yb, (size_t)ctx->elt * 3 * ctx->fs), "alloc");
  CKC(cudaMalloc(&ctx->acc, (size_t)ctx->elt * 3 * ctx->fs), "alloc");
  CKC(cudaMemsetAsync(ctx->ya, 0, (size_t)ctx->elt * 3 * ctx->fs, ctx->st), "memset");
  CKC(cudaMemsetAsync(ctx->yb, 0, (size_t)ctx->elt * 3 * ctx->fs, ctx->st), "memset");
  CKC(cudaMemsetAsync(ctx->acc, 0, (size_t)ctx->elt * 3 * ctx->fs, ctx->st), "memset");
  CKC(cudaMalloc(&ctx->tmp, 14 * fbytes), "alloc work fields");
  CKC(cudaMemsetAsync(ctx->tmp, 0, 14 * fbytes, ctx->st), "memset");
  CKC(cudaMalloc(&ctx->partial, sizeof(double) * REDUCE_BLOCKS), "alloc");
  CKC(cudaMalloc(&ctx->dres, sizeof(double) * 16), "alloc");
  CKC(cudaMallocHost(&ctx->hres, sizeof(double) * 16), "alloc host");
  CKC(cudaMallocHost(&ctx->herr, sizeof(int)), "alloc host");
  *ctx->herr = 0;
  CKC(cudaMalloc(&ctx->derr, sizeof(int)), "alloc");
  CKC(cudaMemsetAsync(ctx->derr, 0, sizeof(int), ctx->st), "memset");
  if (cgrid_order) {
    // the staggered-mesh operator; the Ah stage kernel, metric and
    // quadrature weights are not set up
    ctx->order = cgrid_order;
    int rc = cgrid_create(ctx->g64, ctx->N, cgrid_order, cfg->radius, cfg->grav, cfg->omega, cfg->rotation_axis,
                          ctx->prec == SWM_FP32_FUSED, ctx->st, &ctx->cg, why);
    if (rc) {
      free_ctx(ctx);
      return fail(nullptr, rc == 3 ? SWM_E_NOMEM : rc == 2 ? SWM_E_CUDA : SWM_E_INVALID, why);
    }
    CKC(cudaStreamSynchronize(ctx->st), "sync");
    *out = ctx;
    return SWM_OK;
  }
  CKC(ctx->prec == SWM_FP32_FUSED ? prepare_stage<float>(od, &ctx->shape)
                                  : prepare_stage<double>(od, &ctx->shape),
      "stage kernel attributes");
  if (ctx->shape.tma && !encode_tiled()) {
    free_ctx(ctx);
    return fail(nullptr, SWM_E_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
  }
  CKC(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, cfg->device), "SM count");
  if (int rc = stage_layout(ctx, ctx->shape.cols)) {
    why = ctx->err;
    free_ctx(ctx);
    return fail(nullptr, rc, why);
  }
  CKC(launch_geometry(ctx->g64, ctx->N, cfg->radius, cfg->omega, cfg->rotation_axis, ctx->m64, ctx->qw, ctx->st), "geometry");
  if (ctx->prec == SWM_FP32_FUSED) {
    CKC(cudaMalloc(&ctx->m32, sizeof(float) * NMETRIC * ctx->fs), "alloc");
    CKC(launch_to_f32(ctx->m64, ctx->m32, NMETRIC * ctx->fs, ctx->st), "metric to f32");
  }
  // SBP quadrature weights (quadrature_factory_mod.f90:158-177)
  {
    const SbpC& q = kTables[sbp_index(oq)];
    std::vector<double> A(ctx->n, 1.0);
    for (int i = 0; i < std::min(q.nA, ctx->n); ++i) A[i] = q.A[i];
    for (int i = std::max(ctx->n - q.nA, 0); i < ctx->n; ++i) A[i] = q.A[ctx->n - 1 - i];
    CKC(cudaMemcpy(ctx->Aw, A.data(), sizeof(double) * ctx->n, cudaMemcpyHostToDevice), "copy");
  }
  CKC(cudaStreamSynchronize(ctx->st), "sync");
#undef CKC
  *out = ctx;
  return SWM_OK;
}

int swm_ctx_create(const swm_config* cfg, swm_ctx** out) {
  if (!cfg) return fail(nullptr, SWM_E_INVALID, "null config");
  const int o = cfg->sbp_order;
  if (o != 42 && o != 43 && o != 63)
    return fail(nullptr, SWM_E_UNSUPPORTED, "sbp_order must be 42, 43 or 63 for the model operator");
  char dn[64], gn[64], cn[64], qn[64];
  std::snprintf(dn, sizeof dn, "divergence_ah%d_sbp", o);
  std::snprintf(gn, sizeof gn, "gradient_ah%d_sbp_ecs", o);
  std::snprintf(cn, sizeof cn, "curl_divergence_ah%d_sbp", o);
  std::snprintf(qn, sizeof qn, "SBP_Ah%d_quadrature", o == 43 ? 42 : o);
  return swm_ctx_create_named(cfg, dn, gn, cn, "coriolis_colocated", "KE_colocated",
                              "co2contra_colocated", "massflux_colocated", qn, out);
}

void swm_ctx_destroy(swm_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->cfg.device);
  cudaStreamSynchronize(ctx->st);
  free_ctx(ctx);
}

int swm_ctx_synchronize(swm_ctx* ctx) {
  if (!ctx) return fail(nullptr, SWM_E_INVALID, "null context");
  USE_DEVICE(ctx);
  for (int d = 0; d < 2; ++d)
    if (ctx->xst[d]) CK(cudaStreamSynchronize(ctx->xst[d]), "sync transfers");
  if (int rc_ = sync_check(ctx, ctx->st)) return rc_;
  return SWM_OK;
}

void* swm_ctx_stream(swm_ctx* ctx) { return ctx ? (void*)ctx->st : nullptr; }
size_t swm_ctx_npts(const swm_ctx* ctx) { return ctx ? (size_t)6 * ctx->n * ctx->n : 0; }

int swm_ctx_grid(const swm_ctx* ctx) { return !ctx ? -1 : ctx->cg ? SWM_GRID_C : SWM_GRID_AH; }

int swm_mesh_dims(const swm_ctx* ctx, int mesh, int* nx, int* ny) {
  if (!ctx || !nx || !ny) return fail(nullptr, SWM_E_INVALID, "null argument");
  if (mesh < SWM_MESH_P || mesh > SWM_MESH_Q) return fail(nullptr, SWM_E_INVALID, "unknown mesh");
  mesh_dims(ctx, mesh, nx, ny);
  return SWM_OK;
}

int swm_set_orography(swm_ctx* ctx, const double* hs) {
  if (!ctx || !hs) return fail(ctx, SWM_E_INVALID, "null argument");
  USE_DEVICE(ctx);
  if (!ctx->hs64) {
    CK(cudaMalloc(&ctx->hs64, sizeof(double) * ctx->fs), "alloc");
    CK(cudaMemsetAsync(ctx->hs64, 0, sizeof(double) * ctx->fs, ctx->st), "memset");
  }
  if (ctx->cg) {
    if (int rc = c_copy(ctx, SWM_MESH_P, ctx->hs64, hs, nullptr)) return rc;
  } else if (int rc = put_field(ctx, ctx->hs64, hs)) {
    return rc;
  }
  if (ctx->prec == SWM_FP32_FUSED) {
    if (!ctx->hsT) CK(cudaMalloc(&ctx->hsT, sizeof(float) * ctx->fs), "alloc");
    CK(launch_to_f32(ctx->hs64, (float*)ctx->hsT, ctx->fs, ctx->st), "to f32");
  } else {
    ctx->hsT = nullptr;  // FP64 uses hs64 directly
  }
  for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second.exec);
  ctx->graphs.clear();
  CK(cudaStreamSynchronize(ctx->st), "sync");
  if (ctx->prec == SWM_FP64_PLAIN) ctx->hsT = ctx->hs64;
  return SWM_OK;
}

// ---------------------------------------------------------------- states
int swm_state_create(swm_ctx* ctx, swm_state** out) {
  if (!ctx || !out) return fail(ctx, SWM_E_INVALID, "null argument");
  USE_DEVICE(ctx);
  swm_state* s = new swm_state{ctx, nullptr, nullptr};
  const size_t b = (size_t)ctx->elt * 3 * ctx->fs;
  cudaError_t e = cudaMalloc(&s->hi, b);
  if (e == cudaSuccess) e = cudaMemsetAsync(s->hi, 0, b, ctx->st);
  if (e == cudaSuccess && ctx->prec == SWM_FP32_FUSED) {
    e = cudaMalloc((void**)&s->lo, sizeof(float) * 3 * ctx->fs);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->lo, 0, sizeof(float) * 3 * ctx->fs, ctx->st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
  if (e != cudaSuccess) {
    if (s->hi) cudaFree(s->hi);
    if (s->lo) cudaFree(s->lo);
    delete s;
    return fail(ctx, e == cudaErrorMemoryAllocation ? SWM_E_NOMEM : SWM_E_CUDA,
                std::string("state alloc: ") + cudaGetErrorString(e));
  }
  ctx->states.insert(s);
  *out = s;
  return SWM_OK;
}

int swm_state_create_similar(swm_ctx* ctx, const swm_state* src, swm_state** out) {
  if (int rc = check_state(ctx, src)) return rc;
  return swm_state_create(ctx, out);
}

void swm_state_free(swm_state* s) {
  if (!s) return;
  swm_ctx* c = s->ctx;
  if (c) {  // a state whose context is gone was already released
    cudaSetDevice(c->cfg.device);
    cudaStreamSynchronize(c->st);
    for (auto it = c->graphs.begin(); it != c->graphs.end();) {
      if (std::get<0>(it->first) == (void*)s) { cudaGraphExecDestroy(it->second.exec); it = c->graphs.erase(it); }
      else ++it;
    }
    if (s->hi) cudaFree(s->hi);
    if (s->lo) cudaFree(s->lo);
    c->states.erase(s);
  }
  delete s;
}

int swm_state_upload(swm_ctx* ctx, swm_state* s, const double* h, const double* u, const double* v) {
  TraceRange trace_("swm_state_upload");
  if (int rc = check_state(ctx, s)) return rc;
  if (!h || !u || !v) return fail(ctx, SWM_E_INVALID, "null host array");
  USE_DEVICE(ctx);
  const double* src[3] = {h, u, v};
  if (ctx->cg) {
    for (int c = 0; c < 3; ++c) {
      if (ctx->prec == SWM_FP64_PLAIN) {
        if (int rc = c_copy(ctx, SWM_MESH_P + c, (double*)s->hi + c * ctx->fs, src[c], nullptr)) return rc;
      } else {  // FP64 values through a device field, split into the (hi, lo) pair
        double* t = tmpf(ctx, 11);
        if (int rc = c_copy(ctx, SWM_MESH_P + c, t, src[c], nullptr)) return rc;
        CK(launch_split_f64(ctx->fs, t, (float*)s->hi + c * ctx->fs, s->lo + c * ctx->fs, ctx->st), "split");
      }
    }
    return sync_check(ctx, ctx->st);
  }
  return put_packed(ctx, s, src, cudaMemcpyHostToDevice);
}

int swm_state_download(swm_ctx* ctx, const swm_state* s, double* h, double* u, double* v) {
  TraceRange trace_("swm_state_download");
  if (int rc = check_state(ctx, s)) return rc;
  if (!h || !u || !v) return fail(ctx, SWM_E_INVALID, "null host array");
  USE_DEVICE(ctx);
  double* dst[3] = {h, u, v};
  if (ctx->cg) {
    for (int c = 0; c < 3; ++c) {
      if (ctx->prec == SWM_FP64_PLAIN) {
        if (int rc = c_copy(ctx, SWM_MESH_P + c, (double*)s->hi + c * ctx->fs, nullptr, dst[c])) return rc;
      } else {  // the (hi, lo) pair joined into FP64
        double* t = tmpf(ctx, 11);
        CK(launch_join_f32pair(ctx->fs, (const float*)s->hi + c * ctx->fs, s->lo + c * ctx->fs, t, ctx->st), "join");
        if (int rc = c_copy(ctx, SWM_MESH_P + c, t, nullptr, dst[c])) return rc;
      }
    }
    return SWM_OK;
  }
  if (int rc = get_packed(ctx, s, dst, cudaMemcpyDeviceToHost)) return rc;
  if (int rc_ = sync_check(ctx, ctx->st)) return rc_;
  return SWM_OK;
}

}  // extern "C"

namespace {

// Streams, staging buffers and events of the asynchronous transfers of
// direction d (0: upload, 1: download), created on first use.  The events
// start recorded, so the first waits on them pass.
int transfer_ready(swm_ctx* ctx, int d) {
  if (ctx->xst[d]) return SWM_OK;
  const size_t bytes = sizeof(double) * 3 * 6 * (size_t)ctx->n * ctx->n;
  for (int k = 0; k < 2; ++k) {
    CK(cudaMalloc(&ctx->xbuf[d][k], bytes), "alloc transfer staging");
    CK(cudaEventCreateWithFlags(&ctx->xready[d][k], cudaEventDisableTiming), "event");
    CK(cudaEventCreateWithFlags(&ctx->xdone[d][k], cudaEventDisableTiming), "event");
    CK(cudaEventRecord(ctx->xready[d][k], ctx->st), "event record");
    CK(cudaEventRecord(ctx->xdone[d][k], ctx->st), "event record");
  }
  CK(cudaStreamCreateWithFlags(&ctx->xst[d], cudaStreamNonBlocking), "stream");
  return SWM_OK;
}

}  // namespace

extern "C" {

int swm_state_upload_async(swm_ctx* ctx, swm_state* s, const double* h, const double* u,
                           const double* v) {
  TraceRange trace_("swm_state_upload_async");
  if (int rc = check_state(ctx, s)) return rc;
  if (!h || !u || !v) return fail(ctx, SWM_E_INVALID, "null host array");
  USE_DEVICE(ctx);
  if (int rc = transfer_ready(ctx, 0)) return rc;
  const size_t np = 6 * (size_t)ctx->n * ctx->n;
  const int k = ctx->xnext[0];
  ctx->xnext[0] ^= 1;
  double* B = ctx->xbuf[0][k];
  const double* src[3] = {h, u, v};
  // the copy engine fills buffer k once the unpack that last read it is done
  CK(cudaStreamWaitEvent(ctx->xst[0], ctx->xdone[0][k], 0), "wait");
  for (int c = 0; c < 3; ++c) {
    int nx, ny;
    mesh_dims(ctx, SWM_MESH_P + c, &nx, &ny);   // C grid: the component's own mesh
    CK(cudaMemcpyAsync(B + c * np, src[c], sizeof(double) * 6 * nx * ny, cudaMemcpyHostToDevice, ctx->xst[0]),
       "upload");
  }
  CK(cudaEventRecord(ctx->xready[0][k], ctx->xst[0]), "event record");
  CK(cudaStreamWaitEvent(ctx->st, ctx->xready[0][k], 0), "wait");
  if (ctx->cg) {
    const bool pair = ctx->prec == SWM_FP32_FUSED;
    for (int c = 0; c < 3; ++c)
      CK(cgrid_unpack(ctx->cg, SWM_MESH_P + c, B + c * np,
                      (char*)s->hi + (size_t)ctx->elt * c * ctx->fs, pair ? s->lo + c * ctx->fs : nullptr, ctx->st),
         "unpack");
    CK(cudaEventRecord(ctx->xdone[0][k], ctx->st), "event record");
    return SWM_OK;
  }
  PackedFields pf{{B, B + np, B + 2 * np}};
  CK(launch_unpack_state(ctx->g64, 3, pf, s->hi, ctx->prec == SWM_FP32_FUSED ? s->lo : nullptr,
                         ctx->st),
     "unpack");
  CK(cudaEventRecord(ctx->xdone[0][k], ctx->st), "event record");
  return SWM_OK;
}

int swm_state_download_async(swm_ctx* ctx, const swm_state* s, double* h, double* u, double* v) {
  TraceRange trace_("swm_state_download_async");
  if (int rc = check_state(ctx, s)) return rc;
  if (!h || !u || !v) return fail(ctx, SWM_E_INVALID, "null host array");
  USE_DEVICE(ctx);
  if (int rc = transfer_ready(ctx, 1)) return rc;
  const size_t np = 6 * (size_t)ctx->n * ctx->n;
  const int k = ctx->xnext[1];
  ctx->xnext[1] ^= 1;
  double* B = ctx->xbuf[1][k];
  double* dst[3] = {h, u, v};
  // the state is packed into buffer k once the copy that last read it is done
  CK(cudaStreamWaitEvent(ctx->st, ctx->xdone[1][k], 0), "wait");
  if (ctx->cg) {
    const bool pair = ctx->prec == SWM_FP32_FUSED;
    for (int c = 0; c < 3; ++c)
      CK(cgrid_pack(ctx->cg, SWM_MESH_P + c, (const char*)s->hi + (size_t)ctx->elt * c * ctx->fs,
                    pair ? s->lo + c * ctx->fs : nullptr, B + c * np, ctx->st),
         "pack");
  } else {
    PackedFields pf{{B, B + np, B + 2 * np}};
    CK(launch_pack_state(ctx->g64, 3, s->hi, ctx->prec == SWM_FP32_FUSED ? s->lo : nullptr, pf,
                         ctx->st),
       "pack");
  }
  CK(cudaEventRecord(ctx->xready[1][k], ctx->st), "event record");
  CK(cudaStreamWaitEvent(ctx->xst[1], ctx->xready[1][k], 0), "wait");
  for (int c = 0; c < 3; ++c) {
    int nx, ny;
    mesh_dims(ctx, SWM_MESH_P + c, &nx, &ny);
    CK(cudaMemcpyAsync(dst[c], B + c * np, sizeof(double) * 6 * nx * ny, cudaMemcpyDeviceToHost, ctx->xst[1]),
       "download");
  }
  CK(cudaEventRecord(ctx->xdone[1][k], ctx->xst[1]), "event record");
  return SWM_OK;
}

static int combine(swm_ctx* ctx, swm_state* s, double s1, const swm_state* a, double s2,
                   const swm_state* b, bool update) {
  if (int rc = check_state(ctx, s)) return rc;
  if (a && check_state(ctx, a)) return SWM_E_INVALID;
  if (b && check_state(ctx, b)) return SWM_E_INVALID;
  USE_DEVICE(ctx);
  const long long cnt = 3 * ctx->fs;
  if (ctx->prec == SWM_FP64_PLAIN) {
    double* o = (double*)s->hi;
    if (update) {
      // this = this + s1*a (+ s2*b), evaluated as (this + s1*a) + s2*b
      CK(launch_axpby(cnt, 1.0, o, s1, (const double*)a->hi, o, ctx->st), "update");
      if (b) CK(launch_axpby(cnt, 1.0, o, s2, (const double*)b->hi, o, ctx->st), "update");
    } else if (!a) {
      CK(launch_fill(cnt, s1, o, ctx->st), "assign");
    } else {
      CK(launch_axpby(cnt, s1, (const double*)a->hi, s2, b ? (const double*)b->hi : nullptr, o, ctx->st), "assign");
    }
  } else {
    float* ohi = (float*)s->hi;
    float* olo = s->lo;
    if (update) {
      CK(launch_axpby_f32pair(cnt, 1.0, ohi, olo, s1, (const float*)a->hi, a->lo, ohi, olo, ctx->st), "update");
      if (b) CK(launch_axpby_f32pair(cnt, 1.0, ohi, olo, s2, (const float*)b->hi, b->lo, ohi, olo, ctx->st), "update");
    } else if (!a) {
      CK(launch_fill_f32pair(cnt, s1, ohi, olo, ctx->st), "fill");
    } else {
      CK(launch_axpby_f32pair(cnt, s1, (const float*)a->hi, a->lo, s2,
                              b ? (const float*)b->hi : nullptr, b ? b->lo : nullptr, ohi, olo, ctx->st), "assign");
    }
  }
  return SWM_OK;
}

int swm_assign_s1(swm_ctx* ctx, swm_state* s, double s1) { return combine(ctx, s, s1, nullptr, 0.0, nullptr, false); }
int swm_assign_s1v1(swm_ctx* ctx, swm_state* s, double s1, const swm_state* v1) {
  if (!v1) return fail(ctx, SWM_E_INVALID, "null state");
  return combine(ctx, s, s1, v1, 0.0, nullptr, false);
}
int swm_assign_s1v1s2v2(swm_ctx* ctx, swm_state* s, double s1, const swm_state* v1, double s2, const swm_state* v2) {
  if (!v1 || !v2) return fail(ctx, SWM_E_INVALID, "null state");
  return combine(ctx, s, s1, v1, s2, v2, false);
}
int swm_update_s1v1(swm_ctx* ctx, swm_state* s, double s1, const swm_state* v1) {
  if (!v1) return fail(ctx, SWM_E_INVALID, "null state");
  return combine(ctx, s, s1, v1, 0.0, nullptr, true);
}
int swm_update_s1v1s2v2(swm_ctx* ctx, swm_state* s, double s1, const swm_state* v1, double s2, const swm_state* v2) {
  if (!v1 || !v2) return fail(ctx, SWM_E_INVALID, "null state");
  return combine(ctx, s, s1, v1, s2, v2, true);
}

int swm_dot(swm_ctx* ctx, const swm_state* a, const swm_state* b, double* out) {
  AH_ONLY(ctx, "swm_dot");
  if (int rc = check_state(ctx, a)) return rc;
  if (int rc = check_state(ctx, b)) return rc;
  if (!out) return fail(ctx, SWM_E_INVALID, "null output");
  USE_DEVICE(ctx);
  const double *ah, *au, *av, *bh, *bu, *bv;
  if (ctx->prec == SWM_FP32_FUSED) {
    // join a into 11..13 and b into 8..10
    if (int rc = state64(ctx, a, &ah, &au, &av)) return rc;
    double* d = tmpf(ctx, 8);
    for (int c = 0; c < 3; ++c)
      CK(launch_join_f32pair(ctx->fs, (const float*)b->hi + c * ctx->fs, b->lo + c * ctx->fs, d + c * ctx->fs, ctx->st), "join");
    bh = d; bu = d + ctx->fs; bv = d + 2 * ctx->fs;
  } else {
    if (int rc = state64(ctx, a, &ah, &au, &av)) return rc;
    if (int rc = state64(ctx, b, &bh, &bu, &bv)) return rc;
  }
  if (int rc = reduce(ctx, 0, ah, bh, 0)) return rc;
  if (int rc = reduce(ctx, 0, au, bu, 1)) return rc;
  if (int rc = reduce(ctx, 0, av, bv, 2)) return rc;
  double r[3];
  if (int rc = fetch_results(ctx, 3, r)) return rc;
  *out = r[0] + r[1] + r[2];
  return SWM_OK;
}

int swm_norm2(swm_ctx* ctx, const swm_state* a, double* out) {
  double d;
  if (int rc = swm_dot(ctx, a, a, &d)) return rc;
  *out = std::sqrt(d);
  return SWM_OK;
}

// ------------------------------------------------------------- operator
int swm_apply(swm_ctx* ctx, swm_state* vout, const swm_state* vin) {
  TraceRange trace_("swm_apply");
  if (int rc = check_state(ctx, vout)) return rc;
  if (int rc = check_state(ctx, vin)) return rc;
  if (vout == vin) return fail(ctx, SWM_E_INVALID, "apply needs distinct in/out states");
  USE_DEVICE(ctx);
  if (ctx->cg) {
    if (ctx->prec == SWM_FP64_PLAIN) {
      CK(cgrid_apply(ctx->cg, ctx->topo, ctx->edge64, ctx->hs64, (const double*)vin->hi, (double*)vout->hi, ctx->st),
         "C-grid apply");
    } else {  // tendencies of the high part, in FP32
      CK(cudaMemsetAsync(vout->lo, 0, sizeof(float) * 3 * ctx->fs, ctx->st), "memset");
      CK(cgrid_apply32(ctx->cg, ctx->topo, (float*)ctx->edge, (const float*)ctx->hsT, (const float*)vin->hi,
                       (float*)vout->hi, ctx->st),
         "C-grid apply");
    }
    return SWM_OK;
  }
  if (ctx->prec == SWM_FP64_PLAIN) {
    InstDev<double> I = base_inst<double>(ctx);
    I.in = (const double*)vin->hi; I.out = (double*)vout->hi;
    return run_stage<double>(ctx, I, MODE_APPLY);
  }
  InstDev<float> I = base_inst<float>(ctx);
  I.in = (const float*)vin->hi; I.out = (float*)vout->hi;
  CK(cudaMemsetAsync(vout->lo, 0, sizeof(float) * 3 * ctx->fs, ctx->st), "memset");
  return run_stage<float>(ctx, I, MODE_APPLY);
}

int swm_apply_unfused(swm_ctx* ctx, swm_state* vout, const swm_state* vin) {
  TraceRange trace_("swm_apply_unfused");
  if (int rc = check_state(ctx, vout)) return rc;
  if (int rc = check_state(ctx, vin)) return rc;
  if (ctx->prec != SWM_FP64_PLAIN) return fail(ctx, SWM_E_UNSUPPORTED, "unfused apply is FP64 only");
  USE_DEVICE(ctx);
  const long long fs = ctx->fs;
  const double* h = (const double*)vin->hi;
  const double* u = h + fs;
  const double* v = h + 2 * fs;
  double* oh = (double*)vout->hi;
  double* ou = oh + fs;
  double* ov = oh + 2 * fs;
  double *ut = tmpf(ctx, 0), *vt = tmpf(ctx, 1), *hu = tmpf(ctx, 2), *hv = tmpf(ctx, 3),
         *ke = tmpf(ctx, 4), *gx = tmpf(ctx, 5), *gy = tmpf(ctx, 6), *cu = tmpf(ctx, 7),
         *cor_u = tmpf(ctx, 8), *cor_v = tmpf(ctx, 9), *dv = tmpf(ctx, 10);
  const FieldGeom& g = ctx->g64;
  cudaStream_t st = ctx->st;
  if (CGrid* c = ctx->cg) {
    // the reference's operator sequence, one unfused operator at a time
    CK(cgrid_co2contra(c, u, v, ut, vt, st), "co2contra");
    CK(cgrid_massflux(c, h, ut, vt, hu, hv, st), "massflux");
    CK(cgrid_ke(c, u, v, ut, vt, ke, st), "KE");
    CK(launch_ke_update(g, ctx->cfg.grav, h, ctx->hs64, ke, st), "KE update");
    CK(cgrid_grad(c, ke, gx, gy, st), "grad");
    CK(cgrid_curl(c, ctx->topo, ctx->edge64, u, v, cu, st), "curl");
    CK(cgrid_coriolis(c, hu, hv, h, cu, cor_u, cor_v, st), "coriolis");
    CK(launch_axpby(fs, -1.0, gx, 1.0, cor_u, ou, st), "assign");
    CK(launch_axpby(fs, -1.0, gy, 1.0, cor_v, ov, st), "assign");
    CK(cgrid_div(c, hu, hv, dv, st), "div");
    CK(launch_axpby(fs, -1.0, dv, 0.0, nullptr, oh, st), "assign");
    return SWM_OK;
  }
  CK(launch_co2contra(g, ctx->m64, u, v, ut, vt, st), "co2contra");
  CK(launch_massflux(g, h, ut, vt, hu, hv, st), "massflux");
  CK(launch_ke(g, u, v, ut, vt, ke, st), "KE");
  CK(launch_ke_update(g, ctx->cfg.grav, h, ctx->hs64, ke, st), "KE update");
  if (int rc = op_grad(ctx, ke, gx, gy)) return rc;
  if (int rc = op_curl(ctx, u, v, cu)) return rc;
  CK(launch_coriolis(g, ctx->m64, hu, hv, h, cu, cor_u, cor_v, st), "coriolis");
  CK(launch_axpby(fs, -1.0, gx, 1.0, cor_u, ou, st), "assign");
  CK(launch_axpby(fs, -1.0, gy, 1.0, cor_v, ov, st), "assign");
  if (int rc = op_div(ctx, hu, hv, dv)) return rc;
  CK(launch_axpby(fs, -1.0, dv, 0.0, nullptr, oh, st), "assign");
  return SWM_OK;
}

}  // extern "C"

namespace {

// Run nsteps replays of the CUDA graph of `enqueue` for (state, dt, kind),
// capturing it on first use (at most 8 graphs per context, least recently
// used evicted).
template <class F>
int graph_steps(swm_ctx* ctx, swm_state* v0, double dt, int kind, int nsteps, F enqueue) {
  const auto key = std::make_tuple((void*)v0, dt, kind);
  auto it = ctx->graphs.find(key);
  if (it == ctx->graphs.end()) {
    if (ctx->graphs.size() >= 8) {
      auto old = ctx->graphs.begin();
      for (auto jt = ctx->graphs.begin(); jt != ctx->graphs.end(); ++jt)
        if (jt->second.use < old->second.use) old = jt;
      cudaGraphExecDestroy(old->second.exec);
      ctx->graphs.erase(old);
    }
    cudaGraph_t graph;
    CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal), "begin capture");
    int rc = enqueue();
    cudaError_t ec = cudaStreamEndCapture(ctx->st, &graph);
    if (rc) { if (ec == cudaSuccess) cudaGraphDestroy(graph); return rc; }
    CK(ec, "end capture");
    GraphEntry ge{};
    cudaError_t ei = cudaGraphInstantiate(&ge.exec, graph, 0);
    cudaGraphDestroy(graph);
    CK(ei, "graph instantiate");
    it = ctx->graphs.emplace(key, ge).first;
  }
  it->second.use = ++ctx->graph_clock;
  for (int k = 0; k < nsteps; ++k) CK(cudaGraphLaunch(it->second.exec, ctx->st), "graph launch");
  return SWM_OK;
}

int enqueue_rk4_any(swm_ctx* ctx, swm_state* v0, double dt) {
  if (ctx->cg) {
    if (ctx->prec == SWM_FP64_PLAIN)
      CK(cgrid_rk4(ctx->cg, ctx->topo, ctx->edge64, ctx->hs64, (double*)v0->hi, dt, ctx->st), "C-grid RK4 step");
    else
      CK(cgrid_rk4_32(ctx->cg, ctx->topo, (float*)ctx->edge, (const float*)ctx->hsT, (float*)v0->hi, v0->lo, dt,
                      ctx->st),
         "C-grid RK4 step");
    return SWM_OK;
  }
  return ctx->prec == SWM_FP64_PLAIN ? enqueue_rk4<double>(ctx, v0, dt) : enqueue_rk4<float>(ctx, v0, dt);
}

// ------------------------------------------------------- hyperdiffusion
// Names of operator_swm_diff's operators (hordiff_factory_mod.f90:27-40)
// that this library provides: the narrow-Laplacian ones of the Ah grid
// (SBP 2/1, 4/2 and 6/3).
// kLapCh4: laplace_ch_halo4 with the ECS_xy halo (hordiff_factory_mod.f90:
// 33-34, 37-40, 196-223: "hordiff_scalar_Ah" and "hordiff_vec_xyz_Ah");
// kLapChCov: the same Laplacian on the covariant components as scalars
// ("hordiff_vec_Ah", hordiff_colocated_mod.f90:25-39).  FP64 contexts.
constexpr int kLapCh4 = 4, kLapChCov = 5;
int hordiff_uv_order(const char* name) {
  if (!name) return 0;
  if (!std::strcmp(name, "hordiff_vec_xyz_Ah_sbp_21_narrow")) return 21;
  if (!std::strcmp(name, "hordiff_vec_xyz_Ah_sbp_42_narrow")) return 42;
  if (!std::strcmp(name, "hordiff_vec_xyz_Ah_sbp_63_narrow")) return 63;
  if (!std::strcmp(name, "hordiff_vec_xyz_Ah")) return kLapCh4;
  if (!std::strcmp(name, "hordiff_vec_Ah")) return kLapChCov;
  return 0;
}
int hordiff_h_order(const char* name) {
  if (!name) return 0;
  if (!std::strcmp(name, "hordiff_scalar_Ah_sbp_21_narrow")) return 21;
  if (!std::strcmp(name, "hordiff_scalar_Ah_sbp_42_narrow")) return 42;
  if (!std::strcmp(name, "hordiff_scalar_Ah_sbp_63_narrow")) return 63;
  if (!std::strcmp(name, "hordiff_scalar_Ah")) return kLapCh4;
  return 0;
}
// ... and the C-grid ones (hordiff_factory_mod.f90:19-36): the parts of the
// vector hyperdiffusion (1 div, 2 curl, 3 both), and hordiff_scalar_C for h
// (stored as kHordiffScalarC).
constexpr int kHordiffScalarC = 21;
int hordiff_c_parts(const char* name) {
  if (!name) return 0;
  if (!std::strcmp(name, "hordiff_c_biharm_div")) return 1;
  if (!std::strcmp(name, "hordiff_c_biharm_curl")) return 2;
  if (!std::strcmp(name, "hordiff_c_biharm_curl_div")) return 3;
  return 0;
}
int hordiff_c_h(const char* name) {
  return name && !std::strcmp(name, "hordiff_scalar_C") ? kHordiffScalarC : 0;
}

// work fields of the diffusion step: F 4, L 4, tendencies 3, and (FP64, for
// the two-pass Laplacian) d1x 4, d1y 4
constexpr int kDiffWorkF32 = 11, kDiffWorkF64 = 19;

template <class T>
NarrowTables<T> narrow_tables(swm_ctx* ctx, int narrow) {
  void* const* t = ctx->ntab[narrow == 63 ? 1 : narrow == 21 ? 2 : 0];
  return NarrowTables<T>{narrow, (T*)t[0], (T*)t[1], (T*)t[2], (T*)t[3], (T*)t[4]};
}
template <class T> T* dwork(swm_ctx* ctx, int field) { return (T*)ctx->dw + field * ctx->g64.fs; }

// Workspace, basis vectors and the coefficient tables of order `narrow`, in
// the context precision (outside any capture: allocates on first use).
// The corner-mesh tables of a context: the C grid's own, or on the Ah grid
// (whose node mesh is the corner mesh) the tables-only object made on first
// use.
CGrid* node_tables(swm_ctx* ctx, int* rc) {
  *rc = SWM_OK;
  if (ctx->cg) return ctx->cg;
  if (!ctx->xyg) {
    std::string why;
    const int e = cgrid_create_tables(ctx->g64, ctx->N, ctx->cfg.radius, ctx->st, &ctx->xyg, why);
    if (e) { *rc = fail(ctx, e == 3 ? SWM_E_NOMEM : SWM_E_CUDA, why); return nullptr; }
  }
  return ctx->xyg;
}
int diffusion_ws(swm_ctx* ctx, int narrow) {
  const FieldGeom& g = ctx->g64;
  const size_t elt = (size_t)ctx->elt;
  const bool ch = narrow == kLapCh4 || narrow == kLapChCov;
  if (ch && ctx->prec != SWM_FP64_PLAIN)
    return fail(ctx, SWM_E_UNSUPPORTED, "hordiff_scalar_Ah / hordiff_vec_Ah / hordiff_vec_xyz_Ah run on FP64 contexts");
  if (!ch && ctx->n < 2 * narrow_rows(narrow))
    return fail(ctx, SWM_E_INVALID, "grid too small for the narrow Laplacian closures");
  if (ctx->prec == SWM_FP32_FUSED && !ctx->edge2)
    CK(cudaMalloc(&ctx->edge2, sizeof(float) * 16 * 6 * ctx->n), "alloc");
  if (!ctx->dw) {
    const size_t nw = ctx->prec == SWM_FP64_PLAIN ? kDiffWorkF64 : kDiffWorkF32;
    CK(cudaMalloc(&ctx->dw, elt * nw * g.fs), "alloc");
    CK(cudaMemsetAsync(ctx->dw, 0, elt * nw * g.fs, ctx->st), "memset");
  }
  if (!ctx->b12) {
    CK(cudaMalloc(&ctx->b12, elt * 6 * g.fs), "alloc");
    CK(cudaMemsetAsync(ctx->b12, 0, elt * 6 * g.fs, ctx->st), "memset");
    if (ctx->prec == SWM_FP64_PLAIN) {
      CK(launch_basis(g, ctx->hx, (double*)ctx->b12, ctx->st), "basis");
    } else {
      double* b64 = tmpf(ctx, 0);   // 6 FP64 work fields
      CK(cudaMemsetAsync(b64, 0, sizeof(double) * 6 * g.fs, ctx->st), "memset");
      CK(launch_basis(g, ctx->hx, b64, ctx->st), "basis");
      CK(launch_f64_to_f32(6 * g.fs, b64, (float*)ctx->b12, ctx->st), "basis f32");
    }
  }
  if (ch) {
    // the corner-mesh tables, the ECS_xy scratch and the metric tables, made
    // here, outside any capture
    int rc;
    CGrid* q = node_tables(ctx, &rc);
    if (!q) return rc;
    CK(cgrid_laplace_ch_prepare(q, ctx->st), "laplace_ch tables");
    return SWM_OK;
  }
  void** t = ctx->ntab[narrow == 63 ? 1 : narrow == 21 ? 2 : 0];
  if (!t[2]) {
    // FP32 contexts form the interior coefficients from the two b fields
    const bool f64 = ctx->prec == SWM_FP64_PLAIN;
    const size_t nw = f64 ? (size_t)narrow_width(narrow) * g.fs : 0;
    const size_t ncl = (size_t)narrow_closure_count(narrow, ctx->n);
    void* p[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    cudaError_t e = cudaSuccess;
    if (f64) e = cudaMalloc(&p[0], elt * nw);
    if (f64 && e == cudaSuccess) e = cudaMalloc(&p[1], elt * nw);
    if (e == cudaSuccess) e = cudaMalloc(&p[2], elt * ncl);
    if (e == cudaSuccess) e = cudaMalloc(&p[3], elt * ncl);
    if (e == cudaSuccess) e = cudaMalloc(&p[4], elt * 2 * g.fs);
    if (e == cudaSuccess) e = cudaMemsetAsync(p[4], 0, elt * 2 * g.fs, ctx->st);
    if (e == cudaSuccess) {
      if (f64)
        e = launch_narrow_tables<double>(
            g, NarrowTables<double>{narrow, (double*)p[0], (double*)p[1], (double*)p[2], (double*)p[3],
                                    (double*)p[4]},
            ctx->m64, ctx->st);
      else
        e = launch_narrow_tables<float>(
            g, NarrowTables<float>{narrow, nullptr, nullptr, (float*)p[2], (float*)p[3], (float*)p[4]},
            ctx->m64, ctx->st);
    }
    if (e != cudaSuccess) {
      for (void* q : p) if (q) cudaFree(q);
      return fail(ctx, e == cudaErrorMemoryAllocation ? SWM_E_NOMEM : SWM_E_CUDA,
                  std::string("diffusion tables: ") + cudaGetErrorString(e));
    }
    for (int k = 0; k < 5; ++k) t[k] = p[k];
  }
  return SWM_OK;
}

// Synced Laplacian of nf fields src -> dst (laplace_Ah_sbp42_narrow_mod
// .f90:23-58); src and dst do not overlap; FP64 uses the d1 work fields.
template <class T>
int laplace_fields(swm_ctx* ctx, int narrow, int nf, const T* src, T* dst) {
  const FieldGeom& g = ctx->g64;
  if (narrow == kLapCh4) {
    if constexpr (sizeof(T) == 8) {
      for (int k = 0; k < nf; ++k)
        CK(cgrid_laplace_ch(ctx->xyg, ctx->topo, ctx->edge64, 4, src + (long long)k * g.fs,
                            dst + (long long)k * g.fs, ctx->st),
           "laplace_ch_halo4");
      return SWM_OK;
    } else {
      return fail(ctx, SWM_E_UNSUPPORTED, "laplace_ch_halo4 runs on FP64 contexts");
    }
  }
  T* edge = sizeof(T) == 8 ? (T*)ctx->edge64 : (T*)ctx->edge;
  T* d1 = sizeof(T) == 8 ? dwork<T>(ctx, kDiffWorkF32) : nullptr;
  CK(launch_laplace<T>(g, ctx->topo, narrow_tables<T>(ctx, narrow), nf, src, metric_of<T>(ctx),
                       ctx->hx * ctx->cfg.radius, d1, d1 ? d1 + 4 * g.fs : nullptr, dst, edge,
                       ctx->st),
     "laplace");
  return SWM_OK;
}

// -(c^4) for a diffusion coefficient, c = coeff*radius*hx
// (hordiff_factory_mod.f90:183)
double diff_coeff4(const swm_ctx* ctx, double coeff) {
  const double dc = coeff * ctx->cfg.radius * ctx->hx;
  const double dc2 = dc * dc;
  return -1.0 * (dc2 * dc2);
}

// L(L(.)) of h and of the Cartesian components b1*u + b2*v of the velocity
// into the work fields 0 (h) and 1..3 (x, y, z).
template <class T>
int enqueue_biharmonic(swm_ctx* ctx, const T* h, const T* u, const T* v) {
  const FieldGeom& g = ctx->g64;
  const long long fs = g.fs;
  T* F = dwork<T>(ctx, 0);
  T* L = dwork<T>(ctx, 4);
  CK(launch_to_cart<T>(g, (const T*)ctx->b12, h, u, v, F, F + fs, ctx->st), "to cart");
  if (ctx->diff_uv == ctx->diff_h) {
    if (int rc = laplace_fields<T>(ctx, ctx->diff_h, 4, F, L)) return rc;
    if (int rc = laplace_fields<T>(ctx, ctx->diff_h, 4, L, F)) return rc;
  } else {
    if (int rc = laplace_fields<T>(ctx, ctx->diff_h, 1, F, L)) return rc;
    if (int rc = laplace_fields<T>(ctx, ctx->diff_h, 1, L, F)) return rc;
    if (int rc = laplace_fields<T>(ctx, ctx->diff_uv, 3, F + fs, L + fs)) return rc;
    if (int rc = laplace_fields<T>(ctx, ctx->diff_uv, 3, L + fs, F + fs)) return rc;
  }
  return SWM_OK;
}

// Diffusion tendencies of the fields (h, u, v) into (th, tu, tv)
// (operator_swm_diff_mod.f90:25-46): the xyz-vector operator on (u, v)
// (hordiff_colocated_mod.f90:41-58) and the scalar one on h
// (hordiff_scalar_mod.f90:33-53), each -(c^4) L(L(.)).
template <class T>
int enqueue_diffusion_tend(swm_ctx* ctx, const T* h, const T* u, const T* v, T* th, T* tu, T* tv) {
  const FieldGeom& g = ctx->g64;
  if (ctx->diff_uv == kLapChCov) {
    // hordiff_vec_Ah (hordiff_colocated_mod.f90:25-39): u and v diffused as
    // scalars, -(c^4) L(L(.)), then the covariant vector sync; h with its own
    // operator
    if constexpr (sizeof(T) == 8) {
      const long long fs = g.fs;
      T* F = dwork<T>(ctx, 0);
      T* L = dwork<T>(ctx, 4);
      CK(cudaMemcpyAsync(F, h, sizeof(T) * fs, cudaMemcpyDeviceToDevice, ctx->st), "copy");
      CK(cudaMemcpyAsync(F + fs, u, sizeof(T) * fs, cudaMemcpyDeviceToDevice, ctx->st), "copy");
      CK(cudaMemcpyAsync(F + 2 * fs, v, sizeof(T) * fs, cudaMemcpyDeviceToDevice, ctx->st), "copy");
      if (int rc = laplace_fields<T>(ctx, ctx->diff_h, 1, F, L)) return rc;
      if (int rc = laplace_fields<T>(ctx, ctx->diff_h, 1, L, F)) return rc;
      if (int rc = laplace_fields<T>(ctx, kLapCh4, 2, F + fs, L + fs)) return rc;
      if (int rc = laplace_fields<T>(ctx, kLapCh4, 2, L + fs, F + fs)) return rc;
      const double ch = diff_coeff4(ctx, ctx->diff_h_coeff), cu = diff_coeff4(ctx, ctx->diff_uv_coeff);
      CK(launch_axpby(fs, ch, F, 0.0, F, th, ctx->st), "tendency");
      CK(launch_axpby(fs, cu, F + fs, 0.0, F + fs, tu, ctx->st), "tendency");
      CK(launch_axpby(fs, cu, F + 2 * fs, 0.0, F + 2 * fs, tv, ctx->st), "tendency");
      CK(launch_sync_vector_t<T>(g, ctx->topo, ctx->qw, tu, tv, (T*)ctx->edge64, ctx->st), "vector sync");
      return SWM_OK;
    } else {
      return fail(ctx, SWM_E_UNSUPPORTED, "hordiff_vec_Ah runs on FP64 contexts");
    }
  }
  if (int rc = enqueue_biharmonic<T>(ctx, h, u, v)) return rc;
  const T* F = dwork<T>(ctx, 0);
  CK(launch_diff_tendency<T>(g, (const T*)ctx->b12, diff_coeff4(ctx, ctx->diff_uv_coeff), F + g.fs,
                             tu, tv, diff_coeff4(ctx, ctx->diff_h_coeff), F, th, ctx->st),
     "tendency");
  T* edge = sizeof(T) == 8 ? (T*)ctx->edge64 : (T*)ctx->edge;
  CK(launch_sync_vector_t<T>(g, ctx->topo, ctx->qw, tu, tv, edge, ctx->st), "vector sync");
  return SWM_OK;
}

// One explicit Euler step of the diffusion operator (explicit_Eul1_mod.f90:
// 20-30): v0 = v0 + dt * D(v0).  FP32 contexts take the tendency of the
// high part in FP32 and add it to the (hi, lo) pair with a two-sum, fused
// with the tendency and the sync (launch_diff_update_f32); with the 4/2
// order for h and the velocity the Laplacians' syncs ride in the next
// launch's reads (launch_biharmonic_f32).
int enqueue_diffusion_step(swm_ctx* ctx, swm_state* v0, double dt) {
  const long long fs = ctx->g64.fs;
  if (ctx->cg) {
    const double cu = diff_coeff4(ctx, ctx->diff_uv_coeff), ch = diff_coeff4(ctx, ctx->diff_h_coeff);
    if (ctx->prec == SWM_FP64_PLAIN)
      CK(cgrid_diffusion_step(ctx->cg, ctx->topo, ctx->edge64, ctx->diff_uv, cu, ch, (double*)v0->hi, dt, ctx->st),
         "C-grid diffusion step");
    else
      CK(cgrid_diffusion_step32(ctx->cg, ctx->topo, (float*)ctx->edge, ctx->diff_uv, cu, ch, (float*)v0->hi, v0->lo,
                                dt, ctx->st),
         "C-grid diffusion step");
    return SWM_OK;
  }
  if (ctx->prec == SWM_FP64_PLAIN) {
    double* x = (double*)v0->hi;
    double* T = dwork<double>(ctx, 8);
    if (int rc = enqueue_diffusion_tend<double>(ctx, x, x + fs, x + 2 * fs, T, T + fs, T + 2 * fs))
      return rc;
    CK(launch_axpby(3 * fs, 1.0, x, dt, T, x, ctx->st), "update");
  } else {
    float* x = (float*)v0->hi;
    float* F = dwork<float>(ctx, 0);
    float* T = dwork<float>(ctx, 8);
    const float* edge_in = nullptr;
    if (ctx->diff_uv == ctx->diff_h && ctx->diff_h == 42) {
      // the 4/2 order for h and the velocity: two Laplacian launches of the
      // 4 fields, their syncs folded into the next launch's reads
      const FieldGeom& g = ctx->g64;
      CK(launch_to_cart<float>(g, (const float*)ctx->b12, x, x + fs, x + 2 * fs, F, F + fs, ctx->st),
         "to cart");
      CK(launch_biharmonic_f32(g, ctx->topo, narrow_tables<float>(ctx, ctx->diff_h), F,
                               dwork<float>(ctx, 4), metric_of<float>(ctx), ctx->hx * ctx->cfg.radius,
                               (float*)ctx->edge, (float*)ctx->edge2, ctx->st),
         "biharmonic");
      edge_in = (const float*)ctx->edge2;
    } else if (int rc = enqueue_biharmonic<float>(ctx, x, x + fs, x + 2 * fs)) {
      return rc;
    }
    CK(launch_diff_update_f32(ctx->g64, ctx->topo, ctx->qw, (const float*)ctx->b12,
                              diff_coeff4(ctx, ctx->diff_uv_coeff), F + fs,
                              diff_coeff4(ctx, ctx->diff_h_coeff), F, dt, x, v0->lo, T + fs,
                              T + 2 * fs, (float*)ctx->edge, edge_in, ctx->st),
       "update");
  }
  return SWM_OK;
}

int diffusion_ready(swm_ctx* ctx) {
  if (!ctx->diff_uv) return fail(ctx, SWM_E_INVALID, "diffusion is not configured (swm_diffusion_set)");
  if (ctx->cg) {
    CK(cgrid_diffusion_prepare(ctx->cg), "C-grid diffusion workspace");
    return SWM_OK;
  }
  if (int rc = diffusion_ws(ctx, ctx->diff_uv)) return rc;
  return diffusion_ws(ctx, ctx->diff_h);
}

}  // namespace

extern "C" {

int swm_rk4_step(swm_ctx* ctx, swm_state* v0, double dt, int nsteps) {
  TraceRange trace_("swm_rk4_step");
  if (int rc = check_state(ctx, v0)) return rc;
  if (nsteps < 0 || !std::isfinite(dt)) return fail(ctx, SWM_E_INVALID, "bad dt or nsteps");
  if (nsteps == 0) return SWM_OK;
  USE_DEVICE(ctx);
  if (ctx->timing) {
    for (int k = 0; k < nsteps; ++k)
      if (int rc = enqueue_rk4_any(ctx, v0, dt)) return rc;
    return SWM_OK;
  }
  return graph_steps(ctx, v0, dt, 0, nsteps, [&] { return enqueue_rk4_any(ctx, v0, dt); });
}

int swm_diffusion_set(swm_ctx* ctx, const char* hordiff_uv_name, double uv_diff_coeff,
                      const char* hordiff_h_name, double h_diff_coeff) {
  if (!ctx) return fail(nullptr, SWM_E_INVALID, "null context");
  const int uv = ctx->cg ? hordiff_c_parts(hordiff_uv_name) : hordiff_uv_order(hordiff_uv_name);
  const int h = ctx->cg ? hordiff_c_h(hordiff_h_name) : hordiff_h_order(hordiff_h_name);
  if (!uv || !h)
    return fail(ctx, SWM_E_UNSUPPORTED,
                std::string("unsupported hordiff operator: ") +
                    (!uv ? (hordiff_uv_name ? hordiff_uv_name : "(null)")
                         : (hordiff_h_name ? hordiff_h_name : "(null)")));
  if (!std::isfinite(uv_diff_coeff) || !std::isfinite(h_diff_coeff))
    return fail(ctx, SWM_E_INVALID, "bad diffusion coefficient");
  USE_DEVICE(ctx);
  const int old_uv = ctx->diff_uv, old_h = ctx->diff_h;
  const double old_cu = ctx->diff_uv_coeff, old_ch = ctx->diff_h_coeff;
  ctx->diff_uv = uv; ctx->diff_h = h;
  ctx->diff_uv_coeff = uv_diff_coeff; ctx->diff_h_coeff = h_diff_coeff;
  if (int rc = diffusion_ready(ctx)) {
    ctx->diff_uv = old_uv; ctx->diff_h = old_h;
    ctx->diff_uv_coeff = old_cu; ctx->diff_h_coeff = old_ch;
    return rc;
  }
  // captured graphs hold the old coefficients
  for (auto it = ctx->graphs.begin(); it != ctx->graphs.end();) {
    if (std::get<2>(it->first) != 0) { cudaGraphExecDestroy(it->second.exec); it = ctx->graphs.erase(it); }
    else ++it;
  }
  return SWM_OK;
}

int swm_apply_diffusion(swm_ctx* ctx, swm_state* vout, const swm_state* vin) {
  TraceRange trace_("swm_apply_diffusion");
  if (int rc = check_state(ctx, vout)) return rc;
  if (int rc = check_state(ctx, vin)) return rc;
  if (vout == vin) return fail(ctx, SWM_E_INVALID, "apply needs distinct in/out states");
  USE_DEVICE(ctx);
  if (int rc = diffusion_ready(ctx)) return rc;
  const long long fs = ctx->g64.fs;
  if (ctx->cg) {
    const double cu = diff_coeff4(ctx, ctx->diff_uv_coeff), ch = diff_coeff4(ctx, ctx->diff_h_coeff);
    if (ctx->prec == SWM_FP64_PLAIN) {
      CK(cgrid_diffusion(ctx->cg, ctx->topo, ctx->edge64, ctx->diff_uv, cu, ch, (const double*)vin->hi,
                         (double*)vout->hi, ctx->st),
         "C-grid diffusion");
    } else {
      CK(cudaMemsetAsync(vout->lo, 0, sizeof(float) * 3 * fs, ctx->st), "memset");
      CK(cgrid_diffusion32(ctx->cg, ctx->topo, (float*)ctx->edge, ctx->diff_uv, cu, ch, (const float*)vin->hi,
                           (float*)vout->hi, ctx->st),
         "C-grid diffusion");
    }
    return SWM_OK;
  }
  if (ctx->prec == SWM_FP64_PLAIN) {
    const double* x = (const double*)vin->hi;
    double* o = (double*)vout->hi;
    return enqueue_diffusion_tend<double>(ctx, x, x + fs, x + 2 * fs, o, o + fs, o + 2 * fs);
  }
  const float* x = (const float*)vin->hi;
  float* o = (float*)vout->hi;
  CK(cudaMemsetAsync(vout->lo, 0, sizeof(float) * 3 * fs, ctx->st), "memset");
  return enqueue_diffusion_tend<float>(ctx, x, x + fs, x + 2 * fs, o, o + fs, o + 2 * fs);
}

int swm_diffusion_step(swm_ctx* ctx, swm_state* v0, double dt, int nsteps) {
  TraceRange trace_("swm_diffusion_step");
  if (int rc = check_state(ctx, v0)) return rc;
  if (nsteps < 0 || !std::isfinite(dt)) return fail(ctx, SWM_E_INVALID, "bad dt or nsteps");
  USE_DEVICE(ctx);
  if (int rc = diffusion_ready(ctx)) return rc;
  if (nsteps == 0) return SWM_OK;
  return graph_steps(ctx, v0, dt, 2, nsteps, [&] { return enqueue_diffusion_step(ctx, v0, dt); });
}

int swm_model_step(swm_ctx* ctx, swm_state* v0, double dt, int nsteps) {
  TraceRange trace_("swm_model_step");
  if (int rc = check_state(ctx, v0)) return rc;
  if (nsteps < 0 || !std::isfinite(dt)) return fail(ctx, SWM_E_INVALID, "bad dt or nsteps");
  USE_DEVICE(ctx);
  if (!ctx->diff_uv) return swm_rk4_step(ctx, v0, dt, nsteps);
  if (int rc = diffusion_ready(ctx)) return rc;
  if (nsteps == 0) return SWM_OK;
  return graph_steps(ctx, v0, dt, 1, nsteps, [&] {
    if (int rc = enqueue_rk4_any(ctx, v0, dt)) return rc;
    return enqueue_diffusion_step(ctx, v0, dt);
  });
}

int swm_laplace(swm_ctx* ctx, swm_field* out, const swm_field* in, int narrow_order) {
  AH_ONLY(ctx, "swm_laplace");
  TraceRange trace_("swm_laplace");
  if (int rc = check_field(ctx, out)) return rc;
  if (int rc = check_field(ctx, in)) return rc;
  if (narrow_order != 21 && narrow_order != 42 && narrow_order != 63)
    return fail(ctx, SWM_E_UNSUPPORTED, "narrow Laplacian order must be 21, 42 or 63");
  if (ctx->prec != SWM_FP64_PLAIN)
    return fail(ctx, SWM_E_UNSUPPORTED, "swm_laplace works on FP64 contexts");
  USE_DEVICE(ctx);
  if (int rc = diffusion_ws(ctx, narrow_order)) return rc;
  double* F = dwork<double>(ctx, 0);   // the input may be the output
  CK(cudaMemcpyAsync(F, in->p, sizeof(double) * ctx->g64.fs, cudaMemcpyDeviceToDevice, ctx->st), "copy");
  return laplace_fields<double>(ctx, narrow_order, 1, F, out->p);
}

int swm_diagnostics(swm_ctx* ctx, const swm_state* s, double out[7]) {
  AH_ONLY(ctx, "swm_diagnostics");
  TraceRange trace_("swm_diagnostics");
  if (int rc = check_state(ctx, s)) return rc;
  if (!out) return fail(ctx, SWM_E_INVALID, "null output");
  USE_DEVICE(ctx);
  const double *h, *u, *v;
  if (int rc = state64(ctx, s, &h, &u, &v)) return rc;
  double* z = tmpf(ctx, 0);
  double *ku = tmpf(ctx, 1), *kv = tmpf(ctx, 2), *pe = tmpf(ctx, 3), *en = tmpf(ctx, 4);
  if (int rc = op_curl(ctx, u, v, z)) return rc;
  CK(launch_diag_integrands(ctx->g64, ctx->m64, ctx->cfg.grav, h, u, v, ctx->hs64, z, ku, kv, pe, en, ctx->st), "diag");
  if (int rc = reduce(ctx, 2, h, nullptr, 0)) return rc;
  if (int rc = reduce(ctx, 3, h, nullptr, 1)) return rc;
  if (int rc = reduce(ctx, 1, h, nullptr, 2)) return rc;
  if (int rc = reduce(ctx, 1, ku, nullptr, 3)) return rc;
  if (int rc = reduce(ctx, 1, kv, nullptr, 4)) return rc;
  if (int rc = reduce(ctx, 1, pe, nullptr, 5)) return rc;
  if (int rc = reduce(ctx, 1, en, nullptr, 6)) return rc;
  double r[7];
  if (int rc = fetch_results(ctx, 7, r)) return rc;
  const double ke = r[3] + r[4];
  out[0] = r[0]; out[1] = r[1]; out[2] = r[2];
  out[3] = ke + r[5]; out[4] = ke; out[5] = r[5]; out[6] = r[6];
  return SWM_OK;
}

// ---------------------------------------------------------------- fields
int swm_field_create(swm_ctx* ctx, swm_field** out) { return swm_field_create_mesh(ctx, SWM_MESH_P, out); }

int swm_field_create_mesh(swm_ctx* ctx, int mesh, swm_field** out) {
  if (!ctx || !out) return fail(ctx, SWM_E_INVALID, "null argument");
  if (mesh < SWM_MESH_P || mesh > SWM_MESH_Q) return fail(ctx, SWM_E_INVALID, "unknown mesh");
  USE_DEVICE(ctx);
  swm_field* f = new swm_field{ctx, nullptr, mesh};
  cudaError_t e = cudaMalloc(&f->p, sizeof(double) * ctx->fs);
  if (e == cudaSuccess) e = cudaMemsetAsync(f->p, 0, sizeof(double) * ctx->fs, ctx->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
  if (e != cudaSuccess) {
    if (f->p) cudaFree(f->p);
    delete f;
    return fail(ctx, SWM_E_NOMEM, std::string("field alloc: ") + cudaGetErrorString(e));
  }
  ctx->fields.insert(f);
  *out = f;
  return SWM_OK;
}

void swm_field_free(swm_field* f) {
  if (!f) return;
  if (swm_ctx* c = f->ctx) {
    cudaSetDevice(c->cfg.device);
    cudaStreamSynchronize(c->st);
    if (f->p) cudaFree(f->p);
    c->fields.erase(f);
  }
  delete f;
}

int swm_field_upload(swm_ctx* ctx, swm_field* f, const double* host) {
  if (int rc = check_field(ctx, f)) return rc;
  if (!host) return fail(ctx, SWM_E_INVALID, "null host array");
  USE_DEVICE(ctx);
  if (ctx->cg) return c_copy(ctx, f->mesh, f->p, host, nullptr);
  return put_field(ctx, f->p, host);
}

int swm_field_download(swm_ctx* ctx, const swm_field* f, double* host) {
  if (int rc = check_field(ctx, f)) return rc;
  if (!host) return fail(ctx, SWM_E_INVALID, "null host array");
  USE_DEVICE(ctx);
  if (ctx->cg) return c_copy(ctx, f->mesh, f->p, nullptr, host);
  const size_t bytes = sizeof(double) * 6 * (size_t)ctx->n * ctx->n;
  PackedFields pf{{(double*)mapped_host(host, bytes), nullptr, nullptr}};
  const bool staged = !pf.f[0];
  if (staged) pf.f[0] = tmpf(ctx, 11);
  CK(launch_pack_state(ctx->g64, 1, f->p, nullptr, pf, ctx->st), "pack");
  if (staged) CK(cudaMemcpyAsync(host, pf.f[0], bytes, cudaMemcpyDeviceToHost, ctx->st), "download");
  if (int rc_ = sync_check(ctx, ctx->st)) return rc_;
  return SWM_OK;
}

#define CHECK_FIELDS(...)                                       \
  do {                                                          \
    const swm_field* fl_[] = {__VA_ARGS__};                     \
    for (const swm_field* f_ : fl_)                             \
      if (int rc_ = check_field(ctx, f_)) return rc_;           \
    USE_DEVICE(ctx);                                            \
  } while (0)

int swm_op_co2contra(swm_ctx* ctx, swm_field* ut, swm_field* vt, const swm_field* u, const swm_field* v) {
  CHECK_FIELDS(ut, vt, u, v);
  if (ctx->cg) {
    for (auto fm : {std::make_pair((const swm_field*)ut, SWM_MESH_U), std::make_pair((const swm_field*)vt, SWM_MESH_V),
                    std::make_pair(u, SWM_MESH_U), std::make_pair(v, SWM_MESH_V)})
      if (int rc = check_mesh(ctx, fm.first, fm.second, "co2contra")) return rc;
    CK(cgrid_co2contra(ctx->cg, u->p, v->p, ut->p, vt->p, ctx->st), "co2contra");
    return SWM_OK;
  }
  CK(launch_co2contra(ctx->g64, ctx->m64, u->p, v->p, ut->p, vt->p, ctx->st), "co2contra");
  return SWM_OK;
}
int swm_op_massflux(swm_ctx* ctx, swm_field* hu, swm_field* hv, const swm_field* h, const swm_field* ut, const swm_field* vt) {
  CHECK_FIELDS(hu, hv, h, ut, vt);
  if (ctx->cg) {
    for (auto fm : {std::make_pair((const swm_field*)hu, SWM_MESH_U), std::make_pair((const swm_field*)hv, SWM_MESH_V),
                    std::make_pair(h, SWM_MESH_P), std::make_pair(ut, SWM_MESH_U), std::make_pair(vt, SWM_MESH_V)})
      if (int rc = check_mesh(ctx, fm.first, fm.second, "massflux")) return rc;
    CK(cgrid_massflux(ctx->cg, h->p, ut->p, vt->p, hu->p, hv->p, ctx->st), "massflux");
    return SWM_OK;
  }
  CK(launch_massflux(ctx->g64, h->p, ut->p, vt->p, hu->p, hv->p, ctx->st), "massflux");
  return SWM_OK;
}
int swm_op_ke(swm_ctx* ctx, swm_field* ke, const swm_field* u, const swm_field* v, const swm_field* ut, const swm_field* vt) {
  CHECK_FIELDS(ke, u, v, ut, vt);
  if (ctx->cg) {
    for (auto fm : {std::make_pair((const swm_field*)ke, SWM_MESH_P), std::make_pair(u, SWM_MESH_U),
                    std::make_pair(v, SWM_MESH_V), std::make_pair(ut, SWM_MESH_U), std::make_pair(vt, SWM_MESH_V)})
      if (int rc = check_mesh(ctx, fm.first, fm.second, "KE")) return rc;
    CK(cgrid_ke(ctx->cg, u->p, v->p, ut->p, vt->p, ke->p, ctx->st), "KE");
    return SWM_OK;
  }
  CK(launch_ke(ctx->g64, u->p, v->p, ut->p, vt->p, ke->p, ctx->st), "KE");
  return SWM_OK;
}
int swm_op_grad(swm_ctx* ctx, swm_field* gx, swm_field* gy, const swm_field* f) {
  CHECK_FIELDS(gx, gy, f);
  if (ctx->cg) {
    for (auto fm : {std::make_pair((const swm_field*)gx, SWM_MESH_U), std::make_pair((const swm_field*)gy, SWM_MESH_V),
                    std::make_pair(f, SWM_MESH_P)})
      if (int rc = check_mesh(ctx, fm.first, fm.second, "grad")) return rc;
    CK(cgrid_grad(ctx->cg, f->p, gx->p, gy->p, ctx->st), "grad");
    return SWM_OK;
  }
  return op_grad(ctx, f->p, gx->p, gy->p);
}
int swm_op_div(swm_ctx* ctx, swm_field* div, const swm_field* u, const swm_field* v) {
  CHECK_FIELDS(div, u, v);
  if (ctx->cg) {
    for (auto fm : {std::make_pair((const swm_field*)div, SWM_MESH_P), std::make_pair(u, SWM_MESH_U),
                    std::make_pair(v, SWM_MESH_V)})
      if (int rc = check_mesh(ctx, fm.first, fm.second, "div")) return rc;
    CK(cgrid_div(ctx->cg, u->p, v->p, div->p, ctx->st), "div");
    return SWM_OK;
  }
  return op_div(ctx, u->p, v->p, div->p);
}
int swm_op_curl(swm_ctx* ctx, swm_field* curl, const swm_field* u, const swm_field* v) {
  CHECK_FIELDS(curl, u, v);
  if (ctx->cg) {
    for (auto fm : {std::make_pair((const swm_field*)curl, SWM_MESH_Q), std::make_pair(u, SWM_MESH_U),
                    std::make_pair(v, SWM_MESH_V)})
      if (int rc = check_mesh(ctx, fm.first, fm.second, "curl")) return rc;
    CK(cgrid_curl(ctx->cg, ctx->topo, ctx->edge64, u->p, v->p, curl->p, ctx->st), "curl");
    return SWM_OK;
  }
  return op_curl(ctx, u->p, v->p, curl->p);
}
int swm_op_coriolis(swm_ctx* ctx, swm_field* cor_u, swm_field* cor_v, const swm_field* hu, const swm_field* hv,
                    const swm_field* h, const swm_field* curl) {
  CHECK_FIELDS(cor_u, cor_v, hu, hv, h, curl);
  if (ctx->cg) {
    for (auto fm : {std::make_pair((const swm_field*)cor_u, SWM_MESH_U), std::make_pair((const swm_field*)cor_v, SWM_MESH_V),
                    std::make_pair(hu, SWM_MESH_U), std::make_pair(hv, SWM_MESH_V), std::make_pair(h, SWM_MESH_P),
                    std::make_pair(curl, SWM_MESH_Q)})
      if (int rc = check_mesh(ctx, fm.first, fm.second, "coriolis")) return rc;
    CK(cgrid_coriolis(ctx->cg, hu->p, hv->p, h->p, curl->p, cor_u->p, cor_v->p, ctx->st), "coriolis");
    return SWM_OK;
  }
  CK(launch_coriolis(ctx->g64, ctx->m64, hu->p, hv->p, h->p, curl->p, cor_u->p, cor_v->p, ctx->st), "coriolis");
  return SWM_OK;
}
int swm_op_grad_perp(swm_ctx* ctx, swm_field* gu, swm_field* gv, const swm_field* w) {
  if (ctx && !ctx->cg) return fail(ctx, SWM_E_UNSUPPORTED, "grad_perp is provided on the C grid only");
  CHECK_FIELDS(gu, gv, w);
  for (auto fm : {std::make_pair((const swm_field*)gu, SWM_MESH_U), std::make_pair((const swm_field*)gv, SWM_MESH_V),
                  std::make_pair(w, SWM_MESH_Q)})
    if (int rc = check_mesh(ctx, fm.first, fm.second, "grad_perp")) return rc;
  CK(cgrid_grad_perp(ctx->cg, w->p, gu->p, gv->p, ctx->st), "grad_perp");
  return SWM_OK;
}
int swm_op_contra2co(swm_ctx* ctx, swm_field* u, swm_field* v, const swm_field* ut, const swm_field* vt) {
  if (ctx && !ctx->cg) return fail(ctx, SWM_E_UNSUPPORTED, "contra2co is provided on the C grid only");
  CHECK_FIELDS(u, v, ut, vt);
  for (auto fm : {std::make_pair((const swm_field*)u, SWM_MESH_U), std::make_pair((const swm_field*)v, SWM_MESH_V),
                  std::make_pair(ut, SWM_MESH_U), std::make_pair(vt, SWM_MESH_V)})
    if (int rc = check_mesh(ctx, fm.first, fm.second, "contra2co")) return rc;
  CK(cgrid_contra2co(ctx->cg, ut->p, vt->p, u->p, v->p, ctx->st), "contra2co");
  return SWM_OK;
}
int swm_op_grad_a2_ecs(swm_ctx* ctx, swm_field* gx, swm_field* gy, const swm_field* f) {
  if (ctx && !ctx->cg) return fail(ctx, SWM_E_UNSUPPORTED, "gradient_a2_ecs needs the cell-centre mesh of the C grid");
  CHECK_FIELDS(gx, gy, f);
  for (const swm_field* x : {(const swm_field*)gx, (const swm_field*)gy, f})
    if (int rc = check_mesh(ctx, x, SWM_MESH_P, "gradient_a2_ecs")) return rc;
  if (gx == f || gy == f || gx == gy) return fail(ctx, SWM_E_INVALID, "gradient_a2_ecs needs distinct fields");
  CK(cgrid_grad_a2_ecs(ctx->cg, f->p, gx->p, gy->p, ctx->st), "gradient_a2_ecs");
  return SWM_OK;
}
int swm_halo_ecs_o(swm_ctx* ctx, const swm_field* f, int halo_width, double* ext) {
  if (ctx && !ctx->cg) return fail(ctx, SWM_E_UNSUPPORTED, "the ECS_O halo needs the cell-centre mesh of the C grid");
  CHECK_FIELDS(f);
  if (int rc = check_mesh(ctx, f, SWM_MESH_P, "ECS_O halo")) return rc;
  if (halo_width < 1 || halo_width > 2) return fail(ctx, SWM_E_INVALID, "ECS_O halo width must be 1 or 2");
  if (!ext) return fail(ctx, SWM_E_INVALID, "null output");
  CK(cgrid_ecs_o_halo(ctx->cg, f->p, halo_width, ext, ctx->st), "ECS_O halo");
  return SWM_OK;
}
int swm_halo_ecs_xy(swm_ctx* ctx, const swm_field* f, int halo_width, double* ext) {
  CHECK_FIELDS(f);
  if (int rc = check_mesh(ctx, f, SWM_MESH_Q, "ECS_xy halo")) return rc;
  if (halo_width < 1 || halo_width > 4) return fail(ctx, SWM_E_INVALID, "ECS_xy halo width must be 1..4");
  if (!ext) return fail(ctx, SWM_E_INVALID, "null output");
  int rc;
  CGrid* q = node_tables(ctx, &rc);
  if (!q) return rc;
  CK(cgrid_ecs_xy_halo(q, f->p, halo_width, ext, ctx->st), "ECS_xy halo");
  return SWM_OK;
}
int swm_laplace_ch(swm_ctx* ctx, swm_field* out, const swm_field* in, int order) {
  CHECK_FIELDS(out, in);
  for (const swm_field* x : {(const swm_field*)out, in})
    if (int rc = check_mesh(ctx, x, SWM_MESH_Q, "laplace_ch_halo")) return rc;
  if (order != 2 && order != 4) return fail(ctx, SWM_E_INVALID, "laplace_ch_halo order must be 2 or 4");
  int rc;
  CGrid* q = node_tables(ctx, &rc);
  if (!q) return rc;
  CK(cgrid_laplace_ch(q, ctx->topo, ctx->edge64, order, in->p, out->p, ctx->st), "laplace_ch_halo");
  return SWM_OK;
}
int swm_op_grad_c2_ecs(swm_ctx* ctx, swm_field* gx, swm_field* gy, const swm_field* f) {
  if (ctx && !ctx->cg) return fail(ctx, SWM_E_UNSUPPORTED, "gradient_c2_ecs is provided on the C grid only");
  CHECK_FIELDS(gx, gy, f);
  for (auto fm : {std::make_pair((const swm_field*)gx, SWM_MESH_U), std::make_pair((const swm_field*)gy, SWM_MESH_V),
                  std::make_pair(f, SWM_MESH_P)})
    if (int rc = check_mesh(ctx, fm.first, fm.second, "gradient_c2_ecs")) return rc;
  CK(cgrid_grad_c2_ecs(ctx->cg, f->p, gx->p, gy->p, ctx->st), "gradient_c2_ecs");
  return SWM_OK;
}
int swm_op_div_a2_ecs(swm_ctx* ctx, swm_field* div, const swm_field* u, const swm_field* v) {
  if (ctx && !ctx->cg) return fail(ctx, SWM_E_UNSUPPORTED, "divergence_a2_ecs needs the cell-centre mesh of the C grid");
  CHECK_FIELDS(div, u, v);
  for (const swm_field* x : {(const swm_field*)div, u, v})
    if (int rc = check_mesh(ctx, x, SWM_MESH_P, "divergence_a2_ecs")) return rc;
  if (div == u || div == v) return fail(ctx, SWM_E_INVALID, "divergence_a2_ecs needs an output distinct from its inputs");
  CK(cgrid_div_a2_ecs(ctx->cg, u->p, v->p, div->p, ctx->st), "divergence_a2_ecs");
  return SWM_OK;
}
int swm_halo_ecs_a_vec(swm_ctx* ctx, const swm_field* u, const swm_field* v, int halo_width, double* ext_u,
                       double* ext_v) {
  if (ctx && !ctx->cg) return fail(ctx, SWM_E_UNSUPPORTED, "the ecs_A_vec halo needs the cell-centre mesh of the C grid");
  CHECK_FIELDS(u, v);
  for (const swm_field* x : {u, v})
    if (int rc = check_mesh(ctx, x, SWM_MESH_P, "ecs_A_vec halo")) return rc;
  if (halo_width < 1 || halo_width > 2) return fail(ctx, SWM_E_INVALID, "ecs_A_vec halo width must be 1 or 2");
  if (!ext_u || !ext_v) return fail(ctx, SWM_E_INVALID, "null output");
  CK(cgrid_ecs_a_vec_halo(ctx->cg, u->p, v->p, halo_width, ext_u, ext_v, ctx->st), "ecs_A_vec halo");
  return SWM_OK;
}
int swm_sync_scalar(swm_ctx* ctx, swm_field* f) {
  CHECK_FIELDS(f);
  // on the C grid the corner mesh is the one with duplicated edge points
  if (int rc = check_mesh(ctx, f, SWM_MESH_Q, "sync_scalar")) return rc;
  CK(launch_sync_scalar(ctx->g64, ctx->topo, f->p, ctx->edge64, ctx->st), "sync");
  return SWM_OK;
}
int swm_sync_vector_cov(swm_ctx* ctx, swm_field* gx, swm_field* gy) {
  AH_ONLY(ctx, "swm_sync_vector_cov");
  CHECK_FIELDS(gx, gy);
  CK(launch_sync_vector(ctx->g64, ctx->topo, ctx->qw, gx->p, gy->p, ctx->edge64, ctx->st), "sync");
  return SWM_OK;
}
int swm_quadrature_mass(swm_ctx* ctx, const swm_field* f, double* out) {
  CHECK_FIELDS(f);
  if (!out) return fail(ctx, SWM_E_INVALID, "null output");
  if (ctx->cg) {
    CK(cgrid_mass(ctx->cg, f->mesh, f->p, ctx->dres, ctx->st), "C-grid quadrature");
    return fetch_results(ctx, 1, out);
  }
  if (int rc = reduce(ctx, 1, f->p, nullptr, 0)) return rc;
  return fetch_results(ctx, 1, out);
}

// ---------------------------------------------------------------- static scratch
int swm_sync_scalar_static(swm_ctx* ctx, swm_field* f) {
  AH_ONLY(ctx, "swm_sync_scalar_static");
  CHECK_FIELDS(f);
  if (ctx->N > SWM_SYNC_STATIC_MAX_N) {
    char m[160];
    std::snprintf(m, sizeof m,
                  "swm_sync_scalar_static: N=%d exceeds the static scratch limit N<=%d "
                  "(swm_sync_scalar has no limit)",
                  ctx->N, SWM_SYNC_STATIC_MAX_N);
    return fail(ctx, SWM_E_INVALID, m);
  }
  double* scratch = nullptr;
  if (int rc = static_sync_scratch(ctx, &scratch)) return rc;
  CK(launch_sync_scalar(ctx->g64, ctx->topo, f->p, scratch, ctx->st), "sync");
  return SWM_OK;
}

// ---------------------------------------------------------------- timing
int swm_timing_enable(swm_ctx* ctx, int on) {
  if (!ctx) return fail(nullptr, SWM_E_INVALID, "null context");
  ctx->timing = on != 0;
  return SWM_OK;
}

int swm_timing_read(swm_ctx* ctx, double* stage_ms, long* stage_launches, double* edge_ms, long* edge_launches) {
  if (!ctx) return fail(nullptr, SWM_E_INVALID, "null context");
  if (int rc_ = sync_check(ctx, ctx->st)) return rc_;
  double ts = 0.0, te = 0.0;
  for (auto& e : ctx->ev_stage) { float ms; CK(cudaEventElapsedTime(&ms, e.first, e.second), "elapsed"); ts += ms; }
  for (auto& e : ctx->ev_edge) { float ms; CK(cudaEventElapsedTime(&ms, e.first, e.second), "elapsed"); te += ms; }
  if (stage_ms) *stage_ms = ts;
  if (stage_launches) *stage_launches = (long)ctx->ev_stage.size();
  if (edge_ms) *edge_ms = te;
  if (edge_launches) *edge_launches = (long)ctx->ev_edge.size();
  for (auto& e : ctx->ev_stage) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
  for (auto& e : ctx->ev_edge) { cudaEventDestroy(e.first); cudaEventDestroy(e.second); }
  ctx->ev_stage.clear();
  ctx->ev_edge.clear();
  return SWM_OK;
}

}  // extern "C"

// ===========================================================================
// Ensembles: independent instances (each with its own N, initial state and
// time step) advanced together.  Every member is a full context (geometry,
// buffers, diagnostics); the ensemble adds one table of instances and tensor
// maps per RK stage, the work units of all members in one list, and one
// CUDA graph of the RK4 step: per stage one persistent stage-kernel launch
// and one edge-kernel launch for all members.
// ===========================================================================
struct swm_ensemble {
  int nmem = 0, order = 42, prec = SWM_FP32_FUSED, device = 0;
  std::vector<swm_ctx*> mem;
  std::vector<swm_state*> state;
  std::vector<double> dt;
  cudaStream_t st = nullptr;
  int boxw = 0, max_n = 0, num_sms = 0, occ = 0, cols = 0;
  bool fixbw = false;   // every member uses its width's widest (compile-time) box
  StageMaps* dmaps = nullptr;        // [4 stages][nmem]
  void* dinst = nullptr;             // InstDev<T> [4 stages][nmem]
  WorkUnit* dunits = nullptr;
  int nunits = 0, cap_units = 0;
  int seg_rows = 0;                  // rows per work unit (0: whole panel height)
  int grid = 0;                      // persistent CTAs (0: one CTA per unit)
  cudaGraphExec_t graph = nullptr;
  std::string err;
};

namespace {

int efail(swm_ensemble* e, int code, const std::string& msg) {
  if (e) e->err = msg; else g_err = msg;
  return code;
}
#define USE_ENS_DEVICE(en)                                                  \
  do {                                                                      \
    cudaError_t e_ = cudaSetDevice((en)->device);                           \
    if (e_ != cudaSuccess)                                                  \
      return efail((en), SWM_E_CUDA, std::string("set device: ") + cudaGetErrorString(e_)); \
  } while (0)
#define ECK(call, where)                                                              \
  do {                                                                                \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
      return efail(ens, e_ == cudaErrorMemoryAllocation ? SWM_E_NOMEM : SWM_E_CUDA,   \
                   std::string(where) + ": " + cudaGetErrorString(e_));               \
  } while (0)
#define EMEM(call)                                                                    \
  do {                                                                                \
    if (int rc_ = (call)) return efail(ens, rc_, mem_err(ens));                        \
  } while (0)

std::string mem_err(swm_ensemble* ens) {
  for (swm_ctx* c : ens->mem)
    if (c && !c->err.empty()) return c->err;
  return g_err;
}

// Work units of every member: `seg_rows` rows per unit (0: one segment per
// strip), largest units first so the persistent CTAs finish together.
int ens_units(swm_ensemble* ens, int seg_rows) {
  std::vector<WorkUnit> all;
  std::string why;
  for (int m = 0; m < ens->nmem; ++m) {
    const swm_ctx* c = ens->mem[m];
    const int nseg = seg_rows > 0 ? std::max(1, (c->n + seg_rows - 1) / seg_rows) : 1;
    std::vector<WorkUnit> u;
    if (!make_units(kTables[sbp_index(c->order)], c->n, ens->cols, 1, u, why, nseg))
      return efail(ens, SWM_E_INVALID, why);
    for (WorkUnit& w : u) { w.inst = (int16_t)m; all.push_back(w); }
  }
  std::stable_sort(all.begin(), all.end(), [](const WorkUnit& a, const WorkUnit& b) {
    return (a.rl1 - a.rl0) * (a.cl1 - a.cl0) > (b.rl1 - b.rl0) * (b.cl1 - b.cl0);
  });
  if ((int)all.size() > ens->cap_units) {
    if (ens->dunits) cudaFree(ens->dunits);
    ens->dunits = nullptr;
    ens->cap_units = 0;
    ECK(cudaMalloc(&ens->dunits, sizeof(WorkUnit) * all.size()), "alloc units");
    ens->cap_units = (int)all.size();
  }
  ECK(cudaMemcpy(ens->dunits, all.data(), sizeof(WorkUnit) * all.size(), cudaMemcpyHostToDevice),
      "copy units");
  ens->nunits = (int)all.size();
  ens->seg_rows = seg_rows;
  return SWM_OK;
}

// Instance and tensor-map tables of the four RK stages (the member time
// steps are in the stage coefficients).
template <class T>
int ens_tables(swm_ensemble* ens) {
  const int M = ens->nmem;
  std::vector<InstDev<T>> inst(4 * M);
  std::vector<StageMaps> maps(4 * M);
  for (int m = 0; m < M; ++m) {
    swm_ctx* c = ens->mem[m];
    swm_state* s = ens->state[m];
    const double dt = ens->dt[m];
    T* v0 = (T*)s->hi;
    T* ya = (T*)c->ya;
    T* yb = (T*)c->yb;
    T* acc = (T*)c->acc;
    for (int i = 0; i < 4; ++i) {
      InstDev<T> I = base_inst<T>(c);
      I.acc = acc;
      switch (i) {   // the stage coefficients of enqueue_rk4 (rk4_mod.f90:20-42)
        case 0: I.in = v0; I.base = v0; I.out = ya; I.c_in = (T)(0.5 * dt); I.c_acc = (T)(dt / 6.0); break;
        case 1: I.in = ya; I.base = v0; I.out = yb; I.c_in = (T)(0.5 * dt); I.c_acc = (T)(dt / 3.0); break;
        case 2: I.in = yb; I.base = v0; I.out = ya; I.c_in = (T)dt; I.c_acc = (T)(dt / 3.0); break;
        default:
          I.in = ya; I.base = v0; I.out = nullptr; I.base_out = v0;
          I.base_lo = s->lo ? (T*)(void*)s->lo : nullptr; I.c_acc = (T)(dt / 6.0);
      }
      if (int rc = make_maps<T>(c, I, MODE_RK1 + i, &maps[i * M + m])) return efail(ens, rc, c->err);
      I.maps = c->shape.tma ? ens->dmaps + i * M + m : nullptr;
      inst[i * M + m] = I;
    }
  }
  ECK(cudaMemcpy(ens->dmaps, maps.data(), sizeof(StageMaps) * maps.size(), cudaMemcpyHostToDevice),
      "copy maps");
  ECK(cudaMemcpy(ens->dinst, inst.data(), sizeof(InstDev<T>) * inst.size(), cudaMemcpyHostToDevice),
      "copy instances");
  return SWM_OK;
}

// Capture one ensemble RK4 step into ens->graph.
template <class T>
int ens_capture(swm_ensemble* ens) {
  if (ens->graph) { cudaGraphExecDestroy(ens->graph); ens->graph = nullptr; }
  const InstDev<T>* I = (const InstDev<T>*)ens->dinst;
  const Topology& tp = ens->mem[0]->topo;
  int* derr = ens->mem[0]->derr;
  cudaGraph_t g;
  ECK(cudaStreamBeginCapture(ens->st, cudaStreamCaptureModeThreadLocal), "begin capture");
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 4 && e == cudaSuccess; ++i) {
    e = launch_stage<T>(ens->order, ens->cols, ens->fixbw, nullptr, InstDev<T>{}, I + i * ens->nmem,
                        ens->dunits, ens->nunits, MODE_RK1 + i, ens->boxw, ens->grid, derr, ens->st);
    if (e == cudaSuccess)
      e = launch_edge<T>(InstDev<T>{}, I + i * ens->nmem, ens->nmem, ens->max_n, tp, MODE_RK1 + i,
                         ens->st);
  }
  cudaError_t ec = cudaStreamEndCapture(ens->st, &g);
  if (e != cudaSuccess) { if (ec == cudaSuccess) cudaGraphDestroy(g); ECK(e, "ensemble stage launch"); }
  ECK(ec, "end capture");
  cudaError_t ei = cudaGraphInstantiate(&ens->graph, g, 0);
  cudaGraphDestroy(g);
  ECK(ei, "graph instantiate");
  return SWM_OK;
}

// Box mode, widest box and occupancy of the ensemble's stage launches: the
// compile-time widest box only when every member's maps use it.
void ens_box(swm_ensemble* ens) {
  int boxw = 0;
  bool fixed = true;
  for (swm_ctx* c : ens->mem) {
    boxw = std::max(boxw, c->shape.boxw);
    fixed = fixed && c->shape.fixbw != 0;
  }
  ens->boxw = boxw;
  ens->fixbw = fixed;
  ens->occ = ens->prec == SWM_FP32_FUSED ? stage_occupancy<float>(ens->order, ens->boxw, ens->cols, fixed)
                                         : stage_occupancy<double>(ens->order, ens->boxw, ens->cols, fixed);
}

// Consumer width of the members' FP32 stage kernel: every member's box and
// the ensemble's widest box and occupancy follow it.
int ens_set_width(swm_ensemble* ens, int cols) {
  for (swm_ctx* c : ens->mem)
    if (c->shape.cols != cols && stage_layout(c, cols, 0, 0) != SWM_OK) return efail(ens, SWM_E_INVALID, c->err);
  ens->cols = cols;
  ens_box(ens);
  return SWM_OK;
}

int ens_rebuild(swm_ensemble* ens, int seg_rows, int grid) {
  if (int rc = ens_units(ens, seg_rows)) return rc;
  ens->grid = grid;
  const bool f32 = ens->prec == SWM_FP32_FUSED;
  if (int rc = f32 ? ens_tables<float>(ens) : ens_tables<double>(ens)) return rc;
  return f32 ? ens_capture<float>(ens) : ens_capture<double>(ens);
}

int ens_check_member(swm_ensemble* ens, int m) {
  if (!ens) return efail(nullptr, SWM_E_INVALID, "null ensemble");
  if (m < 0 || m >= ens->nmem) return efail(ens, SWM_E_INVALID, "member index out of range");
  USE_ENS_DEVICE(ens);
  ECK(cudaStreamSynchronize(ens->st), "sync");
  return SWM_OK;
}

void free_ensemble(swm_ensemble* ens) {
  if (!ens) return;
  cudaSetDevice(ens->device);
  if (ens->st) cudaStreamSynchronize(ens->st);
  if (ens->graph) cudaGraphExecDestroy(ens->graph);
  if (ens->dmaps) cudaFree(ens->dmaps);
  if (ens->dinst) cudaFree(ens->dinst);
  if (ens->dunits) cudaFree(ens->dunits);
  for (size_t m = 0; m < ens->mem.size(); ++m) {
    if (m < ens->state.size() && ens->state[m]) swm_state_free(ens->state[m]);
    swm_ctx_destroy(ens->mem[m]);
  }
  if (ens->st) cudaStreamDestroy(ens->st);
  delete ens;
}

}  // namespace

extern "C" {

int swm_ensemble_create(const swm_config* base, int nmembers, const int* member_N,
                        const double* member_dt, swm_ensemble** out) {
  swm_ensemble* ens = nullptr;
  if (!base || !member_N || !member_dt || !out) return efail(nullptr, SWM_E_INVALID, "null argument");
  if (nmembers < 1 || nmembers > 32767) return efail(nullptr, SWM_E_INVALID, "member count out of range");
  for (int m = 0; m < nmembers; ++m)
    if (!(member_dt[m] > 0.0)) return efail(nullptr, SWM_E_INVALID, "member time steps must be positive");
  ens = new swm_ensemble();
  ens->nmem = nmembers;
  ens->order = base->sbp_order;
  ens->prec = base->precision;
  ens->device = base->device;
  ens->dt.assign(member_dt, member_dt + nmembers);
  auto bail = [&](int rc, const std::string& msg) {
    free_ensemble(ens);
    return efail(nullptr, rc, msg);
  };
  for (int m = 0; m < nmembers; ++m) {
    swm_config c = *base;
    c.N = member_N[m];
    swm_ctx* ctx = nullptr;
    if (int rc = swm_ctx_create(&c, &ctx)) return bail(rc, "member " + std::to_string(m) + ": " + g_err);
    ens->mem.push_back(ctx);
    swm_state* s = nullptr;
    if (int rc = swm_state_create(ctx, &s)) return bail(rc, ctx->err);
    ens->state.push_back(s);
    ens->max_n = std::max(ens->max_n, ctx->n);
    ens->cols = ctx->shape.cols;
    ens->num_sms = ctx->num_sms;
  }
  cudaError_t e = cudaStreamCreateWithFlags(&ens->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&ens->dmaps, sizeof(StageMaps) * 4 * nmembers);
  if (e == cudaSuccess)
    e = cudaMalloc(&ens->dinst, (ens->prec == SWM_FP32_FUSED ? sizeof(InstDev<float>) : sizeof(InstDev<double>)) *
                                    4 * nmembers);
  if (e != cudaSuccess)
    return bail(e == cudaErrorMemoryAllocation ? SWM_E_NOMEM : SWM_E_CUDA,
                std::string("ensemble alloc: ") + cudaGetErrorString(e));
  ens_box(ens);
  // default tile shape: whole-panel strips on persistent CTAs (FP32) or one
  // CTA per unit of 64 rows (FP64); swm_ensemble_tune measures the others
  const bool f32 = ens->prec == SWM_FP32_FUSED;
  if (int rc = ens_rebuild(ens, f32 ? 0 : 64, f32 ? std::max(1, ens->occ) * ens->num_sms : 0))
    return bail(rc, ens->err);
  *out = ens;
  return SWM_OK;
}

void swm_ensemble_destroy(swm_ensemble* ens) { free_ensemble(ens); }

const char* swm_ensemble_last_error(const swm_ensemble* ens) {
  return ens ? ens->err.c_str() : g_err.c_str();
}

int swm_ensemble_size(const swm_ensemble* ens) { return ens ? ens->nmem : 0; }

int swm_ensemble_member(swm_ensemble* ens, int m, swm_ctx** ctx, swm_state** state) {
  if (int rc = ens_check_member(ens, m)) return rc;
  if (ctx) *ctx = ens->mem[m];
  if (state) *state = ens->state[m];
  return SWM_OK;
}

int swm_ensemble_upload(swm_ensemble* ens, int m, const double* h, const double* u, const double* v) {
  if (int rc = ens_check_member(ens, m)) return rc;
  EMEM(swm_state_upload(ens->mem[m], ens->state[m], h, u, v));
  ECK(cudaStreamSynchronize(ens->mem[m]->st), "sync");
  return SWM_OK;
}

int swm_ensemble_download(swm_ensemble* ens, int m, double* h, double* u, double* v) {
  if (int rc = ens_check_member(ens, m)) return rc;
  EMEM(swm_state_download(ens->mem[m], ens->state[m], h, u, v));
  return SWM_OK;
}

int swm_ensemble_diagnostics(swm_ensemble* ens, int m, double out[7]) {
  if (int rc = ens_check_member(ens, m)) return rc;
  EMEM(swm_diagnostics(ens->mem[m], ens->state[m], out));
  return SWM_OK;
}

int swm_ensemble_step(swm_ensemble* ens, int nsteps) {
  TraceRange trace_("swm_ensemble_step");
  if (!ens) return efail(nullptr, SWM_E_INVALID, "null ensemble");
  if (nsteps < 0) return efail(ens, SWM_E_INVALID, "nsteps must be >= 0");
  USE_ENS_DEVICE(ens);
  for (int k = 0; k < nsteps; ++k) ECK(cudaGraphLaunch(ens->graph, ens->st), "graph launch");
  return SWM_OK;
}

int swm_ensemble_synchronize(swm_ensemble* ens) {
  if (!ens) return efail(nullptr, SWM_E_INVALID, "null ensemble");
  USE_ENS_DEVICE(ens);
  EMEM(sync_check(ens->mem[0], ens->st));
  return SWM_OK;
}

void* swm_ensemble_stream(swm_ensemble* ens) { return ens ? (void*)ens->st : nullptr; }

int swm_ensemble_set_shape(swm_ensemble* ens, int seg_rows, int grid) {
  if (!ens) return efail(nullptr, SWM_E_INVALID, "null ensemble");
  if (seg_rows < 0 || grid < 0) return efail(ens, SWM_E_INVALID, "tile shape must be >= 0");
  USE_ENS_DEVICE(ens);
  ECK(cudaStreamSynchronize(ens->st), "sync");
  return ens_rebuild(ens, seg_rows, grid);
}

int swm_ensemble_set_width(swm_ensemble* ens, int cols) {
  if (!ens) return efail(nullptr, SWM_E_INVALID, "null ensemble");
  USE_ENS_DEVICE(ens);
  ECK(cudaStreamSynchronize(ens->st), "sync");
  if (ens->prec != SWM_FP32_FUSED && cols != ens->cols)
    return efail(ens, SWM_E_UNSUPPORTED, "the FP64 stage kernel has a single width");
  const int grid = ens->grid;
  if (int rc = ens_set_width(ens, cols)) return rc;
  // a persistent grid follows the new occupancy
  return ens_rebuild(ens, ens->seg_rows, grid > 0 ? std::max(1, ens->occ) * ens->num_sms : 0);
}

int swm_ensemble_get_width(const swm_ensemble* ens, int* cols) {
  if (!ens || !cols) return efail(nullptr, SWM_E_INVALID, "null argument");
  *cols = ens->cols;
  return SWM_OK;
}

int swm_ensemble_get_shape(const swm_ensemble* ens, int* seg_rows, int* grid, int* nunits) {
  if (!ens) return efail(nullptr, SWM_E_INVALID, "null ensemble");
  if (seg_rows) *seg_rows = ens->seg_rows;
  if (grid) *grid = ens->grid;
  if (nunits) *nunits = ens->nunits;
  return SWM_OK;
}

int swm_ensemble_tune(swm_ensemble* ens, int steps, int* seg_rows_out, int* grid_out,
                      double* ms_per_step_out) {
  TraceRange trace_("swm_ensemble_tune");
  if (!ens) return efail(nullptr, SWM_E_INVALID, "null ensemble");
  if (steps < 1) return efail(ens, SWM_E_INVALID, "steps must be >= 1");
  USE_ENS_DEVICE(ens);
  ECK(cudaStreamSynchronize(ens->st), "sync");
  // the trial steps advance the members: keep their states and restore them
  const int M = ens->nmem;
  std::vector<void*> keep(M, nullptr);
  std::vector<size_t> hib(M), lob(M);
  int rc = SWM_OK;
  for (int m = 0; m < M && rc == SWM_OK; ++m) {
    swm_ctx* c = ens->mem[m];
    hib[m] = (size_t)c->elt * 3 * c->fs;
    lob[m] = ens->state[m]->lo ? sizeof(float) * 3 * c->fs : 0;
    if (cudaMalloc(&keep[m], hib[m] + lob[m]) != cudaSuccess) { rc = efail(ens, SWM_E_NOMEM, "tune: alloc"); break; }
    cudaMemcpyAsync(keep[m], ens->state[m]->hi, hib[m], cudaMemcpyDeviceToDevice, ens->st);
    if (lob[m]) cudaMemcpyAsync((char*)keep[m] + hib[m], ens->state[m]->lo, lob[m], cudaMemcpyDeviceToDevice, ens->st);
  }
  auto restore = [&]() {
    for (int m = 0; m < M; ++m) {
      if (!keep[m]) continue;
      cudaMemcpyAsync(ens->state[m]->hi, keep[m], hib[m], cudaMemcpyDeviceToDevice, ens->st);
      if (lob[m]) cudaMemcpyAsync(ens->state[m]->lo, (char*)keep[m] + hib[m], lob[m], cudaMemcpyDeviceToDevice, ens->st);
    }
  };
  const int segs[] = {0, 192, 128, 96, 64, 48, 32, 24, 16};
  const bool f32 = ens->prec == SWM_FP32_FUSED;
  double best = 1e30;
  int best_seg = ens->seg_rows, best_grid = ens->grid, best_cols = ens->cols;
  cudaEvent_t a = nullptr, b = nullptr;
  if (rc == SWM_OK && (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess))
    rc = efail(ens, SWM_E_CUDA, "tune: events");
  constexpr int kNumWidths = (int)(sizeof(kStageWidths) / sizeof(kStageWidths[0]));
  for (int wi = 0; wi < kNumWidths && rc == SWM_OK; ++wi) {   // consumer widths (FP32 kernel only)
    const int cols = f32 ? kStageWidths[wi] : ens->cols;
    if (!f32 && wi > 0) break;
    if (ens_set_width(ens, cols) != SWM_OK) continue;   // width cannot cover a member
    const int persistent = std::max(1, ens->occ) * ens->num_sms;
    const int grids[] = {persistent, 0};
    for (int si = 0; si < (int)(sizeof(segs) / sizeof(segs[0])) && rc == SWM_OK; ++si) {
      if (segs[si] > 0 && segs[si] >= ens->max_n) continue;
      for (int gi = 0; gi < 2 && rc == SWM_OK; ++gi) {
        if (!f32 && grids[gi] != 0) continue;  // FP64 kernel: one CTA per unit
        if ((rc = ens_rebuild(ens, segs[si], grids[gi]))) break;
        cudaGraphLaunch(ens->graph, ens->st);                          // warm-up
        cudaEventRecord(a, ens->st);
        for (int k = 0; k < steps; ++k) cudaGraphLaunch(ens->graph, ens->st);
        cudaEventRecord(b, ens->st);
        if (cudaEventSynchronize(b) != cudaSuccess) { rc = efail(ens, SWM_E_CUDA, "tune: sync"); break; }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        restore();
        if (ms / steps < best) {
          best = ms / steps; best_seg = segs[si]; best_grid = grids[gi]; best_cols = cols;
        }
      }
    }
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  restore();
  cudaStreamSynchronize(ens->st);
  for (void* p : keep) if (p) cudaFree(p);
  if (rc == SWM_OK) rc = ens_set_width(ens, best_cols);
  if (rc == SWM_OK) rc = ens_rebuild(ens, best_seg, best_grid);
  if (rc == SWM_OK) {
    EMEM(sync_check(ens->mem[0], ens->st));
    if (seg_rows_out) *seg_rows_out = best_seg;
    if (grid_out) *grid_out = best_grid;
    if (ms_per_step_out) *ms_per_step_out = best;
  }
  return rc;
}

}  // extern "C"

// ===========================================================================
// Tangent-linear and adjoint of the FP64 model operator and RK4 step, and
// the binomially checkpointed gradient of a trajectory (no counterpart in the
// reference).  The adjoint is the exact transpose of the tangent-linear
// model of the discrete step in the algebraic inner product of all stored
// nodes (the one swm_dot computes).
// ===========================================================================
namespace {

constexpr int kAdWork = 10, kAdStates = 7;

template <class T = double>
T* adf(swm_ctx* c, int k) { return (T*)c->adw + (long long)k * c->fs; }           // work field
template <class T = double>
T* ads(swm_ctx* c, int s) { return adf<T>(c, kAdWork + 3 * s); }                   // work state

SbpT make_sbpT(const SbpC& s) {
  SbpT t{};
  int maxlast = 0;
  for (int r = 0; r < s.ne; ++r) maxlast = std::max(maxlast, s.last[r]);
  t.ct = std::max(maxlast, s.ne + s.H);
  t.kr = t.ct + s.H;
  t.nin = s.nin;
  t.inshift = s.inshift;
  for (int m = 0; m < s.nin; ++m) t.qin[m] = s.Qin[m];
  // D[r][c] near the left end (closure rows, then interior rows)
  auto D = [&](int r, int c) -> double {
    if (r < s.ne) return c < s.last[r] ? s.Ql[r * MAXNW + c] : 0.0;
    const int m = c - r - s.inshift;
    return (m >= 0 && m < s.nin) ? s.Qin[m] : 0.0;
  };
  for (int c = 0; c < t.ct; ++c)
    for (int r = 0; r < t.kr; ++r) t.t[c * t.kr + r] = D(r, c);
  return t;
}

// tl: the caller needs the tangent-linear model (FP64 contexts only); the
// adjoint runs in either precision
int adjoint_ws(swm_ctx* ctx, bool tl) {
  if (tl && ctx->prec != SWM_FP64_PLAIN)
    return fail(ctx, SWM_E_UNSUPPORTED, "the tangent-linear model needs an FP64 (plain) context");
  if (ctx->adw) return SWM_OK;
  ctx->sbpT = make_sbpT(kTables[sbp_index(ctx->order)]);
  if (ctx->sbpT.ct != adjoint_table_ct(ctx->order))
    return fail(ctx, SWM_E_UNSUPPORTED, "transposed SBP table does not match the adjoint kernels");
  if (ctx->n < 2 * ctx->sbpT.kr) return fail(ctx, SWM_E_INVALID, "grid too small for the adjoint");
  const size_t b = (size_t)ctx->elt * (size_t)(kAdWork + 3 * kAdStates) * ctx->fs;
  CK(cudaMalloc(&ctx->adw, b), "alloc adjoint work");
  CK(cudaMemsetAsync(ctx->adw, 0, b, ctx->st), "memset");
  // two edge buffers: transposed-sync pulls, base-curl edge values
  const size_t eb = (size_t)ctx->elt * 2 * 16 * 6 * ctx->n;
  CK(cudaMalloc(&ctx->adC, eb), "alloc adjoint edge buffers");
  CK(cudaMemsetAsync(ctx->adC, 0, eb, ctx->st), "memset");
  return SWM_OK;
}

int apply_fused64(swm_ctx* ctx, const double* in, double* out) {
  InstDev<double> I = base_inst<double>(ctx);
  I.in = in;
  I.out = out;
  return run_stage<double>(ctx, I, MODE_APPLY);
}

// dk = F'(y) dx
int tl_apply(swm_ctx* ctx, const double* y, const double* dx, double* dk) {
  const long long fs = ctx->fs;
  int rc;
  if ((rc = op_curl(ctx, y + fs, y + 2 * fs, adf(ctx, 9)))) return rc;            // base zeta
  CK(launch_tl_pre(ctx->g64, ctx->m64, ctx->cfg.grav, y, dx, adf(ctx, 0), ctx->st), "tl pre");
  if ((rc = op_grad(ctx, adf(ctx, 0), adf(ctx, 5), adf(ctx, 6)))) return rc;       // dGX, dGY
  if ((rc = op_curl(ctx, dx + fs, dx + 2 * fs, adf(ctx, 7)))) return rc;          // dZ
  if ((rc = op_div(ctx, adf(ctx, 1), adf(ctx, 2), adf(ctx, 8)))) return rc;       // dDIV
  CK(launch_tl_post(ctx->g64, ctx->m64, y, adf(ctx, 9), adf(ctx, 0), adf(ctx, 5), adf(ctx, 6),
                    adf(ctx, 7), adf(ctx, 8), dk, ctx->st),
     "tl post");
  return SWM_OK;
}

// mu_out = F'(y)^T (alpha*lam + beta*mu_in) and acc_out = acc_in + mu_out
// (mu_in, mu_out, acc_in/acc_out nullable; outputs may alias inputs)
template <class T>
int ad_stage(swm_ctx* ctx, const T* y, const T* lam, const T* mu_in, double alpha, double beta,
             T* mu_out, const T* acc_in, T* acc_out) {
  T* C = (T*)ctx->adC;
  T* Zedge = C + 16LL * 6 * ctx->n;   // edge values of the base curl
  const T* m = metric_of<T>(ctx);
  CK(launch_zeta_pre<T>(ctx->g, ctx->order, m, y, adf<T>(ctx, 9), Zedge, ctx->st), "ad curl");
  CK(launch_ad_pre<T>(ctx->g, ctx->topo, ctx->qw, m, y, adf<T>(ctx, 9), Zedge, lam, mu_in, (T)alpha,
                      (T)beta, adf<T>(ctx, 0), C, ctx->st),
     "ad pre");
  CK(launch_adsync_gather<T>(ctx->g, ctx->topo, m, C, adf<T>(ctx, 0), ctx->st), "ad syncs");
  CK(launch_ad_main<T>(ctx->g, ctx->order, ctx->sbpT, m, (T)ctx->ghs, (T)ctx->cfg.grav, y,
                       adf<T>(ctx, 0), mu_out, acc_in, acc_out, ctx->st),
     "ad main");
  return SWM_OK;
}

// out = F'(y)^T lk
template <class T>
int ad_apply(swm_ctx* ctx, const T* y, const T* lk, T* out) {
  return ad_stage<T>(ctx, y, lk, nullptr, 1.0, 0.0, out, nullptr, nullptr);
}

// out = base + c F(in) by the fused stage kernel (RK stage mode; scratch
// takes its running-sum output)
template <class T>
int stage_state(swm_ctx* ctx, const T* in, const T* base, double c, T* out, T* scratch) {
  InstDev<T> I = base_inst<T>(ctx);
  I.in = in;
  I.base = base;
  I.out = out;
  I.acc = scratch;
  I.c_in = (T)c;
  I.c_acc = T(0);
  return run_stage<T>(ctx, I, MODE_RK1);
}

// dx <- Phi'(x) dx for one RK4 step Phi (rk4_mod.f90:20-42)
int rk4_tl(swm_ctx* ctx, const double* x, double* dx, double dt) {
  const long long c = 3 * ctx->fs;
  double *Y = ads(ctx, 0), *K = ads(ctx, 1), *DK = ads(ctx, 2), *DY = ads(ctx, 3), *ACC = ads(ctx, 4);
  const cudaStream_t st = ctx->st;
  int rc;
  if ((rc = tl_apply(ctx, x, dx, DK))) return rc;
  CK(launch_axpby(c, 1.0, dx, dt / 6.0, DK, ACC, st), "axpby");
  CK(launch_axpby(c, 1.0, dx, 0.5 * dt, DK, DY, st), "axpby");
  if ((rc = apply_fused64(ctx, x, K))) return rc;
  CK(launch_axpby(c, 1.0, x, 0.5 * dt, K, Y, st), "axpby");
  if ((rc = tl_apply(ctx, Y, DY, DK))) return rc;
  CK(launch_axpby(c, 1.0, ACC, dt / 3.0, DK, ACC, st), "axpby");
  CK(launch_axpby(c, 1.0, dx, 0.5 * dt, DK, DY, st), "axpby");
  if ((rc = apply_fused64(ctx, Y, K))) return rc;
  CK(launch_axpby(c, 1.0, x, 0.5 * dt, K, Y, st), "axpby");
  if ((rc = tl_apply(ctx, Y, DY, DK))) return rc;
  CK(launch_axpby(c, 1.0, ACC, dt / 3.0, DK, ACC, st), "axpby");
  CK(launch_axpby(c, 1.0, dx, dt, DK, DY, st), "axpby");
  if ((rc = apply_fused64(ctx, Y, K))) return rc;
  CK(launch_axpby(c, 1.0, x, dt, K, Y, st), "axpby");
  if ((rc = tl_apply(ctx, Y, DY, DK))) return rc;
  CK(launch_axpby(c, 1.0, ACC, dt / 6.0, DK, dx, st), "axpby");
  return SWM_OK;
}

// lx <- Phi'(x)^T lx: recompute the stage states, then run the stages back
// (the RK combinations are folded into the adjoint kernels)
template <class T>
int rk4_ad(swm_ctx* ctx, const T* x, T* lx, double dt) {
  T *Y2 = ads<T>(ctx, 0), *Y3 = ads<T>(ctx, 1), *Y4 = ads<T>(ctx, 2), *K = ads<T>(ctx, 3);
  T *MU = ads<T>(ctx, 5), *ACC = ads<T>(ctx, 6);
  int rc;
  if ((rc = stage_state<T>(ctx, x, x, 0.5 * dt, Y2, K))) return rc;
  if ((rc = stage_state<T>(ctx, Y2, x, 0.5 * dt, Y3, K))) return rc;
  if ((rc = stage_state<T>(ctx, Y3, x, dt, Y4, K))) return rc;
  if ((rc = ad_stage<T>(ctx, Y4, lx, nullptr, dt / 6.0, 0.0, MU, lx, ACC))) return rc;     // ACC = l + mu4
  if ((rc = ad_stage<T>(ctx, Y3, lx, MU, dt / 3.0, dt, MU, ACC, ACC))) return rc;          // ACC += mu3
  if ((rc = ad_stage<T>(ctx, Y2, lx, MU, dt / 3.0, 0.5 * dt, MU, ACC, ACC))) return rc;    // ACC += mu2
  return ad_stage<T>(ctx, x, lx, MU, dt / 6.0, 0.5 * dt, nullptr, ACC, lx);                // l = ACC + mu1
}

// rk4_ad through a CUDA graph captured for the last (x, lx, dt)
int rk4_ad_graph(swm_ctx* ctx, const void* x, void* lx, double dt) {
  if (!(ctx->ad_graph && ctx->ad_key[0] == x && ctx->ad_key[1] == lx && ctx->ad_dt == dt)) {
    if (ctx->ad_graph) { cudaGraphExecDestroy(ctx->ad_graph); ctx->ad_graph = nullptr; }
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal), "begin capture");
    const int rc = ctx->prec == SWM_FP32_FUSED ? rk4_ad<float>(ctx, (const float*)x, (float*)lx, dt)
                                               : rk4_ad<double>(ctx, (const double*)x, (double*)lx, dt);
    const cudaError_t ec = cudaStreamEndCapture(ctx->st, &g);
    if (rc) { if (ec == cudaSuccess) cudaGraphDestroy(g); return rc; }
    CK(ec, "end capture");
    const cudaError_t ei = cudaGraphInstantiate(&ctx->ad_graph, g, 0);
    cudaGraphDestroy(g);
    CK(ei, "graph instantiate");
    ctx->ad_key[0] = x; ctx->ad_key[1] = lx; ctx->ad_dt = dt;
  }
  CK(cudaGraphLaunch(ctx->ad_graph, ctx->st), "graph launch");
  return SWM_OK;
}

int check_tl_args(swm_ctx* ctx, const swm_state* a, const swm_state* b, const swm_state* c,
                  bool tl) {
  if (int rc = check_state(ctx, a)) return rc;
  if (int rc = check_state(ctx, b)) return rc;
  if (c && check_state(ctx, c)) return SWM_E_INVALID;
  if (a == b || (c && (c == a || c == b)))
    return fail(ctx, SWM_E_INVALID, "tangent-linear / adjoint calls need distinct states");
  USE_DEVICE(ctx);
  return adjoint_ws(ctx, tl);
}

// FP32 cotangents live in the high part of the state pair: clear the low part
int clear_lo(swm_ctx* ctx, swm_state* s) {
  if (s->lo) CK(cudaMemsetAsync(s->lo, 0, sizeof(float) * 3 * ctx->fs, ctx->st), "memset");
  return SWM_OK;
}

}  // namespace

// Binomial checkpointing (Griewank's "revolve" recursion) over nsteps RK4
// steps with nsnap stored states, the initial state included.  The plan is a
// list of actions on one working state: restore it from a snapshot, advance
// it k steps, store it in a snapshot, or run the adjoint step at step n (the
// working state then holds x_n).
struct swm_adjoint {
  enum Kind { RESTORE, ADVANCE, STORE, ADJ };
  struct Act { int kind, arg; };
  swm_ctx* ctx = nullptr;
  int nsteps = 0, nsnap = 0;
  double dt = 0.0;
  std::vector<swm_state*> slot;
  swm_state* cur = nullptr;
  swm_state* lam = nullptr;
  std::vector<Act> plan;
  size_t first_adj = 0;
  bool ready = false;          // forward run done, backward sweep pending
  long fwd_steps = 0, adj_steps = 0;
};

namespace {

long long beta(int c, int r) {   // C(c + r, c), saturating
  long double v = 1.0L;
  for (int k = 1; k <= c; ++k) { v = v * (r + k) / k; if (v > 4e18L) return (long long)4e18; }
  return (long long)(v + 0.5L);
}

void plan_reverse(std::vector<swm_adjoint::Act>& acts, int a, int b, int sa, std::vector<int>& freeslots) {
  using A = swm_adjoint;
  if (b - a == 1) { acts.push_back({A::RESTORE, sa}); acts.push_back({A::ADJ, a}); return; }
  if (freeslots.empty()) {
    for (int k = b - 1; k >= a; --k) {
      acts.push_back({A::RESTORE, sa});
      if (k > a) acts.push_back({A::ADVANCE, k - a});
      acts.push_back({A::ADJ, k});
    }
    return;
  }
  const int c = (int)freeslots.size() + 1, l = b - a;
  int r = 1;
  while (beta(c, r) < l) ++r;
  const long long right = std::min<long long>(l - 1, beta(c - 1, r));
  const int m = b - (int)right;
  acts.push_back({A::RESTORE, sa});
  acts.push_back({A::ADVANCE, m - a});
  const int sm = freeslots.back();
  freeslots.pop_back();
  acts.push_back({A::STORE, sm});
  plan_reverse(acts, m, b, sm, freeslots);
  freeslots.push_back(sm);
  plan_reverse(acts, a, m, sa, freeslots);
}

int copy_state(swm_ctx* ctx, swm_state* dst, const swm_state* src) {
  CK(cudaMemcpyAsync(dst->hi, src->hi, (size_t)ctx->elt * 3 * ctx->fs, cudaMemcpyDeviceToDevice, ctx->st),
     "copy");
  if (dst->lo && src->lo)
    CK(cudaMemcpyAsync(dst->lo, src->lo, sizeof(float) * 3 * ctx->fs, cudaMemcpyDeviceToDevice, ctx->st),
       "copy");
  return SWM_OK;
}

int run_action(swm_adjoint* adj, const swm_adjoint::Act& a) {
  swm_ctx* ctx = adj->ctx;
  switch (a.kind) {
    case swm_adjoint::RESTORE: return copy_state(ctx, adj->cur, adj->slot[a.arg]);
    case swm_adjoint::STORE: return copy_state(ctx, adj->slot[a.arg], adj->cur);
    case swm_adjoint::ADVANCE:
      adj->fwd_steps += a.arg;
      return swm_rk4_step(ctx, adj->cur, adj->dt, a.arg);
    default:
      adj->adj_steps += 1;
      return rk4_ad_graph(ctx, adj->cur->hi, adj->lam->hi, adj->dt);
  }
}

void free_adjoint(swm_adjoint* adj) {
  if (!adj) return;
  for (swm_state* s : adj->slot) swm_state_free(s);
  swm_state_free(adj->cur);
  swm_state_free(adj->lam);
  delete adj;
}

}  // namespace

extern "C" {

int swm_apply_tl(swm_ctx* ctx, const swm_state* y, const swm_state* dx, swm_state* dk) {
  AH_ONLY(ctx, "swm_apply_tl");
  TraceRange trace_("swm_apply_tl");
  if (int rc = check_tl_args(ctx, y, dx, dk, true)) return rc;
  return tl_apply(ctx, (const double*)y->hi, (const double*)dx->hi, (double*)dk->hi);
}

int swm_apply_ad(swm_ctx* ctx, const swm_state* y, const swm_state* lk, swm_state* lx) {
  AH_ONLY(ctx, "swm_apply_ad");
  TraceRange trace_("swm_apply_ad");
  if (int rc = check_tl_args(ctx, y, lk, lx, false)) return rc;
  if (ctx->prec == SWM_FP32_FUSED) {
    if (int rc = ad_apply<float>(ctx, (const float*)y->hi, (const float*)lk->hi, (float*)lx->hi)) return rc;
    return clear_lo(ctx, lx);
  }
  return ad_apply<double>(ctx, (const double*)y->hi, (const double*)lk->hi, (double*)lx->hi);
}

int swm_rk4_tl(swm_ctx* ctx, const swm_state* x, swm_state* dx, double dt) {
  AH_ONLY(ctx, "swm_rk4_tl");
  TraceRange trace_("swm_rk4_tl");
  if (int rc = check_tl_args(ctx, x, dx, nullptr, true)) return rc;
  return rk4_tl(ctx, (const double*)x->hi, (double*)dx->hi, dt);
}

int swm_rk4_ad(swm_ctx* ctx, const swm_state* x, swm_state* lx, double dt) {
  AH_ONLY(ctx, "swm_rk4_ad");
  TraceRange trace_("swm_rk4_ad");
  if (int rc = check_tl_args(ctx, x, lx, nullptr, false)) return rc;
  if (int rc = rk4_ad_graph(ctx, x->hi, lx->hi, dt)) return rc;
  return clear_lo(ctx, lx);
}

int swm_adjoint_create(swm_ctx* ctx, int nsteps, int nsnap, double dt, swm_adjoint** out) {
  AH_ONLY(ctx, "swm_adjoint_create");
  if (!ctx || !out) return fail(ctx, SWM_E_INVALID, "null argument");
  if (nsteps < 1 || nsnap < 1 || !(dt > 0.0))
    return fail(ctx, SWM_E_INVALID, "need nsteps >= 1, nsnap >= 1 and dt > 0");
  USE_DEVICE(ctx);
  if (int rc = adjoint_ws(ctx, false)) return rc;
  swm_adjoint* adj = new swm_adjoint();
  adj->ctx = ctx; adj->nsteps = nsteps; adj->nsnap = std::min(nsnap, nsteps); adj->dt = dt;
  for (int k = 0; k < adj->nsnap; ++k) {
    swm_state* s = nullptr;
    if (int rc = swm_state_create(ctx, &s)) { free_adjoint(adj); return rc; }
    adj->slot.push_back(s);
  }
  if (int rc = swm_state_create(ctx, &adj->cur)) { free_adjoint(adj); return rc; }
  if (int rc = swm_state_create(ctx, &adj->lam)) { free_adjoint(adj); return rc; }
  std::vector<int> freeslots;
  for (int k = adj->nsnap - 1; k >= 1; --k) freeslots.push_back(k);
  plan_reverse(adj->plan, 0, nsteps, 0, freeslots);
  for (size_t k = 0; k < adj->plan.size(); ++k)
    if (adj->plan[k].kind == swm_adjoint::ADJ) { adj->first_adj = k; break; }
  *out = adj;
  return SWM_OK;
}

void swm_adjoint_destroy(swm_adjoint* adj) {
  if (adj && adj->ctx) cudaSetDevice(adj->ctx->cfg.device);
  free_adjoint(adj);
}

int swm_adjoint_forward(swm_adjoint* adj, const swm_state* x0, swm_state* xT) {
  TraceRange trace_("swm_adjoint_forward");
  if (!adj) return fail(nullptr, SWM_E_INVALID, "null adjoint");
  swm_ctx* ctx = adj->ctx;
  if (int rc = check_state(ctx, x0)) return rc;
  if (int rc = check_state(ctx, xT)) return rc;
  USE_DEVICE(ctx);
  adj->fwd_steps = adj->adj_steps = 0;
  if (int rc = copy_state(ctx, adj->slot[0], x0)) return rc;
  for (size_t k = 0; k < adj->first_adj; ++k)
    if (int rc = run_action(adj, adj->plan[k])) return rc;
  // the working state holds x_{T-1}: one more step gives x_T
  if (int rc = copy_state(ctx, xT, adj->cur)) return rc;
  if (int rc = swm_rk4_step(ctx, xT, adj->dt, 1)) return rc;
  adj->fwd_steps += 1;
  adj->ready = true;
  return SWM_OK;
}

int swm_adjoint_backward(swm_adjoint* adj, swm_state* lambda) {
  TraceRange trace_("swm_adjoint_backward");
  if (!adj) return fail(nullptr, SWM_E_INVALID, "null adjoint");
  swm_ctx* ctx = adj->ctx;
  if (int rc = check_state(ctx, lambda)) return rc;
  if (!adj->ready) return fail(ctx, SWM_E_INVALID, "swm_adjoint_backward needs a forward run first");
  USE_DEVICE(ctx);
  if (int rc = copy_state(ctx, adj->lam, lambda)) return rc;
  for (size_t k = adj->first_adj; k < adj->plan.size(); ++k)
    if (int rc = run_action(adj, adj->plan[k])) return rc;
  if (int rc = copy_state(ctx, lambda, adj->lam)) return rc;
  if (int rc = clear_lo(ctx, lambda)) return rc;
  adj->ready = false;
  return sync_check(ctx, ctx->st);
}

int swm_adjoint_counts(const swm_adjoint* adj, long* forward_steps, long* adjoint_steps,
                       long* planned_forward_steps) {
  if (!adj) return fail(nullptr, SWM_E_INVALID, "null adjoint");
  if (forward_steps) *forward_steps = adj->fwd_steps;
  if (adjoint_steps) *adjoint_steps = adj->adj_steps;
  if (planned_forward_steps) {
    long p = 1;   // the extra step to x_T
    for (const auto& a : adj->plan) if (a.kind == swm_adjoint::ADVANCE) p += a.arg;
    *planned_forward_steps = p;
  }
  return SWM_OK;
}

int swm_state_upload_device(swm_ctx* ctx, swm_state* s, const double* h, const double* u,
                            const double* v) {
  AH_ONLY(ctx, "swm_state_upload_device");
  TraceRange trace_("swm_state_upload_device");
  if (int rc = check_state(ctx, s)) return rc;
  if (!h || !u || !v) return fail(ctx, SWM_E_INVALID, "null device array");
  USE_DEVICE(ctx);
  const double* src[3] = {h, u, v};
  return put_packed(ctx, s, src, cudaMemcpyDeviceToDevice);
}

int swm_state_download_device(swm_ctx* ctx, const swm_state* s, double* h, double* u, double* v) {
  AH_ONLY(ctx, "swm_state_download_device");
  TraceRange trace_("swm_state_download_device");
  if (int rc = check_state(ctx, s)) return rc;
  if (!h || !u || !v) return fail(ctx, SWM_E_INVALID, "null device array");
  USE_DEVICE(ctx);
  double* dst[3] = {h, u, v};
  return get_packed(ctx, s, dst, cudaMemcpyDeviceToDevice);
}

int swm_quadrature_weights(swm_ctx* ctx, double* w_host) {
  AH_ONLY(ctx, "swm_quadrature_weights");
  if (!ctx || !w_host) return fail(ctx, SWM_E_INVALID, "null argument");
  USE_DEVICE(ctx);
  const int n = ctx->n;
  std::vector<double> A(n), J((size_t)6 * n * n);
  CK(cudaMemcpy(A.data(), ctx->Aw, sizeof(double) * n, cudaMemcpyDeviceToHost), "copy");
  CK(cudaMemcpy2D(J.data(), sizeof(double) * n, ctx->m64 + MJ * ctx->fs, sizeof(double) * ctx->P,
                  sizeof(double) * n, (size_t)6 * n, cudaMemcpyDeviceToHost),
     "copy");
  const double hx2 = ctx->hx * ctx->hx;
  for (int p = 0; p < 6; ++p)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const size_t k = ((size_t)p * n + j) * n + i;
        w_host[k] = J[k] * hx2 * A[i] * A[j];
      }
  return SWM_OK;
}

}  // extern "C"

// ===========================================================================
// Lat-lon and paneled output (regridders/, outputer/)
// ===========================================================================
namespace {

int check_latlon(swm_ctx* ctx, const swm_latlon* r) {
  if (!ctx) return fail(nullptr, SWM_E_INVALID, "null context");
  if (!r || r->ctx != ctx || !r->base) return fail(ctx, SWM_E_INVALID, "latlon interpolator not of this context");
  return SWM_OK;
}

LatLonDev latlon_dev(const swm_latlon* r) {
  return LatLonDev{r->nlon, r->nlat, r->w, r->base, r->wx, r->wy, r->rot};
}

// Regrid the scalar h (component 0) or the vector (u, v) (components 1, 2)
// of a state into the interpolator's output planes.
int latlon_state(swm_ctx* ctx, swm_latlon* r, const swm_state* s, bool vector, bool f32) {
  const LatLonDev L = latlon_dev(r);
  const long long fs = ctx->fs;
  const int nf = vector ? 2 : 1;
  const long long c0 = vector ? 1 : 0;
  double* out = f32 ? nullptr : r->out;
  float* out32 = f32 ? r->out32 : nullptr;
  if (ctx->prec == SWM_FP64_PLAIN) {
    const double* x = (const double*)s->hi;
    CK(launch_latlon<double>(ctx->g64, L, nf, x + c0 * fs, x + (c0 + 1) * fs, nullptr, nullptr, out, out32,
                             ctx->st),
       "latlon");
  } else {
    const float* x = (const float*)s->hi;
    CK(launch_latlon<float>(ctx->g64, L, nf, x + c0 * fs, x + (c0 + 1) * fs, s->lo + c0 * fs,
                            s->lo + (c0 + 1) * fs, out, out32, ctx->st),
       "latlon");
  }
  return SWM_OK;
}

// Write `count` FP32 values as record rec_num (1-based) of a direct-access
// file of records of `count` values (the outputers' open(access="direct",
// recl=count) with 4-byte record units).
int write_record(swm_ctx* ctx, const char* path, int rec_num, const float* data, size_t count) {
  if (!path || !*path) return SWM_OK;
  if (rec_num < 1) return fail(ctx, SWM_E_INVALID, "record numbers start at 1");
  FILE* fp = std::fopen(path, "r+b");
  if (!fp) fp = std::fopen(path, "w+b");
  if (!fp) return fail(ctx, SWM_E_IO, std::string("cannot open ") + path);
  const long long off = (long long)(rec_num - 1) * (long long)count * 4;
  bool ok = fseeko(fp, (off_t)off, SEEK_SET) == 0 && std::fwrite(data, 4, count, fp) == count;
  ok = (std::fclose(fp) == 0) && ok;
  if (!ok) return fail(ctx, SWM_E_IO, std::string("cannot write ") + path);
  return SWM_OK;
}

}  // namespace

extern "C" {

int swm_latlon_create(swm_ctx* ctx, int nlon, int nlat, const char* interp_type,
                      const char* components_type, swm_latlon** out) {
  AH_ONLY(ctx, "swm_latlon_create");
  if (!ctx || !out) return fail(ctx, SWM_E_INVALID, "null argument");
  *out = nullptr;
  int w = 0, contra = 0;
  const char* it = interp_type ? interp_type : "cubic";
  if (!std::strcmp(it, "linear")) w = 2;
  else if (!std::strcmp(it, "cubic")) w = 4;
  else return fail(ctx, SWM_E_UNSUPPORTED, std::string("unknown interpolation type: ") + it);
  const char* ct = components_type ? components_type : "covariant";
  if (!std::strcmp(ct, "covariant")) contra = 0;
  else if (!std::strcmp(ct, "contravariant")) contra = 1;
  else return fail(ctx, SWM_E_UNSUPPORTED, std::string("unknown vector components type: ") + ct);
  if (nlon < 1 || nlat < 2 || (long long)nlon * nlat > (1LL << 30))
    return fail(ctx, SWM_E_INVALID, "bad lat-lon grid size");
  LatLonHost h;
  if (latlon_setup(ctx->N, nlon, nlat, w, contra, ctx->g64, h))
    return fail(ctx, SWM_E_INVALID, "lat-lon set-up failed");
  USE_DEVICE(ctx);
  swm_latlon* r = new swm_latlon{ctx, nlon, nlat, w, contra, nullptr, nullptr, nullptr, nullptr,
                                 nullptr, nullptr, nullptr, nullptr};
  const size_t np = (size_t)nlon * nlat;
  cudaError_t e = cudaMalloc(&r->base, sizeof(long long) * np);
  if (e == cudaSuccess) e = cudaMalloc(&r->wx, sizeof(double) * 4 * np);
  if (e == cudaSuccess) e = cudaMalloc(&r->wy, sizeof(double) * 4 * np);
  if (e == cudaSuccess) e = cudaMalloc(&r->rot, sizeof(double) * 4 * np);
  if (e == cudaSuccess) e = cudaMalloc(&r->out, sizeof(double) * 2 * np);
  if (e == cudaSuccess) e = cudaMalloc(&r->out32, sizeof(float) * 2 * np);
  if (e == cudaSuccess) e = cudaMallocHost(&r->hout, sizeof(double) * 2 * np);
  if (e == cudaSuccess) e = cudaMallocHost(&r->hout32, sizeof(float) * 2 * np);
  if (e == cudaSuccess) e = cudaMemcpy(r->base, h.base.data(), sizeof(long long) * np, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(r->wx, h.wx.data(), sizeof(double) * 4 * np, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(r->wy, h.wy.data(), sizeof(double) * 4 * np, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(r->rot, h.rot.data(), sizeof(double) * 4 * np, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    release_latlon(r);
    delete r;
    return fail(ctx, e == cudaErrorMemoryAllocation ? SWM_E_NOMEM : SWM_E_CUDA,
                std::string("latlon: ") + cudaGetErrorString(e));
  }
  ctx->latlons.insert(r);
  *out = r;
  return SWM_OK;
}

void swm_latlon_destroy(swm_latlon* r) {
  if (!r) return;
  if (r->ctx) {
    cudaSetDevice(r->ctx->cfg.device);
    release_latlon(r);
    r->ctx->latlons.erase(r);
  }
  delete r;
}

int swm_latlon_regrid_field(swm_ctx* ctx, swm_latlon* r, const swm_field* f, double* out) {
  if (int rc = check_latlon(ctx, r)) return rc;
  if (int rc = check_field(ctx, f)) return rc;
  if (!out) return fail(ctx, SWM_E_INVALID, "null output");
  USE_DEVICE(ctx);
  const size_t np = (size_t)r->nlon * r->nlat;
  CK(launch_latlon<double>(ctx->g64, latlon_dev(r), 1, f->p, nullptr, nullptr, nullptr, r->out, nullptr,
                           ctx->st),
     "latlon");
  CK(cudaMemcpyAsync(r->hout, r->out, sizeof(double) * np, cudaMemcpyDeviceToHost, ctx->st), "copy");
  if (int rc = sync_check(ctx, ctx->st)) return rc;
  std::memcpy(out, r->hout, sizeof(double) * np);
  return SWM_OK;
}

int swm_latlon_regrid_vector(swm_ctx* ctx, swm_latlon* r, const swm_field* u, const swm_field* v,
                             double* uo, double* vo) {
  if (int rc = check_latlon(ctx, r)) return rc;
  if (int rc = check_field(ctx, u)) return rc;
  if (int rc = check_field(ctx, v)) return rc;
  if (!uo || !vo) return fail(ctx, SWM_E_INVALID, "null output");
  USE_DEVICE(ctx);
  const size_t np = (size_t)r->nlon * r->nlat;
  CK(launch_latlon<double>(ctx->g64, latlon_dev(r), 2, u->p, v->p, nullptr, nullptr, r->out, nullptr,
                           ctx->st),
     "latlon");
  CK(cudaMemcpyAsync(r->hout, r->out, sizeof(double) * 2 * np, cudaMemcpyDeviceToHost, ctx->st), "copy");
  if (int rc = sync_check(ctx, ctx->st)) return rc;
  std::memcpy(uo, r->hout, sizeof(double) * np);
  std::memcpy(vo, r->hout + np, sizeof(double) * np);
  return SWM_OK;
}

int swm_latlon_regrid_state(swm_ctx* ctx, swm_latlon* r, const swm_state* s, double* h, double* u,
                            double* v) {
  TraceRange trace_("swm_latlon_regrid_state");
  if (int rc = check_latlon(ctx, r)) return rc;
  if (int rc = check_state(ctx, s)) return rc;
  USE_DEVICE(ctx);
  const size_t np = (size_t)r->nlon * r->nlat;
  if (h) {
    if (int rc = latlon_state(ctx, r, s, false, false)) return rc;
    CK(cudaMemcpyAsync(r->hout, r->out, sizeof(double) * np, cudaMemcpyDeviceToHost, ctx->st), "copy");
    if (int rc = sync_check(ctx, ctx->st)) return rc;
    std::memcpy(h, r->hout, sizeof(double) * np);
  }
  if (u || v) {
    if (int rc = latlon_state(ctx, r, s, true, false)) return rc;
    CK(cudaMemcpyAsync(r->hout, r->out, sizeof(double) * 2 * np, cudaMemcpyDeviceToHost, ctx->st), "copy");
    if (int rc = sync_check(ctx, ctx->st)) return rc;
    if (u) std::memcpy(u, r->hout, sizeof(double) * np);
    if (v) std::memcpy(v, r->hout + np, sizeof(double) * np);
  }
  return SWM_OK;
}

int swm_latlon_write(swm_ctx* ctx, swm_latlon* r, const swm_state* s, const char* h_file,
                     const char* u_file, const char* v_file, int rec_num) {
  TraceRange trace_("swm_latlon_write");
  if (int rc = check_latlon(ctx, r)) return rc;
  if (int rc = check_state(ctx, s)) return rc;
  if (rec_num < 1) return fail(ctx, SWM_E_INVALID, "record numbers start at 1");
  USE_DEVICE(ctx);
  const size_t np = (size_t)r->nlon * r->nlat;
  if (h_file && *h_file) {
    if (int rc = latlon_state(ctx, r, s, false, true)) return rc;
    CK(cudaMemcpyAsync(r->hout32, r->out32, sizeof(float) * np, cudaMemcpyDeviceToHost, ctx->st), "copy");
    if (int rc = sync_check(ctx, ctx->st)) return rc;
    if (int rc = write_record(ctx, h_file, rec_num, r->hout32, np)) return rc;
  }
  if ((u_file && *u_file) || (v_file && *v_file)) {
    if (int rc = latlon_state(ctx, r, s, true, true)) return rc;
    CK(cudaMemcpyAsync(r->hout32, r->out32, sizeof(float) * 2 * np, cudaMemcpyDeviceToHost, ctx->st), "copy");
    if (int rc = sync_check(ctx, ctx->st)) return rc;
    if (int rc = write_record(ctx, u_file, rec_num, r->hout32, np)) return rc;
    if (int rc = write_record(ctx, v_file, rec_num, r->hout32 + np, np)) return rc;
  }
  return SWM_OK;
}

int swm_paneled_write(swm_ctx* ctx, const swm_state* s, int component, const char* file, int rec_num) {
  AH_ONLY(ctx, "swm_paneled_write");
  TraceRange trace_("swm_paneled_write");
  if (int rc = check_state(ctx, s)) return rc;
  if (component < 0 || component > 2 || !file) return fail(ctx, SWM_E_INVALID, "bad component or file");
  if (rec_num < 1) return fail(ctx, SWM_E_INVALID, "record numbers start at 1");
  USE_DEVICE(ctx);
  const size_t np = (size_t)6 * ctx->n * ctx->n;
  PackedFields pf{{tmpf(ctx, 11), nullptr, nullptr}};
  const long long off = (long long)component * ctx->fs;
  if (ctx->prec == SWM_FP64_PLAIN)
    CK(launch_pack_state(ctx->g64, 1, (const double*)s->hi + off, nullptr, pf, ctx->st), "pack");
  else
    CK(launch_pack_state(ctx->g64, 1, (const float*)s->hi + off, s->lo + off, pf, ctx->st), "pack");
  std::vector<double> d(np);
  CK(cudaMemcpyAsync(d.data(), pf.f[0], sizeof(double) * np, cudaMemcpyDeviceToHost, ctx->st), "copy");
  if (int rc = sync_check(ctx, ctx->st)) return rc;
  std::vector<float> f(np);
  for (size_t k = 0; k < np; ++k) f[k] = (float)d[k];
  return write_record(ctx, file, rec_num, f.data(), np);
}

// ------------------------------------------------------------ tuning
int swm_tune_stage(swm_ctx* ctx, const swm_state* s, double dt, int steps, int* cols_out,
                   int* seg_rows_out, int* grid_out, int* box_out, double* ms_out) {
  AH_ONLY(ctx, "swm_tune_stage");
  TraceRange trace_("swm_tune_stage");
  if (int rc = check_state(ctx, s)) return rc;
  if (steps < 1 || !std::isfinite(dt)) return fail(ctx, SWM_E_INVALID, "bad dt or steps");
  USE_DEVICE(ctx);
  auto report = [&](int c, int r, int g, int b, double ms) {
    if (cols_out) *cols_out = c;
    if (seg_rows_out) *seg_rows_out = r;
    if (grid_out) *grid_out = g;
    if (box_out) *box_out = b;
    if (ms_out) *ms_out = ms;
  };
  if (!ctx->shape.tma) {   // the FP64 kernel has one shape
    report(ctx->shape.cols, ctx->seg_rows, ctx->stage_grid, SWM_BOX_STRIP, 0.0);
    return SWM_OK;
  }
  swm_state* x = nullptr;
  if (int rc = swm_state_create_similar(ctx, s, &x)) return rc;
  cudaEvent_t a = nullptr, b = nullptr;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  const int c0 = ctx->shape.cols, r0 = ctx->seg_rows, g0 = ctx->stage_grid;
  const int x0 = ctx->shape.fixbw ? SWM_BOX_WIDEST : SWM_BOX_STRIP;
  int bc = c0, br = r0, bg = g0, bx = x0, rc = SWM_OK;
  double best_ms = 1e30;
  auto trial = [&](int cols, int seg, int grid, int box) {
    if (stage_layout(ctx, cols, seg, grid, box) != SWM_OK) return;   // shape cannot cover the grid
    std::vector<float> ms;
    for (int k = -2; k < steps && rc == SWM_OK; ++k) {   // two untimed steps capture the graph
      rc = copy_state(ctx, x, s);
      if (rc == SWM_OK && cudaEventRecord(a, ctx->st) != cudaSuccess) rc = cuda_fail(ctx, cudaGetLastError(), "event");
      if (rc == SWM_OK) rc = swm_rk4_step(ctx, x, dt, 1);
      if (rc == SWM_OK && cudaEventRecord(b, ctx->st) != cudaSuccess) rc = cuda_fail(ctx, cudaGetLastError(), "event");
      if (rc == SWM_OK) rc = sync_check(ctx, ctx->st);
      float t = 0.0f;
      if (rc == SWM_OK && k >= 0 && cudaEventElapsedTime(&t, a, b) == cudaSuccess) ms.push_back(t);
    }
    if (rc != SWM_OK || ms.empty()) return;
    std::sort(ms.begin(), ms.end());
    const double med = ms[ms.size() / 2];
    if (med < best_ms) { best_ms = med; bc = cols; br = seg; bg = grid; bx = box; }
  };
  // widths x rows per unit (0: one wave of units) x one CTA per unit or a
  // persistent wave of CTAs x both box modes
  const int seg_opts[] = {0, 16, 24, 32, 48, 64, 96};
  for (int w : kStageWidths) {
    for (int seg : seg_opts) {
      for (int box : {SWM_BOX_STRIP, SWM_BOX_WIDEST}) {
        if (rc != SWM_OK) break;
        if (seg >= ctx->n) continue;
        trial(w, seg, 0, box);
        if (rc != SWM_OK || seg == 0) continue;
        const int wave = std::max(1, ctx->shape.ctas_per_sm) * ctx->num_sms;
        if (ctx->shape.cols == w && ctx->nunits > wave) trial(w, seg, wave, box);
      }
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  swm_state_free(x);
  const int rc2 = rc == SWM_OK ? stage_layout(ctx, bc, br, bg, bx) : stage_layout(ctx, c0, r0, g0, x0);
  if (rc != SWM_OK) return rc;
  if (rc2 != SWM_OK) return rc2;
  report(bc, br, bg, bx, best_ms);
  return SWM_OK;
}

int swm_work_split(int N, int sbp_order, int cols, int target_units, int seg_rows, int* units_out,
                   int max_units, int* nunits) {
  if (!units_out || !nunits) return fail(nullptr, SWM_E_INVALID, "null argument");
  if (N < 16 || N > 8190 || cols < 32 || target_units < 1 || seg_rows < 0)
    return fail(nullptr, SWM_E_INVALID, "bad work split arguments");
  if (sbp_order != 21 && sbp_order != 42 && sbp_order != 43 && sbp_order != 63)
    return fail(nullptr, SWM_E_UNSUPPORTED, "unknown SBP order");
  const int n = N + 1;
  std::vector<WorkUnit> units;
  std::string why;
  const int nseg = seg_rows > 0 ? (n + seg_rows - 1) / seg_rows : 0;
  if (!make_units(kTables[sbp_index(sbp_order)], n, cols, target_units, units, why, nseg))
    return fail(nullptr, SWM_E_INVALID, why);
  *nunits = (int)units.size();
  if ((int)units.size() > max_units) return fail(nullptr, SWM_E_INVALID, "max_units too small");
  for (size_t k = 0; k < units.size(); ++k) {
    const WorkUnit& w = units[k];
    const int v[9] = {w.panel, w.i0, w.i1, w.j0, w.j1, w.cl0, w.cl1, w.rl0, w.rl1};
    for (int e = 0; e < 9; ++e) units_out[9 * k + e] = v[e];
  }
  return SWM_OK;
}

int swm_get_stage_shape(swm_ctx* ctx, int* cols, int* seg_rows, int* grid, int* box, int* nunits) {
  AH_ONLY(ctx, "swm_get_stage_shape");
  if (!ctx) return fail(nullptr, SWM_E_INVALID, "null context");
  if (cols) *cols = ctx->shape.cols;
  if (seg_rows) *seg_rows = ctx->seg_rows;
  if (grid) *grid = ctx->stage_grid;
  if (box) *box = ctx->shape.fixbw ? SWM_BOX_WIDEST : SWM_BOX_STRIP;
  if (nunits) *nunits = ctx->nunits;
  return SWM_OK;
}

int swm_set_stage_shape(swm_ctx* ctx, int cols, int seg_rows, int grid, int box) {
  AH_ONLY(ctx, "swm_set_stage_shape");
  if (!ctx) return fail(nullptr, SWM_E_INVALID, "null context");
  if (seg_rows < 0 || grid < 0) return fail(ctx, SWM_E_INVALID, "shape values must be >= 0");
  if (box < SWM_BOX_AUTO || box > SWM_BOX_WIDEST) return fail(ctx, SWM_E_INVALID, "unknown box mode");
  USE_DEVICE(ctx);
  if (!ctx->shape.tma && cols != ctx->shape.cols)
    return fail(ctx, SWM_E_UNSUPPORTED, "the FP64 stage kernel has a single width");
  return stage_layout(ctx, cols, seg_rows, grid, ctx->shape.tma ? box : SWM_BOX_AUTO);
}

// ------------------------------------------------------- checkpoint / resume
// State file: a 64-byte header (magic "SWMSTATE", format version, N, SBP
// order, the writer's precision, the caller's model time) followed by the
// FP64 fields h, u, v, each 6*(N+1)^2 values in the reference layout (per
// panel (N+1)^2 values, i fastest).  An FP32 pair is stored as its exact
// FP64 sum and split again on load, so a round trip restores it.
struct StateFileHeader {
  char magic[8];
  uint32_t version, N, order, precision;
  double time;
  uint8_t pad[32];
};
static_assert(sizeof(StateFileHeader) == 64, "state file header is 64 bytes");

int swm_state_save(swm_ctx* ctx, const swm_state* s, const char* path, double time) {
  AH_ONLY(ctx, "swm_state_save");
  TraceRange trace_("swm_state_save");
  if (int rc = check_state(ctx, s)) return rc;
  if (!path || !*path) return fail(ctx, SWM_E_INVALID, "null path");
  USE_DEVICE(ctx);
  const size_t np = (size_t)6 * ctx->n * ctx->n;
  std::vector<double> buf(3 * np);
  double* dst[3] = {buf.data(), buf.data() + np, buf.data() + 2 * np};
  if (int rc = get_packed(ctx, s, dst, cudaMemcpyDeviceToHost)) return rc;
  if (int rc = sync_check(ctx, ctx->st)) return rc;
  StateFileHeader hd{};
  std::memcpy(hd.magic, "SWMSTATE", 8);
  hd.version = 1; hd.N = (uint32_t)ctx->N; hd.order = (uint32_t)ctx->order;
  hd.precision = (uint32_t)ctx->prec; hd.time = time;
  // Written to path + ".tmp" and renamed over path only when complete, so a
  // failed or interrupted write leaves an earlier restart file at path intact.
  const std::string tmp = std::string(path) + ".tmp";
  FILE* fp = std::fopen(tmp.c_str(), "wb");
  if (!fp) return fail(ctx, SWM_E_IO, "cannot open " + tmp);
  bool ok = std::fwrite(&hd, sizeof(hd), 1, fp) == 1 &&
            std::fwrite(buf.data(), sizeof(double), buf.size(), fp) == buf.size();
  ok = (std::fflush(fp) == 0) && ok;
  ok = (std::fclose(fp) == 0) && ok;
  if (!ok) {
    std::remove(tmp.c_str());
    return fail(ctx, SWM_E_IO, std::string("cannot write ") + path);
  }
  if (std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    return fail(ctx, SWM_E_IO, std::string("cannot rename the restart file to ") + path);
  }
  return SWM_OK;
}

int swm_state_load(swm_ctx* ctx, swm_state* s, const char* path, double* time) {
  AH_ONLY(ctx, "swm_state_load");
  TraceRange trace_("swm_state_load");
  if (int rc = check_state(ctx, s)) return rc;
  if (!path || !*path) return fail(ctx, SWM_E_INVALID, "null path");
  USE_DEVICE(ctx);
  FILE* fp = std::fopen(path, "rb");
  if (!fp) return fail(ctx, SWM_E_IO, std::string("cannot open ") + path);
  StateFileHeader hd{};
  const size_t np = (size_t)6 * ctx->n * ctx->n;
  std::vector<double> buf(3 * np);
  bool ok = std::fread(&hd, sizeof(hd), 1, fp) == 1;
  if (ok && (std::memcmp(hd.magic, "SWMSTATE", 8) != 0 || hd.version != 1)) {
    std::fclose(fp);
    return fail(ctx, SWM_E_INVALID, std::string(path) + " is not a state file");
  }
  if (ok && (int)hd.N != ctx->N) {
    std::fclose(fp);
    return fail(ctx, SWM_E_INVALID, "state file N=" + std::to_string(hd.N) + " does not match the context");
  }
  ok = ok && std::fread(buf.data(), sizeof(double), buf.size(), fp) == buf.size();
  std::fclose(fp);
  if (!ok) return fail(ctx, SWM_E_IO, std::string("cannot read ") + path);
  const double* src[3] = {buf.data(), buf.data() + np, buf.data() + 2 * np};
  if (int rc = put_packed(ctx, s, src, cudaMemcpyHostToDevice)) return rc;
  if (int rc = sync_check(ctx, ctx->st)) return rc;   // the host buffer goes out of scope
  if (time) *time = hd.time;
  return SWM_OK;
}

}  // extern "C"
