// swm_stage_tma.cuh -- fused RHS + RK stage kernel, TMA-pipelined.
//
// Same arithmetic as stage_kernel (swm_stage.cuh), different data movement.
// Every buffer is described to the TMA unit as a 3-D tensor (column, row of
// all panels, field).  One producer warp streams a work unit (a panel strip
// plus its halo columns) through an NST-deep shared-memory pipeline: each
// stage is RPS consecutive rows, brought in by a handful of
// cp.async.bulk.tensor.3d copies -- the state rows and metric rows the
// stencils need next, plus the RK inputs of the rows being finished RMAX
// behind -- completing on an mbarrier.  Four consumer warps (one thread per
// column) turn each landed row into the derived stencil fields and finish
// the row RMAX behind it.  Each thread derives every row of its own column,
// so the y stencils read a register window of the last 2*RMAX+1 rows; only
// the values other threads need along a row (KE, v, J h ut) and the
// thread's own (ut, vt, J) of the row being finished go through a small
// shared-memory ring.  Boundary-closure columns keep their closure row in
// registers; closure rows of the y stencil are compile-time cases.
// Every mbarrier wait is bounded: on expiry the kernel raises the device
// error flag, stops waiting, still passes every barrier, and drains its
// copies before exit.
#pragma once

#include <cuda.h>

#include "swm_stage.cuh"

namespace swm {

// ---------------------------------------------------------------------------
// PTX wrappers (mbarrier, TMA tensor copy, named barrier, global timer)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t tx) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(tx)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// Wait for phase `parity` of bar to complete, at most limit_ns.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}
// 3-D tiled TMA load of one box into shared memory, completing on bar.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}
constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s: far beyond any legal wait
// Consumer threads per CTA (one per column of the unit's strip): a template
// parameter CONS of the kernel, one of the widths below; a context picks one
// (default 128, or the fastest for its grid, see swm_tune_stage).  The
// strip width changes only the work split, not any node's arithmetic.
constexpr int TMA_CONS_DEFAULT = 128;

template <int CONS>
__device__ __forceinline__ void consumers_sync() {  // the consumer threads only
  asm volatile("bar.sync 1, %0;" ::"n"(CONS) : "memory");
}



#ifndef SWM_TMA_RPS
#define SWM_TMA_RPS 2
#endif
// Two stages: measured on GB300 against three (and against four stages of
// one row), the smaller shared-memory footprint gives more resident CTAs and
// is 3% faster at N=384 and 7% at N=1024; one stage in flight already covers
// the TMA latency.
#ifndef SWM_TMA_NST
#define SWM_TMA_NST 2
#endif

// x-ring fields: what other threads read along the row (KE, v, J h ut) and
// what the owning thread reads RMAX rows later (ut, vt, J)
enum { X_KE = 0, X_V, X_GU, X_UT, X_VT, X_J, NX_FIELDS };

template <class T, int ORD, int CONS>
struct TmaLayout {
  static constexpr int RPS = SWM_TMA_RPS;    // rows per pipeline stage
  static constexpr int NST = SWM_TMA_NST;    // pipeline stages
  static constexpr int RMAX = Ord<ORD>::RMAX;
  static constexpr int WS = 2 * RMAX + 1;    // y window (registers): rows j-RMAX..j+RMAX
  static constexpr int RBX = RMAX + 2;       // x-ring rows: row r written, read at r+RMAX
  static constexpr int ALIGN = 16 / (int)sizeof(T);
  static constexpr int BOXW_MAX = CONS + ALIGN;  // widest box (16-byte multiple)
  static constexpr int NF = 2;               // metric f, rJ of the finished rows
  static constexpr size_t head = 256;        // mbarriers + abort flag
  static constexpr size_t xring = sizeof(T) * RBX * NX_FIELDS * CONS;
  __host__ __device__ static constexpr size_t r128(size_t b) { return (b + 127) / 128 * 128; }
  // stage layout for a box width bw: in(3) met(4) metf(2) base(3) acc(3) lo(3) hs(1)
  struct Stage {
    size_t o_in, o_met, o_metf, o_base, o_acc, o_lo, o_hs, bytes;
  };
  __host__ __device__ static constexpr Stage stage(int bw) {
    const size_t rb = sizeof(T) * (size_t)bw * RPS;
    Stage s{};
    s.o_in = 0;
    s.o_met = s.o_in + r128(3 * rb);
    s.o_metf = s.o_met + r128(4 * rb);
    s.o_base = s.o_metf + r128(NF * rb);
    s.o_acc = s.o_base + r128(3 * rb);
    s.o_lo = s.o_acc + r128(3 * rb);
    s.o_hs = s.o_lo + r128(3 * rb);
    s.bytes = s.o_hs + r128(rb);
    return s;
  }
  __host__ __device__ static constexpr size_t smem_bytes(int bw) {
    return 128 + head + r128(xring) + NST * stage(bw).bytes;
  }
  static_assert(2 * NST * 8 + 16 <= head, "barrier area");
  static_assert(BOXW_MAX <= 256 && RPS <= 256, "TMA box limits");
};

// y derivative at row j from the register window w (w[i] holds row j-RMAX+i).
// A closure row takes every window slot with the row's coefficient of that
// slot (zero outside the stencil, adding exact zeros), so the window is only
// ever indexed by compile-time constants and stays in registers.  (Selecting
// among the compile-time closure rows instead, with the taps at their rows,
// made the compiler keep a 4/2 window in local memory, rewritten every row.)
template <int ORD, class T, int WS>
__device__ __forceinline__ T ydiff(const T (&w)[WS], int j, int n) {
  constexpr int NE = Ord<ORD>::NE, RMAX = Ord<ORD>::RMAX, ID = Ord<ORD>::idx;
  if (j >= NE && j < n - NE) return d_interior<ORD, T>([&](int o) { return w[RMAX + o]; });
  T acc = T(0);
  if (j < NE) {
    const int last = c_sbp[ID].last[j];
#pragma unroll
    for (int i = 0; i < WS; ++i) {
      const int m = j - RMAX + i;            // panel row of slot i
      const T c = (m >= 0 && m < last) ? sbp_ql<T>(ID, j, m) : T(0);
      acc += c * w[i];
    }
  } else {
    const int R = n - 1 - j;
    const int last = c_sbp[ID].last[R];
#pragma unroll
    for (int i = 0; i < WS; ++i) {
      const int m = R + RMAX - i;            // slot i holds panel row n-1-m
      const T c = (m >= 0 && m < last) ? sbp_qr<T>(ID, R, m) : T(0);
      acc += c * w[i];
    }
  }
  return acc;
}

// RK stage epilogue of one field at global offset o: k is the tendency, sc
// points at this field's row of the stage (base at +eb, running sum at +ea,
// FP32 low part at +el).
template <class T, int MODE>
__device__ __forceinline__ void rk_store(T* outp, T* accp, T* bop, T* blp, int o, T k, const T* sc,
                                         int eb, int ea, int el, int fstride, T c_in, T c_acc) {
  (void)fstride;
  constexpr bool FP32 = sizeof(T) == 4;
  if constexpr (MODE == MODE_APPLY) {
    outp[o] = k;
  } else if constexpr (!FP32) {
    if constexpr (MODE == MODE_RK1) {
      const T b = sc[eb];
      outp[o] = T(1.0) * b + c_in * k;
      accp[o] = b + c_acc * k;
    } else if constexpr (MODE == MODE_RK4) {
      bop[o] = sc[ea] + c_acc * k;
    } else {
      outp[o] = T(1.0) * sc[eb] + c_in * k;
      accp[o] = sc[ea] + c_acc * k;
    }
  } else {
    if constexpr (MODE == MODE_RK1) {
      outp[o] = sc[eb] + c_in * k;
      accp[o] = c_acc * k;
    } else if constexpr (MODE == MODE_RK4) {
      const T d = sc[ea] + c_acc * k;
      const T hi = sc[eb], lo = sc[el];
      const T tt = lo + d;
      const T sm = hi + tt;
      const T bb = sm - hi;
      bop[o] = sm;
      blp[o] = (hi - (sm - bb)) + (tt - bb);
    } else {
      outp[o] = sc[eb] + c_in * k;
      accp[o] = sc[ea] + c_acc * k;
    }
  }
}

// Stage-ring slot layout of one work unit: element offsets of its boxes for
// the unit's box width bw (the slots themselves are sized for the widest box
// of the launch).
struct StageOffsets {
  int in, met, metf, base, acc, lo, hs;
};
template <class L>
__device__ __forceinline__ StageOffsets stage_offsets(int bw, int esz) {
  const auto sl = L::stage(bw);
  return StageOffsets{(int)(sl.o_in / esz), (int)(sl.o_met / esz), (int)(sl.o_metf / esz),
                      (int)(sl.o_base / esz), (int)(sl.o_acc / esz), (int)(sl.o_lo / esz),
                      (int)(sl.o_hs / esz)};
}

__device__ __forceinline__ void tensormap_acquire(const CUtensorMap* m) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(
                   reinterpret_cast<uint64_t>(m))
               : "memory");
}

// Persistent over work units: CTA b runs units b, b + gridDim.x, ...; the
// pipeline's chunk count (and so every mbarrier phase) runs on across units,
// so the producer streams the next unit while the consumers finish the last.
// A unit takes its tensor maps from its instance (InstDev::maps, global
// memory; batched launches) or from the kernel parameter (one instance).
// slot_bw is the widest box width of the launch (ring slot size).
template <class T, int ORD, int MODE, int CONS, bool FIXBW>
__global__ void __launch_bounds__(CONS + 32)
    stage_tma_kernel(const __grid_constant__ StageMaps maps, InstDev<T> one,
                     const InstDev<T>* many, const WorkUnit* units, int nunits, int slot_bw,
                     int* err) {
  using L = TmaLayout<T, ORD, CONS>;
  constexpr int RMAX = L::RMAX, RPS = L::RPS, NST = L::NST, AL = L::ALIGN, WS = L::WS,
                RBX = L::RBX;
  constexpr int XS = NX_FIELDS * CONS;   // x-ring slot stride
  constexpr int NE = Ord<ORD>::NE, NW = Ord<ORD>::NW;
  constexpr bool FP32 = sizeof(T) == 4;
  constexpr bool needB = MODE == MODE_RK1 || MODE == MODE_RK2 || MODE == MODE_RK3 ||
                         (FP32 && MODE == MODE_RK4);
  constexpr bool needA = MODE == MODE_RK2 || MODE == MODE_RK3 || MODE == MODE_RK4;
  constexpr bool needL = FP32 && MODE == MODE_RK4;

  extern __shared__ unsigned char smem_dyn[];
  // 128-byte aligned base (TMA tensor destinations)
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_dyn) + 127) & ~uintptr_t(127));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + NST;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + 2 * NST * 8);
  T* xring = reinterpret_cast<T*>(smem + L::head);
  unsigned char* stg = smem + L::head + L::r128(L::xring);
  // FIXBW: every box is the widest one, so every shared-memory offset is a
  // compile-time constant (fewer address instructions and registers, more
  // shared memory for narrow strips)
  const size_t st_bytes = L::stage(FIXBW ? int(L::BOXW_MAX) : slot_bw).bytes;   // ring slot stride
  const int tid = threadIdx.x;

  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], CONS / 32);
    }
    *abort_flag = 0;
    mbar_fence_init();
  }
  __syncthreads();

  // ------------------------------------------------------------ producer
  if (tid >= CONS) {
    if (tid == CONS) {
      int gc = 0;   // chunks issued over all units of this CTA
      for (int u = blockIdx.x; u < nunits && !*abort_flag; u += gridDim.x) {
        const WorkUnit wu = units[u];
        const InstDev<T>& I = many ? many[wu.inst] : one;
        const StageMaps* M = I.maps ? I.maps : &maps;
        if (I.maps) {
          tensormap_acquire(&M->in); tensormap_acquire(&M->met); tensormap_acquire(&M->metf);
          tensormap_acquire(&M->base); tensormap_acquire(&M->acc); tensormap_acquire(&M->lo);
          tensormap_acquire(&M->hs);
        }
        const int rl0 = wu.rl0, rl1 = wu.rl1, j0u = wu.j0, j1u = wu.j1;
        const int cal = wu.cl0 & ~(AL - 1);     // 16-byte aligned box start column
        const int prow = wu.panel * I.n;        // row of this panel in the (6n)-row tensors
        const int nch = (j1u + RMAX - rl0 + RPS - 1) / RPS;
        const bool hasHs = I.hs != nullptr;
        const int bw = FIXBW ? int(L::BOXW_MAX) : I.boxw;
        const StageOffsets e = stage_offsets<L>(bw, (int)sizeof(T));
        const uint32_t rowb = (uint32_t)(bw * RPS * (int)sizeof(T));  // one field, RPS rows
        for (int c = 0; c < nch; ++c, ++gc) {
          const int s = gc % NST;
          const uint32_t ph = (uint32_t)(gc / NST) & 1u;
          if (*abort_flag) break;
          if (gc >= NST && !mbar_wait_bounded(&empty[s], ph ^ 1u, kWaitLimitNs)) {
            *abort_flag = 1;
            atomicExch(err, 1);
            break;
          }
          const int r0 = rl0 + c * RPS, j0 = r0 - RMAX;
          const bool in_any = r0 < rl1;
          const bool out_any = j0 + RPS > j0u && j0 < j1u;
          uint32_t tx = 0;
          if (in_any) tx += (uint32_t)(3 + 4 + (hasHs ? 1 : 0)) * rowb;
          if (out_any)
            tx += (uint32_t)(L::NF + (needB ? 3 : 0) + (needA ? 3 : 0) + (needL ? 3 : 0)) * rowb;
          T* sb = reinterpret_cast<T*>(stg + (size_t)s * st_bytes);
          mbar_arrive_expect_tx(&full[s], tx);
          if (in_any) {
            tma_load_3d(sb + e.in, &M->in, cal, prow + r0, 0, &full[s]);
            tma_load_3d(sb + e.met, &M->met, cal, prow + r0, MJ, &full[s]);
            if (hasHs) tma_load_3d(sb + e.hs, &M->hs, cal, prow + r0, 0, &full[s]);
          }
          if (out_any) {
            tma_load_3d(sb + e.metf, &M->metf, cal, prow + j0, MF, &full[s]);
            if (needB) tma_load_3d(sb + e.base, &M->base, cal, prow + j0, 0, &full[s]);
            if (needA) tma_load_3d(sb + e.acc, &M->acc, cal, prow + j0, 0, &full[s]);
            if (needL) tma_load_3d(sb + e.lo, &M->lo, cal, prow + j0, 0, &full[s]);
          }
        }
      }
      // drain: the copies of the last stages must have landed before exit
      for (int c = max(0, gc - NST); c < gc; ++c)
        if (!mbar_wait_bounded(&full[c % NST], (uint32_t)(c / NST) & 1u, kWaitLimitNs))
          atomicExch(err, 2);
    }
    return;
  }

  // ------------------------------------------------------------ consumers
  const int t = tid;
  int gc = 0;   // chunks consumed over all units of this CTA
  for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
  const WorkUnit wu = units[u];
  const InstDev<T>& I = many ? many[wu.inst] : one;
  const int n = I.n, P = I.P;
  const int rl0 = wu.rl0, rl1 = wu.rl1, j0u = wu.j0, j1u = wu.j1;
  const int cal = wu.cl0 & ~(AL - 1);
  const int nch = (j1u + RMAX - rl0 + RPS - 1) / RPS;
  const bool hasHs = I.hs != nullptr;
  const int bw = FIXBW ? int(L::BOXW_MAX) : I.boxw;
  const StageOffsets eo = stage_offsets<L>(bw, (int)sizeof(T));
  const int e_in = eo.in, e_met = eo.met, e_metf = eo.metf, e_base = eo.base, e_acc = eo.acc,
            e_lo = eo.lo, e_hs = eo.hs;
  // every consumer is done with the previous unit's x-ring rows
  if (u != (int)blockIdx.x) consumers_sync<CONS>();
  const int col = wu.cl0 + t;
  const bool ld = col < wu.cl1;
  const bool own = col >= wu.i0 && col < wu.i1;
  const bool xint = col >= NE && col < n - NE;   // interior stencil along the row
  const int x = t + (wu.cl0 - cal);               // column inside a box row
  // A boundary-closure column keeps its closure row in registers: taps at
  // columns xs + m with coefficients cx[m] (the right block is the mirrored,
  // sign-flipped left block).
  T cx[NW];
  int xs = 0;
#pragma unroll
  for (int m = 0; m < NW; ++m) cx[m] = T(0);
  if (!xint && own) {
    const bool left = col < NE;
    const int rr = left ? col : n - 1 - col;
    const int last = c_sbp[Ord<ORD>::idx].last[rr];
    xs = left ? 0 : n - NW;
#pragma unroll
    for (int m = 0; m < NW; ++m) {
      const int mm = left ? m : NW - 1 - m;
      cx[m] = mm < last ? (left ? sbp_ql<T>(Ord<ORD>::idx, rr, mm) : sbp_qr<T>(Ord<ORD>::idx, rr, mm))
                        : T(0);
    }
  }
  const T grav = I.grav, ghs = I.ghs, c_in = I.c_in, c_acc = I.c_acc;
  const int fs = (int)I.fs;
  const int gcol = (int)((long long)wu.panel * I.ps) + col;  // node (col, 0) of this panel
  T* const outp = I.out;
  T* const accp = I.acc;
  T* const bop = I.base_out;
  T* const blp = I.base_lo;
  // y windows of the derived fields this thread needs along its column
  T yke[WS], yu[WS], ygv[WS];
#pragma unroll
  for (int i = 0; i < WS; ++i) { yke[i] = T(0); yu[i] = T(0); ygv[i] = T(0); }
  // x-ring slots of the row being derived (r) and of the row being finished
  // (j = r - RMAX), counted from the unit's first row
  int slot_r = 0, slot_j = RBX - RMAX;

  for (int c = 0; c < nch; ++c, ++gc) {
    const int s = gc % NST;
    const uint32_t ph = (uint32_t)(gc / NST) & 1u;
    // After an abort nothing of this chunk is read or stored: its copies may
    // not have landed, and the caller's state stays as it was.
    bool ok = false;
    if (!*abort_flag) {
      ok = mbar_wait_bounded(&full[s], ph, kWaitLimitNs);
      if (!ok) { *abort_flag = 1; atomicExch(err, 3); }
    }
    // this thread's column in the stage; element (field f, box row q) of the
    // box at element offset e is sx[e + (f * RPS + q) * bw]
    const T* sx = reinterpret_cast<const T*>(stg + (size_t)s * st_bytes) + x;
#pragma unroll
    for (int q = 0; q < RPS; ++q) {
      const int r = rl0 + c * RPS + q, j = r - RMAX;
      T ke = T(0), u = T(0), gv = T(0);
      if (ok && r < rl1 && ld) {
        const T h = sx[e_in + (0 * RPS + q) * bw];
        u = sx[e_in + (1 * RPS + q) * bw];
        const T v = sx[e_in + (2 * RPS + q) * bw];
        const T J = sx[e_met + (0 * RPS + q) * bw];
        const T q1 = sx[e_met + (1 * RPS + q) * bw], q2 = sx[e_met + (2 * RPS + q) * bw], q3 = sx[e_met + (3 * RPS + q) * bw];
        const T ut = q1 * u + q2 * v;
        const T vt = q2 * u + q3 * v;
        ke = (u * ut + v * vt) * T(0.5);
        ke = ke + grav * h;
        if (hasHs) ke = ke + grav * sx[e_hs + (0 * RPS + q) * bw];
        gv = J * (h * vt);
        T* xw = xring + slot_r * XS + t;
        xw[X_KE * CONS] = ke;
        xw[X_V * CONS] = v;
        xw[X_GU * CONS] = J * (h * ut);
        xw[X_UT * CONS] = ut;
        xw[X_VT * CONS] = vt;
        xw[X_J * CONS] = J;
      }
      // push row r into the window: w[i] holds row r-2RMAX+i = j-RMAX+i
#pragma unroll
      for (int i = 0; i < WS - 1; ++i) { yke[i] = yke[i + 1]; yu[i] = yu[i + 1]; ygv[i] = ygv[i + 1]; }
      yke[WS - 1] = ke; yu[WS - 1] = u; ygv[WS - 1] = gv;
      consumers_sync<CONS>();
      const int sj = slot_j;
      slot_r = slot_r + 1 == RBX ? 0 : slot_r + 1;
      slot_j = slot_j + 1 == RBX ? 0 : slot_j + 1;
      if (*abort_flag || !own || j < j0u || j >= j1u) continue;
      const T* xr = xring + sj * XS + t;      // row j, this thread's column
      T dxke, dxv, dxgu;
      if (xint) {
        dxke = d_interior<ORD, T>([&](int o) { return xr[X_KE * CONS + o]; });
        dxv = d_interior<ORD, T>([&](int o) { return xr[X_V * CONS + o]; });
        dxgu = d_interior<ORD, T>([&](int o) { return xr[X_GU * CONS + o]; });
      } else {
        dxke = T(0); dxv = T(0); dxgu = T(0);
#pragma unroll
        for (int m = 0; m < NW; ++m) {
          const int o = xs + m - col;
          dxke += cx[m] * xr[X_KE * CONS + o];
          dxv += cx[m] * xr[X_V * CONS + o];
          dxgu += cx[m] * xr[X_GU * CONS + o];
        }
      }
      const T dyke = ydiff<ORD, T, WS>(yke, j, n);
      const T dyu = ydiff<ORD, T, WS>(yu, j, n);
      const T dygv = ydiff<ORD, T, WS>(ygv, j, n);
      const T J = xr[X_J * CONS];
      const T rJ = sx[e_metf + (1 * RPS + q) * bw];
      const T gx = dxke * ghs, gy = dyke * ghs;
      const T zeta = (dxv - dyu) * rJ;
      const T dv = (dxgu + dygv) * rJ;
      if ((col == 0) | (col == n - 1) | (j == 0) | (j == n - 1)) {
        T* E = I.edge + wu.panel * 16 * n;
        const T vals[4] = {gx, gy, zeta, dv};
        if (col == 0)
#pragma unroll
          for (int e = 0; e < 4; ++e) E[(SIDE_L * 4 + e) * n + j] = vals[e];
        if (col == n - 1)
#pragma unroll
          for (int e = 0; e < 4; ++e) E[(SIDE_R * 4 + e) * n + j] = vals[e];
        if (j == 0)
#pragma unroll
          for (int e = 0; e < 4; ++e) E[(SIDE_B * 4 + e) * n + col] = vals[e];
        if (j == n - 1)
#pragma unroll
          for (int e = 0; e < 4; ++e) E[(SIDE_T * 4 + e) * n + col] = vals[e];
        continue;
      }
      T k0, k1, k2;
      node_tendency<T>(gx, gy, zeta, dv, sx[e_metf + (0 * RPS + q) * bw], J, xr[X_UT * CONS],
                       xr[X_VT * CONS], k0, k1, k2);
      const int g = gcol + j * P;
      const int qb = q * bw;
      rk_store<T, MODE>(outp, accp, bop, blp, g, k0, sx + qb, e_base, e_acc, e_lo, RPS * bw, c_in, c_acc);
      rk_store<T, MODE>(outp, accp, bop, blp, fs + g, k1, sx + qb + RPS * bw, e_base, e_acc, e_lo, RPS * bw, c_in, c_acc);
      rk_store<T, MODE>(outp, accp, bop, blp, 2 * fs + g, k2, sx + qb + 2 * RPS * bw, e_base, e_acc, e_lo, RPS * bw, c_in, c_acc);
    }
    __syncwarp();
    if ((t & 31) == 0) mbar_arrive(&empty[s]);
  }
  }  // units
}

template <class T, int ORD, int MODE, int CONS, bool FIXBW>
cudaError_t launch_stage_tma_mode(const StageMaps& maps, const InstDev<T>& one,
                                  const InstDev<T>* many, const WorkUnit* units, int nunits,
                                  int boxw, int grid, int* err, cudaStream_t st) {
  using L = TmaLayout<T, ORD, CONS>;
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(stage_tma_kernel<T, ORD, MODE, CONS, FIXBW>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)L::smem_bytes(L::BOXW_MAX));
    if (e != cudaSuccess) return e;
    configured = true;
  }
  if (nunits <= 0) return cudaSuccess;
  if (boxw < 1 || boxw > L::BOXW_MAX || (FIXBW && boxw != L::BOXW_MAX)) return cudaErrorInvalidValue;
  const int g = (grid > 0 && grid < nunits) ? grid : nunits;
  stage_tma_kernel<T, ORD, MODE, CONS, FIXBW><<<g, CONS + 32, L::smem_bytes(boxw), st>>>(
      maps, one, many, units, nunits, boxw, err);
  return cudaGetLastError();
}

template <class T, int ORD, int CONS, bool FIXBW>
cudaError_t launch_stage_tma_ord(const StageMaps& maps, const InstDev<T>& one,
                                 const InstDev<T>* many, const WorkUnit* units, int nunits,
                                 int mode, int boxw, int grid, int* err, cudaStream_t st) {
  switch (mode) {
    case MODE_APPLY: return launch_stage_tma_mode<T, ORD, MODE_APPLY, CONS, FIXBW>(maps, one, many, units, nunits, boxw, grid, err, st);
    case MODE_RK1: return launch_stage_tma_mode<T, ORD, MODE_RK1, CONS, FIXBW>(maps, one, many, units, nunits, boxw, grid, err, st);
    case MODE_RK2: return launch_stage_tma_mode<T, ORD, MODE_RK2, CONS, FIXBW>(maps, one, many, units, nunits, boxw, grid, err, st);
    case MODE_RK3: return launch_stage_tma_mode<T, ORD, MODE_RK3, CONS, FIXBW>(maps, one, many, units, nunits, boxw, grid, err, st);
    case MODE_RK4: return launch_stage_tma_mode<T, ORD, MODE_RK4, CONS, FIXBW>(maps, one, many, units, nunits, boxw, grid, err, st);
    default: return cudaErrorInvalidValue;
  }
}

// configure every mode (outside any capture)
template <class T, int ORD, int CONS, bool FIXBW>
cudaError_t prepare_stage_tma_ord() {
  static const StageMaps kNone{};
  for (int m = MODE_APPLY; m <= MODE_RK4; ++m) {
    cudaError_t e = launch_stage_tma_ord<T, ORD, CONS, FIXBW>(kNone, InstDev<T>{}, nullptr, nullptr,
                                                              0, m, TmaLayout<T, ORD, CONS>::BOXW_MAX,
                                                              0, nullptr, nullptr);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// resident CTAs per SM at box width bw
template <class T, int ORD, int CONS, bool FIXBW>
int stage_tma_occupancy(int bw) {
  int blocks = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, stage_tma_kernel<T, ORD, MODE_RK2, CONS, FIXBW>,
                                                CONS + 32, TmaLayout<T, ORD, CONS>::smem_bytes(bw));
  return blocks;
}

// The FP32 stage kernel of one consumer width CONS for every SBP order and
// both box modes (instantiated by swm_stage_f32_w<CONS>.cu).
template <int CONS>
struct StageF32Width {
  template <bool FIXBW>
  static cudaError_t launch_fb(int order, const StageMaps& m, const InstDev<float>& one,
                               const InstDev<float>* many, const WorkUnit* units, int nunits,
                               int mode, int boxw, int grid, int* err, cudaStream_t st) {
    switch (order) {
      case 21: return launch_stage_tma_ord<float, 21, CONS, FIXBW>(m, one, many, units, nunits, mode, boxw, grid, err, st);
      case 42: return launch_stage_tma_ord<float, 42, CONS, FIXBW>(m, one, many, units, nunits, mode, boxw, grid, err, st);
      case 43: return launch_stage_tma_ord<float, 43, CONS, FIXBW>(m, one, many, units, nunits, mode, boxw, grid, err, st);
      case 63: return launch_stage_tma_ord<float, 63, CONS, FIXBW>(m, one, many, units, nunits, mode, boxw, grid, err, st);
      default: return cudaErrorInvalidValue;
    }
  }
  static cudaError_t launch(int order, bool fixbw, const StageMaps& m, const InstDev<float>& one,
                            const InstDev<float>* many, const WorkUnit* units, int nunits,
                            int mode, int boxw, int grid, int* err, cudaStream_t st) {
    return fixbw ? launch_fb<true>(order, m, one, many, units, nunits, mode, boxw, grid, err, st)
                 : launch_fb<false>(order, m, one, many, units, nunits, mode, boxw, grid, err, st);
  }
  template <bool FIXBW>
  static int occupancy_fb(int order, int boxw) {
    switch (order) {
      case 21: return stage_tma_occupancy<float, 21, CONS, FIXBW>(boxw);
      case 42: return stage_tma_occupancy<float, 42, CONS, FIXBW>(boxw);
      case 43: return stage_tma_occupancy<float, 43, CONS, FIXBW>(boxw);
      default: return stage_tma_occupancy<float, 63, CONS, FIXBW>(boxw);
    }
  }
  static int occupancy(int order, bool fixbw, int boxw) {
    return fixbw ? occupancy_fb<true>(order, boxw) : occupancy_fb<false>(order, boxw);
  }
  template <bool FIXBW>
  static cudaError_t prepare_fb(int order) {
    switch (order) {
      case 21: return prepare_stage_tma_ord<float, 21, CONS, FIXBW>();
      case 42: return prepare_stage_tma_ord<float, 42, CONS, FIXBW>();
      case 43: return prepare_stage_tma_ord<float, 43, CONS, FIXBW>();
      case 63: return prepare_stage_tma_ord<float, 63, CONS, FIXBW>();
      default: return cudaErrorInvalidValue;
    }
  }
  static cudaError_t prepare(int order) {
    cudaError_t e = prepare_fb<false>(order);
    return e == cudaSuccess ? prepare_fb<true>(order) : e;
  }
};

}  // namespace swm
