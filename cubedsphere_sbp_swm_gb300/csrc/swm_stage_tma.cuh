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
// column) turn each landed row into the derived stencil fields (KE, u, v,
// J h ut, J h vt in a shared-memory ring) and finish one row per landed row.
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
__device__ __forceinline__ void consumers_sync() {  // the 128 consumer threads only
  asm volatile("bar.sync 1, 128;" ::: "memory");
}

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s: far beyond any legal wait
constexpr int TMA_CONS = 128;                     // consumer threads, one per column
constexpr int TMA_THREADS = TMA_CONS + 32;        // + one producer warp

enum { W_KE = 0, W_U, W_V, W_GU, W_GV, NW_FIELDS };   // stencil (wide) ring
enum { N_UT = 0, N_VT, N_J, NN_FIELDS };              // own-node (narrow) ring

template <class T, int ORD, int RPS, int NST>
struct TmaLayout {
  static constexpr int RMAX = Ord<ORD>::RMAX;
  static constexpr int RBW = 2 * RMAX + 2;   // written row r, read rows r-2RMAX..r
  static constexpr int RBN = RMAX + 2;       // written row r, read at row r+RMAX
  static constexpr int ALIGN = 16 / (int)sizeof(T);
  static constexpr int BOXW = TMA_CONS + ALIGN;  // columns per box (16-byte multiple)
  static constexpr int NF = sizeof(T) == 8 ? 2 : 1;  // f (+ rJ)
  static constexpr size_t r128(size_t b) { return (b + 127) / 128 * 128; }
  static constexpr size_t row_bytes = sizeof(T) * BOXW * RPS;  // one field, RPS rows
  static constexpr size_t b_in = r128(3 * row_bytes), b_met = r128(4 * row_bytes),
                          b_metf = r128(NF * row_bytes), b_rk = r128(3 * row_bytes),
                          b_hs = r128(row_bytes);
  static constexpr size_t o_in = 0, o_met = o_in + b_in, o_metf = o_met + b_met,
                          o_base = o_metf + b_metf, o_acc = o_base + b_rk, o_lo = o_acc + b_rk,
                          o_hs = o_lo + b_rk, stage = o_hs + b_hs;
  static constexpr size_t head = 256;        // mbarriers + abort flag
  static constexpr size_t wide = sizeof(T) * RBW * NW_FIELDS * TMA_CONS;
  static constexpr size_t narrow = sizeof(T) * RBN * NN_FIELDS * TMA_CONS;
  static constexpr size_t bytes = 128 + head + r128(wide) + r128(narrow) + NST * stage;
  static_assert(2 * NST * 8 + 16 <= head, "barrier area");
  static_assert(BOXW <= 256 && RPS <= 256, "TMA box limits");
};

template <class T, int ORD, int RPS, int NST>
__global__ void __launch_bounds__(TMA_THREADS)
    stage_tma_kernel(const __grid_constant__ StageMaps maps, InstDev<T> one,
                     const InstDev<T>* many, const WorkUnit* units, int mode, int* err) {
  using L = TmaLayout<T, ORD, RPS, NST>;
  constexpr int RMAX = L::RMAX, RBW = L::RBW, RBN = L::RBN, BOXW = L::BOXW, AL = L::ALIGN;
  extern __shared__ unsigned char smem_dyn[];
  // 128-byte aligned base (TMA tensor destinations)
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_dyn) + 127) & ~uintptr_t(127));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + NST;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + 2 * NST * 8);
  T* wide = reinterpret_cast<T*>(smem + L::head);
  T* narrow = reinterpret_cast<T*>(smem + L::head + L::r128(L::wide));
  unsigned char* stg = smem + L::head + L::r128(L::wide) + L::r128(L::narrow);

  const WorkUnit wu = units[blockIdx.x];
  const InstDev<T>& I = many ? many[wu.inst] : one;
  const int n = I.n, P = I.P;
  const long long fs = I.fs;
  const long long pbase = (long long)wu.panel * I.ps;
  const int tid = threadIdx.x;
  const int cal = wu.cl0 & ~(AL - 1);         // 16-byte aligned box start column
  const int off = wu.cl0 - cal;
  const int prow = wu.panel * n;              // row of this panel in the (6n)-row tensors
  const int nch = (wu.j1 + RMAX - wu.rl0 + RPS - 1) / RPS;
  const bool fp32 = sizeof(T) == 4;
  const bool needB = mode == MODE_RK1 || mode == MODE_RK2 || mode == MODE_RK3 ||
                     (fp32 && mode == MODE_RK4);
  const bool needA = mode == MODE_RK2 || mode == MODE_RK3 || mode == MODE_RK4;
  const bool needL = fp32 && mode == MODE_RK4;
  const bool hasHs = I.hs != nullptr;

  if (tid == 0) {
    for (int s = 0; s < NST; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], TMA_CONS / 32);
    }
    *abort_flag = 0;
    mbar_fence_init();
  }
  __syncthreads();

  // ------------------------------------------------------------ producer
  if (tid >= TMA_CONS) {
    if (tid == TMA_CONS) {
      int issued = 0;
      for (int c = 0; c < nch; ++c) {
        const int s = c % NST;
        const uint32_t ph = (uint32_t)(c / NST) & 1u;
        if (*abort_flag) break;
        if (c >= NST && !mbar_wait_bounded(&empty[s], ph ^ 1u, kWaitLimitNs)) {
          *abort_flag = 1;
          atomicExch(err, 1);
          break;
        }
        const int r0 = wu.rl0 + c * RPS, j0 = r0 - RMAX;
        const bool in_any = r0 < wu.rl1;
        const bool out_any = j0 + RPS > wu.j0 && j0 < wu.j1;
        uint32_t tx = 0;
        if (in_any) tx += (uint32_t)(3 + 4 + (hasHs ? 1 : 0)) * (uint32_t)L::row_bytes;
        if (out_any)
          tx += (uint32_t)(L::NF + (needB ? 3 : 0) + (needA ? 3 : 0) + (needL ? 3 : 0)) *
                (uint32_t)L::row_bytes;
        unsigned char* sb = stg + (size_t)s * L::stage;
        mbar_arrive_expect_tx(&full[s], tx);
        if (in_any) {
          tma_load_3d(sb + L::o_in, &maps.in, cal, prow + r0, 0, &full[s]);
          tma_load_3d(sb + L::o_met, &maps.met, cal, prow + r0, MJ, &full[s]);
          if (hasHs) tma_load_3d(sb + L::o_hs, &maps.hs, cal, prow + r0, 0, &full[s]);
        }
        if (out_any) {
          tma_load_3d(sb + L::o_metf, &maps.metf, cal, prow + j0, MF, &full[s]);
          if (needB) tma_load_3d(sb + L::o_base, &maps.base, cal, prow + j0, 0, &full[s]);
          if (needA) tma_load_3d(sb + L::o_acc, &maps.acc, cal, prow + j0, 0, &full[s]);
          if (needL) tma_load_3d(sb + L::o_lo, &maps.lo, cal, prow + j0, 0, &full[s]);
        }
        issued = c + 1;
      }
      // drain: the copies of the last stages must have landed before exit
      for (int c = max(0, issued - NST); c < issued; ++c)
        if (!mbar_wait_bounded(&full[c % NST], (uint32_t)(c / NST) & 1u, kWaitLimitNs))
          atomicExch(err, 2);
    }
    return;
  }

  // ------------------------------------------------------------ consumers
  const int t = tid;
  const int col = wu.cl0 + t;
  const bool ld = col < wu.cl1;
  const bool own = col >= wu.i0 && col < wu.i1;
  const int x = t + off;                   // column inside a box row
  const T grav = I.grav;
  for (int c = 0; c < nch; ++c) {
    const int s = c % NST;
    const uint32_t ph = (uint32_t)(c / NST) & 1u;
    bool ok = true;
    if (!*abort_flag) ok = mbar_wait_bounded(&full[s], ph, kWaitLimitNs);
    if (!ok) { *abort_flag = 1; atomicExch(err, 3); }
    const unsigned char* sb = stg + (size_t)s * L::stage;
    // element (field f, box row q) of a box at byte offset o
    auto bx = [&](size_t o, int f, int q) {
      return reinterpret_cast<const T*>(sb + o)[(f * RPS + q) * BOXW + x];
    };
#pragma unroll 1
    for (int q = 0; q < RPS; ++q) {
      const int r = wu.rl0 + c * RPS + q, j = r - RMAX;
      if (ok && r < wu.rl1 && ld) {
        const T h = bx(L::o_in, 0, q), u = bx(L::o_in, 1, q), v = bx(L::o_in, 2, q);
        const T J = bx(L::o_met, 0, q);
        const T q1 = bx(L::o_met, 1, q), q2 = bx(L::o_met, 2, q), q3 = bx(L::o_met, 3, q);
        const T ut = q1 * u + q2 * v;
        const T vt = q2 * u + q3 * v;
        T ke = (u * ut + v * vt) / T(2.0);
        ke = ke + grav * h;
        if (hasHs) ke = ke + grav * bx(L::o_hs, 0, q);
        T* w = wide + (size_t)(r % RBW) * NW_FIELDS * TMA_CONS;
        w[W_KE * TMA_CONS + t] = ke;
        w[W_U * TMA_CONS + t] = u;
        w[W_V * TMA_CONS + t] = v;
        w[W_GU * TMA_CONS + t] = J * (h * ut);
        w[W_GV * TMA_CONS + t] = J * (h * vt);
        T* nr = narrow + (size_t)(r % RBN) * NN_FIELDS * TMA_CONS;
        nr[N_UT * TMA_CONS + t] = ut;
        nr[N_VT * TMA_CONS + t] = vt;
        nr[N_J * TMA_CONS + t] = J;
      }
      consumers_sync();
      if (*abort_flag || !own || j < wu.j0 || j >= wu.j1) continue;
      const T* wj = wide + (size_t)(j % RBW) * NW_FIELDS * TMA_CONS;
      auto xa = [&](int f) {
        return d_line<ORD, T>(col, n, [&](int m) { return wj[f * TMA_CONS + (m - wu.cl0)]; });
      };
      auto ya = [&](int f) {
        return d_line<ORD, T>(j, n, [&](int m) {
          return wide[(size_t)(m % RBW) * NW_FIELDS * TMA_CONS + f * TMA_CONS + t];
        });
      };
      const T dxke = xa(W_KE), dyke = ya(W_KE);
      const T dxv = xa(W_V), dyu = ya(W_U);
      const T dxgu = xa(W_GU), dygv = ya(W_GV);
      const T* nj = narrow + (size_t)(j % RBN) * NN_FIELDS * TMA_CONS;
      const T J = nj[N_J * TMA_CONS + t];
      T rJ;
      if constexpr (sizeof(T) == 8) rJ = bx(L::o_metf, 1, q);
      else rJ = I.ghs / J;
      const T gx = dxke * I.ghs, gy = dyke * I.ghs;
      const T zeta = (dxv - dyu) * rJ;
      const T dv = (dxgu + dygv) * rJ;
      const long long idx = pbase + (long long)j * P + col;
      if ((col == 0) | (col == n - 1) | (j == 0) | (j == n - 1)) {
        T* E = I.edge + (long long)wu.panel * 16 * n;
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
      T kk[3];
      node_tendency<T>(gx, gy, zeta, dv, bx(L::o_metf, 0, q), J, nj[N_UT * TMA_CONS + t],
                       nj[N_VT * TMA_CONS + t], kk[0], kk[1], kk[2]);
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) {
        const long long o = cc * fs + idx;
        if (mode == MODE_APPLY) {
          I.out[o] = kk[cc];
        } else if constexpr (sizeof(T) == 8) {
          if (mode == MODE_RK1) {
            const T b = bx(L::o_base, cc, q);
            I.out[o] = T(1.0) * b + I.c_in * kk[cc];
            I.acc[o] = b + I.c_acc * kk[cc];
          } else if (mode == MODE_RK4) {
            I.base_out[o] = bx(L::o_acc, cc, q) + I.c_acc * kk[cc];
          } else {
            I.out[o] = T(1.0) * bx(L::o_base, cc, q) + I.c_in * kk[cc];
            I.acc[o] = bx(L::o_acc, cc, q) + I.c_acc * kk[cc];
          }
        } else {
          if (mode == MODE_RK1) {
            I.out[o] = bx(L::o_base, cc, q) + I.c_in * kk[cc];
            I.acc[o] = I.c_acc * kk[cc];
          } else if (mode == MODE_RK4) {
            const T d = bx(L::o_acc, cc, q) + I.c_acc * kk[cc];
            const T hi = bx(L::o_base, cc, q), lo = bx(L::o_lo, cc, q);
            const T tt = lo + d;
            const T sm = hi + tt;
            const T bb = sm - hi;
            I.base_out[o] = sm;
            I.base_lo[o] = (hi - (sm - bb)) + (tt - bb);
          } else {
            I.out[o] = bx(L::o_base, cc, q) + I.c_in * kk[cc];
            I.acc[o] = bx(L::o_acc, cc, q) + I.c_acc * kk[cc];
          }
        }
      }
    }
    __syncwarp();
    if ((t & 31) == 0) mbar_arrive(&empty[s]);
  }
}

template <class T, int ORD, int RPS, int NST>
cudaError_t launch_stage_tma_ord(const StageMaps& maps, const InstDev<T>& one,
                                 const InstDev<T>* many, const WorkUnit* units, int nunits,
                                 int mode, int* err, cudaStream_t st) {
  constexpr size_t smem = TmaLayout<T, ORD, RPS, NST>::bytes;
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(stage_tma_kernel<T, ORD, RPS, NST>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  if (nunits <= 0) return cudaSuccess;
  stage_tma_kernel<T, ORD, RPS, NST><<<nunits, TMA_THREADS, smem, st>>>(maps, one, many, units,
                                                                         mode, err);
  return cudaGetLastError();
}

template <class T, int ORD, int RPS, int NST>
int stage_tma_occupancy() {
  int blocks = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, stage_tma_kernel<T, ORD, RPS, NST>,
                                                TMA_THREADS, TmaLayout<T, ORD, RPS, NST>::bytes);
  return blocks;
}

}  // namespace swm
