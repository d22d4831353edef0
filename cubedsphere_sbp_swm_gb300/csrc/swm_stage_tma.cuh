// swm_stage_tma.cuh -- fused RHS + RK stage kernel, TMA-pipelined.
//
// Same arithmetic as stage_kernel (swm_stage.cuh), different data movement:
// one producer warp streams the rows of a work unit (panel strip incl. its
// halo columns) into an NST-deep shared-memory pipeline with TMA bulk copies
// (cp.async.bulk ... mbarrier::complete_tx) -- the state and metric row the
// stencils need next plus the RK inputs of the row being finished -- while
// four consumer warps (one thread per column) turn each landed row into the
// derived stencil fields and finish the row RMAX behind it.  Every mbarrier
// wait is bounded: on expiry the kernel raises the device error flag, stops
// waiting, still passes every barrier (no deadlock) and drains its copies.
#pragma once

#include "swm_stage.cuh"

namespace swm {

// ---------------------------------------------------------------------------
// PTX wrappers (mbarrier, TMA bulk copy, named barrier, global timer)
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
__device__ __forceinline__ void tma_row(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void consumers_sync() {  // the 128 consumer threads only
  asm volatile("bar.sync 1, 128;" ::: "memory");
}

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s: far beyond any legal wait
constexpr int TMA_CONS = 128;                     // consumer threads, one per column
constexpr int TMA_THREADS = TMA_CONS + 32;        // + one producer warp

// row slots of one pipeline stage
enum {
  S_H = 0, S_U, S_V, S_J, S_Q1, S_Q2, S_Q3, S_HS,   // stencil input row
  S_F, S_RJ, S_B0, S_B1, S_B2, S_A0, S_A1, S_A2, S_L0, S_L1, S_L2,  // finished row
  NSLOT
};
enum { W_KE = 0, W_U, W_V, W_GU, W_GV, NW_FIELDS };   // stencil (wide) ring
enum { N_UT = 0, N_VT, N_J, NN_FIELDS };              // own-node (narrow) ring

template <class T, int ORD, int NST>
struct TmaLayout {
  static constexpr int RMAX = Ord<ORD>::RMAX;
  static constexpr int RBW = 2 * RMAX + 2;   // written row r, read rows r-2RMAX..r
  static constexpr int RBN = RMAX + 2;       // written row r, read at row r+RMAX
  static constexpr int ALIGN = 16 / (int)sizeof(T);
  static constexpr int ROWW = TMA_CONS + ALIGN;
  static constexpr size_t head = 256;        // mbarriers + abort flag
  static constexpr size_t wide = sizeof(T) * RBW * NW_FIELDS * TMA_CONS;
  static constexpr size_t narrow = sizeof(T) * RBN * NN_FIELDS * TMA_CONS;
  static constexpr size_t stage = sizeof(T) * NSLOT * ROWW;
  static constexpr size_t bytes = head + wide + narrow + NST * stage;
  static_assert(2 * NST * 8 + 16 <= head, "barrier area");
};

template <class T, int ORD, int NST>
__global__ void __launch_bounds__(TMA_THREADS)
    stage_tma_kernel(InstDev<T> one, const InstDev<T>* many, const WorkUnit* units, int mode,
                     int* err) {
  using L = TmaLayout<T, ORD, NST>;
  constexpr int RMAX = L::RMAX, RBW = L::RBW, RBN = L::RBN, ROWW = L::ROWW, AL = L::ALIGN;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  uint64_t* empty = full + NST;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + 2 * NST * 8);
  T* wide = reinterpret_cast<T*>(smem + L::head);
  T* narrow = wide + RBW * NW_FIELDS * TMA_CONS;
  T* stg = narrow + RBN * NN_FIELDS * TMA_CONS;

  const WorkUnit wu = units[blockIdx.x];
  const InstDev<T>& I = many ? many[wu.inst] : one;
  const int n = I.n, P = I.P;
  const long long fs = I.fs;
  const long long pbase = (long long)wu.panel * I.ps;
  const int tid = threadIdx.x;
  const int cal = wu.cl0 & ~(AL - 1);         // 16-byte aligned copy start
  const int off = wu.cl0 - cal;
  const uint32_t rbytes = (uint32_t)(((wu.cl1 - cal + AL - 1) / AL) * AL * (int)sizeof(T));
  const int niter = wu.j1 + RMAX - wu.rl0;

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
      const bool fp32 = sizeof(T) == 4;
      int issued = 0;
      for (int k = 0; k < niter; ++k) {
        const int s = k % NST;
        const uint32_t ph = (uint32_t)(k / NST) & 1u;
        if (*abort_flag) break;
        if (k >= NST && !mbar_wait_bounded(&empty[s], ph ^ 1u, kWaitLimitNs)) {
          *abort_flag = 1;
          atomicExch(err, 1);
          break;
        }
        const int r = wu.rl0 + k, j = r - RMAX;
        const bool in_row = r < wu.rl1;
        const bool out_row = j >= wu.j0 && j < wu.j1;
        T* sb = stg + (size_t)s * NSLOT * ROWW;
        const long long rin = pbase + (long long)r * P + cal;
        const long long rout = pbase + (long long)j * P + cal;
        // which rows this stage carries
        const T* src[NSLOT];
        int slot[NSLOT];
        int nc = 0;
        if (in_row) {
          for (int c = 0; c < 3; ++c) { src[nc] = I.in + c * fs + rin; slot[nc++] = S_H + c; }
          src[nc] = I.metric + MJ * fs + rin; slot[nc++] = S_J;
          src[nc] = I.metric + MQI1 * fs + rin; slot[nc++] = S_Q1;
          src[nc] = I.metric + MQI2 * fs + rin; slot[nc++] = S_Q2;
          src[nc] = I.metric + MQI3 * fs + rin; slot[nc++] = S_Q3;
          if (I.hs) { src[nc] = I.hs + rin; slot[nc++] = S_HS; }
        }
        if (out_row) {
          src[nc] = I.metric + MF * fs + rout; slot[nc++] = S_F;
          if (!fp32) { src[nc] = I.metric + MRJ * fs + rout; slot[nc++] = S_RJ; }
          const bool needB = mode == MODE_RK1 || mode == MODE_RK2 || mode == MODE_RK3 ||
                             (fp32 && mode == MODE_RK4);
          const bool needA = mode == MODE_RK2 || mode == MODE_RK3 || mode == MODE_RK4;
          const T* bsrc = (mode == MODE_RK4) ? I.base_out : I.base;
          if (needB)
            for (int c = 0; c < 3; ++c) { src[nc] = bsrc + c * fs + rout; slot[nc++] = S_B0 + c; }
          if (needA)
            for (int c = 0; c < 3; ++c) { src[nc] = I.acc + c * fs + rout; slot[nc++] = S_A0 + c; }
          if (fp32 && mode == MODE_RK4)
            for (int c = 0; c < 3; ++c) { src[nc] = I.base_lo + c * fs + rout; slot[nc++] = S_L0 + c; }
        }
        mbar_arrive_expect_tx(&full[s], rbytes * (uint32_t)nc);
        for (int q = 0; q < nc; ++q) tma_row(sb + (size_t)slot[q] * ROWW, src[q], rbytes, &full[s]);
        issued = k + 1;
      }
      // drain: the copies of the last stages must have landed before exit
      for (int k = max(0, issued - NST); k < issued; ++k)
        if (!mbar_wait_bounded(&full[k % NST], (uint32_t)(k / NST) & 1u, kWaitLimitNs))
          atomicExch(err, 2);
    }
    return;
  }

  // ------------------------------------------------------------ consumers
  const int t = tid;
  const int col = wu.cl0 + t;
  const bool ld = col < wu.cl1;
  const bool own = col >= wu.i0 && col < wu.i1;
  const int x = t + off;                   // column index inside a staged row
  const T grav = I.grav;
  const bool fp32 = sizeof(T) == 4;
  for (int k = 0; k < niter; ++k) {
    const int s = k % NST;
    const uint32_t ph = (uint32_t)(k / NST) & 1u;
    bool ok = true;
    if (!*abort_flag) ok = mbar_wait_bounded(&full[s], ph, kWaitLimitNs);
    if (!ok) { *abort_flag = 1; atomicExch(err, 3); }
    const T* sb = stg + (size_t)s * NSLOT * ROWW;
    const int r = wu.rl0 + k, j = r - RMAX;
    if (ok && r < wu.rl1 && ld) {
      const T h = sb[S_H * ROWW + x], u = sb[S_U * ROWW + x], v = sb[S_V * ROWW + x];
      const T J = sb[S_J * ROWW + x];
      const T q1 = sb[S_Q1 * ROWW + x], q2 = sb[S_Q2 * ROWW + x], q3 = sb[S_Q3 * ROWW + x];
      const T ut = q1 * u + q2 * v;
      const T vt = q2 * u + q3 * v;
      T ke = (u * ut + v * vt) / T(2.0);
      ke = ke + grav * h;
      if (I.hs) ke = ke + grav * sb[S_HS * ROWW + x];
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
    if (!*abort_flag && own && j >= wu.j0 && j < wu.j1) {
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
      if constexpr (sizeof(T) == 8) rJ = sb[S_RJ * ROWW + x];
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
      } else {
        T kk[3];
        node_tendency<T>(gx, gy, zeta, dv, sb[S_F * ROWW + x], J, nj[N_UT * TMA_CONS + t],
                         nj[N_VT * TMA_CONS + t], kk[0], kk[1], kk[2]);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const long long o = c * fs + idx;
          if (mode == MODE_APPLY) {
            I.out[o] = kk[c];
          } else if constexpr (sizeof(T) == 8) {
            if (mode == MODE_RK1) {
              const T b = sb[(S_B0 + c) * ROWW + x];
              I.out[o] = T(1.0) * b + I.c_in * kk[c];
              I.acc[o] = b + I.c_acc * kk[c];
            } else if (mode == MODE_RK4) {
              I.base_out[o] = sb[(S_A0 + c) * ROWW + x] + I.c_acc * kk[c];
            } else {
              I.out[o] = T(1.0) * sb[(S_B0 + c) * ROWW + x] + I.c_in * kk[c];
              I.acc[o] = sb[(S_A0 + c) * ROWW + x] + I.c_acc * kk[c];
            }
          } else {
            if (mode == MODE_RK1) {
              I.out[o] = sb[(S_B0 + c) * ROWW + x] + I.c_in * kk[c];
              I.acc[o] = I.c_acc * kk[c];
            } else if (mode == MODE_RK4) {
              const T d = sb[(S_A0 + c) * ROWW + x] + I.c_acc * kk[c];
              const T hi = sb[(S_B0 + c) * ROWW + x], lo = sb[(S_L0 + c) * ROWW + x];
              const T tt = lo + d;
              const T sm = hi + tt;
              const T bb = sm - hi;
              I.base_out[o] = sm;
              I.base_lo[o] = (hi - (sm - bb)) + (tt - bb);
            } else {
              I.out[o] = sb[(S_B0 + c) * ROWW + x] + I.c_in * kk[c];
              I.acc[o] = sb[(S_A0 + c) * ROWW + x] + I.c_acc * kk[c];
            }
          }
        }
      }
    }
    (void)fp32;
    __syncwarp();
    if ((t & 31) == 0) mbar_arrive(&empty[s]);
  }
}

template <class T, int ORD, int NST>
cudaError_t launch_stage_tma_ord(const InstDev<T>& one, const InstDev<T>* many,
                                 const WorkUnit* units, int nunits, int mode, int* err,
                                 cudaStream_t st) {
  constexpr size_t smem = TmaLayout<T, ORD, NST>::bytes;
  static bool configured = false;
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(stage_tma_kernel<T, ORD, NST>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  if (nunits <= 0) return cudaSuccess;
  stage_tma_kernel<T, ORD, NST><<<nunits, TMA_THREADS, smem, st>>>(one, many, units, mode, err);
  return cudaGetLastError();
}

template <class T, int ORD, int NST>
int stage_tma_occupancy() {
  int blocks = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, stage_tma_kernel<T, ORD, NST>, TMA_THREADS,
                                                TmaLayout<T, ORD, NST>::bytes);
  return blocks;
}

}  // namespace swm
