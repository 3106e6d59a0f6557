// lbm_tma.cuh - the A-A step kernel fed by TMA (cp.async.bulk.tensor) through
// a multi-stage shared-memory pipeline.  Used for the float32-collision
// storages (float32, float16, bfloat16 populations).
//
// Work: the fluid segments (32 cells along k, one warp each) in tiles of 8
// segments = 256 cells.  Persistent blocks walk their tiles; every tile's
// inputs arrive by TMA into one pipeline stage, completion is tracked by one
// mbarrier per stage, and the copies of the next STAGES-1 tiles are in
// flight while a tile is computed.  So the bytes in flight per SM do not
// depend on registers per thread.
//
//   even step: per segment one 2-D box {32 cells, 19 planes} of A at x = base
//   odd step:  per segment and direction q one row of plane opp(q) at
//              base - (cx*ny + cy)*nzp; rows of the +-z directions start 16
//              bytes earlier and are 32 bytes wider, so that x stays 16-byte
//              aligned and the +-1 shift along k is covered.  Every copy lands
//              in its own 128-byte-aligned slot of shared memory.
//   both:      the 32 mask words; with averaging, the 4 x 32 running sums
// Results are stored straight to global memory (coalesced, streaming).
//
// Correctness of prefetching in the in-place A-A scheme: every location a
// thread uses is read and written by that thread only, and the window cells
// outside [x, x+32) are never used, so a prefetch may read a location at any
// time before its owning thread runs.
#pragma once
#include <cuda.h>
#include <stdint.h>

#include "d3q19.cuh"
#include "lbm_iface.h"
#include "lbm_kernels.cuh"

namespace abx {

constexpr int kTmaSegs = 8;            // segments (warps) per tile
constexpr int kTmaThreads = 32 * kTmaSegs;

template <int K> struct TmaGeom {
  using T = typename Store<K>::T;
  static constexpr int kElem = sizeof(T);
  static constexpr int kPad = 16 / kElem;                  // cells before a shifted window (16 bytes)
  static constexpr int kWin = 32 + 2 * kPad;               // width of a window for directions with c_z != 0
  static constexpr int kEvenPop = 19 * 32 * kElem;         // bytes per segment, even step
  // odd step: one 128-byte-aligned slot per direction; c_z = 0 rows are exact 32-cell rows
  __host__ __device__ static constexpr int row_bytes(int q) { return (cz(q) == 0 ? 32 : kWin) * kElem; }
  __host__ __device__ static constexpr int slot_bytes(int q) { return (row_bytes(q) + 127) / 128 * 128; }
  // directions before q with c_z != 0 (5, 6, 11..18), closed form (no recursion, any q)
  __host__ __device__ static constexpr int nz_before(int q) {
    return (q > 5) + (q > 6) + (q > 11) + (q > 12) + (q > 13) + (q > 14) + (q > 15) + (q > 16) + (q > 17) + (q > 18);
  }
  __host__ __device__ static constexpr int slot_off(int q) {
    return q * slot_bytes(0) + nz_before(q) * (slot_bytes(5) - slot_bytes(0));
  }
  static constexpr int kOddStride = slot_off(19);          // bytes of one segment's slots
  static constexpr int kOddPop = 9 * 32 * kElem + 10 * kWin * kElem;   // transaction bytes per segment
};

// Tensor maps of one simulation, passed as const __grid_constant__ kernel
// parameters (the TMA instruction reads a descriptor from parameter space).
enum { kMapPopEven = 0,   // 2-D {Np, 19}, box {32, 19}
       kMapPopWide = 1,   // 2-D {Np, 19}, box {kWin, 1}
       kMapPopRow = 2,    // 2-D {Np, 19}, box {32, 1}
       kMapMask = 3,      // 1-D {Np}, box {32}
       kMapAcc = 4 };     // 2-D {Np, 4}, box {32, 4}

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up after 2^18 polls (each poll may suspend for a few
// microseconds, so well under a second), far above a tile's copy time.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int i = 0; i < (1 << 18); i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void fence_barrier_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// Bring a descriptor into the TMA unit's cache ahead of its first use.
__device__ __forceinline__ void tensormap_prefetch(const CUtensorMap *m) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(m) : "memory");
}

__device__ __forceinline__ void tma_load_1d(uint32_t dst, const CUtensorMap *map, int x, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.1d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2}], [%3];" ::"r"(dst),
      "l"(map), "r"(x), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(map), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// ------------------------------------------------------------------ the kernel
template <int K, bool ODD, bool ACC, bool HAS_NS, int STAGES>
struct TmaStage {
  using T = typename Store<K>::T;
  static constexpr int kPopBytes = ODD ? TmaGeom<K>::kOddPop : TmaGeom<K>::kEvenPop;
  static constexpr int kPopStride = ODD ? TmaGeom<K>::kOddStride : (kPopBytes + 127) / 128 * 128;  // 128-byte aligned
  static constexpr int kMaskOff = kTmaSegs * kPopStride;
  static constexpr int kAccOff = kMaskOff + kTmaSegs * 128;
  static constexpr int kBytes = kAccOff + (ACC ? kTmaSegs * 512 : 0);    // one stage
  static constexpr int kSegBytes = kPopBytes + 128 + (ACC ? 512 : 0);    // transaction bytes per segment
  static constexpr int kSmem = STAGES * kBytes + 1024;                    // + barriers, segment table, alignment slack
};

// The one copy a lane issues for its warp's segment of every tile, fixed for
// the whole launch.  Odd step: lanes 0..18 copy direction q = lane (plane
// opp(q), shifted by -(cx*ny + cy)*nzp, +-z rows kPad cells earlier); even
// step: lane 0 copies the 19-plane box.  Lane 19 copies the mask words, lane
// 20 (with averaging) the running sums.
struct LaneCopy {
  const CUtensorMap *map;
  int dx;          // x = segment base + dx
  int y;           // plane (row copies) or 0
  uint32_t soff;   // byte offset of the destination inside the warp's stage slice
  bool use;
};

template <int K, bool ODD, bool ACC, int STAGES>
__device__ __forceinline__ LaneCopy lane_copy(int lane, long long offq, const CUtensorMap *m_even,
                                              const CUtensorMap *m_wide, const CUtensorMap *m_row,
                                              const CUtensorMap *m_mask, const CUtensorMap *m_acc) {
  using G = TmaGeom<K>;
  using ST = TmaStage<K, ODD, ACC, false, STAGES>;
  LaneCopy c{nullptr, 0, 0, 0, false};
  if (ODD && lane < 19) {
    const int q = lane;
    const uint32_t slot = (uint32_t)G::slot_off(q);
    c.map = cz(q) == 0 ? m_row : m_wide;
    c.dx = (int)(-(offq - cz(q))) - (cz(q) == 0 ? 0 : G::kPad);
    c.y = opp(q);
    c.soff = slot;
    c.use = true;
  } else if (!ODD && lane == 0) {
    c.map = m_even; c.dx = 0; c.y = 0; c.soff = 0; c.use = true;
  } else if (lane == 19) {
    c.map = m_mask; c.dx = 0; c.y = -1; c.soff = (uint32_t)ST::kMaskOff; c.use = true;
  } else if (ACC && lane == 20) {
    c.map = m_acc; c.dx = 0; c.y = 0; c.soff = (uint32_t)ST::kAccOff; c.use = true;
  }
  return c;
}

template <int K, bool ODD, bool ACC, bool HAS_NS, int STAGES>
__global__ void __launch_bounds__(kTmaThreads, 2)
    aa_step_tma_kernel(const __grid_constant__ CUtensorMap m_even, const __grid_constant__ CUtensorMap m_wide,
                       const __grid_constant__ CUtensorMap m_row, const __grid_constant__ CUtensorMap m_mask,
                       const __grid_constant__ CUtensorMap m_acc, const StepArgs a, uint32_t ntiles) {
  using S = Store<K>;
  using T = typename S::T;
  using L = typename S::L;
  using G = TmaGeom<K>;
  using ST = TmaStage<K, ODD, ACC, HAS_NS, STAGES>;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127);
  uint64_t *bars = (uint64_t *)(smem + STAGES * ST::kBytes);
  uint2 *segtab = (uint2 *)(bars + STAGES);   // [STAGES][kTmaSegs]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (a.status && *a.status) return;   // the run is halted: the whole block leaves before any copy
  const uint32_t G0 = gridDim.x;
  const uint32_t Np = (uint32_t)a.Np;
  const uint32_t nseg = a.nseg;
  const uint2 *seg = a.seg;
  int *status = (int *)a.status;
  const LaneCopy cp = lane_copy<K, ODD, ACC, STAGES>(lane, lane < 19 ? a.off[lane] : 0, &m_even, &m_wide, &m_row,
                                                     &m_mask, &m_acc);
  const uint32_t smem_base = smem_u32(smem);

  // copies of this warp's segment of tile t into stage st (segment table entry by lane 0);
  // sgv_ is the segment entry, loaded ahead by the caller
  #define ABX_ISSUE(t_, st_, sgv_)                                                                \
    do {                                                                                          \
      const uint32_t s_ = (t_) * kTmaSegs + warp;                                                 \
      const uint2 sg_ = (sgv_);                                                                   \
      if (lane == 0) segtab[(st_) * kTmaSegs + warp] = sg_;                                       \
      if (s_ < nseg && cp.use) {                                                                  \
        const uint32_t dst_ = smem_base + (st_) * ST::kBytes +                                    \
                              (cp.soff >= (uint32_t)ST::kMaskOff                                  \
                                   ? cp.soff + warp * (cp.soff == (uint32_t)ST::kMaskOff ? 128 : 512) \
                                   : warp * ST::kPopStride + cp.soff);                            \
        const int x_ = (int)sg_.x + cp.dx;                                                        \
        const uint32_t bar_ = smem_u32(&bars[st_]);                                               \
        if ((dst_ & 127u) != 0 || (((long long)x_ * (cp.y < 0 ? 4 : (cp.soff >= (uint32_t)ST::kMaskOff ? 4 : G::kElem))) & 15) != 0) { \
          atomicExch(status, -2);                                                                 \
        } else if (cp.y < 0) {                                                                    \
          tma_load_1d(dst_, cp.map, x_, bar_);                                                    \
        } else {                                                                                  \
          tma_load_2d(dst_, cp.map, x_, cp.y, bar_);                                              \
        }                                                                                         \
      }                                                                                           \
    } while (0)

  if (threadIdx.x == 0) {
    tensormap_prefetch(ODD ? &m_wide : &m_even);
    if (ODD) tensormap_prefetch(&m_row);
    tensormap_prefetch(&m_mask);
    if (ACC) tensormap_prefetch(&m_acc);
    for (int i = 0; i < STAGES; i++) mbar_init(smem_u32(&bars[i]), 1);
    fence_barrier_init();   // initialised barriers visible to the other threads
    fence_proxy_async();    // ... and to the async proxy that completes the copies
  }
  __syncthreads();
  // prologue: the first STAGES tiles of this block (tile n = blockIdx.x + n * G0)
  if (threadIdx.x == 0)
    for (int i = 0; i < STAGES; i++) {
      const uint32_t t = blockIdx.x + i * G0;
      if (t < ntiles) mbar_expect_tx(smem_u32(&bars[i]), min((uint32_t)kTmaSegs, nseg - t * kTmaSegs) * ST::kSegBytes);
    }
  __syncthreads();
  for (int i = 0; i < STAGES; i++) {
    const uint32_t t = blockIdx.x + i * G0;
    if (t >= ntiles) break;
    const uint32_t s0 = t * kTmaSegs + warp;
    ABX_ISSUE(t, i, (s0 < nseg ? make_uint2(seg_base(seg[s0]), seg[s0].y) : make_uint2(0, 0)));
  }
  __syncthreads();   // the segment table of the first stages is visible to every lane

  const CollideParams<L> CP = make_params<L>(a);
  T *f = (T *)a.f;
  bool failed = false;
  uint32_t fail_n = 0;
  for (uint32_t n = 0;; n++) {
    const uint32_t t = blockIdx.x + n * G0;
    if (t >= ntiles) break;
    const int st = (int)(n % STAGES);
    const uint32_t parity = (n / STAGES) & 1u;
    const uint32_t bar = smem_u32(&bars[st]);
    // next use of this stage: tile n + STAGES; its segment entry is loaded now, used after the compute
    const uint32_t tn = blockIdx.x + (n + STAGES) * G0;
    const uint32_t sn = tn * kTmaSegs + warp;
    uint2 sg_next = (tn < ntiles && sn < nseg) ? seg[sn] : make_uint2(0, 0);
    sg_next.x = seg_base(sg_next);   // this kernel stages every segment's mask words
    const bool ok = mbar_wait(bar, parity);
    if (ok && threadIdx.x == 0 && tn < ntiles)
      mbar_expect_tx(bar, min((uint32_t)kTmaSegs, nseg - tn * kTmaSegs) * ST::kSegBytes);

    const uint2 sg = segtab[st * kTmaSegs + warp];
    const bool active = ok && (t * kTmaSegs + warp < nseg) && ((sg.y >> lane) & 1u);
    if (active) {
      unsigned char *base = smem + st * ST::kBytes;
      const T *sp = (const T *)(base + warp * ST::kPopStride);
      const uint32_t m = ((const uint32_t *)(base + ST::kMaskOff + warp * 128))[lane];
      const uint32_t p = sg.x + lane;
      L fi[19];
#pragma unroll
      for (int q = 0; q < 19; q++) {
        if (ODD) {
          const T *row = (const T *)((const unsigned char *)sp + G::slot_off(q));
          fi[q] = toc<K>(S::ldsr(row + (cz(q) == 0 ? lane : G::kPad + lane - cz(q))), q);
        } else {
          fi[q] = toc<K>(S::ldsr(sp + q * 32 + lane), q);
        }
      }
      if (ODD && m != 0x7FFFFu) {
#pragma unroll
        for (int q = 1; q < 19; q++)
          if (!((m >> q) & 1u)) fi[q] = toc<K>(S::ldr(f + ((uint32_t)q * Np + p)), q);  // bounce-back
      }
      const uint32_t cls = (m >> kClassShift) & 3u;
      L nsv = (L)0;
      if (HAS_NS) nsv = (L)a.ns[p];
      L fo[19], ux, uy, uz, rho;
      collide_fast<HAS_NS, S::kCollideShifted, S::kFastMath>(fi, cls, nsv, CP, fo, ux, uy, uz, rho);
#pragma unroll
      for (int q = 0; q < 19; q++) {
        uint32_t idx;
        if (ODD) idx = ((m >> opp(q)) & 1u) ? (uint32_t)q * Np + p + (uint32_t)a.off[q] : (uint32_t)opp(q) * Np + p;
        else idx = (uint32_t)opp(q) * Np + p;
        S::str(f + idx, fromc<K>(fo[q], q));
      }
      if (ACC) {
        const float *ac = (const float *)(base + ST::kAccOff + warp * 512);
        float *acc = (float *)a.acc;
        __stcs(acc + p, ac[lane] + ux);
        __stcs(acc + Np + p, ac[32 + lane] + uy);
        __stcs(acc + 2u * Np + p, ac[64 + lane] + uz);
        __stcs(acc + 3u * Np + p, ac[96 + lane] + rho);
      }
    }
    // every thread is done with stage st; a wait that gave up anywhere stops the whole block
    if (__syncthreads_or(!ok)) { failed = true; fail_n = n; break; }
    if (tn < ntiles) {
      fence_proxy_async();
      ABX_ISSUE(tn, st, sg_next);
    }
  }
  #undef ABX_ISSUE
  if (failed) {
    // A copy never completed: flag the run, record where (first block to fail),
    // and wait (bounded) for the copies this block may still have in flight
    // before its shared memory goes away.
    if (threadIdx.x == 0) {
      atomicCAS(status, 0, -1);
      if (a.diag && atomicCAS(a.diag, 0ull, 1ull) == 0ull) {
        const uint32_t t = blockIdx.x + fail_n * G0;
        a.diag[1] = blockIdx.x;
        a.diag[2] = *(volatile unsigned long long *)&bars[fail_n % STAGES];
        a.diag[3] = ntiles | ((unsigned long long)gridDim.x << 32);
        a.diag[4] = fail_n | ((unsigned long long)t << 32);
        a.diag[5] = min((uint32_t)kTmaSegs, nseg - t * kTmaSegs) * ST::kSegBytes;
        a.diag[6] = ST::kSmem | ((unsigned long long)ODD << 32) | ((unsigned long long)ACC << 33);
        a.diag[7] = nseg;
      }
    }
    for (int i = 0; i < STAGES; i++) {
      mbar_wait(smem_u32(&bars[i]), 0);
      mbar_wait(smem_u32(&bars[i]), 1);
    }
  }
}

}  // namespace abx
