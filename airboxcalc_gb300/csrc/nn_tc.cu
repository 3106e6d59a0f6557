// nn_tc.cu - the warm-start network's 3x3x3 convolutions on the tensor cores
// (tcgen05): bf16 activations and weights, float32 accumulation in tensor
// memory, operands staged by TMA, one CTA of 128 threads per output tile.
//
// Forward (and data gradient) as an implicit GEMM
//     D[m][co] = sum_{tap, ci} X[voxel(m) * s + tap - 1][ci] * W[tap][co][ci]
// M = 128 output voxels (a bw x bh x bd box of the output grid), N = Cout
// (padded to 16), K = 27 taps x Cin.  A comes from a channels-last bf16 copy of
// the input, one 5-D TMA box per (tap, 64-channel chunk): the box's outer
// coordinates are the output box's shifted by the tap, element strides give
// the stride-2 gather, and the TMA's zero fill outside the grid is the
// convolution's zero padding.  B is the tap's [Cout][Cin] weight slice.  Both
// land in the canonical K-major swizzled layout (rows of 32, 64 or 128 bytes)
// that the MMA's shared-memory descriptors describe.  The epilogue reads the
// accumulator back from tensor memory (tcgen05.ld) and writes float32
// [B][C][D][H][W] with bias, ReLU and accumulation, like nn.cu's conv3d.
// The data gradient is the same kernel on the output gradient with the
// weights flipped and transposed (stride 2: on the gradient zero-inserted to
// the input's size first).
//
// Weight gradient as a GEMM over voxels:
//     dW[tap][co][ci] = sum_v dY[co][v] * X[ci][v * s + tap - 1]
// M = 128 (Cout rows), N = Cin (padded to 16), K = one row of bw output voxels
// per pipeline stage.  A and B come from channels-first bf16 copies (voxels
// contiguous: the K-major layout here); the input copy is shifted (and, for
// stride 2, decimated) along W per tap column kx, so that every TMA box starts
// at an x coordinate that is a multiple of 8 elements (16 bytes).  One CTA per
// (tap, slice of the rows); partial sums are reduced in a fixed order.
//
// Every wait on an mbarrier is bounded; a wait that gives up records an
// error, lets the CTA skip its remaining work, waits (bounded) for the copies
// it started, frees its tensor memory and returns.  No counterpart in the
// reference (it has no learned part).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include <algorithm>

#include "lbm_iface.h"

namespace abx {
namespace tc {

// ------------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t saddr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
               : "=r"(ok)
               : "r"(bar), "r"(parity)
               : "memory");
  return ok != 0;
}
// Bounded wait: 2^22 polls, about 45 ms on GB300 (a launch whose first copies were never issued ended in 0.09 s
// with its error flag set), three orders of magnitude above any stage's copy or MMA time.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  for (int i = 0; i < (1 << 22); i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void tma_load_5d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3, int c4,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
      "%6}], [%7];" ::"r"(dst),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int c0, int c1, int c2, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(
          dst),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(bar)
      : "memory");
}
__device__ __forceinline__ void tmem_alloc(uint32_t dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem), "r"(ncols) : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// D (tensor memory) (+)= A (shared, descriptor) x B (shared, descriptor)^T, bf16 in, float32 accumulate
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
      : "memory");
}
// arrive on the mbarrier once every MMA this thread issued so far has completed
__device__ __forceinline__ void mma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
// 16 consecutive float32 columns of the warp's 32 tensor-memory lanes (one lane per thread)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, "
      "[%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Shared-memory matrix descriptor of a K-major operand whose rows are `row` bytes (32, 64 or 128) and swizzled in
// that width (the layout TMA writes with the matching swizzle mode): 8-row groups `8 * row` bytes apart; the start
// address advances by 32 bytes per K-step of 16 bf16 elements.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, int row) {
  const uint64_t layout = row == 128 ? 2 : row == 64 ? 4 : 6;   // 128-, 64-, 32-byte swizzle
  uint64_t d = 0;
  d |= (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)1 << 16;                                      // leading byte offset (unused when swizzled)
  d |= (uint64_t)(((uint32_t)(8 * row) >> 4) & 0x3FFFu) << 32; // stride byte offset: 8 rows
  d |= (uint64_t)1 << 46;                                      // descriptor version
  d |= layout << 61;
  return d;
}
// Instruction descriptor: kind::f16 with bf16 A and B, float32 D, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
__host__ __device__ constexpr int tmem_cols(int N) { return N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256; }

// ------------------------------------------------------------------ forward / data gradient
struct FwdArgs {
  float *y;              // [B][Cout][Do][Ho][Wo]
  const float *bias;     // Cout, or null
  int Cout, Do, Ho, Wo;
  int s;                 // stride
  int bw, bh, bd;        // output box of one tile (bw * bh * bd <= 128 voxels: the accumulator rows in use)
  int tw, th;            // tiles along W and H
  int nchunk;            // K chunks per tap (Cin_pad * 2 / ROW)
  int relu, accum;
  int *err;              // set to 1 when a wait gave up
  int drop;              // test hook: the K-step whose copies are never issued (-1: none), so that a wait runs out
};

// ROW: bytes of one operand row per chunk (32, 64 or 128: 16, 32 or 64 channels); N: Cout padded to 16.
template <int ROW, int N, int STAGES>
struct FwdCfg {
  static constexpr int kA = 128 * ROW, kB = N * ROW;
  static constexpr int kStage = (kA + kB + 1023) / 1024 * 1024;
  static constexpr int kSmem = STAGES * kStage + 1024;   // + alignment slack
};

template <int ROW, int N, int STAGES>
__global__ void __launch_bounds__(128, 1) conv_fwd_kernel(const __grid_constant__ CUtensorMap mapX,
                                                          const __grid_constant__ CUtensorMap mapW, const FwdArgs p) {
  using C = FwdCfg<ROW, N, STAGES>;
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long full[STAGES], empty[STAGES], accf;
  __shared__ uint32_t tmem_base;
  __shared__ int fail;
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.y;
  const int t = blockIdx.x;
  const int ox0 = (t % p.tw) * p.bw, oy0 = ((t / p.tw) % p.th) * p.bh, oz0 = (t / (p.tw * p.th)) * p.bd;
  const int nk = 27 * p.nchunk;
  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; i++) { mbar_init(saddr(&full[i]), 1); mbar_init(saddr(&empty[i]), 1); }
    mbar_init(saddr(&accf), 1);
    fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(saddr(&tmem_base), tmem_cols(N));
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  if (warp == 0 && lane == 0) {
    // producer: the A box and the W slice of every (tap, chunk)
    int armed = 0;
    for (int k = 0; k < nk; k++) {
      const int s = k % STAGES, use = k / STAGES;
      if (use > 0 && !mbar_wait(saddr(&empty[s]), (use - 1) & 1)) { fail = 1; break; }
      if (k == p.drop) continue;
      const int tap = k / p.nchunk, ch = k % p.nchunk;
      const int kz = tap / 9, ky = (tap / 3) % 3, kx = tap % 3;
      const uint32_t a = saddr(smem + s * C::kStage), bb = a + C::kA, bar = saddr(&full[s]);
      // rows of the A tile past the box (tiles of grids under 128 voxels) keep what they held: they feed only
      // accumulator rows the epilogue does not store
      mbar_expect_tx(bar, (uint32_t)(p.bw * p.bh * p.bd * ROW) + C::kB);
      tma_load_5d(a, &mapX, ch * (ROW / 2), ox0 * p.s + kx - 1, oy0 * p.s + ky - 1, oz0 * p.s + kz - 1, b, bar);
      tma_load_3d(bb, &mapW, ch * (ROW / 2), 0, tap, bar);
      armed = k + 1;
    }
    // a stopped run waits (bounded) for the copies it started, so that none lands after the CTA has gone
    if (fail)
      for (int k = armed > STAGES ? armed - STAGES : 0; k < armed; k++)
        if (k != p.drop) mbar_wait(saddr(&full[k % STAGES]), (k / STAGES) & 1);
  } else if (warp == 1 && lane == 0) {
    // MMA issuer: ROW / 32 MMAs of K = 16 per chunk
    constexpr uint32_t id = idesc_bf16(128, N);
    bool ok = true;
    for (int k = 0; k < nk; k++) {
      const int s = k % STAGES;
      if (!mbar_wait(saddr(&full[s]), (k / STAGES) & 1)) { ok = false; break; }
      tc_fence_after();
      const uint32_t a = saddr(smem + s * C::kStage), bb = a + C::kA;
#pragma unroll
      for (int j = 0; j < ROW / 32; j++)
        mma_bf16(tmem, smem_desc(a + 32 * j, ROW), smem_desc(bb + 32 * j, ROW), id, (k > 0 || j > 0) ? 1u : 0u);
      mma_commit(saddr(&empty[s]));   // the stage is free once these MMAs have read it
    }
    if (!ok) fail = 1;
    mma_commit(saddr(&accf));          // the accumulator is complete once every MMA has finished
  }
  __syncwarp();
  // epilogue: row m of the accumulator is voxel m of the tile (lane m of tensor memory)
  const bool got = mbar_wait(saddr(&accf), 0);
  tc_fence_after();
  __syncthreads();
  if (got && !fail) {
    const int m = threadIdx.x;
    const int ox = ox0 + m % p.bw, oy = oy0 + (m / p.bw) % p.bh, oz = oz0 + m / (p.bw * p.bh);
    const bool live = m < p.bw * p.bh * p.bd && ox < p.Wo && oy < p.Ho && oz < p.Do;
    const int64_t V = (int64_t)p.Do * p.Ho * p.Wo;
    const int64_t vox = ((int64_t)oz * p.Ho + oy) * p.Wo + ox;
#pragma unroll
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
      for (int j = 0; j < 16; j++) {
        const int co = c0 + j;
        if (!live || co >= p.Cout) continue;
        float r = v[j] + (p.bias ? p.bias[co] : 0.0f);
        if (p.relu && r < 0.0f) r = 0.0f;
        float *o = p.y + ((int64_t)b * p.Cout + co) * V + vox;
        *o = p.accum ? *o + r : r;
      }
    }
  } else if (threadIdx.x == 0) {
    atomicExch(p.err, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, tmem_cols(N));
}

// ------------------------------------------------------------------ weight gradient
struct WgradArgs {
  float *part;           // [nsplit][27][Cout][Cin]
  int Cout, Cin, Do, Ho, Wo, s;
  int bw;                // voxels of one K-step (a row segment): Wo, at most 64; 64 in the plane form
  int plane;             // plane form (rows narrower than 16 voxels): a K-step is 64 consecutive voxels of an output
                         // plane (64 / Wo whole rows), read through 4-D maps over flattened planes
  int nyb;               // plane form: 64-voxel blocks per output plane
  int arows, brows;      // rows of the A and B boxes (Cout, min(Cin, N)); the tiles' other rows feed only
                         // accumulator rows and columns that are not stored
  int abytes, stage;     // bytes of a stage's A region (Cout rows, whole 1024-byte swizzle atoms) and of a stage
  int rows;              // K-steps in all: B * Do * Ho * (Wo / bw), or B * Do * nyb in the plane form
  int per;               // K-steps per CTA
  int *err;
};
// A stage holds the Cout rows of A and the N rows of B.  The MMA (M = 128) reads 128 rows of A from the stage's
// start; the rows past Cout are whatever follows in shared memory (this stage's B, the next stage), which feeds
// only accumulator rows that are not stored, and the last stage is followed by 128 rows of slack.
template <int ROW, int N, int STAGES>
struct WgradCfg {
  static constexpr int kSlack = 128 * ROW + 1024;   // + alignment
  static int stage_bytes(int abytes) { return (abytes + N * ROW + 1023) / 1024 * 1024; }
  static int smem(int abytes) { return STAGES * stage_bytes(abytes) + kSlack; }
};

// grid (27, nsplit).  Row form: mapDY is the channels-first dY {Wo, Ho, Do, Cout, B}, box {bw, 1, 1, Cout, 1};
// mx.m[kx] the input copy for tap column kx, shifted by kx - 1 along W and decimated by s: {Wo, H, D, Cin, B}, box
// {bw, 1, 1, brows, 1}.  Each channel's box row is one K-major operand row of bw voxels (bw * 2 bytes = the swizzle
// span).  Plane form (rows of 8 voxels): dY as {Ho * Wo, Do, Cout, B}, box {64, 1, Cout, 1}, and mx.m[3 ky + kx] the
// input copy shifted by (ky - 1, kx - 1) and decimated by s along H and W: {Ho * Wo, D, Cin, B}, box {64, 1, brows,
// 1}: a K-step is 64 consecutive voxels of one output plane, again one 128-byte operand row per channel.  (Stacking
// several 16-byte rows of a 5-D box into one K-step does not work: a box whose inner dimension is narrower than the
// 128-byte swizzle span does not land as one dense operand row - tried: wrong sums, and the largest such box wrote
// past the stage.)
struct WgradMaps {
  CUtensorMap m[9];
};
template <int ROW, int N, int STAGES>
__global__ void __launch_bounds__(128, 1) conv_wgrad_kernel(const __grid_constant__ CUtensorMap mapDY,
                                                            const __grid_constant__ WgradMaps mx, const WgradArgs p) {
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) unsigned long long full[STAGES], empty[STAGES], accf;
  __shared__ uint32_t tmem_base;
  __shared__ int fail;
  unsigned char *smem = (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tap = blockIdx.x, split = blockIdx.y;
  const int kz = tap / 9, ky = (tap / 3) % 3, kx = tap % 3;
  const CUtensorMap *mapX = &mx.m[p.plane ? 3 * ky + kx : kx];
  const int k0 = split * p.per, k1 = p.rows < k0 + p.per ? p.rows : k0 + p.per;
  const int nk = k1 > k0 ? k1 - k0 : 0;
  const int nwb = p.Wo / p.bw;
  if (threadIdx.x == 0) {
    for (int i = 0; i < STAGES; i++) { mbar_init(saddr(&full[i]), 1); mbar_init(saddr(&empty[i]), 1); }
    mbar_init(saddr(&accf), 1);
    fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) tmem_alloc(saddr(&tmem_base), tmem_cols(N));
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;
  if (warp == 0 && lane == 0) {
    int armed = 0;
    for (int k = 0; k < nk; k++) {
      const int s = k % STAGES, use = k / STAGES;
      if (use > 0 && !mbar_wait(saddr(&empty[s]), (use - 1) & 1)) { fail = 1; break; }
      const int r = k0 + k;
      const uint32_t a = saddr(smem + s * p.stage), bb = a + p.abytes, bar = saddr(&full[s]);
      mbar_expect_tx(bar, (uint32_t)((p.arows + p.brows) * ROW));
      if (p.plane) {                            // (b, oz, 64-voxel block of the plane)
        const int yb = r % p.nyb, oz = (r / p.nyb) % p.Do, b = r / (p.nyb * p.Do);
        tma_load_4d(a, &mapDY, yb * 64, oz, 0, b, bar);
        tma_load_4d(bb, mapX, yb * 64, oz * p.s + kz - 1, 0, b, bar);
      } else {                                  // (b, oz, oy, x-chunk)
        const int xc = r % nwb, oy = (r / nwb) % p.Ho, oz = (r / (nwb * p.Ho)) % p.Do, b = r / (nwb * p.Ho * p.Do);
        tma_load_5d(a, &mapDY, xc * p.bw, oy, oz, 0, b, bar);
        tma_load_5d(bb, mapX, xc * p.bw, oy * p.s + ky - 1, oz * p.s + kz - 1, 0, b, bar);
      }
      armed = k + 1;
    }
    if (fail)
      for (int k = armed > STAGES ? armed - STAGES : 0; k < armed; k++) mbar_wait(saddr(&full[k % STAGES]), (k / STAGES) & 1);
  } else if (warp == 1 && lane == 0) {
    constexpr uint32_t id = idesc_bf16(128, N);
    bool ok = true;
    for (int k = 0; k < nk; k++) {
      const int s = k % STAGES;
      if (!mbar_wait(saddr(&full[s]), (k / STAGES) & 1)) { ok = false; break; }
      tc_fence_after();
      const uint32_t a = saddr(smem + s * p.stage), bb = a + p.abytes;
#pragma unroll
      for (int j = 0; j < ROW / 32; j++)
        mma_bf16(tmem, smem_desc(a + 32 * j, ROW), smem_desc(bb + 32 * j, ROW), id, (k > 0 || j > 0) ? 1u : 0u);
      mma_commit(saddr(&empty[s]));
    }
    if (!ok) fail = 1;
    mma_commit(saddr(&accf));
  }
  __syncwarp();
  const bool got = mbar_wait(saddr(&accf), 0);
  tc_fence_after();
  __syncthreads();
  if (got && !fail) {
    const int co = threadIdx.x;   // accumulator row = output channel
#pragma unroll
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
      if (co < p.Cout) {
#pragma unroll
        for (int j = 0; j < 16; j++) {
          const int ci = c0 + j;
          // a CTA without K-steps accumulated nothing: its partial is zero
          if (ci < p.Cin) p.part[(((int64_t)split * 27 + tap) * p.Cout + co) * p.Cin + ci] = nk > 0 ? v[j] : 0.0f;
        }
      }
    }
  } else if (threadIdx.x == 0) {
    atomicExch(p.err, 1);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) tmem_dealloc(tmem, tmem_cols(N));
}

// ------------------------------------------------------------------ layout conversions
// x [B][C][D][H][W] float32 -> [B][D][H][W][Cp] bf16, channels >= C zero.  up2: the gradient of a stride-2
// convolution zero-inserted to the input's size: voxel q holds x[q / 2] where every coordinate of q is even, zero
// elsewhere (x is then a D/2 x H/2 x W/2 grid).  Grid (voxel blocks, B); voxel indices within a sample are 32-bit
// (the host checks D * H * W < 2^31).
__global__ void to_cl_kernel(const float *__restrict__ x, __nv_bfloat16 *__restrict__ out, int C, int Cp, int D,
                             int H, int W, int up2) {
  const int Dx = up2 ? D / 2 : D, Hx = up2 ? H / 2 : H, Wx = up2 ? W / 2 : W;
  const uint32_t Vx = (uint32_t)Dx * Hx * Wx, V = (uint32_t)D * H * W, HW = (uint32_t)H * W;
  const float *xb = x + (int64_t)blockIdx.y * C * Vx;
  __nv_bfloat16 *ob = out + (int64_t)blockIdx.y * V * Cp;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
    const uint32_t w = v % (uint32_t)W, h = (v / (uint32_t)W) % (uint32_t)H, d = v / HW;
    bool on = true;
    uint32_t src = v;
    if (up2) {
      on = !(w & 1) && !(h & 1) && !(d & 1);
      src = ((d >> 1) * (uint32_t)Hx + (h >> 1)) * (uint32_t)Wx + (w >> 1);
    }
    __nv_bfloat16 *o = ob + (size_t)v * Cp;
    for (int c0 = 0; c0 < Cp; c0 += 8) {
      __align__(16) __nv_bfloat16 q[8];
#pragma unroll
      for (int j = 0; j < 8; j++) {
        const int c = c0 + j;
        q[j] = __float2bfloat16_rn((on && c < C) ? xb[(size_t)c * Vx + src] : 0.0f);
      }
      *reinterpret_cast<uint4 *>(o + c0) = *reinterpret_cast<const uint4 *>(q);
    }
  }
}

// x [B][C][D][H][W] float32 -> three bf16 copies [3][B][C][D][H][Wo]: copy kx holds x[..][s * w + kx - 1] (zero
// outside the grid), Wo = (W - 1) / s + 1.  n = B * C * D * H * Wo (the copies' stride); grid (blocks, B), indices
// within a sample 32-bit (the host checks C * D * H * W < 2^31).
__global__ void to_cf_shift_kernel(const float *__restrict__ x, __nv_bfloat16 *__restrict__ out, int64_t n,
                                   uint32_t rows, int W, int Wo, int s) {
  const uint32_t m = rows * (uint32_t)Wo;   // one sample's elements per copy
  const float *xb = x + (int64_t)blockIdx.y * rows * W;
  __nv_bfloat16 *ob = out + (int64_t)blockIdx.y * m;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += gridDim.x * blockDim.x) {
    const uint32_t r = j / (uint32_t)Wo, w = j % (uint32_t)Wo;
    const float *xr = xb + (size_t)r * W;
#pragma unroll
    for (int kx = 0; kx < 3; kx++) {
      const int src = s * (int)w + kx - 1;
      ob[kx * n + j] = __float2bfloat16_rn((src >= 0 && src < W) ? xr[src] : 0.0f);
    }
  }
}

// x [B][C][D][H][W] float32 -> nine bf16 copies [9][B][C][D][Ho][Wo]: copy 3 ky + kx holds
// x[..][s * oy + ky - 1][s * ox + kx - 1] (zero outside the grid).  n = B * C * D * Ho * Wo (the copies' stride); grid
// (blocks, B), indices within a sample 32-bit (the host checks C * D * H * W < 2^31).
__global__ void to_cf_shift9_kernel(const float *__restrict__ x, __nv_bfloat16 *__restrict__ out, int64_t n,
                                    uint32_t planes, int H, int W, int Ho, int Wo, int s) {
  const uint32_t pl = (uint32_t)Ho * Wo, m = planes * pl;   // one sample's elements per copy
  const float *xb = x + (int64_t)blockIdx.y * planes * H * W;
  __nv_bfloat16 *ob = out + (int64_t)blockIdx.y * m;
  for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += gridDim.x * blockDim.x) {
    const uint32_t q = j / pl, r = j % pl, oy = r / (uint32_t)Wo, ox = r % (uint32_t)Wo;
    const float *xp = xb + (size_t)q * H * W;
#pragma unroll
    for (int ky = 0; ky < 3; ky++) {
      const int yy = s * (int)oy + ky - 1;
#pragma unroll
      for (int kx = 0; kx < 3; kx++) {
        const int xx = s * (int)ox + kx - 1;
        const bool in = yy >= 0 && yy < H && xx >= 0 && xx < W;
        ob[(3 * ky + kx) * n + j] = __float2bfloat16_rn(in ? xp[(size_t)yy * W + xx] : 0.0f);
      }
    }
  }
}

__global__ void to_bf16_kernel(const float *__restrict__ x, __nv_bfloat16 *__restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16_rn(x[i]);
}

// w [Cout][Cin][27] float32 (the forward convolution's) -> bf16 slices [27][Np][Kp]: rows co, K = ci; or (flip) the
// data gradient's, rows ci, K = co, taps reversed.  Padding zero.
__global__ void weights_kernel(const float *__restrict__ w, __nv_bfloat16 *__restrict__ out, int Cout, int Cin, int Np,
                               int Kp, int flip) {
  const int n = 27 * Np * Kp;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int k = i % Kp, r = (i / Kp) % Np, tap = i / (Kp * Np);
    float v = 0.0f;
    if (!flip) {
      if (r < Cout && k < Cin) v = w[((int64_t)r * Cin + k) * 27 + tap];
    } else {
      if (r < Cin && k < Cout) v = w[((int64_t)k * Cin + r) * 27 + (26 - tap)];
    }
    out[i] = __float2bfloat16_rn(v);
  }
}

// dw[co][ci][tap] = sum over splits (fixed order) of part[split][tap][co][ci]
__global__ void wgrad_sum_kernel(const float *__restrict__ part, float *__restrict__ dw, int Cout, int Cin, int nsplit) {
  const int n = Cout * Cin * 27;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int tap = i % 27, ci = (i / 27) % Cin, co = i / (27 * Cin);
    float t = 0.0f;
    for (int sp = 0; sp < nsplit; sp++) t += part[(((int64_t)sp * 27 + tap) * Cout + co) * Cin + ci];
    dw[i] = t;
  }
}

// db[co] = sum over samples and voxels of dy[b][co][v], in two fixed-order passes: grid (kBiasParts, Cout) blocks
// of 256 threads each sum one slice of the voxels over every sample into part[co][slice]; then one thread per channel
// adds the slices.
constexpr int kBiasParts = 64;
__global__ void bias_part_kernel(const float *__restrict__ dy, float *__restrict__ part, int B, int Cout, int64_t V) {
  __shared__ float red[256];
  const int co = blockIdx.y, sl = blockIdx.x;
  const uint32_t lo = (uint32_t)(V * sl / kBiasParts), hi = (uint32_t)(V * (sl + 1) / kBiasParts);
  float t = 0.0f;
  for (int b = 0; b < B; b++) {
    const float *row = dy + ((int64_t)b * Cout + co) * V;
    for (uint32_t v = lo + threadIdx.x; v < hi; v += blockDim.x) t += row[v];
  }
  red[threadIdx.x] = t;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[co * kBiasParts + sl] = red[0];
}
__global__ void bias_sum_kernel(const float *__restrict__ part, float *__restrict__ db, int Cout) {
  const int co = blockIdx.x * blockDim.x + threadIdx.x;
  if (co >= Cout) return;
  float t = 0.0f;
  for (int sl = 0; sl < kBiasParts; sl++) t += part[co * kBiasParts + sl];
  db[co] = t;
}

__global__ void relu_mask_kernel(const float *__restrict__ y, float *__restrict__ dy, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (!(y[i] > 0.0f)) dy[i] = 0.0f;
}

// The output gradient's ReLU mask (when y is given) and its bf16 copy for the weight gradient in one pass, four
// elements per thread (n a multiple of 4, 16-byte aligned buffers: the host checks): dy[i] = 0 where y[i] <= 0,
// out[i] = bf16(dy[i]).
__global__ void mask_bf16_kernel(const float *__restrict__ y, float *__restrict__ dy, __nv_bfloat16 *__restrict__ out,
                                 int64_t n4) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4; i += (int64_t)gridDim.x * blockDim.x) {
    float4 d = reinterpret_cast<const float4 *>(dy)[i];
    if (y) {
      const float4 v = reinterpret_cast<const float4 *>(y)[i];
      const bool keep = (v.x > 0.0f) && (v.y > 0.0f) && (v.z > 0.0f) && (v.w > 0.0f);
      if (!keep) {
        d.x = v.x > 0.0f ? d.x : 0.0f; d.y = v.y > 0.0f ? d.y : 0.0f;
        d.z = v.z > 0.0f ? d.z : 0.0f; d.w = v.w > 0.0f ? d.w : 0.0f;
        reinterpret_cast<float4 *>(dy)[i] = d;
      }
    }
    __align__(8) __nv_bfloat16 q[4] = {__float2bfloat16_rn(d.x), __float2bfloat16_rn(d.y), __float2bfloat16_rn(d.z),
                                       __float2bfloat16_rn(d.w)};
    reinterpret_cast<uint2 *>(out)[i] = *reinterpret_cast<const uint2 *>(q);
  }
}

// ======================================================================== host side
static unsigned blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (unsigned)(b < 1 ? 1 : b);
}

static PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  }
  return fn;
}

static CUtensorMapSwizzle swizzle_of(int row) {
  return row == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : row == 64 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B;
}

// A bf16 tensor map of `rank` dimensions (innermost first); strides in bytes of dimensions 1.. .
static cudaError_t make_map(CUtensorMap *m, const void *base, int rank, const cuuint64_t *dims, const cuuint64_t *strides,
                            const cuuint32_t *box, const cuuint32_t *estr, int row) {
  auto enc = encoder();
  if (!enc) return cudaErrorNotSupported;
  const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, const_cast<void *>(base), dims, strides, box,
                         estr, CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_of(row), CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

// Channels padded for the GEMM's K: 16, 32, or a multiple of 64; the operand row width in bytes; N padded to 16.
static int k_pad(int c) { return c <= 16 ? 16 : c <= 32 ? 32 : (c + 63) / 64 * 64; }
static int k_row(int cp) { return cp == 16 ? 32 : cp == 32 ? 64 : 128; }
static int n_pad(int c) { return c <= 16 ? 16 : c <= 32 ? 32 : c <= 64 ? 64 : 128; }

constexpr int kStages = 4;
// Test hook of the forward kernel (FwdArgs::drop): -1 in every product path; the native check of the failure path
// sets it to make one K-step's copies go missing.
static int g_test_drop_kstep = -1;
// pipeline depth of the weight-gradient kernel (its stages are small: one row of voxels each)
#ifndef ABX_TC_WSTAGES
#define ABX_TC_WSTAGES 4
#endif
constexpr int kWStages = ABX_TC_WSTAGES;

template <int ROW, int N>
static cudaError_t launch_fwd(const CUtensorMap &mx, const CUtensorMap &mw, const FwdArgs &a, dim3 grid, cudaStream_t st) {
  constexpr int smem = FwdCfg<ROW, N, kStages>::kSmem;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(conv_fwd_kernel<ROW, N, kStages>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  conv_fwd_kernel<ROW, N, kStages><<<grid, 128, smem, st>>>(mx, mw, a);
  return cudaGetLastError();
}
template <int ROW>
static cudaError_t launch_fwd_n(int N, const CUtensorMap &mx, const CUtensorMap &mw, const FwdArgs &a, dim3 grid,
                                cudaStream_t st) {
  switch (N) {
    case 16: return launch_fwd<ROW, 16>(mx, mw, a, grid, st);
    case 32: return launch_fwd<ROW, 32>(mx, mw, a, grid, st);
    case 64: return launch_fwd<ROW, 64>(mx, mw, a, grid, st);
    case 128: return launch_fwd<ROW, 128>(mx, mw, a, grid, st);
  }
  return cudaErrorInvalidValue;
}

template <int ROW, int N>
static cudaError_t launch_wgrad(const CUtensorMap &mdy, const WgradMaps &mx, const WgradArgs &a, dim3 grid,
                                cudaStream_t st) {
  using C = WgradCfg<ROW, N, kWStages>;
  const int smem = C::smem(a.abytes);
  static int attr = 0;   // the largest dynamic shared memory set so far for this instantiation
  if (smem > attr) {
    cudaError_t e =
        cudaFuncSetAttribute(conv_wgrad_kernel<ROW, N, kWStages>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    attr = smem;
  }
  WgradArgs b = a;
  b.stage = C::stage_bytes(a.abytes);
  conv_wgrad_kernel<ROW, N, kWStages><<<grid, 128, smem, st>>>(mdy, mx, b);
  return cudaGetLastError();
}
template <int ROW>
static cudaError_t launch_wgrad_n(int N, const CUtensorMap &mdy, const WgradMaps &mx, const WgradArgs &a, dim3 grid,
                                  cudaStream_t st) {
  switch (N) {
    case 16: return launch_wgrad<ROW, 16>(mdy, mx, a, grid, st);
    case 32: return launch_wgrad<ROW, 32>(mdy, mx, a, grid, st);
    case 64: return launch_wgrad<ROW, 64>(mdy, mx, a, grid, st);
    case 128: return launch_wgrad<ROW, 128>(mdy, mx, a, grid, st);
  }
  return cudaErrorInvalidValue;
}

// One convolution y (+)= conv(x) through the forward kernel: x [B][Cin][D][H][W] float32 is copied channels-last
// (zero-inserted to D x H x W first when up2), the weights into bf16 slices (flipped and transposed when flip).
static cudaError_t conv_forward(const float *x, int Cin, bool up2, const float *w, bool flip, const float *bias, float *y,
                                int B, int Cout, int D, int H, int W, int s, int relu, int accum, const TcScratch &sc,
                                cudaStream_t st) {
  const int Kp = k_pad(Cin), row = k_row(Kp), N = n_pad(Cout);
  if (Cout > 128 || Kp > 128) return cudaErrorInvalidValue;
  if ((int64_t)B * D * H * W * Kp > sc.cl_elems || (int64_t)27 * N * Kp > sc.w_elems) return cudaErrorInvalidValue;
  // flip: this call is the data gradient of the convolution whose weights w are [Cout_f][Cin_f][27] with
  // Cout_f = Cin (the gradient's input channels) and Cin_f = Cout; weights_kernel takes the forward's sizes
  weights_kernel<<<blocks_for((int64_t)27 * N * Kp), 256, 0, st>>>(w, sc.w, flip ? Cin : Cout, flip ? Cout : Cin, N, Kp,
                                                                  flip ? 1 : 0);
  if ((int64_t)D * H * W >= (1ll << 31)) return cudaErrorInvalidValue;
  to_cl_kernel<<<dim3(blocks_for((int64_t)D * H * W), (unsigned)B), 256, 0, st>>>(x, sc.cl, Cin, Kp, D, H, W, up2 ? 1 : 0);
  const int Do = (D - 1) / s + 1, Ho = (H - 1) / s + 1, Wo = (W - 1) / s + 1;
  FwdArgs a{};
  a.y = y; a.bias = bias; a.Cout = Cout; a.Do = Do; a.Ho = Ho; a.Wo = Wo; a.s = s;
  a.bw = std::min(Wo, 128); a.bh = std::min(Ho, 128 / a.bw); a.bd = std::min(Do, 128 / (a.bw * a.bh));
  a.tw = (Wo + a.bw - 1) / a.bw; a.th = (Ho + a.bh - 1) / a.bh;
  const int td = (Do + a.bd - 1) / a.bd;
  a.nchunk = Kp * 2 / row;
  a.relu = relu; a.accum = accum; a.err = sc.err; a.drop = g_test_drop_kstep;
  CUtensorMap mx, mw;
  {
    const cuuint64_t dims[5] = {(cuuint64_t)Kp, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)D, (cuuint64_t)B};
    const cuuint64_t strides[4] = {(cuuint64_t)Kp * 2, (cuuint64_t)Kp * 2 * W, (cuuint64_t)Kp * 2 * W * H,
                                   (cuuint64_t)Kp * 2 * W * H * D};
    const cuuint32_t box[5] = {(cuuint32_t)(row / 2), (cuuint32_t)(a.bw * s), (cuuint32_t)(a.bh * s),
                               (cuuint32_t)(a.bd * s), 1};
    const cuuint32_t estr[5] = {1, (cuuint32_t)s, (cuuint32_t)s, (cuuint32_t)s, 1};
    cudaError_t e = make_map(&mx, sc.cl, 5, dims, strides, box, estr, row);
    if (e != cudaSuccess) return e;
  }
  {
    const cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)N, 27};
    const cuuint64_t strides[2] = {(cuuint64_t)Kp * 2, (cuuint64_t)Kp * 2 * N};
    const cuuint32_t box[3] = {(cuuint32_t)(row / 2), (cuuint32_t)N, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    cudaError_t e = make_map(&mw, sc.w, 3, dims, strides, box, estr, row);
    if (e != cudaSuccess) return e;
  }
  const dim3 grid((unsigned)(a.tw * a.th * td), (unsigned)B);
  switch (row) {
    case 32: return launch_fwd_n<32>(N, mx, mw, a, grid, st);
    case 64: return launch_fwd_n<64>(N, mx, mw, a, grid, st);
    case 128: return launch_fwd_n<128>(N, mx, mw, a, grid, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace tc

bool nn_tc_available() {
  int dev = 0, major = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return false;
  if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess) return false;
  return major == 10 && tc::encoder() != nullptr;
}

// CTAs per tap of the weight-gradient kernel (each sums a slice of the K-steps into its own partial; 27 x 48 CTAs
// fill the 152 SMs several times over; 96 measured the same at 64^3 and 32^3, 144 slower)
#ifndef ABX_TC_WSPLITS
#define ABX_TC_WSPLITS 48
#endif
int tc_wgrad_splits() { return ABX_TC_WSPLITS; }

void nn_tc_need(int B, int Cin, int Cout, int D, int s, TcNeed *n) {
  const int64_t V = (int64_t)D * D * D;
  const int Do = (D - 1) / s + 1;
  const int64_t Vo = (int64_t)Do * Do * Do;
  const int kf = tc::k_pad(Cin), kb = tc::k_pad(Cout);
  n->cl_elems = std::max(n->cl_elems, (int64_t)B * V * std::max(kf, kb));
  n->w_elems = std::max(n->w_elems, (int64_t)27 * std::max(tc::n_pad(Cout) * kf, tc::n_pad(Cin) * kb));
  n->xs_elems = std::max(n->xs_elems, std::max((int64_t)3 * B * Cin * D * D * Do, (int64_t)9 * B * Cin * D * Do * Do));
  n->dyc_elems = std::max(n->dyc_elems, (int64_t)B * Cout * Vo);
  n->part_floats = std::max(n->part_floats, (int64_t)std::max(tc_wgrad_splits() * 27 * Cin, tc::kBiasParts) * Cout);
}

cudaError_t nn_tc_conv3d(const float *x, const float *w, const float *b, float *y, int B, int Cin, int Cout, int D, int H,
                         int W, int s, int relu, int accum, const TcScratch &sc, cudaStream_t st) {
  if (B <= 0 || B > 65535 || Cin <= 0 || Cout <= 0 || D <= 0 || H <= 0 || W <= 0 || (s != 1 && s != 2))
    return cudaErrorInvalidValue;
  return tc::conv_forward(x, Cin, false, w, false, b, y, B, Cout, D, H, W, s, relu, accum, sc, st);
}

cudaError_t nn_tc_conv3d_backward(const float *x, const float *w, const float *y, float *dy, float *dx, float *dw,
                                  float *db, float *part, int64_t part_floats, int B, int Cin, int Cout, int D, int H,
                                  int W, int s, int relu, int accum_dx, const TcScratch &sc, cudaStream_t st) {
  if (B <= 0 || B > 65535 || Cin <= 0 || Cout <= 0 || D <= 0 || H <= 0 || W <= 0 || (s != 1 && s != 2))
    return cudaErrorInvalidValue;
  if (s == 2 && ((D | H | W) & 1)) return cudaErrorInvalidValue;
  const int Do = (D - 1) / s + 1, Ho = (H - 1) / s + 1, Wo = (W - 1) / s + 1;
  const int64_t Vo = (int64_t)Do * Ho * Wo;
  const int bw = std::min(Wo, 64);
  const bool row_form = (bw == 16 || bw == 32 || bw == 64) && Wo % bw == 0;
  const bool plane_form = !row_form && Wo < 16 && (Ho * Wo) % 64 == 0;
  const bool tc_wgrad = Cout <= 128 && (row_form || plane_form);
  const int64_t ny = (int64_t)B * Cout * Vo;
  // ReLU mask and (for the tensor-core weight gradient) the bf16 copy of the output gradient: one vectorised pass
  // where the sizes and addresses allow, else two
  const bool fused = tc_wgrad && ny % 4 == 0 && ny <= sc.dyc_elems &&
                     (((uintptr_t)dy | (uintptr_t)y | (uintptr_t)sc.dyc) & 15) == 0;
  if (fused)
    tc::mask_bf16_kernel<<<tc::blocks_for(ny / 4), 256, 0, st>>>(relu ? y : nullptr, dy, sc.dyc, ny / 4);
  else if (relu)
    tc::relu_mask_kernel<<<tc::blocks_for(ny), 256, 0, st>>>(y, dy, ny);
  // data gradient: the forward kernel on dy (zero-inserted for stride 2) with flipped, transposed weights
  if (dx) {
    cudaError_t e = tc::conv_forward(dy, Cout, s == 2, w, true, nullptr, dx, B, Cin, D, H, W, 1, 0, accum_dx, sc, st);
    if (e != cudaSuccess) return e;
  }
  // weight and bias gradients: K-steps of one row segment of 16, 32 or 64 voxels (row form), or of 64 voxels of an
  // output plane of rows narrower than 16 voxels (plane form)
  if (tc_wgrad) {
    const int N = tc::n_pad(Cin), row = row_form ? bw * 2 : 128;
    const int64_t nxs = row_form ? (int64_t)3 * B * Cin * D * H * Wo : (int64_t)9 * B * Cin * D * Ho * Wo;
    if (nxs > sc.xs_elems || (int64_t)B * Cout * Vo > sc.dyc_elems) return cudaErrorInvalidValue;
    if ((int64_t)Cin * D * H * W >= (1ll << 31)) return cudaErrorInvalidValue;
    if (!fused) tc::to_bf16_kernel<<<tc::blocks_for(ny), 256, 0, st>>>(dy, sc.dyc, ny);
    CUtensorMap mdy{};
    tc::WgradMaps mx{};
    const cuuint32_t brows = (cuuint32_t)std::min(Cin, N);
    if (row_form) {
      const int64_t rows_x = (int64_t)B * Cin * D * H;
      tc::to_cf_shift_kernel<<<dim3(tc::blocks_for(rows_x / B * Wo), (unsigned)B), 256, 0, st>>>(
          x, sc.xs, rows_x * Wo, (uint32_t)(rows_x / B), W, Wo, s);
      const cuuint64_t dims[5] = {(cuuint64_t)Wo, (cuuint64_t)Ho, (cuuint64_t)Do, (cuuint64_t)Cout, (cuuint64_t)B};
      const cuuint64_t strides[4] = {(cuuint64_t)Wo * 2, (cuuint64_t)Wo * Ho * 2, (cuuint64_t)Vo * 2, (cuuint64_t)Vo * Cout * 2};
      const cuuint32_t box[5] = {(cuuint32_t)bw, 1, 1, (cuuint32_t)Cout, 1};
      const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
      cudaError_t e = tc::make_map(&mdy, sc.dyc, 5, dims, strides, box, estr, row);
      if (e != cudaSuccess) return e;
      for (int kx = 0; kx < 3; kx++) {
        const cuuint64_t xdims[5] = {(cuuint64_t)Wo, (cuuint64_t)H, (cuuint64_t)D, (cuuint64_t)Cin, (cuuint64_t)B};
        const cuuint64_t xstrides[4] = {(cuuint64_t)Wo * 2, (cuuint64_t)Wo * H * 2, (cuuint64_t)Wo * H * D * 2,
                                        (cuuint64_t)Wo * H * D * Cin * 2};
        const cuuint32_t xbox[5] = {(cuuint32_t)bw, 1, 1, brows, 1};
        e = tc::make_map(&mx.m[kx], sc.xs + (int64_t)kx * rows_x * Wo, 5, xdims, xstrides, xbox, estr, row);
        if (e != cudaSuccess) return e;
      }
    } else {
      const int64_t n9 = (int64_t)B * Cin * D * Ho * Wo, pl = (int64_t)Ho * Wo;
      tc::to_cf_shift9_kernel<<<dim3(tc::blocks_for(n9 / B), (unsigned)B), 256, 0, st>>>(
          x, sc.xs, n9, (uint32_t)(Cin * D), H, W, Ho, Wo, s);
      const cuuint64_t dims[4] = {(cuuint64_t)pl, (cuuint64_t)Do, (cuuint64_t)Cout, (cuuint64_t)B};
      const cuuint64_t strides[3] = {(cuuint64_t)pl * 2, (cuuint64_t)Vo * 2, (cuuint64_t)Vo * Cout * 2};
      const cuuint32_t box[4] = {64, 1, (cuuint32_t)Cout, 1};
      const cuuint32_t estr[4] = {1, 1, 1, 1};
      cudaError_t e = tc::make_map(&mdy, sc.dyc, 4, dims, strides, box, estr, row);
      if (e != cudaSuccess) return e;
      for (int c = 0; c < 9; c++) {
        const cuuint64_t xdims[4] = {(cuuint64_t)pl, (cuuint64_t)D, (cuuint64_t)Cin, (cuuint64_t)B};
        const cuuint64_t xstrides[3] = {(cuuint64_t)pl * 2, (cuuint64_t)pl * D * 2, (cuuint64_t)pl * D * Cin * 2};
        const cuuint32_t xbox[4] = {64, 1, brows, 1};
        e = tc::make_map(&mx.m[c], sc.xs + (int64_t)c * n9, 4, xdims, xstrides, xbox, estr, row);
        if (e != cudaSuccess) return e;
      }
    }
    tc::WgradArgs a{};
    a.part = sc.part; a.Cout = Cout; a.Cin = Cin; a.Do = Do; a.Ho = Ho; a.Wo = Wo; a.s = s; a.bw = row_form ? bw : 64;
    a.plane = plane_form ? 1 : 0; a.nyb = plane_form ? Ho * Wo / 64 : 0;
    a.arows = Cout; a.brows = std::min(Cin, N);
    a.abytes = (Cout * row + 1023) / 1024 * 1024;
    a.rows = plane_form ? B * Do * a.nyb : B * Do * Ho * (Wo / bw);
    const int nsplit = std::min(tc_wgrad_splits(), a.rows);
    a.per = (a.rows + nsplit - 1) / nsplit;
    a.err = sc.err;
    if ((int64_t)nsplit * 27 * Cout * Cin > sc.part_floats) return cudaErrorInvalidValue;
    const dim3 grid(27, (unsigned)nsplit);
    cudaError_t e;
    switch (row) {
      case 32: e = tc::launch_wgrad_n<32>(N, mdy, mx, a, grid, st); break;
      case 64: e = tc::launch_wgrad_n<64>(N, mdy, mx, a, grid, st); break;
      case 128: e = tc::launch_wgrad_n<128>(N, mdy, mx, a, grid, st); break;
      default: e = cudaErrorInvalidValue;
    }
    if (e != cudaSuccess) return e;
    tc::wgrad_sum_kernel<<<tc::blocks_for((int64_t)Cout * Cin * 27), 256, 0, st>>>(sc.part, dw, Cout, Cin, nsplit);
    // the bias partials reuse the weight-gradient scratch after the sums above have read it (same stream)
    tc::bias_part_kernel<<<dim3(tc::kBiasParts, Cout), 256, 0, st>>>(dy, sc.part, B, Cout, Vo);
    tc::bias_sum_kernel<<<(Cout + 127) / 128, 128, 0, st>>>(sc.part, db, Cout);
    return cudaGetLastError();
  }
  // other shapes (planes of fewer than 64 voxels, more than 128 output channels): the float32 kernels (the ReLU
  // mask is already applied)
  return nn_conv3d_backward(x, w, y, dy, nullptr, dw, db, part, part_floats, B, Cin, Cout, D, H, W, s, 0, 0, st);
}

}  // namespace abx
