// d3q19.cuh - D3Q19 lattice, population storage formats and the collision of
// one cell, shared by the step-kernel translation units.
//
// Lattice tables: src/engine.js:4-12 (velocity set CX/CY/CZ, weights WT,
// opposite directions OPP).  Collision: cpuStep, src/engine.js:277-319 (the
// WGSL lbm_step, :395-444, is the same arithmetic in f32).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace abx {

__host__ __device__ constexpr int cx(int q) {
  return q == 1 || q == 7 || q == 9 || q == 11 || q == 13 ? 1 : q == 2 || q == 8 || q == 10 || q == 12 || q == 14 ? -1 : 0;
}
__host__ __device__ constexpr int cy(int q) {
  return q == 3 || q == 7 || q == 10 || q == 15 || q == 17 ? 1 : q == 4 || q == 8 || q == 9 || q == 16 || q == 18 ? -1 : 0;
}
__host__ __device__ constexpr int cz(int q) {
  return q == 5 || q == 11 || q == 14 || q == 15 || q == 18 ? 1 : q == 6 || q == 12 || q == 13 || q == 16 || q == 17 ? -1 : 0;
}
__host__ __device__ constexpr int opp(int q) { return q == 0 ? 0 : ((q & 1) ? q + 1 : q - 1); }
// weight class: 0 -> 1/3, 1..6 -> 1/18, 7..18 -> 1/36
__host__ __device__ constexpr int wclass(int q) { return q == 0 ? 0 : (q <= 6 ? 1 : 2); }

// Cell mask word (one uint32 per padded cell):
//   bits 0..18  direction q's pull neighbour x - c_q is fluid (bit 0: the cell itself is fluid)
//   bits 19..20 boundary class (src/engine.js:252-254): 0 bulk, 1 inlet, 2 outlet, 3 filter
constexpr uint32_t kFluidBit = 1u;
constexpr int kClassShift = 19;
constexpr uint32_t kClsBulk = 0, kClsInlet = 1, kClsOutlet = 2, kClsFilter = 3;
// mask word of a bulk cell whose 18 pull neighbours are all fluid
constexpr uint32_t kMaskInterior = 0x7FFFFu;
// Segment entry {base | flag, lane mask}: bit 31 of the base marks a segment whose fluid cells all have the
// mask word kMaskInterior (the step kernels then skip the mask load).  Bases stay below 2^31 (19 Np < 2^32).
constexpr uint32_t kSegInterior = 0x80000000u;
__host__ __device__ __forceinline__ uint32_t seg_base(uint2 s) { return s.x & ~kSegInterior; }

// Storage formats of the populations.  Shifted formats hold f - w_q.
enum StoreKind { kStoreF32 = 0, kStoreF32Exact = 1, kStoreF16 = 2, kStoreBF16 = 3, kStoreF64 = 4 };

// Reciprocal and square root of collide_fast: correctly rounded, or (FAST) the hardware approximations
// (rcp.approx / sqrt.approx: about one unit in the last place, one MUFU instruction instead of an iteration
// with a special-case branch).  The 16-bit storages take FAST (ABX_FAST_MATH16, default 1): their kernels are
// short of issue slots and their stored values carry 11 or 8 significant bits (config2 float16 step 38.8 ->
// 37.0 us); the float32 kernels keep the correctly rounded forms (no gain there: config3 1038 vs 1049 us).
#ifndef ABX_FAST_MATH16
#define ABX_FAST_MATH16 1
#endif

template <int K> struct Store;
// Cache hints for the float32 populations.  A population written by a step is read only by the next step,
// so stores are marked evict-first; loads stay default: the odd step's neighbour pulls read each line from
// up to three warps (neighbouring columns), and evict-first loads dropped lines before those re-reads
// (config3: 1224 vs 1103 us per step).  0: no hints; 1 (default): evict-first stores; 2: evict-first
// loads and stores.
#ifndef ABX_CACHE_HINTS
#define ABX_CACHE_HINTS 1
#endif
// ld/st address global memory; lds reads a value staged in shared memory.
// Every format also has raw accessors (ldr / ldsr / str) that the step kernels use: the stored value itself,
// i.e. f for the plain formats and h = f - w_q for the shifted ones (whose collision then works on h).
// Collision convention of every format: kCollideShifted - the float32 collision works on h = f - w_q (toc maps a
// stored value to it, fromc back); kFastMath - approximate reciprocal and square root in that collision.
// float32 storage keeps f itself but collides on h: the density and stress sums of values near w_q then keep
// the small deviations that carry rho - 1 (colliding on f loses them to the rounding of sums near 1: on a
// 512x256x384-cell airbox the time-averaged rho - 1 came out 1.9e-3 (relative L2) off the float64 run, against
// 1e-5 with cpuStep's float64 arithmetic on the same float32 storage).
template <> struct Store<kStoreF32> {
  using T = float; using L = float; using Acc = float;
  static constexpr bool kShifted = false;
  static constexpr bool kCollideShifted = true, kFastMath = false;
  __device__ static __forceinline__ L lds(const T *p, L) { return *p; }
  __device__ static __forceinline__ L ldsr(const T *p) { return *p; }
#if ABX_CACHE_HINTS == 2
  __device__ static __forceinline__ L ld(const T *p, L) { return __ldcs(p); }
#else
  __device__ static __forceinline__ L ld(const T *p, L) { return *p; }
#endif
#if ABX_CACHE_HINTS >= 1
  __device__ static __forceinline__ void st(T *p, L v, L) { __stcs(p, v); }
#else
  __device__ static __forceinline__ void st(T *p, L v, L) { *p = v; }
#endif
  __device__ static __forceinline__ L ldr(const T *p) { return ld(p, 0.0f); }
  __device__ static __forceinline__ void str(T *p, L v) { st(p, v, 0.0f); }
};
template <> struct Store<kStoreF32Exact> {
  using T = float; using L = double; using Acc = float;
  static constexpr bool kShifted = false;
  static constexpr bool kCollideShifted = false, kFastMath = false;
  __device__ static __forceinline__ L lds(const T *p, L) { return (L)*p; }
  __device__ static __forceinline__ L ld(const T *p, L) { return (L)*p; }
  __device__ static __forceinline__ void st(T *p, L v, L) { *p = (float)v; }
  __device__ static __forceinline__ L ldsr(const T *p) { return (L)*p; }
  __device__ static __forceinline__ L ldr(const T *p) { return (L)*p; }
  __device__ static __forceinline__ void str(T *p, L v) { *p = (float)v; }
};
template <> struct Store<kStoreF16> {
  using T = __half; using L = float; using Acc = float;
  static constexpr bool kShifted = true;
  static constexpr bool kCollideShifted = true, kFastMath = ABX_FAST_MATH16;
  __device__ static __forceinline__ L lds(const T *p, L w) { return w + __half2float(*p); }
  __device__ static __forceinline__ L ld(const T *p, L w) { return w + __half2float(*p); }
  __device__ static __forceinline__ void st(T *p, L v, L w) { *p = __float2half_rn(v - w); }
  __device__ static __forceinline__ L ldsr(const T *p) { return __half2float(*p); }
  __device__ static __forceinline__ L ldr(const T *p) { return __half2float(*p); }
  __device__ static __forceinline__ void str(T *p, L h) { *p = __float2half_rn(h); }
};
template <> struct Store<kStoreBF16> {
  using T = __nv_bfloat16; using L = float; using Acc = float;
  static constexpr bool kShifted = true;
  static constexpr bool kCollideShifted = true, kFastMath = ABX_FAST_MATH16;
  __device__ static __forceinline__ L lds(const T *p, L w) { return w + __bfloat162float(*p); }
  __device__ static __forceinline__ L ld(const T *p, L w) { return w + __bfloat162float(*p); }
  __device__ static __forceinline__ void st(T *p, L v, L w) { *p = __float2bfloat16_rn(v - w); }
  __device__ static __forceinline__ L ldsr(const T *p) { return __bfloat162float(*p); }
  __device__ static __forceinline__ L ldr(const T *p) { return __bfloat162float(*p); }
  __device__ static __forceinline__ void str(T *p, L h) { *p = __float2bfloat16_rn(h); }
};
template <> struct Store<kStoreF64> {
  using T = double; using L = double; using Acc = double;
  static constexpr bool kShifted = false;
  static constexpr bool kCollideShifted = false, kFastMath = false;
  __device__ static __forceinline__ L lds(const T *p, L) { return *p; }
  __device__ static __forceinline__ L ld(const T *p, L) { return *p; }
  __device__ static __forceinline__ void st(T *p, L v, L) { *p = v; }
  __device__ static __forceinline__ L ldsr(const T *p) { return *p; }
  __device__ static __forceinline__ L ldr(const T *p) { return *p; }
  __device__ static __forceinline__ void str(T *p, L v) { *p = v; }
};

template <class L> __device__ __forceinline__ L weight(int q) {
  return wclass(q) == 0 ? (L)1 / (L)3 : (wclass(q) == 1 ? (L)1 / (L)18 : (L)1 / (L)36);
}

// Stored value of direction q -> the value the collision works on, and back (see kCollideShifted).
template <int K, class L> __device__ __forceinline__ L toc(L raw, int q) {
  if constexpr (Store<K>::kCollideShifted && !Store<K>::kShifted) return raw - weight<L>(q);
  else return raw;
}
template <int K, class L> __device__ __forceinline__ L fromc(L v, int q) {
  if constexpr (Store<K>::kCollideShifted && !Store<K>::kShifted) return v + weight<L>(q);
  else return v;
}

// c_q . u with the zero components left out: exactly the value of
// CX*ux + CY*uy + CZ*uz in src/engine.js:288 for finite u.
template <class L> __device__ __forceinline__ L cdot(int q, L ux, L uy, L uz) {
  L s = (L)0;
  bool first = true;
  if (cx(q) != 0) { s = cx(q) > 0 ? ux : -ux; first = false; }
  if (cy(q) != 0) { const L t = cy(q) > 0 ? uy : -uy; s = first ? t : s + t; first = false; }
  if (cz(q) != 0) { const L t = cz(q) > 0 ? uz : -uz; s = first ? t : s + t; }
  return s;
}

template <class L> struct CollideParams {
  L u0, tau0, sig, aniso, cs2s;
};

// Collision of one cell (src/engine.js:277-319): moments, inlet (Zou/He
// density from the populations coming from the interior, u = (0,0,u0)),
// outlet (rho = 1, local u), Smagorinsky tau from the non-equilibrium stress,
// anisotropic filter velocity shift, BGK, optional partial bounce-back.
// The operation order is cpuStep's, so with L = double and no contraction
// the result is cpuStep's bit for bit.  On return (ux,uy,uz,rho) are the
// values cpuStep adds to the averages.
template <class L, bool HAS_NS>
__device__ __forceinline__ void collide(const L (&fi)[19], uint32_t cls, L nsv, const CollideParams<L> &P,
                                        L (&fo)[19], L &ux, L &uy, L &uz, L &rho) {
  rho = (L)0;
  L mx = (L)0, my = (L)0, mz = (L)0;
#pragma unroll
  for (int q = 0; q < 19; q++) {
    rho += fi[q];
    if (cx(q) != 0) mx = cx(q) > 0 ? mx + fi[q] : mx - fi[q];
    if (cy(q) != 0) my = cy(q) > 0 ? my + fi[q] : my - fi[q];
    if (cz(q) != 0) mz = cz(q) > 0 ? mz + fi[q] : mz - fi[q];
  }
  ux = mx / rho; uy = my / rho; uz = mz / rho;
  if (cls == kClsInlet || cls == kClsOutlet) {
    if (cls == kClsInlet) {
      L s0 = (L)0, sm = (L)0;
#pragma unroll
      for (int q = 0; q < 19; q++) {
        if (cz(q) == 0) s0 += fi[q];
        else if (cz(q) < 0) sm += fi[q];
      }
      rho = (s0 + (L)2 * sm) / ((L)1 - P.u0);
      ux = (L)0; uy = (L)0; uz = P.u0;
    } else {
      rho = (L)1;
    }
    const L usq = (L)1.5 * (ux * ux + uy * uy + uz * uz);
#pragma unroll
    for (int q = 0; q < 19; q++) {
      const L cu = (L)3 * cdot<L>(q, ux, uy, uz);
      fo[q] = weight<L>(q) * rho * ((L)1 + cu + (L)0.5 * cu * cu - usq);
    }
    return;
  }
  L fe[19];
  L usq = (L)1.5 * (ux * ux + uy * uy + uz * uz);
  L pxx = (L)0, pyy = (L)0, pzz = (L)0, pxy = (L)0, pxz = (L)0, pyz = (L)0;
#pragma unroll
  for (int q = 0; q < 19; q++) {
    const L cu = (L)3 * cdot<L>(q, ux, uy, uz);
    const L e = weight<L>(q) * rho * ((L)1 + cu + (L)0.5 * cu * cu - usq);
    fe[q] = e;
    const L ne = fi[q] - e;
    if (cx(q) != 0) pxx += ne;
    if (cy(q) != 0) pyy += ne;
    if (cz(q) != 0) pzz += ne;
    if (cx(q) * cy(q) != 0) pxy = cx(q) * cy(q) > 0 ? pxy + ne : pxy - ne;
    if (cx(q) * cz(q) != 0) pxz = cx(q) * cz(q) > 0 ? pxz + ne : pxz - ne;
    if (cy(q) * cz(q) != 0) pyz = cy(q) * cz(q) > 0 ? pyz + ne : pyz - ne;
  }
  const L Qn = sqrt(pxx * pxx + pyy * pyy + pzz * pzz + (L)2 * (pxy * pxy + pxz * pxz + pyz * pyz));
  const L tau = (L)0.5 * (P.tau0 + sqrt(P.tau0 * P.tau0 + P.cs2s * Qn / rho));
  if (cls == kClsFilter) {
    const L a1 = tau * P.sig * P.aniso, a2 = tau * P.sig;
    // Math.min(a, 0.9): a NaN coefficient (e.g. sigma = 0/0 with zero inflow) propagates as in the reference
    const L sl = (L)1 - (a1 >= (L)0.9 ? (L)0.9 : a1), sv = (L)1 - (a2 >= (L)0.9 ? (L)0.9 : a2);
    const L ex = ux * sl, ey = uy * sv, ez = uz * sl;
    usq = (L)1.5 * (ex * ex + ey * ey + ez * ez);
#pragma unroll
    for (int q = 0; q < 19; q++) {
      const L cu = (L)3 * cdot<L>(q, ex, ey, ez);
      fe[q] = weight<L>(q) * rho * ((L)1 + cu + (L)0.5 * cu * cu - usq);
    }
    ux = (L)0.5 * (ux + ex); uy = (L)0.5 * (uy + ey); uz = (L)0.5 * (uz + ez);
  }
  const L it = (L)1 / tau;
  if (HAS_NS && nsv > (L)0) {
#pragma unroll
    for (int q = 0; q < 19; q++) fo[q] = ((L)1 - nsv) * (fi[q] - (fi[q] - fe[q]) * it) + nsv * fi[opp(q)];
    ux *= (L)1 - nsv; uy *= (L)1 - nsv; uz *= (L)1 - nsv;
  } else {
#pragma unroll
    for (int q = 0; q < 19; q++) fo[q] = fi[q] - (fi[q] - fe[q]) * it;
  }
}

template <bool FAST> __device__ __forceinline__ float cf_rcp(float x) {
  if constexpr (FAST) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
  } else {
    return 1.0f / x;
  }
}
template <bool FAST> __device__ __forceinline__ float cf_sqrt(float x) {
  if constexpr (FAST) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
  } else {
    return sqrtf(x);
  }
}

// The same collision in float32 with the algebra rearranged for the GPU:
// moments and the stress tensor from the nine opposite-pair sums s and
// differences d (f_q +- f_opp(q)), the non-equilibrium stress as
// Pi(f) - rho/3 I - j u (the second moment of the quadratic equilibrium is
// exactly rho/3 I + rho u u on D3Q19), and equilibrium plus BGK per opposite
// pair from a shared even part and an odd part.  Same model as collide();
// about a third of its arithmetic.
template <bool HAS_NS, bool SHIFTED = false, bool FAST = false>
__device__ __forceinline__ void collide_fast(const float (&f)[19], uint32_t cls, float nsv_in,
                                             const CollideParams<float> &P, float (&fo)[19], float &ux, float &uy,
                                             float &uz, float &rho) {
  // partial bounce-back acts on bulk and filter cells only (src/engine.js:313-317)
  const float nsv = (HAS_NS && (cls == kClsBulk || cls == kClsFilter) && nsv_in > 0.0f) ? nsv_in : 0.0f;
  // opposite pairs: (1,2) x, (3,4) y, (5,6) z, (7,8) +x+y, (9,10) +x-y,
  // (11,12) +x+z, (13,14) +x-z, (15,16) +y+z, (17,18) +y-z
  const float s1 = f[1] + f[2], d1 = f[1] - f[2];
  const float s3 = f[3] + f[4], d3 = f[3] - f[4];
  const float s5 = f[5] + f[6], d5 = f[5] - f[6];
  const float s7 = f[7] + f[8], d7 = f[7] - f[8];
  const float s9 = f[9] + f[10], d9 = f[9] - f[10];
  const float s11 = f[11] + f[12], d11 = f[11] - f[12];
  const float s13 = f[13] + f[14], d13 = f[13] - f[14];
  const float s15 = f[15] + f[16], d15 = f[15] - f[16];
  const float s17 = f[17] + f[18], d17 = f[17] - f[18];
  const float sxy = s7 + s9, sxz = s11 + s13, syz = s15 + s17;
  // SHIFTED: f holds h = f - w_q; the weights add 1 to the density and 1/3 to each diagonal stress sum and
  // cancel from every odd moment
  const float tot = f[0] + ((s1 + s3) + s5) + ((sxy + sxz) + syz);
  rho = SHIFTED ? 1.0f + tot : tot;
  const float jx = d1 + (d7 + d9) + (d11 + d13);
  const float jy = d3 + (d7 - d9) + (d15 + d17);
  const float jz = d5 + (d11 - d13) + (d15 - d17);
  const float inv = cf_rcp<FAST>(rho);
  ux = jx * inv; uy = jy * inv; uz = jz * inv;
  float vx = ux, vy = uy, vz = uz;   // velocity of the equilibrium
  float r = rho, omega = 1.0f;       // omega = 1: equilibrium overwrite (inlet/outlet)
  if (cls == kClsInlet) {
    // Zou/He density from populations with c_z <= 0 (src/engine.js:282-284)
    const float s0 = f[0] + s1 + s3 + sxy;
    const float sm = f[6] + f[12] + f[13] + f[16] + f[17];
    r = rho = (SHIFTED ? 1.0f + (s0 + 2.0f * sm) : s0 + 2.0f * sm) / (1.0f - P.u0);
    vx = ux = 0.0f; vy = uy = 0.0f; vz = uz = P.u0;
  } else if (cls == kClsOutlet) {
    r = rho = 1.0f;
  } else {
    const float r3 = (SHIFTED ? tot : rho) * (1.0f / 3.0f);
    const float nxx = (s1 + sxy + sxz) - r3 - jx * ux;
    const float nyy = (s3 + sxy + syz) - r3 - jy * uy;
    const float nzz = (s5 + sxz + syz) - r3 - jz * uz;
    const float nxy = (s7 - s9) - jx * uy;
    const float nxz = (s11 - s13) - jx * uz;
    const float nyz = (s15 - s17) - jy * uz;
    const float q2 = nxx * nxx + nyy * nyy + nzz * nzz + 2.0f * (nxy * nxy + nxz * nxz + nyz * nyz);
    const float tau = 0.5f * (P.tau0 + cf_sqrt<FAST>(P.tau0 * P.tau0 + P.cs2s * cf_sqrt<FAST>(q2) * inv));
    if (cls == kClsFilter) {
      const float a1 = tau * P.sig * P.aniso, a2 = tau * P.sig;
      const float sl = 1.0f - (a1 >= 0.9f ? 0.9f : a1), sv = 1.0f - (a2 >= 0.9f ? 0.9f : a2);  // Math.min, NaN kept
      vx = ux * sl; vy = uy * sv; vz = uz * sl;
      ux = 0.5f * (ux + vx); uy = 0.5f * (uy + vy); uz = 0.5f * (uz + vz);
    }
    omega = cf_rcp<FAST>(tau);
  }
  const float base = 1.0f - 1.5f * (vx * vx + vy * vy + vz * vz);
  const float w1 = r * (1.0f / 18.0f), w2 = r * (1.0f / 36.0f);
  const float keep = 1.0f - nsv;
  // one opposite pair: equilibrium = even +- odd (SHIFTED: minus the pair's weight W), then relax both
  auto pair = [&](int q, float cu, float w, float W) {
    const float even = SHIFTED ? fmaf(w, fmaf(4.5f * cu, cu, base), -W) : w * fmaf(4.5f * cu, cu, base);
    const float odd = (3.0f * w) * cu;
    const float ep = even + odd, em = even - odd;
    const float bp = fmaf(omega, ep - f[q], f[q]), bm = fmaf(omega, em - f[q + 1], f[q + 1]);
    if (HAS_NS) {
      fo[q] = keep * bp + nsv * f[q + 1];
      fo[q + 1] = keep * bm + nsv * f[q];
    } else {
      fo[q] = bp; fo[q + 1] = bm;
    }
  };
  {
    const float e0 = SHIFTED ? fmaf(r * (1.0f / 3.0f), base, -1.0f / 3.0f) : r * (1.0f / 3.0f) * base;
    const float b0 = fmaf(omega, e0 - f[0], f[0]);
    fo[0] = HAS_NS ? keep * b0 + nsv * f[0] : b0;
  }
  constexpr float W1 = 1.0f / 18.0f, W2 = 1.0f / 36.0f;
  pair(1, vx, w1, W1); pair(3, vy, w1, W1); pair(5, vz, w1, W1);
  pair(7, vx + vy, w2, W2); pair(9, vx - vy, w2, W2); pair(11, vx + vz, w2, W2);
  pair(13, vx - vz, w2, W2); pair(15, vy + vz, w2, W2); pair(17, vy - vz, w2, W2);
  if (HAS_NS) { ux *= keep; uy *= keep; uz *= keep; }
}

}  // namespace abx
