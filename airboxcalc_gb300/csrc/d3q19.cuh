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

// Storage formats of the populations.  Shifted formats hold f - w_q.
enum StoreKind { kStoreF32 = 0, kStoreF32Exact = 1, kStoreF16 = 2, kStoreBF16 = 3, kStoreF64 = 4 };

template <int K> struct Store;
template <> struct Store<kStoreF32> {
  using T = float; using L = float; using Acc = float;
  __device__ static __forceinline__ L ld(const T *p, L) { return __ldcs(p); }
  __device__ static __forceinline__ void st(T *p, L v, L) { __stcs(p, v); }
};
template <> struct Store<kStoreF32Exact> {
  using T = float; using L = double; using Acc = float;
  __device__ static __forceinline__ L ld(const T *p, L) { return (L)*p; }
  __device__ static __forceinline__ void st(T *p, L v, L) { *p = (float)v; }
};
template <> struct Store<kStoreF16> {
  using T = __half; using L = float; using Acc = float;
  __device__ static __forceinline__ L ld(const T *p, L w) { return w + __half2float(*p); }
  __device__ static __forceinline__ void st(T *p, L v, L w) { *p = __float2half_rn(v - w); }
};
template <> struct Store<kStoreBF16> {
  using T = __nv_bfloat16; using L = float; using Acc = float;
  __device__ static __forceinline__ L ld(const T *p, L w) { return w + __bfloat162float(*p); }
  __device__ static __forceinline__ void st(T *p, L v, L w) { *p = __float2bfloat16_rn(v - w); }
};
template <> struct Store<kStoreF64> {
  using T = double; using L = double; using Acc = double;
  __device__ static __forceinline__ L ld(const T *p, L) { return *p; }
  __device__ static __forceinline__ void st(T *p, L v, L) { *p = v; }
};

template <class L> __device__ __forceinline__ L weight(int q) {
  return wclass(q) == 0 ? (L)1 / (L)3 : (wclass(q) == 1 ? (L)1 / (L)18 : (L)1 / (L)36);
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
    const L sl = (L)1 - (a1 < (L)0.9 ? a1 : (L)0.9), sv = (L)1 - (a2 < (L)0.9 ? a2 : (L)0.9);
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

}  // namespace abx
