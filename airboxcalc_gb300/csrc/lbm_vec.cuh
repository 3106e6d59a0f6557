// lbm_vec.cuh - the A-A step with V cells per thread: V consecutive cells along k
// ("a block") whose populations move as one aligned 8- or 16-byte vector per
// direction (float32: V = 2 or 4; float16 / bfloat16: V = 4 or 8).
//
// The cells of a geometry fall into
//   interior blocks  V fluid cells, every one with all 18 pull neighbours fluid and
//                    all of one class (bulk or filter): no bounce-back, so every
//                    population moves as a vector; a warp takes 32 blocks of one class
//   boundary cells   the fluid cells of every other block, in a dense list run 32 at
//                    a time by the one-cell-per-lane body of lbm_kernels.cuh (step_cells)
// (prep_vec_lists builds both lists; on the 50 M-cell airbox 96 % of the fluid
// cells are in interior blocks of 8).
//
// Even step (cell-local): direction q of the block is the vector A[q][b .. b+V),
// written back as A[opp q][b .. b+V).
// Odd step: the slots of direction q are the block's cells shifted by c_q.  For
// c_z = 0 they are an aligned vector in the neighbouring column.  For c_z = +-1
// they are shifted by one cell along k: the aligned vector holds V - 1 of them and
// the last one is the first (c_z = -1) or last (c_z = +1) element of the
// k-adjacent block's vector.  When that block sits on the next or previous lane
// of the same warp ("linked"), the value travels by a shuffle and the aligned
// vector is written whole by the thread that owns most of it; otherwise the thread
// loads / stores its edge slot on its own and writes the rest of the vector in
// aligned pieces.  Every slot is still read and written by the thread of the cell
// it belongs to (the A-A property), and a thread that loads a whole vector uses
// only its own elements of it.
#pragma once
#include "lbm_kernels.cuh"

namespace abx {

// Aligned vectors of V stored values (f, or h = f - w_q for the 16-bit storages), 4, 8 or 16 bytes.
template <int K, int V> struct VecIO {
  using T = typename Store<K>::T;
  static constexpr int kE = (int)sizeof(T);
  static constexpr int kBytes = V * kE;
  static constexpr int kW = kBytes / 4;
  static_assert(kBytes == 4 || kBytes == 8 || kBytes == 16, "vectors of 4, 8 or 16 bytes");
  static_assert(kE == 2 || kE == 4, "16- or 32-bit storage");
  struct Vec { uint32_t w[kW]; };

  __device__ static __forceinline__ Vec ld(const T *p) {
    Vec v;
    if constexpr (kW == 4) {
      const uint4 r = *reinterpret_cast<const uint4 *>(p);
      v.w[0] = r.x; v.w[1] = r.y; v.w[2] = r.z; v.w[3] = r.w;
    } else if constexpr (kW == 2) {
      const uint2 r = *reinterpret_cast<const uint2 *>(p);
      v.w[0] = r.x; v.w[1] = r.y;
    } else {
      v.w[0] = *reinterpret_cast<const uint32_t *>(p);
    }
    return v;
  }
  __device__ static __forceinline__ Vec lds(const unsigned char *p) {   // from shared memory
    Vec v;
    if constexpr (kW == 4) {
      const uint4 r = *reinterpret_cast<const uint4 *>(p);
      v.w[0] = r.x; v.w[1] = r.y; v.w[2] = r.z; v.w[3] = r.w;
    } else if constexpr (kW == 2) {
      const uint2 r = *reinterpret_cast<const uint2 *>(p);
      v.w[0] = r.x; v.w[1] = r.y;
    } else {
      v.w[0] = *reinterpret_cast<const uint32_t *>(p);
    }
    return v;
  }
  // whole vector, evict-first: a population written by a step is read only by the next one
  __device__ static __forceinline__ void st(T *p, const Vec &v) {
    if constexpr (kW == 4) __stcs(reinterpret_cast<uint4 *>(p), make_uint4(v.w[0], v.w[1], v.w[2], v.w[3]));
    else if constexpr (kW == 2) __stcs(reinterpret_cast<uint2 *>(p), make_uint2(v.w[0], v.w[1]));
    else __stcs(reinterpret_cast<unsigned int *>(p), v.w[0]);
  }
  // element e (a constant after unrolling) as float
  __device__ static __forceinline__ float get(const Vec &v, int e) {
    if constexpr (kE == 4) {
      return __uint_as_float(v.w[e]);
    } else if constexpr (K == kStoreF16) {
      const uint32_t w = v.w[e >> 1];
      return __half2float(__ushort_as_half((unsigned short)((e & 1) ? (w >> 16) : (w & 0xffffu))));
    } else {
      const uint32_t w = v.w[e >> 1];
      return __uint_as_float((e & 1) ? (w & 0xffff0000u) : (w << 16));
    }
  }
  __device__ static __forceinline__ uint32_t pack2(float lo, float hi) {
    if constexpr (K == kStoreF16) {
      const __half2 h = __floats2half2_rn(lo, hi);
      return *reinterpret_cast<const uint32_t *>(&h);
    } else {
      const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
      return *reinterpret_cast<const uint32_t *>(&h);
    }
  }
  __device__ static __forceinline__ Vec pack(const float (&x)[V]) {
    Vec v;
    if constexpr (kE == 4) {
#pragma unroll
      for (int e = 0; e < V; e++) v.w[e] = __float_as_uint(x[e]);
    } else {
#pragma unroll
      for (int i = 0; i < kW; i++) v.w[i] = pack2(x[2 * i], x[2 * i + 1]);
    }
    return v;
  }
  // the widest aligned piece (elements) that starts at element lo and ends by hi
  __host__ __device__ static constexpr int piece(int lo, int hi) {
    int n = 16 / kE;
    while (n > 1 && (lo % n != 0 || lo + n > hi)) n >>= 1;
    return n;
  }
  template <int LO, int N> __device__ static __forceinline__ void st_piece(T *p, const Vec &v) {
    constexpr int bytes = N * kE;
    if constexpr (bytes == 2) {
      const uint32_t w = v.w[LO >> 1];
      *reinterpret_cast<unsigned short *>(p + LO) = (unsigned short)((LO & 1) ? (w >> 16) : (w & 0xffffu));
    } else if constexpr (bytes == 4) {
      *reinterpret_cast<uint32_t *>(p + LO) = v.w[LO * kE / 4];
    } else if constexpr (bytes == 8) {
      *reinterpret_cast<uint2 *>(p + LO) = make_uint2(v.w[LO * kE / 4], v.w[LO * kE / 4 + 1]);
    } else {
      *reinterpret_cast<uint4 *>(p + LO) = make_uint4(v.w[0], v.w[1], v.w[2], v.w[3]);
    }
  }
  // elements [LO, HI) of the vector whose element 0 is at p, in aligned pieces
  template <int LO, int HI> __device__ static __forceinline__ void st_range(T *p, const Vec &v) {
    if constexpr (LO < HI) {
      constexpr int n = piece(LO, HI);
      st_piece<LO, n>(p, v);
      st_range<LO + n, HI>(p, v);
    }
  }
};

// Averages of V cells: acc[c][b .. b+V), float32, as 16-byte vectors (V = 4 or 8) or an 8-byte one (V = 2).
// (The averaging steps are a quarter of a solve or less; the float32 sums need no narrower form.)
template <int V> __device__ __forceinline__ void acc_ld(const float *p, float (&x)[V]) {
  if constexpr (V == 2) {
    const float2 r = *reinterpret_cast<const float2 *>(p);
    x[0] = r.x; x[1] = r.y;
  } else {
#pragma unroll
    for (int i = 0; i < V / 4; i++) {
      const float4 r = *reinterpret_cast<const float4 *>(p + 4 * i);
      x[4 * i] = r.x; x[4 * i + 1] = r.y; x[4 * i + 2] = r.z; x[4 * i + 3] = r.w;
    }
  }
}
template <int V> __device__ __forceinline__ void acc_st(float *p, const float (&x)[V]) {
  if constexpr (V == 2) {
    *reinterpret_cast<float2 *>(p) = make_float2(x[0], x[1]);
  } else {
#pragma unroll
    for (int i = 0; i < V / 4; i++)
      *reinterpret_cast<float4 *>(p + 4 * i) = make_float4(x[4 * i], x[4 * i + 1], x[4 * i + 2], x[4 * i + 3]);
  }
}

// Asynchronous global -> shared copies of 4, 8 or 16 bytes (no registers held while they fly).
template <int BYTES> __device__ __forceinline__ void cp_async(unsigned char *smem, const void *gmem) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(smem);
  if constexpr (BYTES == 16) asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gmem) : "memory");
  else asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(d), "l"(gmem), "n"(BYTES) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// One warp's stage in shared memory: the 19 population vectors of its 32 lanes ([q][lane]) and, in averaging
// steps, the 4 running-sum vectors ([c][lane]).  Two stages per warp: one being filled, one being computed.
// Odd steps also stage, for the lanes whose k-adjacent block is not on the next / previous lane, the 32-bit word
// holding the edge slot of each direction with c_z != 0 ([e][lane], e = edge_index(q)).
__host__ __device__ constexpr int edge_index(int q) {
  return q == 5 ? 0 : q == 6 ? 1 : q >= 11 && q <= 18 ? q - 9 : -1;
}
template <int K, int V, bool ACC> struct VecStage {
  static constexpr int kVec = VecIO<K, V>::kBytes;
  static constexpr int kAccOff = 19 * 32 * kVec;
  static constexpr int kEdgeOff = kAccOff + (ACC ? 4 * 32 * V * 4 : 0);
  static constexpr int kBytes = kEdgeOff + 10 * 32 * 4;
};
// The 32-bit word holding the edge slot of direction q (c_z = +1: element -1 of the aligned source vector at
// src, c_z = -1: element V) and the slot's value in it.
template <int K, int V> __device__ __forceinline__ const void *edge_word(const typename Store<K>::T *f, uint32_t src, int q) {
  constexpr int perw = 4 / (int)sizeof(typename Store<K>::T);   // elements per word
  return cz(q) > 0 ? (const void *)(f + (src - (uint32_t)perw)) : (const void *)(f + (src + (uint32_t)V));
}
template <int K> __device__ __forceinline__ float edge_value(uint32_t w, int q) {
  if constexpr (sizeof(typename Store<K>::T) == 4) return __uint_as_float(w);
  else {
    const uint32_t h = cz(q) > 0 ? (w >> 16) : (w & 0xffffu);   // element -1 is the high half, element V the low one
    if constexpr (K == kStoreF16) return __half2float(__ushort_as_half((unsigned short)h));
    else return __uint_as_float(h << 16);
  }
}

// Issue the copies of one interior block (first cell b) into a stage: the vectors the step reads.
template <int K, int V, bool ODD, bool ACC>
__device__ __forceinline__ void vec_fetch(const StepArgs &a, const uint32_t b, const bool prev_link,
                                          const bool next_link, unsigned char *stage, uint32_t lane) {
  using IO = VecIO<K, V>;
  using T = typename Store<K>::T;
  using ST = VecStage<K, V, ACC>;
  const T *f = (const T *)a.f;
  const uint32_t Np = (uint32_t)a.Np;
#pragma unroll
  for (int q = 0; q < 19; q++) {
    const uint32_t src = ODD ? (uint32_t)opp(q) * Np + b - (uint32_t)(a.off[q] - cz(q)) : (uint32_t)q * Np + b;
    cp_async<IO::kBytes>(stage + (q * 32 + lane) * IO::kBytes, f + src);
    if (ODD && cz(q) != 0 && !(cz(q) > 0 ? prev_link : next_link))
      cp_async<4>(stage + ST::kEdgeOff + (edge_index(q) * 32 + lane) * 4, edge_word<K, V>(f, src, q));
  }
  if (ACC) {
    const float *acc = (const float *)a.acc;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      unsigned char *d = stage + ST::kAccOff + (c * 32 + lane) * V * 4;
#pragma unroll
      for (int i = 0; i < (V * 4 + 15) / 16; i++)
        cp_async<(V * 4 < 16 ? V * 4 : 16)>(d + 16 * i, acc + (uint32_t)c * Np + b + 4 * i);
    }
  }
}

// One interior block: V cells from padded index b, all of class CLS.  act: the lane holds a block (an idle lane
// repeats its warp's last block and stores nothing); prev_link / next_link: lane - 1 / lane + 1 holds the
// k-adjacent block b - V / b + V of the same column.
// stage: the block's vectors already copied to shared memory (vec_fetch), or null to load them here.
template <int K, int V, bool ODD, bool ACC, uint32_t CLS>
__device__ __forceinline__ void vec_block(const StepArgs &a, const uint32_t b, const bool act, const bool prev_link,
                                          const bool next_link, const unsigned char *stage = nullptr) {
  using IO = VecIO<K, V>;
  using Vec = typename IO::Vec;
  using T = typename Store<K>::T;
  constexpr unsigned kFull = 0xffffffffu;
  T *f = (T *)a.f;
  const uint32_t Np = (uint32_t)a.Np;
  const CollideParams<float> P = make_params<float>(a);
  // aligned vector of every direction: the cell's own slots (even), the pull column's (odd)
  const uint32_t lane = threadIdx.x & 31u;
  Vec in[19];
  float av[4][V];
  if (stage) {
#pragma unroll
    for (int q = 0; q < 19; q++) in[q] = IO::lds(stage + (q * 32 + lane) * IO::kBytes);
    if (ACC) {
#pragma unroll
      for (int c = 0; c < 4; c++)
        acc_ld<V>(reinterpret_cast<const float *>(stage + VecStage<K, V, ACC>::kAccOff + (c * 32 + lane) * V * 4), av[c]);
    }
  } else {
#pragma unroll
    for (int q = 0; q < 19; q++) {
      const uint32_t src = ODD ? (uint32_t)opp(q) * Np + b - (uint32_t)(a.off[q] - cz(q)) : (uint32_t)q * Np + b;
      in[q] = IO::ld(f + src);
    }
    if (ACC) {
      const float *acc = (const float *)a.acc;
#pragma unroll
      for (int c = 0; c < 4; c++) acc_ld<V>(acc + (uint32_t)c * Np + b, av[c]);
    }
  }
  // odd step, c_z != 0: the slot one cell beyond the aligned vector
  float edge[19];
  if (ODD) {
#pragma unroll
    for (int q = 0; q < 19; q++) {
      if (cz(q) == 0) continue;
      const uint32_t src = (uint32_t)opp(q) * Np + b - (uint32_t)(a.off[q] - cz(q));
      const bool linked = cz(q) > 0 ? prev_link : next_link;
      edge[q] = cz(q) > 0 ? __shfl_up_sync(kFull, IO::get(in[q], V - 1), 1) : __shfl_down_sync(kFull, IO::get(in[q], 0), 1);
      if (!linked) {
        if (stage)
          edge[q] = edge_value<K>(*reinterpret_cast<const uint32_t *>(
                                      stage + VecStage<K, V, ACC>::kEdgeOff + (edge_index(q) * 32 + lane) * 4), q);
        else
          edge[q] = Store<K>::ldr(f + (cz(q) > 0 ? src - 1u : src + (uint32_t)V));
      }
      edge[q] = toc<K>(edge[q], q);
    }
  }
  // Cells one after another.  Cell c's output of direction q goes to element pos(c) of the outgoing vector
  // (c, or c +- 1 for the shifted directions of an odd step); a 32-bit word of two 16-bit elements is packed
  // as soon as both are known, so few outputs stay live as floats.
  float ov[19][V];
  uint32_t ow[19][IO::kW];
  float keep[19];   // odd, c_z != 0: the output that leaves the vector (edge slot and the shuffle to the neighbour)
#pragma unroll
  for (int c = 0; c < V; c++) {
    float fi[19], fo[19], ux, uy, uz, rho;
#pragma unroll
    for (int q = 0; q < 19; q++) {
      if (!ODD || cz(q) == 0) fi[q] = toc<K>(IO::get(in[q], c), q);
      else if (cz(q) > 0) fi[q] = c == 0 ? edge[q] : toc<K>(IO::get(in[q], c - 1), q);
      else fi[q] = c == V - 1 ? edge[q] : toc<K>(IO::get(in[q], c + 1), q);
    }
    collide_fast<false, Store<K>::kCollideShifted, Store<K>::kFastMath>(fi, CLS, 0.0f, P, fo, ux, uy, uz, rho);
    // back to stored values (f for float32, h for the 16-bit formats)
#pragma unroll
    for (int q = 0; q < 19; q++) fo[q] = fromc<K>(fo[q], q);
    if (ACC) { av[0][c] += ux; av[1][c] += uy; av[2][c] += uz; av[3][c] += rho; }
#pragma unroll
    for (int q = 0; q < 19; q++) {
      // even step: A[opp q][x] = f*_q(x), collected under array index r = opp(q)
      const int r = ODD ? q : opp(q);
      const int dz = ODD ? cz(q) : 0;
      const int e = c + dz;   // element of the outgoing vector
      if (e < 0 || e >= V) { keep[r] = fo[q]; continue; }
      ov[r][e] = fo[q];
      if constexpr (IO::kE == 4) {
        ow[r][e] = __float_as_uint(fo[q]);
      } else {
        // word e/2 is complete when its second element arrives (element 0 of a c_z = +1 vector comes last)
        if ((e & 1) && !(dz > 0 && e == 1)) ow[r][e >> 1] = IO::pack2(ov[r][e - 1], fo[q]);
      }
    }
  }
  constexpr unsigned kFull2 = 0xffffffffu;
#pragma unroll
  for (int r = 0; r < 19; r++) {
    const int dz = ODD ? cz(r) : 0;
    typename IO::Vec v;
    if (dz > 0) {
      // slots b+1 .. b+V: element 0 holds the previous block's last cell
      const float from = __shfl_up_sync(kFull2, keep[r], 1);
      if constexpr (IO::kE == 4) ow[r][0] = __float_as_uint(from);
      else ow[r][0] = IO::pack2(from, ov[r][1]);
    } else if (dz < 0) {
      // slots b-1 .. b+V-2: the last element holds the next block's first cell
      const float from = __shfl_down_sync(kFull2, keep[r], 1);
      if constexpr (IO::kE == 4) ow[r][V - 1] = __float_as_uint(from);
      else ow[r][IO::kW - 1] = IO::pack2(ov[r][V - 2], from);
    }
#pragma unroll
    for (int i = 0; i < IO::kW; i++) v.w[i] = ow[r][i];
    if (!act) continue;
    if (!ODD) {
      IO::st(f + ((uint32_t)r * Np + b), v);
      continue;
    }
    // A[q][x + c_q] = f*_q(x): the aligned vector of the destination column
    T *dst = f + ((uint32_t)r * Np + b + (uint32_t)(a.off[r] - cz(r)));
    if (dz == 0) {
      IO::st(dst, v);
    } else if (dz > 0) {
      if (prev_link) IO::st(dst, v);
      else IO::template st_range<1, V>(dst, v);
      if (!next_link) Store<K>::str(dst + V, keep[r]);
    } else {
      if (next_link) IO::st(dst, v);
      else IO::template st_range<0, V - 1>(dst, v);
      if (!prev_link) Store<K>::str(dst - 1, keep[r]);
    }
  }
  if (ACC && act) {
    float *acc = (float *)a.acc;
#pragma unroll
    for (int c = 0; c < 4; c++) acc_st<V>(acc + (uint32_t)c * Np + b, av[c]);
  }
}

// Block shape of the vectorised kernel per storage and V: threads per block and resident blocks per SM that the
// registers are sized for (registers per thread = 65536 / (threads * blocks), rounded down to a multiple of 8).
#ifndef ABX_VEC2_MINB
#define ABX_VEC2_MINB 2
#endif
template <int K, int V> struct VecShape {
  static constexpr int kThreads = V >= 4 ? 128 : 256;
  static constexpr int kMinBlocks = V >= 4 ? 3 : ABX_VEC2_MINB;
};

// One step.  Each warp first takes interior items (32 blocks of one class), two at a time in flight: the copies
// of its next item land in shared memory while it computes the current one; then boundary items (32 boundary
// cells, one per lane).  Persistent like aa_step_kernel; odd steps walk the items backwards.
#ifndef ABX_VEC_PIPE
#define ABX_VEC_PIPE 1
#endif
template <int K, int V, bool ODD, bool ACC>
__global__ void __launch_bounds__(VecShape<K, V>::kThreads, VecShape<K, V>::kMinBlocks)
    aa_vec_kernel(const StepArgs a, const VecArgs v) {
  extern __shared__ __align__(16) unsigned char vec_smem[];
  step_dependency_wait();
  using ST = VecStage<K, V, ACC>;
  constexpr unsigned kFull = 0xffffffffu;
  constexpr uint32_t kWarps = VecShape<K, V>::kThreads / 32;
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t nbi = (v.n_bulk + 31u) / 32u, nfi = (v.n_filter + 31u) / 32u, nint = nbi + nfi;
  const uint32_t nci = (v.nbcell + 31u) / 32u;
  const uint32_t warp = blockIdx.x * kWarps + (threadIdx.x >> 5), nw = gridDim.x * kWarps;
  // the run-state word changes only between launches
  if (a.status && *a.status) return;
  // interior item i (walked backwards on odd steps): its lane's block, whether the lane holds one, its class
  auto item = [&](uint32_t i, uint32_t &b, bool &act, bool &filt) {
    const uint32_t it = (ABX_STEP_ALTERNATE && ODD) ? nint - 1u - i : i;
    filt = it >= nbi;
    const uint32_t first = filt ? v.n_bulk + (it - nbi) * 32u : it * 32u;
    const uint32_t end = filt ? v.n_bulk + v.n_filter : v.n_bulk;
    act = first + lane < end;
    b = v.blk[act ? first + lane : end - 1u];
  };
  // lanes holding the k-adjacent blocks of the same column (all lanes take part)
  auto links = [&](uint32_t b, bool act, bool &prev_link, bool &next_link) {
    const uint32_t bp = __shfl_up_sync(kFull, b, 1), bn = __shfl_down_sync(kFull, b, 1);
    const uint32_t am = __ballot_sync(kFull, act);
    prev_link = act && lane > 0 && ((am >> (lane - 1)) & 1u) && bp + (uint32_t)V == b;
    next_link = act && lane < 31 && ((am >> (lane + 1)) & 1u) && b + (uint32_t)V == bn;
  };
  auto compute = [&](uint32_t b, bool act, bool filt, bool pl, bool nl, const unsigned char *stage) {
    if (filt) vec_block<K, V, ODD, ACC, kClsFilter>(a, b, act, pl, nl, stage);
    else vec_block<K, V, ODD, ACC, kClsBulk>(a, b, act, pl, nl, stage);
  };
  if (ABX_VEC_PIPE) {
    unsigned char *stages = vec_smem + (threadIdx.x >> 5) * 2 * ST::kBytes;
    uint32_t b0 = 0, b1 = 0, b2 = 0;
    bool a0 = false, a1 = false, a2 = false, f0 = false, f1 = false, f2 = false, p0 = false, n0 = false, p1 = false,
         n1 = false;
    uint32_t i = warp;
    if (i < nint) {
      item(i, b0, a0, f0);
      links(b0, a0, p0, n0);
      vec_fetch<K, V, ODD, ACC>(a, b0, p0, n0, stages, lane);
    }
    cp_async_commit();
    if (i + nw < nint) item(i + nw, b1, a1, f1);
    int s = 0;
    for (; i < nint; i += nw) {
      if (i + nw < nint) {
        links(b1, a1, p1, n1);
        vec_fetch<K, V, ODD, ACC>(a, b1, p1, n1, stages + (s ^ 1) * ST::kBytes, lane);
      }
      cp_async_commit();
      if (i + 2 * nw < nint) item(i + 2 * nw, b2, a2, f2);   // used next round
      cp_async_wait<1>();   // this item's copies have landed; the next item's may still fly
      __syncwarp();
      compute(b0, a0, f0, p0, n0, stages + s * ST::kBytes);
      __syncwarp();         // every lane is done with this stage before it is filled again
      b0 = b1; a0 = a1; f0 = f1; p0 = p1; n0 = n1;
      b1 = b2; a1 = a2; f1 = f2;
      s ^= 1;
    }
    cp_async_wait<0>();
  } else {
    for (uint32_t i = warp; i < nint; i += nw) {
      uint32_t b;
      bool act, filt, pl, nl;
      item(i, b, act, filt);
      links(b, act, pl, nl);
      compute(b, act, filt, pl, nl, nullptr);
    }
  }
  for (uint32_t w = warp; w < nci; w += nw) {
    // 32 boundary cells, one per lane, as a segment entry of each lane's own: base p - lane (p >= 32, since no
    // fluid cell lies in the grid's first column), lane bit set when the lane holds a cell
    const uint32_t ci = (ABX_STEP_ALTERNATE && ODD) ? nci - 1u - w : w;
    const uint32_t idx = ci * 32u + lane;
    const bool act = idx < v.nbcell;
    const uint32_t p = v.bcell[act ? idx : v.nbcell - 1u];
    const uint2 sg[1] = {make_uint2(p - lane, act ? 1u << lane : 0u)};
    step_cells<K, ODD, ACC, false, 1>(a, sg, lane);
  }
}

// Dynamic shared memory of one block of aa_vec_kernel (both stages of every warp).
template <int K, int V, bool ACC> constexpr int vec_smem_bytes() {
  return ABX_VEC_PIPE ? (VecShape<K, V>::kThreads / 32) * 2 * VecStage<K, V, ACC>::kBytes : 0;
}

}  // namespace abx
