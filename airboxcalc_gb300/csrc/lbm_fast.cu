// lbm_fast.cu - step kernels with float32 collision: float32 populations (the
// WGSL lbm_step contract, src/engine.js:378-450) and float16 / bfloat16
// shifted-deviation storage.  Compiled with the default contraction (FMA).
// Two forms: the TMA-pipelined persistent kernel (lbm_tma.cuh), used when the
// tensor maps could be made, and the direct-load kernel (lbm_kernels.cuh).
#include "lbm_kernels.cuh"
#include "lbm_tma.cuh"
#include "lbm_vec.cuh"

#include <cudaTypedefs.h>

#include <cstring>
#include <utility>

#ifndef ABX_TMA_STAGES
#define ABX_TMA_STAGES 3
#endif

namespace abx {

// Step kernels are launched with programmatic stream serialization (ABX_PDL=0: plain launches): the next
// step may be launched while the previous one finishes; the kernels wait for it before touching memory.
#ifndef ABX_PDL
#define ABX_PDL 1
#endif
template <class... KArgs, class... Args>
static cudaError_t launch_step_kernel_t(void (*kern)(KArgs...), unsigned grid, unsigned threads, cudaStream_t st,
                                       Args &&...args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = ABX_PDL ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}
template <class... KArgs, class... Args>
static cudaError_t launch_step_kernel(void (*kern)(KArgs...), unsigned grid, cudaStream_t st, Args &&...args) {
  return launch_step_kernel_t(kern, grid, 256, st, std::forward<Args>(args)...);
}

template <int K>
static cudaError_t step_k(bool odd, bool acc, bool has_ns, const StepArgs &a, cudaStream_t st) {
  if (a.nseg == 0) return cudaSuccess;
  const unsigned grid = step_grid(a.nseg);
#define ABX_L(O, A, N) return launch_step_kernel(aa_step_kernel<K, O, A, N>, grid, st, a)
  if (odd) {
    if (acc) { if (has_ns) ABX_L(true, true, true); else ABX_L(true, true, false); }
    else { if (has_ns) ABX_L(true, false, true); else ABX_L(true, false, false); }
  } else {
    if (acc) { if (has_ns) ABX_L(false, true, true); else ABX_L(false, true, false); }
    else { if (has_ns) ABX_L(false, false, true); else ABX_L(false, false, false); }
  }
#undef ABX_L
  return cudaGetLastError();
}

// ------------------------------------------------------------------ vectorised step (V cells per thread)
template <class... KArgs, class... Args>
static cudaError_t launch_vec_kernel(void (*kern)(KArgs...), unsigned grid, unsigned threads, size_t smem,
                                     cudaStream_t st, Args &&...args) {
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = ABX_PDL ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

template <int K, int V>
static cudaError_t vec_attrs() {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(aa_vec_kernel<K, V, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                vec_smem_bytes<K, V, true>())) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(aa_vec_kernel<K, V, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                vec_smem_bytes<K, V, true>())) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(aa_vec_kernel<K, V, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                vec_smem_bytes<K, V, false>())) != cudaSuccess) return e;
  return cudaFuncSetAttribute(aa_vec_kernel<K, V, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              vec_smem_bytes<K, V, false>());
}

cudaError_t prepare_step_vec(int storage, int V) {
  switch (storage) {
    case kStoreF32: if (V == 4) return vec_attrs<kStoreF32, 4>(); if (V == 2) return vec_attrs<kStoreF32, 2>(); break;
    case kStoreF16: if (V == 4) return vec_attrs<kStoreF16, 4>(); if (V == 2) return vec_attrs<kStoreF16, 2>(); break;
    case kStoreBF16: if (V == 4) return vec_attrs<kStoreBF16, 4>(); if (V == 2) return vec_attrs<kStoreBF16, 2>(); break;
  }
  return cudaErrorInvalidValue;
}

template <int K, int V>
static cudaError_t step_vec_k(bool odd, bool acc, const StepArgs &a, const VecArgs &v, cudaStream_t st) {
  const uint32_t items = (v.n_bulk + 31u) / 32u + (v.n_filter + 31u) / 32u + (v.nbcell + 31u) / 32u;
  if (items == 0) return cudaSuccess;
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm <= 0) nsm = 1;
  }
  constexpr unsigned T = VecShape<K, V>::kThreads, W = T / 32;
  const unsigned need = (items + W - 1) / W, res = (unsigned)nsm * VecShape<K, V>::kMinBlocks;
  const unsigned grid = need < res ? need : res;
  if (odd) {
    if (acc) return launch_vec_kernel(aa_vec_kernel<K, V, true, true>, grid, T, vec_smem_bytes<K, V, true>(), st, a, v);
    return launch_vec_kernel(aa_vec_kernel<K, V, true, false>, grid, T, vec_smem_bytes<K, V, false>(), st, a, v);
  }
  if (acc) return launch_vec_kernel(aa_vec_kernel<K, V, false, true>, grid, T, vec_smem_bytes<K, V, true>(), st, a, v);
  return launch_vec_kernel(aa_vec_kernel<K, V, false, false>, grid, T, vec_smem_bytes<K, V, false>(), st, a, v);
}

cudaError_t launch_step_vec(int storage, int V, bool odd, bool acc, const StepArgs &a, const VecArgs &v,
                            cudaStream_t st) {
  switch (storage) {
    case kStoreF32:
      if (V == 4) return step_vec_k<kStoreF32, 4>(odd, acc, a, v, st);
      if (V == 2) return step_vec_k<kStoreF32, 2>(odd, acc, a, v, st);
      break;
    case kStoreF16:
      if (V == 4) return step_vec_k<kStoreF16, 4>(odd, acc, a, v, st);
      if (V == 2) return step_vec_k<kStoreF16, 2>(odd, acc, a, v, st);
      break;
    case kStoreBF16:
      if (V == 4) return step_vec_k<kStoreBF16, 4>(odd, acc, a, v, st);
      if (V == 2) return step_vec_k<kStoreBF16, 2>(odd, acc, a, v, st);
      break;
  }
  return cudaErrorInvalidValue;
}

// ------------------------------------------------------------------ batched step (many domains)
template <int K, int SPW, int MINB>
static cudaError_t step_batch_k(bool odd, bool acc, const BatchParams &P, const uint2 *tiles, uint32_t t0, uint32_t t1,
                                uint32_t grid, cudaStream_t st) {
  if (t1 <= t0) return cudaSuccess;
  if (odd) {
    if (acc) return launch_step_kernel(aa_step_batch_kernel<K, true, true, SPW, MINB>, grid, st, P, tiles, t0, t1);
    return launch_step_kernel(aa_step_batch_kernel<K, true, false, SPW, MINB>, grid, st, P, tiles, t0, t1);
  }
  if (acc) return launch_step_kernel(aa_step_batch_kernel<K, false, true, SPW, MINB>, grid, st, P, tiles, t0, t1);
  return launch_step_kernel(aa_step_batch_kernel<K, false, false, SPW, MINB>, grid, st, P, tiles, t0, t1);
}

template <int K>
static cudaError_t step_batch_shape(int shape, bool odd, bool acc, const BatchParams &P, const uint2 *tiles,
                                    uint32_t t0, uint32_t t1, uint32_t grid, cudaStream_t st) {
  switch (shape) {
    case 0: return step_batch_k<K, 1, 4>(odd, acc, P, tiles, t0, t1, grid, st);
    case 1: return step_batch_k<K, 1, 3>(odd, acc, P, tiles, t0, t1, grid, st);
    case 2: return step_batch_k<K, 2, 2>(odd, acc, P, tiles, t0, t1, grid, st);
  }
  return cudaErrorInvalidValue;
}

int batch_shape_spw(int shape) { return shape == 2 ? 2 : 1; }
int batch_shape_minblocks(int shape) { return shape == 0 ? 4 : shape == 1 ? 3 : 2; }

cudaError_t launch_step_batch(int storage, bool odd, bool acc, int shape, const BatchParams &P, const uint2 *tiles,
                              uint32_t t0, uint32_t t1, uint32_t grid, cudaStream_t st) {
  if (grid == 0 || shape < 0 || shape >= kBatchShapes) return cudaErrorInvalidValue;
  switch (storage) {
    case kStoreF32: return step_batch_shape<kStoreF32>(shape, odd, acc, P, tiles, t0, t1, grid, st);
    case kStoreF16: return step_batch_shape<kStoreF16>(shape, odd, acc, P, tiles, t0, t1, grid, st);
    case kStoreBF16: return step_batch_shape<kStoreBF16>(shape, odd, acc, P, tiles, t0, t1, grid, st);
  }
  return cudaErrorInvalidValue;
}

// ------------------------------------------------------------------ TMA path
template <int K, bool O, bool A, bool N>
static cudaError_t tma_one(const StepArgs &a, const TmaBlob &b, cudaStream_t st) {
  CUtensorMap m[5];
  std::memcpy(m, b.maps, sizeof m);
  aa_step_tma_kernel<K, O, A, N, ABX_TMA_STAGES><<<b.grid, kTmaThreads, TmaStage<K, O, A, N, ABX_TMA_STAGES>::kSmem, st>>>(
      m[kMapPopEven], m[kMapPopWide], m[kMapPopRow], m[kMapMask], m[kMapAcc], a, b.ntiles);
  return cudaGetLastError();
}

template <int K>
static cudaError_t step_tma(bool odd, bool acc, bool has_ns, const StepArgs &a, const TmaBlob &b, cudaStream_t st) {
  if (a.nseg == 0) return cudaSuccess;
  if (odd) {
    if (acc) return has_ns ? tma_one<K, true, true, true>(a, b, st) : tma_one<K, true, true, false>(a, b, st);
    return has_ns ? tma_one<K, true, false, true>(a, b, st) : tma_one<K, true, false, false>(a, b, st);
  }
  if (acc) return has_ns ? tma_one<K, false, true, true>(a, b, st) : tma_one<K, false, true, false>(a, b, st);
  return has_ns ? tma_one<K, false, false, true>(a, b, st) : tma_one<K, false, false, false>(a, b, st);
}

template <int K, bool O, bool A, bool N>
static cudaError_t tma_attr(int *blocks) {
  constexpr int smem = TmaStage<K, O, A, N, ABX_TMA_STAGES>::kSmem;
  auto fn = aa_step_tma_kernel<K, O, A, N, ABX_TMA_STAGES>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  int nb = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kTmaThreads, smem);
  if (e != cudaSuccess) return e;
  *blocks = *blocks == 0 ? nb : std::min(*blocks, nb);
  return cudaSuccess;
}

template <int K>
static cudaError_t tma_prepare(int *blocks) {
  cudaError_t e;
#define ABX_A(O, A, N) if ((e = tma_attr<K, O, A, N>(blocks)) != cudaSuccess) return e;
  ABX_A(true, true, true) ABX_A(true, true, false) ABX_A(true, false, true) ABX_A(true, false, false)
  ABX_A(false, true, true) ABX_A(false, true, false) ABX_A(false, false, true) ABX_A(false, false, false)
#undef ABX_A
  return cudaSuccess;
}

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
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

cudaError_t make_tma(int storage, const StepArgs &a, TmaBlob *out) {
  out->ready = false;
  CUtensorMapDataType dt;
  int elem, win;
  switch (storage) {
    case kStoreF32: dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT32; elem = 4; win = TmaGeom<kStoreF32>::kWin; break;
    case kStoreF16: dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT16; elem = 2; win = TmaGeom<kStoreF16>::kWin; break;
    case kStoreBF16: dt = CU_TENSOR_MAP_DATA_TYPE_BFLOAT16; elem = 2; win = TmaGeom<kStoreBF16>::kWin; break;
    default: return cudaErrorNotSupported;
  }
  auto enc = encode_fn();
  if (!enc) return cudaErrorNotSupported;
  if (a.Np % 32 != 0 || a.Np >= (1ll << 31)) return cudaErrorNotSupported;
  CUtensorMap maps[5];
  const cuuint64_t np = (cuuint64_t)a.Np;
  const cuuint32_t ones[2] = {1, 1};
  {  // populations, even-step box {32, 19}
    const cuuint64_t dims[2] = {np, 19}, strides[1] = {np * elem};
    const cuuint32_t box[2] = {32, 19};
    if (enc(&maps[0], dt, 2, a.f, dims, strides, box, ones, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  }
  for (int m = 1; m <= 2; m++) {  // populations, odd-step rows: {win, 1} for +-z directions, {32, 1} otherwise
    const cuuint64_t dims[2] = {np, 19}, strides[1] = {np * elem};
    const cuuint32_t box[2] = {(cuuint32_t)(m == 1 ? win : 32), 1};
    if (enc(&maps[m], dt, 2, a.f, dims, strides, box, ones, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  }
  {  // cell mask words
    const cuuint64_t dims[1] = {np}, strides[1] = {np * 4};
    const cuuint32_t box[1] = {32};
    if (enc(&maps[3], CU_TENSOR_MAP_DATA_TYPE_UINT32, 1, (void *)a.mask, dims, strides, box, ones,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  }
  {  // running sums of the averages, box {32, 4}
    const cuuint64_t dims[2] = {np, 4}, strides[1] = {np * 4};
    const cuuint32_t box[2] = {32, 4};
    if (enc(&maps[4], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, a.acc, dims, strides, box, ones,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return cudaErrorInvalidValue;
  }
  static_assert(sizeof maps == sizeof out->maps, "five descriptors");
  std::memcpy(out->maps, maps, sizeof maps);
  int blocks = 0;
  cudaError_t e;
  switch (storage) {
    case kStoreF32: e = tma_prepare<kStoreF32>(&blocks); break;
    case kStoreF16: e = tma_prepare<kStoreF16>(&blocks); break;
    default: e = tma_prepare<kStoreBF16>(&blocks); break;
  }
  if (e != cudaSuccess) return e;
  if (blocks < 1) return cudaErrorNotSupported;
  int dev = 0, nsm = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
  out->ntiles = (a.nseg + kTmaSegs - 1) / kTmaSegs;
  out->grid = std::min<uint32_t>(out->ntiles, (uint32_t)(nsm * blocks));
  if (out->grid == 0) out->grid = 1;
  out->ready = true;
  return cudaSuccess;
}

void free_tma(TmaBlob *b) { b->ready = false; }

cudaError_t launch_step_fast(int storage, bool odd, bool acc, bool has_ns, const StepArgs &a, const TmaBlob *tma,
                             cudaStream_t st) {
  if (tma && tma->ready) {
    switch (storage) {
      case kStoreF32: return step_tma<kStoreF32>(odd, acc, has_ns, a, *tma, st);
      case kStoreF16: return step_tma<kStoreF16>(odd, acc, has_ns, a, *tma, st);
      case kStoreBF16: return step_tma<kStoreBF16>(odd, acc, has_ns, a, *tma, st);
      default: break;
    }
  }
  switch (storage) {
    case kStoreF32: return step_k<kStoreF32>(odd, acc, has_ns, a, st);
    case kStoreF16: return step_k<kStoreF16>(odd, acc, has_ns, a, st);
    case kStoreBF16: return step_k<kStoreBF16>(odd, acc, has_ns, a, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace abx
