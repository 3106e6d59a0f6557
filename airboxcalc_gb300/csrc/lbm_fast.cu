// lbm_fast.cu - step kernels with float32 collision: float32 populations (the
// WGSL lbm_step contract, src/engine.js:378-450) and float16 / bfloat16
// shifted-deviation storage.  Compiled with the default contraction (FMA).
#include "lbm_kernels.cuh"

namespace abx {

template <int K>
static cudaError_t step_k(bool odd, bool acc, bool has_ns, const StepArgs &a, cudaStream_t st) {
  if (a.nseg == 0) return cudaSuccess;
  const dim3 grid((a.nseg + 7) / 8), block(256);
#define ABX_L(O, A, N) aa_step_kernel<K, O, A, N><<<grid, block, 0, st>>>(a)
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

cudaError_t launch_step_fast(int storage, bool odd, bool acc, bool has_ns, const StepArgs &a, cudaStream_t st) {
  switch (storage) {
    case kStoreF32: return step_k<kStoreF32>(odd, acc, has_ns, a, st);
    case kStoreF16: return step_k<kStoreF16>(odd, acc, has_ns, a, st);
    case kStoreBF16: return step_k<kStoreBF16>(odd, acc, has_ns, a, st);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace abx
