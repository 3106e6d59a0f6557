// lbm_exact.cu - compiled with -fmad=false, so every multiply and add rounds
// separately, as in the reference's JavaScript arithmetic.  Holds:
//   * the step kernel with float32 storage and float64 collision in
//     cpuStep's operation order (src/engine.js:266-321), bit-exact with it;
//   * the float64 run (float64 storage and collision);
//   * state, probe and evaluate kernels for every storage (float64 sums);
//   * the cell-mask construction.
#include "lbm_kernels.cuh"

namespace abx {

template <int K>
static cudaError_t step_k(bool odd, bool acc, bool has_ns, const StepArgs &a, cudaStream_t st) {
  if (a.nseg == 0) return cudaSuccess;
  const dim3 grid(step_grid(a.nseg)), block(256);
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

cudaError_t launch_step(int storage, bool odd, bool acc, bool has_ns, const StepArgs &a, const TmaBlob *tma,
                        cudaStream_t st) {
  switch (storage) {
    case kStoreF32Exact: return step_k<kStoreF32Exact>(odd, acc, has_ns, a, st);
    case kStoreF64: return step_k<kStoreF64>(odd, acc, has_ns, a, st);
    case kStoreF32: case kStoreF16: case kStoreBF16: return launch_step_fast(storage, odd, acc, has_ns, a, tma, st);
    default: return cudaErrorInvalidValue;
  }
}

static dim3 stride_grid(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  if (b < 1) b = 1;
  return dim3((unsigned)b);
}

#define ABX_DISPATCH(storage, CALL)                  \
  switch (storage) {                                 \
    case kStoreF32: { constexpr int K = kStoreF32; CALL; break; }           \
    case kStoreF32Exact: { constexpr int K = kStoreF32Exact; CALL; break; } \
    case kStoreF16: { constexpr int K = kStoreF16; CALL; break; }           \
    case kStoreBF16: { constexpr int K = kStoreBF16; CALL; break; }         \
    case kStoreF64: { constexpr int K = kStoreF64; CALL; break; }           \
    default: return cudaErrorInvalidValue;           \
  }

cudaError_t launch_init(int storage, const StateArgs &a, cudaStream_t st) {
  ABX_DISPATCH(storage, (init_state_kernel<K><<<stride_grid(a.Np), 256, 0, st>>>(a)));
  return cudaGetLastError();
}
cudaError_t launch_get_f(int storage, const StateArgs &a, float *out, cudaStream_t st) {
  ABX_DISPATCH(storage, (get_f_kernel<K><<<stride_grid(a.ncells), 256, 0, st>>>(a, out)));
  return cudaGetLastError();
}
cudaError_t launch_set_f(int storage, const StateArgs &a, const float *in, cudaStream_t st) {
  ABX_DISPATCH(storage, (set_f_kernel<K><<<stride_grid(a.ncells), 256, 0, st>>>(a, in)));
  return cudaGetLastError();
}
cudaError_t launch_get_acc(int storage, const StateArgs &a, float *out, int nacc, cudaStream_t st) {
  ABX_DISPATCH(storage, (get_acc_kernel<K><<<stride_grid(a.ncells), 256, 0, st>>>(a, out, nacc)));
  return cudaGetLastError();
}
cudaError_t launch_probe(int storage, const StateArgs &a, const ProbeArgs &p, cudaStream_t st) {
  if (p.nblocks < 1) return cudaErrorInvalidValue;
  ABX_DISPATCH(storage, (probe_pass1_kernel<K><<<p.nblocks, kProbeThreads, 0, st>>>(a, p)));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  probe_pass2_kernel<<<1, 1024, 0, st>>>(p, a.status);
  return cudaGetLastError();
}
cudaError_t launch_evaluate(int storage, const StateArgs &a, const EvalArgs &e, cudaStream_t st) {
  ABX_DISPATCH(storage, (evaluate_kernel<K><<<1, 1024, 0, st>>>(a, e)));
  return cudaGetLastError();
}

// Mask words from class bytes; the pull neighbour of direction q is
// (i - cx, j - cy, k - cz), fluid when inside the grid and of nonzero class.
// This is the nb table of setupSim (src/engine.js:243,251) with explicit
// bounds instead of linear wrap-around; the two agree because fluid never
// touches the grid faces that a wrap could cross (the leak check of
// src/engine.js:191-195 and the closed last row of :177-178 ensure it).
__global__ void build_mask_kernel(const uint8_t *cls, int nx, int ny, int nz, int64_t nzp, int64_t kpad,
                                  uint32_t *mask) {
  const int64_t total = (int64_t)nx * ny * nzp;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < total; p += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(p % nzp - kpad);
    const int64_t ij = p / nzp;
    const int j = (int)(ij % ny), i = (int)(ij / ny);
    uint32_t m = 0;
    if (k >= 0 && k < nz) {
      const uint8_t c = cls[ij * nz + k];
      if (c) {
#pragma unroll
        for (int q = 0; q < 19; q++) {
          const int ii = i - cx(q), jj = j - cy(q), kk = k - cz(q);
          if (ii >= 0 && ii < nx && jj >= 0 && jj < ny && kk >= 0 && kk < nz &&
              cls[((int64_t)ii * ny + jj) * nz + kk])
            m |= 1u << q;
        }
        m |= (uint32_t)(c == 2 ? kClsInlet : c == 3 ? kClsOutlet : c == 4 ? kClsFilter : kClsBulk) << kClassShift;
      }
    }
    mask[p] = m;
  }
}

cudaError_t launch_build_mask(const uint8_t *cls, int nx, int ny, int nz, int64_t nzp, int64_t kpad, uint32_t *mask,
                              cudaStream_t st) {
  build_mask_kernel<<<stride_grid((int64_t)nx * ny * nzp), 256, 0, st>>>(cls, nx, ny, nz, nzp, kpad, mask);
  return cudaGetLastError();
}

__global__ void scatter_f32_kernel(const float *src, const int64_t *cells, int64_t n, float *dst) {
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < n; a += (int64_t)gridDim.x * blockDim.x)
    dst[cells[a]] = src[a];
}
cudaError_t launch_scatter_f32(const float *src, const int64_t *cells, int64_t n, float *dst, cudaStream_t st) {
  scatter_f32_kernel<<<stride_grid(n), 256, 0, st>>>(src, cells, n, dst);
  return cudaGetLastError();
}

}  // namespace abx
