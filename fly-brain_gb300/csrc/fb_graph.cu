// On-device graph compile: the reference's writeGraph (src/lifwasm.js:14-34), which turns raw
// synapse counts and per-neuron scales into the kernel's weights and signs.
//
//   sign[j] = f32(s_j * wSyn)
//   W[k]    = (c_k >= minSyn && keep_k) ? f32(((c_k * eg_k) * inScale[q]) * ig_j) : 0,
//             ig_j = (s_j < 0 ? inhGain : 1) * og_j,  keep_k = !sensory[q] || (preInh > 0 && s_j < 0)
//
// every product formed in double in the reference's operand order and rounded once to f32, as a
// JS Float32Array store rounds the double it is given.
#include <cuda_runtime.h>

#include "fb_internal.cuh"

namespace fb {

struct CompileArgs {
  int32_t N;
  const uint32_t *indptr, *indices;
  const float *counts;      // per edge (synapse count)
  const float *edgeGain;    // per edge or null
  const float *preSign;     // per neuron: the sign before wSyn
  const float *inScale;     // per neuron or null
  const float *outScale;    // per neuron or null
  const uint8_t *sensory;   // per neuron or null
  double wSyn, inhGain, minSyn, preInh;
  float *W, *sign;
};

// One warp per presynaptic row: lanes stride over the row's edges.
__global__ void compile_kernel(CompileArgs a) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t j = warp; j < a.N; j += nw) {
    const double s = (double)a.preSign[j];
    if (lane == 0) a.sign[j] = __double2float_rn(__dmul_rn(s, a.wSyn));
    const double og = a.outScale ? (double)a.outScale[j] : 1.0;
    const double ig = __dmul_rn(s < 0 ? a.inhGain : 1.0, og);
    const bool keepInh = a.preInh > 0 && s < 0;
    for (uint32_t k = a.indptr[j] + lane; k < a.indptr[j + 1]; k += 32) {
      const uint32_t q = a.indices[k];
      const double c = (double)a.counts[k];
      const bool keep = !(a.sensory && a.sensory[q]) || keepInh;
      float w = 0.f;
      if (c >= a.minSyn && keep) {
        double v = __dmul_rn(c, a.edgeGain ? (double)a.edgeGain[k] : 1.0);
        v = __dmul_rn(v, a.inScale ? (double)a.inScale[q] : 1.0);
        w = __double2float_rn(__dmul_rn(v, ig));
      }
      a.W[k] = w;
    }
  }
}

cudaError_t launch_compile(const CompileArgs &a, cudaStream_t st) {
  compile_kernel<<<608, 256, 0, st>>>(a);
  return cudaGetLastError();
}

}  // namespace fb
