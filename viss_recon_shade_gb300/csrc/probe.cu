// probe.cu -- SFU (XU pipe) throughput probe: the denominator of the
// roofline of the DFT kernels, whose per-term cost is two SFU operations
// (sin, cos).  Each thread runs 8 independent __sincosf chains; the caller
// times the launch and divides 2 * 8 * iters * threads by the duration.
#include "viss_internal.cuh"

namespace viss {

__global__ void __launch_bounds__(256) sfu_probe_kernel(int iters, float seed, float* out) {
  float x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = seed * (float)(threadIdx.x + 1 + i * 37);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      float s, c;
      __sincosf(x[i], &s, &c);
      x[i] = s + c;  // stays in [-1.5, 1.5]
    }
  }
  float acc = 0.f;
#pragma unroll
  for (int i = 0; i < 8; ++i) acc += x[i];
  if (acc == 12345.678f) out[0] = acc;  // keep the chains live
}

}  // namespace viss

using namespace viss;

extern "C" {

int viss_sfu_probe(int iters, int blocks_per_sm, float* out, int64_t* sfu_ops, void* stream) {
  if (iters < 1 || blocks_per_sm < 1 || !out || !sfu_ops) return fail(VISS_ERR_INVALID, "bad probe arguments");
  const int nb = device_sm_count() * blocks_per_sm;
  sfu_probe_kernel<<<nb, 256, 0, static_cast<cudaStream_t>(stream)>>>(iters, 1e-3f, out);
  VISS_LAUNCH_CHECK("sfu_probe_kernel");
  *sfu_ops = (int64_t)nb * 256 * 8 * 2 * (int64_t)iters;
  return VISS_OK;
}

}  // extern "C"
