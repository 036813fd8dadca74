// order.cu -- spatial permutation of the sky (cube-face Morton order), used by
// the geometric-mask passes so that a warp's pixels form a compact patch.
#include <cub/cub.cuh>

#include "viss_internal.cuh"

namespace viss {

namespace {
struct OrderScratch {
  uint32_t *k0 = nullptr, *k1 = nullptr;
  int32_t* i0 = nullptr;
  void* cub = nullptr;
  size_t cub_bytes = 0, bytes = 0;
  void layout(void* ws, int64_t J) {
    Carver c(ws);
    k0 = c.take<uint32_t>(J);
    k1 = c.take<uint32_t>(J);
    i0 = c.take<int32_t>(J);
    size_t a = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, a, (uint32_t*)nullptr, (uint32_t*)nullptr, (int32_t*)nullptr,
                                    (int32_t*)nullptr, (int64_t)J, 0, 23);
    cub_bytes = a;
    cub = c.take<char>(a);
    bytes = c.size();
  }
};
}  // namespace

size_t pixel_order_scratch(int64_t J) {
  if (J <= 0) return 0;
  OrderScratch s;
  s.layout(nullptr, J);
  return s.bytes;
}

int pixel_order(const float* l, const float* m, const float* n, int64_t J, void* scratch, size_t scratch_bytes,
                int32_t* perm, cudaStream_t st) {
  if (J <= 0) return VISS_OK;
  OrderScratch s;
  s.layout(nullptr, J);
  if (!scratch || scratch_bytes < s.bytes) return fail(VISS_ERR_WORKSPACE, "pixel order scratch too small");
  s.layout(scratch, J);
  int rc = launch_pixel_keys(l, m, n, J, s.k0, s.i0, st);
  if (rc) return rc;
  size_t cb = s.cub_bytes;
  VISS_CUDA(cub::DeviceRadixSort::SortPairs(s.cub, cb, s.k0, s.k1, s.i0, perm, J, 0, 23, st));
  return VISS_OK;
}

}  // namespace viss
