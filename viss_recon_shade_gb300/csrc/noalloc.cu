// noalloc.cu -- the shaded visibility DFT for callers that cannot allocate
// device memory.
//
// Who needs it: a host that sizes and owns all GPU memory up front (a
// correlator or beam-former running a fixed-budget real-time loop, or an
// application whose own pool hands out every byte) must not see a library
// call cudaMalloc behind its back, and a latency-bound loop cannot afford the
// device-wide synchronisation cudaMalloc/cudaFree may imply.  viss_vis_dft
// already takes a caller workspace; this entry point removes even that
// obligation by using a scratch buffer that is part of the library image.
//
// The scratch is a file-scope __device__ array of VISS_NOALLOC_SCRATCH_BYTES
// (32 MiB).  Every GPU that loads the library keeps it resident until the
// process exits.  Host code cannot use the array's name as a device address;
// the first call on each device asks the runtime for that device's address
// (cudaGetSymbolAddress, with the device current) and caches it, so that first
// call on a device should come before any stream capture.  All calls share the
// one buffer and it keeps the previous call's contents: the pass clears what
// must start at zero (its flag words) itself, and calls whose work overlaps on
// the GPU (different streams or threads without ordering) race on the buffer.
#include <mutex>

#include "viss_internal.cuh"

namespace viss {

static __device__ __align__(256) unsigned char g_noalloc_scratch[VISS_NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set up once per device).
int scratch_address(void** out) {
  int dev = 0;
  VISS_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(VISS_ERR_UNSUPPORTED, "device ordinal beyond the scratch table");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    VISS_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return VISS_OK;
}
}  // namespace

}  // namespace viss

using namespace viss;

// Few sky chunks: their partial sums (chunks x K complex values) are the largest
// part of the scratch.  ~4 work items per resident CTA.
static viss_tuning noalloc_tuning(int64_t K) {
  viss_tuning t{};
  const int64_t nrb = (K + VIS_ROWS - 1) / VIS_ROWS, slots = (int64_t)device_sm_count() * VISS_VIS_MINB;
  t.vis_split = (nrb > 0 && nrb < 4 * slots) ? (int32_t)((4 * slots + nrb - 1) / nrb) : 1;
  return t;
}

extern "C" int viss_vis_dft_noalloc(const viss_dft_cfg* cfg, const viss_sky* sky, const viss_vis_set* vis,
                                    const viss_geometry* geo, float* V, void* stream) {
  if (!cfg || !sky || !vis) return fail(VISS_ERR_INVALID, "cfg, sky or vis is NULL");
  const viss_tuning tn = noalloc_tuning(vis->K);
  const size_t need = viss_vis_dft_batch_workspace(cfg, nullptr, vis->K, sky->J, geo, &tn);
  if (need > (size_t)VISS_NOALLOC_SCRATCH_BYTES)
    return fail(VISS_ERR_RANGE, "viss_vis_dft_noalloc: this pass needs " + std::to_string(need) +
                                    " bytes of scratch, more than the built-in " +
                                    std::to_string((size_t)VISS_NOALLOC_SCRATCH_BYTES) +
                                    " (use viss_vis_dft with a caller workspace)");
  void* scratch = nullptr;
  int rc = scratch_address(&scratch);
  if (rc) return rc;
  // the same checks and pass as viss_vis_dft, on the built-in scratch
  return viss_vis_dft_batch(cfg, sky, vis, nullptr, geo, &tn, V, scratch, (size_t)VISS_NOALLOC_SCRATCH_BYTES, stream);
}
