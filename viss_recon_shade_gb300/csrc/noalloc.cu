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
// process exits.  Host code cannot use the array's name as a device address:
// every call asks the runtime for the current device's address of the array
// (cudaGetSymbolAddress, with that device current).  After the module is
// loaded this is a host-side lookup, and because it is repeated on every call a
// context torn down and rebuilt (cudaDeviceReset) gets the new address.  The
// first call on a device (or after a reset) loads the module, so it should come
// before any stream capture.  All calls share the one buffer and it keeps the
// previous call's contents: the pass clears what must start at zero (its flag
// words) itself, and calls whose work overlaps on the GPU (different streams or
// threads without ordering) race on the buffer.
//
// The pass records input problems in the scratch's flag words instead of
// reading out of bounds (viss_workspace_flags reads them for a caller
// workspace).  A caller of this entry point cannot reach the scratch, so the
// call reads them itself once the pass has completed: it synchronises `stream`
// and returns the problem as a status.
#include "viss_internal.cuh"

namespace viss {

static __device__ __align__(256) unsigned char g_noalloc_scratch[VISS_NOALLOC_SCRATCH_BYTES];

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
  // the current device's address of the array, looked up on every call
  void* scratch = nullptr;
  VISS_CUDA(cudaGetSymbolAddress(&scratch, g_noalloc_scratch));
  // the same checks and pass as viss_vis_dft, on the built-in scratch
  int rc = viss_vis_dft_batch(cfg, sky, vis, nullptr, geo, &tn, V, scratch, (size_t)VISS_NOALLOC_SCRATCH_BYTES,
                              stream);
  if (rc != VISS_OK || vis->K == 0 || sky->J == 0) return rc;
  // input problems the pass recorded (the flag words are the scratch's first carve)
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int32_t err = 0;
  VISS_CUDA(cudaMemcpyAsync(&err, static_cast<const int32_t*>(scratch) + FLAG_ERR, sizeof(err),
                            cudaMemcpyDeviceToHost, st));
  VISS_CUDA(cudaStreamSynchronize(st));
  if (err & 1) return fail(VISS_ERR_RANGE, "viss_vis_dft_noalloc: a |u|, |v| or |w| of 2^30 or more");
  if (err & 2)
    return fail(VISS_ERR_INVALID, "viss_vis_dft_noalloc: a snapshot or satellite index outside the geometry");
  if (err) return fail(VISS_ERR_INVALID, "viss_vis_dft_noalloc: input flags " + std::to_string(err));
  return VISS_OK;
}
