// finemap.cu -- non-identity fine->coarse sky maps.
//
// The reference's skies are a fine grid (X = RES^2 pixels, brightness FF) mapped
// onto J coarse pixels (directions l, m, n): NX[i] is the 1-based coarse pixel of
// fine pixel i; (countLoc, NXq) is its inverse, the fine pixels of every coarse
// pixel in ascending order (built in-program at 1M, vissGen1M_shade_optim1.cu:54-115,
// read from lmn10M/{countLoc,NXq}.txt at 10M, vissGen10M_shade.cu:261-286).
// visscal averages a coarse pixel's fine members, each replaced by 240 inside
// the visibility's window (vissGen10M_shade.cu:120-136).
//
//   viss_nxq:          NX -> (countLoc, NXq) with a stable radix sort (the
//                      reference counts and scans NX once per coarse pixel, O(J X)).
//   prep_fine_map:     per coarse pixel the mean brightness of its members, their
//                      bounding box on the fine grid and their range in the member
//                      list; per sky tile the range of fine indices it covers.
//                      The vis kernel decides most (visibility, pixel) terms from
//                      the box and walks the members only where a window cuts it.
#include <cub/cub.cuh>

#include "viss_internal.cuh"

namespace viss {

// key = coarse pixel q when NX[i] - 1 is exactly the float value of an integer
// q in [0, J) (the reference's `NX[i] - 1 == q` float test), J otherwise.
__global__ void nxq_keys_kernel(const float* __restrict__ NX, int64_t X, int J, uint32_t* keys, int32_t* vals,
                                int32_t* countLoc) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= X) return;
  const float v = NX[i] - 1.0f;
  uint32_t key = (uint32_t)J;
  if (v >= 0.f && v < (float)J && v == floorf(v)) key = (uint32_t)v;
  keys[i] = key;
  vals[i] = (int32_t)i;
  if (key < (uint32_t)J) atomicAdd(countLoc + key, 1);
}

static int key_bits(int64_t J) {
  int b = 1;
  while (b < 32 && ((int64_t)1 << b) <= J) ++b;
  return b;
}

struct NxqLayout {
  uint32_t *keys = nullptr, *keys_out = nullptr;
  int32_t* vals = nullptr;
  void* temp = nullptr;
  size_t temp_bytes = 0, bytes = 0;
  void layout(void* ws, int64_t X, int64_t J) {
    Carver c(ws);
    keys = c.take<uint32_t>(X > 0 ? X : 1);
    keys_out = c.take<uint32_t>(X > 0 ? X : 1);
    vals = c.take<int32_t>(X > 0 ? X : 1);
    temp_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, (uint32_t*)nullptr, (uint32_t*)nullptr,
                                    (int32_t*)nullptr, (int32_t*)nullptr, (int)(X > 0 ? X : 1), 0, key_bits(J));
    temp = c.take<char>(temp_bytes);
    bytes = c.size();
  }
};

// ------------------------------------------------------------------ map prep
// Per coarse pixel: its members as ints (NXq[c] truncated as the reference does,
// `long long locViss = NXq[...]`; indices outside [0, X), or a member list
// running past X, set flag bit 8 and make the pixel NaN), their mean brightness,
// bounding box on the fine grid and range in the list.
__global__ void map_pixels_kernel(const float* __restrict__ NXq_f, const int32_t* __restrict__ NXq_i,
                                  const int32_t* __restrict__ countLoc, const int* __restrict__ start,
                                  const float* __restrict__ FF, int64_t J, int64_t Jpad, int64_t X, int res, int trunc,
                                  int* members, float* base, int4* box, int2* mem, int2* tile_rng, int* flags) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= Jpad) return;
  if (j >= J) {
    base[j] = 0.f;
    box[j] = make_int4(1, 0, 1, 0);  // empty
    mem[j] = make_int2(0, 0);
    return;
  }
  const int s = start[j];
  int cnt = countLoc[j];
  double sum = 0.0;
  if (cnt < 0 || (int64_t)s + cnt > X) {
    atomicOr(flags + FLAG_ERR, 8);
    cnt = 0;
    sum = nan("");
  }
  int qmin = 0x7fffffff, qmax = -1, rmin = 0x7fffffff, rmax = -1, imin = 0x7fffffff, imax = -1;
  for (int c = 0; c < cnt; ++c) {
    const int64_t i64 = NXq_f ? (int64_t)NXq_f[s + c] : (int64_t)NXq_i[s + c];
    if (i64 < 0 || i64 >= X) {
      atomicOr(flags + FLAG_ERR, 8);
      members[s + c] = -1;
      sum = nan("");
      continue;
    }
    const int i = (int)i64;
    members[s + c] = i;
    float ff = FF[i];
    if (trunc) ff = (float)(int)ff;
    sum += ff;
    const int q = i / res, r = i - q * res;
    qmin = min(qmin, q); qmax = max(qmax, q);
    rmin = min(rmin, r); rmax = max(rmax, r);
    imin = min(imin, i); imax = max(imax, i);
  }
  base[j] = (float)(sum / (double)cnt);  // 0/0 = NaN for an empty pixel, as the reference
  box[j] = make_int4(qmin, qmax, rmin, rmax);
  mem[j] = make_int2(s, cnt);
  if (cnt > 0) {
    atomicMin(&tile_rng[j / VIS_P].x, imin);
    atomicMax(&tile_rng[j / VIS_P].y, imax);
  }
}

__global__ void tile_rng_init_kernel(int2* tile_rng, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) tile_rng[t] = make_int2(0x7fffffff, -1);
}

size_t fine_map_scratch(int64_t J) {
  size_t temp = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, temp, (const int32_t*)nullptr, (int*)nullptr, (int)(J > 0 ? J : 1));
  Carver c(nullptr);
  c.take<int>(J > 0 ? J : 1);
  c.take<char>(temp);
  return c.size();
}

int prep_fine_map(const float* NXq_f, const int32_t* NXq_i, const int32_t* countLoc, const float* FF, int64_t J,
                  int64_t X, int res, int trunc, int64_t Jpad, float* base, int4* box, int2* mem, int* members,
                  int2* tile_rng, void* scratch, size_t scratch_bytes, int* flags, cudaStream_t st) {
  if (J <= 0) return VISS_OK;
  Carver c(scratch);
  int* start = c.take<int>(J);
  size_t temp = 0;
  cub::DeviceScan::ExclusiveSum(nullptr, temp, countLoc, start, (int)J);
  void* tmp = c.take<char>(temp);
  if (c.size() > scratch_bytes) return fail(VISS_ERR_WORKSPACE, "fine map scratch too small");
  VISS_CUDA(cub::DeviceScan::ExclusiveSum(tmp, temp, countLoc, start, (int)J, st));
  count_launch();
  const int64_t ntiles = Jpad / VIS_P;
  tile_rng_init_kernel<<<(unsigned)((ntiles + 255) / 256), 256, 0, st>>>(tile_rng, ntiles);
  VISS_LAUNCH_CHECK("tile_rng_init_kernel");
  map_pixels_kernel<<<(unsigned)((Jpad + 255) / 256), 256, 0, st>>>(NXq_f, NXq_i, countLoc, start, FF, J, Jpad, X,
                                                                     res > 0 ? res : 1, trunc, members, base, box,
                                                                     mem, tile_rng, flags);
  VISS_LAUNCH_CHECK("map_pixels_kernel");
  return VISS_OK;
}

}  // namespace viss

using namespace viss;

extern "C" size_t viss_nxq_workspace(int64_t X, int64_t J) {
  if (X < 0 || J < 0) return 0;
  NxqLayout L;
  L.layout(nullptr, X, J);
  return L.bytes;
}

extern "C" int viss_nxq(const float* NX, int64_t X, int64_t J, int32_t* countLoc, int32_t* NXq, void* workspace,
                        size_t workspace_bytes, void* stream) {
  if (X < 0 || J < 1 || X > ((int64_t)1 << 31) - 1 || J > ((int64_t)1 << 24))
    return fail(VISS_ERR_RANGE, "viss_nxq: need 0 <= X < 2^31 and 1 <= J <= 2^24 (float coarse ids)");
  if ((X > 0 && (!NX || !NXq)) || !countLoc) return fail(VISS_ERR_INVALID, "viss_nxq: NULL argument");
  NxqLayout L;
  L.layout(nullptr, X, J);
  if (!workspace || workspace_bytes < L.bytes || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return fail(VISS_ERR_WORKSPACE, "viss_nxq: workspace missing, misaligned or below " + std::to_string(L.bytes));
  L.layout(workspace, X, J);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  VISS_CUDA(cudaMemsetAsync(countLoc, 0, sizeof(int32_t) * (size_t)J, st));
  if (X == 0) return VISS_OK;
  nxq_keys_kernel<<<(unsigned)((X + 255) / 256), 256, 0, st>>>(NX, X, (int)J, L.keys, L.vals, countLoc);
  VISS_LAUNCH_CHECK("nxq_keys_kernel");
  // stable: fine indices of one coarse pixel stay ascending; unmapped ones go last
  VISS_CUDA(cub::DeviceRadixSort::SortPairs(L.temp, L.temp_bytes, L.keys, L.keys_out, L.vals, NXq, (int)X, 0,
                                            key_bits(J), st));
  count_launch();
  return VISS_OK;
}
