// shade.cu -- Moon shade windows per uvw (shade1M.cu:62-105, 218-225) and the
// shadeM normalisation of the vis programs (vissGen10M_shade.cu:383-399).
//
// The reference materialises r, theta, phi as complex arrays (Cart2SphKernel),
// reduces r with thrust in FP32, then forms the windows (ShadeMatrix).  Here a
// deterministic two-level double reduction gives the mean radius and one
// kernel evaluates the window arithmetic of ShadeMatrix per uvw in the same
// float operation order, with r, theta, phi kept in registers.
#include "viss_internal.cuh"

namespace viss {

constexpr int SHADE_BS = 256;

__global__ void shade_rsum_kernel(const float* u, const float* v, const float* w, int64_t K, double* part) {
  __shared__ double red[SHADE_BS / 32];
  double acc = 0.0;
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < K; k += (int64_t)gridDim.x * blockDim.x) {
    const float r = sqrtf(u[k] * u[k] + v[k] * v[k] + w[k] * w[k]);
    acc += (double)r;
  }
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < SHADE_BS / 32; ++i) s += red[i];
    part[blockIdx.x] = s;
  }
}

__global__ void shade_mean_kernel(const double* part, int nb, int64_t K, double* mean) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < nb; ++i) s += part[i];
    mean[0] = s / (double)K;
  }
}

// ShadeMatrix (shade1M.cu:73-105) for one uvw.  mean_r is read from device
// memory so the pass needs no host round trip.
__global__ void shade_windows_kernel(const float* u, const float* v, const float* w, int64_t K, int RES,
                                     const double* mean_r_dev, double mean_r_host, int32_t* out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  const float mean_r = (float)(mean_r_dev ? mean_r_dev[0] : mean_r_host);
  const float r0 = atanf(1737.74f / (mean_r + 1737.74f));  // shade1M.cu:223
  const float dtheta = (float)(2 * kPi / RES);
  const float dphi = (float)(kPi / RES);
  const float uk = u[k], vk = v[k], wk = w[k];
  const float r = sqrtf(uk * uk + vk * vk + wk * wk);     // Cart2SphKernel (:67-69)
  float theta = atan2f(vk, uk);
  float phi = asinf(wk / r);
  theta = theta + (float)kPi;                              // :78-83
  phi = phi + (float)(kPi / 2);
  theta = (float)(2 * kPi) - theta;
  phi = (float)kPi - phi;
  const int thetaInd = (int)roundf(theta / dtheta);        // :86-89
  const int phiInd = (int)roundf(phi / dphi);
  const int thetaR = (int)roundf(r0 / dtheta);
  const int phiR = (int)roundf((float)(thetaR / 2));
  int tS = thetaInd - thetaR, tE = thetaInd + thetaR;
  int pS = phiInd - phiR, pE = phiInd + phiR;
  if (tS <= 0) tS += RES;
  if (tE > RES) tE -= RES;
  if (pS <= 0) pS += RES;
  if (pE > RES) pE -= RES;
  reinterpret_cast<int4*>(out)[k] = make_int4(tS, tE, pS, pE);
}

__global__ void normalise_shade_kernel(const int32_t* raw, int64_t K, int32_t* M) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  const int4 a = reinterpret_cast<const int4*>(raw)[k];
  reinterpret_cast<int4*>(M)[k] = make_int4(min(a.x, a.y) - 1, max(a.x, a.y) - 1, min(a.z, a.w) - 1,
                                            max(a.z, a.w) - 1);
}

}  // namespace viss

using namespace viss;

extern "C" {

size_t viss_shade_windows_workspace(int64_t K) {
  (void)K;
  Carver c(nullptr);
  c.take<double>(1024);
  c.take<double>(4);
  return c.size();
}

int viss_shade_windows(const float* u, const float* v, const float* w, int64_t K, int RES, double mean_r_km,
                       int32_t* out, double* mean_r_out, void* workspace, size_t workspace_bytes, void* stream) {
  if (K < 0) return fail(VISS_ERR_RANGE, "K < 0");
  if (RES < 1) return fail(VISS_ERR_RANGE, "RES >= 1");
  if (K == 0) return VISS_OK;
  if (!u || !v || !w || !out) return fail(VISS_ERR_INVALID, "NULL argument");
  if (reinterpret_cast<uintptr_t>(out) & 15) return fail(VISS_ERR_INVALID, "out must be 16-byte aligned");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned nbk = (unsigned)((K + 255) / 256);
  if (mean_r_km > 0.0) {
    shade_windows_kernel<<<nbk, 256, 0, st>>>(u, v, w, K, RES, nullptr, mean_r_km, out);
    VISS_LAUNCH_CHECK("shade_windows_kernel");
    if (mean_r_out) *mean_r_out = mean_r_km;
    return VISS_OK;
  }
  const size_t need = viss_shade_windows_workspace(K);
  if (!workspace || workspace_bytes < need) return fail(VISS_ERR_WORKSPACE, "shade workspace too small");
  if (reinterpret_cast<uintptr_t>(workspace) & 255) return fail(VISS_ERR_WORKSPACE, "workspace misaligned");
  Carver c(workspace);
  double* part = c.take<double>(1024);
  double* mean = c.take<double>(4);
  int nb = (int)((K + SHADE_BS - 1) / SHADE_BS);
  if (nb > 1024) nb = 1024;
  shade_rsum_kernel<<<nb, SHADE_BS, 0, st>>>(u, v, w, K, part);
  VISS_LAUNCH_CHECK("shade_rsum_kernel");
  shade_mean_kernel<<<1, 32, 0, st>>>(part, nb, K, mean);
  VISS_LAUNCH_CHECK("shade_mean_kernel");
  shade_windows_kernel<<<nbk, 256, 0, st>>>(u, v, w, K, RES, mean, 0.0, out);
  VISS_LAUNCH_CHECK("shade_windows_kernel");
  if (mean_r_out) {
    VISS_CUDA(cudaMemcpyAsync(mean_r_out, mean, sizeof(double), cudaMemcpyDeviceToHost, st));
    VISS_CUDA(cudaStreamSynchronize(st));
  }
  return VISS_OK;
}

int viss_normalise_shade(const int32_t* raw, int64_t K, int32_t* M, void* stream) {
  if (K < 0) return fail(VISS_ERR_RANGE, "K < 0");
  if (K == 0) return VISS_OK;
  if (!raw || !M) return fail(VISS_ERR_INVALID, "NULL argument");
  if ((reinterpret_cast<uintptr_t>(raw) | reinterpret_cast<uintptr_t>(M)) & 15)
    return fail(VISS_ERR_INVALID, "arrays must be 16-byte aligned");
  normalise_shade_kernel<<<(unsigned)((K + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(raw, K, M);
  VISS_LAUNCH_CHECK("normalise_shade_kernel");
  return VISS_OK;
}

}  // extern "C"
