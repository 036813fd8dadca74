// shade.cu -- Moon shade windows per uvw (shade1M.cu:62-105, 218-225; the same code in
// shade10M.cu:63-105, 188-224 and shade30M.cu:56-98, 158-179) and the shadeM
// normalisation of the vis programs (vissGen10M_shade.cu:383-399).
//
// The windows are integers, so they are reproduced bit for bit:
//   - r = sqrtf(u*u + v*v + w*w) as the reference's kernel evaluates it:
//     fma(w, w, fma(u, u, v*v)), rounded once per operation (the contraction
//     nvcc picks for that expression; written out so no other one is possible);
//   - the mean radius is the reference's FP32 sum, thrust::transform_reduce over
//     the complex r array with plus<float> from 0.0f (shade1M.cu:219): the same
//     CUB reduction with the same iterator, offset and operator types, hence the
//     same tiling and summation order on the same GPU, then `sum / K` in float
//     on the host;
//   - r0 = atanf(1737.74f / (mean_r + 1737.74f)), dtheta = (float)(2 pi / RES) and
//     dphi = (float)(pi / RES) are computed on the host, as the reference does
//     (shade1M.cu:222-224), and passed to the window kernel;
//   - the window arithmetic follows ShadeMatrix's float operation order.
// The reference materialises r, theta and phi as complex arrays; only r is
// materialised here (for the sum), theta and phi stay in registers.
#include <cub/device/device_reduce.cuh>
#include <thrust/complex.h>
#include <thrust/device_ptr.h>
#include <thrust/device_vector.h>
#include <thrust/functional.h>

#include "viss_internal.cuh"

namespace viss {

// r of Cart2SphKernel (shade1M.cu:67): the reference's contraction of u*u + v*v + w*w.
__device__ __forceinline__ float shade_radius(float u, float v, float w) {
  return __fsqrt_rn(__fmaf_rn(w, w, __fmaf_rn(u, u, __fmul_rn(v, v))));
}

// r as the reference stores it: complex<float>(r, 0) per uvw.
__global__ void shade_radius_kernel(const float* u, const float* v, const float* w, int64_t K, float2* r) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < K) r[k] = make_float2(shade_radius(u[k], v[k], w[k]), 0.f);
}

// The transform of the reference's sum: the real part of a complex r.
struct ShadeRealPart {
  __host__ __device__ float operator()(const thrust::complex<float>& c) const { return c.real(); }
};

// The iterator type of `r.begin()` for the reference's device_vector<complex<float>> r.
using ShadeRIter = thrust::device_vector<thrust::complex<float>>::iterator;

// The reference's FP32 sum of r (thrust::transform_reduce -> this CUB call, 32-bit
// offsets below 2^31 items).  d_temp == nullptr: returns the temporary size in *bytes.
static cudaError_t shade_rsum(void* d_temp, size_t* bytes, const float2* r, int64_t K, float* out,
                              cudaStream_t st) {
  ShadeRIter first(thrust::device_pointer_cast(reinterpret_cast<thrust::complex<float>*>(const_cast<float2*>(r))));
  if (K <= (int64_t)INT32_MAX)
    return cub::DeviceReduce::TransformReduce(d_temp, *bytes, first, out, (int32_t)K, thrust::plus<float>(),
                                              ShadeRealPart(), 0.0f, st);
  return cub::DeviceReduce::TransformReduce(d_temp, *bytes, first, out, (int64_t)K, thrust::plus<float>(),
                                            ShadeRealPart(), 0.0f, st);
}

// ShadeMatrix (shade1M.cu:73-105) for one uvw, with the host's r0, dtheta, dphi.
__global__ void shade_windows_kernel(const float* u, const float* v, const float* w, int64_t K, int RES, float r0,
                                     float dtheta, float dphi, int32_t* out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= K) return;
  const float uk = u[k], vk = v[k], wk = w[k];
  const float r = shade_radius(uk, vk, wk);               // Cart2SphKernel (:67-69)
  float theta = atan2f(vk, uk);
  float phi = asinf(__fdiv_rn(wk, r));
  theta = __fadd_rn(theta, (float)kPi);                    // :78-83
  phi = __fadd_rn(phi, (float)(kPi / 2));
  theta = __fsub_rn((float)(2 * kPi), theta);
  phi = __fsub_rn((float)kPi, phi);
  const int thetaInd = (int)roundf(__fdiv_rn(theta, dtheta));  // :86-89
  const int phiInd = (int)roundf(__fdiv_rn(phi, dphi));
  const int thetaR = (int)roundf(__fdiv_rn(r0, dtheta));
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
  if (K < 0) return 0;
  size_t tmp = 0;
  if (K > 0 && shade_rsum(nullptr, &tmp, nullptr, K, nullptr, nullptr) != cudaSuccess) return 0;
  Carver c(nullptr);
  c.take<float2>((size_t)K);  // r as complex
  c.take<float>(64);          // the sum
  c.take<char>(tmp);          // CUB's temporary storage
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
  float mean_r = (float)mean_r_km;
  if (!(mean_r_km > 0.0)) {
    size_t tmp = 0;
    VISS_CUDA(shade_rsum(nullptr, &tmp, nullptr, K, nullptr, st));
    const size_t need = viss_shade_windows_workspace(K);
    if (!workspace || workspace_bytes < need) return fail(VISS_ERR_WORKSPACE, "shade workspace too small");
    if (reinterpret_cast<uintptr_t>(workspace) & 255) return fail(VISS_ERR_WORKSPACE, "workspace misaligned");
    Carver c(workspace);
    float2* r = c.take<float2>((size_t)K);
    float* sum = c.take<float>(64);
    void* temp = c.take<char>(tmp);
    shade_radius_kernel<<<nbk, 256, 0, st>>>(u, v, w, K, r);
    VISS_LAUNCH_CHECK("shade_radius_kernel");
    VISS_CUDA(shade_rsum(temp, &tmp, r, K, sum, st));
    float sum_r = 0.f;
    VISS_CUDA(cudaMemcpyAsync(&sum_r, sum, sizeof(float), cudaMemcpyDeviceToHost, st));
    VISS_CUDA(cudaStreamSynchronize(st));
    mean_r = sum_r / (float)(size_t)K;  // `sum_r / r.size()` (shade1M.cu:220)
  }
  // shade1M.cu:222-224, on the host as there
  const float r0 = atanf(1737.74f / (mean_r + 1737.74f));
  const float dtheta = (float)(2 * M_PI / RES);
  const float dphi = (float)(M_PI / RES);
  shade_windows_kernel<<<nbk, 256, 0, st>>>(u, v, w, K, RES, r0, dtheta, dphi, out);
  VISS_LAUNCH_CHECK("shade_windows_kernel");
  if (mean_r_out) *mean_r_out = (double)mean_r;
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
