// ref_thrust.cu -- the reference's thrust call sites, restated.
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/ and by bench.py's reference legs
// (oracle/ref_thrust.py), never by the product.  The reference's kernels run
// from its own sources (oracle/ref_cuda.py); what it does between them with
// thrust (NVIDIA CCCL, shipped with CUDA 13.0: CCCL 3.0.1) is restated here
// with the same calls on the same element, iterator and functor types, so the
// summation order and the sort/unique results are the reference's.
//
//   shade1M.cu:54-59, 219-220   mean radius: thrust::transform_reduce over the
//                               device_vector<complex<float>> r (real parts),
//                               plus<float> from 0.0f, then sum / r.size()
//   MIncline_generate_uvw_float.cu:60-80, 374-397
//                               per satellite pair: thrust::sort with SortCompare
//                               (u, then v, then w) and thrust::unique with
//                               UniqueCompare (all three equal) on the pair's
//                               tuple<float,float,float> rows; the unique rows are
//                               appended to a global vector, which is sorted and
//                               uniqued the same way at the end
#include <cuda_runtime.h>
#include <stdint.h>

#include <thrust/complex.h>
#include <thrust/device_ptr.h>
#include <thrust/device_vector.h>
#include <thrust/execution_policy.h>
#include <thrust/functional.h>
#include <thrust/sort.h>
#include <thrust/transform_reduce.h>
#include <thrust/tuple.h>
#include <thrust/unique.h>

namespace {

struct RealPartExtractor {  // shade1M.cu:54-59
  __host__ __device__ float operator()(const thrust::complex<float>& c) const { return c.real(); }
};

using Row = thrust::tuple<float, float, float>;
static_assert(sizeof(Row) == 12, "a row is three packed floats, as computeUVW writes them");

struct RowLess {  // SortCompare, MIncline_generate_uvw_float.cu:60-71
  __host__ __device__ bool operator()(const Row& a, const Row& b) const {
    if (thrust::get<0>(a) != thrust::get<0>(b)) return thrust::get<0>(a) < thrust::get<0>(b);
    if (thrust::get<1>(a) != thrust::get<1>(b)) return thrust::get<1>(a) < thrust::get<1>(b);
    return thrust::get<2>(a) < thrust::get<2>(b);
  }
};

struct RowEqual {  // UniqueCompare, :73-80
  __host__ __device__ bool operator()(const Row& a, const Row& b) const {
    return thrust::get<0>(a) == thrust::get<0>(b) && thrust::get<1>(a) == thrust::get<1>(b) &&
           thrust::get<2>(a) == thrust::get<2>(b);
  }
};

}  // namespace

extern "C" {

// Sum and mean of the real parts of K complex<float> (device pointer, e.g. the
// r array of the reference's Cart2SphKernel), the reference's way.
int ref_thrust_mean_r(const void* r_complex, int64_t K, float* sum_out, float* mean_out) {
  try {
    thrust::device_vector<thrust::complex<float>> r((size_t)K);
    if (cudaMemcpy(thrust::raw_pointer_cast(r.data()), r_complex, sizeof(thrust::complex<float>) * (size_t)K,
                   cudaMemcpyDeviceToDevice) != cudaSuccess)
      return -1;
    const float sum_r = thrust::transform_reduce(r.begin(), r.end(), RealPartExtractor(), 0.0f, thrust::plus<float>());
    *sum_out = sum_r;
    *mean_out = sum_r / r.size();
    return 0;
  } catch (...) {
    return -1;
  }
}

// In place on n rows of (u, v, w) floats (device, 12 bytes a row): sort with
// SortCompare, unique with UniqueCompare; returns the unique count (< 0 on error).
int64_t ref_thrust_sort_unique(void* rows, int64_t n) {
  try {
    thrust::device_ptr<Row> first(static_cast<Row*>(rows));
    thrust::sort(thrust::device, first, first + n, RowLess());
    auto e = thrust::unique(thrust::device, first, first + n, RowEqual());
    if (cudaDeviceSynchronize() != cudaSuccess) return -1;
    return (int64_t)(e - first);
  } catch (...) {
    return -1;
  }
}

}  // extern "C"
