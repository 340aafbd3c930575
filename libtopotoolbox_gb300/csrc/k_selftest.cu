// Self-checks of device arithmetic that the kernels rely on for
// bit-exactness (no counterpart in the reference).
#include "tt_internal.cuh"

namespace tt {
namespace {

// Every float32 bit pattern: div_by_sqrt2 against the IEEE division.
__global__ void check_div_sqrt2_kernel(unsigned long long *__restrict__ bad,
                                       unsigned *__restrict__ first) {
  const float s = 1.41421353816986083984375f;
  unsigned long long nbad = 0;
  unsigned fb = 0xffffffffu;
  for (unsigned long long b = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
       b < (1ULL << 32); b += (unsigned long long)gridDim.x * blockDim.x) {
    const float x = __uint_as_float((unsigned)b);
    const float a = div_by_sqrt2(x), c = __fdiv_rn(x, s);
    const bool same = __float_as_uint(a) == __float_as_uint(c) || (isnan(a) && isnan(c));
    if (!same) {
      nbad++;
      fb = min(fb, (unsigned)b);
    }
  }
  if (nbad) {
    atomicAdd(bad, nbad);
    atomicMin(first, fb);
  }
}

}  // namespace
}  // namespace tt

extern "C" tt_cuda_status tt_cuda_selftest_div_sqrt2(unsigned long long *mismatches,
                                                     unsigned *first_bad) {
  using namespace tt;
  tt_cuda_status s = TT_CUDA_SUCCESS;
  int ndev = 0;
  if (!mismatches || !first_bad) {
    s = TT_CUDA_ERR_INVALID_ARGUMENT;
  } else if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    s = TT_CUDA_ERR_NO_DEVICE;
  } else {
    unsigned long long *d = nullptr;
    if (cudaMalloc(&d, 16) != cudaSuccess) {
      cudaGetLastError();
      s = TT_CUDA_ERR_ALLOC;
    } else {
      unsigned long long init[2] = {0, 0xffffffffULL};
      cudaMemcpy(d, init, 16, cudaMemcpyHostToDevice);
      TT_LAUNCH(check_div_sqrt2_kernel, sm_count() * 8, 256, 0, 0, d,
                reinterpret_cast<unsigned *>(d + 1));
      unsigned long long h[2] = {0, 0};
      if (cudaMemcpy(h, d, 16, cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        s = TT_CUDA_ERR_CUDA;
      }
      *mismatches = h[0];
      *first_bad = (unsigned)h[1];
      cudaFree(d);
    }
  }
  set_status(s);
  return s;
}
