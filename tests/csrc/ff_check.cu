// ff_check.cu — test kernel for the double-float conversions of pc_ff.cuh:
// ff_of_fast and f2d_fast (the integer-pipe forms, where ff_fast_ok /
// f2d_fast_ok admit them) against CUDA's conversions, element by element.
#include "pc_ff.cuh"

namespace {

__global__ void ff_check_kernel(const double* __restrict__ x, const float* __restrict__ f, long long n,
                                float* __restrict__ split, double* __restrict__ widen) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  // the fast forms where they apply, else the dispatching ones
  const pcg::ff a = pcg::ff_fast_ok(x[i]) ? pcg::ff_of_fast(x[i]) : pcg::ff_of(x[i]);
  const float h = __double2float_rn(x[i]);
  split[4 * i + 0] = a.hi;
  split[4 * i + 1] = a.lo;
  split[4 * i + 2] = h;
  split[4 * i + 3] = __double2float_rn(x[i] - (double)h);
  widen[2 * i + 0] = pcg::f2d_fast_ok(f[i]) ? pcg::f2d_fast(f[i]) : pcg::f2d_exact(f[i]);
  widen[2 * i + 1] = (double)f[i];
}

}  // namespace

// split: 4 n floats (ff_of hi, lo; the conversions' hi, lo); widen: 2 n
// doubles (f2d_exact, the conversion).  0 on success, else the CUDA error.
extern "C" int ff_check(const double* x, const float* f, long long n, float* split, double* widen) {
  if (n <= 0) return 0;
  ff_check_kernel<<<(unsigned)((n + 255) / 256), 256>>>(x, f, n, split, widen);
  const cudaError_t e = cudaDeviceSynchronize();
  return e == cudaSuccess ? 0 : (int)e;
}
