// Diagnostic translation unit, compiled with nvcc's DEFAULT floating-point
// contraction (-fmad=true), unlike the prover's main unit.  It evaluates the
// equal-split expression the way the reference writes it in
// subintervals.hpp:35-41 (a plain `lb + diff * i`), so a test can check that
// nvcc's contraction of it equals the explicit FMA in cc::subinterval.
#include <cuda_runtime.h>
#include <stddef.h>

__global__ void k_split_plain(const double* lo, const double* hi, const int* idx, const int* cnt, double* out, size_t n) {
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    double lb = lo[t];
    double ub = hi[t];
    int i = idx[t];
    int k = cnt[t];
    double diff = ub - lb;
    diff /= k;
    double l = lb + diff * i;
    double u = lb + diff * (i + 1);
    if (i + 1 == k) u = ub;
    out[2 * t] = l;
    out[2 * t + 1] = u;
}

extern "C" int cc_selftest_subinterval_contracted(const double* lo, const double* hi, const int* idx, const int* cnt,
                                                  double* out, size_t n, void* stream) {
    k_split_plain<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(lo, hi, idx, cnt, out, n);
    return cudaGetLastError() == cudaSuccess ? 0 : 1;
}
