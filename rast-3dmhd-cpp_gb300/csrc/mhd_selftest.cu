// mhd_selftest.cu -- on-device check of the integer-pipe conversions of
// mhd_convert.cuh against the hardware conversions.
#include "mhd_context.h"
#include "mhd_convert.cuh"

namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

__device__ __forceinline__ bool same_f32(float a, float b) {
    return (a != a && b != b) || __float_as_uint(a) == __float_as_uint(b);
}
__device__ __forceinline__ bool same_f64(double a, double b) {
    return (a != a && b != b) || __double_as_longlong(a) == __double_as_longlong(b);
}

// Test patterns: random bits; doubles near the float range edges and on
// rounding ties; random floats (all exponents, subnormals included).
__global__ void k_selftest(long long n, unsigned long long seed, unsigned long long* bad) {
    unsigned long long nb = 0;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        const unsigned long long h = mix64(seed ^ mix64((unsigned long long)t));
        double d;
        switch (t & 3) {
            case 0: d = __longlong_as_double((long long)h); break;
            case 1: {  // exponents around the float range, low bits forming ties
                const unsigned long long e = 1023 - 160 + (h >> 56) % 330;
                unsigned long long m = h & 0xfffffffffffffull;
                if ((h >> 40) & 1) m = (m & ~0x1fffffffull) | 0x10000000ull;  // exact tie
                d = __longlong_as_double((long long)((e << 52) | m | (h & 0x8000000000000000ull)));
                break;
            }
            case 2: d = 1.0 + (double)(h >> 11) * 0x1p-53; break;
            default: {
                const float f = __uint_as_float((unsigned)(h >> 32));
                if (!same_f64(mhd::widen_f32(f), (double)f)) nb++;
                d = __longlong_as_double((long long)h) * 0x1p-900;
            }
        }
        if (!same_f32(mhd::narrow_f64(d), __double2float_rn(d))) nb++;
        const float f = __double2float_rn(d);
        if (!same_f64(mhd::widen_f32(f), (double)f)) nb++;
    }
    if (nb) atomicAdd(bad, nb);
}

}  // namespace

extern "C" int mhd_selftest_convert(long long n, unsigned long long seed, long long* mismatches) {
    if (n < 0 || !mismatches) return MHD_ERR_INVALID;
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, sizeof(unsigned long long)) != cudaSuccess) return MHD_ERR_NOMEM;
    cudaMemset(d, 0, sizeof(unsigned long long));
    k_selftest<<<152 * 8, 256>>>(n, seed, d);
    unsigned long long h = 0;
    cudaError_t e = cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return MHD_ERR_CUDA;
    *mismatches = (long long)h;
    return MHD_OK;
}
