// Self-test of the integer-pipe float <-> double conversions (f2d, d2f in dyn_common.cuh) against the
// hardware conversions, bit for bit. The mixed-precision kernels use them wherever an FP32 value meets an
// FP64 one, so the mixed path's results equal those of plain casts only while this test finds nothing.
#include "dyn_common.cuh"

namespace atsat {
namespace {

__device__ __forceinline__ uint64_t mix64(uint64_t x) {          // splitmix64's output function
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// A copy the compiler cannot see through: (float)(double)f would otherwise fold to f, which keeps a
// signaling NaN that the hardware narrowing quiets.
__device__ __forceinline__ double opaque(double d) {
    double r;
    asm volatile("mov.b64 %0, %1;" : "=d"(r) : "d"(d));
    return r;
}

__device__ __forceinline__ uint64_t bits_of(double d) {
    uint32_t lo, hi;
    split_f64(d, lo, hi);
    return ((uint64_t)hi << 32) | lo;
}

// every binary32 encoding: widening, and narrowing of the widened value
__global__ void __launch_bounds__(256) conv_float_kernel(unsigned long long* bad) {
    unsigned long long nw = 0, nn = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; n < (1ull << 32); n += stride) {
        const float f = __uint_as_float((uint32_t)n);
        const double mine = f2d(f), hw = opaque((double)f);
        nw += bits_of(mine) != bits_of(hw);
        nn += __float_as_uint(d2f(hw)) != __float_as_uint((float)hw);
    }
    if (nw) atomicAdd(bad, nw);
    if (nn) atomicAdd(bad + 1, nn);
}

// hashed binary64 encodings, narrowing: a quarter raw patterns; the rest with biased exponents
// 860..1179 (binary32's normal range is 897..1150), of those a third exact ties of the rounding
// (the 29 dropped bits 0x10000000) and a third one unit either side of a tie
__global__ void __launch_bounds__(256) conv_double_kernel(uint64_t n_total, unsigned long long* bad) {
    unsigned long long nn = 0;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t n = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; n < n_total; n += stride) {
        const uint64_t h = mix64(n);
        uint64_t b = h;
        const int kind = (int)(n & 3u);
        if (kind != 0) {
            const uint64_t e = 860u + (h >> 52) % 320u;
            b = (h & 0x800FFFFFFFFFFFFFull) | (e << 52);
            if (kind == 2) b = (b & ~0x1FFFFFFFull) | 0x10000000ull;
            if (kind == 3) b = (b & ~0x1FFFFFFFull) | (((h >> 7) & 1u) ? 0x10000001ull : 0x0FFFFFFFull);
        }
        const double d = __longlong_as_double((long long)b);
        nn += __float_as_uint(d2f(d)) != __float_as_uint((float)d);
    }
    if (nn) atomicAdd(bad + 2, nn);
}

}  // namespace

cudaError_t run_conv_selftest(uint64_t n_doubles, unsigned long long* bad3, cudaStream_t s) {
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int blocks = 8 * (sms > 0 ? sms : 1);
    conv_float_kernel<<<blocks, 256, 0, s>>>(bad3);
    if (n_doubles) conv_double_kernel<<<blocks, 256, 0, s>>>(n_doubles, bad3);
    return cudaGetLastError();
}

}  // namespace atsat

extern "C" int atsat_dyn_conv_selftest(int32_t device, uint64_t n_doubles, uint64_t* bad_widen,
                                       uint64_t* bad_narrow) {
    if (!bad_widen || !bad_narrow) return ATSAT_DYN_E_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) return ATSAT_DYN_E_CUDA;
    unsigned long long* d = nullptr;
    if (cudaMalloc(&d, 3 * sizeof(unsigned long long)) != cudaSuccess) return ATSAT_DYN_E_NOMEM;
    unsigned long long h[3] = {0, 0, 0};
    cudaError_t e = cudaMemset(d, 0, sizeof(h));
    if (e == cudaSuccess) e = atsat::run_conv_selftest(n_doubles, d, nullptr);
    if (e == cudaSuccess) e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return ATSAT_DYN_E_CUDA;
    *bad_widen = h[0];
    *bad_narrow = h[1] + h[2];
    return ATSAT_DYN_OK;
}
