// The buoyancy reference level (the sin(theta)-weighted level mean of g p_stat / (r_mix R_mix t t_ref),
// RungeKutta_Sat_Turb.cpp:31-50) for callers that must not allocate device memory.
//
// Who needs this: a host program that hands all of the GPU's memory to its own pool allocator and
// forbids anyone else to call cudaMalloc (a fixed device-memory budget, no fragmentation from a
// library), and a time-stepping loop that cannot afford cudaMalloc / cudaFree on its critical path,
// where each of them costs latency and can synchronise the whole device. Such a caller already holds
// t and p_stat on the device (for example the device copies a handle exposes through
// atsat_dyn_device_field, or its own pool's buffers) and an output buffer; what it cannot provide is
// the reduction's scratch space. Here that scratch is a fixed array compiled into the library.
//
// The scratch is file-scope `static __device__` memory: every GPU that loads this library holds it
// (192 KB) until the process exits. In host code its name only stands for the symbol, so the host
// asks the runtime for its device address (cudaGetSymbolAddress) once per device, with that device
// current, and passes that address to the kernels.
#include <cstdio>
#include <mutex>

#include "dyn_common.cuh"

namespace atsat {
namespace {

constexpr int NA_CHUNKS = 16;          // j-chunks per level in the partial sums
constexpr int NA_THREADS = 256;
constexpr int NA_PARTIAL = ATSAT_DYN_NOALLOC_MAX_IM * NA_CHUNKS * 2;
constexpr int NA_TOTAL = NA_PARTIAL + ATSAT_DYN_NOALLOC_MAX_JM;   // partial sums, then the_z

// Shared by every call on a device; each call overwrites the parts it reads before reading them.
static __device__ __align__(256) double g_noalloc_scratch[NA_TOTAL];

constexpr int NA_MAX_DEVICES = 64;
double* g_scratch_dev[NA_MAX_DEVICES] = {};
std::mutex g_scratch_mu;

__global__ void __launch_bounds__(NA_THREADS) na_partial_kernel(const double* __restrict__ t,
                                                                const double* __restrict__ ps,
                                                                int64_t pitch, int jm, int km,
                                                                double g, double rR, double t_ref,
                                                                double* __restrict__ scratch) {
    const int i = blockIdx.x, chunk = blockIdx.y;
    const double* the_z = scratch + NA_PARTIAL;
    const int j0 = (int)((int64_t)jm * chunk / NA_CHUNKS), j1 = (int)((int64_t)jm * (chunk + 1) / NA_CHUNKS);
    double sum = 0.0, wsum = 0.0;
    const int n = (j1 - j0) * km;
    for (int e = threadIdx.x; e < n; e += NA_THREADS) {
        const int j = j0 + e / km, k = e % km;
        const int64_t c = ((int64_t)i * jm + j) * pitch + k;
        const double tc = t[c];
        if (!(tc > 0.0)) continue;                      // also skips NaN, as the reference does
        const double b = g * ps[c] / (rR * tc * t_ref);
        if (!isfinite(b)) continue;
        const double wgt = sin(the_z[j]);
        sum += wgt * b;
        wsum += wgt;
    }
    __shared__ double s_sum[NA_THREADS / 32], s_w[NA_THREADS / 32];
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_down_sync(0xffffffffu, sum, o);
        wsum += __shfl_down_sync(0xffffffffu, wsum, o);
    }
    if ((threadIdx.x & 31) == 0) { s_sum[threadIdx.x >> 5] = sum; s_w[threadIdx.x >> 5] = wsum; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int q = 0; q < NA_THREADS / 32; q++) { a += s_sum[q]; b += s_w[q]; }
        scratch[((int64_t)i * NA_CHUNKS + chunk) * 2 + 0] = a;   // every slot is written each call
        scratch[((int64_t)i * NA_CHUNKS + chunk) * 2 + 1] = b;
    }
}

__global__ void na_final_kernel(const double* __restrict__ scratch, int im, double* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= im) return;
    double s = 0.0, w = 0.0;
    for (int q = 0; q < NA_CHUNKS; q++) {
        s += scratch[((int64_t)i * NA_CHUNKS + q) * 2 + 0];
        w += scratch[((int64_t)i * NA_CHUNKS + q) * 2 + 1];
    }
    out[i] = (w > 0.0) ? s / w : 0.0;
}

// The scratch array's device address on the current device, looked up on the first call there.
cudaError_t scratch_address(double** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= NA_MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_dev[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_dev[dev] = static_cast<double*>(p);
    }
    *out = g_scratch_dev[dev];
    return cudaSuccess;
}

}  // namespace
}  // namespace atsat

extern "C" int atsat_dyn_buoyancy_ref_level_noalloc(const double* t, const double* p_stat, int64_t pitch,
                                                    int32_t im, int32_t jm, int32_t km, const double* the_z,
                                                    double g, double r_mix, double R_mix, double t_ref,
                                                    double* buoy_out, void* stream) {
    using namespace atsat;
    if (!t || !p_stat || !the_z || !buoy_out || im < 1 || jm < 1 || km < 1 || pitch < km)
        return ATSAT_DYN_E_INVALID;
    if (im > ATSAT_DYN_NOALLOC_MAX_IM || jm > ATSAT_DYN_NOALLOC_MAX_JM) {
        fprintf(stderr, "atsat_dyn_buoyancy_ref_level_noalloc: grid %d x %d exceeds the fixed scratch "
                        "(at most %d radial levels and %d latitude rows)\n",
                im, jm, ATSAT_DYN_NOALLOC_MAX_IM, ATSAT_DYN_NOALLOC_MAX_JM);
        return ATSAT_DYN_E_TOO_LARGE;
    }
    // an error left pending by earlier, unrelated work belongs to its owner: leave it there and stop
    if (cudaPeekAtLastError() != cudaSuccess) return ATSAT_DYN_E_CUDA;
    // the kernels run on the current device, so the caller's arrays must live there
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return ATSAT_DYN_E_CUDA;
    const void* on_device[3] = {t, p_stat, buoy_out};
    for (const void* q : on_device) {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
            cudaGetLastError();   // the lookup's own error, not a pending one (checked above)
            return ATSAT_DYN_E_INVALID;
        }
        const bool here = (a.type == cudaMemoryTypeDevice && a.device == dev) || a.type == cudaMemoryTypeManaged;
        if (!here) return ATSAT_DYN_E_INVALID;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    double* scratch = nullptr;
    if (scratch_address(&scratch) != cudaSuccess) return ATSAT_DYN_E_CUDA;
    // the colatitudes go into the scratch's tail; the partial sums are overwritten in full below
    if (cudaMemcpyAsync(scratch + NA_PARTIAL, the_z, sizeof(double) * (size_t)jm, cudaMemcpyHostToDevice, s) !=
        cudaSuccess)
        return ATSAT_DYN_E_CUDA;
    na_partial_kernel<<<dim3(im, NA_CHUNKS), NA_THREADS, 0, s>>>(t, p_stat, pitch, jm, km, g, r_mix * R_mix, t_ref,
                                                                 scratch);
    if (cudaGetLastError() != cudaSuccess) return ATSAT_DYN_E_CUDA;
    na_final_kernel<<<(im + 63) / 64, 64, 0, s>>>(scratch, im, buoy_out);
    if (cudaGetLastError() != cudaSuccess) return ATSAT_DYN_E_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return ATSAT_DYN_E_CUDA;
    return ATSAT_DYN_OK;
}
