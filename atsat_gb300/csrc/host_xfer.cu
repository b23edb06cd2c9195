// Host <-> device transfers of bound fields by the SMs themselves: one kernel reads (or writes) the host
// arrays of every field of an upload (download) and the device field in its pitched layout, with no
// staging copy and no per-field copy-engine hop. An upload also writes a field's FP32 copy when asked (the
// mixed path's copies of the point inputs), from the values it already holds.
//
// On a Grace-Blackwell node the GPU reaches host memory over NVLink-C2C through the CPU's page tables
// (cudaDevAttrPageableMemoryAccessUsesHostPageTables): pinned and pageable memory alike, contiguous arrays
// and the reference's ragged rows (one allocation of km doubles per (i, j), lib/Array.cpp) alike. The
// host decides per binding whether this path applies (atsat_dyn.cu); it never runs where the device
// cannot address the memory.
#include <algorithm>
#include <cstdint>

#include "dyn_common.cuh"

namespace atsat {

namespace {

constexpr int XF_WARPS = 8;          // rows in flight per block: one warp per row
constexpr int XF_UNROLL = 4;         // 16-byte accesses in flight per lane before the stores

// One row of km doubles. The host side moves in 16-byte words from its first 16-byte boundary (a host row
// of km doubles starts 8 bytes past one every other row in a contiguous array): one leading and one
// trailing double go alone, lane 0 takes them. Device rows start on a 16-byte boundary (kp even, fields
// 256-byte aligned), so the device side uses 16-byte words when the host's boundary falls on its own.
__device__ __forceinline__ void gather_row(const double* src, double* dst, float* dst32, int km, int lane) {
    const int a = (int)((reinterpret_cast<uintptr_t>(src) >> 3) & 1u);
    const int np = (km - a) >> 1;
    const double2* s2 = reinterpret_cast<const double2*>(src + a);
    for (int p0 = 0; p0 < np; p0 += 32 * XF_UNROLL) {
        double2 v[XF_UNROLL];
#pragma unroll
        for (int q = 0; q < XF_UNROLL; q++) {
            const int p = p0 + lane + 32 * q;
            if (p < np) v[q] = s2[p];
        }
#pragma unroll
        for (int q = 0; q < XF_UNROLL; q++) {
            const int p = p0 + lane + 32 * q;
            if (p >= np) continue;
            double* d = dst + a + 2 * p;
            if (a) { d[0] = v[q].x; d[1] = v[q].y; }
            else *reinterpret_cast<double2*>(d) = v[q];
            if (dst32) { dst32[a + 2 * p] = d2f(v[q].x); dst32[a + 2 * p + 1] = d2f(v[q].y); }
        }
    }
    if (lane == 0) {
        if (a) { dst[0] = src[0]; if (dst32) dst32[0] = d2f(src[0]); }
        if ((km - a) & 1) { dst[km - 1] = src[km - 1]; if (dst32) dst32[km - 1] = d2f(src[km - 1]); }
    }
}

__device__ __forceinline__ void scatter_row(const double* src, double* dst, int km, int lane) {
    const int a = (int)((reinterpret_cast<uintptr_t>(dst) >> 3) & 1u);
    const int np = (km - a) >> 1;
    double2* d2 = reinterpret_cast<double2*>(dst + a);
    for (int p0 = 0; p0 < np; p0 += 32 * XF_UNROLL) {
        double2 v[XF_UNROLL];
#pragma unroll
        for (int q = 0; q < XF_UNROLL; q++) {
            const int p = p0 + lane + 32 * q;
            if (p >= np) continue;
            const double* s = src + a + 2 * p;
            v[q] = a ? make_double2(s[0], s[1]) : *reinterpret_cast<const double2*>(s);
        }
#pragma unroll
        for (int q = 0; q < XF_UNROLL; q++) {
            const int p = p0 + lane + 32 * q;
            if (p < np) d2[p] = v[q];
        }
    }
    if (lane == 0) {
        if (a) dst[0] = src[0];
        if ((km - a) & 1) dst[km - 1] = src[km - 1];
    }
}

// A contiguous host array is moved as one flat stream of 16-byte words (full host cache lines, none shared
// between warps); element e sits at device row e / km, column e % km. The row comes from an FP32 estimate
// corrected once: exact while e < 2^24 (the host keeps larger fields on the row path).
struct FlatPos {
    float inv_km;
    int km, kp;
    __device__ __forceinline__ int64_t dev(uint32_t e) const {
        int r = (int)((float)e * inv_km);
        int k = (int)e - r * km;
        if (k < 0) { r--; k += km; }
        else if (k >= km) { r++; k -= km; }
        return (int64_t)r * kp + k;
    }
};

// blockIdx.y: the field. Ragged rows: warps stride over the rows r = i * jm + j. Contiguous arrays: threads
// stride over the 16-byte words of the flat array, XF_UNROLL at a time.
__global__ void __launch_bounds__(XF_WARPS * 32)
host_gather_kernel(const __grid_constant__ HostBatch B, int64_t nrows, int km, int kp, int flat, float inv_km) {
    const HostField& fd = B.f[blockIdx.y];
    const int lane = threadIdx.x & 31;
    if (fd.rows || !flat) {
        const int64_t nw = (int64_t)gridDim.x * XF_WARPS;
        for (int64_t r = (int64_t)blockIdx.x * XF_WARPS + (threadIdx.x >> 5); r < nrows; r += nw) {
            const double* src = fd.rows ? fd.rows[r] : fd.base + r * km;
            gather_row(src, fd.dev + r * kp, fd.dev32 ? fd.dev32 + r * kp : nullptr, km, lane);
        }
        return;
    }
    const FlatPos pos{inv_km, km, kp};
    const uint32_t n = (uint32_t)(nrows * km);
    const uint32_t a = (uint32_t)((reinterpret_cast<uintptr_t>(fd.base) >> 3) & 1u);
    const uint32_t nwords = (n - a) >> 1;
    const double2* s2 = reinterpret_cast<const double2*>(fd.base + a);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t w0 = blockIdx.x * blockDim.x + threadIdx.x; w0 < nwords; w0 += stride * XF_UNROLL) {
        double2 v[XF_UNROLL];
#pragma unroll
        for (int q = 0; q < XF_UNROLL; q++) {
            const uint32_t w = w0 + q * stride;
            if (w < nwords) v[q] = s2[w];
        }
#pragma unroll
        for (int q = 0; q < XF_UNROLL; q++) {
            const uint32_t w = w0 + q * stride;
            if (w >= nwords) continue;
            const uint32_t e = a + 2 * w;
            const int64_t d0 = pos.dev(e), d1 = pos.dev(e + 1);
            fd.dev[d0] = v[q].x;
            fd.dev[d1] = v[q].y;
            if (fd.dev32) { fd.dev32[d0] = d2f(v[q].x); fd.dev32[d1] = d2f(v[q].y); }
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (a) {
            fd.dev[pos.dev(0)] = fd.base[0];
            if (fd.dev32) fd.dev32[pos.dev(0)] = d2f(fd.base[0]);
        }
        if ((n - a) & 1u) {
            fd.dev[pos.dev(n - 1)] = fd.base[n - 1];
            if (fd.dev32) fd.dev32[pos.dev(n - 1)] = d2f(fd.base[n - 1]);
        }
    }
}

__global__ void __launch_bounds__(XF_WARPS * 32)
host_scatter_kernel(const __grid_constant__ HostBatch B, int64_t nrows, int km, int kp, int flat, float inv_km) {
    const HostField& fd = B.f[blockIdx.y];
    const int lane = threadIdx.x & 31;
    if (fd.rows || !flat) {
        const int64_t nw = (int64_t)gridDim.x * XF_WARPS;
        for (int64_t r = (int64_t)blockIdx.x * XF_WARPS + (threadIdx.x >> 5); r < nrows; r += nw) {
            double* dst = fd.rows ? fd.rows[r] : fd.base + r * km;
            scatter_row(fd.dev + r * kp, dst, km, lane);
        }
        return;
    }
    const FlatPos pos{inv_km, km, kp};
    const uint32_t n = (uint32_t)(nrows * km);
    const uint32_t a = (uint32_t)((reinterpret_cast<uintptr_t>(fd.base) >> 3) & 1u);
    const uint32_t nwords = (n - a) >> 1;
    double2* d2 = reinterpret_cast<double2*>(fd.base + a);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t w0 = blockIdx.x * blockDim.x + threadIdx.x; w0 < nwords; w0 += stride * XF_UNROLL) {
        double2 v[XF_UNROLL];
#pragma unroll
        for (int q = 0; q < XF_UNROLL; q++) {
            const uint32_t w = w0 + q * stride;
            if (w >= nwords) continue;
            const uint32_t e = a + 2 * w;
            v[q] = make_double2(fd.dev[pos.dev(e)], fd.dev[pos.dev(e + 1)]);
        }
#pragma unroll
        for (int q = 0; q < XF_UNROLL; q++) {
            const uint32_t w = w0 + q * stride;
            if (w < nwords) d2[w] = v[q];
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (a) fd.base[0] = fd.dev[pos.dev(0)];
        if ((n - a) & 1u) fd.base[n - 1] = fd.dev[pos.dev(n - 1)];
    }
}

}  // namespace

// Ragged rows: about four rows per warp. Contiguous arrays below 2^24 elements: about four 16-byte words
// per thread and pass. Enough blocks to keep the link's latency covered, few enough to stay cheap.
cudaError_t launch_host_transfer(const HostBatch& b, int to_device, int64_t nrows, int km, int kp, cudaStream_t s) {
    if (b.n <= 0) return cudaSuccess;
    if (b.n > HOST_BATCH_MAX || km <= 0 || kp < km || (kp & 1) || nrows <= 0) return cudaErrorInvalidValue;
    const int64_t n = nrows * km;
    const int flat = n < (1 << 24) ? 1 : 0;
    const int64_t per_block = flat ? (int64_t)XF_WARPS * 32 * XF_UNROLL * 2 : (int64_t)XF_WARPS * 4;
    const int64_t gx = std::min<int64_t>(((flat ? n : nrows) + per_block - 1) / per_block, 65535);
    const dim3 grid((unsigned)gx, (unsigned)b.n);
    const float inv_km = 1.0f / (float)km;
    if (to_device) host_gather_kernel<<<grid, XF_WARPS * 32, 0, s>>>(b, nrows, km, kp, flat, inv_km);
    else host_scatter_kernel<<<grid, XF_WARPS * 32, 0, s>>>(b, nrows, km, kp, flat, inv_km);
    return cudaGetLastError();
}

}  // namespace atsat
