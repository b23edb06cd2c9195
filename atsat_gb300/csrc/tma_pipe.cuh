// The shared-memory pipeline of the TMA-tiled stage kernels: mbarrier operations, the 4-D tensor copy,
// and the consumer side of a ring of NSLOT slots (inline PTX for sm_100-class GPUs).
//
// Item n of a block's stream lands in slot n % NSLOT. Its "full" barrier (count 1) completes when the
// producer's arrive.expect_tx and the copy's transaction bytes are in; its "empty" barrier (one arrival per
// consumer warp) completes when every consumer warp is done with the slot. Every wait is bounded: after
// WAIT_LIMIT SM clocks it gives up and the caller sets a bit of the device status word.
#pragma once

#include <cstdint>

#include <cuda.h>

#include "dyn_common.cuh"

namespace atsat {
namespace tma {

constexpr long long WAIT_LIMIT = TILE_WAIT_LIMIT;   // SM clocks, about a second

enum : unsigned int { ERR_PRODUCER = 1u, ERR_CONSUMER = 2u, ERR_PLAN = 4u, ERR_ALIGN = 8u };

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// wait for the phase of parity `parity` to complete; false after `limit` clocks
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long limit = WAIT_LIMIT) {
    if (mbar_try(bar, parity)) return true;
    const long long t0 = clock64();
    do {
        if (mbar_try(bar, parity)) return true;
    } while (clock64() - t0 < limit);
    return false;
}
__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int x, int y, int z, int w,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(w), "r"(bar)
        : "memory");
}

// a contiguous copy global -> shared (both addresses 16-byte aligned, bytes a multiple of 16)
__device__ __forceinline__ void bulk_load(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(bar)
        : "memory");
}

struct Ring {
    uint32_t full0, empty0;     // shared addresses of full[0], empty[0]
    __device__ __forceinline__ uint32_t full(int s) const { return full0 + 8u * (uint32_t)s; }
    __device__ __forceinline__ uint32_t empty(int s) const { return empty0 + 8u * (uint32_t)s; }
};

// consumer side: wait for items [n0, n1); false (warp-uniform) when a wait gave up. Thread 0 also checks
// that the producer streams the arrays the consumer expects (`expect`), against the host-built plan.
template <int NSLOT>
__device__ __forceinline__ bool acquire(const Ring& rg, int n0, int n1, const TilePlan& plan, const int* expect) {
    bool ok = true;
#pragma unroll
    for (int n = n0; n < n1; n++) ok = ok && mbar_wait(rg.full(n % NSLOT), (uint32_t)((n / NSLOT) & 1), plan.wait_limit);
    if (threadIdx.x == 0) {
        bool same = true;
#pragma unroll
        for (int n = n0; n < n1; n++) same = same && plan.item[n] == expect[n - n0];
        if (!same) atomicOr(plan.err, ERR_PLAN);
    }
    return !__any_sync(0xffffffffu, !ok);
}

// Handing a slot back: the producer refills it by a tensor copy (async proxy) as soon as the empty barrier
// completes, so every lane's shared-memory loads from it must have been performed before the arrive. Where
// the loaded values have gone into global stores before the release, they have. Where they feed registers
// only (stencil differences, wind factors), the compiler is free to schedule that arithmetic after the
// arrive, and the copy could then overtake the loads and hand them the next item's data: such a release is
// preceded by slot_reads_done, a proxy fence that orders each lane's generic-proxy reads before the
// async-proxy writes that follow the barrier.
__device__ __forceinline__ void slot_reads_done() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

template <int NSLOT>
__device__ __forceinline__ void release(const Ring& rg, int n0, int n1) {
    __syncwarp();
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int n = n0; n < n1; n++) mbar_arrive(rg.empty(n % NSLOT));
    }
}

// Producer: stream the plan's items into the ring (main halo box plus, when `seam`, the seam box at xs),
// then wait (bounded, always with the full WAIT_LIMIT: a copy in flight lands by itself) for the last copy
// of every slot so that none lands after the block is gone.
template <int NSLOT>
__device__ __forceinline__ void produce(const Ring& rg, float* smem, int slot_f, uint32_t box_bytes,
                                        uint32_t seam_bytes, const CUtensorMap* map_main, const CUtensorMap* map_seam,
                                        int x, int y, int z, int seam, int xs, int ys, int zs, const TilePlan& plan) {
    const uint32_t bytes = box_bytes + (seam ? seam_bytes : 0u);
    int n = 0;
    bool ok = true;
    for (; n < plan.n_items; n++) {
        const int s = n % NSLOT;
        if (n >= NSLOT && !mbar_wait(rg.empty(s), (uint32_t)(((n / NSLOT) - 1) & 1), plan.wait_limit)) {
            ok = false;
            break;
        }
        const uint32_t dst = smem_u32(smem + s * slot_f);
        mbar_expect_tx(rg.full(s), bytes);
        tma_load_4d(dst, map_main, x, y, z, plan.item[n], rg.full(s));
        if (seam) tma_load_4d(dst + box_bytes, map_seam, xs, ys, zs, plan.item[n], rg.full(s));
    }
    if (!ok) atomicOr(plan.err, ERR_PRODUCER);
    for (int m = (n > NSLOT ? n - NSLOT : 0); m < n; m++)
        if (!mbar_wait(rg.full(m % NSLOT), (uint32_t)((m / NSLOT) & 1))) break;
}

}  // namespace tma
}  // namespace atsat
