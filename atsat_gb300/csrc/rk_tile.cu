// TMA-tiled mixed-precision RK stage (RungeKuttaSat's stage loop over RHSSat,
// planet/RungeKutta_Sat_Turb.cpp:110-387, planet/RHS_Sat_Turb.cpp:25-1016), the GB300 form of the
// direct kernel in rk_mixed.cu: same per-cell physics (mixed_physics.cuh), different data movement.
//
// A block owns TILE_K x TILE_J x TILE_I cells (k, j, i) of the integrated interior. One producer warp
// streams, with cp.async.bulk.tensor, a halo box of every stencil array (y_n copies, w's low word, the
// stage increments) into a ring of NSLOT shared-memory slots; eight consumer warps -- one per row j,
// a lane per meridian k, two radial levels per lane -- read the 7-point stencils from shared memory
// with constant offsets. mbarriers pair each slot's "full" (transaction bytes of the copy) and "empty"
// (one arrival per consumer warp) phases. The point inputs (frozen terms, sources, dl_1/dl_2 and y_n
// at the final stage) are plain loads. Every mbarrier wait is bounded (about a second); a wait that
// gives up sets a bit of the device status word, the producer waits (again bounded) for its own copies
// in flight, and the block returns.
#include <cuda.h>

#include "mixed_physics.cuh"
#include "tma_pipe.cuh"

namespace atsat {

namespace {

using namespace mixed;
using namespace tma;

constexpr int PL = TILE_BX * TILE_BY;                     // floats per plane of a box (400)
constexpr int BOX_F = PL * TILE_BZ;                       // 1600
constexpr int SEAM_F = TILE_SEAM_X * TILE_J * TILE_I;     // 64
constexpr int SLOT_F = BOX_F + SEAM_F;                    // 1664 floats = 6656 bytes (52 x 128)
constexpr uint32_t BOX_BYTES = BOX_F * 4;
constexpr uint32_t SEAM_BYTES = SEAM_F * 4;
constexpr int NSLOT = 12;                                 // >= the 9 arrays held at once for momentum
constexpr int NCW = TILE_J;                               // consumer warps
constexpr int THREADS = (NCW + 1) * 32;
constexpr int GEO_F = TILE_I * TILE_J * 16;               // ColGeoF of the block's columns
constexpr size_t SMEM_BYTES = (size_t)NSLOT * SLOT_F * 4 + (size_t)GEO_F * 4 + 2 * NSLOT * 8;

static_assert((SLOT_F * 4) % 128 == 0, "slots stay 128-byte aligned");
static_assert((BOX_F * 4) % 128 == 0, "the seam box starts 128-byte aligned");

// position of the items of field q in the stream (compile-time once q is): per field y_n, then w's low
// word, then the increment
template <bool HAS_DL>
__host__ __device__ constexpr int item_yn(int q) { return (HAS_DL ? 2 * q : q) + (q > ATSAT_F_W ? 1 : 0); }
template <bool HAS_DL>
__host__ __device__ constexpr int item_lo() { return item_yn<HAS_DL>(ATSAT_F_W) + 1; }
template <bool HAS_DL>
__host__ __device__ constexpr int item_dl(int q) { return item_yn<HAS_DL>(q) + (q == ATSAT_F_W ? 2 : 1); }

// stencils out of the slot ring: slot of item n = n % NSLOT
template <bool HAS_DL>
struct TileSrc {
    const float* sm;       // slot 0
    int o, ow, oe;         // centre, west and east neighbour, in floats from a slot's start

    __device__ __forceinline__ const float* slot(int n) const { return sm + (n % NSLOT) * SLOT_F; }
    __device__ __forceinline__ float cyn(int q) const { return slot(item_yn<HAS_DL>(q))[o]; }
    __device__ __forceinline__ float cdl(int q) const { return HAS_DL ? slot(item_dl<HAS_DL>(q))[o] : 0.0f; }
    __device__ __forceinline__ float clo() const { return slot(item_lo<HAS_DL>())[o]; }
    __device__ __forceinline__ void d7(const float* s, float* e) const {
        const float x = s[o];
        const float rp = s[o + PL], rn = s[o - PL];
        const float tp = s[o + TILE_BX], tn = s[o - TILE_BX];
        const float pe = s[oe], pw = s[ow];
        e[0] = rp - rn;
        e[1] = rp - 2.0f * x + rn;
        e[2] = tp - tn;
        e[3] = tp - 2.0f * x + tn;
        e[4] = pe - pw;
        e[5] = pe - 2.0f * x + pw;
    }
    __device__ __forceinline__ void raw6(int q, float* a) const {
        d7(slot(item_yn<HAS_DL>(q)), a);
        if (q == ATSAT_F_W) {
            float b[6];
            d7(slot(item_lo<HAS_DL>()), b);
#pragma unroll
            for (int r = 0; r < 6; r++) a[r] += b[r];
        }
        if (HAS_DL) {
            float b[6];
            d7(slot(item_dl<HAS_DL>(q)), b);
#pragma unroll
            for (int r = 0; r < 6; r++) a[r] += b[r];
        }
    }
};

template <int MODE, bool HAS_DL>
__global__ void __launch_bounds__(THREADS, 2)
rk_tile_kernel(const __grid_constant__ CUtensorMap map_main, const __grid_constant__ CUtensorMap map_seam,
               const MixedConstF K, const MixedIO io, const StageParams sp, const TilePlan plan) {
    extern __shared__ __align__(128) float smem[];
    float* sgeo = smem + NSLOT * SLOT_F;
    uint64_t* bars = reinterpret_cast<uint64_t*>(sgeo + GEO_F);
    const Ring rg{smem_u32(bars), smem_u32(bars + NSLOT)};
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    const int k0 = blockIdx.x * TILE_K;
    const int j0 = 2 + blockIdx.y * TILE_J;
    const int i0 = 1 + blockIdx.z * TILE_I;
    // the periodic partner of k = 0 (km-2) or of k = km-2 (0) when it lies outside the main box
    int seam = 0, xs = 0;
    if (k0 == 0 && K.km - 2 > k0 + TILE_K + 3) { seam = 1; xs = (K.km - 2) & ~3; }
    else if (k0 > 0 && K.km - 2 >= k0 && K.km - 2 < k0 + TILE_K) { seam = 2; xs = 0; }

    if (smem_u32(smem) & 127u) {              // the tensor copies need 128-byte aligned slots
        if (threadIdx.x == 0) atomicOr(plan.err, ERR_ALIGN);
        return;
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < NSLOT; s++) {
            mbar_init(rg.full(s), 1);
            mbar_init(rg.empty(s), NCW);
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == NCW) {
        // ---- producer ----
        if (lane == 0)
            produce<NSLOT>(rg, smem, SLOT_F, BOX_BYTES, SEAM_BYTES, &map_main, &map_seam, k0 - 4, j0 - 1, i0 - 1, seam,
                           xs, j0, i0, plan);
        return;
    }

    // ---- consumers: warp w owns row j = j0 + w, lane the meridian k = k0 + lane, levels i0, i0 + 1 ----
    const int j = j0 + warp, k = k0 + lane;
    {
        // the row's two columns of FP32 geometry into shared memory (one float per lane)
        const int ii = lane >> 4, f = lane & 15;
        const int i = i0 + ii;
        float v = 0.0f;
        if (i < K.im && j < K.jm) v = __ldg(reinterpret_cast<const float*>(io.geof + ((int64_t)i * K.jm + j)) + f);
        sgeo[(ii * TILE_J + warp) * 16 + f] = v;
        __syncwarp();
    }
    bool valid[TILE_I];
    int64_t c[TILE_I];
    TileSrc<HAS_DL> S[TILE_I];
#pragma unroll
    for (int ii = 0; ii < TILE_I; ii++) {
        const int i = i0 + ii;
        valid[ii] = (k <= K.km - 2) && (j <= K.jm - 3) && (i <= K.im - 2);
        c[ii] = ((int64_t)i * K.jm + j) * K.kp + k;
        const int row = (1 + ii) * PL + (warp + 1) * TILE_BX;
        S[ii].sm = smem;
        S[ii].o = row + lane + 4;
        S[ii].ow = S[ii].o - 1;
        S[ii].oe = S[ii].o + 1;
        if (k == 0)
            S[ii].ow = (seam == 1) ? BOX_F + (ii * TILE_J + warp) * TILE_SEAM_X + ((K.km - 2) - xs)
                                   : row + (K.km - 2) - (k0 - 4);
        if (k == K.km - 2)
            S[ii].oe = (seam == 2) ? BOX_F + (ii * TILE_J + warp) * TILE_SEAM_X + (0 - xs) : row + 0 - (k0 - 4);
    }

    // momentum and temperature: u, v, w, t held together
    constexpr int N_MOM = item_yn<HAS_DL>(ATSAT_F_T) + (HAS_DL ? 2 : 1);
    {
        int expect[N_MOM];
#pragma unroll
        for (int q = 0; q <= ATSAT_F_T; q++) {
            expect[item_yn<HAS_DL>(q)] = plan.arr_yn[q];
            if (q == ATSAT_F_W) expect[item_lo<HAS_DL>()] = plan.arr_lo;
            if (HAS_DL) expect[item_dl<HAS_DL>(q)] = plan.arr_dl[q];
        }
        if (!acquire<NSLOT>(rg, 0, N_MOM, plan, expect)) {
            if (lane == 0) atomicOr(plan.err, ERR_CONSUMER);
            return;
        }
    }
    CellState cs[TILE_I];
#pragma unroll
    for (int ii = 0; ii < TILE_I; ii++) {
        if (valid[ii]) {
            const ColGeoF& g = *reinterpret_cast<const ColGeoF*>(sgeo + (ii * TILE_J + warp) * 16);
            cs[ii] = momentum_t<MODE>(K, io, sp, S[ii], i0 + ii, c[ii], g);
        }
    }
    release<NSLOT>(rg, 0, N_MOM);

    // the tracers, one field (one or two arrays) at a time
    const int q_last = K.turb ? ATSAT_F_DIS : ATSAT_F_NH4SH;
#pragma unroll
    for (int q = ATSAT_F_H2O; q <= ATSAT_F_DIS; q++) {
        if (q > q_last) break;
        const int n0 = item_yn<HAS_DL>(q), n1 = n0 + (HAS_DL ? 2 : 1);
        int expect[2] = {plan.arr_yn[q], plan.arr_dl[q]};
        if (!acquire<NSLOT>(rg, n0, n1, plan, expect)) {
            if (lane == 0) atomicOr(plan.err, ERR_CONSUMER);
            return;
        }
#pragma unroll
        for (int ii = 0; ii < TILE_I; ii++) {
            if (valid[ii]) {
                const ColGeoF& g = *reinterpret_cast<const ColGeoF*>(sgeo + (ii * TILE_J + warp) * 16);
                scalar<MODE>(q, K, io, sp, S[ii], c[ii], g, cs[ii]);
            }
        }
        release<NSLOT>(rg, n0, n1);
    }
    if (!K.turb && MODE == MODE_FINAL && sp.write_all_rhs) {
#pragma unroll
        for (int ii = 0; ii < TILE_I; ii++)
            if (valid[ii]) {
                io.rhs[ATSAT_F_TKE][c[ii]] = 0.0;
                io.rhs[ATSAT_F_DIS][c[ii]] = 0.0;
            }
    }
}

template <int MODE, bool HAS_DL>
cudaError_t launch_one(const TileMaps& maps, const MixedConstF& kf, const MixedIO& io, const StageParams& sp,
                       const TilePlan& plan, dim3 grid, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = cudaFuncSetAttribute(rk_tile_kernel<MODE, HAS_DL>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_BYTES);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    rk_tile_kernel<MODE, HAS_DL><<<grid, THREADS, SMEM_BYTES, s>>>(
        *reinterpret_cast<const CUtensorMap*>(maps.main), *reinterpret_cast<const CUtensorMap*>(maps.seam), kf, io,
        sp, plan);
    return cudaGetLastError();
}

}  // namespace

size_t rk_tile_smem_bytes() { return SMEM_BYTES; }

cudaError_t launch_rk_tile(const TileMaps& maps, const MixedConstF& kf, const MixedIO& io, const StageParams& sp,
                           const TilePlan& plan, int mode, cudaStream_t s) {
    const int nk = (kf.km - 1 + TILE_K - 1) / TILE_K;
    const int nj = (kf.jm - 4 + TILE_J - 1) / TILE_J;
    const int ni = (kf.im - 2 + TILE_I - 1) / TILE_I;
    if (nk <= 0 || nj <= 0 || ni <= 0) return cudaSuccess;   // no interior cells
    if (mode == MODE_RHS || plan.n_items > TILE_MAX_ITEMS) return cudaErrorInvalidValue;
    const dim3 grid(nk, nj, ni);
    const bool has_dl = io.dl_in[0] != nullptr;
    if (mode == MODE_STAGE)
        return has_dl ? launch_one<MODE_STAGE, true>(maps, kf, io, sp, plan, grid, s)
                      : launch_one<MODE_STAGE, false>(maps, kf, io, sp, plan, grid, s);
    return has_dl ? launch_one<MODE_FINAL, true>(maps, kf, io, sp, plan, grid, s)
                  : launch_one<MODE_FINAL, false>(maps, kf, io, sp, plan, grid, s);
}

}  // namespace atsat
