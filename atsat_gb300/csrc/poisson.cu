// Standalone solves of the pressure equation the reference relaxes (PressureSolver.h:318-495, 718-746):
//
//   num1 (p[i+1] + p[i-1]) + num2 (p[j+1] + p[j-1]) + num3 (p[k+1] + p[k-1]) - den p = f
//
// on the interior P cells (i = 1..im-2, j = 1..jm-2, k = 0..km-2), with the reference's boundary planes
// p[0] = c43 p[1] - c13 p[2] in r and theta (folded into the rows next to them) and the periodic seam in
// phi. num1..3 and den are the sweep weights of the column geometry (PressureSolver.h:349-353).
//
// The reference only smooths (one red-black Gauss-Seidel sweep per call). This file solves:
//   * SOR: the reference's red-black update with over-relaxation, FP64 or FP32;
//   * DIRECT: the coefficients do not depend on phi, so a real DFT over the km-1 meridians decouples
//     the modes; each mode is a block-tridiagonal system in theta with tridiagonal radial blocks, solved by
//     block Thomas with the inverse pivot blocks W_j = S_j^-1 factored once on the host (FP64, stored in
//     FP64 and FP32). The zero mode is singular (constants): one cell is pinned and the result is shifted to
//     zero interior mean; sources are made compatible by `project` (the component along the zero mode's
//     left null vector is removed);
//   * REFINE: FP64 defect correction with FP32 inner solves (direct or SOR sweeps): r = f - L p in FP64,
//     e = L^-1 r in FP32, p += e, until ||r|| / ||f|| <= tol.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <omp.h>

#include "dyn_common.cuh"

namespace atsat {

namespace {

// ---- stencil helpers over the pitched layout ----
template <typename T>
__device__ __forceinline__ T pv_i(const KConst& K, const T* p, int i, int j, int k) {
    const int64_t row = (int64_t)j * K.kp + k;
    const T c43 = (T)K.c43, c13 = (T)K.c13;
    if (i == 0) return c43 * p[K.plane + row] - c13 * p[2 * K.plane + row];
    if (i == K.im - 1) return c43 * p[(K.im - 2) * K.plane + row] - c13 * p[(K.im - 3) * K.plane + row];
    return p[(int64_t)i * K.plane + row];
}

template <typename T>
__device__ __forceinline__ T pv(const KConst& K, const T* p, int i, int j, int k) {
    const T c43 = (T)K.c43, c13 = (T)K.c13;
    if (j == 0) return c43 * pv_i(K, p, i, 1, k) - c13 * pv_i(K, p, i, 2, k);
    if (j == K.jm - 1) return c43 * pv_i(K, p, i, K.jm - 2, k) - c13 * pv_i(K, p, i, K.jm - 3, k);
    return pv_i(K, p, i, j, k);
}

// boundary planes and seam from the interior (the reference's order: radial, polar, seam)
template <typename T>
__global__ void fold_kernel(const KConst K, T* __restrict__ p) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int im = K.im, jm = K.jm, km = K.km;
    const int64_t nA = (int64_t)im * jm, nB = 2LL * jm * (km - 1), nC = 2LL * (im - 2) * (km - 1);
    int i, j, k;
    if (e < nA) {
        i = (int)(e / jm); j = (int)(e % jm); k = km - 1;
    } else if (e < nA + nB) {
        const int64_t q = e - nA;
        k = (int)(q % (km - 1));
        const int64_t r = q / (km - 1);
        j = (int)(r % jm);
        i = (r / jm) ? im - 1 : 0;
    } else if (e < nA + nB + nC) {
        const int64_t q = e - nA - nB;
        k = (int)(q % (km - 1));
        const int64_t r = q / (km - 1);
        i = 1 + (int)(r % (im - 2));
        j = (r / (im - 2)) ? jm - 1 : 0;
    } else {
        return;
    }
    p[((int64_t)i * jm + j) * K.kp + k] = pv(K, p, i, j, (k == km - 1) ? 0 : k);
}

// one colour of red-black SOR: p <- (1 - w) p + w (acc - f) / den; the seam partner k = km-2 of an odd
// ring is done by sor_seam_kernel after k = 0 (the reference's row order)
template <typename T>
__device__ __forceinline__ void sor_cell(const KConst& K, const ColGeo* __restrict__ geo, const T* __restrict__ f,
                                         T* __restrict__ p, int i, int j, int k, T w) {
    const int64_t c = ((int64_t)i * K.jm + j) * K.kp + k;
    const int kw = (k == 0) ? K.km - 2 : k - 1, ke = (k == K.km - 2) ? 0 : k + 1;
    const ColGeo* g = geo + ((int64_t)i * K.jm + j);
    const T acc = (p[c + K.plane] + p[c - K.plane]) * (T)__ldg(&g->p_num1) + (p[c + K.kp] + p[c - K.kp]) * (T)__ldg(&g->p_num2)
                + (p[c - k + ke] + p[c - k + kw]) * (T)__ldg(&g->p_num3);
    const T nv = (acc - f[c]) / (T)__ldg(&g->p_den);
    p[c] = p[c] + w * (nv - p[c]);
}

template <typename T>
__global__ void __launch_bounds__(256) sor_kernel(const KConst K, const ColGeo* __restrict__ geo,
                                                  const T* __restrict__ f, T* __restrict__ p, int colour, T w) {
    const int m = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    if (j < 1 || j > K.jm - 2 || i < 1 || i > K.im - 2) return;
    const int k = 2 * m + ((colour - i - j) & 1);
    if (k > K.km - 2) return;
    if (k == K.km - 2 && k > 0 && ((K.km - 1) & 1)) return;
    sor_cell(K, geo, f, p, i, j, k, w);
}

template <typename T>
__global__ void sor_seam_kernel(const KConst K, const ColGeo* __restrict__ geo, const T* __restrict__ f,
                                T* __restrict__ p, int colour, T w) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = 1 + e / (K.jm - 2), j = 1 + e % (K.jm - 2);
    if (i > K.im - 2) return;
    const int k = K.km - 2;
    if (((i + j + k) & 1) != colour) return;
    sor_cell(K, geo, f, p, i, j, k, w);
}

// ---- checkerboard-packed red-black SOR, many sweeps per launch ----
// With an even ring (km-1 = n even) the colour (i + j + k) & 1 is consistent across the periodic seam, and
// every colour-c cell of row (i, j) is k = 2m + ((i + j + c) & 1), m = k >> 1: colour c is stored packed as
// Pk[c][(i * jm + j) * kh + m] (kh = n / 2 rounded up to 32). A colour-c cell's four theta / radial
// neighbours sit at the same m of the other colour's array, its phi neighbours at m and m +- 1; a
// half-sweep reads the other colour's packed array and its own packed source, and writes its own colour:
// every access is a coalesced run, none drags the other colour's half of a cache line along.
//
// One cooperative launch runs `nsweeps` sweeps; the blocks meet at a grid barrier after each half-sweep.
// The reference folds the boundary planes after each sweep (p[0] = c43 p[1] - c13 p[2] in r and theta); here
// the thread that updates the cell at distance two from a boundary writes that boundary cell's folded value
// itself, at the moment the reference's stored value would hold it: in the first half-sweep from its old
// value (the other colour reads it in the second half-sweep, as the previous sweep's fold), in the second
// from its new value (read in the next sweep's first half-sweep, as this sweep's fold). The neighbour at
// distance one is of the other colour and does not change in that half-sweep. So a sweep is two phases
// and two barriers, and every value equals the unpacked red, black, fold sequence.
struct GridBar {
    unsigned int count, gen, err, pad;
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned* p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

// all blocks of the cooperative launch meet here; false (block-uniform) when the wait gave up after
// `limit` clocks (the error word is then set)
__device__ __forceinline__ bool grid_barrier(GridBar* b, unsigned nblocks, long long limit) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        int ok = 1;
        __threadfence();                  // the block's writes of this phase, before its arrival
        const unsigned g = ld_acquire(&b->gen);
        if (atom_add_acq_rel(&b->count, 1u) == nblocks - 1) {
            b->count = 0;
            st_release(&b->gen, g + 1u);
        } else {
            const long long t0 = clock64();
            while (ld_acquire(&b->gen) == g) {
                __nanosleep(32);           // fewer polls of the one line the arrivals update
                if (clock64() - t0 > limit) {
                    ok = 0;
                    atomicOr(&b->err, 1u);
                    break;
                }
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

template <typename T>
struct alignas(4 * sizeof(T)) SorW {
    T num1, num2, num3, rden;     // the sweep weights and 1 / den (formed in FP64 on the host)
};

constexpr int SORP_WARPS = 32;   // large blocks: few arrivals at each grid barrier

// A warp's position in the item list (level i, row j, chunk mc of 32 packed columns) and the step of the
// grid's stride in the same terms, so that the walk needs no division: integer division and int <-> float
// conversion run at the FP64 rate on this GPU.
struct ItemWalk {
    int i, j, mc;          // the first item of this warp
    int di, dj, dmc;       // the stride nw as levels, rows and chunks (dj < NJ, dmc < nch)
};

__device__ __forceinline__ ItemWalk item_walk(const KConst& K, int gw, int nw) {
    const int n = K.km - 1, nch = ((n >> 1) + 31) >> 5, NJ = K.jm - 2;
    ItemWalk W;
    int r = gw / nch;
    W.mc = gw - r * nch;
    W.i = 1 + r / NJ;
    W.j = 1 + (r - (W.i - 1) * NJ);
    r = nw / nch;
    W.dmc = nw - r * nch;
    W.di = r / NJ;
    W.dj = r - W.di * NJ;
    return W;
}

// One half-sweep of colour c over the warps of the grid. A work item is 32 consecutive cells of one packed
// row; the arrays are distinct (restrict), so the loads of the next items can be issued ahead of this
// item's stores.
template <typename T>
__device__ __forceinline__ void sor_phase(const KConst& K, const SorW<T>* __restrict__ wt, T* __restrict__ Pc,
                                          const T* __restrict__ Po, const T* __restrict__ Fc, int kh, int c, T w,
                                          ItemWalk it) {
    const int n = K.km - 1, nh = n >> 1, nch = (nh + 31) >> 5;
    const int64_t plane = (int64_t)K.jm * kh;
    const int lane = threadIdx.x;
    const T c43 = (T)K.c43, c13 = (T)K.c13;
    int i = it.i, j = it.j, mc = it.mc;
#pragma unroll 4
    for (; i <= K.im - 2;) {
        const int m = mc * 32 + lane;
        const int ci = i, cj = j;
        mc += it.dmc;
        if (mc >= nch) { mc -= nch; j++; }
        j += it.dj;
        if (j > K.jm - 2) { j -= K.jm - 2; i++; }
        i += it.di;
        if (m >= nh) continue;
        const int64_t row = ((int64_t)ci * K.jm + cj) * kh;
        const SorW<T> W = wt[(int64_t)ci * K.jm + cj];
        const int k = 2 * m + ((ci + cj + c) & 1);
        const int me = (k == n - 1) ? 0 : ((k + 1) >> 1);
        const int mw = (k == 0) ? ((n - 1) >> 1) : ((k - 1) >> 1);
        const T acc = (__ldcg(Po + row + plane + m) + __ldcg(Po + row - plane + m)) * W.num1
                    + (__ldcg(Po + row + kh + m) + __ldcg(Po + row - kh + m)) * W.num2
                    + (__ldcg(Po + row + me) + __ldcg(Po + row + mw)) * W.num3;
        const T old = __ldcg(Pc + row + m);
        const T nv = (acc - Fc[row + m]) * W.rden;
        const T pn = old + w * (nv - old);
        Pc[row + m] = pn;
        // the folded boundary cells this cell stands two away from (the same colour as it)
        const T self = (c == 0) ? old : pn;
        if (ci == 2) Pc[row - 2 * plane + m] = c43 * __ldcg(Po + row - plane + m) - c13 * self;
        if (ci == K.im - 3) Pc[row + 2 * plane + m] = c43 * __ldcg(Po + row + plane + m) - c13 * self;
        if (cj == 2) Pc[row - 2 * kh + m] = c43 * __ldcg(Po + row - kh + m) - c13 * self;
        if (cj == K.jm - 3) Pc[row + 2 * kh + m] = c43 * __ldcg(Po + row + kh + m) - c13 * self;
    }
}

template <typename T>
__global__ void __launch_bounds__(32 * SORP_WARPS) sor_packed_kernel(const KConst K, const SorW<T>* __restrict__ wt,
                                                                     T* p0, T* p1, const T* __restrict__ f0,
                                                                     const T* __restrict__ f1, int kh, int nsweeps,
                                                                     T w, GridBar* bar, long long limit) {
    const ItemWalk it = item_walk(K, blockIdx.x * SORP_WARPS + threadIdx.y, gridDim.x * SORP_WARPS);
    for (int sweep = 0; sweep < nsweeps; sweep++) {
        sor_phase<T>(K, wt, p0, p1, f0, kh, 0, w, it);
        if (!grid_barrier(bar, gridDim.x, limit)) return;
        sor_phase<T>(K, wt, p1, p0, f1, kh, 1, w, it);
        if (!grid_barrier(bar, gridDim.x, limit)) return;
    }
}

// ---- the same sweeps temporally blocked (FP32): S sweeps per grid barrier ----
// A block owns a tile of rows j0 .. j1-1 and packed columns m0 .. m1-1 over every radial level (the folded
// planes i = 0 and im-1 included) and holds it in shared memory, both colours, with a halo of 2S rows and
// S packed columns (2S cells along phi) on each side: TB_LANES packed columns per shared row, a pair of them
// per lane of a half-warp (tiles start on even columns and the half-ring is even, so a pair never straddles
// the periodic wrap).
// A pass loads the halo'd tile from the current packed arrays, runs 2S half-sweeps in shared memory --
// half-sweep h updates the cells within 2S - h cells of the owned tile, the cone the owned cells depend
// on -- and writes the owned cells (with the folded rows j = 0 / jm-1 where it owns the rows next to them)
// to the other pair of packed arrays; the blocks meet at the grid barrier between passes. Every cell gets
// the operations of sor_phase in the same order (the folds included), so the two kernels agree bit for
// bit; halo cells are computed by each tile whose cone holds them.
constexpr int TB_WARPS = 32;
constexpr int TB_LANES = 32;
constexpr int TB_MAX_TILES = 1024;

struct TbPlan {
    int ntiles, RJ, nh;          // tiles, shared rows per tile, n / 2
};

// one tile: packed columns m0 .. m0+TM-1, rows j0 .. j1-1 (formed on the host: no division on the device,
// where integer division and int <-> float conversion run at the FP64 rate)
struct TbTile {
    int m0, TM, j0, j1;
};

// shared memory of one tile: both colours of p over im x RJ rows of TB_LANES, then the rows' weights
__host__ __device__ inline size_t tb_smem_bytes(int im, int RJ) {
    return (size_t)2 * im * RJ * TB_LANES * sizeof(float) + (size_t)im * RJ * sizeof(SorW<float>);
}

// (a, b) += step in a row-major walk with b in [0, nb): b wraps into a (b, step >= 0)
__device__ __forceinline__ void walk(int& a, int& b, int step, int nb) {
    b += step;
    while (b >= nb) { b -= nb; a++; }
}

// asynchronous copy of a pair of floats global -> shared (no register round trip; many in flight per thread)
__device__ __forceinline__ void cp_async8(float* dst, const float* src) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

constexpr int TB_SEG = 2;        // radial levels per work item of a half-sweep

// One work item of a half-warp: the cells of one shared row jj at levels i0 .. i0+nl-1 of colour c, a pair of
// adjacent packed columns per lane (8-byte shared loads and stores). The pair's cells share the parity
// par (k = 2 m + par), so their phi neighbours in the other colour are the pair (q, q+1) and one of q-1,
// q+2: par 0: east, west = (q, q-1) and (q+1, q); par 1: (q+1, q) and (q+2, q+1). vx / vy: whether each
// cell of the pair is updated for parity 0 (a) and 1 (b); a cell that is not keeps its value.
// FOLDS: the item may hold a cell two away from a folded boundary (levels 2 or im-3, rows 2 or jm-3).
template <bool FOLDS>
__device__ __forceinline__ void tb_segment(float* __restrict__ own, const float* __restrict__ oth,
                                           const SorW<float>* wp, const float2 (&fv)[TB_SEG], int q, int par,
                                           bool a0, bool a1, bool b0, bool b1, int PL, int RJ, int nl, int i0,
                                           int im, bool jlow, bool jhigh, float w, float c43, float c13, int c) {
#pragma unroll
    for (int u = 0; u < TB_SEG; u++) {
        const bool vx = par ? b0 : a0, vy = par ? b1 : a1;
        if (u < nl && (vx || vy)) {
            const SorW<float> W = wp[u * RJ];
            const float2 up = *reinterpret_cast<const float2*>(oth + q + PL);
            const float2 dn = *reinterpret_cast<const float2*>(oth + q - PL);
            const float2 nn = *reinterpret_cast<const float2*>(oth + q + TB_LANES);
            const float2 ss = *reinterpret_cast<const float2*>(oth + q - TB_LANES);
            const float2 pq = *reinterpret_cast<const float2*>(oth + q);
            const float wl = oth[q - 1], er = oth[q + 2];
            const float ex = par ? pq.y : pq.x, wx = par ? pq.x : wl;
            const float ey = par ? er : pq.y, wy = par ? pq.y : pq.x;
            const float accx = (up.x + dn.x) * W.num1 + (nn.x + ss.x) * W.num2 + (ex + wx) * W.num3;
            const float accy = (up.y + dn.y) * W.num1 + (nn.y + ss.y) * W.num2 + (ey + wy) * W.num3;
            const float2 old = *reinterpret_cast<const float2*>(own + q);
            const float nvx = (accx - fv[u].x) * W.rden, nvy = (accy - fv[u].y) * W.rden;
            const float pnx = old.x + w * (nvx - old.x), pny = old.y + w * (nvy - old.y);
            *reinterpret_cast<float2*>(own + q) = make_float2(vx ? pnx : old.x, vy ? pny : old.y);
            if (FOLDS) {
                // the folded boundary cells the pair's cells stand two away from (same colour)
                const float sx = (c == 0) ? old.x : pnx, sy = (c == 0) ? old.y : pny;
                const int i = i0 + u;
                if (i == 2) {
                    if (vx) own[q - 2 * PL] = c43 * dn.x - c13 * sx;
                    if (vy) own[q + 1 - 2 * PL] = c43 * dn.y - c13 * sy;
                }
                if (i == im - 3) {
                    if (vx) own[q + 2 * PL] = c43 * up.x - c13 * sx;
                    if (vy) own[q + 1 + 2 * PL] = c43 * up.y - c13 * sy;
                }
                if (jlow) {
                    if (vx) own[q - 2 * TB_LANES] = c43 * ss.x - c13 * sx;
                    if (vy) own[q + 1 - 2 * TB_LANES] = c43 * ss.y - c13 * sy;
                }
                if (jhigh) {
                    if (vx) own[q + 2 * TB_LANES] = c43 * nn.x - c13 * sx;
                    if (vy) own[q + 1 + 2 * TB_LANES] = c43 * nn.y - c13 * sy;
                }
            }
        }
        q += PL;
        par ^= 1;
    }
}

template <int S>
__global__ void __launch_bounds__(32 * TB_WARPS) sor_tb_kernel(const KConst K, const SorW<float>* __restrict__ wt,
                                                               const TbTile* __restrict__ tiles,
                                                               float* A0, float* A1, float* B0, float* B1,
                                                               const float* __restrict__ f0,
                                                               const float* __restrict__ f1, int kh, int nsweeps,
                                                               float w, TbPlan pl, GridBar* bar, long long limit) {
    extern __shared__ float4 tb_smem[];
    float* const sp = reinterpret_cast<float*>(tb_smem);
    const int RJ = pl.RJ, im = K.im, jm = K.jm, nh = pl.nh, NI = im - 2;
    const int lane = threadIdx.x, warp = threadIdx.y;
    const int cs = im * RJ * TB_LANES;          // floats per colour
    const int PL = RJ * TB_LANES;               // floats per radial level
    const int64_t GP = (int64_t)jm * kh;        // global floats per radial level (packed)
    const int nseg = (NI + TB_SEG - 1) / TB_SEG;
    SorW<float>* const sw = reinterpret_cast<SorW<float>*>(sp + 2 * cs);
    const float c43 = (float)K.c43, c13 = (float)K.c13;
    for (int done = 0; done < nsweeps;) {
        const int ns = min(S, nsweeps - done);
        done += ns;
        for (int t = blockIdx.x; t < pl.ntiles; t += gridDim.x) {
            const TbTile T = tiles[t];
            const int m0 = T.m0, TM = T.TM, j0 = T.j0, j1 = T.j1;
            const int jb = j0 - 2 * S;          // the row of shared row 0
            {
                // two shared rows per warp instruction, a pair of packed columns per lane: tiles start on
                // even columns and the half-ring is even, so a pair never straddles the wrap and its
                // global address is 8-byte aligned
                const int half = lane >> 4, pc = 2 * (lane & 15);
                int gp = m0 - S + pc;
                gp = gp < 0 ? gp + nh : (gp >= nh ? gp - nh : gp);
                int i = 0, jj = 2 * warp + half;
                walk(i, jj, 0, RJ);
                for (; i < im; walk(i, jj, 2 * TB_WARPS, RJ)) {
                    const int j = jb + jj;
                    if (j < 0 || j >= jm) continue;
                    const int r = i * RJ + jj;
                    const int64_t g = ((int64_t)i * jm + j) * kh + gp;
                    if (pc < TM + 2 * S) {
                        cp_async8(sp + r * TB_LANES + pc, A0 + g);
                        cp_async8(sp + cs + r * TB_LANES + pc, A1 + g);
                    }
                    if (pc < 4) cp_async8(reinterpret_cast<float*>(sw + r) + pc,
                                          reinterpret_cast<const float*>(wt + (int64_t)i * jm + j) + pc);
                }
                cp_async_wait_all();
            }
            __syncthreads();
            for (int h = 1; h <= 2 * ns; h++) {
                const int c = (h - 1) & 1, e = 2 * ns - h;
                float* const own = sp + c * cs;
                const float* const oth = sp + (1 - c) * cs;
                const float* const fc = c ? f1 : f0;
                const int jlo = max(1, j0 - e), nj = min(jm - 2, j1 - 1 + e) - jlo + 1;
                const int klo = -e, khi = 2 * TM + e;          // phi range relative to 2 m0
                // this lane's pair of packed columns pc, pc+1 (phi 2 (pc - S) + par and 2 (pc + 1 - S) + par
                // relative to 2 m0) and whether each is updated for parity 0 (a0, a1) and 1 (b0, b1)
                const int half = lane >> 4, pc = 2 * (lane & 15), kl = 2 * (pc - S);
                const bool a0 = kl >= klo && kl < khi, a1 = kl + 2 >= klo && kl + 2 < khi;
                const bool b0 = kl + 1 >= klo && kl + 1 < khi, b1 = kl + 3 >= klo && kl + 3 < khi;
                int gp = m0 - S + pc;
                gp = gp < 0 ? gp + nh : (gp >= nh ? gp - nh : gp);
                // work items of the half-warps: (row jr, segment sg of TB_SEG levels), segment fastest
                int jr = 0, sg = 2 * warp + half;
                walk(jr, sg, 0, nseg);
                for (; jr < nj; walk(jr, sg, 2 * TB_WARPS, nseg)) {
                    const int j = jlo + jr, jj = j - jb;
                    const int i0 = 1 + sg * TB_SEG, nl = min(TB_SEG, NI + 1 - i0);
                    const float* fp = fc + ((int64_t)i0 * jm + j) * kh + gp;
                    float2 fv[TB_SEG];
#pragma unroll
                    for (int u = 0; u < TB_SEG; u++)
                        fv[u] = (u < nl) ? __ldg(reinterpret_cast<const float2*>(fp + u * GP)) : make_float2(0.0f, 0.0f);
                    const bool jlow = (j == 2 && jj >= 2), jhigh = (j == jm - 3 && jj + 2 < RJ);
                    const int q0 = i0 * PL + jj * TB_LANES + pc, par0 = (i0 + j + c) & 1;
                    const SorW<float>* wp = sw + i0 * RJ + jj;
                    if (nl == TB_SEG && i0 > 2 && i0 + TB_SEG <= im - 3 && !jlow && !jhigh)
                        tb_segment<false>(own, oth, wp, fv, q0, par0, a0, a1, b0, b1, PL, RJ, TB_SEG, i0, im, false,
                                          false, w, c43, c13, c);
                    else
                        tb_segment<true>(own, oth, wp, fv, q0, par0, a0, a1, b0, b1, PL, RJ, nl, i0, im, jlow, jhigh,
                                         w, c43, c13, c);
                }
                __syncthreads();
            }
            // the owned cells, with the folded rows next to the owned boundary rows: a pair of columns per
            // lane, two rows per warp instruction
            const int jsl = (j0 == 1) ? 0 : j0, nrow = ((j1 == jm - 1) ? jm - 1 : j1 - 1) - jsl + 1;
            {
                const int half = lane >> 4, pc = 2 * (lane & 15);
                if (pc >= S && pc < S + TM) {
                    int jr = 0, i = 2 * warp + half;
                    walk(jr, i, 0, im);
                    for (; jr < nrow; walk(jr, i, 2 * TB_WARPS, im)) {
                        const int j = jsl + jr;
                        const int q = i * PL + (j - jb) * TB_LANES + pc;
                        const int64_t g = ((int64_t)i * jm + j) * kh + (m0 + pc - S);
                        *reinterpret_cast<float2*>(B0 + g) = *reinterpret_cast<const float2*>(sp + q);
                        *reinterpret_cast<float2*>(B1 + g) = *reinterpret_cast<const float2*>(sp + cs + q);
                    }
                }
            }
            __syncthreads();
        }
        if (done < nsweeps) {
            if (!grid_barrier(bar, gridDim.x, limit)) return;
            float* t0 = A0; A0 = B0; B0 = t0;
            float* t1 = A1; A1 = B1; B1 = t1;
        }
    }
}

// pitched -> packed (every (i, j) row, the folded boundary rows and planes included); unpacked back for the
// interior cells only (the fold kernel then sets the boundary)
template <typename T>
__global__ void pack_kernel(const KConst K, const T* __restrict__ src, T* __restrict__ d0, T* __restrict__ d1, int kh) {
    const int m = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    const int n = K.km - 1;
    if (m >= (n >> 1) || j >= K.jm) return;
    const int64_t c = ((int64_t)i * K.jm + j) * K.kp;
    const int64_t o = ((int64_t)i * K.jm + j) * kh + m;
    d0[o] = src[c + 2 * m + ((i + j) & 1)];
    d1[o] = src[c + 2 * m + ((i + j + 1) & 1)];
}

template <typename T>
__global__ void unpack_kernel(const KConst K, T* __restrict__ dst, const T* __restrict__ s0, const T* __restrict__ s1,
                              int kh) {
    const int m = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    const int n = K.km - 1;
    if (m >= (n >> 1) || j < 1 || j > K.jm - 2 || i < 1 || i > K.im - 2) return;
    const int64_t c = ((int64_t)i * K.jm + j) * K.kp;
    const int64_t o = ((int64_t)i * K.jm + j) * kh + m;
    dst[c + 2 * m + ((i + j) & 1)] = s0[o];
    dst[c + 2 * m + ((i + j + 1) & 1)] = s1[o];
}

// r = f - L p on the interior P cells, in FP64 (p FP64), with an FP32 copy of r and the sums
// sum r^2 and sum f^2 (sq[0], sq[1])
__global__ void __launch_bounds__(256) residual_kernel(const KConst K, const ColGeo* __restrict__ geo,
                                                       const double* __restrict__ f, const double* __restrict__ p,
                                                       double* __restrict__ r, float* __restrict__ r32,
                                                       double* __restrict__ sq) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    double rr = 0.0, ff = 0.0;
    if (k <= K.km - 2 && j >= 1 && j <= K.jm - 2 && i >= 1 && i <= K.im - 2) {
        const int64_t c = ((int64_t)i * K.jm + j) * K.kp + k;
        const int kw = (k == 0) ? K.km - 2 : k - 1, ke = (k == K.km - 2) ? 0 : k + 1;
        const ColGeo* g = geo + ((int64_t)i * K.jm + j);
        const double lp = (p[c + K.plane] + p[c - K.plane]) * __ldg(&g->p_num1)
                        + (p[c + K.kp] + p[c - K.kp]) * __ldg(&g->p_num2)
                        + (p[c - k + ke] + p[c - k + kw]) * __ldg(&g->p_num3) - __ldg(&g->p_den) * p[c];
        const double fc = f[c];
        const double x = fc - lp;
        r[c] = x;
        if (r32) r32[c] = d2f(x);
        rr = x * x;
        ff = fc * fc;
    }
    for (int o = 16; o > 0; o >>= 1) {
        rr += __shfl_down_sync(0xffffffffu, rr, o);
        ff += __shfl_down_sync(0xffffffffu, ff, o);
    }
    __shared__ double s[2][8];
    if (threadIdx.x == 0) { s[0][threadIdx.y] = rr; s[1][threadIdx.y] = ff; }
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        double a = 0.0, b = 0.0;
        for (int q = 0; q < 8; q++) { a += s[0][q]; b += s[1][q]; }
        atomicAdd(sq, a);
        atomicAdd(sq + 1, b);
    }
}

// p64 += e32 on the interior P cells
__global__ void axpy_kernel(const KConst K, double* __restrict__ p, const float* __restrict__ e) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    if (k > K.km - 2 || j < 1 || j > K.jm - 2 || i < 1 || i > K.im - 2) return;
    const int64_t c = ((int64_t)i * K.jm + j) * K.kp + k;
    p[c] += f2d(e[c]);
}

template <typename To, typename Ti>
__global__ void convert_kernel(const KConst K, To* __restrict__ out, const Ti* __restrict__ in) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= K.km || j >= K.jm) return;
    const int64_t c = ((int64_t)i * K.jm + j) * K.kp + k;
    if (sizeof(To) == 8) out[c] = (To)f2d((float)in[c]);
    else out[c] = (To)d2f((double)in[c]);
}

// sum of p over the interior P cells (for the zero-mean normalisation)
template <typename T>
__global__ void __launch_bounds__(256) sum_kernel(const KConst K, const T* __restrict__ p, double* __restrict__ out) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    double v = 0.0;
    if (k <= K.km - 2 && j >= 1 && j <= K.jm - 2 && i >= 1 && i <= K.im - 2)
        v = (double)p[((int64_t)i * K.jm + j) * K.kp + k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __shared__ double s[8];
    if (threadIdx.x == 0) s[threadIdx.y] = v;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        double a = 0.0;
        for (int q = 0; q < 8; q++) a += s[q];
        atomicAdd(out, a);
    }
}

template <typename T>
__global__ void shift_kernel(const KConst K, T* __restrict__ p, const double* __restrict__ sum, double inv_n) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= K.km || j >= K.jm) return;
    const int64_t c = ((int64_t)i * K.jm + j) * K.kp + k;
    p[c] = (T)((double)p[c] - sum[0] * inv_n);
}

// ---- spectral solve ----
// spec layout: [(m * 2 + part) * NJ + jj] * NI + ii, part 0 = cosine, 1 = sine coefficients
struct Spec {
    int n, M, NI, NJ;     // ring length km-1, modes n/2+1, radial and polar unknowns
};

template <typename T>
__global__ void dft_fwd_kernel(const KConst K, const Spec S, const T* __restrict__ x, const T* __restrict__ tw,
                               T* __restrict__ spec) {
    extern __shared__ __align__(16) unsigned char dsm[];
    T* row = reinterpret_cast<T*>(dsm);             // n
    T* tc = row + S.n;                              // cos table, n
    T* ts = tc + S.n;                               // sin table, n
    const int ii = blockIdx.x, jj = blockIdx.y;
    const int i = ii + 1, j = jj + 1;
    const int64_t base = ((int64_t)i * K.jm + j) * K.kp;
    for (int k = threadIdx.x; k < S.n; k += blockDim.x) {
        row[k] = x[base + k];
        tc[k] = tw[k];
        ts[k] = tw[S.n + k];
    }
    __syncthreads();
    for (int m = threadIdx.x; m < S.M; m += blockDim.x) {
        T a = 0, b = 0;
        int idx = 0;
        for (int k = 0; k < S.n; k++) {
            a += row[k] * tc[idx];
            b += row[k] * ts[idx];
            idx += m;
            if (idx >= S.n) idx -= S.n;
        }
        spec[((int64_t)(m * 2 + 0) * S.NJ + jj) * S.NI + ii] = a;
        spec[((int64_t)(m * 2 + 1) * S.NJ + jj) * S.NI + ii] = b;
    }
}

template <typename T>
__global__ void dft_inv_kernel(const KConst K, const Spec S, const T* __restrict__ spec, const T* __restrict__ tw,
                               T* __restrict__ x) {
    extern __shared__ __align__(16) unsigned char dsm[];
    T* a = reinterpret_cast<T*>(dsm);               // M
    T* b = a + S.M;                                 // M
    T* tc = b + S.M;                                // n
    T* ts = tc + S.n;                               // n
    const int ii = blockIdx.x, jj = blockIdx.y;
    const int i = ii + 1, j = jj + 1;
    for (int m = threadIdx.x; m < S.M; m += blockDim.x) {
        a[m] = spec[((int64_t)(m * 2 + 0) * S.NJ + jj) * S.NI + ii];
        b[m] = spec[((int64_t)(m * 2 + 1) * S.NJ + jj) * S.NI + ii];
    }
    for (int k = threadIdx.x; k < S.n; k += blockDim.x) { tc[k] = tw[k]; ts[k] = tw[S.n + k]; }
    __syncthreads();
    const bool even = (S.n & 1) == 0;
    const int mtop = even ? S.M - 1 : S.M;          // modes with a conjugate partner: 1 .. mtop-1
    const T inv_n = (T)1 / (T)S.n;
    const int64_t base = ((int64_t)i * K.jm + j) * K.kp;
    for (int k = threadIdx.x; k < S.n; k += blockDim.x) {
        T s = 0;
        int idx = k;                                  // (m k) mod n for m = 1
        for (int m = 1; m < mtop; m++) {
            s += a[m] * tc[idx] + b[m] * ts[idx];
            idx += k;
            if (idx >= S.n) idx -= S.n;
        }
        T v = a[0] + (T)2 * s;
        if (even) v += a[S.M - 1] * ((k & 1) ? (T)-1 : (T)1);
        x[base + k] = v * inv_n;
    }
}

// Block Thomas for one (mode, part): g_j = f_j - b_j * (W_{j-1} g_{j-1}); x_NJ = W_NJ g_NJ;
// x_j = W_j (g_j - c_j * x_{j+1}). W is column-major per block; b, c are the theta couplings (mode
// independent); the zero mode pins the cell (1, 1) (its row of D_1 is the identity, its c is 0, f = 0).
template <typename T>
__global__ void bt_solve_kernel(const Spec S, const T* __restrict__ W, const double* __restrict__ bvec,
                                const double* __restrict__ cvec, T* __restrict__ spec) {
    const int m = blockIdx.x >> 1, part = blockIdx.x & 1;
    const bool even = (S.n & 1) == 0;
    if (part == 1 && (m == 0 || (even && m == S.M - 1))) return;   // sine part identically zero
    const int NI = S.NI, NJ = S.NJ;
    extern __shared__ __align__(16) unsigned char dsm[];
    T* g = reinterpret_cast<T*>(dsm);   // NI
    T* t = g + NI;                      // NI
    T* f = spec + (int64_t)(m * 2 + part) * NJ * NI;
    const T* Wm = W + (int64_t)m * NJ * NI * NI;
    const int r = threadIdx.x;
    const bool pin = (m == 0 && part == 0);
    // forward
    if (r < NI) g[r] = (pin && r == 0) ? (T)0 : f[r];
    __syncthreads();
    for (int jj = 1; jj < NJ; jj++) {
        if (r < NI) {
            const T* Wp = Wm + (int64_t)(jj - 1) * NI * NI;
            T acc = 0;
            for (int c = 0; c < NI; c++) acc += Wp[(int64_t)c * NI + r] * g[c];
            t[r] = f[(int64_t)jj * NI + r] - (T)bvec[jj * NI + r] * acc;
        }
        __syncthreads();
        if (r < NI) {
            f[(int64_t)(jj - 1) * NI + r] = g[r];     // keep g_{j-1} for the backward pass
            g[r] = t[r];
        }
        __syncthreads();
    }
    // backward: x_NJ = W_NJ g_NJ
    {
        const T* Wp = Wm + (int64_t)(NJ - 1) * NI * NI;
        T acc = 0;
        if (r < NI) for (int c = 0; c < NI; c++) acc += Wp[(int64_t)c * NI + r] * g[c];
        __syncthreads();
        if (r < NI) { g[r] = acc; f[(int64_t)(NJ - 1) * NI + r] = acc; }
        __syncthreads();
    }
    for (int jj = NJ - 2; jj >= 0; jj--) {
        if (r < NI) {
            T cc = (T)cvec[jj * NI + r];
            if (pin && jj == 0 && r == 0) cc = 0;
            t[r] = f[(int64_t)jj * NI + r] - cc * g[r];
        }
        __syncthreads();
        if (r < NI) {
            const T* Wp = Wm + (int64_t)jj * NI * NI;
            T acc = 0;
            for (int c = 0; c < NI; c++) acc += Wp[(int64_t)c * NI + r] * t[c];
            g[r] = acc;
            f[(int64_t)jj * NI + r] = acc;
        }
        __syncthreads();
    }
}

dim3 cell_grid(const KConst& K) { return dim3((K.km + 31) / 32, (K.jm + 7) / 8, K.im); }

// Gauss-Jordan inverse with partial pivoting of an n x n row-major matrix (in place into inv)
bool invert(int n, std::vector<double>& a, std::vector<double>& inv) {
    inv.assign((size_t)n * n, 0.0);
    for (int q = 0; q < n; q++) inv[(size_t)q * n + q] = 1.0;
    for (int c = 0; c < n; c++) {
        int piv = c;
        for (int r = c + 1; r < n; r++)
            if (std::fabs(a[(size_t)r * n + c]) > std::fabs(a[(size_t)piv * n + c])) piv = r;
        if (!(std::fabs(a[(size_t)piv * n + c]) > 0.0)) return false;
        if (piv != c)
            for (int q = 0; q < n; q++) {
                std::swap(a[(size_t)c * n + q], a[(size_t)piv * n + q]);
                std::swap(inv[(size_t)c * n + q], inv[(size_t)piv * n + q]);
            }
        const double d = 1.0 / a[(size_t)c * n + c];
        for (int q = 0; q < n; q++) { a[(size_t)c * n + q] *= d; inv[(size_t)c * n + q] *= d; }
        for (int r = 0; r < n; r++) {
            if (r == c) continue;
            const double fct = a[(size_t)r * n + c];
            if (fct == 0.0) continue;
            for (int q = 0; q < n; q++) {
                a[(size_t)r * n + q] -= fct * a[(size_t)c * n + q];
                inv[(size_t)r * n + q] -= fct * inv[(size_t)c * n + q];
            }
        }
    }
    return true;
}

}  // namespace

struct PoissonSolver {
    KConst K{};
    Spec S{};
    cudaStream_t stream = nullptr;
    const ColGeo* geo = nullptr;          // device column geometry (owned by the handle)
    std::vector<double> num1, num2, num3, den;   // host, [jj * NI + ii]
    std::vector<double> bvec, cvec;       // host theta couplings
    // device
    double *f64 = nullptr, *p64 = nullptr, *r64 = nullptr, *sq = nullptr, *W64 = nullptr, *spec64 = nullptr;
    double *bvec_d = nullptr, *cvec_d = nullptr, *tw64 = nullptr;
    float *p32 = nullptr, *r32 = nullptr, *e32 = nullptr, *W32 = nullptr, *spec32 = nullptr, *tw32 = nullptr;
    std::vector<double> ynull;            // left null vector of the zero mode, [jj * NI + ii]
    void* block = nullptr;
    int64_t n_interior = 0;
    // the checkerboard-packed SOR (even rings only): per precision both colours of p and f, the column
    // weights, the grid barrier's words, and the cooperative launch's grid
    int kh = 0;
    bool packed = false;
    double *pk64[2] = {}, *fk64[2] = {};
    float *pk32[2] = {}, *fk32[2] = {};
    SorW<double>* w64 = nullptr;
    SorW<float>* w32 = nullptr;
    GridBar* bar = nullptr;
    int coop_blocks64 = 0, coop_blocks32 = 0;
    // the temporally blocked FP32 sweeps: the second pair of packed p arrays (passes alternate between the
    // pairs), sweeps per pass (0: not available on this grid), the tiling, its shared memory and grid
    float* pkb32[2] = {};
    int tb_S = 0, tb_grid = 0;
    size_t tb_smem = 0;
    TbPlan tb{};
    std::vector<TbTile> tb_tiles_h;
    TbTile* tb_tiles = nullptr;
    // the last solve's sweeps between barriers and device time of its sweep launches (events around them)
    cudaEvent_t sev[2] = {};
    int spp = 0;
    double sweep_ms = 0.0;
};

namespace {

// D_j(m) as a dense NI x NI row-major matrix; `pin`: the zero mode's cell (1, 1) becomes x = 0
void build_D(const PoissonSolver& P, int m, int jj, std::vector<double>& D, bool pin = true) {
    const int NI = P.S.NI, NJ = P.S.NJ;
    const double c43 = P.K.c43, c13 = P.K.c13;
    const double cth = std::cos(2.0 * M_PI * (double)m / (double)P.S.n);
    D.assign((size_t)NI * NI, 0.0);
    for (int ii = 0; ii < NI; ii++) {
        const size_t q = (size_t)jj * NI + ii;
        double d = -P.den[q] + 2.0 * P.num3[q] * cth;
        if (jj == 0) d += c43 * P.num2[q];
        if (jj == NJ - 1) d += c43 * P.num2[q];
        if (ii == 0) d += c43 * P.num1[q];
        if (ii == NI - 1) d += c43 * P.num1[q];
        D[(size_t)ii * NI + ii] = d;
        if (ii + 1 < NI) D[(size_t)ii * NI + ii + 1] = P.num1[q] * (ii == 0 ? 1.0 - c13 : 1.0);
        if (ii > 0) D[(size_t)ii * NI + ii - 1] = P.num1[q] * (ii == NI - 1 ? 1.0 - c13 : 1.0);
    }
    if (pin && m == 0 && jj == 0) {           // the pinned cell (1, 1)
        for (int q = 0; q < NI; q++) D[q] = 0.0;
        D[0] = 1.0;
    }
}

// The tiling of the temporally blocked sweeps with S sweeps per pass: packed columns in tiles of at most
// TB_LANES - 2S (so that tile and halo fit one shared row); rows split evenly into as many tiles as fill the
// co-resident blocks, each of at least two rows (so that the tile owning j = 1 or jm-2 also updates j = 2 or
// jm-3, whose updates write the folded rows it owns), and fewer, larger ones only if the shared memory
// allows no more. Leaves tb_S = 0 where no tiling fits (the one-sweep-per-phase kernel then runs).
void plan_tb(PoissonSolver* P, int S, int dev, int nsm) {
    const KConst& K = P->K;
    const int nh = P->S.n / 2, NJ = K.jm - 2;
    if ((nh & 1) || (S & 1)) return;          // column pairs: an even half-ring, an even halo
    const int ntm = (nh + TB_LANES - 2 * S - 1) / (TB_LANES - 2 * S);
    int optin = 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    const void* fn = (const void*)sor_tb_kernel<2>;
    // the kernel's limit: the device's, less the kernel's static shared memory (handles on other grids
    // share the function)
    cudaFuncAttributes fa{};
    if (cudaFuncGetAttributes(&fa, fn) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    optin -= (int)fa.sharedSizeBytes;
    if (optin <= 0 || cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    for (int ntj = std::max(1, std::min(nsm / ntm, NJ / 2)); ntj <= NJ / 2 && ntm * ntj <= TB_MAX_TILES; ntj++) {
        const int tjmax = (NJ + ntj - 1) / ntj;
        const size_t smem = tb_smem_bytes(K.im, tjmax + 4 * S);
        if (smem > (size_t)optin) continue;
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fn, 32 * TB_WARPS, smem) != cudaSuccess || b < 1) {
            cudaGetLastError();
            return;
        }
        // tile boundaries along m rounded to even columns (the pairs of the tile loads and stores)
        auto mb = [&](int tm) { return (tm * nh / ntm) & ~1; };
        P->tb_tiles_h.clear();
        for (int t = 0; t < ntm * ntj; t++) {
            const int tm = t % ntm, tj = t / ntm;
            const int m0 = mb(tm), m1 = (tm + 1 == ntm) ? nh : mb(tm + 1), j0 = 1 + tj * NJ / ntj;
            if (m1 - m0 < 2 || m1 - m0 + 2 * S > TB_LANES) return;
            P->tb_tiles_h.push_back(TbTile{m0, m1 - m0, j0, 1 + (tj + 1) * NJ / ntj});
        }
        P->tb = TbPlan{ntm * ntj, tjmax + 4 * S, nh};
        P->tb_S = S;
        P->tb_smem = smem;
        P->tb_grid = std::min(ntm * ntj, b * nsm);
        return;
    }
}

}  // namespace

PoissonSolver* poisson_create(const KConst& kc, const ColGeo* geo_dev, const std::vector<ColGeo>& geo_h,
                              cudaStream_t s, std::string* err) {
    if (kc.im < 5 || kc.jm < 5 || kc.km < 4) { *err = "poisson: grid too small (im, jm >= 5, km >= 4)"; return nullptr; }
    auto* P = new PoissonSolver();
    P->K = kc;
    P->stream = s;
    P->geo = geo_dev;
    Spec& S = P->S;
    S.n = kc.km - 1;
    S.M = S.n / 2 + 1;
    S.NI = kc.im - 2;
    S.NJ = kc.jm - 2;
    if (S.NI > 1024) { *err = "poisson: im too large"; delete P; return nullptr; }
    const int NI = S.NI, NJ = S.NJ;
    P->n_interior = (int64_t)NI * NJ * S.n;
    const size_t nc = (size_t)NI * NJ;
    P->num1.resize(nc); P->num2.resize(nc); P->num3.resize(nc); P->den.resize(nc);
    for (int jj = 0; jj < NJ; jj++)
        for (int ii = 0; ii < NI; ii++) {
            const ColGeo& g = geo_h[(size_t)(ii + 1) * kc.jm + (jj + 1)];
            const size_t q = (size_t)jj * NI + ii;
            P->num1[q] = g.p_num1; P->num2[q] = g.p_num2; P->num3[q] = g.p_num3; P->den[q] = g.p_den;
        }
    P->bvec.assign(nc, 0.0);
    P->cvec.assign(nc, 0.0);
    for (int jj = 0; jj < NJ; jj++)
        for (int ii = 0; ii < NI; ii++) {
            const size_t q = (size_t)jj * NI + ii;
            P->bvec[q] = P->num2[q] * (jj == NJ - 1 ? 1.0 - kc.c13 : 1.0);   // coefficient of x_{j-1}
            P->cvec[q] = P->num2[q] * (jj == 0 ? 1.0 - kc.c13 : 1.0);        // coefficient of x_{j+1}
        }
    // the inverse pivot blocks of every mode (FP64), then an FP32 copy
    const size_t blk = (size_t)NI * NI;
    std::vector<double> W((size_t)S.M * NJ * blk);
    bool ok = true;
#pragma omp parallel for schedule(dynamic)
    for (int m = 0; m < S.M; m++) {
        std::vector<double> D, Sm, inv;
        double* Wm = W.data() + (size_t)m * NJ * blk;
        for (int jj = 0; jj < NJ; jj++) {
            build_D(*P, m, jj, D);
            Sm = D;
            if (jj > 0) {
                const double* Wp = Wm + (size_t)(jj - 1) * blk;     // column-major W_{j-1}
                for (int r = 0; r < NI; r++) {
                    const double b = P->bvec[(size_t)jj * NI + r];
                    for (int c = 0; c < NI; c++) {
                        double cc = P->cvec[(size_t)(jj - 1) * NI + c];
                        if (m == 0 && jj - 1 == 0 && c == 0) cc = 0.0;
                        Sm[(size_t)r * NI + c] -= b * Wp[(size_t)c * NI + r] * cc;
                    }
                }
            }
            if (!invert(NI, Sm, inv)) {
#pragma omp atomic write
                ok = false;
                break;
            }
            double* Wj = Wm + (size_t)jj * blk;
            for (int r = 0; r < NI; r++)
                for (int c = 0; c < NI; c++) Wj[(size_t)c * NI + r] = inv[(size_t)r * NI + c];
        }
    }
    if (!ok) { *err = "poisson: singular pivot block"; delete P; return nullptr; }
    // Left null vector of the unpinned zero-mode operator A0 (host, once): A0^T y = 0 with the transposed
    // equation of cell (1, 1) replaced by y(1, 1) = 1. A0^T is block tridiagonal: block row j holds
    // diag(cvec[j-1]) y_{j-1} + D_j^T y_j + diag(bvec[j+1]) y_{j+1}.
    {
        std::vector<std::vector<double>> Winv(NJ), g(NJ);
        std::vector<double> D, Sm(blk), inv;
        auto upper = [&](int jj, int c) {            // U_jj = diag(bvec[jj+1]), its pinned row zeroed
            return (jj == 0 && c == 0) ? 0.0 : P->bvec[(size_t)(jj + 1) * NI + c];
        };
        for (int jj = 0; jj < NJ; jj++) {
            build_D(*P, 0, jj, D, false);
            for (int r = 0; r < NI; r++)
                for (int c = 0; c < NI; c++) Sm[(size_t)r * NI + c] = D[(size_t)c * NI + r];
            std::vector<double> rhs(NI, 0.0);
            if (jj == 0) {
                for (int c = 0; c < NI; c++) Sm[c] = (c == 0) ? 1.0 : 0.0;
                rhs[0] = 1.0;
            } else {
                std::vector<double> wg(NI, 0.0);
                for (int r = 0; r < NI; r++) {
                    const double low = P->cvec[(size_t)(jj - 1) * NI + r];
                    for (int c = 0; c < NI; c++) {
                        Sm[(size_t)r * NI + c] -= low * Winv[jj - 1][(size_t)r * NI + c] * upper(jj - 1, c);
                        wg[r] += Winv[jj - 1][(size_t)r * NI + c] * g[jj - 1][c];
                    }
                    rhs[r] -= low * wg[r];
                }
            }
            if (!invert(NI, Sm, inv)) { *err = "poisson: singular block (null vector)"; delete P; return nullptr; }
            Winv[jj] = inv;
            g[jj] = rhs;
        }
        P->ynull.assign(nc, 0.0);
        std::vector<double> t(NI), ynext(NI, 0.0);
        for (int jj = NJ - 1; jj >= 0; jj--) {
            for (int r = 0; r < NI; r++) t[r] = g[jj][r] - ((jj + 1 < NJ) ? upper(jj, r) * ynext[r] : 0.0);
            for (int r = 0; r < NI; r++) {
                double a = 0.0;
                for (int c = 0; c < NI; c++) a += Winv[jj][(size_t)r * NI + c] * t[c];
                P->ynull[(size_t)jj * NI + r] = a;
            }
            for (int r = 0; r < NI; r++) ynext[r] = P->ynull[(size_t)jj * NI + r];
        }
    }
    // device buffers
    const size_t fsz = (size_t)kc.fsz;
    const size_t nspec = (size_t)S.M * 2 * nc;
    const size_t nW = (size_t)S.M * NJ * blk;
    size_t bytes = 0;
    auto take = [&](size_t b) { size_t o = bytes; bytes += (b + 255) & ~size_t(255); return o; };
    const size_t o_f = take(fsz * 8), o_p = take(fsz * 8), o_r = take(fsz * 8), o_sq = take(64);
    const size_t o_W64 = take(nW * 8), o_s64 = take(nspec * 8), o_b = take(nc * 8), o_c = take(nc * 8);
    const size_t o_tw64 = take((size_t)2 * S.n * 8), o_p32 = take(fsz * 4), o_r32 = take(fsz * 4), o_e32 = take(fsz * 4);
    const size_t o_W32 = take(nW * 4), o_s32 = take(nspec * 4), o_tw32 = take((size_t)2 * S.n * 4);
    // the packed SOR's arrays (even rings): p and f of both colours in each precision, the column weights
    P->packed = (S.n % 2) == 0;
    P->kh = ((S.n / 2 + 31) / 32) * 32;
    const size_t npk = P->packed ? (size_t)kc.im * kc.jm * P->kh : 0, ncol = (size_t)kc.im * kc.jm;
    const size_t o_pk64 = take(4 * npk * 8), o_pk32 = take(4 * npk * 4), o_pkb32 = take(2 * npk * 4);
    const size_t o_w64 = take(P->packed ? ncol * sizeof(SorW<double>) : 0);
    const size_t o_w32 = take(P->packed ? ncol * sizeof(SorW<float>) : 0), o_bar = take(sizeof(GridBar));
    const size_t o_tiles = take(P->packed ? TB_MAX_TILES * sizeof(TbTile) : 0);
    cudaError_t e = cudaMalloc(&P->block, bytes);
    if (e != cudaSuccess) { *err = std::string("poisson: cudaMalloc: ") + cudaGetErrorString(e); delete P; return nullptr; }
    if ((e = cudaEventCreate(&P->sev[0])) != cudaSuccess || (e = cudaEventCreate(&P->sev[1])) != cudaSuccess) {
        *err = std::string("poisson: cudaEventCreate: ") + cudaGetErrorString(e);
        poisson_destroy(P);
        return nullptr;
    }
    char* b0 = static_cast<char*>(P->block);
    P->f64 = reinterpret_cast<double*>(b0 + o_f);
    P->p64 = reinterpret_cast<double*>(b0 + o_p);
    P->r64 = reinterpret_cast<double*>(b0 + o_r);
    P->sq = reinterpret_cast<double*>(b0 + o_sq);
    P->W64 = reinterpret_cast<double*>(b0 + o_W64);
    P->spec64 = reinterpret_cast<double*>(b0 + o_s64);
    P->bvec_d = reinterpret_cast<double*>(b0 + o_b);
    P->cvec_d = reinterpret_cast<double*>(b0 + o_c);
    P->tw64 = reinterpret_cast<double*>(b0 + o_tw64);
    P->p32 = reinterpret_cast<float*>(b0 + o_p32);
    P->r32 = reinterpret_cast<float*>(b0 + o_r32);
    P->e32 = reinterpret_cast<float*>(b0 + o_e32);
    P->W32 = reinterpret_cast<float*>(b0 + o_W32);
    P->spec32 = reinterpret_cast<float*>(b0 + o_s32);
    P->tw32 = reinterpret_cast<float*>(b0 + o_tw32);
    P->bar = reinterpret_cast<GridBar*>(b0 + o_bar);
    std::vector<SorW<double>> w64h;
    std::vector<SorW<float>> w32h;
    if (P->packed) {
        for (int q = 0; q < 4; q++) {
            double* d = reinterpret_cast<double*>(b0 + o_pk64) + q * npk;
            float* f = reinterpret_cast<float*>(b0 + o_pk32) + q * npk;
            if (q < 2) { P->pk64[q] = d; P->pk32[q] = f; } else { P->fk64[q - 2] = d; P->fk32[q - 2] = f; }
        }
        P->pkb32[0] = reinterpret_cast<float*>(b0 + o_pkb32);
        P->pkb32[1] = P->pkb32[0] + npk;
        P->tb_tiles = reinterpret_cast<TbTile*>(b0 + o_tiles);
        P->w64 = reinterpret_cast<SorW<double>*>(b0 + o_w64);
        P->w32 = reinterpret_cast<SorW<float>*>(b0 + o_w32);
        w64h.resize(ncol);
        w32h.resize(ncol);
        for (size_t q = 0; q < ncol; q++) {
            const ColGeo& c = geo_h[q];
            const double rden = 1.0 / c.p_den;
            w64h[q] = SorW<double>{c.p_num1, c.p_num2, c.p_num3, rden};
            w32h[q] = SorW<float>{(float)c.p_num1, (float)c.p_num2, (float)c.p_num3, (float)rden};
        }
        // the cooperative launch's grid: as many blocks as fit on the GPU at once
        int dev = 0, nsm = 0, b64 = 0, b32 = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b64, sor_packed_kernel<double>, 32 * SORP_WARPS, 0) !=
                cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b32, sor_packed_kernel<float>, 32 * SORP_WARPS, 0) !=
                cudaSuccess) {
            cudaGetLastError();
            P->packed = false;
        } else {
            P->coop_blocks64 = nsm * b64;
            P->coop_blocks32 = nsm * b32;
            if (P->coop_blocks64 < 1 || P->coop_blocks32 < 1) P->packed = false;
        }
        if (P->packed) {
            // ATSAT_SOR_SWEEPS_PER_PASS=1 keeps the one-sweep-per-phase kernel (a comparison switch)
            const char* ev = std::getenv("ATSAT_SOR_SWEEPS_PER_PASS");
            if (!(ev && std::atoi(ev) == 1)) plan_tb(P, 2, dev, nsm);
        }
    }
    std::vector<float> W32(nW);
    for (size_t q = 0; q < nW; q++) W32[q] = (float)W[q];
    std::vector<double> tw(2 * S.n);
    std::vector<float> tw32(2 * S.n);
    for (int k = 0; k < S.n; k++) {
        tw[k] = std::cos(2.0 * M_PI * k / S.n);
        tw[S.n + k] = std::sin(2.0 * M_PI * k / S.n);
    }
    for (int q = 0; q < 2 * S.n; q++) tw32[q] = (float)tw[q];
    if ((e = cudaMemsetAsync(P->block, 0, bytes, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(P->W64, W.data(), nW * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(P->W32, W32.data(), nW * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(P->bvec_d, P->bvec.data(), nc * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(P->cvec_d, P->cvec.data(), nc * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(P->tw64, tw.data(), 2 * S.n * 8, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (e = cudaMemcpyAsync(P->tw32, tw32.data(), 2 * S.n * 4, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (!w64h.empty() && (e = cudaMemcpyAsync(P->w64, w64h.data(), w64h.size() * sizeof(SorW<double>),
                                               cudaMemcpyHostToDevice, s)) != cudaSuccess) ||
        (!w32h.empty() && (e = cudaMemcpyAsync(P->w32, w32h.data(), w32h.size() * sizeof(SorW<float>),
                                               cudaMemcpyHostToDevice, s)) != cudaSuccess) ||
        (!P->tb_tiles_h.empty() && (e = cudaMemcpyAsync(P->tb_tiles, P->tb_tiles_h.data(),
                                                        P->tb_tiles_h.size() * sizeof(TbTile),
                                                        cudaMemcpyHostToDevice, s)) != cudaSuccess) ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess) {
        *err = std::string("poisson: upload: ") + cudaGetErrorString(e);
        poisson_destroy(P);
        return nullptr;
    }
    return P;
}

void poisson_destroy(PoissonSolver* P) {
    if (!P) return;
    for (cudaEvent_t& ev : P->sev)
        if (ev) cudaEventDestroy(ev);
    if (P->block) cudaFree(P->block);
    delete P;
}

void poisson_sweep_stats(PoissonSolver* P, int* sweeps_per_pass, double* sweep_ms) {
    *sweeps_per_pass = P->spp;
    *sweep_ms = P->sweep_ms;
}

double* poisson_f(PoissonSolver* P) { return P->f64; }
double* poisson_p(PoissonSolver* P) { return P->p64; }
const std::vector<double>& poisson_null_vector(PoissonSolver* P) { return P->ynull; }
int poisson_modes(PoissonSolver* P) { return P->S.M; }

namespace {

template <typename T>
cudaError_t fold(PoissonSolver* P, T* p) {
    const KConst& K = P->K;
    const int64_t n = (int64_t)K.im * K.jm + 2LL * K.jm * (K.km - 1) + 2LL * (K.im - 2) * (K.km - 1);
    fold_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, P->stream>>>(K, p);
    return cudaGetLastError();
}

template <typename T>
cudaError_t sor_sweep(PoissonSolver* P, const T* f, T* p, T w) {
    const KConst& K = P->K;
    const int nm = (K.km - 1 + 1) / 2;
    const dim3 grid((nm + 31) / 32, (K.jm + 7) / 8, K.im), block(32, 8);
    for (int colour = 0; colour < 2; colour++) {
        sor_kernel<T><<<grid, block, 0, P->stream>>>(K, P->geo, f, p, colour, w);
        if (((K.km - 1) & 1) && K.km - 2 > 0) {
            const int n = (K.im - 2) * (K.jm - 2);
            sor_seam_kernel<T><<<(n + 255) / 256, 256, 0, P->stream>>>(K, P->geo, f, p, colour, w);
        }
    }
    return fold(P, p);
}

template <typename T> T** packed_p(PoissonSolver* P);
template <> double** packed_p<double>(PoissonSolver* P) { return P->pk64; }
template <> float** packed_p<float>(PoissonSolver* P) { return P->pk32; }
template <typename T> T** packed_f(PoissonSolver* P);
template <> double** packed_f<double>(PoissonSolver* P) { return P->fk64; }
template <> float** packed_f<float>(PoissonSolver* P) { return P->fk32; }
template <typename T> const SorW<T>* packed_w(PoissonSolver* P);
template <> const SorW<double>* packed_w<double>(PoissonSolver* P) { return P->w64; }
template <> const SorW<float>* packed_w<float>(PoissonSolver* P) { return P->w32; }

// `nsweeps` sweeps of the checkerboard-packed SOR in one cooperative launch: f and p packed first where
// asked (p keeps its packed copy between calls), p unpacked and folded after. FP32 runs the temporally
// blocked kernel where the grid has a tiling (tb_S > 0); its passes alternate between the two pairs of
// packed p arrays, and the pair holding the result becomes the current one. The barrier's error word is
// read back: a barrier wait that gave up returns cudaErrorLaunchTimeout.
template <typename T>
cudaError_t sor_packed_run(PoissonSolver* P, const T* f, T* p, T w, int nsweeps, bool pack_f, bool pack_p) {
    const KConst& K = P->K;
    const int kh = P->kh;
    T** pk = packed_p<T>(P);
    T** fk = packed_f<T>(P);
    const dim3 pg((K.km - 1) / 2 / 32 + 1, (K.jm + 7) / 8, K.im), pb(32, 8);
    if (pack_f) pack_kernel<T><<<pg, pb, 0, P->stream>>>(K, f, fk[0], fk[1], kh);
    if (pack_p) pack_kernel<T><<<pg, pb, 0, P->stream>>>(K, p, pk[0], pk[1], kh);
    cudaError_t e = cudaMemsetAsync(P->bar, 0, sizeof(GridBar), P->stream);
    if (e != cudaSuccess) return e;
    const SorW<T>* wt = packed_w<T>(P);
    T* p0 = pk[0];
    T* p1 = pk[1];
    const T* f0 = fk[0];
    const T* f1 = fk[1];
    long long limit = TILE_WAIT_LIMIT;
    if ((e = cudaEventRecord(P->sev[0], P->stream)) != cudaSuccess) return e;
    P->spp = (sizeof(T) == 4 && P->tb_S > 0) ? P->tb_S : 1;
    if (sizeof(T) == 4 && P->tb_S > 0) {
        float* b0 = P->pkb32[0];
        float* b1 = P->pkb32[1];
        TbPlan pl = P->tb;
        const TbTile* tiles = P->tb_tiles;
        void* args[] = {(void*)&K, (void*)&wt, (void*)&tiles, (void*)&p0, (void*)&p1, (void*)&b0, (void*)&b1,
                        (void*)&f0, (void*)&f1, (void*)&kh, (void*)&nsweeps, (void*)&w, (void*)&pl,
                        (void*)&P->bar, (void*)&limit};
        const void* fn = (const void*)sor_tb_kernel<2>;
        e = cudaLaunchCooperativeKernel(fn, dim3(P->tb_grid), dim3(32, TB_WARPS), args, P->tb_smem, P->stream);
        if (e != cudaSuccess) return e;
        if ((((nsweeps + P->tb_S - 1) / P->tb_S) & 1) == 1) {     // an odd number of passes: the result is in B
            std::swap(P->pk32[0], P->pkb32[0]);
            std::swap(P->pk32[1], P->pkb32[1]);
        }
    } else {
        void* args[] = {(void*)&K, (void*)&wt, (void*)&p0, (void*)&p1, (void*)&f0, (void*)&f1, (void*)&kh,
                        (void*)&nsweeps, (void*)&w, (void*)&P->bar, (void*)&limit};
        const int nb = sizeof(T) == 8 ? P->coop_blocks64 : P->coop_blocks32;
        e = cudaLaunchCooperativeKernel((const void*)sor_packed_kernel<T>, dim3(nb), dim3(32, SORP_WARPS), args, 0,
                                        P->stream);
        if (e != cudaSuccess) return e;
    }
    if ((e = cudaEventRecord(P->sev[1], P->stream)) != cudaSuccess) return e;
    unpack_kernel<T><<<pg, pb, 0, P->stream>>>(K, p, pk[0], pk[1], kh);
    if ((e = fold(P, p)) != cudaSuccess) return e;
    unsigned herr = 0;
    if ((e = cudaMemcpyAsync(&herr, &P->bar->err, sizeof(herr), cudaMemcpyDeviceToHost, P->stream)) != cudaSuccess)
        return e;
    if ((e = cudaStreamSynchronize(P->stream)) != cudaSuccess) return e;
    float ms = 0.0f;
    if ((e = cudaEventElapsedTime(&ms, P->sev[0], P->sev[1])) != cudaSuccess) return e;
    P->sweep_ms += ms;
    return herr ? cudaErrorLaunchTimeout : cudaSuccess;
}

// x = L^-1 rhs by the spectral block solve in precision T (rhs and x pitched; x may alias rhs)
template <typename T>
cudaError_t direct(PoissonSolver* P, const T* rhs, T* x, T* spec, const T* W, const T* tw) {
    const KConst& K = P->K;
    const Spec& S = P->S;
    const dim3 rows(S.NI, S.NJ);
    dft_fwd_kernel<T><<<rows, 128, (size_t)3 * S.n * sizeof(T), P->stream>>>(K, S, rhs, tw, spec);
    const int thr = ((S.NI + 31) / 32) * 32;
    bt_solve_kernel<T><<<2 * S.M, thr, (size_t)2 * S.NI * sizeof(T), P->stream>>>(S, W, P->bvec_d, P->cvec_d, spec);
    dft_inv_kernel<T><<<rows, 128, (size_t)(2 * S.M + 2 * S.n) * sizeof(T), P->stream>>>(K, S, spec, tw, x);
    // zero interior mean (the zero mode's pinned constant), then the boundary planes
    cudaMemsetAsync(P->sq + 2, 0, sizeof(double), P->stream);
    sum_kernel<T><<<cell_grid(K), dim3(32, 8), 0, P->stream>>>(K, x, P->sq + 2);
    shift_kernel<T><<<cell_grid(K), dim3(32, 8), 0, P->stream>>>(K, x, P->sq + 2, 1.0 / (double)P->n_interior);
    return fold(P, x);
}

// ||f - L p|| / ||f|| with r64 (and r32) written
cudaError_t residual(PoissonSolver* P, double* rel) {
    const KConst& K = P->K;
    cudaError_t e = cudaMemsetAsync(P->sq, 0, 2 * sizeof(double), P->stream);
    if (e != cudaSuccess) return e;
    residual_kernel<<<cell_grid(K), dim3(32, 8), 0, P->stream>>>(K, P->geo, P->f64, P->p64, P->r64, P->r32, P->sq);
    double h[2];
    if ((e = cudaMemcpyAsync(h, P->sq, sizeof(h), cudaMemcpyDeviceToHost, P->stream)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(P->stream)) != cudaSuccess) return e;
    *rel = h[1] > 0.0 ? std::sqrt(h[0] / h[1]) : std::sqrt(h[0]);
    return cudaSuccess;
}

}  // namespace

// Solve L p = f (f in P->f64, result in P->p64, both pitched, boundary planes folded).
// method: 0 SOR64, 1 SOR32, 2 REFINE with FP32 SOR inner sweeps, 3 DIRECT64, 4 DIRECT32,
// 5 REFINE with FP32 direct inner solves. Iterations: sweeps (0, 1), outer corrections (2, 5), 1 (3, 4).
cudaError_t poisson_run_inner(PoissonSolver* P, int method, double tol, int max_iter, int inner, double omega,
                              int* iters, int* inner_total, double* rel);

// the solve, then the result shifted to zero interior mean (solutions are defined up to a constant)
cudaError_t poisson_run(PoissonSolver* P, int method, double tol, int max_iter, int inner, double omega,
                        int* iters, int* inner_total, double* rel) {
    cudaError_t e = poisson_run_inner(P, method, tol, max_iter, inner, omega, iters, inner_total, rel);
    if (e != cudaSuccess) return e;
    const KConst& K = P->K;
    if ((e = cudaMemsetAsync(P->sq + 2, 0, sizeof(double), P->stream)) != cudaSuccess) return e;
    sum_kernel<double><<<cell_grid(K), dim3(32, 8), 0, P->stream>>>(K, P->p64, P->sq + 2);
    shift_kernel<double><<<cell_grid(K), dim3(32, 8), 0, P->stream>>>(K, P->p64, P->sq + 2, 1.0 / (double)P->n_interior);
    if ((e = fold<double>(P, P->p64)) != cudaSuccess) return e;
    return cudaStreamSynchronize(P->stream);
}

cudaError_t poisson_run_inner(PoissonSolver* P, int method, double tol, int max_iter, int inner, double omega,
                              int* iters, int* inner_total, double* rel) {
    const KConst& K = P->K;
    cudaError_t e;
    *iters = 0;
    *inner_total = 0;
    P->spp = 0;
    P->sweep_ms = 0.0;
    const size_t fsz = (size_t)K.fsz;
    if (method == 3) {
        e = direct<double>(P, P->f64, P->p64, P->spec64, P->W64, P->tw64);
        if (e != cudaSuccess) return e;
        *iters = 1;
        return residual(P, rel);
    }
    if (method == 4) {
        convert_kernel<float, double><<<cell_grid(K), dim3(32, 8), 0, P->stream>>>(K, P->r32, P->f64);
        e = direct<float>(P, P->r32, P->p32, P->spec32, P->W32, P->tw32);
        if (e != cudaSuccess) return e;
        convert_kernel<double, float><<<cell_grid(K), dim3(32, 8), 0, P->stream>>>(K, P->p64, P->p32);
        *iters = 1;
        return residual(P, rel);
    }
    if ((e = cudaMemsetAsync(P->p64, 0, fsz * 8, P->stream)) != cudaSuccess) return e;
    if (method == 0 || method == 1) {
        const int check = 200;     // sweeps per launch between residual checks
        if (method == 1) {
            if ((e = cudaMemsetAsync(P->p32, 0, fsz * 4, P->stream)) != cudaSuccess) return e;
            convert_kernel<float, double><<<cell_grid(K), dim3(32, 8), 0, P->stream>>>(K, P->e32, P->f64);
        }
        *rel = 1.0;
        if (P->packed) {
            // runs of `check` sweeps in one launch each, the residual between them
            for (int it = 0; it < max_iter;) {
                const int run = std::min(check, max_iter - it);
                e = (method == 0) ? sor_packed_run<double>(P, P->f64, P->p64, omega, run, it == 0, it == 0)
                                  : sor_packed_run<float>(P, P->e32, P->p32, (float)omega, run, it == 0, it == 0);
                if (e != cudaSuccess) return e;
                it += run;
                *iters = it;
                if (method == 1) convert_kernel<double, float><<<cell_grid(K), dim3(32, 8), 0, P->stream>>>(K, P->p64, P->p32);
                if ((e = residual(P, rel)) != cudaSuccess) return e;
                if (*rel <= tol) break;
            }
            return cudaSuccess;
        }
        for (int it = 1; it <= max_iter; it++) {
            e = (method == 0) ? sor_sweep<double>(P, P->f64, P->p64, omega)
                              : sor_sweep<float>(P, P->e32, P->p32, (float)omega);
            if (e != cudaSuccess) return e;
            *iters = it;
            if (it % check == 0 || it == max_iter) {
                if (method == 1) convert_kernel<double, float><<<cell_grid(K), dim3(32, 8), 0, P->stream>>>(K, P->p64, P->p32);
                if ((e = residual(P, rel)) != cudaSuccess) return e;
                if (*rel <= tol) break;
            }
        }
        return cudaSuccess;
    }
    // defect correction: p64 = 0; r = f - L p; e = L^-1 r (FP32); p += e
    for (int it = 0; it <= max_iter; it++) {
        if ((e = residual(P, rel)) != cudaSuccess) return e;
        if (*rel <= tol || it == max_iter) break;
        if (method == 5) {
            e = direct<float>(P, P->r32, P->e32, P->spec32, P->W32, P->tw32);
            *inner_total += 1;
        } else {
            if ((e = cudaMemsetAsync(P->e32, 0, fsz * 4, P->stream)) != cudaSuccess) return e;
            if (P->packed) e = sor_packed_run<float>(P, P->r32, P->e32, (float)omega, inner, true, true);
            else
                for (int s = 0; s < inner && e == cudaSuccess; s++) e = sor_sweep<float>(P, P->r32, P->e32, (float)omega);
            *inner_total += inner;
        }
        if (e != cudaSuccess) return e;
        axpy_kernel<<<cell_grid(K), dim3(32, 8), 0, P->stream>>>(K, P->p64, P->e32);
        if ((e = fold<double>(P, P->p64)) != cudaSuccess) return e;
        *iters = it + 1;
    }
    return cudaGetLastError();
}

}  // namespace atsat
