// Kernels of PressureSolver<cSaturnModel>::run (planet/PressureSolver.h:145-766, pointwise sweep)
// and of its model hook prepareProjectionBoundaries (planet/Pressure_Sat.cpp:78-194).
//
// The source of every interior cell (projection divergence, clamp, defect-correction term lc_old)
// does not depend on p, so it is formed once per call by press_source_kernel, from p_dyn as the call
// finds it -- exactly when the reference forms lc_old (:249-282). Each half-sweep then reads only
// the other colour's p and its own source. The outer boundary of the relaxation (:718-746: radial
// planes, then polar planes, then the seam copy) is one kernel that writes boundary cells only and
// reads interior cells only, so it has no ordering hazard of its own.
#include <algorithm>

#include "dyn_common.cuh"

namespace atsat {

namespace {

__device__ __forceinline__ double ldg(const double* p) { return __ldg(p); }

__device__ __forceinline__ double cubic(double a, double b, double c) { return c - 3.0 * b + 3.0 * a; }

// Radial (z = 0) and polar (z = 1) planes of aux_* and rhs_* (Pressure_Sat.cpp:85-148).
__global__ void prep_planes_kernel(const KConst K, double* const* __restrict__ six_) {
    double* au = six_[0]; double* av = six_[1]; double* aw = six_[2];
    double* ru = six_[3]; double* rv = six_[4]; double* rw = six_[5];
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int r = blockIdx.y * 8 + threadIdx.y;
    if (k > K.km - 2) return;
    const int64_t P = K.plane, kp = K.kp;
    const int im = K.im, jm = K.jm;
    if (blockIdx.z == 0) {
        const int j = r;
        if (j < 1 || j > jm - 2) return;
        const int64_t c0 = (int64_t)j * kp + k;                       // (0, j, k)
        const int64_t c1 = c0 + (int64_t)(im - 1) * P;                 // (im-1, j, k)
#define R0(F_) F_[c0] = cubic(F_[c0 + P], F_[c0 + 2 * P], F_[c0 + 3 * P])
#define R1(F_) F_[c1] = cubic(F_[c1 - P], F_[c1 - 2 * P], F_[c1 - 3 * P])
        if (K.rigid_lid) { au[c0] = 0.0; au[c1] = 0.0; }
        else { R0(au); R1(au); }
        R0(av); R1(av); R0(aw); R1(aw);
        R0(ru); R1(ru); R0(rv); R1(rv); R0(rw); R1(rw);
#undef R0
#undef R1
    } else {
        const int i = r;
        if (i < 1 || i > im - 2) return;
        const int64_t c0 = (int64_t)i * P + k;                         // (i, 0, k)
        const int64_t c1 = c0 + (int64_t)(jm - 1) * kp;                // (i, jm-1, k)
        au[c0] = cubic(au[c0 + kp], au[c0 + 2 * kp], au[c0 + 3 * kp]);
        av[c0] = 0.0; aw[c0] = 0.0;
        au[c1] = cubic(au[c1 - kp], au[c1 - 2 * kp], au[c1 - 3 * kp]);
        av[c1] = 0.0; aw[c1] = 0.0;
        ru[c0] = cubic(ru[c0 + kp], ru[c0 + 2 * kp], ru[c0 + 3 * kp]);
        rv[c0] = 0.0; rw[c0] = 0.0;
        ru[c1] = cubic(ru[c1 - kp], ru[c1 - 2 * kp], ru[c1 - 3 * kp]);
        rv[c1] = 0.0; rw[c1] = 0.0;
    }
}

// Seam copy k = km-1 <- k = 0 of the six arrays (Pressure_Sat.cpp:150-161).
__global__ void prep_seam_kernel(const KConst K, double* const* __restrict__ six_) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= K.im * K.jm * 6) return;
    const int s = e % 6, row = e / 6;
    double* f = six_[s];
    const int64_t c = (int64_t)row * K.kp;
    f[c + K.km - 1] = f[c];
}

__global__ void __launch_bounds__(256) press_source_kernel(
        const KConst K, const ColGeo* __restrict__ geo, const double* __restrict__ su,
        const double* __restrict__ sv, const double* __restrict__ sw, const double* __restrict__ aux_u,
        const double* __restrict__ aux_v, const double* __restrict__ aux_w, const double* __restrict__ rhs_u,
        const double* __restrict__ rhs_v, const double* __restrict__ rhs_w, const double* __restrict__ p,
        double* __restrict__ src, unsigned long long* __restrict__ nclamp) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    bool clamped = false;
    if (k <= K.km - 2 && j >= 1 && j <= K.jm - 2 && i >= 1 && i <= K.im - 2) {
        const int64_t P = K.plane, kp = K.kp;
        const int64_t c = ((int64_t)i * K.jm + j) * kp + k;
        const int kw = (k == 0) ? K.km - 2 : k - 1;
        const int ke = (k == K.km - 2) ? 0 : k + 1;
        const int64_t cw = c - k + kw, ce = c - k + ke;
        const ColGeo* g = geo + ((int64_t)i * K.jm + j);
        // GB300 issues two FP64 operations per SM per cycle: the scales of each difference are one
        // product from the column table, the clamp one compare (finiteness is an exponent test), and
        // lc_old's three second differences accumulate into div by fma (17 operations per cell)
        double dr_, dthe_, dphi_;
        if (K.press_src == 0) {     // legacy div(aux - rhs), PressureSolver.h:373-381
            dr_ = (ldg(aux_u + c + P) - ldg(aux_u + c - P)) - (ldg(rhs_u + c + P) - ldg(rhs_u + c - P));
            dthe_ = (ldg(aux_v + c + kp) - ldg(aux_v + c - kp)) - (ldg(rhs_v + c + kp) - ldg(rhs_v + c - kp));
            dphi_ = (ldg(aux_w + ce) - ldg(aux_w + cw)) - (ldg(rhs_w + ce) - ldg(rhs_w + cw));
        } else {                    // projection source, rigid-lid zero of S_u on the radial walls (:246-248)
            const bool wall0 = K.press_incr && K.rigid_lid;
            const double sup = (wall0 && i + 1 == K.im - 1) ? 0.0 : ldg(su + c + P);
            const double sdn = (wall0 && i - 1 == 0) ? 0.0 : ldg(su + c - P);
            dr_ = sup - sdn;
            dthe_ = ldg(sv + c + kp) - ldg(sv + c - kp);
            dphi_ = ldg(sw + ce) - ldg(sw + cw);
        }
        double div = fma(dphi_, ldg(&g->src_phi), fma(dthe_, ldg(&g->src_the), dr_ * ldg(&g->src_r)));
        const double src_max = ldg(&g->p_den) * K.pdyn_cap;
        uint32_t lo, hi;
        split_f64(div, lo, hi);
        if (((hi >> 20) & 0x7FFu) == 0x7FFu) { div = 0.0; clamped = true; }
        else if (fabs(div) > src_max) { div = (div > src_max) ? src_max : -src_max; clamped = true; }
        if (K.press_incr) {         // lc_old = Lc(p_dyn) before the sweep (:249-282)
            const double p0 = ldg(p + c);      // fma(-2, p0, s) == s - 2 p0: the product is exact
            div = fma(ldg(&g->lc_num1), fma(-2.0, p0, ldg(p + c + P) + ldg(p + c - P)), div);
            div = fma(ldg(&g->lc_num2), fma(-2.0, p0, ldg(p + c + kp) + ldg(p + c - kp)), div);
            div = fma(ldg(&g->lc_num3), fma(-2.0, p0, ldg(p + ce) + ldg(p + cw)), div);
        }
        src[c] = div;
    }
    const unsigned m = __ballot_sync(0xffffffffu, clamped);
    if ((threadIdx.x & 31) == 0 && m && nclamp) atomicAdd(nclamp, (unsigned long long)__popc(m));
}

// One colour of the red-black sweep (PressureSolver.h:318-495): cells with (i + j + k) & 1 == colour.
// The reference visits a row's meridians in increasing k. Neighbours of one colour never touch except
// across the periodic seam when km-1 is odd: then k = 0 and k = km-2 share a colour and km-2 reads
// the value k = 0 received earlier in the same sweep. That cell waits for press_sweep_seam_kernel.
__device__ __forceinline__ void sweep_cell(const KConst& K, const ColGeo* __restrict__ geo,
                                           const double* __restrict__ src, double* __restrict__ p, int i, int j,
                                           int k) {
    const int64_t P = K.plane, kp = K.kp;
    const int64_t c = ((int64_t)i * K.jm + j) * kp + k;
    const int kw = (k == 0) ? K.km - 2 : k - 1;
    const int ke = (k == K.km - 2) ? 0 : k + 1;
    const ColGeo* g = geo + ((int64_t)i * K.jm + j);
    const double acc = (p[c + P] + p[c - P]) * ldg(&g->p_num1) + (p[c + kp] + p[c - kp]) * ldg(&g->p_num2)
                     + (p[c - k + ke] + p[c - k + kw]) * ldg(&g->p_num3);
    p[c] = (acc - ldg(src + c)) * ldg(&g->p_inv_den);
}

__global__ void __launch_bounds__(256) press_sweep_kernel(const KConst K, const ColGeo* __restrict__ geo,
                                                          const double* __restrict__ src, double* __restrict__ p,
                                                          int colour) {
    const int m = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    if (j < 1 || j > K.jm - 2 || i < 1 || i > K.im - 2) return;
    const int k = 2 * m + ((colour - i - j) & 1);
    if (k > K.km - 2) return;
    if (k == K.km - 2 && k > 0 && ((K.km - 1) & 1)) return;      // after its seam partner
    sweep_cell(K, geo, src, p, i, j, k);
}

__global__ void __launch_bounds__(256) press_sweep_seam_kernel(const KConst K, const ColGeo* __restrict__ geo,
                                                               const double* __restrict__ src,
                                                               double* __restrict__ p, int colour) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = 1 + e / (K.jm - 2), j = 1 + e % (K.jm - 2);
    if (i > K.im - 2) return;
    const int k = K.km - 2;
    if (((i + j + k) & 1) != colour) return;
    sweep_cell(K, geo, src, p, i, j, k);
}

// Neumann planes i = 0, im-1 (all j), then j = 0, jm-1 (all i), then the seam copy -- composed per
// boundary cell from interior values (PressureSolver.h:718-746).
__device__ __forceinline__ double pval_i(const KConst& K, const double* p, int i, int j, int k) {
    const int64_t row = (int64_t)j * K.kp + k;
    if (i == 0) return K.c43 * p[K.plane + row] - K.c13 * p[2 * K.plane + row];
    if (i == K.im - 1) return K.c43 * p[(K.im - 2) * K.plane + row] - K.c13 * p[(K.im - 3) * K.plane + row];
    return p[(int64_t)i * K.plane + row];
}

__device__ __forceinline__ double pval(const KConst& K, const double* p, int i, int j, int k) {
    if (j == 0) return K.c43 * pval_i(K, p, i, 1, k) - K.c13 * pval_i(K, p, i, 2, k);
    if (j == K.jm - 1) return K.c43 * pval_i(K, p, i, K.jm - 2, k) - K.c13 * pval_i(K, p, i, K.jm - 3, k);
    return pval_i(K, p, i, j, k);
}

// blockIdx.z picks the part: 0 the seam column k = km-1 of every (i, j) (row blockIdx.y = i, j along x);
// 1 the radial planes i = 0 and im-1 (row blockIdx.y = side * jm + j, k along x); 2 the polar planes
// j = 0 and jm-1 at interior i (row blockIdx.y = side * (im-2) + i-1, k along x). Every value is formed from
// interior cells only, so the parts are independent; no index needs a division.
__global__ void press_boundary_kernel(const KConst K, double* __restrict__ p) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    const int im = K.im, jm = K.jm, km = K.km;
    int i, j, k;
    if (blockIdx.z == 0) {
        if (y >= im || x >= jm) return;
        i = y; j = x; k = km - 1;
    } else if (blockIdx.z == 1) {
        if (y >= 2 * jm || x >= km - 1) return;
        const bool top = y >= jm;
        i = top ? im - 1 : 0; j = top ? y - jm : y; k = x;
    } else {
        if (y >= 2 * (im - 2) || x >= km - 1) return;
        const bool top = y >= im - 2;
        i = 1 + (top ? y - (im - 2) : y); j = top ? jm - 1 : 0; k = x;
    }
    const int ks = (k == km - 1) ? 0 : k;
    p[((int64_t)i * jm + j) * K.kp + k] = pval(K, p, i, j, ks);
}

__global__ void __launch_bounds__(256) count_nonfinite_kernel(const KConst K, const double* __restrict__ x,
                                                              unsigned long long* __restrict__ count) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    bool bad = false;
    if (k < K.km && j < K.jm) bad = !isfinite(__ldg(x + ((int64_t)i * K.jm + j) * K.kp + k));
    const unsigned m = __ballot_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(count, (unsigned long long)__popc(m));
}

}  // namespace

cudaError_t launch_projection_prep(const KConst& kc, double* const six[6], cudaStream_t s) {
    // the six pointers travel in a small device array owned by the caller (six is device memory)
    const int rows = (kc.im > kc.jm ? kc.im : kc.jm);
    dim3 block(32, 8), grid((kc.km - 1 + 31) / 32, (rows + 7) / 8, 2);
    prep_planes_kernel<<<grid, block, 0, s>>>(kc, six);
    const int n = kc.im * kc.jm * 6;
    prep_seam_kernel<<<(n + 255) / 256, 256, 0, s>>>(kc, six);
    return cudaGetLastError();
}

cudaError_t launch_press_source(const KConst& kc, const ColGeo* geo, const double* su, const double* sv,
                                const double* sw, const double* aux_u, const double* aux_v, const double* aux_w,
                                const double* rhs_u, const double* rhs_v, const double* rhs_w, const double* p,
                                double* src, unsigned long long* nclamp, cudaStream_t s) {
    dim3 block(32, 8), grid((kc.km - 1 + 31) / 32, (kc.jm + 7) / 8, kc.im);
    press_source_kernel<<<grid, block, 0, s>>>(kc, geo, su, sv, sw, aux_u, aux_v, aux_w, rhs_u, rhs_v, rhs_w, p,
                                               src, nclamp);
    return cudaGetLastError();
}

cudaError_t launch_press_sweep(const KConst& kc, const ColGeo* geo, const double* src, double* p, int colour,
                               cudaStream_t s) {
    const int nm = (kc.km - 1 + 1) / 2;
    dim3 block(32, 8), grid((nm + 31) / 32, (kc.jm + 7) / 8, kc.im);
    press_sweep_kernel<<<grid, block, 0, s>>>(kc, geo, src, p, colour);
    if (((kc.km - 1) & 1) && kc.km - 2 > 0 && kc.jm > 2) {
        const int n = (kc.im - 2) * (kc.jm - 2);
        press_sweep_seam_kernel<<<(n + 255) / 256, 256, 0, s>>>(kc, geo, src, p, colour);
    }
    return cudaGetLastError();
}

cudaError_t launch_press_boundary(const KConst& kc, double* p, cudaStream_t s) {
    const int width = std::max(kc.jm, kc.km), rows = std::max(kc.im, 2 * std::max(kc.jm, kc.im - 2));
    press_boundary_kernel<<<dim3((width + 127) / 128, rows, 3), 128, 0, s>>>(kc, p);
    return cudaGetLastError();
}

cudaError_t launch_count_nonfinite(const KConst& kc, const double* x, unsigned long long* count, cudaStream_t s) {
    dim3 block(32, 8), grid((kc.km + 31) / 32, (kc.jm + 7) / 8, kc.im);
    count_nonfinite_kernel<<<grid, block, 0, s>>>(kc, x, count);
    return cudaGetLastError();
}

}  // namespace atsat
