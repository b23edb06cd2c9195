// The two optional passes of PressureSolver<cSaturnModel>::run, FP64, run after each sweep's red-black
// colours (PressureSolver.h:300-316, 502-708, 750-755):
//
// PRESS_LINE: per colour ((j + k) & 1) every (j, k) column is relaxed exactly in r -- a Thomas solve over
// i = 1..im-2 with the theta / phi neighbours lagged and both radial ends folded (p0 = c43 p1 - c13 p2) --
// and after the boundary pass the interior mean of p_dyn is held at its value on entry. One thread per
// column; the forward coefficients go to two scratch fields at the column's own cells. The columns of one
// colour read only the other colour, except across an odd periodic seam where k = 0 and k = km-2 share a
// colour: as in a single thread's visit of the reference's loop, k = km-2 is solved after k = 0 (a second
// launch) and reads its new values.
//
// PRESS_BAROTROPIC: the column residual R(j, k) = sum_i (src - Lc(p)) / sum_i 1/rm^2, its real DFT over
// the N = km-1 meridians (sequential sums, modes below 1e-12 of the row's sum |R| dropped), per mode a
// tridiagonal in theta (mode 0 made consistent, pinned at j = 1, shifted to zero sin-weighted mean), and
// the correction q(j, k) added to every level of the column. The cos / sin tables, the modes' eigenvalue
// factors and the sine tables come from the host, formed with the reference's own expressions.
//
// Weights: lc_num1..3 of ColGeo are the line pass's num1, num2, num3 expression for expression.
#include "dyn_common.cuh"

namespace atsat {
namespace {

__device__ __forceinline__ double ldg(const double* p) { return __ldg(p); }

// PressureSolver.h:506-567 for one column
__device__ void line_column(const KConst& K, const ColGeo* __restrict__ geo, const double* __restrict__ src,
                            double* __restrict__ p, double* __restrict__ cpb, double* __restrict__ dpb, int j, int k) {
    const int64_t P = K.plane, kp = K.kp;
    const int kw = (k == 0) ? K.km - 2 : k - 1;
    const int ke = (k == K.km - 2) ? 0 : k + 1;
    const int lo = 1, hi = K.im - 2;
    const bool fold = hi > lo;
    double cprev = 0.0, dprev = 0.0;
    for (int i = lo; i <= hi; i++) {
        const int64_t c = ((int64_t)i * K.jm + j) * kp + k;
        const ColGeo* g = geo + ((int64_t)i * K.jm + j);
        const double num1 = ldg(&g->lc_num1), num2 = ldg(&g->lc_num2), num3 = ldg(&g->lc_num3);
        const double acc_h = num2 * (p[c + kp] + p[c - kp]) + num3 * (p[c - k + ke] + p[c - k + kw]);
        double a = -num1, b = 2.0 * (num1 + num2 + num3), cc = -num1;
        double d = acc_h - ldg(src + c);
        if (i == lo) {
            if (fold) { b += a * K.c43; cc -= a * K.c13; }
            else d -= a * p[c - P];
        }
        if (i == hi) {
            if (fold) { b += cc * K.c43; a -= cc * K.c13; }
            else d -= cc * p[c + P];
        }
        double cpi, dpi;
        if (i == lo) {
            cpi = cc / b;
            dpi = d / b;
        } else {
            const double dn = b - a * cprev;
            cpi = cc / dn;
            dpi = (d - a * dprev) / dn;
        }
        cpb[c] = cpi;
        dpb[c] = dpi;
        cprev = cpi;
        dprev = dpi;
    }
    double x = dprev;
    {
        const int64_t c = ((int64_t)hi * K.jm + j) * kp + k;
        if (isfinite(x)) p[c] = x;
    }
    for (int i = hi - 1; i >= lo; i--) {
        const int64_t c = ((int64_t)i * K.jm + j) * kp + k;
        x = dpb[c] - cpb[c] * x;
        if (isfinite(x)) p[c] = x;
    }
}

__global__ void __launch_bounds__(128) line_kernel(const KConst K, const ColGeo* __restrict__ geo,
                                                   const double* __restrict__ src, double* __restrict__ p,
                                                   double* __restrict__ cpb, double* __restrict__ dpb, int colour) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y;
    if (j > K.jm - 2) return;
    const int k = 2 * m + ((colour - j) & 1);
    if (k > K.km - 2) return;
    if (k == K.km - 2 && k > 0 && ((K.km - 1) & 1)) return;     // after its seam partner k = 0
    line_column(K, geo, src, p, cpb, dpb, j, k);
}

__global__ void line_seam_kernel(const KConst K, const ColGeo* __restrict__ geo, const double* __restrict__ src,
                                 double* __restrict__ p, double* __restrict__ cpb, double* __restrict__ dpb,
                                 int colour) {
    const int j = 1 + blockIdx.x * blockDim.x + threadIdx.x;
    if (j > K.jm - 2) return;
    const int k = K.km - 2;
    if (((j + k) & 1) != colour) return;
    line_column(K, geo, src, p, cpb, dpb, j, k);
}

// ---- interior mean (PressureSolver.h:310-316): per level partial sums over row chunks, then in order ----
constexpr int IM_CHUNKS = 8;

__global__ void __launch_bounds__(128) imean_partial_kernel(const KConst K, const double* __restrict__ p,
                                                            double* __restrict__ partial) {
    const int i = 1 + blockIdx.x, chunk = blockIdx.y;
    const int nj = K.jm - 2;
    const int j0 = 1 + (int)((int64_t)nj * chunk / IM_CHUNKS), j1 = 1 + (int)((int64_t)nj * (chunk + 1) / IM_CHUNKS);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double s = 0.0;
    for (int j = j0 + warp; j < j1; j += 4) {
        const double* row = p + ((int64_t)i * K.jm + j) * K.kp;
        for (int k = lane; k <= K.km - 2; k += 32) s += ldg(row + k);
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __shared__ double ws[4];
    if (lane == 0) ws[warp] = s;
    __syncthreads();
    if (threadIdx.x == 0) partial[(int64_t)(i - 1) * IM_CHUNKS + chunk] = ((ws[0] + ws[1]) + ws[2]) + ws[3];
}

__global__ void imean_final_kernel(const double* __restrict__ partial, int n, double count, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    for (int q = 0; q < n; q++) s += partial[q];
    *out = s / count;
}

// p -= mean_now - mean_entry on every cell (PressureSolver.h:750-755)
__global__ void __launch_bounds__(256) mean_shift_kernel(const KConst K, double* __restrict__ p,
                                                         const double* __restrict__ mean) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= K.km || j >= K.jm) return;
    const double shift = mean[1] - mean[0];
    p[((int64_t)i * K.jm + j) * K.kp + k] -= shift;
}

// ---- PRESS_BAROTROPIC (PressureSolver.h:573-708) ----
// the column residual of PressureSolver.h:581-604, end rows read as the boundary pass sets them
__device__ __forceinline__ double pb_i(const KConst& K, const double* p, int i, int j, int k) {
    const int64_t row = (int64_t)j * K.kp + k;
    if (i == 0) return K.c43 * p[K.plane + row] - K.c13 * p[2 * K.plane + row];
    if (i == K.im - 1) return K.c43 * p[(K.im - 2) * K.plane + row] - K.c13 * p[(K.im - 3) * K.plane + row];
    return p[(int64_t)i * K.plane + row];
}
__device__ __forceinline__ double pb_j(const KConst& K, const double* p, int i, int j, int k) {
    const int64_t base = (int64_t)i * K.plane + k;
    if (j == 0) return K.c43 * p[base + K.kp] - K.c13 * p[base + 2 * K.kp];
    if (j == K.jm - 1) return K.c43 * p[base + (int64_t)(K.jm - 2) * K.kp] - K.c13 * p[base + (int64_t)(K.jm - 3) * K.kp];
    return p[base + (int64_t)j * K.kp];
}

__global__ void __launch_bounds__(128) baro_resid_kernel(const KConst K, const ColGeo* __restrict__ geo,
                                                         const double* __restrict__ src, const double* __restrict__ p,
                                                         double A2, double* __restrict__ R) {
    const int N = K.km - 1;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = 1 + blockIdx.y;
    if (k >= N || j > K.jm - 2) return;
    const int kw = (k == 0) ? N - 1 : k - 1;
    const int ke = (k == N - 1) ? 0 : k + 1;
    double s = 0.0;
    for (int i = 1; i < K.im - 1; i++) {
        const ColGeo* g = geo + ((int64_t)i * K.jm + j);
        const int64_t c = ((int64_t)i * K.jm + j) * K.kp + k;
        const double p0 = p[c];
        const double lc = ldg(&g->lc_num1) * (pb_i(K, p, i + 1, j, k) + pb_i(K, p, i - 1, j, k) - 2.0 * p0)
                        + ldg(&g->lc_num2) * (pb_j(K, p, i, j + 1, k) + pb_j(K, p, i, j - 1, k) - 2.0 * p0)
                        + ldg(&g->lc_num3) * (p[c - k + ke] + p[c - k + kw] - 2.0 * p0);
        s += ldg(src + c) - lc;
    }
    R[(int64_t)(j - 1) * N + k] = s / A2;
}

// sum_k |R(j, k)| per row, in order
__global__ void baro_rowabs_kernel(int J, int N, const double* __restrict__ R, double* __restrict__ ra) {
    const int jj = blockIdx.x * blockDim.x + threadIdx.x;
    if (jj >= J) return;
    double s = 0.0;
    for (int k = 0; k < N; k++) s += fabs(R[(int64_t)jj * N + k]);
    ra[jj] = s;
}

// Ac[m][j] = sum_k R cos(2 pi m k / N), As likewise with sin; one thread per (mode, row), sums in k order
__global__ void __launch_bounds__(128) baro_dft_kernel(int J, int N, int NM, const double* __restrict__ R,
                                                       const double* __restrict__ ct, const double* __restrict__ st,
                                                       const double* __restrict__ ra, double* __restrict__ Ac,
                                                       double* __restrict__ As) {
    const int jj = blockIdx.x * blockDim.x + threadIdx.x;
    const int mm = blockIdx.y;
    if (jj >= J || mm > NM) return;
    const double* r_ = R + (int64_t)jj * N;
    const double* c_ = ct + (int64_t)mm * N;
    const double* s_ = st + (int64_t)mm * N;
    double sc = 0.0, ss = 0.0;
    for (int k = 0; k < N; k++) {
        const double r = ldg(r_ + k);
        sc += r * ldg(c_ + k);
        ss += r * ldg(s_ + k);
    }
    if (mm > 0) {
        const double tol = 1.0e-12 * ra[jj];
        if (fabs(sc) < tol) sc = 0.0;
        if (fabs(ss) < tol) ss = 0.0;
    }
    Ac[(int64_t)mm * J + jj] = sc;
    As[(int64_t)mm * J + jj] = ss;
}

struct BaroModes {
    int J, N, NM;
    double e, c43, c13;
    const double* lam;         // NM+1: 4 sin^2(pi m / N) / dphi^2
    const double* sinthe;      // jm: the solver's guarded sine table
    const double* abs_sin;     // J: |sin(the_z[jj+1])|
    double *Ac, *As, *cp, *dp; // cp, dp: (NM+1) x J scratch
};

// PressureSolver.h:638-680: one thread per mode, both parts
__global__ void baro_modes_kernel(const BaroModes B) {
    const int mm = blockIdx.x * blockDim.x + threadIdx.x;
    if (mm > B.NM) return;
    const int J = B.J;
    const double e = B.e, lam = B.lam[mm];
    auto coef = [&](int jj, double& a, double& b, double& c) {
        const double s_ = B.sinthe[jj + 1];
        a = e;
        c = e;
        b = -2.0 * e - lam / (s_ * s_);
        if (jj == 0) { a = 0.0; b += B.c43 * e; c -= B.c13 * e; }
        if (jj == J - 1) { c = 0.0; b += B.c43 * e; a -= B.c13 * e; }
    };
    double* cp = B.cp + (int64_t)mm * J;
    double* dp = B.dp + (int64_t)mm * J;
    for (int part = 0; part < 2; part++) {
        if (mm == 0 && part == 1) continue;
        if (2 * mm == B.N && part == 1) continue;
        double* d = (part == 0 ? B.Ac : B.As) + (int64_t)mm * J;
        double a0, b0, c0;
        coef(0, a0, b0, c0);
        if (mm == 0) {
            double yr = 0.0, ys = 0.0;
            for (int jj = 0; jj < J; jj++) {
                const double y = (jj == 0 || jj == J - 1) ? 1.5 : 1.0;
                yr += y * d[jj];
                ys += y * B.abs_sin[jj];
            }
            for (int jj = 0; jj < J; jj++) d[jj] -= yr / ys * B.abs_sin[jj];
            b0 = 1.0;
            c0 = 0.0;
            d[0] = 0.0;
        }
        cp[0] = c0 / b0;
        dp[0] = d[0] / b0;
        for (int jj = 1; jj < J; jj++) {
            double a, b, c;
            coef(jj, a, b, c);
            const double dn = b - a * cp[jj - 1];
            cp[jj] = c / dn;
            dp[jj] = (d[jj] - a * dp[jj - 1]) / dn;
        }
        d[J - 1] = dp[J - 1];
        for (int jj = J - 2; jj >= 0; jj--) d[jj] = dp[jj] - cp[jj] * d[jj + 1];
        if (mm == 0) {
            double sq = 0.0, sw = 0.0;
            for (int jj = 0; jj < J; jj++) {
                sq += B.abs_sin[jj] * d[jj];
                sw += B.abs_sin[jj];
            }
            for (int jj = 0; jj < J; jj++) d[jj] -= sq / sw;
        }
    }
}

// PressureSolver.h:684-697: q(j, k) back in phi, added to every level of the column
__global__ void __launch_bounds__(128) baro_apply_kernel(const KConst K, int J, int N, int NM,
                                                         const double* __restrict__ Ac, const double* __restrict__ As,
                                                         const double* __restrict__ ct, const double* __restrict__ st,
                                                         double* __restrict__ p) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int jj = blockIdx.y;
    if (k >= N || jj >= J) return;
    double q = 0.0;
    for (int mm = 0; mm <= NM; mm++) {
        const bool real = (mm == 0 || 2 * mm == N);
        const double w_ = real ? 1.0 : 2.0;
        q += w_ * (ldg(Ac + (int64_t)mm * J + jj) * ldg(ct + (int64_t)mm * N + k)
                   + (real ? 0.0 : ldg(As + (int64_t)mm * J + jj) * ldg(st + (int64_t)mm * N + k)));
    }
    q /= N;
    for (int i = 0; i < K.im; i++) p[((int64_t)i * K.jm + (jj + 1)) * K.kp + k] += q;
}

}  // namespace

cudaError_t launch_line_pass(const KConst& kc, const ColGeo* geo, const double* src, double* p, double* cpb,
                             double* dpb, int colour, cudaStream_t s, int* launches) {
    const int nm = (kc.km - 1 + 1) / 2 + 1;
    line_kernel<<<dim3((nm + 127) / 128, kc.jm - 2), 128, 0, s>>>(kc, geo, src, p, cpb, dpb, colour);
    *launches += 1;
    if (((kc.km - 1) & 1) && kc.km - 2 > 0) {
        line_seam_kernel<<<(kc.jm - 2 + 127) / 128, 128, 0, s>>>(kc, geo, src, p, cpb, dpb, colour);
        *launches += 1;
    }
    return cudaGetLastError();
}

// the interior mean of p into *out; partial holds (im-2) * IM_CHUNKS doubles
cudaError_t launch_interior_mean(const KConst& kc, const double* p, double* partial, double* out, cudaStream_t s,
                                 int* launches) {
    const int n = (kc.im - 2) * IM_CHUNKS;
    const double count = (double)((int64_t)(kc.im - 2) * (kc.jm - 2) * (kc.km - 1));
    imean_partial_kernel<<<dim3(kc.im - 2, IM_CHUNKS), 128, 0, s>>>(kc, p, partial);
    imean_final_kernel<<<1, 32, 0, s>>>(partial, n, count, out);
    *launches += 2;
    return cudaGetLastError();
}

int interior_mean_partials(const KConst& kc) { return (kc.im - 2) * IM_CHUNKS; }

cudaError_t launch_mean_shift(const KConst& kc, double* p, const double* mean, cudaStream_t s) {
    mean_shift_kernel<<<dim3((kc.km + 31) / 32, (kc.jm + 7) / 8, kc.im), dim3(32, 8), 0, s>>>(kc, p, mean);
    return cudaGetLastError();
}

cudaError_t launch_barotropic(const KConst& kc, const ColGeo* geo, const double* src, double* p, const BaroTables& T,
                              cudaStream_t s, int* launches) {
    const int N = kc.km - 1, J = kc.jm - 2, NM = N / 2;
    baro_resid_kernel<<<dim3((N + 127) / 128, J), 128, 0, s>>>(kc, geo, src, p, T.A2, T.R);
    baro_rowabs_kernel<<<(J + 127) / 128, 128, 0, s>>>(J, N, T.R, T.ra);
    baro_dft_kernel<<<dim3((J + 127) / 128, NM + 1), 128, 0, s>>>(J, N, NM, T.R, T.ct, T.st, T.ra, T.Ac, T.As);
    BaroModes B{J, N, NM, kc.inv_dthe2, kc.c43, kc.c13, T.lam, T.sinthe, T.abs_sin, T.Ac, T.As, T.cp, T.dp};
    baro_modes_kernel<<<(NM + 1 + 63) / 64, 64, 0, s>>>(B);
    baro_apply_kernel<<<dim3((N + 127) / 128, J), 128, 0, s>>>(kc, J, N, NM, T.Ac, T.As, T.ct, T.st, p);
    *launches += 5;
    return cudaGetLastError();
}

}  // namespace atsat
