// Device glue for resident multi-iteration runs: the boundary conditions BC_Sat applies between
// RK4 steps (planet/BoundaryConditions.h:150-518 with BC_Sat.cpp:61-179), on the fields of the dycore.
//
// Each of the three routines only moves data along one grid direction, so each is one kernel whose
// threads own disjoint (line, field) pairs: bcTheta works along j for every (i, k), bcPhi along k for
// every (i, j), bcRadius (with the rigid-wall u, the top taper and the species lid / wall copies) along i
// for every (j, k). They run in the order cSaturnModel::Run calls them (cSaturnModel.cpp:1091-1093).
//
// In a resident mixed-precision run the prognostic fields also have FP32 copies (and w a second FP32
// word) that the next step's stencils read; every value written here is written to them too.
#include "dyn_common.cuh"

namespace atsat {

namespace {

struct BCArgs {
    double* f[ATSAT_NFIELDS];
    float* s32[ATSAT_NFIELDS];     // FP32 copies (null: none)
    float* wlo;                    // second FP32 word of w (null: none)
    int radius[20];                // bc_fields_radius() restricted to the dycore; bcPhi uses the same list
    int theta_extrap[17];
    int theta_zero[3];
    int turb[3];
    double turb_floor[3];
    int species[11];
    int turb_on;
    double r_mix;
    int radius_form, bottom_form, pole_form, pole_fill, lid_u, top_taper, lid_copy, wall_copy, local_rho;
};

__device__ __forceinline__ double form3(int form, double a, double b, double c, double c43, double c13) {
    const int f = (form == 0) ? 3 : form;
    if (f == 1) return a;
    if (f == 2) return c43 * a - c13 * b;
    return c - 3.0 * b + 3.0 * a;
}

__device__ __forceinline__ double smax(double a, double b) { return (a < b) ? b : a; }

__device__ __forceinline__ double get(const BCArgs& A, int id, int64_t c) { return A.f[id][c]; }

__device__ __forceinline__ void put(const BCArgs& A, int id, int64_t c, double x) {
    A.f[id][c] = x;
    if (A.s32[id]) {
        // the FP32 copy (and w's low word) by the integer-pipe conversions: GB300 runs the hardware
        // float <-> double conversions at its FP64 rate
        const float hi = d2f(x);
        A.s32[id][c] = hi;
        if (id == ATSAT_F_W && A.wlo) A.wlo[c] = d2f(x - f2d(hi));
    }
}

// Each kernel runs one thread per (line, field): a field's boundary steps depend only on that field (and
// rho_mix for the wall copy), so the fields of a line are independent and go to separate threads.
// blockIdx.z is the field's task: an index into the kernel's field lists.

__global__ void bc_theta_kernel(const KConst K, const BCArgs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = 1 + blockIdx.y;
    const int task = blockIdx.z;                      // 0..16 extrapolated, 17..19 zeroed, 20..22 turbulence
    if (k > K.km - 2 || i > K.im - 2) return;
    if (task >= 20 && !A.turb_on) return;
    const int64_t kp = K.kp, jm = K.jm;
    const int64_t base = (int64_t)i * K.plane + k;     // (i, 0, k)
    auto at = [&](int j) { return base + (int64_t)j * kp; };
    const int jf = 2;
    if (task < 17) {
        const int F = A.theta_extrap[task];
        if (A.pole_fill) {
            put(A, F, at(1), get(A, F, at(jf)));
            put(A, F, at(jm - 2), get(A, F, at(jm - 1 - jf)));
        }
        put(A, F, at(0), form3(A.pole_form, get(A, F, at(1)), get(A, F, at(2)), get(A, F, at(3)), K.c43, K.c13));
        put(A, F, at(jm - 1), form3(A.pole_form, get(A, F, at(jm - 2)), get(A, F, at(jm - 3)), get(A, F, at(jm - 4)),
                                    K.c43, K.c13));
    } else if (task < 20) {
        const int F = A.theta_zero[task - 17];
        if (A.pole_fill) {
            const double ramp = 1.0 / 2.0;
            put(A, F, at(1), ramp * get(A, F, at(jf)));
            put(A, F, at(jm - 2), ramp * get(A, F, at(jm - 1 - jf)));
        }
        put(A, F, at(0), 0.0);
        put(A, F, at(jm - 1), 0.0);
    } else {
        const int q = task - 20;
        const int F = A.turb[q];
        if (A.pole_fill) {
            put(A, F, at(1), smax(A.turb_floor[q], get(A, F, at(jf))));
            put(A, F, at(jm - 2), smax(A.turb_floor[q], get(A, F, at(jm - 1 - jf))));
        }
        put(A, F, at(0), smax(A.turb_floor[q], K.c43 * get(A, F, at(1)) - K.c13 * get(A, F, at(2))));
        put(A, F, at(jm - 1), smax(A.turb_floor[q], K.c43 * get(A, F, at(jm - 2)) - K.c13 * get(A, F, at(jm - 3))));
    }
}

__global__ void bc_phi_kernel(const KConst K, const BCArgs A) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;     // i * jm + j
    const int task = blockIdx.z;                                // 0..19 copied, 20..22 turbulence
    if (row >= K.im * K.jm) return;
    const int64_t c0 = (int64_t)row * K.kp, c1 = c0 + K.km - 1;
    if (task < 20) {
        put(A, A.radius[task], c1, get(A, A.radius[task], c0));
    } else if (A.turb_on) {
        const int q = task - 20;
        const int F = A.turb[q];
        const double x = smax(A.turb_floor[q], get(A, F, c0));
        put(A, F, c0, x);
        put(A, F, c1, x);
    }
}

__global__ void bc_radius_kernel(const KConst K, const BCArgs A) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    const int task = blockIdx.z;                                // 0..19 radius fields, 20..22 turbulence
    if (k >= K.km || j >= K.jm) return;
    const int64_t P = K.plane;
    const int64_t c0 = (int64_t)j * K.kp + k;                  // (0, j, k)
    const int im = K.im;
    auto at = [&](int i) { return c0 + (int64_t)i * P; };
    const bool inner = j >= 1 && j <= K.jm - 2 && k <= K.km - 2;
    if (task >= 20) {
        if (!A.turb_on || !inner) return;
        const int q = task - 20;
        const int F = A.turb[q];
        const double a1 = get(A, F, at(1)), a2 = get(A, F, at(2)), b2 = get(A, F, at(im - 2)),
                     b3 = get(A, F, at(im - 3));
        put(A, F, at(0), smax(A.turb_floor[q], K.c43 * a1 - K.c13 * a2));
        put(A, F, at(im - 1), smax(A.turb_floor[q], K.c43 * b2 - K.c13 * b3));
        return;
    }
    const int F = A.radius[task];
    if (im >= 8) {
        // The same steps with every load issued before the first store (one memory round trip instead of
        // several). With im >= 8 the planes read (1..3 and im-4..im-2) are disjoint from the extrapolated
        // walls (0 and im-1); the taper (v, w only) reads planes nothing before it wrote; the species
        // copies read planes 1 and im-2, which only the taper writes, and never in a species field.
        bool species = false;
        for (int q = 0; q < 11; q++) species = species || (A.species[q] == F);
        const bool copies = species && (A.lid_copy != 0 || A.wall_copy != 0);
        const bool taper = (F == ATSAT_F_V || F == ATSAT_F_W) && A.top_taper;
        const bool rho = copies && A.wall_copy == 2 && A.local_rho;
        if (!inner && !taper && !copies && !(F == ATSAT_F_U && A.lid_u)) return;
        const double x1 = get(A, F, at(1)), x2 = get(A, F, at(2)), x3 = get(A, F, at(3));
        const double y2 = get(A, F, at(im - 2)), y3 = get(A, F, at(im - 3)), y4 = get(A, F, at(im - 4));
        const double ra = rho ? get(A, ATSAT_F_RHO_MIX, at(0)) : 0.0;
        const double rb = rho ? get(A, ATSAT_F_RHO_MIX, at(1)) : 0.0;
        double w0 = 0.0, w1 = 0.0;                        // planes 0 and im-1
        bool s0 = false, s1 = false;
        if (inner) {
            const int fb = (A.bottom_form != 0 && F != ATSAT_F_U) ? A.bottom_form : A.radius_form;
            w0 = form3(fb, x1, x2, x3, K.c43, K.c13);
            w1 = form3(A.radius_form, y2, y3, y4, K.c43, K.c13);
            s0 = s1 = true;
        }
        if (F == ATSAT_F_U && A.lid_u) { w0 = 0.0; w1 = 0.0; s0 = s1 = true; }
        if (taper) {
            w1 = 0.0;
            s1 = true;
            put(A, F, at(im - 2), A.top_taper == 2 ? (1.0 / 3.0) * y4 : y2 * (1.0 / 3.0));
            put(A, F, at(im - 3), A.top_taper == 2 ? (2.0 / 3.0) * y4 : y3 * (2.0 / 3.0));
        }
        if (copies) {
            double fr = 1.0;
            if (A.wall_copy == 2) {
                double r0 = A.r_mix, r1 = A.r_mix;
                if (A.local_rho) {
                    r0 = (ra > 0.0 && isfinite(ra)) ? ra : A.r_mix;
                    r1 = (rb > 0.0 && isfinite(rb)) ? rb : A.r_mix;
                }
                fr = r0 / r1;
            }
            if (A.lid_copy != 0) { w1 = y2; s1 = true; }
            if (A.wall_copy != 0) { w0 = x1 * fr; s0 = true; }
        }
        if (s0) put(A, F, at(0), w0);
        if (s1) put(A, F, at(im - 1), w1);
        return;
    }
    if (inner) {
        const int fb = (A.bottom_form != 0 && F != ATSAT_F_U) ? A.bottom_form : A.radius_form;
        put(A, F, at(0), form3(fb, get(A, F, at(1)), get(A, F, at(2)), get(A, F, at(3)), K.c43, K.c13));
        put(A, F, at(im - 1), form3(A.radius_form, get(A, F, at(im - 2)), get(A, F, at(im - 3)),
                                    get(A, F, at(im - 4)), K.c43, K.c13));
    }
    if (F == ATSAT_F_U && A.lid_u) { put(A, ATSAT_F_U, at(0), 0.0); put(A, ATSAT_F_U, at(im - 1), 0.0); }
    if ((F == ATSAT_F_V || F == ATSAT_F_W) && A.top_taper) {
        const int iml = im - 1;
        put(A, F, at(iml), 0.0);
        if (A.top_taper == 2) {
            put(A, F, at(iml - 1), (1.0 / 3.0) * get(A, F, at(iml - 3)));
            put(A, F, at(iml - 2), (2.0 / 3.0) * get(A, F, at(iml - 3)));
        } else {
            put(A, F, at(iml - 1), get(A, F, at(iml - 1)) * (1.0 / 3.0));
            put(A, F, at(iml - 2), get(A, F, at(iml - 2)) * (2.0 / 3.0));
        }
    }
    if (A.lid_copy == 0 && A.wall_copy == 0) return;
    bool species = false;
    for (int q = 0; q < 11; q++) species = species || (A.species[q] == F);
    if (!species) return;
    double fr = 1.0;
    if (A.wall_copy == 2) {
        double r0 = A.r_mix, r1 = A.r_mix;
        if (A.local_rho) {
            const double a = get(A, ATSAT_F_RHO_MIX, at(0)), b = get(A, ATSAT_F_RHO_MIX, at(1));
            r0 = (a > 0.0 && isfinite(a)) ? a : A.r_mix;
            r1 = (b > 0.0 && isfinite(b)) ? b : A.r_mix;
        }
        fr = r0 / r1;
    }
    if (A.lid_copy != 0) put(A, F, at(im - 1), get(A, F, at(im - 2)));
    if (A.wall_copy != 0) put(A, F, at(0), get(A, F, at(1)) * fr);
}

// dst[r * dst_pitch + k] = src[r * src_pitch + k] for k < width: host arrays are contiguous rows of km
// values, the device layout pads them to kp, so host copies go through a contiguous staging field
__global__ void repitch_kernel(double* __restrict__ dst, int dst_pitch, const double* __restrict__ src, int src_pitch,
                               int width, int64_t rows) {
    const int64_t r = (int64_t)blockIdx.y * gridDim.z + blockIdx.z;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows || k >= width) return;
    dst[r * dst_pitch + k] = src[r * src_pitch + k];
}

// ---- AtomUtils::damp_wiggles (lib/Utils.cpp:229-322), no surface mask: one axis of the 1-2-1 filter,
// f = t + coeff (t[-1] - 2 t + t[+1]) with t the field's copy. axis 0: k, periodic over the km-1 distinct
// meridians with k = km-1 their copy (seam), else over all km; axis 1: j, clamped at the poles; axis 2: i,
// clamped at the walls.
__global__ void __launch_bounds__(256) damp_axis_kernel(const KConst K, const double* __restrict__ t,
                                                        double* __restrict__ f, double coeff, int axis, int seam) {
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int i = blockIdx.z;
    if (k >= K.km || j >= K.jm) return;
    const int64_t row = ((int64_t)i * K.jm + j) * K.kp;
    const int64_t c = row + k;
    const double t0 = t[c];
    double a, b;
    if (axis == 0) {
        if (seam) {
            if (k == K.km - 1) return;                      // the copy, written with k = 0
            a = t[row + ((k == 0) ? K.km - 2 : k - 1)];
            b = t[row + ((k == K.km - 2) ? 0 : k + 1)];
        } else {
            a = t[row + (k - 1 + K.km) % K.km];
            b = t[row + (k + 1) % K.km];
        }
    } else if (axis == 1) {
        a = t[c + (int64_t)((j > 0 ? j - 1 : 0) - j) * K.kp];
        b = t[c + (int64_t)((j < K.jm - 1 ? j + 1 : K.jm - 1) - j) * K.kp];
    } else {
        a = t[c + (int64_t)((i > 0 ? i - 1 : 0) - i) * K.plane];
        b = t[c + (int64_t)((i < K.im - 1 ? i + 1 : K.im - 1) - i) * K.plane];
    }
    const double v = t0 + coeff * (a - 2.0 * t0 + b);
    f[c] = v;
    if (axis == 0 && seam && k == 0) f[row + K.km - 1] = v;
}

// ---- cSaturnModel::clampNegativeSpecies (FileIO_Sat.cpp:716-772) ----
// !(v >= 0) (NaN included) becomes 0 in the FP64 field and, when given, its FP32 copy. The finite amounts
// clipped and the cells, in the whole field and on the radial planes i = 0, im-1, form the budget:
// added[11], added_bnd[11] (doubles), then cells[11], cells_bnd[11] (64-bit counts). An evolved state has
// undershoots in most cells of some species, so the sums are two-level and deterministic: each of CL_NB
// blocks per species walks a contiguous range of the field's cells and writes its four sums to `partial`;
// one small kernel adds the blocks' sums in block order to the budget (no atomics on the 22 totals).
constexpr int CL_NB = 128, CL_THREADS = 256;

struct ClampArgs {
    double* f[11];
    float* s32[11];
    double* added;
    unsigned long long* cells;
    double* partial;               // [11][CL_NB][4]
};

__global__ void __launch_bounds__(CL_THREADS) clamp_species_kernel(const KConst K, const ClampArgs A) {
    const int q = blockIdx.y;
    const int64_t n = (int64_t)K.im * K.jm * K.km;
    const int64_t per = (n + CL_NB - 1) / CL_NB;
    const int64_t e0 = per * blockIdx.x, e1 = e0 + per < n ? e0 + per : n;
    const int64_t rb_lo = K.jm, rb_hi = (int64_t)(K.im - 1) * K.jm;   // rows r = i jm + j of i = 0 and im-1
    const bool small = n < (1 << 24);                                  // the FP32 row estimate is exact
    const float inv_km = 1.0f / (float)K.km;
    double* f = A.f[q];
    float* s32 = A.s32[q];
    double s[4] = {0.0, 0.0, 0.0, 0.0};                               // added, added_bnd, cells, cells_bnd
    auto cell = [&](int64_t e, int64_t& r) -> int64_t {                // (row, device index) of flat cell e
        int64_t k;
        if (small) {
            int ri = (int)((float)e * inv_km);
            int ki = (int)e - ri * K.km;
            if (ki < 0) { ri--; ki += K.km; }
            else if (ki >= K.km) { ri++; ki -= K.km; }
            r = ri;
            k = ki;
        } else {
            r = e / K.km;
            k = e - r * K.km;
        }
        return r * K.kp + k;
    };
    // four cells per thread and pass: their loads are in flight together
    constexpr int U = 4;
    for (int64_t e0t = e0 + threadIdx.x; e0t < e1; e0t += (int64_t)CL_THREADS * U) {
        int64_t rr[U], cc[U];
        double vv[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const int64_t e = e0t + (int64_t)u * CL_THREADS;
            cc[u] = e < e1 ? cell(e, rr[u]) : -1;
            vv[u] = cc[u] >= 0 ? f[cc[u]] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
            const double v = vv[u];
            if (cc[u] < 0 || v >= 0.0) continue;
            f[cc[u]] = 0.0;
            if (s32) s32[cc[u]] = 0.0f;
            if (isfinite(v)) {
                s[0] -= v;
                s[2] += 1.0;
                if (rr[u] < rb_lo || rr[u] >= rb_hi) { s[1] -= v; s[3] += 1.0; }
            }
        }
    }
    __shared__ double red[CL_THREADS / 32][4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int m = 0; m < 4; m++) {
        for (int o = 16; o > 0; o >>= 1) s[m] += __shfl_down_sync(0xffffffffu, s[m], o);
        if (lane == 0) red[warp][m] = s[m];
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0.0;
        for (int w = 0; w < CL_THREADS / 32; w++) t += red[w][threadIdx.x];
        A.partial[((int64_t)q * CL_NB + blockIdx.x) * 4 + threadIdx.x] = t;
    }
}

// one thread per (species, sum): the blocks' partial sums added in block order
__global__ void clamp_budget_kernel(const ClampArgs A) {
    const int q = threadIdx.x >> 2, m = threadIdx.x & 3;
    if (q >= 11) return;
    double t = 0.0;
#pragma unroll 8
    for (int b = 0; b < CL_NB; b++) t += A.partial[((int64_t)q * CL_NB + b) * 4 + m];
    if (m == 0) A.added[q] += t;
    else if (m == 1) A.added[11 + q] += t;
    else if (m == 2) A.cells[q] += (unsigned long long)t;
    else A.cells[11 + q] += (unsigned long long)t;
}

// cSaturnModel::restart_state_is_clean (FileIO_Sat.cpp:676-695): cells whose exponent bits are all ones
struct NonfiniteArgs {
    const double* f[40];
    int n;
};
__global__ void __launch_bounds__(256) nonfinite_fields_kernel(const KConst K, const NonfiniteArgs A,
                                                               unsigned long long* count) {
    const int k = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
    const int q = blockIdx.z / K.im, i = blockIdx.z % K.im;
    bool bad = false;
    if (k < K.km && j < K.jm && q < A.n) {
        const uint64_t b = (uint64_t)__double_as_longlong(A.f[q][((int64_t)i * K.jm + j) * K.kp + k]);
        bad = (b & 0x7FF0000000000000ull) == 0x7FF0000000000000ull;
    }
    const unsigned m = __ballot_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(count, (unsigned long long)__popc(m));
}

}  // namespace

cudaError_t launch_nonfinite_fields(const KConst& kc, const double* const* f, int n, unsigned long long* count,
                                    cudaStream_t s) {
    if (n > 40) return cudaErrorInvalidValue;
    NonfiniteArgs A{};
    for (int q = 0; q < n; q++) A.f[q] = f[q];
    A.n = n;
    nonfinite_fields_kernel<<<dim3((kc.km + 31) / 32, (kc.jm + 7) / 8, kc.im * n), dim3(32, 8), 0, s>>>(kc, A, count);
    return cudaGetLastError();
}

cudaError_t launch_damp_axis(const KConst& kc, const double* tmp, double* f, double coeff, int axis, int seam,
                             cudaStream_t s) {
    damp_axis_kernel<<<dim3((kc.km + 31) / 32, (kc.jm + 7) / 8, kc.im), dim3(32, 8), 0, s>>>(kc, tmp, f, coeff, axis,
                                                                                           seam);
    return cudaGetLastError();
}

size_t clamp_partial_doubles() { return (size_t)11 * CL_NB * 4; }

cudaError_t launch_clamp_species(const KConst& kc, double* const f[11], float* const s32[11], double* added,
                                 unsigned long long* cells, double* partial, cudaStream_t s) {
    ClampArgs A{};
    for (int q = 0; q < 11; q++) {
        A.f[q] = f[q];
        A.s32[q] = s32 ? s32[q] : nullptr;
    }
    A.added = added;
    A.cells = cells;
    A.partial = partial;
    clamp_species_kernel<<<dim3(CL_NB, 11), CL_THREADS, 0, s>>>(kc, A);
    clamp_budget_kernel<<<1, 64, 0, s>>>(A);
    return cudaGetLastError();
}

cudaError_t launch_repitch(double* dst, int dst_pitch, const double* src, int src_pitch, int width, int64_t rows,
                           cudaStream_t s) {
    // rows split over grid y and z (each below 65536)
    const int64_t gz = rows < 1024 ? rows : 1024;
    const int64_t gy = (rows + gz - 1) / gz;
    repitch_kernel<<<dim3((width + 127) / 128, (unsigned)gy, (unsigned)gz), 128, 0, s>>>(dst, dst_pitch, src, src_pitch,
                                                                                        width, rows);
    return cudaGetLastError();
}

cudaError_t launch_boundary_conditions(const KConst& kc, const atsat_dyn_params& p, double* const* f,
                                       float* const* s32, float* wlo, cudaStream_t s) {
    BCArgs A{};
    for (int q = 0; q < ATSAT_NFIELDS; q++) {
        A.f[q] = f[q];
        A.s32[q] = s32 ? s32[q] : nullptr;
    }
    A.wlo = wlo;
    const int radius[20] = {ATSAT_F_T, ATSAT_F_U, ATSAT_F_V, ATSAT_F_W, ATSAT_F_CH4, ATSAT_F_CH4_CLOUD,
                            ATSAT_F_CH4_ICE, ATSAT_F_H2O, ATSAT_F_H2O_CLOUD, ATSAT_F_H2O_ICE, ATSAT_F_H2S,
                            ATSAT_F_NH3, ATSAT_F_NH3_CLOUD, ATSAT_F_NH3_ICE, ATSAT_F_NH4SH,
                            ATSAT_F_MASSFLUX_H2S, ATSAT_F_MASSFLUX_NH3, ATSAT_F_MASSFLUX_NH4SH,
                            ATSAT_F_FLUXLIM_NH4SH, ATSAT_F_THERMALMASSFLUX};
    const int theta_extrap[17] = {ATSAT_F_T, ATSAT_F_U, ATSAT_F_CH4, ATSAT_F_CH4_CLOUD, ATSAT_F_CH4_ICE,
                                  ATSAT_F_H2O, ATSAT_F_H2O_CLOUD, ATSAT_F_H2O_ICE, ATSAT_F_H2S, ATSAT_F_NH3,
                                  ATSAT_F_NH3_CLOUD, ATSAT_F_NH3_ICE, ATSAT_F_NH4SH, ATSAT_F_MASSFLUX_H2S,
                                  ATSAT_F_MASSFLUX_NH3, ATSAT_F_MASSFLUX_NH4SH, ATSAT_F_THERMALMASSFLUX};
    const int theta_zero[3] = {ATSAT_F_V, ATSAT_F_W, ATSAT_F_FLUXLIM_NH4SH};
    const int turb[3] = {ATSAT_F_TKE, ATSAT_F_DIS, ATSAT_F_NUE};
    const int species[11] = {ATSAT_F_H2O, ATSAT_F_H2O_CLOUD, ATSAT_F_H2O_ICE, ATSAT_F_H2S, ATSAT_F_NH3,
                             ATSAT_F_NH3_CLOUD, ATSAT_F_NH3_ICE, ATSAT_F_CH4, ATSAT_F_CH4_CLOUD,
                             ATSAT_F_CH4_ICE, ATSAT_F_NH4SH};
    for (int q = 0; q < 20; q++) A.radius[q] = radius[q];
    for (int q = 0; q < 17; q++) A.theta_extrap[q] = theta_extrap[q];
    for (int q = 0; q < 3; q++) { A.theta_zero[q] = theta_zero[q]; A.turb[q] = turb[q]; }
    for (int q = 0; q < 11; q++) A.species[q] = species[q];
    A.turb_floor[0] = 0.0;
    A.turb_floor[1] = 1.0e-10;
    A.turb_floor[2] = 0.0;
    A.turb_on = p.turb_active;
    A.r_mix = p.r_mix;
    A.radius_form = p.bc_radius_form;
    A.bottom_form = p.bc_bottom_form;
    A.pole_form = p.bc_pole_form;
    A.pole_fill = p.bc_pole_fill;
    A.lid_u = p.bc_lid_u;
    A.top_taper = p.bc_top_taper;
    A.lid_copy = p.bc_species_lid_copy;
    A.wall_copy = p.bc_species_wall_copy;
    A.local_rho = p.local_rho;
    bc_theta_kernel<<<dim3((kc.km - 1 + 127) / 128, kc.im - 2, 23), 128, 0, s>>>(kc, A);
    bc_phi_kernel<<<dim3((kc.im * kc.jm + 127) / 128, 1, 23), 128, 0, s>>>(kc, A);
    bc_radius_kernel<<<dim3((kc.km + 127) / 128, kc.jm, 23), 128, 0, s>>>(kc, A);
    return cudaGetLastError();
}

}  // namespace atsat
