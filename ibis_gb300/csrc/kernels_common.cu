// Precision-independent device work: the Runge-Kutta time-step control block
// and reductions of residual norms.
#include "engine.hpp"

namespace ibisgb {

namespace {

// linear CFL schedule (LinearSchedule::eval, cfl.cpp:108-127)
__device__ double cfl_eval(const StepCtl& c, double t) {
    if (c.n_cfl == 0) return c.cfl;
    if (t <= c.cfl_t[0]) return c.cfl_v[0];
    int n = c.n_cfl;
    if (t >= c.cfl_t[n - 1]) return c.cfl_v[n - 1];
    for (int i = 0; i + 1 < n; i++) {
        if (t >= c.cfl_t[i] && t < c.cfl_t[i + 1]) {
            double frac = (t - c.cfl_t[i]) / (c.cfl_t[i + 1] - c.cfl_t[i]);
            return c.cfl_v[i] + frac * (c.cfl_v[i + 1] - c.cfl_v[i]);
        }
    }
    return c.cfl_v[n - 1];
}

__device__ double dmin(double a, double b) { return (b < a) ? b : a; }

// RungeKutta::estimate_dt (runge_kutta.cpp:108-119) and the coefficients of the step
__global__ void k_dt_finalize(StepCtl* ctl, int n_cases) {
    const int cs = blockIdx.x * blockDim.x + threadIdx.x;
    if (cs >= n_cases) return;
    StepCtl* c = ctl + cs;
    if (c->halt) return;
    if (c->bad_cells > 0 || c->t >= c->max_time) {
        c->halt = 1;
        return;
    }
    double stable = __longlong_as_double((long long)c->dt_bits);
    c->stable_dt = stable;
    double dt_startup = dmin(cfl_eval(*c, c->t) * stable, 1.5 * c->dt);
    double dt = dmin(dt_startup, c->max_time - c->t);
    if (c->plot_frequency > 0.0 && c->time_since_last_plot < c->plot_frequency)
        dt = dmin(dt, c->plot_frequency - c->time_since_last_plot);
    c->dt = dt;
    for (int i = 1; i < c->stages; i++)
        for (int j = 0; j < i; j++) c->ca[i][j] = c->a[i][j] * dt;
    for (int i = 0; i < c->stages; i++) c->cb[i] = c->b[i] * dt;
    c->t += dt;
    c->time_since_last_plot += dt;
    c->dt_bits = 0x7FF0000000000000ull;  // +inf for the next step
    c->steps += 1;
}

__global__ void k_reset_dt(StepCtl* ctl, int n_cases) {
    const int cs = blockIdx.x * blockDim.x + threadIdx.x;
    if (cs < n_cases) ctl[cs].dt_bits = 0x7FF0000000000000ull;
}

// sums of squares of k0 per component and in total; one block per chunk,
// deterministic two-pass reduction (block partials, then one block)
constexpr int kRB = 256;

__global__ void k_l2_partial(const double* k0, int N, int nc, double* partial) {
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * kRB + threadIdx.x; i < N; i += gridDim.x * kRB) {
        for (int q = 0; q < nc; q++) {
            double x = k0[(size_t)q * N + i];
            int slot = q == 0 ? 1 : (q == nc - 1 ? 5 : 1 + q);  // mass, mx, my, [mz], energy
            s[slot] += x * x;
            s[0] += x * x;
        }
    }
    __shared__ double sh[6][kRB];
    for (int k = 0; k < 6; k++) sh[k][threadIdx.x] = s[k];
    __syncthreads();
    for (int w = kRB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w)
            for (int k = 0; k < 6; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = 0; k < 6; k++) partial[blockIdx.x * 6 + k] = sh[k][0];
}

__global__ void k_l2_final(const double* partial, int nblocks, double* out6) {
    if (threadIdx.x != 0) return;
    double s[6] = {0, 0, 0, 0, 0, 0};
    for (int b = 0; b < nblocks; b++)
        for (int k = 0; k < 6; k++) s[k] += partial[b * 6 + k];
    for (int k = 0; k < 6; k++) out6[k] = sqrt(s[k]);
}

}  // namespace

void launch_dt_finalize(StepCtl* ctl, int n_cases, cudaStream_t s) {
    k_dt_finalize<<<(n_cases + 63) / 64, 64, 0, s>>>(ctl, n_cases);
}
void launch_reset_dt(StepCtl* ctl, int n_cases, cudaStream_t s) {
    k_reset_dt<<<(n_cases + 63) / 64, 64, 0, s>>>(ctl, n_cases);
}

// out6 must hold 6 + 6*nblocks doubles of scratch after the 6 results
void launch_l2_norms(const double* k0, int N, int nc, double* out6, cudaStream_t s) {
    const int nblocks = 304;
    k_l2_partial<<<nblocks, kRB, 0, s>>>(k0, N, nc, out6 + 6);
    k_l2_final<<<1, 32, 0, s>>>(out6 + 6, nblocks, out6);
}

// ---------------------------------------------------------------------------
// Krylov vector kernels (dense_linear_algebra.h:184-309 on the device).  Dots
// and norms are deterministic two-pass reductions whose result stays in device
// memory, so a modified Gram-Schmidt sweep never waits for the host.
// ---------------------------------------------------------------------------
namespace {
constexpr int kDotBlocks = 608;  // 4 per SM

__global__ void k_dot_partial(const double* a, const double* b, long long n, double* partial) {
    double s = 0.0;
    for (long long i = (long long)blockIdx.x * kRB + threadIdx.x; i < n; i += (long long)gridDim.x * kRB)
        s += a[i] * b[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __shared__ double w[kRB / 32];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < kRB / 32; k++) t += w[k];
        partial[blockIdx.x] = t;
    }
}

__global__ void k_dot_final(const double* partial, int nb, double* out, int take_sqrt) {
    __shared__ double sh[kRB];
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += kRB) s += partial[b];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = kRB / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = take_sqrt ? sqrt(sh[0]) : sh[0];
}

// y += x * (-c[0])   (add_scaled_vector(w, v_i, -H(i, j)), gmres.cpp:147)
__global__ void k_axpy_neg(double* y, const double* x, long long n, const double* c) {
    const double a = -c[0];
    for (long long i = (long long)blockIdx.x * kRB + threadIdx.x; i < n; i += (long long)gridDim.x * kRB)
        y[i] += x[i] * a;
}

// out = in * (1 / d[0])   (scale(w, v, 1.0 / H(j+1, j)), gmres.cpp:150)
__global__ void k_scale_inv(double* out, const double* in, long long n, const double* d) {
    const double a = 1.0 / d[0];
    for (long long i = (long long)blockIdx.x * kRB + threadIdx.x; i < n; i += (long long)gridDim.x * kRB)
        out[i] = in[i] * a;
}

__global__ void k_sub(double* out, const double* a, const double* b, long long n) {
    for (long long i = (long long)blockIdx.x * kRB + threadIdx.x; i < n; i += (long long)gridDim.x * kRB)
        out[i] = a[i] - b[i];
}

// x += V y with V column c at V + c * n   (gemv + add_scaled_vector, gmres.cpp:170-179)
__global__ void k_gemv_add(double* x, const double* V, long long n, int m, const double* y) {
    for (long long i = (long long)blockIdx.x * kRB + threadIdx.x; i < n; i += (long long)gridDim.x * kRB) {
        double d = 0.0;
        for (int c = 0; c < m; c++) d += V[(size_t)c * n + i] * y[c];
        x[i] += d * 1.0;
    }
}

// y = a x + b y
__global__ void k_axpby(double* y, const double* x, long long n, double a, double b) {
    for (long long i = (long long)blockIdx.x * kRB + threadIdx.x; i < n; i += (long long)gridDim.x * kRB)
        y[i] = a * x[i] + b * y[i];
}

// out[i * nc + q] = in[i * nc + q] * s[q]  (per-variable scaling of row vectors)
__global__ void k_scale_rows(double* out, const double* in, long long n, int nc, RowScale sc) {
    for (long long i = (long long)blockIdx.x * kRB + threadIdx.x; i < n; i += (long long)gridDim.x * kRB)
        out[i] = in[i] * sc.s[i % nc];
}

// dst[i * w + q] = src[map[i] * w + q]   (rows between two cell numberings)
__global__ void k_gather_rows(double* dst, const double* src, const int32_t* map, int N, int w) {
    const long long n = (long long)N * w;
    for (long long t = (long long)blockIdx.x * kRB + threadIdx.x; t < n; t += (long long)gridDim.x * kRB) {
        const long long i = t / w;
        dst[t] = src[(long long)map[i] * w + (t - i * w)];
    }
}

// U[q][i] += dU[i * nc + q]   (Jfnk::apply_update_, jfnk.cpp:63-76)
__global__ void k_add_rows(double* U, const double* dU, int N, int nc) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * nc) return;
    int i = (int)(t / nc), q = (int)(t % nc);
    U[(size_t)q * N + i] += dU[t];
}
}  // namespace

void launch_dot(const double* a, const double* b, long long n, double* partial, double* out,
                bool take_sqrt, cudaStream_t s) {
    k_dot_partial<<<kDotBlocks, kRB, 0, s>>>(a, b, n, partial);
    k_dot_final<<<1, kRB, 0, s>>>(partial, kDotBlocks, out, take_sqrt ? 1 : 0);
}
void launch_axpy_neg(double* y, const double* x, long long n, const double* c, cudaStream_t s) {
    k_axpy_neg<<<kDotBlocks, kRB, 0, s>>>(y, x, n, c);
}
void launch_scale_inv(double* out, const double* in, long long n, const double* d, cudaStream_t s) {
    k_scale_inv<<<kDotBlocks, kRB, 0, s>>>(out, in, n, d);
}
void launch_sub(double* out, const double* a, const double* b, long long n, cudaStream_t s) {
    k_sub<<<kDotBlocks, kRB, 0, s>>>(out, a, b, n);
}
void launch_gemv_add(double* x, const double* V, long long n, int m, const double* y, cudaStream_t s) {
    k_gemv_add<<<kDotBlocks, kRB, 0, s>>>(x, V, n, m, y);
}
void launch_axpby(double* y, const double* x, long long n, double a, double b, cudaStream_t s) {
    k_axpby<<<kDotBlocks, kRB, 0, s>>>(y, x, n, a, b);
}
void launch_scale_rows(double* out, const double* in, long long n, int nc, const RowScale& sc, cudaStream_t s) {
    k_scale_rows<<<kDotBlocks, kRB, 0, s>>>(out, in, n, nc, sc);
}
void launch_gather_rows(double* dst, const double* src, const int32_t* map, int N, int w, cudaStream_t s) {
    k_gather_rows<<<kDotBlocks, kRB, 0, s>>>(dst, src, map, N, w);
}
void launch_add_rows(double* U, const double* dU, int N, int nc, cudaStream_t s) {
    long long n = (long long)N * nc;
    k_add_rows<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(U, dU, N, nc);
}
int dot_scratch_doubles() { return kDotBlocks; }

namespace {
__global__ void k_rows_to_soa(const double* rows, double* soa, int N, int nc) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * nc) return;
    int i = (int)(t / nc), q = (int)(t % nc);
    soa[(size_t)q * N + i] = rows[t];
}
__global__ void k_soa_to_rows(const double* soa, double* rows, int N, int nc) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * nc) return;
    int i = (int)(t / nc), q = (int)(t % nc);
    rows[t] = soa[(size_t)q * N + i];
}

// The same with 16-byte accesses on the row side (two doubles per thread; the row
// array holds an even number of doubles and is 16-byte aligned): half as many
// requests when the rows are pinned host memory read or written over the C2C link.
__global__ void k_rows_to_soa2(const double2* rows, double* soa, int N, int nc) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * nc / 2) return;
    const double2 v = rows[t];
    const long long e = 2 * t;
    soa[(size_t)(e % nc) * N + e / nc] = v.x;
    soa[(size_t)((e + 1) % nc) * N + (e + 1) / nc] = v.y;
}
__global__ void k_soa_to_rows2(const double* soa, double2* rows, int N, int nc) {
    long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)N * nc / 2) return;
    const long long e = 2 * t;
    double2 v;
    v.x = soa[(size_t)(e % nc) * N + e / nc];
    v.y = soa[(size_t)((e + 1) % nc) * N + (e + 1) / nc];
    rows[t] = v;
}

// One block per boundary: the ghosts of boundary b, visited in a fixed strided
// order and summed by a tree, so the result does not depend on scheduling.
__global__ void __launch_bounds__(256) k_sum_ghost_rows(const double* rows, const int* gb, int G, double* out) {
    __shared__ double red[7][256];
    const int b = blockIdx.x, t = threadIdx.x;
    double acc[7] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int g = t; g < G; g += 256)
        if (gb[g] == b)
            for (int k = 0; k < 7; k++) acc[k] += rows[(size_t)g * 7 + k];
    for (int k = 0; k < 7; k++) red[k][t] = acc[k];
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if (t < h)
            for (int k = 0; k < 7; k++) red[k][t] += red[k][t + h];
        __syncthreads();
    }
    if (t < 7) out[b * 7 + t] = red[t][0];
}
}  // namespace

void launch_sum_ghost_rows(const double* rows, const int* ghost_bound, int G, int nb, double* out, cudaStream_t s) {
    if (nb > 0) k_sum_ghost_rows<<<(unsigned)nb, 256, 0, s>>>(rows, ghost_bound, G, out);
}

void launch_rows_to_soa(const double* rows, double* soa, int N, int nc, cudaStream_t s) {
    long long n = (long long)N * nc;
    if (n % 2 == 0 && ((uintptr_t)rows & 15) == 0)
        k_rows_to_soa2<<<(unsigned)((n / 2 + 255) / 256), 256, 0, s>>>((const double2*)rows, soa, N, nc);
    else
        k_rows_to_soa<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(rows, soa, N, nc);
}
void launch_soa_to_rows(const double* soa, double* rows, int N, int nc, cudaStream_t s) {
    long long n = (long long)N * nc;
    if (n % 2 == 0 && ((uintptr_t)rows & 15) == 0)
        k_soa_to_rows2<<<(unsigned)((n / 2 + 255) / 256), 256, 0, s>>>(soa, (double2*)rows, N, nc);
    else
        k_soa_to_rows<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(soa, rows, N, nc);
}

}  // namespace ibisgb
