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
__global__ void k_dt_finalize(StepCtl* c) {
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

__global__ void k_reset_dt(StepCtl* c) { c->dt_bits = 0x7FF0000000000000ull; }

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

void launch_dt_finalize(StepCtl* ctl, cudaStream_t s) { k_dt_finalize<<<1, 1, 0, s>>>(ctl); }
void launch_reset_dt(StepCtl* ctl, cudaStream_t s) { k_reset_dt<<<1, 1, 0, s>>>(ctl); }

// out6 must hold 6 + 6*nblocks doubles of scratch after the 6 results
void launch_l2_norms(const double* k0, int N, int nc, double* out6, cudaStream_t s) {
    const int nblocks = 304;
    k_l2_partial<<<nblocks, kRB, 0, s>>>(k0, N, nc, out6 + 6);
    k_l2_final<<<1, 32, 0, s>>>(out6 + 6, nblocks, out6);
}

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
}  // namespace

void launch_rows_to_soa(const double* rows, double* soa, int N, int nc, cudaStream_t s) {
    long long n = (long long)N * nc;
    k_rows_to_soa<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(rows, soa, N, nc);
}
void launch_soa_to_rows(const double* soa, double* rows, int N, int nc, cudaStream_t s) {
    long long n = (long long)N * nc;
    k_soa_to_rows<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(soa, rows, N, nc);
}

}  // namespace ibisgb
