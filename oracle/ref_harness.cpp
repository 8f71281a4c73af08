// ORACLE (test infrastructure only): a C interface over the reference's own
// classes, compiled unchanged from an ibis checkout (Makefile.ref).  It drives
// the reference exactly as its solvers do -- FiniteVolume<T>::compute_dudt
// (src/finite_volume/finite_volume/finite_volume.cpp:56-96),
// RungeKutta::initialise / take_step (src/solvers/solvers/runge_kutta.cpp:82-203),
// SteadyState::initialise / take_step and SteadyStateLinearisation::
// matrix_vector_product (src/solvers/solvers/steady_state.cpp:52-128,
// 175-326) -- and copies results out as plain arrays.  Members that ibis keeps
// private (the limiter values, the solver state) are read by compiling the
// reference headers with private/protected access opened in this file only.
// Every entry point returns 0 on success (1: the solver stopped on bad cells)
// or -1 with a message in ref_last_error(); no C++ exception crosses this
// interface.
#include <algorithm>
#include <array>
#include <cassert>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <functional>
#include <iomanip>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <numeric>
#include <optional>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <tuple>
#include <unordered_map>
#include <utility>
#include <variant>
#include <vector>

#include <Kokkos_Core.hpp>
#include <doctest/doctest.h>
#include <nlohmann/json.hpp>
#include <spdlog/spdlog.h>
#include <spdlog/stopwatch.h>

#define private public
#define protected public
#include <finite_volume/finite_volume.h>
#include <finite_volume/primative_conserved_conversion.h>
#include <solvers/runge_kutta.h>
#include <solvers/steady_state.h>
#undef private
#undef protected

using json = nlohmann::json;

namespace {

std::string g_error;

template <class F>
int guarded(F&& f) {
    try {
        f();
        return 0;
    } catch (const std::exception& e) {
        g_error = e.what();
    } catch (const std::exception* e) {  // ibis throws new std::runtime_error(...)
        g_error = e->what();
    } catch (...) {
        g_error = "unknown exception";
    }
    return -1;
}

// Runs f with the working directory set to dir (ibis's solvers read and write
// relative paths: config/, io/, log/).
template <class F>
void in_dir(const std::string& dir, F&& f) {
    const auto old = std::filesystem::current_path();
    std::filesystem::current_path(dir);
    try {
        f();
    } catch (...) {
        std::filesystem::current_path(old);
        throw;
    }
    std::filesystem::current_path(old);
}

json read_json(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw std::runtime_error("cannot open " + path);
    return json::parse(f);
}

// One grid block with a FiniteVolume, as a RungeKutta builds them.
struct FvCase {
    json config;
    GridBlock<Ibis::real> grid;
    FiniteVolume<Ibis::real> fv;
    IdealGas<Ibis::real> gas;
    TransportProperties<Ibis::real> tp;
    FlowStates<Ibis::real> fs;
    ConservedQuantities<Ibis::real> dudt;
};

template <class T>
void copy_rows(const ConservedQuantities<T>& cq, size_t n, double* out) {
    const size_t nc = cq.dim() + 2;
    for (size_t i = 0; i < n; i++)
        for (size_t q = 0; q < nc; q++) out[i * nc + q] = Ibis::real_part(cq(i, q));
}

template <class T>
void copy_prims(const FlowStates<T>& fs, size_t n, double* out) {
    for (size_t i = 0; i < n; i++) {
        out[0 * n + i] = Ibis::real_part(fs.gas.rho(i));
        out[1 * n + i] = Ibis::real_part(fs.gas.pressure(i));
        out[2 * n + i] = Ibis::real_part(fs.gas.temp(i));
        out[3 * n + i] = Ibis::real_part(fs.gas.energy(i));
        out[4 * n + i] = Ibis::real_part(fs.vel.x(i));
        out[5 * n + i] = Ibis::real_part(fs.vel.y(i));
        out[6 * n + i] = Ibis::real_part(fs.vel.z(i));
    }
}

}  // namespace

extern "C" {

const char* ref_last_error() { return g_error.c_str(); }

int ref_threads() { return Kokkos::DefaultExecutionSpace::concurrency(); }

// ------------------------------------------------------------------ residual
void* ref_fv_create(const char* config_text, const char* su2_path) {
    FvCase* c = nullptr;
    const int rc = guarded([&] {
        auto h = std::make_unique<FvCase>();
        h->config = json::parse(std::string(config_text));
        json grid_config = h->config.at("grid");
        h->grid = GridBlock<Ibis::real>(std::string(su2_path), grid_config);
        h->fv = FiniteVolume<Ibis::real>(h->grid, h->config);
        h->gas = IdealGas<Ibis::real>(h->config.at("gas_model"));
        h->tp = TransportProperties<Ibis::real>(h->config.at("transport_properties"));
        h->fs = FlowStates<Ibis::real>(h->grid.num_total_cells());
        h->dudt = ConservedQuantities<Ibis::real>(h->grid.num_total_cells(), h->grid.dim());
        c = h.release();
    });
    return rc == 0 ? c : nullptr;
}

void ref_fv_destroy(void* h) { delete (FvCase*)h; }

int ref_fv_sizes(void* hp, long long* out) {
    return guarded([&] {
        FvCase& c = *(FvCase*)hp;
        out[0] = (long long)c.grid.num_cells();
        out[1] = (long long)c.grid.num_ghost_cells();
        out[2] = (long long)c.grid.num_interfaces();
        out[3] = (long long)c.grid.dim();
    });
}

// The initial condition of the valid cells as the native flow reader leaves it
// (T, p, v), then the thermodynamic state from (p, T) on every cell.
int ref_fv_set_prims(void* hp, const double* T, const double* p, const double* vx, const double* vy,
                     const double* vz) {
    return guarded([&] {
        FvCase& c = *(FvCase*)hp;
        const size_t n = c.grid.num_cells();
        for (size_t i = 0; i < n; i++) {
            c.fs.gas.temp(i) = T[i];
            c.fs.gas.pressure(i) = p[i];
            c.fs.vel.x(i) = vx[i];
            c.fs.vel.y(i) = vy[i];
            c.fs.vel.z(i) = vz ? vz[i] : 0.0;
        }
        c.gas.update_thermo_from_pT(c.fs.gas);
    });
}

// FiniteVolume::compute_dudt at the current state: dudt of the valid cells,
// N x n_conserved row-major
int ref_fv_residual(void* hp, double* dudt, int allow_reconstruction) {
    return guarded([&] {
        FvCase& c = *(FvCase*)hp;
        c.fv.compute_dudt(c.fs, c.grid, c.dudt, c.gas, c.tp, allow_reconstruction != 0);
        copy_rows(c.dudt, c.grid.num_cells(), dudt);
    });
}

// The limiter values of the last residual, N x 7 in the order rho, p, T, u
// (internal energy), vx, vy, vz; NaN where the reference keeps no value
int ref_fv_limiters(void* hp, double* out) {
    return guarded([&] {
        FvCase& c = *(FvCase*)hp;
        const auto& L = c.fv.convective_flux_.limiters_;
        const size_t n = c.grid.num_cells();
        const Field<Ibis::real>* f[7] = {&L.rho, &L.p, &L.temp, &L.u, &L.vx, &L.vy, &L.vz};
        for (int k = 0; k < 7; k++)
            for (size_t i = 0; i < n; i++)
                out[i * 7 + k] = f[k]->size() == n ? (*f[k])(i) : std::numeric_limits<double>::quiet_NaN();
    });
}

// The gradients of the last residual, N x 7 x 3 (same variable order)
int ref_fv_gradients(void* hp, double* out) {
    return guarded([&] {
        FvCase& c = *(FvCase*)hp;
        const auto& g = c.fv.cell_grad_;
        const size_t n = c.grid.num_cells();
        const Vector3s<Ibis::real>* v[7] = {&g.rho, &g.p, &g.temp, &g.u, &g.vx, &g.vy, &g.vz};
        for (int k = 0; k < 7; k++)
            for (size_t i = 0; i < n; i++)
                for (int a = 0; a < 3; a++)
                    out[(i * 7 + k) * 3 + a] =
                        v[k]->size() >= n ? (*v[k])(i, a) : std::numeric_limits<double>::quiet_NaN();
    });
}

// Primitives of every cell (valid, then ghosts as the last residual's boundary
// actions left them): 7 x (N + G), rho, p, T, e, vx, vy, vz
int ref_fv_prims(void* hp, double* out) {
    return guarded([&] {
        FvCase& c = *(FvCase*)hp;
        copy_prims(c.fs, c.grid.num_total_cells(), out);
    });
}

int ref_fv_estimate_dt(void* hp, double* dt) {
    return guarded([&] {
        FvCase& c = *(FvCase*)hp;
        *dt = c.fv.estimate_dt(c.fs, c.grid, c.gas, c.tp);
    });
}

// ------------------------------------------------------------------ Runge-Kutta
struct RkCase {
    std::string dir;
    std::unique_ptr<RungeKutta> rk;
    size_t steps = 0;
};

// A RungeKutta solver of a case directory (config/config.json,
// io/grid/0000/block_0000.su2, io/flow/0000), initialised from its flow files.
void* ref_rk_create(const char* case_dir) {
    RkCase* out = nullptr;
    const int rc = guarded([&] {
        auto c = std::make_unique<RkCase>();
        c->dir = case_dir;
        in_dir(c->dir, [&] {
            json config = read_json("config/config.json");
            json grid_config = config.at("grid");
            GridBlock<Ibis::real> grid("io/grid/0000/block_0000.su2", grid_config);
            c->rk = std::make_unique<RungeKutta>(config, grid, "io/grid", "io/flow");
            if (c->rk->initialise() != 0) throw std::runtime_error("RungeKutta::initialise failed");
        });
        out = c.release();
    });
    return rc == 0 ? out : nullptr;
}

void ref_rk_destroy(void* h) { delete (RkCase*)h; }

// n steps of RungeKutta::take_step, stopping (rc 1) at bad cells as
// Solver::solve does; t and dt after the last step; wall seconds of the steps
int ref_rk_steps(void* hp, long long n, double* t, double* dt, double* seconds) {
    int status = 0;
    const int rc = guarded([&] {
        RkCase& c = *(RkCase*)hp;
        const auto t0 = std::chrono::steady_clock::now();
        for (long long s = 0; s < n; s++) {
            if (c.rk->take_step(c.steps++) != 0 || c.rk->count_bad_cells() > 0) {
                status = 1;
                break;
            }
        }
        if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        if (t) *t = c.rk->t_;
        if (dt) *dt = c.rk->dt_;
    });
    return rc != 0 ? rc : status;
}

// conserved state of the valid cells, N x n_conserved row-major
int ref_rk_conserved(void* hp, double* U) {
    return guarded([&] {
        RkCase& c = *(RkCase*)hp;
        copy_rows(c.rk->conserved_quantities_, c.rk->grid_.num_cells(), U);
    });
}

int ref_rk_sizes(void* hp, long long* out) {
    return guarded([&] {
        RkCase& c = *(RkCase*)hp;
        out[0] = (long long)c.rk->grid_.num_cells();
        out[1] = (long long)c.rk->grid_.num_ghost_cells();
        out[2] = (long long)c.rk->grid_.num_interfaces();
        out[3] = (long long)c.rk->grid_.dim();
    });
}

// The reference's own driver on a case directory: make_solver + Solver::solve
// (solver.cpp:18-85), reading config/, io/grid/0000 and io/flow/0000 and writing
// io/flow/NNNN, io/flow/flows and log/ as `ibis run` does.  Returns solve()'s result.
int ref_run_case(const char* case_dir) {
    int result = -1;
    const int rc = guarded([&] {
        in_dir(case_dir, [&] {
            json config = read_json("config/config.json");
            std::unique_ptr<Solver> solver = make_solver(config, "io/grid", "io/flow");
            result = solver->solve();
        });
    });
    return rc != 0 ? rc : result;
}

// ------------------------------------------------------------------ steady state
struct SsCase {
    std::string dir;
    std::unique_ptr<SteadyState> ss;
    size_t steps = 0;
};

void* ref_ss_create(const char* case_dir) {
    SsCase* out = nullptr;
    const int rc = guarded([&] {
        auto c = std::make_unique<SsCase>();
        c->dir = case_dir;
        in_dir(c->dir, [&] {
            json config = read_json("config/config.json");
            json grid_config = config.at("grid");
            GridBlock<Ibis::dual> grid("io/grid/0000/block_0000.su2", grid_config);
            c->ss = std::make_unique<SteadyState>(config, grid, "io/grid", "io/flow");
            if (c->ss->initialise() != 0) throw std::runtime_error("SteadyState::initialise failed");
        });
        out = c.release();
    });
    return rc == 0 ? out : nullptr;
}

void ref_ss_destroy(void* h) { delete (SsCase*)h; }

// SteadyStateLinearisation::matrix_vector_product at the solver's current
// state: result = v / dt_star - dR/dU v (valid cells, cell-major n_conserved)
int ref_ss_jv(void* hp, const double* v, double* result, double dt_star, int allow_reconstruction) {
    return guarded([&] {
        SsCase& c = *(SsCase*)hp;
        SteadyState& s = *c.ss;
        SteadyStateLinearisation lin(s.sim_, s.residuals_, s.cq_, s.fs_, s.vertex_vel_, allow_reconstruction != 0);
        lin.set_pseudo_time_step(dt_star);
        const size_t n = lin.num_vars();
        Ibis::Vector<Ibis::real> vec("ref_jv_v", n), res("ref_jv_result", n);
        for (size_t i = 0; i < n; i++) vec(i) = v[i];
        lin.matrix_vector_product(vec, res);
        for (size_t i = 0; i < n; i++) result[i] = res(i);
    });
}

// One Newton step (SteadyState::take_step); the global relative residual norm
// after it, the pseudo time step and the GMRES iterations of the step
int ref_ss_step(void* hp, double* rel_residual, double* dt_star, long long* gmres_iters) {
    return guarded([&] {
        SsCase& c = *(SsCase*)hp;
        in_dir(c.dir, [&] {
            if (c.ss->take_step(c.steps++) != 0) throw std::runtime_error("SteadyState::take_step failed");
        });
        const Jfnk& j = c.ss->jfnk_;
        if (rel_residual) *rel_residual = Ibis::real_part(j.relative_residual_norms().global());
        if (dt_star) *dt_star = j.pseudo_time_step_size();
        if (gmres_iters) *gmres_iters = (long long)j.last_gmres_result().n_iters;
    });
}

int ref_ss_conserved(void* hp, double* U) {
    return guarded([&] {
        SsCase& c = *(SsCase*)hp;
        copy_rows(*c.ss->cq_, c.ss->sim_->grid.num_cells(), U);
    });
}

}  // extern "C"
