// ibisgb-run: runs an ibis case directory on the GB300 engine, as `ibis run`
// does with the reference build (Solver::solve, src/solvers/solvers/solver.cpp:18-85).
//
// Run from the case directory that ibis's prep step produced:
//   config/config.json, io/grid/0000/block_0000.su2, io/flow/0000/{T, p, vx, vy[, vz], meta_data.json}
// It writes what the reference writes: io/flow/NNNN/{T, p, vx, vy[, vz], meta_data.json}
// (native binary or text, per config io.flow_format), the io/flow/flows index,
// and log/residuals.dat (Runge-Kutta) or log/{absolute,relative}_residuals.dat and
// log/gmres_diagnostics.dat (steady state).  The work goes through the C ABI of
// libibisgb.so only.
//
//   ibisgb-run [--precision f64|mixed|mixed_ff|mixed_grad|f64_exact] [--case DIR]
//
// Exit status: 0 on success, 1 when a step fails or leaves bad cells (as
// Solver::solve), 2 for unreadable input or a refused configuration.
#include <sys/stat.h>
#include <unistd.h>

#include <charconv>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "../../../include/ibisgb.h"
#include "../json_lite.hpp"

using ibisgb::Json;

namespace {

struct Failure {
    int code;
    std::string what;
};

std::string read_text(const std::string& path) {
    std::ifstream f(path);
    if (!f) throw Failure{2, "unable to read " + path};
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

void make_dir(const std::string& d) { ::mkdir(d.c_str(), 0755); }

// pad_time_index (src/io/io/io.cpp:32-37)
std::string pad4(int i) {
    std::string s = std::to_string(i);
    return std::string(s.size() < 4 ? 4 - s.size() : 0, '0') + s;
}

// A double as nlohmann::json::dump writes it: the shortest representation that
// reads back exactly, with ".0" added to integral values.
std::string json_number(double v) {
    char buf[64];
    auto r = std::to_chars(buf, buf + sizeof(buf), v);
    std::string s(buf, r.ptr);
    if (s.find_first_of(".eEn") == std::string::npos) s += ".0";
    return s;
}

struct Fields {
    std::vector<double> T, p, vx, vy, vz;
};

const char* kNames[5] = {"T", "p", "vx", "vy", "vz"};

// NativeBinaryInput / NativeTextInput::read (src/io/io/native.cpp:104-339)
Fields read_flow(const std::string& dir, int64_t n, int dim, bool binary) {
    Fields fl;
    std::vector<double>* dst[5] = {&fl.T, &fl.p, &fl.vx, &fl.vy, &fl.vz};
    for (int k = 0; k < (dim == 3 ? 5 : 4); k++) {
        const std::string path = dir + "/" + kNames[k];
        std::vector<double>& v = *dst[k];
        if (binary) {
            std::ifstream f(path, std::ios::binary);
            if (!f) throw Failure{2, "Unable to load " + path};
            v.resize(n);
            f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(sizeof(double) * n));
            if (f.gcount() != (std::streamsize)(sizeof(double) * n))
                throw Failure{2, "too few values in " + path};
        } else {
            std::ifstream f(path);
            if (!f) throw Failure{2, "Unable to load " + path};
            std::string line;
            while (std::getline(f, line))
                if (!line.empty()) v.push_back(std::stod(line));
            if ((int64_t)v.size() != n)
                throw Failure{2, "Incorrect number of values in " + path + ": " + std::to_string(n) +
                                     " cells, but " + std::to_string(v.size()) + " values"};
        }
    }
    return fl;
}

class Case {
   public:
    Case(const std::string& precision) {
        if (precision == "f64") prec_ = IBISGB_F64;
        else if (precision == "mixed") prec_ = IBISGB_MIXED;
        else if (precision == "f64_exact") prec_ = IBISGB_F64_EXACT;
        else if (precision == "mixed_grad") prec_ = IBISGB_MIXED_GRAD;
        else if (precision == "mixed_ff") prec_ = IBISGB_MIXED_FF;
        else throw Failure{2, "unknown precision " + precision};
        text_ = read_text("config/config.json");
        try {
            cfg_ = Json::parse(text_);
        } catch (const std::exception& e) {
            throw Failure{2, std::string("config/config.json: ") + e.what()};
        }
        const std::string fmt = cfg_.at("io").at("flow_format").as_string();
        if (fmt != "native_binary" && fmt != "native_text")
            throw Failure{2, "flow_format " + fmt + " is not written by ibisgb-run (native formats only)"};
        binary_ = fmt == "native_binary";
        if (ibisgb_create(text_.c_str(), "io/grid/0000/block_0000.su2", &ctx_) != IBISGB_OK)
            throw Failure{2, ibisgb_last_error(nullptr)};
        ibisgb_sizes sz;
        ibisgb_get_sizes(ctx_, &sz);
        n_ = sz.num_cells;
        dim_ = sz.dim;
        Fields f = read_flow("io/flow/0000", n_, dim_, binary_);
        check(ibisgb_set_primitives(ctx_, f.T.data(), f.p.data(), f.vx.data(), f.vy.data(),
                                    dim_ == 3 ? f.vz.data() : nullptr));
        make_dir("log");
    }
    ~Case() { ibisgb_destroy(ctx_); }

    int run() {
        const std::string name = cfg_.at("solver").at("name").as_string();
        if (name == "runge_kutta") return run_rk();
        if (name == "steady_state") return run_steady();
        throw Failure{2, "Unknown solver " + name};
    }

   private:
    ibisgb_ctx* ctx_ = nullptr;
    std::string text_;
    Json cfg_;
    int prec_ = IBISGB_F64;
    bool binary_ = true;
    int64_t n_ = 0;
    int dim_ = 2;
    int out_index_ = 1;  // FVIO(config, 1)
    std::chrono::steady_clock::time_point t0_ = std::chrono::steady_clock::now();

    void check(int rc) {
        if (rc != IBISGB_OK) throw Failure{rc == IBISGB_ERR_BAD_CELLS ? 1 : 2, ibisgb_last_error(ctx_)};
    }
    double wall() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
    }

    // FVIO::write + NativeBinaryOutput / NativeTextOutput::write (io.cpp:106-129, native.cpp:7-260)
    void plot(double time) {
        std::vector<double> rho(n_), p(n_), T(n_), e(n_), vx(n_), vy(n_), vz(n_);
        check(ibisgb_get_primitives(ctx_, rho.data(), p.data(), T.data(), e.data(), vx.data(), vy.data(),
                                    vz.data()));
        const std::string idx = pad4(out_index_++);
        make_dir("io/flow");
        const std::string dir = "io/flow/" + idx;
        make_dir(dir);
        {
            std::ofstream meta(dir + "/meta_data.json");
            meta << "{\n    \"time\": " << json_number(time) << "\n}";
        }
        {
            std::ofstream flows("io/flow/flows", std::ios_base::app);
            flows << idx << std::endl;
        }
        const std::vector<double>* src[5] = {&T, &p, &vx, &vy, &vz};
        for (int k = 0; k < (dim_ == 3 ? 5 : 4); k++) {
            const std::string path = dir + "/" + kNames[k];
            if (binary_) {
                std::ofstream f(path, std::ios::binary);
                if (!f) throw Failure{1, "failed to open " + path};
                f.write(reinterpret_cast<const char*>(src[k]->data()), (std::streamsize)(sizeof(double) * n_));
            } else {
                std::ofstream f(path);
                if (!f) throw Failure{1, "failed to open " + path};
                f << std::fixed << std::setprecision(16);
                for (double x : *src[k]) f << x << std::endl;
            }
        }
    }

    // ConservedQuantitiesNorm::write_to_file (conserved_quantities.cpp:5-11)
    static void norms_line(std::ofstream& f, const double* n6, double wc, double time, size_t step) {
        f << time << " " << step << " " << wc << " " << n6[0] << " " << n6[1] << " " << n6[2] << " " << n6[3]
          << " " << n6[4] << " " << n6[5] << std::endl;
    }

    // RungeKutta::initialise / take_step and Solver::solve (runge_kutta.cpp:82-290, solver.cpp:18-61)
    int run_rk() {
        const Json& sc = cfg_.at("solver");
        const double max_time = sc.at("max_time").as_double();
        const size_t max_step = (size_t)sc.at("max_step").as_double();
        const size_t print_frequency = (size_t)sc.at("print_frequency").as_double();
        const double plot_frequency = sc.at("plot_frequency").as_double();
        const double residual_frequency = sc.at("residual_frequency").as_double();
        const int64_t residuals_every = (int64_t)sc.at("residuals_every_n_steps").as_double();
        const int64_t plot_every = (int64_t)sc.at("plot_every_n_steps").as_double();
        double t = 0.0, since_plot = 0.0, since_res = 0.0;
        // the residual of the initial state (function_eval_ at initialise) as the first line
        std::vector<double> scratch((size_t)n_ * (dim_ + 2));
        check(ibisgb_residual(ctx_, prec_, scratch.data()));
        auto write_res = [&](size_t step) {
            double n6[6];
            check(ibisgb_l2_norms(ctx_, n6));
            std::ofstream f("log/residuals.dat", std::ios_base::app);
            norms_line(f, n6, wall(), t, step);
            since_res = 0.0;
        };
        if (residuals_every > 0 || residual_frequency > 0) {
            {
                std::ofstream f("log/residuals.dat", std::ios_base::out);
                f << "time step wall_clock global mass momentum_x momentum_y momentum_z energy\n";
            }
            // ibisgb_residual wrote the stage-0 derivative the norms read
            write_res(0);
        }
        for (size_t step = 0; step < max_step; step++) {
            ibisgb_rk_status st{};
            const int rc = ibisgb_rk_run(ctx_, prec_, 1, &st);
            const double dt = st.dt;
            t = st.t;
            since_plot += dt;
            since_res += dt;
            const bool res_now = (residuals_every > 0 && (step != 0 || step % residuals_every == 0)) ||
                                 (residual_frequency > 0 && since_res >= residual_frequency - 1e-15);
            if (res_now) write_res(step);
            if (rc != IBISGB_OK) {
                std::fprintf(stderr, "step %zu failed: %s\n", step, ibisgb_last_error(ctx_));
                if (rc == IBISGB_ERR_BAD_CELLS)
                    std::fprintf(stderr, "Encountered %lld bad cells on step %zu\n", (long long)st.bad_cells, step);
                plot(t);
                return 1;
            }
            const bool stop = step >= max_step - 1 || t >= max_time;
            if (stop) {
                std::printf("STOPPING: %s\n", t >= max_time - 1e-15 ? "reached max time" : "reached max step");
                plot(t);
                since_plot = 0.0;
                break;
            }
            if (step != 0 && print_frequency > 0 && step % print_frequency == 0)
                std::printf("  step: %8zu, t = %.6e (%.1f%%), dt = %.6e (cfl=%.1f), wc = %.1fs\n", step, t,
                            t / max_time * 100, dt, dt / st.stable_dt, wall());
            const bool plot_now = (plot_every > 0 && step != 0 && step % plot_every == 0) ||
                                  (plot_frequency > 0 && since_plot >= plot_frequency - 1e-15);
            if (plot_now) {
                plot(t);
                since_plot = 0.0;
            }
        }
        std::printf("Elapsed Wall Clock: %.3fs\n", wall());
        return 0;
    }

    // SteadyState::initialise / take_step with Jfnk (steady_state.cpp:176-326, jfnk.cpp:25-93)
    int run_steady() {
        const Json& sc = cfg_.at("solver");
        const size_t max_step = (size_t)sc.at("max_steps").as_double();
        const double target = sc.at("tolerance").as_double();
        const size_t print_frequency = (size_t)sc.at("print_frequency").as_double();
        const size_t plot_frequency = (size_t)sc.at("plot_frequency").as_double();
        const size_t diagnostics = (size_t)sc.at("diagnostics_frequency").as_double();
        check(ibisgb_steady_initialise(ctx_, prec_));
        ibisgb_newton_status st{};
        bool have = false;
        double init[6], cur[6];
        check(ibisgb_steady_norms(ctx_, cur, init));
        auto write_res = [&](size_t step) {
            double rel[6];
            for (int q = 0; q < 6; q++) rel[q] = init[q] != 0.0 ? cur[q] / init[q] : 0.0;
            std::ofstream fa("log/absolute_residuals.dat", std::ios_base::app);
            norms_line(fa, cur, wall(), (double)step, step);
            std::ofstream fr("log/relative_residuals.dat", std::ios_base::app);
            norms_line(fr, rel, wall(), (double)step, step);
            std::ofstream fg("log/gmres_diagnostics.dat", std::ios_base::app);
            fg << step << " " << (have ? st.gmres_converged : 0) << " " << (have ? st.gmres_residual : 0.0) << " "
               << sc.at("linear_solver").get("tol", sc.at("linear_solver").get("tolerance", 0.0)) << " "
               << (have ? st.gmres_iterations : 0) << std::endl;
        };
        if (diagnostics > 0) {
            {
                std::ofstream fa("log/absolute_residuals.dat", std::ios_base::out);
                fa << "step step wall_clock global mass momentum_x momentum_y momentum_z energy\n";
                std::ofstream fr("log/relative_residuals.dat", std::ios_base::out);
                fr << "step step wall_clock global mass momentum_x momentum_y momentum_z energy\n";
            }
            write_res(0);
            std::ofstream fg("log/gmres_diagnostics.dat", std::ios_base::out);
            fg << "step converged residual tolerance n_iters\n";
        }
        for (size_t step = 0; step < max_step; step++) {
            check(ibisgb_newton_step(ctx_, prec_, &st));
            have = true;
            for (int q = 0; q < 6; q++) { cur[q] = st.residual_norms[q]; init[q] = st.initial_norms[q]; }
            if (diagnostics > 0 && step != 0 && step % diagnostics == 0) write_res(step);
            int64_t bad = 0;
            check(ibisgb_count_bad_cells(ctx_, &bad));
            if (bad > 0) {
                std::fprintf(stderr, "Encountered %lld bad cells on step %zu\n", (long long)bad, step);
                plot((double)step);
                return 1;
            }
            const bool converged = st.relative_residual < target;
            if (step >= max_step - 1 || converged) {
                std::printf("STOPPING: %s\n", converged ? "reached target residual" : "reached max_step");
                plot((double)step);
                break;
            }
            if (step != 0 && print_frequency > 0 && step % print_frequency == 0)
                std::printf("  step: %8zu, relative global residual %.2e, cfl = %.1f, wc = %.1fs\n", step,
                            st.relative_residual, st.cfl, wall());
            if (step != 0 && plot_frequency > 0 && step % plot_frequency == 0) plot((double)step);
        }
        std::printf("Elapsed Wall Clock: %.3fs\n", wall());
        return 0;
    }
};

}  // namespace

int main(int argc, char** argv) {
    std::string precision = "f64", dir;
    for (int a = 1; a < argc; a++) {
        const std::string s = argv[a];
        if (s == "--precision" && a + 1 < argc) precision = argv[++a];
        else if (s == "--case" && a + 1 < argc) dir = argv[++a];
        else {
            std::fprintf(stderr, "usage: ibisgb-run [--precision f64|mixed|mixed_ff|mixed_grad|f64_exact] [--case DIR]\n");
            return 2;
        }
    }
    if (!dir.empty() && ::chdir(dir.c_str()) != 0) {
        std::fprintf(stderr, "cannot enter %s\n", dir.c_str());
        return 2;
    }
    try {
        Case c(precision);
        return c.run();
    } catch (const Failure& f) {
        std::fprintf(stderr, "ibisgb-run: %s\n", f.what.c_str());
        return f.code;
    } catch (const std::exception& e) {
        std::fprintf(stderr, "ibisgb-run: %s\n", e.what());
        return 2;
    }
}
