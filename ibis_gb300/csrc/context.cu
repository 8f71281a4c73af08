// Host side of libibisgb: the context behind the C ABI (include/ibisgb.h).
// Reads ibis's config.json, builds the mesh, owns the device memory and one
// CUDA stream, and drives the residual / Runge-Kutta kernels (one CUDA graph
// per Runge-Kutta step).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/ibisgb.h"
#include "engine.hpp"
#include "json_lite.hpp"
#include "mesh.hpp"
#include "profile.hpp"
#include "structured.hpp"

using namespace ibisgb;

namespace {

#define CUDA_OK(x)                                                                          \
    do {                                                                                    \
        cudaError_t e_ = (x);                                                               \
        if (e_ != cudaSuccess)                                                              \
            throw CudaError(std::string(#x) + ": " + cudaGetErrorString(e_));               \
    } while (0)

struct CudaError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct ConfigError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct ArgError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct StateError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// Device allocation owned by the context.
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { if (p) cudaFree(p); }
    void alloc(size_t n) {
        if (p && bytes >= n) return;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        if (n == 0) return;
        CUDA_OK(cudaMalloc(&p, n));
        bytes = n;
    }
    template <class T>
    T* as() const { return (T*)p; }
};

template <class T>
void upload(DBuf& b, const std::vector<T>& v, cudaStream_t s) {
    b.alloc(v.size() * sizeof(T));
    if (!v.empty()) CUDA_OK(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}

// State buffers of one storage type (double for F64 / F64_EXACT, float for MIXED).
struct StateBufs {
    DBuf cc, r, face, lsqw, lsqd;                  // geometry
    DBuf prim, vghost, grad, phi, vgrad, flux;     // state and intermediates
    DBuf prim_lo, cc_lo, face_lo, flux_lo;         // float-float build: lo companions of the float arrays
    DBuf lsqw_lo, lsqd_lo, grad_lo, vgrad_lo, vghost_lo;
    bool geometry = false;
    bool prims_current = false;
    bool lsq_shared = false;  // lsqw / lsqd (and their lo parts) hold one row per slot, the same for every cell
    DBuf face_class, face_class_tab;  // float build: class of each face, and each class's row (kFaceClassRow)
    int n_face_classes = 0;           // 0: the face kernels read the per-face arrays
};

// Whether every column c of the rows x N array a (row-major [rows][N]) is
// bitwise equal to column 0, and if so its first column.
template <class T>
bool shared_column(const std::vector<T>& a, int64_t rows, int64_t N, std::vector<T>& col) {
    if (N < 1 || (int64_t)a.size() != rows * N) return false;
    for (int64_t r = 0; r < rows; r++)
        for (int64_t c = 1; c < N; c++)
            if (std::memcmp(&a[r * N + c], &a[r * N], sizeof(T)) != 0) return false;
    col.resize(rows);
    for (int64_t r = 0; r < rows; r++) col[r] = a[r * N];
    return true;
}

// The faces of a uniform lattice fall into a few classes whose geometry, as the
// float kernels read it, is bitwise the same: the normal, the 2-D tangents (t1 x,
// t1 y, t2 z; the 3-D face kernel forms its frame from n), each valid side's
// reconstruction offset (face centre - centroid, the float subtraction the face
// kernel does) and the area (the local time step's).  On success cls holds each face's class and tab one kFaceClassRow row per
// class; false when the faces have more than kMaxFaceClasses distinct rows.
bool face_classes(const std::vector<float>& fc, const std::vector<float>& cc, const Mesh& mesh,
                  std::vector<uint8_t>& cls, std::vector<float>& tab) {
    const int64_t F = mesh.F, N = mesh.N, NT = mesh.NT();
    const bool three = mesh.dim == 3;
    int n = 0, last = 0;  // classes so far; the last face's (neighbouring faces mostly share one)
    cls.assign(F, 0);
    tab.clear();
    for (int64_t f = 0; f < F; f++) {
        float row[kFaceClassRow] = {};
        for (int k = 0; k < 3; k++) row[k] = fc[k * F + f];
        if (!three) { row[3] = fc[3 * F + f]; row[4] = fc[4 * F + f]; row[5] = fc[8 * F + f]; }
        row[12] = fc[12 * F + f];
        const int64_t side[2] = {mesh.left[f], mesh.right[f]};
        for (int sd = 0; sd < 2; sd++) {
            const int64_t c = side[sd];
            if (c >= N) continue;
            for (int k = 0; k < 3; k++) {
                const float a = fc[(9 + k) * F + f], b = cc[k * NT + c];
                row[6 + 3 * sd + k] = a - b;
            }
        }
        auto same = [&](int k) { return std::memcmp(&tab[(size_t)k * kFaceClassRow], row, sizeof(row)) == 0; };
        int k = n > 0 && same(last) ? last : -1;
        for (int j = 0; k < 0 && j < n; j++)
            if (same(j)) k = j;
        if (k < 0) {
            if (n == kMaxFaceClasses) return false;
            tab.insert(tab.end(), row, row + kFaceClassRow);
            k = n++;
        }
        cls[f] = (uint8_t)k;
        last = k;
    }
    return F > 0;
}

ActionKind parse_action_kind(const std::string& t) {
    if (t == "flow_state_copy") return aFlowStateCopy;
    if (t == "internal_copy") return aInternalCopy;
    if (t == "internal_copy_reflect_normal") return aReflectNormal;
    if (t == "internal_vel_copy_reflect") return aVelReflect;
    if (t == "fix_temperature") return aFixTemperature;
    if (t == "subsonic_inflow") return aSubsonicInflow;
    if (t == "subsonic_outflow") return aSubsonicOutflow;
    if (t == "periodic_copy") return aPeriodicCopy;
    if (t == "boundary_layer_profile") return aBoundaryLayer;
    throw ConfigError("Unknown boundary action " + t);
}

// build_boundary_action, boundary.cpp:448-479; a boundary_layer_profile's
// splines go to `profiles` and the action keeps their index.
Action parse_action(const Json& a, std::vector<BoundaryLayerProfile>& profiles) {
    Action out{};
    out.kind = parse_action_kind(a.at("type").as_string());
    auto fs = [&](const Json& j) {
        out.fs[0] = j.at("T").as_double(); out.fs[1] = j.at("p").as_double();
        out.fs[2] = j.at("rho").as_double(); out.fs[3] = j.at("energy").as_double();
        out.fs[4] = j.at("vx").as_double(); out.fs[5] = j.at("vy").as_double();
        out.fs[6] = j.at("vz").as_double();
    };
    if (out.kind == aFlowStateCopy || out.kind == aSubsonicInflow) fs(a.at("flow_state"));
    if (out.kind == aFixTemperature) out.value = a.at("temperature").as_double();
    if (out.kind == aSubsonicOutflow) out.value = a.at("pressure").as_double();
    if (out.kind == aBoundaryLayer) {  // BoundaryLayerProfile ctor, boundary.cpp:48-57
        const Json& pj = a.at("profile");
        const std::vector<double> h = pj.at("height").as_doubles();
        BoundaryLayerProfile bl;
        try {
            bl.vx = NaturalSpline(h, pj.at("v").as_doubles());
            bl.T = NaturalSpline(h, pj.at("T").as_doubles());
        } catch (const std::runtime_error& e) {
            throw ConfigError(std::string("boundary_layer_profile: ") + e.what());
        }
        bl.p = pj.at("p").as_double();
        out.table = (int)profiles.size();
        profiles.push_back(bl);
    }
    return out;
}

}  // namespace

struct ibisgb_ctx {
    std::string err;
    Json config;
    FvParams prm{};
    Mesh mesh;
    std::vector<BoundDev> bounds_host;
    std::vector<BoundaryLayerProfile> profiles;  // tables of the boundary_layer_profile actions

    // steady-state / JFNK settings (SteadyState ctor steady_state.cpp:176-221, Jfnk jfnk.cpp:7-23)
    struct Steady {
        bool configured = false;
        int max_steps = 1000;
        double tolerance = 1e-5;
        bool fgmres = false;
        int max_iters = 50, max_prec_iters = 5;
        double tol = 1e-2, prec_tol = 1e-1;
        int cfl_kind = 0;  // 0 constant, 1 linear_interpolate(step), 2 residual_based
        double cfl = 0.5;
        std::vector<double> cfl_t, cfl_v;
        double rb_threshold = 0.1, rb_power = 0.8, rb_start = 1.0, rb_max = 1e8;
        double rb_prev_cfl = 1.0, rb_prev_res = 1.0;
        double norms[6] = {0, 0, 0, 0, 0, 0}, initial[6] = {0, 0, 0, 0, 0, 0};
        int64_t step = 0;
        bool initialised = false;
    } steady;
    StateBufs sdual;        // dual-number state of the tangent (double geometry from s64)
    DBuf rhs, dU, kv, kw, kr0, kz, kH, kpart, kscal;  // Krylov storage

    // Runge-Kutta settings (RungeKutta ctor, runge_kutta.cpp:21-80)
    bool rk_configured = false;
    StepCtl ctl_host{};
    double dt_init = -1.0;

    // batched ensembles: one control block (and dt_init) per case, the case of
    // every valid cell, and the offsets of each case's cells / faces / ghosts
    int n_cases = 1;
    std::vector<StepCtl> case_ctl;
    std::vector<double> case_dt_init;
    std::vector<int64_t> cell_off, face_off, ghost_off;
    std::vector<StepCtl> last_ctl;
    DBuf case_of;

    cudaStream_t stream = nullptr;
    int device = 0;

    // connectivity and per-cell data shared by all arithmetics
    DBuf cell_face, cell_nbr, outsign, nfaces, left, right, ghost_src, ghost_face, ghost_bound,
        bounds, gfix, feed_off, feed_ghost, vol, inv_vol, inv_vol2;
    DBuf U, k, vsig, ctl, l2, out, branches;
    StateBufs s64, s32, sff;
    std::vector<double> ic_prims;  // host IC primitives (7 x NT), kept until the first update
    bool have_state = false;
    bool k_alias = false;  // stage derivatives share slot 0 (the reference's RungeKutta)
    cudaGraphExec_t graph[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    // launch variants of recon / face / update per precision (autotuned)
    int var[5][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    bool tuned[5] = {false, false, false, false, false};
    double tune_ms[5][3][kNumVariants] = {};
    static int gidx(int prec) {
        switch (prec) {
            case IBISGB_MIXED: return 1;
            case IBISGB_F64_EXACT: return 2;
            case IBISGB_MIXED_GRAD: return 3;
            case IBISGB_MIXED_FF: return 4;
            default: return 0;
        }
    }

    // Fused stage on structured blocks (mixed build, inviscid, second order).
    // The mixed primitives live in two buffers that the fused stages alternate
    // between; prim_cur names the one holding the current state.
    int fused_elig = -1;  // -1 not checked yet, 0 not eligible, 1 eligible
    std::string fused_why;
    StructuredLayout slay;
    DBuf sb_blocks, sb_tiles, sb_face, sb_ghost, prim_alt;
    bool fused_uploaded = false;
    int prim_cur = 0;
    int fused_mode = -1;  // -1 the autotuner decides, 0 off, 1 on
    bool fused_on = false;
    cudaGraphExec_t graph_fused[2] = {nullptr, nullptr};
    double fused_ms = 0.0, generic_ms = 0.0;
    // Plane-marching variant of the fused stage (one 3-D block, TMA-staged
    // planes): the autotuner times it beside the tile kernel and keeps the faster.
    int march_elig = -1;  // -1 not checked yet, 0 not eligible, 1 eligible
    std::string march_why;
    int march_mode = -1;  // -1 the autotuner decides, 0 tile kernel, 1 plane-marching kernel
    int march_kc_req = 0;  // planes per CTA requested (0: tuned)
    bool march_on = false;
    int march_kc = 32;
    double tile_ms = 0.0, march_ms = 0.0;
    TmaMap march_map_prim[2], march_map_cc;
    const void* march_map_base[3] = {nullptr, nullptr, nullptr};
    DBuf march_fault;
    // Per-cell flux path (mixed, inviscid): recon + k_cell_update per stage, on
    // the same alternating primitive buffers and per-parity graphs as the fused stage.
    int cell_mode = -1;  // -1 the autotuner decides, 0 off, 1 on
    bool cell_on = false;
    int cell_var = 0;
    double cell_ms = 0.0;
    DBuf tune_save;
    double last_l2[6] = {0, 0, 0, 0, 0, 0};
    double last_ms = 0.0;

    ~ibisgb_ctx() {
        for (auto& g : graph)
            if (g) cudaGraphExecDestroy(g);
        for (auto& g : graph_fused)
            if (g) cudaGraphExecDestroy(g);
        for (auto& e : pipe_ev)
            if (e) cudaEventDestroy(e);
        if (pipe_h2d) cudaStreamDestroy(pipe_h2d);
        if (pipe_d2h) cudaStreamDestroy(pipe_d2h);
        if (stream) cudaStreamDestroy(stream);
    }

    int nc() const { return mesh.dim + 2; }
    int stages() const { return rk_configured ? ctl_host.stages : 1; }

    void parse_config(const std::string& text) {
        try {
            config = Json::parse(text);
        } catch (const std::exception& e) {
            throw ConfigError(std::string("config.json: ") + e.what());
        }
        try {
            const Json& cf = config.at("convective_flux");  // ConvectiveFlux ctor, convective_flux.cpp:60-82
            std::string ft = cf.at("flux_calculator").at("type").as_string();
            if (ft == "hanel") prm.flux = kHanel;
            else if (ft == "ausmdv") prm.flux = kAusmdv;
            else if (ft == "ldfss2") { prm.flux = kLdfss2; prm.delta = cf.at("flux_calculator").at("delta").as_double(); }
            else if (ft == "rusanov") prm.flux = kRusanov;
            else throw ConfigError("Unknown flux calculator " + ft);
            prm.order = (int)cf.at("reconstruction_order").as_int();
            prm.thermo = kRhoU;
            prm.limiter = 0;
            prm.eps = 1e-25;
            if (prm.order > 1) {
                std::string th = cf.at("thermo_interpolator").as_string();
                if (th == "rho_p") prm.thermo = kRhoP;
                else if (th == "rho_T") prm.thermo = kRhoT;
                else if (th == "rho_u") prm.thermo = kRhoU;
                else if (th == "p_T") prm.thermo = kPT;
                else throw ConfigError("Unknown thermo interpolator " + th);
                std::string lt = cf.at("limiter").at("type").as_string();
                if (lt == "barth_jespersen") { prm.limiter = 1; prm.eps = cf.at("limiter").at("epsilon").as_double(); }
                else if (lt == "unlimited") prm.limiter = 0;
                else throw ConfigError("Unknown limiter " + lt);
            }
            if (prm.order != 1 && prm.order != 2) throw ConfigError("Invalid reconstruction order");
            const Json& vf = config.at("viscous_flux");
            prm.viscous = vf.at("enabled").as_bool() ? 1 : 0;
            prm.signal_factor = vf.at("signal_factor").as_double();
            const Json& gm = config.at("gas_model");  // IdealGas(json), gas_model.h:58-62
            prm.R = gm.at("R").as_double(); prm.Cv = gm.at("Cv").as_double();
            prm.Cp = gm.at("Cp").as_double(); prm.gamma = gm.at("gamma").as_double();
            prm.mu0 = 1.716e-5; prm.T0 = 273.0; prm.Ts = 110.0; prm.Pr = 0.72;
            if (config.contains("transport_properties")) {  // transport_properties.h:91-109
                const Json& tp = config.at("transport_properties");
                const Json& vi = tp.at("viscosity");
                if (vi.at("type").as_string() != "sutherland") throw ConfigError("Unknown viscosity model");
                prm.mu0 = vi.at("mu_0").as_double(); prm.T0 = vi.at("T_0").as_double(); prm.Ts = vi.at("T_s").as_double();
                const Json& kc = tp.at("thermal_conductivity");
                if (kc.at("type").as_string() != "constant_prandtl_number") throw ConfigError("Unknown thermal conductivity model");
                prm.Pr = kc.at("Pr").as_double();
            }
            const Json& grid = config.at("grid");
            if (grid.contains("motion") && grid.at("motion").contains("enabled") &&
                grid.at("motion").at("enabled").as_bool())
                throw ConfigError("moving grids are not supported");
            renumber_mode = 0;
            if (grid.contains("renumber")) {  // not a reference key: the internal cell order
                const std::string r = grid.at("renumber").as_string();
                if (r == "auto") renumber_mode = 0;
                else if (r == "rcm") renumber_mode = 1;
                else if (r == "none") renumber_mode = 2;
                else throw ConfigError("grid.renumber must be auto, rcm or none");
            }
            shared_tables_mode = 0;
            if (grid.contains("geometry_tables")) {  // not a reference key: the layout of the geometry tables
                const std::string t = grid.at("geometry_tables").as_string();
                if (t == "auto") shared_tables_mode = 0;
                else if (t == "per_element") shared_tables_mode = 1;
                else throw ConfigError("grid.geometry_tables must be auto or per_element");
            }
            prm.fR = (float)prm.R; prm.fCv = (float)prm.Cv; prm.fCp = (float)prm.Cp;
            prm.fgamma = (float)prm.gamma; prm.fgR = prm.fgamma * prm.fR; prm.feps = (float)prm.eps;
            prm.fdelta = (float)prm.delta; prm.fmu0 = (float)prm.mu0; prm.fT0 = (float)prm.T0;
            prm.fTs = (float)prm.Ts; prm.fPr = (float)prm.Pr; prm.inv_Cv = 1.0 / prm.Cv;
            prm.finv_Cv = (float)prm.inv_Cv;
            auto lo = [](double d, float f) { return (float)(d - (double)f); };
            prm.loR = lo(prm.R, prm.fR); prm.loCv = lo(prm.Cv, prm.fCv); prm.loCp = lo(prm.Cp, prm.fCp);
            prm.logamma = lo(prm.gamma, prm.fgamma); prm.logR = lo(prm.gamma * prm.R, prm.fgR);
            prm.lodelta = lo(prm.delta, prm.fdelta); prm.lomu0 = lo(prm.mu0, prm.fmu0);
            prm.loT0 = lo(prm.T0, prm.fT0); prm.loTs = lo(prm.Ts, prm.fTs); prm.loPr = lo(prm.Pr, prm.fPr);
            prm.loinv_Cv = lo(prm.inv_Cv, prm.finv_Cv);
            const Json& solver = config.at("solver");
            if (solver.at("name").as_string() == "runge_kutta") parse_rk(solver);
            if (solver.at("name").as_string() == "steady_state") parse_steady(solver);
        } catch (const ConfigError&) {
            throw;
        } catch (const std::exception& e) {
            throw ConfigError(std::string("config.json: ") + e.what());
        }
    }

    void parse_rk(const Json& sc) {
        StepCtl& c = ctl_host;
        const Json& bt = sc.at("butcher_tableau");
        auto b = bt.at("b").as_doubles();
        if (b.empty() || b.size() > (size_t)kMaxStages) throw ConfigError("unsupported Butcher tableau size");
        c.stages = (int)b.size();
        const auto& rows = bt.at("a").elements();
        for (int i = 1; i < c.stages; i++) {
            auto row = rows.at(i - 1).as_doubles();
            for (int j = 0; j < i && j < (int)row.size(); j++) c.a[i][j] = row[j];
            // the stage combinations skip a(i, j) < 1e-14 (runge_kutta.cpp:161-168)
            for (int j = 0; j < i; j++)
                if (!(c.a[i][j] < 1e-14)) c.a_used[i] |= 1u << j;
        }
        for (int i = 0; i < c.stages; i++) c.b[i] = b[i];
        const Json& cfl = sc.at("cfl");  // make_cfl_schedule, cfl.cpp:157-169
        std::string ct = cfl.at("type").as_string();
        if (ct == "constant") {
            c.cfl = cfl.at("value").as_double();
        } else if (ct == "linear_interpolate") {
            auto ts = cfl.at("times").as_doubles(), vs = cfl.at("cfls").as_doubles();
            if (ts.size() != vs.size() || ts.empty() || ts.size() > 16) throw ConfigError("bad cfl schedule");
            c.n_cfl = (int)ts.size();
            for (size_t i = 0; i < ts.size(); i++) { c.cfl_t[i] = ts[i]; c.cfl_v[i] = vs[i]; }
        } else {
            throw ConfigError("unsupported CFL schedule for runge_kutta: " + ct);
        }
        c.max_time = sc.at("max_time").as_double();
        c.plot_frequency = sc.at("plot_frequency").as_double();
        dt_init = sc.at("dt_init").as_double();
        // extension: "stage_derivatives": "aliased" reproduces the reference's
        // RungeKutta, whose stage derivatives are copies of one Kokkos View and so
        // share one array (runge_kutta.cpp:47-48); "separate" (the default) keeps
        // one array per stage, as the tableau is written
        if (sc.contains("stage_derivatives")) {
            const std::string sd = sc.at("stage_derivatives").as_string();
            if (sd != "aliased" && sd != "separate") throw ConfigError("stage_derivatives must be aliased or separate");
            k_alias = sd == "aliased";
        }
        rk_configured = true;
    }

    void parse_steady(const Json& sc) {
        Steady& st = steady;
        st.max_steps = (int)sc.at("max_steps").as_int();
        st.tolerance = sc.at("tolerance").as_double();
        const Json& ls = sc.at("linear_solver");  // make_linear_solver, gmres.cpp:305-318
        std::string lt = ls.at("type").as_string();
        if (lt == "gmres") {
            st.max_iters = (int)ls.at("max_iters").as_int();
            st.tol = ls.at("tol").as_double();
        } else if (lt == "fgmres") {
            st.fgmres = true;
            st.max_iters = (int)ls.at("max_iters").as_int();
            st.tol = ls.at("tolerance").as_double();
            st.max_prec_iters = (int)ls.at("max_preconditioner_iters").as_int();
            st.prec_tol = ls.at("preconditioner_tolerance").as_double();
        } else {
            throw ConfigError("Unknown linear solver " + lt);
        }
        const Json& cfl = sc.at("cfl");  // make_cfl_schedule, cfl.cpp:157-169
        if (cfl.is_number()) {
            st.cfl = cfl.as_double();
        } else {
            std::string ct = cfl.at("type").as_string();
            if (ct == "constant") {
                st.cfl = cfl.at("value").as_double();
            } else if (ct == "linear_interpolate") {
                st.cfl_kind = 1;
                st.cfl_t = cfl.at("times").as_doubles();
                st.cfl_v = cfl.at("cfls").as_doubles();
            } else if (ct == "residual_based") {
                st.cfl_kind = 2;
                st.rb_threshold = cfl.at("growth_threshold").as_double();
                st.rb_power = cfl.at("power").as_double();
                st.rb_start = cfl.at("start_cfl").as_double();
                st.rb_max = cfl.at("max_cfl").as_double();
                st.rb_prev_cfl = st.rb_start;
            } else {
                throw ConfigError("Unknown CFL schedule " + ct);
            }
        }
        st.configured = true;
    }

    std::vector<BoundarySpec> boundary_specs() {
        std::vector<BoundarySpec> out;
        for (const auto& [tag, b] : config.at("grid").at("boundaries").items()) {
            BoundarySpec s;
            s.tag = tag;
            s.ghost_cells = b.at("ghost_cells").as_bool();
            for (const Json& a : b.at("pre_reconstruction").elements()) {
                if (a.at("type").as_string() == "periodic_copy") {
                    s.periodic = true;
                    s.partner = a.at("partner").as_string();
                    auto off = a.at("offset").as_doubles();
                    for (int d = 0; d < 3; d++) s.offset[d] = off.at(d);
                }
            }
            out.push_back(s);
        }
        return out;
    }

    void build(const GridInput& in) {
        if (in.dim != 2 && in.dim != 3) throw ConfigError("grid dimension must be 2 or 3");
        prm.dim = in.dim;
        std::vector<BoundarySpec> specs = boundary_specs();
        build_mesh(in, specs, prm.viscous || prm.order > 1, mesh);
        check_index_range();
        choose_numbering();
        // the fast kernels visit at most 6 face slots per cell in 3-D, 4 in 2-D (the
        // most faces of any element type the reference reads)
        if (mesh.MF > (in.dim == 3 ? 6 : 4)) throw ConfigError("a cell has more faces than any supported element");
        // every face needs two sides (boundaries without ghost cells are not supported)
        for (int64_t f = 0; f < mesh.F; f++)
            if (mesh.left[f] < 0 || mesh.right[f] < 0)
                throw ConfigError("a boundary face has no ghost cell (ghost_cells false is not supported)");
        for (const auto& b : mesh.bounds) {  // BoundaryCondition ctor, boundary.cpp:494-515
            const Json& bj = config.at("grid").at("boundaries").at(b.tag);
            BoundDev d{};
            for (const Json& a : bj.at("pre_reconstruction").elements()) {
                if (d.n_pre == kMaxActions) throw ConfigError("too many boundary actions");
                d.pre[d.n_pre++] = parse_action(a, profiles);
            }
            for (const Json& a : bj.at("pre_viscous_grad").elements()) {
                if (d.n_visc == kMaxActions) throw ConfigError("too many boundary actions");
                d.visc[d.n_visc++] = parse_action(a, profiles);
            }
            // post_convective_flux (build_flux_action, boundary.cpp:481-492): each
            // action overwrites the face flux, so the last one is the one that counts
            for (const Json& a : bj.at("post_convective_flux").elements()) {
                const std::string t = a.at("type").as_string();
                if (t != "constant_flux") throw ConfigError("Unknown flux action " + t);
                const Json& fs = a.at("flow_state");
                const char* keys[7] = {"T", "p", "rho", "energy", "vx", "vy", "vz"};
                for (int q = 0; q < 7; q++) d.cfs[q] = fs.at(keys[q]).as_double();
                d.cflux = 1;
                prm.cflux = 1;
            }
            bounds_host.push_back(d);
        }
    }

    // ----- internal cell / face numbering ---------------------------------------
    // The device arrays are in an internal order (reverse Cuthill-McKee of the
    // cell graph, faces by their lower then higher cell) when that shortens the
    // cell graph's bandwidth; every array and id that crosses the ABI stays in the
    // reference's numbering (grid.h:113-133).  Per-cell and per-face arithmetic and
    // summation orders are unchanged, so the results are the same bits.
    int renumber_mode = 0;  // 0 auto, 1 rcm, 2 none
    // 0 auto: on a uniform lattice, the least-squares weights and face offsets stored
    // once per slot (every cell's bitwise the same) and, for the float build, each
    // face's normal and side offsets as a class index into a small table; 1: always
    // per cell and per face
    int shared_tables_mode = 0;
    MeshNumbering num;
    int64_t bandwidth_ref = 0, bandwidth_internal = 0;
    DBuf d_cell_to_new, d_cell_to_ref, map_a, map_b;
    bool renumbered() const { return num.active(); }

    void choose_numbering() {
        bandwidth_ref = bandwidth_internal = cell_bandwidth(mesh);
        if (renumber_mode == 2 || mesh.N < 2) return;
        if (renumber_mode == 0) {  // auto: unstructured grids only (quad / hex blocks keep their lattice)
            bool all_lattice = true;
            for (int64_t c = 0; c < mesh.N && all_lattice; c++)
                all_lattice = mesh.cell_kind[c] == (mesh.dim == 2 ? kQuad : kHex);
            if (all_lattice) return;
        }
        std::vector<int64_t> order = rcm_cell_order(mesh);
        Mesh trial = mesh;
        MeshNumbering tn;
        renumber_mesh(trial, order, tn);
        const int64_t bw = cell_bandwidth(trial);
        if (renumber_mode == 0 && 2 * bw > bandwidth_ref) return;  // auto: only for a 2x shorter bandwidth
        mesh = std::move(trial);
        num = std::move(tn);
        bandwidth_internal = bw;
    }

    void ensure_maps() {
        if (!renumbered() || d_cell_to_new.p) return;
        const int64_t N = mesh.N;
        std::vector<int32_t> a(N), b(N);
        for (int64_t i = 0; i < N; i++) {
            a[i] = (int32_t)num.cell_ref_of_new[i];
            b[i] = (int32_t)num.cell_new_of_ref[i];
        }
        d_cell_to_new.alloc(sizeof(int32_t) * N);
        d_cell_to_ref.alloc(sizeof(int32_t) * N);
        CUDA_OK(cudaMemcpyAsync(d_cell_to_new.p, a.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice, stream));
        CUDA_OK(cudaMemcpyAsync(d_cell_to_ref.p, b.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice, stream));
        CUDA_OK(cudaStreamSynchronize(stream));
    }
    // device rows (N x w): reference numbering -> internal (to_internal) or back
    void map_rows_device(const double* src, double* dst, int w, bool to_internal) {
        ensure_maps();
        launch_gather_rows(dst, src, (to_internal ? d_cell_to_new : d_cell_to_ref).as<int32_t>(), (int)mesh.N, w,
                           stream);
        CUDA_OK(cudaGetLastError());
    }
    // host per-cell values (N x w rows) between the numberings
    template <class T>
    void map_rows_host(const T* src, T* dst, int w, bool to_internal) const {
        const auto& m = to_internal ? num.cell_ref_of_new : num.cell_new_of_ref;
        for (int64_t i = 0; i < mesh.N; i++)
            for (int q = 0; q < w; q++) dst[i * w + q] = src[m[i] * w + q];
    }
    int64_t cell_id_to_ref(int64_t c) const {
        return (renumbered() && c >= 0 && c < mesh.N) ? num.cell_ref_of_new[c] : c;
    }
    int64_t face_id_to_ref(int64_t f) const { return (renumbered() && f >= 0) ? num.face_ref_of_new[f] : f; }

    // the residual / tangent / adjoint entry points on rows in the reference numbering
    void residual_rows(int prec, double* out_rows) {
        if (!renumbered()) return residual(prec, out_rows, true);
        map_b.alloc(sizeof(double) * nvars());
        residual(prec, map_b.as<double>(), true);
        map_rows_device(map_b.as<double>(), out_rows, nc(), false);
    }
    void jvp_rows(const double* v, double* out_rows, double inv_dt_star, bool reconstruct) {
        if (!renumbered()) return jvp(v, out_rows, inv_dt_star, reconstruct);
        map_a.alloc(sizeof(double) * nvars());
        map_b.alloc(sizeof(double) * nvars());
        map_rows_device(v, map_a.as<double>(), nc(), true);
        jvp(map_a.as<double>(), map_b.as<double>(), inv_dt_star, reconstruct);
        map_rows_device(map_b.as<double>(), out_rows, nc(), false);
    }
    void vjp_rows(const double* w, double* out_rows, double* ghost_out, bool reconstruct) {
        if (!renumbered()) return vjp(w, out_rows, ghost_out, reconstruct);
        map_a.alloc(sizeof(double) * nvars());
        map_b.alloc(sizeof(double) * nvars());
        map_rows_device(w, map_a.as<double>(), nc(), true);
        vjp(map_a.as<double>(), map_b.as<double>(), ghost_out, reconstruct);  // ghost ids are not renumbered
        map_rows_device(map_b.as<double>(), out_rows, nc(), false);
    }
    void adjoint_step_rows(const double* g, double* lam, double cfl, ibisgb_adjoint_status* st) {
        if (!renumbered()) return adjoint_step(g, lam, cfl, st);
        map_a.alloc(sizeof(double) * nvars());
        map_b.alloc(sizeof(double) * nvars());
        map_rows_device(g, map_a.as<double>(), nc(), true);
        map_rows_device(lam, map_b.as<double>(), nc(), true);
        adjoint_step(map_a.as<double>(), map_b.as<double>(), cfl, st);
        map_rows_device(map_b.as<double>(), lam, nc(), false);
        CUDA_OK(cudaStreamSynchronize(stream));
    }

    void check_index_range() const {
        const int64_t N = mesh.N, F = mesh.F, G = mesh.G;
        const int64_t lim = std::numeric_limits<int>::max();
        if (15 * N >= lim || 5 * F >= lim || 7 * (N + G) >= lim || 3 * (int64_t)mesh.MF * N >= lim)
            throw ConfigError("grid too large for 32-bit device indexing");
    }

    // Batched ensemble from single-case contexts (see ibisgb_batch_create).
    void merge(ibisgb_ctx* const* cs, int n) {
        std::vector<const Mesh*> parts;
        for (int i = 0; i < n; i++) {
            if (!cs[i]) throw ArgError("case " + std::to_string(i) + " is null");
            const ibisgb_ctx& c = *cs[i];
            if (c.n_cases != 1) throw ArgError("case " + std::to_string(i) + " is itself a batch");
            if (!same_scheme(cs[0]->prm, c.prm))
                throw ConfigError("case " + std::to_string(i) +
                                  ": cases of a batch must share flux, reconstruction, gas and transport settings");
            if (!c.rk_configured || !cs[0]->rk_configured || !same_tableau(cs[0]->ctl_host, c.ctl_host) ||
                c.k_alias != cs[0]->k_alias)
                throw ConfigError("case " + std::to_string(i) +
                                  ": cases of a batch must use runge_kutta with the same Butcher tableau and "
                                  "stage_derivatives");
            parts.push_back(&c.mesh);
        }
        const ibisgb_ctx& a = *cs[0];
        config = a.config;
        prm = a.prm;
        rk_configured = true;
        ctl_host = a.ctl_host;
        dt_init = a.dt_init;
        k_alias = a.k_alias;
        std::vector<int64_t> bound_off;
        try {
            merge_meshes(parts, mesh, cell_off, ghost_off, face_off, bound_off);
        } catch (const std::runtime_error& e) {
            throw ConfigError(e.what());
        }
        check_index_range();
        bandwidth_ref = bandwidth_internal = 0;
        bool any = false;
        for (int i = 0; i < n; i++) any = any || cs[i]->num.active();
        if (any) {  // each case's numbering at its offsets (merge_meshes keeps the cases' own orders)
            num.cell_ref_of_new.resize(mesh.N);
            num.cell_new_of_ref.resize(mesh.N);
            num.face_ref_of_new.resize(mesh.F);
            num.face_new_of_ref.resize(mesh.F);
            for (int i = 0; i < n; i++) {
                const MeshNumbering& ci = cs[i]->num;
                for (int64_t c = 0; c < cell_off[i + 1] - cell_off[i]; c++) {
                    num.cell_ref_of_new[cell_off[i] + c] = cell_off[i] + (ci.active() ? ci.cell_ref_of_new[c] : c);
                    num.cell_new_of_ref[cell_off[i] + c] = cell_off[i] + (ci.active() ? ci.cell_new_of_ref[c] : c);
                }
                for (int64_t f = 0; f < face_off[i + 1] - face_off[i]; f++) {
                    num.face_ref_of_new[face_off[i] + f] = face_off[i] + (ci.active() ? ci.face_ref_of_new[f] : f);
                    num.face_new_of_ref[face_off[i] + f] = face_off[i] + (ci.active() ? ci.face_new_of_ref[f] : f);
                }
            }
        }
        prm.cflux = 0;
        for (int i = 0; i < n; i++) {
            // profile tables of case i follow those of the cases before it
            const int t0 = (int)profiles.size();
            profiles.insert(profiles.end(), cs[i]->profiles.begin(), cs[i]->profiles.end());
            for (BoundDev d : cs[i]->bounds_host) {
                for (int k = 0; k < d.n_pre; k++) d.pre[k].table += t0;
                for (int k = 0; k < d.n_visc; k++) d.visc[k].table += t0;
                bounds_host.push_back(d);
            }
            prm.cflux |= cs[i]->prm.cflux;
            case_ctl.push_back(cs[i]->ctl_host);
            case_dt_init.push_back(cs[i]->dt_init);
        }
        n_cases = n;
    }

    static bool same_scheme(const FvParams& a, const FvParams& b) {
        return a.dim == b.dim && a.flux == b.flux && a.thermo == b.thermo && a.order == b.order &&
               a.limiter == b.limiter && a.viscous == b.viscous && a.eps == b.eps && a.delta == b.delta &&
               a.signal_factor == b.signal_factor && a.R == b.R && a.Cv == b.Cv && a.Cp == b.Cp &&
               a.gamma == b.gamma && a.mu0 == b.mu0 && a.T0 == b.T0 && a.Ts == b.Ts && a.Pr == b.Pr;
    }
    static bool same_tableau(const StepCtl& a, const StepCtl& b) {
        if (a.stages != b.stages) return false;
        for (int i = 0; i < a.stages; i++) {
            if (a.b[i] != b.b[i]) return false;
            for (int j = 0; j < i; j++)
                if (a.a[i][j] != b.a[i][j]) return false;
        }
        return true;
    }

    // Device buffers are created on the first call that needs the GPU, so that
    // the host-side numbering and geometry can be inspected without one.
    bool uploaded = false;
    void ensure_device() {
        if (uploaded) return;
        upload_mesh();
        uploaded = true;
    }

    void upload_mesh() {
        CUDA_OK(cudaGetDevice(&device));
        CUDA_OK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        const int64_t N = mesh.N, F = mesh.F, G = mesh.G, MF = mesh.MF;
        std::vector<int> cf(MF * N, -1), nb(MF * N, -1), nfa(N);
        std::vector<signed char> os(MF * N, 0);
        for (int64_t c = 0; c < N; c++) {
            nfa[c] = mesh.nfaces[c];
            for (int64_t k = 0; k < MF; k++) {
                cf[k * N + c] = (int)mesh.cell_face[c * MF + k];
                nb[k * N + c] = (int)mesh.cell_nbr[c * MF + k];
                os[k * N + c] = mesh.outsign[c * MF + k];
            }
        }
        upload(cell_face, cf, stream); upload(cell_nbr, nb, stream); upload(outsign, os, stream);
        upload(nfaces, nfa, stream);
        std::vector<int> l(F), r(F);
        for (int64_t f = 0; f < F; f++) { l[f] = (int)mesh.left[f]; r[f] = (int)mesh.right[f]; }
        upload(left, l, stream); upload(right, r, stream);
        std::vector<int> gs(G), gf(G), gb(G);
        for (int64_t g = 0; g < G; g++) {
            gs[g] = (int)mesh.ghost_src[g]; gf[g] = (int)mesh.ghost_face[g]; gb[g] = (int)mesh.ghost_bound[g];
        }
        upload(ghost_src, gs, stream); upload(ghost_face, gf, stream); upload(ghost_bound, gb, stream);
        upload(bounds, bounds_host, stream);
        if (!profiles.empty()) {
            // boundary-layer ghost states (boundary.cpp:59-94): T(y), p, rho = p / (R T),
            // e = Cv T, vx(y) at the ghost centroid's height y
            const size_t nt = profiles.size();
            std::vector<double> t(nt * 5 * (size_t)std::max<int64_t>(G, 1), 0.0);
            for (int64_t g = 0; g < G; g++) {
                const BoundDev& d = bounds_host[gb[g]];
                auto fill = [&](const Action& a) {
                    if (a.kind != aBoundaryLayer) return;
                    const BoundaryLayerProfile& bl = profiles[a.table];
                    const double y = mesh.ccy[N + g];
                    double* o = t.data() + (size_t)a.table * 5 * G;
                    const double T = bl.T(y);
                    o[g] = T;
                    o[G + g] = bl.p;
                    o[2 * G + g] = bl.p / (prm.R * T);
                    o[3 * G + g] = prm.Cv * T;
                    o[4 * G + g] = bl.vx(y);
                };
                for (int k = 0; k < d.n_pre; k++) fill(d.pre[k]);
                for (int k = 0; k < d.n_visc; k++) fill(d.visc[k]);
            }
            upload(gfix, t, stream);
        }
        // ghosts fed by each valid cell (CSR)
        std::vector<int> off(N + 1, 0), fg(G);
        for (int64_t g = 0; g < G; g++) off[gs[g] + 1]++;
        for (int64_t c = 0; c < N; c++) off[c + 1] += off[c];
        std::vector<int> cur(off.begin(), off.end() - 1);
        for (int64_t g = 0; g < G; g++) fg[cur[gs[g]]++] = (int)g;
        upload(feed_off, off, stream); upload(feed_ghost, fg, stream);
        upload_volumes();
        U.alloc(sizeof(double) * nc() * N);
        k.alloc(sizeof(double) * nc() * N * stages());
        vsig.alloc(sizeof(double) * F);
        CUDA_OK(cudaMemsetAsync(vsig.p, 0, sizeof(double) * F, stream));
        ctl.alloc(sizeof(StepCtl) * n_cases);
        if (n_cases > 1) {
            std::vector<int> co(N);
            for (int c = 0; c < n_cases; c++)
                for (int64_t i = cell_off[c]; i < cell_off[c + 1]; i++) co[i] = c;
            upload(case_of, co, stream);
        }
        l2.alloc(sizeof(double) * (6 + 6 * 304));
        CUDA_OK(cudaStreamSynchronize(stream));
    }

    void upload_volumes() {
        const int64_t N = mesh.N;
        std::vector<double> v(mesh.volume.begin(), mesh.volume.begin() + N);
        upload(vol, v, stream);
        for (auto& x : v) x = 1.0 / x;
        upload(inv_vol, v, stream);
        // 1/volume as two floats whose sum is it to ~2^-48 (the mixed build's residual scaling)
        std::vector<float> p(2 * (size_t)N);
        for (int64_t c = 0; c < N; c++) {
            p[2 * c] = (float)v[c];
            p[2 * c + 1] = (float)(v[c] - (double)p[2 * c]);
        }
        upload(inv_vol2, p, stream);
        CUDA_OK(cudaStreamSynchronize(stream));
    }

    // Replaces the grid geometry (face rows 13 x F: n, t1, t2, centre, area; cell
    // rows 4 x (N+G): centroid, volume; the layouts of dumps 6 and 7, reference
    // numbering) and forms the least-squares factors again from the centroids.
    // The connectivity and the boundary-layer profile's ghost states stay; the
    // structured-block stages, which hold their own lattice geometry, are switched off.
    void set_geometry(const double* face, const double* cell) {
        if (n_cases > 1) throw StateError("a batch's geometry belongs to its cases");
        const int64_t N = mesh.N, F = mesh.F, NT = mesh.NT();
        std::vector<double>* fa[13] = {&mesh.nx, &mesh.ny, &mesh.nz, &mesh.t1x, &mesh.t1y, &mesh.t1z,
                                       &mesh.t2x, &mesh.t2y, &mesh.t2z, &mesh.fcx, &mesh.fcy, &mesh.fcz, &mesh.area};
        std::vector<double>* ca[4] = {&mesh.ccx, &mesh.ccy, &mesh.ccz, &mesh.volume};
        for (int q = 0; q < 13; q++)
            for (int64_t f = 0; f < F; f++) (*fa[q])[f] = face[q * F + (renumbered() ? num.face_ref_of_new[f] : f)];
        for (int q = 0; q < 4; q++)
            for (int64_t c = 0; c < NT; c++) {
                if (q == 3 && c >= N) continue;  // ghost volumes are not inputs
                (*ca[q])[c] = cell[q * NT + (c < N ? cell_id_to_ref(c) : c)];
            }
        if (!mesh.r.empty()) compute_lsq(mesh);
        s64.geometry = s32.geometry = sff.geometry = false;
        s64.prims_current = s32.prims_current = sff.prims_current = false;
        fused_elig = march_elig = 0;
        fused_on = false;
        fused_why = march_why = "the geometry was replaced (ibisgb_set_geometry)";
        if (uploaded) upload_volumes();
    }

    template <class Gm>
    void upload_geometry(StateBufs& s, bool with_lo = false) {
        if (s.geometry) return;
        if (with_lo) {  // what the float copies of the geometry leave out
            const int64_t NT = mesh.NT(), F = mesh.F;
            auto lo = [](double d) { return (float)(d - (double)(float)d); };
            std::vector<float> cl(3 * NT), fl(13 * F);
            for (int64_t c = 0; c < NT; c++) {
                cl[c] = lo(mesh.ccx[c]); cl[NT + c] = lo(mesh.ccy[c]); cl[2 * NT + c] = lo(mesh.ccz[c]);
            }
            const std::vector<double>* fa[13] = {&mesh.nx, &mesh.ny, &mesh.nz, &mesh.t1x, &mesh.t1y, &mesh.t1z,
                                                 &mesh.t2x, &mesh.t2y, &mesh.t2z, &mesh.fcx, &mesh.fcy, &mesh.fcz,
                                                 &mesh.area};
            for (int q = 0; q < 13; q++)
                for (int64_t f = 0; f < F; f++) fl[q * F + f] = lo((*fa[q])[f]);
            upload(s.cc_lo, cl, stream); upload(s.face_lo, fl, stream);
            s.prim_lo.alloc(sizeof(float) * 7 * NT);
            s.flux_lo.alloc(sizeof(float) * nc() * F);
            s.grad_lo.alloc(sizeof(float) * 16 * mesh.N);
            s.vgrad_lo.alloc(sizeof(float) * 12 * mesh.N);
            s.vghost_lo.alloc(sizeof(float) * 5 * std::max<int64_t>(mesh.G, 1));
        }
        const int64_t N = mesh.N, NT = mesh.NT(), F = mesh.F;
        std::vector<Gm> cc(3 * NT), r(6 * N, Gm(0)), fc(13 * F);
        for (int64_t c = 0; c < NT; c++) { cc[c] = (Gm)mesh.ccx[c]; cc[NT + c] = (Gm)mesh.ccy[c]; cc[2 * NT + c] = (Gm)mesh.ccz[c]; }
        if (!mesh.r.empty())
            for (int64_t c = 0; c < N; c++)
                for (int q = 0; q < 6; q++) r[q * N + c] = (Gm)mesh.r[c * 6 + q];
        const std::vector<double>* fa[13] = {&mesh.nx, &mesh.ny, &mesh.nz, &mesh.t1x, &mesh.t1y, &mesh.t1z,
                                             &mesh.t2x, &mesh.t2y, &mesh.t2z, &mesh.fcx, &mesh.fcy, &mesh.fcz, &mesh.area};
        for (int q = 0; q < 13; q++)
            for (int64_t f = 0; f < F; f++) fc[q * F + f] = (Gm)(*fa[q])[f];
        upload(s.cc, cc, stream); upload(s.r, r, stream); upload(s.face, fc, stream);
        // least-squares weights per neighbour slot and, for the float builds, the
        // limiter's face offsets per face slot: coalesced instead of gathered
        const int64_t MF = mesh.MF, rows = 3 * MF;
        auto lo = [](double d) { return (float)(d - (double)(float)d); };
        std::vector<Gm> w, d;
        std::vector<float> wl, dl;
        if (!mesh.lsqw.empty()) {
            w.assign(mesh.lsqw.begin(), mesh.lsqw.end());
            if (with_lo) {
                wl.resize(mesh.lsqw.size());
                for (size_t q = 0; q < wl.size(); q++) wl[q] = lo(mesh.lsqw[q]);
            }
        }
        if (sizeof(Gm) == sizeof(float) && prm.order == 2) {
            d.assign(rows * N, Gm(0));
            const std::vector<double>* fcs[3] = {&mesh.fcx, &mesh.fcy, &mesh.fcz};
            const std::vector<double>* ccs[3] = {&mesh.ccx, &mesh.ccy, &mesh.ccz};
            dl.assign(with_lo ? rows * N : 0, 0.f);
            for (int64_t c = 0; c < N; c++)
                for (int64_t k = 0; k < mesh.nfaces[c]; k++) {
                    const int64_t f = mesh.cell_face[c * MF + k];
                    for (int a = 0; a < 3; a++) {
                        const double x = (*fcs[a])[f] - (*ccs[a])[c];
                        d[(a * MF + k) * N + c] = (Gm)x;
                        if (with_lo) dl[(a * MF + k) * N + c] = lo(x);
                    }
                }
        }
        // On a uniform lattice every cell's tables are bitwise the same: keep one
        // row per slot, read by every thread at the same address.  The values, and
        // so the results, do not change.
        std::vector<Gm> w1, d1;
        std::vector<float> wl1, dl1;
        s.lsq_shared = shared_tables_mode == 0 && !w.empty() && shared_column(w, rows, N, w1) &&
                       (d.empty() || shared_column(d, rows, N, d1)) &&
                       (wl.empty() || shared_column(wl, rows, N, wl1)) &&
                       (dl.empty() || shared_column(dl, rows, N, dl1));
        if (!w.empty()) upload(s.lsqw, s.lsq_shared ? w1 : w, stream);
        if (!d.empty()) upload(s.lsqd, s.lsq_shared ? d1 : d, stream);
        if (!wl.empty()) upload(s.lsqw_lo, s.lsq_shared ? wl1 : wl, stream);
        if (!dl.empty()) upload(s.lsqd_lo, s.lsq_shared ? dl1 : dl, stream);
        if constexpr (sizeof(Gm) == sizeof(float)) {
            s.n_face_classes = 0;
            std::vector<uint8_t> fcls;
            std::vector<float> ftab;
            if (shared_tables_mode == 0 && !with_lo && face_classes(fc, cc, mesh, fcls, ftab)) {
                upload(s.face_class, fcls, stream);
                upload(s.face_class_tab, ftab, stream);
                s.n_face_classes = (int)(ftab.size() / kFaceClassRow);
            }
        }
        size_t P = sizeof(Gm);
        s.prim.alloc(P * 7 * NT);
        s.vghost.alloc(P * 5 * std::max<int64_t>(mesh.G, 1));
        s.grad.alloc(P * 16 * N);  // 15 x N, or the mixed build's 16 packed floats per cell
        s.phi.alloc(P * 5 * N);
        if (s.phi.p) CUDA_OK(cudaMemsetAsync(s.phi.p, 0, P * 5 * N, stream));  // 2-D leaves the fifth row unwritten
        s.vgrad.alloc(P * 12 * N);
        s.flux.alloc(P * nc() * F);
        s.geometry = true;
        CUDA_OK(cudaStreamSynchronize(stream));
    }

    static bool is_mixed(int prec) { return prec == IBISGB_MIXED; }
    static bool is_ff(int prec) { return prec == IBISGB_MIXED_FF; }
    // float state and geometry arrays (MIXED, and MIXED_FF with its lo companions)
    static bool float_storage(int prec) { return prec == IBISGB_MIXED || prec == IBISGB_MIXED_FF; }
    StateBufs& bufs(int prec) { return is_mixed(prec) ? s32 : (is_ff(prec) ? sff : s64); }
    KernelOps ops(int prec) const {
        if (prec == IBISGB_MIXED) return kernels_mixed();
        if (prec == IBISGB_F64_EXACT) return kernels_f64_exact();
        if (prec == IBISGB_MIXED_GRAD) return kernels_mixed_grad();
        if (prec == IBISGB_MIXED_FF) return kernels_mixed_ff();
        return kernels_f64();
    }

    DevView view(int prec) {
        StateBufs& s = bufs(prec);
        DevView v{};
        v.dim = mesh.dim; v.N = (int)mesh.N; v.G = (int)mesh.G; v.F = (int)mesh.F; v.MF = mesh.MF;
        v.NT = (int)mesh.NT();
        v.cell_face = cell_face.as<int>(); v.cell_nbr = cell_nbr.as<int>();
        v.outsign = outsign.as<signed char>(); v.nfaces = nfaces.as<int>();
        v.left = left.as<int>(); v.right = right.as<int>();
        v.ghost_src = ghost_src.as<int>(); v.ghost_face = ghost_face.as<int>();
        v.ghost_bound = ghost_bound.as<int>(); v.bounds = bounds.as<BoundDev>(); v.gfix = gfix.as<double>();
        v.feed_off = feed_off.as<int>(); v.feed_ghost = feed_ghost.as<int>();
        v.cc = s.cc.p; v.r = s.r.p; v.face = s.face.p; v.vol = vol.as<double>();
        v.inv_vol = inv_vol.as<double>(); v.inv_vol2 = inv_vol2.as<float2>(); v.lsqw = s.lsqw.p;
        v.lsqd = s.lsqd.p;
        v.lsq_shared = s.lsq_shared ? 1 : 0;
        v.face_class = s.n_face_classes ? s.face_class.as<uint8_t>() : nullptr;
        v.face_class_tab = s.n_face_classes ? s.face_class_tab.as<float>() : nullptr;
        v.prim = (is_mixed(prec) && prim_cur) ? prim_alt.p : s.prim.p;
        v.vghost = s.vghost.p; v.grad = s.grad.p; v.phi = s.phi.p;
        v.vgrad = s.vgrad.p; v.flux = s.flux.p; v.vsig = vsig.as<double>();
        v.prim_lo = s.prim_lo.as<float>(); v.cc_lo = s.cc_lo.as<float>();
        v.face_lo = s.face_lo.as<float>(); v.flux_lo = s.flux_lo.as<float>();
        v.lsqw_lo = s.lsqw_lo.as<float>(); v.lsqd_lo = s.lsqd_lo.as<float>(); v.grad_lo = s.grad_lo.as<float>();
        v.vgrad_lo = s.vgrad_lo.as<float>(); v.vghost_lo = s.vghost_lo.as<float>();
        v.U = U.as<double>(); v.k = k.as<double>(); v.ctl = ctl.as<StepCtl>();
        v.k_alias = k_alias ? 1 : 0;
        v.case_of = n_cases > 1 ? case_of.as<int>() : nullptr;
        v.n_cases = n_cases;
        v.branches = nullptr;
        return v;
    }

    void ensure_geometry(int prec) {
        ensure_device();
        if (is_mixed(prec)) upload_geometry<float>(s32);
        else if (is_ff(prec)) upload_geometry<float>(sff, true);
        else upload_geometry<double>(s64);
    }
    // Make the primitives (and ghosts) of arithmetic `prec` reflect the current state.
    void ensure_prims(int prec) {
        ensure_device();
        if (!have_state) throw StateError("no initial condition: call ibisgb_set_primitives first");
        ensure_geometry(prec);
        StateBufs& s = bufs(prec);
        if (s.prims_current) return;
        DevView v = view(prec);
        if (!ic_prims.empty()) {
            const int64_t NT = mesh.NT();
            if (float_storage(prec)) {
                std::vector<float> f(ic_prims.begin(), ic_prims.end());
                CUDA_OK(cudaMemcpyAsync(v.prim, f.data(), sizeof(float) * 7 * NT, cudaMemcpyHostToDevice, stream));
                if (is_ff(prec)) {
                    std::vector<float> lo(f.size());
                    for (size_t q = 0; q < f.size(); q++) lo[q] = (float)(ic_prims[q] - (double)f[q]);
                    CUDA_OK(cudaMemcpyAsync(v.prim_lo, lo.data(), sizeof(float) * 7 * NT, cudaMemcpyHostToDevice,
                                            stream));
                    CUDA_OK(cudaStreamSynchronize(stream));
                }
                CUDA_OK(cudaStreamSynchronize(stream));
            } else {
                CUDA_OK(cudaMemcpyAsync(v.prim, ic_prims.data(), sizeof(double) * 7 * NT, cudaMemcpyHostToDevice, stream));
            }
            ops(prec).ghost_fill(v, prm, stream);
        } else {
            ops(prec).prims_from_U(v, prm, stream);
        }
        CUDA_OK(cudaGetLastError());
        s.prims_current = true;
    }

    // prec < 0: the conserved state changed outside a kernel build (no prims current)
    void state_changed(int prec) {
        ic_prims.clear();
        s64.prims_current = prec >= 0 && !float_storage(prec);
        s32.prims_current = prec >= 0 && is_mixed(prec);
        sff.prims_current = prec >= 0 && is_ff(prec);
    }

    void set_primitives(const double* T, const double* p, const double* vx, const double* vy, const double* vz) {
        if (!T || !p || !vx || !vy) throw ArgError("T, p, vx and vy are required");
        if (mesh.dim == 3 && !vz) throw ArgError("vz is required in 3-D");
        ensure_device();
        const int64_t N = mesh.N, NT = mesh.NT();
        // NativeBinaryInput::read (native.cpp:263-339): update_thermo_from_pT per cell
        ic_prims.assign(7 * NT, 0.0);
        std::vector<double> u(nc() * N);
        for (int64_t i = 0; i < N; i++) {
            double rho = p[i] / (prm.R * T[i]);
            double e = prm.Cv * T[i];
            double w = vz ? vz[i] : 0.0;
            ic_prims[i] = rho; ic_prims[NT + i] = p[i]; ic_prims[2 * NT + i] = T[i]; ic_prims[3 * NT + i] = e;
            ic_prims[4 * NT + i] = vx[i]; ic_prims[5 * NT + i] = vy[i]; ic_prims[6 * NT + i] = w;
            // primatives_to_conserved (primative_conserved_conversion.cpp:31-51)
            u[i] = rho;
            u[N + i] = rho * vx[i];
            u[2 * N + i] = rho * vy[i];
            if (mesh.dim == 3) u[3 * N + i] = rho * w;
            double ke = 0.5 * (vx[i] * vx[i] + vy[i] * vy[i] + w * w);
            u[(mesh.dim + 1) * N + i] = rho * (ke + e);
        }
        CUDA_OK(cudaMemcpyAsync(U.p, u.data(), sizeof(double) * u.size(), cudaMemcpyHostToDevice, stream));
        CUDA_OK(cudaStreamSynchronize(stream));
        have_state = true;
        s64.prims_current = false;
        s32.prims_current = false;
        sff.prims_current = false;
        // RungeKutta::initialise: t = 0, dt = dt_init or max (runge_kutta.cpp:82-104)
        reset_rk();
    }

    void reset_rk() {
        std::vector<StepCtl> all(n_cases);
        for (int cs = 0; cs < n_cases; cs++) {
            StepCtl c = n_cases > 1 ? case_ctl[cs] : ctl_host;
            const double dti = n_cases > 1 ? case_dt_init[cs] : dt_init;
            c.t = 0.0;
            c.time_since_last_plot = 0.0;
            c.dt = dti > 0 ? dti : std::numeric_limits<double>::max();
            c.dt_bits = 0x7FF0000000000000ull;
            c.bad_cells = 0;
            c.steps = 0;
            if (!rk_configured) c.stages = 1;
            c.halt = 0;
            if (!rk_configured) c.max_time = std::numeric_limits<double>::max();
            all[cs] = c;
        }
        last_ctl = all;
        CUDA_OK(cudaMemcpyAsync(ctl.p, all.data(), sizeof(StepCtl) * n_cases, cudaMemcpyHostToDevice, stream));
        CUDA_OK(cudaStreamSynchronize(stream));
    }

    void residual(int prec, double* out_device, bool record_branches) {
        ensure_prims(prec);
        if (scratch_poison) {  // the stage's intermediates: each is written before it is read
            StateBufs& sb = bufs(prec);
            for (DBuf* b : {&sb.grad, &sb.phi, &sb.vgrad, &sb.flux, &sb.grad_lo, &sb.vgrad_lo, &sb.flux_lo, &vsig})
                poison(*b);
        }
        DevView v = view(prec);
        KernelOps o = ops(prec);
        // compute_dudt applies the pre-reconstruction actions first (finite_volume.cpp:62)
        o.ghost_fill(v, prm, stream);
        if (record_branches && prm.order == 2 && prm.limiter) {
            if (!branches.p) {  // a 2-D grid leaves the fifth row unwritten
                branches.alloc(sizeof(unsigned) * 5 * mesh.N);
                if (branches.p) CUDA_OK(cudaMemsetAsync(branches.p, 0, sizeof(unsigned) * 5 * mesh.N, stream));
            }
            v.branches = branches.as<unsigned>();
        }
        bool reco = prm.order == 2;
        const int* vr = var[gidx(prec)];
        o.recon(v, prm, reco, vr[0], stream);
        o.face_flux(v, prm, reco, vr[1], stream);
        o.update(v, prm, 0, 0, out_device, 0, vr[2], stream);
        CUDA_OK(cudaGetLastError());
    }

    double estimate_dt(int prec) {
        ensure_prims(prec);
        DevView v = view(prec);
        launch_reset_dt(v.ctl, n_cases, stream);
        ops(prec).local_dt(v, prm, stream);
        CUDA_OK(cudaGetLastError());
        std::vector<StepCtl> c(n_cases);
        CUDA_OK(cudaMemcpyAsync(c.data(), ctl.p, sizeof(StepCtl) * n_cases, cudaMemcpyDeviceToHost, stream));
        CUDA_OK(cudaStreamSynchronize(stream));
        double dt = std::numeric_limits<double>::infinity();
        for (const StepCtl& x : c) {
            double d;
            std::memcpy(&d, &x.dt_bits, sizeof(d));
            dt = std::min(dt, d);
        }
        return dt;
    }

    // Host-side eligibility of the fused stage (no GPU needed).
    bool check_fused() {
        if (fused_elig >= 0) return fused_elig == 1;
        fused_elig = 0;
        if (prm.viscous) fused_why = "viscous fluxes take the generic kernels";
        else if (k_alias) fused_why = "aliased stage derivatives take the generic kernels";
        else if (prm.cflux) fused_why = "constant-flux boundaries take the generic kernels";
        else if (prm.order != 2) fused_why = "first-order reconstruction takes the generic kernels";
        else {
            std::vector<int64_t> offs = n_cases > 1 ? cell_off : std::vector<int64_t>{0, mesh.N};
            int tx, ty, tz;
            fused_tile_shape(mesh.dim, &tx, &ty, &tz);
            if (detect_structured(mesh, offs, tx, ty, tz, slay, &fused_why)) {
                fused_elig = 1;
                fused_why.clear();
            }
        }
        return fused_elig == 1;
    }

    void upload_fused() {
        if (fused_uploaded) return;
        ensure_device();
        upload_geometry<float>(s32);
        upload(sb_blocks, slay.blocks, stream);
        upload(sb_tiles, slay.tiles, stream);
        std::vector<float> fc(slay.face.begin(), slay.face.end());
        upload(sb_face, fc, stream);
        upload(sb_ghost, slay.ghost_map, stream);
        prim_alt.alloc(sizeof(float) * 7 * mesh.NT());
        CUDA_OK(prepare_fused_stage());
        CUDA_OK(cudaStreamSynchronize(stream));
        fused_uploaded = true;
    }

    // Host-side eligibility of the plane-marching kernel (no GPU needed).
    bool check_march() {
        if (march_elig >= 0) return march_elig == 1;
        march_elig = 0;
        if (!check_fused()) march_why = fused_why;
        else if (mesh.dim != 3) march_why = "the plane-marching stage is three-dimensional";
        else if (slay.blocks.size() != 1 || n_cases != 1) march_why = "the plane-marching stage takes one structured block";
        else if (slay.blocks[0].c0 % 4 || slay.blocks[0].ni % 4 || mesh.NT() % 4)
            march_why = "TMA copies need the block's first cell, i-extent and N+G to be multiples of 4";
        else march_elig = 1;
        return march_elig == 1;
    }

    // Tensor maps of the two mixed primitive buffers and of the float centroids
    // (re-encoded if a buffer moved).
    void upload_march() {
        upload_fused();
        if (!march_fault.p) {
            march_fault.alloc(sizeof(unsigned));
            CUDA_OK(cudaMemsetAsync(march_fault.p, 0, sizeof(unsigned), stream));
            CUDA_OK(prepare_march_stage());
        }
        const SBlock& B = slay.blocks[0];
        const void* bases[3] = {s32.prim.p, prim_alt.p, s32.cc.p};
        for (int b = 0; b < 3; b++) {
            if (bases[b] == march_map_base[b]) continue;
            std::string why;
            const float* base = (const float*)bases[b] + B.c0;
            TmaMap* out = b < 2 ? &march_map_prim[b] : &march_map_cc;
            if (march_encode_map(out, base, B.ni, B.nj, B.nk, b < 2 ? 7 : 3, mesh.NT(), &why) != 0)
                throw CudaError("plane-marching stage: " + why);
            march_map_base[b] = bases[b];
        }
    }

    // The fused stage the context uses (tile or plane-marching kernel), reading
    // primitive buffer `cur` and writing the other one.
    void launch_fused_any(const DevView& v, int cur, int mode, int stage, int with_dt, bool march, int kc) {
        SbView sb = sb_view(mixed_prim(cur ^ 1));
        if (march)
            launch_march_stage(v, sb, slay.blocks[0], prm, march_map_prim[cur], march_map_cc, mode, stage, with_dt, kc,
                               stream);
        else
            launch_fused_stage(v, sb, prm, mode, stage, with_dt, stream);
    }

    // A TMA copy of the plane-marching stage that did not complete within its wait
    // limit is reported once, as a CUDA failure of the call that ran it.
    void check_march_fault() {
        if (!march_fault.p) return;
        unsigned f = 0;
        CUDA_OK(cudaMemcpyAsync(&f, march_fault.p, sizeof(f), cudaMemcpyDeviceToHost, stream));
        CUDA_OK(cudaStreamSynchronize(stream));
        if (f) {
            CUDA_OK(cudaMemsetAsync(march_fault.p, 0, sizeof(unsigned), stream));
            throw CudaError("plane-marching stage: a TMA copy did not complete within its wait limit");
        }
    }

    SbView sb_view(void* prim_out) const {
        SbView sb{};
        sb.blocks = sb_blocks.as<SBlock>();
        sb.tiles = sb_tiles.as<STile>();
        sb.num_tiles = (int)slay.tiles.size();
        sb.face = sb_face.as<float>();
        sb.SF = (int)slay.num_faces;
        sb.ghost_map = sb_ghost.as<int>();
        sb.prim_out = prim_out;
        sb.fault = march_fault.as<unsigned>();
        return sb;
    }
    void* mixed_prim(int which) { return which ? prim_alt.p : s32.prim.p; }

    bool cell_eligible() const {
        return rk_configured && !prm.viscous && !prm.cflux && !k_alias && kernels_mixed().cell_update != nullptr;
    }
    std::string cell_why() const {
        if (!rk_configured) return "the solver is not runge_kutta";
        if (prm.viscous) return "viscous fluxes take the generic kernels";
        if (prm.cflux) return "constant-flux boundaries take the generic kernels";
        return "";
    }

    // one Runge-Kutta step of the per-cell flux path starting from primitive buffer `start`
    void enqueue_cell_step(int start) {
        const int S = ctl_host.stages;
        DevView v = view(IBISGB_MIXED);
        KernelOps o = ops(IBISGB_MIXED);
        const bool reco = prm.order == 2;
        launch_dt_finalize(v.ctl, n_cases, stream);
        int cur = start;
        for (int s = 0; s < S; s++) {
            v.prim = mixed_prim(cur);
            o.recon(v, prm, reco, var[1][0], stream);
            o.cell_update(v, prm, reco, s == S - 1 ? 3 : 2, s, s == S - 1, cell_var, mixed_prim(cur ^ 1), stream);
            cur ^= 1;
        }
    }

    // one fused Runge-Kutta step starting from primitive buffer `start`
    void enqueue_fused_step(int start) {
        const int S = ctl_host.stages;
        DevView v = view(IBISGB_MIXED);
        launch_dt_finalize(v.ctl, n_cases, stream);
        int cur = start;
        for (int s = 0; s < S; s++) {
            v.prim = mixed_prim(cur);
            launch_fused_any(v, cur, s == S - 1 ? 3 : 2, s, s == S - 1, march_on, march_kc);
            cur ^= 1;
        }
    }

    void drop_mixed_graphs() {
        for (auto* g : {&graph[1], &graph_fused[0], &graph_fused[1]})
            if (*g) {
                cudaGraphExecDestroy(*g);
                *g = nullptr;
            }
    }

    // one Runge-Kutta step (RungeKutta::take_step, runge_kutta.cpp:131-203)
    void enqueue_step(int prec) {
        DevView v = view(prec);
        KernelOps o = ops(prec);
        const bool reco = prm.order == 2;
        const int S = ctl_host.stages;
        const int* vr = var[gidx(prec)];
        if (!prm.viscous) {
            // Inviscid: the step's dt depends only on the primitives of U^n, so
            // the previous step's last update (or rk_run's prologue) has already
            // min-reduced it; the first stage's update then forms the next
            // stage state directly, and the last one reduces the next step's dt.
            launch_dt_finalize(v.ctl, n_cases, stream);
            for (int s = 0; s < S; s++) {
                o.recon(v, prm, reco, vr[0], stream);
                o.face_flux(v, prm, reco, vr[1], stream);
                o.update(v, prm, s == S - 1 ? 3 : 2, s, nullptr, s == S - 1, vr[2], stream);
            }
            return;
        }
        // Viscous: the dt signal needs the viscous face state of stage 0.
        o.recon(v, prm, reco, vr[0], stream);
        o.face_flux(v, prm, reco, vr[1], stream);
        o.update(v, prm, 1, 0, nullptr, 0, vr[2], stream);
        o.local_dt(v, prm, stream);
        launch_dt_finalize(v.ctl, n_cases, stream);
        if (S == 1) {
            o.finalize(v, prm, stream);
            return;
        }
        o.combine(v, prm, 1, stream);
        for (int s = 1; s < S; s++) {
            o.recon(v, prm, reco, vr[0], stream);
            o.face_flux(v, prm, reco, vr[1], stream);
            o.update(v, prm, s == S - 1 ? 3 : 2, s, nullptr, 0, vr[2], stream);
        }
    }

    // Tuning and the per-step graphs of precision prec; returns whether the fused
    // (or per-cell flux) stage runs.  The primitives of the current state are made current.
    bool prepare_rk(int prec) {
        if (!rk_configured) throw ConfigError("config.json solver is not runge_kutta");
        ensure_prims(prec);
        int gi = gidx(prec);
        if (!tuned[gi]) autotune(prec);
        // the fused stage and the per-cell flux path alternate primitive buffers
        const bool fused = is_mixed(prec) && (fused_on || cell_on);
        if (fused && fused_on && march_on) upload_march();
        if (fused) {
            for (int par = 0; par < 2; par++) {
                if (graph_fused[par]) continue;
                cudaGraph_t g;
                CUDA_OK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                if (fused_on) enqueue_fused_step(par);
                else enqueue_cell_step(par);
                cudaError_t le = cudaGetLastError();
                CUDA_OK(cudaStreamEndCapture(stream, &g));
                CUDA_OK(le);
                CUDA_OK(cudaGraphInstantiate(&graph_fused[par], g, 0));
                CUDA_OK(cudaGraphDestroy(g));
            }
        } else if (!graph[gi]) {
            cudaGraph_t g;
            CUDA_OK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
            enqueue_step(prec);
            cudaError_t le = cudaGetLastError();
            CUDA_OK(cudaStreamEndCapture(stream, &g));
            CUDA_OK(le);
            CUDA_OK(cudaGraphInstantiate(&graph[gi], g, 0));
            CUDA_OK(cudaGraphDestroy(g));
        }
        return fused;
    }

    // n steps on the context stream (the local-dt prologue unless the caller formed
    // it already, then one graph per step)
    void enqueue_rk(int prec, int64_t n, bool fused, bool prologue = true) {
        if (prologue && !prm.viscous && n > 0) {  // local dt of the current state for the first step
            DevView v = view(prec);
            launch_reset_dt(v.ctl, n_cases, stream);
            ops(prec).local_dt(v, prm, stream);
            CUDA_OK(cudaGetLastError());
        }
        if (fused) {
            for (int64_t i = 0; i < n; i++) {
                CUDA_OK(cudaGraphLaunch(graph_fused[prim_cur], stream));
                prim_cur ^= (ctl_host.stages & 1);
            }
        } else {
            const int gi = gidx(prec);
            for (int64_t i = 0; i < n; i++) CUDA_OK(cudaGraphLaunch(graph[gi], stream));
        }
        state_changed(prec);
    }

    void rk_run(int prec, int64_t n, ibisgb_rk_status* st) {
        const bool fused = prepare_rk(prec);
        cudaEvent_t e0, e1;
        CUDA_OK(cudaEventCreate(&e0));
        CUDA_OK(cudaEventCreate(&e1));
        CUDA_OK(cudaEventRecord(e0, stream));
        enqueue_rk(prec, n, fused);
        CUDA_OK(cudaEventRecord(e1, stream));
        float ms = finish_rk(prec, fused, e0, e1, st);
        (void)ms;
    }

    // The step control after the last enqueued step (t, dt, steps, bad cells: a batch
    // reports its minimum times, maximum steps and total bad cells); throws on bad cells.
    float finish_rk(int prec, bool fused, cudaEvent_t e0, cudaEvent_t e1, ibisgb_rk_status* st) {
        (void)prec;
        last_ctl.resize(n_cases);
        CUDA_OK(cudaMemcpyAsync(last_ctl.data(), ctl.p, sizeof(StepCtl) * n_cases, cudaMemcpyDeviceToHost, stream));
        CUDA_OK(cudaStreamSynchronize(stream));
        if (fused && fused_on && march_on) check_march_fault();
        float ms = 0.f;
        CUDA_OK(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        last_ms = ms;
        StepCtl c = last_ctl[0];
        for (const StepCtl& x : last_ctl) {  // batch: minimum times, maximum steps, total bad cells
            c.t = std::min(c.t, x.t); c.dt = std::min(c.dt, x.dt); c.stable_dt = std::min(c.stable_dt, x.stable_dt);
            c.steps = std::max(c.steps, x.steps);
        }
        c.bad_cells = 0;
        for (const StepCtl& x : last_ctl) c.bad_cells += x.bad_cells;
        if (st) {
            st->t = c.t; st->dt = c.dt; st->stable_dt = c.stable_dt; st->steps = c.steps;
            st->bad_cells = (int64_t)c.bad_cells;
            st->device_ms = ms;
        }
        if (c.bad_cells > 0) throw std::runtime_error("bad cells");
        return ms;
    }

    // n_jobs Runge-Kutta runs from host rows: job j replaces the state by U_in[j],
    // takes `steps` steps and writes the new state to U_out[j] -- what
    // set_conserved + rk_run + get_conserved do per job, with job j+1's upload and
    // job j-1's read-back on two copy streams while job j's steps run (two device
    // staging buffers each way).  Pinned host rows make the copies asynchronous.
    DBuf pipe_in[2], pipe_out[2];
    cudaStream_t pipe_h2d = nullptr, pipe_d2h = nullptr;
    cudaEvent_t pipe_ev[8] = {};
    void rk_run_host(int prec, int64_t n_jobs, int64_t steps, const double* const* U_in, double* const* U_out,
                     ibisgb_rk_status* st) {
        if (n_jobs <= 0) throw ArgError("n_jobs must be positive");
        for (int64_t j = 0; j < n_jobs; j++)
            if (!U_in[j] || !U_out[j]) throw ArgError("a job's host rows are null");
        ensure_device();
        if (!have_state) set_conserved(U_in[0]);
        const bool fused = prepare_rk(prec);
        const size_t bytes = sizeof(double) * nvars();
        if (!pipe_h2d) {
            CUDA_OK(cudaStreamCreateWithFlags(&pipe_h2d, cudaStreamNonBlocking));
            CUDA_OK(cudaStreamCreateWithFlags(&pipe_d2h, cudaStreamNonBlocking));
            for (auto& e : pipe_ev) CUDA_OK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        }
        for (int b = 0; b < 2; b++) {
            pipe_in[b].alloc(bytes);
            pipe_out[b].alloc(bytes);
        }
        if (renumbered()) map_a.alloc(bytes);
        cudaEvent_t* ev_in = pipe_ev, *ev_used = pipe_ev + 2, *ev_packed = pipe_ev + 4, *ev_read = pipe_ev + 6;
        cudaEvent_t e0, e1;
        CUDA_OK(cudaEventCreate(&e0));
        CUDA_OK(cudaEventCreate(&e1));
        CUDA_OK(cudaEventRecord(e0, stream));
        CUDA_OK(cudaStreamWaitEvent(pipe_h2d, e0, 0));
        CUDA_OK(cudaStreamWaitEvent(pipe_d2h, e0, 0));
        auto upload = [&](int64_t j) {
            const int b = (int)(j & 1);
            if (j >= 2) CUDA_OK(cudaStreamWaitEvent(pipe_h2d, ev_used[b], 0));  // job j-2 consumed buffer b
            CUDA_OK(cudaMemcpyAsync(pipe_in[b].p, U_in[j], bytes, cudaMemcpyHostToDevice, pipe_h2d));
            CUDA_OK(cudaEventRecord(ev_in[b], pipe_h2d));
        };
        upload(0);
        for (int64_t j = 0; j < n_jobs; j++) {
            const int b = (int)(j & 1);
            if (j + 1 < n_jobs) upload(j + 1);
            CUDA_OK(cudaStreamWaitEvent(stream, ev_in[b], 0));
            // the state, its primitives and ghosts and the first step's local dt in one pass
            DevView v = view(prec);
            const bool with_dt = !prm.viscous && steps > 0;
            if (with_dt) launch_reset_dt(v.ctl, n_cases, stream);
            if (renumbered()) ensure_maps();
            ops(prec).load_state(v, prm, pipe_in[b].as<double>(),
                                 renumbered() ? d_cell_to_new.as<int32_t>() : nullptr, with_dt ? 1 : 0, stream);
            CUDA_OK(cudaGetLastError());
            CUDA_OK(cudaEventRecord(ev_used[b], stream));
            ic_prims.clear();
            state_changed(prec);
            enqueue_rk(prec, steps, fused, false);
            if (j >= 2) CUDA_OK(cudaStreamWaitEvent(stream, ev_read[b], 0));  // job j-2's read-back is done
            if (renumbered()) {
                launch_soa_to_rows(U.as<double>(), map_a.as<double>(), (int)mesh.N, nc(), stream);
                map_rows_device(map_a.as<double>(), pipe_out[b].as<double>(), nc(), false);
            } else {
                launch_soa_to_rows(U.as<double>(), pipe_out[b].as<double>(), (int)mesh.N, nc(), stream);
            }
            CUDA_OK(cudaGetLastError());
            CUDA_OK(cudaEventRecord(ev_packed[b], stream));
            CUDA_OK(cudaStreamWaitEvent(pipe_d2h, ev_packed[b], 0));
            CUDA_OK(cudaMemcpyAsync(U_out[j], pipe_out[b].p, bytes, cudaMemcpyDeviceToHost, pipe_d2h));
            CUDA_OK(cudaEventRecord(ev_read[b], pipe_d2h));
        }
        CUDA_OK(cudaStreamWaitEvent(stream, ev_read[(n_jobs - 1) & 1], 0));
        CUDA_OK(cudaEventRecord(e1, stream));
        // every copy has completed before the call returns, bad cells or not
        CUDA_OK(cudaStreamSynchronize(pipe_h2d));
        CUDA_OK(cudaStreamSynchronize(pipe_d2h));
        finish_rk(prec, fused, e0, e1, st);
    }

    // ----- tangent (SteadyStateLinearisation::matrix_vector_product) ---------
    // Scratch poisoning (ibisgb_set_scratch_poison): every buffer the derivative
    // kernels use as scratch is filled with NaN before each call, so that a read of
    // an entry the call did not write shows in its result.
    bool scratch_poison = false;
    void poison(DBuf& b) {
        if (scratch_poison && b.p) CUDA_OK(cudaMemsetAsync(b.p, 0xFF, b.bytes, stream));
    }
    void poison_tangent() {
        if (!scratch_poison) return;
        for (DBuf* b : {&sdual.prim, &sdual.vghost, &sdual.grad, &sdual.phi, &sdual.vgrad, &sdual.flux}) poison(*b);
    }
    void poison_adjoint() {
        if (!scratch_poison) return;
        poison_tangent();
        for (DBuf* b : {&adj_qf, &adj_self, &adj_nba, &adj_ga, &adj_qv, &adj_qg, &adj_gav}) poison(*b);
    }
    DevView tangent_view() {
        ensure_device();
        upload_geometry<double>(s64);
        if (!sdual.geometry) {
            const int64_t N = mesh.N, NT = mesh.NT(), F = mesh.F;
            const size_t D = 2 * sizeof(double);
            sdual.prim.alloc(D * 7 * NT);
            sdual.vghost.alloc(D * 5 * std::max<int64_t>(mesh.G, 1));
            sdual.grad.alloc(D * 15 * N);
            sdual.phi.alloc(D * 5 * N);
            sdual.vgrad.alloc(D * 12 * N);
            sdual.flux.alloc(D * nc() * F);
            sdual.geometry = true;
        }
        DevView v = view(IBISGB_F64);
        v.prim = sdual.prim.p; v.vghost = sdual.vghost.p; v.grad = sdual.grad.p; v.phi = sdual.phi.p;
        v.vgrad = sdual.vgrad.p; v.flux = sdual.flux.p;
        return v;
    }

    // out = inv_dt * v - dR/dU v on device rows (N x nc)
    void jvp(const double* v_dev, double* out_dev, double inv_dt, bool reconstruct) {
        if (!have_state) throw StateError("no state: call ibisgb_set_primitives first");
        DevView v = tangent_view();
        poison_tangent();
        launch_tangent(v, prm, v_dev, inv_dt, reconstruct && prm.order == 2, out_dev, stream);
        CUDA_OK(cudaGetLastError());
    }

    // ----- adjoint: (dR/dU)^T w ------------------------------------------------
    DBuf adj_qf, adj_self, adj_nba, adj_ga, adj_back, adj_gout, adj_qv, adj_qg, adj_gav;
    bool adj_ready = false;
    void ensure_adjoint() {
        if (adj_ready) return;
        ensure_device();
        const int64_t N = mesh.N, F = mesh.F, MF = mesh.MF;
        adj_qf.alloc(sizeof(double) * 12 * F);
        adj_self.alloc(sizeof(double) * 7 * N);
        adj_nba.alloc(sizeof(double) * 7 * MF * N);
        adj_ga.alloc(sizeof(double) * 7 * std::max<int64_t>(mesh.G, 1));
        if (prm.viscous) {
            adj_qv.alloc(sizeof(double) * 10 * F);
            adj_qg.alloc(sizeof(double) * 24 * F);
            adj_gav.alloc(sizeof(double) * 5 * std::max<int64_t>(mesh.G, 1));
        }
        // slot of each valid neighbour that points back through the same face
        std::vector<signed char> back(MF * N, -1);
        for (int64_t c = 0; c < N; c++)
            for (int64_t k = 0; k < MF; k++) {
                const int64_t nb = mesh.cell_nbr[c * MF + k];
                if (nb < 0 || nb >= N) continue;
                const int64_t f = mesh.cell_face[c * MF + k];
                for (int64_t t = 0; t < MF; t++)
                    if (mesh.cell_face[nb * MF + t] == f) back[k * N + c] = (signed char)t;
            }
        upload(adj_back, back, stream);
        CUDA_OK(cudaStreamSynchronize(stream));
        adj_ready = true;
    }

    void vjp(const double* w_dev, double* out_dev, double* ghost_out_dev, bool reconstruct) {
        if (!have_state) throw StateError("no state: call ibisgb_set_primitives first");
        DevView v = tangent_view();
        ensure_adjoint();
        poison_adjoint();
        AdjScratch a{adj_qf.as<double>(), adj_self.as<double>(), adj_nba.as<double>(), adj_ga.as<double>(),
                     adj_back.as<signed char>(), adj_qv.as<double>(), adj_qg.as<double>(), adj_gav.as<double>()};
        launch_adjoint(v, prm, w_dev, reconstruct && prm.order == 2, a, out_dev, ghost_out_dev, stream);
        CUDA_OK(cudaGetLastError());
    }

    // w^T dR/dgeometry: face rows (13 x F: n, t1, t2, centre, area) and cell rows
    // (4 x (N+G): centroid, volume), internal numbering
    DBuf geo_fcb, geo_vb, geo_nbc, geo_ceb;
    void vjp_geometry(const double* w_dev, double* face_out, double* cell_out, bool reconstruct) {
        if (!have_state) throw StateError("no state: call ibisgb_set_primitives first");
        DevView v = tangent_view();
        ensure_adjoint();
        const int64_t N = mesh.N, F = mesh.F, MF = mesh.MF;
        geo_fcb.alloc(sizeof(double) * 6 * F);
        geo_vb.alloc(sizeof(double) * 2 * F);
        geo_nbc.alloc(sizeof(double) * 3 * MF * std::max<int64_t>(N, 1));
        geo_ceb.alloc(sizeof(double) * 3 * F);
        poison_adjoint();
        for (DBuf* b : {&geo_fcb, &geo_vb, &geo_nbc, &geo_ceb}) poison(*b);
        AdjScratch a{adj_qf.as<double>(), adj_self.as<double>(), adj_nba.as<double>(), adj_ga.as<double>(),
                     adj_back.as<signed char>(), adj_qv.as<double>(), adj_qg.as<double>(), adj_gav.as<double>()};
        a.geo_face = face_out;
        a.geo_cell = cell_out;
        a.geo_fcb = geo_fcb.as<double>();
        a.geo_vb = geo_vb.as<double>();
        a.geo_nbc = geo_nbc.as<double>();
        a.geo_ceb = geo_ceb.as<double>();
        launch_adjoint_geometry(v, prm, w_dev, reconstruct && prm.order == 2, a, stream);
        CUDA_OK(cudaGetLastError());
    }
    // dR/dgeometry . (dface, dcell) (N x nc rows, internal numbering)
    DBuf gt_face, gt_cc, gt_vol, gt_r;
    void jvp_geometry(const double* dface, const double* dcell, double* out, bool reconstruct) {
        if (!have_state) throw StateError("no state: call ibisgb_set_primitives first");
        DevView v = tangent_view();
        const int64_t N = mesh.N, F = mesh.F, NT = mesh.NT();
        const size_t D = 2 * sizeof(double);
        gt_face.alloc(D * 13 * F);
        gt_cc.alloc(D * 3 * NT);
        gt_vol.alloc(D * std::max<int64_t>(N, 1));
        gt_r.alloc(D * 6 * std::max<int64_t>(N, 1));
        poison_tangent();
        for (DBuf* b : {&gt_face, &gt_cc, &gt_vol, &gt_r}) poison(*b);
        GeoTangent g{gt_face.p, gt_cc.p, gt_vol.p, gt_r.p};
        launch_tangent_geometry(v, prm, dface, dcell, reconstruct && prm.order == 2, g, out, stream);
        CUDA_OK(cudaGetLastError());
    }

    // the same on rows and geometry arrays in the reference numbering
    DBuf map_fg, map_cg, d_face_to_ref, d_face_to_new, geo_out_face, geo_out_cell;
    void jvp_geometry_rows(const double* dface, const double* dcell, double* out, bool reconstruct) {
        if (!renumbered()) return jvp_geometry(dface, dcell, out, reconstruct);
        const int64_t N = mesh.N, F = mesh.F, NT = mesh.NT();
        if (!d_face_to_new.p) {
            std::vector<int32_t> fm(F);
            for (int64_t f = 0; f < F; f++) fm[f] = (int32_t)num.face_ref_of_new[f];
            d_face_to_new.alloc(sizeof(int32_t) * F);
            CUDA_OK(cudaMemcpyAsync(d_face_to_new.p, fm.data(), sizeof(int32_t) * F, cudaMemcpyHostToDevice, stream));
            CUDA_OK(cudaStreamSynchronize(stream));
        }
        ensure_maps();
        map_fg.alloc(sizeof(double) * 13 * F);
        map_cg.alloc(sizeof(double) * 4 * NT);
        map_b.alloc(sizeof(double) * nvars());
        for (int r = 0; r < 13; r++)
            launch_gather_rows(map_fg.as<double>() + r * F, dface + r * F, d_face_to_new.as<int32_t>(), (int)F, 1,
                               stream);
        for (int r = 0; r < 4; r++) {
            launch_gather_rows(map_cg.as<double>() + r * NT, dcell + r * NT, d_cell_to_new.as<int32_t>(), (int)N, 1,
                               stream);
            if (NT > N)
                CUDA_OK(cudaMemcpyAsync(map_cg.as<double>() + r * NT + N, dcell + r * NT + N,
                                        sizeof(double) * (NT - N), cudaMemcpyDeviceToDevice, stream));
        }
        jvp_geometry(map_fg.as<double>(), map_cg.as<double>(), map_b.as<double>(), reconstruct);
        map_rows_device(map_b.as<double>(), out, nc(), false);
    }
    void vjp_geometry_rows(const double* w, double* face_out, double* cell_out, bool reconstruct) {
        if (!renumbered()) return vjp_geometry(w, face_out, cell_out, reconstruct);
        const int64_t N = mesh.N, F = mesh.F, NT = mesh.NT();
        if (!d_face_to_ref.p) {
            std::vector<int32_t> fm(F);
            for (int64_t f = 0; f < F; f++) fm[f] = (int32_t)num.face_new_of_ref[f];
            d_face_to_ref.alloc(sizeof(int32_t) * F);
            CUDA_OK(cudaMemcpyAsync(d_face_to_ref.p, fm.data(), sizeof(int32_t) * F, cudaMemcpyHostToDevice, stream));
            CUDA_OK(cudaStreamSynchronize(stream));
        }
        map_a.alloc(sizeof(double) * nvars());
        map_fg.alloc(sizeof(double) * 13 * F);
        map_cg.alloc(sizeof(double) * 4 * NT);
        map_rows_device(w, map_a.as<double>(), nc(), true);
        vjp_geometry(map_a.as<double>(), map_fg.as<double>(), map_cg.as<double>(), reconstruct);
        ensure_maps();
        for (int r = 0; r < 13; r++)
            launch_gather_rows(face_out + r * F, map_fg.as<double>() + r * F, d_face_to_ref.as<int32_t>(), (int)F, 1,
                               stream);
        for (int r = 0; r < 4; r++) {
            launch_gather_rows(cell_out + r * NT, map_cg.as<double>() + r * NT, d_cell_to_ref.as<int32_t>(), (int)N,
                               1, stream);
            if (NT > N)
                CUDA_OK(cudaMemcpyAsync(cell_out + r * NT + N, map_cg.as<double>() + r * NT + N,
                                        sizeof(double) * (NT - N), cudaMemcpyDeviceToDevice, stream));
        }
        CUDA_OK(cudaGetLastError());
    }

    // The flow state (T, p, rho, energy, vx, vy, vz) of boundary `tag`: every
    // action that carries one (flow_state_copy, subsonic_inflow before
    // reconstruction or the viscous gradients, constant_flux after the convective
    // flux) takes `fs`, as if the config had given it.
    int bound_index(const char* tag) const {
        for (size_t b = 0; b < mesh.bounds.size(); b++)
            if (mesh.bounds[b].tag == tag) return (int)b;
        throw ArgError(std::string("no boundary ") + tag);
    }
    static bool carries_flow_state(const Action& a) { return a.kind == aFlowStateCopy || a.kind == aSubsonicInflow; }
    bool has_flow_state(const BoundDev& d) const {
        bool any = d.cflux != 0;
        for (int k = 0; k < d.n_pre; k++) any |= carries_flow_state(d.pre[k]);
        for (int k = 0; k < d.n_visc; k++) any |= carries_flow_state(d.visc[k]);
        return any;
    }
    void flow_state(const char* tag, double* fs) const {
        if (n_cases > 1) throw StateError("a batch's boundary states belong to its cases");
        const BoundDev& d = bounds_host[bound_index(tag)];
        for (int k = 0; k < d.n_pre; k++)
            if (carries_flow_state(d.pre[k])) return (void)std::copy(d.pre[k].fs, d.pre[k].fs + 7, fs);
        for (int k = 0; k < d.n_visc; k++)
            if (carries_flow_state(d.visc[k])) return (void)std::copy(d.visc[k].fs, d.visc[k].fs + 7, fs);
        if (d.cflux) return (void)std::copy(d.cfs, d.cfs + 7, fs);
        throw ArgError(std::string("boundary ") + tag + " has no flow state");
    }
    void set_flow_state(const char* tag, const double* fs) {
        if (n_cases > 1) throw StateError("a batch's boundary states belong to its cases");
        for (int k = 0; k < 7; k++)
            if (!std::isfinite(fs[k])) throw ArgError("flow state entries must be finite");
        BoundDev& d = bounds_host[bound_index(tag)];
        if (!has_flow_state(d)) throw ArgError(std::string("boundary ") + tag + " has no flow state");
        for (int k = 0; k < d.n_pre; k++)
            if (carries_flow_state(d.pre[k])) std::copy(fs, fs + 7, d.pre[k].fs);
        for (int k = 0; k < d.n_visc; k++)
            if (carries_flow_state(d.visc[k])) std::copy(fs, fs + 7, d.visc[k].fs);
        if (d.cflux) std::copy(fs, fs + 7, d.cfs);
        s64.prims_current = s32.prims_current = sff.prims_current = false;  // ghosts carry the old state
        if (uploaded) {
            upload(bounds, bounds_host, stream);
            CUDA_OK(cudaStreamSynchronize(stream));
        }
    }

    // out (num_boundaries x 7, sorted tag order) = w^T dR/d(flow state of each
    // boundary), the derivative taken with every action of the boundary that
    // carries a flow state moving together (set_flow_state's semantics)
    DBuf fs_ghost, fs_io;  // per-ghost partials; the host calls' flow-state rows (num_boundaries x 7)
    void vjp_flow_state(const double* w_dev, double* out_dev, bool reconstruct) {
        if (!have_state) throw StateError("no state: call ibisgb_set_primitives first");
        if (n_cases > 1) throw StateError("a batch's boundary states belong to its cases");
        DevView v = tangent_view();
        ensure_adjoint();
        const int64_t G = mesh.G;
        fs_ghost.alloc(sizeof(double) * 7 * std::max<int64_t>(G, 1));
        poison_adjoint();
        CUDA_OK(cudaMemsetAsync(fs_ghost.p, 0, sizeof(double) * 7 * std::max<int64_t>(G, 1), stream));
        AdjScratch a{adj_qf.as<double>(), adj_self.as<double>(), adj_nba.as<double>(), adj_ga.as<double>(),
                     adj_back.as<signed char>(), adj_qv.as<double>(), adj_qg.as<double>(), adj_gav.as<double>()};
        a.fs_ghost = fs_ghost.as<double>();
        launch_adjoint(v, prm, w_dev, reconstruct && prm.order == 2, a, nullptr, nullptr, stream);
        launch_sum_ghost_rows(fs_ghost.as<double>(), ghost_bound.as<int>(), (int)G, (int)mesh.bounds.size(), out_dev,
                              stream);
        CUDA_OK(cudaGetLastError());
    }
    // out (N x nc rows, internal numbering) = dR/dfs . dfs for a direction dfs of
    // every boundary's flow state (num_boundaries x 7, device), the actions of a
    // boundary that carry a flow state moving together
    void jvp_flow_state(const double* dfs_dev, double* out_dev, bool reconstruct) {
        if (!have_state) throw StateError("no state: call ibisgb_set_primitives first");
        if (n_cases > 1) throw StateError("a batch's boundary states belong to its cases");
        DevView v = tangent_view();
        poison_tangent();
        v.fs_tan = dfs_dev;
        launch_tangent(v, prm, nullptr, 0.0, reconstruct && prm.order == 2, out_dev, stream);  // -dR/dfs . dfs
        RowScale neg{{-1.0, -1.0, -1.0, -1.0, -1.0}};
        launch_scale_rows(out_dev, out_dev, (long long)nvars(), nc(), neg, stream);
        CUDA_OK(cudaGetLastError());
    }
    void jvp_flow_state_rows(const double* dfs_dev, double* out_rows, bool reconstruct) {
        if (!renumbered()) return jvp_flow_state(dfs_dev, out_rows, reconstruct);
        map_b.alloc(sizeof(double) * nvars());
        jvp_flow_state(dfs_dev, map_b.as<double>(), reconstruct);
        map_rows_device(map_b.as<double>(), out_rows, nc(), false);
    }
    void vjp_flow_state_rows(const double* w, double* out_dev, bool reconstruct) {
        if (!renumbered()) return vjp_flow_state(w, out_dev, reconstruct);
        map_a.alloc(sizeof(double) * nvars());
        map_rows_device(w, map_a.as<double>(), nc(), true);
        vjp_flow_state(map_a.as<double>(), out_dev, reconstruct);  // ghost ids are not renumbered
    }

    size_t nvars() const { return (size_t)mesh.N * nc(); }

    void ensure_krylov(int m) {
        const size_t n = nvars();
        rhs.alloc(sizeof(double) * n);
        dU.alloc(sizeof(double) * n);
        kw.alloc(sizeof(double) * n);
        kr0.alloc(sizeof(double) * n);
        kv.alloc(sizeof(double) * n * (m + 1));
        kz.alloc(sizeof(double) * n * (m + 1));
        kH.alloc(sizeof(double) * (m + 1) * (m + 1));
        kpart.alloc(sizeof(double) * dot_scratch_doubles());
        kscal.alloc(sizeof(double) * (2 * m + 8));
    }

    struct GmresOut {
        bool success = false;
        int iters = 0;
        double residual = -1.0;
    };

    // Un-restarted GMRES with modified Gram-Schmidt (Gmres::solve, gmres.cpp:119-182).
    // A(x, out) applies the operator on device rows; the Krylov basis lives in V
    // (m+1 columns of n), Hessenberg entries are produced on the device and
    // copied once per Arnoldi step for the Givens rotations on the host.
    template <class Op>
    GmresOut gmres(Op&& A, const double* b, double* x, int m_cfg, double tol, double* V, double* Z,
                   const std::function<void(const double*, double*)>* precond) {
        const size_t n = nvars();
        const int m = (int)std::min<size_t>((size_t)m_cfg, n);
        double* w = kw.as<double>();
        double* r0 = kr0.as<double>();
        double* H = kH.as<double>();  // column-major (m+1) per column
        double* scal = kscal.as<double>();
        double* part = kpart.as<double>();
        GmresOut res;
        A(x, w);  // compute_r0_
        launch_sub(r0, b, w, (long long)n, stream);
        launch_dot(r0, r0, (long long)n, part, scal, true, stream);
        double beta = 0.0;
        CUDA_OK(cudaMemcpyAsync(&beta, scal, sizeof(double), cudaMemcpyDeviceToHost, stream));
        CUDA_OK(cudaStreamSynchronize(stream));
        if (beta < tol) {
            res.success = true;
            res.residual = beta;
            return res;
        }
        launch_scale_inv(V, r0, (long long)n, scal, stream);
        std::vector<double> h((m + 1) * (m + 1), 0.0), cs(m + 1, 0.0), sn(m + 1, 0.0), g(m + 2, 0.0);
        g[0] = beta;
        res.residual = 1.0;
        for (int j = 0; j < m; j++) {
            double* vj = V + (size_t)j * n;
            const double* col = vj;
            if (precond) {  // FGmres::solve: z_j = P^-1 v_j (gmres.cpp:257-264)
                (*precond)(vj, Z + (size_t)j * n);
                col = Z + (size_t)j * n;
            }
            A(col, w);
            double* Hj = H + (size_t)j * (m + 1);
            for (int i = 0; i <= j; i++) {
                launch_dot(w, V + (size_t)i * n, (long long)n, part, Hj + i, false, stream);
                launch_axpy_neg(w, V + (size_t)i * n, (long long)n, Hj + i, stream);
            }
            launch_dot(w, w, (long long)n, part, Hj + j + 1, true, stream);
            launch_scale_inv(V + (size_t)(j + 1) * n, w, (long long)n, Hj + j + 1, stream);
            CUDA_OK(cudaGetLastError());
            CUDA_OK(cudaMemcpyAsync(&h[(size_t)j * (m + 1)], Hj, sizeof(double) * (j + 2), cudaMemcpyDeviceToHost, stream));
            CUDA_OK(cudaStreamSynchronize(stream));
            double* hc = &h[(size_t)j * (m + 1)];
            // rotate the new column into upper-triangular form (apply_rotations_to_hessenberg_, gmres.cpp:22-74)
            for (int i = 0; i < j; i++) {
                double t = cs[i] * hc[i] + sn[i] * hc[i + 1];
                hc[i + 1] = -sn[i] * hc[i] + cs[i] * hc[i + 1];
                hc[i] = t;
            }
            double denom = std::sqrt(hc[j] * hc[j] + hc[j + 1] * hc[j + 1]);
            sn[j] = hc[j + 1] / denom;
            cs[j] = hc[j] / denom;
            hc[j] = cs[j] * hc[j] + sn[j] * hc[j + 1];
            hc[j + 1] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            double r = std::fabs(g[j + 1]);
            res.residual = r / beta;
            res.iters = j + 1;
            if (r < tol * beta) {
                res.success = true;
                break;
            }
        }
        // upper-triangular solve and x += V y (or Z y)   (gmres.cpp:170-179)
        const int k = res.iters;
        std::vector<double> y(k, 0.0);
        for (int i = k - 1; i >= 0; i--) {
            double sum = g[i];
            for (int c = i + 1; c < k; c++) sum -= h[(size_t)c * (m + 1) + i] * y[c];
            y[i] = sum / h[(size_t)i * (m + 1) + i];
        }
        CUDA_OK(cudaMemcpyAsync(scal, y.data(), sizeof(double) * k, cudaMemcpyHostToDevice, stream));
        launch_gemv_add(x, precond ? Z : V, (long long)n, k, scal, stream);
        CUDA_OK(cudaGetLastError());
        CUDA_OK(cudaStreamSynchronize(stream));
        return res;
    }

    // real residual rows into rhs and the norms of it (SteadyStateLinearisation::eval_rhs, steady_state.cpp:130-165)
    void eval_rhs(int prec) {
        residual(prec, rhs.as<double>(), false);
        launch_l2_norms(k.as<double>(), (int)mesh.N, nc(), l2.as<double>(), stream);
        CUDA_OK(cudaGetLastError());
        CUDA_OK(cudaMemcpyAsync(steady.norms, l2.p, sizeof(double) * 6, cudaMemcpyDeviceToHost, stream));
        CUDA_OK(cudaStreamSynchronize(stream));
    }

    void steady_initialise(int prec) {  // Jfnk::initialise, jfnk.cpp:25-30
        if (n_cases > 1) throw StateError("steady-state solves run one case per context, not on a batch");
        if (!steady.configured) throw ConfigError("config.json solver is not steady_state");
        ensure_prims(prec);
        ensure_krylov(steady.max_iters);
        eval_rhs(prec);
        std::memcpy(steady.initial, steady.norms, sizeof(steady.norms));
        steady.step = 0;
        steady.rb_prev_cfl = steady.rb_start;
        steady.rb_prev_res = 1.0;
        steady.initialised = true;
    }

    double steady_cfl(int64_t step) {  // Jfnk::calculate_cfl (jfnk.h:39-47), cfl.cpp:94-155
        Steady& st = steady;
        if (st.cfl_kind == 2) {
            double t = st.norms[0] / st.initial[0];
            if (t > st.rb_threshold) {
                st.rb_prev_res = t;
                return st.rb_prev_cfl;
            }
            double ratio = st.rb_prev_res / t;
            double c = st.rb_prev_cfl * std::pow(ratio, st.rb_power);
            c = std::min(c, st.rb_max);
            c = std::max(st.rb_start, c);
            st.rb_prev_res = t;
            st.rb_prev_cfl = c;
            return c;
        }
        if (st.cfl_kind == 0) return st.cfl;
        double t = (double)step;
        const auto &ts = st.cfl_t, &cs = st.cfl_v;
        if (t <= ts[0]) return cs[0];
        size_t nn = ts.size();
        if (t >= ts[nn - 1]) return cs[nn - 1];
        for (size_t i = 0; i + 1 < nn; i++)
            if (t >= ts[i] && t < ts[i + 1]) return cs[i] + (t - ts[i]) / (ts[i + 1] - ts[i]) * (cs[i + 1] - cs[i]);
        return cs[nn - 1];
    }

    // one Newton step of the JFNK solver (Jfnk::step, jfnk.cpp:39-61)
    void newton_step(int prec, ibisgb_newton_status* out) {
        if (n_cases > 1) throw StateError("steady-state solves run one case per context, not on a batch");
        if (!steady.initialised) steady_initialise(prec);
        Steady& st = steady;
        const size_t n = nvars();
        double stable = estimate_dt(prec);
        double cfl = steady_cfl(st.step);
        double dt_star = cfl * stable;
        double inv = 1 / dt_star;
        CUDA_OK(cudaMemsetAsync(dU.p, 0, sizeof(double) * n, stream));
        auto A = [&](const double* x, double* y) { jvp(x, y, inv, true); };
        GmresOut r;
        if (st.fgmres) {
            // FGmres with an inner GMRES on the first-order linearisation (steady_state.cpp:47-50)
            std::function<void(const double*, double*)> P = [&](const double* vin, double* zout) {
                CUDA_OK(cudaMemsetAsync(zout, 0, sizeof(double) * n, stream));
                auto A1 = [&](const double* x, double* y) { jvp(x, y, inv, false); };
                inner_gmres(A1, vin, zout, st.max_prec_iters, st.prec_tol);
            };
            r = gmres(A, rhs.as<double>(), dU.as<double>(), st.max_iters, st.tol, kv.as<double>(),
                      kz.as<double>(), &P);
        } else {
            r = gmres(A, rhs.as<double>(), dU.as<double>(), st.max_iters, st.tol, kv.as<double>(), nullptr, nullptr);
        }
        // apply_update_ (jfnk.cpp:63-93) and the new residual
        launch_add_rows(U.as<double>(), dU.as<double>(), (int)mesh.N, nc(), stream);
        CUDA_OK(cudaGetLastError());
        state_changed(-1);
        ensure_prims(prec);
        eval_rhs(prec);
        st.step++;
        if (out) {
            out->relative_residual = st.norms[0] / st.initial[0];
            for (int q = 0; q < 6; q++) out->residual_norms[q] = st.norms[q];
            out->gmres_iterations = r.iters;
            out->gmres_converged = r.success ? 1 : 0;
            out->gmres_residual = r.residual;
            out->dt_star = dt_star;
            out->cfl = cfl;
            out->step = st.step;
            for (int q = 0; q < 6; q++) out->initial_norms[q] = st.initial[q];
        }
    }

    // One pseudo-time step of the steady adjoint J^T lambda + g = 0 (J = dR/dU at
    // the current state): r = J^T lambda + g, GMRES on S (I/dt* - J^T) S^-1 y = S r
    // with the steady solver's settings, lambda += S^-1 y.  S scales each conserved
    // variable to its RMS over the cells (density and energy; sqrt of their product
    // for the momenta): density and energy differ by ~1e5, and GMRES on the
    // unscaled operator stagnates on the energy rows.  The continuation converges
    // wherever the forward pseudo-time iteration does (J^T has J's spectrum) and
    // becomes restarted GMRES on the scaled J^T as the CFL grows.
    DBuf adj_r, adj_d, adj_t, adj_norm;
    int adj_krylov = 0;  // GMRES length of the adjoint step (0: the steady solver's)
    void adjoint_step(const double* g, double* lam, double cfl, ibisgb_adjoint_status* out) {
        if (n_cases > 1) throw StateError("steady-state solves run one case per context, not on a batch");
        if (!have_state) throw StateError("no state: call ibisgb_set_primitives first");
        const Steady& st = steady;
        const size_t n = nvars();
        const int ncv = nc();
        const int m = adj_krylov > 0 ? adj_krylov : st.max_iters;
        ensure_krylov(m);
        adj_r.alloc(sizeof(double) * n);
        adj_d.alloc(sizeof(double) * n);
        adj_t.alloc(sizeof(double) * n);
        adj_norm.alloc(sizeof(double) * 8);
        double* r = adj_r.as<double>();
        double* d = adj_d.as<double>();
        double* t = adj_t.as<double>();
        double* nrm = adj_norm.as<double>();
        // RMS of each conserved variable (U is one array per variable)
        const int64_t N = mesh.N;
        for (int q = 0; q < ncv; q++)
            launch_dot(U.as<double>() + q * N, U.as<double>() + q * N, N, kpart.as<double>(), nrm + 2 + q, true,
                       stream);
        vjp(lam, r, nullptr, true);
        launch_axpby(r, g, (long long)n, 1.0, 1.0, stream);  // r = J^T lambda + g
        launch_dot(r, r, (long long)n, kpart.as<double>(), nrm, true, stream);
        double hn[8] = {};
        CUDA_OK(cudaMemcpyAsync(hn, nrm, sizeof(double) * (2 + ncv), cudaMemcpyDeviceToHost, stream));
        CUDA_OK(cudaStreamSynchronize(stream));
        const double rnorm = hn[0];
        const double inv_sqrt_n = 1.0 / std::sqrt((double)N);
        const double rho_s = hn[2] * inv_sqrt_n, e_s = hn[2 + ncv - 1] * inv_sqrt_n;
        if (!(rho_s > 0.0) || !(e_s > 0.0)) throw StateError("adjoint scaling: the state has no density or energy");
        RowScale sc{}, isc{};
        for (int q = 0; q < ncv; q++) {
            sc.s[q] = (q == 0) ? rho_s : (q == ncv - 1) ? e_s : std::sqrt(rho_s * e_s);
            isc.s[q] = 1.0 / sc.s[q];
        }
        launch_scale_rows(r, r, (long long)n, ncv, sc, stream);  // S r
        launch_dot(r, r, (long long)n, kpart.as<double>(), nrm + 1, true, stream);
        double srnorm = 0.0;
        CUDA_OK(cudaMemcpyAsync(&srnorm, nrm + 1, sizeof(double), cudaMemcpyDeviceToHost, stream));
        const double stable = estimate_dt(IBISGB_F64);  // synchronizes the stream
        const double dt_star = cfl * stable, inv = 1.0 / dt_star;
        CUDA_OK(cudaMemsetAsync(d, 0, sizeof(double) * n, stream));
        auto A = [&](const double* x, double* y) {  // y = S (I/dt* - J^T) S^-1 x
            launch_scale_rows(t, x, (long long)n, ncv, isc, stream);
            vjp(t, y, nullptr, true);
            launch_axpby(y, t, (long long)n, inv, -1.0, stream);
            launch_scale_rows(y, y, (long long)n, ncv, sc, stream);
        };
        GmresOut res = gmres(A, r, d, m, st.tol, kv.as<double>(), nullptr, nullptr);
        launch_scale_rows(d, d, (long long)n, ncv, isc, stream);
        launch_axpby(lam, d, (long long)n, 1.0, 1.0, stream);
        CUDA_OK(cudaGetLastError());
        CUDA_OK(cudaStreamSynchronize(stream));
        if (out) {
            out->residual_norm = rnorm;
            out->scaled_residual_norm = srnorm;
            out->gmres_iterations = res.iters;
            out->gmres_converged = res.success ? 1 : 0;
            out->gmres_residual = res.residual;
            out->dt_star = dt_star;
        }
    }

    // the preconditioner's own GMRES, with separate Krylov storage
    DBuf pv, pw, pr0, pH, ppart, pscal;
    template <class Op>
    void inner_gmres(Op&& A, const double* b, double* x, int m, double tol) {
        const size_t n = nvars();
        pv.alloc(sizeof(double) * n * (m + 1));
        // reuse the outer storage layout through a temporary swap of the work buffers
        std::swap(kw.p, pw.p); std::swap(kw.bytes, pw.bytes);
        std::swap(kr0.p, pr0.p); std::swap(kr0.bytes, pr0.bytes);
        std::swap(kH.p, pH.p); std::swap(kH.bytes, pH.bytes);
        std::swap(kscal.p, pscal.p); std::swap(kscal.bytes, pscal.bytes);
        kw.alloc(sizeof(double) * n);
        kr0.alloc(sizeof(double) * n);
        kH.alloc(sizeof(double) * (m + 1) * (m + 1));
        kscal.alloc(sizeof(double) * (2 * m + 8));
        gmres(A, b, x, m, tol, pv.as<double>(), nullptr, nullptr);
        std::swap(kw.p, pw.p); std::swap(kw.bytes, pw.bytes);
        std::swap(kr0.p, pr0.p); std::swap(kr0.bytes, pr0.bytes);
        std::swap(kH.p, pH.p); std::swap(kH.bytes, pH.bytes);
        std::swap(kscal.p, pscal.p); std::swap(kscal.bytes, pscal.bytes);
    }

    // Launch-variant autotuner: times every variant of the recon, face and update
    // kernels on this grid and state (CUDA events, one warm-up launch, then the
    // fastest of three; update in its first-stage Runge-Kutta mode, the
    // primitives it changes restored afterwards) and keeps the fastest.
    // A variant must be 2% faster than the lower-numbered best to be chosen.
    // Every variant computes the same bits, so tuning changes only the speed.
    // Leaves the residual of the current state in stage 0 of k.
    // (The fused stage, timed in the same mode, writes only the other primitive buffer.)
    void autotune(int prec) {
        ensure_prims(prec);
        const int gi = gidx(prec);
        int* vr = var[gi];
        vr[0] = vr[1] = vr[2] = 0;
        if (prec != IBISGB_F64_EXACT) {
            DevView v = view(prec);
            KernelOps o = ops(prec);
            const bool reco = prm.order == 2;
            cudaEvent_t ev[4];
            for (auto& e : ev) CUDA_OK(cudaEventCreate(&e));
            // one warm-up launch, then the fastest of three individually timed ones
            auto timed = [&](const std::function<void()>& launch) {
                launch();
                CUDA_OK(cudaEventRecord(ev[0], stream));
                for (int r = 0; r < 3; r++) {
                    launch();
                    CUDA_OK(cudaEventRecord(ev[r + 1], stream));
                }
                CUDA_OK(cudaGetLastError());
                CUDA_OK(cudaEventSynchronize(ev[3]));
                double best = 0.0;
                for (int r = 0; r < 3; r++) {
                    float ms = 0.f;
                    CUDA_OK(cudaEventElapsedTime(&ms, ev[r], ev[r + 1]));
                    if (r == 0 || ms < best) best = ms;
                }
                return best;
            };
            // The update kernel is timed in its first-stage Runge-Kutta mode (it also forms
            // and commits the next stage state); the primitives it overwrites are restored.
            const size_t pbytes = (float_storage(prec) ? sizeof(float) : sizeof(double)) * 7 * mesh.NT();
            const size_t gbytes = (float_storage(prec) ? sizeof(float) : sizeof(double)) * 5 * mesh.G;
            const size_t lbytes = is_ff(prec) ? sizeof(float) * 7 * mesh.NT() : 0;
            const size_t vlbytes = is_ff(prec) ? sizeof(float) * 5 * mesh.G : 0;
            tune_save.alloc(pbytes + gbytes + lbytes + vlbytes + 16);
            CUDA_OK(cudaMemcpyAsync(tune_save.p, v.prim, pbytes, cudaMemcpyDeviceToDevice, stream));
            if (gbytes)
                CUDA_OK(cudaMemcpyAsync((char*)tune_save.p + pbytes, v.vghost, gbytes, cudaMemcpyDeviceToDevice, stream));
            if (lbytes)
                CUDA_OK(cudaMemcpyAsync((char*)tune_save.p + pbytes + gbytes, v.prim_lo, lbytes,
                                        cudaMemcpyDeviceToDevice, stream));
            if (vlbytes)
                CUDA_OK(cudaMemcpyAsync((char*)tune_save.p + pbytes + gbytes + lbytes, v.vghost_lo, vlbytes,
                                        cudaMemcpyDeviceToDevice, stream));
            auto launch_k = [&](int k, int w) {
                if (k == 0) o.recon(v, prm, reco, w, stream);
                else if (k == 1) o.face_flux(v, prm, reco, w, stream);
                else o.update(v, prm, ctl_host.stages > 1 ? 2 : 0, 0, nullptr, 0, w, stream);
            };
            for (int k = 0; k < 3; k++) {
                if (k == 0 && !reco && !prm.viscous) continue;  // no recon kernel
                double* t = tune_ms[gi][k];
                for (int w = 0; w < kNumVariants; w++) t[w] = timed([&] { launch_k(k, w); });
                // a time far above the others is an outside disturbance: measure it again
                const double tmin = *std::min_element(t, t + kNumVariants);
                for (int w = 0; w < kNumVariants; w++)
                    if (t[w] > 3.0 * tmin) t[w] = std::min(t[w], timed([&] { launch_k(k, w); }));
                double best = 0.0;
                for (int w = 0; w < kNumVariants; w++)
                    if (w == 0 || t[w] < 0.98 * best) { best = t[w]; vr[k] = w; }
                // leave the chosen kernel's outputs for the next kernel's timing
                if (k == 0) o.recon(v, prm, reco, vr[0], stream);
                if (k == 1) o.face_flux(v, prm, reco, vr[1], stream);
            }
            CUDA_OK(cudaMemcpyAsync(v.prim, tune_save.p, pbytes, cudaMemcpyDeviceToDevice, stream));
            if (gbytes)
                CUDA_OK(cudaMemcpyAsync(v.vghost, (char*)tune_save.p + pbytes, gbytes, cudaMemcpyDeviceToDevice, stream));
            if (lbytes)
                CUDA_OK(cudaMemcpyAsync(v.prim_lo, (char*)tune_save.p + pbytes + gbytes, lbytes,
                                        cudaMemcpyDeviceToDevice, stream));
            if (vlbytes)
                CUDA_OK(cudaMemcpyAsync(v.vghost_lo, (char*)tune_save.p + pbytes + gbytes + lbytes, vlbytes,
                                        cudaMemcpyDeviceToDevice, stream));
            if (is_mixed(prec)) {
                generic_ms = tune_ms[gi][0][vr[0]] + tune_ms[gi][1][vr[1]] + tune_ms[gi][2][vr[2]];
                fused_ms = 0.0;
                tile_ms = march_ms = 0.0;
                if (fused_mode != 0 && check_fused()) {
                    upload_fused();
                    // the fused stage in the same first-stage mode, writing the other buffer:
                    // the tile kernel and, on one 3-D block, the plane-marching kernel at
                    // several chunk lengths; the faster kernel is the fused stage
                    const int fm = ctl_host.stages > 1 ? 2 : 0;
                    auto time_fused = [&](bool march, int kc) {
                        const double a = timed([&] { launch_fused_any(v, prim_cur, fm, 0, 0, march, kc); });
                        const double b = timed([&] { launch_fused_any(v, prim_cur, fm, 0, 0, march, kc); });
                        return std::min(a, b);
                    };
                    if (march_mode != 1) tile_ms = time_fused(false, 0);
                    if (march_mode != 0 && check_march()) {
                        upload_march();
                        const int nk = slay.blocks[0].nk;
                        std::vector<int> kcs;
                        if (march_kc_req > 0) kcs.push_back(march_kc_req);
                        else
                            for (int kc : {16, 32, 64})
                                if (kc < 2 * nk) kcs.push_back(kc);
                        for (int kc : kcs) {
                            const double t = time_fused(true, kc);
                            if (march_ms == 0.0 || t < march_ms) { march_ms = t; march_kc = kc; }
                        }
                        check_march_fault();
                    }
                    march_on = march_ms > 0.0 && (tile_ms == 0.0 || march_ms < tile_ms);
                    fused_ms = march_on ? march_ms : tile_ms;
                }
                // the per-cell flux path: recon (as chosen) + k_cell_update in the same mode,
                // writing the other primitive buffer (the current one stays as it is)
                cell_ms = 0.0;
                if (cell_mode != 0 && cell_eligible()) {
                    prim_alt.alloc(sizeof(float) * 7 * mesh.NT());
                    void* other = mixed_prim(prim_cur ^ 1);
                    const int cm = ctl_host.stages > 1 ? 2 : 0;
                    double best = 0.0;
                    for (int w = 0; w < kNumVariants; w++) {
                        double t = timed([&] { o.cell_update(v, prm, reco, cm, 0, 0, w, other, stream); });
                        if (w == 0 || t < 0.98 * best) { best = t; cell_var = w; }
                    }
                    cell_ms = tune_ms[gi][0][vr[0]] + best;
                }
                const double generic = generic_ms;
                bool f_ok = fused_ms > 0.0, c_ok = cell_ms > 0.0;
                if (fused_mode == 1) {
                    fused_on = true;
                    cell_on = false;
                } else if (cell_mode == 1 && c_ok) {
                    fused_on = false;
                    cell_on = true;
                } else {
                    fused_on = fused_mode == -1 && f_ok && fused_ms < generic && (!c_ok || fused_ms < cell_ms);
                    cell_on = !fused_on && cell_mode == -1 && c_ok && cell_ms < generic;
                }
            }
            CUDA_OK(cudaStreamSynchronize(stream));
            for (auto& e : ev) cudaEventDestroy(e);
        }
        tuned[gi] = true;
        if (graph[gi]) {
            cudaGraphExecDestroy(graph[gi]);
            graph[gi] = nullptr;
        }
        if (is_mixed(prec)) drop_mixed_graphs();
    }

    // fused stage: -1 the autotuner decides, 0 never, 1 always (if eligible)
    void set_fused(int mode) {
        if (mode < -1 || mode > 1) throw ArgError("fused mode must be -1, 0 or 1");
        if (mode == 1 && !check_fused()) throw ArgError("the fused stage does not apply: " + fused_why);
        fused_mode = mode;
        if (mode == 1) {
            upload_fused();
            if (march_mode == 1 || (march_mode == -1 && march_on)) {
                upload_march();
                march_on = true;
                if (march_kc_req > 0) march_kc = march_kc_req;
            } else {
                march_on = false;
            }
        }
        if (mode >= 0) fused_on = mode == 1;
        if (fused_on) cell_on = false;
        if (mode < 0) tuned[1] = false;
        drop_mixed_graphs();
    }

    // kernel of the fused stage: -1 the autotuner decides, 0 the tile kernel, 1 the
    // plane-marching kernel (kc planes per CTA, 0: tuned)
    void set_fused_kind(int kind, int kc) {
        if (kind < -1 || kind > 1) throw ArgError("fused kind must be -1, 0 or 1");
        if (kc < 0) throw ArgError("planes per CTA must be >= 0");
        if (kind == 1 && !check_march()) throw ArgError("the plane-marching stage does not apply: " + march_why);
        march_mode = kind;
        march_kc_req = kc;
        if (kind == 1) {
            upload_march();
            if (kc > 0) march_kc = kc;
        }
        if (kind >= 0) march_on = kind == 1;
        if (kind < 0 || (kind == 1 && kc == 0)) tuned[1] = false;
        drop_mixed_graphs();
    }

    // per-cell flux path: -1 the autotuner decides, 0 never, 1 always (if eligible)
    void set_cell_flux(int mode) {
        if (mode < -1 || mode > 1) throw ArgError("cell flux mode must be -1, 0 or 1");
        if (mode == 1 && !cell_eligible()) throw ArgError("the per-cell flux path does not apply: " + cell_why());
        cell_mode = mode;
        if (mode == 1) {
            ensure_device();
            prim_alt.alloc(sizeof(float) * 7 * mesh.NT());
            cell_on = true;
            fused_on = false;
            if (fused_mode == 1) fused_mode = -1;
        }
        if (mode == 0) cell_on = false;
        if (mode < 0) tuned[1] = false;
        drop_mixed_graphs();
    }

    void set_variants(int prec, const int* w) {
        const int gi = gidx(prec);
        for (int k = 0; k < 3; k++) {
            if (w[k] < 0 || w[k] >= kNumVariants) throw ArgError("launch variant out of range");
            var[gi][k] = prec == IBISGB_F64_EXACT ? 0 : w[k];
        }
        tuned[gi] = true;
        if (graph[gi]) {
            cudaGraphExecDestroy(graph[gi]);
            graph[gi] = nullptr;
        }
        if (is_mixed(prec)) {
            cell_var = w[2];  // the per-cell flux kernel takes the update's variant
            drop_mixed_graphs();
        }
    }

    void kernel_times(int prec, int reps, double out[4]) {
        ensure_prims(prec);
        DevView v = view(prec);
        KernelOps o = ops(prec);
        const bool reco = prm.order == 2;
        cudaEvent_t ev[5];
        for (auto& e : ev) CUDA_OK(cudaEventCreate(&e));
        double acc[4] = {0, 0, 0, 0};
        for (int r = 0; r < reps + 1; r++) {  // first round is a warm-up
            CUDA_OK(cudaEventRecord(ev[0], stream));
            const int* vr = var[gidx(prec)];
            o.recon(v, prm, reco, vr[0], stream);
            CUDA_OK(cudaEventRecord(ev[1], stream));
            o.face_flux(v, prm, reco, vr[1], stream);
            CUDA_OK(cudaEventRecord(ev[2], stream));
            o.update(v, prm, 0, 0, nullptr, 0, vr[2], stream);
            CUDA_OK(cudaEventRecord(ev[3], stream));
            CUDA_OK(cudaGetLastError());
            CUDA_OK(cudaEventSynchronize(ev[3]));
            if (r == 0) continue;
            float a, b, c, d;
            CUDA_OK(cudaEventElapsedTime(&a, ev[0], ev[1]));
            CUDA_OK(cudaEventElapsedTime(&b, ev[1], ev[2]));
            CUDA_OK(cudaEventElapsedTime(&c, ev[2], ev[3]));
            CUDA_OK(cudaEventElapsedTime(&d, ev[0], ev[3]));
            acc[0] += a; acc[1] += b; acc[2] += c; acc[3] += d;
        }
        for (auto& e : ev) cudaEventDestroy(e);
        for (int k = 0; k < 4; k++) out[k] = reps > 0 ? acc[k] / reps : 0.0;
    }

    // Device address of pinned host memory mapped into this device's address space
    // (on Grace the GPU reads and writes it over the coherent C2C link), or null.
    static void* mapped_host(const void* p) {
        cudaPointerAttributes a{};
        if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
            cudaGetLastError();  // not a CUDA allocation: pageable memory
            return nullptr;
        }
        return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
    }

    void set_conserved(const double* rows, bool device = false) {
        if (!rows) throw ArgError("U is null");
        ensure_device();
        const int64_t N = mesh.N;
        const size_t bytes = sizeof(double) * nc() * N;
        // rows in the reference numbering -> the internal one (renumbered grids)
        auto internal_rows = [&](const double* r) {
            if (!renumbered()) return r;
            map_a.alloc(bytes);
            map_rows_device(r, map_a.as<double>(), nc(), true);
            return (const double*)map_a.as<double>();
        };
        if (device) {
            launch_rows_to_soa(internal_rows(rows), U.as<double>(), (int)N, nc(), stream);
        } else if (const void* d = mapped_host(rows)) {
            // pinned host rows: the layout kernel reads them in place (one pass, all SMs)
            launch_rows_to_soa(internal_rows((const double*)d), U.as<double>(), (int)N, nc(), stream);
            CUDA_OK(cudaGetLastError());
            CUDA_OK(cudaStreamSynchronize(stream));  // the caller may reuse its buffer on return
        } else {
            out.alloc(bytes);
            CUDA_OK(cudaMemcpyAsync(out.p, rows, bytes, cudaMemcpyHostToDevice, stream));
            launch_rows_to_soa(internal_rows(out.as<double>()), U.as<double>(), (int)N, nc(), stream);
        }
        CUDA_OK(cudaGetLastError());
        if (!have_state) reset_rk();
        have_state = true;
        ic_prims.clear();
        s64.prims_current = false;
        s32.prims_current = false;
        sff.prims_current = false;
    }

    void get_conserved(double* rows) {
        if (!have_state) throw StateError("no initial condition");
        const int64_t N = mesh.N;
        const size_t bytes = sizeof(double) * nc() * N;
        if (renumbered()) {  // internal rows, then gathered into the reference numbering
            map_a.alloc(bytes);
            out.alloc(bytes);
            launch_soa_to_rows(U.as<double>(), map_a.as<double>(), (int)N, nc(), stream);
            void* d = mapped_host(rows);
            map_rows_device(map_a.as<double>(), d ? (double*)d : out.as<double>(), nc(), false);
            if (!d) CUDA_OK(cudaMemcpyAsync(rows, out.p, bytes, cudaMemcpyDeviceToHost, stream));
            CUDA_OK(cudaStreamSynchronize(stream));
            return;
        }
        if (void* d = mapped_host(rows)) {
            // pinned host rows: the layout kernel writes them in place
            launch_soa_to_rows(U.as<double>(), (double*)d, (int)N, nc(), stream);
            CUDA_OK(cudaGetLastError());
            CUDA_OK(cudaStreamSynchronize(stream));
            return;
        }
        out.alloc(bytes);
        launch_soa_to_rows(U.as<double>(), out.as<double>(), (int)N, nc(), stream);
        CUDA_OK(cudaGetLastError());
        CUDA_OK(cudaMemcpyAsync(rows, out.p, bytes, cudaMemcpyDeviceToHost, stream));
        CUDA_OK(cudaStreamSynchronize(stream));
    }

    void get_primitives(double* out7[7]) {
        if (!have_state) throw StateError("no initial condition");
        const int64_t N = mesh.N, NT = mesh.NT();
        if (!ic_prims.empty()) {
            for (int q = 0; q < 7; q++)
                if (out7[q]) std::memcpy(out7[q], &ic_prims[q * NT], sizeof(double) * N);
            return;
        }
        if (!s64.prims_current) {
            upload_geometry<double>(s64);
            ops(IBISGB_F64).prims_from_U(view(IBISGB_F64), prm, stream);
            CUDA_OK(cudaGetLastError());
            s64.prims_current = true;
        }
        for (int q = 0; q < 7; q++)
            if (out7[q])
                CUDA_OK(cudaMemcpyAsync(out7[q], s64.prim.as<double>() + q * NT, sizeof(double) * N,
                                        cudaMemcpyDeviceToHost, stream));
        CUDA_OK(cudaStreamSynchronize(stream));
    }
};

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

namespace {
thread_local std::string g_create_error;
}  // namespace

void ibisgb::set_thread_error(const std::string& msg) { g_create_error = msg; }

namespace {

template <class F>
int guarded(ibisgb_ctx* ctx, F&& f) {
    try {
        f();
        return IBISGB_OK;
    } catch (const ConfigError& e) {
        if (ctx) ctx->err = e.what();
        return IBISGB_ERR_CONFIG;
    } catch (const CudaError& e) {
        if (ctx) ctx->err = e.what();
        return IBISGB_ERR_CUDA;
    } catch (const ArgError& e) {
        if (ctx) ctx->err = e.what();
        return IBISGB_ERR_ARG;
    } catch (const StateError& e) {
        if (ctx) ctx->err = e.what();
        return IBISGB_ERR_STATE;
    } catch (const std::exception& e) {
        if (ctx) ctx->err = e.what();
        return std::string(e.what()) == "bad cells" ? IBISGB_ERR_BAD_CELLS : IBISGB_ERR_GRID;
    }
}

int create_common(const char* config_json, const GridInput* in_arrays, const char* su2_path,
                  ibisgb_ctx** out) {
    if (!out || !config_json) {
        g_create_error = "null argument";
        return IBISGB_ERR_ARG;
    }
    *out = nullptr;
    auto ctx = std::make_unique<ibisgb_ctx>();
    int rc = guarded(ctx.get(), [&] {
        ctx->parse_config(config_json);
        if (su2_path) {
            GridInput in;
            try {
                in = read_su2(su2_path);
            } catch (const std::exception& e) {
                throw std::runtime_error(std::string("grid: ") + e.what());
            }
            ctx->build(in);
        } else {
            ctx->build(*in_arrays);
        }
    });
    if (rc != IBISGB_OK) {
        g_create_error = ctx->err;
        return rc;
    }
    *out = ctx.release();
    return IBISGB_OK;
}
}  // namespace

extern "C" {

int ibisgb_create(const char* config_json, const char* su2_path, ibisgb_ctx** out) {
    if (!su2_path) {
        g_create_error = "su2_path is null";
        return IBISGB_ERR_ARG;
    }
    return create_common(config_json, nullptr, su2_path, out);
}

int ibisgb_create_from_arrays(const char* config_json, int32_t dim, int64_t num_vertices,
                              const double* xyz, int64_t num_cells, const int32_t* cell_types,
                              const int64_t* cell_offsets, const int64_t* cell_vertices,
                              int32_t num_markers, const char* marker_names,
                              const int64_t* marker_offsets, const int32_t* element_types,
                              const int64_t* element_offsets, const int64_t* element_vertices,
                              ibisgb_ctx** out) {
    GridInput in;
    try {
        if (!xyz || !cell_types || !cell_offsets || !cell_vertices || num_vertices < 0 || num_cells < 0)
            throw ArgError("null or negative grid argument");
        in.dim = dim;
        in.xyz.assign(xyz, xyz + 3 * num_vertices);
        for (int64_t c = 0; c < num_cells; c++) {
            ElemKind k = elem_kind_from_vtk(cell_types[c]);
            int64_t n = cell_offsets[c + 1] - cell_offsets[c];
            if (n != vertices_per_elem(k)) throw ArgError("cell vertex count does not match its type");
            in.cells.push(k, cell_vertices + cell_offsets[c], (int)n);
        }
        std::string names = marker_names ? marker_names : "";
        size_t pos = 0;
        for (int32_t m = 0; m < num_markers; m++) {
            size_t nl = names.find('\n', pos);
            std::string tag = names.substr(pos, nl == std::string::npos ? std::string::npos : nl - pos);
            pos = nl == std::string::npos ? names.size() : nl + 1;
            ElemList& dst = in.markers[tag];
            for (int64_t e = marker_offsets[m]; e < marker_offsets[m + 1]; e++) {
                ElemKind k = elem_kind_from_vtk(element_types[e]);
                int64_t n = element_offsets[e + 1] - element_offsets[e];
                dst.push(k, element_vertices + element_offsets[e], (int)n);
            }
        }
    } catch (const std::exception& e) {
        g_create_error = e.what();
        return IBISGB_ERR_ARG;
    }
    return create_common(config_json, &in, nullptr, out);
}

void ibisgb_destroy(ibisgb_ctx* ctx) { delete ctx; }

const char* ibisgb_last_error(const ibisgb_ctx* ctx) {
    return ctx ? ctx->err.c_str() : g_create_error.c_str();
}

int ibisgb_get_sizes(const ibisgb_ctx* ctx, ibisgb_sizes* out) {
    if (!ctx || !out) return IBISGB_ERR_ARG;
    out->num_cells = ctx->mesh.N;
    out->num_ghost_cells = ctx->mesh.G;
    out->num_faces = ctx->mesh.F;
    out->dim = ctx->mesh.dim;
    out->max_faces_per_cell = ctx->mesh.MF;
    out->n_conserved = ctx->mesh.dim + 2;
    out->num_boundaries = (int32_t)ctx->mesh.bounds.size();
    return IBISGB_OK;
}

int ibisgb_set_primitives(ibisgb_ctx* ctx, const double* T, const double* p, const double* vx,
                          const double* vy, const double* vz) {
    if (!ctx) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        if (!ctx->renumbered()) return ctx->set_primitives(T, p, vx, vy, vz);
        const double* in[5] = {T, p, vx, vy, vz};
        std::vector<double> mapped[5];
        const double* pp[5];
        for (int q = 0; q < 5; q++) {
            pp[q] = nullptr;
            if (!in[q]) continue;
            mapped[q].resize(ctx->mesh.N);
            ctx->map_rows_host(in[q], mapped[q].data(), 1, true);
            pp[q] = mapped[q].data();
        }
        ctx->set_primitives(pp[0], pp[1], pp[2], pp[3], pp[4]);
    });
}

int ibisgb_get_primitives(ibisgb_ctx* ctx, double* rho, double* p, double* T, double* e, double* vx,
                          double* vy, double* vz) {
    if (!ctx) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        double* o[7] = {rho, p, T, e, vx, vy, vz};
        if (!ctx->renumbered()) return ctx->get_primitives(o);
        std::vector<double> internal[7];
        double* io[7];
        for (int q = 0; q < 7; q++) {
            io[q] = nullptr;
            if (!o[q]) continue;
            internal[q].resize(ctx->mesh.N);
            io[q] = internal[q].data();
        }
        ctx->get_primitives(io);
        for (int q = 0; q < 7; q++)
            if (o[q]) ctx->map_rows_host(io[q], o[q], 1, false);
    });
}

int ibisgb_get_conserved(ibisgb_ctx* ctx, double* out) {
    if (!ctx || !out) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] { ctx->get_conserved(out); });
}

int ibisgb_set_conserved(ibisgb_ctx* ctx, const double* U) {
    if (!ctx) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] { ctx->set_conserved(U); });
}

int ibisgb_set_conserved_device(ibisgb_ctx* ctx, const double* U_device, void* stream) {
    if (!ctx || !U_device) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        ctx->ensure_device();
        cudaStream_t user = (cudaStream_t)stream;
        cudaEvent_t ev = nullptr;
        if (user && user != ctx->stream) {
            CUDA_OK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            CUDA_OK(cudaEventRecord(ev, user));
            CUDA_OK(cudaStreamWaitEvent(ctx->stream, ev, 0));
        }
        ctx->set_conserved(U_device, true);
        if (ev) {
            CUDA_OK(cudaEventRecord(ev, ctx->stream));
            CUDA_OK(cudaStreamWaitEvent(user, ev, 0));
            CUDA_OK(cudaEventDestroy(ev));
        }
    });
}

int ibisgb_get_stream(ibisgb_ctx* ctx, void** stream) {
    if (!ctx || !stream) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        ctx->ensure_device();
        *stream = (void*)ctx->stream;
    });
}

int ibisgb_kernel_times(ibisgb_ctx* ctx, int32_t precision, int32_t reps, double out[4]) {
    if (!ctx || !out || reps < 0) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        if (precision < 0 || precision > 4) throw ArgError("unknown precision");
        ctx->kernel_times(precision, reps, out);
    });
}

int ibisgb_residual_device(ibisgb_ctx* ctx, int32_t precision, double* dudt_device, void* stream) {
    if (!ctx) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        if (precision < 0 || precision > 4) throw ArgError("unknown precision");
        cudaStream_t user = (cudaStream_t)stream;
        if (user && user != ctx->stream) {  // order the context stream after the caller's work
            cudaEvent_t ev;
            CUDA_OK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            CUDA_OK(cudaEventRecord(ev, user));
            CUDA_OK(cudaStreamWaitEvent(ctx->stream, ev, 0));
            ctx->residual_rows(precision, dudt_device);
            CUDA_OK(cudaEventRecord(ev, ctx->stream));
            CUDA_OK(cudaStreamWaitEvent(user, ev, 0));
            CUDA_OK(cudaEventDestroy(ev));
        } else {
            ctx->residual_rows(precision, dudt_device);
        }
    });
}

int ibisgb_residual(ibisgb_ctx* ctx, int32_t precision, double* dudt) {
    if (!ctx || !dudt) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        if (precision < 0 || precision > 4) throw ArgError("unknown precision");
        const size_t bytes = sizeof(double) * ctx->nc() * ctx->mesh.N;
        ctx->out.alloc(bytes);
        ctx->residual_rows(precision, ctx->out.as<double>());
        CUDA_OK(cudaMemcpyAsync(dudt, ctx->out.p, bytes, cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_OK(cudaStreamSynchronize(ctx->stream));
    });
}

int ibisgb_estimate_dt(ibisgb_ctx* ctx, double* dt) {
    if (!ctx || !dt) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] { *dt = ctx->estimate_dt(IBISGB_F64); });
}

int ibisgb_count_bad_cells(ibisgb_ctx* ctx, int64_t* n) {
    if (!ctx || !n) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        const int64_t N = ctx->mesh.N;
        std::vector<double> rho(N), T(N);
        double* o[7] = {rho.data(), nullptr, T.data(), nullptr, nullptr, nullptr, nullptr};
        ctx->get_primitives(o);
        int64_t bad = 0;  // count_bad_cells, finite_volume.cpp:257-270
        for (int64_t i = 0; i < N; i++)
            if (T[i] < 0.0 || rho[i] < 0.0 || std::isnan(rho[i]) || std::isinf(rho[i])) bad++;
        *n = bad;
    });
}

int ibisgb_rk_run(ibisgb_ctx* ctx, int32_t precision, int64_t n_steps, ibisgb_rk_status* status) {
    if (!ctx || n_steps < 0) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        if (precision < 0 || precision > 4) throw ArgError("unknown precision");
        ctx->rk_run(precision, n_steps, status);
    });
}

int ibisgb_rk_run_host(ibisgb_ctx* ctx, int32_t precision, int64_t n_jobs, int64_t steps_per_job,
                       const double* const* U_in, double* const* U_out, ibisgb_rk_status* status) {
    if (!ctx || !U_in || !U_out || n_jobs <= 0 || steps_per_job < 0) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        if (precision < 0 || precision > 4) throw ArgError("unknown precision");
        ctx->rk_run_host(precision, n_jobs, steps_per_job, U_in, U_out, status);
    });
}

int ibisgb_l2_norms(ibisgb_ctx* ctx, double out[6]) {
    if (!ctx || !out) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        if (!ctx->have_state) throw StateError("no initial condition");
        launch_l2_norms(ctx->k.as<double>(), (int)ctx->mesh.N, ctx->nc(), ctx->l2.as<double>(), ctx->stream);
        CUDA_OK(cudaGetLastError());
        CUDA_OK(cudaMemcpyAsync(out, ctx->l2.p, sizeof(double) * 6, cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_OK(cudaStreamSynchronize(ctx->stream));
    });
}

int ibisgb_get_dump(ibisgb_ctx* ctx, int32_t which, void* buf, int64_t bytes) {
    if (!ctx || !buf) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        const Mesh& m = ctx->mesh;
        const int64_t N = m.N, F = m.F, G = m.G, MF = m.MF, NT = m.NT();
        const int nc = ctx->nc();
        // the dump in the internal numbering first, then (renumbered grids) in the reference's
        std::vector<unsigned char> raw;
        auto put = [&](const void* src, size_t n) {
            if ((int64_t)n > bytes) throw ArgError("dump buffer too small");
            raw.assign((const unsigned char*)src, (const unsigned char*)src + n);
        };
        auto dev = [&](const void* src, size_t n) {
            if ((int64_t)n > bytes) throw ArgError("dump buffer too small");
            if (!src) throw StateError("nothing to dump yet");
            raw.resize(n);
            CUDA_OK(cudaMemcpyAsync(raw.data(), src, n, cudaMemcpyDeviceToHost, ctx->stream));
            CUDA_OK(cudaStreamSynchronize(ctx->stream));
        };
        auto face_rows = [&](const auto& soa_host) {  // SoA face values -> F x nc rows
            std::vector<double> o(soa_host.size());
            for (int64_t f = 0; f < F; f++)
                for (int q = 0; q < nc; q++) o[f * nc + q] = soa_host[q * F + f];
            put(o.data(), sizeof(double) * o.size());
        };
        switch (which) {
            case 0: put(m.left.data(), sizeof(int64_t) * F); break;
            case 1: put(m.right.data(), sizeof(int64_t) * F); break;
            case 2: put(m.cell_face.data(), sizeof(int64_t) * N * MF); break;
            case 3: {
                std::vector<int32_t> o(m.outsign.begin(), m.outsign.end());
                put(o.data(), sizeof(int32_t) * N * MF);
                break;
            }
            case 4: put(m.cell_nbr.data(), sizeof(int64_t) * N * MF); break;
            case 5: put(m.ghost_src.data(), sizeof(int64_t) * G); break;
            case 6: {
                std::vector<double> o;
                for (auto* a : {&m.nx, &m.ny, &m.nz, &m.t1x, &m.t1y, &m.t1z, &m.t2x, &m.t2y, &m.t2z,
                                &m.fcx, &m.fcy, &m.fcz, &m.area})
                    o.insert(o.end(), a->begin(), a->end());
                put(o.data(), sizeof(double) * 13 * F);
                break;
            }
            case 7: {
                std::vector<double> o;
                for (auto* a : {&m.ccx, &m.ccy, &m.ccz, &m.volume}) o.insert(o.end(), a->begin(), a->end());
                put(o.data(), sizeof(double) * 4 * NT);
                break;
            }
            case 8: dev(ctx->branches.p, sizeof(unsigned) * 5 * N); break;
            case 9: {
                if (!ctx->s64.prims_current && !ctx->s32.prims_current) throw StateError("nothing to dump yet");
                dev(ctx->s64.phi.p, sizeof(double) * 5 * N);
                break;
            }
            case 10: {
                if (!ctx->s64.flux.p) throw StateError("nothing to dump yet");
                std::vector<double> soa(nc * F);
                CUDA_OK(cudaMemcpyAsync(soa.data(), ctx->s64.flux.p, sizeof(double) * soa.size(),
                                        cudaMemcpyDeviceToHost, ctx->stream));
                CUDA_OK(cudaStreamSynchronize(ctx->stream));
                face_rows(soa);
                break;
            }
            case 13: {  // face fluxes of the last mixed-precision residual / stage
                if (!ctx->s32.flux.p) throw StateError("nothing to dump yet");
                std::vector<float> soa(nc * F);
                CUDA_OK(cudaMemcpyAsync(soa.data(), ctx->s32.flux.p, sizeof(float) * soa.size(),
                                        cudaMemcpyDeviceToHost, ctx->stream));
                CUDA_OK(cudaStreamSynchronize(ctx->stream));
                face_rows(soa);
                break;
            }
            case 11: put(m.ghost_face.data(), sizeof(int64_t) * G); break;
            case 12: put(m.ghost_bound.data(), sizeof(int64_t) * G); break;
            case 14: {  // the reference id of each internal cell
                std::vector<int64_t> o(N);
                for (int64_t c = 0; c < N; c++) o[c] = ctx->cell_id_to_ref(c);
                put(o.data(), sizeof(int64_t) * N);
                break;
            }
            case 16: {  // the vertices of each face (int64 F x 4, -1 padded)
                if ((int64_t)m.face_vtx_off.size() != F + 1) throw StateError("a batch keeps no face vertices");
                std::vector<int64_t> o(4 * F, -1);
                for (int64_t f = 0; f < F; f++)
                    for (int64_t j = m.face_vtx_off[f], k = 0; j < m.face_vtx_off[f + 1] && k < 4; j++, k++)
                        o[4 * f + k] = m.face_vtx[j];
                put(o.data(), sizeof(int64_t) * 4 * F);
                break;
            }
            case 15: {  // the reference id of each internal face
                std::vector<int64_t> o(F);
                for (int64_t f = 0; f < F; f++) o[f] = ctx->face_id_to_ref(f);
                put(o.data(), sizeof(int64_t) * F);
                break;
            }
            default: throw ArgError("unknown dump");
        }
        if (!ctx->renumbered() || which == 14 || which == 15) {
            std::memcpy(buf, raw.data(), raw.size());
            return;
        }
        const MeshNumbering& nm = ctx->num;
        // rows of w elements of T over n items (cells or faces), reordered to the reference
        // numbering, the values of id arrays mapped by `val`
        auto reorder = [&](auto tag, int64_t n, int64_t w, const std::vector<int64_t>& new_of_ref, int64_t blocks,
                           int64_t block_stride, auto val) {
            using T = decltype(tag);
            const T* in = (const T*)raw.data();
            T* out = (T*)buf;
            std::memcpy(buf, raw.data(), raw.size());  // anything outside the reordered rows (ghosts) as is
            for (int64_t b = 0; b < blocks; b++)
                for (int64_t r = 0; r < n; r++)
                    for (int64_t k = 0; k < w; k++)
                        out[b * block_stride + r * w + k] = val(in[b * block_stride + new_of_ref[r] * w + k]);
        };
        auto same = [](auto x) { return x; };
        auto cell_val = [&](int64_t c) { return ctx->cell_id_to_ref(c); };
        auto face_val = [&](int64_t f) { return ctx->face_id_to_ref(f); };
        switch (which) {
            case 0: case 1: reorder(int64_t{}, F, 1, nm.face_new_of_ref, 1, 0, cell_val); break;
            case 2: reorder(int64_t{}, N, MF, nm.cell_new_of_ref, 1, 0, face_val); break;
            case 3: reorder(int32_t{}, N, MF, nm.cell_new_of_ref, 1, 0, same); break;
            case 4: reorder(int64_t{}, N, MF, nm.cell_new_of_ref, 1, 0, cell_val); break;
            case 5: {
                const int64_t* in = (const int64_t*)raw.data();
                for (int64_t g = 0; g < G; g++) ((int64_t*)buf)[g] = cell_val(in[g]);
                break;
            }
            case 6: reorder(double{}, F, 1, nm.face_new_of_ref, 13, F, same); break;
            case 7: reorder(double{}, N, 1, nm.cell_new_of_ref, 4, NT, same); break;
            case 8: reorder(uint32_t{}, N, 5, nm.cell_new_of_ref, 1, 0, same); break;
            case 9: reorder(double{}, N, 1, nm.cell_new_of_ref, 5, N, same); break;
            case 10: case 13: reorder(double{}, F, nc, nm.face_new_of_ref, 1, 0, same); break;
            case 16: reorder(int64_t{}, F, 4, nm.face_new_of_ref, 1, 0, same); break;
            case 11: {
                const int64_t* in = (const int64_t*)raw.data();
                for (int64_t g = 0; g < G; g++) ((int64_t*)buf)[g] = face_val(in[g]);
                break;
            }
            default: std::memcpy(buf, raw.data(), raw.size());  // 12: per ghost, ghost ids are not renumbered
        }
    });
}

int ibisgb_set_geometry(ibisgb_ctx* ctx, const double* face, const double* cell) {
    if (!ctx || !face || !cell) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] { ctx->set_geometry(face, cell); });
}

int ibisgb_set_scratch_poison(ibisgb_ctx* ctx, int32_t on) {
    if (!ctx) return IBISGB_ERR_ARG;
    ctx->scratch_poison = on != 0;
    return IBISGB_OK;
}

int ibisgb_set_flow_state(ibisgb_ctx* ctx, const char* tag, const double* fs) {
    if (!ctx || !tag || !fs) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] { ctx->set_flow_state(tag, fs); });
}

int ibisgb_get_flow_state(ibisgb_ctx* ctx, const char* tag, double* fs) {
    if (!ctx || !tag || !fs) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] { ctx->flow_state(tag, fs); });
}

int ibisgb_vjp_flow_state_device(ibisgb_ctx* ctx, const double* w_device, double* out_device,
                                 int32_t allow_reconstruction, void* stream) {
    if (!ctx || !w_device || !out_device) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        cudaStream_t user = (cudaStream_t)stream;
        cudaEvent_t ev = nullptr;
        ctx->ensure_device();
        if (user && user != ctx->stream) {
            CUDA_OK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            CUDA_OK(cudaEventRecord(ev, user));
            CUDA_OK(cudaStreamWaitEvent(ctx->stream, ev, 0));
        }
        ctx->vjp_flow_state_rows(w_device, out_device, allow_reconstruction != 0);
        if (ev) {
            CUDA_OK(cudaEventRecord(ev, ctx->stream));
            CUDA_OK(cudaStreamWaitEvent(user, ev, 0));
            CUDA_OK(cudaEventDestroy(ev));
        }
    });
}

int ibisgb_jvp_flow_state_device(ibisgb_ctx* ctx, const double* dfs_device, double* out_device,
                                 int32_t allow_reconstruction, void* stream) {
    if (!ctx || !dfs_device || !out_device) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        cudaStream_t user = (cudaStream_t)stream;
        cudaEvent_t ev = nullptr;
        ctx->ensure_device();
        if (user && user != ctx->stream) {
            CUDA_OK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            CUDA_OK(cudaEventRecord(ev, user));
            CUDA_OK(cudaStreamWaitEvent(ctx->stream, ev, 0));
        }
        ctx->jvp_flow_state_rows(dfs_device, out_device, allow_reconstruction != 0);
        if (ev) {
            CUDA_OK(cudaEventRecord(ev, ctx->stream));
            CUDA_OK(cudaStreamWaitEvent(user, ev, 0));
            CUDA_OK(cudaEventDestroy(ev));
        }
    });
}

int ibisgb_jvp_flow_state(ibisgb_ctx* ctx, const double* dfs, double* out, int32_t allow_reconstruction) {
    if (!ctx || !dfs || !out) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        ctx->ensure_device();
        const size_t n = ctx->nvars(), nb = 7 * ctx->mesh.bounds.size();
        ctx->ensure_krylov(1);
        ctx->fs_io.alloc(sizeof(double) * std::max(nb, (size_t)1));
        if (nb) CUDA_OK(cudaMemcpyAsync(ctx->fs_io.p, dfs, sizeof(double) * nb, cudaMemcpyHostToDevice, ctx->stream));
        ctx->jvp_flow_state_rows(ctx->fs_io.as<double>(), ctx->kw.as<double>(), allow_reconstruction != 0);
        CUDA_OK(cudaMemcpyAsync(out, ctx->kw.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_OK(cudaStreamSynchronize(ctx->stream));
    });
}

int ibisgb_vjp_flow_state(ibisgb_ctx* ctx, const double* w, double* out, int32_t allow_reconstruction) {
    if (!ctx || !w || !out) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        ctx->ensure_device();
        const size_t n = ctx->nvars(), nb = 7 * ctx->mesh.bounds.size();
        ctx->ensure_krylov(1);
        ctx->fs_io.alloc(sizeof(double) * std::max(nb, (size_t)1));
        CUDA_OK(cudaMemcpyAsync(ctx->kr0.p, w, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
        ctx->vjp_flow_state_rows(ctx->kr0.as<double>(), ctx->fs_io.as<double>(), allow_reconstruction != 0);
        if (nb)
            CUDA_OK(cudaMemcpyAsync(out, ctx->fs_io.p, sizeof(double) * nb, cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_OK(cudaStreamSynchronize(ctx->stream));
    });
}

int ibisgb_shared_tables(ibisgb_ctx* ctx, int32_t precision, int32_t* lsq_shared, int32_t* face_classes) {
    if (!ctx || precision < 0 || precision > IBISGB_MIXED_FF) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        ctx->ensure_geometry(precision);
        if (lsq_shared) *lsq_shared = ctx->bufs(precision).lsq_shared ? 1 : 0;
        if (face_classes) *face_classes = ctx->bufs(precision).n_face_classes;
    });
}

int ibisgb_numbering(const ibisgb_ctx* ctx, int32_t* renumbered, int64_t* bandwidth_reference,
                     int64_t* bandwidth_internal) {
    if (!ctx) return IBISGB_ERR_ARG;
    if (renumbered) *renumbered = ctx->renumbered() ? 1 : 0;
    if (bandwidth_reference) *bandwidth_reference = ctx->bandwidth_ref;
    if (bandwidth_internal) *bandwidth_internal = ctx->bandwidth_internal;
    return IBISGB_OK;
}

int ibisgb_jvp_device(ibisgb_ctx* ctx, const double* v_device, double* out_device, double inv_dt_star,
                      int32_t allow_reconstruction, void* stream) {
    if (!ctx || !v_device || !out_device) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        cudaStream_t user = (cudaStream_t)stream;
        cudaEvent_t ev = nullptr;
        ctx->ensure_device();
        if (user && user != ctx->stream) {
            CUDA_OK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            CUDA_OK(cudaEventRecord(ev, user));
            CUDA_OK(cudaStreamWaitEvent(ctx->stream, ev, 0));
        }
        ctx->jvp_rows(v_device, out_device, inv_dt_star, allow_reconstruction != 0);
        if (ev) {
            CUDA_OK(cudaEventRecord(ev, ctx->stream));
            CUDA_OK(cudaStreamWaitEvent(user, ev, 0));
            CUDA_OK(cudaEventDestroy(ev));
        }
    });
}

int ibisgb_jvp(ibisgb_ctx* ctx, const double* v, double* out, double inv_dt_star,
               int32_t allow_reconstruction) {
    if (!ctx || !v || !out) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        ctx->ensure_device();
        const size_t n = ctx->nvars();
        ctx->ensure_krylov(1);
        CUDA_OK(cudaMemcpyAsync(ctx->kr0.p, v, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
        ctx->jvp_rows(ctx->kr0.as<double>(), ctx->kw.as<double>(), inv_dt_star, allow_reconstruction != 0);
        CUDA_OK(cudaMemcpyAsync(out, ctx->kw.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_OK(cudaStreamSynchronize(ctx->stream));
    });
}

int ibisgb_vjp_device(ibisgb_ctx* ctx, const double* w_device, double* out_device, double* ghost_out_device,
                      int32_t allow_reconstruction, void* stream) {
    if (!ctx || !w_device || !out_device) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        cudaStream_t user = (cudaStream_t)stream;
        cudaEvent_t ev = nullptr;
        ctx->ensure_device();
        if (user && user != ctx->stream) {
            CUDA_OK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            CUDA_OK(cudaEventRecord(ev, user));
            CUDA_OK(cudaStreamWaitEvent(ctx->stream, ev, 0));
        }
        ctx->vjp_rows(w_device, out_device, ghost_out_device, allow_reconstruction != 0);
        if (ev) {
            CUDA_OK(cudaEventRecord(ev, ctx->stream));
            CUDA_OK(cudaStreamWaitEvent(user, ev, 0));
            CUDA_OK(cudaEventDestroy(ev));
        }
    });
}

int ibisgb_vjp(ibisgb_ctx* ctx, const double* w, double* out, double* ghost_out, int32_t allow_reconstruction) {
    if (!ctx || !w || !out) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        ctx->ensure_device();
        const size_t n = ctx->nvars();
        const size_t ng = 7 * (size_t)ctx->mesh.G;
        ctx->ensure_krylov(1);
        ctx->adj_gout.alloc(sizeof(double) * std::max(ng, (size_t)1));
        CUDA_OK(cudaMemcpyAsync(ctx->kr0.p, w, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
        ctx->vjp_rows(ctx->kr0.as<double>(), ctx->kw.as<double>(), ghost_out ? ctx->adj_gout.as<double>() : nullptr,
                      allow_reconstruction != 0);
        CUDA_OK(cudaMemcpyAsync(out, ctx->kw.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
        if (ghost_out && ng)
            CUDA_OK(cudaMemcpyAsync(ghost_out, ctx->adj_gout.p, sizeof(double) * ng, cudaMemcpyDeviceToHost,
                                    ctx->stream));
        CUDA_OK(cudaStreamSynchronize(ctx->stream));
    });
}

int ibisgb_vjp_geometry_device(ibisgb_ctx* ctx, const double* w_device, double* face_out_device,
                               double* cell_out_device, int32_t allow_reconstruction, void* stream) {
    if (!ctx || !w_device || !face_out_device || !cell_out_device) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        cudaStream_t user = (cudaStream_t)stream;
        cudaEvent_t ev = nullptr;
        ctx->ensure_device();
        if (user && user != ctx->stream) {
            CUDA_OK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            CUDA_OK(cudaEventRecord(ev, user));
            CUDA_OK(cudaStreamWaitEvent(ctx->stream, ev, 0));
        }
        ctx->vjp_geometry_rows(w_device, face_out_device, cell_out_device, allow_reconstruction != 0);
        if (ev) {
            CUDA_OK(cudaEventRecord(ev, ctx->stream));
            CUDA_OK(cudaStreamWaitEvent(user, ev, 0));
            CUDA_OK(cudaEventDestroy(ev));
        }
    });
}

int ibisgb_jvp_geometry_device(ibisgb_ctx* ctx, const double* dface_device, const double* dcell_device,
                               double* out_device, int32_t allow_reconstruction, void* stream) {
    if (!ctx || !dface_device || !dcell_device || !out_device) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        cudaStream_t user = (cudaStream_t)stream;
        cudaEvent_t ev = nullptr;
        ctx->ensure_device();
        if (user && user != ctx->stream) {
            CUDA_OK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            CUDA_OK(cudaEventRecord(ev, user));
            CUDA_OK(cudaStreamWaitEvent(ctx->stream, ev, 0));
        }
        ctx->jvp_geometry_rows(dface_device, dcell_device, out_device, allow_reconstruction != 0);
        if (ev) {
            CUDA_OK(cudaEventRecord(ev, ctx->stream));
            CUDA_OK(cudaStreamWaitEvent(user, ev, 0));
            CUDA_OK(cudaEventDestroy(ev));
        }
    });
}

int ibisgb_jvp_geometry(ibisgb_ctx* ctx, const double* dface, const double* dcell, double* out,
                        int32_t allow_reconstruction) {
    if (!ctx || !dface || !dcell || !out) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        ctx->ensure_device();
        const size_t n = ctx->nvars(), nf = 13 * (size_t)ctx->mesh.F, ncl = 4 * (size_t)ctx->mesh.NT();
        ctx->ensure_krylov(1);
        ctx->geo_out_face.alloc(sizeof(double) * nf);
        ctx->geo_out_cell.alloc(sizeof(double) * ncl);
        CUDA_OK(cudaMemcpyAsync(ctx->geo_out_face.p, dface, sizeof(double) * nf, cudaMemcpyHostToDevice, ctx->stream));
        CUDA_OK(cudaMemcpyAsync(ctx->geo_out_cell.p, dcell, sizeof(double) * ncl, cudaMemcpyHostToDevice, ctx->stream));
        ctx->jvp_geometry_rows(ctx->geo_out_face.as<double>(), ctx->geo_out_cell.as<double>(), ctx->kw.as<double>(),
                               allow_reconstruction != 0);
        CUDA_OK(cudaMemcpyAsync(out, ctx->kw.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
        CUDA_OK(cudaStreamSynchronize(ctx->stream));
    });
}

int ibisgb_vjp_geometry(ibisgb_ctx* ctx, const double* w, double* face_out, double* cell_out,
                        int32_t allow_reconstruction) {
    if (!ctx || !w || !face_out || !cell_out) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        ctx->ensure_device();
        const size_t n = ctx->nvars(), nf = 13 * (size_t)ctx->mesh.F, ncl = 4 * (size_t)ctx->mesh.NT();
        ctx->ensure_krylov(1);
        ctx->geo_out_face.alloc(sizeof(double) * nf);
        ctx->geo_out_cell.alloc(sizeof(double) * ncl);
        CUDA_OK(cudaMemcpyAsync(ctx->kr0.p, w, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
        ctx->vjp_geometry_rows(ctx->kr0.as<double>(), ctx->geo_out_face.as<double>(), ctx->geo_out_cell.as<double>(),
                               allow_reconstruction != 0);
        CUDA_OK(cudaMemcpyAsync(face_out, ctx->geo_out_face.p, sizeof(double) * nf, cudaMemcpyDeviceToHost,
                                ctx->stream));
        CUDA_OK(cudaMemcpyAsync(cell_out, ctx->geo_out_cell.p, sizeof(double) * ncl, cudaMemcpyDeviceToHost,
                                ctx->stream));
        CUDA_OK(cudaStreamSynchronize(ctx->stream));
    });
}

int ibisgb_adjoint_step(ibisgb_ctx* ctx, const double* g_device, double* lambda_device, double cfl,
                        ibisgb_adjoint_status* status) {
    if (!ctx || !g_device || !lambda_device || !(cfl > 0.0)) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] { ctx->adjoint_step_rows(g_device, lambda_device, cfl, status); });
}

int ibisgb_set_adjoint_krylov(ibisgb_ctx* ctx, int32_t max_iters) {
    if (!ctx || max_iters < 0 || max_iters > 1000) return IBISGB_ERR_ARG;
    ctx->adj_krylov = max_iters;
    return IBISGB_OK;
}

int ibisgb_steady_initialise(ibisgb_ctx* ctx, int32_t precision) {
    if (!ctx) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        if (precision < 0 || precision > 4) throw ArgError("unknown precision");
        ctx->steady_initialise(precision);
    });
}

int ibisgb_steady_norms(ibisgb_ctx* ctx, double norms[6], double initial[6]) {
    if (!ctx) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        if (!ctx->steady.initialised) throw StateError("call ibisgb_steady_initialise first");
        for (int q = 0; q < 6; q++) {
            if (norms) norms[q] = ctx->steady.norms[q];
            if (initial) initial[q] = ctx->steady.initial[q];
        }
    });
}

int ibisgb_newton_step(ibisgb_ctx* ctx, int32_t precision, ibisgb_newton_status* status) {
    if (!ctx) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        if (precision < 0 || precision > 4) throw ArgError("unknown precision");
        ctx->newton_step(precision, status);
    });
}

int ibisgb_autotune(ibisgb_ctx* ctx, int32_t precision, int32_t variants[3], double* times_ms) {
    if (!ctx) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        if (precision < 0 || precision > 4) throw ArgError("unknown precision");
        ctx->autotune(precision);
        const int gi = ibisgb_ctx::gidx(precision);
        for (int k = 0; k < 3; k++) {
            if (variants) variants[k] = ctx->var[gi][k];
            if (times_ms)
                for (int w = 0; w < kNumVariants; w++) times_ms[k * kNumVariants + w] = ctx->tune_ms[gi][k][w];
        }
    });
}

int ibisgb_set_launch_variants(ibisgb_ctx* ctx, int32_t precision, const int32_t variants[3]) {
    if (!ctx || !variants) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        if (precision < 0 || precision > 4) throw ArgError("unknown precision");
        int w[3] = {variants[0], variants[1], variants[2]};
        ctx->set_variants(precision, w);
    });
}

int ibisgb_launch_variants(int32_t* count, int32_t* threads, int32_t* min_blocks) {
    if (!count) return IBISGB_ERR_ARG;
    *count = kNumVariants;
    for (int w = 0; w < kNumVariants; w++) {
        if (threads) threads[w] = kVariantThreads[w];
        if (min_blocks) min_blocks[w] = kVariantMinBlocks[w];
    }
    return IBISGB_OK;
}

int ibisgb_check_conversions(int64_t samples, uint64_t seed, int64_t* mismatches) {
    if (!mismatches || samples < 0) return IBISGB_ERR_ARG;
    unsigned long long m = 0;
    if (check_float_conversions((long long)samples, (unsigned long long)seed, &m) != 0) {
        g_create_error = "CUDA failure in the conversion self-check";
        return IBISGB_ERR_CUDA;
    }
    *mismatches = (int64_t)m;
    return IBISGB_OK;
}

int ibisgb_set_fused(ibisgb_ctx* ctx, int32_t mode) {
    if (!ctx) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] { ctx->set_fused(mode); });
}

int ibisgb_fused_info(ibisgb_ctx* ctx, int32_t* eligible, int32_t* enabled, double* times_ms, char* reason,
                      int32_t reason_len) {
    if (!ctx) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        const bool el = ctx->check_fused();
        if (eligible) *eligible = el ? 1 : 0;
        if (enabled) *enabled = ctx->fused_on ? 1 : 0;
        if (times_ms) { times_ms[0] = ctx->fused_ms; times_ms[1] = ctx->generic_ms; }
        if (reason && reason_len > 0) {
            std::snprintf(reason, (size_t)reason_len, "%s", ctx->fused_why.c_str());
        }
    });
}

int ibisgb_set_fused_kind(ibisgb_ctx* ctx, int32_t kind, int32_t planes_per_cta) {
    if (!ctx) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] { ctx->set_fused_kind(kind, planes_per_cta); });
}

int ibisgb_fused_kind(ibisgb_ctx* ctx, int32_t* march_eligible, int32_t* march_in_use, int32_t* planes_per_cta,
                      double* times_ms, char* reason, int32_t reason_len) {
    if (!ctx) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        const bool el = ctx->check_march();
        if (march_eligible) *march_eligible = el ? 1 : 0;
        if (march_in_use) *march_in_use = ctx->march_on ? 1 : 0;
        if (planes_per_cta) *planes_per_cta = ctx->march_kc;
        if (times_ms) { times_ms[0] = ctx->tile_ms; times_ms[1] = ctx->march_ms; }
        if (reason && reason_len > 0) std::snprintf(reason, (size_t)reason_len, "%s", ctx->march_why.c_str());
    });
}

int ibisgb_set_cell_flux(ibisgb_ctx* ctx, int32_t mode) {
    if (!ctx) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] { ctx->set_cell_flux(mode); });
}

int ibisgb_cell_flux_info(ibisgb_ctx* ctx, int32_t* eligible, int32_t* enabled, int32_t* variant,
                          double* times_ms) {
    if (!ctx) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        if (eligible) *eligible = ctx->cell_eligible() ? 1 : 0;
        if (enabled) *enabled = ctx->cell_on ? 1 : 0;
        if (variant) *variant = ctx->cell_var;
        if (times_ms) { times_ms[0] = ctx->cell_ms; times_ms[1] = ctx->generic_ms; }
    });
}

int ibisgb_batch_create(ibisgb_ctx* const* cases, int32_t n_cases, ibisgb_ctx** out) {
    if (!out || !cases || n_cases < 1) {
        g_create_error = "ibisgb_batch_create: null argument or no cases";
        return IBISGB_ERR_ARG;
    }
    *out = nullptr;
    auto ctx = std::make_unique<ibisgb_ctx>();
    int rc = guarded(ctx.get(), [&] { ctx->merge(cases, n_cases); });
    if (rc != IBISGB_OK) {
        g_create_error = ctx->err;
        return rc;
    }
    *out = ctx.release();
    return IBISGB_OK;
}

int ibisgb_batch_layout(const ibisgb_ctx* ctx, int32_t* n_cases, int64_t* cell_offsets,
                        int64_t* face_offsets, int64_t* ghost_offsets) {
    if (!ctx) return IBISGB_ERR_ARG;
    const int n = ctx->n_cases;
    if (n_cases) *n_cases = n;
    for (int c = 0; c <= n; c++) {
        const bool one = n == 1;
        if (cell_offsets) cell_offsets[c] = one ? (c ? ctx->mesh.N : 0) : ctx->cell_off[c];
        if (face_offsets) face_offsets[c] = one ? (c ? ctx->mesh.F : 0) : ctx->face_off[c];
        if (ghost_offsets) ghost_offsets[c] = one ? (c ? ctx->mesh.G : 0) : ctx->ghost_off[c];
    }
    return IBISGB_OK;
}

int ibisgb_batch_status(ibisgb_ctx* ctx, ibisgb_rk_status* per_case) {
    if (!ctx || !per_case) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        if (ctx->last_ctl.size() != (size_t)ctx->n_cases) throw StateError("no Runge-Kutta state yet");
        for (int c = 0; c < ctx->n_cases; c++) {
            const StepCtl& x = ctx->last_ctl[c];
            per_case[c].t = x.t; per_case[c].dt = x.dt; per_case[c].stable_dt = x.stable_dt;
            per_case[c].steps = x.steps; per_case[c].bad_cells = (int64_t)x.bad_cells;
            per_case[c].device_ms = ctx->last_ms;
        }
    });
}

int ibisgb_synchronize(ibisgb_ctx* ctx) {
    if (!ctx) return IBISGB_ERR_ARG;
    return guarded(ctx, [&] {
        if (ctx->stream) CUDA_OK(cudaStreamSynchronize(ctx->stream));
    });
}

}  // extern "C"
