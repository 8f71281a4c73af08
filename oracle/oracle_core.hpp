// ORACLE — test infrastructure only. Never linked into the product.
//
// A CPU restatement of ibis's compressible finite-volume residual path
// (grid preprocessing, ghost-cell boundary actions, least-squares gradients,
// Barth-Jespersen limiting, MUSCL reconstruction, the Hanel / AUSMDV /
// LDFSS2 / Rusanov flux calculators, viscous fluxes, the face->cell surface
// integral, the CFL time-step estimate, explicit Runge-Kutta, and the
// dual-number Jacobian-vector product + GMRES of the steady solver).
// Every function cites the reference file:line it restates; operation order
// follows the reference so that results can be compared bit for bit where no
// library math function (pow) is involved. Build with -ffp-contract=off.
//
// The reference itself cannot be compiled here: it needs Kokkos,
// nlohmann/json and spdlog, none of which is installed (its git submodules
// are empty). Parity of this restatement is pinned by the golden vectors in
// the reference's own unit tests (grid numbering, outsigns, neighbours,
// ghost-cell centres, LSQ gradient of a linear field, GMRES/FGMRES solutions,
// CFL schedule) and by the free-stream-preservation property of its
// integration tests; flux calculators, limiter, reconstruction, viscous flux,
// boundary actions, RK and JFNK have no reference test, so parity there is
// "unpinned" beyond this line-by-line restatement.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "../ibis_gb300/csrc/json_lite.hpp"

namespace oracle {

using ibisgb::Json;
static constexpr size_t NONE = std::numeric_limits<size_t>::max();

// ---------------------------------------------------------------------------
// Dual numbers with the reference's semantics (src/util/util/dual.h:11-346):
// comparisons use the real part, min/max pick an operand by real part
// (ties pick the second operand), abs flips on real<0, floor applies floor to
// BOTH parts, pow(b, p) includes the p.dual*real*log(b) term, copysign keeps
// or flips the dual part.
// ---------------------------------------------------------------------------
struct Dual {
    double re = 0.0, du = 0.0;
    Dual() = default;
    Dual(double r) : re(r), du(0.0) {}
    Dual(double r, double d) : re(r), du(d) {}
    Dual& operator=(double r) { re = r; du = 0.0; return *this; }
    Dual operator-() const { return {-re, -du}; }
    Dual& operator+=(const Dual& o) { re += o.re; du += o.du; return *this; }
    Dual& operator-=(const Dual& o) { re -= o.re; du -= o.du; return *this; }
    Dual& operator*=(const Dual& o) { du = re * o.du + du * o.re; re *= o.re; return *this; }
};
// dual.h:139-141, 170-175, 183
inline Dual operator+(const Dual& a, const Dual& b) { return {a.re + b.re, a.du + b.du}; }
inline Dual operator-(const Dual& a, const Dual& b) { return {a.re - b.re, a.du - b.du}; }
inline Dual operator*(const Dual& a, const Dual& b) { return {a.re * b.re, a.re * b.du + a.du * b.re}; }
inline Dual operator/(const Dual& a, const Dual& b) {
    return {a.re / b.re, (a.du * b.re - a.re * b.du) / (b.re * b.re)};
}
inline Dual operator+(const Dual& a, double b) { return {a.re + b, a.du}; }
inline Dual operator+(double a, const Dual& b) { return {a + b.re, b.du}; }
inline Dual operator-(const Dual& a, double b) { return {a.re - b, a.du}; }
inline Dual operator-(double a, const Dual& b) { return {a - b.re, -b.du}; }
inline Dual operator*(const Dual& a, double b) { return {a.re * b, a.du * b}; }
inline Dual operator*(double a, const Dual& b) { return {b.re * a, b.du * a}; }
inline Dual operator/(const Dual& a, double b) { return {a.re / b, a.du / b}; }
inline Dual operator/(double a, const Dual& b) { return {a / b.re, -b.du * a / (b.re * b.re)}; }
inline bool operator<(const Dual& a, const Dual& b) { return a.re < b.re; }
inline bool operator>(const Dual& a, const Dual& b) { return a.re > b.re; }
inline bool operator<=(const Dual& a, const Dual& b) { return a.re <= b.re; }
inline bool operator>=(const Dual& a, const Dual& b) { return a.re >= b.re; }
inline bool operator==(const Dual& a, const Dual& b) { return a.re == b.re; }
inline bool operator!=(const Dual& a, const Dual& b) { return a.re != b.re; }

inline double real_part(double x) { return x; }
inline double real_part(const Dual& x) { return x.re; }
inline double dual_part(double) { return 0.0; }
inline double dual_part(const Dual& x) { return x.du; }
inline void set_real(double& x, double v) { x = v; }
inline void set_real(Dual& x, double v) { x.re = v; }
inline void set_dual(double&, double) {}
inline void set_dual(Dual& x, double v) { x.du = v; }

// src/util/util/real.h:15-68 (Kokkos math forwarding for doubles)
inline double o_sqrt(double x) { return std::sqrt(x); }
inline double o_pow(double b, double p) { return std::pow(b, p); }
inline double o_abs(double x) { return std::fabs(x); }
inline double o_min(double a, double b) { return (b < a) ? b : a; }
inline double o_max(double a, double b) { return (a < b) ? b : a; }
inline double o_floor(double x) { return std::floor(x); }
inline double o_copysign(double m, double s) { return std::copysign(m, s); }
inline bool o_isnan(double x) { return std::isnan(x); }
inline bool o_isinf(double x) { return std::isinf(x); }
// src/util/util/dual.h:226-314
inline Dual o_sqrt(const Dual& d) {
    double r = std::sqrt(d.re);
    return {r, d.du / (2.0 * r)};
}
inline Dual o_pow(const Dual& b, const Dual& p) {
    double r = std::pow(b.re, p.re);
    double d = b.du * p.re * std::pow(b.re, p.re - 1.0) + p.du * r * std::log(b.re);
    return {r, d};
}
inline Dual o_abs(const Dual& d) { return (d.re < 0.0) ? -d : d; }
inline Dual o_max(const Dual& a, const Dual& b) { return a.re > b.re ? a : b; }
inline Dual o_max(double a, const Dual& b) { return a > b.re ? Dual(a) : b; }
inline Dual o_max(const Dual& a, double b) { return a.re > b ? a : Dual(b); }
inline Dual o_min(const Dual& a, const Dual& b) { return a.re < b.re ? a : b; }
inline Dual o_min(double a, const Dual& b) { return a < b.re ? Dual(a) : b; }
inline Dual o_min(const Dual& a, double b) { return a.re < b ? a : Dual(b); }
inline Dual o_floor(const Dual& d) { return {std::floor(d.re), std::floor(d.du)}; }
inline Dual o_copysign(const Dual& m, const Dual& s) {
    double r = std::copysign(m.re, s.re);
    double d = (r - m.re) < 1e-15 ? m.du : -m.du;
    return {r, d};
}
inline bool o_isnan(const Dual& d) { return std::isnan(d.re) || std::isnan(d.du); }
inline bool o_isinf(const Dual& d) { return std::isinf(d.re) || std::isinf(d.du); }

// ---------------------------------------------------------------------------
// Counting scalar: a double that counts the floating-point operations applied to
// it, so that instantiating the templated restatement on it gives the exact
// operation count of a residual evaluation or Runge-Kutta step (the plain FP64
// path's FP64-issue roofline).  The counts are global: count with one thread.
// abs, min, max, floor and copysign are counted apart from the arithmetic.
// ---------------------------------------------------------------------------
struct FlopCounts {
    unsigned long long add = 0, mul = 0, div = 0, sqrt = 0, pow = 0, other = 0;
};
extern FlopCounts g_flops;
struct Cnt {
    double v = 0.0;
    Cnt() = default;
    Cnt(double x) : v(x) {}
    Cnt& operator=(double x) { v = x; return *this; }
    Cnt operator-() const { return Cnt(-v); }
    Cnt& operator+=(const Cnt& o) { g_flops.add++; v += o.v; return *this; }
    Cnt& operator-=(const Cnt& o) { g_flops.add++; v -= o.v; return *this; }
    Cnt& operator*=(const Cnt& o) { g_flops.mul++; v *= o.v; return *this; }
    Cnt& operator/=(const Cnt& o) { g_flops.div++; v /= o.v; return *this; }
};
inline Cnt operator+(const Cnt& a, const Cnt& b) { g_flops.add++; return Cnt(a.v + b.v); }
inline Cnt operator-(const Cnt& a, const Cnt& b) { g_flops.add++; return Cnt(a.v - b.v); }
inline Cnt operator*(const Cnt& a, const Cnt& b) { g_flops.mul++; return Cnt(a.v * b.v); }
inline Cnt operator/(const Cnt& a, const Cnt& b) { g_flops.div++; return Cnt(a.v / b.v); }
inline bool operator<(const Cnt& a, const Cnt& b) { return a.v < b.v; }
inline bool operator>(const Cnt& a, const Cnt& b) { return a.v > b.v; }
inline bool operator<=(const Cnt& a, const Cnt& b) { return a.v <= b.v; }
inline bool operator>=(const Cnt& a, const Cnt& b) { return a.v >= b.v; }
inline bool operator==(const Cnt& a, const Cnt& b) { return a.v == b.v; }
inline bool operator!=(const Cnt& a, const Cnt& b) { return a.v != b.v; }
inline double real_part(const Cnt& x) { return x.v; }
inline double dual_part(const Cnt&) { return 0.0; }
inline void set_real(Cnt& x, double v) { x.v = v; }
inline void set_dual(Cnt&, double) {}
inline Cnt o_sqrt(const Cnt& x) { g_flops.sqrt++; return Cnt(std::sqrt(x.v)); }
inline Cnt o_pow(const Cnt& b, const Cnt& p) { g_flops.pow++; return Cnt(std::pow(b.v, p.v)); }
inline Cnt o_abs(const Cnt& x) { g_flops.other++; return Cnt(std::fabs(x.v)); }
inline Cnt o_min(const Cnt& a, const Cnt& b) { g_flops.other++; return (b.v < a.v) ? b : a; }
inline Cnt o_max(const Cnt& a, const Cnt& b) { g_flops.other++; return (a.v < b.v) ? b : a; }
inline Cnt o_floor(const Cnt& x) { g_flops.other++; return Cnt(std::floor(x.v)); }
inline Cnt o_copysign(const Cnt& m, const Cnt& s) { g_flops.other++; return Cnt(std::copysign(m.v, s.v)); }
inline bool o_isnan(const Cnt& x) { return std::isnan(x.v); }
inline bool o_isinf(const Cnt& x) { return std::isinf(x.v); }

// ---------------------------------------------------------------------------
// Grid input (src/grid/grid/grid_io.{h,cpp})
// ---------------------------------------------------------------------------
enum class ElemType { Line, Tri, Tetra, Quad, Hex, Wedge, Pyramid };

struct ElemIO {
    std::vector<size_t> ids;
    ElemType type;
};

// grid_io.cpp:28-48
ElemType elem_type_from_vtk(size_t t);
// grid_io.cpp:72-91
size_t vertices_of(ElemType t);
// grid_io.cpp:298-348
std::vector<ElemIO> vtk_face_order(const std::vector<size_t>& ids, ElemType type);

struct GridIO {
    size_t dim = 0;
    std::vector<std::array<double, 3>> vertices;
    std::vector<ElemIO> cells;
    std::unordered_map<std::string, std::vector<ElemIO>> markers;
    // grid_io.cpp:218-268
    void read_su2(const std::string& path);
};

// ---------------------------------------------------------------------------
// Grid block (src/grid/grid/grid.h, interface.{h,cpp}, cell.h, geom.h)
// ---------------------------------------------------------------------------
struct PeriodicLink {
    std::string partner;
    double offset[3];
};

template <typename T>
struct Grid {
    size_t dim = 0, N = 0, G = 0, F = 0, NV = 0;
    std::vector<T> vx, vy, vz;

    std::vector<std::vector<size_t>> face_vertices;
    std::vector<ElemType> face_shape;
    std::vector<size_t> left, right;
    std::vector<T> nx, ny, nz, t1x, t1y, t1z, t2x, t2y, t2z, cx, cy, cz, area;

    std::vector<std::vector<size_t>> cell_vertices, cell_faces, cell_nbrs;
    std::vector<std::vector<int>> outsigns;
    std::vector<ElemType> cell_shape;
    std::vector<T> volume, ccx, ccy, ccz;  // length N+G

    std::vector<std::string> boundary_tags;                 // sorted (json object order)
    std::map<std::string, std::vector<size_t>> ghost_cells;     // per tag
    std::map<std::string, std::vector<size_t>> boundary_faces;  // per tag

    // WLS QR factors r11,r12,r22,r13,r23,r33 per valid cell (gradient.h:119-162)
    std::vector<std::array<T, 6>> r;

    // periodic extension: donor valid cell for each ghost (NONE otherwise)
    std::vector<size_t> ghost_donor;

    void init(const GridIO& io, const Json& boundaries,
              const std::map<std::string, PeriodicLink>& periodic);
    void compute_gradient_weights();
};

// ---------------------------------------------------------------------------
// Flow and conserved storage
// ---------------------------------------------------------------------------
template <typename T>
struct FlowStates {  // src/gas/gas/flow_state.h:49-110, gas_state.h:134-243
    std::vector<T> rho, p, temp, e, vx, vy, vz;
    FlowStates() = default;
    explicit FlowStates(size_t n) { resize(n); }
    void resize(size_t n) {
        rho.assign(n, T(0.0)); p.assign(n, T(0.0)); temp.assign(n, T(0.0)); e.assign(n, T(0.0));
        vx.assign(n, T(0.0)); vy.assign(n, T(0.0)); vz.assign(n, T(0.0));
    }
    size_t size() const { return rho.size(); }
};

template <typename T>
struct Conserved {  // src/finite_volume/finite_volume/conserved_quantities.{h,cpp}
    size_t n = 0, dim = 0, nc = 0;
    std::vector<T> q;  // row-major (cell, component), like View<T**>(n, dim+2)
    Conserved() = default;
    Conserved(size_t n_, size_t dim_) : n(n_), dim(dim_), nc(dim_ + 2), q(n_ * (dim_ + 2), T(0.0)) {}
    T& mass(size_t i) { return q[i * nc]; }
    T& mx(size_t i) { return q[i * nc + 1]; }
    T& my(size_t i) { return q[i * nc + 2]; }
    T& mz(size_t i) { return q[i * nc + 3]; }
    T& energy(size_t i) { return q[i * nc + 1 + dim]; }
    const T& mass(size_t i) const { return q[i * nc]; }
    const T& mx(size_t i) const { return q[i * nc + 1]; }
    const T& my(size_t i) const { return q[i * nc + 2]; }
    const T& mz(size_t i) const { return q[i * nc + 3]; }
    const T& energy(size_t i) const { return q[i * nc + 1 + dim]; }
};

struct Norms {  // ConservedQuantitiesNorm, conserved_quantities.h:9-96
    double global = 0, mass = 0, mx = 0, my = 0, mz = 0, energy = 0;
};

// ---------------------------------------------------------------------------
// Gas model and transport (src/gas/gas/gas_model.h:46-189, transport_properties.h)
// ---------------------------------------------------------------------------
struct IdealGas {
    double R = 287.0, Cv = 717.5, Cp = 1004.5, gamma = 1.4;
};
struct Transport {
    double mu0 = 1.716e-5, T0 = 273.0, Ts = 110.0, Pr = 0.72;
};

// ---------------------------------------------------------------------------
// Boundary actions (src/finite_volume/finite_volume/boundaries/boundary.cpp)
// ---------------------------------------------------------------------------
enum class ActionKind {
    FlowStateCopy, InternalCopy, InternalCopyReflectNormal, InternalVelCopyReflect,
    FixTemperature, SubsonicInflow, SubsonicOutflow, ConstantFlux, PeriodicCopy,
    BoundaryLayerProfile
};

// Natural cubic spline (src/util/util/cubic_spline.{h,cpp}): second
// derivatives from the tridiagonal system of the interior knots, assembled and
// solved (Thomas algorithm) in the reference's operation order; eval clamps to
// the end values outside [x0, x_{n-1}].  m holds the second derivative at every
// knot with m[0] = m[n-1] = 0.  The reference stores only n-2 of them and reads
// the last two knots' values past the end of its array (cubic_spline.cpp:47-48,
// 80-84; cubic_spline.h:27-37); this restatement uses the natural-spline values
// that code intends (the solved m[n-2], and m[n-1] = 0).
struct CubicSpline {
    std::vector<double> x, y, m;
    void fit(const std::vector<double>& xs, const std::vector<double>& ys);  // cubic_spline.cpp:9-89
    double eval(double t) const;                                            // cubic_spline.h:13-38
};

struct Action {
    ActionKind kind;
    // flow_state_copy / subsonic_inflow / constant_flux: T, p, rho, energy, vx, vy, vz
    double fs[7] = {0, 0, 0, 0, 0, 0, 0};
    // the dual parts of fs in the Dual build (a directional derivative with
    // respect to the flow state; zero otherwise, and unread by the real build)
    double fs_du[7] = {0, 0, 0, 0, 0, 0, 0};
    double value = 0.0;  // fix_temperature temperature / subsonic_outflow pressure / profile pressure
    CubicSpline spline_v, spline_T;  // boundary_layer_profile: vx(y) and T(y)
};
struct BoundaryCondition {
    std::vector<Action> pre_reconstruction, post_convective_flux, pre_viscous_grad;
};
// Entry k of an action's flow state in the arithmetic T (with its dual part in
// the Dual build).
template <typename T>
inline T fs_value(const Action& a, int k) { return T(a.fs[k]); }
template <>
inline Dual fs_value<Dual>(const Action& a, int k) { return Dual(a.fs[k], a.fs_du[k]); }

enum class FluxKind { Hanel, Ausmdv, Ldfss2, Rusanov };
enum class Thermo { rho_p, rho_T, rho_u, p_T };

struct FvConfig {
    FluxKind flux = FluxKind::Hanel;
    double ldfss_delta = 2.0;
    int order = 2;
    bool limiter_enabled = true;   // barth_jespersen (true) or unlimited (false)
    double epsilon = 1e-25;
    Thermo thermo = Thermo::rho_u;
    bool viscous = false;
    double signal_factor = 4.0;
};

// Branch record of one Barth-Jespersen evaluation: 2 bits per face slot
// (0: delta_2 == 0, 1: > 0 -> U_max branch, 2: < 0 -> U_min branch) in the low
// 16 bits, and (slot + 1) of the face that set phi in bits 16..23 (0 = phi is 1).
using BranchCode = uint32_t;

template <typename T>
struct FiniteVolume {
    FvConfig cfg;
    size_t dim = 0;
    std::vector<BoundaryCondition> bcs;     // in boundary_tags order
    std::vector<std::vector<size_t>> bc_faces;

    // scratch (finite_volume.h:114-143, convective_flux.h:69-87)
    Conserved<T> flux;
    FlowStates<T> left, right, face_fs;
    // gradients of p, rho, u(=energy), temp, vx, vy, vz on valid cells, 3 comps
    std::vector<std::array<T, 3>> g_p, g_rho, g_u, g_temp, g_vx, g_vy, g_vz;
    std::vector<T> l_p, l_rho, l_u, l_temp, l_vx, l_vy, l_vz;
    // branch records of the last convective limiter evaluation, 5 per cell:
    // the two thermo variables (in reference call order), vx, vy, vz
    std::vector<BranchCode> branches;
    bool record_branches = false;

    void setup(const Grid<T>& grid, const FvConfig& c, const std::vector<BoundaryCondition>& b);
    // finite_volume.cpp:87-96 / 56-85
    void compute_dudt(FlowStates<T>& fs, const Grid<T>& grid, Conserved<T>& dudt,
                      const IdealGas& gas, const Transport& tp, bool allow_reconstruction = true);
    // finite_volume.cpp:130-184
    double estimate_dt(const FlowStates<T>& fs, const Grid<T>& grid, const IdealGas& gas,
                       const Transport& tp);
    // finite_volume.cpp:257-270
    size_t count_bad_cells(const FlowStates<T>& fs, size_t n);

    void apply_ghost_actions(const std::vector<Action>& acts, FlowStates<T>& fs,
                             const Grid<T>& grid, const std::vector<size_t>& faces,
                             const IdealGas& gas);
    void convective_flux(const FlowStates<T>& fs, const Grid<T>& grid, const IdealGas& gas,
                         bool allow_reconstruction);
    void viscous_flux(const FlowStates<T>& fs, const Grid<T>& grid, const IdealGas& gas,
                      const Transport& tp);
    void surface_integral(const Grid<T>& grid, Conserved<T>& dudt);
};

// conserved <-> primitive (primative_conserved_conversion.cpp:4-57)
template <typename T>
void conserved_to_primatives(const Conserved<T>& cq, FlowStates<T>& fs, const IdealGas& gas);
template <typename T>
void primatives_to_conserved(Conserved<T>& cq, const FlowStates<T>& fs);
// conserved_quantities.cpp:40-69
template <typename T>
Norms l2_norms(const Conserved<T>& cq);

// RK driver state (src/solvers/solvers/runge_kutta.cpp)
struct Tableau {
    std::vector<std::vector<double>> a;
    std::vector<double> b, c;
    size_t stages() const { return b.size(); }
    double A(size_t i, size_t j) const { return a[i - 1][j]; }
};

struct RkState {
    Tableau tab;
    double cfl = 0.5, max_time = 1e300, plot_frequency = -1.0, dt_init = -1.0;
    // The stage derivatives of the reference's RungeKutta share one array: it
    // builds them as copies of one ConservedQuantities (runge_kutta.cpp:47-48),
    // and copies of a Kokkos View alias its storage, so every stage reads the
    // derivative the previous stage wrote.  "stage_derivatives": "aliased" in
    // the solver block reproduces that; the default keeps one array per stage
    // (the tableau as written).
    bool aliased_stages = false;
    double t = 0.0, dt = 0.0, stable_dt = 0.0, time_since_last_plot = 0.0;
    // linear CFL schedule (cfl.cpp:101-127) when non-empty
    std::vector<double> cfl_times, cfl_values;
};

// One ibis simulation on one grid: the aggregate Sim<T> (simulation.h:13-23)
template <typename T>
struct Sim {
    Grid<T> grid;
    FiniteVolume<T> fv;
    IdealGas gas;
    Transport tp;
    FlowStates<T> fs;        // N+G rows
    Conserved<T> U;          // N+G rows
    RkState rk;
    std::vector<Conserved<T>> k;
    Conserved<T> k_tmp;
    FlowStates<T> fs_tmp;

    void init_rk(const Json& solver_cfg);
    // runge_kutta.cpp:82-104 after the initial condition is in fs
    void rk_initialise();
    double cfl_eval(double t) const;
    // runge_kutta.cpp:108-119
    void rk_estimate_dt();
    // runge_kutta.cpp:131-203
    void rk_take_step();
};

// Builds a simulation from a config.json object and a grid.
// The "periodic_copy" ghost action is an extension (ibis has no periodic BC).
template <typename T>
std::unique_ptr<Sim<T>> build_sim(const Json& config, const GridIO& io);

FvConfig parse_fv_config(const Json& config);

// WLSGradient::compute_gradients on a real-valued grid (gradient.h:65-116)
void lsq_gradient_real(const Grid<double>& g, const std::vector<double>& values,
                       std::vector<std::array<double, 3>>& grad);

// ---------------------------------------------------------------------------
// Steady-state linearisation + GMRES (steady_state.cpp, gmres.cpp, jfnk.cpp)
// ---------------------------------------------------------------------------
struct GmresResult {
    bool success = false;
    size_t n_iters = 0;
    double tol = -1, residual = -1;
};

// A linear operator y = A x on flat vectors.
using MatVec = std::function<void(const std::vector<double>&, std::vector<double>&)>;

// gmres.cpp:119-182 (un-restarted GMRES, MGS Arnoldi, Givens on the host)
GmresResult gmres_solve(const MatVec& A, const std::vector<double>& rhs, std::vector<double>& x,
                        size_t max_iters, double tol);
// gmres.cpp:234-303 (flexible GMRES with an inner GMRES preconditioner)
GmresResult fgmres_solve(const MatVec& A, const MatVec& P, std::vector<double>& x,
                         const std::vector<double>& rhs, size_t max_iters, double tol,
                         size_t max_prec_iters, double prec_tol);

// SteadyStateLinearisation on a dual simulation
struct Steady {
    std::unique_ptr<Sim<Dual>> sim;
    Conserved<Dual> residuals, cq_tmp;
    FlowStates<Dual> fs_tmp;
    std::vector<double> rhs, dU;
    double dt_star = 1.0;
    size_t n_vars = 0;
    Norms residual_norms, initial_norms;
    GmresResult last;
    // jfnk config
    size_t max_iters = 50;
    double gmres_tol = 1e-2;
    std::vector<double> cfl_times, cfl_values;  // linear schedule when non-empty
    double cfl_const = 0.5;
    bool residual_based = false;
    double rb_threshold = 0.1, rb_power = 0.8, rb_start = 1.0, rb_max = 1e8;
    double rb_prev_cfl = 1.0, rb_prev_res = 1.0;
    bool fgmres = false;
    size_t max_prec_iters = 5;
    double prec_tol = 1e-1;

    void setup(const Json& config, const GridIO& io);
    // steady_state.cpp:52-128
    void matvec(const std::vector<double>& v, std::vector<double>& out, bool allow_reconstruction);
    // steady_state.cpp:130-165
    void eval_rhs();
    // jfnk.cpp:25-30
    void initialise();
    double calculate_cfl(size_t step);
    // jfnk.cpp:39-61
    GmresResult step(size_t step_index);
};

}  // namespace oracle
