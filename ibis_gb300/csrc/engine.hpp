// Types shared by the host context and the device kernels of the residual engine.
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

#include "sblock.hpp"

namespace ibisgb {

enum FluxKind : int { kHanel = 0, kAusmdv = 1, kLdfss2 = 2, kRusanov = 3 };
enum ThermoKind : int { kRhoP = 0, kRhoT = 1, kRhoU = 2, kPT = 3 };

// Ghost-cell actions (src/finite_volume/finite_volume/boundaries/boundary.cpp)
enum ActionKind : int {
    aFlowStateCopy = 0,
    aInternalCopy = 1,
    aReflectNormal = 2,  // internal_copy_reflect_normal
    aVelReflect = 3,     // internal_vel_copy_reflect
    aFixTemperature = 4,
    aSubsonicInflow = 5,
    aSubsonicOutflow = 6,
    aPeriodicCopy = 7,   // extension: copy of the periodic donor cell
    aBoundaryLayer = 8,  // boundary_layer_profile: a fixed state per ghost (its centroid height)
};

constexpr int kMaxActions = 4;
constexpr int kMaxStages = 8;
// Face classes of a uniform lattice: n (3); 2-D t1 x, t1 y, t2 z (3); the left and
// right sides' face centre - centroid (3 + 3, zero for a ghost side); the area; 3 pads.
constexpr int kFaceClassRow = 16;
constexpr int kMaxFaceClasses = 64;

struct Action {
    int kind;
    int table;     // boundary_layer_profile: its table of per-ghost states (DevView::gfix)
    double fs[7];  // T, p, rho, energy, vx, vy, vz
    double value;  // fix_temperature temperature / subsonic_outflow pressure
};

// The ghost-cell and flux actions of one boundary tag.
struct BoundDev {
    int n_pre, n_visc;
    Action pre[kMaxActions];   // pre_reconstruction
    Action visc[kMaxActions];  // pre_viscous_grad
    int cflux;                 // post_convective_flux: a constant_flux action (the last one wins)
    double cfs[7];             // its flow state: T, p, rho, energy, vx, vy, vz
};

// Gas, transport and finite-volume settings (FiniteVolume ctor, finite_volume.cpp:13-54).
struct FvParams {
    int dim;
    int flux;     // FluxKind
    int thermo;   // ThermoKind
    int order;    // reconstruction order 1 or 2
    int limiter;  // 1: Barth-Jespersen, 0: unlimited
    int viscous;
    int cflux;             // some boundary has a constant_flux action
    double eps;            // Barth-Jespersen epsilon
    double delta;          // LDFSS2 delta
    double signal_factor;  // viscous dt signal factor
    double R, Cv, Cp, gamma;
    double mu0, T0, Ts, Pr;
    // float copies for the float kernels (rounded on the host, so that the
    // device does no double->float conversions) and host-side reciprocals
    float fR, fCv, fCp, fgamma, fgR, feps, fdelta, fmu0, fT0, fTs, fPr, finv_Cv;
    // what the float copies leave out (the double minus its float copy, rounded to
    // float): float-float kernels take each constant as the pair (f*, lo*)
    float loR, loCv, loCp, logamma, logR, lodelta, lomu0, loT0, loTs, loPr, loinv_Cv;
    double inv_Cv;
};

// Device-side control block of the explicit Runge-Kutta step
// (RungeKutta::estimate_dt / take_step, runge_kutta.cpp:108-203).
struct StepCtl {
    double t, dt, stable_dt, time_since_last_plot;
    double cfl, max_time, plot_frequency;
    int n_cfl;  // linear CFL schedule points (0: constant cfl)
    double cfl_t[16], cfl_v[16];
    int stages;
    double a[kMaxStages][kMaxStages];  // tableau a(i, j), row i = stage i (>= 1)
    unsigned a_used[kMaxStages];       // bit j of row i: a(i, j) >= 1e-14 (the terms the stages add)
    double b[kMaxStages];
    double ca[kMaxStages][kMaxStages];  // a(i, j) * dt of the current step
    double cb[kMaxStages];              // b(i) * dt
    unsigned long long dt_bits;         // min over cells of the local dt (bits of a positive double)
    unsigned long long bad_cells;       // bad cells left by the last solution update
    long long steps;
    int halt;  // set when a step left bad cells or t >= max_time (Solver::solve, solver.cpp:38-49)
};

// Raw device pointers of one context for one arithmetic (P = primitive
// storage type, Gm = geometry type, both double or float; see layouts below).
struct DevView {
    int dim, N, G, F, MF, NT;
    // connectivity, slot-major: slot k of cell c at [k * N + c]
    const int* cell_face;
    const int* cell_nbr;
    const signed char* outsign;
    const int* nfaces;
    const int* left;
    const int* right;
    // ghosts (index g = ghost id - N)
    const int* ghost_src;
    const int* ghost_face;
    const int* ghost_bound;
    const BoundDev* bounds;
    const double* gfix;  // [tables][5][G]: T, p, rho, e, vx of each boundary-layer profile's ghosts
    // ghosts fed by each valid cell (CSR over valid cells)
    const int* feed_off;
    const int* feed_ghost;
    // geometry (type Gm): cc[3][NT], r[6][N], face[13][F] = n, t1, t2, centre, area
    const void* cc;
    const void* r;
    const void* face;
    const double* vol;      // N
    const double* inv_vol;  // N, 1/volume (fast paths)
    const float2* inv_vol2; // N, 1/volume as a float pair (hi, lo) (mixed build)
    const void* lsqw;       // [3][MF][N] least-squares weights per neighbour slot (type Gm, fast paths)
    const void* lsqd;       // [3][MF][N] face centre minus cell centroid per face slot (float build), or null
    int lsq_shared;         // 1: lsqw, lsqd and their lo parts are [3][MF], the same for every cell
    // float build on a uniform lattice, else null: each face's class and the
    // classes' rows (n; 2-D t1 x, t1 y, t2 z; left and right offsets face centre - centroid; area)
    const unsigned char* face_class;  // [F]
    const float* face_class_tab;      // [classes][kFaceClassRow]
    // flow-state tangent only, else null: a tangent direction of each boundary's
    // flow state (T, p, rho, energy, vx, vy, vz), seeded by the dual ghost fill and
    // the dual constant-flux faces
    const double* fs_tan;  // [bounds][7]
    // state (type P)
    void* prim;    // [7][NT]: rho, p, T, e, vx, vy, vz
    void* vghost;  // [5][G]: p, T, vx, vy, vz after the pre-viscous-gradient actions
    void* grad;    // [5*3][N]: gradients of the 5 reconstructed variables
    void* phi;     // [5][N]: their limiter values
    void* vgrad;   // [4*3][N]: gradients of T, vx, vy, vz for the viscous flux
    void* flux;    // [nc][F]
    // float-float build (MIXED_FF) only, else null: what the float arrays above
    // leave out of each double value (value - float copy, rounded to float), so
    // that prim + prim_lo etc. hold the value to about 48 bits
    float* prim_lo;        // [7][NT]
    const float* cc_lo;    // [3][NT]
    const float* face_lo;  // [13][F]
    float* flux_lo;        // [nc][F]
    const float* lsqw_lo;  // [3][MF][N]
    const float* lsqd_lo;  // [3][MF][N]
    float* grad_lo;        // [N][16]: lo parts of the packed limiter-scaled gradients
    float* vgrad_lo;       // [4*3][N]: lo parts of the viscous gradients
    float* vghost_lo;      // [5][G]: lo parts of the pre-viscous ghost values
    double* vsig;  // [F]: viscous time-step signal (gamma/rho)(mu/Pr) per face
    double* U;     // [nc][N]
    double* k;     // [stages][nc][N]
    int k_alias;   // 1: every stage derivative in slot 0 (the reference's aliased stages)
    StepCtl* ctl;            // one control block per case
    const int* case_of;      // case of each valid cell (batched ensembles), or null for one case
    int n_cases;
    unsigned* branches;  // optional [N][5] limiter branch codes
};

// Launch entry points of one kernel build (one arithmetic).
// Launch variants of the stage kernels (recon, face, update) for the
// autotuner: threads per block and minimum resident blocks per SM (which caps
// the registers per thread at 65536 / (threads x blocks)).  The FP64_EXACT
// build always uses variant 0.
constexpr int kNumVariants = 5;
constexpr int kVariantThreads[kNumVariants] = {256, 256, 256, 256, 512};
constexpr int kVariantMinBlocks[kNumVariants] = {1, 3, 4, 5, 2};

struct KernelOps {
    // ghosts from their source cells (pre-reconstruction and pre-viscous actions)
    void (*ghost_fill)(const DevView&, const FvParams&, cudaStream_t);
    // gradients + limiters (+ viscous gradients) of every valid cell
    void (*recon)(const DevView&, const FvParams&, bool reconstruct, int variant, cudaStream_t);
    // face fluxes (convective + viscous)
    void (*face_flux)(const DevView&, const FvParams&, bool reconstruct, int variant, cudaStream_t);
    // surface integral into stage `stage`; mode: 0 residual only (writes k[stage]),
    // 1 stage 0 of a step whose dt is not known yet, 2 a stage followed by another
    // (+ next stage state), 3 last stage (+ solution update). with_dt: also min-reduce
    // the local time step of the new state into the control blocks (mode 3 only).
    // out_rowmajor: optional N x nc output of dU/dt.
    void (*update)(const DevView&, const FvParams&, int mode, int stage, double* out_rowmajor,
                   int with_dt, int variant, cudaStream_t);
    // stage-1 state U + a(1,0) dt k0 -> primitives and ghosts (after dt is known)
    void (*combine)(const DevView&, const FvParams&, int stage, cudaStream_t);
    // primitives (and ghosts) from U
    void (*prims_from_U)(const DevView&, const FvParams&, cudaStream_t);
    // local CFL dt of every valid cell reduced into ctl->dt_bits (face signal of the last flux)
    void (*local_dt)(const DevView&, const FvParams&, cudaStream_t);
    // U += sum_j b(j) dt k_j, primitives and ghosts (single-stage tableaus)
    void (*finalize)(const DevView&, const FvParams&, cudaStream_t);
    // mixed build only (else null): face_flux + update of an inviscid Runge-Kutta
    // stage (mode 2 or 3) in one kernel that recomputes each cell's face fluxes;
    // the new primitives go to prim_out (not the buffer the view reads)
    void (*cell_update)(const DevView&, const FvParams&, bool reconstruct, int mode, int stage, int with_dt,
                        int variant, void* prim_out, cudaStream_t);
    // U from N x nc device rows (rows[map[i]] for cell i when map is not null), the
    // primitives and ghosts from it, and (with_dt) the local time step of the new
    // state min-reduced into the control blocks: the layout pass, prims_from_U and
    // local_dt in one kernel
    void (*load_state)(const DevView&, const FvParams&, const double* rows, const int32_t* map, int with_dt,
                       cudaStream_t);
};

KernelOps kernels_f64();
KernelOps kernels_f64_exact();
KernelOps kernels_mixed();
KernelOps kernels_mixed_grad();
KernelOps kernels_mixed_ff();

// precision-independent kernels (kernels_common.cu)
// Fused Runge-Kutta stage on structured blocks (mixed build, inviscid, second
// order): reads the primitives of v.prim, writes the new state's into
// sb.prim_out; mode / stage / with_dt as KernelOps::update.
void launch_fused_stage(const DevView& v, const SbView& sb, const FvParams& prm, int mode, int stage, int with_dt,
                        cudaStream_t s);
cudaError_t prepare_fused_stage();              // shared-memory opt-in, once per device
void fused_tile_shape(int dim, int* tx, int* ty, int* tz);
// Plane-marching fused stage for one 3-D structured block (kernels_march.cuh):
// the same stage as launch_fused_stage, with the block's planes staged into
// shared memory by TMA; hb is the host copy of sb.blocks[0], kc the planes per CTA.
struct alignas(128) TmaMap {
    unsigned char bytes[128];  // a CUtensorMap
};
void launch_march_stage(const DevView& v, const SbView& sb, const SBlock& hb, const FvParams& prm,
                        const TmaMap& prim, const TmaMap& cc, int mode, int stage, int with_dt, int kc,
                        cudaStream_t s);
cudaError_t prepare_march_stage();  // shared-memory opt-in, once per device
// The tensor map of nvar float arrays of one block (base: its first cell;
// var_stride: elements between variables) in the layout the stage copies.
// Returns 0, or -1 with *why set.
int march_encode_map(TmaMap* out, const float* base, int ni, int nj, int nk, int nvar, long long var_stride,
                     std::string* why);
constexpr int kMarchTileX = 32, kMarchTileY = 8;
// The mixed build's integer-pipe float -> double conversion against the
// conversion instruction on n pseudo-random bit patterns; mismatches counted.
int check_float_conversions(long long n, unsigned long long seed, unsigned long long* mismatches);

// Scratch of the adjoint passes (device pointers; sizes in launch_adjoint's callers).
struct AdjScratch {
    double* qf;               // [2][6][F] adjoints of the faces' reconstructed inputs
    double* self;             // [7][N]    each cell's own primitive adjoint
    double* nba;              // [7][MF][N] primitive adjoints each cell sends to the neighbour of slot s
    double* ga;               // [7][G]    ghost primitive adjoints
    const signed char* back;  // [MF][N]   slot of cell_nbr(i, s) that points back to i
    double* qv;               // [2][5][F] viscous: adjoints of the sides' p, T, v (valid sides)
    double* qg;               // [2][12][F] viscous: adjoints of the sides' viscous gradients
    double* gav;              // [5][G]    viscous: adjoints of the ghosts' pre-viscous p, T, v
    // geometry adjoint (ibisgb_vjp_geometry; null for the state-only product)
    double* geo_face = nullptr;  // [13][F]   out: n, t1, t2, face centre, area
    double* geo_cell = nullptr;  // [4][N+G]  out: centroid, volume (ghost rows: centroid only)
    double* geo_fcb = nullptr;   // [2][3][F] face-centre adjoint from each side's cell
    double* geo_vb = nullptr;    // [2][F]    volume adjoint of each side's cell from the face
    double* geo_nbc = nullptr;   // [3][MF][N] centroid adjoint each cell sends to the neighbour of slot s
    double* geo_ceb = nullptr;   // [3][F]    viscous: adjoint of an interior face's centroid offset x_r - x_l
    // boundary flow-state adjoint (ibisgb_vjp_flow_state; null otherwise)
    double* fs_ghost = nullptr;  // [G][7]    out, added to: each ghost's share of w^T dR/d(its boundary's flow
                                 //           state: T, p, rho, energy, vx, vy, vz)
};
// out = (dR/dU)^T w for w, out of N x nc rows; ghost_out (optional, G x 7 rows):
// the adjoint of every ghost cell's primitives (rho, p, T, e, v).
void launch_adjoint(const DevView& v, const FvParams& p, const double* w, bool reconstruct, const AdjScratch& a,
                    double* out, double* ghost_out, cudaStream_t s);
// The adjoint of the residual with respect to the grid geometry, w^T dR/dgeom, into
// a.geo_face / a.geo_cell (residuals without constant-flux boundaries; the
// least-squares factors are differentiated through the centroids).
void launch_adjoint_geometry(const DevView& v, const FvParams& p, const double* w, bool reconstruct,
                             const AdjScratch& a, cudaStream_t s);
// out[b * 7 + k] = sum over the ghosts g of boundary b of rows[g * 7 + k] (nb
// boundaries, G ghosts, ghost_bound per ghost), in a fixed order.
void launch_sum_ghost_rows(const double* rows, const int* ghost_bound, int G, int nb, double* out, cudaStream_t s);
// The geometry tangent: out = dR/dgeometry . (dface [13][F], dcell [4][N+G]) at the
// current state, on dual copies of the geometry (each element 2 doubles).
struct GeoTangent {
    void* face;  // [13][F]
    void* cc;    // [3][N+G]
    void* vol;   // [N]
    void* r;     // [6][N] least-squares factors
};
void launch_tangent_geometry(const DevView& v, const FvParams& p, const double* dface, const double* dcell,
                             bool reconstruct, const GeoTangent& g, double* out, cudaStream_t s);

void launch_dt_finalize(StepCtl* ctl, int n_cases, cudaStream_t s);
void launch_reset_dt(StepCtl* ctl, int n_cases, cudaStream_t s);
void launch_l2_norms(const double* k0, int N, int nc, double* out6, cudaStream_t s);
// Krylov vector kernels (kernels_common.cu); results stay in device memory
void launch_dot(const double* a, const double* b, long long n, double* partial, double* out,
                bool take_sqrt, cudaStream_t s);
void launch_axpy_neg(double* y, const double* x, long long n, const double* c, cudaStream_t s);
void launch_scale_inv(double* out, const double* in, long long n, const double* d, cudaStream_t s);
void launch_sub(double* out, const double* a, const double* b, long long n, cudaStream_t s);
void launch_gemv_add(double* x, const double* V, long long n, int m, const double* y, cudaStream_t s);
void launch_add_rows(double* U, const double* dU, int N, int nc, cudaStream_t s);
void launch_axpby(double* y, const double* x, long long n, double a, double b, cudaStream_t s);  // y = a x + b y
int dot_scratch_doubles();

// tangent of the residual: out = inv_dt * v - dR/dU v (kernels_tangent.cu); v, out: N x nc rows
void launch_tangent(const DevView& v, const FvParams& p, const double* vt, double inv_dt,
                    bool reconstruct, double* out, cudaStream_t s);

// message returned by ibisgb_last_error(NULL) on this thread
void set_thread_error(const std::string& msg);

// row-major (N x nc) <-> slot-major ([nc][N]) conserved state
struct RowScale { double s[5]; };
void launch_scale_rows(double* out, const double* in, long long n, int nc, const RowScale& sc, cudaStream_t s);
void launch_gather_rows(double* dst, const double* src, const int32_t* map, int N, int w, cudaStream_t s);
void launch_rows_to_soa(const double* rows, double* soa, int N, int nc, cudaStream_t s);
void launch_soa_to_rows(const double* soa, double* rows, int N, int nc, cudaStream_t s);

}  // namespace ibisgb
