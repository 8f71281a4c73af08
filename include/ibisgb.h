/*
 * ibisgb — GB300-native residual engine for ibis's compressible finite-volume path.
 *
 * C ABI of libibisgb.so.  Plain pointers and sizes only; no C++ exceptions cross
 * this boundary.  Every function returns 0 on success or a negative IBISGB_ERR_*
 * code, with a message from ibisgb_last_error().
 *
 * A context owns one grid, its device memory and one CUDA stream.  It is not
 * thread-safe: use one context per host thread.  Host pointers passed in are
 * owned by the caller and copied before the call returns; *_device entry points
 * take device pointers and run on the context's stream, ordered after the work
 * already queued on the caller's `stream` and before what the caller queues
 * on it next.  NULL means no ordering (the context stream alone); pass
 * cudaStreamLegacy, not NULL, for the legacy default stream.
 *
 * Array conventions follow ibis: cells and faces are in the reference's
 * numbering (cells in SU2 file order; faces numbered by first appearance while
 * scanning cells, src/grid/grid/grid.h:113-133; ghost cells N.. in boundary-tag
 * order, grid.h:406-443).  Conserved quantities are row-major (cell, component)
 * with components (mass, momentum_x, momentum_y[, momentum_z], energy), like
 * ConservedQuantities' View<T**>(n, dim+2) (conserved_quantities.cpp:15-23).
 */
#ifndef IBISGB_H
#define IBISGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IBISGB_OK 0
#define IBISGB_ERR_CONFIG (-1)    /* bad or unsupported config.json content */
#define IBISGB_ERR_GRID (-2)      /* unreadable or inconsistent grid */
#define IBISGB_ERR_CUDA (-3)      /* CUDA runtime failure (no device, OOM, launch error) */
#define IBISGB_ERR_BAD_CELLS (-4) /* T < 0, rho < 0 or non-finite rho after a step */
#define IBISGB_ERR_ARG (-5)       /* null or inconsistent argument */
#define IBISGB_ERR_TIMEOUT (-6)   /* a bounded device wait ran out */
#define IBISGB_ERR_STATE (-7)     /* call out of order (e.g. no initial condition yet) */

/* Arithmetic of the residual.  F64: everything in double (fused multiply-add
 * allowed).  MIXED: reconstruction, gradients, limiters and fluxes in float,
 * face fluxes accumulated into cell residuals, state update and
 * conserved->primitive inversion in double.  F64_EXACT: double with the
 * reference's operation order and no fused multiply-add, for bitwise parity. */
#define IBISGB_F64 0
#define IBISGB_MIXED 1
#define IBISGB_F64_EXACT 2
/* MIXED_GRAD: least-squares gradients and Barth-Jespersen limiters in float, on
 * neighbour values and face offsets taken relative to the cell's own value and
 * centroid in double (float rounds only these increments); face states,
 * fluxes, accumulation, update and inversion in double.  For long runs through
 * shock transients, where the float states and fluxes of MIXED drift beyond
 * 1e-6 of the FP64 solution. */
#define IBISGB_MIXED_GRAD 3
/* MIXED_FF: the float arrays of MIXED plus, for every state, geometry and flux
 * value, the float remainder that the float copy leaves out (value = hi + lo,
 * about 48 bits).  Gradients and limiters in float on cell-relative values;
 * face states, thermo closure, flux calculators and the local time step in
 * float-float arithmetic on the FP32 pipe (an FP64-like result without GB300's
 * narrow FP64 pipe); ghost actions with the normals as hi + lo; fluxes summed
 * as float pairs; update and inversion in double.  For long runs through shock
 * transients at MIXED-like speed. */
#define IBISGB_MIXED_FF 4

typedef struct ibisgb_ctx ibisgb_ctx;

typedef struct {
    int64_t num_cells;       /* valid cells N */
    int64_t num_ghost_cells; /* ghost cells G (ids N..N+G-1) */
    int64_t num_faces;       /* faces F */
    int32_t dim;             /* 2 or 3 */
    int32_t max_faces_per_cell;
    int32_t n_conserved;     /* dim + 2 */
    int32_t num_boundaries;  /* boundary tags in config.json */
} ibisgb_sizes;

typedef struct {
    double t;          /* simulated time after the last step */
    double dt;         /* last time step */
    double stable_dt;  /* last CFL-stable estimate (FiniteVolume::estimate_dt) */
    int64_t steps;     /* steps taken by this context */
    int64_t bad_cells; /* bad cells after the last step */
    double device_ms;  /* device time of the steps of this call (CUDA events on the context stream) */
} ibisgb_rk_status;

/* Build a context from a config.json document and an SU2 grid file.
 * Replaces GridBlock<T>(file, config) (src/grid/grid/grid.h:40-42, 89-167),
 * FiniteVolume<T>(grid, config) (src/finite_volume/finite_volume/finite_volume.cpp:13-54),
 * IdealGas(json)/TransportProperties(json) (src/gas/gas/gas_model.h:58-62,
 * transport_properties.h:91-109) and RungeKutta's tableau/CFL set-up
 * (src/solvers/solvers/runge_kutta.cpp:21-80). */
int ibisgb_create(const char* config_json, const char* su2_path, ibisgb_ctx** out);

/* Same, from grid arrays instead of an SU2 file: VTK element codes (3 line,
 * 5 tri, 9 quad, 10 tet, 12 hex, 13 wedge, 14 pyramid), CSR connectivity;
 * markers named by newline-separated marker_names, marker m owning elements
 * marker_offsets[m]..marker_offsets[m+1]-1.  Equivalent to GridIO's SU2 reader
 * output (src/grid/grid/grid_io.cpp:218-268). */
int ibisgb_create_from_arrays(const char* config_json, int32_t dim, int64_t num_vertices,
                              const double* xyz, int64_t num_cells, const int32_t* cell_types,
                              const int64_t* cell_offsets, const int64_t* cell_vertices,
                              int32_t num_markers, const char* marker_names,
                              const int64_t* marker_offsets, const int32_t* element_types,
                              const int64_t* element_offsets, const int64_t* element_vertices,
                              ibisgb_ctx** out);

void ibisgb_destroy(ibisgb_ctx* ctx);

/* Message of the last error on ctx (or of the last failed create when ctx is NULL). */
const char* ibisgb_last_error(const ibisgb_ctx* ctx);

int ibisgb_get_sizes(const ibisgb_ctx* ctx, ibisgb_sizes* out);

/* Initial condition on the valid cells (T, p, vx, vy[, vz]; vz may be NULL in 2-D);
 * rho and internal energy follow from update_thermo_from_pT.  Replaces
 * NativeBinaryInput::read (src/io/io/native.cpp:263-339) + primatives_to_conserved
 * (src/finite_volume/finite_volume/primative_conserved_conversion.cpp:31-51). */
int ibisgb_set_primitives(ibisgb_ctx* ctx, const double* T, const double* p, const double* vx,
                          const double* vy, const double* vz);

/* Primitives of the valid cells in the current state (any pointer may be NULL).
 * Replaces the FlowStates read-back of FVIO::write (src/io/io/io.cpp:106-129). */
int ibisgb_get_primitives(ibisgb_ctx* ctx, double* rho, double* p, double* T, double* e,
                          double* vx, double* vy, double* vz);

/* Conserved state of the valid cells, N x n_conserved row-major.  Pinned host
 * memory (mapped into the device's address space, as cudaHostAlloc memory is
 * under unified addressing) is written in place by the layout kernel; other
 * memory receives a copy of a device staging buffer. */
int ibisgb_get_conserved(ibisgb_ctx* ctx, double* U);

/* Replace the conserved state of the valid cells (N x n_conserved row-major,
 * host memory; pinned memory is read in place by the layout kernel, other memory
 * is copied through a device staging buffer; U may be reused once the call
 * returns from pinned memory); primitives and ghost cells follow
 * from conserved_to_primatives (primative_conserved_conversion.cpp:4-23).  The
 * state write of Jfnk::apply_update_ (src/solvers/solvers/jfnk.cpp:63-93) and
 * of a restart. */
int ibisgb_set_conserved(ibisgb_ctx* ctx, const double* U);

/* As ibisgb_set_conserved from device memory (N x n_conserved rows), ordered
 * after the work on `stream` (NULL: the context stream). */
int ibisgb_set_conserved_device(ibisgb_ctx* ctx, const double* U_device, void* stream);

/* The context's CUDA stream (a cudaStream_t), for callers that record events
 * or order their own work against the context. */
int ibisgb_get_stream(ibisgb_ctx* ctx, void** stream);

/* Mean device time in milliseconds, over `reps` launches timed with CUDA
 * events on the context stream, of the kernels of one residual evaluation:
 * out[0] gradients + limiters, out[1] face fluxes, out[2] surface integral,
 * out[3] the whole evaluation.  A profiling aid with no counterpart in ibis,
 * which only labels its Kokkos kernels. */
int ibisgb_kernel_times(ibisgb_ctx* ctx, int32_t precision, int32_t reps, double out[4]);

/* dU/dt of the valid cells (N x n_conserved row-major) at the current state,
 * including the pre-reconstruction / pre-viscous boundary actions and the
 * post-convective constant_flux action.  Replaces
 * FiniteVolume<T>::compute_dudt (src/finite_volume/finite_volume/finite_volume.cpp:56-96). */
int ibisgb_residual(ibisgb_ctx* ctx, int32_t precision, double* dudt);

/* As ibisgb_residual with a device output pointer, on `stream` (a cudaStream_t,
 * NULL for the context's stream).  For callers that keep data in HBM (torch). */
int ibisgb_residual_device(ibisgb_ctx* ctx, int32_t precision, double* dudt_device, void* stream);

/* CFL-stable time step of the current state.  Replaces FiniteVolume<T>::estimate_dt
 * (finite_volume.cpp:130-184); in viscous runs the face states of the last
 * residual evaluation are used, as in the reference. */
int ibisgb_estimate_dt(ibisgb_ctx* ctx, double* dt);

/* Bad cells (T<0, rho<0, NaN/Inf rho) in the current state.  Replaces
 * FiniteVolume<T>::count_bad_cells (finite_volume.cpp:257-270). */
int ibisgb_count_bad_cells(ibisgb_ctx* ctx, int64_t* n);

/* n_steps explicit Runge-Kutta steps on the device (CUDA graph per step),
 * dt = min(cfl(t) * stable_dt, 1.5 * dt_prev, max_time - t[, plot clip]).
 * Replaces RungeKutta::take_step (src/solvers/solvers/runge_kutta.cpp:131-203)
 * inside Solver::solve's loop (src/solvers/solvers/solver.cpp:25-59); returns
 * IBISGB_ERR_BAD_CELLS after the first step that leaves bad cells. */
int ibisgb_rk_run(ibisgb_ctx* ctx, int32_t precision, int64_t n_steps, ibisgb_rk_status* status);

/* n_jobs Runge-Kutta runs between host buffers: job j replaces the state by the
 * rows U_in[j] (N x n_conserved, reference cell order), takes steps_per_job steps
 * and writes the new state to U_out[j] -- the same results as
 * ibisgb_set_conserved + ibisgb_rk_run + ibisgb_get_conserved per job, with job
 * j+1's upload and job j-1's read-back on copy streams while job j's steps run.
 * Pinned host buffers (cudaHostAlloc, torch pin_memory) make the copies overlap;
 * the buffers of a job may be reused once the call returns.  The status is the
 * last job's (IBISGB_ERR_BAD_CELLS when it left bad cells).  A driver that
 * advances a stream of states (ensembles kept on the host, sampling, surrogate
 * training) calls this instead of the three calls per state. */
int ibisgb_rk_run_host(ibisgb_ctx* ctx, int32_t precision, int64_t n_jobs, int64_t steps_per_job,
                       const double* const* U_in, double* const* U_out, ibisgb_rk_status* status);

/* L2 norms of the first-stage residual of the last step: global, mass,
 * momentum_x, momentum_y, momentum_z, energy.  Replaces
 * ConservedQuantities<T>::L2_norms (conserved_quantities.cpp:40-69) on k_[0]
 * (runge_kutta.cpp:264). */
int ibisgb_l2_norms(ibisgb_ctx* ctx, double out[6]);

/* Internal arrays in reference numbering, for parity checks.
 * which: 0 face left cell (int64 F), 1 face right cell (int64 F),
 * 2 cell faces (int64 N x max_faces, -1 padded), 3 outsigns (int32 N x max_faces),
 * 4 cell neighbours (int64 N x max_faces), 5 ghost source cell (int64 G),
 * 6 face geometry (double 13 x F: n, t1, t2, centre, area),
 * 7 cell geometry (double 4 x (N+G): centroid, volume),
 * 8 limiter branch codes of the last residual (uint32 N x 5),
 * 9 limiter values of the last residual (double 5 x N),
 * 10 face fluxes of the last residual (double F x n_conserved),
 * 11 boundary face of each ghost cell (int64 G), 12 boundary (index in sorted
 * tag order) of each ghost cell (int64 G), 13 face fluxes of the last MIXED
 * residual evaluation (double F x n_conserved, from the float fluxes),
 * 14 the reference id of each internal cell (int64 N), 15 the reference id of
 * each internal face (int64 F), 16 the vertices of each face (int64 F x 4, -1
 * padded; the grid's vertex ids). */
int ibisgb_get_dump(ibisgb_ctx* ctx, int32_t which, void* buf, int64_t bytes);

/* Replaces the grid geometry: face (13 x F: normal, tangents t1 and t2, centre,
 * area) and cell (4 x (N+G): centroid, volume; ghost volumes ignored), host
 * arrays in the layouts of dumps 6 and 7, reference numbering.  The
 * least-squares factors are formed again from the centroids; connectivity,
 * boundary actions and the boundary-layer profile's ghost states are kept, and
 * the structured-block stages (which hold their own lattice geometry) are
 * switched off.  With ibisgb_vjp_geometry / ibisgb_jvp_geometry this makes the
 * residual a differentiable function of the geometry arrays.  No counterpart in
 * the reference (its GridBlock is built once from the SU2 file). */
int ibisgb_set_geometry(ibisgb_ctx* ctx, const double* face, const double* cell);

/* A check for the tangent and adjoint calls (ibisgb_jvp*, ibisgb_vjp*,
 * ibisgb_adjoint_step's products) and the residual (ibisgb_residual*): with
 * on != 0, every device buffer those kernels use as scratch (dual primitives,
 * gradients, limiters and fluxes, the adjoint's per-face and per-slot partials,
 * the geometry and flow-state scratch; the residual's gradients, limiters, face
 * fluxes and viscous time-step signal) is filled with NaN before each call, so
 * that a read of an entry the call did not write shows in its result.  Results
 * are the same bits with it on or off; it costs one memset per buffer per call.
 * The limiter dump of a 2-D grid then shows NaN in its unused fifth row.  No
 * counterpart in the reference. */
int ibisgb_set_scratch_poison(ibisgb_ctx* ctx, int32_t on);

/* The geometry-table layout of arithmetic `precision` on this grid.  On a
 * uniform lattice -- the benchmark's periodic box -- and with the config's
 * grid.geometry_tables "auto" (the default; "per_element" keeps every table per
 * cell and per face):
 *  - *lsq_shared = 1 when the least-squares weights and the limiter's face
 *    offsets are stored once per face slot, every cell's being bitwise the same
 *    in that arithmetic's storage type; the reconstruction then reads one row per
 *    slot that every thread shares instead of 24 values per cell;
 *  - *face_classes = the number of face classes (MIXED only, else 0): faces whose
 *    normal, 2-D tangents and side offsets (face centre - centroid, as the float
 *    face kernel forms them) and area are bitwise the same share a row, and each
 *    face keeps a one-byte class instead of its normal, centre and area and the
 *    gathers of its cells' centroids (the face kernel and the local time step
 *    read the class's row); 0 when there are more than 64 distinct rows.
 * The values, and so the results, are the same as with the per-element tables.
 * Uploads the geometry of that arithmetic if it is not on the device yet.  Either
 * pointer may be NULL.  No counterpart in the reference (WLSGradient and the
 * interfaces keep per-cell and per-face geometry, gradient.h:89-162,
 * interface.h:180-251). */
int ibisgb_shared_tables(ibisgb_ctx* ctx, int32_t precision, int32_t* lsq_shared, int32_t* face_classes);

/* Replaces the flow state (7 doubles: T, p, rho, energy, vx, vy, vz -- the
 * "flow_state" object of the config) of boundary `tag`: every action of it that
 * carries one takes fs, as if the config had given it (FlowStateCopy and
 * SubsonicInflow, src/finite_volume/finite_volume/boundaries/boundary.cpp:10-12,
 * 280-282, in the pre-reconstruction and pre-viscous-gradient lists; the
 * constant_flux flux action, boundary.cpp:404-444).  rho and energy are inputs
 * as in the config (the reference takes them as given); keep them consistent
 * with the gas model (rho = p / (R T), energy = Cv T) for a physical state.
 * IBISGB_ERR_ARG for an unknown tag, a boundary with no flow state or a
 * non-finite entry; IBISGB_ERR_STATE on a batch (its cases' states are fixed
 * when it is made).  No counterpart in the reference (its boundary conditions
 * are built once from the config). */
int ibisgb_set_flow_state(ibisgb_ctx* ctx, const char* tag, const double* fs);

/* The flow state of boundary `tag` (7 doubles, as ibisgb_set_flow_state). */
int ibisgb_get_flow_state(ibisgb_ctx* ctx, const char* tag, double* fs);

/* out = w^T dR/d(flow state): for w (N x n_conserved rows), the adjoint of the
 * residual with respect to each boundary's flow state (num_boundaries x 7, the
 * boundaries in sorted tag order, the entries as ibisgb_set_flow_state; zero
 * rows for boundaries without one).  Every action of a boundary that carries a
 * flow state moves together, ibisgb_set_flow_state's semantics; through the
 * ghost cells (each ghost's actions differentiated with the flow state seeded,
 * the viscous ghost values included) and the constant-flux faces.  out_device
 * is device memory, on `stream` (NULL: the context stream).  The transposed
 * derivative the steady adjoint needs for inflow parameters: with lambda from
 * ibisgb_adjoint_step, dObjective/dfs = dObjective/dfs|_U + lambda . dR/dfs.
 * No counterpart in the reference. */
int ibisgb_vjp_flow_state_device(ibisgb_ctx* ctx, const double* w_device, double* out_device,
                                 int32_t allow_reconstruction, void* stream);

/* As ibisgb_vjp_flow_state_device with host vectors. */
int ibisgb_vjp_flow_state(ibisgb_ctx* ctx, const double* w, double* out, int32_t allow_reconstruction);

/* out = dR/dfs . dfs: the tangent of the residual (N x n_conserved rows) along a
 * direction dfs of every boundary's flow state (num_boundaries x 7, the layout of
 * ibisgb_vjp_flow_state's output; rows of boundaries without a flow state are not
 * read).  The dual ghost fill and the dual constant-flux faces carry the direction
 * (every action of a boundary that carries a flow state moves together), on a
 * state of zero tangent; ibisgb_vjp_flow_state is its transpose.  dfs_device and
 * out_device are device memory, on `stream` (NULL: the context stream).  No
 * counterpart in the reference. */
int ibisgb_jvp_flow_state_device(ibisgb_ctx* ctx, const double* dfs_device, double* out_device,
                                 int32_t allow_reconstruction, void* stream);

/* As ibisgb_jvp_flow_state_device with host vectors. */
int ibisgb_jvp_flow_state(ibisgb_ctx* ctx, const double* dfs, double* out, int32_t allow_reconstruction);

/* The device arrays' cell and face order.  The grid's optional "renumber" key
 * ("auto" when absent, "rcm", "none"; not a reference key) selects it: "rcm"
 * orders the valid cells by reverse Cuthill-McKee over the interior-face graph
 * and the faces by their lower, then higher, cell; "auto" does so for grids with
 * cells other than quadrilaterals (2-D) or hexahedra (3-D) when that at least
 * halves the cell graph's bandwidth (max |left - right| over interior faces).
 * Every array and id that crosses this ABI stays in the reference's numbering
 * (grid.h:113-133); each cell's face slots and every summation keep their order,
 * so results do not depend on the numbering.  Ghost cells keep their ids. */
int ibisgb_numbering(const ibisgb_ctx* ctx, int32_t* renumbered, int64_t* bandwidth_reference,
                     int64_t* bandwidth_internal);

/* Result of one Newton step of the steady solver. */
typedef struct {
    double relative_residual; /* global L2 norm of the residual / its initial value */
    double residual_norms[6]; /* global, mass, momentum_x, momentum_y, momentum_z, energy */
    int32_t gmres_iterations;
    int32_t gmres_converged;
    double gmres_residual;    /* |g_{k}| / beta of the last GMRES iteration */
    double dt_star;           /* pseudo time step cfl * stable dt */
    double cfl;
    int64_t step;             /* Newton steps taken since ibisgb_steady_initialise */
    double initial_norms[6];  /* the residual norms at ibisgb_steady_initialise */
} ibisgb_newton_status;

/* out = inv_dt_star * v - (dR/dU) v on device vectors of N x n_conserved rows
 * (index cell * n_conserved + component), at the current state, on `stream`
 * (NULL: the context stream).  Replaces the dual-number evaluation of
 * SteadyStateLinearisation::matrix_vector_product
 * (src/solvers/solvers/steady_state.cpp:52-128) with a hand-written tangent of
 * the residual kernels that follows ibis's Dual<T> rules (dual.h:11-346).
 * inv_dt_star = 1/dt* gives the reference's operator; 0 gives -J v.
 * allow_reconstruction = 0 is the first-order linearisation used as the
 * FGMRES preconditioner (steady_state.cpp:47-50). */
int ibisgb_jvp_device(ibisgb_ctx* ctx, const double* v_device, double* out_device, double inv_dt_star,
                      int32_t allow_reconstruction, void* stream);

/* As ibisgb_jvp_device with host vectors. */
int ibisgb_jvp(ibisgb_ctx* ctx, const double* v, double* out, double inv_dt_star,
               int32_t allow_reconstruction);

/* out = (dR/dU)^T w: the adjoint (vector-Jacobian product) of the residual
 * dU/dt at the current state, for device vectors of N x n_conserved rows, on
 * `stream` (NULL: the context stream).  No counterpart in the reference, which
 * has no adjoint; it is the exact transpose of the tangent of
 * ibisgb_jvp_device (the same Dual rules, every branch -- limiter face,
 * min/max neighbour, flux splitting -- recomputed from the current state), so
 * <w, J v> = <J^T w, v> to rounding.  ghost_out_device (may be NULL) receives
 * the adjoint of every ghost cell's primitives (G x 7 rows: rho, p, T, e, vx,
 * vy, vz), from which derivatives with respect to boundary states (an inflow
 * Mach number) follow.  allow_reconstruction = 0 gives the transpose of the
 * first-order linearisation.  Viscous fluxes are included. */
int ibisgb_vjp_device(ibisgb_ctx* ctx, const double* w_device, double* out_device, double* ghost_out_device,
                      int32_t allow_reconstruction, void* stream);

/* As ibisgb_vjp_device with host vectors (ghost_out: G x 7, may be NULL). */
int ibisgb_vjp(ibisgb_ctx* ctx, const double* w, double* out, double* ghost_out, int32_t allow_reconstruction);

/* The adjoint of the residual with respect to the grid geometry at the current
 * state: for w (N x n_conserved rows), w^T dR/dgeom into face_out (13 x F: the
 * face normal, tangents t1 and t2, centre and area, the layout of dump 6) and
 * cell_out (4 x (N+G): centroid and volume, the layout of dump 7; ghost rows hold
 * the ghost centroids' adjoint, ghost volumes are not inputs).  Covers what the
 * inviscid residual reads: the face frame in the flux rotation and in the
 * slip-wall ghost reflection (ghost_cells.cpp / boundary.cpp), areas and volumes
 * in the surface integral (finite_volume.cpp:220-255), face centres and centroids
 * in the reconstruction and the Barth-Jespersen limiter (limiter.cpp:23-63) and
 * the centroids (ghosts included) through the least-squares factors
 * (gradient.h:89-162), and in viscous residuals the normal and the centroid
 * offset of the face gradient (viscous_flux.cpp:36-80) and the viscous least
 * squares.  The boundary-layer profile is evaluated at the ghost centroid's real
 * height, as the reference's spline (cubic_spline.cpp, on doubles) does under its
 * dual type, so it carries no geometry derivative.  2-D grids
 * have no n_z, t1_z, t2_x, t2_y inputs (rows 0).  A constant-flux face's flux
 * depends on the geometry through its normal only.  No counterpart in the
 * reference. */
int ibisgb_vjp_geometry_device(ibisgb_ctx* ctx, const double* w_device, double* face_out_device,
                               double* cell_out_device, int32_t allow_reconstruction, void* stream);
int ibisgb_vjp_geometry(ibisgb_ctx* ctx, const double* w, double* face_out, double* cell_out,
                        int32_t allow_reconstruction);

/* The geometry tangent, the transpose of ibisgb_vjp_geometry: out (N x
 * n_conserved rows) = dR/dgeometry . (dface, dcell) at the current state, with
 * dface (13 x F) and dcell (4 x (N+G)) in the layouts of dumps 6 and 7 (ghost
 * volumes ignored).  The residual kernels run on dual copies of the geometry,
 * the least-squares factors formed again from the dual centroids -- the
 * reference's Dual<T> seeded in GridBlock<Dual>'s geometry. */
int ibisgb_jvp_geometry_device(ibisgb_ctx* ctx, const double* dface_device, const double* dcell_device,
                               double* out_device, int32_t allow_reconstruction, void* stream);
int ibisgb_jvp_geometry(ibisgb_ctx* ctx, const double* dface, const double* dcell, double* out,
                        int32_t allow_reconstruction);

/* Result of one pseudo-time step of the steady adjoint. */
typedef struct {
    double residual_norm;   /* |J^T lambda + g| before the step */
    int32_t gmres_iterations;
    int32_t gmres_converged;
    double gmres_residual;  /* |g_k| / beta of the last GMRES iteration */
    double dt_star;         /* cfl * stable dt of the current state */
    double scaled_residual_norm;  /* |S (J^T lambda + g)| before the step (S below) */
} ibisgb_adjoint_status;

/* One step of the discrete adjoint of the steady problem, J^T lambda = -g with
 * J = dR/dU at the current (converged) state and g = dObjective/dU (device
 * vectors, N x n_conserved rows): r = J^T lambda + g, then GMRES on
 * S (I/dt* - J^T) S^-1 y = S r and lambda += S^-1 y, in place (dt* = cfl * the
 * stable time step; GMRES length and tolerance from the config's steady solver,
 * or 50 and 1e-2).  S is diagonal per conserved variable: the RMS over the cells
 * of density and total energy, sqrt(RMS density * RMS energy) for the momenta --
 * the conserved variables differ by ~1e5 in magnitude, and unscaled GMRES
 * stagnates on that spread.  The transposed counterpart of ibisgb_newton_step; no
 * counterpart in the reference.  Iterate with a growing cfl until
 * scaled_residual_norm is small.
 * With lambda, dObjective/dp = dObjective/dp|_U + lambda . dR/dp for any
 * parameter p of the boundary states (through ibisgb_vjp's ghost adjoint) or of
 * the grid. */
int ibisgb_adjoint_step(ibisgb_ctx* ctx, const double* g_device, double* lambda_device, double cfl,
                        ibisgb_adjoint_status* status);

/* GMRES length of ibisgb_adjoint_step (1..1000; 0 restores the steady solver's
 * max_iters).  The adjoint is a linear solve, so a longer Krylov space than the
 * forward Newton steps' (whose length is the reference's, for parity) pays. */
int ibisgb_set_adjoint_krylov(ibisgb_ctx* ctx, int32_t max_iters);

/* Residual and initial norms of the steady solver at the current state
 * (Jfnk::initialise, src/solvers/solvers/jfnk.cpp:25-30).  `precision` is the
 * arithmetic of the real residual; the tangent is always double. */
int ibisgb_steady_initialise(ibisgb_ctx* ctx, int32_t precision);

/* The steady solver's residual norms at the current state and at
 * ibisgb_steady_initialise (global, mass, momentum x, y, z, energy; either may
 * be NULL): Jfnk::residual_norms and the initial norms behind
 * Jfnk::relative_residual_norms (jfnk.h). */
int ibisgb_steady_norms(ibisgb_ctx* ctx, double norms[6], double initial[6]);

/* One Jacobian-free Newton-Krylov step: dt* = cfl * estimate_dt, GMRES (or
 * FGMRES) on (I/dt* - J) dU = R(U) with the tangent operator, U += dU, new
 * residual norms.  Replaces Jfnk::step / apply_update_ (jfnk.cpp:39-93) with
 * Gmres::solve / FGmres::solve (src/linear_algebra/linear_algebra/gmres.cpp:119-303)
 * on device vectors. */
int ibisgb_newton_step(ibisgb_ctx* ctx, int32_t precision, ibisgb_newton_status* status);

/* Wait for all work on the context's stream. */
int ibisgb_synchronize(ibisgb_ctx* ctx);

/* Launch-configuration autotuner (no counterpart in the reference, whose
 * kernels take Kokkos's default launch shape).  The recon, face and update
 * kernels of the F64 and MIXED builds each come in ibisgb_launch_variants()
 * launch variants (threads per block x minimum resident blocks per SM, which
 * caps registers per thread).  ibisgb_autotune times every variant on the
 * context's grid and current state (CUDA events; the update kernel in its
 * first-stage Runge-Kutta mode, with the primitives it overwrites restored),
 * keeps the fastest and returns the choice in variants
 * (recon, face, update) and, if times_ms is not NULL, the time of every
 * variant (fastest of three launches; 3 x count doubles, kernel-major).  ibisgb_rk_run tunes a precision
 * by itself on its first call unless variants were set.  All variants give
 * bit-identical results.  The residual of the current state is left as the
 * first-stage derivative (what ibisgb_l2_norms reads).  F64_EXACT always uses
 * variant 0. */
int ibisgb_autotune(ibisgb_ctx* ctx, int32_t precision, int32_t variants[3], double* times_ms);

/* Fix the launch variants (recon, face, update) of a precision instead of tuning.
 * For MIXED the update's variant also applies to the per-cell flux kernel. */
int ibisgb_set_launch_variants(ibisgb_ctx* ctx, int32_t precision, const int32_t variants[3]);

/* The variant table: count, and per variant the threads per block and minimum
 * resident blocks per SM (arrays of at least count entries, may be NULL). */
int ibisgb_launch_variants(int32_t* count, int32_t* threads, int32_t* min_blocks);

/* Fused Runge-Kutta stage on structured blocks (no counterpart in the
 * reference).  When every case of the context is a structured block -- quads
 * or hexahedra numbered lexicographically on an ni x nj [x nk] lattice, the way
 * a structured grid is written as SU2 -- and the scheme is inviscid and second
 * order, the MIXED build can run each stage as one tiled kernel that keeps the
 * tile's state, gradients and fluxes in shared memory.  mode -1 (the default)
 * lets ibisgb_autotune / the first ibisgb_rk_run choose it when it is faster
 * than the three-kernel stage, 0 never uses it, 1 always does (IBISGB_ERR_ARG if
 * the grid or scheme does not qualify).  Its results agree with the
 * three-kernel MIXED path to rounding (faces are evaluated along the lattice
 * directions). */
int ibisgb_set_fused(ibisgb_ctx* ctx, int32_t mode);

/* Whether the fused stage applies to this context (host-side check, no GPU
 * needed) and is in use, the last tuning times (fused stage, best three-kernel
 * stage; ms, 2 doubles, may be NULL) and, when it does not apply, why (written
 * into reason, at most reason_len bytes with the terminating zero). */
int ibisgb_fused_info(ibisgb_ctx* ctx, int32_t* eligible, int32_t* enabled, double* times_ms, char* reason,
                      int32_t reason_len);

/* Kernel of the fused stage.  On one 3-D structured block whose first cell
 * index, i-extent and N+G are multiples of 4, the fused stage also has a
 * plane-marching kernel: each CTA owns a 32 x 8 column of cells and marches
 * along k, with every plane of primitives and centroids staged into shared
 * memory once by TMA tensor copies, gradients, limiters and fluxes kept on the
 * SM, and the double update as in the tile kernel.  kind -1 (the default) lets
 * ibisgb_autotune / the first ibisgb_rk_run time both kernels (and the
 * marching kernel at 16, 32 and 64 planes per CTA, or at planes_per_cta when
 * it is > 0) and keep the faster; 0 always takes the tile kernel; 1 always the
 * plane-marching kernel (IBISGB_ERR_ARG if it does not apply).  Applies when the
 * fused stage is in use (ibisgb_set_fused).  A scheduling choice with no
 * counterpart in ibis; the same formulas as the tile kernel. */
int ibisgb_set_fused_kind(ibisgb_ctx* ctx, int32_t kind, int32_t planes_per_cta);

/* Whether the plane-marching kernel applies (host-side check) and is the fused
 * stage's kernel, its planes per CTA, the last tuning times of one stage (ms:
 * tile kernel, plane-marching kernel; 2 doubles, may be NULL; 0 when not timed)
 * and, when it does not apply, why. */
int ibisgb_fused_kind(ibisgb_ctx* ctx, int32_t* march_eligible, int32_t* march_in_use, int32_t* planes_per_cta,
                      double* times_ms, char* reason, int32_t reason_len);

/* Per-cell flux path of the MIXED build (inviscid Runge-Kutta stages without
 * constant-flux boundaries; any grid).  Each stage runs the gradient kernel and
 * then one kernel in which every cell recomputes the convective fluxes of its
 * faces and applies the surface integral and the stage update, instead of a
 * face-flux kernel that stores the fluxes and an update kernel that gathers
 * them.  Results are bit-identical to the three-kernel stage.  mode -1 (the
 * default) lets ibisgb_autotune / the first ibisgb_rk_run choose among the
 * three-kernel stage, this path and the fused stage by their timings; 0 never
 * uses it; 1 always does (IBISGB_ERR_ARG if the scheme does not qualify).  A
 * scheduling choice with no counterpart in ibis. */
int ibisgb_set_cell_flux(ibisgb_ctx* ctx, int32_t mode);

/* Whether the per-cell flux path applies and is in use, its launch variant (an
 * index into ibisgb_launch_variants) and the last tuning times of one stage
 * (ms: per-cell flux path, best three-kernel stage; 2 doubles, may be NULL). */
int ibisgb_cell_flux_info(ibisgb_ctx* ctx, int32_t* eligible, int32_t* enabled, int32_t* variant,
                          double* times_ms);

/* Self-check of the mixed build's float -> double and double -> float
 * conversions, which run on the integer pipe (GB300's FP64 pipe is its scarcest
 * unit): compares them bit for bit with the conversion instructions on `samples`
 * pseudo-random float bit patterns and as many doubles (any bit pattern,
 * exponents around the float range, exact rounding ties), seeded, on the current
 * device.  No counterpart in the reference. */
int ibisgb_check_conversions(int64_t samples, uint64_t seed, int64_t* mismatches);

/* Batched ensembles (no counterpart in the reference, which runs one case per
 * process through Solver::solve, src/solvers/solvers/solver.cpp:25-59).
 * Merges already-created single-case contexts into one new context whose valid
 * cells are the cases' cells concatenated in case order, followed by the ghost
 * cells of all cases; faces and boundaries are concatenated in case order too.
 * The cases must share the dimension, flux calculator, reconstruction, limiter,
 * gas and transport settings and the Runge-Kutta tableau; each keeps its own
 * grid, boundary conditions (inflow states) and Runge-Kutta control (CFL
 * schedule, max_time, dt_init, and its own t and dt), so one ibisgb_rk_run
 * advances every case by one step of its own dt in the same kernel launches,
 * with the results of running each case alone.  A case that reaches max_time
 * or gets bad cells stops while the others go on.  The batch starts without
 * state: pass the cases' fields, concatenated in case order, to
 * ibisgb_set_primitives.  On a batch, ibisgb_rk_run's status holds the minimum
 * t, dt and stable_dt, the maximum step count and the total bad cells over the
 * cases, ibisgb_estimate_dt the minimum over the cases, ibisgb_l2_norms the
 * norms over all cells of all cases, and the steady-state calls are rejected
 * (IBISGB_ERR_STATE).  The source contexts are not changed and may be destroyed
 * afterwards. */
int ibisgb_batch_create(ibisgb_ctx* const* cases, int32_t n_cases, ibisgb_ctx** out);

/* Number of cases of a context (1 for a single case) and, for each case, the
 * first index of its valid cells, faces and ghost cells (n_cases + 1 entries
 * each, the last one the total; ghost offsets count from N).  Array arguments
 * may be NULL. */
int ibisgb_batch_layout(const ibisgb_ctx* ctx, int32_t* n_cases, int64_t* cell_offsets,
                        int64_t* face_offsets, int64_t* ghost_offsets);

/* Runge-Kutta status of every case (n_cases entries) after the last
 * ibisgb_rk_run; device_ms is that of the whole call. */
int ibisgb_batch_status(ibisgb_ctx* ctx, ibisgb_rk_status* per_case);

/* Largest residual (in cells) that ibisgb_l2_norms_noalloc accepts.  Its
 * scratch is one fixed array of 4096 x 6 doubles (192 KiB) that every GPU
 * which loads the library keeps until the process exits. */
#define IBISGB_NOALLOC_MAX_CELLS 16777216

/* L2 norms (global, mass, momentum_x, momentum_y, momentum_z, energy) of a
 * residual already in device memory (dudt_device: num_cells x n_conserved
 * row-major, as ibisgb_residual_device writes it) into norms_device (6 doubles
 * of device memory), on `stream`, without allocating anything.  This entry
 * point has no counterpart in the reference; it is ibisgb_l2_norms for callers
 * that cannot call cudaMalloc: code whose device memory is owned by a caching
 * allocator that leaves no room for a raw allocation, and time loops that must
 * not stall on the device synchronization of cudaMalloc/cudaFree.
 * num_cells above IBISGB_NOALLOC_MAX_CELLS, or n_conserved other than 4 or 5,
 * are rejected with IBISGB_ERR_ARG; errors are read with ibisgb_last_error(NULL).
 * The norms are a deterministic two-pass sum (the same bits for the same
 * input); they equal ibisgb_l2_norms's to rounding, not bit for bit, because
 * the two sum the cells in different orders.
 * The first call on a device (and the first after the device's context was
 * reset) looks up the scratch array's device address with that device
 * current: make that first call before any stream capture.  All
 * calls share the one scratch array (each call writes every slot it reads), so
 * calls whose work overlaps on the GPU race: serialize them. */
int ibisgb_l2_norms_noalloc(const double* dudt_device, int64_t num_cells, int32_t n_conserved,
                            double* norms_device, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* IBISGB_H */
