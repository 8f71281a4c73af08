// ORACLE — test infrastructure only. extern "C" surface of the CPU restatement
// (oracle_core.hpp), loaded by the tests and by the CPU-baseline leg of bench.py.
#include <algorithm>
#include <cstring>
#include <string>

#include "oracle_core.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace oracle;

namespace {

struct Handle {
    Json config;
    GridIO io;
    std::unique_ptr<Sim<double>> sim;  // real-valued simulation
    std::unique_ptr<Steady> steady;    // dual-valued steady linearisation
    std::string error;
    size_t N() const { return sim ? sim->grid.N : steady->sim->grid.N; }
};

template <typename T>
Grid<T>& grid_of(Handle* h);
template <>
Grid<double>& grid_of<double>(Handle* h) { return h->sim->grid; }

void set_ic(Sim<double>& s, const double* T, const double* p, const double* vx, const double* vy,
            const double* vz) {
    // NativeBinaryInput::read, native.cpp:263-339 (valid cells, then update_thermo_from_pT)
    for (size_t i = 0; i < s.grid.N; i++) {
        s.fs.temp[i] = T[i];
        s.fs.p[i] = p[i];
        s.fs.vx[i] = vx[i];
        s.fs.vy[i] = vy[i];
        s.fs.vz[i] = vz ? vz[i] : 0.0;
        s.fs.rho[i] = s.fs.p[i] / (s.gas.R * s.fs.temp[i]);
        s.fs.e[i] = s.gas.Cv * s.fs.temp[i];
    }
}

}  // namespace

#define GUARD_BEGIN try {
#define GUARD_END(h, rv)                        \
    }                                           \
    catch (const std::exception& e) {           \
        if (h) ((Handle*)h)->error = e.what();  \
        return rv;                              \
    }

extern "C" {

const char* orc_last_error(void* h) { return h ? ((Handle*)h)->error.c_str() : "null handle"; }

// Create from a config.json text and either an SU2 path or, when su2_path is
// null, grid arrays (vtk element codes, CSR connectivity). kind 0 = real, 1 = dual/steady.
void* orc_create(const char* config_text, const char* su2_path, int kind, int dim, long long nv,
                 const double* xyz, long long ncells, const int* cell_types,
                 const long long* cell_offsets, const long long* cell_conn, int nmark,
                 const char* mark_names, const long long* mark_offsets, const int* elem_types,
                 const long long* elem_offsets, const long long* elem_conn, char* err, int errlen) {
    Handle* h = new Handle();
    try {
        h->config = Json::parse(config_text);
        if (su2_path) {
            h->io.read_su2(su2_path);
        } else {
            h->io.dim = (size_t)dim;
            h->io.vertices.resize((size_t)nv);
            for (long long i = 0; i < nv; i++) h->io.vertices[i] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
            h->io.cells.resize((size_t)ncells);
            for (long long c = 0; c < ncells; c++) {
                ElemIO& e = h->io.cells[c];
                e.type = elem_type_from_vtk((size_t)cell_types[c]);
                for (long long k = cell_offsets[c]; k < cell_offsets[c + 1]; k++) e.ids.push_back((size_t)cell_conn[k]);
            }
            std::string names(mark_names);
            size_t pos = 0;
            for (int m = 0; m < nmark; m++) {
                size_t nl = names.find('\n', pos);
                std::string tag = names.substr(pos, nl == std::string::npos ? std::string::npos : nl - pos);
                pos = nl + 1;
                auto& dst = h->io.markers[tag];
                for (long long el = mark_offsets[m]; el < mark_offsets[m + 1]; el++) {
                    ElemIO e;
                    e.type = elem_type_from_vtk((size_t)elem_types[el]);
                    for (long long k = elem_offsets[el]; k < elem_offsets[el + 1]; k++) e.ids.push_back((size_t)elem_conn[k]);
                    dst.push_back(e);
                }
            }
        }
        if (kind == 0) {
            h->sim = build_sim<double>(h->config, h->io);
            if (h->config.at("solver").at("name").as_string() == "runge_kutta") h->sim->init_rk(h->config.at("solver"));
        } else {
            h->steady = std::make_unique<Steady>();
            h->steady->setup(h->config, h->io);
        }
    } catch (const std::exception& e) {
        std::snprintf(err, errlen, "%s", e.what());
        delete h;
        return nullptr;
    }
    return h;
}

void orc_destroy(void* h) { delete (Handle*)h; }

// sizes: N, G, F, dim, max faces per cell
int orc_sizes(void* hp, long long* out) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    size_t mf = 0, N, G, F, dim;
    if (h->sim) {
        auto& g = h->sim->grid;
        N = g.N; G = g.G; F = g.F; dim = g.dim;
        for (auto& c : g.cell_faces) mf = std::max(mf, c.size());
    } else {
        auto& g = h->steady->sim->grid;
        N = g.N; G = g.G; F = g.F; dim = g.dim;
        for (auto& c : g.cell_faces) mf = std::max(mf, c.size());
    }
    out[0] = (long long)N; out[1] = (long long)G; out[2] = (long long)F; out[3] = (long long)dim;
    out[4] = (long long)mf;
    return 0;
    GUARD_END(h, -1)
}

// connectivity in reference numbering: left/right per face (NONE -> -1), per cell
// face ids / outsigns / neighbours padded to mf slots with -1 / 0
int orc_connectivity(void* hp, long long* left, long long* right, long long* cell_faces,
                     int* outsigns, long long* nbrs, int mf) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    auto& g = h->sim->grid;
    for (size_t f = 0; f < g.F; f++) {
        left[f] = g.left[f] == NONE ? -1 : (long long)g.left[f];
        right[f] = g.right[f] == NONE ? -1 : (long long)g.right[f];
    }
    for (size_t c = 0; c < g.N; c++) {
        for (int k = 0; k < mf; k++) {
            bool has = (size_t)k < g.cell_faces[c].size();
            cell_faces[c * mf + k] = has ? (long long)g.cell_faces[c][k] : -1;
            outsigns[c * mf + k] = has ? g.outsigns[c][k] : 0;
            nbrs[c * mf + k] = has ? (long long)g.cell_nbrs[c][k] : -1;
        }
    }
    return 0;
    GUARD_END(h, -1)
}

// ghost cells of one boundary tag (ids, in the order they were created)
int orc_ghosts(void* hp, const char* tag, long long* ids, long long* faces, long long cap) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    auto& g = h->sim->grid;
    const auto& gc = g.ghost_cells.at(tag);
    const auto& bf = g.boundary_faces.at(tag);
    for (size_t i = 0; i < gc.size() && (long long)i < cap; i++) ids[i] = (long long)gc[i];
    for (size_t i = 0; i < bf.size() && (long long)i < cap; i++) faces[i] = (long long)bf[i];
    return (int)std::max(gc.size(), bf.size());
    GUARD_END(h, -1)
}

// geometry: face (nx,ny,nz,t1x..,t2x..,cx,cy,cz,area) 13*F; cell (ccx,ccy,ccz,volume) 4*(N+G)
int orc_geometry(void* hp, double* face, double* cell) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    auto& g = h->sim->grid;
    const std::vector<double>* fa[13] = {&g.nx, &g.ny, &g.nz, &g.t1x, &g.t1y, &g.t1z, &g.t2x,
                                         &g.t2y, &g.t2z, &g.cx, &g.cy, &g.cz, &g.area};
    for (int k = 0; k < 13; k++) std::memcpy(face + k * g.F, fa[k]->data(), g.F * sizeof(double));
    size_t NT = g.N + g.G;
    const std::vector<double>* ca[4] = {&g.ccx, &g.ccy, &g.ccz, &g.volume};
    for (int k = 0; k < 4; k++) std::memcpy(cell + k * NT, ca[k]->data(), NT * sizeof(double));
    return 0;
    GUARD_END(h, -1)
}

int orc_lsq_r(void* hp, double* r6) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    auto& g = h->sim->grid;
    if (g.r.empty()) g.compute_gradient_weights();
    for (size_t i = 0; i < g.N; i++) for (int k = 0; k < 6; k++) r6[i * 6 + k] = g.r[i][k];
    return 0;
    GUARD_END(h, -1)
}

// LSQ gradient of an arbitrary cell scalar (N+G values) -> N x 3
int orc_gradient(void* hp, const double* values, double* grad) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    auto& g = h->sim->grid;
    if (g.r.empty()) g.compute_gradient_weights();
    std::vector<double> v(values, values + g.N + g.G);
    std::vector<std::array<double, 3>> gr(g.N);
    lsq_gradient_real(g, v, gr);
    for (size_t i = 0; i < g.N; i++) for (int k = 0; k < 3; k++) grad[i * 3 + k] = gr[i][k];
    return 0;
    GUARD_END(h, -1)
}

// initial condition of the valid cells (T, p, vx, vy, vz; vz may be null in 2-D)
int orc_set_ic(void* hp, const double* T, const double* p, const double* vx, const double* vy,
               const double* vz) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    if (h->sim) {
        set_ic(*h->sim, T, p, vx, vy, vz);
    } else {
        Sim<Dual>& s = *h->steady->sim;
        for (size_t i = 0; i < s.grid.N; i++) {
            s.fs.temp[i] = T[i]; s.fs.p[i] = p[i]; s.fs.vx[i] = vx[i]; s.fs.vy[i] = vy[i];
            s.fs.vz[i] = vz ? vz[i] : 0.0;
            s.fs.rho[i] = s.fs.p[i] / (s.gas.R * s.fs.temp[i]);
            s.fs.e[i] = s.gas.Cv * s.fs.temp[i];
        }
    }
    return 0;
    GUARD_END(h, -1)
}

// primitives of all N+G cells: rho, p, T, e, vx, vy, vz (7 x (N+G))
int orc_get_prims(void* hp, double* out) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    auto& g = h->sim->grid;
    auto& fs = h->sim->fs;
    size_t NT = g.N + g.G;
    const std::vector<double>* a[7] = {&fs.rho, &fs.p, &fs.temp, &fs.e, &fs.vx, &fs.vy, &fs.vz};
    for (int k = 0; k < 7; k++) std::memcpy(out + k * NT, a[k]->data(), NT * sizeof(double));
    return 0;
    GUARD_END(h, -1)
}

// Overwrite the primitives of all N+G cells (7 x (N+G)), e.g. to restart from a GPU state.
int orc_put_prims(void* hp, const double* in) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    auto& g = h->sim->grid;
    auto& fs = h->sim->fs;
    size_t NT = g.N + g.G;
    std::vector<double>* a[7] = {&fs.rho, &fs.p, &fs.temp, &fs.e, &fs.vx, &fs.vy, &fs.vz};
    for (int k = 0; k < 7; k++) std::memcpy(a[k]->data(), in + k * NT, NT * sizeof(double));
    primatives_to_conserved(h->sim->U, fs);
    return 0;
    GUARD_END(h, -1)
}

// dU/dt of the valid cells (N x nc, row-major), as compute_dudt on the current
// primitives; record=1 also stores limiter branch codes (N x 5)
int orc_residual(void* hp, double* dudt, int allow_reconstruction, unsigned* branches) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    Sim<double>& s = *h->sim;
    Conserved<double> d(s.grid.N + s.grid.G, s.grid.dim);
    s.fv.record_branches = branches != nullptr;
    s.fv.compute_dudt(s.fs, s.grid, d, s.gas, s.tp, allow_reconstruction != 0);
    s.fv.record_branches = false;
    size_t nc = s.grid.dim + 2;
    std::memcpy(dudt, d.q.data(), s.grid.N * nc * sizeof(double));
    if (branches) std::memcpy(branches, s.fv.branches.data(), s.grid.N * 5 * sizeof(unsigned));
    return 0;
    GUARD_END(h, -1)
}

// limiter values and convective gradients after the last residual: per cell
// [l_rho, l_u, l_p, l_T, l_vx, l_vy, l_vz] (7) and gradients of rho,u,p,T,vx,vy,vz (21)
int orc_recon_dump(void* hp, double* lim, double* grad) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    auto& fv = h->sim->fv;
    size_t N = h->sim->grid.N;
    const std::vector<double>* ls[7] = {&fv.l_rho, &fv.l_u, &fv.l_p, &fv.l_temp, &fv.l_vx, &fv.l_vy, &fv.l_vz};
    const std::vector<std::array<double, 3>>* gs[7] = {&fv.g_rho, &fv.g_u, &fv.g_p, &fv.g_temp, &fv.g_vx, &fv.g_vy, &fv.g_vz};
    for (size_t i = 0; i < N; i++) {
        for (int k = 0; k < 7; k++) {
            lim[i * 7 + k] = (*ls[k])[i];
            for (int d = 0; d < 3; d++) grad[i * 21 + k * 3 + d] = (*gs[k])[i][d];
        }
    }
    return 0;
    GUARD_END(h, -1)
}

// face flux after the last residual (F x nc) and viscous face state (rho,p,T,e,vx,vy,vz x F)
int orc_face_dump(void* hp, double* flux, double* face_fs) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    auto& fv = h->sim->fv;
    size_t F = h->sim->grid.F;
    std::memcpy(flux, fv.flux.q.data(), fv.flux.q.size() * sizeof(double));
    if (face_fs) {
        const std::vector<double>* a[7] = {&fv.face_fs.rho, &fv.face_fs.p, &fv.face_fs.temp, &fv.face_fs.e,
                                           &fv.face_fs.vx, &fv.face_fs.vy, &fv.face_fs.vz};
        for (int k = 0; k < 7; k++) std::memcpy(face_fs + k * F, a[k]->data(), F * sizeof(double));
    }
    return 0;
    GUARD_END(h, -1)
}

double orc_estimate_dt(void* hp) {
    Handle* h = (Handle*)hp;
    Sim<double>& s = *h->sim;
    return s.fv.estimate_dt(s.fs, s.grid, s.gas, s.tp);
}

long long orc_count_bad_cells(void* hp) {
    Handle* h = (Handle*)hp;
    return (long long)h->sim->fv.count_bad_cells(h->sim->fs, h->sim->grid.N);
}

// RungeKutta::initialise (after orc_set_ic)
int orc_rk_initialise(void* hp) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    h->sim->rk_initialise();
    return 0;
    GUARD_END(h, -1)
}

// n RungeKutta::take_step calls; out: t, dt, stable_dt, then the 6 L2 norms of k0
int orc_rk_steps(void* hp, int n, double* out) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    Sim<double>& s = *h->sim;
    for (int i = 0; i < n; i++) s.rk_take_step();
    Norms nm = l2_norms(s.k[0]);
    double v[9] = {s.rk.t, s.rk.dt, s.rk.stable_dt, nm.global, nm.mass, nm.mx, nm.my, nm.mz, nm.energy};
    std::memcpy(out, v, sizeof(v));
    return 0;
    GUARD_END(h, -1)
}

// conserved state of the valid cells (N x nc)
int orc_get_conserved(void* hp, double* out) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    Sim<double>& s = *h->sim;
    size_t nc = s.grid.dim + 2;
    std::memcpy(out, s.U.q.data(), s.grid.N * nc * sizeof(double));
    return 0;
    GUARD_END(h, -1)
}

// ---- steady / dual -------------------------------------------------------

int orc_steady_initialise(void* hp) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    h->steady->initialise();
    return 0;
    GUARD_END(h, -1)
}

// (I/dt* - dR/dU) v with the reference's dual numbers; dt_star<=0 gives -dR/dU v
// with the 1/dt* term dropped. allow_reconstruction=0 is the first-order preconditioner.
int orc_jvp(void* hp, const double* v, double* out, double dt_star, int allow_reconstruction) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    Steady& st = *h->steady;
    std::vector<double> vv(v, v + st.n_vars), oo(st.n_vars);
    st.dt_star = dt_star > 0 ? dt_star : 1e300;
    st.matvec(vv, oo, allow_reconstruction != 0);
    std::memcpy(out, oo.data(), st.n_vars * sizeof(double));
    return 0;
    GUARD_END(h, -1)
}

// Directional derivative of the residual at the steady simulation's current state
// along a perturbation of the grid geometry: dface (13 x F: n, t1, t2, face
// centre, area) and dcell (4 x (N+G): centroid, volume) seeded into the dual
// parts of the Grid<Dual> arrays; the least-squares factors are recomputed from
// the dual centroids (gradient.h:119-162), so they carry the centroids'
// perturbation.  The geometry's dual parts are cleared afterwards.
int orc_geometry_jvp(void* hp, const double* dface, const double* dcell, double* out, int allow_reconstruction) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    Steady& st = *h->steady;
    Sim<Dual>& s = *st.sim;
    Grid<Dual>& g = s.grid;
    std::vector<Dual>* fa[13] = {&g.nx, &g.ny, &g.nz, &g.t1x, &g.t1y, &g.t1z, &g.t2x, &g.t2y, &g.t2z,
                                 &g.cx, &g.cy, &g.cz, &g.area};
    std::vector<Dual>* ca[4] = {&g.ccx, &g.ccy, &g.ccz, &g.volume};
    const size_t NT = g.N + g.G;
    auto seed = [&](bool on) {
        for (int k = 0; k < 13; k++)
            for (size_t f = 0; f < g.F; f++) (*fa[k])[f].du = on ? dface[k * g.F + f] : 0.0;
        for (int k = 0; k < 4; k++)
            for (size_t c = 0; c < NT; c++) (*ca[k])[c].du = on ? dcell[k * NT + c] : 0.0;
        if (!g.r.empty()) g.compute_gradient_weights();
    };
    seed(true);
    size_t nc = g.dim + 2;
    for (size_t c = 0; c < g.N; c++)
        for (size_t q = 0; q < nc; q++) {
            st.cq_tmp.q[c * nc + q].re = s.U.q[c * nc + q].re;
            st.cq_tmp.q[c * nc + q].du = 0.0;
        }
    conserved_to_primatives(st.cq_tmp, st.fs_tmp, s.gas);
    s.fv.compute_dudt(st.fs_tmp, g, st.residuals, s.gas, s.tp, allow_reconstruction != 0);
    for (size_t i = 0; i < g.N * nc; i++) out[i] = st.residuals.q[i].du;
    seed(false);
    return 0;
    GUARD_END(h, -1)
}

// Directional derivative of the residual at the steady simulation's current state
// along a perturbation dfs (T, p, rho, energy, vx, vy, vz) of boundary `tag`'s
// flow state, seeded into the dual parts of every action of that boundary that
// carries one (flow_state_copy, subsonic_inflow, constant_flux); cleared afterwards.
int orc_flow_state_jvp(void* hp, const char* tag, const double* dfs, double* out, int allow_reconstruction) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    Steady& st = *h->steady;
    Sim<Dual>& s = *st.sim;
    Grid<Dual>& g = s.grid;
    const auto& tags = g.boundary_tags;
    const size_t b = (size_t)(std::find(tags.begin(), tags.end(), std::string(tag)) - tags.begin());
    if (b == tags.size()) throw std::runtime_error(std::string("no boundary ") + tag);
    BoundaryCondition& bc = s.fv.bcs[b];
    auto seed = [&](bool on) {
        for (auto* list : {&bc.pre_reconstruction, &bc.post_convective_flux, &bc.pre_viscous_grad})
            for (Action& a : *list)
                if (a.kind == ActionKind::FlowStateCopy || a.kind == ActionKind::SubsonicInflow ||
                    a.kind == ActionKind::ConstantFlux)
                    for (int k = 0; k < 7; k++) a.fs_du[k] = on ? dfs[k] : 0.0;
    };
    seed(true);
    size_t nc = g.dim + 2;
    for (size_t c = 0; c < g.N; c++)
        for (size_t q = 0; q < nc; q++) {
            st.cq_tmp.q[c * nc + q].re = s.U.q[c * nc + q].re;
            st.cq_tmp.q[c * nc + q].du = 0.0;
        }
    conserved_to_primatives(st.cq_tmp, st.fs_tmp, s.gas);
    s.fv.compute_dudt(st.fs_tmp, g, st.residuals, s.gas, s.tp, allow_reconstruction != 0);
    for (size_t i = 0; i < g.N * nc; i++) out[i] = st.residuals.q[i].du;
    seed(false);
    return 0;
    GUARD_END(h, -1)
}

// real residual of the steady simulation at its current state (N x nc)
int orc_steady_rhs(void* hp, double* out) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    Steady& st = *h->steady;
    st.eval_rhs();
    std::memcpy(out, st.rhs.data(), st.n_vars * sizeof(double));
    return 0;
    GUARD_END(h, -1)
}

// n JFNK steps; out per step: [relative global residual, gmres iters, gmres residual, dt_star]
int orc_steady_steps(void* hp, int n, double* out) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    Steady& st = *h->steady;
    for (int i = 0; i < n; i++) {
        GmresResult r = st.step((size_t)i);
        out[4 * i + 0] = st.residual_norms.global / st.initial_norms.global;
        out[4 * i + 1] = (double)r.n_iters;
        out[4 * i + 2] = r.residual;
        out[4 * i + 3] = st.dt_star;
    }
    return 0;
    GUARD_END(h, -1)
}

int orc_steady_conserved(void* hp, double* out) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    Sim<Dual>& s = *h->steady->sim;
    size_t nc = s.grid.dim + 2;
    for (size_t i = 0; i < s.grid.N * nc; i++) out[i] = s.U.q[i].re;
    return 0;
    GUARD_END(h, -1)
}

// ---- dense GMRES / FGMRES on a small matrix (gmres.cpp:320-500 tests) ----
int orc_dense_gmres(int n, const double* A, const double* rhs, double* x, int max_iters,
                    double tol, const double* P, int max_prec_iters, double prec_tol,
                    double* info) {
    try {
        auto mv = [n](const double* M) {
            return MatVec([n, M](const std::vector<double>& v, std::vector<double>& o) {
                for (int r = 0; r < n; r++) {
                    double d = 0.0;
                    for (int c = 0; c < n; c++) d += M[r * n + c] * v[c];
                    o[r] = d;
                }
            });
        };
        std::vector<double> b(rhs, rhs + n), xx(n, 0.0);
        GmresResult r;
        if (P) r = fgmres_solve(mv(A), mv(P), xx, b, (size_t)max_iters, tol, (size_t)max_prec_iters, prec_tol);
        else r = gmres_solve(mv(A), b, xx, (size_t)max_iters, tol);
        std::memcpy(x, xx.data(), n * sizeof(double));
        info[0] = r.success; info[1] = (double)r.n_iters; info[2] = r.residual;
        return 0;
    } catch (...) {
        return -1;
    }
}

// ---- natural cubic spline of the boundary-layer profile (cubic_spline.cpp:91-159 tests) ----
int orc_cubic_spline(int n, const double* x, const double* y, int nq, const double* q, double* out) {
    try {
        CubicSpline sp;
        sp.fit(std::vector<double>(x, x + n), std::vector<double>(y, y + n));
        for (int i = 0; i < nq; i++) out[i] = sp.eval(q[i]);
        return 0;
    } catch (...) {
        return -1;
    }
}

// Exact floating-point operation counts of one RungeKutta::take_step from the
// real simulation's current primitive state, on a copy of it instantiated on
// the counting scalar (one thread).  The step includes its estimate_dt.
// out: additions (and subtractions), multiplications, divisions, square roots,
// powers, and abs/min/max/floor/copysign, in that order.
int orc_count_step_flops(void* hp, long long* out) {
    Handle* h = (Handle*)hp;
    GUARD_BEGIN
    if (!h->sim) throw std::runtime_error("orc_count_step_flops: not a real-valued (kind 0) oracle");
    const Sim<double>& src = *h->sim;
    std::unique_ptr<Sim<Cnt>> s = build_sim<Cnt>(h->config, h->io);
    s->init_rk(h->config.at("solver"));
    for (size_t i = 0; i < src.grid.N; i++) {
        s->fs.temp[i] = src.fs.temp[i]; s->fs.p[i] = src.fs.p[i]; s->fs.rho[i] = src.fs.rho[i];
        s->fs.e[i] = src.fs.e[i]; s->fs.vx[i] = src.fs.vx[i]; s->fs.vy[i] = src.fs.vy[i];
        s->fs.vz[i] = src.fs.vz[i];
    }
#ifdef _OPENMP
    const int nt = omp_get_max_threads();
    omp_set_num_threads(1);
#endif
    s->rk_initialise();
    g_flops = FlopCounts{};
    s->rk_take_step();
    const FlopCounts c = g_flops;
#ifdef _OPENMP
    omp_set_num_threads(nt);
#endif
    const unsigned long long v[6] = {c.add, c.mul, c.div, c.sqrt, c.pow, c.other};
    for (int q = 0; q < 6; q++) out[q] = (long long)v[q];
    return 0;
    GUARD_END(h, -1)
}

int orc_num_threads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
