// _ibisgb_py: a pybind11 module beside the reference's own python_api
// (src/python/python/python_api.cpp:14-70, which exposes GasState, IdealGas,
// Vector3 and the flux-calculator names to the prep step) with the residual, its
// tangent and its adjoint on CUDA tensors, for torch.autograd
// (ibis_gb300/autograd.py).  A client of the C ABI only (include/ibisgb.h): each
// call takes a context handle (a Simulation's) and torch tensors, passes their
// device pointers and the current torch CUDA stream, and raises RuntimeError
// with the context's message when the call fails.  Built against the pybind11
// headers that ship with torch; no torch headers are needed.
#include <pybind11/pybind11.h>

#include <cstdint>
#include <stdexcept>
#include <string>

#include <cuda_runtime_api.h>

#include "ibisgb.h"

namespace py = pybind11;

namespace {

ibisgb_ctx* handle(py::object sim) {
    py::object h = sim.attr("_h");
    py::object v = h.attr("value");
    if (v.is_none()) throw std::invalid_argument("the simulation has no context");
    return reinterpret_cast<ibisgb_ctx*>(v.cast<uintptr_t>());
}

// a contiguous float64 CUDA tensor's device pointer, checked against n elements (0: any)
void* device_ptr(py::object t, const char* what, int64_t n = 0) {
    if (!t.attr("is_cuda").cast<bool>()) throw std::invalid_argument(std::string(what) + " must be a CUDA tensor");
    if (py::str(t.attr("dtype")).cast<std::string>() != "torch.float64")
        throw std::invalid_argument(std::string(what) + " must be float64");
    if (!t.attr("is_contiguous")().cast<bool>()) throw std::invalid_argument(std::string(what) + " must be contiguous");
    if (n > 0 && t.attr("numel")().cast<int64_t>() != n)
        throw std::invalid_argument(std::string(what) + " has the wrong number of elements");
    return reinterpret_cast<void*>(t.attr("data_ptr")().cast<uintptr_t>());
}

// the current torch stream as the C ABI's stream argument: the ABI reads NULL as
// "no ordering", so torch's legacy default stream (handle 0) goes as cudaStreamLegacy
void* current_stream() {
    py::object s = py::module_::import("torch.cuda").attr("current_stream")();
    const uintptr_t h = s.attr("cuda_stream").cast<uintptr_t>();
    return h ? reinterpret_cast<void*>(h) : (void*)cudaStreamLegacy;
}

void check(ibisgb_ctx* ctx, int rc) {
    if (rc != IBISGB_OK) throw std::runtime_error("ibisgb: " + std::string(ibisgb_last_error(ctx)));
}

struct Sizes {
    int64_t n = 0, n_rows = 0, F = 0, NT = 0, nb = 0;
};
Sizes sizes(ibisgb_ctx* ctx) {
    ibisgb_sizes s{};
    check(ctx, ibisgb_get_sizes(ctx, &s));
    return {s.num_cells * s.n_conserved, s.num_cells, s.num_faces, s.num_cells + s.num_ghost_cells,
            s.num_boundaries};
}

const char* precision_doc =
    "precision: 0 FP64, 1 MIXED, 2 FP64_EXACT (the reference's operation order), 3 MIXED_GRAD, 4 MIXED_FF";

}  // namespace

PYBIND11_MODULE(_ibisgb_py, m) {
    m.doc() = "Residual, tangent and adjoint of an ibis_gb300 Simulation on CUDA tensors (C ABI client)";
    m.def(
        "set_conserved",
        [](py::object sim, py::object U) {
            ibisgb_ctx* c = handle(sim);
            const double* u = (const double*)device_ptr(U, "U", sizes(c).n);
            check(c, ibisgb_set_conserved_device(c, u, current_stream()));
        },
        "The context's conserved state from U (N x n_conserved rows, reference cell order).");
    m.def(
        "residual",
        [](py::object sim, int precision, py::object out) {
            ibisgb_ctx* c = handle(sim);
            double* o = (double*)device_ptr(out, "out", sizes(c).n);
            check(c, ibisgb_residual_device(c, precision, o, current_stream()));
        },
        py::arg("sim"), py::arg("precision"), py::arg("out"),
        (std::string("dU/dt of the context's state into out (FiniteVolume::compute_dudt); ") + precision_doc)
            .c_str());
    m.def(
        "jvp",
        [](py::object sim, py::object v, py::object out, double inv_dt_star, bool allow_reconstruction) {
            ibisgb_ctx* c = handle(sim);
            const int64_t n = sizes(c).n;
            const double* x = (const double*)device_ptr(v, "v", n);
            double* o = (double*)device_ptr(out, "out", n);
            check(c, ibisgb_jvp_device(c, x, o, inv_dt_star, allow_reconstruction ? 1 : 0, current_stream()));
        },
        py::arg("sim"), py::arg("v"), py::arg("out"), py::arg("inv_dt_star") = 0.0,
        py::arg("allow_reconstruction") = true,
        "out = v inv_dt_star - (dR/dU) v (SteadyStateLinearisation's product, steady_state.cpp:52-128).");
    m.def(
        "vjp",
        [](py::object sim, py::object w, py::object out, bool allow_reconstruction) {
            ibisgb_ctx* c = handle(sim);
            const int64_t n = sizes(c).n;
            const double* x = (const double*)device_ptr(w, "w", n);
            double* o = (double*)device_ptr(out, "out", n);
            check(c, ibisgb_vjp_device(c, x, o, nullptr, allow_reconstruction ? 1 : 0, current_stream()));
        },
        py::arg("sim"), py::arg("w"), py::arg("out"), py::arg("allow_reconstruction") = true,
        "out = (dR/dU)^T w.");
    m.def(
        "vjp_geometry",
        [](py::object sim, py::object w, py::object face_out, py::object cell_out, bool allow_reconstruction) {
            ibisgb_ctx* c = handle(sim);
            const Sizes s = sizes(c);
            const double* x = (const double*)device_ptr(w, "w", s.n);
            double* fo = (double*)device_ptr(face_out, "face_out", 13 * s.F);
            double* co = (double*)device_ptr(cell_out, "cell_out", 4 * s.NT);
            check(c, ibisgb_vjp_geometry_device(c, x, fo, co, allow_reconstruction ? 1 : 0, current_stream()));
        },
        py::arg("sim"), py::arg("w"), py::arg("face_out"), py::arg("cell_out"), py::arg("allow_reconstruction") = true,
        "face_out (13 x F) and cell_out (4 x (N+G)) = w^T dR/dgeometry.");
    m.def(
        "jvp_geometry",
        [](py::object sim, py::object dface, py::object dcell, py::object out, bool allow_reconstruction) {
            ibisgb_ctx* c = handle(sim);
            const Sizes s = sizes(c);
            const double* df = (const double*)device_ptr(dface, "dface", 13 * s.F);
            const double* dc = (const double*)device_ptr(dcell, "dcell", 4 * s.NT);
            double* o = (double*)device_ptr(out, "out", s.n);
            check(c, ibisgb_jvp_geometry_device(c, df, dc, o, allow_reconstruction ? 1 : 0, current_stream()));
        },
        py::arg("sim"), py::arg("dface"), py::arg("dcell"), py::arg("out"), py::arg("allow_reconstruction") = true,
        "out (N x n_conserved) = dR/dgeometry . (dface, dcell).");
    m.def(
        "set_flow_state",
        [](py::object sim, const std::string& tag, py::sequence fs) {
            ibisgb_ctx* c = handle(sim);
            if (py::len(fs) != 7) throw std::invalid_argument("fs must hold 7 values: T, p, rho, energy, vx, vy, vz");
            double a[7];
            for (int k = 0; k < 7; k++) a[k] = fs[k].cast<double>();
            check(c, ibisgb_set_flow_state(c, tag.c_str(), a));
        },
        py::arg("sim"), py::arg("tag"), py::arg("fs"),
        "The flow state (T, p, rho, energy, vx, vy, vz) of every action of boundary tag that carries one.");
    m.def(
        "vjp_flow_state",
        [](py::object sim, py::object w, py::object out, bool allow_reconstruction) {
            ibisgb_ctx* c = handle(sim);
            const Sizes s = sizes(c);
            const double* x = (const double*)device_ptr(w, "w", s.n);
            double* o = (double*)device_ptr(out, "out", 7 * s.nb);
            check(c, ibisgb_vjp_flow_state_device(c, x, o, allow_reconstruction ? 1 : 0, current_stream()));
        },
        py::arg("sim"), py::arg("w"), py::arg("out"), py::arg("allow_reconstruction") = true,
        "out (num_boundaries x 7, sorted tag order) = w^T dR/d(each boundary's flow state).");
    m.def(
        "jvp_flow_state",
        [](py::object sim, py::object dfs, py::object out, bool allow_reconstruction) {
            ibisgb_ctx* c = handle(sim);
            const Sizes s = sizes(c);
            const double* d = (const double*)device_ptr(dfs, "dfs", 7 * s.nb);
            double* o = (double*)device_ptr(out, "out", s.n);
            check(c, ibisgb_jvp_flow_state_device(c, d, o, allow_reconstruction ? 1 : 0, current_stream()));
        },
        py::arg("sim"), py::arg("dfs"), py::arg("out"), py::arg("allow_reconstruction") = true,
        "out (N x n_conserved) = dR/dfs . dfs for dfs (num_boundaries x 7) a direction of every flow state.");
}
