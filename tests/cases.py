"""Matched test cases for the GPU engine and the oracle: small grids of every
kind the benchmark uses, random but physical initial states, and the per-cell
relative error measure used by the parity tests."""
import numpy as np

from ibis_gb300 import grids


def random_state(n, T0, p0, u0, dim, seed=0, amp=0.08):
    """Smooth-ish random primitives around a reference state (exercises every
    limiter branch and flux-splitting branch)."""
    rng = np.random.default_rng(seed)
    T = T0 * (1 + amp * rng.standard_normal(n))
    p = p0 * (1 + amp * rng.standard_normal(n))
    vx = u0 * (1 + amp * rng.standard_normal(n))
    vy = 0.2 * u0 * rng.standard_normal(n)
    vz = 0.2 * u0 * rng.standard_normal(n) if dim == 3 else None
    return T, p, vx, vy, vz


def case(name, **kw):
    """Returns (grid, config, (T, p, vx, vy, vz))."""
    gas = grids.ideal_gas(287.0)
    if name == "ramp":
        g, c, inf = grids.ramp_case(kw.pop("ni", 24), kw.pop("nj", 12), **kw)
        st = random_state(g.num_cells, inf["T"], inf["p"], inf["vx"], 2, seed=1)
        return g, c, st
    if name == "plate":
        g, c, inf = grids.flat_plate_case(kw.pop("ni", 24), kw.pop("nj", 12), **kw)
        st = random_state(g.num_cells, inf["T"], inf["p"], inf["vx"], 2, seed=2)
        return g, c, st
    if name == "box":
        n = kw.pop("n", 6)
        g, c = grids.box_case(n, **kw)
        T, p, vx, vy, vz = grids.box_initial_condition(n, c["gas_model"], seed=3)
        return g, c, (T, p, vx, vy, vz)
    if name == "box_ragged":  # periodic box whose extents are not multiples of the kernels' tiles
        ni, nj, nk = kw.pop("shape", (36, 12, 10))
        g, c = grids.box_case(ni, ny=nj, nz=nk, **kw)
        return g, c, random_state(g.num_cells, 1.0, 1.0, 0.3, 3, seed=10, amp=0.05)
    if name == "box_inout":  # 3-D channel: supersonic in/out, slip walls
        n = kw.pop("n", 5)
        g = grids.box_3d(*n) if isinstance(n, tuple) else grids.box_3d(n)
        inflow = grids.flow_state(gas, 300.0, 1e5, 700.0, 30.0, 20.0)
        b = {"west": grids.supersonic_inflow(inflow), "east": grids.supersonic_outflow(),
             "south": grids.slip_wall(), "north": grids.slip_wall(), "bottom": grids.slip_wall(),
             "top": grids.slip_wall()}
        c = grids.make_config(3, b, gas=gas, **kw)
        return g, c, random_state(g.num_cells, 300.0, 1e5, 700.0, 3, seed=4)
    if name == "subsonic":  # subsonic in/out and a fixed-temperature no-slip wall, viscous
        X, Y = np.meshgrid(np.linspace(0, 1, 21), np.linspace(0, 0.5, 11), indexing="ij")
        g = grids.structured_2d(X, Y)
        inflow = grids.flow_state(gas, 300.0, 1e5, 100.0, 0.0)
        b = {"west": grids.subsonic_inflow(inflow), "east": grids.subsonic_outflow(0.98e5),
             "south": grids.fixed_temperature_no_slip_wall(320.0), "north": grids.slip_wall()}
        c = grids.make_config(2, b, gas=gas, viscous=True, **kw)
        return g, c, random_state(g.num_cells, 300.0, 1e5, 100.0, 2, seed=5, amp=0.03)
    if name == "bl_plate":  # viscous: boundary-layer inflow profile, constant-flux top, no-slip wall
        y = 0.05 * (np.linspace(0, 1, 13) ** 1.3)
        X, Y = np.meshgrid(np.linspace(0, 0.2, 17), y, indexing="ij")
        g = grids.structured_2d(X, Y)
        # profile heights start above the first ghost centroid and end below the
        # top ones, so both clamps of the spline are used
        h = [0.0015, 0.004, 0.008, 0.013, 0.02, 0.03, 0.04]
        u = [60.0, 180.0, 320.0, 420.0, 480.0, 500.0, 505.0]
        T = [340.0, 328.0, 315.0, 306.0, 301.0, 300.0, 300.0]
        top = grids.flow_state(gas, 300.0, 1e5, 505.0, -15.0)
        b = {"west": grids.boundary_layer_inflow(h, u, T, 1e5), "east": grids.supersonic_outflow(),
             "south": grids.adiabatic_no_slip_wall(), "north": grids.constant_flux(top)}
        kw.setdefault("viscous", True)
        c = grids.make_config(2, b, gas=gas, **kw)
        return g, c, random_state(g.num_cells, 300.0, 1e5, 450.0, 2, seed=7, amp=0.04)
    if name == "cflux_ramp":  # the ramp with a constant-flux inflow (vy != 0: the vy n.x term counts)
        g, c, inf = grids.ramp_case(kw.pop("ni", 24), kw.pop("nj", 12), **kw)
        fs = grids.flow_state(gas, inf["T"], inf["p"], inf["vx"], 0.1 * inf["vx"])
        c["grid"]["boundaries"]["inflow"] = grids.constant_flux(fs)
        return g, c, random_state(g.num_cells, inf["T"], inf["p"], inf["vx"], 2, seed=8)
    if name == "cflux_box":  # 3-D channel with a constant-flux inflow
        n = kw.pop("n", 5)
        g = grids.box_3d(n)
        inflow = grids.flow_state(gas, 300.0, 1e5, 700.0, 30.0, 20.0)
        b = {"west": grids.constant_flux(inflow), "east": grids.supersonic_outflow(),
             "south": grids.slip_wall(), "north": grids.slip_wall(), "bottom": grids.slip_wall(),
             "top": grids.constant_flux(grids.flow_state(gas, 310.0, 1.02e5, 690.0, 25.0, -10.0))}
        c = grids.make_config(3, b, gas=gas, **kw)
        return g, c, random_state(g.num_cells, 300.0, 1e5, 700.0, 3, seed=9)
    if name in ("tri", "tet", "wedge", "pyramid", "tiny2d", "tiny3d"):
        # other element types (every one the reference reads) and the smallest grids,
        # supersonic inflow on the first tag, slip walls and outflow on the others
        if name == "tri":
            X, Y = np.meshgrid(np.linspace(0, 1, 9), np.linspace(0, 0.5, 6), indexing="ij")
            g = grids.triangulate_2d(grids.structured_2d(X, Y))
        elif name == "tiny2d":
            X, Y = np.meshgrid(np.linspace(0, 1, 3), np.linspace(0, 0.5, 2), indexing="ij")
            g = grids.structured_2d(X, Y)  # 2 x 1 cells
        elif name == "tiny3d":
            g = grids.box_3d(1)  # one hexahedron
        else:
            make = {"tet": grids.tetrahedralize, "wedge": grids.prisms_3d, "pyramid": grids.pyramids_3d}[name]
            g = make(grids.box_3d(3))
        dim = g.dim
        inflow = grids.flow_state(gas, 300.0, 1e5, 600.0, 80.0, 40.0 if dim == 3 else 0.0)
        b = {t: (grids.supersonic_inflow(inflow) if i == 0 else
                 grids.slip_wall() if i % 2 else grids.supersonic_outflow()) for i, t in enumerate(g.markers)}
        c = grids.make_config(dim, b, gas=gas, **kw)
        return g, c, random_state(g.num_cells, 300.0, 1e5, 600.0, dim, seed=6, amp=0.05)
    raise KeyError(name)


def gross_flux_scale(oracle):
    """Per-cell, per-component sum of |F_f| A_f / V over the cell's faces, from
    the oracle's last residual evaluation: the natural size of a residual that
    is a difference of face fluxes."""
    flux, _ = oracle.face_dump()
    conn = oracle.connectivity()
    geo = oracle.geometry()
    cf = conn["cell_faces"]
    mask = cf >= 0
    A = np.where(mask, geo["area"][np.where(mask, cf, 0)], 0.0)
    s = np.zeros((oracle.N, oracle.nc))
    for k in range(cf.shape[1]):
        f = np.where(mask[:, k], cf[:, k], 0)
        s += np.abs(flux[f]) * A[:, k:k + 1]
    return s / geo["volume"][: oracle.N, None]


def per_cell_rel_err(r_gpu, r_ref, scale):
    return np.abs(r_gpu - r_ref) / np.maximum(scale, 1e-300)
