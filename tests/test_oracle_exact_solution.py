"""The oracle against exact solutions.

1. Mach 3 flow over a 15-degree expansion corner, the reference's exact-solution
   case (tests/exact_solutions/prandtl_meyer_expansion/job.py: AUSMDV,
   second-order unlimited reconstruction, ssp-rk3 at CFL 2 for three flow-through
   times, ideal air, rho = 1.225 kg/m^3 and T = 300 K upstream).  Downstream of
   the centred expansion fan the flow is uniform, turned by 15 degrees, at the
   Mach number whose Prandtl-Meyer angle exceeds the upstream one by 15 degrees,
   with temperature, pressure and density from the isentropic relations.  The
   corner is a true 15-degree turn on a structured quad grid written here (the
   reference meshes the same domain with gmsh, which is absent; its wall drops by
   (length - x0) sin 15 deg instead of tan 15 deg).  The analytic state uses the
   standard isentropic relations p2/p1 = (T2/T1)^(g/(g-1)), rho2/rho1 =
   (T2/T1)^(1/(g-1)).  The second-order error falls about 4x when the cells are
   halved.

2. The compression ramp of the benchmarks (Mach 2 at 300 K, 15 degrees; Hanel,
   second-order MUSCL with Barth-Jespersen, ssp-rk3 at CFL 0.5 for three
   flow-through times): between the attached oblique shock and the ramp the flow
   is uniform, turned by 15 degrees, with the weak-shock angle of the
   theta-beta-M relation and the normal-shock jumps of the Mach number normal to
   the shock.  At 128 x 64 the mean errors are 0.07-0.11%.

3. Sod's shock tube (left rho = 1, p = 1; right rho = 0.125, p = 0.1; at rest,
   gamma = 1.4) to t = 0.2 with the default numerics, one row of cells between
   slip walls: against the exact Riemann solution (Toro's iterative solver for
   the star pressure, written here from the published method), the L1 errors
   fall as the cells shrink (order about 0.8 with the discontinuities) and the
   star state p* = 0.30313, u* = 0.92745 is reproduced between the rarefaction
   and the contact.

4. The same ramp extruded into two layers of hexahedra between slip walls (the
   3-D path): the post-shock state matches the oblique shock as in 2-D.  With
   first-order reconstruction the z-mirror symmetry holds to round-off.  With
   Barth-Jespersen it does not, at the shock: a cell's z-gradient there is pure
   round-off, so its projections onto the z faces are +-1e-17; in a cell that is
   a local extremum the reference's ratio (U_min - U_i) / d2 is then 0 for the
   sign that rounding picked, and the limiter drops the cell to first order in
   one layer and not the other (v_z reaches 5e-4 of |v| in the shock cells).

5. The structure of a normal shock in air (Mach 2 at 300 K, Sutherland
   viscosity, Prandtl number 3/4) on one row of cells between slip walls, with
   the Rankine-Hugoniot downstream pressure at a subsonic outflow.  At Pr = 3/4
   the total enthalpy is constant through the shock (Becker's integral, for any
   mu(T)), and the exact Navier-Stokes profile follows from the momentum
   equation (4/3) mu(T) du/dx = m (u - u1) + p - p1, with T and p functions of u,
   integrated here.  This checks the viscous stress, the heat flux and the
   Sutherland transport.  The velocity error within five shock thicknesses is
   1.0% of the jump at 3 cells per thickness and 0.39% at 5.

The GPU builds equal the oracle (tests/test_residual_gpu.py,
tests/test_ramp_full_gpu.py), so they inherit these checks."""
import math

import numpy as np
import pytest

from ibis_gb300 import grids
from oracle.oracle import Oracle


def prandtl_meyer(M, g):
    a = math.sqrt((g + 1) / (g - 1))
    return a * math.atan(math.sqrt((g - 1) / (g + 1) * (M * M - 1))) - math.atan(math.sqrt(M * M - 1))


def mach_after_turn(M1, theta, g):
    """The Mach number whose Prandtl-Meyer angle is nu(M1) + theta (bisection)."""
    target = prandtl_meyer(M1, g) + theta
    lo, hi = M1, 50.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        lo, hi = (mid, hi) if prandtl_meyer(mid, g) < target else (lo, mid)
    return 0.5 * (lo + hi)


def expansion_corner(h):
    """Run the corner to t = 3 L / u on cells of size h; returns the mean relative
    errors of M, T, p, rho and the mean flow angle over the uniform region
    downstream of the fan (0.5 <= x <= 0.85, between 0.02 m above the wall and
    y = -0.05, clear of the fan's last characteristic)."""
    th = math.radians(15.0)
    L, x0, H = 0.9, 0.05, 0.6
    ni, nj = int(round(L / h)), int(round(H / h))
    x = np.linspace(0.0, L, ni + 1)
    yw = np.where(x <= x0, 0.0, -(x - x0) * math.tan(th))
    X = np.repeat(x[:, None], nj + 1, 1)
    Y = yw[:, None] + (H - yw[:, None]) * np.linspace(0.0, 1.0, nj + 1)[None, :]
    g = grids.structured_2d(X, Y, bottom_tags=lambda i: "wall")
    gas = grids.ideal_gas(287.0)
    gm = gas["gamma"]
    M1, T1, rho1 = 3.0, 300.0, 1.225
    p1 = rho1 * gas["R"] * T1
    inflow = grids.mach_state(gas, M1, T1, p1)
    b = {"west": grids.supersonic_inflow(inflow), "east": grids.supersonic_outflow(),
         "north": grids.supersonic_outflow(), "wall": grids.slip_wall()}
    tmax = 3 * 1.0 / inflow["vx"]
    c = grids.make_config(2, b, gas=gas, flux="ausmdv", order=2, limiter="unlimited",
                          solver=grids.runge_kutta(cfl=2.0, max_step=100000, max_time=tmax))
    o = Oracle(c, g)
    n = g.num_cells
    o.set_initial_condition(np.full(n, T1), np.full(n, p1), np.full(n, inflow["vx"]), np.zeros(n))
    o.rk_initialise()
    t = 0.0
    for _ in range(400):
        t = o.rk_steps(50)["t"]
        if t >= tmax * (1 - 1e-12):
            break
    assert t >= tmax * (1 - 1e-12) and o.count_bad_cells() == 0
    M2 = mach_after_turn(M1, th, gm)
    k = (1 + 0.5 * (gm - 1) * M1 ** 2) / (1 + 0.5 * (gm - 1) * M2 ** 2)
    exact = {"M": M2, "T": T1 * k, "p": p1 * k ** (gm / (gm - 1)), "rho": rho1 * k ** (1 / (gm - 1))}
    pr = o.primitives()[:, :o.N]  # rho, p, T, e, vx, vy, vz
    cen = o.geometry()["centroid"]
    cx, cy = cen[0][:o.N], cen[1][:o.N]
    sel = (cx >= 0.5) & (cx <= 0.85) & (cy <= -0.05) & (cy >= -(cx - x0) * math.tan(th) + 0.02)
    rho, p, T, vx, vy = pr[0][sel], pr[1][sel], pr[2][sel], pr[4][sel], pr[5][sel]
    got = {"M": np.hypot(vx, vy) / np.sqrt(gm * gas["R"] * T), "T": T, "p": p, "rho": rho}
    err = {q: float(np.mean(np.abs(got[q] / exact[q] - 1))) for q in exact}
    return err, float(np.degrees(np.mean(np.arctan2(vy, vx)))), int(sel.sum())


@pytest.fixture(scope="module")
def coarse():
    return expansion_corner(0.01)


def test_expanded_state_matches_prandtl_meyer(coarse):
    err, angle, cells = coarse
    assert cells > 200
    for q, e in err.items():
        assert e <= 5e-3, (q, err)
    assert angle == pytest.approx(-15.0, abs=0.05)


def test_error_falls_at_second_order(coarse):
    err, _, _ = coarse
    fine, angle, _ = expansion_corner(0.005)
    assert fine["p"] <= err["p"] / 3.0, (err, fine)
    assert max(fine.values()) <= 1e-3, fine
    assert angle == pytest.approx(-15.0, abs=0.01)


def weak_shock_angle(M, theta, g):
    """The weak root beta of tan(theta) = 2 cot(beta) (M^2 sin^2(beta) - 1) / (M^2 (g + cos 2 beta) + 2)."""
    def f(b):
        return 2 / math.tan(b) * (M * M * math.sin(b) ** 2 - 1) / (M * M * (g + math.cos(2 * b)) + 2) - math.tan(theta)
    bs = np.linspace(math.asin(1 / M) + 1e-9, math.pi / 2 - 1e-6, 20000)
    i = int(np.argmax([f(b) > 0 for b in bs]))
    lo, hi = bs[i - 1], bs[i]
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        lo, hi = (lo, mid) if f(mid) > 0 else (mid, hi)
    return 0.5 * (lo + hi)


def test_compression_ramp_matches_the_oblique_shock():
    g, c, inf = grids.ramp_case(128, 64)
    tmax = 3.0 * 1.0 / inf["vx"]
    c = dict(c, solver=grids.runge_kutta(cfl=0.5, max_step=100000, max_time=tmax))
    o = Oracle(c, g)
    n = g.num_cells
    o.set_initial_condition(np.full(n, inf["T"]), np.full(n, inf["p"]), np.full(n, inf["vx"]), np.full(n, inf["vy"]))
    o.rk_initialise()
    t = 0.0
    for _ in range(200):
        t = o.rk_steps(100)["t"]
        if t >= tmax * (1 - 1e-12):
            break
    assert t >= tmax * (1 - 1e-12) and o.count_bad_cells() == 0
    gm, R, M1, th = 1.4, 287.0, 2.0, math.radians(15.0)
    b = weak_shock_angle(M1, th, gm)
    Mn1 = M1 * math.sin(b)
    p21 = 1 + 2 * gm / (gm + 1) * (Mn1 ** 2 - 1)
    r21 = (gm + 1) * Mn1 ** 2 / ((gm - 1) * Mn1 ** 2 + 2)
    Mn2 = math.sqrt((1 + 0.5 * (gm - 1) * Mn1 ** 2) / (gm * Mn1 ** 2 - 0.5 * (gm - 1)))
    exact = {"M": Mn2 / math.sin(b - th), "T": inf["T"] * p21 / r21, "p": inf["p"] * p21, "rho": inf["rho"] * r21}
    pr = o.primitives()[:, :o.N]
    cen = o.geometry()["centroid"]
    cx, cy = cen[0][:o.N], cen[1][:o.N]
    # clear of the ramp's first cells and of the shock; the shock's reflection off the
    # top wall (x ~ 0.7) comes back down downstream of x = 0.55
    sel = (cx >= 0.3) & (cx <= 0.55) & (cy >= (cx - 0.2) * math.tan(th) + 0.02) & (cy <= (cx - 0.2) * math.tan(b) - 0.04)
    assert sel.sum() > 400
    rho, p, T, vx, vy = pr[0][sel], pr[1][sel], pr[2][sel], pr[4][sel], pr[5][sel]
    got = {"M": np.hypot(vx, vy) / np.sqrt(gm * R * T), "T": T, "p": p, "rho": rho}
    for q in exact:
        assert np.mean(np.abs(got[q] / exact[q] - 1)) <= 3e-3, q
    assert float(np.degrees(np.mean(np.arctan2(vy, vx)))) == pytest.approx(15.0, abs=0.02)


GAMMA = 1.4


def _f_side(p, rk, pk, ak):
    """Toro's pressure function of one side: a shock for p > pk, a rarefaction otherwise."""
    if p > pk:
        A, B = 2 / ((GAMMA + 1) * rk), (GAMMA - 1) / (GAMMA + 1) * pk
        return (p - pk) * math.sqrt(A / (p + B))
    return 2 * ak / (GAMMA - 1) * ((p / pk) ** ((GAMMA - 1) / (2 * GAMMA)) - 1)


def riemann_star(left, right):
    """Star pressure and velocity: the root of f_L(p) + f_R(p) + (u_R - u_L), monotone in p."""
    (rl, ul, pl), (rr, ur, pr) = left, right
    al, ar = math.sqrt(GAMMA * pl / rl), math.sqrt(GAMMA * pr / rr)
    lo, hi = 1e-12, 10 * max(pl, pr)
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        lo, hi = (lo, mid) if _f_side(mid, rl, pl, al) + _f_side(mid, rr, pr, ar) + (ur - ul) > 0 else (mid, hi)
    ps = 0.5 * (lo + hi)
    return ps, 0.5 * (ul + ur) + 0.5 * (_f_side(ps, rr, pr, ar) - _f_side(ps, rl, pl, al))


def riemann_exact(left, right, s):
    """Exact solution (rho, u, p) of the Riemann problem at x/t = s (Toro, ch. 4)."""
    (rl, ul, pl), (rr, ur, pr) = left, right
    al, ar = math.sqrt(GAMMA * pl / rl), math.sqrt(GAMMA * pr / rr)
    ps, us = riemann_star(left, right)
    g1, g2 = (GAMMA - 1) / (GAMMA + 1), (GAMMA - 1) / (2 * GAMMA)
    if s <= us:
        if ps > pl:  # left shock
            S = ul - al * math.sqrt((GAMMA + 1) / (2 * GAMMA) * ps / pl + g2)
            return (rl, ul, pl) if s < S else (rl * (ps / pl + g1) / (g1 * ps / pl + 1), us, ps)
        if s < ul - al:
            return rl, ul, pl
        if s > us - al * (ps / pl) ** g2:
            return rl * (ps / pl) ** (1 / GAMMA), us, ps
        u = 2 / (GAMMA + 1) * (al + (GAMMA - 1) / 2 * ul + s)
        c = 2 / (GAMMA + 1) * (al + (GAMMA - 1) / 2 * (ul - s))
        return rl * (c / al) ** (2 / (GAMMA - 1)), u, pl * (c / al) ** (2 * GAMMA / (GAMMA - 1))
    if ps > pr:  # right shock
        S = ur + ar * math.sqrt((GAMMA + 1) / (2 * GAMMA) * ps / pr + g2)
        return (rr, ur, pr) if s > S else (rr * (ps / pr + g1) / (g1 * ps / pr + 1), us, ps)
    if s > ur + ar:
        return rr, ur, pr
    if s < us + ar * (ps / pr) ** g2:
        return rr * (ps / pr) ** (1 / GAMMA), us, ps
    u = 2 / (GAMMA + 1) * (-ar + (GAMMA - 1) / 2 * ur + s)
    c = 2 / (GAMMA + 1) * (ar - (GAMMA - 1) / 2 * (ur - s))
    return rr * (c / ar) ** (2 / (GAMMA - 1)), u, pr * (c / ar) ** (2 * GAMMA / (GAMMA - 1))


def sod(ni, tend=0.2, **kw):
    x = np.linspace(0.0, 1.0, ni + 1)
    X = np.repeat(x[:, None], 2, 1)
    Y = np.repeat(np.array([0.0, 1.0 / ni])[None, :], ni + 1, 0)
    g = grids.structured_2d(X, Y)
    b = {"west": grids.supersonic_outflow(), "east": grids.supersonic_outflow(),
         "south": grids.slip_wall(), "north": grids.slip_wall()}
    c = grids.make_config(2, b, gas=grids.ideal_gas(1.0),
                          solver=grids.runge_kutta(cfl=0.5, max_step=100000, max_time=tend), **kw)
    o = Oracle(c, g)
    xc = 0.5 * (x[1:] + x[:-1])
    rho, p = np.where(xc < 0.5, 1.0, 0.125), np.where(xc < 0.5, 1.0, 0.1)
    o.set_initial_condition(p / rho, p, np.zeros(ni), np.zeros(ni))  # R = 1: T = p / rho
    o.rk_initialise()
    t = 0.0
    for _ in range(1000):
        t = o.rk_steps(20)["t"]
        if t >= tend * (1 - 1e-12):
            break
    assert t == pytest.approx(tend, rel=1e-12) and o.count_bad_cells() == 0
    ex = np.array([riemann_exact((1.0, 0.0, 1.0), (0.125, 0.0, 0.1), (xx - 0.5) / t) for xx in xc])
    pr = o.primitives()[:, :o.N]  # rho, p, T, e, vx, vy, vz
    l1 = {q: float(np.mean(np.abs(pr[k] - ex[:, j]))) for q, k, j in (("rho", 0, 0), ("u", 4, 1), ("p", 1, 2))}
    star = (xc > 0.55) & (xc < 0.65)  # between the rarefaction's tail (0.486) and the contact (0.685)
    return l1, float(pr[1][star].mean()), float(pr[4][star].mean())


def test_sod_shock_tube_matches_the_exact_riemann_solution():
    ps, us = riemann_star((1.0, 0.0, 1.0), (0.125, 0.0, 0.1))
    assert ps == pytest.approx(0.30313, abs=1e-5) and us == pytest.approx(0.92745, abs=1e-5)
    coarse, _, _ = sod(200)
    fine, p_star, u_star = sod(400)
    for q in ("rho", "u", "p"):
        assert fine[q] <= 3e-3, fine
        assert fine[q] <= coarse[q] / 1.5, (q, coarse, fine)
    assert p_star == pytest.approx(ps, rel=2e-3) and u_star == pytest.approx(us, rel=2e-3)


@pytest.mark.parametrize("kw", [{"flux": "ausmdv"}, {"flux": "ldfss2"}, {"flux": "rusanov"}, {"thermo": "rho_p"},
                                {"thermo": "rho_T"}, {"thermo": "p_T"}],
                         ids=lambda kw: "-".join(f"{k}={v}" for k, v in kw.items()))
def test_sod_shock_tube_with_every_flux_and_thermo_pair(kw):
    """Every flux calculator and interpolated thermodynamic pair reproduces the exact
    Riemann solution (at 400 cells the L1 density errors are 1.3e-3, Rusanov, the
    most diffusive, 2.0e-3)."""
    l1, p_star, u_star = sod(400, **kw)
    assert l1["rho"] <= 2.5e-3 and l1["u"] <= 4e-3 and l1["p"] <= 1.6e-3, l1
    ps, us = riemann_star((1.0, 0.0, 1.0), (0.125, 0.0, 0.1))
    assert p_star == pytest.approx(ps, rel=5e-3) and u_star == pytest.approx(us, rel=5e-3)


def extruded_ramp(ni, nj, **kw):
    """The compression ramp as two layers of hexahedra (dz = 1/ni) between slip walls, run to steady state."""
    th = math.radians(15.0)
    g = grids.box_3d(ni, nj, 2, lx=1.0, ly=0.5, lz=2.0 / ni)
    x, y = g.xyz[:, 0], g.xyz[:, 1]
    yb = np.where(x > 0.2, (x - 0.2) * math.tan(th), 0.0)
    g.xyz[:, 1] = yb + (0.5 - yb) * (y / 0.5)
    gas = grids.ideal_gas(287.0)
    inf = grids.mach_state(gas, 2.0, 300.0, 101325.0)
    tmax = 3.0 / inf["vx"]
    b = {"west": grids.supersonic_inflow(inf), "east": grids.supersonic_outflow(), "south": grids.slip_wall(),
         "north": grids.slip_wall(), "bottom": grids.slip_wall(), "top": grids.slip_wall()}
    c = grids.make_config(3, b, gas=gas, solver=grids.runge_kutta(cfl=0.5, max_step=100000, max_time=tmax), **kw)
    o = Oracle(c, g)
    n = g.num_cells
    o.set_initial_condition(np.full(n, inf["T"]), np.full(n, inf["p"]), np.full(n, inf["vx"]), np.full(n, inf["vy"]),
                            np.zeros(n))
    o.rk_initialise()
    t = 0.0
    for _ in range(200):
        t = o.rk_steps(100)["t"]
        if t >= tmax * (1 - 1e-12):
            break
    assert t >= tmax * (1 - 1e-12) and o.count_bad_cells() == 0
    cen = o.geometry()["centroid"]
    return o.primitives()[:, :o.N], cen[0][:o.N], cen[1][:o.N], inf


def test_extruded_ramp_in_3d_matches_the_oblique_shock():
    pr, cx, cy, inf = extruded_ramp(64, 32)
    th = math.radians(15.0)
    b = weak_shock_angle(2.0, th, 1.4)
    p21 = 1 + 2 * 1.4 / 2.4 * ((2.0 * math.sin(b)) ** 2 - 1)
    sel = (cx >= 0.3) & (cx <= 0.55) & (cy >= (cx - 0.2) * math.tan(th) + 0.02) & (cy <= (cx - 0.2) * math.tan(b) - 0.04)
    assert sel.sum() > 200
    assert np.mean(np.abs(pr[1][sel] / (inf["p"] * p21) - 1)) <= 3e-3
    assert float(np.degrees(np.mean(np.arctan2(pr[5][sel], pr[4][sel])))) == pytest.approx(15.0, abs=0.05)
    assert np.abs(pr[6][sel]).max() <= 1e-3 * inf["vx"]  # the symmetry breaking stays at the shock


def test_extruded_ramp_keeps_z_symmetry_at_first_order():
    pr, _, _, inf = extruded_ramp(32, 16, order=1)
    assert np.abs(pr[6]).max() <= 1e-12 * inf["vx"]


def viscous_shock(cells_per_thickness_x40):
    """The Mach 2 normal shock on 40 exact shock thicknesses, run for one
    flow-through time from the Rankine-Hugoniot step; returns the largest
    velocity error within five thicknesses of the shock (a fraction of the
    jump), the shock position (a fraction of the domain) and the outflow
    temperature with its Rankine-Hugoniot value."""
    integrate = pytest.importorskip("scipy.integrate")
    R, g = 287.0, 1.4
    cp = g * R / (g - 1)
    mu0, T0, Ts = 1.716e-5, 273.0, 110.0
    mu = lambda T: mu0 * (T / T0) ** 1.5 * (T0 + Ts) / (T + Ts)  # noqa: E731  (Sutherland)
    M1, T1, p1 = 2.0, 300.0, 101325.0
    rho1 = p1 / (R * T1)
    u1 = M1 * math.sqrt(g * R * T1)
    p2 = p1 * (1 + 2 * g / (g + 1) * (M1 ** 2 - 1))
    r21 = (g + 1) * M1 ** 2 / ((g - 1) * M1 ** 2 + 2)
    u2, T2 = u1 / r21, p2 / (rho1 * r21 * R)
    m, h0 = rho1 * u1, cp * T1 + 0.5 * u1 ** 2
    Tu = lambda u: (h0 - 0.5 * u * u) / cp  # noqa: E731  (constant total enthalpy)

    def dudx(x, y):
        u = y[0]
        return [(m * (u - u1) + m * R * Tu(u) / u - p1) * 3.0 / (4.0 * mu(Tu(u)))]

    um = 0.5 * (u1 + u2)
    fw = integrate.solve_ivp(dudx, [0, 5e-6], [um], rtol=1e-10, atol=1e-12, dense_output=True, max_step=1e-9)
    bw = integrate.solve_ivp(dudx, [0, -5e-6], [um], rtol=1e-10, atol=1e-12, dense_output=True, max_step=1e-9)

    def u_exact(x):
        return np.where(x >= 0, fw.sol(np.clip(x, 0, 5e-6))[0], bw.sol(np.clip(x, -5e-6, 0))[0])

    xs = np.linspace(-1e-6, 1e-6, 2001)
    delta = (u1 - u2) / np.abs(np.gradient(u_exact(xs), xs)).max()  # maximum-slope thickness
    L, ni = 40 * delta, cells_per_thickness_x40
    x = np.linspace(0.0, L, ni + 1)
    X = np.repeat(x[:, None], 2, 1)
    Y = np.repeat(np.array([0.0, L / ni])[None, :], ni + 1, 0)
    gas = grids.ideal_gas(R)
    b = {"west": grids.supersonic_inflow(grids.flow_state(gas, T1, p1, u1, 0.0)), "east": grids.subsonic_outflow(p2),
         "south": grids.slip_wall(), "north": grids.slip_wall()}
    tmax = L / u2
    c = grids.make_config(2, b, gas=gas, viscous=True, Pr=0.75,
                          solver=grids.runge_kutta(cfl=0.5, max_step=10_000_000, max_time=tmax))
    o = Oracle(c, grids.structured_2d(X, Y))
    xc = 0.5 * (x[1:] + x[:-1])
    up = xc < 0.5 * L
    o.set_initial_condition(np.where(up, T1, T2), np.where(up, p1, p2), np.where(up, u1, u2), np.zeros(ni))
    o.rk_initialise()
    t = 0.0
    for _ in range(2000):
        t = o.rk_steps(200)["t"]
        if t >= tmax * (1 - 1e-12):
            break
    assert t >= tmax * (1 - 1e-12) and o.count_bad_cells() == 0
    pr = o.primitives()[:, :o.N]
    u = pr[4]
    k = int(np.argmax(u < um))
    xm = xc[k - 1] + (um - u[k - 1]) * (xc[k] - xc[k - 1]) / (u[k] - u[k - 1])
    inner = np.abs(xc - xm) < 5 * delta
    err = float(np.abs(u - u_exact(xc - xm))[inner].max() / (u1 - u2))
    return err, xm / L, float(pr[2][-1]), T2


def test_viscous_shock_structure_matches_the_navier_stokes_profile():
    coarse, _, _, _ = viscous_shock(120)
    fine, pos, T_out, T2 = viscous_shock(200)
    assert fine <= 6e-3, fine
    assert coarse / fine >= 2.0, (coarse, fine)  # about second order (3 -> 5 cells per thickness)
    assert abs(pos - 0.5) <= 0.01
    assert T_out == pytest.approx(T2, rel=1e-6)
