"""MappingQ1 cells: the semi-Lagrangian operator on deformed (non-Cartesian) grids.

The reference streams with MappingQ1 whenever the problem is not Cartesian
(advection/AdvectionOperator.cpp:59-63): faceCrossedFirst works on the
inverse-mapped points (SemiLagrangian.cpp:525-699), the shape values come
from the inverse map of the departure point (SemiLagrangianTools.cpp:15-64),
periodic faces translate by the offset between the faces' vertices
(PeriodicBoundary.cpp:184-270).  Its non-Cartesian benchmark is the
LubricationSine channel (benchmarks/LubricationSine.cpp).

Oracle properties (no reference golden vectors exist for deformed grids):
  * a vertex grid equal to the box gives the Cartesian operator (1e-14);
  * constant streaming A 1 = 1 on deformed periodic grids and in the
    LubricationSine channel with bounce-back walls at rest;
  * a linear field is streamed exactly on a deformed grid (Q_p on a
    multilinear cell contains the linear functions), away from the periodic
    seam.
GPU parity through the C ABI: relative L2 <= 1e-12 in FP64 and <= 1e-6 in
FP32 deviation storage against the oracle, for periodic deformed grids
(FE_Q and DG, 2-D and 3-D, BGK and KBC), the LubricationSine channel with a
moving wall, stream-only, and the compressible two-population model.
"""
import dataclasses
import math

import numpy as np
import pytest

import natrium_gb300 as N
import oracle as O
from natrium_gb300 import problems as P
from tests.gpu_cases import rel_l2


def _box_grid(cells, L):
    axes = [np.linspace(0.0, L[a], cells[a] + 1) for a in range(len(cells))]
    return np.stack(np.meshgrid(*axes, indexing="ij"), -1)


@pytest.mark.parametrize("D,cells,p,dg,stencil", [
    (2, (3, 4), 2, True, "D2Q9"), (2, (3, 3), 3, False, "D2Q9"), (3, (2, 3, 2), 2, True, "D3Q19"),
    (3, (2, 2, 2), 2, False, "D3Q27")])
def test_box_vertices_give_the_cartesian_operator(D, cells, p, dg, stencil):
    L = (1.0, 1.5, 1.2)[:D]
    st = O.stencil(stencil, 1.0)
    m0 = O.Mesh(D, cells, p, dg, L)
    m1 = O.Mesh(D, cells, p, dg, L, vertices=_box_grid(cells, L))
    assert m1.h_min() == pytest.approx(m0.h_min(), rel=1e-15)
    dt = O.time_step(m0.h_min(), p, st.max_speed, 0.4)
    a, b = O.SLOperator(m0, st, dt), O.SLOperator(m1, st, dt)
    f = np.random.default_rng(0).random((st.Q, m0.n_nodes))
    assert np.abs(a.stream(f) - b.stream(f)).max() < 1e-14
    assert np.abs(m0.coords() - m1.coords()).max() < 1e-15


WAVY = [(2, (4, 5), 1, True, "D2Q9"), (2, (4, 4), 2, False, "D2Q9"), (2, (5, 4), 3, True, "D2Q9"),
        (3, (3, 3, 3), 2, True, "D3Q19"), (3, (3, 3, 3), 2, False, "D3Q27")]


@pytest.mark.parametrize("D,cells,p,dg,stencil", WAVY)
def test_deformed_grid_constant_and_linear_fields(D, cells, p, dg, stencil):
    L = (1.0, 1.3, 0.9)[:D]
    V = P.wavy_grid(cells, L, 0.12 if D == 2 else 0.05)
    m = O.Mesh(D, cells, p, dg, L, vertices=V)
    st = O.stencil(stencil, 1.0)
    dt = O.time_step(m.h_min(), p, st.max_speed, 0.8)
    S = O.SLOperator(m, st, dt)
    assert np.abs(S.stream(np.ones((st.Q, m.n_nodes))) - 1.0).max() < 1e-14
    X = m.coords()
    assert np.abs(X - P.mapped_node_coords(V, p, "dg" if dg else "feq")).max() < 1e-15
    lin = X[:, 0] + 2 * X[:, 1]
    out = S.stream(np.tile(lin, (st.Q, 1)))
    ex = lin[None, :] - dt * (st.e[:, 0][:, None] + 2 * st.e[:, 1][:, None])
    inner = (X[:, 0] > 0.2) & (X[:, 0] < 0.8) & (X[:, 1] > 0.2) & (X[:, 1] < 1.0)
    assert np.abs(out - ex)[:, inner].max() < 1e-13


@pytest.mark.parametrize("p", [1, 2, 3])
def test_lubrication_sine_channel_constant_streaming(p):
    V = P.lubrication_sine_grid(refinement=1)
    cells = tuple(s - 1 for s in V.shape[:2])
    st = O.stencil("D2Q9", 1.0)
    m = O.Mesh(2, cells, p, True, (1.0, 0.25), bc=(0, 0, 1, 1, 0, 0), uw=((0, 0, 0),) * 6, vertices=V)
    dt = O.time_step(m.h_min(), p, st.max_speed, 0.4)
    S = O.SLOperator(m, st, dt)
    assert np.abs(S.stream(np.ones((9, m.n_nodes))) - 1.0).max() < 1e-14
    assert S.wall_hits > 0


@pytest.mark.parametrize("p", [2, 3])
def test_sinusoidal_shear_gap_constant_streaming(p):
    V = P.sinusoidal_shear_grid(refinement=2)
    cells = tuple(s - 1 for s in V.shape[:2])
    assert np.abs(V[-1, :, 0] - V[0, :, 0] - 1.0).max() < 1e-12  # one translation along x
    st = O.stencil("D2Q9", 1.0)
    m = O.Mesh(2, cells, p, True, (1.0, 1.0), bc=(0, 0, 1, 1, 0, 0), uw=((0, 0, 0),) * 6, vertices=V)
    dt = O.time_step(m.h_min(), p, st.max_speed, 0.4)
    S = O.SLOperator(m, st, dt)
    assert np.abs(S.stream(np.ones((9, m.n_nodes))) - 1.0).max() < 1e-14
    assert S.wall_hits > 0


def test_periodic_axis_needs_one_translation():
    V = P.wavy_grid((3, 3), (1.0, 1.0), 0.1)
    V[-1, 1, 1] += 0.01  # x+ face no longer a translate of the x- face
    m = O.Mesh(2, (3, 3), 2, True, (1.0, 1.0), vertices=V)
    st = O.stencil("D2Q9", 1.0)
    with pytest.raises(RuntimeError):
        O.SLOperator(m, st, 0.01)


def test_spec_vertex_layout():
    V = P.wavy_grid((3, 2), (1.0, 1.0), 0.1)
    spec = N.SolverSpec(stencil="D2Q9", order=2, cells=(3, 2), length=(1.0, 1.0), vertices=V)
    flat = spec.vertex_array()
    assert flat.shape == (4 * 3, 3)
    assert np.array_equal(flat[1 * 4 + 2, :2], V[2, 1])  # x fastest
    with pytest.raises(ValueError):
        N.SolverSpec(stencil="D2Q9", order=2, cells=(3, 3), vertices=V).vertex_array()


# ---------------------------------------------------------------------------
# GPU parity
# ---------------------------------------------------------------------------

def _mapped_case(stencil, cells, p, dg, V, model="BGK_STANDARD", precision="fp64", Ma=0.1, nu=2e-3, bc=None,
                 uw=None, cfl=0.4):
    st = O.stencil(stencil, math.sqrt(3) / Ma)
    D = st.D
    bc = bc or (0,) * 6
    uw = uw or ((0, 0, 0),) * 6
    L = tuple(float(V[..., a].max() - V[..., a].min()) for a in range(D)) + (1.0,) * (3 - D)
    m = O.Mesh(D, tuple(cells), p, dg, L, bc=bc, uw=uw, vertices=V)
    dt = O.time_step(m.h_min(), p, st.max_speed, cfl)
    tau = nu / (dt * st.cs2) + 0.5
    periodic = tuple(bc[2 * a] == 0 for a in range(3))
    spec = N.SolverSpec(stencil=stencil, order=p, cells=tuple(cells), length=L, scaling=st.scaling, viscosity=nu,
                        dt=dt, collision=model, precision=precision, topology="dg" if dg else "feq",
                        periodic=periodic, vertices=V)
    return st, m, dt, tau, spec


def _state(m, st, seed):
    X = m.coords()
    rng = np.random.default_rng(seed)
    k = 2 * math.pi
    rho = 1.0 + 0.02 * np.sin(k * X[:, 0]) * np.cos(k * X[:, 1] + 0.3)
    u = 0.03 * np.stack([np.cos(k * X[:, 1]), np.sin(k * X[:, 0] + 0.2)] + ([0.5 * np.sin(k * X[:, 2])]
                                                                                if st.D == 3 else []))
    f = O.equilibrium(st, rho, u * st.scaling)
    f = f * (1.0 + 1e-3 * rng.standard_normal(f.shape))
    if not m.dg:  # FE_Q: equal values on the periodic duplicates
        shape = [m.nodes_per_axis(a) for a in range(st.D)][::-1]
        v = f.reshape((st.Q,) + tuple(shape))
        for a in range(st.D):
            ax = st.D - a  # numpy axis of lattice axis a
            sl_last = [slice(None)] * v.ndim
            sl_first = [slice(None)] * v.ndim
            sl_last[ax], sl_first[ax] = -1, 0
            v[tuple(sl_last)] = v[tuple(sl_first)]
    return np.ascontiguousarray(f)


MAPPED_CASES = [
    ("D2Q9", (4, 5), 2, True, "BGK_STANDARD", "d2q9 p2 dg"),
    ("D2Q9", (4, 4), 3, False, "BGK_STANDARD", "d2q9 p3 feq"),
    ("D2Q9", (5, 4), 4, True, "KBC_STANDARD", "d2q9 p4 dg kbc"),
    ("D3Q19", (3, 3, 3), 2, True, "BGK_STANDARD", "d3q19 p2 dg"),
    ("D3Q27", (3, 3, 3), 2, False, "KBC_STANDARD", "d3q27 p2 feq kbc"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
@pytest.mark.parametrize("case", MAPPED_CASES, ids=[c[5] for c in MAPPED_CASES])
def test_mapped_step_matches_oracle(gpu_lib, case, precision):
    stencil, cells, p, dg, model, _ = case
    D = len(cells)
    V = P.wavy_grid(cells, (1.0, 1.3, 0.9)[:D], 0.12 if D == 2 else 0.05)
    st, m, dt, tau, spec = _mapped_case(stencil, cells, p, dg, V, model=model, precision=precision)
    f0 = _state(m, st, seed=7)
    S = O.SLOperator(m, st, dt)
    f1 = f0.copy()
    rho1, u1 = np.zeros(m.n_nodes), np.zeros((D, m.n_nodes))
    for _ in range(3):
        f1 = S.stream(f1)
        O.collide(st, model, tau, f1, rho1, u1)
    with N.Solver(spec) as sol:
        assert sol.kernel_variant == 8
        sol.upload_f(f0)
        sol.step(3)
        f = sol.download_f()
        rho, u = sol.download_macro()
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert rel_l2(f, f1) <= tol
    assert rel_l2(rho, rho1) <= tol
    assert rel_l2(u, u1) <= (1e-11 if precision == "fp64" else 1e-5)


@pytest.mark.gpu
def test_mapped_stream_only_matches_oracle(gpu_lib):
    V = P.wavy_grid((4, 4), (1.0, 1.0), 0.12)
    st, m, dt, tau, spec = _mapped_case("D2Q9", (4, 4), 3, True, V)
    f0 = _state(m, st, seed=2)
    fo = O.SLOperator(m, st, dt).stream(f0)
    with N.Solver(spec) as sol:
        sol.upload_f(f0)
        sol.stream()
        f = sol.download_f()
    assert rel_l2(f, fo) <= 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
def test_lubrication_sine_channel_matches_oracle(gpu_lib, precision):
    V = P.lubrication_sine_grid(refinement=1)
    cells = tuple(s - 1 for s in V.shape[:2])
    scaling = math.sqrt(3) / 0.1
    U = 0.05 * scaling
    bc = (0, 0, 1, 1, 0, 0)
    uw = ((0, 0, 0), (0, 0, 0), (U, 0, 0), (0, 0, 0), (0, 0, 0), (0, 0, 0))
    st, m, dt, tau, spec = _mapped_case("D2Q9", cells, 2, True, V, precision=precision, bc=bc, uw=uw, nu=0.01)
    X = m.coords()
    u0 = P.lubrication_sine_velocity(X, U, 0.25, 0.05)
    f0 = O.equilibrium(st, np.ones(m.n_nodes), u0)
    S = O.SLOperator(m, st, dt)
    f1 = f0.copy()
    rho1, u1 = S.step_bgk(f1, tau, 4)
    with N.Solver(spec) as sol:
        sol.set_boundary(2, "VELOCITY_BOUNCE_BACK", np.array([U, 0.0, 0.0]))
        sol.upload_f(f0)
        sol.step(4)
        f = sol.download_f()
        rho, u = sol.download_macro()
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert rel_l2(f, f1) <= tol
    assert rel_l2(u, u1) <= (1e-11 if precision == "fp64" else 1e-5)


@pytest.mark.gpu
def test_sinusoidal_shear_gap_matches_oracle(gpu_lib):
    V = P.sinusoidal_shear_grid(refinement=2)
    cells = tuple(s - 1 for s in V.shape[:2])
    scaling = math.sqrt(3) / 0.1
    U = 0.05 * scaling
    bc = (0, 0, 1, 1, 0, 0)
    uw = ((0, 0, 0), (0, 0, 0), (U, 0, 0), (0, 0, 0), (0, 0, 0), (0, 0, 0))
    st, m, dt, tau, spec = _mapped_case("D2Q9", cells, 3, True, V, bc=bc, uw=uw, nu=0.01, model="KBC_STANDARD")
    f0 = _state(m, st, seed=11)
    S = O.SLOperator(m, st, dt)
    f1 = f0.copy()
    rho1, u1 = np.zeros(m.n_nodes), np.zeros((2, m.n_nodes))
    for _ in range(3):
        f1 = S.stream(f1)
        O.collide(st, "KBC_STANDARD", tau, f1, rho1, u1)
    with N.Solver(spec) as sol:
        sol.set_boundary(2, "VELOCITY_BOUNCE_BACK", np.array([U, 0.0, 0.0]))
        sol.upload_f(f0)
        sol.step(3)
        f = sol.download_f()
    assert rel_l2(f, f1) <= 1e-12


@pytest.mark.gpu
def test_mapped_box_equals_cartesian_solver(gpu_lib):
    """The same box given as vertices runs the sparse departure-point path and
    must agree with the Cartesian fused kernel."""
    cells, L = (4, 4), (1.0, 1.0)
    st, m, dt, tau, spec = _mapped_case("D2Q9", cells, 3, True, _box_grid(cells, L))
    f0 = _state(m, st, seed=9)
    spec_c = dataclasses.replace(spec, vertices=None)
    out = []
    for sp in (spec, spec_c):
        with N.Solver(sp) as sol:
            sol.upload_f(f0)
            sol.step(3)
            out.append(sol.download_f())
    assert rel_l2(out[0], out[1]) <= 1e-12


@pytest.mark.gpu
def test_mapped_mass_uses_the_cell_jacobians(gpu_lib):
    V = P.wavy_grid((4, 4), (1.0, 1.0), 0.12)
    st, m, dt, tau, spec = _mapped_case("D2Q9", (4, 4), 2, True, V)
    n = m.n_nodes
    f0 = O.equilibrium(st, np.full(n, 1.5), np.zeros((2, n)))
    with N.Solver(spec) as sol:
        sol.upload_f(f0)
        sol.collide()
        mass, ke = sol.mass_energy()
    # the deformed grid still covers the unit square: mass = 1.5 * area
    assert mass == pytest.approx(1.5, rel=1e-12)
    assert abs(ke) < 1e-20


@pytest.mark.gpu
def test_mapped_compressible_model_matches_oracle(gpu_lib):
    V = P.wavy_grid((4, 4), (1.0, 1.0), 0.1)
    st = O.stencil("D2Q25H", 1.0)
    m = O.Mesh(2, (4, 4), 2, True, (1.0, 1.0), vertices=V)
    dt = O.time_step(m.h_min(), 2, st.max_speed, 0.4)
    nu = 1e-3
    tau = nu / (dt * st.cs2) + 0.5
    from tests.gpu_cases import thermal_state
    rho0, u0, T0, f0, g0 = thermal_state(m, st, seed=4)
    S = O.SLOperator(m, st, dt)
    f1, g1 = f0.copy(), g0.copy()
    r1, u1, T1, m1 = S.step_compressible(f1, g1, tau, nsteps=2)
    spec = N.SolverSpec(stencil="D2Q25H", order=2, cells=(4, 4), length=(1.0, 1.0), scaling=1.0, viscosity=nu, dt=dt,
                        collision="BGK_COMPRESSIBLE", precision="fp64", topology="dg", vertices=V)
    with N.Solver(spec) as sol:
        sol.upload_f(f0)
        sol.upload_g(g0)
        sol.step(2)
        f, g = sol.download_f(), sol.download_g()
        T, _ = sol.download_thermal()
    assert rel_l2(f, f1) <= 1e-12
    assert rel_l2(g, g1) <= 1e-12
    assert rel_l2(T, T1) <= 1e-12


@pytest.mark.gpu
def test_mapped_grid_errors(gpu_lib):
    V = P.wavy_grid((3, 3), (1.0, 1.0), 0.1)
    bad = V.copy()
    bad[-1, 1, 1] += 0.01
    spec = N.SolverSpec(stencil="D2Q9", order=2, cells=(3, 3), length=(1.0, 1.0), topology="dg", vertices=bad)
    with pytest.raises(N.NatError) as ei:
        N.Solver(spec)
    assert ei.value.code == N.NAT_ERR_INVALID_ARG
    flip = V.copy()
    flip[1, 1], flip[2, 1] = V[2, 1].copy(), V[1, 1].copy()  # two vertices swapped: inverted cells
    spec = N.SolverSpec(stencil="D2Q9", order=2, cells=(3, 3), length=(1.0, 1.0), topology="dg", vertices=flip)
    with pytest.raises(N.NatError) as ei:
        N.Solver(spec)
    assert ei.value.code == N.NAT_ERR_INVALID_ARG


TRACK_CASES = [
    (2, (4, 5), 2, True, "D2Q9", "BGK_STANDARD", "fp32dev"),
    (2, (4, 4), 3, False, "D2Q9", "KBC_STANDARD", "fp64"),
    (2, (5, 4), 4, True, "D2Q9", "BGK_STANDARD", "fp64"),
    (3, (3, 3, 3), 2, True, "D3Q19", "BGK_STANDARD", "fp32dev"),
    (3, (3, 3, 3), 2, False, "D3Q27", "KBC_STANDARD", "fp64"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("D,cells,p,dg,stencil,model,precision", TRACK_CASES)
def test_device_departure_search_equals_host_bitwise(gpu_lib, D, cells, p, dg, stencil, model, precision):
    """The departure-point search and the Newton inverse of MappingQ1
    (SemiLagrangian.cpp:525-757, SemiLagrangianTools.cpp:15-64) run on the
    device (one thread per row, the rows nat_create uses) and on the host
    tracker: every row is the same, bit for bit."""
    L = (1.0, 1.0, 1.0)[:D]
    V = P.wavy_grid(cells, L, 0.12 if D == 2 else 0.05)
    st = O.stencil(stencil, math.sqrt(3) / 0.1)
    m = O.Mesh(D, cells, p, dg, L, vertices=V)
    dt = O.time_step(m.h_min(), p, st.max_speed, 0.4)
    spec = N.SolverSpec(stencil=stencil, order=p, cells=cells, length=L, scaling=st.scaling, viscosity=2e-3,
                        dt=dt, collision=model, precision=precision, topology="dg" if dg else "feq", vertices=V)
    with N.Solver(spec) as sol:
        host = sol.mapped_rows("host")
        dev = sol.mapped_rows("device")
    for h, d in zip(host, dev):
        assert h.dtype == d.dtype and h.shape == d.shape
        assert np.array_equal(h.view(np.uint8), d.view(np.uint8))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32dev", "fp64"])
def test_device_departure_search_equals_host_in_the_lubrication_channel(gpu_lib, precision):
    """The same in the LubricationSine channel: bounce-back walls (one moving)
    and the wavy top wall, where paths hit walls."""
    V = P.lubrication_sine_grid(refinement=2)
    cells = tuple(s - 1 for s in V.shape[:2])
    scaling = math.sqrt(3) / 0.1
    spec = N.SolverSpec(stencil="D2Q9", order=3, cells=cells, length=(1.0, 0.25), scaling=scaling, viscosity=1e-3,
                        cfl=0.4, collision="BGK_STANDARD", precision=precision, topology="dg",
                        periodic=(True, False, True), vertices=V)
    with N.Solver(spec) as sol:
        sol.set_boundary(2, "VELOCITY_BOUNCE_BACK", np.array([0.05 * scaling, 0.0, 0.0]))
        host = sol.mapped_rows("host")
        dev = sol.mapped_rows("device")
    for h, d in zip(host, dev):
        assert np.array_equal(h.view(np.uint8), d.view(np.uint8))
