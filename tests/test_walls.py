"""Wall boundaries of the semi-Lagrangian streaming (SemiLagrangian.cpp:354-399).

Oracle known answers, restated from the reference's own tests
(boundaries/VelocityNeqBounceBack_SL_test.cpp, WallFixture.h, WallTestDomain2D.h):
[0, 1]^2, 2 x 2 cells, periodic in x, VelocityNeqBounceBack walls at y = 0 and
y = 1 moving with u = (0.01, 0), nu = 0.2, D2Q9, scaling 1, FE_Q:
  * p = 1, CFL 0.4, 10 steps from rest: the mean density stays 1 within 1e-10;
  * p = 2, CFL 1, 100 steps: |u - 0.01| <= 1e-3 and |v| <= 1e-5 at every node.
The boundary handler's hit counts on CouetteFlow2D
(boundaries/SemiLagrangianBoundaryHandler_test.cpp): 102 hits at dt = 0.001,
204 at dt = 0.1.
GPU parity (DG topology, through the C ABI): relative L2 <= 1e-12 per step in
FP64 and <= 1e-6 in FP32 deviation storage against the oracle's tracker.
"""
import math

import numpy as np
import pytest

import natrium_gb300 as N
import oracle as O
from tests.gpu_cases import rel_l2

UW = ((0, 0, 0), (0, 0, 0), (0.01, 0, 0), (0.01, 0, 0), (0, 0, 0), (0, 0, 0))


def _wall_domain(p, cfl, dg=False, bc=(0, 0, 1, 1, 0, 0), uw=UW, cells=(2, 2), nu=0.2, scaling=1.0):
    st = O.stencil("D2Q9", scaling)
    m = O.Mesh(2, cells, p, dg, (1.0, 1.0), bc=bc, uw=uw)
    dt = O.time_step(m.h_min(), p, st.max_speed, cfl)
    tau = nu / (dt * st.cs2) + 0.5
    return st, m, dt, tau


def test_bounce_back_mass_conservation_known_answer():
    st, m, dt, tau = _wall_domain(1, 0.4)
    S = O.SLOperator(m, st, dt)
    f = np.ascontiguousarray(np.repeat(st.w[:, None], m.n_nodes, axis=1))
    rho, u = S.step_bgk(f, tau, 10)
    assert S.wall_hits > 0
    assert abs(rho.mean() - 1.0) < 1e-10


def test_bounce_back_wall_velocity_known_answer():
    st, m, dt, tau = _wall_domain(2, 1.0)
    S = O.SLOperator(m, st, dt)
    f = np.ascontiguousarray(np.repeat(st.w[:, None], m.n_nodes, axis=1))
    rho, u = S.step_bgk(f, tau, 100)
    assert np.abs(u[0] - 0.01).max() <= 1e-3
    assert np.abs(u[1]).max() <= 1e-5


@pytest.mark.parametrize("dt,layers", [(0.001, 1), (0.1, 2)])
def test_wall_hit_counts_known_answer(dt, layers):
    """SemiLagrangianBoundaryHandler_DataStructures_test / _offSupportHits_test
    (boundaries/SemiLagrangianBoundaryHandler_test.cpp:98-176): CouetteFlow2D on
    [0, 1]^2, refinement 3 (8 x 8 cells), FE_Q p = 2, D2Q9, walls at y = 0 and
    y = 1, periodic x.  A small step hits the walls from the support points on
    them only: (2^3 * 2 * 2 + 2) points x 3 directions = 102 hits; dt = 0.1
    reaches the second node layer: twice that."""
    st = O.stencil("D2Q9", 1.0)
    uw = ((0, 0, 0), (0, 0, 0), (0, 0, 0), (0.1, 0, 0), (0, 0, 0), (0, 0, 0))
    m = O.Mesh(2, (8, 8), 2, False, (1.0, 1.0), bc=(0, 0, 1, 1, 0, 0), uw=uw)
    S = O.SLOperator(m, st, dt)
    n_points = 2 ** 3 * 2 * 2 + 2
    assert S.wall_hits == layers * n_points * 3


def test_bounce_back_rows_reverse_the_population():
    st, m, dt, tau = _wall_domain(2, 0.4, dg=True)
    S = O.SLOperator(m, st, dt)
    # direction 2 (0, 1): departure below y = 0 for the bottom nodes -> taken
    # from direction 4 (0, -1), with the wall term 2 w e.u / cs2 = 0 here
    d = S.csr_dirs(2)
    assert set(np.unique(d)) == {2, 4}
    # direction 5 (1, 1): wall term 2 w_5 (1 * 0.01) / (1/3) on the reversed rows
    b = S.bconst(5)
    assert np.isclose(b.max(), 2 * st.w[5] * 0.01 / st.cs2)


def test_do_nothing_keeps_a_uniform_flow():
    st, m, dt, tau = _wall_domain(2, 0.4, dg=True, bc=(0, 0, 2, 2, 0, 0), uw=((0, 0, 0),) * 6, nu=0.01)
    S = O.SLOperator(m, st, dt)
    n = m.n_nodes
    rho = np.full(n, 1.0)
    u = np.stack([np.full(n, 0.02), np.full(n, 0.01)])
    f = O.equilibrium(st, rho, u)
    f0 = f.copy()
    r, uu = S.step_bgk(f, tau, 5)
    assert S.wall_hits > 0
    assert np.abs(f - f0).max() < 1e-14


# ---------------------------------------------------------------------------
# GPU parity (DG)
# ---------------------------------------------------------------------------

def _dg_wall_case(stencil, cells, p, bc, uw, model="BGK_STANDARD", precision="fp64", Ma=0.1, nu=2e-3):
    st = O.stencil(stencil, math.sqrt(3) / Ma)
    dim = st.D
    L = (1.0, 1.0, 1.0)
    m = O.Mesh(dim, tuple(cells), p, True, L, bc=bc, uw=uw)
    dt = O.time_step(m.h_min(), p, st.max_speed, 0.4)
    tau = nu / (dt * st.cs2) + 0.5
    periodic = tuple(bc[2 * a] == 0 for a in range(3))
    spec = N.SolverSpec(stencil=stencil, order=p, cells=tuple(cells), length=L, scaling=st.scaling, viscosity=nu,
                        dt=dt, collision=model, precision=precision, topology="dg", periodic=periodic)
    return st, m, dt, tau, spec


def _smooth_state(m, st, seed):
    X = m.coords()
    rng = np.random.default_rng(seed)
    k = 2 * math.pi
    rho = 1.0 + 0.02 * np.sin(k * X[:, 0]) * np.cos(k * X[:, 1] + 0.3)
    u = 0.03 * np.stack([np.cos(k * X[:, 1]), np.sin(k * X[:, 0] + 0.2)] + ([0.5 * np.sin(k * X[:, 2])]
                                                                                if st.D == 3 else []))
    f = O.equilibrium(st, rho, u * st.scaling)
    return np.ascontiguousarray(f * (1.0 + 1e-3 * rng.standard_normal(f.shape)))


def _set_walls(sol, bc, uw, scaling):
    for face in range(6):
        if bc[face] == 1:
            sol.set_boundary(face, "VELOCITY_BOUNCE_BACK", np.asarray(uw[face]) * 1.0)
        elif bc[face] == 2:
            sol.set_boundary(face, "DO_NOTHING")


WALL_CASES = [
    ("D2Q9", (4, 3), 3, (0, 0, 1, 1, 0, 0), "moving walls y"),
    ("D2Q9", (3, 4), 2, (1, 1, 2, 2, 0, 0), "walls x, do-nothing y"),
    ("D2Q9", (3, 3), 4, (2, 2, 0, 0, 0, 0), "do-nothing x"),
    ("D3Q19", (2, 2, 3), 2, (0, 0, 0, 0, 1, 1), "walls z"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
@pytest.mark.parametrize("case", WALL_CASES, ids=[c[4] for c in WALL_CASES])
def test_walls_match_oracle(gpu_lib, case, precision):
    stencil, cells, p, bc, _ = case
    scaling = math.sqrt(3) / 0.1
    uw = tuple((0.05 * scaling * (1 if f % 2 else -1), 0.02 * scaling, 0.0) if bc[f] == 1 else (0, 0, 0)
               for f in range(6))
    st, m, dt, tau, spec = _dg_wall_case(stencil, cells, p, bc, uw, precision=precision)
    f0 = _smooth_state(m, st, seed=3)
    S = O.SLOperator(m, st, dt)
    f1 = f0.copy()
    rho1, u1 = S.step_bgk(f1, tau, 3)
    with N.Solver(spec) as sol:
        _set_walls(sol, bc, uw, scaling)
        sol.upload_f(f0)
        sol.step(3)
        f = sol.download_f()
        rho, u = sol.download_macro()
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert rel_l2(f, f1) <= tol
    assert rel_l2(rho, rho1) <= tol
    assert rel_l2(u, u1) <= (1e-11 if precision == "fp64" else 1e-5)


@pytest.mark.gpu
def test_wall_stream_only_matches_oracle(gpu_lib):
    bc = (0, 0, 1, 1, 0, 0)
    scaling = math.sqrt(3) / 0.1
    uw = ((0, 0, 0), (0, 0, 0), (0.05 * scaling, 0, 0), (-0.03 * scaling, 0, 0), (0, 0, 0), (0, 0, 0))
    st, m, dt, tau, spec = _dg_wall_case("D2Q9", (3, 3), 3, bc, uw)
    f0 = _smooth_state(m, st, seed=5)
    S = O.SLOperator(m, st, dt)
    fo = S.stream(f0)
    with N.Solver(spec) as sol:
        _set_walls(sol, bc, uw, scaling)
        sol.upload_f(f0)
        sol.stream()
        f = sol.download_f()
    assert rel_l2(f, fo) <= 1e-12


@pytest.mark.gpu
def test_walls_compressible_model_matches_oracle(gpu_lib):
    bc = (0, 0, 1, 1, 0, 0)
    uw = ((0, 0, 0), (0, 0, 0), (0.05, 0, 0), (-0.05, 0, 0), (0, 0, 0), (0, 0, 0))
    st = O.stencil("D2Q25H", 1.0)
    m = O.Mesh(2, (4, 3), 2, True, (1.0, 1.0), bc=bc, uw=uw)
    dt = O.time_step(m.h_min(), 2, st.max_speed, 0.4)
    nu = 1e-3
    tau = nu / (dt * st.cs2) + 0.5
    from tests.gpu_cases import thermal_state
    rho0, u0, T0, f0, g0 = thermal_state(m, st, seed=4)
    S = O.SLOperator(m, st, dt)
    f1, g1 = f0.copy(), g0.copy()
    r1, u1, T1, m1 = S.step_compressible(f1, g1, tau, nsteps=2)
    spec = N.SolverSpec(stencil="D2Q25H", order=2, cells=(4, 3), length=(1.0, 1.0), scaling=1.0, viscosity=nu, dt=dt,
                        collision="BGK_COMPRESSIBLE", precision="fp64", topology="dg", periodic=(True, False, True))
    with N.Solver(spec) as sol:
        _set_walls(sol, bc, uw, 1.0)
        sol.upload_f(f0)
        sol.upload_g(g0)
        sol.step(2)
        f, g = sol.download_f(), sol.download_g()
        T, _ = sol.download_thermal()
    assert rel_l2(f, f1) <= 1e-12
    assert rel_l2(g, g1) <= 1e-12
    assert rel_l2(T, T1) <= 1e-12


THERMAL_WALL_FORMS = [("fp64", 0), ("fp32dev", 0), ("fp32dev", 1), ("fp32dev", 2), ("fp32dev", 3)]


@pytest.mark.gpu
@pytest.mark.parametrize("bc", [(0, 0, 1, 1, 0, 0), (2, 2, 2, 2, 0, 0)], ids=["moving walls y", "do-nothing all"])
@pytest.mark.parametrize("precision,form", THERMAL_WALL_FORMS,
                         ids=["fp64", "fp32-registers", "fp32-smem-20-warps", "fp32-smem-24-warps", "fp32-staged"])
def test_walls_compressible_model_fused_forms(gpu_lib, bc, precision, form):
    """The step kernel collides the wall nodes of the two-population model
    after their sparse rows: 36 nodes along x (two 32-node row segments, the
    second partial) so the per-segment wall words of both segments are used,
    in every kernel form."""
    uw = ((0, 0, 0), (0, 0, 0), (0.05, 0, 0), (-0.05, 0, 0), (0, 0, 0), (0, 0, 0))
    st = O.stencil("D2Q25H", 1.0)
    m = O.Mesh(2, (12, 4), 2, True, (1.0, 1.0), bc=bc, uw=uw)
    dt = O.time_step(m.h_min(), 2, st.max_speed, 0.4)
    nu = 1e-3
    tau = nu / (dt * st.cs2) + 0.5
    from tests.gpu_cases import thermal_state
    rho0, u0, T0, f0, g0 = thermal_state(m, st, seed=6)
    S = O.SLOperator(m, st, dt)
    f1, g1 = f0.copy(), g0.copy()
    r1, u1, T1, m1 = S.step_compressible(f1, g1, tau, nsteps=3)
    periodic = (bc[0] == 0, False, True)
    spec = N.SolverSpec(stencil="D2Q25H", order=2, cells=(12, 4), length=(1.0, 1.0), scaling=1.0, viscosity=nu,
                        dt=dt, collision="BGK_COMPRESSIBLE", precision=precision, topology="dg", periodic=periodic)
    with N.Solver(spec) as sol:
        _set_walls(sol, bc, uw, 1.0)
        if precision == "fp32dev":
            sol.select_candidate(form)
        sol.upload_f(f0)
        sol.upload_g(g0)
        sol.step(3)
        f, g = sol.download_f(), sol.download_g()
        T, _ = sol.download_thermal()
        r, _ = sol.download_macro()
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert rel_l2(f, f1) <= tol
    assert rel_l2(g, g1) <= tol
    assert rel_l2(T, T1) <= tol
    assert rel_l2(r, r1) <= tol


@pytest.mark.gpu
def test_walls_compressible_stream_only_matches_oracle(gpu_lib):
    """nat_stream on a two-population handle with walls: the lattice streamed
    without collision, then the wall nodes' rows overwrite f (with the wall
    terms) and g (without them)."""
    bc = (0, 0, 1, 1, 0, 0)
    uw = ((0, 0, 0), (0, 0, 0), (0.05, 0, 0), (-0.05, 0, 0), (0, 0, 0), (0, 0, 0))
    st = O.stencil("D2Q25H", 1.0)
    m = O.Mesh(2, (12, 4), 2, True, (1.0, 1.0), bc=bc, uw=uw)
    dt = O.time_step(m.h_min(), 2, st.max_speed, 0.4)
    from tests.gpu_cases import thermal_state
    rho0, u0, T0, f0, g0 = thermal_state(m, st, seed=8)
    S = O.SLOperator(m, st, dt)
    fo, go = S.stream(f0), S.stream_g(g0)
    spec = N.SolverSpec(stencil="D2Q25H", order=2, cells=(12, 4), length=(1.0, 1.0), scaling=1.0, viscosity=1e-3,
                        dt=dt, collision="BGK_COMPRESSIBLE", precision="fp64", topology="dg",
                        periodic=(True, False, True))
    with N.Solver(spec) as sol:
        _set_walls(sol, bc, uw, 1.0)
        sol.upload_f(f0)
        sol.upload_g(g0)
        sol.stream()
        f, g = sol.download_f(), sol.download_g()
    assert rel_l2(f, fo) <= 1e-12
    assert rel_l2(g, go) <= 1e-12
    assert rel_l2(g, S.stream(g0)) > 1e-9  # the wall terms would have changed g


def test_walls_need_dg_topology():
    spec = N.SolverSpec(stencil="D2Q9", order=2, cells=(2, 2), length=(1, 1), scaling=1.0, viscosity=0.1,
                        topology="feq", periodic=(True, False, True))
    with pytest.raises(N.NatError) as ei:
        N.Solver(spec)
    assert ei.value.code == N.NAT_ERR_UNSUPPORTED
