"""Constant body force in the BGK collision (the advanced collision of the
time loop: collision_advanced/CollisionOperator.h:76-90 and
AuxiliaryCollisionFunctions.h:332-414, schemes SHIFTING_VELOCITY and
EXACT_DIFFERENCE; the legacy BGKStandard::collideAll's GUO scheme,
collision/BGKStandard.cpp:222-225 and 470-473 with
ExternalForceFunctions.h:119-200 and 385-520).

Oracle properties: a collision adds exactly dt F / scaling of (unscaled)
momentum per node and keeps the mass; the reported velocity carries
+ dt F / (2 rho).  GPU parity through the C ABI: relative L2 <= 1e-12 in FP64
and <= 1e-6 in FP32 deviation storage against the oracle (periodic D2Q9 and
D3Q19, a walled D2Q9 channel).  Known answer: the reference's
SemiLagrangianBoundaryHandler_PoiseuilleBB_test
(boundaries/SemiLagrangianBoundaryHandler_test.cpp:178-226): a force-driven
Poiseuille channel with bounce-back walls reaches a mean velocity within
10 % of the bulk velocity.
"""
import math

import numpy as np
import pytest

import natrium_gb300 as N
import oracle as O
from tests.gpu_cases import make_case, periodic_state, rel_l2


@pytest.mark.parametrize("scheme", [O.FORCE_SHIFTING_VELOCITY, O.FORCE_EXACT_DIFFERENCE])
@pytest.mark.parametrize("stencil", ["D2Q9", "D3Q19"])
def test_force_adds_momentum_and_keeps_mass(stencil, scheme):
    st = O.stencil(stencil, 10.0)
    n = 40
    rng = np.random.default_rng(1)
    rho = 1 + 0.1 * rng.random(n)
    u = 0.3 * (rng.random((st.D, n)) - 0.5)
    f = O.equilibrium(st, rho, u) * (1 + 1e-3 * rng.standard_normal((st.Q, n)))
    e = st.e_unit[:, : st.D]
    F = np.array([0.3, -0.2, 0.1][: st.D])
    dt, tau = 0.01, 0.8
    m0, j0 = f.sum(0), e.T @ f
    r, uu = np.zeros(n), np.zeros((st.D, n))
    O.collide_bgk_force(st, tau, dt, f, r, uu, scheme, F)
    assert np.abs(f.sum(0) - m0).max() < 1e-14
    assert np.abs(e.T @ f - j0 - dt * F[:, None] / st.scaling).max() < 1e-14
    # reported velocity: the moments' velocity plus dt F / (2 rho)
    assert np.allclose(uu, st.scaling * j0 / m0 + 0.5 * dt * F[:, None] / m0, atol=1e-14)


def test_no_force_is_the_plain_collision():
    st = O.stencil("D2Q9", 5.0)
    n = 20
    rng = np.random.default_rng(2)
    f = O.equilibrium(st, np.ones(n), 0.1 * rng.standard_normal((2, n))) * (1 + 1e-3 * rng.random((9, n)))
    a, b = f.copy(), f.copy()
    O.collide_bgk(st, 0.7, a, np.zeros(n), np.zeros((2, n)))
    O.collide_bgk_force(st, 0.7, 0.01, b, np.zeros(n), np.zeros((2, n)), O.FORCE_NONE, (0.0, 0.0))
    assert np.array_equal(a, b)


def _oracle_steps(S, st, tau, dt, f, scheme, F, nsteps):
    f = f.copy()
    n = f.shape[1]
    rho, u = np.zeros(n), np.zeros((st.D, n))
    for _ in range(nsteps):
        f = S.stream(f)
        O.collide_bgk_force(st, tau, dt, f, rho, u, scheme, F)
    return f, rho, u


FORCE_CASES = [
    ("D2Q9", (6, 5), 3, False, "periodic"),
    ("D3Q19", (3, 3, 2), 2, True, "periodic"),
    ("D2Q9", (4, 3), 2, True, "walls"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
@pytest.mark.parametrize("scheme", ["SHIFTING_VELOCITY", "EXACT_DIFFERENCE"])
@pytest.mark.parametrize("case", FORCE_CASES, ids=[f"{c[0]}-{c[4]}" for c in FORCE_CASES])
def test_forced_step_matches_oracle(gpu_lib, case, scheme, precision):
    stencil, cells, p, dg, kind = case
    st, mesh, dt, tau, spec = make_case(stencil, cells, p, dg, "BGK_STANDARD", precision=precision)
    F = np.array([0.02, -0.01, 0.015][: st.D]) * st.scaling
    if kind == "walls":
        bc = (0, 0, 1, 1, 0, 0)
        mesh = O.Mesh(2, cells, p, True, mesh.L, bc=bc, uw=((0, 0, 0),) * 6)
        spec = N.SolverSpec(**{**spec.__dict__, "periodic": (True, False, True)})
    f0 = periodic_state(O.Mesh(st.D, cells, p, dg, mesh.L), st, seed=13)
    S = O.SLOperator(mesh, st, dt)
    f1, rho1, u1 = _oracle_steps(S, st, tau, dt, f0, O.FORCE_SHIFTING_VELOCITY if scheme == "SHIFTING_VELOCITY"
                                 else O.FORCE_EXACT_DIFFERENCE, F, 3)
    with N.Solver(spec) as sol:
        sol.set_force(scheme, F)
        assert sol.kernel_variant == 1  # the generic kernel carries the force term
        sol.upload_f(f0)
        sol.step(3)
        f = sol.download_f()
        rho, u = sol.download_macro()
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert rel_l2(f, f1) <= tol
    assert rel_l2(rho, rho1) <= tol
    assert rel_l2(u, u1) <= (1e-11 if precision == "fp64" else 1e-5)


@pytest.mark.gpu
def test_force_needs_bgk(gpu_lib):
    st, mesh, dt, tau, spec = make_case("D2Q9", (4, 4), 2, False, "KBC_STANDARD")
    with N.Solver(spec) as sol:
        with pytest.raises(N.NatError) as ei:
            sol.set_force("SHIFTING_VELOCITY", (0.1, 0.0))
        assert ei.value.code == N.NAT_ERR_UNSUPPORTED


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", ["SHIFTING_VELOCITY", "EXACT_DIFFERENCE"])
def test_poiseuille_bounce_back_known_answer(gpu_lib, scheme):
    """PoiseuilleFlow2D with VelocityNeqBounceBack walls
    (SemiLagrangianBoundaryHandler_test.cpp:178-226; PoiseuilleFlow2D.cpp:22-40):
    Re 10, u_bulk = 1e-4 / 1.5, height 1, length 2, refinement 2 (4 x 4 cells),
    p = 2, Ma 0.1, CFL 1.5, scaling sqrt(3) 1.5 u_bulk / Ma, body force
    F_x = 8 u_max nu / H^2 with u_max = 1.5 u_bulk; at steady state the mean
    velocity lies within 10 % of u_bulk.  (FE_DGQ here: walls need the DG node
    topology.)"""
    Re, u_bulk, H, L, p, Ma, cfl = 10.0, 1e-4 / 1.5, 1.0, 2.0, 2, 0.1, 1.5
    nu = u_bulk * H / Re
    scaling = math.sqrt(3) * 1.5 * u_bulk / Ma
    Fx = 8 * 1.5 * u_bulk * nu / (H * H)
    spec = N.SolverSpec(stencil="D2Q9", order=p, cells=(4, 4), length=(L, H), scaling=scaling, viscosity=nu,
                        cfl=cfl, collision="BGK_STANDARD", precision="fp64", topology="dg",
                        periodic=(True, False, True))
    with N.Solver(spec) as sol:
        sol.set_force(scheme, (Fx, 0.0))
        n = sol.n_ref
        from natrium_gb300 import problems as P
        sol.upload_f(P.equilibrium("D2Q9", scaling, np.ones(n), np.zeros((2, n))))
        # about ten viscous times H^2 / nu
        nsteps = int(10 * H * H / nu / sol.dt)
        sol.step(nsteps)
        rho, u = sol.download_macro()
    mean_u = float(u[0].mean())
    assert 0.9 * u_bulk < mean_u < 1.1 * u_bulk, (mean_u, u_bulk)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
def test_forced_mapped_mesh_matches_oracle(gpu_lib, precision):
    """The departure-point kernel's body-force form on a deformed periodic grid."""
    from natrium_gb300 import problems as P
    V = P.wavy_grid((4, 4), (1.0, 1.0), 0.1)
    st = O.stencil("D2Q9", math.sqrt(3) / 0.1)
    m = O.Mesh(2, (4, 4), 3, True, (1.0, 1.0), vertices=V)
    dt = O.time_step(m.h_min(), 3, st.max_speed, 0.4)
    nu = 2e-3
    tau = nu / (dt * st.cs2) + 0.5
    F = np.array([0.02, 0.01]) * st.scaling
    X = m.coords()
    u0 = 0.03 * np.stack([np.cos(2 * math.pi * X[:, 1]), np.sin(2 * math.pi * X[:, 0])]) * st.scaling
    f0 = O.equilibrium(st, np.ones(m.n_nodes), u0)
    f1, rho1, u1 = _oracle_steps(O.SLOperator(m, st, dt), st, tau, dt, f0, O.FORCE_EXACT_DIFFERENCE, F, 3)
    spec = N.SolverSpec(stencil="D2Q9", order=3, cells=(4, 4), length=(1.0, 1.0), scaling=st.scaling, viscosity=nu,
                        dt=dt, precision=precision, topology="dg", vertices=V)
    with N.Solver(spec) as sol:
        sol.set_force("EXACT_DIFFERENCE", F)
        sol.upload_f(f0)
        sol.step(3)
        f = sol.download_f()
        rho, u = sol.download_macro()
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert rel_l2(f, f1) <= tol
    assert rel_l2(u, u1) <= (1e-11 if precision == "fp64" else 1e-5)


# ---------------------------------------------------------------------------
# GUO (legacy BGKStandard::collideAll)
# ---------------------------------------------------------------------------

def _guo_d2q9_reference_form(f, F, scaling, tau, dt):
    """One node of BGKStandard::collideAllD2Q9 with GUO, written out per
    direction as the reference writes it (BGKStandard.cpp:110-239,
    ExternalForceFunctions.h:119-200): scaled u and F, unit directions."""
    cs2 = scaling * scaling / 3
    pre = scaling / cs2
    rf = -1.0 / tau
    rho = f.sum()
    u0 = scaling / rho * (f[1] + f[5] + f[8] - f[3] - f[6] - f[7]) + 0.5 * dt * F[0] / rho
    u1 = scaling / rho * (f[2] + f[5] + f[6] - f[4] - f[7] - f[8]) + 0.5 * dt * F[1] / rho
    usq = -(u0 * u0 + u1 * u1) / (2 * cs2)
    E = [(0, 0), (1, 0), (0, 1), (-1, 0), (0, -1), (1, 1), (-1, 1), (-1, -1), (1, -1)]
    W = [4 / 9] + [1 / 9] * 4 + [1 / 36] * 4
    out = f.copy()
    ug = u0 * F[0] + u1 * F[1]
    for i, (ex, ey) in enumerate(E):
        m = pre * (ex * u0 + ey * u1)
        feq = W[i] * rho * (1 + m * (1 + 0.5 * m) + usq)
        out[i] += rf * (f[i] - feq)
        eu, eF = ex * u0 + ey * u1, ex * F[0] + ey * F[1]
        out[i] += dt * W[i] * (1 - 0.5 / tau) * (pre * (eF - ug) + pre * pre * eu * eF)
    return out, rho, (u0, u1)


def test_guo_oracle_matches_the_reference_form_d2q9():
    st = O.stencil("D2Q9", 7.0)
    rng = np.random.default_rng(5)
    n = 16
    f = O.equilibrium(st, 1 + 0.1 * rng.random(n), 0.5 * (rng.random((2, n)) - 0.5)) * \
        (1 + 1e-3 * rng.standard_normal((9, n)))
    F = np.array([0.4, -0.3])
    dt, tau = 0.02, 0.9
    g, r, u = f.copy(), np.zeros(n), np.zeros((2, n))
    O.collide_bgk_force(st, tau, dt, g, r, u, O.FORCE_GUO, F)
    for k in range(n):
        ref, rho, uk = _guo_d2q9_reference_form(f[:, k], F, st.scaling, tau, dt)
        assert np.abs(g[:, k] - ref).max() <= 1e-15 * np.abs(ref).max() * 10
        assert abs(r[k] - rho) <= 1e-15
        assert np.allclose(u[:, k], uk, rtol=0, atol=1e-14)


@pytest.mark.parametrize("stencil", ["D2Q9", "D3Q19"])
def test_guo_momentum_and_mass(stencil):
    """The GUO collision adds dt F / scaling of unscaled momentum (omega/2 of
    it by relaxing towards the shifted velocity u', the rest from the source
    term) and dt (1 - omega/2)(3/s)(1/s - 1) u'.F of mass (the reference's
    u.F term carries p = 3/s where Guo's form has 3/s^2).  For D3Q19 the
    reference drops the source term: momentum + omega/2 dt F / s, mass kept."""
    st = O.stencil(stencil, 10.0)
    s = st.scaling
    n = 40
    rng = np.random.default_rng(3)
    rho = 1 + 0.1 * rng.random(n)
    u = 0.3 * (rng.random((st.D, n)) - 0.5)
    f = O.equilibrium(st, rho, u) * (1 + 1e-3 * rng.standard_normal((st.Q, n)))
    e = st.e_unit[:, : st.D]
    F = np.array([0.3, -0.2, 0.1][: st.D])
    dt, tau = 0.01, 0.8
    omega = 1 / tau
    m0, j0 = f.sum(0), e.T @ f
    r, uu = np.zeros(n), np.zeros((st.D, n))
    O.collide_bgk_force(st, tau, dt, f, r, uu, O.FORCE_GUO, F)
    assert np.allclose(uu, s * j0 / m0 + 0.5 * dt * F[:, None] / m0, rtol=0, atol=1e-14)
    uF = (uu * F[:, None]).sum(0)
    if stencil == "D2Q9":
        dm = dt * (1 - omega / 2) * (3 / s) * (1 / s - 1) * uF
        dj = dt * F[:, None] / s
    else:
        dm = 0 * uF
        dj = 0.5 * omega * dt * F[:, None] / s
    assert np.abs(f.sum(0) - m0 - dm).max() < 1e-14
    assert np.abs(e.T @ f - j0 - dj).max() < 1e-14


GUO_CASES = [
    ("D2Q9", (6, 5), 3, False, "periodic"),
    ("D3Q19", (3, 3, 2), 2, True, "periodic"),
    ("D2Q9", (4, 3), 2, True, "walls"),
]


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
@pytest.mark.parametrize("case", GUO_CASES, ids=[f"{c[0]}-{c[4]}" for c in GUO_CASES])
def test_guo_step_matches_oracle(gpu_lib, case, precision):
    stencil, cells, p, dg, kind = case
    st, mesh, dt, tau, spec = make_case(stencil, cells, p, dg, "BGK_STANDARD", precision=precision)
    F = np.array([0.02, -0.01, 0.015][: st.D]) * st.scaling
    if kind == "walls":
        mesh = O.Mesh(2, cells, p, True, mesh.L, bc=(0, 0, 1, 1, 0, 0), uw=((0, 0, 0),) * 6)
        spec = N.SolverSpec(**{**spec.__dict__, "periodic": (True, False, True)})
    f0 = periodic_state(O.Mesh(st.D, cells, p, dg, mesh.L), st, seed=17)
    S = O.SLOperator(mesh, st, dt)
    f1, rho1, u1 = _oracle_steps(S, st, tau, dt, f0, O.FORCE_GUO, F, 3)
    with N.Solver(spec) as sol:
        sol.set_force("GUO", F)
        sol.upload_f(f0)
        sol.step(3)
        f = sol.download_f()
        rho, u = sol.download_macro()
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert rel_l2(f, f1) <= tol
    assert rel_l2(rho, rho1) <= tol
    assert rel_l2(u, u1) <= (1e-11 if precision == "fp64" else 1e-5)


@pytest.mark.gpu
def test_guo_collide_all_mirror_matches_oracle(gpu_lib):
    """BGKStandard.collideAll through the Python mirror with the GUO force set."""
    st, mesh, dt, tau, spec = make_case("D2Q9", (4, 4), 2, False, "BGK_STANDARD")
    F = np.array([0.03, 0.01]) * st.scaling
    f0 = periodic_state(mesh, st, seed=19)
    fr, rr, ur = f0.copy(), np.zeros(mesh.n_nodes), np.zeros((2, mesh.n_nodes))
    O.collide_bgk_force(st, tau, dt, fr, rr, ur, O.FORCE_GUO, F)
    with N.Solver(spec) as sol:
        sol.set_force("GUO", F)
        f = N.DistributionFunctions(f0.copy())
        rho, u = np.zeros(mesh.n_nodes), np.zeros((2, mesh.n_nodes))
        N.BGKStandard(sol).collideAll(f, rho, u, None, False)
    # compare on the nodes the device stores once (periodic duplicates folded)
    nx = mesh.nodes_per_axis(0)
    keep = np.ones((nx, nx), bool)
    keep[:, -1] = keep[-1, :] = False
    keep = keep.reshape(-1)
    assert rel_l2(f.f[:, keep], fr[:, keep]) <= 1e-12
    assert rel_l2(u[:, keep], ur[:, keep]) <= 1e-11


@pytest.mark.gpu
def test_guo_unsupported_on_d3q27(gpu_lib):
    st, mesh, dt, tau, spec = make_case("D3Q27", (2, 2, 2), 2, False, "BGK_STANDARD")
    with N.Solver(spec) as sol:
        with pytest.raises(N.NatError) as ei:
            sol.set_force("GUO", (0.1, 0.0, 0.0))
        assert ei.value.code == N.NAT_ERR_UNSUPPORTED
