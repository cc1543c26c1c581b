"""Parity of the CUDA path (through the C ABI) with the CPU oracle.

Plain FP64: relative L2 <= 1e-12 per step against the oracle's restatement
of the reference (copy + per-direction CSR SpMV + collide sweep); the same
bound over 20 steps.  FP32 deviation storage: relative L2 of f <= 1e-6 per
step and of the velocity <= 1e-6 after the multi-step runs below.
"""
import glob
import math
import os

import numpy as np
import pytest

import natrium_gb300 as N
import oracle as O
from tests.gpu_cases import make_case, oracle_step, periodic_state, rel_l2

pytestmark = pytest.mark.gpu

TOL64 = 1e-12

CASES = [
    ("D2Q9", (8, 8), 4, False, "BGK_STANDARD"),
    ("D2Q9", (4, 4), 3, True, "BGK_STANDARD"),
    ("D2Q9", (6, 6), 2, False, "BGK_INCOMPRESSIBLE"),
    ("D2Q9", (4, 4), 3, False, "KBC_STANDARD"),
    ("D2Q9", (4, 6), 3, True, "KBC_STANDARD"),
    ("D2Q9", (5, 3), 1, False, "BGK_STANDARD"),
    ("D2Q9", (2, 2), 6, False, "BGK_STANDARD"),
    ("D2Q9", (3, 2), 6, True, "BGK_STANDARD"),
    ("D3Q19", (3, 3, 3), 2, False, "BGK_STANDARD"),
    ("D3Q19", (4, 4, 4), 4, False, "BGK_STANDARD"),
    ("D3Q19", (2, 4, 2), 4, True, "BGK_STANDARD"),
    ("D3Q27", (4, 4, 4), 3, False, "BGK_STANDARD"),
    ("D3Q27", (3, 3, 3), 2, True, "BGK_STANDARD"),
    ("D3Q27", (4, 4, 4), 2, False, "KBC_STANDARD"),
    ("D3Q27", (2, 2, 2), 3, True, "KBC_STANDARD"),
]


def _ids(c):
    return f"{c[0]}-{'x'.join(map(str, c[1]))}-p{c[2]}-{'dg' if c[3] else 'feq'}-{c[4]}"


@pytest.mark.parametrize("case", CASES, ids=[_ids(c) for c in CASES])
def test_fp64_step_matches_oracle(gpu_lib, case):
    stencil, cells, p, dg, model = case
    st, mesh, dt, tau, spec = make_case(stencil, cells, p, dg, model)
    f0 = periodic_state(mesh, st, seed=3)
    S = O.SLOperator(mesh, st, dt)
    f1, rho1, u1 = oracle_step(S, st, model, tau, f0)
    with N.Solver(spec) as sol:
        assert sol.n_ref == mesh.n_nodes
        assert sol.dt == pytest.approx(dt, rel=1e-15)
        assert sol.tau == pytest.approx(tau, rel=1e-14)
        sol.upload_f(f0)
        sol.step(1)
        g1 = sol.download_f()
        rho, u = sol.download_macro()
    assert rel_l2(g1, f1) <= TOL64
    assert rel_l2(rho, rho1) <= TOL64
    assert rel_l2(u, u1) <= 1e-11


@pytest.mark.parametrize("case", [CASES[0], CASES[3], CASES[9], CASES[13]], ids=_ids)
def test_fp64_twenty_steps(gpu_lib, case):
    stencil, cells, p, dg, model = case
    st, mesh, dt, tau, spec = make_case(stencil, cells, p, dg, model)
    f0 = periodic_state(mesh, st, seed=5)
    S = O.SLOperator(mesh, st, dt)
    f20, rho20, u20 = oracle_step(S, st, model, tau, f0, nsteps=20)
    with N.Solver(spec) as sol:
        sol.upload_f(f0)
        sol.step(20)
        g = sol.download_f()
        rho, u = sol.download_macro()
    assert rel_l2(g, f20) <= TOL64
    assert rel_l2(u, u20) <= 1e-10


@pytest.mark.parametrize("case", [CASES[0], CASES[1], CASES[9], CASES[12]], ids=_ids)
def test_stream_only_matches_spmv(gpu_lib, case):
    """AdvectionOperator::stream == the oracle's CSR SpMV (f_0 unchanged)."""
    stencil, cells, p, dg, model = case
    st, mesh, dt, tau, spec = make_case(stencil, cells, p, dg, model)
    f0 = periodic_state(mesh, st, seed=7)
    S = O.SLOperator(mesh, st, dt)
    ref = S.stream(f0)
    with N.Solver(spec) as sol:
        sol.upload_f(f0)
        assert sol.stream(0.0) == pytest.approx(dt)
        g = sol.download_f()
    assert rel_l2(g, ref) <= TOL64
    uniq = _unique_mask(mesh)
    assert np.array_equal(g[0][uniq], f0[0][uniq])


@pytest.mark.parametrize("model,stencil", [("BGK_STANDARD", "D2Q9"), ("BGK_INCOMPRESSIBLE", "D2Q9"),
                                           ("KBC_STANDARD", "D2Q9"), ("BGK_STANDARD", "D3Q19"),
                                           ("BGK_STANDARD", "D3Q27"), ("KBC_STANDARD", "D3Q27")])
@pytest.mark.parametrize("in_init", [False, True])
def test_collide_all_matches_oracle(gpu_lib, model, stencil, in_init):
    """CollisionModel::collideAll, including inInitializationProcedure."""
    cells = (4, 4) if stencil == "D2Q9" else (2, 2, 2)
    st, mesh, dt, tau, spec = make_case(stencil, cells, 2, False, model)
    f0 = periodic_state(mesh, st, seed=11)
    rng = np.random.default_rng(0)
    rho_in = np.zeros(mesh.n_nodes)
    u_in = np.ascontiguousarray(0.03 * st.scaling * np.sin(np.arange(st.D * mesh.n_nodes)).reshape(st.D, -1))
    fr = f0.copy()
    rr = rho_in.copy()
    ur = u_in.copy()
    O.collide(st, model, tau, fr, rr, ur, in_init)
    with N.Solver(spec) as sol:
        f = N.DistributionFunctions(f0.copy())
        rho = rho_in.copy()
        u = u_in.copy()
        {"BGK_STANDARD": N.BGKStandard, "BGK_INCOMPRESSIBLE": N.BGKIncompressible,
         "KBC_STANDARD": N.KBCStandard}[model](sol).collideAll(f, rho, u, None, in_init)
    # periodic duplicates of u_in are not equal in this synthetic input; the
    # device keeps one copy per periodic node, so compare on the unique nodes
    uniq = _unique_mask(mesh)
    assert rel_l2(f.f[:, uniq], fr[:, uniq]) <= TOL64
    assert rel_l2(rho[uniq], rr[uniq]) <= TOL64
    if not in_init:
        assert rel_l2(u[:, uniq], ur[:, uniq]) <= 1e-11


def _unique_mask(mesh):
    X = [np.arange(mesh.nodes_per_axis(a)) for a in range(3)]
    keep = np.ones((mesh.nodes_per_axis(2), mesh.nodes_per_axis(1), mesh.nodes_per_axis(0)), bool)
    if not mesh.dg:
        keep[:, :, -1] = False
        if mesh.dim >= 2:
            keep[:, -1, :] = False
        if mesh.dim == 3:
            keep[-1, :, :] = False
    return keep.reshape(-1)


def test_semilagrangian_mirror_stream(gpu_lib):
    """SemiLagrangian::stream(f_old, f, t) through the Python mirror."""
    st, mesh, dt, tau, spec = make_case("D2Q9", (4, 4), 4, False, "BGK_STANDARD")
    f0 = periodic_state(mesh, st, seed=2)
    ref = O.SLOperator(mesh, st, dt).stream(f0)
    with N.Solver(spec) as sol:
        sl = N.SemiLagrangian(sol)
        f_old = N.DistributionFunctions(np.zeros_like(f0))
        f = N.DistributionFunctions(f0.copy())
        assert sl.stream(f_old, f, 0.0) == pytest.approx(dt)
        assert np.array_equal(f_old.f, f0)
        assert rel_l2(f.f, ref) <= TOL64
        with pytest.raises(ValueError):
            sl.stream(f, f, 0.0)


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "oracle_*.npz"))),
                         ids=lambda p: os.path.basename(p))
def test_golden_fixtures(gpu_lib, path):
    z = np.load(path)
    stencil, model = str(z["stencil"]), str(z["model"])
    Ma = float(z["Ma"])
    st = O.stencil(stencil, math.sqrt(3) / Ma)
    spec = N.SolverSpec(stencil=stencil, order=int(z["p"]), cells=tuple(int(x) for x in z["N"]),
                        length=(2 * math.pi,) * 3, scaling=st.scaling, viscosity=float(z["nu"]),
                        dt=float(z["dt"]), collision=model, topology="dg" if bool(z["dg"]) else "feq")
    with N.Solver(spec) as sol:
        sol.upload_f(z["f0"])
        sol.step(1)
        assert rel_l2(sol.download_f(), z["f1"]) <= TOL64
        rho, u = sol.download_macro()
        assert rel_l2(rho, z["rho"]) <= TOL64


def test_density_underflow_is_reported(gpu_lib):
    """rho < 1e-10 -> CollisionException (the reference throws
    DensityZeroException, CollisionOperator.h:106-109)."""
    st, mesh, dt, tau, spec = make_case("D2Q9", (4, 4), 2, False, "BGK_STANDARD")
    f0 = periodic_state(mesh, st, seed=1)
    f0[:, :] = 0.0
    with N.Solver(spec) as sol:
        sol.upload_f(f0)
        with pytest.raises(N.CollisionException):
            sol.step(1)
        # the status is cleared and the handle stays usable
        sol.upload_f(periodic_state(mesh, st, seed=1))
        sol.step(1)


def test_mass_energy_reduction(gpu_lib):
    st, mesh, dt, tau, spec = make_case("D2Q9", (8, 8), 4, False, "BGK_STANDARD", Ma=0.05)
    rho0, u0 = O.tgv2d_init(mesh.coords(), 0.05)
    u0 = np.ascontiguousarray(u0)
    f0 = O.equilibrium(st, rho0, u0)
    S = O.SLOperator(mesh, st, dt)
    f1, rho1, u1 = oracle_step(S, st, "BGK_STANDARD", tau, f0, 3)
    with N.Solver(spec) as sol:
        sol.upload_f(f0)
        sol.step(3)
        m, e = sol.mass_energy()
    assert e == pytest.approx(O.kinetic_energy(mesh, rho1, u1), rel=1e-12)
    assert m == pytest.approx(_mass(mesh, rho1), rel=1e-12)


@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
def test_tgv2d_integration_known_answer(gpu_lib, precision):
    """The reference's semi-Lagrangian Taylor-Green integration test
    (ConvergenceTestSemiLagrangianPeriodic, IntegrationTestCases.cpp:885-961),
    run on the device: 8 x 8 cells, FE_Q p = 4, D2Q9 BGK, nu = 1, Ma = 0.05,
    CFL 0.4; after t = 1 / (2 nu), E_kin / E_kin(0) = e^-2 within 1e-2 and the
    velocity's relative L2 error against the analytic decay below 5e-2."""
    import json
    import os
    from natrium_gb300 import problems as P
    with open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")) as fh:
        c = json.load(fh)["tgv2d_sl"]
    Ma, nu, p = c["Ma"], c["viscosity"], c["order"]
    n = 2 ** c["refinement"]
    scaling = math.sqrt(3) / Ma
    spec = N.SolverSpec(stencil="D2Q9", order=p, cells=(n, n), length=(2 * math.pi,) * 2, scaling=scaling,
                        viscosity=nu, cfl=c["cfl"], collision="BGK_STANDARD", precision=precision, topology="feq")
    X = P.node_coords((n, n), p, spec.length, "feq")
    rho0, u0 = P.taylor_green_2d(X, Ma)
    with N.Solver(spec) as sol:
        sol.upload_macro(rho0, u0)  # E_kin(0) of the initial fields
        _, e0 = sol.mass_energy()
        nsteps = int(round(1.0 / (2 * nu) / sol.dt))
        sol.upload_f(P.equilibrium("D2Q9", scaling, rho0, u0))
        sol.step(nsteps)
        _, e1 = sol.mass_energy()
        rho, u = sol.download_macro()
        t = nsteps * sol.dt
    assert abs(e1 / e0 - math.exp(-2)) < c["ekin_tol"]
    ua = np.stack([np.sin(X[:, 0]) * np.cos(X[:, 1]), -np.cos(X[:, 0]) * np.sin(X[:, 1])]) * math.exp(-2 * nu * t)
    assert rel_l2(u, ua) < c["l2_velocity_tol"]


def test_physical_properties_known_answers(gpu_lib):
    """solver/PhysicalProperties_test.cpp:46-91.  Mass of CouetteFlow2D on the unit
    square (rho = 1): 1 within 1e-4 %.  Kinetic energy of the ShearLayer2D
    initial state (Minion & Brown: u0 = 1, kappa = 80, nu = 1e-4, refinement 3
    -> 8 x 8 cells, scaling 10, FE_Q p = 2): 0.476 within 10 %."""
    from natrium_gb300 import problems as P
    spec = N.SolverSpec(stencil="D2Q9", order=2, cells=(8, 8), length=(1.0, 1.0), scaling=10.0, viscosity=1e-4,
                        cfl=0.4, topology="feq")
    X = P.node_coords((8, 8), 2, (1.0, 1.0), "feq")
    rho, u = P.shear_layer_2d(X, kappa=80.0, delta=0.05, L=1.0)
    with N.Solver(spec) as sol:
        sol.upload_f(P.equilibrium("D2Q9", 10.0, rho, u))
        sol.collide()  # rho and u (scaled) from the moments of f
        m, e = sol.mass_energy()
    assert m == pytest.approx(1.0, rel=1e-6)
    assert e == pytest.approx(0.476, rel=0.10)


def _mass(mesh, rho):
    # sum_cells sum_q rho w_q |J| via the oracle's quadrature (KE with |u| = 1)
    one = np.ones((mesh.dim, rho.size)) / math.sqrt(mesh.dim)
    return 2 * O.kinetic_energy(mesh, rho, one)


@pytest.mark.parametrize("stencil,cells,p,dg,model", [
    ("D2Q9", (8, 8), 4, False, "BGK_STANDARD"),
    ("D2Q9", (8, 8), 3, False, "KBC_STANDARD"),
    ("D2Q9", (8, 8), 3, False, "BGK_INCOMPRESSIBLE"),
    ("D3Q19", (4, 4, 4), 3, False, "BGK_STANDARD"),
    ("D3Q27", (4, 4, 4), 2, True, "KBC_STANDARD"),
])
def test_fp32_deviation_against_fp64_oracle(gpu_lib, stencil, cells, p, dg, model):
    """FP32 deviation storage: f within 1e-6 relative L2 after one step and
    the velocity within 1e-6 relative L2 after 50 steps (10 for the
    incompressible model), against the FP64 oracle on the same input."""
    st, mesh, dt, tau, spec = make_case(stencil, cells, p, dg, model, precision="fp32dev")
    f0 = periodic_state(mesh, st, seed=4)
    if model == "BGK_INCOMPRESSIBLE":
        f0 = incompressible_equilibrium(st, f0)
    S = O.SLOperator(mesh, st, dt)
    # the reference's incompressible model, restated as written, is unstable
    # (its equilibrium does not conserve mass) and blows up after ~30 steps:
    # compare it over 10 steps
    nmore = 9 if model == "BGK_INCOMPRESSIBLE" else 49
    f1, _, _ = oracle_step(S, st, model, tau, f0, 1)
    f50, rho50, u50 = oracle_step(S, st, model, tau, f1, nmore)
    with N.Solver(spec) as sol:
        sol.upload_f(f0)
        sol.step(1)
        assert rel_l2(sol.download_f(), f1) <= 1e-6
        sol.step(nmore)
        rho, u = sol.download_macro()
    assert rel_l2(u, u50) <= 1e-6
    assert rel_l2(rho, rho50) <= 1e-7


def incompressible_equilibrium(st, f):
    """The incompressible model's own equilibrium at the (rho, u) of f: one
    oracle collision with tau = 1 and the velocity prescribed (f -> feq)."""
    rho = f.sum(0)
    u = np.ascontiguousarray((st.e[:, :st.D].T @ f) / rho)
    g = np.ascontiguousarray(f.copy())
    O.collide_bgk_incompressible_d2q9(st, 1.0, g, np.zeros_like(rho), u, in_init=True)
    return g


V2_CASES = [
    ("D3Q19", (4, 2, 2), 4, True, "BGK_STANDARD"),
    ("D3Q19", (4, 4, 4), 4, False, "BGK_STANDARD"),
    ("D3Q19", (4, 4, 2), 4, True, "BGK_STANDARD"),
    ("D3Q27", (4, 2, 2), 3, True, "BGK_STANDARD"),
    ("D3Q27", (4, 2, 2), 3, True, "KBC_STANDARD"),
    ("D3Q27", (4, 4, 2), 3, True, "KBC_STANDARD"),
]


@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
@pytest.mark.parametrize("case", V2_CASES, ids=[_ids(c) for c in V2_CASES])
def test_specialised_and_generic_kernels_agree(gpu_lib, case, precision):
    """Every fused kernel that applies (generic, tile, row-segment) against
    the oracle on the same input, each forced in turn."""
    stencil, cells, p, dg, model = case
    st, mesh, dt, tau, spec = make_case(stencil, cells, p, dg, model, precision=precision)
    f0 = periodic_state(mesh, st, seed=9)
    S = O.SLOperator(mesh, st, dt)
    f1, rho1, u1 = oracle_step(S, st, model, tau, f0, 2)
    tol = TOL64 if precision == "fp64" else 1e-6
    out = {}
    for variant, kind in ((1, 1), (3, 2), (4, 3)):
        with N.Solver(spec) as sol:
            try:
                sol.set_kernel_variant(variant)
            except N.NatError:
                continue
            assert sol.kernel_variant == kind
            sol.upload_f(f0)
            sol.step(2)
            out[kind] = sol.download_f()
            rho, u = sol.download_macro()
        assert rel_l2(out[kind], f1) <= tol, kind
        assert rel_l2(u, u1) <= (1e-11 if precision == "fp64" else 1e-6), kind
    assert 1 in out and len(out) >= 2
    if precision == "fp64":
        for k in out:
            assert rel_l2(out[k], out[1]) <= TOL64


def test_automatic_variant_choice(gpu_lib):
    st, mesh, dt, tau, spec = make_case("D3Q19", (4, 2, 2), 4, True, "BGK_STANDARD", precision="fp32dev")
    with N.Solver(spec) as sol:
        assert sol.kernel_variant in (2, 3)
    st, mesh, dt, tau, spec = make_case("D3Q19", (3, 3, 3), 2, False, "BGK_STANDARD")
    with N.Solver(spec) as sol:
        assert sol.kernel_variant == 1
        with pytest.raises(N.NatError):
            sol.set_kernel_variant(2)


def test_cell_variants_refused_where_they_do_not_apply(gpu_lib):
    """Variants 11-13 need DG rows of 16 or 32 cells; 12 only exists for
    D3Q27 FP32 and 13 not for D3Q27 FP32 BGK: asking for one where it does
    not apply is refused (NAT_ERR_UNSUPPORTED), and the handle steps
    correctly after the automatic choice is restored."""
    st, mesh, dt, tau, spec = make_case("D3Q19", (16, 8, 1), 4, True, "BGK_STANDARD", precision="fp32dev")
    with N.Solver(spec) as sol:
        for v in (11, 13):
            sol.set_kernel_variant(v)
            assert sol.kernel_variant == v
        with pytest.raises(N.NatError):
            sol.set_kernel_variant(12)
    st, mesh, dt, tau, spec = make_case("D3Q27", (32, 2, 1), 3, True, "BGK_STANDARD", precision="fp32dev")
    with N.Solver(spec) as sol:
        sol.set_kernel_variant(12)
        assert sol.kernel_variant == 12
        with pytest.raises(N.NatError):
            sol.set_kernel_variant(13)
    st, mesh, dt, tau, spec = make_case("D3Q19", (12, 2, 1), 4, True, "BGK_STANDARD", precision="fp32dev")
    with N.Solver(spec) as sol:  # 12 cells per x row: no cell-row kernel
        with pytest.raises(N.NatError):
            sol.set_kernel_variant(11)
        f0 = periodic_state(mesh, st, seed=5)
        S = O.SLOperator(mesh, st, dt)
        f1, rho1, u1 = oracle_step(S, st, "BGK_STANDARD", tau, f0, 2)
        sol.set_kernel_variant(0)
        sol.upload_f(f0)
        sol.step(2)
        assert rel_l2(sol.download_f(), f1) <= 1e-6


@pytest.mark.parametrize("stencil,p,model", [("D3Q19", 4, "BGK_STANDARD"), ("D3Q27", 3, "KBC_STANDARD")])
def test_fp32_tgv3d_long_run_against_fp64(gpu_lib, stencil, p, model):
    """3-D Taylor-Green (Ma 0.1, Re 1600), FP32 deviation storage against the
    FP64 path (itself pinned to the oracle above): relative L2 of u and rho
    after 1000 steps within 1e-6."""
    from natrium_gb300 import problems as P
    cells = (4, 4, 4)
    Ma, Re = 0.1, 1600.0
    scaling = math.sqrt(3) / Ma
    out = {}
    for prec in ("fp64", "fp32dev"):
        spec = N.SolverSpec(stencil=stencil, order=p, cells=cells, length=(2 * math.pi,) * 3, scaling=scaling,
                            viscosity=1 / Re, cfl=0.4, collision=model, precision=prec, topology="dg")
        X = P.node_coords(cells, p, spec.length, "dg")
        rho, u = P.taylor_green_3d(X, Ma)
        f0 = P.equilibrium(stencil, scaling, rho, u)
        with N.Solver(spec) as sol:
            sol.upload_f(f0)
            sol.step(1000)
            out[prec] = sol.download_macro()
    assert rel_l2(out["fp32dev"][1], out["fp64"][1]) <= 1e-6
    assert rel_l2(out["fp32dev"][0], out["fp64"][0]) <= 1e-7


@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
def test_autotune_keeps_state_and_parity(gpu_lib, precision):
    """nat_autotune times every applicable kernel, restores f, and the
    chosen kernel still matches the oracle."""
    st, mesh, dt, tau, spec = make_case("D3Q19", (4, 4, 2), 4, True, "BGK_STANDARD", precision=precision)
    f0 = periodic_state(mesh, st, seed=21)
    S = O.SLOperator(mesh, st, dt)
    f1, _, _ = oracle_step(S, st, "BGK_STANDARD", tau, f0, 1)
    with N.Solver(spec) as sol:
        sol.upload_f(f0)
        nc, ch = sol.autotune(3)
        assert nc >= 2 and 0 <= ch < nc
        info = sol.kernel_info()
        assert info["variant"] in (1, 2, 3)
        assert rel_l2(sol.download_f(), f0) <= (TOL64 if precision == "fp64" else 1e-7)
        sol.step(1)
        assert rel_l2(sol.download_f(), f1) <= (TOL64 if precision == "fp64" else 1e-6)


ROW_CASES = [(st, cells, p, dg, m) for (st, cells, m) in (("D2Q9", (2, 4), "BGK_STANDARD"), ("D2Q9", (4, 2), "KBC_STANDARD"),
                                                          ("D2Q9", (2, 2), "BGK_INCOMPRESSIBLE"))
             for p in (1, 2, 3, 4, 5, 6) for dg in (False, True)] + [
    ("D3Q19", (2, 2, 2), p, dg, "BGK_STANDARD") for p in (2, 3, 5, 6) for dg in (False, True)] + [
    ("D3Q27", (2, 2, 2), p, dg, m) for p in (2, 3) for dg in (False, True) for m in ("BGK_STANDARD", "KBC_STANDARD")]


@pytest.mark.parametrize("case", ROW_CASES, ids=[_ids(c) for c in ROW_CASES])
def test_row_kernel_all_orders(gpu_lib, case):
    """The row-segment kernel (forced when it applies, else the automatic
    choice) against the oracle for every FE order and both topologies."""
    stencil, cells, p, dg, model = case
    st, mesh, dt, tau, spec = make_case(stencil, cells, p, dg, model)
    f0 = periodic_state(mesh, st, seed=13)
    if model == "BGK_INCOMPRESSIBLE":
        f0 = incompressible_equilibrium(st, f0)
    S = O.SLOperator(mesh, st, dt)
    f1, rho1, u1 = oracle_step(S, st, model, tau, f0, 1)
    with N.Solver(spec) as sol:
        try:
            sol.set_kernel_variant(4)
        except N.NatError:
            sol.set_kernel_variant(0)
        sol.upload_f(f0)
        sol.step(1)
        assert rel_l2(sol.download_f(), f1) <= TOL64


# The bulk-copy row kernel (sl_rowt.cuh, kernel kind 6) needs x rows of at
# least one copy width and 16-byte aligned row starts, so these meshes are
# longer in x than the cases above.
ROWT_CASES = [
    ("D3Q19", (12, 4, 2), 4, True, "BGK_STANDARD"),
    ("D3Q19", (32, 2, 2), 2, False, "BGK_STANDARD"),
    ("D3Q19", (16, 4, 2), 3, False, "BGK_STANDARD"),
    ("D3Q27", (12, 2, 2), 3, True, "BGK_STANDARD"),
    ("D3Q27", (16, 4, 2), 2, True, "KBC_STANDARD"),
]


@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
@pytest.mark.parametrize("case", ROWT_CASES, ids=[_ids(c) for c in ROWT_CASES])
def test_bulk_copy_row_kernel_matches_oracle(gpu_lib, case, precision):
    stencil, cells, p, dg, model = case
    st, mesh, dt, tau, spec = make_case(stencil, cells, p, dg, model, precision=precision)
    f0 = periodic_state(mesh, st, seed=21)
    S = O.SLOperator(mesh, st, dt)
    f1, rho1, u1 = oracle_step(S, st, model, tau, f0, 2)
    with N.Solver(spec) as sol:
        sol.set_kernel_variant(6)
        assert sol.kernel_variant == 6
        assert sol.kernel_info()["smem_bytes"] > 0
        sol.upload_f(f0)
        sol.step(2)
        f = sol.download_f()
        rho, u = sol.download_macro()
        sol.set_kernel_variant(1)
        sol.upload_f(f0)
        sol.step(2)
        fg = sol.download_f()
    tol = TOL64 if precision == "fp64" else 1e-6
    assert rel_l2(f, f1) <= tol
    assert rel_l2(rho, rho1) <= tol
    assert rel_l2(u, u1) <= (1e-11 if precision == "fp64" else 1e-6)
    if precision == "fp64":
        assert rel_l2(f, fg) <= TOL64


# The row kernel with its streamed values in shared memory (FP32, 3-D, one
# z row per CTA of 4 or 8 warps) is the first row candidate when ny is a
# multiple of 4.
SS_CASES = [
    ("D3Q19", (4, 4, 2), 4, True, "BGK_STANDARD"),
    ("D3Q19", (3, 4, 3), 2, False, "BGK_STANDARD"),
    ("D3Q19", (2, 8, 2), 1, True, "BGK_STANDARD"),
    ("D3Q27", (3, 4, 2), 3, True, "BGK_STANDARD"),
    ("D3Q27", (4, 4, 2), 3, False, "KBC_STANDARD"),
]


@pytest.mark.parametrize("case", SS_CASES, ids=[_ids(c) for c in SS_CASES])
def test_shared_state_row_kernel_matches_oracle(gpu_lib, case):
    stencil, cells, p, dg, model = case
    st, mesh, dt, tau, spec = make_case(stencil, cells, p, dg, model, precision="fp32dev")
    f0 = periodic_state(mesh, st, seed=23)
    S = O.SLOperator(mesh, st, dt)
    f1, rho1, u1 = oracle_step(S, st, model, tau, f0, 3)
    with N.Solver(spec) as sol:
        sol.set_kernel_variant(4)
        info = sol.kernel_info()
        assert info["variant"] == 3 and info["tile_nodes"][2] == 1, info
        sol.upload_f(f0)
        sol.step(3)
        f = sol.download_f()
        rho, u = sol.download_macro()
    assert rel_l2(f, f1) <= 1e-6
    assert rel_l2(rho, rho1) <= 1e-6
    assert rel_l2(u, u1) <= 1e-6


# Every kernel the autotuner can choose, one by one (nat_select_candidate):
# the row-segment kernels in all their CTA shapes (incl. the z-sharing form),
# the row-group, bulk-copy, tile and generic kernels.
EVERY_CASES = [
    ("D3Q19", (4, 4, 2), 4, True, "BGK_STANDARD", "fp32dev"),
    ("D3Q19", (3, 4, 3), 2, False, "BGK_STANDARD", "fp32dev"),
    ("D3Q27", (3, 4, 2), 3, True, "BGK_STANDARD", "fp32dev"),
    ("D3Q27", (4, 4, 2), 3, False, "KBC_STANDARD", "fp32dev"),
    # DG p = 3 with cells divisible by every D3Q27 tile (4 x 2 x 2 down to 4 x 1 x 1)
    ("D3Q27", (4, 2, 2), 3, True, "KBC_STANDARD", "fp32dev"),
    ("D3Q27", (4, 2, 2), 3, True, "BGK_STANDARD", "fp32dev"),
    ("D3Q27", (4, 2, 2), 3, True, "KBC_STANDARD", "fp64"),
    ("D3Q27", (3, 4, 2), 3, False, "BGK_STANDARD", "fp64"),
    ("D3Q19", (4, 4, 2), 4, True, "BGK_STANDARD", "fp64"),
    ("D2Q9", (8, 8), 4, True, "BGK_STANDARD", "fp32dev"),
    # cell-row kernel shapes (nx = L (p + 1), L = 16 or 32 cells per x row)
    ("D3Q27", (16, 2, 2), 3, True, "KBC_STANDARD", "fp32dev"),
    ("D3Q27", (32, 2, 1), 3, True, "BGK_STANDARD", "fp32dev"),
    ("D3Q27", (32, 2, 2), 3, True, "KBC_STANDARD", "fp32dev"),
    ("D3Q27", (32, 2, 1), 3, True, "KBC_STANDARD", "fp64"),
    ("D3Q19", (16, 4, 2), 4, True, "BGK_STANDARD", "fp32dev"),
    ("D3Q19", (16, 4, 2), 4, True, "BGK_STANDARD", "fp64"),
    ("D3Q19", (32, 2, 1), 3, True, "BGK_STANDARD", "fp32dev"),
    # x rows of 64 cells: two warps per row, edge values through shared memory
    ("D3Q19", (64, 2, 1), 4, True, "BGK_STANDARD", "fp32dev"),
    ("D3Q19", (64, 2, 1), 4, True, "BGK_STANDARD", "fp64"),
    ("D3Q19", (64, 2, 2), 4, False, "BGK_STANDARD", "fp32dev"),
    ("D3Q27", (64, 2, 1), 3, True, "KBC_STANDARD", "fp32dev"),
    # x rows of 128 cells: four warps per row
    ("D3Q19", (128, 2, 1), 4, True, "BGK_STANDARD", "fp32dev"),
    ("D3Q19", (128, 2, 1), 4, True, "BGK_STANDARD", "fp64"),
    ("D3Q19", (128, 2, 2), 4, False, "BGK_STANDARD", "fp32dev"),
    ("D3Q27", (128, 2, 1), 3, True, "KBC_STANDARD", "fp32dev"),
    # the cell-row kernel on FE_Q nodes (a lane owns its cell's p nodes)
    ("D3Q19", (16, 4, 2), 4, False, "BGK_STANDARD", "fp32dev"),
    ("D3Q19", (16, 4, 2), 4, False, "BGK_STANDARD", "fp64"),
    ("D3Q27", (32, 4, 2), 3, False, "KBC_STANDARD", "fp32dev"),
]


@pytest.mark.parametrize("case", EVERY_CASES, ids=[_ids(c[:5]) + "-" + c[5] for c in EVERY_CASES])
def test_every_autotune_candidate_matches_oracle(gpu_lib, case):
    stencil, cells, p, dg, model, precision = case
    st, mesh, dt, tau, spec = make_case(stencil, cells, p, dg, model, precision=precision)
    f0 = periodic_state(mesh, st, seed=29)
    S = O.SLOperator(mesh, st, dt)
    f1, rho1, u1 = oracle_step(S, st, model, tau, f0, 3)
    with N.Solver(spec) as sol:
        sol.upload_f(f0)
        n, _ = sol.autotune(1)
        kinds = [r["variant"] for r in sol.autotune_report()]
    assert n >= 1 and len(kinds) == n
    tol = 1e-6 if precision == "fp32dev" else 1e-12
    for i in range(n):
        with N.Solver(spec) as sol:
            sol.select_candidate(i)
            assert sol.kernel_variant == kinds[i]
            sol.upload_f(f0)
            sol.step(3)
            f = sol.download_f()
            rho, u = sol.download_macro()
        assert rel_l2(f, f1) <= tol, (i, kinds[i])
        assert rel_l2(rho, rho1) <= tol
        assert rel_l2(u, u1) <= (1e-6 if precision == "fp32dev" else 1e-11)


# Cell-row kernel with the 8 corner directions of D3Q27 as tf32x3 tensor-core
# tiles (kernel variant 12, only when asked for): 32 cells per x row, y and z
# with several cells so that the upwind windows wrap.
TC_CASES = [
    ("D3Q27", (32, 2, 2), 3, True, "KBC_STANDARD"),
    ("D3Q27", (32, 3, 2), 3, True, "BGK_STANDARD"),
]


@pytest.mark.parametrize("case", TC_CASES, ids=[_ids(c) for c in TC_CASES])
def test_tensor_core_corner_kernel_matches_oracle(gpu_lib, case):
    stencil, cells, p, dg, model = case
    st, mesh, dt, tau, spec = make_case(stencil, cells, p, dg, model, precision="fp32dev")
    f0 = periodic_state(mesh, st, seed=31)
    S = O.SLOperator(mesh, st, dt)
    f1, rho1, u1 = oracle_step(S, st, model, tau, f0, 3)
    with N.Solver(spec) as sol:
        sol.set_kernel_variant(12)
        assert sol.kernel_variant == 12
        sol.upload_f(f0)
        sol.step(3)
        f = sol.download_f()
        rho, u = sol.download_macro()
    assert rel_l2(f, f1) <= 1e-6
    assert rel_l2(rho, rho1) <= 1e-6
    assert rel_l2(u, u1) <= 1e-6


def test_tensor_core_corner_kernel_not_chosen_automatically(gpu_lib):
    st, mesh, dt, tau, spec = make_case("D3Q27", (32, 2, 1), 3, True, "KBC_STANDARD", precision="fp32dev")
    with N.Solver(spec) as sol:
        n, _ = sol.autotune(1)
        kinds = [r["variant"] for r in sol.autotune_report()]
    assert 11 in kinds and 12 not in kinds


# Row-group kernel (sl_rowg.cuh, kernel kind 7): G warps own a whole x row
# (32 (G - 1) < nx <= 32 G, G = 2..4).
ROWG_CASES = [
    ("D3Q19", (16, 4, 2), 4, True, "BGK_STANDARD"),
    ("D3Q19", (20, 4, 2), 2, False, "BGK_STANDARD"),
    ("D3Q19", (32, 2, 2), 3, False, "BGK_STANDARD"),
    ("D3Q27", (12, 2, 2), 3, True, "BGK_STANDARD"),
    ("D3Q27", (16, 4, 2), 2, True, "KBC_STANDARD"),
]


@pytest.mark.parametrize("case", ROWG_CASES, ids=[_ids(c) for c in ROWG_CASES])
def test_row_group_kernel_matches_oracle(gpu_lib, case):
    stencil, cells, p, dg, model = case
    st, mesh, dt, tau, spec = make_case(stencil, cells, p, dg, model, precision="fp32dev")
    f0 = periodic_state(mesh, st, seed=29)
    S = O.SLOperator(mesh, st, dt)
    f1, rho1, u1 = oracle_step(S, st, model, tau, f0, 3)
    with N.Solver(spec) as sol:
        sol.set_kernel_variant(7)
        assert sol.kernel_variant == 7
        sol.upload_f(f0)
        sol.step(3)
        f = sol.download_f()
        rho, u = sol.download_macro()
    assert rel_l2(f, f1) <= 1e-6
    assert rel_l2(rho, rho1) <= 1e-6
    assert rel_l2(u, u1) <= 1e-6
