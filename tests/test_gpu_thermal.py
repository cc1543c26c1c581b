"""Parity of the compressible two-population path (D2Q25H, quartic
equilibrium, relaxWithG) on the GPU with the CPU oracle.

Plain FP64: relative L2 <= 1e-12 per step for f, g, rho, u and T against the
oracle's restatement (copy + CSR SpMV of f and of g with the same operator,
then CollisionOperator::collideAll(f, g, ...)); the shock-sensor mask (a sum
of |f - f^eq|, i.e. of small differences) within 1e-9.
"""
import numpy as np
import pytest

import natrium_gb300 as N
import oracle as O
from tests.gpu_cases import rel_l2, thermal_case, thermal_state

pytestmark = pytest.mark.gpu

TOL64 = 1e-12

CASES = [((4, 4), p, dg) for p in (1, 2, 3, 4, 5, 6) for dg in (False, True)]


def _th(settings: N.ThermalSettings) -> O.Thermal:
    return O.Thermal(settings.gamma, settings.prandtl, settings.prandtl_set, settings.sutherland,
                     settings.equilibrium == "QUARTIC")


def _run(spec, f0, g0, settings=None, nsteps=1):
    with N.Solver(spec) as sol:
        if settings is not None:
            sol.set_thermal(settings)
        sol.upload_f(f0)
        sol.upload_g(g0)
        sol.step(nsteps)
        f, g = sol.download_f(), sol.download_g()
        rho, u = sol.download_macro()
        T, m = sol.download_thermal()
        assert sol.kernel_variant == 5
    return f, g, rho, u, T, m


@pytest.mark.parametrize("case", CASES, ids=[f"p{c[1]}-{'dg' if c[2] else 'feq'}" for c in CASES])
def test_fp64_step_matches_oracle(gpu_lib, case):
    cells, p, dg = case
    st, mesh, dt, tau, spec = thermal_case(cells, p, dg)
    rho0, u0, T0, f0, g0 = thermal_state(mesh, st, seed=p)
    S = O.SLOperator(mesh, st, dt)
    f1, g1 = f0.copy(), g0.copy()
    r1, u1, T1, m1 = S.step_compressible(f1, g1, tau)
    f, g, rho, u, T, m = _run(spec, f0, g0)
    assert rel_l2(f, f1) <= TOL64
    assert rel_l2(g, g1) <= TOL64
    assert rel_l2(rho, r1) <= TOL64
    assert rel_l2(u, u1) <= 1e-11
    assert rel_l2(T, T1) <= TOL64
    assert rel_l2(m, m1) <= 1e-9


SETTINGS = [
    N.ThermalSettings(prandtl=0.71, prandtl_set=True),
    N.ThermalSettings(sutherland=True),
    N.ThermalSettings(equilibrium="BGK"),
    N.ThermalSettings(gamma=1.67, prandtl=2.0, prandtl_set=True, sutherland=True),
]


@pytest.mark.parametrize("settings", SETTINGS, ids=["prandtl", "sutherland", "bgk-eq", "all"])
def test_fp64_settings_match_oracle(gpu_lib, settings):
    st, mesh, dt, tau, spec = thermal_case((4, 3), 2, True, scaling=1.3, nu=2e-3)
    rho0, u0, T0, f0, g0 = thermal_state(mesh, st, seed=7, gamma=settings.gamma)
    S = O.SLOperator(mesh, st, dt)
    f1, g1 = f0.copy(), g0.copy()
    r1, u1, T1, m1 = S.step_compressible(f1, g1, tau, _th(settings))
    f, g, rho, u, T, m = _run(spec, f0, g0, settings)
    assert rel_l2(f, f1) <= TOL64
    assert rel_l2(g, g1) <= TOL64
    assert rel_l2(T, T1) <= TOL64
    assert rel_l2(m, m1) <= 1e-9


def test_fp64_ten_steps(gpu_lib):
    st, mesh, dt, tau, spec = thermal_case((6, 5), 2, True)
    rho0, u0, T0, f0, g0 = thermal_state(mesh, st, seed=11)
    S = O.SLOperator(mesh, st, dt)
    f1, g1 = f0.copy(), g0.copy()
    r1, u1, T1, m1 = S.step_compressible(f1, g1, tau, nsteps=10)
    f, g, rho, u, T, m = _run(spec, f0, g0, nsteps=10)
    assert rel_l2(f, f1) <= TOL64
    assert rel_l2(g, g1) <= TOL64
    assert rel_l2(T, T1) <= TOL64
    assert rel_l2(u, u1) <= 1e-10


@pytest.mark.parametrize("dg", [False, True])
def test_stream_only_streams_both_populations(gpu_lib, dg):
    st, mesh, dt, tau, spec = thermal_case((4, 4), 3, dg)
    rho0, u0, T0, f0, g0 = thermal_state(mesh, st, seed=2)
    S = O.SLOperator(mesh, st, dt)
    fo, go = S.stream(f0), S.stream(g0)
    f, g = N.DistributionFunctions(f0.copy()), N.DistributionFunctions(g0.copy())
    with N.Solver(spec) as sol:
        dt_out = N.CompressibleStep(sol).stream(f, g)
    assert dt_out == pytest.approx(dt, rel=1e-15)
    assert rel_l2(f.f, fo) <= TOL64
    assert rel_l2(g.f, go) <= TOL64


@pytest.mark.parametrize("in_init", [False, True])
def test_collide_all_matches_oracle(gpu_lib, in_init):
    st, mesh, dt, tau, spec = thermal_case((3, 4), 2, True, scaling=1.2)
    rho0, u0, T0, f0, g0 = thermal_state(mesh, st, seed=4, amp=5e-3)
    n = mesh.n_nodes
    fo, go = f0.copy(), g0.copy()
    ro, To, mo = np.zeros(n), np.zeros(n), np.zeros(n)
    uo = (u0 * 1.1).copy() if in_init else np.zeros((2, n))
    O.collide_compressible(st, tau, fo, go, ro, uo, To, mo, in_init=in_init)
    f, g = N.DistributionFunctions(f0.copy()), N.DistributionFunctions(g0.copy())
    rho, T, m = np.zeros(n), np.zeros(n), np.zeros(n)
    u = (u0 * 1.1).copy() if in_init else np.zeros((2, n))
    with N.Solver(spec) as sol:
        N.BGKCompressible(sol).collideAll(f, g, rho, u, T, m, None, in_init)
    assert rel_l2(f.f, fo) <= TOL64
    assert rel_l2(g.f, go) <= TOL64
    assert rel_l2(rho, ro) <= TOL64
    assert rel_l2(u, uo) <= 1e-11
    assert rel_l2(T, To) <= TOL64
    assert rel_l2(m, mo) <= 1e-9


@pytest.mark.parametrize("dg", [False, True])
def test_equilibrium_initialisation_matches_oracle(gpu_lib, dg):
    st, mesh, dt, tau, spec = thermal_case((4, 4), 4, dg, scaling=1.5)
    rho0, u0, T0, f0, g0 = thermal_state(mesh, st, seed=1, gamma=1.3)
    fo, go = O.thermal_init(st, rho0, u0, T0, gamma=1.3)
    with N.Solver(spec) as sol:
        sol.set_thermal(N.ThermalSettings(gamma=1.3))
        sol.init_thermal(rho0, u0, T0)
        f, g = sol.download_f(), sol.download_g()
        rho, u = sol.download_macro()
    assert rel_l2(f, fo) <= 1e-14
    assert rel_l2(g, go) <= 1e-14
    assert rel_l2(rho, rho0) == 0.0


def test_uniform_state_is_stationary_on_device(gpu_lib):
    st, mesh, dt, tau, spec = thermal_case((5, 4), 3, False, scaling=1.1)
    n = mesh.n_nodes
    rho = np.full(n, 0.9)
    u = np.stack([np.full(n, 0.07), np.full(n, -0.02)]) * st.scaling
    T = np.full(n, 1.05)
    with N.Solver(spec) as sol:
        sol.init_thermal(rho, u, T)
        f0 = sol.download_f()
        sol.step(5)
        f = sol.download_f()
        T1, m = sol.download_thermal()
    assert np.abs(f - f0).max() < 1e-13
    assert np.allclose(T1, 1.05, rtol=1e-13)
    assert np.abs(m).max() < 1e-12


@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
@pytest.mark.parametrize("T0", [1.1, 1.2])
def test_quartic_equilibrium_moment_recovery_on_device(gpu_lib, T0, precision):
    """The known answers of the reference's Equilibrium_D2Q19H_test and
    Equilibrium_D3Q45_test (test/collision_advanced/Equilibrium_test.cpp:
    111-206), run on this build's compressible stencil D2Q25H on the device:
    the quartic equilibrium at rho = 1, u = (0.1, 0.2), T = 1.1 (1.2), scaling
    1, c_s^2 = 1/3, returns its density and velocity (BOOST_CHECK_CLOSE
    10e-6 %, i.e. 1e-7 relative); here also its temperature, from the
    device collision's moments of f and g."""
    spec = N.SolverSpec(stencil="D2Q25H", order=2, cells=(2, 2), length=(1.0, 1.0), scaling=1.0, viscosity=1.0,
                        dt=0.1, collision="BGK_COMPRESSIBLE", precision=precision, topology="dg")
    st = O.stencil("D2Q25H", 1.0)
    with N.Solver(spec) as sol:
        n = sol.n_ref
        rho0 = np.ones(n)
        u0 = np.stack([np.full(n, 0.1), np.full(n, 0.2)])
        sol.init_thermal(rho0, u0, np.full(n, T0))
        f = sol.download_f()
        sol.collide()
        rho, u = sol.download_macro()
        T, _ = sol.download_thermal()
    e = st.e_unit[:, :2]
    r = f.sum(0)
    v = (e.T @ f) / r
    tol = 1e-7
    assert np.allclose(r, 1.0, rtol=tol, atol=0)
    assert np.allclose(v[0], 0.1, rtol=tol, atol=0) and np.allclose(v[1], 0.2, rtol=tol, atol=0)
    assert np.allclose(rho, 1.0, rtol=tol, atol=0)
    assert np.allclose(u[0], 0.1, rtol=tol, atol=0) and np.allclose(u[1], 0.2, rtol=tol, atol=0)
    assert np.allclose(T, T0, rtol=tol, atol=0)


def test_density_underflow_is_reported(gpu_lib):
    st, mesh, dt, tau, spec = thermal_case((2, 2), 2, True)
    n = mesh.n_nodes
    f = np.zeros((25, n))
    f[0] = 1.0
    f[0, 3] = 0.0
    with N.Solver(spec) as sol:
        sol.upload_f(f)
        sol.upload_g(np.zeros((25, n)))
        with pytest.raises(N.CollisionException):
            sol.collide()


# ---------------------------------------------------------------------------
# FP32 deviation storage (f - w_i, g - w_i g_ref in float) against the FP64
# oracle.  Tolerances: one step, relative L2 <= 2e-7 for f, g, rho and T and
# <= 2e-6 for u; 200 steps of the smooth state, <= 1e-5 for rho and T and
# <= 1e-4 for u (float rounding accumulates over the steps).
# ---------------------------------------------------------------------------

def _spec32(spec):
    spec.precision = "fp32dev"
    return spec


@pytest.mark.parametrize("dg", [False, True])
def test_fp32_step_close_to_oracle(gpu_lib, dg):
    st, mesh, dt, tau, spec = thermal_case((6, 6), 3, dg, scaling=1.2)
    rho0, u0, T0, f0, g0 = thermal_state(mesh, st, seed=9)
    S = O.SLOperator(mesh, st, dt)
    f1, g1 = f0.copy(), g0.copy()
    r1, u1, T1, m1 = S.step_compressible(f1, g1, tau)
    f, g, rho, u, T, m = _run(_spec32(spec), f0, g0)
    assert rel_l2(f, f1) <= 2e-7
    assert rel_l2(g, g1) <= 2e-7
    assert rel_l2(rho, r1) <= 2e-7
    assert rel_l2(T, T1) <= 2e-7
    assert rel_l2(u, u1) <= 2e-6


@pytest.mark.parametrize("settings", [N.ThermalSettings(), N.ThermalSettings(prandtl=0.71, prandtl_set=True,
                                                                             sutherland=True, gamma=1.67)],
                         ids=["default", "prandtl-sutherland-gamma"])
def test_fp32_200_steps_close_to_oracle(gpu_lib, settings):
    st, mesh, dt, tau, spec = thermal_case((8, 8), 2, True)
    rho0, u0, T0, f0, g0 = thermal_state(mesh, st, seed=12, gamma=settings.gamma, amp=0.0)
    S = O.SLOperator(mesh, st, dt)
    f1, g1 = f0.copy(), g0.copy()
    r1, u1, T1, m1 = S.step_compressible(f1, g1, tau, _th(settings), nsteps=200, nthreads=O.max_threads())
    f, g, rho, u, T, m = _run(_spec32(spec), f0, g0, settings, nsteps=200)
    assert rel_l2(rho, r1) <= 1e-5
    assert rel_l2(T, T1) <= 1e-5
    assert rel_l2(u, u1) <= 1e-4


@pytest.mark.parametrize("form", [0, 1, 2], ids=["registers", "smem-20-warps", "smem-24-warps"])
@pytest.mark.parametrize("settings", [N.ThermalSettings(), N.ThermalSettings(prandtl=0.71, prandtl_set=True,
                                                                             sutherland=True)],
                         ids=["default", "prandtl-sutherland"])
def test_fp32_kernel_forms_close_to_oracle(gpu_lib, form, settings):
    """The three forms of the FP32 fused kernel (nat_select_candidate: f and
    g in registers, or in shared memory with 20 / 24 resident warps)."""
    st, mesh, dt, tau, spec = thermal_case((6, 6), 3, True, scaling=1.2)
    rho0, u0, T0, f0, g0 = thermal_state(mesh, st, seed=9, gamma=settings.gamma)
    S = O.SLOperator(mesh, st, dt)
    f1, g1 = f0.copy(), g0.copy()
    r1, u1, T1, m1 = S.step_compressible(f1, g1, tau, _th(settings), nsteps=3)
    with N.Solver(_spec32(spec)) as sol:
        sol.set_thermal(settings)
        sol.select_candidate(form)
        assert sol.kernel_variant == (5 if form == 0 else 8 + form)
        sol.upload_f(f0)
        sol.upload_g(g0)
        sol.step(3)
        f, g = sol.download_f(), sol.download_g()
        T, _ = sol.download_thermal()
        n, ch = sol.autotune(2)
        rep = sol.autotune_report()
        assert n == 3 and len(rep) == 3 and sol.kernel_variant == rep[ch]["variant"]
        assert rel_l2(sol.download_f(), f) <= 1e-7  # the autotuner restored f
    assert rel_l2(f, f1) <= 1e-6
    assert rel_l2(g, g1) <= 1e-6
    assert rel_l2(T, T1) <= 1e-6


STAGED_CASES = [((5, 4), True), ((12, 6), True), ((12, 6), False)]


@pytest.mark.parametrize("cells,dg", STAGED_CASES, ids=["dg-15-nodes", "dg-36-nodes", "feq-24-nodes"])
def test_fp32_staged_form_order2_close_to_oracle(gpu_lib, cells, dg):
    """Order 2 has a fourth FP32 form (variant 14): the register form whose
    y-window rows arrive by cp.async one direction ahead.  Rows narrower
    than a warp (the buffer slots wrap more than once) and rows of two
    32-node segments, DG and FE_Q; the same values as the register form, and
    the autotuner offers all four forms."""
    st, mesh, dt, tau, spec = thermal_case(cells, 2, dg, scaling=1.2)
    rho0, u0, T0, f0, g0 = thermal_state(mesh, st, seed=21)
    S = O.SLOperator(mesh, st, dt)
    f1, g1 = f0.copy(), g0.copy()
    r1, u1, T1, m1 = S.step_compressible(f1, g1, tau, nsteps=3)
    out = {}
    for form in (0, 3):
        with N.Solver(_spec32(spec)) as sol:
            sol.select_candidate(form)
            assert sol.kernel_variant == (5 if form == 0 else 14)
            sol.upload_f(f0)
            sol.upload_g(g0)
            sol.step(3)
            out[form] = (sol.download_f(), sol.download_g(), sol.download_thermal()[0])
            if form == 3:
                n, ch = sol.autotune(2)
                rep = sol.autotune_report()
                assert n == 4 and [r["variant"] for r in rep] == [5, 9, 10, 14]
                assert sol.kernel_variant == rep[ch]["variant"]
    f, g, T = out[3]
    assert rel_l2(f, f1) <= 1e-6
    assert rel_l2(g, g1) <= 1e-6
    assert rel_l2(T, T1) <= 1e-6
    for a, b in zip(out[3], out[0]):
        assert rel_l2(a, b) <= 1e-7


def test_fp32_initialisation_and_uniform_state(gpu_lib):
    st, mesh, dt, tau, spec = thermal_case((4, 4), 2, False, scaling=1.1)
    n = mesh.n_nodes
    rho = np.full(n, 1.2)
    u = np.stack([np.full(n, 0.05), np.full(n, 0.02)]) * st.scaling
    T = np.full(n, 0.9)
    fo, go = O.thermal_init(st, rho, u, T)
    with N.Solver(_spec32(spec)) as sol:
        sol.init_thermal(rho, u, T)
        f, g = sol.download_f(), sol.download_g()
        sol.step(10)
        f10 = sol.download_f()
        T10, _ = sol.download_thermal()
    assert rel_l2(f, fo) <= 1e-7 and rel_l2(g, go) <= 1e-7
    assert rel_l2(f10, fo) <= 1e-6
    assert np.allclose(T10, 0.9, rtol=1e-6)
