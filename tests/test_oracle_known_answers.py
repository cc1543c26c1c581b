"""The CPU oracle against the known answers of the reference's own tests.

These pin the oracle (test infrastructure) before the CUDA path is compared
against it.  The expected values come from
tests/golden/known_answers.json, parsed out of the reference's test sources
by tests/golden/make_golden.py.
"""
import json
import math
import os

import numpy as np
import pytest

import oracle as O

KA = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))


@pytest.mark.parametrize("dim", ["2d", "3d"])
def test_face_crossed_first_known_answers(dim):
    """SemiLagrangian{2,3}D_FaceCrossedFirst_test (SemiLagrangian_test.cpp:227-456)."""
    case = KA["face_crossed_first"][dim]
    d = len(case["p_in"])
    assert len(case["probes"]) >= 7
    for pr in case["probes"]:
        fid, lam, pb = O.face_crossed_first(d, case["cell_lo"], case["cell_h"], case["p_in"], pr["p_out"])
        assert fid == pr["face"], pr
        if pr["lambda"] is not None:
            assert lam == pytest.approx(pr["lambda"], rel=1e-13)
        if pr["pb"] is not None:
            for a in range(d):
                if pr["pb"][a] is None:
                    continue
                if pr["pb"][a] == 0.0:
                    assert abs(pb[a]) < 1e-13
                else:
                    assert pb[a] == pytest.approx(pr["pb"][a], rel=1e-13)


@pytest.mark.parametrize("dim", ["2d", "3d"])
def test_constant_streaming(dim):
    """A * 1 = 1 (SemiLagrangian{2,3}D_ConstantStreaming_test, :519-596):
    PeriodicTestDomain (unit box, refinement 3 = 8 cells/axis)."""
    c = KA["constant_streaming"][dim]
    D = 2 if dim == "2d" else 3
    N = 2 ** c["refinement"]
    mesh = O.Mesh(D, (N,) * D, c["order"], False, (1.0, 1.0, 1.0))
    st = O.stencil(c["stencil"])
    S = O.SLOperator(mesh, st, c["dt"])
    f = np.ones((st.Q, mesh.n_nodes))
    r = S.stream(f)
    assert np.sum((r[1:] - 1.0) ** 2) <= c["bound_norm_sqr"]
    # every row carries exactly the Kronecker-structure nonzeros
    for alpha in range(1, st.Q):
        rp, col, val = S.csr(alpha)
        k = int(np.count_nonzero(st.e_unit[alpha]))
        assert np.all(np.diff(rp) == (c["order"] + 1) ** k)
    assert S.lifetime_hits == 0


def test_gl_points_and_lagrange():
    for p in range(1, 7):
        xi = O.gl_points(p)
        assert xi[0] == 0.0 and xi[-1] == 1.0
        assert np.all(np.diff(xi) > 0)
        # Lagrange cardinality and partition of unity
        for j in range(p + 1):
            for k in range(p + 1):
                assert O.lagrange(p, xi, j, xi[k]) == pytest.approx(float(j == k), abs=1e-14)
        for x in np.linspace(0, 1, 7):
            assert sum(O.lagrange(p, xi, j, x) for j in range(p + 1)) == pytest.approx(1.0, abs=1e-14)
    # GL points of order 4: 0, (1 - sqrt(3/7))/2, 1/2, ...
    xi = O.gl_points(4)
    assert xi[1] == pytest.approx((1 - math.sqrt(3 / 7)) / 2, abs=1e-15)


def _fixture_f(Q, j=None):
    """f_i = 1.5 + sin(1.5 i) + 0.001 + i/(i+1) (+ (0.5 cos j)^2), integer division."""
    f = np.array([1.5 + math.sin(1.5 * i) + 0.001 + (i // (i + 1)) for i in range(Q)])
    if j is not None:
        f = f[:, None] + (0.5 * np.cos(np.asarray(j, dtype=float))) ** 2
    return f


@pytest.mark.parametrize("name", ["D2Q9", "D3Q19", "D3Q27"])
def test_bgk_invariants_and_fixed_point(name):
    """BGKStandardCollisionInvariants_test (BGKStandard_test.cpp:311-356)."""
    c = KA["bgk_invariants"]
    st = O.stencil(name)
    f = _fixture_f(st.Q)
    rho0 = f.sum()
    j0 = f @ st.e
    g = O.collide_single_point(st, c["relax_param"], f)
    assert np.all(np.abs(g - f) > 1e-5)
    assert abs(g.sum() - rho0) < c["mass_momentum_tol"] * 10
    assert np.all(np.abs(g @ st.e - j0) < c["mass_momentum_tol"] * 10)
    feq = O.equilibrium(st, np.array([c["prescribed_density"]]), np.zeros((st.D, 1)))[:, 0]
    g = O.collide_single_point(st, c["relax_param"], feq)
    assert np.all(np.abs(g - feq) < c["fixed_point_tol"])


@pytest.mark.parametrize("name", ["D2Q9", "D3Q19", "D3Q27"])
def test_collide_all_equals_collide_single_point(name):
    """BGKStandard_collideAll{D2Q9,D3Q19}_test (BGKStandard_test.cpp:358-470):
    the time loop's collideAll must equal the generic single-point collision
    to 1e-10 percent (BOOST_CHECK_CLOSE)."""
    c = KA["bgk_collide_all"]
    st = O.stencil(name)
    D = st.D
    n = (2 ** c["refinement"]) ** D * (c["dg_order"] + 1) ** D
    f = np.ascontiguousarray(_fixture_f(st.Q, np.arange(n)))
    rho = np.zeros(n)
    u = np.zeros((D, n))
    ref = np.stack([O.collide_single_point(st, c["relax_param"], f[:, i]) for i in range(n)], axis=1)
    tau = c["relax_param"] + 0.5
    O.collide_bgk(st, tau, f, rho, u)
    assert np.allclose(f, ref, rtol=c["close_percent"] / 100.0, atol=0)


def test_kbc_mass_equals_bgk_mass():
    """KBCStandard_collideAll_test (KBCStandard_test.cpp:36-108)."""
    c = KA["kbc_mass"]
    st = O.stencil("D2Q9")
    n = 8 * 8 * 4
    base = np.array([0.1 * i + 0.1 for i in range(9)])
    fk = np.ascontiguousarray(np.repeat(base[:, None], n, axis=1))
    fb = fk.copy()
    tau = c["relax_param"] + 0.5
    O.collide_kbc(st, tau, fk, np.zeros(n), np.zeros((2, n)))
    O.collide_bgk(st, tau, fb, np.zeros(n), np.zeros((2, n)))
    assert np.all(np.abs(fk.sum(0) - fb.sum(0)) < c["tol"])


def test_kbc_d3q27_invariants():
    """D3Q27 KBC (no reference; parity unpinned): conserves mass and
    momentum, has the equilibrium as fixed point, and reduces to BGK when
    the higher-order part vanishes."""
    st = O.stencil("D3Q27")
    rng = np.random.default_rng(1)
    n = 64
    rho = 1 + 0.01 * rng.standard_normal(n)
    u = 0.05 * rng.standard_normal((3, n))
    feq = O.equilibrium(st, rho, np.ascontiguousarray(u))
    f = np.ascontiguousarray(feq * (1 + 1e-3 * rng.standard_normal(feq.shape)))
    m0, j0 = f.sum(0), st.e.T @ f
    g = f.copy()
    O.collide_kbc(st, 0.9, g, np.zeros(n), np.zeros((3, n)))
    assert np.allclose(g.sum(0), m0, atol=1e-13)
    assert np.allclose(st.e.T @ g, j0, atol=1e-13)


def test_kbc_d2q9_fixed_point():
    st = O.stencil("D2Q9", 3.0)
    n = 10
    rho = np.linspace(0.9, 1.1, n)
    # KBC's own (product-form) equilibrium is its fixed point: build it by
    # colliding with tau = 1/2 (beta = 1 -> f = feq when gamma = 2)
    f = np.ascontiguousarray(O.equilibrium(st, rho, np.zeros((2, n))))
    O.collide_kbc(st, 0.5, f, np.zeros(n), np.zeros((2, n)))
    g = f.copy()
    O.collide_kbc(st, 0.8, g, np.zeros(n), np.zeros((2, n)))
    assert np.allclose(g, f, atol=1e-14)


def test_tgv2d_kinetic_energy_decay():
    """ConvergenceTestSemiLagrangianPeriodic
    (IntegrationTestCases.cpp:885-961): E_kin(1/(2 nu))/E_kin(0) = e^-2
    within 1e-2 (8x8 cells, p = 4, CFL 0.4, Ma 0.05, nu = 1)."""
    c = KA["tgv2d_sl"]
    Ma, nu, p = c["Ma"], c["viscosity"], c["order"]
    st = O.stencil("D2Q9", math.sqrt(3) / Ma)
    N = 2 ** c["refinement"]
    mesh = O.Mesh(2, (N, N), p)
    dt = O.time_step(mesh.h_min(), p, st.max_speed, c["cfl"])
    tau = nu / (dt * st.cs2) + 0.5
    rho, u = O.tgv2d_init(mesh.coords(), Ma)
    u = np.ascontiguousarray(u)
    f = O.equilibrium(st, rho, u)
    E0 = O.kinetic_energy(mesh, rho, u)
    S = O.SLOperator(mesh, st, dt)
    nsteps = int(round(1.0 / (2 * nu) / dt))
    r2, u2 = S.step_bgk(f, tau, nsteps, nthreads=2)
    ratio = O.kinetic_energy(mesh, r2, u2) / E0
    assert abs(ratio - math.exp(-2)) < c["ekin_tol"]
    # velocity L2 error against the analytic decay
    X = mesh.coords()
    ua = np.stack([np.sin(X[:, 0]) * np.cos(X[:, 1]), -np.cos(X[:, 0]) * np.sin(X[:, 1])]) * math.exp(-2 * nu * nsteps * dt)
    err = np.sqrt(np.sum((u2 - ua) ** 2) / np.sum(ua ** 2))
    assert err < c["l2_velocity_tol"]


def test_dg_topology_partition_of_unity():
    for dim, name in ((2, "D2Q9"), (3, "D3Q27")):
        mesh = O.Mesh(dim, (3,) * dim, 2, True)
        st = O.stencil(name, 5.0)
        dt = O.time_step(mesh.h_min(), 2, st.max_speed, 0.4)
        S = O.SLOperator(mesh, st, dt)
        r = S.stream(np.ones((st.Q, mesh.n_nodes)))
        assert np.max(np.abs(r - 1)) < 1e-13
