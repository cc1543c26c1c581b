"""Known answers and invariants of the compressible two-population oracle (D2Q25H).

The reference states these in its own tests or they follow from its formulas:
  * D2Q25H construction and scaled construction (stencils/D2Q25H_test.cpp:25-62);
  * the quartic equilibrium returns the density and velocity it was built
    from (collision_advanced/Equilibrium_test.cpp:111-150, written there for
    D2Q19V and D3Q45; restated for D2Q25H with the same state rho = 1,
    u = (0.1, 0.2), T = 1.1 and BOOST_CHECK_CLOSE tolerance 10e-6 %);
  * calculateTemperature of (f^eq, g^eq) returns T (AuxiliaryCollisionFunctions.h:289-307
    with g^eq = f^eq T (2 C_v - D), :420-431), so the equilibrium is a fixed
    point of relaxWithG;
  * relaxWithG conserves mass, momentum and total energy sum(|e|^2 f / c_s^2 + g),
    with and without the Prandtl correction and the Sutherland law;
  * the initialisation's tensor form of the quartic equilibrium
    (CompressibleCFDSolver.h:790-840) equals the collision's expanded form
    (Equilibria.h:130-267);
  * the semi-Lagrangian operator of D2Q25H reproduces a constant field (A 1 = 1,
    the SemiLagrangian{2,3}D_ConstantStreaming_test criterion).
"""
import math

import numpy as np
import pytest

import oracle as O


def _state(n, seed=0):
    rng = np.random.default_rng(seed)
    rho = 1.0 + 0.2 * rng.random(n)
    u = 0.15 * (rng.random((2, n)) - 0.5)
    T = 0.9 + 0.3 * rng.random(n)
    return rho, u, T


def test_d2q25h_construction():
    st = O.stencil("D2Q25H", 1.0)
    assert (st.D, st.Q) == (2, 25)
    assert st.cs2 == pytest.approx(1.0 / 3.0, rel=1e-8)
    assert math.sqrt(st.cs2) == pytest.approx(math.sqrt(1.0 / 3.0), rel=1e-8)
    sc = O.stencil("D2Q25H", 0.5)
    assert sc.cs2 == pytest.approx(0.25 / 3.0, rel=1e-8)
    assert np.allclose(sc.e, 0.5 * st.e, rtol=0, atol=1e-15)


def test_d2q25h_lattice_moments():
    st = O.stencil("D2Q25H", 1.0)
    e, w = st.e_unit[:, :2], st.w
    assert w.sum() == pytest.approx(1.0, abs=1e-14)
    cs2 = 1.0 / 3.0
    m2 = np.einsum("i,ia,ib->ab", w, e, e)
    assert np.allclose(m2, cs2 * np.eye(2), atol=1e-14)
    m4 = np.einsum("i,ia,ib,ic,id->abcd", w, e, e, e, e)
    d = np.eye(2)
    iso = cs2 ** 2 * (np.einsum("ab,cd->abcd", d, d) + np.einsum("ac,bd->abcd", d, d) + np.einsum("ad,bc->abcd", d, d))
    assert np.allclose(m4, iso, atol=1e-14)
    # odd moments vanish
    assert np.allclose(np.einsum("i,ia->a", w, e), 0, atol=1e-15)
    assert np.allclose(np.einsum("i,ia,ib,ic->abc", w, e, e, e), 0, atol=1e-15)


def test_quartic_equilibrium_recovers_density_and_velocity():
    st = O.stencil("D2Q25H", 1.0)
    rho = np.array([1.0])
    u = np.array([[0.1], [0.2]])
    T = np.array([1.1])
    feq = O.thermal_feq(st, rho, u, T)[:, 0]
    r = feq.sum()
    v = (st.e_unit[:, :2] * feq[:, None]).sum(0) / r
    assert r == pytest.approx(1.0, rel=1e-7)
    assert v[0] == pytest.approx(0.1, rel=1e-7)
    assert v[1] == pytest.approx(0.2, rel=1e-7)


def test_quartic_equilibrium_hermite_moments():
    st = O.stencil("D2Q25H", 1.0)
    rho, u, T = _state(7, seed=3)
    feq = O.thermal_feq(st, rho, u, T)
    e = st.e_unit[:, :2]
    cs2 = 1.0 / 3.0
    d = np.eye(2)
    for k in range(rho.size):
        f = feq[:, k]
        uu = u[:, k]
        m2 = np.einsum("i,ia,ib->ab", f, e, e)
        assert np.allclose(m2, rho[k] * (np.outer(uu, uu) + cs2 * T[k] * d), atol=1e-14)
        m3 = np.einsum("i,ia,ib,ic->abc", f, e, e, e)
        ref3 = rho[k] * (np.einsum("a,b,c->abc", uu, uu, uu) + cs2 * T[k] * (
            np.einsum("a,bc->abc", uu, d) + np.einsum("b,ac->abc", uu, d) + np.einsum("c,ab->abc", uu, d)))
        assert np.allclose(m3, ref3, atol=1e-14)


def test_init_tensor_form_equals_collision_form():
    st = O.stencil("D2Q25H", 1.7)
    rho, u, T = _state(50, seed=1)
    f, g = O.thermal_init(st, rho, u * st.scaling, T)
    feq = O.thermal_feq(st, rho, u * st.scaling, T)
    assert np.abs(f - feq).max() <= 1e-14
    C_v = 1.0 / (1.4 - 1.0)
    assert np.allclose(g, f * T * (2 * C_v - 2), rtol=1e-15, atol=0)


@pytest.mark.parametrize("th", [O.Thermal(), O.Thermal(prandtl=0.71, prandtl_set=True),
                                O.Thermal(sutherland=True), O.Thermal(gamma=1.67)])
def test_equilibrium_is_fixed_point(th):
    st = O.stencil("D2Q25H", 1.3)
    rho, u, T = _state(20, seed=2)
    f, g = O.thermal_init(st, rho, u * st.scaling, T, gamma=th.gamma)
    f0, g0 = f.copy(), g.copy()
    r, uu, TT, m = np.zeros(20), np.zeros((2, 20)), np.zeros(20), np.zeros(20)
    O.collide_compressible(st, 0.8, f, g, r, uu, TT, m, th)
    assert np.allclose(r, rho, rtol=1e-14)
    assert np.allclose(uu, u * st.scaling, atol=1e-14)
    assert np.allclose(TT, T, rtol=1e-13)
    assert np.abs(m).max() < 1e-12
    assert np.abs(f - f0).max() < 1e-14 and np.abs(g - g0).max() < 1e-13


@pytest.mark.parametrize("th", [O.Thermal(), O.Thermal(prandtl=0.71, prandtl_set=True),
                                O.Thermal(sutherland=True), O.Thermal(prandtl=2.0, prandtl_set=True,
                                                                      sutherland=True)])
def test_collision_invariants(th):
    st = O.stencil("D2Q25H", 1.0)
    n = 40
    rho, u, T = _state(n, seed=4)
    f, g = O.thermal_init(st, rho, u, T, gamma=th.gamma)
    rng = np.random.default_rng(5)
    f *= 1.0 + 0.02 * (rng.random(f.shape) - 0.5)
    g *= 1.0 + 0.02 * (rng.random(g.shape) - 0.5)
    e = st.e_unit[:, :2]
    cs2 = 1.0 / 3.0
    e2 = (e * e).sum(1)

    def inv(f, g):
        return f.sum(0), e.T @ f, (e2[:, None] * f).sum(0) / cs2 + g.sum(0)

    m0, j0, E0 = inv(f, g)
    fb, gb = f.copy(), g.copy()
    r, uu, TT, mk = np.zeros(n), np.zeros((2, n)), np.zeros(n), np.zeros(n)
    O.collide_compressible(st, 0.9, f, g, r, uu, TT, mk, th)
    m1, j1, E1 = inv(f, g)
    assert np.allclose(m1, m0, rtol=1e-14)
    assert np.allclose(j1, j0, atol=1e-14)
    assert np.allclose(E1, E0, rtol=1e-13)
    assert np.abs(f - fb).max() > 1e-6  # something relaxed
    assert (mk > 0).all()
    # the Knudsen estimate of the input state
    feq = O.thermal_feq(st, r, uu, TT)
    kn = (np.abs(fb - feq) / st.w[:, None]).sum(0) / st.Q
    assert np.allclose(mk, kn, rtol=1e-12)


@pytest.mark.parametrize("dg", [False, True])
@pytest.mark.parametrize("p", [1, 2, 3])
def test_d2q25h_constant_streaming(p, dg):
    st = O.stencil("D2Q25H", 1.5)
    m = O.Mesh(2, (4, 4), p, dg, (1.0, 1.0))
    dt = O.time_step(m.h_min(), p, st.max_speed, 0.4)
    sl = O.SLOperator(m, st, dt)
    f = np.ones((25, m.n_nodes))
    assert np.abs(sl.stream(f) - 1.0).max() < 1e-13
    assert sl.lifetime_hits == 0


def test_uniform_state_is_stationary():
    st = O.stencil("D2Q25H", 1.2)
    m = O.Mesh(2, (3, 3), 2, True, (1.0, 1.0))
    n = m.n_nodes
    dt = O.time_step(m.h_min(), 2, st.max_speed, 0.4)
    sl = O.SLOperator(m, st, dt)
    rho = np.full(n, 1.1)
    u = np.stack([np.full(n, 0.05), np.full(n, -0.03)]) * st.scaling
    T = np.full(n, 0.95)
    f, g = O.thermal_init(st, rho, u, T)
    f0, g0 = f.copy(), g.copy()
    tau = 1e-3 / (dt * st.cs2) + 0.5
    r, uu, TT, mk = sl.step_compressible(f, g, tau, nsteps=3)
    assert np.abs(f - f0).max() < 1e-13 and np.abs(g - g0).max() < 1e-12
    assert np.allclose(TT, 0.95, rtol=1e-13)


def test_density_underflow_raises():
    st = O.stencil("D2Q25H", 1.0)
    n = 4
    f = np.zeros((25, n))
    g = np.zeros((25, n))
    f[0] = 1.0
    f[0, 2] = 0.0
    z = lambda *s: np.zeros(s)
    with pytest.raises(O.DensityZeroError):
        O.collide_compressible(st, 0.8, f, g, z(n), z(2, n), z(n), z(n))
