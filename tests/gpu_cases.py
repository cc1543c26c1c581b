"""Shared helpers of the GPU parity tests: a seeded periodic state, the
oracle's reference step, and relative L2 norms."""
import math

import numpy as np

import natrium_gb300 as N
import oracle as O


def rel_l2(a, b):
    return float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b ** 2)))


def make_case(stencil, N_cells, p, dg=False, model="BGK_STANDARD", Ma=0.1, nu=1e-2, precision="fp64",
              L=2 * math.pi, cfl=0.4):
    st = O.stencil(stencil, math.sqrt(3) / Ma)
    dim = st.D
    mesh = O.Mesh(dim, tuple(N_cells), p, dg, (L, L, L))
    dt = O.time_step(mesh.h_min(), p, st.max_speed, cfl)
    tau = nu / (dt * st.cs2) + 0.5
    spec = N.SolverSpec(stencil=stencil, order=p, cells=tuple(N_cells), length=(L, L, L), scaling=st.scaling,
                        viscosity=nu, dt=dt, collision=model, precision=precision,
                        topology="dg" if dg else "feq")
    return st, mesh, dt, tau, spec


def periodic_state(mesh, st, seed=0, amp=0.05):
    import importlib.util, os
    here = os.path.dirname(os.path.abspath(__file__))
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(here, "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg.periodic_field(mesh, st, seed, amp)


def oracle_step(S, st, model, tau, f, nsteps=1):
    f = np.ascontiguousarray(f.copy())
    rho = np.zeros(f.shape[1])
    u = np.zeros((st.D, f.shape[1]))
    for _ in range(nsteps):
        f = S.stream(f)
        O.collide(st, model, tau, f, rho, u)
    return f, rho, u


# ---------------------------------------------------------------------------
# compressible two-population model (D2Q25H)
# ---------------------------------------------------------------------------

def thermal_case(N_cells, p, dg=True, scaling=1.0, nu=1e-3, L=1.0, cfl=0.4):
    st = O.stencil("D2Q25H", scaling)
    mesh = O.Mesh(2, tuple(N_cells), p, dg, (L, L, L))
    dt = O.time_step(mesh.h_min(), p, st.max_speed, cfl)
    tau = nu / (dt * st.cs2) + 0.5
    spec = N.SolverSpec(stencil="D2Q25H", order=p, cells=tuple(N_cells), length=(L, L), scaling=scaling,
                        viscosity=nu, dt=dt, collision="BGK_COMPRESSIBLE", precision="fp64",
                        topology="dg" if dg else "feq")
    return st, mesh, dt, tau, spec


def thermal_state(mesh, st, seed=0, gamma=1.4, amp=1e-3):
    """Smooth periodic rho, u (scaled), T on the support points, the
    equilibrium f, g of the oracle, and a seeded non-equilibrium perturbation."""
    X = mesh.coords()
    k = 2 * math.pi / mesh.L[0]
    x, y = X[:, 0] * k, X[:, 1] * k
    rho = 1.0 + 0.1 * np.sin(x) * np.cos(y)
    u = np.stack([0.1 * np.sin(x + 0.3) * np.cos(y), -0.08 * np.cos(x) * np.sin(2 * y)]) * st.scaling
    T = 1.0 + 0.1 * np.cos(x - 0.2) * np.sin(y + 0.1)
    f, g = O.thermal_init(st, rho, u, T, gamma)
    rng = np.random.default_rng(seed)
    # perturb consistently on periodic duplicates of the FE_Q lattice
    pf = rng.standard_normal(f.shape)
    pg = rng.standard_normal(g.shape)
    if not mesh.dg:
        nx, ny = mesh.nodes_per_axis(0), mesh.nodes_per_axis(1)
        for a in (pf, pg):
            v = a.reshape(a.shape[0], ny, nx)
            v[:, :, nx - 1] = v[:, :, 0]
            v[:, ny - 1, :] = v[:, 0, :]
    f = f * (1.0 + amp * pf)
    g = g * (1.0 + amp * pg)
    return rho, u, T, np.ascontiguousarray(f), np.ascontiguousarray(g)
