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
