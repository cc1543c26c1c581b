"""Initial states of the benchmark flows (host setup, FP64 numpy).

Equivalent of CFDSolver::initializeDistributions with the EQUILIBRIUM
option (solver/CFDSolver.cpp:1103-1130): evaluate the problem's initial
density and velocity at the support points and set f = f^eq(rho, u).

Node coordinates follow the lattice layout of include/natgpu.h (reference
layout, x fastest; FE_Q keeps the periodic duplicate nodes).
"""
from __future__ import annotations

import math

import numpy as np

# unit velocities and weights (stencils/D2Q9.cpp:40-61, D3Q19.cpp:37-67,
# D3Q27.cpp:36-112 of the reference)
_E = {
    "D2Q9": [(0, 0, 0), (1, 0, 0), (0, 1, 0), (-1, 0, 0), (0, -1, 0), (1, 1, 0), (-1, 1, 0), (-1, -1, 0),
             (1, -1, 0)],
    "D3Q19": [(0, 0, 0), (1, 0, 0), (0, 0, 1), (-1, 0, 0), (0, 0, -1), (0, -1, 0), (0, 1, 0), (1, 0, 1),
              (-1, 0, 1), (-1, 0, -1), (1, 0, -1), (1, -1, 0), (1, 1, 0), (-1, 1, 0), (-1, -1, 0),
              (0, -1, 1), (0, 1, 1), (0, 1, -1), (0, -1, -1)],
    "D3Q27": [(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1), (0, 1, 1),
              (0, -1, -1), (0, 1, -1), (0, -1, 1), (1, 0, 1), (-1, 0, -1), (1, 0, -1), (-1, 0, 1),
              (1, 1, 0), (-1, -1, 0), (1, -1, 0), (-1, 1, 0), (1, 1, 1), (-1, -1, -1), (1, 1, -1),
              (-1, -1, 1), (1, -1, 1), (-1, 1, -1), (1, -1, -1), (-1, 1, 1)],
}


def _weights(name: str) -> np.ndarray:
    e = np.array(_E[name])
    nz = np.count_nonzero(e, axis=1)
    if name == "D2Q9":
        table = {0: 4 / 9, 1: 1 / 9, 2: 1 / 36}
    elif name == "D3Q19":
        table = {0: 1 / 3, 1: 1 / 18, 2: 1 / 36}
    else:
        table = {0: 8 / 27, 1: 2 / 27, 2: 1 / 54, 3: 1 / 216}
    return np.array([table[int(k)] for k in nz])


def unit_velocities(name: str) -> np.ndarray:
    return np.array(_E[name], dtype=np.float64)


def gl_points(p: int) -> np.ndarray:
    """Gauss-Lobatto points on [0, 1]: end points and the roots of P_p'."""
    if p == 1:
        return np.array([0.0, 1.0])
    P = np.polynomial.legendre.Legendre.basis(p)
    r = np.sort(np.real(P.deriv().roots()))
    xi = np.concatenate([[0.0], (r + 1) / 2, [1.0]])
    xi = 0.5 * (xi + (1 - xi[::-1]))
    return xi


def node_coords(cells, order: int, lengths, topology: str = "feq") -> np.ndarray:
    """(n_ref, 3) coordinates of the lattice nodes."""
    dim = len(cells)
    xi = gl_points(order)
    axes = []
    for a in range(3):
        if a >= dim:
            axes.append(np.zeros(1))
            continue
        N, h = cells[a], lengths[a] / cells[a]
        if topology == "dg":
            x = np.array([(c + xi[l]) * h for c in range(N) for l in range(order + 1)])
        else:
            x = np.array([(c + xi[l]) * h for c in range(N) for l in range(order)] + [N * h])
        axes.append(x)
    Z, Y, X = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)


def mapped_node_coords(vertices, order: int, topology: str = "feq") -> np.ndarray:
    """(n_ref, 3) coordinates of the lattice nodes of a MappingQ1 grid: the
    multilinear map of each cell (vertices of shape (N0+1, N1+1[, N2+1], dim))
    at its Gauss-Lobatto points; FE_Q nodes on a cell face come from the
    lower cell except at the last face of an axis."""
    v = np.asarray(vertices, dtype=np.float64)
    dim = v.shape[-1]
    cells = tuple(s - 1 for s in v.shape[:dim])
    xi = gl_points(order)
    per = order + 1 if topology == "dg" else order
    idx = []
    for a in range(3):
        if a >= dim:
            idx.append((np.zeros(1, int), np.zeros(1)))
            continue
        n = cells[a] * per + (0 if topology == "dg" else 1)
        i = np.arange(n)
        c = np.minimum(i // per, cells[a] - 1)
        u = xi[i - c * per]
        idx.append((c, u))
    out = np.zeros((len(idx[2][0]), len(idx[1][0]), len(idx[0][0]), 3))
    for k in range(1 << dim):
        b = [(k >> a) & 1 for a in range(dim)]
        phi = [(u if b[a] else 1.0 - u) for a, (c, u) in enumerate(idx[:dim])]
        cidx = [c + b[a] for a, (c, u) in enumerate(idx[:dim])]
        if dim == 2:
            w = phi[1][:, None] * phi[0][None, :]
            vv = v[cidx[0][None, :], cidx[1][:, None]]
            out[0, :, :, :2] += w[..., None] * vv
        else:
            w = phi[2][:, None, None] * phi[1][None, :, None] * phi[0][None, None, :]
            vv = v[cidx[0][None, None, :], cidx[1][None, :, None], cidx[2][:, None, None]]
            out[..., :3] += w[..., None] * vv
    return out.reshape(-1, 3)


def wavy_grid(cells, lengths, amplitude: float) -> np.ndarray:
    """A smoothly deformed periodic grid: the box vertices moved by
    amplitude * h_a * (1 + 0.3 a) * prod_b sin(2 pi x_b / L_b) along each
    axis a (zero on every face, so each axis keeps the translation L_a e_a)."""
    dim = len(cells)
    axes = [np.linspace(0.0, lengths[a], cells[a] + 1) for a in range(dim)]
    X = np.stack(np.meshgrid(*axes, indexing="ij"), -1)
    ph = np.ones(X.shape[:-1])
    for a in range(dim):
        ph = ph * np.sin(2 * math.pi * X[..., a] / lengths[a])
    V = X.copy()
    for a in range(dim):
        V[..., a] += amplitude * lengths[a] / cells[a] * (1 + 0.3 * a) * ph
    return V


def lubrication_sine_grid(length: float = 1.0, average_height: float = 0.25, amplitude: float = 0.05,
                          cell_aspect_ratio: float = 1.0, refinement: int = 2, roughness_height: float = 0.0,
                          roughness_length_ratio: int = 1) -> np.ndarray:
    """Vertices of the LubricationSine channel (benchmarks/LubricationSine.cpp:33-54,
    95-104, LubricationSine.h:80-105): a box [0, L] x [0, H] of
    L / H / aspect x 1 cells refined `refinement` times, mapped by
    x -> x + lambda A / (2 pi H) sin(2 pi x / lambda) and
    y -> y_r(y) / H * (H + A cos(2 pi x' / lambda) + R cos(2 pi x' ratio / lambda)),
    y_r(y) = H (1/2 + tanh(pi (y / H - 1/2)) / (2 tanh(pi / 2))), lambda = L.
    x is periodic; the bottom (y = 0) and the wavy top are the walls."""
    H, A, lam = average_height, amplitude, length
    nx = int(length / average_height / cell_aspect_ratio) * 2 ** refinement
    ny = 2 ** refinement
    x = np.linspace(0.0, length, nx + 1)
    y = np.linspace(0.0, H, ny + 1)
    X, Y = np.meshgrid(x, y, indexing="ij")
    xr = X + lam * A / H / (2 * math.pi) * np.sin(2 * math.pi * X / lam)
    yr = H * (0.5 + 0.5 * np.tanh((Y / H - 0.5) * math.pi) / math.tanh(0.5 * math.pi))
    upper = H + A * np.cos(2 * math.pi * xr / lam) + roughness_height * np.cos(
        2 * math.pi * xr / (lam / roughness_length_ratio))
    return np.stack([xr, yr / H * upper], -1)


def sinusoidal_shear_grid(length: float = 1.0, average_height: float = 1.0, amplitude: float = 0.1,
                          cell_aspect_ratio: float = 1.0, refinement: int = 2) -> np.ndarray:
    """Vertices of the SinusoidalShear2D gap (benchmarks/SinusoidalShear2D.cpp:33-52 and
    .h:80-105): the unit square of 1 / aspect x 1 cells refined `refinement` times, mapped by
    x -> L x_r, x_r = x - 0.019 A / 0.49 sin(4 pi x), and
    y -> y_r(y) (H + A sin(2 pi x_r)), y_r(y) = 1/2 + tanh(pi (y - 1/2)) / (2 tanh(pi / 2)).
    x is periodic; the bottom (y = 0, moving) and the wavy top are walls."""
    H, A = average_height, amplitude
    nx = int(1.0 / cell_aspect_ratio) * 2 ** refinement
    ny = 2 ** refinement
    X, Y = np.meshgrid(np.linspace(0.0, 1.0, nx + 1), np.linspace(0.0, 1.0, ny + 1), indexing="ij")
    xr = X - 0.019 * A / 0.49 * np.sin(4 * math.pi * X)
    yr = 0.5 + 0.5 * np.tanh((Y - 0.5) * math.pi) / math.tanh(0.5 * math.pi)
    return np.stack([length * xr, yr * (H + A * np.sin(2 * math.pi * xr))], -1)


def lubrication_sine_velocity(X: np.ndarray, bottom_velocity: float, average_height: float, amplitude: float):
    """Initial velocity (LubricationSine.cpp:78-87): u = U (1 - y / (H - A))^2, v = 0."""
    upper = average_height - amplitude
    u = np.zeros((2, X.shape[0]))
    u[0] = bottom_velocity * (1.0 - X[:, 1] / upper) ** 2
    return u


def equilibrium(stencil: str, scaling: float, rho: np.ndarray, u_scaled: np.ndarray) -> np.ndarray:
    """Second-order equilibrium with scaled velocities (the legacy
    getEquilibriumDistribution, collision/BGKStandard.cpp:23-41)."""
    e = unit_velocities(stencil)[:, : u_scaled.shape[0]]
    w = _weights(stencil)
    u = u_scaled / scaling
    ue = 3.0 * (e @ u)
    uu = 1.5 * np.sum(u * u, axis=0)
    return np.ascontiguousarray(w[:, None] * rho[None, :] * (1 + ue * (1 + 0.5 * ue) - uu[None, :]))


def taylor_green_3d(X: np.ndarray, Ma: float):
    """TaylorGreenVortex3D initial state (benchmarks/TaylorGreenVortex3D.cpp:38-58):
    u = (sin x cos y cos z, -cos x sin y cos z, 0),
    rho = 1 + Ma^2 (cos 2x + cos 2y)(cos 2z + 2) / 16."""
    x, y, z = X[:, 0], X[:, 1], X[:, 2]
    u = np.stack([np.sin(x) * np.cos(y) * np.cos(z), -np.cos(x) * np.sin(y) * np.cos(z), np.zeros_like(x)])
    rho = 1.0 + Ma * Ma / 16.0 * (np.cos(2 * x) + np.cos(2 * y)) * (np.cos(2 * z) + 2)
    return rho, u


def taylor_green_2d(X: np.ndarray, Ma: float, L: float = 2 * math.pi, rho_sign: float = 1.0):
    """TaylorGreenVortex2D at t = 0 (benchmarks/TaylorGreenVortex2D.cpp:36-59):
    u = (sin x' cos y', -cos x' sin y'), rho = 1 + rho_sign Ma^2 (cos 2x' + cos 2y')/4,
    x' = 2 pi x / L.  rho_sign = +1 is the reference's sign."""
    k = 2 * math.pi / L
    x, y = X[:, 0] * k, X[:, 1] * k
    u = np.stack([np.sin(x) * np.cos(y), -np.cos(x) * np.sin(y)])
    rho = 1.0 + rho_sign * Ma * Ma * 0.25 * (np.cos(2 * x) + np.cos(2 * y))
    return rho, u


def shear_layer_2d(X: np.ndarray, kappa: float = 80.0, delta: float = 0.05, L: float = 1.0):
    """Double-periodic shear layer (benchmarks/ShearLayer2D.cpp:39-53 with
    u0 = 1): u = tanh(kappa (y - L/4)) for y <= L/2, tanh(kappa (3L/4 - y))
    above; v = delta sin(2 pi (x/L + 1/4)); rho = 1."""
    x, y = X[:, 0] / L, X[:, 1] / L
    ux = np.where(y <= 0.5, np.tanh(kappa * (y - 0.25)), np.tanh(kappa * (0.75 - y)))
    uy = delta * np.sin(2 * math.pi * (x + 0.25))
    return np.ones_like(x), np.stack([ux, uy])


# Four-quadrant 2-D Riemann problem on [0, 1]^2 (discontinuities at x = 1/2
# and y = 1/2); states (rho, u, v, p) per quadrant.
RIEMANN2D_QUADRANTS = {
    "upper_right": (1.5, 0.0, 0.0, 1.5),
    "upper_left": (0.5323, 1.206, 0.0, 0.3),
    "lower_left": (0.138, 1.206, 1.206, 0.029),
    "lower_right": (0.5323, 0.0, 1.206, 0.3),
}


def riemann_2d(X: np.ndarray, velocity_unit: float = 1.58, scaling: float = 1.0):
    """Initial rho, scaled u and lattice temperature of the four-quadrant
    Riemann problem at the points X.  A physical velocity u maps to the
    lattice velocity u / velocity_unit, and p / rho to the lattice temperature
    T = (p / rho) / (c_s^2 velocity_unit^2) with c_s^2 = 1/3 (T = 1 is the
    lattice reference temperature of the quartic equilibrium).  The
    compressible solver of the reference states its Riemann problem directly
    in these lattice units (benchmarks/Riemann2D.cpp:41-106)."""
    x, y = X[:, 0], X[:, 1]
    n = X.shape[0]
    rho = np.empty(n)
    u = np.empty((2, n))
    T = np.empty(n)
    right, up = x > 0.5, y > 0.5
    for mask, key in ((right & up, "upper_right"), (~right & up, "upper_left"), (~right & ~up, "lower_left"),
                      (right & ~up, "lower_right")):
        r, ux, uy, p = RIEMANN2D_QUADRANTS[key]
        rho[mask] = r
        u[0, mask] = ux / velocity_unit
        u[1, mask] = uy / velocity_unit
        T[mask] = 3.0 * (p / r) / velocity_unit ** 2
    return rho, u * scaling, T
