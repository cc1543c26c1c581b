"""CPU oracle for the semi-Lagrangian stream + collide path.

TEST INFRASTRUCTURE ONLY: a numpy/ctypes front-end for ``natoracle.c``, the
plain-C FP64 restatement of NATriuM's reference algorithm (see the header of
``natoracle.c`` for the reference file:line each function follows).  Only the
tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg and
reference arm may use it: to check results and as the timed CPU baseline.  The
product package ``natrium_gb300`` never imports it.

Parity status: pinned against the known answers and invariants of the
reference's own tests; the reference itself cannot be built or run (deal.II,
Trilinos, p4est, Boost and MPI are absent), so no reference-run outputs exist.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "natoracle.c")
_LIB = os.path.join(_HERE, "_build", "liboracle.so")

D2Q9, D3Q19, D3Q27, D2Q25H = 0, 1, 2, 3
STENCIL_IDS = {"D2Q9": D2Q9, "D3Q19": D3Q19, "D3Q27": D3Q27, "D2Q25H": D2Q25H}


def build(force: bool = False) -> str:
    """Compile natoracle.c into oracle/_build/liboracle.so (gcc, OpenMP)."""
    os.makedirs(os.path.dirname(_LIB), exist_ok=True)
    if force or not os.path.exists(_LIB) or os.path.getmtime(_LIB) < os.path.getmtime(_SRC):
        cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-o", _LIB, _SRC, "-lm"]
        subprocess.run(cmd, check=True)
    return _LIB


class _Mesh(C.Structure):
    _fields_ = [("dim", C.c_int), ("N", C.c_int * 3), ("p", C.c_int), ("dg", C.c_int),
                ("L", C.c_double * 3), ("bc", C.c_int * 6), ("uw", (C.c_double * 3) * 6),
                ("vtx", C.POINTER(C.c_double))]


# boundary kinds of the six faces x-, x+, y-, y+, z-, z+
BC_PERIODIC, BC_VELOCITY_BOUNCE_BACK, BC_DO_NOTHING = 0, 1, 2


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        L.orc_stencil.argtypes = [C.c_int, C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_int), dp, dp, dp, dp]
        L.orc_gl_points.argtypes = [C.c_int, dp]
        L.orc_lagrange.argtypes = [C.c_int, dp, C.c_int, C.c_double]
        L.orc_lagrange.restype = C.c_double
        L.orc_n_nodes.argtypes = [C.POINTER(_Mesh)]
        L.orc_n_nodes.restype = C.c_int64
        L.orc_node_coords.argtypes = [C.POINTER(_Mesh), dp]
        L.orc_face_crossed_first.argtypes = [C.c_int, dp, dp, dp, dp, dp, dp]
        L.orc_face_crossed_first.restype = C.c_int
        L.orc_sl_assemble.argtypes = [C.POINTER(_Mesh), C.c_int, C.c_double, C.c_double]
        L.orc_sl_assemble.restype = C.c_void_p
        L.orc_sl_free.argtypes = [C.c_void_p]
        L.orc_sl_nnz.argtypes = [C.c_void_p, C.c_int]
        L.orc_sl_nnz.restype = C.c_int64
        L.orc_sl_lifetime_hits.argtypes = [C.c_void_p]
        L.orc_sl_csr.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int32), dp]
        L.orc_sl_stream.argtypes = [C.c_void_p, dp, dp, C.c_int]
        L.orc_sl_stream_g.argtypes = [C.c_void_p, dp, dp, C.c_int]
        L.orc_sl_csr_dirs.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int32)]
        L.orc_sl_bconst.argtypes = [C.c_void_p, C.c_int, dp]
        L.orc_sl_wall_hits.argtypes = [C.c_void_p]
        L.orc_collide_bgk.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int64, dp, dp, dp, C.c_int, C.c_int]
        L.orc_collide_bgk_force.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int64, dp, dp, dp,
                                            C.c_int, C.c_int, dp, C.c_int]
        L.orc_equilibrium.argtypes = [C.c_int, C.c_double, C.c_int64, dp, dp, dp]
        L.orc_bgk_collide_single_point.argtypes = [C.c_int, C.c_double, C.c_double, dp]
        L.orc_collide_bgk_incompressible_d2q9.argtypes = [C.c_double, C.c_double, C.c_int64, dp, dp, dp, C.c_int]
        L.orc_collide_kbc_d2q9.argtypes = [C.c_double, C.c_double, C.c_int64, dp, dp, dp, C.c_int, dp]
        L.orc_collide_kbc_d3q27.argtypes = [C.c_double, C.c_double, C.c_int64, dp, dp, dp, C.c_int, dp]
        L.orc_step_bgk.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, dp, dp, dp, dp, C.c_int, C.c_int]
        L.orc_time_step.argtypes = [C.c_double, C.c_int, C.c_double, C.c_double]
        L.orc_time_step.restype = C.c_double
        L.orc_max_threads.restype = C.c_int
        L.orc_thermal_init.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int64, dp, dp, dp, dp, dp]
        L.orc_thermal_feq.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int64, dp, dp, dp, dp]
        L.orc_collide_compressible.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int,
                                               C.c_int, C.c_int, C.c_int64, dp, dp, dp, dp, dp, dp, C.c_int,
                                               C.c_int]
        L.orc_step_compressible.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                            C.c_int, C.c_int, C.c_int, dp, dp, dp, dp, dp, dp, dp, C.c_int,
                                            C.c_int]
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(C.c_double))


# --------------------------------------------------------------------------
# stencils, points, basis
# --------------------------------------------------------------------------

@dataclass
class Stencil:
    name: str
    id: int
    D: int
    Q: int
    scaling: float
    e: np.ndarray          # (Q, 3) scaled directions
    w: np.ndarray          # (Q,)
    cs2: float             # scaled c_s^2 = scaling^2 / 3
    max_speed: float       # sqrt(2) * scaling

    @property
    def e_unit(self):
        return self.e / self.scaling


def stencil(name: str, scaling: float = 1.0) -> Stencil:
    sid = STENCIL_IDS[name]
    D, Q = C.c_int(), C.c_int()
    e = np.zeros(3 * 32)
    w = np.zeros(32)
    cs2, vmax = C.c_double(), C.c_double()
    rc = lib().orc_stencil(sid, scaling, C.byref(D), C.byref(Q), _dp(e), _dp(w), C.byref(cs2), C.byref(vmax))
    assert rc == 0
    q = Q.value
    return Stencil(name, sid, D.value, q, scaling, e[: 3 * q].reshape(q, 3).copy(), w[:q].copy(), cs2.value, vmax.value)


def gl_points(p: int) -> np.ndarray:
    xi = np.zeros(p + 1)
    lib().orc_gl_points(p, _dp(xi))
    return xi


def lagrange(p: int, xi: np.ndarray, j: int, x: float) -> float:
    xi = np.ascontiguousarray(xi, dtype=np.float64)
    return lib().orc_lagrange(p, _dp(xi), j, x)


def face_crossed_first(dim, lo, h, p_in, p_out):
    """SemiLagrangian::faceCrossedFirst for an axis-aligned cell.
    Returns (face_id, lambda, p_boundary)."""
    arr = lambda v: np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(-1))
    lo, h, pi, po = arr(lo), arr(h), arr(p_in), arr(p_out)
    pb = np.zeros(3)
    lam = C.c_double(0)
    fid = lib().orc_face_crossed_first(dim, _dp(lo), _dp(h), _dp(pi), _dp(po), _dp(pb), C.byref(lam))
    return fid, lam.value, pb[:dim].copy()


def time_step(dx_min: float, p: int, max_speed: float, cfl: float) -> float:
    return lib().orc_time_step(dx_min, p, max_speed, cfl)


# --------------------------------------------------------------------------
# mesh and semi-Lagrangian operator
# --------------------------------------------------------------------------

@dataclass
class Mesh:
    dim: int
    N: tuple
    p: int
    dg: bool = False
    L: tuple = (2 * math.pi, 2 * math.pi, 2 * math.pi)
    bc: tuple = (0, 0, 0, 0, 0, 0)          # per face x-, x+, y-, y+, z-, z+: BC_*
    uw: tuple = ((0.0, 0.0, 0.0),) * 6      # wall velocity of bounce-back faces (scaled)
    # MappingQ1 cells: grid vertices, array of shape (N0+1, N1+1[, N2+1], D)
    # indexed [i, j(, k)]; None = the Cartesian box of lengths L
    vertices: object = None

    def vertex_array(self):
        """The vertices as the C layout wants them: x fastest, 3 doubles each."""
        if self.vertices is None:
            return None
        v = np.asarray(self.vertices, dtype=np.float64)
        shape = tuple(self.N[a] + 1 for a in range(self.dim))
        if v.shape != shape + (self.dim,):
            raise ValueError(f"vertices must have shape {shape + (self.dim,)}")
        out = np.zeros(shape[::-1] + (3,))
        out[..., :self.dim] = np.transpose(v, tuple(range(self.dim))[::-1] + (self.dim,))
        return np.ascontiguousarray(out.reshape(-1, 3))

    def c(self) -> _Mesh:
        m = _Mesh()
        m.dim = self.dim
        for a in range(3):
            m.N[a] = int(self.N[a]) if a < self.dim else 1
            m.L[a] = float(self.L[a]) if a < self.dim else 1.0
        m.p = self.p
        m.dg = 1 if self.dg else 0
        for f in range(6):
            m.bc[f] = int(self.bc[f])
            for a in range(3):
                m.uw[f][a] = float(self.uw[f][a])
        v = self.vertex_array()
        if v is not None:
            m._keep = v
            m.vtx = _dp(v)
        return m

    def nodes_per_axis(self, a: int) -> int:
        if a >= self.dim:
            return 1
        return self.N[a] * (self.p + 1) if self.dg else self.N[a] * self.p + 1

    @property
    def n_nodes(self) -> int:
        m = self.c()
        return int(lib().orc_n_nodes(C.byref(m)))

    def coords(self) -> np.ndarray:
        m = self.c()
        X = np.zeros((self.n_nodes, 3))
        lib().orc_node_coords(C.byref(m), _dp(X))
        return X

    def h_min(self) -> float:
        if self.vertices is not None:
            # minimum over cells of the smallest distance between two of the
            # cell's vertices (CFDSolverUtilities.cpp:69-84)
            v = np.asarray(self.vertices, dtype=np.float64)
            D = self.dim
            corners = [tuple((k >> a) & 1 for a in range(D)) for k in range(1 << D)]

            def corner(b):
                return v[tuple(slice(b[a], v.shape[a] - 1 + b[a]) for a in range(D))]
            d = min(np.linalg.norm(corner(b1) - corner(b2), axis=-1).min()
                    for i, b1 in enumerate(corners) for b2 in corners[i + 1:])
            return float(d)
        return min(self.L[a] / self.N[a] for a in range(self.dim))


class SLOperator:
    """Per-direction CSR streaming operator assembled by the restated tracker."""

    def __init__(self, mesh: Mesh, st: Stencil, dt: float):
        self.mesh, self.st, self.dt = mesh, st, dt
        m = mesh.c()
        self._h = lib().orc_sl_assemble(C.byref(m), st.id, st.scaling, dt)
        if not self._h:
            raise RuntimeError("oracle assembly failed")
        self.n = mesh.n_nodes

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_sl_free(self._h)
            self._h = None

    def csr(self, alpha: int):
        nnz = lib().orc_sl_nnz(self._h, alpha)
        rp = np.zeros(self.n + 1, dtype=np.int64)
        col = np.zeros(max(nnz, 1), dtype=np.int32)
        val = np.zeros(max(nnz, 1))
        lib().orc_sl_csr(self._h, alpha, rp.ctypes.data_as(C.POINTER(C.c_int64)),
                         col.ctypes.data_as(C.POINTER(C.c_int32)), _dp(val))
        return rp, col[:nnz], val[:nnz]

    @property
    def lifetime_hits(self) -> int:
        return lib().orc_sl_lifetime_hits(self._h)

    @property
    def wall_hits(self) -> int:
        return lib().orc_sl_wall_hits(self._h)

    def csr_dirs(self, alpha: int) -> np.ndarray:
        nnz = lib().orc_sl_nnz(self._h, alpha)
        d = np.zeros(max(nnz, 1), dtype=np.int32)
        lib().orc_sl_csr_dirs(self._h, alpha, d.ctypes.data_as(C.POINTER(C.c_int32)))
        return d[:nnz]

    def bconst(self, alpha: int) -> np.ndarray:
        b = np.zeros(self.n)
        lib().orc_sl_bconst(self._h, alpha, _dp(b))
        return b

    def stream(self, f: np.ndarray, nthreads: int = 1) -> np.ndarray:
        f = np.ascontiguousarray(f, dtype=np.float64)
        out = np.empty_like(f)
        lib().orc_sl_stream(self._h, _dp(f), _dp(out), nthreads)
        return out

    def stream_g(self, g: np.ndarray, nthreads: int = 1) -> np.ndarray:
        """The compressible model's second population through the same
        operator without the wall-velocity terms (CompressibleCFDSolver::gStream,
        CompressibleCFDSolver.h:279-314)."""
        g = np.ascontiguousarray(g, dtype=np.float64)
        out = np.empty_like(g)
        lib().orc_sl_stream_g(self._h, _dp(g), _dp(out), nthreads)
        return out

    def step_bgk(self, f, tau, nsteps=1, nthreads=1):
        """nsteps of copy + SpMV + collide sweep, in place on f (Q, n)."""
        assert f.dtype == np.float64 and f.flags["C_CONTIGUOUS"]
        work = np.empty_like(f)
        rho = np.empty(self.n)
        u = np.empty((self.st.D, self.n))
        rc = lib().orc_step_bgk(self._h, self.st.id, self.st.scaling, tau, _dp(f), _dp(work), _dp(rho), _dp(u),
                                nsteps, nthreads)
        if rc != 0:
            raise RuntimeError(f"oracle step failed rc={rc}")
        return rho, u


    def step_compressible(self, f, g, tau, th=None, nsteps=1, nthreads=1):
        """nsteps of stream(f), gStream(g), collide (CompressibleCFDSolver::run),
        in place on f and g (Q, n).  Returns rho, u (scaled), T, mask."""
        th = th or Thermal()
        for a in (f, g):
            assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
        work = np.empty_like(f)
        rho = np.empty(self.n)
        u = np.empty((self.st.D, self.n))
        T = np.empty(self.n)
        mask = np.empty(self.n)
        rc = lib().orc_step_compressible(self._h, self.st.id, self.st.scaling, tau, th.gamma, th.prandtl,
                                         int(th.prandtl_set), int(th.sutherland), int(th.quartic), _dp(f), _dp(g),
                                         _dp(work), _dp(rho), _dp(u), _dp(T), _dp(mask), nsteps, nthreads)
        _check(rc)
        return rho, u, T, mask


# --------------------------------------------------------------------------
# collisions (all arrays (Q, n) / (D, n), float64, modified in place)
# --------------------------------------------------------------------------

class DensityZeroError(RuntimeError):
    pass


def _check(rc):
    if rc == -2:
        raise DensityZeroError("Densities too small (< 1e-10) for collisions.")
    if rc != 0:
        raise RuntimeError(f"oracle rc={rc}")


def collide_bgk(st: Stencil, tau: float, f, rho, u, in_init=False, nthreads=1):
    n = f.shape[1]
    _check(lib().orc_collide_bgk(st.id, st.scaling, tau, n, _dp(f), _dp(rho), _dp(u), int(in_init), nthreads))


# forcing schemes of the advanced collision (SolverConfiguration::setForcingScheme)
# (3: GUO, the legacy BGKStandard scheme, collision/BGKStandard.cpp:222-225, 470-473)
FORCE_NONE, FORCE_SHIFTING_VELOCITY, FORCE_EXACT_DIFFERENCE, FORCE_GUO = 0, 1, 2, 3


def collide_bgk_force(st: Stencil, tau: float, dt: float, f, rho, u, scheme: int, force, in_init=False,
                      nthreads=1):
    """Advanced BGK with a constant body force (scaled units)."""
    F = np.zeros(3)
    F[: len(force)] = force
    n = f.shape[1]
    _check(lib().orc_collide_bgk_force(st.id, st.scaling, tau, dt, n, _dp(f), _dp(rho), _dp(u), int(in_init),
                                       int(scheme), _dp(F), nthreads))


def collide_bgk_incompressible_d2q9(st: Stencil, tau: float, f, rho, u, in_init=False):
    _check(lib().orc_collide_bgk_incompressible_d2q9(st.scaling, tau, f.shape[1], _dp(f), _dp(rho), _dp(u),
                                                     int(in_init)))


def collide_kbc(st: Stencil, tau: float, f, rho, u, in_init=False, gamma=None):
    g = _dp(gamma) if gamma is not None else C.POINTER(C.c_double)()
    fn = {"D2Q9": lib().orc_collide_kbc_d2q9, "D3Q27": lib().orc_collide_kbc_d3q27}[st.name]
    _check(fn(st.scaling, tau, f.shape[1], _dp(f), _dp(rho), _dp(u), int(in_init), g))


def collide(st: Stencil, model: str, tau: float, f, rho, u, in_init=False):
    if model == "BGK_STANDARD":
        collide_bgk(st, tau, f, rho, u, in_init)
    elif model == "BGK_INCOMPRESSIBLE":
        collide_bgk_incompressible_d2q9(st, tau, f, rho, u, in_init)
    elif model == "KBC_STANDARD":
        collide_kbc(st, tau, f, rho, u, in_init)
    else:
        raise ValueError(model)


def equilibrium(st: Stencil, rho: np.ndarray, u: np.ndarray) -> np.ndarray:
    n = rho.shape[0]
    f = np.zeros((st.Q, n))
    lib().orc_equilibrium(st.id, st.scaling, n, _dp(np.ascontiguousarray(rho)), _dp(np.ascontiguousarray(u)), _dp(f))
    return f


def collide_single_point(st: Stencil, relax_param: float, fq: np.ndarray) -> np.ndarray:
    fq = np.ascontiguousarray(fq, dtype=np.float64).copy()
    lib().orc_bgk_collide_single_point(st.id, st.scaling, relax_param, _dp(fq))
    return fq


@dataclass
class Thermal:
    """Compressible-model settings (SolverConfiguration: heat capacity ratio,
    Prandtl number and its switch, Sutherland law switch; equilibrium scheme
    QUARTIC_EQUILIBRIUM or BGK_EQUILIBRIUM)."""
    gamma: float = 1.4
    prandtl: float = 1.0
    prandtl_set: bool = False
    sutherland: bool = False
    quartic: bool = True


def thermal_init(st: Stencil, rho, u, T, gamma: float = 1.4):
    """Equilibrium initialisation of f and g (CompressibleCFDSolver.h:849-899);
    u scaled.  Returns (f, g), each (Q, n)."""
    n = rho.shape[0]
    f = np.zeros((st.Q, n))
    g = np.zeros((st.Q, n))
    c = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    rc = lib().orc_thermal_init(st.id, st.scaling, gamma, n, _dp(c(rho)), _dp(c(u)), _dp(c(T)), _dp(f), _dp(g))
    _check(rc)
    return f, g


def thermal_feq(st: Stencil, rho, u, T, quartic: bool = True):
    """The collision's equilibrium (quartic, Equilibria.h:130-267, or second
    order, :66-83) at (rho, u scaled, T); (Q, n)."""
    n = rho.shape[0]
    feq = np.zeros((st.Q, n))
    c = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    _check(lib().orc_thermal_feq(st.id, st.scaling, int(quartic), n, _dp(c(rho)), _dp(c(u)), _dp(c(T)), _dp(feq)))
    return feq


def collide_compressible(st: Stencil, tau: float, f, g, rho, u, T, mask, th: Thermal = Thermal(),
                         in_init=False, nthreads=1):
    """CollisionOperator::collideAll(f, g, rho, u, T, mask) with relaxWithG;
    in place on f, g; writes rho, u (scaled, unless in_init), T, mask."""
    _check(lib().orc_collide_compressible(st.id, st.scaling, tau, th.gamma, th.prandtl, int(th.prandtl_set),
                                          int(th.sutherland), int(th.quartic), f.shape[1], _dp(f), _dp(g),
                                          _dp(rho), _dp(u), _dp(T), _dp(mask), int(in_init), nthreads))


def max_threads() -> int:
    return lib().orc_max_threads()


# --------------------------------------------------------------------------
# problems: Taylor-Green initial conditions, kinetic energy
# --------------------------------------------------------------------------

def tgv2d_init(X: np.ndarray, Ma: float, L: float = 2 * math.pi, rho_sign: float = 1.0):
    """TaylorGreenVortex2D (benchmarks/TaylorGreenVortex2D.cpp:36-59) at t=0,
    analytic density rho = 1 + rho_sign * p / c_s^2 with c_s = 1/Ma, p = 1/4
    (cos 2x' + cos 2y'), x' = 2 pi x / L.  rho_sign=+1 is the reference's sign."""
    k = 2 * math.pi / L
    x, y = X[:, 0] * k, X[:, 1] * k
    u = np.stack([np.sin(x) * np.cos(y), -np.cos(x) * np.sin(y)])
    p = 0.25 * (np.cos(2 * x) + np.cos(2 * y))
    rho = 1.0 + rho_sign * p * Ma * Ma
    return rho, u


def tgv3d_init(X: np.ndarray, Ma: float):
    """TaylorGreenVortex3D (benchmarks/TaylorGreenVortex3D.cpp:38-58)."""
    x, y, z = X[:, 0], X[:, 1], X[:, 2]
    u = np.stack([np.sin(x) * np.cos(y) * np.cos(z), -np.cos(x) * np.sin(y) * np.cos(z), np.zeros_like(x)])
    p = 1.0 / 16.0 * (np.cos(2 * x) + np.cos(2 * y)) * (np.cos(2 * z) + 2)
    rho = 1.0 + p * Ma * Ma
    return rho, u


def kinetic_energy(mesh: Mesh, rho: np.ndarray, u: np.ndarray) -> float:
    """PhysicalProperties::kineticEnergy (solver/PhysicalProperties.cpp:29-79)
    with Gauss-Lobatto quadrature on the support points: 0.5 sum_cells sum_q
    rho |u|^2 w_q |J|; at GL support points shape_value(i,q) = delta_iq."""
    p, D = mesh.p, mesh.dim
    xi = gl_points(p)
    # GL weights on [0,1]
    P = np.polynomial.legendre.Legendre.basis(p)
    wq = 1.0 / (p * (p + 1)) * 2.0 / (P(2 * xi - 1) ** 2) / 2.0
    e = rho * np.sum(u * u, axis=0)
    n_ax = [mesh.nodes_per_axis(a) for a in range(3)]
    E = e.reshape(n_ax[2], n_ax[1], n_ax[0])
    total = 0.0
    jac = 1.0
    for a in range(D):
        jac *= mesh.L[a] / mesh.N[a]
    per = (lambda c: slice(c * (p + 1), c * (p + 1) + p + 1)) if mesh.dg else (lambda c: slice(c * p, c * p + p + 1))
    if D == 2:
        W = np.outer(wq, wq)
        for cy in range(mesh.N[1]):
            for cx in range(mesh.N[0]):
                total += np.sum(E[0, per(cy), per(cx)] * W)
    else:
        W = np.einsum("i,j,k->ijk", wq, wq, wq)
        for cz in range(mesh.N[2]):
            for cy in range(mesh.N[1]):
                for cx in range(mesh.N[0]):
                    total += np.sum(E[per(cz), per(cy), per(cx)] * W)
    return 0.5 * total * jac
