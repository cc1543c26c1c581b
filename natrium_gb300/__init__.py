"""natrium_gb300 -- GB300-native semi-Lagrangian stream + collide for NATriuM.

Python host mirror of the reference's operator interfaces for the hot path,
on top of the C ABI of ``libnatgpu.so`` (``include/natgpu.h``):

* :class:`Solver` -- one device-resident solve (the state a ``CFDSolver``
  keeps in ``m_f``, ``m_density``, ``m_velocity``).
* :class:`SemiLagrangian` -- ``AdvectionOperator::stream(f_old, f, t)``
  (advection/SemiLagrangian.h:150-161) and ``setDeltaT`` (:175-179).
* :class:`BGKStandard`, :class:`BGKIncompressible`, :class:`KBCStandard` --
  ``CollisionModel::collideAll(f, rho, u, owned, inInitializationProcedure)``
  (collision/CollisionModel.h:74-78).
* :class:`DistributionFunctions` -- host mirror of
  solver/DistributionFunctions.h: Q blocks of n doubles, block 0 = f_0.
* :class:`CompressibleStep`, :class:`BGKCompressible` -- the compressible
  two-population model on D2Q25H: ``CompressibleCFDSolver::stream()`` +
  ``gStream()`` (solver/CompressibleCFDSolver.h:181-314) and
  ``collideAll(f, g, rho, u, T, mask, owned, init)``
  (collision_advanced/CollisionOperator.h:113-224).

There is no CPU fallback: importing the package raises if the CUDA library is
missing, and every call goes through the CUDA kernels.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libnatgpu.so")

# status codes (include/natgpu.h)
NAT_OK = 0
NAT_ERR_INVALID_ARG = 1
NAT_ERR_OOM = 2
NAT_ERR_DENSITY_UNDERFLOW = 3
NAT_ERR_NAN = 4
NAT_ERR_TIMEOUT = 5
NAT_ERR_CUDA = 6
NAT_ERR_UNSUPPORTED = 7

STENCILS = {"D2Q9": 0, "D3Q19": 1, "D3Q27": 2, "D2Q25H": 3}
STENCIL_DQ = {"D2Q9": (2, 9), "D3Q19": (3, 19), "D3Q27": (3, 27), "D2Q25H": (2, 25)}
COLLISIONS = {"BGK_STANDARD": 0, "BGK_INCOMPRESSIBLE": 1, "KBC_STANDARD": 2, "BGK_COMPRESSIBLE": 3}
FORCE_SCHEMES = {"NONE": 0, "SHIFTING_VELOCITY": 1, "EXACT_DIFFERENCE": 2, "GUO": 3}
EQUILIBRIA = {"BGK": 0, "QUARTIC": 1}
TOPOLOGIES = {"feq": 0, "dg": 1}
PRECISIONS = {"fp64": 0, "fp32dev": 1}

# every symbol include/natgpu.h declares
EXPORTS = [
    "nat_create", "nat_destroy", "nat_sizes", "nat_get_dt", "nat_set_dt", "nat_set_stream",
    "nat_upload_f", "nat_download_f", "nat_download_macro", "nat_upload_macro", "nat_stream",
    "nat_collide", "nat_step", "nat_step_async", "nat_status", "nat_last_error",
    "nat_mass_energy", "nat_device_f", "nat_launch_count", "nat_version", "nat_set_kernel_variant",
    "nat_kernel_variant", "nat_autotune", "nat_autotune_report", "nat_select_candidate", "nat_kernel_info",
    "nat_mapped_rows", "nat_server_create", "nat_server_destroy", "nat_server_submit", "nat_server_step", "nat_server_run",
    "nat_server_poll",
    "nat_server_result", "nat_server_stats", "nat_server_last_error", "nat_mass_energy_noalloc",
    "nat_set_thermal", "nat_get_thermal", "nat_upload_g", "nat_download_g", "nat_download_thermal",
    "nat_init_thermal", "nat_set_boundary", "nat_set_force", "nat_checkpoint_save", "nat_checkpoint_load",
    "nat_write_vtu", "nat_download_macro_async", "nat_wait", "nat_set_wait_limit",
]


class NatError(RuntimeError):
    """Error returned through the C ABI (code + text of nat_last_error)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class CollisionException(NatError):
    """rho < 1e-10 in a collision (the reference's CollisionException /
    DensityZeroException, collision_advanced/AuxiliaryCollisionFunctions.h:53-56)."""


class _Spec(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("stencil", C.c_int), ("order", C.c_int), ("topology", C.c_int),
        ("cells", C.c_int * 3), ("length", C.c_double * 3), ("periodic", C.c_int * 3),
        ("scaling", C.c_double), ("viscosity", C.c_double), ("cfl", C.c_double), ("dt", C.c_double),
        ("collision", C.c_int), ("precision", C.c_int), ("vertices", C.POINTER(C.c_double)),
    ]


class _Thermal(C.Structure):
    _fields_ = [("gamma", C.c_double), ("prandtl", C.c_double), ("prandtl_set", C.c_int),
                ("sutherland_set", C.c_int), ("equilibrium", C.c_int)]


@dataclass
class ThermalSettings:
    """Compressible-model settings (SolverConfiguration: heat capacity ratio
    gamma, Prandtl number and its switch, Sutherland law switch; equilibrium
    QUARTIC or BGK).  Defaults are the reference's
    (solver/SolverConfiguration.cpp:21-31)."""
    gamma: float = 1.4
    prandtl: float = 1.0
    prandtl_set: bool = False
    sutherland: bool = False
    equilibrium: str = "QUARTIC"


_lib = None


def load_library(path: str | None = None):
    """Load libnatgpu.so (fails loudly when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(f"libnatgpu.so not found at {path}; build it with "
                          "`python -m natrium_gb300.build` (nvcc, sm_103a)")
    L = C.CDLL(path)
    vp, dp, i64p = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)
    L.nat_create.argtypes = [C.POINTER(_Spec), C.POINTER(vp)]
    L.nat_destroy.argtypes = [vp]
    L.nat_sizes.argtypes = [vp, i64p, i64p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.nat_get_dt.argtypes = [vp, dp, dp]
    L.nat_set_dt.argtypes = [vp, C.c_double]
    L.nat_set_stream.argtypes = [vp, vp]
    L.nat_upload_f.argtypes = [vp, dp]
    L.nat_download_f.argtypes = [vp, dp]
    L.nat_download_macro.argtypes = [vp, dp, dp]
    L.nat_upload_macro.argtypes = [vp, dp, dp]
    L.nat_download_macro_async.argtypes = [vp, dp, dp, C.POINTER(C.c_uint64)]
    L.nat_wait.argtypes = [vp, C.c_uint64]
    L.nat_set_wait_limit.argtypes = [vp, C.c_uint32]
    L.nat_stream.argtypes = [vp, C.c_double, dp]
    L.nat_collide.argtypes = [vp, C.c_int]
    L.nat_step.argtypes = [vp, C.c_int]
    L.nat_step_async.argtypes = [vp, C.c_int, C.c_int]
    L.nat_status.argtypes = [vp]
    L.nat_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    L.nat_mass_energy.argtypes = [vp, dp, dp]
    L.nat_device_f.argtypes = [vp, C.POINTER(vp)]
    L.nat_launch_count.argtypes = [vp]
    L.nat_launch_count.restype = C.c_int64
    L.nat_version.restype = C.c_char_p
    L.nat_set_kernel_variant.argtypes = [vp, C.c_int]
    L.nat_mass_energy_noalloc.argtypes = [vp, vp, C.c_int, C.POINTER(C.c_int), C.c_int, C.c_int,
                                          C.POINTER(C.c_double), vp, vp]
    L.nat_kernel_variant.argtypes = [vp]
    L.nat_autotune.argtypes = [vp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.nat_autotune_report.argtypes = [vp, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_int)]
    L.nat_select_candidate.argtypes = [vp, C.c_int]
    L.nat_kernel_info.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), i64p]
    L.nat_set_thermal.argtypes = [vp, C.POINTER(_Thermal)]
    L.nat_get_thermal.argtypes = [vp, C.POINTER(_Thermal)]
    L.nat_upload_g.argtypes = [vp, dp]
    L.nat_download_g.argtypes = [vp, dp]
    L.nat_download_thermal.argtypes = [vp, dp, dp]
    L.nat_init_thermal.argtypes = [vp, dp, dp, dp]
    L.nat_set_boundary.argtypes = [vp, C.c_int, C.c_int, dp]
    L.nat_set_force.argtypes = [vp, C.c_int, dp]
    L.nat_mapped_rows.argtypes = [vp, C.c_int, vp, vp, vp, vp]
    L.nat_checkpoint_save.argtypes = [vp, C.c_char_p, C.c_int64, C.c_double]
    L.nat_checkpoint_load.argtypes = [vp, C.c_char_p, C.POINTER(C.c_int64), C.POINTER(C.c_double)]
    L.nat_write_vtu.argtypes = [vp, C.c_char_p]
    _lib = L
    return L


def _dp(a: np.ndarray):
    if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"]:
        raise TypeError("expected a C-contiguous float64 array")
    return a.ctypes.data_as(C.POINTER(C.c_double))


@dataclass
class SolverSpec:
    """Problem + numerics of one stream-collide solve (a plain struct in
    place of SolverConfiguration / ProblemDescription)."""
    stencil: str = "D2Q9"
    order: int = 4
    cells: tuple = (8, 8)
    length: tuple = (2 * np.pi, 2 * np.pi)
    scaling: float = 1.0
    viscosity: float = 1e-3
    cfl: float = 0.4
    dt: float = 0.0
    collision: str = "BGK_STANDARD"
    precision: str = "fp64"
    topology: str = "feq"
    periodic: tuple = (True, True, True)  # False: two wall faces on that axis (DG only)
    # MappingQ1 cells: grid vertices of shape (N0+1, N1+1[, N2+1], dim) indexed
    # [i, j(, k)]; None = the Cartesian box of `length`
    vertices: object = None

    @property
    def dim(self) -> int:
        return STENCIL_DQ[self.stencil][0]

    def c(self) -> _Spec:
        s = _Spec()
        s.dim = self.dim
        s.stencil = STENCILS[self.stencil]
        s.order = int(self.order)
        s.topology = TOPOLOGIES[self.topology]
        for a in range(3):
            s.cells[a] = int(self.cells[a]) if a < self.dim else 1
            s.length[a] = float(self.length[a]) if a < self.dim else 1.0
            s.periodic[a] = 1 if (a >= self.dim or self.periodic[a]) else 0
        s.scaling = float(self.scaling)
        s.viscosity = float(self.viscosity)
        s.cfl = float(self.cfl)
        s.dt = float(self.dt)
        s.collision = COLLISIONS[self.collision]
        s.precision = PRECISIONS[self.precision]
        v = self.vertex_array()
        if v is not None:
            s._keep = v  # alive until nat_create has copied it
            s.vertices = v.ctypes.data_as(C.POINTER(C.c_double))
        return s

    def vertex_array(self):
        """The vertices in the C layout: x fastest, 3 doubles per vertex."""
        if self.vertices is None:
            return None
        D = self.dim
        v = np.asarray(self.vertices, dtype=np.float64)
        shape = tuple(int(self.cells[a]) + 1 for a in range(D))
        if v.shape != shape + (D,):
            raise ValueError(f"vertices must have shape {shape + (D,)}, got {v.shape}")
        out = np.zeros(shape[::-1] + (3,))
        out[..., :D] = np.transpose(v, tuple(range(D))[::-1] + (D,))
        return np.ascontiguousarray(out.reshape(-1, 3))


class Solver:
    """One device-resident solve driven through the C ABI."""

    def __init__(self, spec: SolverSpec):
        self.spec = spec
        self._L = load_library()
        self._pending = {}  # ticket -> host arrays of an asynchronous read-back
        self._h = C.c_void_p()
        cs = spec.c()
        rc = self._L.nat_create(C.byref(cs), C.byref(self._h))
        if rc != NAT_OK:
            msg = self._err()
            self._L.nat_destroy(self._h)
            self._h = C.c_void_p()
            raise NatError(rc, msg)
        nr, nd = C.c_int64(), C.c_int64()
        q, d = C.c_int(), C.c_int()
        self._L.nat_sizes(self._h, C.byref(nr), C.byref(nd), C.byref(q), C.byref(d))
        self.n_ref, self.n_dev, self.Q, self.D = nr.value, nd.value, q.value, d.value

    # -- plumbing ----------------------------------------------------------
    def _err(self) -> str:
        buf = C.create_string_buffer(512)
        self._L.nat_last_error(self._h, buf, 512)
        return buf.value.decode()

    def _check(self, rc: int):
        if rc == NAT_OK:
            return
        msg = self._err()
        if rc in (NAT_ERR_DENSITY_UNDERFLOW, NAT_ERR_NAN):
            raise CollisionException(rc, msg)
        raise NatError(rc, msg)

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._L.nat_destroy(self._h)  # waits for outstanding read-backs
            self._h = C.c_void_p()
            self._pending = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- properties ----------------------------------------------------------
    @property
    def dt(self) -> float:
        dt, tau = C.c_double(), C.c_double()
        self._L.nat_get_dt(self._h, C.byref(dt), C.byref(tau))
        return dt.value

    @property
    def tau(self) -> float:
        dt, tau = C.c_double(), C.c_double()
        self._L.nat_get_dt(self._h, C.byref(dt), C.byref(tau))
        return tau.value

    @property
    def launches(self) -> int:
        return int(self._L.nat_launch_count(self._h))

    # -- state transfer -------------------------------------------------------
    def upload_f(self, f: np.ndarray):
        f = np.ascontiguousarray(f, dtype=np.float64)
        if f.shape != (self.Q, self.n_ref):
            raise ValueError(f"f must have shape {(self.Q, self.n_ref)}")
        self._check(self._L.nat_upload_f(self._h, _dp(f)))

    def download_f(self) -> np.ndarray:
        out = np.empty((self.Q, self.n_ref))
        self._check(self._L.nat_download_f(self._h, _dp(out)))
        return out

    def download_macro(self, rho: np.ndarray = None, u: np.ndarray = None):
        """rho (n_ref) and u (D, n_ref) of the last collision, into the given
        float64 arrays when passed (e.g. page-locked ones, so the copy runs as
        DMA), else into new ones."""
        if rho is None:
            rho = np.empty(self.n_ref)
        if u is None:
            u = np.empty((self.D, self.n_ref))
        if rho.shape != (self.n_ref,) or u.shape != (self.D, self.n_ref):
            raise ValueError("rho / u have the wrong shape")
        self._check(self._L.nat_download_macro(self._h, _dp(rho), _dp(u)))
        return rho, u

    def download_macro_async(self, rho: np.ndarray, u: np.ndarray) -> int:
        """Enqueue the read-back of rho (n_ref) and u (D, n_ref) into the given
        C-contiguous float64 arrays (page-locked ones for an asynchronous
        copy) and return a ticket; the arrays are filled, and the status of
        the steps before it checked, by wait(ticket).  The arrays are kept
        alive here until then."""
        if rho.shape != (self.n_ref,) or u.shape != (self.D, self.n_ref):
            raise ValueError("rho / u have the wrong shape")
        for a in (rho, u):
            if a.dtype != np.float64 or not a.flags.c_contiguous or not a.flags.writeable:
                raise ValueError("rho / u must be writeable C-contiguous float64 arrays")
        t = C.c_uint64()
        self._check(self._L.nat_download_macro_async(self._h, _dp(rho), _dp(u), C.byref(t)))
        self._pending[t.value] = (rho, u)
        # issuing ticket t waited for ticket t - 8 (its slot was reused)
        for old in [k for k in self._pending if k <= t.value - 8]:
            del self._pending[old]
        return t.value

    def wait(self, ticket: int):
        """Wait for the read-back of a ticket; raises CollisionException when
        a step before it met a density below 1e-10 or a NaN."""
        try:
            self._check(self._L.nat_wait(self._h, ticket))
        finally:
            self._pending.pop(ticket, None)

    def upload_macro(self, rho: np.ndarray, u: np.ndarray):
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        u = np.ascontiguousarray(u, dtype=np.float64)
        self._check(self._L.nat_upload_macro(self._h, _dp(rho), _dp(u)))

    # -- operators --------------------------------------------------------------
    def set_dt(self, dt: float):
        self._check(self._L.nat_set_dt(self._h, dt))

    def set_stream(self, cuda_stream_ptr: int):
        self._check(self._L.nat_set_stream(self._h, C.c_void_p(cuda_stream_ptr)))

    def stream(self, t: float = 0.0) -> float:
        dt = C.c_double()
        self._check(self._L.nat_stream(self._h, t, C.byref(dt)))
        return dt.value

    def collide(self, in_init: bool = False):
        self._check(self._L.nat_collide(self._h, int(in_init)))

    def step(self, n: int = 1):
        self._check(self._L.nat_step(self._h, int(n)))

    def step_async(self, n: int = 1, write_macro: bool = True):
        self._check(self._L.nat_step_async(self._h, int(n), int(write_macro)))

    def status(self):
        self._check(self._L.nat_status(self._h))

    def set_wait_limit(self, polls: int):
        """Limit of each wait of the bulk-copy kernels for a copy (mbarrier
        polls; default 2^24).  A wait that runs out ends the step with
        NatError(NAT_ERR_TIMEOUT) instead of hanging; 0 makes every such wait
        run out at once (tests that path)."""
        self._check(self._L.nat_set_wait_limit(self._h, int(polls)))

    def mass_energy(self):
        m, e = C.c_double(), C.c_double()
        self._check(self._L.nat_mass_energy(self._h, C.byref(m), C.byref(e)))
        return m.value, e.value

    def set_kernel_variant(self, variant: int):
        """0 automatic, 1 generic kernel, 2 specialised kernel required,
        3 tile kernel required, 4 row-segment kernel required, 6 bulk-copy
        row-segment kernel required, 7 row-group kernel required, 11 cell-row
        kernel required, 12 cell-row kernel with the D3Q27 corner directions
        on the tensor cores (only when asked for), 13 cell-row kernel with z
        sharing of the yz-diagonal directions."""
        self._check(self._L.nat_set_kernel_variant(self._h, int(variant)))

    @property
    def kernel_variant(self) -> int:
        return int(self._L.nat_kernel_variant(self._h))

    def autotune(self, steps: int = 5):
        """Time every applicable kernel for `steps` steps and keep the
        fastest (the state is restored).  Returns (n_candidates, chosen)."""
        nc, ch = C.c_int(), C.c_int()
        self._check(self._L.nat_autotune(self._h, int(steps), C.byref(nc), C.byref(ch)))
        return nc.value, ch.value

    def select_candidate(self, index: int):
        """Use candidate `index` of the autotuner's list (no timing)."""
        self._check(self._L.nat_select_candidate(self._h, int(index)))

    def autotune_report(self) -> list:
        """Per candidate of the last autotune: dict(variant, tile_nodes,
        threads, ms_per_step)."""
        n = int(self._L.nat_autotune_report(self._h, 0, None, None))
        if n <= 0:
            return []
        ms = (C.c_float * n)()
        desc = (C.c_int * (5 * n))()
        self._L.nat_autotune_report(self._h, n, ms, desc)
        return [dict(variant=desc[5 * i], tile_nodes=[desc[5 * i + 1], desc[5 * i + 2], desc[5 * i + 3]],
                     threads=desc[5 * i + 4], ms_per_step=float(ms[i])) for i in range(n)]

    def kernel_info(self) -> dict:
        v, th = C.c_int(), C.c_int()
        tile = (C.c_int * 3)()
        sm = C.c_int64()
        self._check(self._L.nat_kernel_info(self._h, C.byref(v), tile, C.byref(th), C.byref(sm)))
        return {"variant": v.value, "tile_nodes": list(tile), "threads": th.value, "smem_bytes": sm.value}

    def device_f_ptr(self) -> int:
        p = C.c_void_p()
        self._check(self._L.nat_device_f(self._h, C.byref(p)))
        return p.value or 0

    # -- checkpoint and output ---------------------------------------------------------
    def save_checkpoint(self, path: str, iteration: int = 0, time: float = 0.0):
        self._check(self._L.nat_checkpoint_save(self._h, os.fsencode(path), int(iteration), float(time)))

    def load_checkpoint(self, path: str):
        """Restore f (and g); returns (iteration, time) of the checkpoint."""
        it, t = C.c_int64(), C.c_double()
        self._check(self._L.nat_checkpoint_load(self._h, os.fsencode(path), C.byref(it), C.byref(t)))
        return it.value, t.value

    def write_vtu(self, path: str):
        self._check(self._L.nat_write_vtu(self._h, os.fsencode(path)))

    # -- wall boundaries -------------------------------------------------------------
    def mapped_rows(self, where: str = "device", copy: bool = True):
        """Departure-point rows of a mapped one-population mesh, searched by
        the host tracker (where="host") or the device tracker ("device"):
        (base int32 [(Q-1) n], u, c, flags uint8 [(Q-1) n]) with u and c
        float32 (FP32 deviation storage: unit coordinates, deviation
        constant) or float64 (FP64: 1-D Lagrange values, plain constant).
        copy=False runs the search only (for timing) and returns None."""
        fp64 = self.spec.precision == "fp64"
        dt = np.float64 if fp64 else np.float32
        nr = (self.Q - 1) * self.n_dev
        per = self.D * (self.spec.order + 1 if fp64 else 1)
        if copy:
            base = np.empty(nr, dtype=np.int32)
            u = np.empty(nr * per, dtype=dt)
            c = np.empty(nr, dtype=dt)
            fl = np.empty(nr, dtype=np.uint8)
            ptrs = [a.ctypes.data_as(C.c_void_p) for a in (base, u, c, fl)]
        else:
            ptrs = [None] * 4
        self._check(self._L.nat_mapped_rows(self._h, {"host": 0, "device": 1}[where], *ptrs))
        return (base, u, c, fl) if copy else None

    def set_force(self, scheme: str = "SHIFTING_VELOCITY", force=(0.0, 0.0, 0.0)):
        """Constant body force in scaled units (ConstantExternalForce) with the
        forcing scheme NONE, SHIFTING_VELOCITY, EXACT_DIFFERENCE (the advanced
        collision) or GUO (the legacy BGKStandard collision, D2Q9 and D3Q19)."""
        F = np.zeros(3)
        F[: len(force)] = force
        self._check(self._L.nat_set_force(self._h, FORCE_SCHEMES[scheme], _dp(F)))

    def set_boundary(self, face: int, kind: str = "VELOCITY_BOUNCE_BACK", u_wall=(0.0, 0.0, 0.0)):
        """Kind of wall face `face` (0 x-, 1 x+, 2 y-, 3 y+, 4 z-, 5 z+) of a
        non-periodic axis: VELOCITY_BOUNCE_BACK (wall velocity u_wall, scaled)
        or DO_NOTHING."""
        k = {"VELOCITY_BOUNCE_BACK": 1, "DO_NOTHING": 2}[kind]
        uw = np.ascontiguousarray(np.asarray(u_wall, dtype=np.float64).reshape(3))
        self._check(self._L.nat_set_boundary(self._h, int(face), k, _dp(uw)))

    # -- compressible two-population model (collision BGK_COMPRESSIBLE) ---------
    def set_thermal(self, t: ThermalSettings):
        c = _Thermal(float(t.gamma), float(t.prandtl), int(t.prandtl_set), int(t.sutherland),
                     EQUILIBRIA[t.equilibrium])
        self._check(self._L.nat_set_thermal(self._h, C.byref(c)))

    def get_thermal(self) -> ThermalSettings:
        c = _Thermal()
        self._check(self._L.nat_get_thermal(self._h, C.byref(c)))
        eq = {v: k for k, v in EQUILIBRIA.items()}[c.equilibrium]
        return ThermalSettings(c.gamma, c.prandtl, bool(c.prandtl_set), bool(c.sutherland_set), eq)

    def upload_g(self, g: np.ndarray):
        g = np.ascontiguousarray(g, dtype=np.float64)
        if g.shape != (self.Q, self.n_ref):
            raise ValueError(f"g must have shape {(self.Q, self.n_ref)}")
        self._check(self._L.nat_upload_g(self._h, _dp(g)))

    def download_g(self) -> np.ndarray:
        out = np.empty((self.Q, self.n_ref))
        self._check(self._L.nat_download_g(self._h, _dp(out)))
        return out

    def download_thermal(self):
        """Temperature and shock-sensor mask of the last collision."""
        T = np.empty(self.n_ref)
        m = np.empty(self.n_ref)
        self._check(self._L.nat_download_thermal(self._h, _dp(T), _dp(m)))
        return T, m

    def init_thermal(self, rho: np.ndarray, u: np.ndarray, T: np.ndarray):
        """Equilibrium initialisation of f and g from rho, u (scaled), T."""
        c = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        self._check(self._L.nat_init_thermal(self._h, _dp(c(rho)), _dp(c(u)), _dp(c(T))))


# ---------------------------------------------------------------------------
# mirrors of the reference interfaces
# ---------------------------------------------------------------------------

@dataclass
class DistributionFunctions:
    """Host mirror of solver/DistributionFunctions.h: f.at(i) is block i."""
    f: np.ndarray = field(default_factory=lambda: np.zeros((0, 0)))

    def at(self, i: int) -> np.ndarray:
        return self.f[i]

    def getFStream(self) -> np.ndarray:
        return self.f[1:]

    def size(self) -> int:
        return self.f.shape[0]

    def copy(self) -> "DistributionFunctions":
        return DistributionFunctions(self.f.copy())


class SemiLagrangian:
    """advection/SemiLagrangian.h: stream(f_old, f, t) on the device."""

    def __init__(self, solver: Solver):
        self.solver = solver

    def setDeltaT(self, dt: float):
        self.solver.set_dt(dt)

    def getDeltaT(self) -> float:
        return self.solver.dt

    def stream(self, f_old: DistributionFunctions, f: DistributionFunctions, t: float = 0.0) -> float:
        if f_old is f:
            raise ValueError("f_old and f must be different objects (SemiLagrangian.h:153)")
        f_old.f = f.f.copy()
        self.solver.upload_f(f_old.f)
        dt = self.solver.stream(t)
        f.f = self.solver.download_f()
        return dt


class _CollisionModel:
    MODEL = "BGK_STANDARD"

    def __init__(self, solver: Solver):
        if solver.spec.collision != self.MODEL:
            raise ValueError(f"solver was created for {solver.spec.collision}, not {self.MODEL}")
        self.solver = solver

    def collideAll(self, f: DistributionFunctions, densities: np.ndarray, velocities: np.ndarray,
                   locally_owned_dofs=None, inInitializationProcedure: bool = False):
        """In-place collision of every node; densities and (unless in init)
        velocities are overwritten like the reference's vectors."""
        s = self.solver
        s.upload_f(f.f)
        if inInitializationProcedure:
            s.upload_macro(np.ascontiguousarray(densities), np.ascontiguousarray(velocities))
        s.collide(inInitializationProcedure)
        f.f[...] = s.download_f()
        rho, u = s.download_macro()
        densities[...] = rho
        if not inInitializationProcedure:
            velocities[...] = u


class BGKStandard(_CollisionModel):
    MODEL = "BGK_STANDARD"


class BGKIncompressible(_CollisionModel):
    MODEL = "BGK_INCOMPRESSIBLE"


class KBCStandard(_CollisionModel):
    MODEL = "KBC_STANDARD"


class CompressibleStep:
    """CompressibleCFDSolver's streaming: stream() of f and gStream() of g with
    the same semi-Lagrangian operator (solver/CompressibleCFDSolver.h:181-314)."""

    def __init__(self, solver: Solver):
        if solver.spec.collision != "BGK_COMPRESSIBLE":
            raise ValueError("the solver must be created with collision BGK_COMPRESSIBLE")
        self.solver = solver

    def stream(self, f: DistributionFunctions, g: DistributionFunctions, t: float = 0.0) -> float:
        s = self.solver
        s.upload_f(f.f)
        s.upload_g(g.f)
        dt = s.stream(t)
        f.f = s.download_f()
        g.f = s.download_g()
        return dt


class BGKCompressible:
    """CollisionOperator<2,25,QuarticEquilibrium,BGKCollision>::collideAll(f, g,
    rho, u, T, mask, owned, inInitializationProcedure) with relaxWithG."""

    def __init__(self, solver: Solver):
        if solver.spec.collision != "BGK_COMPRESSIBLE":
            raise ValueError("the solver must be created with collision BGK_COMPRESSIBLE")
        self.solver = solver

    def collideAll(self, f: DistributionFunctions, g: DistributionFunctions, densities: np.ndarray,
                   velocities: np.ndarray, temperature: np.ndarray, maskShockSensor: np.ndarray,
                   locally_owned_dofs=None, inInitializationProcedure: bool = False):
        s = self.solver
        s.upload_f(f.f)
        s.upload_g(g.f)
        if inInitializationProcedure:
            s.upload_macro(np.ascontiguousarray(densities), np.ascontiguousarray(velocities))
        s.collide(inInitializationProcedure)
        f.f[...] = s.download_f()
        g.f[...] = s.download_g()
        rho, u = s.download_macro()
        T, m = s.download_thermal()
        densities[...] = rho
        if not inInitializationProcedure:
            velocities[...] = u
        temperature[...] = T
        maskShockSensor[...] = m


def version() -> str:
    return load_library().nat_version().decode()
