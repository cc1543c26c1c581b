"""Continuous-batching serving of independent 2-D solves (host driver).

Wraps the server of ``libnatgpu.so`` (``nat_server_*`` in include/natgpu.h):
requests are admitted by HBM footprint, all live solves advance together in
one persistent graph-captured launch per server step, finished solves are
copied out after an event.  ``run_workload`` replays a seeded request stream
(Poisson arrivals) against wall-clock time and reports solves/s and the
p50 / p99 latency (arrival to result).
"""
from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass

import numpy as np

from . import NatError, NAT_OK, load_library, STENCILS, COLLISIONS

INIT_TAYLOR_GREEN = 0
INIT_SHEAR_LAYER = 1


class _Request(C.Structure):
    _fields_ = [
        ("stencil", C.c_int), ("collision", C.c_int), ("order", C.c_int), ("cells", C.c_int * 2),
        ("length", C.c_double * 2), ("scaling", C.c_double), ("viscosity", C.c_double), ("cfl", C.c_double),
        ("dt", C.c_double), ("steps", C.c_int), ("init", C.c_int), ("Ma", C.c_double), ("u0", C.c_double),
        ("kappa", C.c_double), ("delta", C.c_double),
    ]


class _Stats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("pending", "live", "completing", "finished", "steps", "node_updates",
                                         "pool_used", "pool_bytes", "launches", "graph_builds",
                                         "graph_updates", "rebuild_ns")]


@dataclass
class Request:
    """One independent periodic D2Q9 solve."""
    collision: str = "BGK_STANDARD"
    order: int = 4
    cells: tuple = (8, 8)
    length: tuple = (2 * math.pi, 2 * math.pi)
    Ma: float = 0.05
    Re: float = 1000.0
    steps: int = 100
    init: int = INIT_TAYLOR_GREEN
    cfl: float = 0.4
    kappa: float = 80.0
    delta: float = 0.05

    @property
    def scaling(self) -> float:
        return math.sqrt(3) / self.Ma

    @property
    def viscosity(self) -> float:
        # U = 1 in scaled units; characteristic length L (TaylorGreenVortex2D
        # uses the box length, ShearLayer2D uses 1)
        L = self.length[0] if self.init == INIT_TAYLOR_GREEN else 1.0
        return L / self.Re

    def c(self) -> _Request:
        r = _Request()
        r.stencil = STENCILS["D2Q9"]
        r.collision = COLLISIONS[self.collision]
        r.order = self.order
        r.cells[0], r.cells[1] = self.cells
        r.length[0], r.length[1] = self.length
        r.scaling = self.scaling
        r.viscosity = self.viscosity
        r.cfl = self.cfl
        r.dt = 0.0
        r.steps = self.steps
        r.init = self.init
        r.Ma = self.Ma
        r.u0 = 1.0
        r.kappa = self.kappa
        r.delta = self.delta
        return r

    @property
    def nodes(self) -> int:
        return (self.cells[0] * self.order) * (self.cells[1] * self.order)


def _bind(L):
    if getattr(L, "_serve_bound", False):
        return L
    vp = C.c_void_p
    L.nat_server_create.argtypes = [C.c_size_t, C.c_int, C.POINTER(vp)]
    L.nat_server_destroy.argtypes = [vp]
    L.nat_server_submit.argtypes = [vp, C.POINTER(_Request), C.POINTER(C.c_int64)]
    L.nat_server_step.argtypes = [vp]
    L.nat_server_run.argtypes = [vp, C.c_int, C.POINTER(C.c_int)]
    L.nat_server_poll.argtypes = [vp, C.POINTER(C.c_int64), C.c_int, C.POINTER(C.c_int), C.c_int]
    L.nat_server_result.argtypes = [vp, C.c_int64, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                    C.POINTER(C.c_int64), C.POINTER(C.c_int)]
    L.nat_server_stats.argtypes = [vp, C.POINTER(_Stats)]
    L.nat_server_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
    L._serve_bound = True
    return L


class Server:
    """Device-resident continuous-batching server."""

    def __init__(self, pool_bytes: int = 4 << 30, max_slots: int = 256):
        self._L = _bind(load_library())
        self._h = C.c_void_p()
        rc = self._L.nat_server_create(pool_bytes, max_slots, C.byref(self._h))
        if rc != NAT_OK:
            msg = self._err()
            self._L.nat_server_destroy(self._h)
            raise NatError(rc, msg)

    def _err(self) -> str:
        buf = C.create_string_buffer(512)
        self._L.nat_server_last_error(self._h, buf, 512)
        return buf.value.decode()

    def _check(self, rc):
        if rc != NAT_OK:
            raise NatError(rc, self._err())

    def close(self):
        if self._h and self._h.value:
            self._L.nat_server_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, req: Request) -> int:
        rid = C.c_int64()
        r = req.c()
        self._check(self._L.nat_server_submit(self._h, C.byref(r), C.byref(rid)))
        return rid.value

    def step(self):
        self._check(self._L.nat_server_step(self._h))

    def run(self, max_steps: int) -> int:
        """Up to max_steps server steps in one call; returns the number run
        (fewer when no solve is live)."""
        done = C.c_int()
        self._check(self._L.nat_server_run(self._h, int(max_steps), C.byref(done)))
        return done.value

    def poll(self, wait: bool = False, max_ids: int = 4096):
        ids = (C.c_int64 * max_ids)()
        n = C.c_int()
        self._check(self._L.nat_server_poll(self._h, ids, max_ids, C.byref(n), int(wait)))
        return [ids[i] for i in range(n.value)]

    def result_arrays(self, rid: int, n_nodes: int):
        rho = np.empty(n_nodes)
        u = np.empty((2, n_nodes))
        n = C.c_int64()
        st = C.c_int()
        self._check(self._L.nat_server_result(self._h, rid, rho.ctypes.data_as(C.POINTER(C.c_double)),
                                              u.ctypes.data_as(C.POINTER(C.c_double)), C.byref(n), C.byref(st)))
        return rho[: n.value], u[:, : n.value], st.value

    def stats(self) -> dict:
        s = _Stats()
        self._check(self._L.nat_server_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in _Stats._fields_}

    @property
    def busy(self) -> bool:
        st = self.stats()
        return st["pending"] + st["live"] + st["completing"] > 0


def workload(n: int = 512, seed: int = 0, rate: float = 200.0, steps_range=(50, 2000)):
    """The serving workload: n independent 2-D periodic solves, Poisson
    arrivals at `rate` per second; per request (seeded): Taylor-Green or
    double shear layer, BGK or KBC, cells per side in {4, 8, 16, 32, 64},
    FE order 2..6, Ma in [0.02, 0.1], Re in [100, 5000], steps in steps_range."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n))
    reqs = []
    for i in range(n):
        kind = int(rng.integers(0, 2))
        N = int(rng.choice([4, 8, 16, 32, 64]))
        L = 2 * math.pi if kind == INIT_TAYLOR_GREEN else 1.0
        reqs.append(Request(collision="BGK_STANDARD" if rng.integers(0, 2) == 0 else "KBC_STANDARD",
                            order=int(rng.integers(2, 7)), cells=(N, N), length=(L, L),
                            Ma=float(rng.uniform(0.02, 0.1)), Re=float(rng.uniform(100, 5000)),
                            steps=int(rng.integers(steps_range[0], steps_range[1] + 1)), init=kind))
    return arrivals, reqs


def run_workload(arrivals, reqs, pool_bytes: int = 8 << 30, max_slots: int = 512, steps_per_call: int = 8):
    """Replay the request stream in wall-clock time through one server.
    Requests are submitted as their arrival time passes; between checks the
    server runs up to steps_per_call steps in one C call.  Returns throughput
    (over the whole run, and over the arrival window: completions while
    requests were still arriving) and latency statistics (arrival to result
    on the host)."""
    lat = {}
    with Server(pool_bytes, max_slots) as srv:
        t0 = time.perf_counter()
        nxt = 0
        submit_t = {}
        done_t = {}
        id2req = {}
        n = len(reqs)
        while len(lat) < n:
            now = time.perf_counter() - t0
            while nxt < n and arrivals[nxt] <= now:
                rid = srv.submit(reqs[nxt])
                submit_t[rid] = t0 + arrivals[nxt]
                id2req[rid] = reqs[nxt]
                nxt += 1
            ran = srv.run(steps_per_call) if srv.busy else 0
            if not ran and nxt < n:
                time.sleep(max(0.0, min(1e-3, arrivals[nxt] - now)))
            for rid in srv.poll(wait=False):
                rho, u, st = srv.result_arrays(rid, id2req[rid].nodes)
                if st != 0:
                    raise NatError(st, f"request {rid} failed")
                done_t[rid] = time.perf_counter() - t0
                lat[rid] = time.perf_counter() - submit_t[rid]
        wall = time.perf_counter() - t0
        stats = srv.stats()
    l = np.array(sorted(lat.values()))
    first, last = float(arrivals[0]), float(arrivals[-1])
    in_window = sum(1 for t in done_t.values() if t <= last)
    return {
        "solves": n,
        "wall_s": wall,
        "solves_per_s": n / (wall - first),
        "solves_per_s_arrival_window": in_window / (last - first) if last > first else None,
        "offered_per_s": (n - 1) / (last - first) if last > first else None,
        "latency_p50_s": float(np.percentile(l, 50)),
        "latency_p99_s": float(np.percentile(l, 99)),
        "node_updates_per_s": stats["node_updates"] / (wall - first),
        "server_steps": stats["steps"],
        "launches": stats["launches"],
        "graph_builds": stats["graph_builds"],
        "graph_updates": stats["graph_updates"],
        "host_rebuild_s": stats["rebuild_ns"] * 1e-9,
    }


def run_sequential(reqs, precision: str = "fp64"):
    """The plain path: the same requests one at a time through the
    single-solve C ABI (create, upload the initial state, run, read rho / u).
    Returns solves/s and the per-solve service times."""
    from . import Solver, SolverSpec
    from . import problems as P
    times = []
    t0 = time.perf_counter()
    for r in reqs:
        t1 = time.perf_counter()
        spec = SolverSpec(stencil="D2Q9", order=r.order, cells=r.cells, length=r.length, scaling=r.scaling,
                          viscosity=r.viscosity, cfl=r.cfl, collision=r.collision, precision=precision)
        X = P.node_coords(r.cells, r.order, r.length)
        if r.init == INIT_TAYLOR_GREEN:
            rho, u = P.taylor_green_2d(X, r.Ma, L=r.length[0])
        else:
            rho, u = P.shear_layer_2d(X, r.kappa, r.delta, L=r.length[0])
        with Solver(spec) as sol:
            sol.upload_f(P.equilibrium("D2Q9", r.scaling, rho, u))
            sol.step(r.steps)
            sol.download_macro()
        times.append(time.perf_counter() - t1)
    wall = time.perf_counter() - t0
    return {"solves": len(reqs), "wall_s": wall, "solves_per_s": len(reqs) / wall,
            "service_p50_s": float(np.percentile(times, 50)), "service_p99_s": float(np.percentile(times, 99))}
