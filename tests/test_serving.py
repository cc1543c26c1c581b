"""Continuous-batching server: each result is the same alone and in the
mix, matches the single-solve path, and admission by HBM footprint works."""
import math

import numpy as np
import pytest

import natrium_gb300 as N
import oracle as O
from natrium_gb300 import problems as P
from natrium_gb300.serving import INIT_SHEAR_LAYER, INIT_TAYLOR_GREEN, Request, Server, workload


def test_workload_is_seeded_and_in_range():
    a1, r1 = workload(64, seed=3)
    a2, r2 = workload(64, seed=3)
    assert np.array_equal(a1, a2) and r1 == r2
    assert np.all(np.diff(a1) > 0)
    for r in r1:
        assert r.cells[0] in (4, 8, 16, 32, 64) and 2 <= r.order <= 6
        assert 0.02 <= r.Ma <= 0.1 and 100 <= r.Re <= 5000 and 50 <= r.steps <= 2000
        assert r.collision in ("BGK_STANDARD", "KBC_STANDARD")


def _run(srv, reqs):
    ids = [srv.submit(r) for r in reqs]
    out = {}
    while len(out) < len(ids):
        if srv.busy:
            srv.step()
        for rid in srv.poll(wait=not srv.stats()["live"]):
            out[rid] = srv.result_arrays(rid, reqs[ids.index(rid)].nodes)
    return [out[i] for i in ids]


MIX = [
    Request("BGK_STANDARD", 4, (8, 8), steps=37),
    Request("KBC_STANDARD", 3, (4, 8), steps=20, Ma=0.08, Re=300),
    Request("BGK_STANDARD", 2, (16, 16), steps=55, init=INIT_SHEAR_LAYER, length=(1.0, 1.0), Re=2000),
    Request("KBC_STANDARD", 6, (4, 4), steps=12, init=INIT_SHEAR_LAYER, length=(1.0, 1.0)),
    Request("BGK_STANDARD", 5, (8, 4), steps=30, Ma=0.03),
    Request("BGK_STANDARD", 1, (32, 32), steps=25),
]


@pytest.mark.gpu
def test_alone_equals_in_mix(gpu_lib):
    with Server(1 << 30, 64) as srv:
        mixed = _run(srv, MIX)
    for i, r in enumerate(MIX):
        with Server(1 << 30, 4) as srv:
            alone = _run(srv, [r])[0]
        assert mixed[i][2] == 0 and alone[2] == 0
        assert np.array_equal(mixed[i][0], alone[0]), i
        assert np.array_equal(mixed[i][1], alone[1]), i


@pytest.mark.gpu
@pytest.mark.parametrize("req", MIX[:5], ids=lambda r: f"{r.collision}-p{r.order}-{r.cells[0]}x{r.cells[1]}-{r.init}")
def test_served_matches_single_solve(gpu_lib, req):
    """Same request through the single-solve C ABI (FP32 deviation): rho and
    u within 1e-6 relative L2 (the initial states are built by different
    code, host numpy vs device, and differ in the last float bit)."""
    with Server(1 << 30, 4) as srv:
        rho_s, u_s, st = _run(srv, [req])[0]
    spec = N.SolverSpec(stencil="D2Q9", order=req.order, cells=req.cells, length=req.length,
                        scaling=req.scaling, viscosity=req.viscosity, cfl=req.cfl, collision=req.collision,
                        precision="fp32dev")
    X = P.node_coords(req.cells, req.order, req.length)
    if req.init == INIT_TAYLOR_GREEN:
        rho, u = P.taylor_green_2d(X, req.Ma, L=req.length[0])
    else:
        rho, u = P.shear_layer_2d(X, req.kappa, req.delta, L=req.length[0])
    f0 = P.equilibrium("D2Q9", req.scaling, rho, u)
    with N.Solver(spec) as sol:
        sol.upload_f(f0)
        sol.step(req.steps)
        rho1, u1 = sol.download_macro()
    # device lattice order (periodic duplicates folded) -> drop duplicates
    nx = req.cells[0] * req.order
    ny = req.cells[1] * req.order
    keep = np.ones((ny + 1, nx + 1), bool)
    keep[-1, :] = False
    keep[:, -1] = False
    k = keep.ravel()
    r1 = rho1[k]
    v1 = u1[:, k]
    assert np.sqrt(np.sum((rho_s - r1) ** 2) / np.sum(r1 ** 2)) <= 1e-7
    assert np.sqrt(np.sum((u_s - v1) ** 2) / np.sum(v1 ** 2)) <= 1e-6


@pytest.mark.gpu
def test_admission_waits_for_memory(gpu_lib):
    """A pool that holds only one of the solves at a time: they are admitted
    one after another and all finish."""
    reqs = [Request("BGK_STANDARD", 4, (32, 32), steps=5) for _ in range(4)]
    nodes = reqs[0].nodes
    one = 2 * 9 * nodes * 4 + 3 * nodes * 8
    assert one + 4096 > (1 << 20)
    with Server(one + 4096, 8) as srv:
        ids = [srv.submit(r) for r in reqs]
        srv.step()
        st = srv.stats()
        assert st["live"] == 1 and st["pending"] == 3
        done = 0
        while done < len(ids):
            if srv.busy:
                srv.step()
            for rid in srv.poll(wait=not srv.stats()["live"]):
                srv.result_arrays(rid, nodes)
                done += 1
    assert done == 4


@pytest.mark.gpu
def test_invalid_request_rejected(gpu_lib):
    with Server(1 << 24, 4) as srv:
        with pytest.raises(N.NatError):
            srv.submit(Request("BGK_STANDARD", 9, (4, 4)))
        with pytest.raises(N.NatError):
            srv.submit(Request("BGK_STANDARD", 4, (4096, 4096)))  # larger than the pool


@pytest.mark.gpu
@pytest.mark.parametrize("req", [Request("BGK_STANDARD", 3, (8, 8), steps=40, Ma=0.05, Re=500),
                                 Request("KBC_STANDARD", 4, (4, 8), steps=30, Ma=0.08, Re=300)],
                         ids=["bgk-p3-8x8", "kbc-p4-4x8"])
def test_served_matches_oracle(gpu_lib, req):
    """A served solve (FP32 deviation storage, in a mix with another request)
    against the CPU oracle's FP64 run of the same request: the reference's
    copy + CSR SpMV + collide per step from the same Taylor-Green equilibrium
    (TaylorGreenVortex2D.cpp:36-59).  Relative L2 of u within 1e-6, of rho
    within 1e-7."""
    other = Request("BGK_STANDARD", 2, (16, 16), steps=60, init=INIT_SHEAR_LAYER, length=(1.0, 1.0), Re=2000)
    with Server(1 << 30, 8) as srv:
        rho_s, u_s, st = _run(srv, [req, other])[0]
    assert st == 0
    so = O.stencil("D2Q9", req.scaling)
    mesh = O.Mesh(2, req.cells, req.order, False, (req.length[0], req.length[1], 1.0))
    dt = O.time_step(mesh.h_min(), req.order, so.max_speed, req.cfl)
    tau = req.viscosity / (dt * so.cs2) + 0.5
    rho0, u0 = O.tgv2d_init(mesh.coords(), req.Ma, L=req.length[0])
    f = O.equilibrium(so, rho0, np.ascontiguousarray(u0))
    S = O.SLOperator(mesh, so, dt)
    rho = np.zeros(mesh.n_nodes)
    u = np.zeros((2, mesh.n_nodes))
    for _ in range(req.steps):
        f = S.stream(f)
        O.collide(so, req.collision, tau, f, rho, u)
    # oracle lattice (N p + 1 per axis) -> the served lattice (periodic duplicates folded)
    nx, ny = req.cells[0] * req.order, req.cells[1] * req.order
    keep = np.ones((ny + 1, nx + 1), bool)
    keep[-1, :] = False
    keep[:, -1] = False
    k = keep.ravel()
    r1, v1 = rho[k], u[:, k]
    assert np.sqrt(np.sum((rho_s - r1) ** 2) / np.sum(r1 ** 2)) <= 1e-7
    assert np.sqrt(np.sum((u_s - v1) ** 2) / np.sum(v1 ** 2)) <= 1e-6


@pytest.mark.gpu
def test_server_run_batches_steps(gpu_lib):
    """nat_server_run advances several steps per call and gives the same
    results as single steps."""
    reqs = [Request("BGK_STANDARD", 3, (8, 8), steps=33), Request("KBC_STANDARD", 2, (8, 4), steps=17)]
    with Server(1 << 30, 8) as srv:
        single = _run(srv, reqs)
    with Server(1 << 30, 8) as srv:
        ids = [srv.submit(r) for r in reqs]
        out = {}
        while len(out) < len(ids):
            if srv.busy:
                assert srv.run(7) >= 0
            for rid in srv.poll(wait=not srv.stats()["live"]):
                out[rid] = srv.result_arrays(rid, reqs[ids.index(rid)].nodes)
        batched = [out[i] for i in ids]
    for a, b in zip(single, batched):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
