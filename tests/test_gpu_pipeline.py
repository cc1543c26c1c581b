"""Pipelined host I/O through the C ABI: nat_upload_f on its own copy stream
(two input staging buffers) and conversion stream (into a spare state
buffer), asynchronous read-back tickets (nat_download_macro_async /
nat_wait).

Each pipelined result must equal, bit for bit, the blocking
upload -> step -> download of the same state, while the next state's upload
is already enqueued (the double-buffered staging must not leak one state into
another).  Ticket status: a density underflow in a step is reported by the
wait of the ticket that follows it; tickets reused by the ring (more than 8
outstanding) stay valid and keep their status.
"""
import numpy as np
import pytest

import natrium_gb300 as N
from tests.gpu_cases import make_case, periodic_state

pytestmark = pytest.mark.gpu


def _pinned(shape):
    torch = pytest.importorskip("torch")
    return torch.empty(shape, dtype=torch.float64).pin_memory().numpy()


def _blocking(sol, f):
    sol.upload_f(f)
    sol.step(1)
    return sol.download_macro()


@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
@pytest.mark.parametrize("stencil,cells,p", [("D2Q9", (6, 5), 3), ("D3Q19", (4, 4, 4), 4)])
def test_pipelined_readback_equals_blocking(gpu_lib, stencil, cells, p, precision):
    st, mesh, dt, tau, spec = make_case(stencil, cells, p, True, "BGK_STANDARD", precision=precision)
    states = [np.ascontiguousarray(periodic_state(mesh, st, seed=s)) for s in range(5)]
    with N.Solver(spec) as sol:
        expect = [_blocking(sol, f) for f in states]
        f_pin = [_pinned(f.shape) for f in states]
        for a, b in zip(f_pin, states):
            a[...] = b
        rho = [_pinned(sol.n_ref) for _ in states]
        u = [_pinned((sol.D, sol.n_ref)) for _ in states]
        tickets = []
        for k in range(len(states)):
            sol.upload_f(f_pin[k])
            sol.step_async(1, True)
            tickets.append(sol.download_macro_async(rho[k], u[k]))
            if k >= 1:
                sol.wait(tickets[k - 1])
        sol.wait(tickets[-1])
        for k, (r, v) in enumerate(expect):
            assert np.array_equal(rho[k], r), k
            assert np.array_equal(u[k], v), k


@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
@pytest.mark.parametrize("stencil,cells,p,dg", [("D2Q9", (6, 5), 3, False), ("D3Q19", (4, 4, 4), 4, True)])
def test_upload_into_spare_buffer(gpu_lib, stencil, cells, p, dg, precision):
    """nat_upload_f converts into a spare state buffer on its own streams and
    then makes it the current one: two uploads in a row leave the second
    state; an upload while steps are in flight replaces the state only for
    the steps after it; the previous current buffer, now the spare, is
    reused by the next upload without corrupting anything in flight."""
    st, mesh, dt, tau, spec = make_case(stencil, cells, p, dg, "BGK_STANDARD", precision=precision)
    states = [np.ascontiguousarray(periodic_state(mesh, st, seed=s)) for s in range(4)]
    with N.Solver(spec) as sol:
        # the reference for each: upload, read back f, one step, read back rho/u
        ref_f, ref_m = [], []
        for f in states:
            sol.upload_f(f)
            ref_f.append(sol.download_f())
            sol.step(1)
            ref_m.append(sol.download_macro())
        # two uploads in a row: the second state is the current one
        sol.upload_f(states[0])
        sol.upload_f(states[1])
        assert np.array_equal(sol.download_f(), ref_f[1])
        # upload, step (async), upload, step, ... with no synchronisation
        for k in range(4):
            sol.upload_f(states[k])
            sol.step_async(1, True)
        r, u = sol.download_macro()
        assert np.array_equal(r, ref_m[3][0]) and np.array_equal(u, ref_m[3][1])
        # a step after an upload continues from the uploaded state
        sol.upload_f(states[2])
        sol.step(1)
        r, u = sol.download_macro()
        assert np.array_equal(r, ref_m[2][0]) and np.array_equal(u, ref_m[2][1])


def test_ticket_ring_reuse(gpu_lib):
    st, mesh, dt, tau, spec = make_case("D2Q9", (4, 4), 2, True, "BGK_STANDARD")
    f0 = np.ascontiguousarray(periodic_state(mesh, st, seed=3))
    with N.Solver(spec) as sol:
        r_ref, u_ref = _blocking(sol, f0)
        bufs = [(np.empty(sol.n_ref), np.empty((sol.D, sol.n_ref))) for _ in range(11)]
        tickets = []
        for r, u in bufs:
            sol.upload_f(f0)
            sol.step_async(1, True)
            tickets.append(sol.download_macro_async(r, u))
        assert tickets == list(range(tickets[0], tickets[0] + 11))
        sol.wait(tickets[0])  # its slot was reused: complete, status kept
        sol.wait(tickets[-1])
        for r, u in bufs:
            assert np.array_equal(r, r_ref) and np.array_equal(u, u_ref)
        for bad in (0, tickets[-1] + 1):
            with pytest.raises(N.NatError) as ei:
                sol.wait(bad)
            assert ei.value.code == N.NAT_ERR_INVALID_ARG


def test_ticket_reports_density_underflow(gpu_lib):
    """rho < 1e-10 in a pipelined step -> CollisionException from the wait of
    the ticket after it (CollisionOperator.h:106-109); the next ticket is
    clean."""
    st, mesh, dt, tau, spec = make_case("D2Q9", (4, 4), 2, False, "BGK_STANDARD")
    good = np.ascontiguousarray(periodic_state(mesh, st, seed=1))
    bad = np.zeros_like(good)
    with N.Solver(spec) as sol:
        r, u = np.empty(sol.n_ref), np.empty((sol.D, sol.n_ref))
        sol.upload_f(bad)
        sol.step_async(1, True)
        t1 = sol.download_macro_async(r, u)
        sol.upload_f(good)
        sol.step_async(1, True)
        t2 = sol.download_macro_async(r, u)
        with pytest.raises(N.CollisionException):
            sol.wait(t1)
        sol.wait(t2)


def test_unwaited_ticket_status_is_not_lost(gpu_lib):
    """A failing ticket nobody waited for, whose slot the ring reused: its
    status comes with the next wait."""
    st, mesh, dt, tau, spec = make_case("D2Q9", (4, 4), 2, False, "BGK_STANDARD")
    good = np.ascontiguousarray(periodic_state(mesh, st, seed=2))
    with N.Solver(spec) as sol:
        r, u = np.empty(sol.n_ref), np.empty((sol.D, sol.n_ref))
        sol.upload_f(np.zeros_like(good))
        sol.step_async(1, True)
        sol.download_macro_async(r, u)  # never waited for
        last = None
        for _ in range(8):
            sol.upload_f(good)
            sol.step_async(1, True)
            last = sol.download_macro_async(r, u)
        with pytest.raises(N.CollisionException):
            sol.wait(last)
        sol.upload_f(good)
        sol.step_async(1, True)
        sol.wait(sol.download_macro_async(r, u))
