"""Failure detection on the GPU without a fault: the bounded waits of the
bulk-copy kernels.

The tile kernel (sl_step_v2.cuh) and the bulk-copy row kernel (sl_rowt.cuh)
wait on mbarriers for their cp.async.bulk copies.  Every such wait has a poll
limit; one that runs out sets the TIMEOUT bit of the status word, waits
(bounded) for the copies still in flight and stops its tile, and the host
returns NAT_ERR_TIMEOUT.  A wait limit of 0 makes every wait run out at once
while the copies themselves are ordinary, so this path runs here without a
hang or a fault.  Afterwards the context is usable: the same step with the
default limit matches the oracle.
"""
import numpy as np
import pytest

import natrium_gb300 as N
import oracle as O
from tests.gpu_cases import make_case, oracle_step, periodic_state, rel_l2

pytestmark = pytest.mark.gpu


# 12 x 4 x 2 cells: x rows long enough for the bulk-copy row kernel's copies
@pytest.mark.parametrize("variant,kind", [(3, 2), (6, 6)], ids=["tile", "bulk-copy-row"])
def test_copy_wait_that_runs_out_is_reported(gpu_lib, variant, kind):
    st, mesh, dt, tau, spec = make_case("D3Q19", (12, 4, 2), 4, True, "BGK_STANDARD", precision="fp32dev")
    f0 = periodic_state(mesh, st, seed=5)
    f1, rho1, u1 = oracle_step(O.SLOperator(mesh, st, dt), st, "BGK_STANDARD", tau, f0, 1)
    with N.Solver(spec) as sol:
        sol.set_kernel_variant(variant)
        assert sol.kernel_variant == kind
        sol.upload_f(f0)
        sol.set_wait_limit(0)
        with pytest.raises(N.NatError) as ei:
            sol.step(1)
        assert ei.value.code == N.NAT_ERR_TIMEOUT
        assert "ran out" in str(ei.value)
        # the status was cleared and the context stays usable
        sol.set_wait_limit(1 << 24)
        sol.upload_f(f0)
        sol.step(1)
        assert rel_l2(sol.download_f(), f1) <= 1e-6


def test_timeout_reaches_a_readback_ticket(gpu_lib):
    st, mesh, dt, tau, spec = make_case("D3Q19", (4, 4, 2), 4, True, "BGK_STANDARD", precision="fp32dev")
    f0 = np.ascontiguousarray(periodic_state(mesh, st, seed=6))
    with N.Solver(spec) as sol:
        sol.set_kernel_variant(3)
        r, u = np.empty(sol.n_ref), np.empty((sol.D, sol.n_ref))
        sol.set_wait_limit(0)
        sol.upload_f(f0)
        sol.step_async(1, True)
        t = sol.download_macro_async(r, u)
        with pytest.raises(N.NatError) as ei:
            sol.wait(t)
        assert ei.value.code == N.NAT_ERR_TIMEOUT


def test_kernels_without_copies_ignore_the_limit(gpu_lib):
    """The row kernels that load with plain loads have no waits: a limit of
    0 changes nothing for them."""
    st, mesh, dt, tau, spec = make_case("D3Q19", (4, 4, 2), 4, True, "BGK_STANDARD", precision="fp32dev")
    f0 = periodic_state(mesh, st, seed=7)
    f1, _, _ = oracle_step(O.SLOperator(mesh, st, dt), st, "BGK_STANDARD", tau, f0, 1)
    with N.Solver(spec) as sol:
        sol.set_kernel_variant(4)
        assert sol.kernel_variant == 3
        sol.set_wait_limit(0)
        sol.upload_f(f0)
        sol.step(1)
        assert rel_l2(sol.download_f(), f1) <= 1e-6
