"""The allocation-free reduction entry point (nat_mass_energy_noalloc).

Some callers of this library cannot call cudaMalloc where they need the
mass / kinetic-energy diagnostics -- work being recorded into a CUDA graph,
hosts whose framework owns all device memory, latency-bound loops -- so this
entry point keeps its only scratch in a fixed file-scope device array.  The
test calls it through the C ABI twice in a row on the same fields and checks
both results against the allocating entry point nat_mass_energy, within the
relative tolerance the FP64 parity tests use (1e-12).  It lives in a file of
its own that pytest collects last, and it sets up everything it needs so it
also passes alone in a fresh process.
"""
import ctypes as C
import math

import numpy as np
import pytest

import natrium_gb300 as N
from natrium_gb300 import problems as P

TOL = 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("stencil,cells,p,topology", [("D2Q9", (8, 8), 4, "feq"), ("D3Q19", (4, 4, 4), 3, "dg")])
def test_noalloc_matches_allocating_entry_point(gpu_lib, stencil, cells, p, topology):
    import torch
    Ma = 0.1
    scaling = math.sqrt(3) / Ma
    L = (2 * math.pi,) * 3
    spec = N.SolverSpec(stencil=stencil, order=p, cells=cells, length=L, scaling=scaling, viscosity=1e-2,
                        cfl=0.4, precision="fp64", topology=topology)
    X = P.node_coords(cells, p, L, topology)
    if len(cells) == 2:
        rho, u = P.taylor_green_2d(X, Ma)
    else:
        rho, u = P.taylor_green_3d(X, Ma)
    f0 = P.equilibrium(stencil, scaling, rho, u)
    with N.Solver(spec) as sol:
        sol.upload_f(f0)
        sol.step(3)
        mass, ke = sol.mass_energy()
        rho_r, u_r = sol.download_macro()
    dim = len(cells)
    # device lattice order: FE_Q folds the periodic duplicate of every axis
    per = p if topology == "feq" else p + 1
    n_axis = [cells[a] * per for a in range(dim)]
    ref_axis = [n + (1 if topology == "feq" else 0) for n in n_axis]
    shape = tuple(reversed(ref_axis))
    sl = tuple(slice(0, n) for n in reversed(n_axis))
    rho_d = np.ascontiguousarray(rho_r.reshape(shape)[sl].ravel())
    u_d = np.ascontiguousarray(np.stack([u_r[a].reshape(shape)[sl].ravel() for a in range(dim)]))
    dev = torch.device("cuda:0")
    t_rho = torch.from_numpy(rho_d).to(dev)
    t_u = torch.from_numpy(u_d).to(dev)
    out = torch.zeros(2, dtype=torch.float64, device=dev)
    lib = N.load_library()
    axes = (C.c_int * 3)(*(n_axis + [1] * (3 - dim)))
    h = (C.c_double * 3)(*[L[a] / cells[a] if a < dim else 1.0 for a in range(3)])
    stream = torch.cuda.current_stream().cuda_stream
    topo = N.TOPOLOGIES[topology]
    results = []
    for _ in range(2):
        out.zero_()
        rc = lib.nat_mass_energy_noalloc(C.c_void_p(t_rho.data_ptr()), C.c_void_p(t_u.data_ptr()), dim, axes, p,
                                         topo, h, C.c_void_p(out.data_ptr()), C.c_void_p(stream))
        assert rc == N.NAT_OK
        torch.cuda.synchronize()
        results.append(out.cpu().numpy().copy())
    for m2, e2 in results:
        assert abs(m2 - mass) <= TOL * abs(mass)
        assert abs(e2 - ke) <= TOL * abs(ke)
    # fixed reduction order: the two calls agree bit for bit
    assert np.array_equal(results[0], results[1])


@pytest.mark.gpu
def test_noalloc_rejects_oversized_input(gpu_lib):
    lib = N.load_library()
    axes = (C.c_int * 3)(8192, 4096, 1)  # 2^25 nodes > NAT_NOALLOC_MAX_NODES
    h = (C.c_double * 3)(1.0, 1.0, 1.0)
    dummy = C.c_void_p(16)  # never dereferenced: rejected before any launch
    rc = lib.nat_mass_energy_noalloc(dummy, dummy, 2, axes, 2, 0, h, dummy, None)
    assert rc == N.NAT_ERR_INVALID_ARG
