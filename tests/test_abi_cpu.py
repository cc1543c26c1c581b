"""C-ABI checks that need no GPU: the library builds/loads, exports every
symbol include/natgpu.h declares, and rejects bad specs before touching CUDA."""
import ctypes as C
import os
import re

import pytest

import natrium_gb300 as N
from natrium_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "natgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(nat_[a-z_0-9]+)\s*\(", txt)))


def test_library_builds_and_exports_header_symbols():
    path = B.build()
    assert os.path.exists(path)
    L = N.load_library()
    syms = header_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(L, s), s
    assert sorted(N.EXPORTS) == syms
    assert "sm_103a" in N.version()


@pytest.mark.parametrize("bad", [
    dict(order=0), dict(order=9), dict(scaling=-1.0), dict(viscosity=0.0),
    dict(cells=(0, 4)), dict(collision="BGK_STANDARD", topology="feq", length=(0.0, 1.0)),
])
def test_invalid_specs_are_rejected_without_gpu(bad):
    spec = N.SolverSpec(**{**dict(stencil="D2Q9", order=2, cells=(4, 4), scaling=1.0, viscosity=0.1), **bad})
    with pytest.raises(N.NatError) as ei:
        N.Solver(spec)
    assert ei.value.code == N.NAT_ERR_INVALID_ARG


def test_unsupported_combination_is_reported():
    # the reference throws for BGKIncompressible on anything but D2Q9
    # (collision/BGKIncompressible.cpp:54-55) and for KBC on D3Q19 (KBCStandard.cpp:79-81)
    for st, coll in (("D3Q19", "BGK_INCOMPRESSIBLE"), ("D3Q19", "KBC_STANDARD")):
        spec = N.SolverSpec(stencil=st, order=2, cells=(2, 2, 2), length=(1, 1, 1), scaling=1.0,
                            viscosity=0.1, collision=coll)
        with pytest.raises(N.NatError) as ei:
            N.Solver(spec)
        assert ei.value.code == N.NAT_ERR_UNSUPPORTED


def test_compressible_model_combinations_are_checked():
    # the compressible two-population model runs on D2Q25H only, and D2Q25H
    # only runs that model
    for st, coll, prec in (("D2Q9", "BGK_COMPRESSIBLE", "fp64"), ("D2Q25H", "BGK_STANDARD", "fp64"),
                           ("D2Q25H", "KBC_STANDARD", "fp32dev")):
        spec = N.SolverSpec(stencil=st, order=2, cells=(2, 2), length=(1, 1), scaling=1.0,
                            viscosity=0.1, collision=coll, precision=prec)
        with pytest.raises(N.NatError) as ei:
            N.Solver(spec)
        assert ei.value.code == N.NAT_ERR_UNSUPPORTED


def test_last_error_null_handle():
    L = N.load_library()
    buf = C.create_string_buffer(64)
    assert L.nat_last_error(None, buf, 64) == 0
    assert buf.value == b"null handle"


def test_lattice_beyond_32bit_indexing_is_refused_without_gpu():
    # 200^3 cells of p = 4 DG: 10^9 nodes x 19 populations > 2^31 -- refused
    # before anything is allocated or launched
    spec = N.SolverSpec(stencil="D3Q19", order=4, cells=(200, 200, 200), length=(1, 1, 1), scaling=1.0,
                        viscosity=0.1, topology="dg", precision="fp32dev")
    with pytest.raises(N.NatError) as ei:
        N.Solver(spec)
    assert ei.value.code == N.NAT_ERR_UNSUPPORTED
    assert "2^31" in str(ei.value)


def test_transfer_entry_points_check_arguments_without_gpu():
    """The pipelined-transfer and wait-limit entry points reject a null handle
    or null buffers before touching CUDA."""
    L = N.load_library()
    t = C.c_uint64(7)
    buf = (C.c_double * 4)()
    assert L.nat_download_macro_async(None, buf, buf, C.byref(t)) == N.NAT_ERR_INVALID_ARG
    assert t.value == 7  # untouched
    assert L.nat_wait(None, 1) == N.NAT_ERR_INVALID_ARG
    assert L.nat_set_wait_limit(None, 0) == N.NAT_ERR_INVALID_ARG
    assert L.nat_upload_f(None, buf) == N.NAT_ERR_INVALID_ARG


def test_async_readback_validates_host_arrays_without_gpu():
    """Solver.download_macro_async checks the host arrays before any C call
    (a handle-less Solver: the checks must raise before the library is
    reached)."""
    import numpy as np

    sol = N.Solver.__new__(N.Solver)
    sol.n_ref, sol.D = 10, 2
    sol._pending = {}
    sol._L = None  # any C call would fail with AttributeError, not ValueError
    good_r, good_u = np.empty(10), np.empty((2, 10))
    for r, u in [(np.empty(9), good_u), (good_r, np.empty((3, 10))), (good_r.astype(np.float32), good_u),
                 (good_r, np.empty((10, 2)).T), (np.empty(20)[::2], good_u)]:
        with pytest.raises(ValueError):
            sol.download_macro_async(r, u)
    ro = np.empty(10)
    ro.flags.writeable = False
    with pytest.raises(ValueError):
        sol.download_macro_async(ro, good_u)
    assert sol._pending == {}


def test_noalloc_reduction_checks_arguments_without_gpu():
    """nat_mass_energy_noalloc rejects, before any CUDA call, an axis that does
    not hold whole cells: its node weights repeat with the cell's period (p
    nodes per cell for FE_Q with the periodic duplicates folded, p + 1 for DG),
    so the reference layout's N p + 1 FE_Q count would silently give a wrong
    mass."""
    L = N.load_library()
    dummy = C.c_void_p(16)  # never dereferenced: every case is rejected before a launch
    h = (C.c_double * 3)(1.0, 1.0, 1.0)
    for n_axis, order, topo in (((33, 32, 1), 4, N.TOPOLOGIES["feq"]),   # 8 cells p=4 + the duplicate
                                ((32, 33, 1), 4, N.TOPOLOGIES["feq"]),
                                ((40, 41, 1), 4, N.TOPOLOGIES["dg"]),    # not a multiple of p + 1 = 5
                                ((0, 40, 1), 4, N.TOPOLOGIES["dg"])):
        axes = (C.c_int * 3)(*n_axis)
        rc = L.nat_mass_energy_noalloc(dummy, dummy, 2, axes, order, topo, h, dummy, None)
        assert rc == N.NAT_ERR_INVALID_ARG, n_axis
    axes = (C.c_int * 3)(32, 32, 1)
    assert L.nat_mass_energy_noalloc(dummy, dummy, 4, axes, 4, 0, h, dummy, None) == N.NAT_ERR_INVALID_ARG
    assert L.nat_mass_energy_noalloc(dummy, dummy, 2, axes, 0, 0, h, dummy, None) == N.NAT_ERR_INVALID_ARG
    assert L.nat_mass_energy_noalloc(None, dummy, 2, axes, 4, 0, h, dummy, None) == N.NAT_ERR_INVALID_ARG
