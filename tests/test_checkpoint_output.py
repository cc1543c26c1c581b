"""Checkpoint and solution output (the reference's solver/Checkpoint.cpp and
CFDSolver.cpp:1001-1069).

A run interrupted by a checkpoint and resumed in a fresh solver gives the
same f bit for bit as the uninterrupted run; the VTU output carries the
lattice nodes, the p^D sub-cells of every element and the fields of the last
collision.
"""
import dataclasses
import xml.etree.ElementTree as ET

import numpy as np
import pytest

import natrium_gb300 as N
from tests.gpu_cases import make_case, periodic_state, thermal_case, thermal_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "fp32dev"])
def test_checkpoint_resume_is_bitwise(gpu_lib, tmp_path, precision):
    st, mesh, dt, tau, spec = make_case("D3Q19", (4, 4, 2), 2, True, "BGK_STANDARD", precision=precision)
    f0 = periodic_state(mesh, st, seed=17)
    path = str(tmp_path / "run.ckpt")
    with N.Solver(spec) as a:
        a.upload_f(f0)
        a.step(4)
        a.save_checkpoint(path, iteration=4, time=4 * a.dt)
        a.step(3)
        fa = a.download_f()
    with N.Solver(spec) as b:
        it, t = b.load_checkpoint(path)
        assert it == 4 and t == pytest.approx(4 * b.dt, rel=0, abs=0)
        b.step(3)
        fb = b.download_f()
    assert np.array_equal(fa, fb)


def test_checkpoint_resume_two_populations_with_walls(gpu_lib, tmp_path):
    st, mesh, dt, tau, spec = thermal_case((4, 4), 2, True)
    spec.precision = "fp32dev"
    spec.periodic = (True, False, True)
    rho0, u0, T0, f0, g0 = thermal_state(mesh, st, seed=6)
    path = str(tmp_path / "thermal.ckpt")
    with N.Solver(spec) as a:
        a.set_boundary(2, "DO_NOTHING")
        a.upload_f(f0)
        a.upload_g(g0)
        a.step(3)
        a.save_checkpoint(path, 3, 0.5)
        a.step(2)
        fa, ga = a.download_f(), a.download_g()
    with N.Solver(spec) as b:
        b.set_boundary(2, "DO_NOTHING")
        assert b.load_checkpoint(path) == (3, 0.5)
        b.step(2)
        fb, gb = b.download_f(), b.download_g()
    assert np.array_equal(fa, fb) and np.array_equal(ga, gb)


def test_checkpoint_of_another_lattice_is_refused(gpu_lib, tmp_path):
    st, mesh, dt, tau, spec = make_case("D2Q9", (4, 4), 2, False, "BGK_STANDARD")
    path = str(tmp_path / "a.ckpt")
    with N.Solver(spec) as a:
        a.upload_f(periodic_state(mesh, st, seed=1))
        a.save_checkpoint(path)
    st2, mesh2, dt2, tau2, spec2 = make_case("D2Q9", (4, 4), 3, False, "BGK_STANDARD")
    with N.Solver(spec2) as b:
        with pytest.raises(N.NatError):
            b.load_checkpoint(path)
    bad = tmp_path / "junk.ckpt"
    bad.write_bytes(b"not a checkpoint at all" * 8)
    with N.Solver(spec) as c:
        with pytest.raises(N.NatError):
            c.load_checkpoint(str(bad))


def test_checkpoint_of_a_mapped_mesh(gpu_lib, tmp_path):
    """Resume on the same vertex grid is bitwise; another grid of the same
    size is refused."""
    from natrium_gb300 import problems as P
    V = P.wavy_grid((4, 4), (1.0, 1.0), 0.1)
    spec = N.SolverSpec(stencil="D2Q9", order=2, cells=(4, 4), length=(1.0, 1.0), scaling=10.0, viscosity=1e-3,
                        topology="dg", vertices=V)
    X = P.mapped_node_coords(V, 2, "dg")
    u = 0.05 * np.stack([np.sin(2 * np.pi * X[:, 1]), np.cos(2 * np.pi * X[:, 0])]) * 10.0
    f0 = P.equilibrium("D2Q9", 10.0, np.ones(X.shape[0]), u)
    path = str(tmp_path / "mapped.ckpt")
    with N.Solver(spec) as a:
        a.upload_f(f0)
        a.step(3)
        a.save_checkpoint(path, iteration=3, time=3 * a.dt)
        a.step(2)
        fa = a.download_f()
    with N.Solver(spec) as b:
        it, t = b.load_checkpoint(path)
        assert it == 3
        b.step(2)
        assert np.array_equal(b.download_f(), fa)
    other = dataclasses.replace(spec, vertices=P.wavy_grid((4, 4), (1.0, 1.0), 0.05))
    with N.Solver(other) as c:
        with pytest.raises(N.NatError):
            c.load_checkpoint(path)


@pytest.mark.parametrize("dg", [False, True])
def test_vtu_output(gpu_lib, tmp_path, dg):
    st, mesh, dt, tau, spec = make_case("D2Q9", (3, 2), 3, dg, "BGK_STANDARD")
    f0 = periodic_state(mesh, st, seed=2)
    path = str(tmp_path / "t.vtu")
    with N.Solver(spec) as sol:
        sol.upload_f(f0)
        sol.step(2)
        rho, u = sol.download_macro()
        sol.write_vtu(path)
    root = ET.parse(path).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    assert int(piece.get("NumberOfPoints")) == mesh.n_nodes
    assert int(piece.get("NumberOfCells")) == 3 * 2 * 3 * 3
    arrays = {a.get("Name"): np.array(a.text.split(), dtype=float) for a in piece.iter("DataArray") if a.get("Name")}
    assert np.array_equal(arrays["rho"], rho)
    assert np.array_equal(arrays["ux"], u[0]) and np.array_equal(arrays["uy"], u[1])
    pts = np.array(piece.find("Points/DataArray").text.split(), dtype=float).reshape(-1, 3)
    assert np.allclose(pts[:, :2], mesh.coords()[:, :2], rtol=0, atol=1e-14)
    conn = arrays["connectivity"].astype(int).reshape(-1, 4)
    assert conn.min() == 0 and conn.max() < mesh.n_nodes
