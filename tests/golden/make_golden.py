"""Regenerate the golden fixtures in tests/golden/.

1. ``known_answers.json`` -- the known answers that the reference's own unit
   and integration tests state for the stream + collide path, extracted from
   the reference's test sources (read as text; the reference cannot be built
   here):
     * SemiLagrangian{2,3}D_FaceCrossedFirst_test
       (test/advection/SemiLagrangian_test.cpp:227-456): every probe point
       p2, the expected face id, lambda and boundary point, parsed from the
       p2[...] assignments and BOOST_CHECK_* lines;
     * the tolerances and parameters of the constant-streaming tests
       (:519-596), the BGK invariant / collideAll tests
       (test/collision/BGKStandard_test.cpp:311-425), the KBC mass test
       (test/collision/KBCStandard_test.cpp:36-108) and the semi-Lagrangian
       Taylor-Green integration test
       (test/integrationtest/IntegrationTestCases.cpp:885-961).
2. ``oracle_*.npz`` -- small oracle outputs (one stream + collide step on
   seeded periodic inputs) that the GPU parity tests check against in
   addition to the live oracle.

Usage: python tests/golden/make_golden.py [--reference PATH]
PATH is the root of a NATriuM source tree; without --reference the
environment variable NATRIUM_REFERENCE is used.  Without either (or when the
directory does not exist), step 1 is skipped and the committed JSON is kept.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def _num(expr: str) -> float:
    expr = expr.strip()
    if not re.fullmatch(r"[0-9eE+\-*/. ()]+", expr):
        raise ValueError(expr)
    return float(eval(expr, {"__builtins__": {}}, {}))


def parse_face_crossed_first(src: str, test_name: str, dim: int):
    """Walk the body of one FaceCrossedFirst test statement by statement and
    record each probe (p2, expected face, lambda, boundary point)."""
    start = src.index(f"BOOST_AUTO_TEST_CASE({test_name})")
    end = src.index("/* with/without mapping */", start)
    body = re.sub(r"//[^\n]*", "", src[start:end])
    m = re.search(r"dealii::Point<%d> p2\(([^)]*)\)" % dim, body)
    p2 = [_num(x) for x in m.group(1).split(",")]
    probes = []
    cur = None
    for stmt in body.split(";"):
        st = " ".join(stmt.split())
        ma = re.search(r"p2\[(\d)\] = (.+)$", st)
        if ma and "faceCrossedFirst" not in st:
            p2[int(ma.group(1))] = _num(ma.group(2))
            continue
        mi = re.search(r"BOOST_CHECK_EQUAL\( sl\.faceCrossedFirst\(.*\), (-?\d+)\)$", st)
        if mi:
            probes.append({"p_out": list(p2), "face": int(mi.group(1)), "lambda": None, "pb": None})
            cur = None
            continue
        if re.search(r"result = sl\.faceCrossedFirst", st):
            cur = {"p_out": list(p2), "face": None, "lambda": None, "pb": [None] * dim}
            probes.append(cur)
            continue
        if cur is None:
            continue
        mf = re.search(r"BOOST_CHECK_EQUAL\(result, (-?\d+)\)$", st)
        if mf:
            cur["face"] = int(mf.group(1))
        ml = re.search(r"BOOST_CHECK_CLOSE\(lambda, ([^,]+),", st)
        if ml:
            cur["lambda"] = _num(ml.group(1))
        mc = re.search(r"BOOST_CHECK_CLOSE\(pb\[(\d)\], ([^,]+),", st)
        if mc:
            cur["pb"][int(mc.group(1))] = _num(mc.group(2))
        ms = re.search(r"BOOST_CHECK_SMALL\(pb\[(\d)\],", st)
        if ms:
            cur["pb"][int(ms.group(1))] = 0.0
    return probes


def known_answers(reference: str) -> dict:
    test_dir = os.path.join(reference, "src", "test")
    sl = open(os.path.join(test_dir, "advection", "SemiLagrangian_test.cpp")).read()
    out = {
        "source": "reference test sources (src/test/...), parsed by tests/golden/make_golden.py",
        "face_crossed_first": {
            "2d": {
                "cite": "test/advection/SemiLagrangian_test.cpp:227-321",
                "cell_lo": [0.0, 0.0], "cell_h": [0.125, 0.125], "p_in": [0.0625, 0.0625],
                "probes": parse_face_crossed_first(sl, "SemiLagrangian2D_FaceCrossedFirst_test", 2),
            },
            "3d": {
                "cite": "test/advection/SemiLagrangian_test.cpp:323-456",
                "cell_lo": [0.0, 0.0, 0.0], "cell_h": [0.125, 0.125, 0.125],
                "p_in": [0.0625, 0.0625, 0.0625],
                "probes": parse_face_crossed_first(sl, "SemiLagrangian3D_FaceCrossedFirst_test", 3),
            },
        },
    }
    # constant streaming: parameters and bound
    def grab(pattern, text, cast=float):
        m = re.search(pattern, text, re.S)
        return cast(m.group(1))

    cs2 = sl[sl.index("SemiLagrangian2D_ConstantStreaming_test) {"):]
    cs3 = sl[sl.index("SemiLagrangian3D_ConstantStreaming_test) {"):]
    out["constant_streaming"] = {
        "cite": "test/advection/SemiLagrangian_test.cpp:519-596",
        "2d": {"stencil": "D2Q9", "order": grab(r"fe_order = (\d+);", cs2, int),
               "refinement": grab(r"refinementLevel = (\d+);", cs2, int),
               "dt": grab(r"setDeltaT\(([0-9.]+)\)", cs2), "L": 1.0,
               "bound_norm_sqr": grab(r"BOOST_CHECK_LE\(result.norm_sqr\(\), ([0-9e.\-]+)\)", cs2)},
        "3d": {"stencil": "D3Q19", "order": grab(r"fe_order = (\d+);", cs3, int),
               "refinement": grab(r"refinementLevel = (\d+);", cs3, int),
               "dt": grab(r"setDeltaT\(([0-9.]+)\)", cs3), "L": 1.0,
               "bound_norm_sqr": grab(r"BOOST_CHECK_LE\(result.norm_sqr\(\), ([0-9e.\-]+)\)", cs3)},
    }
    bgk = open(os.path.join(test_dir, "collision", "BGKStandard_test.cpp")).read()
    inv = bgk[bgk.index("BGKStandardCollisionInvariants_test) {"):]
    out["bgk_invariants"] = {
        "cite": "test/collision/BGKStandard_test.cpp:311-356",
        "relax_param": grab(r"double tau = ([0-9.]+);", inv),
        "dt": grab(r"BGKStandard bgk\(tau, ([0-9.]+),", inv),
        "fixture": "f_i = 1.5 + sin(1.5 i) + 0.001 + i/(i+1) (integer division)",
        "mass_momentum_tol": grab(r"BOOST_CHECK_SMALL\(rhoBefore - rhoAfter, ([0-9e.\-]+)\)", inv),
        "prescribed_density": grab(r"prescribedDensity = ([0-9.]+);", inv),
        "fixed_point_tol": grab(r"BOOST_CHECK_SMALL\(feq.at\(i\) - feqAfterCollision.at\(i\), ([0-9e.\-]+)\)", inv),
    }
    ca = bgk[bgk.index("BGKStandard_collideAllD2Q9_test) {"):]
    out["bgk_collide_all"] = {
        "cite": "test/collision/BGKStandard_test.cpp:358-425 (D2Q9), :428-... (D3Q19)",
        "relax_param": grab(r"double tau = ([0-9.]+);", ca),
        "fixture": "f_i(j) = 1.5 + sin(1.5 i) + 0.001 + i/(i+1) + (0.5 cos j)^2 (integer division)",
        "refinement": 3, "dg_order": 1,
        "close_percent": grab(r"BOOST_CHECK_CLOSE\(localF.at\(0\), 0.0 \+ fAfterCollision.at\(0\)\(i\), ([0-9e.\-]+)\)", ca),
    }
    kbc = open(os.path.join(test_dir, "collision", "KBCStandard_test.cpp")).read()
    kb = kbc[kbc.index("KBCStandard_collideAll_test) {"):]
    out["kbc_mass"] = {
        "cite": "test/collision/KBCStandard_test.cpp:36-108",
        "relax_param": grab(r"double tau = ([0-9.]+);", kb),
        "fixture": "f_i = 0.1 i + 0.1",
        "tol": grab(r"BOOST_CHECK_SMALL\(rho_bgk - rho_kbc, ([0-9e.\-]+)\)", kb),
    }
    it = open(os.path.join(test_dir, "integrationtest", "IntegrationTestCases.cpp")).read()
    tg = it[it.index("TestResult ConvergenceTestSemiLagrangianPeriodic() {"):]
    tg = tg[: tg.index("} /* ConvergenceTestSemiLagrangianPeriodic */")]
    out["tgv2d_sl"] = {
        "cite": "test/integrationtest/IntegrationTestCases.cpp:885-961",
        "viscosity": grab(r"const double viscosity = ([0-9.]+);", tg),
        "Ma": grab(r"const double Ma = ([0-9.]+);", tg),
        "order": grab(r"orderOfFiniteElement = ([0-9.]+);", tg, lambda x: int(float(x))),
        "refinement": grab(r"refinementLevel = ([0-9.]+);", tg, lambda x: int(float(x))),
        "cfl": grab(r"const double CFL = ([0-9.]+);", tg),
        "ekin_ratio_expected": "exp(-2)",
        "ekin_tol": grab(r"result.threshold.push_back\(([0-9e.\-]+)\);", tg),
        "l2_velocity_tol": float(re.findall(r"result.threshold.push_back\(([0-9e.\-]+)\);", tg)[1]),
    }
    return out


def periodic_field(mesh, st, seed: int, amp: float = 0.05):
    """Seeded smooth periodic state (equilibrium + small non-equilibrium
    noise), equal on periodic duplicate nodes."""
    import oracle as O
    rng = np.random.default_rng(seed)
    X = mesh.coords()
    D = mesh.dim
    k = [2 * math.pi / mesh.L[a] for a in range(D)]
    ph = rng.uniform(0, 2 * math.pi, size=(D + 1, D))
    def wave(c):
        s = 0.0
        for a in range(D):
            s = s + np.sin(k[a] * X[:, a] + ph[c, a])
        return s / D
    rho = 1.0 + 0.01 * wave(0)
    u = np.stack([amp * st.scaling * wave(c + 1) for c in range(D)])
    f = O.equilibrium(st, rho, np.ascontiguousarray(u))
    # non-equilibrium noise that is a periodic function of position
    noise = np.zeros_like(f)
    for q in range(st.Q):
        ph2 = rng.uniform(0, 2 * math.pi, size=D)
        s = 0.0
        for a in range(D):
            s = s + np.cos(k[a] * X[:, a] + ph2[a])
        noise[q] = 1e-3 * st.w[q] * s
    return np.ascontiguousarray(f + noise)


def oracle_fixtures():
    import oracle as O
    cases = {
        "d2q9_bgk_feq_p4": dict(stencil="D2Q9", dim=2, N=(4, 4), p=4, dg=False, model="BGK_STANDARD"),
        "d3q19_bgk_feq_p2": dict(stencil="D3Q19", dim=3, N=(3, 3, 3), p=2, dg=False, model="BGK_STANDARD"),
        "d2q9_kbc_dg_p3": dict(stencil="D2Q9", dim=2, N=(4, 4), p=3, dg=True, model="KBC_STANDARD"),
    }
    for name, c in cases.items():
        Ma = 0.1
        st = O.stencil(c["stencil"], math.sqrt(3) / Ma)
        L = tuple([2 * math.pi] * 3)
        mesh = O.Mesh(c["dim"], c["N"], c["p"], c["dg"], L)
        dt = O.time_step(mesh.h_min(), c["p"], st.max_speed, 0.4)
        nu = 1e-2
        tau = nu / (dt * st.cs2) + 0.5
        f0 = periodic_field(mesh, st, seed=0)
        S = O.SLOperator(mesh, st, dt)
        f1 = S.stream(f0)
        rho = np.zeros(mesh.n_nodes)
        u = np.zeros((c["dim"], mesh.n_nodes))
        O.collide(st, c["model"], tau, f1, rho, u)
        np.savez_compressed(os.path.join(HERE, f"oracle_{name}.npz"), f0=f0, f1=f1, rho=rho, u=u,
                            dt=dt, tau=tau, nu=nu, Ma=Ma, p=c["p"], N=np.array(c["N"]),
                            dg=c["dg"], stencil=c["stencil"], model=c["model"])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("NATRIUM_REFERENCE"),
                    help="root of the NATriuM source tree (default: $NATRIUM_REFERENCE)")
    a = ap.parse_args()
    if a.reference and os.path.isdir(a.reference):
        ka = known_answers(a.reference)
        with open(os.path.join(HERE, "known_answers.json"), "w") as fh:
            json.dump(ka, fh, indent=1)
        print("wrote known_answers.json")
    else:
        print("reference tree not found; kept known_answers.json")
    oracle_fixtures()
    print("wrote oracle fixtures")


if __name__ == "__main__":
    main()
