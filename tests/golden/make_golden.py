"""Generate the golden fixtures in this directory from the reference's tests.

Run with the environment variable SPECTRE_ROOT set to a checkout of the
SpECTRE source tree (release 2024.09.29); the script stops with a message if
it is unset.  The generated JSON files are committed; nothing at test time
reads the reference tree.

Fixtures:
  lgl_golden.json      LGL points/weights, D-matrices and Vandermonde matrices
                       read as text from
                       tests/Unit/NumericalAlgorithms/Spectral/Test_LegendreGaussLobatto.cpp
  gauss_golden.json    Legendre-Gauss points/weights, D-matrices and
                       Vandermonde matrices read as text from
                       tests/Unit/NumericalAlgorithms/Spectral/Test_LegendreGauss.cpp
  curved_golden.json   seeded inputs and outputs of the CurvedScalarWave pypp
                       golden functions: BoundaryCorrections/UpwindPenalty.py
                       and BoundaryConditions/ConstraintPreservingSphericalRadiation.py
                       under tests/Unit/Evolution/Systems/CurvedScalarWave
  adams_golden.json    Adams-Bashforth known answers read as text from
                       tests/Unit/Time/TimeSteppers/Test_AdamsCoefficients.cpp
                       (exact variable_coefficients cases) and
                       tests/Unit/Time/TimeSteppers/Test_AdamsLts.cpp (every
                       explicit "AB ..." lts_coefficients step case; the
                       Adams-Moulton cases and dense output are not taken)
  upwind_golden.json   seeded inputs and the outputs of the reference's pypp
                       golden functions
                       tests/Unit/Evolution/Systems/ScalarWave/BoundaryCorrections/UpwindPenalty.py
                       (dg_package_data, dg_boundary_terms), evaluated point
                       by point as pypp does for DataVector arguments.
"""
import importlib.util
import json
import os
import re
import sys

import numpy as np

ROOT = os.environ.get("SPECTRE_ROOT")
HERE = os.path.dirname(os.path.abspath(__file__))


def _cpp_expr_to_py(s):
    s = re.sub(r"Matrix\(\s*\{", "Matrix({", s)
    s = re.sub(r"\}\s*\)", "})", s)
    s = s.replace("DataVector{", "np.array([").replace("Matrix({", "np.array([")
    # close the constructors: count braces by a tiny state machine
    out, depth_stack = [], []
    i = 0
    while i < len(s):
        c = s[i]
        if s.startswith("np.array([", i):
            out.append("np.array([")
            depth_stack.append("arr")
            i += len("np.array([")
            continue
        if c == "{":
            out.append("[")
            depth_stack.append("br")
        elif c == "}":
            kind = depth_stack.pop()
            out.append("])" if kind == "arr" else "]")
            if kind == "arr" and i + 1 < len(s) and s[i + 1] == ")":
                i += 1  # Matrix({ ... }) closing paren
        else:
            out.append(c)
        i += 1
    return "".join(out)


def _split_args(text):
    depth, cur, args = 0, [], []
    for c in text:
        if c in "({[":
            depth += 1
        elif c in ")}]":
            depth -= 1
        if c == "," and depth == 0:
            args.append("".join(cur))
            cur = []
        else:
            cur.append(c)
    args.append("".join(cur))
    return [a.strip() for a in args]


def _calls(src, fname):
    out = []
    for m in re.finditer(re.escape(fname) + r"\(", src):
        if src[m.start() - 5 : m.start()].strip().endswith("void"):
            continue
        i, depth = m.end(), 1
        while depth:
            depth += {"(": 1, ")": -1}.get(src[i], 0)
            i += 1
        out.append(_split_args(src[m.end() : i - 1]))
    return out


def lgl_golden():
    return spectral_golden("tests/Unit/NumericalAlgorithms/Spectral/Test_LegendreGaussLobatto.cpp")


def spectral_golden(rel):
    path = os.path.join(ROOT, rel)
    src = open(path).read()
    src = re.sub(r"//[^\n]*", "", src)
    res = {"source": rel,
           "points_weights": {}, "diff_matrix": {}, "modal_to_nodal": {},
           "nodal_to_modal": {}}
    for args in _calls(src, "test_points_and_weights"):
        if len(args) != 3 or not args[0].isdigit() or int(args[0]) < 2:
            continue
        n = int(args[0])
        x = eval(_cpp_expr_to_py(args[1]), {"np": np})
        w = eval(_cpp_expr_to_py(args[2]), {"np": np})
        res["points_weights"][n] = {"x": list(map(float, np.ravel(x))),
                                   "w": list(map(float, np.ravel(w)))}
    for key, fname in (("diff_matrix", "test_diff_matrix"),
                       ("modal_to_nodal", "test_modal_to_nodal_matrix"),
                       ("nodal_to_modal", "test_nodal_to_modal_matrix")):
        for args in _calls(src, fname):
            if len(args) != 2 or not args[0].isdigit() or int(args[0]) < 2:
                continue
            n = int(args[0])
            M = eval(_cpp_expr_to_py(args[1]), {"np": np})
            res[key][n] = np.asarray(M, dtype=float).tolist()
    return res


def upwind_golden(seed=20241204, npts=40):
    path = os.path.join(
        ROOT, "tests/Unit/Evolution/Systems/ScalarWave/BoundaryCorrections/UpwindPenalty.py")
    spec = importlib.util.spec_from_file_location("ref_upwind", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    rng = np.random.default_rng(seed)
    cases = []
    for side in range(2):
        psi = rng.uniform(-1, 1, npts)
        pi = rng.uniform(-1, 1, npts)
        phi = rng.uniform(-1, 1, (3, npts))
        g2 = rng.uniform(0, 2, npts)
        nrm = rng.normal(size=(3, npts))
        nrm /= np.linalg.norm(nrm, axis=0)
        cases.append((psi, pi, phi, g2, nrm))
    pkgs = []
    for (psi, pi, phi, g2, nrm) in cases:
        pk = np.zeros((16, npts))
        for p in range(npts):
            r = mod.dg_package_data(psi[p], pi[p], phi[:, p], g2[p], nrm[:, p], None, None)
            flat = [np.atleast_1d(np.asarray(f, dtype=float)) for f in r]
            pk[:, p] = np.concatenate(flat)
        pkgs.append(pk)
    bt = np.zeros((5, npts))
    for p in range(npts):
        def fields(pk):
            return (pk[0, p], pk[1:4, p], pk[4, p], pk[5, p], pk[6:9, p], pk[9:12, p],
                    pk[12, p], pk[13:16, p])
        r = mod.dg_boundary_terms(*fields(pkgs[0]), *fields(pkgs[1]), True)
        bt[:, p] = np.concatenate([np.atleast_1d(np.asarray(f, dtype=float)) for f in r])
    # exterior package with non-default char speeds so every Theta branch is hit
    sp = np.array([[0.0, 1.0, -1.0], [-0.3, 0.7, -1.3], [0.4, 1.4, -0.6]])
    pk_int2 = pkgs[0].copy()
    pk_ext2 = pkgs[1].copy()
    for p in range(npts):
        pk_int2[13:16, p] = sp[p % 3]
        pk_ext2[13:16, p] = sp[(p + 1) % 3]
    bt2 = np.zeros((5, npts))
    for p in range(npts):
        def fields2(pk):
            return (pk[0, p], pk[1:4, p], pk[4, p], pk[5, p], pk[6:9, p], pk[9:12, p],
                    pk[12, p], pk[13:16, p])
        r = mod.dg_boundary_terms(*fields2(pk_int2), *fields2(pk_ext2), True)
        bt2[:, p] = np.concatenate([np.atleast_1d(np.asarray(f, dtype=float)) for f in r])
    return {
        "source": "tests/Unit/Evolution/Systems/ScalarWave/BoundaryCorrections/UpwindPenalty.py",
        "seed": seed,
        "npts": npts,
        "inputs": [{"psi": c[0].tolist(), "pi": c[1].tolist(), "phi": c[2].tolist(),
                    "gamma2": c[3].tolist(), "normal": c[4].tolist()} for c in cases],
        "packaged": [p.tolist() for p in pkgs],
        "boundary_terms": bt.tolist(),
        "speeds_case": {"pkg_int": pk_int2.tolist(), "pkg_ext": pk_ext2.tolist(),
                        "boundary_terms": bt2.tolist()},
    }


def curved_golden(seed=20241205, npts=30):
    unit = os.path.join(ROOT, "tests/Unit")
    if unit not in sys.path:
        sys.path.insert(0, unit)
    base = os.path.join(ROOT, "tests/Unit/Evolution/Systems/CurvedScalarWave")

    def load(rel, name):
        spec = importlib.util.spec_from_file_location(name, os.path.join(base, rel))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        return mod

    up = load("BoundaryCorrections/UpwindPenalty.py", "ref_csw_upwind")
    cp = load("BoundaryConditions/ConstraintPreservingSphericalRadiation.py", "ref_csw_cpsr")
    rng = np.random.default_rng(seed)

    def side():
        d = {
            "psi": rng.uniform(-1, 1, npts), "pi": rng.uniform(-1, 1, npts),
            "phi": rng.uniform(-1, 1, (3, npts)), "lapse": rng.uniform(0.3, 1.0, npts),
            "shift": rng.uniform(-0.6, 0.6, (3, npts)), "gamma1": rng.uniform(-1, 1, npts),
            "gamma2": rng.uniform(0, 2, npts),
        }
        nrm = rng.normal(size=(3, npts))
        nrm /= np.linalg.norm(nrm, axis=0)
        # a normal vector raised with a random symmetric positive matrix
        nvec = np.zeros((3, npts))
        for p in range(npts):
            A = rng.normal(size=(3, 3)) * 0.2
            g = np.eye(3) + A @ A.T
            v = g @ nrm[:, p]
            nvec[:, p] = v / np.sqrt(v @ nrm[:, p])
        d["normal"] = nrm
        d["normal_vector"] = nvec
        return d

    sides = [side(), side()]
    pk = []
    for d in sides:
        out = np.zeros((14, npts))
        for p in range(npts):
            r = up.dg_package_data(d["psi"][p], d["pi"][p], d["phi"][:, p], d["lapse"][p],
                                   d["shift"][:, p], d["gamma1"][p], d["gamma2"][p],
                                   d["normal"][:, p], d["normal_vector"][:, p], None, None)
            out[:, p] = np.concatenate([np.atleast_1d(np.asarray(f, dtype=float)) for f in r])
        pk.append(out)
    bt = np.zeros((5, npts))
    for p in range(npts):
        def f(pkx):
            return (pkx[0, p], pkx[1:4, p].copy(), pkx[4, p], pkx[5, p], pkx[6, p], pkx[7:10, p],
                    pkx[10:14, p])
        r = up.dg_boundary_terms(*f(pk[0]), *f(pk[1]), True)
        bt[:, p] = np.concatenate([np.atleast_1d(np.asarray(x, dtype=float)) for x in r])
    # CPSR dt corrections on side 0 with extra volume data
    d = sides[0]
    xyz = rng.uniform(5, 20, (3, npts)) * rng.choice([-1, 1], (3, npts))
    dpsi = rng.uniform(-1, 1, (3, npts))
    dpi = rng.uniform(-1, 1, (3, npts))
    dphi = rng.uniform(-1, 1, (3, 3, npts))
    dtpsi = rng.uniform(-1, 1, npts)
    dtpi = rng.uniform(-1, 1, npts)
    dtphi = rng.uniform(-1, 1, (3, npts))
    cps = np.zeros((5, npts))
    for p in range(npts):
        args = (None, d["normal"][:, p], d["normal_vector"][:, p], d["psi"][p], d["phi"][:, p],
                xyz[:, p], d["gamma1"][p], d["gamma2"][p], d["lapse"][p], d["shift"][:, p],
                dtpsi[p], dtpi[p], dtphi[:, p], dpsi[:, p], dpi[:, p], dphi[:, :, p])
        cps[0, p] = cp.dt_psi_constraint_preserving_spherical_radiation(*args)
        cps[1, p] = cp.dt_pi_constraint_preserving_spherical_radiation(*args)
        cps[2:5, p] = cp.dt_phi_constraint_preserving_spherical_radiation(*args)
    tolist = lambda a: np.asarray(a).tolist()
    return {
        "source": "tests/Unit/Evolution/Systems/CurvedScalarWave/{BoundaryCorrections/UpwindPenalty.py,"
                  "BoundaryConditions/ConstraintPreservingSphericalRadiation.py}",
        "seed": seed, "npts": npts,
        "sides": [{k: tolist(v) for k, v in d.items()} for d in sides],
        "packaged": [tolist(x) for x in pk], "boundary_terms": tolist(bt),
        "cpsr": {"xyz": tolist(xyz), "d_psi": tolist(dpsi), "d_pi": tolist(dpi),
                 "d_phi": tolist(dphi), "dt_psi": tolist(dtpsi), "dt_pi": tolist(dtpi),
                 "dt_phi": tolist(dtphi), "out": tolist(cps)},
    }


def _rational(text):
    """'{-5, 2}' -> -2.5, '3' -> 3.0"""
    text = text.strip()
    m = re.fullmatch(r"\{\s*(-?\d+)\s*,\s*(-?\d+)\s*\}", text)
    if m:
        return int(m.group(1)) / int(m.group(2))
    return float(int(text))


def _rational_list(text):
    """'{{5, 12}, {-4, 3}, 2}' -> [5/12, -4/3, 2]"""
    body = text.strip()[1:-1]
    items, depth, cur = [], 0, ""
    for c in body:
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
        if c == "," and depth == 0:
            items.append(cur)
            cur = ""
        else:
            cur += c
    if cur.strip():
        items.append(cur)
    return [_rational(i) for i in items]


def _fake_id(text):
    """FakeId text -> [slab, time]; None for a substep id (Adams-Moulton)."""
    parts = [p.strip() for p in _split_args(text.strip()[1:-1])]
    if len(parts) == 1:
        return [0, int(parts[0])]
    if len(parts) == 3 and parts[1] == "{}":
        return [int(parts[2]), int(parts[0])]
    return None


def _brace_items(body):
    items, depth, start = [], 0, None
    for i, c in enumerate(body):
        if c == "{":
            if depth == 0:
                start = i
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                items.append(body[start:i + 1])
    return items


def adams_golden():
    out = {"source": ["tests/Unit/Time/TimeSteppers/Test_AdamsCoefficients.cpp",
                      "tests/Unit/Time/TimeSteppers/Test_AdamsLts.cpp"],
           "variable": [], "lts": []}
    src = open(os.path.join(ROOT, out["source"][0])).read()
    for m in re.finditer(r"ac::variable_coefficients<Rational>\((.*?)\)\s*==\s*"
                         r"ac::OrderVector<Rational>(\{.*?\})\);", src, re.S):
        args = _split_args(m.group(1))
        out["variable"].append({"control_times": _rational_list(args[0]),
                                "step_start": _rational(args[1]),
                                "step_end": _rational(args[2]),
                                "expected": _rational_list(m.group(2))})
    src = open(os.path.join(ROOT, out["source"][1])).read()
    body = src[src.index("void test_lts_coefficients()"):]
    body = body[:body.index("SPECTRE_TEST_CASE")]
    arrays = {}
    for m in re.finditer(r"const std::array (\w+)\{(.*?)\};", body, re.S):
        arrays[m.group(1)] = [eval(v) for v in _split_args(m.group(2))]
    infos = [(m.start(), m.group(1)) for m in re.finditer(r'INFO\("([^"]+)"\)', body)]
    for i, (pos, name) in enumerate(infos):
        if not name.startswith("AB "):
            continue
        block = body[pos:infos[i + 1][0] if i + 1 < len(infos) else len(body)]
        orders = {m.group(1): int(m.group(3)) for m in re.finditer(
            r"adams_lts::AdamsScheme (\w+)\{adams_lts::SchemeType::(\w+), (\d+)\}", block)
            if m.group(2) == "Explicit"}
        steps = {}
        for m in re.finditer(r"const std::vector<FakeId> (\w+)\{(.*?)\};", block, re.S):
            steps[m.group(1)] = [_fake_id(t) for t in _brace_items(m.group(2))]
        expected = {}
        for m in re.finditer(r"const ExpectedCoefficients (\w+)\{(.*?)\};", block, re.S):
            entries = []
            for item in _brace_items(m.group(2)):
                inner = item[1:-1]
                ids_text = _brace_items(inner)[0]
                value = inner[len(ids_text):].strip().lstrip(",").strip()
                value = re.sub(r"(\w+)\[(\d+)\]", lambda a: repr(arrays[a.group(1)][int(a.group(2))]),
                               value)
                pair = [_fake_id(t) for t in _brace_items(ids_text[1:-1])]
                entries.append({"local": pair[0], "remote": pair[1], "coef": eval(value)})
            expected[m.group(1)] = entries
        for m in re.finditer(r"step_coefficients\(\s*(\w+),\s*(\w+),\s*(\w+),\s*(\w+),"
                             r"\s*(\w+),\s*(-?\d+),\s*(-?\d+)(?:,\s*false)?\),\s*(\w+)\);",
                             block):
            loc, rem, sl, sr, ss, t0, t1, exp = m.groups()
            out["lts"].append({
                "case": name, "local": steps[loc], "remote": steps[rem],
                "orders": [orders[sl], orders[sr], orders[ss]],
                "step_start": int(t0), "step_end": int(t1), "expected": expected[exp]})
    return out


def main():
    if not ROOT or not os.path.isdir(ROOT):
        sys.stderr.write("set SPECTRE_ROOT to a checkout of the SpECTRE source tree "
                         "(release 2024.09.29)\n")
        return 2
    with open(os.path.join(HERE, "adams_golden.json"), "w") as f:
        json.dump(adams_golden(), f, indent=1)
    with open(os.path.join(HERE, "lgl_golden.json"), "w") as f:
        json.dump(lgl_golden(), f, indent=1)
    with open(os.path.join(HERE, "upwind_golden.json"), "w") as f:
        json.dump(upwind_golden(), f)
    with open(os.path.join(HERE, "curved_golden.json"), "w") as f:
        json.dump(curved_golden(), f)
    with open(os.path.join(HERE, "gauss_golden.json"), "w") as f:
        json.dump(spectral_golden(
            "tests/Unit/NumericalAlgorithms/Spectral/Test_LegendreGauss.cpp"), f, indent=1)
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    sys.exit(main())
