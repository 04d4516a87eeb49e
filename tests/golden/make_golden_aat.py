"""AAT fixtures from the reference's own code.

1. tests/golden/aat_small.npz: the reference's determinant-sum AAT terms
   (apyib/aats.py:120-555 spin-orbital, :558-1067 spatial) evaluated on small
   seeded inputs: spin-blocked overlap matrices near the identity (the shape
   compute_so_overlap gives, apyib/utils.py:393-423) and random amplitudes, for
   a few (nuclear, field) component pairs, CISD (all nine terms) in full and
   intermediate normalisation.  The reference's ``AAT`` object is made with
   ``object.__new__`` and given the attributes its term methods read (overlaps,
   amplitudes, sizes, strengths), so no psi4 call is made.
2. tests/golden/aat_goldens.json: the golden AAT arrays of
   apyib/tests/test_011_AAT.py, test_012_AAT_SO.py and test_013_AAT_parallel.py (read as text with the
   Python AST), with the geometry, basis, method, normalisation and steps of
   each test.

Run where the reference sources are available:
    APYIB_REF=/path/to/apyib-checkout python tests/golden/make_golden_aat.py
"""
import ast
import importlib.util
import json
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("APYIB_REF")
if not REF_ROOT:
    raise SystemExit("set APYIB_REF to an apyib source checkout (the directory holding apyib/)")
NBF, NDOCC, NATOM = 4, 2, 1         # spatial sizes: SO o = 4, v = 4
PAIRS = [(0, 0), (1, 2), (2, 1)]
TERMS = ["I_00", "I_0D", "I_D0", "I_DD", "I_0S", "I_S0", "I_SS", "I_SD", "I_DS"]


def load_reference_aats():
    sys.path.insert(0, HERE)
    from ref_loader import _stub_psi4, load_reference
    _stub_psi4()
    load_reference()
    sys.modules["psi4"].core = types.SimpleNamespace()
    spec = importlib.util.spec_from_file_location("apyib.aats", os.path.join(REF_ROOT, "apyib", "aats.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["apyib.aats"] = mod
    spec.loader.exec_module(mod)
    return mod


def so_overlap(M):
    n = M.shape[0]
    S = np.zeros((2 * n, 2 * n), dtype=complex)
    S[0::2, 0::2] = M
    S[1::2, 1::2] = M
    return S


def seeded_inputs(seed, spatial):
    rng = np.random.default_rng(seed)
    n = NBF

    def mo():
        return np.eye(n) + 0.08 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    o, v = (NDOCC, NBF - NDOCC) if spatial else (2 * NDOCC, 2 * (NBF - NDOCC))

    def amps():
        t1 = 0.05 * (rng.standard_normal((o, v)) + 1j * rng.standard_normal((o, v)))
        t2 = 0.05 * (rng.standard_normal((o, o, v, v)) + 1j * rng.standard_normal((o, o, v, v)))
        if spatial:
            t2 = 0.5 * (t2 + t2.transpose(1, 0, 3, 2))                     # t_ijab = t_jiba
        else:
            t2 = t2 - t2.transpose(1, 0, 2, 3) - t2.transpose(0, 1, 3, 2) + t2.transpose(1, 0, 3, 2)
        return [1.0, t1, t2]
    n3 = 3 * NATOM
    ov = {"uu": mo()}
    for b in range(3):
        ov["up", b], ov["un", b] = mo(), mo()
    for a in range(n3):
        ov["pu", a], ov["nu", a] = mo(), mo()
        for b in range(3):
            for k in ("pp", "pn", "np", "nn"):
                ov[k, a, b] = mo()
    T = {"u": amps(), "np": [amps() for _ in range(n3)], "nn": [amps() for _ in range(n3)],
         "mp": [amps() for _ in range(3)], "mn": [amps() for _ in range(3)]}
    return ov, T


def reference_object(mod, ov, T, method, spatial):
    A = object.__new__(mod.AAT)
    conv = (lambda M: M) if spatial else so_overlap
    A.parameters = {"method": method}
    A.nbf, A.ndocc, A.nfzc = NBF, NDOCC, 0
    A.nuc_pert_strength = A.mag_pert_strength = 1e-4
    A.unperturbed_T, A.nuc_pos_T, A.nuc_neg_T, A.mag_pos_T, A.mag_neg_T = T["u"], T["np"], T["nn"], T["mp"], T["mn"]
    n3 = 3 * NATOM
    A.overlap_uu = conv(ov["uu"])
    A.overlap_up = [conv(ov["up", b]) for b in range(3)]
    A.overlap_un = [conv(ov["un", b]) for b in range(3)]
    A.overlap_pu = [conv(ov["pu", a]) for a in range(n3)]
    A.overlap_nu = [conv(ov["nu", a]) for a in range(n3)]
    for k in ("pp", "pn", "np", "nn"):
        setattr(A, "overlap_" + k, [[conv(ov[k, a, b]) for b in range(3)] for a in range(n3)])
    return A


def small_fixture(mod):
    out = {}
    for tag, spatial, method in (("so", False, "CISD_SO"), ("sp", True, "CISD")):
        ov, T = seeded_inputs(11 if not spatial else 12, spatial)
        for k, M in ov.items():
            out[f"{tag}_ov_" + "_".join(map(str, k if isinstance(k, tuple) else (k,)))] = M
        for key in ("u",):
            out[f"{tag}_T_u_1"], out[f"{tag}_T_u_2"] = T["u"][1], T["u"][2]
        for key in ("np", "nn", "mp", "mn"):
            for i, t in enumerate(T[key]):
                out[f"{tag}_T_{key}{i}_1"], out[f"{tag}_T_{key}{i}_2"] = t[1], t[2]
        for norm in ("full", "intermediate"):
            for (a, b) in PAIRS:
                A = reference_object(mod, ov, T, method, spatial)
                if spatial:
                    out[f"{tag}_{norm}_{a}_{b}_total"] = A.compute_spatial_aats(a, b, norm)
                else:
                    for term in TERMS:
                        out[f"{tag}_{norm}_{a}_{b}_{term}"] = getattr(A, "compute_SO_" + term)(a, b, norm)
                print(tag, norm, a, b, "done", flush=True)
    np.savez_compressed(os.path.join(HERE, "aat_small.npz"), **out)


def golden_arrays():
    out = []
    for rel in ("apyib/tests/test_011_AAT.py", "apyib/tests/test_012_AAT_SO.py", "apyib/tests/test_013_AAT_parallel.py"):
        tree = ast.parse(open(os.path.join(REF_ROOT, rel)).read())
        for fn in tree.body:
            if not isinstance(fn, ast.FunctionDef) or not fn.name.startswith("test_"):
                continue
            case = {"name": fn.name, "file": rel, "line": fn.lineno,
                    "skip": any("skip" in ast.unparse(d) for d in fn.decorator_list), "refs": {}}
            for node in ast.walk(fn):
                if isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Name):
                    tgt = node.targets[0].id
                    if tgt == "parameters":
                        case["parameters"] = {ast.literal_eval(k): (
                            {"moldict": v.slice.value} if isinstance(v, ast.Subscript) else ast.literal_eval(v))
                            for k, v in zip(node.value.keys, node.value.values)}
                    elif tgt.endswith("_ref") and isinstance(node.value, ast.Call) and node.value.args:
                        try:
                            case["refs"][tgt] = ast.literal_eval(node.value.args[0])
                        except ValueError:
                            pass
                if isinstance(node, ast.Call) and getattr(node.func, "attr", "") in ("compute_SO_aats",
                                                                                      "compute_spatial_aats"):
                    case["call"] = node.func.attr
                    case["normalization"] = next((ast.literal_eval(k.value) for k in node.keywords
                                                  if k.arg == "normalization"), "full")
                if isinstance(node, ast.Call) and getattr(node.func, "attr", "") in ("compute_AAT",
                                                                                      "compute_parallel_aats"):
                    case["steps"] = [ast.literal_eval(a) for a in node.args if isinstance(a, ast.Constant)]
                    if node.func.attr == "compute_parallel_aats":
                        case["parallel_normalization"] = next((ast.literal_eval(k.value) for k in node.keywords
                                                               if k.arg == "normalization"), "full")
                if isinstance(node, ast.Assert):
                    case["tol"] = ast.literal_eval(node.test.comparators[0])
            out.append(case)
    src = open(os.path.join(REF_ROOT, "apyib/data/molecules.py")).read()
    tree = ast.parse(src)
    strings, moldict = {}, {}
    for node in tree.body:
        if isinstance(node, ast.Assign) and isinstance(node.value, ast.Constant) and isinstance(node.value.value, str):
            strings[node.targets[0].id] = node.value.value
        elif isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Subscript):
            moldict[node.targets[0].slice.value] = strings[node.value.id]
    mols = {c["parameters"]["geom"]["moldict"]: moldict[c["parameters"]["geom"]["moldict"]] for c in out}
    with open(os.path.join(HERE, "aat_goldens.json"), "w") as f:
        json.dump({"molecules": mols, "cases": out}, f, indent=1)
    for c in out:
        print(c["name"], c["skip"], c["parameters"]["basis"], c["parameters"]["method"], c.get("call"),
              c.get("normalization"), list(c["refs"]))


if __name__ == "__main__":
    golden_arrays()
    small_fixture(load_reference_aats())
