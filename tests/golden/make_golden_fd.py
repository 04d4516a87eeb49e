"""Extract the reference's finite-difference (and length-gauge analytic APT) golden values
into tests/golden/fd_goldens.json.

apyib/tests/test_009_Hessian.py and apyib/tests/test_010_APT.py each set up a
``parameters`` dict, compare ``finite_difference.compute_Hessian(h)`` /
``compute_APT(h, f)`` with a ``hess_ref`` / ``apt_ref`` array and assert a
tolerance.  This script reads those files as text (Python AST, nothing is
executed), takes the geometries they name from apyib/data/molecules.py, and
writes per test: the parameters, the step sizes, the reference array, the
tolerance and whether the reference skips the test.

Run where the reference sources are available:
    APYIB_REF=/path/to/apyib-checkout python tests/golden/make_golden_fd.py
"""
import ast
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("APYIB_REF")
if not REF_ROOT:
    raise SystemExit("set APYIB_REF to an apyib source checkout (the directory holding apyib/)")
FILES = {"hessian": "apyib/tests/test_009_Hessian.py", "apt": "apyib/tests/test_010_APT.py"}


def molecules():
    src = open(os.path.join(REF_ROOT, "apyib/data/molecules.py")).read()
    tree = ast.parse(src)
    strings, moldict = {}, {}
    for node in tree.body:
        if isinstance(node, ast.Assign) and isinstance(node.value, ast.Constant) and isinstance(node.value.value, str):
            strings[node.targets[0].id] = node.value.value
        elif (isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Subscript)
              and isinstance(node.value, ast.Name)):
            moldict[node.targets[0].slice.value] = strings[node.value.id]
    return moldict


def _param_value(node):
    if isinstance(node, ast.Subscript) and getattr(node.value, "id", None) == "moldict":
        return {"moldict": node.slice.value}
    return ast.literal_eval(node)


def cases(kind, rel):
    src = open(os.path.join(REF_ROOT, rel)).read()
    tree = ast.parse(src)
    out = []
    for fn in tree.body:
        if not isinstance(fn, ast.FunctionDef) or not fn.name.startswith("test_"):
            continue
        skip = any("skip" in ast.unparse(d) for d in fn.decorator_list)
        case = {"name": fn.name, "file": rel, "line": fn.lineno, "skip": skip}
        for node in ast.walk(fn):
            if isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Name):
                tgt = node.targets[0].id
                if tgt == "parameters":
                    case["parameters"] = {ast.literal_eval(k): _param_value(v)
                                          for k, v in zip(node.value.keys, node.value.values)}
                elif tgt in ("hess_ref", "apt_ref"):
                    case["ref"] = ast.literal_eval(node.value.args[0])
                    case["ref_line"] = node.lineno
                elif tgt in ("hessian", "apt") and isinstance(node.value, ast.Call):
                    case["steps"] = [ast.literal_eval(a) for a in node.value.args]
            if isinstance(node, ast.Assert):
                # assert(np.max(np.abs(x - ref[.reshape(...)])) < tol)
                case["tol"] = ast.literal_eval(node.test.comparators[0])
        out.append(case)
    return out


def analytic_apt_cases():
    """The length- and velocity-gauge analytic APT goldens of
    apyib/tests/test_022_RHF_Analytic_APT.py (geometry given inside each test)."""
    rel = "apyib/tests/test_022_RHF_Analytic_APT.py"
    tree = ast.parse(open(os.path.join(REF_ROOT, rel)).read())
    out = []
    for fn in tree.body:
        if not isinstance(fn, ast.FunctionDef) or not (fn.name.endswith("_LG") or fn.name.endswith("_VG")):
            continue
        local = {n.targets[0].id: n.value.value for n in ast.walk(fn) if isinstance(n, ast.Assign)
                 and isinstance(n.targets[0], ast.Name) and isinstance(n.value, ast.Constant)
                 and isinstance(n.value.value, str)}
        c = {"name": fn.name, "file": rel, "line": fn.lineno}
        for node in ast.walk(fn):
            if isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Name):
                if node.targets[0].id == "parameters":
                    c["parameters"] = {ast.literal_eval(k): (local[v.id] if isinstance(v, ast.Name)
                                                             else ast.literal_eval(v))
                                       for k, v in zip(node.value.keys, node.value.values)}
                elif node.targets[0].id == "apt_ref":
                    c["ref"] = ast.literal_eval(node.value.args[0])
            if isinstance(node, ast.Assert):
                c["tol"] = ast.literal_eval(node.test.comparators[0])
        out.append(c)
    return out


def main():
    mols = molecules()
    data = {"molecules": {}, "hessian": [], "apt": []}
    for kind, rel in FILES.items():
        for c in cases(kind, rel):
            key = c["parameters"]["geom"]["moldict"]
            data["molecules"][key] = mols[key]
            data[kind].append(c)
    data["apt_analytic"] = analytic_apt_cases()
    path = os.path.join(HERE, "fd_goldens.json")
    with open(path, "w") as f:
        json.dump(data, f, indent=1)
    print("wrote", path, {k: len(v) for k, v in data.items()})


if __name__ == "__main__":
    main()
