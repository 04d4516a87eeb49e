"""Extract the golden analytic AATs of apyib/tests/test_018_RHF_Analytic_AAT.py,
test_019_MP2_Analytic_AAT.py, test_020_CID_Analytic_AAT.py and
test_021_CISD_Analytic_AAT.py (read as text with the Python AST) with their
parameters, the method called and the normalisation, and the geometries they
name from apyib/data/molecules.py, into tests/golden/analytic_aat_goldens.json.

    APYIB_REF=/path/to/apyib-checkout python tests/golden/make_golden_analytic_aat.py
"""
import ast
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
REF_ROOT = os.environ.get("APYIB_REF")
if not REF_ROOT:
    raise SystemExit("set APYIB_REF to an apyib source checkout (the directory holding apyib/)")
FILES = ["apyib/tests/test_018_RHF_Analytic_AAT.py", "apyib/tests/test_019_MP2_Analytic_AAT.py",
         "apyib/tests/test_020_CID_Analytic_AAT.py", "apyib/tests/test_021_CISD_Analytic_AAT.py"]


def molecules():
    tree = ast.parse(open(os.path.join(REF_ROOT, "apyib/data/molecules.py")).read())
    strings, moldict = {}, {}
    for node in tree.body:
        if isinstance(node, ast.Assign) and isinstance(node.value, ast.Constant) and isinstance(node.value.value, str):
            strings[node.targets[0].id] = node.value.value
        elif isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Subscript):
            moldict[node.targets[0].slice.value] = strings[node.value.id]
    return moldict


def main():
    mols = molecules()
    cases, used = [], {}
    for rel in FILES:
        tree = ast.parse(open(os.path.join(REF_ROOT, rel)).read())
        for fn in tree.body:
            if not isinstance(fn, ast.FunctionDef) or not fn.name.startswith("test_"):
                continue
            c = {"name": fn.name, "file": rel, "line": fn.lineno,
                 "skip": any("skip" in ast.unparse(d) for d in fn.decorator_list)}
            local = {n.targets[0].id: n.value.value for n in ast.walk(fn)
                     if isinstance(n, ast.Assign) and isinstance(n.targets[0], ast.Name)
                     and isinstance(n.value, ast.Constant) and isinstance(n.value.value, str)}

            def value(v):
                if isinstance(v, ast.Subscript):
                    return {"moldict": v.slice.value}
                if isinstance(v, ast.Name):
                    return {"local": v.id, "text": local[v.id]}
                return ast.literal_eval(v)
            for node in ast.walk(fn):
                if isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Name):
                    if node.targets[0].id == "parameters":
                        c["parameters"] = {ast.literal_eval(k): value(v) for k, v in zip(node.value.keys, node.value.values)}
                    elif node.targets[0].id == "aat_ref":
                        c["ref"] = ast.literal_eval(node.value.args[0])
                if isinstance(node, ast.Call) and getattr(node.func, "attr", "").endswith("_AATs"):
                    c["call"] = node.func.attr
                    c["kwargs"] = {k.arg: ast.literal_eval(k.value) for k in node.keywords}
                if isinstance(node, ast.Assert):
                    c["tol"] = ast.literal_eval(node.test.comparators[0])
            g = c["parameters"]["geom"]
            if "moldict" in g:
                used[g["moldict"]] = mols[g["moldict"]]
            cases.append(c)
    with open(os.path.join(HERE, "analytic_aat_goldens.json"), "w") as f:
        json.dump({"molecules": used, "cases": cases}, f, indent=1)
    for c in cases:
        print(c["name"], c["parameters"]["basis"], c["parameters"]["method"], c["parameters"]["freeze_core"],
              c.get("call"), c.get("kwargs"), c.get("tol"), len(c.get("ref", [])))


if __name__ == "__main__":
    main()
