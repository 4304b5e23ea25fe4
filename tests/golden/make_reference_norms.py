"""Extract the reference's own golden `Solution norm` values for the hexahedral
elliptic cases (C0 and IPDG) from its regression driver (test/testElliptic.py, read as text)
and write reference_norms.json beside this script.

Run where the reference tree is available:
    python tests/golden/make_reference_norms.py /path/to/libparanumal
"""
import ast
import json
import os
import sys


def extract(ref_root):
    path = os.path.join(ref_root, "test", "testElliptic.py")
    src = open(path).read()
    tree = ast.parse(src)
    out = {}
    for node in ast.walk(tree):
        if not (isinstance(node, ast.Call) and getattr(node.func, "id", "") == "test"):
            continue
        kw = {k.arg: k.value for k in node.keywords}
        name = ast.literal_eval(kw["name"])
        if not (name.startswith("testEllipticHex_C0") or name.startswith("testEllipticHex_Ipdg")):
            continue
        settings = {k.arg: ast.literal_eval(k.value) for k in kw["settings"].keywords
                    if k.arg != "data_file"}
        out[name] = {"settings": settings, "norm": ast.literal_eval(kw["referenceNorm"]),
                     "source": "test/testElliptic.py:%d" % node.lineno}
    return out


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LIBPARANUMAL_DIR")
    if not ref:
        sys.exit("usage: make_reference_norms.py <libParanumal source tree> (or set LIBPARANUMAL_DIR)")
    data = {"tolerance": 1e-5, "tolerance_source": "test/test.py:63,129-137",
            "defaults_source": "test/testElliptic.py:34-59 (LAMBDA is not written to the .rc, so the "
                               "default 1.0 of solvers/elliptic/src/ellipticSettings.cpp applies)",
            "cases": extract(ref)}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_norms.json")
    json.dump(data, open(dst, "w"), indent=1, sort_keys=True)
    print(dst, len(data["cases"]))
