"""Generate tests/golden/gauss_legendre_ref.json from the reference's own basis generator.

The reference computes its Gauss-Legendre tables at build time with
script/auto_generate.py + script/Basis.py (sympy, 50 digits) and writes them into a
generated C++ file. This script runs that generator unmodified from a temporary copy
(matplotlib is only imported, never used, so a stub module stands in for it), parses
the emitted ``Gauss_legendre.cpp`` and stores every table as JSON, in the reference's
storage order (column-major for square matrices, ``[side][node]`` for ``boundary``).

It needs the reference checkout and sympy. Give the checkout's root as the argument or in
HEXED_REFERENCE_ROOT:
    python tests/golden/make_basis_golden.py /path/to/hexed
"""
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "gauss_legendre_ref.json")
MAX_ROW_SIZE = 8


def main(ref_root=None):
    ref_root = ref_root or os.environ.get("HEXED_REFERENCE_ROOT")
    if not ref_root:
        sys.exit("usage: make_basis_golden.py /path/to/hexed (or set HEXED_REFERENCE_ROOT)")
    with tempfile.TemporaryDirectory() as tmp:
        script = os.path.join(tmp, "script")
        shutil.copytree(os.path.join(ref_root, "script"), script)
        stub = os.path.join(tmp, "stub", "matplotlib")
        os.makedirs(stub)
        with open(os.path.join(stub, "__init__.py"), "w") as fh:
            fh.write("def __getattr__(name):\n    return None\n")
        open(os.path.join(stub, "pyplot.py"), "w").close()
        out_dir = os.path.join(tmp, "out")
        os.makedirs(out_dir)
        env = dict(os.environ, PYTHONPATH=os.path.join(tmp, "stub") + os.pathsep + script)
        subprocess.run([sys.executable, "auto_generate.py", out_dir + "/", str(MAX_ROW_SIZE)],
                       cwd=script, env=env, check=True)
        with open(os.path.join(out_dir, "Gauss_legendre.cpp")) as fh:
            text = fh.read()
    tables = {}
    for m in re.finditer(r"const double (\w+?)(\d+) \[[^\]]*\] \{([^}]*)\}", text):
        name, rs, body = m.group(1), int(m.group(2)), m.group(3)
        vals = [float(v) for v in body.replace("\n", " ").split(",") if v.strip()]
        tables.setdefault(str(rs), {})[name] = vals
    with open(OUT, "w") as fh:
        json.dump(tables, fh, indent=1)
    print("wrote", OUT, "row sizes", sorted(int(k) for k in tables))


if __name__ == "__main__":
    main(*sys.argv[1:])
