"""Build the golden fixtures in this folder from tincr's own test data.

    python tests/golden/make_golden.py /path/to/tincr

Two sources, both read as data (nothing from tincr is executed):

1. `tests/data/<mol>/*.dat` + `<mol>.xyz` for h2o, ammonia, benzene, uracil, h2 — the fixtures that
   tincr's unit tests load through `src/utils/tests.rs:76-126` (SCC-level S, H0, gamma matrices and
   their gradients, converged orbitals, densities, charges).  Written as `<mol>.npz`, one key per
   `.dat` file plus `symbols` and `xyz_angstrom`.  3-D arrays keep tincr's flattened
   [rows, n*n] layout and are reshaped by the tests exactly like `load_3d` (`utils/tests.rs:60-74`).
2. Known-answer tests in `not_refactored_tests/` whose expected values are literal arrays:
   `solver.rs` `excited_energies_tda_routine` (water TDA from explicit S, orbe, C), `tda_routine`
   (2x2 active space TDA from explicit gamma, gamma_lr, q), `test_apbv_fortran` (A+B products);
   `param/h0_and_s.rs` `test_h0_and_s` / `test_grad_H0_andS` (water S, H0, dS/dR, dH0/dR).
   Each literal `let NAME: ArrayN<f64> = array![...]` in the test body becomes one key of
   `kat_<test>.npz`.
"""

import ast
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
MOLS = ["h2o", "ammonia", "benzene", "uracil", "h2"]


def convert_data(src):
    for mol in MOLS:
        d = os.path.join(src, "tests", "data", mol)
        out = {}
        for fn in sorted(os.listdir(d)):
            if fn.endswith(".dat"):
                rows = [ln.split() for ln in open(os.path.join(d, fn)) if ln.strip() and not ln.startswith("%")]
                a = np.array([[float(v) for v in r] for r in rows])
                out[fn[:-4]] = a
        lines = open(os.path.join(d, mol + ".xyz")).read().split("\n")
        n = int(lines[0])
        sym, xyz = [], []
        for ln in lines[2:2 + n]:
            p = ln.split()
            sym.append(p[0])
            xyz.append([float(v) for v in p[1:4]])
        out["symbols"] = np.array(sym)
        out["xyz_angstrom"] = np.array(xyz)
        np.savez_compressed(os.path.join(HERE, mol + ".npz"), **out)


def _test_body(text, name):
    m = re.search(r"fn\s+" + name + r"\s*\(\s*\)\s*\{", text)
    if not m:
        raise KeyError(name)
    i = m.end()
    depth = 1
    while depth:
        c = text[i]
        if c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
        i += 1
    return text[m.end():i - 1]


def _literal_arrays(body):
    out = {}
    for m in re.finditer(r"let\s+(?:mut\s+)?(\w+)\s*:\s*Array\d<f64>\s*=\s*array!\s*\[", body):
        name = m.group(1)
        i = m.end()
        depth = 1
        while depth:
            c = body[i]
            if c == "[":
                depth += 1
            elif c == "]":
                depth -= 1
            i += 1
        lit = "[" + body[m.end():i - 1] + "]"
        out[name] = np.array(ast.literal_eval(lit), dtype=np.float64)
    return out


def convert_kats(src):
    jobs = [
        ("solver.rs", "excited_energies_tda_routine"),
        ("solver.rs", "tda_routine"),
        ("solver.rs", "test_apbv_fortran"),
        ("solver.rs", "test_apbv_fortran_no_lc"),
        (os.path.join("param", "h0_and_s.rs"), "test_h0_and_s"),
        (os.path.join("param", "h0_and_s.rs"), "test_grad_H0_andS"),
    ]
    for fn, test in jobs:
        text = open(os.path.join(src, "not_refactored_tests", fn)).read()
        arrs = _literal_arrays(_test_body(text, test))
        np.savez_compressed(os.path.join(HERE, "kat_%s.npz" % test), **arrs)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_golden.py <path of the tincr source tree>")
    src = sys.argv[1]
    convert_data(src)
    convert_kats(src)
    print("golden fixtures written to", HERE)
