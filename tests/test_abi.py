"""CPU tests of the C-ABI library: it builds for sm_103a, loads, and exports exactly the entry
points that include/tincr_gb300.h declares.  No compute call is made here."""

import ctypes
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "tincr_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(tincr_\w+)\s*\(", text, re.M)))


@pytest.fixture(scope="module")
def libpath():
    if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
        pytest.skip("nvcc not available")
    from tincr_gb300 import build
    return build.build()


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("tincr_ctx_create", "tincr_ctx_destroy", "tincr_trans_charges", "tincr_tda_setup",
              "tincr_tda_products", "tincr_tda_solve"):
        assert s in syms


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", libpath], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT\s+(tincr_\w+)", out))
    assert set(declared_symbols()) <= exported, set(declared_symbols()) - exported
    lib = ctypes.CDLL(libpath)
    for s in declared_symbols():
        assert getattr(lib, s) is not None


def test_binding_signatures_cover_header(libpath):
    from tincr_gb300 import _lib
    assert set(declared_symbols()) == set(_lib.SIGNATURES)


def test_build_targets_sm103a_only():
    from tincr_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def _declared_arities():
    """Number of parameters of every entry point in the header (comments stripped)."""
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"^\s*(?:const\s+)?\w+\s*\*?\s*(tincr_\w+)\s*\(([^)]*)\)\s*;", text, re.M):
        params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
        out[m.group(1)] = len(params)
    return out


def test_binding_arities_match_header():
    """The ctypes argument lists have as many entries as the C declarations have parameters."""
    from tincr_gb300 import _lib
    ar = _declared_arities()
    assert set(ar) == set(_lib.SIGNATURES)
    for name, (_, args) in _lib.SIGNATURES.items():
        assert len(args) == ar[name], (name, len(args), ar[name])


def test_batch_struct_layouts_match_header(tmp_path):
    """tincr_tda_instance / tincr_tda_result as the C compiler lays them out equal the ctypes (and
    numpy record) layouts the Python mirror passes."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "lay.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "tincr_gb300.h"\n'
                   'int main(void) { printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(tincr_tda_instance), '
                   'offsetof(tincr_tda_instance, orbs_per_atom), offsetof(tincr_tda_instance, xyz), '
                   'sizeof(tincr_tda_result), offsetof(tincr_tda_result, iterations), '
                   'offsetof(tincr_tda_result, status)); return 0; }\n')
    exe = tmp_path / "lay"
    subprocess.run([cc, str(src), "-I", os.path.join(ROOT, "include"), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    from tincr_gb300 import fmo
    I, R = fmo._Instance, fmo._Result
    assert got == [ctypes.sizeof(I), I.orbs_per_atom.offset, I.xyz.offset, ctypes.sizeof(R), R.iterations.offset,
                   R.status.offset]
    assert fmo._INST_DT.itemsize == got[0] and fmo._RES_DT.itemsize == got[3]


def test_exciton_struct_layouts_match_header(tmp_path):
    """tincr_exciton_monomer / _pair / _ct as the C compiler lays them out equal the ctypes structures
    `fmo.exciton_states` passes (every field's offset and the sizes)."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from tincr_gb300 import fmo
    structs = [("tincr_exciton_monomer", fmo._ExMonomer), ("tincr_exciton_pair", fmo._ExPair),
               ("tincr_exciton_ct", fmo._ExCT)]
    body = []
    for cname, cls in structs:
        body.append('printf("%%zu\\n", sizeof(%s));' % cname)
        for f, _ in cls._fields_:
            body.append('printf("%%zu\\n", offsetof(%s, %s));' % (cname, f))
    src = tmp_path / "lay.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "tincr_gb300.h"\nint main(void) { '
                   + " ".join(body) + " return 0; }\n")
    exe = tmp_path / "lay"
    subprocess.run([cc, str(src), "-I", os.path.join(ROOT, "include"), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = []
    for _, cls in structs:
        want.append(ctypes.sizeof(cls))
        want += [getattr(cls, f).offset for f, _ in cls._fields_]
    assert got == want


def test_scc_struct_layouts_match_header(tmp_path):
    """tincr_scc_system as the C compiler lays it out equals the numpy record `scc.scc_batch` packs,
    and tincr_scc_inputs the ctypes structure it passes."""
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from tincr_gb300 import scc
    dt = scc.SYSTEM_DTYPE
    body = ['printf("%zu\\n", sizeof(tincr_scc_system));']
    body += ['printf("%%zu\\n", offsetof(tincr_scc_system, %s));' % f for f in dt.names]
    body += ['printf("%zu\\n", sizeof(tincr_scc_inputs));']
    body += ['printf("%%zu\\n", offsetof(tincr_scc_inputs, %s));' % f for f, _ in scc._Inputs._fields_]
    src = tmp_path / "lay.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "tincr_gb300.h"\nint main(void) { '
                   + " ".join(body) + " return 0; }\n")
    exe = tmp_path / "lay"
    subprocess.run([cc, str(src), "-I", os.path.join(ROOT, "include"), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    want = [dt.itemsize] + [dt.fields[f][1] for f in dt.names]
    want += [ctypes.sizeof(scc._Inputs)] + [getattr(scc._Inputs, f).offset for f, _ in scc._Inputs._fields_]
    assert got == want
