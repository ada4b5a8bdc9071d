"""C-ABI checks that need no GPU: the library loads, exports every function
declared in include/*.h, and its host-side logic (IRD selector, input
validation, error reporting) matches the reference semantics."""
from __future__ import annotations

import ctypes as C
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden_cases, golden_csr, load_golden


def declared_functions() -> list[str]:
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        src = re.sub(r"//[^\n]*", "", src)
        src = re.sub(r"#[^\n]*", "", src)
        src = src.replace('extern "C" {', "")
        prev = None
        while prev != src:  # drop struct / enum bodies
            prev = src
            src = re.sub(r"\{[^{}]*\}", "", src)
        src = src.replace("{", "").replace("}", "")
        for stmt in src.split(";"):
            s = " ".join(stmt.split())
            if not s.endswith(")") or s.startswith("typedef"):
                continue
            m = re.match(r"^(?:extern\s+)?(?:const\s+)?(?:struct\s+)?[A-Za-z_]\w*[\s\*]+\**\s*([A-Za-z_]\w*)\s*\(", s)
            if m:
                names.append(m.group(1))
    return sorted(set(names))


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for f in ("SpB_mxv", "IRD_VNEC", "Build_VNEC_L", "SpMV_VNEC_L_FP64", "SpMV_VNEC_L_FP32"):
        assert f in names


def test_library_exports_every_declared_symbol(built):
    from vnec_gb300 import _loader

    lib = _loader.load("vnec_gb300")
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_generator_library_loads(built):
    from vnec_gb300 import _loader

    assert hasattr(_loader.load("vnec_gen"), "vnec_gen_rmat")


@pytest.mark.parametrize("case", [c for c in golden_cases() if bool(load_golden(c)["vnec_ds_defined"])])
@pytest.mark.parametrize("tag", ["f64", "f32"])
def test_ird_selector_matches_reference(built, case, tag):
    """IRD_VNEC (host computation, no GPU) returns the reference's choice."""
    from vnec_gb300 import api

    g = load_golden(case)
    m = golden_csr(g)
    dt = np.float64 if tag == "f64" else np.float32
    A = api.Matrix.from_csr(m, dtype=dt)
    choice = api.IRD_VNEC(A, api.SpB_FP64 if tag == "f64" else api.SpB_FP32)
    expected = {1: api.SpB_VNEC_D, 2: api.SpB_VNEC_S}[int(g[f"auto_variant_{tag}"])]
    assert choice == expected


def test_ird_selector_matches_oracle_on_fresh_matrices(built):
    from oracle import oracle as O
    from vnec_gb300 import api
    from vnec_gb300 import generators as G

    for m in (G.banded(5000, 5, seed=1), G.banded(5000, 65, seed=2), G.uniform_k(5000, 8, seed=3),
              G.blockdiag(4096, 32, seed=4), G.stencil27(14, seed=5), G.rmat(13, 60000, seed=6)):
        A = api.Matrix.from_csr(m)
        want, _ = O.ird(m, fp64=True)
        assert api.IRD_VNEC(A, api.SpB_FP64) == want


def _bad(m_rows, n_cols, ptr, idx, val, fmt=None):
    from vnec_gb300 import api

    A = api.Matrix(m_rows, n_cols, ptr, idx, val)
    if fmt is not None:
        A._s.matrix_base.format_type = fmt
    return A


@pytest.mark.parametrize("kind", ["csc", "ptr_not_monotone", "col_out_of_range", "nnz_mismatch", "int_type"])
def test_invalid_input_fails_with_message_before_any_device_work(built, kind):
    """The reference exits the process on bad input (SpB_Error.c:4-8); this
    library returns NULL/SpB_FAILURE with a message, before touching the GPU."""
    from vnec_gb300 import api

    ptr = np.array([0, 2, 3, 5])
    idx = np.array([0, 2, 1, 0, 2])
    val = np.arange(5, dtype=np.float64)
    if kind == "csc":
        A = _bad(3, 3, ptr, idx, val, fmt=api.SpB_CSC)
    elif kind == "ptr_not_monotone":
        A = _bad(3, 3, np.array([0, 3, 2, 5]), idx, val)
    elif kind == "col_out_of_range":
        A = _bad(3, 3, ptr, np.array([0, 2, 1, 0, 3]), val)
    elif kind == "nnz_mismatch":
        A = _bad(3, 3, ptr, idx, val)
        A._s.nnz = 4
    else:
        A = _bad(3, 3, ptr, idx, val)
        A._s.matrix_base.element_type = 4  # SpB_INT32
    h = api.lib().Build_VNEC_L(A.handle)
    assert not h
    assert api.last_error() != ""


def test_unknown_handle_is_rejected(built):
    from vnec_gb300 import api

    A = api.Matrix(2, 2, np.array([0, 1, 2]), np.array([0, 1]), np.ones(2))
    x, y = api.Vector(np.ones(2)), api.Vector(n=2)
    bogus = C.c_void_p(12345678)
    assert api.lib().SpB_mxv(y.handle, A.handle, x.handle, bogus) == api.SpB_FAILURE
    assert "unknown" in api.last_error()
    api.lib().SpMV_VNEC_L_FP64(y.handle, A.handle, x.handle, bogus)
    assert "unknown" in api.last_error()


LAYOUT_PROBE = r"""
#include <stdio.h>
#include <stddef.h>
%s
int main(void) {
  printf("%%zu %%zu %%zu %%zu %%zu %%zu %%zu %%zu\n", sizeof(struct SpB_Matrix_opaque),
         offsetof(SpB_Matrix_CSC_or_CSR, val), offsetof(SpB_Matrix_CSC_or_CSR, indices),
         offsetof(SpB_Matrix_CSC_or_CSR, ptr), offsetof(SpB_Matrix_CSC_or_CSR, nnz),
         sizeof(SpB_Matrix_CSC_or_CSR), offsetof(SpB_Vector_Dense, values), sizeof(VNEC_L));
  return 0;
}
"""


def _layout(tmp_path, includes: str, flags: list[str]) -> list[int]:
    import subprocess

    src = tmp_path / "probe.c"
    src.write_text(LAYOUT_PROBE % includes)
    exe = tmp_path / "probe"
    subprocess.run(["gcc", *flags, str(src), "-o", str(exe)], check=True, capture_output=True)
    return [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]


def test_extension_structs_match_c_header(tmp_path):
    """Every field of the ctypes mirrors of SpB_VNEC_options_ext,
    SpB_VNEC_info_ext and SpB_VNEC_batch_options_ext sits at the C header's
    offset, and the sizes agree (new options take reserved slots)."""
    import subprocess

    from vnec_gb300 import api

    structs = {"SpB_VNEC_options_ext": api.Options, "SpB_VNEC_info_ext": api.Info,
               "SpB_VNEC_batch_options_ext": api.BatchOptions}
    lines, want = [], []
    for cname, py in structs.items():
        lines.append(f'  printf("%zu\\n", sizeof({cname}));')
        want.append(C.sizeof(py))
        for fname, _ in py._fields_:
            lines.append(f'  printf("%zu\\n", offsetof({cname}, {fname}));')
            want.append(getattr(py, fname).offset)
    src = tmp_path / "ext_probe.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "vnec_gb300.h"\nint main(void) {\n' +
                   "\n".join(lines) + "\n  return 0;\n}\n")
    exe = tmp_path / "ext_probe"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True,
                   capture_output=True)
    got = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert got == want


def test_struct_layout_matches_c_header(tmp_path):
    """The ctypes mirror and include/vnec_spb_types.h lay out identically
    (and, where the reference headers exist, identically to them)."""
    from vnec_gb300 import api

    mine = _layout(tmp_path, '#include "vnec_spb_types.h"', ["-I", os.path.join(ROOT, "include")])
    py = [C.sizeof(api._MatrixBase), api._CsrStruct.val.offset, api._CsrStruct.indices.offset,
          api._CsrStruct.ptr.offset, api._CsrStruct.nnz.offset, C.sizeof(api._CsrStruct),
          api._DenseStruct.values.offset, mine[7]]
    assert mine == py
    from oracle import oracle as O

    ref = O.reference_tree()
    if ref:
        theirs = _layout(tmp_path, '#include "SpB_Matrix_CSC_or_CSR.h"\n#include "SpB_Vector_Dense.h"',
                         ["-I", f"{ref}/include", "-I", f"{ref}/src/core/include"])
        assert theirs == mine
