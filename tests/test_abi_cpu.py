"""CPU checks of the C ABI: the library builds for sm_103a, loads, exports every symbol
the header declares, and its host-side set-up helpers agree with the oracle."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from oracle import oracle as O
from starfish_gb300 import abi, build
from starfish_gb300 import workloads as W

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return abi.load()


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(sf_[a-z0-9_]+)\s*\(", txt))
    return names


def test_exports_match_header(lib):
    names = declared_symbols()
    assert len(names) >= 15
    for n in sorted(names):
        assert hasattr(lib, n), f"missing export {n}"
    # the Python binding declares exactly what the header declares
    assert set(abi.EXPORTS) <= names


def test_version(lib):
    assert b"sm_103a" in lib.sf_version()


def test_node_segments_match_oracle(lib):
    for spec in (W.es_pic_mesh(81, 41, 1e-3), W.es_pic_mesh(101, 51, 1e-3, electrode_halfwidth=7.3e-3)):
        p1, i1 = abi.build_node_segments(spec.ni, spec.nj, spec.x0, spec.dh, spec.seg_xy)
        om = O.OMesh(spec.ni, spec.nj, spec.x0, spec.dh, spec.domain, spec.node_type, spec.face_type)
        p2, i2 = O.node_segments(om, spec.seg_xy)
        assert np.array_equal(p1, p2)
        assert np.array_equal(i1, i2)


def test_ctx_create_fails_cleanly_without_gpu(lib):
    """Without a device the context call returns an error code, never crashes."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("GPU present")
    except Exception:
        pass
    spec = W.es_pic_mesh(21, 11, 1e-3)
    d = spec.desc()
    h = C.c_void_p()
    rc = lib.sf_ctx_create(C.byref(d), 0, C.byref(h))
    assert rc != abi.SF_OK
    assert lib.sf_last_error(None)


def test_bad_arguments_rejected(lib):
    h = C.c_void_p()
    assert lib.sf_ctx_create(None, 0, C.byref(h)) == abi.SF_ERR_ARG
    spec = W.es_pic_mesh(21, 11, 1e-3)
    d = spec.desc()
    d.ni = 2
    assert lib.sf_ctx_create(C.byref(d), 0, C.byref(h)) == abi.SF_ERR_ARG


def test_struct_layouts_match_header(tmp_path):
    """Every ctypes structure has the size and field offsets that the C compiler gives the
    header's struct of the same name (a shorter Python struct would let the library write
    past its end)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = [(abi.MeshDesc, "sf_mesh_desc"), (abi.PushStats, "sf_push_stats"),
             (abi.PoissonParams, "sf_poisson_params"), (abi.SolveStats, "sf_solve_stats"),
             (abi.Sigma, "sf_sigma"), (abi.BatchStats, "sf_batch_stats")]
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "starfish_gpu.h"', "int main(void) {"]
    expect = []
    for cls, cname in pairs:
        lines.append(f'  printf("%zu\\n", sizeof({cname}));')
        expect.append(C.sizeof(cls))
        for f in cls._fields_:
            lines.append(f'  printf("%zu\\n", offsetof({cname}, {f[0]}));')
            expect.append(getattr(cls, f[0]).offset)
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-std=c11", "-I", inc, str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert got == expect
