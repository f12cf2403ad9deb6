"""CPU checks of the C ABI: the library builds and loads, exports every symbol the header
declares, its structs match the ctypes mirror, and host-only entry points work without a GPU."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from pfem_gb300 import api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pfem_gpu.h")


def header_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"PFG_API\s+[^;(]*?\b(pfg_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol(gpu_lib):
    syms = header_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(gpu_lib, s), s
    assert sorted(api.EXPORTED) == syms


def test_struct_layout_matches_header():
    src = r"""
    #include <stdio.h>
    #include <stddef.h>
    #include "pfem_gpu.h"
    int main(void) {
        printf("%zu %zu %zu %zu %zu\n", sizeof(pfg_params), sizeof(pfg_step_status),
               offsetof(pfg_params, K0), offsetof(pfg_params, hbm_budget_bytes),
               offsetof(pfg_step_status, time));
        return 0;
    }
    """
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        out = subprocess.check_output([exe]).decode().split()
    expect = [ctypes.sizeof(api.Params), ctypes.sizeof(api.StepStatus), api.Params.K0.offset,
              api.Params.hbm_budget_bytes.offset, api.StepStatus.time.offset]
    assert [int(x) for x in out] == expect


def test_default_params_host_only(gpu_lib):
    p = api.default_params(api.KIND_INCOMP_PSPG, 2)
    assert p.dim == 2 and p.rho == 1000.0 and p.mu == 1e-3
    assert p.picard_max_iter == 10 and p.picard_min_res == 1e-6
    assert tuple(p.gravity) == (0.0, -9.81, 0.0)
    q = api.default_params(api.KIND_WC_CDS_DPDT, 3)
    assert q.K0 == 2.2e7 and q.K0p == 7.0 and q.security_coeff == 0.3 and tuple(q.gravity) == (0.0, 0.0, -9.81)
    bad = api.Params()
    assert gpu_lib.pfg_default_params(7, 2, ctypes.byref(bad)) == -1
    assert gpu_lib.pfg_default_params(0, 4, ctypes.byref(bad)) == -1


def test_null_arguments_rejected(gpu_lib):
    assert gpu_lib.pfg_create(None, None) == -1
    assert gpu_lib.pfg_destroy(None) == -1
    assert gpu_lib.pfg_last_error(None) == b"null context"
    assert gpu_lib.pfg_version().startswith(b"pfem_gb300")


REMESH_HEADER = os.path.join(ROOT, "include", "pfem_remesh.h")


def test_remesh_library_exports_every_declared_symbol():
    from pfem_gb300 import build
    from pfem_gb300 import remesh as R

    build.build_remesh()
    lib = R.native_lib()
    txt = open(REMESH_HEADER).read()
    syms = sorted(set(re.findall(r"PFR_API\s+[^;(]*?\b(pfr_\w+)\s*\(", txt)))
    assert len(syms) == 7
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(R.REMESH_EXPORTED) == syms


def test_remesh_struct_layout_matches_header():
    from pfem_gb300 import remesh as R

    src = r"""
    #include <stdio.h>
    #include <stddef.h>
    #include "pfem_remesh.h"
    int main(void) {
        printf("%zu %zu %zu\n", sizeof(pfr_params), offsetof(pfr_params, jitter), offsetof(pfr_params, bounding_box));
        return 0;
    }
    """
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        exe = os.path.join(d, "t")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        out = subprocess.check_output([exe]).decode().split()
    P = R._PfrParams
    assert [int(x) for x in out] == [ctypes.sizeof(P), P.jitter.offset, P.bounding_box.offset]
