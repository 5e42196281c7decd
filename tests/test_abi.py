"""The C-ABI library: builds, loads, exports every declared symbol (no GPU)."""
import os
import re

import numpy as np
import pytest

from demon_simulation_code_gb300 import _lib, workloads as W
from demon_simulation_code_gb300.build import ROOT, build

HEADER = os.path.join(ROOT, "include", "demon_gb300.h")


def declared_symbols():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*int\s+(dm_\w+)\s*\(", src, flags=re.M)))


def test_library_builds_and_exports_every_declared_symbol():
    path = build()
    lib = _lib.load(path)
    syms = declared_symbols()
    assert len(syms) >= 20
    for s in syms:
        assert hasattr(lib, s), s
        assert s in _lib.SIGNATURES, s
    assert lib.dm_version() == 1


def test_create_error_is_reported_without_gpu():
    import torch

    if torch.cuda.is_available():
        pytest.skip("GPU present")
    from demon_simulation_code_gb300 import Context, DemonError

    with pytest.raises(DemonError):
        Context(0)


def test_force_params_layout_matches_oracle():
    import ctypes

    import oracle

    assert ctypes.sizeof(_lib.ForceParams) == ctypes.sizeof(oracle.Params) == 232
    assert [f[0] for f in _lib.ForceParams._fields_] == [f[0] for f in oracle.Params._fields_]


def test_force_params_layout_matches_c_header(tmp_path):
    """ctypes' dm_force_params has the C compiler's size and field offsets."""
    import ctypes
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    names = [f[0] for f in _lib.ForceParams._fields_]
    src = tmp_path / "layout.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "demon_gb300.h"\nint main(void) {\n'
                   '  printf("%zu\\n", sizeof(dm_force_params));\n'
                   + "".join(f'  printf("%zu\\n", offsetof(dm_force_params, {k}));\n' for k in names)
                   + "  return 0;\n}\n")
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-std=c11", "-I", inc, str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True,
                                          text=True).stdout.split()]
    assert got[0] == ctypes.sizeof(_lib.ForceParams)
    assert got[1:] == [getattr(_lib.ForceParams, k).offset for k in names]


def test_workloads_are_seeded():
    a = W.disk16k().clouds[0]
    b = W.disk16k().clouds[0]
    assert np.array_equal(a.x, b.x) and a.n == 16384
    assert np.all(np.hypot(a.x, a.y) <= 2e-2)
    w = W.batch256()
    ns = [c.n for c in w.clouds]
    assert len(ns) == 256 and min(ns) >= 64 and max(ns) <= 4096
    assert W.disk512().pairs_per_eval == 512 * 511


def test_noalloc_rejects_bad_sizes_and_params_before_any_device_call():
    """dm_diagnostics_noalloc checks its size limit and its force parameters
    on the host, before it looks up its scratch or launches anything, with
    the same parameter rules as dm_cloud_set_forces -- so these rejections
    need no GPU."""
    import ctypes

    lib = _lib.load(build())
    fake = 16  # never dereferenced: every case below is rejected on the host
    ok = dict(flags=W.CONFINEMENT | W.DRAG | W.SHIELDED_COULOMB, shielding=2e4, confine=1e8, gamma=3.0)
    cases = [
        (0, ok, _lib.DM_ERR_ARG),
        (524288 + 1, ok, _lib.DM_ERR_ARG),
        (64, {**ok, "shielding": float("inf")}, _lib.DM_ERR_ARG),
        (64, {**ok, "shielding": 0.0}, _lib.DM_ERR_ARG),
        (64, {**ok, "thermal_mode": 2}, _lib.DM_ERR_ARG),
        (64, {**ok, "flags": ok["flags"] | (1 << 20)}, 6),  # DM_ERR_UNSUPPORTED
    ]
    for n, params, want in cases:
        p = _lib.force_params(**params)
        rc = lib.dm_diagnostics_noalloc(n, *([fake] * 6), ctypes.byref(p), fake, None)
        assert rc == want, (n, params, rc)
