"""C-ABI library: builds, loads, exports every declared symbol; host-only
schedule helpers agree with the oracle (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

from pyflowreg_gb300 import _lib, build
from pyflowreg_gb300.api import make_params

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "flowreg_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(frg_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_and_exports_all_symbols():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), f"{name} declared in the header but not exported"
    assert lib.frg_version() == 2


def test_symbols_are_plain_c():
    # nm -D lists the C names unmangled
    import subprocess

    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (frg_[a-z0-9_]+)$", out, flags=re.M))
    assert set(declared_functions()) <= exported


@pytest.mark.parametrize("H,W,eta,levels,min_level", [
    (256, 256, 0.8, 100, 0), (512, 512, 0.8, 100, 0), (512, 796, 0.8, 100, 0), (30, 36, 0.8, 50, 0),
    (64, 300, 0.7, 50, 0), (1024, 1024, 0.8, 100, 0), (100, 90, 0.5, 3, 0), (120, 80, 0.8, 100, 4),
])
def test_schedule_matches_oracle(oracle, H, W, eta, levels, min_level):
    lib = _lib.load()
    p = make_params(alpha=(1.5, 2.5), eta=eta, levels=levels, min_level=min_level)
    n = lib.frg_schedule(ctypes.byref(p), H, W, 0, None, None, None, None)
    h = (ctypes.c_int * n)()
    w = (ctypes.c_int * n)()
    ax = (ctypes.c_double * n)()
    ay = (ctypes.c_double * n)()
    assert lib.frg_schedule(ctypes.byref(p), H, W, n, h, w, ax, ay) == n
    sched, ml = oracle.level_schedule(H, W, levels, eta, min_level)
    assert [s for _, s in sched] == list(zip(h, w))
    for q, (i, _) in enumerate(sched):
        sc = 1.0 if i == ml else eta ** (-0.5 * i)
        assert ax[q] == sc * 1.5 and ay[q] == sc * 2.5


@pytest.mark.parametrize("in_len,out_len", [(512, 9), (512, 410), (512, 512), (256, 205), (410, 512), (796, 637),
                                            (37, 30), (13, 19), (1024, 11)])
def test_resize_tables_match_oracle(oracle, in_len, out_len):
    lib = _lib.load()
    sig = oracle.sigma_for((in_len, in_len), (out_len, out_len))
    P = lib.frg_resize_tables(in_len, out_len, sig, 0, None, None)
    idx = np.empty((out_len, P), np.int32)
    wt = np.empty((out_len, P), np.float32)
    assert lib.frg_resize_tables(in_len, out_len, sig, P, idx.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                 wt.ctypes.data_as(ctypes.POINTER(ctypes.c_float))) == P
    ix, wx = oracle.resize_tables(in_len, out_len, sig, "numba")
    np.testing.assert_array_equal(idx, ix)
    # float32 Gaussian taps come from two exp implementations: allow 2 ulp
    np.testing.assert_allclose(wt, wx, rtol=0, atol=4e-7)


def _passes_model(iterations, lag, gmax=5):
    """Groups start at t = 0 and at every tick (t+1) % lag == 0; each is cut
    into passes of at most gmax iterations; only a group's first pass folds."""
    starts = sorted({0} | {t for t in range(iterations) if (t + 1) % lag == 0})
    out = []
    for i, s in enumerate(starts):
        e = starts[i + 1] if i + 1 < len(starts) else iterations
        mode = (1 if s == 0 else 0) | (2 if (s + 1) % lag == 0 else 0)
        for q in range(s, e, gmax):
            out.append((min(gmax, e - q), mode if q == s else -1))
    return out


@pytest.mark.parametrize("iterations,lag", [(50, 5), (50, 1), (50, 7), (23, 3), (2, 5), (1, 1), (12, 4), (100, 13)])
def test_iteration_passes(iterations, lag):
    lib = _lib.load()
    n = lib.frg_iteration_passes(iterations, lag, 0, None, None)
    G = (ctypes.c_int * n)()
    M = (ctypes.c_int * n)()
    lib.frg_iteration_passes(iterations, lag, n, G, M)
    got = list(zip(G, M))
    assert got == _passes_model(iterations, lag)
    assert sum(G) == iterations


@pytest.mark.parametrize("in_len,out_len", [(512, 9), (512, 410), (256, 205), (410, 512), (37, 30), (1024, 11),
                                            (72, 58), (9, 11)])
def test_host_tables_equal_oracle_bit_for_bit(oracle, in_len, out_len):
    """The plan's tables (pyflowreg_gb300.tables, uploaded into every plan) are
    the reference's numpy construction: identical to the oracle's, bit for bit."""
    from pyflowreg_gb300 import tables

    sig = tables.sigma_for((in_len, in_len), (out_len, out_len))
    assert sig == oracle.sigma_for((in_len, in_len), (out_len, out_len))
    ix, wx = tables.resize_tables(in_len, out_len, sig)
    iy, wy = oracle.resize_tables(in_len, out_len, sig, "numba")
    np.testing.assert_array_equal(ix, iy)
    np.testing.assert_array_equal(wx, wy)


def test_host_tables_pinned_to_golden(golden_dir):
    """Tables of the reference source itself (golden vectors, plain-Python
    typing) agree with the plan's numba-typed tables to float32 rounding."""
    from pyflowreg_gb300 import tables

    g = np.load(os.path.join(golden_dir, "resize.npz"))
    for q, (ih, iw, oh, ow) in enumerate(g["cases"]):
        sig = tables.sigma_for((ih, iw), (oh, ow))
        ix, wx = tables.resize_tables(iw, ow, sig)
        np.testing.assert_array_equal(ix, g[f"ix{q}"])
        np.testing.assert_allclose(wx, g[f"wx{q}"], rtol=0, atol=2e-7)


def test_params_struct_layout_matches_header(tmp_path):
    """The ctypes mirror of frg_params has the C struct's size and offsets."""
    import subprocess

    fields = [f[0] for f in _lib.FrgParams._fields_]
    src = tmp_path / "layout.c"
    src.write_text('#include <stddef.h>\n#include <stdio.h>\n#include "flowreg_gb300.h"\nint main(void){\n'
                   + 'printf("%zu\\n", sizeof(frg_params));\n'
                   + "".join(f'printf("%zu\\n", offsetof(frg_params, {f}));\n' for f in fields) + "return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.dirname(HEADER), str(src), "-o", str(exe)], check=True)
    vals = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert vals[0] == ctypes.sizeof(_lib.FrgParams)
    assert vals[1:] == [getattr(_lib.FrgParams, f).offset for f in fields]


@pytest.mark.parametrize("stages,sched,steps", [
    (1, [0.0], 2), (3, [0.5, 0.7, 1.0], 2), (3, [0.0, 0.7, 0.5], 2), (2, [0.0, 0.9], 2), (2, [0.0, 1.0], 0),
    (17, [0.0] * 16, 2), (2, [0.0, 1.5], 2),
])
def test_plan_create_rejects_bad_gnc_options(stages, sched, steps):
    """normalize_gnc_schedule / normalize_warping_steps (core/optical_flow.py:414-443)
    are checked before anything touches the device."""
    from pyflowreg_gb300.api import make_params

    lib = _lib.load()
    p = make_params()
    p.gnc_stages = stages
    for i, b in enumerate(sched[:_lib.FRG_MAX_GNC_STAGES]):
        p.gnc_schedule[i] = b
    p.warping_steps = steps
    out = ctypes.c_void_p()
    assert lib.frg_plan_create(ctypes.byref(p), 32, 32, 1, 1, ctypes.byref(out)) == 1  # FRG_EINVAL
    assert b"gnc" in lib.frg_last_error() or b"warping" in lib.frg_last_error()
