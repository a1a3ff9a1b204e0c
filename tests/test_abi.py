"""The C ABI library: it loads, exports every entry point include/*.h
declares, and its host-only helpers agree with the oracle (no GPU needed)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from blobs_gb300 import native, scenes
from oracle import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s+\**(blobs_[A-Za-z0-9_]+)\s*\(",
                             text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_entry_points():
    names = declared_symbols()
    assert "blobs_world_step" in names and "blobs_world_load" in names
    assert len(names) >= 15


@pytest.mark.parametrize("name", declared_symbols())
def test_library_exports(name):
    L = ctypes.CDLL(native.LIB_PATH)
    assert hasattr(L, name), name


def test_abi_version_and_status_strings():
    L = native.lib()
    assert L.blobs_abi_version() == 1
    assert native.status_string(0) == "ok"
    assert "NaN" in native.status_string(native.ERR_NAN)


def test_config_defaults_match_physics_new():
    cfg = native.make_config()
    assert cfg.substeps == 8 and cfg.joint_iterations == 4 and cfg.collisions_enabled == 1  # physics.rs:46-62


@pytest.mark.parametrize("seed", [0, 1])
def test_mass_inertia_matches_oracle(seed):
    s = scenes.jointed_bodies(seed=seed, n=3000, n_joints=100, n_springs=100, side=60.0)
    s.col_sensor[::7] = 1
    s.col_mass_override[::5] = 0.75
    m, I = native.mass_inertia(s)
    mo, Io = oracle.mass_inertia_f32(s)
    np.testing.assert_array_equal(m, mo)
    np.testing.assert_array_equal(I, Io)


def test_world_create_without_device_is_an_error_not_a_fallback():
    h = ctypes.c_void_p()
    cfg = native.make_config()
    st = native.lib().blobs_world_create(ctypes.byref(cfg), ctypes.byref(h))
    if st == native.OK:           # a GPU is present: fine, release it
        native.lib().blobs_world_destroy(h)
    else:
        assert st == native.ERR_NO_DEVICE


def test_header_is_plain_c(tmp_path):
    """include/blobs_gpu.h compiles as C99 (no C++ types cross the boundary),
    and a C program can take the address of every entry point."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "abi.c"
    refs = "\n".join("  (void (*)(void))&%s," % n for n in declared_symbols())
    src.write_text('#include "blobs_gpu.h"\nvoid (*entry_points[])(void) = {\n%s\n};\n' % refs)
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only",
                        "-I", os.path.join(ROOT, "include"), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
