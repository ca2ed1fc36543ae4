"""The C ABI library builds, loads and exports every declared entry point;
argument and state errors come back as status codes (no GPU needed)."""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest

from petar_gb300 import gpuforce

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> list[str]:
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        names += re.findall(r"^\s*(?:int|const char\s*\*)\s*(pgf_\w+)\s*\(", text, flags=re.M)
    return names


def test_header_declares_entry_points():
    names = declared_functions()
    for required in ("pgf_initialize", "pgf_dispatch_index", "pgf_dispatch", "pgf_retrieve",
                     "pgf_last_error", "pgf_finalize"):
        assert required in names


def test_library_exports_every_declared_symbol():
    lib_path = gpuforce.load().__dict__.get("_name") or str(gpuforce.library_path())
    out = subprocess.run(["nm", "-D", "--defined-only", lib_path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(\w+)$", out, flags=re.M))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing


def test_status_codes_without_device_or_state():
    lib = gpuforce.load()
    assert lib.pgf_set_precision(7) == 1  # PGF_ERR_ARG
    assert b"precision" in lib.pgf_last_error()
    if lib.pgf_initialize(0, 0.0, 1e-4, 1.0) == 0:
        pytest.skip("a GPU is present; the no-device path is not reachable")
    assert lib.pgf_initialize(0, 0.0, 1e-4, 1.0) == 2  # PGF_ERR_NO_DEVICE
    # Without a successful initialize every call is a state error.
    assert lib.pgf_dispatch_index(0, 0, None, None, None, None, None, None, None,
                                  None, 0, None, None, 0, None, 0) == 4
    assert lib.pgf_retrieve(0, 0, None, None, None) == 4
    assert lib.pgf_recompute(0) == 4


def test_setter_arguments_checked_without_device():
    """The tuning and accuracy setters validate their arguments on the host."""
    lib = gpuforce.load()
    assert lib.pgf_set_walk_split_unit(0) == 1 and lib.pgf_set_walk_split_unit(257) == 1
    assert lib.pgf_set_walk_split_unit(16) == 0
    assert lib.pgf_set_gradient_accuracy(2) == 1 and lib.pgf_set_gradient_accuracy(-1) == 1
    assert lib.pgf_set_gradient_accuracy(1) == 0
    assert lib.pgf_set_dispatch_stages(9) == 1 and lib.pgf_set_dispatch_stages(0) == 0
    with pytest.raises(gpuforce.GpuForceError):
        gpuforce.set_gradient_accuracy(3)
    with pytest.raises(gpuforce.GpuForceError):
        gpuforce.set_walk_split_unit(1000)


def test_bad_initialize_arguments():
    lib = gpuforce.load()
    assert lib.pgf_initialize(0, -1.0, 1e-4, 1.0) == 1
    assert lib.pgf_initialize(0, 0.0, float("nan"), 1.0) == 1


def test_python_errors_raise():
    with pytest.raises(gpuforce.GpuForceError):
        gpuforce.set_precision(9)


def test_record_layouts_match_petar():
    """Offsets the functors pass for PeTar's records (soft_ptcl.hpp field order)."""
    el, jl, sl, fl = gpuforce._layouts()
    assert (el.size, el.off_pos, el.off_r_search) == (48, 8, 32)
    assert (jl.off_mass, jl.off_pos, jl.off_r_search) == (8, 16, 80)
    assert (sl.off_mass, sl.off_pos, sl.off_quad, sl.has_quad) == (0, 8, 32, 1)
    assert (fl.size, fl.off_acc, fl.off_pot, fl.off_n_ngb, fl.n_ngb_bytes) == (40, 0, 24, 32, 8)


def test_variant_count_matches_header():
    import re
    text = (ROOT / "include" / "petar_gpuforce.h").read_text()
    n = int(re.search(r"#define PGF_NUM_KERNEL_VARIANTS (\d+)", text).group(1))
    assert n == gpuforce.NUM_KERNEL_VARIANTS
    d = int(re.search(r"#define PGF_DEFAULT_KERNEL_VARIANT (\d+)", text).group(1))
    assert d == gpuforce.DEFAULT_KERNEL_VARIANT
    assert 0 <= d < n


def test_nbody_entry_points_without_device():
    from petar_gb300 import nbody
    lib = nbody._lib()
    cfg = nbody.Config(0.0, 0.01, 1.0, 0.3, 20, 512, 0, -1, 2.0)
    h = ctypes.c_void_p()
    import numpy as np
    x = np.zeros(3)
    assert lib.pgf_nbody_create(None, 1, None, None, None, None, ctypes.byref(h)) == 1
    bad = nbody.Config(0.0, 0.0, 1.0, 0.3, 20, 512, 0, -1, 2.0)
    assert lib.pgf_nbody_create(ctypes.byref(bad), 1, x.ctypes.data, x.ctypes.data, x.ctypes.data,
                                x.ctypes.data, ctypes.byref(h)) == 1
    assert b"r_out" in lib.pgf_nbody_last_error()
    r = lib.pgf_nbody_create(ctypes.byref(cfg), 1, x.ctypes.data, x.ctypes.data, x.ctypes.data, x.ctypes.data,
                             ctypes.byref(h))
    if r == 0:
        lib.pgf_nbody_destroy(h)
        pytest.skip("a GPU is present")
    assert r == 2  # PGF_ERR_NO_DEVICE
    assert lib.pgf_nbody_force(None) == 1
    assert lib.pgf_nbody_destroy(None) == 0
