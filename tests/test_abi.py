"""The C-ABI library: it builds, loads, and exports every entry point include/vgcuda.h declares.
No compute call is made here (these run without a GPU)."""
import ctypes
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "vgcuda.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib_path():
    from verion_gb300 import build

    return build.build()


def test_library_exports_every_declared_symbol(lib_path):
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib_path)], capture_output=True, text=True, check=True)
    exported = set(re.findall(r" T (vg_[a-z0-9_]+)$", out.stdout, flags=re.M))
    declared = declared_functions()
    assert len(declared) >= 30
    missing = [f for f in declared if f not in exported]
    assert not missing, missing


def test_library_loads_and_binds(lib_path):
    from verion_gb300 import backend

    L = backend.lib()
    for name in declared_functions():
        assert hasattr(L, name)


def test_context_without_a_gpu_reports_no_device(lib_path):
    from verion_gb300 import backend

    L = backend.lib()
    n = ctypes.c_int(0)
    try:
        import torch  # noqa: F401

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = ctypes.c_void_p()
    status = L.vg_context_create(ctypes.byref(h))
    assert status == backend.VG_ERR_NO_DEVICE and not h.value
    buf = ctypes.create_string_buffer(256)
    assert L.vg_last_error(buf, 256) > 0 and buf.value


def test_null_handles_are_rejected(lib_path):
    from verion_gb300 import backend

    L = backend.lib()
    assert L.vg_set_multiscatter(None, 1) == backend.VG_ERR_INVALID
    assert L.vg_accumulate(None, None, 1) == backend.VG_ERR_INVALID
    assert L.vg_accum_samples(None) == 0
    # Batched serving: no context, no requests.
    assert L.vg_batch_render(None, None, 0, None, None, None) == backend.VG_ERR_INVALID
    assert L.vg_set_batch_options(None, 0, 0, 0) == backend.VG_ERR_INVALID
    assert L.vg_set_batch_wave_slots(None, 1 << 21) == backend.VG_ERR_INVALID
    assert L.vg_set_batch_device_loop(None, 1) == backend.VG_ERR_INVALID


def test_oracle_library_loads(oracle_lib):
    assert oracle_lib.lib().or_pcg(0) != 0
