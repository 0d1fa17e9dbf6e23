"""CPU checks of the C ABI: the library loads, exports every declared
symbol, and its structs match the reference layout (no GPU calls)."""
from __future__ import annotations

import ctypes as C
import os

import pytest

from openvort_gb300 import abi, gpu


@pytest.fixture(scope="module")
def lib():
    from openvort_gb300 import build
    build.build()
    return gpu.load()


def test_every_declared_symbol_is_exported(lib):
    """ov_* from libovgpu.so, ovd_* (the drop-in layer) from libovdropin.a."""
    import subprocess
    from openvort_gb300 import build
    names = gpu.declared_symbols()
    assert "ov_update_velocities" in names and "ov_rk4_step" in names and "ovd_update_velocities" in names
    missing = [n for n in names if n.startswith("ov_") and not hasattr(lib, n)]
    assert not missing, missing
    syms = subprocess.run(["nm", build.DROPIN], capture_output=True, text=True).stdout
    defined = {ln.split()[-1] for ln in syms.splitlines() if " T " in ln}
    missing = [n for n in names if n.startswith("ovd_") and n not in defined]
    assert not missing, missing
    assert "__wrap_update_velocities" in defined


def test_defaults_are_the_reference_defaults(lib):
    p = abi.Params()
    lib.ov_params_default(C.byref(p))
    ref = abi.make_params()
    for f, _ in abi.Params._fields_:
        if f in ("vn", "vs", "vb"):
            a, b = getattr(p, f), getattr(ref, f)
            assert (a.type, a.strength, list(a.direction.p)) == (b.type, b.strength, list(b.direction.p))
        else:
            assert getattr(p, f) == getattr(ref, f), f


def test_layouts():
    assert C.sizeof(abi.TangleState) == 168
    assert abi.TangleState.box.offset == 64 and abi.TangleState.N.offset == 152
    assert C.sizeof(abi.ImageTangle) == 28 and C.sizeof(abi.ExtVel) == 56


def test_missing_library_fails_loudly(tmp_path):
    saved = gpu._LIB
    gpu._LIB = None
    try:
        with pytest.raises(RuntimeError):
            gpu.load(str(tmp_path / "nope.so"))
    finally:
        gpu._LIB = saved


def test_no_device_is_reported(lib):
    # on a machine without a GPU the context call reports OV_ERR_NODEVICE
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gpu.OVError) as e:
        gpu.Context(0)
    assert e.value.code == 9
