"""The drop-in links into OpenVort's own program (CPU check, where the
OpenVort checkout and its compiled objects are present).

Builds tests/dropin_link_main.c against the reference's headers and objects
(oracle/_ref/obj) plus ov_dropin.c compiled with -DOV_DROPIN_WRAP, with
-Wl,--wrap for every replaced entry point, and checks that the reference's
calls now resolve to the drop-in.
"""
from __future__ import annotations

import glob
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OBJ = os.path.join(ROOT, "oracle", "_ref", "obj")


def _ref_include() -> str:
    """The reference's include/ directory, as recorded by oracle/Makefile's ref target."""
    rec = os.path.join(ROOT, "oracle", "_ref", "ref_dir.txt")
    if not os.path.exists(rec):
        return ""
    with open(rec) as f:
        return os.path.join(f.read().strip(), "include")


REF_INC = _ref_include()
WRAPPED = ["update_tangents_normals", "update_velocities", "update_velocity", "rk4_step", "reconnect", "remesh",
           "eliminate_small_loops", "enforce_periodic_boundaries", "smooth", "octree_build", "octree_get_vs",
           "octree_destroy", "enforce_wall_boundaries", "save_tangle", "load_tangle", "add_loop", "add_line_in_zdir",
           "inject_vortices"]


@pytest.mark.skipif(not (REF_INC and os.path.isdir(REF_INC) and glob.glob(os.path.join(OBJ, "*.o"))),
                    reason="OpenVort checkout / reference objects not present")
def test_reference_program_links_against_dropin(tmp_path):
    from openvort_gb300 import build
    build.build()
    libdir = os.path.join(ROOT, "openvort_gb300", "lib")
    shim = tmp_path / "dropin.o"
    subprocess.run(["gcc", "-O2", "-DOV_DROPIN_WRAP", "-c", os.path.join(ROOT, "openvort_gb300", "csrc", "ov_dropin.c"),
                    "-o", str(shim)], check=True)
    exe = tmp_path / "vortices_gpu"
    wraps = [f"-Wl,--wrap={n}" for n in WRAPPED]
    cmd = ["gcc", "-O2", "-fopenmp", "-I" + REF_INC, os.path.join(ROOT, "tests", "dropin_link_main.c"),
           *sorted(glob.glob(os.path.join(OBJ, "*.o"))), str(shim), *wraps, "-L" + libdir, "-lovgpu",
           "-Wl,-rpath," + libdir, "-lm", "-o", str(exe)]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    syms = subprocess.run(["nm", str(exe)], capture_output=True, text=True).stdout
    for n in WRAPPED:
        assert f"__wrap_{n}" in syms
    # Run it.  Every wrapped call of the loop goes to the drop-in: with a GPU
    # the loop runs on it; without one each call reports that it found no
    # device and leaves the tangle as it was, and the program still ends.
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300,
                         env={**os.environ, "LD_LIBRARY_PATH": libdir})
    assert run.returncode == 0, run.stderr
    assert run.stdout.startswith("nodes "), run.stdout
    failures = [ln for ln in run.stderr.splitlines() if ln.startswith("libovgpu ")]
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        assert not failures, run.stderr
    else:
        # add_loop, then 3 steps of the main loop's 11 wrapped calls
        # (update_tangle is update_tangents_normals + update_velocities)
        assert len(failures) == 1 + 3 * 11, run.stderr
        assert all("error" in ln for ln in failures)
