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
REF_INC = "/root/reference/include"
OBJ = os.path.join(ROOT, "oracle", "_ref", "obj")
WRAPPED = ["update_tangents_normals", "update_velocities", "update_velocity", "rk4_step", "reconnect", "remesh",
           "eliminate_small_loops", "enforce_periodic_boundaries", "smooth", "octree_build", "octree_get_vs",
           "octree_destroy", "enforce_wall_boundaries", "save_tangle", "load_tangle", "add_loop", "add_line_in_zdir",
           "inject_vortices"]


@pytest.mark.skipif(not (os.path.isdir(REF_INC) and glob.glob(os.path.join(OBJ, "*.o"))),
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
