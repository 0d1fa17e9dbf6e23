"""Smoothing's low-pass filter against FFTW itself, where libfftw3 exists.

OpenVort's low_pass_filter (vortex_smooth.c:134-175) plans
fftw_plan_r2r_1d(N, in, out, FFTW_FORWARD, FFTW_ESTIMATE), zeroes the middle
2*floor(freq_to_cutoff*N/2)+1 bins (2*... for odd N), plans the inverse with
FFTW_BACKWARD and divides by N.  FFTW_FORWARD and FFTW_BACKWARD are the
complex-DFT sign constants (-1, +1) passed where an fftw_r2r_kind belongs.
The C restatement (oracle/ov_oracle.c, orc_low_pass_filter) assumes the
half-complex R2HC / HC2R pair that the reference's comment describes; this
test runs the reference's calls against the host's libfftw3 in a child
process (an out-of-range kind may make FFTW abort) and compares.

Marked gpu so that it runs on the GPU host with the other parity tests; it
uses no GPU.  Skipped where libfftw3 is not installed.
"""
from __future__ import annotations

import ctypes.util
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle.pyoracle import Checker

pytestmark = pytest.mark.gpu
FFTW = ctypes.util.find_library("fftw3")

CHILD = r"""
import ctypes as C, json, sys
import numpy as np
L = C.CDLL(sys.argv[1])
L.fftw_plan_r2r_1d.restype = C.c_void_p
L.fftw_plan_r2r_1d.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_uint]
L.fftw_execute.argtypes = [C.c_void_p]
L.fftw_destroy_plan.argtypes = [C.c_void_p]
FORWARD, BACKWARD, ESTIMATE = -1, 1, 1 << 6
cut = float(sys.argv[2])
out = {}
for n in json.loads(sys.argv[3]):
    x = np.cos(np.arange(n) * 0.7) + 0.3 * np.sin(np.arange(n) * 2.9) + 0.01 * np.arange(n)
    a = np.ascontiguousarray(x, dtype=np.float64)
    b = np.zeros(n)
    pf = L.fftw_plan_r2r_1d(n, a.ctypes.data, b.ctypes.data, FORWARD, ESTIMATE)
    if not pf:
        out[n] = "null forward plan"
        continue
    L.fftw_execute(pf)
    s = int(cut * n / 2)
    if n > 2 * s + 1:
        hi = n // 2 + 1 + s if n % 2 == 0 else n // 2 + s
        b[n // 2 - s:hi] = 0
    pb = L.fftw_plan_r2r_1d(n, b.ctypes.data, a.ctypes.data, BACKWARD, ESTIMATE)
    if not pb:
        out[n] = "null backward plan"
        continue
    L.fftw_execute(pb)
    out[n] = list(a / n)
    L.fftw_destroy_plan(pf)
    L.fftw_destroy_plan(pb)
print(json.dumps(out))
"""

SIZES = [7, 8, 33, 64, 255, 256]
CUTOFF = 0.8


@pytest.mark.skipif(not FFTW, reason="libfftw3 not installed on this host: smoothing parity stays unpinned")
def test_low_pass_filter_matches_fftw():
    p = subprocess.run([sys.executable, "-c", CHILD, FFTW, str(CUTOFF), json.dumps(SIZES)], capture_output=True,
                       text=True, timeout=120, env={**os.environ, "OMP_NUM_THREADS": "1"})
    assert p.returncode == 0, f"FFTW with the reference's kinds failed: rc {p.returncode} {p.stderr[-400:]}"
    got = json.loads(p.stdout)
    port = Checker("port")
    for n in SIZES:
        res = got[str(n)]
        assert not isinstance(res, str), f"N={n}: {res}"
        x = np.cos(np.arange(n) * 0.7) + 0.3 * np.sin(np.arange(n) * 2.9) + 0.01 * np.arange(n)
        ours = port.low_pass_filter(x, CUTOFF)
        err = np.abs(np.asarray(res) - ours).max() / np.abs(ours).max()
        print(f"N={n}: max rel diff {err:.2e}")
        assert err < 1e-12
