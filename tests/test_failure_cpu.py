"""Failure paths that need no GPU: an NVRTC compile error (injected through
the NCA_JIT_EXTRA_SOURCE diagnostic hook) must come back as NCA_ERR_COMPILE
with the compiler's log, never end the process, and leave the library usable
for the next call (the reference exits or throws here: rtcompiler.hh:68-88,
rtcompiler.cc:487-493)."""
import os
import subprocess
import sys
from pathlib import Path

from ncarray_gb300 import _lib

ROOT = Path(__file__).resolve().parent.parent

CHILD = r"""
import ctypes, os
from ncarray_gb300 import _lib
L = _lib.lib()
n = ctypes.c_int32(0)
rc = L.nca_jit_selftest(b"sm_103a", ctypes.byref(n))
print("first", rc)
print("message", L.nca_last_error().decode().replace("\n", " ")[:2000])
del os.environ["NCA_JIT_EXTRA_SOURCE"]
rc = L.nca_jit_selftest(b"sm_103a", ctypes.byref(n))
print("second", rc, n.value)
"""


def test_injected_compile_error_is_a_status(built_lib):
    env = dict(os.environ, NCA_JIT_EXTRA_SOURCE="#error injected-by-the-failure-test",
               PYTHONPATH=str(ROOT) + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, "-c", CHILD], env=env, capture_output=True, text=True, cwd=ROOT,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    out = dict(line.split(" ", 1) for line in r.stdout.splitlines() if " " in line)
    assert int(out["first"]) == _lib.ERR_COMPILE
    assert "injected-by-the-failure-test" in out["message"]
    rc, n = out["second"].split()
    assert int(rc) == _lib.OK and int(n) > 0
