"""Failure paths on the GPU, in the forms that fault and hang nothing:

* a bounded device wait that runs out: nca_wait_probe waits on an mbarrier
  that nothing completes (no copy issued), through the bounded-wait helper of
  the pipeline kernels; the kernel records NCA_ERR_TIMEOUT, returns, and
  nca_device_status reports it once; the context then runs kernels normally;
* a corrupt or truncated cubin in the on-disk JIT cache: a fresh process must
  reject it (magic, length and hash are checked), recompile, store a good
  copy, and a third process must load that copy from disk."""
import ctypes
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import ncarray_gb300 as nca
from ncarray_gb300 import _lib

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent


def test_bounded_wait_times_out_with_status(cuda):
    torch = cuda
    s = torch.cuda.current_stream().cuda_stream
    st = ctypes.c_int32(-1)
    _lib.call("nca_device_status", ctypes.byref(st), s)   # clear anything earlier tests left
    _lib.call("nca_wait_probe", ctypes.c_double(0.2), s)
    _lib.call("nca_device_status", ctypes.byref(st), s)
    assert st.value == _lib.ERR_TIMEOUT
    _lib.call("nca_device_status", ctypes.byref(st), s)
    assert st.value == 0   # read and cleared
    x = np.arange(4096, dtype=np.float32)
    a = nca.NCDevArray.from_host(x)
    with nca.lazy_mode():
        e = a * 2.0 + 1.0
    assert np.array_equal(e.materialize().to_host(), x * np.float32(2.0) + np.float32(1.0))
    with pytest.raises(nca.NcaError):
        _lib.call("nca_wait_probe", ctypes.c_double(5.0), s)   # limits are capped


CHILD = r"""
import ctypes, json
import numpy as np
import ncarray_gb300 as nca
from ncarray_gb300 import _lib
x = np.arange(1000, dtype=np.float32)
a = nca.NCDevArray.from_host(x)
with nca.lazy_mode():
    e = a * 3.0 - 7.0
ok = bool(np.array_equal(e.materialize().to_host(), x * np.float32(3.0) - np.float32(7.0)))
c, d, m = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
_lib.call("nca_jit_stats", ctypes.byref(c), ctypes.byref(d), ctypes.byref(m))
print(json.dumps({"ok": ok, "compiled": c.value, "disk": d.value}))
"""


def _child(cache):
    env = dict(os.environ, NCA_GB300_CACHE_DIR=str(cache),
               PYTHONPATH=str(ROOT) + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, "-c", CHILD], env=env, capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_corrupt_cache_files_are_rejected(cuda, tmp_path):
    first = _child(tmp_path)
    assert first["ok"] and first["compiled"] >= 1 and first["disk"] == 0
    files = sorted(tmp_path.glob("*.cubin"))
    assert files
    for k, f in enumerate(files):
        raw = bytearray(f.read_bytes())
        if k % 3 == 0:
            raw = raw[: len(raw) // 2]           # truncated
        elif k % 3 == 1:
            raw[len(raw) // 2] ^= 0xFF           # one byte flipped: hash mismatch
        else:
            raw[:8] = b"garbage!"                # wrong magic
        f.write_bytes(bytes(raw))
    second = _child(tmp_path)
    assert second["ok"] and second["compiled"] >= 1 and second["disk"] == 0
    third = _child(tmp_path)
    assert third["ok"] and third["compiled"] == 0 and third["disk"] >= 1
