"""The autotuner on the GPU (child processes with their own cache directory):
in search mode the first call of a shape class times the candidates and
stores the winner -- results stay bit-exact --, and a later process in the
default mode reads the stored choice and gives the same results."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

CHILD = r"""
import json, sys
import numpy as np
import ncarray_gb300 as nca
from ncarray_gb300 import tune
from ncarray_gb300.dtype import DType
from ncarray_gb300.stencil import Stencil3D, laplacian7
mode = int(sys.argv[1])
tune.set_mode(mode)
rng = np.random.default_rng(5)
x = rng.normal(size=1 << 22).astype(np.float32)
y = rng.normal(size=1 << 22).astype(np.float32)
a, b = nca.NCDevArray.from_host(x), nca.NCDevArray.from_host(y)
with nca.lazy_mode():
    e = a * b + 1.5
ok_ew = bool(np.array_equal(e.materialize().to_host(), x * y + np.float32(1.5)))
# a transposed view: the strided kernel
with nca.lazy_mode():
    e2 = a.reshape(1024, 4096).transpose(1, 0) - b.reshape(4096, 1024)
ok_nd = bool(np.array_equal(e2.materialize().to_host(), x.reshape(1024, 4096).T - y.reshape(4096, 1024)))
u = rng.normal(size=(96, 128, 256)).astype(np.float32)
src, dst = nca.NCDevArray.from_host(u), nca.NCDevArray((96, 128, 256), DType.float32)
Stencil3D(laplacian7().reshape(27), 0.1).apply(src, dst)
import hashlib
print(json.dumps({"ok_ew": ok_ew, "ok_nd": ok_nd, "stencil": hashlib.sha256(dst.to_host().tobytes()).hexdigest(),
                  "entries": tune.entries()}))
"""


def _child(cache, mode):
    env = dict(os.environ, NCA_GB300_CACHE_DIR=str(cache),
               PYTHONPATH=str(ROOT) + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, "-c", CHILD, str(mode)], env=env, capture_output=True, text=True, cwd=ROOT,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_search_then_reuse(cuda, tmp_path):
    first = _child(tmp_path, 2)
    assert first["ok_ew"] and first["ok_nd"]
    keys = list(first["entries"])
    assert any(k.startswith("stencil3d|f32|1|") for k in keys), keys
    assert any(k.startswith("ew|k1|") for k in keys) and any(k.startswith("ew|k2|") for k in keys), keys
    for k, v in first["entries"].items():
        if k.startswith("stencil3d"):
            assert len(v) == 2 and 0 <= v[0] < 3 and v[1] in (8, 16, 32, 64)
        else:
            assert len(v) == 3 and v[0] in (128, 256, 512) and 1 <= v[1] <= 4
    second = _child(tmp_path, 1)
    assert second["ok_ew"] and second["ok_nd"]
    assert second["entries"] == first["entries"]
    assert second["stencil"] == first["stencil"]   # the same values whatever the tile
