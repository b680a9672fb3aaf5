"""The autotuner's cache (tune.txt in the JIT cache directory): one line per
key, "<key> <values...>"; read back through nca_tune_get, forgotten by
nca_tune_clear; modes outside 0..2 are rejected. Runs without a GPU (in a
child process, so the cache directory it sets is its own)."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

CHILD = r"""
import json, sys
from pathlib import Path
from ncarray_gb300 import _lib, tune
d = Path(sys.argv[1])
(d / "tune.txt").write_text("stencil3d|f32|1|9x9x9 1 32\new|k1|10|10|10.|v4|n24|d1 256 4 2048\nbroken-line\n")
out = {"stencil": tune.get("stencil3d|f32|1|9x9x9"), "ew": tune.get("ew|k1|10|10|10.|v4|n24|d1"),
       "missing": tune.get("nope"), "entries": tune.entries(str(d))}
try:
    tune.set_mode(3)
    out["bad_mode"] = "accepted"
except _lib.NcaError as e:
    out["bad_mode"] = e.status
tune.set_mode(0)
out["mode0_file_kept"] = (d / "tune.txt").exists()
tune.clear()
out["cleared"] = not (d / "tune.txt").exists() and tune.get("stencil3d|f32|1|9x9x9") is None
print(json.dumps(out))
"""


def test_tune_cache_file(built_lib, tmp_path):
    env = dict(os.environ, NCA_GB300_CACHE_DIR=str(tmp_path),
               PYTHONPATH=str(ROOT) + os.pathsep + os.environ.get("PYTHONPATH", ""))
    r = subprocess.run([sys.executable, "-c", CHILD, str(tmp_path)], env=env, capture_output=True, text=True,
                       cwd=ROOT, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["stencil"] == [1, 32]
    assert out["ew"] == [256, 4, 2048]
    assert out["missing"] is None
    assert out["entries"]["stencil3d|f32|1|9x9x9"] == [1, 32]
    assert out["bad_mode"] == 1   # NCA_ERR_INVALID
    assert out["mode0_file_kept"] and out["cleared"]
