"""Builds and runs the drop-in check program (tests/dropin/Makefile) and, with
--write, stores its output as tests/golden/dropin_cases.json: the C-ABI
descriptors (nca_tape, nca_view) that ncarray's own code produces for a few
expressions, a stencil and reduction-axis sets through include/ncarray_dropin.
Needs the reference sources (the Makefile's REF); the GPU test replays the
stored descriptors where they are absent."""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
FIXTURE = HERE.parent / "golden" / "dropin_cases.json"


def have_reference() -> bool:
    return subprocess.run(["make", "-s", "-C", str(HERE), "have-ref"], capture_output=True).returncode == 0


def build_and_run() -> list:
    subprocess.run(["make", "-s", "-C", str(HERE), "check"], check=True)
    out = subprocess.run([str(HERE / "_build" / "check_dropin")], check=True, capture_output=True, text=True)
    return json.loads(out.stdout)


if __name__ == "__main__":
    cases = build_and_run()
    if "--write" in sys.argv:
        FIXTURE.write_text(json.dumps(cases, indent=1) + "\n")
        print(f"wrote {FIXTURE} ({len(cases)} cases)")
    else:
        print(json.dumps(cases, indent=1))
