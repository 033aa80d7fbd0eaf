"""Record the reference executables' diagnostics for the CLI cases.

Runs the reference svo_builder / svo_builder_binary built from the reference's own
sources by ``make -C oracle ref`` (output oracle/_ref/) on every case of
tests/cli_cases.py and stores, per case, the diagnostic lines and the exit status in
cli_messages.json, and for the complete runs (FULL_RUNS) every line with the timer
values masked in cli_full_runs.json.  Regenerate with ``python tests/golden/make_cli_golden.py``
(needs the reference build).
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

import cli_cases  # noqa: E402


def main() -> None:
    ref = os.path.join(ROOT, "oracle", "_ref")
    out = {}
    with tempfile.TemporaryDirectory() as d:
        cli_cases.make_inputs(d)
        for exe, args in cli_cases.CASES:
            r = subprocess.run([os.path.join(ref, exe), *args], cwd=d, stdout=subprocess.PIPE, text=True,
                               timeout=120)
            out[cli_cases.case_id(exe, args)] = {"status": r.returncode, "lines": cli_cases.diagnostics(r.stdout)}
        full = {}
        for exe, args in cli_cases.FULL_RUNS:
            r = subprocess.run([os.path.join(ref, exe), *args], cwd=d, stdout=subprocess.PIPE, text=True,
                               timeout=120)
            full[cli_cases.case_id(exe, args)] = {"status": r.returncode, "lines": cli_cases.full_run_lines(r.stdout)}
    with open(os.path.join(HERE, "cli_messages.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    with open(os.path.join(HERE, "cli_full_runs.json"), "w") as f:
        json.dump(full, f, indent=1)
        f.write("\n")
    print("wrote %d cases and %d complete runs" % (len(out), len(full)))


if __name__ == "__main__":
    main()
