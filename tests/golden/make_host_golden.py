"""Record the reference program's own outputs for the drop-in comparison.

Runs the reference program (oracle/_ref/hsmc_ref, built from the reference
sources by oracle/Makefile) on the inputs in tests/golden/host_inputs/ and
stores, per input, its stdout and output files under tests/golden/host_ref/.
Also records its answers to `-e` and to malformed input files.  Run where the
reference sources are present:

    python tests/golden/make_host_golden.py
"""
from __future__ import annotations

import gzip
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import REF_EXE, build_oracle  # noqa: E402

INPUTS = os.path.join(HERE, "host_inputs")
OUT = os.path.join(HERE, "host_ref")

BAD_INPUTS = {
    "unknown_key.dat": "rho 0.5\nfoo 3\n",
    "missing_value.dat": "rho 0.5\nneigh_list 1.05\n",
    "long_restart.dat": "restart_read 1 " + "x" * 120 + "\n",
}


def main() -> None:
    build_oracle(with_reference=True)
    if os.path.isdir(OUT):
        shutil.rmtree(OUT)
    os.makedirs(OUT)
    ex = subprocess.run([REF_EXE, "-e"], capture_output=True, text=True, check=True)
    open(os.path.join(OUT, "example.txt"), "w").write(ex.stdout)
    for name, text in BAD_INPUTS.items():
        with tempfile.TemporaryDirectory() as td:
            open(os.path.join(td, "in.dat"), "w").write(text)
            r = subprocess.run([REF_EXE, "-i", "in.dat"], cwd=td, capture_output=True, text=True)
            open(os.path.join(OUT, name + ".stdout"), "w").write(r.stdout)
            open(os.path.join(OUT, name + ".rc"), "w").write(str(r.returncode))
    for inp in sorted(os.listdir(INPUTS)):
        case = os.path.splitext(inp)[0]
        dst = os.path.join(OUT, case)
        os.makedirs(dst)
        with tempfile.TemporaryDirectory() as td:
            shutil.copy(os.path.join(INPUTS, inp), os.path.join(td, "in.dat"))
            r = subprocess.run([REF_EXE, "-i", "in.dat"], cwd=td, capture_output=True, text=True, check=True)
            open(os.path.join(dst, "stdout.txt"), "w").write(r.stdout)
            for f in sorted(os.listdir(td)):
                if f == "in.dat":
                    continue
                src = os.path.join(td, f)
                if f.endswith(".gz"):
                    with gzip.open(src, "rt") as fh:
                        open(os.path.join(dst, f[:-3]), "w").write(fh.read())
                else:
                    shutil.copy(src, os.path.join(dst, f))
        print("recorded", case, sorted(os.listdir(dst)))


if __name__ == "__main__":
    main()
