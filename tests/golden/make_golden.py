"""Record golden vectors by running the reference implementation.

Run where the reference package is available: its checkout path comes from
argv[1] or the environment variable ``XGRID_REFERENCE``; further arguments name
the cases to record (default: all).  Each case of ``cases.py`` runs in its own process
with the reference's ``xgrid`` (its C backend compiled by gcc, OpenMP on) and
its outputs are written to ``<case>.npz`` beside this script.  The cases only
use inputs the reference handles correctly (see ``cases.py``).
"""
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))

CHILD = r"""
import sys, os, numpy as np
sys.path.insert(0, {ref!r})
sys.path.insert(1, {here!r})
import xgrid
assert os.path.abspath(xgrid.__file__).startswith(os.path.abspath({ref!r})), xgrid.__file__
from loader import load_cases
mod = load_cases(xgrid, ".xgridgolden", "ref")
out = mod.CASES[{case!r}]()
np.savez_compressed({dst!r}, **out)
"""


def main() -> None:
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("XGRID_REFERENCE")
    if not ref:
        sys.exit("usage: make_golden.py <reference checkout> (or set XGRID_REFERENCE)")
    sys.path.insert(0, HERE)
    names = [l.split("def ", 1)[1].split("(")[0] for l, prev in
             zip(open(os.path.join(HERE, "cases.py")).read().splitlines()[1:],
                 open(os.path.join(HERE, "cases.py")).read().splitlines())
             if prev.strip() == "@case"]
    names = sys.argv[2:] or names
    index = os.path.join(HERE, "golden_index.json")
    meta = json.load(open(index)) if os.path.exists(index) else {}
    for case in names:
        dst = os.path.join(HERE, f"{case}.npz")
        with tempfile.TemporaryDirectory() as tmp:
            code = CHILD.format(ref=ref, here=HERE, case=case, dst=dst)
            env = dict(os.environ, OMP_NUM_THREADS="4")
            proc = subprocess.run([sys.executable, "-c", code], cwd=tmp, capture_output=True, text=True, env=env)
        status = "ok" if proc.returncode == 0 else "failed"
        meta[case] = status
        print(case, status)
        if proc.returncode != 0:
            print(proc.stderr[-2000:])
    with open(index, "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
