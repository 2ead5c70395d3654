"""Record the digests of ``full_cases.py`` by running the reference implementation.

Run where the reference package is available: its checkout path comes from
argv[1] or the environment variable ``XGRID_REFERENCE``; further arguments
name the cases to record (default: all; the others keep their digests).  Each case runs in its own process with the
reference's ``xgrid`` (its C backend compiled by gcc, OpenMP on); the SHA-256 of
every time level of every grid goes to ``full_digests.json`` beside this script.
"""
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))

CHILD = r"""
import json, sys, os
sys.path.insert(0, {ref!r})
sys.path.insert(1, {here!r})
import xgrid
assert os.path.abspath(xgrid.__file__).startswith(os.path.abspath({ref!r})), xgrid.__file__
from loader import load_cases
mod = load_cases(xgrid, ".xgriddigest", "ref", "full_cases.py")
print(json.dumps(mod.FULL[{case!r}]()))
"""


def main() -> None:
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("XGRID_REFERENCE")
    if not ref:
        sys.exit("usage: make_digests.py <reference checkout> [case ...] (or set XGRID_REFERENCE)")
    sys.path.insert(0, HERE)
    from loader import load_cases
    names = sys.argv[2:] or list(load_cases(None, "", "names", "full_cases.py").FULL)
    path = os.path.join(HERE, "full_digests.json")
    out = json.load(open(path)) if os.path.exists(path) else {}
    for case in names:
        with tempfile.TemporaryDirectory() as tmp:
            code = CHILD.format(ref=ref, here=HERE, case=case)
            env = dict(os.environ, OMP_NUM_THREADS=str(os.cpu_count() or 4))
            proc = subprocess.run([sys.executable, "-c", code], cwd=tmp, capture_output=True, text=True, env=env)
        if proc.returncode != 0:
            print(case, "failed")
            print(proc.stderr[-2000:])
            continue
        out[case] = json.loads(proc.stdout.strip().splitlines()[-1])
        print(case, "ok")
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
