"""Write the reference's own generated C for the benchmark programs.

Needs the reference checkout: argv[1] or the environment variable
``XGRID_REFERENCE``.  For each of
the benchmark programs in workloads.py (2-D diffusion and the lid-driven cavity
in FP64, the batched convection-diffusion step in FP32 with periodic edges) it
runs the reference's parser and C generator (xgrid/lang/generator.py), under the
configuration that program runs with, and writes the C source to
oracle/_ref/<kernel>.c.  Those files are not versioned;
they travel with the working tree and ``oracle.native.build_ref`` compiles them
with the reference's compiler flags on whatever host runs the baseline.
"""
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(HERE, "_ref")
# kernel -> (precision, overstep) it is generated under
KERNELS = {"diffusion2d": ("double", "none"), "cavity_kernel": ("double", "none"),
           "convdiff2d": ("float", "wrap")}

CHILD = r"""
import os, sys
sys.path.insert(0, {ref!r})
sys.path.insert(1, {root!r})
import xgrid
assert os.path.abspath(xgrid.__file__).startswith(os.path.abspath({ref!r}))
import workloads
from xgrid.lang.generator import Generator
for name, (precision, overstep) in {kernels!r}.items():
    # the parser fixes the width of float when it first reads a kernel, so each
    # kernel gets a fresh operator under its own configuration
    xgrid.init(parallel=True, precision=precision, overstep=overstep, opt_level=3, cacheroot=".xgridref")
    op = getattr(workloads, name)
    src = Generator(xgrid.kernel()(op.func)).source
    with open(os.path.join({out!r}, name + ".c"), "w") as f:
        f.write(src)
"""


def reference_checkout():
    """Path of the reference checkout from ``XGRID_REFERENCE``, or None."""
    ref = os.environ.get("XGRID_REFERENCE")
    return ref if ref and os.path.isdir(os.path.join(ref, "xgrid")) else None


def generate(ref: str) -> list:
    if not ref or not os.path.isdir(os.path.join(ref, "xgrid")):
        raise FileNotFoundError(f"reference checkout not found at {ref}")
    os.makedirs(OUT, exist_ok=True)
    code = CHILD.format(ref=ref, root=ROOT, kernels=KERNELS, out=OUT)
    with tempfile.TemporaryDirectory() as tmp:
        subprocess.run([sys.executable, "-c", code], cwd=tmp, check=True)
    return [os.path.join(OUT, k + ".c") for k in KERNELS]


if __name__ == "__main__":
    checkout = sys.argv[1] if len(sys.argv) > 1 else reference_checkout()
    if not checkout:
        sys.exit("usage: make_ref.py <reference checkout> (or set XGRID_REFERENCE)")
    for p in generate(checkout):
        print(p)
