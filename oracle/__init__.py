"""Oracle of the GB300 stencil backend — TEST INFRASTRUCTURE, never the product.

* ``interp``/``xgrid_oracle``: numpy restatement of the reference's sweep
  semantics behind the same ``xgrid`` API (any DSL program runs on it).
* ``c/xg_oracle.c``: plain C (OpenMP) restatement of the two benchmark programs
  (2-D diffusion, lid-driven cavity), loop for loop like the reference's
  generated C; used for large-size checks and as the CPU baseline.
* ``make_ref.py``: writes the reference's own generated C for those programs
  into ``oracle/_ref/`` (needs the reference checkout; the output is not
  versioned) so it can be compiled on any host and timed as the reference.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
may import this package.
"""
