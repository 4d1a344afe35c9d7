"""ORACLE: CPU restatements of the reference's algorithms for the fused-tensor path.

Test infrastructure only.  ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline leg use it as the checker or the timed CPU
baseline; the product (compute.scala_gb300/) never imports it.

* ``interp`` - numpy evaluation of an IR text with the reference kernels' semantics;
* ``rng`` - the Wang-hash uniform and Box-Muller normal generators;
* ``clgen`` + ``cl_shim.h`` + ``cref`` - the reference's generated OpenCL C, compiled
  for the host with gcc/OpenMP (the CPU baseline and a second checker);
* ``cbuild`` - pre-builds the C parts.

Parity is pinned: ``interp``, ``rng`` and ``cref`` reproduce every golden
vector of the reference's own tests (tests/test_reference_goldens.py).
"""
