"""CPU oracle for the min-max NUFFT path (test infrastructure only).

Nothing in the product package imports this directory.  It is used only by
``tests/``, by ``__graft_entry__.smoke()`` as the checker, and by ``bench.py``
for its CPU-baseline and reference-arm timings.
"""
