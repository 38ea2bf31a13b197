"""CPU oracle for the crossbar IR-drop solve.  TEST INFRASTRUCTURE ONLY.

Nothing in the product package (``fadesim_gb300``) imports this package.  Only
``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` / reference arm of
``bench.py`` use it, and only as the checker or as the timed CPU baseline.

Contents
--------
nodal      FP64 direct solve of the two-plane nodal system (sparse LU, plus a
           dense solve for small tiles).  This is the accuracy oracle.
sweeps     numpy restatement of the reference's Gauss-Seidel/SOR sweep order
           as PimTorch runs it (fixed sweep count, optional delta break).
au_gs.c    C restatement of crossbarHspice V1 ``array2D::nodeBasedGS`` (the
           lexicographic "Au" algorithm), built into ``oracle/_build``.
intstages  numpy restatement of PimTorch's integer stages: fixed-point
           quantisation, PN split, bit slicing, ADC codes and shift-add.
Makefile   builds the C port and, where the reference tree is present, the
           reference's own V1 ``sim`` into ``oracle/_ref``.

Pinning: the restatements are checked against fixtures produced by the
reference itself (its compiled ``sim`` and its PimTorch Python modules), see
``tests/golden/make_golden.py``.
"""
