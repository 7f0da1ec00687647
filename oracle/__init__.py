"""The oracle: a CPU FP64 restatement of CalChem's XC quadrature (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this package, as the checker.  The product (``calchem_gb300``)
never imports it.
"""
