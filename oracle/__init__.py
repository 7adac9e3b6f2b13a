"""Oracle package: CPU restatements of the reference's per-batch sorting path.

Test infrastructure only -- imported by ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` as the checker, never by the product path.
"""
