"""CPU oracle for the cuPSS pseudospectral step (TEST INFRASTRUCTURE ONLY).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package.  The product never routes through it.
"""
