"""CPU oracle of the XPBD cloth substep -- test infrastructure only.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package.  The product (the CUDA library and its
Python front end) never does.
"""
