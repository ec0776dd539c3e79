"""CPU checker for the GB300 mobility library.  TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` import this package.  The product library never links, calls or
falls back to anything here.
"""
