"""CPU oracle for the GB300 channel-flow step -- TEST INFRASTRUCTURE.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
and reference legs import this package, and only as the checker or the timed
CPU baseline.  The product (``f90_dns_gb300``) never uses it.
"""
