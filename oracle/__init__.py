"""CPU oracle of the fix-eph hot path.  TEST INFRASTRUCTURE ONLY: imported by
tests/, __graft_entry__.smoke() and the cpu_baseline leg of bench.py as the
checker; the product never imports it."""
