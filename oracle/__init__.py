"""CPU oracle of HEAL's sample implementation — test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it,
and only as the checker; the product package never imports it.
"""
