"""CPU oracle for pytreegrav_gb300 -- test infrastructure (parity checker and timed CPU baseline).

Nothing in the pytreegrav_gb300 package imports this; only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg do.
"""
