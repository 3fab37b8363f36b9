"""CPU oracle of the RSF evolution (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use it, and
only as the checker / the timed CPU reference.  See rsf_oracle.c.
"""
