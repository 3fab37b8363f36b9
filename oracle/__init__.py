"""CPU oracle of the RSF evolution (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use it, and
only as the checker / the timed CPU reference.  See rsf_oracle.c.  The
reference's own kernels (ref_build.py, ref_harness.py) are checkers too;
time_ref_kernels.py, run by hand, times them beside the product on a GPU.
"""
