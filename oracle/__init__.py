"""CPU oracle for the SPH-DEM hot path -- test infrastructure only.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package, and only as the checker (or, in bench.py, as the timed CPU
baseline); the product library never calls it.
"""
