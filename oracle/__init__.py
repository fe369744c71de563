"""CPU oracle package (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import this package;
the library under integrator2_gb300/ never does.
"""
