"""CPU oracle for the laser-polio per-tick agent step.

Test infrastructure: only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline use this package.  The product (laser_polio_gb300) never imports it.
"""
