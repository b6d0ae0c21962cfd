"""CPU oracle for the Bubbles 3D SPH/PCISPH step -- test infrastructure only.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU baseline; never by
the product package.
"""
