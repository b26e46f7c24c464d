"""Test infrastructure: the CPU oracle of the field-evaluation and rendering path.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this package.
"""
