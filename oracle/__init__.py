"""CPU oracle of the Blitzen culling path. TEST INFRASTRUCTURE ONLY.

Imported by tests/, by __graft_entry__.smoke() as the checker and by bench.py's CPU-baseline leg;
the product package never imports it.
"""
