"""CPU oracle for the B2R stencil hot path -- test infrastructure only.

Importable from tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg.  The product package (b2r_gb300) never imports it.
"""
