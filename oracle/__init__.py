"""ORACLE: CPU restatement of warp_cfd's SIMPLE/PISO step, used only as the checker by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg.  Never imported by
the product package."""
