"""CPU FP64 oracle of the reference DG scalar-wave step (test infrastructure).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use this
package; the product (spectre_gb300) never imports it.
"""
