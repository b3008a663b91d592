"""TEST INFRASTRUCTURE: CPU restatement of the reference's hot-path algorithms.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package, and only as the oracle that results are compared with or as the timed
CPU baseline.  The product library (fluxcore3d_gb300) never imports it.
"""
