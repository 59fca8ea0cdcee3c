"""CPU oracle and reference harness (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline import this
package; the product never does.
"""
