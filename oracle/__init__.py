"""Test infrastructure only: the CPU oracle for fastlem's generate().

Only `tests/`, `__graft_entry__.smoke()` and `bench.py`'s CPU-baseline legs use this
package, always as the checker or the timed CPU baseline, never as the product.
"""
