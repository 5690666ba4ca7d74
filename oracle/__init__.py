"""CPU oracle for parity tests: a restatement of the reference's algorithm (dsrim/adrt-pinv).

Test infrastructure only. The product (the `adrt-pinv_gb300` package and its CUDA library) never imports,
links or runs anything in this directory; only `tests/`, `__graft_entry__.smoke()` and `bench.py`'s CPU
baseline do, as the checker or as the timed CPU baseline.
"""
