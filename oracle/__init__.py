"""CPU oracle for the GB300 dense-operator Krylov path.

Test infrastructure only: imported by tests/, by __graft_entry__.smoke() to
check its results, and by bench.py's CPU baseline and reference arm.  Never
part of the product path.
"""
