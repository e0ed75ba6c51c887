"""ORACLE -- test infrastructure only.

A CPU restatement of the reference's RKHEVI step (game_oracle.c), its ctypes
binding (bind.py) and the recipe that compiles the reference's own C sources
for pinning it (build_ref.py).  Only tests/, __graft_entry__.smoke() and the
CPU-baseline arm of bench.py may use anything here, and only as the checker.
"""
