"""ORACLE — test infrastructure only: the CPU parity reference of the GPU engine.

Imported only by tests/, __graft_entry__.smoke() and bench.py's CPU legs."""
