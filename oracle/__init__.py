"""ORACLE — test infrastructure only (CPU restatement of the reference loop).

Importable by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg;
never by the product package.
"""
