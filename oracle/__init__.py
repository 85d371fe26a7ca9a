"""CPU oracle for the Black-Scholes map -- TEST INFRASTRUCTURE ONLY.

Importable only by tests/, the smoke check in __graft_entry__.py and the
cpu_baseline / reference legs of bench.py.  The product library never loads
it.  See oracle/bs_oracle.h for what each function restates.
"""
from .oracle import *  # noqa: F401,F403
