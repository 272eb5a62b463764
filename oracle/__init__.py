"""ORACLE — test infrastructure, not product code.

CPU restatement of the reference's training path (oracle.hpp) and the recipe
that compiles the reference itself here (ref/).  Only tests, the smoke check
and the benchmark's CPU-baseline leg import this package, to check results or
as the timed CPU path.
"""
