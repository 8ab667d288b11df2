"""CPU checker for the DDGI probe update (test infrastructure only).

Only the tests, the package smoke check and the benchmark's CPU-baseline leg
load this package.  See ddgi_oracle.cpp for the restated reference code.
"""
from .oracle import Oracle, build_oracle, oracle_lib_path  # noqa: F401
