"""Numeric constants of PGMax (pgmax/utils/__init__.py:22-37, pgmax/factor/logical.py:33)."""

MSG_NEG_INF = -1e32
LOG_POTENTIAL_MAX_ABS = 1e6
NEG_INF = -float("inf")
TEMPERATURE_STABILITY_THRE = 0.5
