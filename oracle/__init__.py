"""CPU oracle (test infrastructure only): see bldfm_oracle.py."""

from .build_oracle import build_oracle  # noqa: F401
