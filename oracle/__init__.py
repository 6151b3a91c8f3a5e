"""Test oracle package (test infrastructure only; see zfp_oracle.h)."""
