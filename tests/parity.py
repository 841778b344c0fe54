"""The parity bar of the GPU tests (shared with bench.py's CPU leg):
hit/miss, meshIndex and triangleIndex agree with the oracle on >= 99.99 % of
rays; every disagreement is a tie with |dt| <= 1e-6 * t; t, b1, b2 agree
within 1e-5 relative where the triangle agrees."""
from oracle.parity import AGREE_MIN, TIE_REL, VAL_REL, check_anyhit, compare  # noqa: F401
