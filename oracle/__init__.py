"""The CPU oracle: a plain-C restatement of the reference renderer's hot
path (oracle/port), plus a build recipe for the reference itself
(oracle/ref, only where its sources are present).

This package is test infrastructure.  Only tests/, the smoke check and the
CPU baseline of bench.py import it, always as the checker; the product
(kodanuki_gb300) never does.
"""
from .port import build, lib  # noqa: F401
