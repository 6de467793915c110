"""ORACLE — test infrastructure, not product code.

CPU restatement of the LSQuantumED hot path (see ``ed_oracle.cpp``).  Only
``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline /
reference arm import this package, and only as the checker or the timed CPU
baseline.  The ``lsquantumed_gb300`` package never imports it.

Parity of this restatement is pinned against the reference's own golden tests
(``tests/golden/reference_golden.json``, extracted from the reference's
``tests/unit_tests`` by ``tests/golden/make_golden.py``).
"""
from .oracle import *  # noqa: F401,F403
from .oracle import build, lib  # noqa: F401
