"""CPU oracle for the TDVP/TEBD local-update path (test infrastructure only).

This package is a NumPy restatement of PyTreeNet's one-site/two-site TDVP
algorithm, used to check the GPU engine. It is imported only by ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py``; the
product path (``pytreenet_gb300``) never imports it.

Parity pin: the restatement is checked against the reference itself in
``tests/test_oracle_golden.py`` through the fixtures in ``tests/golden/``
(generated by ``tests/golden/make_golden.py``, which runs the reference's own
drivers on seeded inputs).
"""
from .ptn_oracle import *  # noqa: F401,F403
