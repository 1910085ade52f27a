"""CPU oracle for torchquad_gb300 — TEST INFRASTRUCTURE ONLY.

A numpy restatement of the reference torchquad (v0.5.0) algorithms on the
integration hot path, each function citing the reference file:line it
follows.  Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s
CPU-baseline / reference arm may import it, and only to check results or as
the timed CPU baseline; the product package never imports it.

Parity pin: ``tests/golden/*.json`` hold outputs of the unmodified reference
(run here through ``tests/golden/make_golden.py``); ``tests/test_oracle.py``
checks this restatement against them and against the reference tests' own
golden vectors.
"""
