"""ORACLE -- test infrastructure, not product code.

CPU restatement of the reference's energy/force/MD hot path
(src/mlff_distiller/models/student_model.py, inference/ase_calculator.py,
testing/nve_harness.py).  Only tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline / reference legs may import this package, and only
to check results (or as the timed CPU baseline); the product path never does.

Parity pins: tests/test_oracle_golden.py checks this restatement against
golden vectors produced by the reference implementation itself
(tests/golden/make_golden.py, run where the reference is importable).
"""
