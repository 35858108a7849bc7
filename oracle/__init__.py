"""CPU restatement of the reference PBD cloth step: test infrastructure only.

The product path never imports this package; tests/, the smoke check and the
cpu_baseline leg of bench.py use it as the checker.
"""
