"""Test infrastructure only: the CPU oracle (NumPy and C++ restatements of the
reference's algorithm) that tests/, the smoke check and bench.py's CPU legs check and
time against; the product never imports it."""
