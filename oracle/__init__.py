"""CPU oracle for the Fletcher TTI path -- TEST INFRASTRUCTURE ONLY.

Imported by tests/, the smoke check and bench.py's CPU-baseline leg; never by
the product package."""
