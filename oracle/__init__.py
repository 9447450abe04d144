"""CPU oracle for the exterior Burton-Miller BEM path (test infrastructure only).

Nothing in the product package imports this package.  Tests, the smoke check and
the benchmark's CPU baseline / reference arm use it as the checker.
"""
