"""TEST INFRASTRUCTURE: the reference-kernel recipe and harness."""
