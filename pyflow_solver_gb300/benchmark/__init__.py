"""Benchmark harness (src/pyflow/benchmark/)."""
