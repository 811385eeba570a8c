"""End-to-end sweeps over the accelerated path (reference: benchmarks/)."""
