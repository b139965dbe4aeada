"""Learned layout selector: workload generator, timing sweep, training."""
