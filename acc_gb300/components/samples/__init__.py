"""Samples (acc/components/samples)."""
