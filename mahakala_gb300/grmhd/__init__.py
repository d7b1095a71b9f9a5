"""Fluid models: resident GRMHD snapshots and the synthetic snapshot generator."""
